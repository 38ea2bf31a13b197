"""The allocation-free entry point against the allocating one, through the C ABI.

fadesim_ir_drop_gs_noalloc_f32 is for callers that cannot allocate device
memory (code inside a stream capture they do not own, allocation-free host
callbacks or real-time loops, fixed device-memory budgets).  It keeps its
scratch in one static device array shared by every call, so this test runs it
twice in a row -- the second call sees the first call's leftovers -- and
compares both results with fadesim_ir_drop_gs_f32 on the same inputs.  The file
is named so pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GW = 1 / 2.93
I_RTOL = 1e-6  # current tolerance the line-solver tests use for weak cells


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import _lib
    from fadesim_gb300.build import build
    build()
    return _lib.load()


def case(seed, B, X, Y, n, m):
    rng = np.random.default_rng(seed)
    G = (1.0 / np.array([2e6, 1.6e6, 1.3e6, 1e6])[rng.integers(0, 4, (X, n, Y * m))]).astype(np.float32)
    inp = (rng.integers(0, 2, (B, X, n)) * 0.2).astype(np.float32)
    return torch.from_numpy(inp).cuda(), torch.from_numpy(G).cuda()


@pytest.mark.parametrize("shape", [(6, 3, 2, 128, 128), (5, 2, 3, 64, 48)])
def test_noalloc_matches_allocating_entry_twice(lib, shape):
    B, X, Y, n, m = shape
    ti, tg = case(sum(shape), B, X, Y, n, m)
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.empty((B, X, Y * m), dtype=torch.float32, device="cuda")
    rc = lib.fadesim_ir_drop_gs_f32(ti.data_ptr(), tg.data_ptr(), B, n, m, X, Y, 600, GW, 1.9, 0, 1e-7, 0, None, 0, 0,
                                    ref.data_ptr(), stream)
    assert rc == 0, lib.fadesim_last_error()
    torch.cuda.synchronize()
    for call in range(2):
        out = torch.full((B, X, Y * m), float("nan"), dtype=torch.float32, device="cuda")
        rc = lib.fadesim_ir_drop_gs_noalloc_f32(ti.data_ptr(), tg.data_ptr(), B, n, m, X, Y, GW, out.data_ptr(),
                                                stream)
        assert rc == 0, lib.fadesim_noalloc_last_error()
        torch.cuda.synchronize()
        err = (out - ref).abs().max().item()
        assert err <= I_RTOL * ref.abs().max().item(), (call, err)


def test_noalloc_rejects_tiles_beyond_its_scratch(lib):
    ti, tg = case(1, 1, 1, 1, 8, 8)
    rc = lib.fadesim_ir_drop_gs_noalloc_f32(ti.data_ptr(), tg.data_ptr(), 1, 256, 256, 1, 1, GW, tg.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert b"2..128" in lib.fadesim_noalloc_last_error()
    assert lib.fadesim_noalloc_scratch_bytes() == 24 << 20
