"""The allocation-free entry point against the allocating one and the FP64
oracle, through the C ABI.

fadesim_ir_drop_gs_noalloc_f32 is for callers that cannot allocate device
memory (code inside a stream capture they do not own, allocation-free host
callbacks or real-time loops, fixed device-memory budgets).  It keeps its
scratch in one static device array shared by every call, so this test runs it
twice in a row -- the second call sees the first call's leftovers -- and
compares both results with fadesim_ir_drop_gs_f32 on the same inputs and with
the FP64 nodal oracle, reading each call's status back from the static array
(fadesim_noalloc_last_status).  The file is named so pytest collects it last.

The grid cap of the entry (CTA pivot slots that fit the 24 MiB array) does not
bind on a 152-SM GB300: the largest tile (128 x 128) needs 135 KB per CTA, 186
slots, for 152 resident CTAs; smaller tiles need less per CTA than the CTAs
they add.  No test here can reach it.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import nodal  # noqa: E402

GW = 1 / 2.93
I_RTOL = 1e-6   # current tolerance the line-solver tests use for weak cells
I_ORACLE = 1e-4  # relative current tolerance against the FP64 oracle
ST_CONVERGED, ST_MAXITER, ST_NONFINITE = 1, 2, 4


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
    return inp, G


def last_status(lib, stream):
    from fadesim_gb300 import _lib
    st = _lib.SolveStats()
    rc = lib.fadesim_noalloc_last_status(ctypes.byref(st), stream)
    assert rc == 0, lib.fadesim_noalloc_last_error()
    return st


@pytest.mark.parametrize("shape", [(6, 3, 2, 128, 128), (5, 2, 3, 64, 48)])
def test_noalloc_matches_allocating_entry_and_oracle_twice(lib, shape):
    B, X, Y, n, m = shape
    inp, G = case(sum(shape), B, X, Y, n, m)
    ti, tg = torch.from_numpy(inp).cuda(), torch.from_numpy(G).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.empty((B, X, Y * m), dtype=torch.float32, device="cuda")
    rc = lib.fadesim_ir_drop_gs_f32(ti.data_ptr(), tg.data_ptr(), B, n, m, X, Y, 600, GW, 1.9, 0, 1e-7, 0, None, 0, 0,
                                    ref.data_ptr(), stream)
    assert rc == 0, lib.fadesim_last_error()
    torch.cuda.synchronize()
    oracle = nodal.solve_layer(inp, G, n, m, X, Y, GW)
    for call in range(2):
        out = torch.full((B, X, Y * m), float("nan"), dtype=torch.float32, device="cuda")
        rc = lib.fadesim_ir_drop_gs_noalloc_f32(ti.data_ptr(), tg.data_ptr(), B, n, m, X, Y, GW, out.data_ptr(),
                                                stream)
        assert rc == 0, lib.fadesim_noalloc_last_error()
        st = last_status(lib, stream)
        assert st.solves == B * X * Y and st.status_or == ST_CONVERGED, (call, st.solves, st.status_or)
        assert 1 <= st.iters_max <= 400
        err = (out - ref).abs().max().item()
        assert err <= I_RTOL * ref.abs().max().item(), (call, err)
        oerr = np.abs(out.double().cpu().numpy() - oracle).max() / np.abs(oracle).max()
        assert oerr <= I_ORACLE, (call, oerr)


def test_noalloc_reports_nonfinite_input(lib):
    """A NaN conductance ends its solve with the non-finite status; the next
    call, on clean inputs, reads back clean counters."""
    inp, G = case(3, 2, 2, 1, 32, 32)
    G_bad = G.copy()
    G_bad[1, 5, 7] = np.nan
    stream = torch.cuda.current_stream().cuda_stream
    ti = torch.from_numpy(inp).cuda()
    out = torch.empty((2, 2, 32), dtype=torch.float32, device="cuda")
    tb = torch.from_numpy(G_bad).cuda()
    assert lib.fadesim_ir_drop_gs_noalloc_f32(ti.data_ptr(), tb.data_ptr(), 2, 32, 32, 2, 1, GW, out.data_ptr(),
                                              stream) == 0
    assert last_status(lib, stream).status_or & ST_NONFINITE
    tg = torch.from_numpy(G).cuda()
    assert lib.fadesim_ir_drop_gs_noalloc_f32(ti.data_ptr(), tg.data_ptr(), 2, 32, 32, 2, 1, GW, out.data_ptr(),
                                              stream) == 0
    assert last_status(lib, stream).status_or == ST_CONVERGED


def test_noalloc_rejects_tiles_beyond_its_scratch(lib):
    inp, G = case(1, 1, 1, 1, 8, 8)
    tg = torch.from_numpy(G).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.fadesim_ir_drop_gs_noalloc_f32(tg.data_ptr(), tg.data_ptr(), 1, 256, 256, 1, 1, GW, tg.data_ptr(), stream)
    assert rc == -1
    assert b"2..128" in lib.fadesim_noalloc_last_error()
    assert lib.fadesim_noalloc_scratch_bytes() == 24 << 20
    for bad in (float("inf"), float("nan"), 0.0):
        rc = lib.fadesim_ir_drop_gs_noalloc_f32(tg.data_ptr(), tg.data_ptr(), 1, 8, 8, 1, 1, bad, tg.data_ptr(), stream)
        assert rc == -1 and b"g_wire" in lib.fadesim_noalloc_last_error()
