"""The layer path's solver strategies on the CPU, with the drop-in's solve
replaced by a recording fake: which method, tolerance and stop mode each
strategy asks for, and that superposition forms the currents by linearity
from the unit responses it requested."""
import pytest

torch = pytest.importorskip("torch")

from fadesim_gb300 import splitarr  # noqa: E402
from fadesim_gb300 import cpp_ir_drop_accelerate as acc  # noqa: E402


@pytest.fixture
def calls(monkeypatch):
    seen = []

    def fake(v, G, B, rows, cols, numX, numY, **kw):
        seen.append(dict(B=B, rows=rows, cols=cols, **kw))
        # currents linear in the inputs: I[b, x, j] = sum_r v[b, x, r] * (r + 1) * (j + 1)
        w = torch.arange(1, rows + 1, dtype=v.dtype)[:, None] * torch.arange(1, numY * cols + 1, dtype=v.dtype)[None]
        return torch.einsum("bxr,rj->bxj", v, w), {"status_or": 1, "solves": B * numX * numY}, None

    monkeypatch.setattr(acc, "ir_drop_gs_ex", fake)
    return seen


def cfg(n):
    return splitarr.ArrayConfig(Ron=1e3, Roff=1e6, cellBits=2, arrRowSize=n, arrColSize=n, inputMaxVoltage=0.2)


@pytest.mark.parametrize("n,fp32_limit,method", [(128, True, "line_coarse"), (128, False, None), (64, True, None)])
def test_superposition_unit_response_call(calls, n, fp32_limit, method):
    B, X = 2 * n, 2
    v = (torch.rand((B, X, n)) < 0.5).float() * 0.2
    G = torch.rand((X, n, n))
    out = splitarr.superposition_solver(cfg(n), fp32_limit=fp32_limit)(v, G, B, n, n, X, 1, None)
    assert len(calls) == 1
    c = calls[0]
    assert c["B"] == n and c["method"] == method
    assert c["fp32_limit"] == (True if method else None)
    assert c["tol_v"] == pytest.approx(acc.options.tol_v * 2e-3)
    w = torch.arange(1, n + 1.0)[:, None] * torch.arange(1, n + 1.0)[None]
    assert torch.allclose(out.reshape(B, X, n), torch.einsum("bxr,rj->bxj", v, w), rtol=1e-5)


def test_direct_solver_uses_the_module_options(calls):
    v = torch.zeros((3, 1, 16))
    splitarr.default_solver(cfg(16))(v, torch.zeros((1, 16, 16)), 3, 16, 16, 1, 1, None)
    assert calls[0]["method"] is None and calls[0]["fp32_limit"] is None and calls[0]["tol_v"] is None
