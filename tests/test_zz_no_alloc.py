"""The allocation-free fused grid entry point (tq_grid_fused_noalloc).

It exists for callers that cannot allocate device memory when they call:
a plugin whose host application owns every device allocation, code that
must not allocate once it runs, or a C caller without an allocator.  Its
scratch is a static device array shared by every call, so this file is
collected last and checks, through the C ABI, that two calls in a row give
the same result as the workspace-taking entry point (tq_grid_fused) and as
the unmodified reference (its recorded golden values), within the
tolerances of the grid-rule parity tests.  It passes alone in a fresh
process (the first call does the per-device set-up) and after the others.
"""
import pytest
import torch

from tests import golden as G
from torchquad_gb300 import _lib as L

CASES = [
    # rule, dtype, dim, n, family, params (c, b, a[dim], u[dim]), domain, rel. tolerance,
    # name of the reference's recorded value for the same integral (or None)
    (L.TQ_RULE_SIMPSON, torch.float64, 3, 101, L.TQ_FN_EXP_SUM, [1.0, 0.0] + [1.0] * 3 + [0.0] * 3,
     [[0.0, 1.0]] * 3, 1e-12, "C1-Simpson-expsum3-101"),
    (L.TQ_RULE_GAUSS, torch.float64, 4, 32, L.TQ_FN_OSCILLATORY,
     [1.0, 0.37, 1.2, -2.1, 0.7, 2.6] + [0.0] * 4, [[0.0, 1.0]] * 4, 1e-12, "C4-GaussLegendre-osc4-32"),
    (L.TQ_RULE_BOOLE, torch.float32, 2, 401, L.TQ_FN_GAUSSIAN, [1.5, 0.0, 2.0, 3.0, 0.3, 0.6],
     [[-1.0, 1.0], [0.0, 2.0]], 1e-6, None),
]


def _reference_value(name):
    if name is None:
        return None
    (case,) = [c for c in G.load("grid_mc_golden.json")["grid"] if c["name"] == name]
    return G.f(case["value"])


def test_scratch_status_string():
    # the rejection of a launch larger than the static scratch has its own
    # status and message (no GPU needed)
    L.load()
    assert L.TQ_ERR_SCRATCH == -10
    msg = L.status_string(L.TQ_ERR_SCRATCH)
    assert msg != "unknown status" and "scratch" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=["simpson-f64", "gauss-f64", "boole-f32"])
def test_noalloc_matches_workspace_entry_point_twice(case, cuda):
    rule, dtype, dim, n, fam, params, dom, tol, golden = case
    want = _reference_value(golden)
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    d = torch.tensor(dom, dtype=dtype, device=cuda)
    p = torch.tensor(params, dtype=torch.float64, device=cuda)
    nodes = weights = None
    if rule == L.TQ_RULE_GAUSS:
        import numpy as np

        r, w = np.polynomial.legendre.leggauss(n)
        nodes = torch.tensor(r, dtype=torch.float64, device=cuda)
        weights = torch.tensor(w, dtype=torch.float64, device=cuda)
    out_dtype = torch.float64 if rule == L.TQ_RULE_GAUSS else dtype
    code = L.dtype_code(dtype)
    ocode = L.dtype_code(out_dtype)

    ref = torch.empty((), dtype=out_dtype, device=cuda)
    ws = torch.zeros(lib.tq_grid_fused_workspace_size(rule, dim, n), dtype=torch.uint8, device=cuda)
    rc = lib.tq_grid_fused(code, rule, dim, n, d.data_ptr(), L.ptr(nodes), L.ptr(weights), fam,
                           p.data_ptr(), ref.data_ptr(), ocode, None, ws.data_ptr(), ws.numel(), stream)
    assert rc == L.TQ_OK, L.status_string(rc)

    for _ in range(2):  # the second call reuses the static scratch the first one left
        out = torch.full((), float("nan"), dtype=out_dtype, device=cuda)
        rc = lib.tq_grid_fused_noalloc(code, rule, dim, n, d.data_ptr(), L.ptr(nodes), L.ptr(weights),
                                       fam, p.data_ptr(), out.data_ptr(), ocode, None, stream)
        assert rc == L.TQ_OK, L.status_string(rc)
        torch.cuda.synchronize()
        a, b = out.item(), ref.item()
        assert abs(a - b) <= tol * max(1.0, abs(b)), (a, b)
        if want is not None:  # the reference's own value for this integral
            assert abs(a - want) <= tol * abs(want), (a, want)
