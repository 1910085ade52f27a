"""GPU parity of the grid rules against the reference's golden outputs."""
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300 import _lib as L
from torchquad_gb300.integration import _kernels as K
from tests import golden as G

pytestmark = pytest.mark.gpu

GRID = G.load("grid_mc_golden.json")["grid"]
FAMS = {"ExpSum": tq.ExpSum, "GaussianPeak": tq.GaussianPeak, "Oscillatory": tq.Oscillatory, "SumSin": tq.SumSin}


def _integrand(case):
    kw = {k: v for k, v in case["family"].items() if k != "kind"}
    return FAMS[case["family"]["kind"]](case["dim"], **kw)


def _tol(case):
    # tolerances: 1e-12 relative in fp64, 1e-6 in fp32
    return 1e-12 if case["result_dtype"] == "float64" and case["dtype"] == "float64" else (
        1e-12 if case["rule"] == "GaussLegendre" else 1e-6)


def _run(case, fused, cuda):
    f = _integrand(case)
    fn = f if fused else (lambda x: f(x))
    domain = torch.tensor(case["domain"], dtype=getattr(torch, case["dtype"]), device=cuda)
    integ = getattr(tq, case["rule"])()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        val = integ.integrate(fn, case["dim"], N=case["N"], integration_domain=domain)
    return integ, val


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "materialised"])
@pytest.mark.parametrize("case", GRID, ids=lambda c: c["name"])
def test_grid_matches_reference(case, fused, cuda):
    integ, val = _run(case, fused, cuda)
    want = G.f(case["value"])
    assert str(val.dtype).replace("torch.", "") == case["result_dtype"]
    assert val.shape == ()
    assert integ._nr_of_fevals == case["fevals"]
    got = val.item()
    assert abs(got - want) <= _tol(case) * max(1.0, abs(want)), (got, want)


def test_points_bitwise_equal_torch_cpu_linspace(cuda):
    for c in G.load("grid_mc_golden.json")["linspace"]:
        dt = getattr(torch, c["dtype"])
        dom = torch.tensor([[G.f(c["a"]), G.f(c["b"])]], dtype=dt, device=cuda)
        pts = K.grid_points(L.TQ_RULE_TRAPEZOID, 1, c["n"], dom, None, 0, c["n"], dt)
        assert np.array_equal(pts[:, 0].double().cpu().numpy(), G.arr(c["values"]))


def test_grid_points_layout_last_dim_fastest(cuda):
    dom = torch.tensor([[0.0, 1.0], [10.0, 12.0], [-1.0, 1.0]], dtype=torch.float64, device=cuda)
    pts = K.grid_points(L.TQ_RULE_TRAPEZOID, 3, 3, dom, None, 0, 27, torch.float64).cpu()
    g = [torch.linspace(0, 1, 3, dtype=torch.float64), torch.linspace(10, 12, 3, dtype=torch.float64),
         torch.linspace(-1, 1, 3, dtype=torch.float64)]
    want = torch.stack([m.ravel() for m in torch.meshgrid(*g, indexing="ij")], dim=1)
    assert torch.equal(pts, want)
    # a sub-range equals the same rows of the full grid
    sub = K.grid_points(L.TQ_RULE_TRAPEZOID, 3, 3, dom, None, 5, 11, torch.float64).cpu()
    assert torch.equal(sub, want[5:16])


def test_calculate_grid_staged_api(cuda):
    simp = tq.Simpson()
    dom = torch.tensor([[0.0, 1.0], [0.0, 2.0]], dtype=torch.float64, device=cuda)
    pts, hs, n = simp.calculate_grid(25, dom)
    assert pts.shape == (25, 2) and n == 5
    assert torch.allclose(hs.cpu(), torch.tensor([0.25, 0.5], dtype=torch.float64))
    f = 1.0 + 2.0 * pts[:, 0] + 3.0 * pts[:, 1] ** 2
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        r = simp.calculate_result(f, 2, n, hs, dom)
    assert abs(r.item() - 12.0) < 1e-12


@pytest.mark.parametrize("case", G.load("grid_mc_golden.json")["multidim"], ids=lambda c: c["rule"])
def test_vector_and_complex_integrands(case, cuda):
    dom = torch.tensor(case["domain"], dtype=torch.float64, device=cuda)

    def vec(x):
        base = torch.exp(0.3 * x[:, 0] - 0.2 * x[:, 1])
        scale = torch.arange(6, dtype=x.dtype, device=x.device).reshape(2, 3) + 1.0
        return base[:, None, None] * scale[None] + x[:, 0:1, None] * x[:, 1:2, None]

    def cplx(x):
        return torch.exp(1j * (x[:, 0] + 0.5 * x[:, 1]))

    integ = getattr(tq, case["rule"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v = integ().integrate(vec, 2, N=case["N"], integration_domain=dom)
        c = integ().integrate(cplx, 2, N=case["N"], integration_domain=dom)
    assert list(v.shape) == case["vec_shape"]
    assert np.allclose(v.cpu().numpy().ravel(), G.arr(case["vec"]), rtol=1e-12, atol=1e-13)
    assert abs(c.real.item() - G.f(case["cplx"][0])) < 1e-12
    assert abs(c.imag.item() - G.f(case["cplx"][1])) < 1e-12


def test_non_vectorised_integrand_raises(cuda):
    with pytest.raises(ValueError, match="vectorized"):
        tq.Trapezoid().integrate(lambda x: torch.ones(3, device=x.device), 1, N=10,
                                 integration_domain=[[0.0, 1.0]])


def test_chunked_materialised_path_equals_single_chunk(cuda):
    f = tq.GaussianPeak(3, a=[2.0, 1.0, 3.0], u=[0.2, 0.5, 0.7])
    dom = torch.tensor([[0.0, 1.0]] * 3, dtype=torch.float64, device=cuda)
    full = tq.Boole().integrate(lambda x: f(x), 3, N=41**3, integration_domain=dom)
    tq.set_materialise_budget(1 << 16)
    try:
        chunked = tq.Boole().integrate(lambda x: f(x), 3, N=41**3, integration_domain=dom)
    finally:
        tq.set_materialise_budget(8 << 30)
    assert abs(full.item() - chunked.item()) <= 1e-6 * abs(full.item())


def test_large_fused_c1_full_size(cuda):
    # plain Simpson at its full 101^3 fp64 size against the reference value
    dom = torch.tensor([[0.0, 1.0]] * 3, dtype=torch.float64, device=cuda)
    v = tq.Simpson().integrate(tq.ExpSum(3), 3, N=1030301, integration_domain=dom)
    assert abs(v.item() - 5.073214112618379) <= 1e-12 * 5.08
