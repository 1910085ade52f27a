"""Gradients: the hand-written adjoint kernel of the fused grid rules against
the reference's torch autograd (golden) and central finite differences, and
the reference's own gradient tests (gradient_test.py:162-259) for every
integrator on arbitrary torch integrands."""
import math
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from tests import golden as G

pytestmark = pytest.mark.gpu

GRADS = G.load("grid_mc_golden.json")["grads"]
F64 = torch.float64


def _build(case, cuda):
    params = {}
    for k, v in case["params"].items():
        if k in case["grad_params"]:
            params[k] = torch.tensor(v, dtype=F64, device=cuda, requires_grad=True)
        else:
            params[k] = v
    f = getattr(tq, case["family"])(case["dim"], **params)
    dom = torch.tensor(case["domain"], dtype=getattr(torch, case["dtype"]), device=cuda, requires_grad=True)
    return f, params, dom


@pytest.mark.parametrize("case", GRADS, ids=lambda c: c["name"])
def test_adjoint_matches_reference_autograd(case, cuda):
    f, params, dom = _build(case, cuda)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        val = getattr(tq, case["rule"])().integrate(f, case["dim"], N=case["N"], integration_domain=dom)
    assert "FusedGridFn" in type(val.grad_fn).__name__  # the adjoint kernel path
    val.backward()
    f32 = case["dtype"] == "float32" and case["rule"] != "GaussLegendre"
    tol = 1e-5 if f32 else 1e-10
    want = G.f(case["value"])
    assert abs(val.item() - want) <= tol * max(1.0, abs(want))
    gd = dom.grad.double().cpu().numpy().ravel()
    # fp32 domains: the reference's node arithmetic is fp32
    gtol = 2e-6 if case["dtype"] == "float32" else 1e-10
    assert np.allclose(gd, G.arr(case["grad_domain"]), rtol=gtol, atol=gtol)
    for k, hs in case["grads"].items():
        got = params[k].grad.double().cpu().numpy().ravel()
        assert np.allclose(got, G.arr(hs), rtol=gtol, atol=gtol), k


def test_adjoint_central_differences_c4(cuda):
    """GaussLegendre, dim 4, 32 nodes per dimension, cos(2 pi u + a.x)."""
    a = [1.2, -2.1, 0.7, 2.6]
    u = torch.tensor(0.37, dtype=F64, device=cuda, requires_grad=True)
    dom = torch.tensor([[0.0, 1.0]] * 4, dtype=F64, device=cuda, requires_grad=True)
    gl = tq.GaussLegendre()
    val = gl.integrate(tq.Oscillatory(4, a=a, b=u), 4, N=32**4, integration_domain=dom)
    val.backward()
    h = 1e-6

    def I(uu, dd):
        with torch.no_grad():
            return gl.integrate(tq.Oscillatory(4, a=a, b=uu), 4, N=32**4, integration_domain=dd).item()

    fd_u = (I(0.37 + h, dom.detach()) - I(0.37 - h, dom.detach())) / (2 * h)
    assert abs(u.grad.item() - fd_u) < 1e-7
    for k in range(4):
        for e in range(2):
            dp, dm = dom.detach().clone(), dom.detach().clone()
            dp[k, e] += h
            dm[k, e] -= h
            fd = (I(0.37, dp) - I(0.37, dm)) / (2 * h)
            assert abs(dom.grad[k, e].item() - fd) < 1e-7
    # analytic: Re[e^{i 2 pi u} prod (e^{i a_k} - 1) / (i a_k)]
    z = complex(math.cos(2 * math.pi * 0.37), math.sin(2 * math.pi * 0.37))
    for ak in a:
        z *= (complex(math.cos(ak), math.sin(ak)) - 1.0) / complex(0.0, ak)
    assert abs(val.item() - z.real) < 1e-12


def _v(x):
    return 2 * torch.abs(x)


def _poly(x):
    return 1.0 + 2.0 * x[:, 0] + 3.0 * x[:, 1] ** 2


@pytest.fixture
def float64_default():
    # gradient_test.py runs under set_up_backend("torch", "float64")
    old = torch.get_default_dtype()
    torch.set_default_dtype(torch.float64)
    yield
    torch.set_default_dtype(old)


@pytest.mark.parametrize("name,N1,N2", [("Trapezoid", 149, 549), ("Simpson", 149, 121), ("Boole", 149, 81),
                                        ("MonteCarlo", 99997, 99997), ("VEGAS", 99997, 99997)])
def test_reference_gradient_cases(name, N1, N2, cuda, float64_default):
    integ = getattr(tq, name)()
    seed = {"seed": 0} if name in ("MonteCarlo", "VEGAS") else {}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        # V-shaped function over the domain: gradient [-2, 2]
        dom = torch.tensor([[-1.0, 1.0]], dtype=F64, device=cuda, requires_grad=True)
        r = integ.integrate(_v, 1, N=N1, integration_domain=dom, **seed)
        r.backward()
        assert abs(r.item() - 2.0) < 1e-2
        assert np.all(np.abs(dom.grad.cpu().numpy() - np.array([-2.0, 2.0])) < 2e-2)
        # 2-D polynomial over the domain: [[-10, 14], [-2, 14]]
        dom = torch.tensor([[0.0, 1.0], [0.0, 2.0]], dtype=F64, device=cuda, requires_grad=True)
        r = integ.integrate(_poly, 2, N=N2, integration_domain=dom, **seed)
        r.backward()
        assert abs(r.item() - 12.0) < 8e-2
        assert np.all(np.abs(dom.grad.cpu().numpy() - np.array([[-10.0, 14.0], [-2.0, 14.0]])) < 0.1)
        # over polynomial coefficients: [2, 1, 8/3]
        p = torch.tensor([1.0, 2.0, 3.0], dtype=F64, device=cuda, requires_grad=True)
        r = integ.integrate(lambda x: p[0] + p[1] * x[:, 0] + p[2] * x[:, 1] ** 2, 2, N=N2,
                            integration_domain=[[0.0, 1.0], [0.0, 2.0]], backend="torch", **seed)
        r.backward()
        assert abs(r.item() - 12.0) < 8e-2
        assert np.all(np.abs(p.grad.cpu().numpy() - np.array([2.0, 1.0, 8.0 / 3.0])) < 5e-2)
        # V-shaped function over an offset: 4
        c = torch.tensor(2.0, dtype=F64, device=cuda, requires_grad=True)
        r = integ.integrate(lambda x: 2 * torch.abs(x + c), 1, N=N1, integration_domain=[[-5.0, 3.0]],
                            backend="torch", **seed)
        r.backward()
        assert abs(r.item() - 34.0) < 0.2
        assert abs(c.grad.item() - 4.0) < 0.15


@pytest.mark.parametrize("case", ["exp_steep_outer", "exp_steep_last", "gauss_narrow_outer", "gauss_narrow_last"])
def test_adjoint_outside_the_double_float_range(case, cuda):
    """Row factors or table entries beyond [2^-30, 2^30] (exp(60 x) up to
    1e26, Gaussian tails below 1e-40): those rows leave the adjoint's
    double-float node loop for its fp64 one.  Value and gradients against
    the numpy restatement of the discrete rule's gradient (oracle/grad.py)."""
    from oracle import grad as OGR

    dim, n = 2, 32
    if case.startswith("exp"):
        a = [60.0, 0.5] if case == "exp_steep_outer" else [0.5, 60.0]
        a_t = torch.tensor(a, dtype=F64, device=cuda, requires_grad=True)
        f = tq.ExpSum(dim, a=a_t, b=0.1)
    else:
        a = [400.0, 1.0] if case == "gauss_narrow_outer" else [1.0, 400.0]
        a_t = torch.tensor(a, dtype=F64, device=cuda, requires_grad=True)
        f = tq.GaussianPeak(dim, a=a_t, u=[0.5, 0.3])
    dom_l = [[0.0, 1.0], [-0.5, 1.0]]
    dom = torch.tensor(dom_l, dtype=F64, device=cuda, requires_grad=True)
    val = tq.GaussLegendre().integrate(f, dim, N=n**dim, integration_domain=dom)
    assert "FusedGridFn" in type(val.grad_fn).__name__
    val.backward()
    I, gdom, gpar = OGR.value_and_grad(f.family, f.params_numpy(), OGR.GAUSS, dim, n, dom_l)
    assert abs(val.item() - I) <= 1e-11 * abs(I)
    gd = dom.grad.cpu().numpy()
    assert np.allclose(gd, gdom, rtol=1e-10, atol=1e-10 * np.abs(gdom).max())
    ga = a_t.grad.cpu().numpy()
    want_a = gpar[2:2 + dim]
    assert np.allclose(ga, want_a, rtol=1e-10, atol=1e-10 * np.abs(want_a).max())
