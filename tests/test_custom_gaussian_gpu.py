"""Custom Gaussian rules and batched domains (the reference's extension
points, gaussian.py:6-20,71-129 and its tutorial's custom integrators):
a subclass with its own roots (_root_fn) and composite rule, a subclass
with only its own roots (fused kernels read its root table), a user
subclass that batches 1-D domains through _resize_roots, and the native
batched-domain launch."""
import math

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300 import batch as B

pytestmark = pytest.mark.gpu


class GaussHermite(tq.Gaussian):
    """Gauss-Hermite: integrals of exp(-x^2) f(x) over the real line
    (scipy's roots_hermite as the root function, plain sums per
    dimension)."""

    def __init__(self):
        super().__init__()
        self.name = "Gauss-Hermite"
        scipy_special = pytest.importorskip("scipy.special")
        self._root_fn = scipy_special.roots_hermite

    @staticmethod
    def _apply_composite_rule(cur_dim_areas, dim, hs, domain):
        for _ in range(dim):
            cur_dim_areas = torch.sum(cur_dim_areas, dim=len(cur_dim_areas.shape) - 1)
        return cur_dim_areas


def test_gauss_hermite_custom_rule(cuda):
    gh = GaussHermite()
    v = gh.integrate(lambda x: 1 - x[:, 0], dim=1, N=200)
    assert abs(v.item() - math.sqrt(math.pi)) < 1e-12  # the reference tutorial's example
    v2 = gh.integrate(lambda x: (x**2).sum(1), dim=2, N=20**2)
    assert abs(v2.item() - math.pi) < 1e-12  # int exp(-x^2-y^2)(x^2+y^2) = pi
    assert gh._nr_of_fevals == 400


class ShiftedLegendre(tq.Gaussian):
    """Only the roots change (Legendre roots from a user function, cached
    under extra root arguments): the fused kernels read this rule's table."""

    def __init__(self):
        super().__init__()
        self._root_fn = lambda n, tag: np.polynomial.legendre.leggauss(n)
        self._root_args = ("user",)


def test_custom_root_function_runs_fused(cuda):
    f = tq.GaussianPeak(3, a=[1.0, 2.0, 0.5], u=[0.1, -0.2, 0.3])
    dom = torch.tensor([[-1.0, 1.0]] * 3, dtype=torch.float64, device=cuda)
    s = ShiftedLegendre()
    assert not s._is_custom()
    got = s.integrate(f, 3, N=12**3, integration_domain=dom)
    assert (12, "user") in s._cache
    want = tq.GaussLegendre().integrate(f, 3, N=12**3, integration_domain=dom)
    mat = s.integrate(lambda x: f(x), 3, N=12**3, integration_domain=dom)
    assert abs(got.item() - want.item()) <= 1e-13 * abs(want.item())
    assert abs(mat.item() - want.item()) <= 1e-13 * abs(want.item())


class Batch1D(tq.Gaussian):
    """A user's batched-domain 1-D Gauss-Legendre: [batch, 2] domains go
    through _resize_roots, one integrand call for all of them."""

    def _resize_roots(self, integration_domain, roots):
        a = integration_domain[:, 0:1]
        b = integration_domain[:, 1:2]
        return ((b - a) / 2) * roots.to(integration_domain.device).unsqueeze(0) + (a + b) / 2

    def integrate(self, fn, dim, N, integration_domain=None, backend="torch"):
        assert dim == 1
        n = self._adjust_N(dim=1, N=N)
        roots = self._roots(n, backend, integration_domain.requires_grad)
        w = self._weights(n, 1, backend)
        pts = self._resize_roots(integration_domain, roots)
        vals = fn(pts.reshape(-1, 1)).reshape(pts.shape[0], n)
        return (integration_domain[:, 1] - integration_domain[:, 0]) / 2 * (vals * w.unsqueeze(0)).sum(1)


def test_user_batched_domain_integrator(cuda):
    upper = torch.linspace(0.1, 5.0, 500, dtype=torch.float64, device=cuda)
    doms = torch.stack([torch.zeros_like(upper), upper], dim=1)
    res = Batch1D().integrate(lambda x: x[:, 0] ** 2, dim=1, N=50, integration_domain=doms)
    assert res.shape == (500,)
    assert torch.allclose(res, upper**3 / 3, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("dim", [1, 2])
def test_native_batched_domains(dim, cuda):
    """integrate_domains: one integrand over many domains in one launch,
    equal to the per-call Gauss-Legendre of each domain, differentiable in
    the domain bounds."""
    rng = np.random.default_rng(9)
    m = 300
    f = tq.GaussianPeak(dim, a=[1.5] * dim, u=[0.2] * dim)
    lo = rng.uniform(-1.0, 0.0, (m, dim))
    doms = torch.tensor(np.stack([lo, lo + rng.uniform(0.5, 2.0, (m, dim))], axis=2), dtype=torch.float64,
                        requires_grad=True)
    N = 40**dim
    vals = B.integrate_domains(f, "gausslegendre", N, doms)
    assert vals.shape == (m,)
    vals.sum().backward()
    for i in range(0, m, 37):
        di = doms[i].detach().to(cuda).requires_grad_(True)
        ref = tq.GaussLegendre().integrate(f, dim, N=N, integration_domain=di)
        ref.backward()
        assert abs(vals[i].item() - ref.item()) <= 1e-12 * max(1.0, abs(ref.item()))
        assert torch.allclose(doms.grad[i], di.grad.cpu(), rtol=1e-10, atol=1e-12)
        assert abs(vals[i].item() - f.exact(doms[i].detach())) <= 1e-9
