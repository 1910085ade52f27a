"""The compiled integrate functions (grid_integrator.py:133-255,
monte_carlo.py:108-225) as the reference's JIT tests use them
(simpson_test.py:90-138, monte_carlo_test.py:78-130): N and dim fixed once,
the returned function reused for several integrands, including complex and
[2, 2, 2]-shaped ones."""
import math
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq

pytestmark = pytest.mark.gpu


def _integrands(dev):
    dom = torch.tensor([[0.0, 2.0]], dtype=torch.float64, device=dev)
    shape_scale = (torch.arange(8, dtype=torch.float64, device=dev) + 1.0).reshape(2, 2, 2)
    return dom, [
        ("exp", lambda x: torch.exp(x[:, 0]), math.exp(2.0) - 1.0),
        ("poly", lambda x: x[:, 0] ** 3 - 2.0 * x[:, 0], 0.0),
        ("complex", lambda x: torch.exp(1j * x[:, 0]), complex(math.sin(2.0), 1.0 - math.cos(2.0))),
        ("shaped", lambda x: torch.exp(x[:, 0])[:, None, None, None] * shape_scale[None],
         (math.exp(2.0) - 1.0) * shape_scale.cpu().numpy()),
    ]


@pytest.mark.parametrize("rule,N,tol", [("Trapezoid", 100001, 2e-9), ("Simpson", 100001, 3e-11),
                                         ("Boole", 100001, 3e-11), ("GaussLegendre", 64, 1e-13)])
def test_compiled_grid_rule_matches_integrate(rule, N, tol, cuda):
    dom, cases = _integrands(cuda)
    integ = getattr(tq, rule)()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        compiled = integ.get_jit_compiled_integrate(dim=1, N=N)
        for name, fn, exact in cases:
            got = compiled(fn, dom)
            plain = getattr(tq, rule)().integrate(fn, 1, N=N, integration_domain=dom)
            assert torch.equal(got, plain), name
            g = got.cpu().numpy()
            assert np.max(np.abs(g - np.asarray(exact))) <= tol * max(1.0, float(np.max(np.abs(exact)))), name


def test_compiled_monte_carlo_draws_fresh_numbers(cuda):
    dom, cases = _integrands(cuda)
    mc = tq.MonteCarlo()
    compiled = mc.get_jit_compiled_integrate(dim=1, N=400000, seed=5)
    fn, exact = cases[0][1], cases[0][2]
    a = compiled(fn, dom).item()
    b = compiled(fn, dom).item()
    assert a != b  # each call continues the stream
    # both within six standard errors of the exact value
    x = torch.linspace(0, 2, 100001, dtype=torch.float64)
    sd = float(2.0 * torch.exp(x).std()) / math.sqrt(400000)
    assert abs(a - exact) < 6 * sd and abs(b - exact) < 6 * sd
    # the first call equals a plain integrate with the same seed
    assert a == tq.MonteCarlo().integrate(fn, 1, N=400000, integration_domain=dom, seed=5).item()
