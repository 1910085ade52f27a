"""GPU parity of the counter-based uniforms and Monte Carlo."""
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from oracle import philox as OP
from tests import golden as G

pytestmark = pytest.mark.gpu

FAMS = {"ExpSum": tq.ExpSum, "GaussianPeak": tq.GaussianPeak, "Oscillatory": tq.Oscillatory, "SumSin": tq.SumSin}


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_uniform_bitwise_equal_oracle(dtype, cuda):
    r = tq.RNG(seed=0x1234_5678_9ABC)
    a = r.uniform([1001, 3], dtype)
    b = r.uniform([7], dtype)
    nd = np.float32 if dtype == torch.float32 else np.float64
    s = OP.ReplayStream(0x1234_5678_9ABC)
    assert np.array_equal(a.cpu().numpy(), s.uniform([1001, 3], nd))
    assert np.array_equal(b.cpu().numpy(), s.uniform([7], nd))
    big = tq.RNG(seed=9).uniform([1 << 22], dtype)
    assert float(big.min()) >= 0.0 and float(big.max()) < 1.0
    assert abs(float(big.double().mean()) - 0.5) < 1e-3


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "materialised"])
@pytest.mark.parametrize("case", G.load("grid_mc_golden.json")["mc"], ids=lambda c: f"{c['dim']}-{c['dtype']}")
def test_mc_matches_reference_on_same_draws(case, fused, cuda):
    kw = {k: v for k, v in case["family"].items() if k != "kind"}
    f = FAMS[case["family"]["kind"]](case["dim"], **kw)
    fn = f if fused else (lambda x: f(x))
    dom = torch.tensor(case["domain"], dtype=getattr(torch, case["dtype"]), device=cuda)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v = tq.MonteCarlo().integrate(fn, case["dim"], N=case["N"], integration_domain=dom, seed=case["seed"])
    want = G.f(case["value"])
    tol = 2e-6 if case["dtype"] == "float32" else 1e-12
    assert v.dtype == dom.dtype
    assert abs(v.item() - want) <= tol * max(1.0, abs(want)), (v.item(), want)


def test_mc_seed_and_rng_exclusive(cuda):
    with pytest.raises(ValueError, match="seed and rng"):
        tq.MonteCarlo().integrate(lambda x: x[:, 0], 1, N=10, integration_domain=[[0, 1]], seed=1,
                                  rng=tq.RNG(seed=2))


def test_mc_constant_exact(cuda):
    v = tq.MonteCarlo().integrate(lambda x: torch.full_like(x[:, 0], 2.0), 2, N=1000,
                                  integration_domain=[[0.0, 3.0], [0.0, 1.0]], seed=0)
    assert abs(v.item() - 6.0) < 1e-6
