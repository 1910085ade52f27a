"""Batched grid rules: every integral of a batch equals its per-call value
(and the reference's golden value), whatever launch shape the tuner picks."""
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300 import batch as B
from tests import golden as G

pytestmark = pytest.mark.gpu

FAMS = {"ExpSum": tq.ExpSum, "GaussianPeak": tq.GaussianPeak, "Oscillatory": tq.Oscillatory, "SumSin": tq.SumSin}


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_of_reference_cases(dtype, cuda):
    cases = [c for c in G.load("grid_mc_golden.json")["grid"] if c["dtype"] == dtype]
    by_fam = {}
    for c in cases:
        by_fam.setdefault(c["family"]["kind"], []).append(c)
    dt = getattr(torch, dtype)
    for kind, cs in by_fam.items():
        fs = [FAMS[kind](c["dim"], **{k: v for k, v in c["family"].items() if k != "kind"}) for c in cs]
        vals = B.BatchedGrid(dtype=dt, autotune=False).integrate(
            fs, [c["rule"] for c in cs], [c["N"] for c in cs], [c["domain"] for c in cs]).cpu()
        for v, c in zip(vals.tolist(), cs):
            want = G.f(c["value"])
            # fp32 batches evaluate Gauss-Legendre in fp32 too
            tol = 1e-12 if dtype == "float64" else 2e-6
            assert abs(v - want) <= tol * max(1.0, abs(want)), (c["name"], v, want)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_equals_per_call(dtype, cuda):
    from bench import c3_workload

    specs, exact = c3_workload(n=200, seed=5)
    fs = [tq.GaussianPeak(d, a=a.tolist(), u=u.tolist()) for (_, d, _, _, a, u) in specs]
    bg = B.BatchedGrid(dtype=dtype, autotune=True)
    vals = bg.integrate(fs, [s[0] for s in specs], [s[2] for s in specs], [s[3] for s in specs]).cpu()
    assert bg.last_shape is not None
    cls = {"trapezoid": tq.Trapezoid, "simpson": tq.Simpson, "boole": tq.Boole, "gausslegendre": tq.GaussLegendre}
    for i, (rule, d, N, dom, a, u) in enumerate(specs[:60]):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ref = cls[rule]().integrate(fs[i], d, N=N, integration_domain=torch.tensor(dom, dtype=dtype, device=cuda)).item()
        tol = 1e-12 if dtype == torch.float64 else 2e-6
        assert abs(vals[i].item() - ref) <= tol * max(1.0, abs(ref)), (i, rule, vals[i].item(), ref)
    # every launch shape gives the same values
    plan = bg.plan(fs, [s[0] for s in specs], [s[2] for s in specs], [s[3] for s in specs])
    for shape in [(128, 4, 8192, 0), (256, 16, 131072, 0)]:
        other = bg.run(bg.retile(plan, shape[2]), shape).cpu()
        tol = 1e-12 if dtype == torch.float64 else 2e-6
        assert torch.allclose(other.double(), vals.double(), rtol=tol, atol=1e-12)


def test_batch_validation(cuda):
    with pytest.raises(ValueError):
        B.BatchedGrid().integrate([tq.ExpSum(1), tq.GaussianPeak(1)], ["simpson"] * 2, [101, 101], [[[0, 1]]] * 2)
    with pytest.raises(ValueError):
        B.BatchedGrid().integrate([tq.ExpSum(1)], ["simpson"], [101], [[[1, 0]]])
