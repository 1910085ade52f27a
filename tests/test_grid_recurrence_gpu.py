"""fp64 grid rows evaluated by recurrence (rows without a node table: one
dimension, or more nodes per dimension than a table holds) against the
numpy oracle, which evaluates every node directly (the reference's
composite rules, simpson.py:29-46, trapezoid.py:27-37, boole.py:29-48).
Covers every family, every Newton-Cotes rule, and parameters for which the
range guards send segments to direct evaluation."""
import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from oracle import grid as OG
from oracle import integrands as OI

pytestmark = pytest.mark.gpu

RULES = {"trapezoid": (tq.Trapezoid, OG.TRAPEZOID), "simpson": (tq.Simpson, OG.SIMPSON),
         "boole": (tq.Boole, OG.BOOLE)}


def _cases():
    return [
        ("exp", tq.ExpSum(1, a=-1.7, b=0.3, c=2.0), [[-1.0, 2.0]]),
        ("gauss", tq.GaussianPeak(1, a=3.0, u=0.4), [[-1.0, 2.0]]),
        ("osc", tq.Oscillatory(1, a=7.0, b=0.2), [[0.0, 3.0]]),
        ("sumsin", tq.SumSin(1, a=5.0, c=0.7), [[-2.0, 1.0]]),
        # guards: a narrow peak whose exponent leaves [-600, 600] over most
        # rows, and an exponent that grows past 600 along the row
        ("gauss_narrow", tq.GaussianPeak(1, a=2.0e5, u=0.5), [[0.0, 1.0]]),
        ("exp_steep", tq.ExpSum(1, a=900.0, b=-700.0), [[0.0, 1.0]]),
        # negative Gaussian coefficient: convex exponent, direct evaluation
        ("gauss_neg", tq.GaussianPeak(1, a=-0.5, u=0.2), [[0.0, 1.0]]),
    ]


@pytest.mark.parametrize("rule", list(RULES))
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_one_dimensional_rows_match_oracle(cuda, rule, case):
    _, f, dom = case
    cls, rid = RULES[rule]
    N = 40_001  # valid for every rule (4k + 1)
    got = cls().integrate(f, 1, N=N, integration_domain=torch.tensor(dom, dtype=torch.float64, device=cuda))
    want = OG.integrate(lambda x: OI.evaluate(f.family, f.params_numpy(), x), rid, 1, N, np.asarray(dom))
    assert np.isfinite(want)
    assert abs(got.item() - want) <= 1e-12 * max(abs(want), 1e-300) + 1e-300, (got.item(), want)


@pytest.mark.parametrize("fam", ["exp", "gauss", "osc", "sumsin"])
def test_long_rows_without_a_table_match_oracle(cuda, fam):
    """dim 2 with 2501 nodes per dimension (more than a per-CTA table
    holds): the outer sum per row, the row by recurrence."""
    f = {"exp": tq.ExpSum(2, a=[0.5, -1.2], b=0.1), "gauss": tq.GaussianPeak(2, a=[2.0, 4.0], u=[0.3, 0.6]),
         "osc": tq.Oscillatory(2, a=[1.5, -3.0], b=0.4), "sumsin": tq.SumSin(2, a=[2.0, 3.0])}[fam]
    dom = [[0.0, 1.0], [-0.5, 1.5]]
    N = 2501**2
    got = tq.Simpson().integrate(f, 2, N=N, integration_domain=torch.tensor(dom, dtype=torch.float64, device=cuda))
    want = OG.integrate(lambda x: OI.evaluate(f.family, f.params_numpy(), x), OG.SIMPSON, 2, N, np.asarray(dom))
    assert abs(got.item() - want) <= 1e-12 * abs(want), (got.item(), want)


def test_batch_one_dimensional_rows_match_oracle(cuda):
    """The batched form's rows without a table (tq_batch_grid) against the
    oracle, all families and rules in one launch."""
    from torchquad_gb300 import batch as B

    fs, rules, Ns, doms, want = [], [], [], [], []
    for name, f, dom in _cases():
        for rule, (_, rid) in RULES.items():
            fs.append(f)
            rules.append(rule)
            Ns.append(20_001)
            doms.append(dom)
            want.append(OG.integrate(lambda x, f=f: OI.evaluate(f.family, f.params_numpy(), x), rid, 1, 20_001,
                                     np.asarray(dom)))
    got = B.integrate_batch(fs, rules, Ns, doms, dtype=torch.float64).cpu().numpy()
    for g, w in zip(got, want):
        assert abs(g - w) <= 1e-12 * max(abs(w), 1e-300) + 1e-300, (g, w)
