"""The materialised path's weighted sum of fp64 integrand values
(tq_weighted_sum, rows of at least 32 nodes), which replaces the weight
multiply of base_integrator.py:77-89 and the per-dimension collapse of
grid_integrator.py:57-91.  Products and sums run as double-floats on the
FP32 pipe, values outside the split's range (2^-40 <= |f| < 2^40) as an
fp64 side sum, grids whose node weights leave [2^-40, 2^40] in fp64; each
case is checked against the exact sum (math.fsum of the fp64 products)
within 2^-44 of the sum of |w_i f_i|, the order of an fp64 pairwise sum's
bound."""
import math

import numpy as np
import pytest
import torch

from torchquad_gb300 import _lib as L
from torchquad_gb300.integration import _kernels as K

pytestmark = pytest.mark.gpu

TOL = 2.0**-44


def _unit(rule, n, gl_w):
    if rule == L.TQ_RULE_SIMPSON:
        c = np.where(np.arange(n) % 2 == 1, 4.0, 2.0)
        c[0] = c[-1] = 1.0
        return c
    if rule == L.TQ_RULE_TRAPEZOID:
        c = np.full(n, 2.0)
        c[0] = c[-1] = 1.0
        return c
    return gl_w


def _weights(rule, dim, n, dom, gl_w=None):
    """w_i of every node, last dimension fastest (meshgrid 'ij')."""
    w = np.ones(1)
    for k in range(dim):
        a, b = dom[k]
        if rule == L.TQ_RULE_GAUSS:
            scale = 0.5 * (b - a)
        else:
            scale = (b - a) / (n - 1) / (3.0 if rule == L.TQ_RULE_SIMPSON else 2.0)
        w = np.multiply.outer(w, scale * _unit(rule, n, gl_w)).ravel()
    return w


def _run(rule, dim, n, dom, values, gl_w=None, chunks=1):
    dev = torch.device("cuda")
    d = torch.tensor(dom, dtype=torch.float64, device=dev)
    glt = None if gl_w is None else torch.tensor(gl_w, dtype=torch.float64, device=dev)
    v = torch.tensor(values, dtype=torch.float64, device=dev).reshape(-1, 1)
    acc = torch.zeros(2, dtype=torch.float64, device=dev)
    bounds = np.linspace(0, len(values), chunks + 1).astype(int)
    for s, e in zip(bounds[:-1], bounds[1:]):
        K.weighted_sum_into(acc, rule, dim, n, d, glt, int(s), v[s:e])
    a = acc.cpu().numpy()
    return float(a[0] + a[1])


def _exact(w, v):
    return math.fsum((w * v).tolist()), float(np.abs(w * v).sum())


def _mixed_values(rng, count):
    mag = 10.0 ** rng.uniform(-20, 20, count)
    v = rng.choice([-1.0, 1.0], count) * mag
    v[rng.random(count) < 0.05] = 0.0
    return v


@pytest.mark.parametrize("rule", [L.TQ_RULE_SIMPSON, L.TQ_RULE_TRAPEZOID])
@pytest.mark.parametrize("dim,n", [(2, 301), (3, 65), (4, 33)])
def test_newton_cotes_rows_match_exact_sum(cuda, rule, dim, n):
    rng = np.random.default_rng(dim * 1000 + n)
    dom = [[-1.0 + 0.1 * k, 0.5 + 0.3 * k] for k in range(dim)]
    v = _mixed_values(rng, n**dim)
    want, scale = _exact(_weights(rule, dim, n, dom), v)
    got = _run(rule, dim, n, dom, v)
    assert abs(got - want) <= TOL * scale, (got, want, scale)


def test_gauss_rows_match_exact_sum(cuda):
    dim, n = 3, 48
    x, glw = np.polynomial.legendre.leggauss(n)
    dom = [[0.0, 1.0], [-2.0, 3.0], [0.5, 0.75]]
    rng = np.random.default_rng(7)
    v = np.exp(rng.standard_normal(n**dim)) * rng.choice([-1.0, 1.0], n**dim)
    want, scale = _exact(_weights(L.TQ_RULE_GAUSS, dim, n, dom, glw), v)
    got = _run(L.TQ_RULE_GAUSS, dim, n, dom, v, gl_w=glw)
    assert abs(got - want) <= TOL * scale, (got, want, scale)


def test_cancelling_values(cuda):
    """Terms of both signs that cancel to a small remainder: the error stays
    within the bound relative to the sum of magnitudes."""
    dim, n = 2, 401
    rng = np.random.default_rng(3)
    dom = [[0.0, 1.0], [0.0, 1.0]]
    w = _weights(L.TQ_RULE_SIMPSON, dim, n, dom)
    v = rng.standard_normal(n**dim) * 1e6
    v -= math.fsum((w * v).tolist()) / w.sum()  # sum of w v is now ~0
    want, scale = _exact(w, v)
    got = _run(L.TQ_RULE_SIMPSON, dim, n, dom, v)
    assert abs(got - want) <= TOL * scale, (got, want, scale)


@pytest.mark.parametrize("kind", ["tiny", "huge", "subnormal", "mixed"])
def test_values_outside_the_split_take_the_fp64_side_sum(cuda, kind):
    dim, n = 2, 257
    rng = np.random.default_rng(11)
    dom = [[0.0, 2.0], [-1.0, 1.0]]
    w = _weights(L.TQ_RULE_SIMPSON, dim, n, dom)
    base = rng.uniform(0.5, 2.0, n**dim)
    if kind == "tiny":
        v = base * 1e-80
    elif kind == "huge":
        v = base * 1e200
    elif kind == "subnormal":
        v = base * 1e-310
    else:  # a few values of each kind among ordinary ones, and the split's range ends
        v = base.copy()
        idx = rng.choice(n**dim, 36, replace=False)
        v[idx[:10]] *= 1e-80
        v[idx[10:20]] *= 1e-310
        v[idx[20:30]] *= 1e30
        v[idx[30:]] = [2.0**40, 2.0**40 * (1 - 2.0**-52), -(2.0**-40), 2.0**-40 * (1 - 2.0**-52), 1e12, -1e-12]
    want, scale = _exact(w, v)
    got = _run(L.TQ_RULE_SIMPSON, dim, n, dom, v)
    # subnormal products: one subnormal spacing per term on top of the bound
    assert abs(got - want) <= TOL * scale + len(v) * 5e-324, (got, want, scale)


def test_non_finite_values_propagate(cuda):
    dim, n = 2, 65
    dom = [[0.0, 1.0], [0.0, 1.0]]
    v = np.ones(n**dim)
    v[100] = np.nan
    assert math.isnan(_run(L.TQ_RULE_SIMPSON, dim, n, dom, v))
    v[100] = np.inf
    assert not math.isfinite(_run(L.TQ_RULE_SIMPSON, dim, n, dom, v))


def test_chunks_equal_one_launch(cuda):
    """The grid cut into chunks that split rows (start offsets, as the
    chunked materialised path calls it) gives the same sum to the bound."""
    dim, n = 3, 101
    rng = np.random.default_rng(5)
    dom = [[0.0, 1.0]] * 3
    v = _mixed_values(rng, n**dim)
    want, scale = _exact(_weights(L.TQ_RULE_SIMPSON, dim, n, dom), v)
    for chunks in (1, 3, 7):
        got = _run(L.TQ_RULE_SIMPSON, dim, n, dom, v, chunks=chunks)
        assert abs(got - want) <= TOL * scale, (chunks, got, want, scale)


@pytest.mark.parametrize("width", [1e20, 1e-20])
def test_extreme_node_weights_are_summed_in_fp64(cuda, width):
    """Node weights far outside the float range (domains of width 1e20 and
    1e-20): the kernel sums the grid in fp64."""
    dim, n = 3, 65
    rng = np.random.default_rng(9)
    dom = [[0.0, width]] * dim
    v = _mixed_values(rng, n**dim)
    want, scale = _exact(_weights(L.TQ_RULE_SIMPSON, dim, n, dom), v)
    got = _run(L.TQ_RULE_SIMPSON, dim, n, dom, v)
    assert abs(got - want) <= TOL * scale, (got, want, scale)
