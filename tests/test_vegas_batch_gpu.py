"""Batched VEGAS (tq_vegas_batch_*, torchquad_gb300.vegas_batch) against the
per-call API: each integral of a batch equals its own VEGAS().integrate
with the same seed (reference vegas.py:100-160 runs one per call)."""
import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300.vegas_batch import VegasBatch

pytestmark = pytest.mark.gpu


def _mixed(rng, n, max_n=200_000):
    """Integrands of every family, dims 1..8, N log-uniform 1e4..max_n."""
    fns, Ns, doms = [], [], []
    for i in range(n):
        dim = int(rng.integers(1, 9))
        fam = i % 4
        if fam == 0:
            f = tq.GaussianPeak.normal(dim, float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.1, 0.3)))
        elif fam == 1:
            f = tq.Oscillatory(dim, a=float(rng.uniform(0.5, 2.0)), b=float(rng.uniform(0, 1)))
        elif fam == 2:
            f = tq.ExpSum(dim, a=float(rng.uniform(-1, 1)), b=0.1)
        else:
            f = tq.SumSin(dim, a=float(rng.uniform(1, 3)))
        fns.append(f)
        Ns.append(int(np.exp(rng.uniform(np.log(1e4), np.log(max_n)))))
        doms.append([[0.0, float(rng.uniform(0.5, 2.0))]] * dim)
    return fns, Ns, doms


def _per_call(fns, Ns, doms, seeds, dtype, **kw):
    out = []
    for f, N, d, s in zip(fns, Ns, doms, seeds):
        v = tq.VEGAS()
        r = v.integrate(f, f.dim, N=N, integration_domain=torch.tensor(d, dtype=dtype, device="cuda"), seed=s,
                        **kw)
        out.append((float(r), v.it, v._nr_of_fevals, v._starting_N))
    return out


def _close(a, b, rtol):
    return abs(a - b) <= rtol * max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("graph_call", [False, True])
def test_batch_matches_per_call_fp64(cuda, graph_call):
    """Every integral of a mixed batch (four families, dims 1..8, N up to
    2e5) equals the per-call result to 1e-9 with the same iterations,
    evaluations and adapted _starting_N; the first call runs the phases
    eagerly, later calls replay the captured graph."""
    rng = np.random.default_rng(7)
    fns, Ns, doms = _mixed(rng, 24)
    seeds = [1000 + i for i in range(len(fns))]
    ref = _per_call(fns, Ns, doms, seeds, torch.float64)
    vb = VegasBatch(fns, Ns, dtype=torch.float64)
    res = vb.integrate(domains=doms, seeds=seeds)
    if graph_call:
        res = vb.integrate(domains=doms, seeds=seeds)
        assert vb.graph is not None
    res = res.cpu().numpy()
    for i, (r, it, ev, sN) in enumerate(ref):
        assert _close(res[i], r, 1e-9), (i, res[i], r)
        assert vb.it[i] == it and vb.nr_of_fevals[i] == ev and vb.starting_N_out[i] == sN, i


def test_batch_stops_each_integral_on_its_own(cuda):
    """An integral that reaches its accuracy early stops there while the
    others go on; each matches its per-call run (iterations and result)."""
    fns = [tq.ExpSum(2, a=0.5), tq.GaussianPeak.normal(4, 0.5, 0.15), tq.Oscillatory(3, a=1.0, b=0.2)]
    Ns = [50_000, 120_000, 80_000]
    doms = [[[0.0, 1.0]] * f.dim for f in fns]
    seeds = [11, 12, 13]
    eps = [1e-1, 0.0, 0.0]
    ref = []
    for f, N, d, s, e in zip(fns, Ns, doms, seeds, eps):
        v = tq.VEGAS()
        r = v.integrate(f, f.dim, N=N, integration_domain=torch.tensor(d, dtype=torch.float64, device="cuda"),
                        seed=s, eps_rel=e)
        ref.append((float(r), v.it))
    assert ref[0][1] < ref[1][1]  # the first stops earlier than the second
    vb = VegasBatch(fns, Ns, dtype=torch.float64)
    for _ in range(2):  # eager, then the graph
        res = vb.integrate(domains=doms, seeds=seeds, eps_rel=eps).cpu().numpy()
        for i, (r, it) in enumerate(ref):
            assert vb.it[i] == it
            assert _close(res[i], r, 1e-9)


def test_batch_fp32_matches_per_call(cuda):
    """fp32 batch: the per-cube and histogram sums are fp64 atomics whose
    order depends on the CTA split, and the fp32 state rounds them, so each
    result equals the per-call result to 1e-5 with the same iterations."""
    rng = np.random.default_rng(3)
    fns, Ns, doms = _mixed(rng, 16, max_n=100_000)
    seeds = list(range(16))
    ref = _per_call(fns, Ns, doms, seeds, torch.float32)
    vb = VegasBatch(fns, Ns, dtype=torch.float32)
    res = vb.integrate(domains=doms, seeds=seeds).cpu().numpy()
    assert res.dtype == np.float32
    for i, (r, it, _, _) in enumerate(ref):
        assert abs(float(res[i]) - r) <= 1e-5 * max(abs(r), 1e-2), (i, res[i], r)
        assert vb.it[i] == it, i


def test_batch_rejects_large_maps(cuda):
    with pytest.raises(ValueError):
        VegasBatch([tq.ExpSum(2)], [2_000_000])


@pytest.mark.parametrize("opts", [dict(use_grid_improve=False), dict(use_warmup=False),
                                  dict(max_iterations=12)])
def test_batch_options_match_per_call(cuda, opts):
    """The reference's VEGAS options (vegas.py:30-44) through the batch:
    each integral equals its per-call run with the same options."""
    fns = [tq.GaussianPeak(3, a=[5.0, 8.0, 3.0], u=[0.3, 0.5, 0.7]), tq.Oscillatory(2, a=[1.0, -2.0], b=0.1),
           tq.ExpSum(5, a=0.3, b=-0.2), tq.SumSin(1, a=2.0)]
    Ns = [40_000, 25_000, 60_000, 12_000]
    doms = [[[0.0, 1.0], [-1.0, 1.0], [0.0, 2.0]], [[0.0, 1.0]] * 2, [[0.0, 0.5]] * 5, [[-1.0, 3.0]]]
    seeds = [21, 22, 23, 24]
    ref = _per_call(fns, Ns, doms, seeds, torch.float64, **opts)
    vb = VegasBatch(fns, Ns, dtype=torch.float64, **opts)
    res = vb.integrate(domains=doms, seeds=seeds).cpu().numpy()
    for i, (r, it, ev, sN) in enumerate(ref):
        assert _close(res[i], r, 1e-9), (i, res[i], r)
        assert vb.it[i] == it and vb.nr_of_fevals[i] == ev and vb.starting_N_out[i] == sN, i


def test_batch_edge_states(cuda):
    """Edge states in one batch: a zero integrand (every map update finds an
    all-zero row of weights and only resets, vegas_map.py:187-196), a tiny
    budget whose warm-up draws no points (_starting_N // 5 = 0), the largest
    dimension (16) and the largest map (1024 intervals); each equals its
    per-call run, the zero integrand exactly 0."""
    fns = [tq.ExpSum(2, c=0.0), tq.GaussianPeak.normal(2, 0.5, 0.2), tq.Oscillatory(16, a=0.2, b=0.3),
           tq.GaussianPeak.normal(3, 0.4, 0.2)]
    Ns = [20_000, 120, 30_000, 256_000]
    doms = [[[0.0, 1.0]] * f.dim for f in fns]
    seeds = [5, 6, 7, 8]
    ref = _per_call(fns, Ns, doms, seeds, torch.float64)
    vb = VegasBatch(fns, Ns, dtype=torch.float64)
    assert vb.warm_samples[1] == 0 and vb.states[3].n_bins == 1024
    res = vb.integrate(domains=doms, seeds=seeds).cpu().numpy()
    assert res[0] == 0.0
    for i, (r, it, ev, _) in enumerate(ref):
        assert _close(res[i], r, 1e-9), (i, res[i], r)
        assert vb.it[i] == it and vb.nr_of_fevals[i] == ev, i


def test_batch_rng_offsets_advance_like_per_call(cuda):
    """RNG objects passed to the batch advance as VEGAS().integrate advances
    them, so a second call continues each stream; results match two
    consecutive per-call runs on the same RNG objects."""
    from torchquad_gb300.integration.rng import RNG

    fns = [tq.GaussianPeak.normal(2, 0.5, 0.2), tq.ExpSum(3, a=0.5)]
    Ns = [30_000, 50_000]
    doms = [[[0.0, 1.0]] * f.dim for f in fns]
    ra, rb = [RNG(seed=1), RNG(seed=2)], [RNG(seed=1), RNG(seed=2)]
    want = []
    for _ in range(2):
        for f, N, d, r in zip(fns, Ns, doms, ra):
            v = tq.VEGAS()
            want.append(float(v.integrate(f, f.dim, N=N, integration_domain=torch.tensor(d, dtype=torch.float64,
                                                                                          device="cuda"), rng=r)))
    vb = VegasBatch(fns, Ns, dtype=torch.float64)
    got = list(vb.integrate(domains=doms, rngs=rb).cpu().numpy()) + list(vb.integrate(domains=doms, rngs=rb).cpu().numpy())
    assert [r.offset for r in ra] == [r.offset for r in rb]
    for g, w in zip(got, want):
        assert _close(g, w, 1e-9)
