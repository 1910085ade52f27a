"""The numpy VEGAS oracle against the reference: the golden vectors of the
reference's own unit tests and states recorded from the reference
(step-wise, on the same Philox draws).  CPU only."""
import math

import numpy as np
import pytest

from oracle import integrands as OI
from oracle import philox as OP
from oracle import vegas as OV
from tests import golden as G

VG = G.load("vegas_golden.json")


def test_interval_ids_and_offsets_reference_golden():
    # vegas_map_test.py:28-48
    for dt in (np.float32, np.float64):
        m = OV.Map(20, 3, dt)
        y = np.array([[0.8121, 0.4319, 0.1612], [0.4746, 0.6501, 0.9241], [0.6143, 0.0724, 0.5818]], dtype=dt)
        assert np.array_equal(m.interval_id(y), [[16, 8, 3], [9, 13, 18], [12, 1, 11]])
        off = np.array([[0.2420, 0.6380, 0.2240], [0.4920, 0.0020, 0.4820], [0.2860, 0.4480, 0.6360]], dtype=dt)
        assert np.max(np.abs(m.interval_offset(y) - off)) <= 6e-5
        assert np.max(np.abs(m.get_X(y) - y)) <= 3e-7


def test_smooth_map_reference_golden():
    # vegas_map_test.py:84-100
    for dt in (np.float32, np.float64):
        w = np.array([[0.0, 0.0, 0.0, 1.0, 1.0, 1.0], [0.0, 0.0, 0.0, 1.0, 0.0, 0.0]], dtype=dt)
        want = np.array([[0.0, 0.0, 0.54913316, 0.75820765, 0.77899047, 0.77899047],
                         [-0.0, -0.0, 0.64868024, 0.93220967, 0.64868024, -0.0]])
        got = OV.Map.smooth_map(w, np.ones(w.shape, dtype=np.int64), 0.5)
        assert np.max(np.abs(got - want)) <= 3e-7


def test_map_update_invariants_reference():
    # vegas_map_test.py:54-128
    for dt in (np.float32, np.float64):
        m = OV.Map(20, 3, dt)
        g = np.linspace(0.0, 0.99999, 100, dtype=dt)
        y = np.stack([a.ravel() for a in np.meshgrid(g, g, g, indexing="ij")], axis=1).astype(dt)
        f = np.prod(np.exp(y), axis=1).astype(dt)
        jac = m.get_Jac(y)
        assert np.max(np.abs(jac - 1.0)) < 1e-14
        m.accumulate_weight(y, (f * jac) ** 2)
        assert np.min(m.weights[:, 1:] - m.weights[:, :-1]) > 0
        assert np.max(np.abs(m.counts - 50000)) == 0
        m.update_map()
        assert np.array_equal(m.x_edges[:, [0, -1]], np.array([[0.0, 1.0]] * 3, dtype=dt))
        assert np.max(np.abs(m.dx_edges.sum(axis=1) - 1.0)) < 3e-7
        assert np.min(m.dx_edges) > 0 and np.max(m.dx_edges[:, 1:] - m.dx_edges[:, :-1]) < 0
        assert np.max(np.abs(m.get_X(y)[0])) == 0.0


def _load(p, dt):
    return G.arr(p["values"]).reshape(p["shape"]).astype(dt)


@pytest.mark.parametrize("case", VG["steps"], ids=lambda c: c["dtype"])
def test_oracle_steps_match_reference(case):
    dt = np.float32 if case["dtype"] == "float32" else np.float64
    params = G.arr(case["params"])
    dom = np.array(case["domain"], dtype=dt)
    sizes = (dom[:, 1] - dom[:, 0]).astype(dt)
    vol = dt(np.prod(sizes))
    fn = lambda x: (OI.evaluate(2, params, ((x * sizes).astype(dt) + dom[:, 0]).astype(dt)) * vol).astype(dt)  # noqa
    for st in case["steps"]:
        m = OV.Map(case["n_bins"], 3, dt)
        m.x_edges = _load(st["x_edges"], dt)
        m.dx_edges = _load(st["dx_edges"], dt)
        s = OV.Strat(case["N"] // 25, 3, dt)
        s.dh = _load(st["dh"], dt)
        neval = s.get_NH(st["starting_N"])
        assert neval.tolist() == st["neval"]  # bit-exact
        M = int(neval.sum())
        u = OP.ReplayStream(case["seed"], 0, st["rng_offset"]).uniform([M, 3], dt)
        y = s.get_Y(neval, u)
        jf = (fn(m.get_X(y)) * m.get_Jac(y)).astype(dt)
        m.accumulate_weight(y, (jf * jf).astype(dt))
        assert m.counts.ravel().tolist() == st["counts"]  # bit-exact
        rtol = 2e-5 if dt == np.float32 else 1e-11
        assert np.allclose(m.weights, _load(st["weights"], dt), rtol=rtol, atol=0)
        JF, JF2 = s.accumulate_weight(neval, jf)
        assert np.allclose(JF, _load(st["JF"], dt), rtol=rtol, atol=1e-30)
        assert np.allclose(JF2, _load(st["JF2"], dt), rtol=rtol, atol=1e-30)
        m.update_map()
        s.update_DH()
        assert np.allclose(m.x_edges, _load(st["x_edges_new"], dt), rtol=0, atol=5e-6 if dt == np.float32 else 1e-12)
        # dh ~ (V^2 JF2/n - (V JF/n)^2)^0.75 cancels catastrophically in fp32 for
        # cubes of small variance: compare against the largest dh
        want = _load(st["dh_new"], dt)
        tol = 2e-3 if dt == np.float32 else 1e-9
        assert np.max(np.abs(s.dh - want)) <= tol * np.max(want)


C2 = G.load_npz("vegas_c2_steps.npz")


@pytest.mark.parametrize("it", [int(i) for i in C2["steps"]])
def test_oracle_c2_steps_match_reference(it):
    """The plain VEGAS configuration at full size (dim 6, 50 intervals, 6^6
    cubes, fp32, seed 0): the oracle given the reference's state before
    iteration `it` reproduces its evaluations per cube and interval counts
    bit for bit, its sums to fp32 rounding, and the next iteration's
    evaluations per cube exactly."""
    dt, p = np.float32, f"it{it}_"
    fn = lambda x: OI.evaluate(2, C2["params"], x).astype(dt)  # noqa: E731
    m = OV.Map(50, 6, dt)
    m.x_edges, m.dx_edges = C2[p + "x_edges"].copy(), C2[p + "dx_edges"].copy()
    s = OV.Strat(400000, 6, dt)
    s.dh = C2[p + "dh"].copy()
    neval = s.get_NH(int(C2[p + "starting_N"]))
    assert np.array_equal(neval, C2[p + "neval"].astype(np.int64))  # bit-exact
    M = int(neval.sum())
    u = OP.ReplayStream(0, 0, int(C2[p + "rng_offset"])).uniform([M, 6], dt)
    y = s.get_Y(neval, u)
    jf = (fn(m.get_X(y)) * m.get_Jac(y)).astype(dt)
    m.accumulate_weight(y, (jf * jf).astype(dt))
    assert np.array_equal(m.counts, C2[p + "counts"])  # bit-exact
    assert np.allclose(m.weights, C2[p + "weights"], rtol=2e-6, atol=0)
    JF, JF2 = s.accumulate_weight(neval, jf)
    assert np.allclose(JF, C2[p + "JF"], rtol=2e-6, atol=1e-35)
    assert np.allclose(JF2, C2[p + "JF2"], rtol=2e-6, atol=1e-35)
    m.update_map()
    s.update_DH()
    assert np.max(np.abs(m.x_edges - C2[p + "x_edges_new"])) <= 1e-6
    want = C2[p + "dh_new"]
    assert np.max(np.abs(s.dh - want)) <= 5e-5 * np.max(want)
    n = int(C2[p + "next_starting_N"])  # get_NH of the next iteration (vegas_stratification.py:92-103)
    nh = np.clip(np.floor((s.dh * dt(n)).astype(dt)), 2, None)
    assert np.array_equal(nh, np.clip(np.floor((want * dt(n)).astype(dt)), 2, None))


def test_oracle_c2_end_to_end_statistically():
    c = VG["c2"]
    params = G.arr(c["params"])
    v = OV.Vegas()
    got = v.integrate(lambda x: OI.evaluate(2, params, x), 6, c["N"], [[0.0, 1.0]] * 6,
                      OP.ReplayStream(c["seed"]), dt=np.float32, n_intervals=50)
    want = G.f(c["value"])
    assert v.it == c["iterations"]
    assert abs(v.fevals - c["fevals"]) <= 2000
    assert abs(got - want) <= 5 * v.get_error() + 1e-6
    assert abs(got - 1.0) < 5e-3


def _abort_vegas(c):
    v = OV.Vegas()
    v.dt = np.float32 if c["dtype"] == "float32" else np.float64
    v.it, v.results, v.sigma2 = c["it"], G.arr(c["r"]).tolist(), G.arr(c["s"]).tolist()
    v.eps_rel, v.eps_abs = c["eps_rel"], c["eps_abs"]
    v.starting_N, v.N_increment, v.N, v.max_iterations = c["sN"], c["inc"], c["N"], c["max_it"]
    v.fevals = c["fevals"]
    return v


def test_oracle_abort_test_matches_reference():
    """_check_abort_conditions (vegas.py:161-209) on blocks of five results
    held as fp32 and fp64 tensors in the reference: same decision, same
    adapted _starting_N, same exception from int()."""
    for c in VG["abort"]:
        v = _abort_vegas(c)
        if c["error"]:
            with pytest.raises({"OverflowError": OverflowError, "ValueError": ValueError}[c["error"]]):
                v.check_abort()
            continue
        assert v.check_abort() == c["stop"], c
        assert v.starting_N == c["starting_N"], c
