"""GPU parity of VEGAS: the reference unit tests' golden vectors, step-wise
states recorded from the reference on the same Philox draws (bin indices,
counts and evaluations per cube bit-exact), the full-size plain VEGAS
configuration, and the reference's special-case and accuracy tests."""
import math
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300 import _lib as L
from torchquad_gb300.integration._vegas_state import VegasDevice
from tests import golden as G

pytestmark = pytest.mark.gpu

VG = G.load("vegas_golden.json")
DT = {"float32": torch.float32, "float64": torch.float64}


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_map_reference_golden_vectors(dtype, cuda):
    # vegas_map_test.py:19-128
    m = tq.VEGASMap(20, 3, "torch", dtype)
    y = torch.tensor([[0.8121, 0.4319, 0.1612], [0.4746, 0.6501, 0.9241], [0.6143, 0.0724, 0.5818]],
                     dtype=dtype, device=cuda)
    assert m._get_interval_ID(y).cpu().tolist() == [[16, 8, 3], [9, 13, 18], [12, 1, 11]]
    off = torch.tensor([[0.2420, 0.6380, 0.2240], [0.4920, 0.0020, 0.4820], [0.2860, 0.4480, 0.6360]],
                       dtype=dtype, device=cuda)
    assert float((m._get_interval_offset(y) - off).abs().max()) <= 6e-5
    assert float((m.get_X(y) - y).abs().max()) <= 3e-7
    g = torch.linspace(0.0, 0.99999, 100, dtype=dtype, device=cuda)
    yy = torch.stack([a.ravel() for a in torch.meshgrid(g, g, g, indexing="ij")], dim=1)
    f = torch.prod(torch.exp(yy), dim=1)
    jac = m.get_Jac(yy)
    assert jac.shape == (100**3,) and jac.dtype == dtype
    assert float((jac - 1.0).abs().max()) < 1e-14
    m.accumulate_weight(yy, (f * jac) ** 2)
    assert m.weights.shape == (3, 20)
    assert float((m.weights[:, 1:] - m.weights[:, :-1]).min()) > 0.0
    assert m.counts.dtype == torch.int64 and int((m.counts - 50000).abs().max()) == 0
    w = torch.tensor([[0.0, 0.0, 0.0, 1.0, 1.0, 1.0], [0.0, 0.0, 0.0, 1.0, 0.0, 0.0]], dtype=dtype)
    want = torch.tensor([[0.0, 0.0, 0.54913316, 0.75820765, 0.77899047, 0.77899047],
                         [-0.0, -0.0, 0.64868024, 0.93220967, 0.64868024, -0.0]], dtype=dtype)
    sm = tq.VEGASMap._smooth_map(w, torch.ones(w.shape, dtype=torch.int64), 0.5)
    assert float((sm.cpu() - want).abs().max()) <= 3e-7
    m.update_map()
    xe = m.x_edges.cpu()
    assert torch.equal(xe[:, [0, -1]], torch.tensor([[0.0, 1.0]] * 3, dtype=dtype))
    dx = m.dx_edges.cpu()
    assert float((dx.sum(dim=1) - 1.0).abs().max()) < 3e-7
    assert float(dx.min()) > 0.0 and float((dx[:, 1:] - dx[:, :-1]).max()) < 0.0
    assert float(m.get_X(yy)[0].abs().max()) == 0.0


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_stratification_reference_invariants(dtype, cuda):
    # vegas_stratification_test.py:10-62
    s = tq.VEGASStratification(1000, dim=3, rng=tq.RNG(seed=0), backend="torch", dtype=dtype)
    neval = s.get_NH(4000)
    assert neval.dtype == torch.int64 and neval.shape == (s.N_cubes,)
    assert int((neval - neval[0]).abs().max()) == 0
    y = s.get_Y(neval)
    assert y.dtype == dtype and y.shape == (int(neval.sum()), 3)
    assert bool((y >= 0).all()) and bool((y <= 1).all())
    f = torch.prod(torch.exp(y), dim=1)
    jf, jf2 = s.accumulate_weight(neval, f)
    assert float(jf2.min()) >= 0.0 and float((jf**2 - jf2).min()) >= 0.0
    s.update_DH()
    assert float(s.dh.min()) >= 0.0
    assert abs(float(s.dh.sum()) - 1.0) < 4e-7
    assert float(s.dh[-1]) > float(s.dh[0])
    neval = s.get_NH(4000)
    assert int(neval[-1]) > int(neval[0])
    y = s.get_Y(neval)
    assert y.shape == (int(neval.sum()), 3) and bool((y >= 0).all()) and bool((y <= 1).all())


def _load(p, dtype, cuda):
    return torch.tensor(G.arr(p["values"]).reshape(p["shape"]), dtype=dtype, device=cuda)


def _step_state(case, st, cuda):
    dtype = DT[case["dtype"]]
    dom = torch.tensor(case["domain"], dtype=dtype, device=cuda)
    dev = VegasDevice(3, dtype, case["n_bins"], case["n_strat"], cuda, dom)
    dev.x_edges.copy_(_load(st["x_edges"], dtype, cuda))
    dev.dx_edges.copy_(_load(st["dx_edges"], dtype, cuda))
    dev.dh.copy_(_load(st["dh"], dtype, cuda))
    dev.rng_offset.fill_(st["rng_offset"])
    return dev, dtype


def _check_step(case, st, dev, dtype, cuda, weights_before_update):
    f32 = dtype == torch.float32
    rtol = 2e-5 if f32 else 1e-11
    assert dev.counts.cpu().ravel().tolist() == st["counts"]  # bit-exact
    assert torch.allclose(weights_before_update, _load(st["weights"], torch.float64, cuda), rtol=rtol, atol=0)
    assert torch.allclose(dev.jf, _load(st["JF"], torch.float64, cuda), rtol=rtol, atol=1e-30)
    assert torch.allclose(dev.jf2, _load(st["JF2"], torch.float64, cuda), rtol=rtol, atol=1e-30)


@pytest.mark.parametrize("case", VG["steps"], ids=lambda c: c["dtype"])
def test_fused_iteration_matches_reference_state(case, cuda):
    f = tq.GaussianPeak(3, **{k: v for k, v in case["family"].items() if k != "kind"})
    params = f.device_params(cuda)
    for st in case["steps"]:
        dev, dtype = _step_state(case, st, cuda)
        dev.get_nh(st["starting_N"], normalize=False)
        assert dev.neval.cpu().tolist() == st["neval"]  # bit-exact
        M = sum(st["neval"])
        dev.set_control(L.TQ_VC_SEED | L.TQ_VC_STREAM, seed=case["seed"], sid=0)
        dev.iterate_fused(f.family, params, True, M)
        w = dev.weights.clone()
        _check_step(case, st, dev, dtype, cuda, w)
        assert int(dev.rng_offset.item()) == st["rng_offset"] + tq.RNG.blocks_for(3 * M, dtype)
        dev.finish(0.75, 0)
        stats = dev.stats[0].cpu()
        tol = 2e-5 if dtype == torch.float32 else 1e-11
        assert abs(float(stats[0]) - G.f(st["result"])) <= tol * abs(G.f(st["result"]))
        assert abs(float(stats[1]) - G.f(st["sigma2"])) <= 50 * tol * abs(G.f(st["sigma2"]))
        assert int(stats[2]) == M
        dev.update_map(0.5)
        xe_tol = 5e-6 if dtype == torch.float32 else 1e-12
        assert float((dev.x_edges - _load(st["x_edges_new"], dtype, cuda)).abs().max()) <= xe_tol
        dev.get_nh(st["starting_N"], normalize=True)  # normalises dh as update_DH does
        want = _load(st["dh_new"], dtype, cuda)
        dtol = 2e-3 if dtype == torch.float32 else 1e-9
        assert float((dev.dh - want).abs().max()) <= dtol * float(want.max())
        # what the next iteration consumes of dh (vegas_stratification.py:
        # 92-103): floor(dh * N) per cube, in dh's dtype, from the
        # reference's normalised dh, exactly
        nd = np.float32 if dtype == torch.float32 else np.float64
        dh_ref = want.cpu().numpy().astype(nd)
        nh_ref = np.clip(np.floor(dh_ref * nd(st["starting_N"])), 2, None).astype(np.int64)
        assert dev.neval.cpu().numpy().tolist() == nh_ref.tolist()


@pytest.mark.parametrize("case", VG["steps"], ids=lambda c: c["dtype"])
def test_materialised_iteration_matches_reference_state(case, cuda):
    f = tq.GaussianPeak(3, **{k: v for k, v in case["family"].items() if k != "kind"})
    for st in case["steps"][:2]:
        dev, dtype = _step_state(case, st, cuda)
        rng = tq.RNG(seed=case["seed"])
        rng.offset = st["rng_offset"]
        s = tq.VEGASStratification(case["N"] // 25, 3, rng, "torch", dtype, _device_state=dev)
        m = tq.VEGASMap(case["n_bins"], 3, "torch", dtype, _device_state=dev)
        neval = s.get_NH(st["starting_N"])
        assert neval.cpu().tolist() == st["neval"]
        y = s.get_Y(neval)
        x, jac = m.get_X_and_Jac(y)
        dom = dev.domain
        sizes = dom[:, 1] - dom[:, 0]
        jf = f(x * sizes + dom[:, 0]) * torch.prod(sizes) * jac
        m.accumulate_weight(y, jf**2)
        s.accumulate_weight(neval, jf)
        _check_step(case, st, dev, dtype, cuda, dev.weights.clone())


C2 = G.load_npz("vegas_c2_steps.npz")
F32 = torch.float32


def _c2_device(cuda):
    dom = torch.tensor([[0.0, 1.0]] * 6, dtype=F32, device=cuda)
    return VegasDevice(6, F32, 50, int(C2["n_strat"]), cuda, dom, stats_slots=32)


def _c2(name, cuda, dtype=F32):
    return torch.from_numpy(np.ascontiguousarray(C2[name])).to(device=cuda, dtype=dtype)


def _floor_nh(dh, n):
    """get_NH (vegas_stratification.py:92-103) in fp32 on the host."""
    return np.clip(np.floor((np.asarray(dh, dtype=np.float32) * np.float32(n)).astype(np.float32)), 2, None)


@pytest.mark.parametrize("it", [int(i) for i in C2["steps"]])
def test_plain_vegas_full_size_step_matches_reference(it, cuda):
    """The plain VEGAS configuration at full size (dim 6, N = 1e7, 50
    intervals, 6^6 = 46656 cubes, fp32, normal peak sigma 0.05, seed 0),
    one iteration from the reference's recorded state before iteration `it`
    on the same Philox draws: evaluations per cube and interval counts bit
    for bit; cube sums, interval weights, the estimate and the new map to
    fp32 rounding; and the next get_NH (floor(dh * N) per cube, the only
    place the next iteration depends on them) exactly."""
    p = f"it{it}_"
    f = tq.GaussianPeak.normal(6, 0.5, 0.05)
    assert np.array_equal(f.params_vector().numpy(), C2["params"])
    params = f.device_params(cuda)
    dev = _c2_device(cuda)
    dev.x_edges.copy_(_c2(p + "x_edges", cuda))
    dev.dx_edges.copy_(_c2(p + "dx_edges", cuda))
    dev.dh.copy_(_c2(p + "dh", cuda))
    dev.rng_offset.fill_(int(C2[p + "rng_offset"]))
    dev.get_nh(int(C2[p + "starting_N"]), normalize=False)
    neval = C2[p + "neval"].astype(np.int64)
    assert np.array_equal(dev.neval.cpu().numpy(), neval)  # bit-exact
    M = int(neval.sum())
    dev.set_control(L.TQ_VC_SEED | L.TQ_VC_STREAM, seed=0, sid=0)
    dev.iterate_fused(f.family, params, True, M)
    assert np.array_equal(dev.counts.cpu().numpy(), C2[p + "counts"])  # bit-exact
    assert torch.allclose(dev.weights, _c2(p + "weights", cuda, torch.float64), rtol=2e-5, atol=0)
    assert torch.allclose(dev.jf, _c2(p + "JF", cuda, torch.float64), rtol=2e-5, atol=1e-35)
    assert torch.allclose(dev.jf2, _c2(p + "JF2", cuda, torch.float64), rtol=2e-5, atol=1e-35)
    assert int(dev.rng_offset.item()) == int(C2[p + "rng_offset"]) + tq.RNG.blocks_for(6 * M, F32)
    dev.finish(0.75, 0)
    stats = dev.stats[0].cpu()
    assert abs(float(stats[0]) - float(C2[p + "result"])) <= 2e-5 * abs(float(C2[p + "result"]))
    assert abs(float(stats[1]) - float(C2[p + "sigma2"])) <= 1e-3 * abs(float(C2[p + "sigma2"]))
    assert int(stats[2]) == M
    dev.update_map(0.5)
    assert float((dev.x_edges - _c2(p + "x_edges_new", cuda)).abs().max()) <= 1e-6
    n = int(C2[p + "next_starting_N"])
    dev.get_nh(n, normalize=True)  # normalises dh as update_DH does
    want = C2[p + "dh_new"]
    got = dev.dh.cpu().numpy()
    assert np.max(np.abs(got - want)) <= 5e-5 * np.max(want)
    nh_ref = _floor_nh(want, n)
    assert np.array_equal(dev.neval.cpu().numpy(), nh_ref)  # the next iteration's counts, exactly
    assert np.array_equal(_floor_nh(got, n), nh_ref)
    nxt = [int(i) for i in C2["steps"]]
    if it + 1 in nxt:  # the reference's next iteration used exactly these counts
        assert np.array_equal(nh_ref, C2[f"it{it + 1}_neval"])


def test_plain_vegas_full_size_trajectory(cuda):
    """The GPU's own run of the plain VEGAS configuration against the
    reference's (both from seed 0 on the same Philox stream): after the
    warm-up the map agrees to a few fp32 ulps and the RNG offset exactly;
    iteration 1 has the same evaluations per cube.  Iteration 2's counts come
    from floor(dh * N) of sums over maps that differ in the last bits (the
    reference adds interval weights one point at a time in fp32, the kernels
    per warp in fp32 and across CTAs in fp64), so a cube whose dh * N lies
    within rounding of an integer can flip by one there; this test lists
    those flips and requires each to be such a near-tie.  After a flip the
    points move to other draws and the runs agree statistically
    (test_plain_vegas_full_size_matches_reference)."""
    f = tq.GaussianPeak.normal(6, 0.5, 0.05)
    params = f.device_params(cuda)
    dev = _c2_device(cuda)
    dev.set_control(L.TQ_VC_SEED | L.TQ_VC_STREAM, seed=0, sid=0)
    dev.rng_offset.fill_(0)
    for _ in range(5):
        dev.warmup_fused(f.family, params, 80000)
        dev.update_map(0.5)
    assert float((dev.x_edges - _c2("it1_x_edges", cuda)).abs().max()) <= 1e-6
    assert int(dev.rng_offset.item()) == int(C2["it1_rng_offset"])
    dev.get_nh(400000, normalize=False)
    assert np.array_equal(dev.neval.cpu().numpy(), C2["it1_neval"].astype(np.int64))
    dev.iterate_fused(f.family, params, True)
    assert np.array_equal(dev.counts.cpu().numpy(), C2["it1_counts"])
    dev.finish(0.75, 0)
    dev.update_map(0.5)
    dev.get_nh(400000, normalize=True)
    got = dev.neval.cpu().numpy()
    want_dh = C2["it2_dh"].astype(np.float64)
    flips = np.nonzero(got != C2["it2_neval"].astype(np.int64))[0]
    assert float(np.max(np.abs(dev.dh.cpu().numpy() - want_dh))) <= 5e-5 * float(want_dh.max())
    assert len(flips) <= 8, len(flips)
    for c in flips:
        x = want_dh[c] * 400000.0
        assert abs(got[c] - C2["it2_neval"][c]) == 1 and abs(x - round(x)) < 1e-2, (c, x, got[c])


def test_plain_vegas_full_size_matches_reference(cuda):
    """dim 6, N = 1e7, 50 intervals, fp32 normal peak, seed 0: the whole
    integration through the public API (graph-captured device loop) against
    the reference's run.  The first iteration is identical; the step-wise
    parity and the trajectory tests above pin the rest."""
    c = VG["c2"]
    f = tq.GaussianPeak.normal(6, 0.5, c["sigma"])
    v = tq.VEGAS()
    dom = torch.tensor([[0.0, 1.0]] * 6, dtype=torch.float32, device=cuda)
    r = v.integrate(f, 6, N=c["N"], integration_domain=dom, seed=c["seed"], n_intervals=c["n_bins"])
    assert r.dtype == torch.float32
    assert v.it == c["iterations"]
    Ms = [int(m) for m in v._dev.stats[: v.it, 2].cpu()]
    ref_Ms = [it["M"] for it in c["iters"]]
    assert Ms[0] == ref_Ms[0]
    # after the first floor flip the counts follow other draws: same budget rule
    assert v._nr_of_fevals <= c["N"] and abs(v._nr_of_fevals - c["fevals"]) <= 0.001 * c["fevals"]
    want = G.f(c["value"])
    assert abs(r.item() - want) <= 5 * v._get_error() + 1e-6
    assert abs(r.item() - 1.0) < 5e-3


def test_fused_and_materialised_paths_agree(cuda):
    f = tq.GaussianPeak(3, a=[5.0, 8.0, 3.0], u=[0.3, 0.5, 0.7])
    dom = torch.tensor([[0.0, 1.0], [-1.0, 1.0], [0.0, 2.0]], dtype=torch.float64, device=cuda)
    a, b = tq.VEGAS(), tq.VEGAS()
    ra = a.integrate(f, 3, N=20000, integration_domain=dom, seed=11)
    rb = b.integrate(lambda x: f(x), 3, N=20000, integration_domain=dom, seed=11)
    assert a._nr_of_fevals == b._nr_of_fevals and a.it == b.it
    assert abs(ra.item() - rb.item()) <= 1e-9 * abs(ra.item())


def test_reference_run_step_sequence(cuda):
    case = [c for c in VG["steps"] if c["dtype"] == "float64"][0]
    f = tq.GaussianPeak(3, **{k: v for k, v in case["family"].items() if k != "kind"})
    dom = torch.tensor(case["domain"], dtype=torch.float64, device=cuda)
    v = tq.VEGAS()
    r = v.integrate(f, 3, N=case["N"], integration_domain=dom, seed=case["seed"])
    assert v.it == case["iterations"] and v._nr_of_fevals == case["fevals"]
    assert abs(r.item() - G.f(case["value"])) <= 1e-9 * abs(G.f(case["value"]))


def test_zero_and_constant_integrands(cuda):
    # vegas_test.py:159-184
    dom = torch.tensor([[0.0, 3.0]] * 2, dtype=torch.float64, device=cuda)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        z = tq.VEGAS().integrate(lambda x: x[:, 0] * 0.0, 2, N=10000, integration_domain=dom, seed=0)
    assert z.item() == 0.0
    c = tq.VEGAS().integrate(lambda x: x[:, 0] * 0.0 + 10.0, 2, N=10000, integration_domain=dom, seed=0)
    assert abs(c.item() - 90.0) < 1e-13
    assert abs(c.item() - G.f(VG["special"]["constant"])) < 1e-13
    with pytest.warns(RuntimeWarning, match="Cannot update the VEGASMap"):
        tq.VEGAS().integrate(tq.ExpSum(2, c=0.0), 2, N=10000, integration_domain=dom, seed=0)


class ModifiedRNG(tq.RNG):
    """Replaces half of the draws with exactly 0.0 or 1.0 (vegas_test.py:143-156)."""

    def uniform(self, size, dtype):
        n = super().uniform(size, dtype)
        return torch.where(n < 0.5, n * 2.0, torch.where(n < 0.75, torch.zeros_like(n), torch.ones_like(n)))


def test_draws_of_exactly_zero_and_one(cuda):
    dom = torch.tensor([[0.0, 1.0]] * 2, dtype=torch.float64, device=cuda)
    r = tq.VEGAS().integrate(lambda x: torch.sum(x, dim=1), 2, N=10000, integration_domain=dom,
                             rng=ModifiedRNG(seed=0))
    assert abs(r.item() - 1.0) < 0.1


def test_peak_accuracy_reference_cases(cuda):
    # vegas_test.py:71-140
    dom = torch.tensor([[1.0, 5.0], [-4.0, 4.0], [2.0, 6.0]], dtype=torch.float64, device=cuda)

    def cube(x):
        return torch.prod((x >= 3.0) * (x < 4.0), dim=1).to(torch.float64) + 0.001

    ref = float(torch.prod(dom[:, 1] - dom[:, 0])) * 0.001 + 1.0
    for seed in [0, 1, 2, 3, 41317]:
        r = tq.VEGAS().integrate(cube, 3, N=30000, integration_domain=dom, seed=seed)
        assert abs(r.item() - ref) < 0.03
    d2 = torch.tensor([[1.0, 101.0], [-4.0, 96.0]], dtype=torch.float64, device=cuda)

    def diag(x):
        return torch.exp(torch.sum(d2[:, 0] - x, dim=1)) + torch.exp(torch.sum(x - d2[:, 1], dim=1))

    ref2 = 2.0 - 4.0 * math.exp(-100.0) + 2.0 * math.exp(-200.0)
    # Two peaks in opposite corners: whether the warm-up finds both depends on
    # the draws.  With this package's Philox stream the reference algorithm
    # itself (the oracle, same draws) finds one peak for two of the
    # reference's five seeds; the GPU must reproduce the algorithm on every
    # seed and be accurate where the algorithm is.
    from oracle import philox as OP
    from oracle import vegas as OV

    d2n = d2.cpu().numpy()

    def diag_np(x):
        return np.exp(np.sum(d2n[:, 0] - x, axis=1)) + np.exp(np.sum(x - d2n[:, 1], axis=1))

    good = 0
    for seed in [0, 1, 2, 3, 41317]:
        r = tq.VEGAS().integrate(diag, 2, N=30000, integration_domain=d2, seed=seed).item()
        o = OV.Vegas().integrate(diag_np, 2, 30000, d2n, OP.ReplayStream(seed), dt=np.float64)
        assert abs(r - o) <= 1e-9 * abs(o)
        good += abs(r - ref2) < 0.03
    assert good >= 3


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_large_map_update_matches_oracle(dtype, cuda):
    """Maps with more than 1024 intervals per dimension use the tiled passes."""
    from oracle import vegas as OV

    B, d = 5000, 2
    rng = np.random.default_rng(4)
    counts = rng.integers(1, 50, size=(d, B)).astype(np.int64)
    weights = rng.uniform(0.1, 3.0, size=(d, B)) * counts
    _check_large_map(OV, dtype, cuda, weights, counts)


def _check_large_map(OV, dtype, cuda, weights, counts, tol32=2e-5):
    d, B = counts.shape
    nd = np.float32 if dtype == torch.float32 else np.float64
    m = OV.Map(B, d, nd)
    m.weights = weights.astype(nd)
    m.counts = counts.copy()
    sw_ref = OV.Map.smooth_map(m.weights, m.counts, 0.5)
    updated = m.update_map()
    dev = VegasDevice(d, dtype, B, 1, cuda)
    dev.weights.copy_(torch.tensor(weights.astype(nd).astype(np.float64), device=cuda))
    dev.counts.copy_(torch.tensor(counts, device=cuda))
    x0 = dev.x_edges.double().cpu().numpy().copy()
    sw = dev.smooth(0.5)
    if sw_ref is not None:
        tol_sw = 1e-5 if dtype == torch.float32 else 1e-12
        assert np.max(np.abs(sw.double().cpu().numpy() - sw_ref) / np.abs(sw_ref).max()) <= tol_sw
    f0 = int(dev.flags[0].item())
    dev.update_map(0.5)
    got = dev.x_edges.double().cpu().numpy()
    if updated:
        tol = tol32 if dtype == torch.float32 else 1e-10
        assert np.max(np.abs(got - m.x_edges.astype(np.float64))) <= tol
        assert np.all(np.diff(got, axis=1) > 0)
        dx = dev.dx_edges.double().cpu().numpy()
        assert np.max(np.abs(dx - np.diff(got, axis=1))) <= (1e-6 if dtype == torch.float32 else 1e-14)
    else:
        assert np.array_equal(got, x0)  # the map cannot be updated: edges stay
        assert int(dev.flags[0].item()) == f0 + 1
    assert int(dev.counts.abs().sum()) == 0  # reset after the update
    assert float(dev.weights.abs().sum()) == 0.0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("case", ["zeros", "raw_zeros", "peaked", "zero_row"])
def test_large_map_cases_match_oracle(case, dtype, cuda):
    """Tiled map update: empty intervals filled across tile boundaries and
    beyond ten neighbours (closed form), empty intervals that carry weights
    (the sweeps themselves), concentrated weights (long runs of equal delta
    multiples, multiples that skip), and a row without weight (map reset)."""
    from oracle import vegas as OV

    rng = np.random.default_rng({"zeros": 5, "raw_zeros": 8, "peaked": 6, "zero_row": 7}[case])
    d, B = (5, 40000) if case != "zero_row" else (3, 3000)
    counts = rng.integers(1, 20, size=(d, B)).astype(np.int64)
    weights = rng.uniform(0.1, 3.0, size=(d, B)) * counts
    if case == "raw_zeros":  # empty intervals with weights set directly: the fill sweeps shift them
        z = rng.random((d, B)) < 0.3
        z[:, 3000:3030] = True
        counts[z] = 0
    if case == "zeros":
        z = rng.random((d, B)) < 0.3
        z[:, 2040:2065] = True  # a run of 25 across the first tile boundary
        z[:, :12] = True
        z[:, -13:] = True
        z[0, 10000:10003] = True
        counts[z] = 0
        weights[z] = 0.0
    elif case == "peaked":
        x = (np.arange(B) + 0.5) / B
        for k in range(d):
            peak = np.exp(-(((x - rng.uniform(0.2, 0.8)) / 0.01) ** 2)) + 1e-7
            weights[k] = peak * counts[k]
    else:
        counts[1] = 0
        weights[1] = 0.0
    _check_large_map(OV, dtype, cuda, weights, counts, tol32=5e-5)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("B", [2, 50, 1024])
@pytest.mark.parametrize("case", ["uniform", "random", "zeros"])
def test_small_map_cases_match_oracle(case, B, dtype, cuda):
    """One-CTA-per-row map update (at most 1024 intervals): uniform weights
    (every cumulative sum an exact multiple of delta), random weights, and
    empty intervals."""
    from oracle import vegas as OV

    rng = np.random.default_rng({"uniform": 11, "random": 12, "zeros": 13}[case] + B)
    d = 4
    counts = rng.integers(1, 30, size=(d, B)).astype(np.int64)
    if case == "uniform":
        weights = 2.5 * counts.astype(np.float64)
    else:
        weights = rng.uniform(0.05, 4.0, size=(d, B)) * counts
    if case == "zeros" and B > 2:
        z = rng.random((d, B)) < 0.35
        z[:, 0] = True
        counts[z] = 0
        weights[z] = 0.0
    _check_large_map(OV, dtype, cuda, weights, counts)


def test_default_interval_count_vegas(cuda):
    """The reference's default map size (N_increment // 10 intervals) at a
    size that takes the large-map path."""
    f = tq.GaussianPeak.normal(3, 0.5, 0.1)
    dom = torch.tensor([[0.0, 1.0]] * 3, dtype=torch.float64, device=cuda)
    v = tq.VEGAS()
    r = v.integrate(f, 3, N=2_000_000, integration_domain=dom, seed=3)
    assert v.map.N_intervals == 2_000_000 // 25 // 10
    assert abs(r.item() - 1.0) < 5 * v._get_error() + 1e-3


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_device_abort_test_matches_reference(dtype, cuda):
    """tq_vegas_abort_test (the every-fifth-iteration test on the device)
    against the reference's _check_abort_conditions on tensors of the
    state's dtype (golden): decision, adapted _starting_N, zero variances,
    x / 0, and the non-finite int() for which the reference raises (stop
    codes 5 / 6)."""
    d = VegasDevice(2, DT[dtype], 4, 2, cuda, stats_slots=64)
    zeros = np.zeros(6)
    cases = [c for c in VG["abort"] if c["dtype"] == dtype]
    assert len(cases) >= 90
    for case in cases:
        it, warm = case["it"], 777
        pts = np.arange(1, it + 1) * 1000
        d.begin_run(case["sN"], case["N"], case["inc"], case["max_it"], warm, case["eps_rel"],
                    case["eps_abs"], 0, 0, 0, zeros)
        st = torch.zeros((it, 4), dtype=torch.float64)
        st[:, 2] = torch.tensor(pts, dtype=torch.float64)
        st[it - 5:, 0] = torch.tensor(G.arr(case["r"]), dtype=torch.float64)
        st[it - 5:, 1] = torch.tensor(G.arr(case["s"]), dtype=torch.float64)
        d.stats[:it] = st.to(cuda)
        d.control[1] = it
        d.control[11] = it - 5
        d.abort_test(0)
        d.read_back()
        c = d.host_control
        assert int(c[L.VC_EVALS]) == case["fevals"] == warm + int(pts.sum())
        assert int(c[L.VC_IT]) == it
        if case["error"]:
            assert int(c[L.VC_STOP]) == {"OverflowError": 5, "ValueError": 6}[case["error"]], case
            continue
        assert bool(c[L.VC_STOP]) == case["stop"], case
        assert int(c[L.VC_NEVALS]) == case["starting_N"], case


def test_fused_graph_and_eager_runs_agree(cuda):
    """The captured run (warm-up + WHILE node with the device abort test)
    and the same launches run eagerly give the same integration."""
    from torchquad_gb300.integration import vegas as V
    f = tq.GaussianPeak.normal(4, 0.5, 0.1)
    dom = torch.tensor([[0.0, 1.0]] * 4, dtype=torch.float32, device=cuda)
    out = []
    for eager in (False, True):
        V.FORCE_EAGER[0] = eager
        try:
            for seed in (1, 2, 3):  # the second call of a shape captures the graph
                v = tq.VEGAS()
                r = v.integrate(f, 4, N=400_000, integration_domain=dom, seed=seed)
            out.append((r.item(), v.it, v._nr_of_fevals, v._starting_N, v.rng.offset,
                        list(v.results), list(v.sigma2)))
        finally:
            V.FORCE_EAGER[0] = False
    assert out[0] == out[1]


def test_fused_host_domain_and_dh_normalised(cuda):
    """A domain given as host values (launch arguments) integrates exactly
    like the same domain as a tensor; dh comes out normalised (once)."""
    f = tq.GaussianPeak.normal(3, 0.4, 0.1)
    dom_list = [[0.0, 1.0], [-0.5, 1.0], [0.1, 0.9]]
    a, b = tq.VEGAS(), tq.VEGAS()
    ra = a.integrate(f, 3, N=200_000, integration_domain=dom_list, seed=4)
    dh_a = a.strat.dh.clone()
    rb = b.integrate(f, 3, N=200_000, seed=4,
                     integration_domain=torch.tensor(dom_list, dtype=torch.get_default_dtype(), device=cuda))
    assert ra.dtype == rb.dtype == torch.get_default_dtype()
    assert ra.item() == rb.item() and a.it == b.it and a._nr_of_fevals == b._nr_of_fevals
    assert abs(float(dh_a.double().sum()) - 1.0) < 1e-5
    assert torch.equal(b.strat.dh, dh_a)
    assert torch.equal(b.strat.dh, dh_a)  # a second access does not divide again


_STATE_TENSORS = ("x_edges", "dx_edges", "weights", "counts", "dh", "jf", "jf2", "neval",
                  "cube_start", "rng_offset", "stats", "flags", "scalars", "control")


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_split_get_nh_matches_get_nh(dtype, cuda):
    """get_NH leaving cube_start split (block offsets added by the sampler,
    written back by finish) gives the same points, counts and final cube
    prefix as get_NH with its fix-up launch."""
    f = tq.GaussianPeak.normal(4, 0.5, 0.1)
    params = f.device_params(cuda)
    d = VegasDevice(4, dtype, 50, 20, cuda)  # 160000 cubes: 625 blocks of 256
    d.set_control(L.TQ_VC_NEVALS | L.TQ_VC_SEED | L.TQ_VC_STREAM, nevals=700000, seed=3, sid=0)
    d.warmup_fused(f.family, params, 50000)
    d.update_map(0.5)
    d.get_nh()
    d.iterate_fused(f.family, params, True)
    d.finish(0.75)
    snap = {n: getattr(d, n).clone() for n in _STATE_TENSORS}
    out = []
    for split in (False, True):
        for n in _STATE_TENSORS:
            getattr(d, n).copy_(snap[n])
        if split:
            d.get_nh_split()
            assert int(d.control[14].item()) == 1
        else:
            d.get_nh()
        d.iterate_fused(f.family, params, True)
        d.finish(0.75)
        out.append({n: getattr(d, n).clone() for n in _STATE_TENSORS})
    a, b = out
    for n in ("neval", "cube_start", "counts", "rng_offset"):
        assert torch.equal(a[n], b[n]), n
    assert torch.equal(a["stats"][:, 2], b["stats"][:, 2])
    assert int(b["control"][14].item()) == 0
    # the cube sums are fp64 atomics (order-dependent rounding), dh follows them
    assert torch.allclose(a["jf"], b["jf"], rtol=1e-12, atol=0)
    assert torch.allclose(a["dh"], b["dh"], rtol=1e-5 if dtype == torch.float32 else 1e-11, atol=0)
    assert torch.allclose(a["weights"], b["weights"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("opts", [dict(use_grid_improve=False), dict(use_warmup=False),
                                  dict(eps_rel=1e-2), dict(eps_rel=1e-3, max_iterations=40),
                                  dict(eps_abs=1e-4)])
def test_fused_options_match_materialised(opts, cuda):
    """The reference's VEGAS options through the device-side loop (fused;
    the second call of a shape replays the captured graph) against the host
    loop of the materialised path on the same draws."""
    f = tq.GaussianPeak(3, a=[5.0, 8.0, 3.0], u=[0.3, 0.5, 0.7])
    dom = torch.tensor([[0.0, 1.0], [-1.0, 1.0], [0.0, 2.0]], dtype=torch.float64, device=cuda)
    for seed in (11, 12):
        a, b = tq.VEGAS(), tq.VEGAS()
        ra = a.integrate(f, 3, N=40000, integration_domain=dom, seed=seed, **opts)
        rb = b.integrate(lambda x: f(x), 3, N=40000, integration_domain=dom, seed=seed, **opts)
        assert (a.it, a._nr_of_fevals, a._starting_N) == (b.it, b._nr_of_fevals, b._starting_N)
        assert abs(ra.item() - rb.item()) <= 1e-9 * abs(rb.item())


def test_integrators_keep_their_own_state(cuda):
    """Integrators of the same shape share one device plan; each keeps its
    own map and stratification afterwards (as the reference's instances
    own theirs), whether it reads them before or after the next run."""
    f = tq.GaussianPeak.normal(3, 0.5, 0.1)
    dom = torch.tensor([[0.0, 1.0]] * 3, dtype=torch.float32, device=cuda)
    a, b, c = tq.VEGAS(), tq.VEGAS(), tq.VEGAS()
    ra = a.integrate(f, 3, N=200_000, integration_domain=dom, seed=1)
    xa, dha = a.map.x_edges.clone(), a.strat.dh.clone()
    rb = b.integrate(f, 3, N=200_000, integration_domain=dom, seed=2)
    xb, dhb = b.map.x_edges.clone(), b.strat.dh.clone()
    assert not torch.equal(xa, xb) and ra.item() != rb.item()
    c.integrate(f, 3, N=200_000, integration_domain=dom, seed=3)
    assert torch.equal(a.map.x_edges, xa) and torch.equal(a.strat.dh, dha)
    assert torch.equal(b.map.x_edges, xb) and torch.equal(b.strat.dh, dhb)
    # d (b's seed) reads its dh only after the next run: still its own,
    # normalised once (equal to b's up to the order of fp64 atomic adds)
    d = tq.VEGAS()
    d.integrate(f, 3, N=200_000, integration_domain=dom, seed=2)
    a.integrate(f, 3, N=200_000, integration_domain=dom, seed=5)
    assert torch.allclose(d.map.x_edges, xb, rtol=0, atol=1e-6)
    assert torch.allclose(d.strat.dh, dhb, rtol=1e-5, atol=0)


def test_more_live_integrators_than_pooled_plans(cuda):
    """Six integrators of one shape alive at once (more than the plans kept
    per shape): the ones whose plan is handed on get a private copy of
    their state first, so every one still reads its own map and dh."""
    f = tq.GaussianPeak.normal(2, 0.5, 0.1)
    dom = torch.tensor([[0.0, 1.0]] * 2, dtype=torch.float64, device=cuda)
    vs, snaps = [], []
    for seed in range(6):
        v = tq.VEGAS()
        v.integrate(f, 2, N=50_000, integration_domain=dom, seed=100 + seed)
        vs.append(v)
        snaps.append((v.map.x_edges.clone(), v.strat.dh.clone(), list(v.results)))
    for v, (xe, dh, res) in zip(vs, snaps):
        assert torch.equal(v.map.x_edges, xe) and torch.equal(v.strat.dh, dh) and v.results == res



def test_fused_sampler_dynamic_smem_near_default_limit(cuda):
    """fp32 d=5 with 94 map intervals: the sampler's dynamic shared memory
    (47.8 KB: map edges plus per-warp histograms) and its static shared
    memory together pass the 48 KB a launch gets without the opt-in, which
    is made for it."""
    f = tq.SumSin(5, a=2.0)
    dom = torch.tensor([[0.0, 1.0]] * 5, dtype=torch.float32, device=cuda)
    v = tq.VEGAS()
    r = v.integrate(f, 5, N=23_672, integration_domain=dom, seed=7)
    exact = f.exact(dom)
    assert v.map.N_intervals == 94
    assert abs(float(r) - exact) < 0.05 * abs(exact)
