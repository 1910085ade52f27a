"""Host-side logic that needs no GPU: N adjustment, input validation and
the RNG's counter bookkeeping, checked against the reference's behaviour."""
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300.integration.base_integrator import BaseIntegrator
from torchquad_gb300.integration.utils import _check_integration_domain, _host_domain_check


def test_simpson_adjust_n_warnings():
    with pytest.warns(UserWarning, match="cannot be lower than 3"):
        assert tq.Simpson._adjust_N(2, 4) == 9
    with pytest.warns(UserWarning, match="cannot be even"):
        assert tq.Simpson._adjust_N(3, 1076890) == 101**3
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        assert tq.Simpson._adjust_N(3, 101**3) == 101**3


def test_boole_adjust_n_warnings():
    with pytest.warns(UserWarning, match="cannot be lower than 5"):
        assert tq.Boole._adjust_N(1, 4) == 5
    with pytest.warns(UserWarning, match="1 \\+ 4n"):
        assert tq.Boole._adjust_N(3, 1000) == 9**3


def test_minimal_n():
    assert tq.Simpson._get_minimal_N(3) == 27
    assert tq.Boole._get_minimal_N(2) == 25


@pytest.mark.parametrize(
    "kwargs",
    [dict(dim=0), dict(N=0), dict(N=2.5), dict(dim=2, integration_domain=[[0, 1]])],
)
def test_check_inputs_errors(kwargs):
    with pytest.raises(ValueError):
        BaseIntegrator._check_inputs(**kwargs)


def test_domain_checks():
    with pytest.raises(ValueError):
        _host_domain_check([[1.0, 0.0]])
    with pytest.raises(ValueError):
        _host_domain_check([[0.0, 1.0, 2.0]])
    with pytest.raises(ValueError):
        _host_domain_check([])
    assert _host_domain_check([[0, 1], [2, 3]]) == 2
    with pytest.raises(ValueError):
        _check_integration_domain(torch.tensor([[1.0, 0.0]]))
    with pytest.raises(ValueError):
        _check_integration_domain(torch.zeros(3))
    assert _check_integration_domain(torch.tensor([[0.0, 1.0]] * 4)) == 4


def test_rng_block_accounting():
    r = tq.RNG(seed=3)
    assert r.reserve(10, torch.float32) == 0
    assert r.offset == 3
    assert r.reserve(3, torch.float64) == 3
    assert r.offset == 5
    with pytest.raises(ValueError):
        tq.RNG(backend="numpy")


def test_non_torch_backend_rejected():
    with pytest.raises(ValueError):
        tq.set_up_backend("jax")


def test_builtin_integrands_match_oracle_on_cpu():
    from oracle import integrands as OI

    x = torch.rand(64, 3, dtype=torch.float64)
    for f in [tq.ExpSum(3, a=[1, 2, 3], b=0.5, c=2.0), tq.GaussianPeak(3, a=[1, 2, 3], u=[0.1, 0.2, 0.3]),
              tq.Oscillatory(3, a=[1, -1, 2], b=0.2), tq.SumSin(3, a=[1, 2, 3], c=0.5)]:
        got = f(x).numpy()
        want = OI.evaluate(f.family, f.params_vector().numpy(), x.numpy())
        assert np.allclose(got, want, rtol=1e-15, atol=0)


def test_batch_pack_layout():
    """Host packing of a batch (numpy only): descriptor fields, offsets, the
    tile prefix and domain checks, against a per-integral loop."""
    import numpy as np

    from torchquad_gb300 import batch as B

    rng = np.random.default_rng(0)
    fs, rules, Ns, doms = [], [], [], []
    names = ["trapezoid", "simpson", "boole", "gausslegendre"]
    for i in range(40):
        d = int(rng.integers(1, 5))
        fs.append(tq.GaussianPeak(d, a=rng.uniform(0.5, 5, d).tolist(), u=rng.uniform(0, 1, d).tolist()))
        rules.append(names[i % 4])
        Ns.append(int(10 ** rng.uniform(2, 4)))
        lo = rng.uniform(-1, 0, d)
        doms.append(np.stack([lo, lo + rng.uniform(0.5, 2, d)], axis=1).tolist())
    desc, ts, par, dom, gln, glw, fam, tp = B.pack(fs, rules, Ns, doms, torch.float64, 1000)
    po = do = 0
    gl = {}
    for i, (f, r, N) in enumerate(zip(fs, rules, Ns)):
        rid = B.rule_id(r)
        n = B.points_per_dim(rid, f.dim, N)
        assert tuple(desc[i])[:4] == (rid, f.dim, n, n ** f.dim)
        assert desc[i]["par_off"] == po and desc[i]["dom_off"] == do
        assert np.array_equal(par[po:po + 2 + 2 * f.dim], f.params_vector().numpy())
        assert np.array_equal(dom[do:do + 2 * f.dim], np.asarray(doms[i]).ravel())
        if rid == 3:
            if n not in gl:
                gl[n] = int(desc[i]["gl_off"])
            assert np.array_equal(gln[gl[n]:gl[n] + n], np.polynomial.legendre.leggauss(n)[0])
        po += 2 + 2 * f.dim
        do += 2 * f.dim
    assert ts[0] == 0 and np.array_equal(np.diff(ts), (desc["total"] + 999) // 1000)
    bad = [list(map(list, dm)) for dm in doms]
    bad[7][0] = [1.0, 0.0]
    with pytest.raises(ValueError, match="integral 7"):
        B.pack(fs, rules, Ns, bad, torch.float64, 1000)


def test_integrand_parameter_vector_cache():
    """The cached host parameter vector follows in-place writes."""
    import numpy as np

    f = tq.GaussianPeak(3, a=[1.0, 2.0, 3.0], u=[0.1, 0.2, 0.3], c=2.0)
    assert np.array_equal(f.params_numpy(), f.params_vector().numpy())
    f.a[1] = 7.0
    assert f.params_numpy()[3] == 7.0
    g = tq.Oscillatory(2, a=[1.0, -1.0], b=torch.tensor(0.3, dtype=torch.float64))
    assert np.array_equal(g.params_numpy(), g.params_vector().numpy())


def test_vegas_abort_helpers_follow_tensor_arithmetic():
    """The abort test's sums run left to right from zero (Python's builtin
    sum of floats is compensated since 3.12), x / 0 gives IEEE values and
    the arithmetic is in the state's dtype, as the reference's 0-d tensor
    arithmetic does."""
    import math

    from torchquad_gb300.integration.vegas import _sum_lr

    xs = [1e16, 1.0, -1e16, 1.0]
    assert _sum_lr(xs) == ((1e16 + 1.0) + -1e16) + 1.0
    for dtype in (torch.float64, torch.float32):
        v = tq.VEGAS()
        v.dtype = dtype
        v.it, v.results, v.sigma2 = 5, [1.0, 2.0, 1.0, 1.0, 1.0], [0.0, 1.0, 1.0, 1.0, 1.0]
        v._eps_rel = v._eps_abs = 0.0
        v._starting_N = v._N_increment = 4000
        v.N, v._max_iterations, v._nr_of_fevals = 10**6, 20, 20000
        assert v._get_chisq() == math.inf  # (1 - 1.2)^2 / 0
        assert v._check_abort_conditions() is False and v._starting_N == 8000
    # fp32 state: the estimate is rounded per operation in fp32
    v = tq.VEGAS()
    v.dtype = torch.float32
    v.results, v.sigma2 = [1.0 + 2**-20, 1.0, 1.0, 1.0, 1.0], [3.0] * 5
    want = np.float32(0)
    for r in v.results:
        want = want + np.float32(r) / np.float32(3.0)
    den = np.float32(0)
    for _ in range(5):
        den = den + np.float32(1) / np.float32(3.0)
    assert v._get_result() == want / den and isinstance(v._get_result(), np.float32)


def test_vegas_abort_test_matches_reference_golden():
    """The host abort test (used by the materialised path and after the
    fused runs for the estimate) against the reference's
    _check_abort_conditions on fp32 and fp64 tensors: decision, adapted
    _starting_N and the exception int() raises for a non-finite value."""
    from tests import golden as G

    for c in G.load("vegas_golden.json")["abort"]:
        v = tq.VEGAS()
        v.dtype = torch.float32 if c["dtype"] == "float32" else torch.float64
        v.it, v.results, v.sigma2 = c["it"], G.arr(c["r"]).tolist(), G.arr(c["s"]).tolist()
        v._eps_rel, v._eps_abs = c["eps_rel"], c["eps_abs"]
        v._starting_N, v._N_increment, v.N = c["sN"], c["inc"], c["N"]
        v._max_iterations, v._nr_of_fevals = c["max_it"], c["fevals"]
        if c["error"]:
            with pytest.raises({"OverflowError": OverflowError, "ValueError": ValueError}[c["error"]]):
                v._check_abort_conditions()
            continue
        assert v._check_abort_conditions() == c["stop"], c
        assert v._starting_N == c["starting_N"], c


def test_host_domain_values():
    from torchquad_gb300.integration.utils import _host_domain_values

    assert _host_domain_values(2, None, None) == [(-1.0, 1.0)] * 2
    assert _host_domain_values(2, [[0, 1], [2, 3.5]], None) == [(0.0, 1.0), (2.0, 3.5)]
    assert _host_domain_values(2, np.array([[0.0, 1.0], [2.0, 3.0]]), None) == [(0.0, 1.0), (2.0, 3.0)]
    assert _host_domain_values(2, torch.zeros(2, 2), None) is None
    with pytest.raises(ValueError):
        _host_domain_values(3, [[0, 1], [0, 1]], None)
    with pytest.raises(ValueError):
        _host_domain_values(2, [[0, 1, 2], [0, 1]], None)
    with pytest.raises(ValueError):
        _host_domain_values(2, [[0, 1], [0, 1]], "jax")


def test_gaussian_root_cache_and_composite_rule():
    """The Gaussian extension points a custom rule relies on
    (gaussian.py:109-143): roots cached under (N, *_root_args), N given as an
    int, a numpy integer or a 0-d tensor, anything else rejected; the
    composite rule collapses the trailing node axes and scales by the
    half-widths, as the reference's one-axis-at-a-time loop does."""
    g = tq.Gaussian()
    r3, w3 = g._cached_points_and_weights(3)
    assert np.allclose(r3, [-np.sqrt(0.6), 0.0, np.sqrt(0.6)]) and np.isclose(w3.sum(), 2.0)
    assert g._cached_points_and_weights(np.int64(3)) is g._cached_points_and_weights(3)
    assert g._cached_points_and_weights(torch.tensor(3)) is g._cached_points_and_weights(3)
    with pytest.raises(NotImplementedError):
        g._cached_points_and_weights(3.0)

    calls = []

    class Tagged(tq.Gaussian):
        def __init__(self):
            super().__init__()
            self._root_args = ("tag",)
            self._root_fn = lambda n, tag: calls.append((n, tag)) or np.polynomial.legendre.leggauss(n)

    t = Tagged()
    t._cached_points_and_weights(4)
    t._cached_points_and_weights(4)
    assert calls == [(4, "tag")]

    v = torch.rand(2, 5, 5, 5, dtype=torch.float64)
    dom = torch.tensor([[-1.0, 2.0], [0.0, 0.5], [1.0, 3.0]], dtype=torch.float64)
    want = v
    for d in range(3):  # the reference's order: last axis first, dimension d's half-width
        want = 0.5 * (dom[d][1] - dom[d][0]) * torch.sum(want, dim=want.dim() - 1)
    got = tq.Gaussian._apply_composite_rule(v, 3, None, dom)
    assert got.shape == want.shape == (2,)
    assert torch.allclose(got, want, rtol=1e-14, atol=0)
