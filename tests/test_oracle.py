"""The CPU oracle against the reference's golden outputs and known-answer
vectors (no GPU)."""
import math

import numpy as np
import pytest

from oracle import grid as OG
from oracle import integrands as OI
from oracle import mc as OM
from oracle import philox as OP
from tests import golden as G


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in kat:
        got = OP.philox4x32_10(*[[c] for c in ctr], *key)
        assert tuple(int(g[0]) for g in got) == want


def test_uniform_layout_and_range():
    u32 = OP.uniform(5, 0, 0, 10, np.float32)
    u64 = OP.uniform(5, 0, 0, 10, np.float64)
    assert u32.dtype == np.float32 and u64.dtype == np.float64
    assert np.all(u32 >= 0) and np.all(u32 < 1) and np.all(u64 >= 0) and np.all(u64 < 1)
    # offsets: a second request continues the counter
    s = OP.ReplayStream(5)
    a = s.uniform([3], np.float32)
    b = s.uniform([5], np.float32)
    assert np.array_equal(a, OP.uniform(5, 0, 0, 3, np.float32))
    assert np.array_equal(b, OP.uniform(5, 0, 1, 5, np.float32))


def test_linspace_matches_torch_cpu_bitwise():
    for c in G.load("grid_mc_golden.json")["linspace"]:
        dt = np.float32 if c["dtype"] == "float32" else np.float64
        got = OG.linspace(G.f(c["a"]), G.f(c["b"]), c["n"], dt)
        assert np.array_equal(got.astype(np.float64), G.arr(c["values"])), c


@pytest.mark.parametrize("case", G.load("grid_mc_golden.json")["grid"], ids=lambda c: c["name"])
def test_oracle_grid_matches_reference(case):
    dt = np.float32 if case["dtype"] == "float32" else np.float64
    params = G.arr(case["params"])
    fam = {"ExpSum": 1, "GaussianPeak": 2, "Oscillatory": 3, "SumSin": 4}[case["family"]["kind"]]
    rule = G.RULES[case["rule"]]
    val = OG.integrate(lambda x: OI.evaluate(fam, params, x), rule, case["dim"], case["N"],
                       np.array(case["domain"]), dt)
    want = G.f(case["value"])
    tol = 1e-12 if (dt == np.float64 or rule == OG.GAUSS) else 1e-6
    assert abs(float(val) - want) <= tol * max(1.0, abs(want)), (float(val), want)


def test_c1_reference_value():
    c = [c for c in G.load("grid_mc_golden.json")["grid"] if c["name"].startswith("C1")][0]
    want = G.f(c["value"])
    assert abs(want - 5.073214112618379) < 1e-15
    assert abs(want - (math.e - 1) ** 3) / (math.e - 1) ** 3 < 2e-10


@pytest.mark.parametrize("case", G.load("grid_mc_golden.json")["mc"], ids=lambda c: f"mc-{c['dim']}-{c['dtype']}")
def test_oracle_mc_matches_reference(case):
    dt = np.float32 if case["dtype"] == "float32" else np.float64
    u = OP.uniform(case["seed"], 0, 0, case["N"] * case["dim"], dt).reshape(case["N"], case["dim"])
    assert np.array_equal(u.ravel()[:16].astype(np.float64), G.arr(case["first_uniforms"]))
    params = G.arr(case["params"])
    fam = {"ExpSum": 1, "GaussianPeak": 2, "Oscillatory": 3, "SumSin": 4}[case["family"]["kind"]]
    val = OM.integrate(lambda x: OI.evaluate(fam, params, x), case["dim"], case["N"], np.array(case["domain"]), u)
    want = G.f(case["value"])
    tol = 1e-5 if dt == np.float32 else 1e-12
    assert abs(float(val) - want) <= tol * max(1.0, abs(want))


def test_adjust_n_matches_reference_rules():
    assert OG.adjust_N(OG.SIMPSON, 3, 1076890) == 101**3
    assert OG.adjust_N(OG.BOOLE, 3, 1000) == 9**3
    assert OG.adjust_N(OG.SIMPSON, 2, 4) == 9
    assert OG.adjust_N(OG.BOOLE, 1, 4) == 5


def test_oracle_gradients_match_reference_autograd():
    """The numpy gradient of the discrete rules (oracle/grad.py) against the
    reference's torch autograd recorded in the golden fixtures (fp64
    cases)."""
    from oracle import grad as OGR

    fams = {"ExpSum": 1, "GaussianPeak": 2, "Oscillatory": 3, "SumSin": 4}
    rules = {"Trapezoid": 0, "Simpson": 1, "Boole": 2, "GaussLegendre": 3}
    cases = [c for c in G.load("grid_mc_golden.json")["grads"] if c["dtype"] == "float64"]
    assert len(cases) >= 4
    for c in cases:
        d = c["dim"]
        p = c["params"]
        a = np.broadcast_to(np.asarray(p["a"], dtype=np.float64), (d,))
        u = np.broadcast_to(np.asarray(p.get("u", 0.0), dtype=np.float64), (d,))
        params = np.concatenate([[p.get("c", 1.0), p.get("b", 0.0)], a, u])
        n = int(round(c["N"] ** (1.0 / d)))
        I, gdom, gpar = OGR.value_and_grad(fams[c["family"]], params, rules[c["rule"]], d, n, c["domain"])
        want = G.f(c["value"])
        assert abs(I - want) <= 1e-12 * max(1.0, abs(want)), c["name"]
        assert np.allclose(gdom.ravel(), G.arr(c["grad_domain"]), rtol=1e-10, atol=1e-12), c["name"]
        names = {"c": [0], "b": [1], "a": list(range(2, 2 + d)), "u": list(range(2 + d, 2 + 2 * d))}
        for k, hs in c["grads"].items():
            assert np.allclose(gpar[names[k]], G.arr(hs), rtol=1e-10, atol=1e-12), (c["name"], k)
