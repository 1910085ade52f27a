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

F64 = torch.float64
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
        B.BatchedGrid().integrate([tq.ExpSum(1), lambda x: x[:, 0]], ["simpson"] * 2, [101, 101], [[[0, 1]]] * 2)
    with pytest.raises(ValueError):
        B.BatchedGrid().integrate([tq.ExpSum(1)], ["simpson"], [101], [[[1, 0]]])


def _mixed_batch(n, seed, max_dim=5):
    """Integrals of all four families, all rules, dims 1..max_dim."""
    rng = np.random.default_rng(seed)
    rules = ["trapezoid", "simpson", "boole", "gausslegendre"]
    fs, rs, Ns, doms = [], [], [], []
    for i in range(n):
        d = int(rng.integers(1, max_dim + 1))
        a = rng.uniform(-2.0, 2.0, d).tolist()
        kind = i % 4
        if kind == 0:
            f = tq.ExpSum(d, a=a, b=float(rng.uniform(-0.5, 0.5)), c=float(rng.uniform(0.5, 2)))
        elif kind == 1:
            f = tq.GaussianPeak(d, a=np.abs(a).tolist(), u=rng.uniform(0, 1, d).tolist(), c=float(rng.uniform(0.5, 2)))
        elif kind == 2:
            f = tq.Oscillatory(d, a=a, b=float(rng.uniform(0, 1)), c=float(rng.uniform(0.5, 2)))
        else:
            f = tq.SumSin(d, a=a, c=float(rng.uniform(0.5, 2)))
        lo = rng.uniform(-1.0, 0.0, d)
        doms.append(np.stack([lo, lo + rng.uniform(0.5, 2.0, d)], axis=1).tolist())
        fs.append(f)
        rs.append(rules[int(rng.integers(0, 4))])
        N = int(10 ** rng.uniform(2, 4.5))
        Ns.append(min(N, 128**d) if rs[-1] == "gausslegendre" else N)
    return fs, rs, Ns, doms


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_mixed_family_batch_is_one_launch(dtype, cuda):
    """Families mixed in one batch: one tq_batch_grid launch (each
    descriptor names its family), and every value equals the per-call form
    and the closed-form integral."""
    from torchquad_gb300 import _lib as L

    fs, rs, Ns, doms = _mixed_batch(160, 3)
    bg = B.BatchedGrid(dtype=dtype, autotune=False)
    plan = bg.plan(fs, rs, Ns, doms)
    assert plan.family == L.TQ_FN_PER_DESC
    n0 = L.launches[0]
    vals = bg.run(plan).cpu()
    assert L.launches[0] - n0 == 2  # the batch and its finalize
    cls = {"trapezoid": tq.Trapezoid, "simpson": tq.Simpson, "boole": tq.Boole, "gausslegendre": tq.GaussLegendre}
    tol = 1e-12 if dtype == torch.float64 else 2e-6
    for i in range(0, 160, 3):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ref = cls[rs[i]]().integrate(fs[i], fs[i].dim, N=Ns[i],
                                         integration_domain=torch.tensor(doms[i], dtype=dtype, device=cuda)).item()
        assert abs(vals[i].item() - ref) <= tol * max(1.0, abs(ref)), (i, rs[i], vals[i].item(), ref)
    # the same integrals split by family give the same values
    for fam in (tq.ExpSum, tq.GaussianPeak, tq.Oscillatory, tq.SumSin):
        idx = [i for i, f in enumerate(fs) if isinstance(f, fam)]
        sub = bg.integrate([fs[i] for i in idx], [rs[i] for i in idx], [Ns[i] for i in idx],
                           [doms[i] for i in idx]).cpu()
        assert torch.allclose(sub.double(), vals[idx].double(), rtol=tol, atol=1e-12)


def test_batched_adjoint_c4_1024(cuda):
    """1024 differentiation integrals (Gauss-Legendre, dim 4, 32 nodes per
    dimension, fp64, c cos(2 pi u + a.x), u and the domain bounds requiring
    gradients) in one batched adjoint launch: value and every gradient equal
    the per-call adjoint (tq_grid_adjoint behind GaussLegendre.integrate +
    backward) to 1e-12, and the reference's recorded autograd for the
    differentiation case."""
    rng = np.random.default_rng(4)
    m = 1024
    a = rng.uniform(-3.0, 3.0, (m, 4))
    u = torch.tensor(rng.uniform(0.0, 1.0, m), dtype=F64, requires_grad=True)
    golden = [c for c in G.load("grid_mc_golden.json")["grads"] if c["name"] == "C4-GaussLegendre-osc4-32"][0]
    a[0] = golden["params"]["a"]
    with torch.no_grad():
        u[0] = golden["params"]["b"]
    doms = torch.tensor([[[0.0, 1.0]] * 4] * m, dtype=F64, requires_grad=True)
    fs = [tq.Oscillatory(4, a=a[i].tolist(), b=u[i]) for i in range(m)]
    bg = B.BatchedGrid(dtype=F64)
    vals = bg.integrate(fs, ["gausslegendre"] * m, [32**4] * m, list(doms))
    assert vals.shape == (m,) and vals.requires_grad
    w = torch.tensor(rng.uniform(0.5, 2.0, m), dtype=F64)
    (vals.cpu() * w).sum().backward()
    g_u, g_dom = u.grad.clone(), doms.grad.clone()
    # the reference's autograd of the differentiation case (integral 0)
    assert abs(vals[0].item() - G.f(golden["value"])) <= 1e-12 * abs(G.f(golden["value"]))
    assert np.allclose(g_dom[0].numpy().ravel() / w[0].item(), G.arr(golden["grad_domain"]), rtol=1e-10, atol=1e-12)
    assert abs(g_u[0].item() / w[0].item() - G.arr(golden["grads"]["b"])[0]) <= 1e-10
    # every integral against the per-call adjoint
    for i in range(m):
        ui = torch.tensor(u[i].item(), dtype=F64, device=cuda, requires_grad=True)
        di = torch.tensor([[0.0, 1.0]] * 4, dtype=F64, device=cuda, requires_grad=True)
        vi = tq.GaussLegendre().integrate(tq.Oscillatory(4, a=a[i].tolist(), b=ui), 4, N=32**4, integration_domain=di)
        vi.backward()
        assert abs(vals[i].item() - vi.item()) <= 1e-12 * max(1.0, abs(vi.item())), i
        assert abs(g_u[i].item() - w[i].item() * ui.grad.item()) <= 1e-12 * max(1.0, abs(g_u[i].item())), i
        assert torch.allclose(g_dom[i], w[i] * di.grad.cpu(), rtol=1e-12, atol=1e-13), i


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batched_adjoint_mixed_matches_per_call(dtype, cuda):
    """Gradients of a batch mixing families, rules and dims (1..5, so the
    wider accumulator set) against the per-call adjoint of each integral."""
    fs0, rs, Ns, doms0 = _mixed_batch(48, 7)
    fs, params, doms = [], [], []
    for f in fs0:
        p = {"a": f.a.clone().requires_grad_(True), "c": f.c.clone().requires_grad_(True)}
        if isinstance(f, tq.GaussianPeak):
            g = tq.GaussianPeak(f.dim, a=p["a"], u=f.u.clone().requires_grad_(True), c=p["c"])
            p["u"] = g.u
        elif isinstance(f, tq.SumSin):
            g = tq.SumSin(f.dim, a=p["a"], c=p["c"])
        else:
            p["b"] = f.b.clone().requires_grad_(True)
            g = type(f)(f.dim, a=p["a"], b=p["b"], c=p["c"])
        fs.append(g)
        params.append(p)
    doms = [torch.tensor(d, dtype=dtype, requires_grad=True) for d in doms0]
    vals = B.BatchedGrid(dtype=dtype).integrate(fs, rs, Ns, doms)
    vals.sum().backward()
    cls = {"trapezoid": tq.Trapezoid, "simpson": tq.Simpson, "boole": tq.Boole, "gausslegendre": tq.GaussLegendre}
    tol = 1e-11 if dtype == torch.float64 else 2e-5
    for i, f in enumerate(fs):
        p2 = {k: v.detach().to(cuda).requires_grad_(True) for k, v in params[i].items()}
        kw = {k: v for k, v in p2.items()}
        g = type(f)(f.dim, **kw)
        d2 = doms[i].detach().to(cuda).requires_grad_(True)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            v = cls[rs[i]]().integrate(g, f.dim, N=Ns[i], integration_domain=d2)
        v.backward()
        scale = max(1.0, abs(v.item()))
        assert abs(vals[i].item() - v.item()) <= tol * scale, (i, rs[i], vals[i].item(), v.item())
        assert torch.allclose(doms[i].grad.double(), d2.grad.double().cpu(), rtol=tol, atol=tol * scale), i
        for k in p2:
            assert torch.allclose(params[i][k].grad.double(), p2[k].grad.double().cpu(), rtol=tol,
                                  atol=tol * scale), (i, k)
