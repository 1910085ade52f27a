"""Record golden fixtures from the unmodified reference torchquad.

Run in a container where the reference source is present:

    python tests/golden/make_golden.py /root/reference [--only grid,vegas,c2_steps,abort]

The reference's hard dependencies autoray and loguru are replaced by the
small stand-ins in ``tests/golden/refshim`` (dispatch only, no arithmetic).
The reference runs on torch CPU in this process; uniform draws for Monte
Carlo / VEGAS are injected from the Philox stream of ``oracle.philox`` through
the reference's own ``rng=`` argument.  Outputs (JSON, floats as hex) are
written next to this script and committed; tests read them on any machine.
"""
from __future__ import annotations

import json
import math
import sys
import warnings
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _import_reference(ref_root: str):
    sys.path[:0] = [str(HERE / "refshim"), ref_root, str(REPO)]
    import torchquad  # noqa: F401  (the reference)

    return torchquad


def hexf(x) -> str:
    return float(x).hex()


def hexarr(a):
    import numpy as np

    return [float(v).hex() for v in np.asarray(a, dtype=np.float64).ravel()]


class ReplayRNG:
    """RNG stand-in handed to the reference (``rng=``): draws come from the
    counter-based Philox stream the GB300 build uses, as torch tensors, and
    every draw is recorded."""

    def __init__(self, seed, stream_id=0):
        from oracle.philox import ReplayStream

        self.stream = ReplayStream(seed, stream_id)
        self.log = []

    def uniform(self, size, dtype):
        import numpy as np
        import torch

        nd = np.float32 if dtype == torch.float32 else np.float64
        a = self.stream.uniform(list(size), nd)
        self.log.append(a)
        return torch.from_numpy(a.copy())


def grid_cases():
    """(name, rule class, dim, N, family spec, domain, dtype)."""
    cases = []
    fams = [
        ("expsum1", 1, dict(kind="ExpSum", a=[1.0], b=0.0), [[-2.0, 1.0]], 101),
        ("expsum3", 3, dict(kind="ExpSum", a=[1.0, 1.0, 1.0], b=0.0), [[0.0, 1.0]] * 3, 21**3),
        ("gauss2", 2, dict(kind="GaussianPeak", a=[2.0, 3.0], u=[0.3, 0.6], c=1.5), [[-1.0, 1.0], [0.0, 2.0]], 33**2),
        ("osc4", 4, dict(kind="Oscillatory", a=[1.0, -2.0, 0.5, 1.5], b=0.3), [[0.0, 1.0]] * 4, 9**4),
        ("sumsin5", 5, dict(kind="SumSin", a=[1.0] * 5), [[0.0, 1.0]] * 5, 5**5),
        ("adjust3", 3, dict(kind="ExpSum", a=[0.5, -1.0, 2.0], b=0.25), [[0.0, 1.0], [-1.0, 0.5], [0.2, 0.4]], 1000),
    ]
    for rule in ["Trapezoid", "Simpson", "Boole", "GaussLegendre"]:
        for dtype in ["float32", "float64"]:
            for name, dim, fam, dom, N in fams:
                cases.append((f"{rule}-{name}-{dtype}", rule, dim, N, fam, dom, dtype))
    cases.append(("C1-Simpson-expsum3-101", "Simpson", 3, 1030301,
                  dict(kind="ExpSum", a=[1.0] * 3, b=0.0), [[0.0, 1.0]] * 3, "float64"))
    cases.append(("C4-GaussLegendre-osc4-32", "GaussLegendre", 4, 32**4,
                  dict(kind="Oscillatory", a=[1.2, -2.1, 0.7, 2.6], b=0.37), [[0.0, 1.0]] * 4, "float64"))
    cases.append(("Simpson-N1076890-expsum3", "Simpson", 3, 1076890,
                  dict(kind="ExpSum", a=[1.0] * 3, b=0.0), [[0.0, 1.0]] * 3, "float64"))
    return cases


def make_integrand(spec, dim):
    import torchquad_gb300.integrands as I

    kw = {k: v for k, v in spec.items() if k != "kind"}
    return getattr(I, spec["kind"])(dim, **kw)


def gen_grid(tq):
    import torch

    out = []
    for name, rule, dim, N, fam, dom, dtype in grid_cases():
        dt = getattr(torch, dtype)
        f = make_integrand(fam, dim)
        domain = torch.tensor(dom, dtype=dt)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            integ = getattr(tq, rule)()
            val = integ.integrate(f, dim, N=N, integration_domain=domain)
        out.append(dict(name=name, rule=rule, dim=dim, N=N, family=fam, domain=dom, dtype=dtype,
                        value=hexf(val.item()), result_dtype=str(val.dtype).replace("torch.", ""),
                        n_per_dim=int(integ._nr_of_fevals ** (1.0 / dim) + 0.5),
                        fevals=int(integ._nr_of_fevals),
                        params=hexarr(f.params_vector().numpy())))
    return out


def gen_multidim(tq):
    """Vector-valued and complex integrands on the materialised path."""
    import torch

    out = []
    dom = [[0.0, 1.0], [-1.0, 2.0]]
    for rule in ["Trapezoid", "Simpson", "Boole", "GaussLegendre"]:
        domain = torch.tensor(dom, dtype=torch.float64)

        def vec(x):
            base = torch.exp(0.3 * x[:, 0] - 0.2 * x[:, 1])
            scale = torch.arange(6, dtype=x.dtype).reshape(2, 3) + 1.0
            return base[:, None, None] * scale[None] + x[:, 0:1, None] * x[:, 1:2, None]

        def cplx(x):
            return torch.exp(1j * (x[:, 0] + 0.5 * x[:, 1]))

        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            v = getattr(tq, rule)().integrate(vec, 2, N=17**2, integration_domain=domain)
            c = getattr(tq, rule)().integrate(cplx, 2, N=17**2, integration_domain=domain)
        out.append(dict(rule=rule, domain=dom, N=17**2, vec=hexarr(v.numpy()), vec_shape=list(v.shape),
                        cplx=[hexf(c.real.item()), hexf(c.imag.item())]))
    return out


def gen_linspace():
    import numpy as np
    import torch

    rng = np.random.default_rng(7)
    out = []
    for i in range(24):
        dt = torch.float32 if i % 2 == 0 else torch.float64
        n = int(rng.integers(2, 400))
        a = float(rng.uniform(-3, 1))
        b = a + float(rng.uniform(0.1, 5))
        x = torch.linspace(torch.tensor(a, dtype=dt), torch.tensor(b, dtype=dt), n, dtype=dt)
        out.append(dict(a=hexf(torch.tensor(a, dtype=dt).item()), b=hexf(torch.tensor(b, dtype=dt).item()),
                        n=n, dtype=str(dt).replace("torch.", ""), values=hexarr(x.numpy())))
    return out


def gen_mc(tq):
    import torch

    out = []
    cases = [
        (1, 1000, [[-2.0, 1.0]], dict(kind="ExpSum", a=[1.0], b=0.0), 0),
        (3, 100000, [[0.0, 1.0]] * 3, dict(kind="ExpSum", a=[1.0] * 3, b=0.0), 1),
        (4, 50000, [[0.0, 1.0], [-1.0, 1.0], [0.5, 2.0], [0.0, 3.0]],
         dict(kind="GaussianPeak", a=[1.0, 2.0, 0.5, 3.0], u=[0.5, 0.1, 1.0, 2.0], c=2.0), 2),
        (6, 20000, [[0.0, 1.0]] * 6, dict(kind="Oscillatory", a=[1.0] * 6, b=0.1), 3),
    ]
    for dim, N, dom, fam, seed in cases:
        for dtype in ["float32", "float64"]:
            dt = getattr(torch, dtype)
            rng = ReplayRNG(seed)
            f = make_integrand(fam, dim)
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                val = tq.MonteCarlo().integrate(f, dim, N=N, integration_domain=torch.tensor(dom, dtype=dt), rng=rng)
            out.append(dict(dim=dim, N=N, domain=dom, family=fam, seed=seed, dtype=dtype,
                            value=hexf(val.item()), params=hexarr(f.params_vector().numpy()),
                            first_uniforms=hexarr(rng.log[0].ravel()[:16])))
    return out


def _vegas_spec():
    return dict(kind="GaussianPeak", a=[5.0, 8.0, 3.0], u=[0.3, 0.5, 0.7], c=1.0)


def gen_vegas_steps(tq):
    """Reference VEGAS state before/after stratified iterations, on the
    Philox draws, for step-wise parity (d=3, N=20000)."""
    import torch
    from torchquad.integration import vegas as V

    out = []
    dom = [[0.0, 1.0], [-1.0, 1.0], [0.0, 2.0]]
    for dtype in ["float32", "float64"]:
        dt = getattr(torch, dtype)
        f = make_integrand(_vegas_spec(), 3)
        integ = tq.VEGAS()
        records = []
        orig_run = V.VEGAS._run_iteration

        def run(self):
            pre = dict(x_edges=self.map.x_edges.clone(), dx_edges=self.map.dx_edges.clone(),
                       dh=self.strat.dh.clone(), starting_N=self._starting_N, it=self.it,
                       rng_offset=self.rng.stream.offset)
            snap = {}
            orig_update = self.map.update_map

            def upd():
                snap["counts"] = self.map.counts.clone()
                snap["weights"] = self.map.weights.clone()
                orig_update()

            self.map.update_map = upd
            acc = orig_run(self)
            del self.map.update_map
            rec = dict(pre=pre, counts=snap["counts"], weights=snap["weights"],
                       neval=self.strat.strat_counts.to(torch.int64).clone(), JF=self.strat.JF.clone(),
                       JF2=self.strat.JF2.clone(), result=self.results[-1].item(), sigma2=self.sigma2[-1].item(),
                       x_edges_new=self.map.x_edges.clone(), dh_new=self.strat.dh.clone())
            records.append(rec)
            return acc

        V.VEGAS._run_iteration = run
        try:
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                val = integ.integrate(f, 3, N=20000, integration_domain=torch.tensor(dom, dtype=dt),
                                      rng=ReplayRNG(11))
        finally:
            V.VEGAS._run_iteration = orig_run

        def pack(t):
            return dict(shape=list(t.shape), values=hexarr(t.double().numpy()))

        steps = []
        for i in (0, 1, 5):
            r = records[i]
            steps.append(dict(
                it=r["pre"]["it"] + 1, starting_N=r["pre"]["starting_N"], rng_offset=r["pre"]["rng_offset"],
                x_edges=pack(r["pre"]["x_edges"]), dx_edges=pack(r["pre"]["dx_edges"]), dh=pack(r["pre"]["dh"]),
                neval=[int(v) for v in r["neval"]], counts=[int(v) for v in r["counts"].ravel()],
                weights=pack(r["weights"]), JF=pack(r["JF"]), JF2=pack(r["JF2"]),
                result=hexf(r["result"]), sigma2=hexf(r["sigma2"]),
                x_edges_new=pack(r["x_edges_new"]), dh_new=pack(r["dh_new"])))
        out.append(dict(dtype=dtype, domain=dom, N=20000, seed=11, family=_vegas_spec(),
                        params=hexarr(f.params_vector().numpy()), n_bins=integ.map.N_intervals,
                        n_strat=integ.strat.N_strat, value=hexf(val.item()), fevals=int(integ._nr_of_fevals),
                        iterations=int(integ.it), steps=steps))
    return out


def gen_vegas_c2(tq):
    """Plain VEGAS at full size: dim 6, N = 1e7, 50 map intervals, fp32,
    normal peak sigma 0.05, seed 0, draws from the Philox stream."""
    import torch
    import torchquad_gb300.integrands as I
    from torchquad.integration import vegas as V

    class Map50(V.VEGASMap):
        def __init__(self, N_intervals, dim, backend, dtype, alpha=0.5):
            super().__init__(50, dim, backend, dtype, alpha)

    f = I.GaussianPeak.normal(6, 0.5, 0.05)
    iters = []
    orig_run = V.VEGAS._run_iteration

    def run(self):
        acc = orig_run(self)
        iters.append(dict(M=int(self.strat.strat_counts.sum().item()), result=hexf(self.results[-1].item()),
                          sigma2=hexf(self.sigma2[-1].item())))
        return acc

    V.VEGAS._run_iteration = run
    orig_map = V.VEGASMap
    V.VEGASMap = Map50
    try:
        integ = tq.VEGAS()
        dom = torch.tensor([[0.0, 1.0]] * 6, dtype=torch.float32)
        val = integ.integrate(f, 6, N=10_000_000, integration_domain=dom, rng=ReplayRNG(0))
    finally:
        V.VEGAS._run_iteration = orig_run
        V.VEGASMap = orig_map
    return dict(dim=6, N=10_000_000, n_bins=50, dtype="float32", seed=0, sigma=0.05,
                params=hexarr(f.params_vector().numpy()), value=hexf(val.item()),
                fevals=int(integ._nr_of_fevals), iterations=int(integ.it), iters=iters)


def gen_vegas_c2_steps(tq, out_path):
    """Step-wise reference states of the plain VEGAS run at full size (dim
    6, N = 1e7, 50 map intervals, 6^6 cubes, fp32, normal peak sigma 0.05,
    seed 0, Philox draws): before and after iterations 1, 2, 5 and 10.
    Written as a compressed .npz (arrays in the reference's own dtypes)."""
    import numpy as np
    import torch
    import torchquad_gb300.integrands as I
    from torchquad.integration import vegas as V

    class Map50(V.VEGASMap):
        def __init__(self, N_intervals, dim, backend, dtype, alpha=0.5):
            super().__init__(50, dim, backend, dtype, alpha)

    f = I.GaussianPeak.normal(6, 0.5, 0.05)
    records = []
    orig_run = V.VEGAS._run_iteration

    def run(self):
        pre = dict(x_edges=self.map.x_edges.clone(), dx_edges=self.map.dx_edges.clone(),
                   dh=self.strat.dh.clone(), starting_N=self._starting_N, it=self.it,
                   rng_offset=self.rng.stream.offset)
        snap = {}
        orig_update = self.map.update_map

        def upd():
            snap["counts"] = self.map.counts.clone()
            snap["weights"] = self.map.weights.clone()
            orig_update()

        self.map.update_map = upd
        acc = orig_run(self)
        del self.map.update_map
        records.append(dict(pre=pre, counts=snap["counts"], weights=snap["weights"],
                            neval=self.strat.strat_counts.to(torch.int64).clone(), JF=self.strat.JF.clone(),
                            JF2=self.strat.JF2.clone(), result=self.results[-1].item(),
                            sigma2=self.sigma2[-1].item(), x_edges_new=self.map.x_edges.clone(),
                            dh_new=self.strat.dh.clone()))
        return acc

    V.VEGAS._run_iteration = run
    orig_map = V.VEGASMap
    V.VEGASMap = Map50
    try:
        integ = tq.VEGAS()
        dom = torch.tensor([[0.0, 1.0]] * 6, dtype=torch.float32)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            val = integ.integrate(f, 6, N=10_000_000, integration_domain=dom, rng=ReplayRNG(0))
    finally:
        V.VEGAS._run_iteration = orig_run
        V.VEGASMap = orig_map
    arrays = dict(params=f.params_vector().numpy(), value=np.float32(val.item()),
                  n_strat=np.int64(integ.strat.N_strat), fevals=np.int64(integ._nr_of_fevals),
                  iterations=np.int64(integ.it))
    picks = [0, 1, 4, 9]
    # the reference numbers iterations from 1 and counts self.it up before
    # _run_iteration
    arrays["steps"] = np.array([records[i]["pre"]["it"] for i in picks], dtype=np.int64)
    for i in picks:
        r, p = records[i], f"it{records[i]['pre']['it']}_"
        nxt = records[i + 1]["pre"]["starting_N"] if i + 1 < len(records) else r["pre"]["starting_N"]
        assert int(r["neval"].max()) < 65536
        arrays.update({
            p + "starting_N": np.int64(r["pre"]["starting_N"]),
            p + "next_starting_N": np.int64(nxt),
            p + "rng_offset": np.int64(r["pre"]["rng_offset"]),
            p + "x_edges": r["pre"]["x_edges"].numpy(), p + "dx_edges": r["pre"]["dx_edges"].numpy(),
            p + "dh": r["pre"]["dh"].numpy(),
            p + "neval": r["neval"].numpy().astype(np.uint16),
            p + "counts": r["counts"].numpy().astype(np.int32), p + "weights": r["weights"].numpy(),
            p + "JF": r["JF"].numpy(), p + "JF2": r["JF2"].numpy(),
            p + "result": np.float32(r["result"]), p + "sigma2": np.float32(r["sigma2"]),
            p + "x_edges_new": r["x_edges_new"].numpy(), p + "dh_new": r["dh_new"].numpy(),
        })
    np.savez_compressed(out_path, **arrays)
    return out_path


def gen_vegas_abort(tq):
    """The reference's _check_abort_conditions (vegas.py:161-209) on
    prescribed blocks of five iteration results, with results and variances
    as 0-d tensors of each dtype: the stop decision and the adapted
    _starting_N (or the exception int() raises)."""
    import numpy as np
    import torch

    rng = np.random.default_rng(5)
    cases = []
    for _ in range(60):
        cases.append(dict(r=list(1.0 + 0.01 * rng.standard_normal(5)),
                          s=list(np.abs(1e-4 * rng.standard_normal(5)) + 1e-8),
                          eps_rel=float(rng.choice([0.0, 1e-6, 1e-2, 1.0])),
                          eps_abs=float(rng.choice([0.0, 1e-3])), it=int(rng.choice([5, 10, 15, 20])),
                          sN=int(rng.integers(1000, 100000)), inc=int(rng.integers(1000, 50000)),
                          N=int(rng.choice([10**6, 10**7])), max_it=int(rng.choice([10, 20, 40]))))
    # rounding-sensitive: results within a few fp32 ulps of each other
    for _ in range(24):
        base = float(rng.uniform(0.5, 2.0))
        cases.append(dict(r=list(base * (1.0 + 3e-7 * rng.standard_normal(5))),
                          s=list(np.abs(1e-13 * rng.standard_normal(5)) + 1e-15),
                          eps_rel=float(rng.choice([0.0, 1e-7, 3e-7])), eps_abs=0.0, it=5,
                          sN=int(rng.integers(1000, 10**6)), inc=int(rng.integers(1000, 10**5)),
                          N=10**8, max_it=20))
    base = dict(eps_rel=0.0, eps_abs=0.0, it=5, sN=4000, inc=4000, N=10**6, max_it=20)
    cases += [
        dict(base, r=[1.0] * 5, s=[0.0] * 5),                                      # constant integrand
        dict(base, r=[0.0] * 5, s=[0.0] * 5),                                      # zero integrand
        dict(base, r=[1.0, 2.0, 1.0, 1.0, 1.0], s=[0.0, 1.0, 1.0, 1.0, 1.0]),      # x / 0 in chi2
        dict(base, r=[1.0, 1.1, 0.9, 1.0, 1.05], s=[1e-2] * 5, eps_rel=1.0),       # accuracy
        dict(base, r=[1.0, 5.0, -3.0, 1.0, 2.0], s=[1e-6] * 5),                    # chi2 / 5 > 1
        dict(base, r=[1.0] * 5, s=[1e-4] * 5, N=30000),                            # budget
        dict(base, r=[1.0] * 5, s=[1e-4] * 5, it=20, max_it=20),                   # iteration limit
        dict(base, r=[1e-30, 1.1e-30, 0.9e-30, 1e-30, 1e-30], s=[1e3] * 5),        # err / res overflows fp32
    ]
    out = []
    for dtype in ("float32", "float64"):
        dt = getattr(torch, dtype)
        for c in cases:
            v = tq.VEGAS()
            v.backend, v.dtype = "torch", dt
            v.it = c["it"]
            v.results = [torch.tensor(x, dtype=dt) for x in c["r"]]
            v.sigma2 = [torch.tensor(x, dtype=dt) for x in c["s"]]
            v._eps_rel, v._eps_abs = c["eps_rel"], c["eps_abs"]
            v._starting_N, v._N_increment, v.N = c["sN"], c["inc"], c["N"]
            v._max_iterations = c["max_it"]
            v._nr_of_fevals = 777 + 1000 * c["it"] * (c["it"] + 1) // 2
            try:
                stop = bool(v._check_abort_conditions())
                err = None
            except (OverflowError, ValueError) as e:
                stop, err = None, type(e).__name__
            out.append(dict(c, dtype=dtype, fevals=v._nr_of_fevals if err is None else 777 + 1000 * c["it"] * (c["it"] + 1) // 2,
                            stop=stop, error=err, starting_N=v._starting_N,
                            r=[float(x).hex() for x in c["r"]], s=[float(x).hex() for x in c["s"]]))
    return out


def gen_vegas_special(tq):
    """Zero and constant integrands (reference vegas_test.py:159-184) on
    the Philox draws."""
    import torch

    out = {}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        z = tq.VEGAS().integrate(lambda x: x[:, 0] * 0.0, 2, N=10000,
                                 integration_domain=torch.tensor([[0.0, 3.0]] * 2, dtype=torch.float64),
                                 rng=ReplayRNG(0))
        c = tq.VEGAS().integrate(lambda x: x[:, 0] * 0.0 + 10.0, 2, N=10000,
                                 integration_domain=torch.tensor([[0.0, 3.0]] * 2, dtype=torch.float64),
                                 rng=ReplayRNG(0))
    out["zero"] = hexf(z.item())
    out["constant"] = hexf(c.item())
    return out


def gen_grads(tq):
    """Reference torch autograd of the grid rules w.r.t. the domain and the
    integrand's parameters (the differentiation configuration and more)."""
    import torch
    import torchquad_gb300.integrands as I

    f64 = torch.float64

    def t(v):
        return torch.tensor(v, dtype=f64, requires_grad=True)

    cases = [
        ("C4-GaussLegendre-osc4-32", "GaussLegendre", 4, 32**4, "Oscillatory",
         dict(a=[1.2, -2.1, 0.7, 2.6], b=0.37), ["b"], [[0.0, 1.0]] * 4, "float64"),
        ("Simpson-gauss2", "Simpson", 2, 33**2, "GaussianPeak",
         dict(a=[2.0, 3.0], u=[0.3, 0.6], c=1.5), ["a", "u", "c"], [[-1.0, 1.0], [0.0, 2.0]], "float64"),
        ("Trapezoid-expsum3", "Trapezoid", 3, 21**3, "ExpSum",
         dict(a=[0.5, -1.0, 2.0], b=0.25), ["a", "b"], [[0.0, 1.0], [-1.0, 0.5], [0.2, 0.4]], "float64"),
        ("Boole-sumsin1", "Boole", 1, 101, "SumSin", dict(a=[2.0], c=0.7), ["a", "c"], [[0.0, 2.0]], "float64"),
        ("GaussLegendre-gauss3-f32", "GaussLegendre", 3, 8**3, "GaussianPeak",
         dict(a=[1.0, 2.0, 0.5], u=[0.2, 0.5, 0.9]), ["a", "u"], [[0.0, 1.0]] * 3, "float32"),
    ]
    out = []
    for name, rule, dim, N, kind, kw, grad_params, dom, dtype in cases:
        kw2 = {}
        for k, v in kw.items():
            kw2[k] = t(v) if k in grad_params else v
        f = getattr(I, kind)(dim, **kw2)
        domain = torch.tensor(dom, dtype=getattr(torch, dtype), requires_grad=True)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            val = getattr(tq, rule)().integrate(f, dim, N=N, integration_domain=domain)
        val.backward()
        grads = {k: hexarr(kw2[k].grad.numpy()) for k in grad_params}
        out.append(dict(name=name, rule=rule, dim=dim, N=N, family=kind, params=kw, grad_params=grad_params,
                        domain=dom, dtype=dtype, value=hexf(val.item()), grad_domain=hexarr(domain.grad.numpy()),
                        grads=grads))
    return out


def main():
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("ref_root", nargs="?", default="/root/reference")
    ap.add_argument("--only", default="", help="comma list of parts to regenerate: "
                    "grid, vegas, c2_steps, abort (default: all)")
    args = ap.parse_args()
    only = set(filter(None, args.only.split(",")))
    tq = _import_reference(args.ref_root)
    import torch

    torch.set_num_threads(4)
    if not only or "grid" in only:
        data = {
            "reference_version": tq.__version__,
            "torch": torch.__version__,
            "grid": gen_grid(tq),
            "multidim": gen_multidim(tq),
            "linspace": gen_linspace(),
            "mc": gen_mc(tq),
            "grads": gen_grads(tq),
        }
        with open(HERE / "grid_mc_golden.json", "w") as fh:
            json.dump(data, fh, indent=0)
        print("wrote", HERE / "grid_mc_golden.json", len(data["grid"]), "grid cases")
    vpath = HERE / "vegas_golden.json"
    if not only or "vegas" in only or "abort" in only:
        vdata = json.loads(vpath.read_text()) if vpath.exists() else {}
        vdata["reference_version"] = tq.__version__
        vdata["torch"] = torch.__version__
        if not only or "vegas" in only:
            vdata["steps"] = gen_vegas_steps(tq)
            vdata["special"] = gen_vegas_special(tq)
            vdata["c2"] = gen_vegas_c2(tq)
        if not only or "abort" in only:
            vdata["abort"] = gen_vegas_abort(tq)
        with open(vpath, "w") as fh:
            json.dump(vdata, fh, indent=0)
        print("wrote", vpath)
    if not only or "c2_steps" in only:
        print("wrote", gen_vegas_c2_steps(tq, HERE / "vegas_c2_steps.npz"))


if __name__ == "__main__":
    main()
