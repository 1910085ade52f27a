"""VEGAS (VEGAS+ / "VEGAS Enhanced", reference: integration/vegas.py:13-362).

Two drivers with the reference's algorithm and defaults:

* fused — built-in integrand and this package's counter-based RNG: every
  warm-up step and iteration is one sampling kernel (Philox draws,
  stratified points, map transform, integrand, histograms and cube sums in
  registers/shared memory) plus the small get_NH / finish / map-update
  kernels.  The every-fifth-iteration abort test (vegas.py:161-209), the
  only place the reference's control flow depends on results, runs on the
  device too, so a whole integration is one CUDA graph launch (a WHILE node
  over blocks of five iterations) and one read-back.
* materialised — any torch integrand or any ``rng`` object: points are
  written to memory, the integrand runs on them, and the same kernels do the
  map transform, histograms, cube sums and updates.
"""
from __future__ import annotations

import ctypes
import math
import warnings
import weakref

import numpy as np
import torch

from .. import _lib as L
from ..integrands import BuiltinIntegrand
from .base_integrator import BaseIntegrator
from .rng import RNG
from .utils import _host_domain_values, _setup_integration_domain
from ._vegas_state import VegasDevice, n_strat_for
from .vegas_map import VEGASMap
from .vegas_stratification import VEGASStratification

ALPHA = 0.5  # vegas.py:220
BETA = 0.75  # vegas_stratification.py:13


class _FusedPlan:
    """Device state plus one captured CUDA graph for a fused VEGAS shape.

    A whole integration is one graph: the warm-up (state reset and five
    warm-up sampling/map-update pairs), then a WHILE conditional node whose
    body is a block of five stratified iterations (get_NH, fused sampling,
    finish and map update) followed by the device-side abort test, which
    ends the loop (vegas.py:141-209).  Every changing input sits in the
    state's control block (written by begin_run), so the graph is captured
    once and launched for every call with the same shape, and the host reads
    the results back once per call.  The first use runs the same launches
    eagerly, with the loop on the host."""

    _cache = {}  # shape key -> [plans]
    _MAX = 8  # shape keys kept
    _PER_KEY = 4  # plans per shape key (integrators of one shape alive at once)

    def __init__(self, dev, family, use_grid_improve, use_warmup, ns, n_inc):
        self.dev, self.family = dev, family
        self.use_grid_improve, self.use_warmup, self.ns = use_grid_improve, use_warmup, ns
        self.points_hint = dev.points_hint(n_inc)
        self.uses = 0
        self.graph = None
        self.owner = None  # weak reference to the VEGAS whose results the state holds
        self._side = torch.cuda.Stream(device=dev.device)
        self._fork, self._join = torch.cuda.Event(), torch.cuda.Event()

    @classmethod
    def get(cls, make_dev, shape_key, family, use_grid_improve, use_warmup, ns, n_inc, max_iterations, requester):
        """A plan of this shape for `requester`: its own from an earlier call,
        else one no live integrator holds, else a new one (up to _PER_KEY);
        when all are held, the least recently used one, whose integrator
        first gets a private copy of its state."""
        key = (*shape_key, family, bool(use_grid_improve), bool(use_warmup), ns, n_inc, max_iterations)
        plans = cls._cache.get(key)
        if plans is None:
            if len(cls._cache) >= cls._MAX:
                cls._cache.pop(next(iter(cls._cache)))
            plans = cls._cache[key] = []
        free = None
        for p in plans:
            owner = p.owner() if p.owner is not None else None
            if owner is requester:
                return p
            if owner is None and free is None:
                free = p
        if free is not None:
            return free
        if len(plans) < cls._PER_KEY:
            p = cls(make_dev(), family, use_grid_improve, use_warmup, ns, n_inc)
            plans.append(p)
            return p
        p = plans.pop(0)  # least recently handed out
        plans.append(p)
        owner = p.owner() if p.owner is not None else None
        if owner is not None and owner._dev is p.dev:
            owner._detach_state()
        return p

    # launch sequences
    def _warm_seq(self):
        d = self.dev
        d.reinit()
        if self.use_warmup:
            for _ in range(5):
                if self.ns > 0:
                    d.warmup_fused(self.family, d.params, self.ns)
                d.update_map(ALPHA)

    def _block_seq(self):
        # The map update of an iteration gates only the next sampling
        # launch, while get_NH needs only the end of the iteration: the map
        # update runs on a side stream, beside finish and the next get_NH.
        d = self.dev
        main = torch.cuda.current_stream()
        side, fork, join = self._side, self._fork, self._join
        for i in range(5):
            d.get_nh_split()
            if i > 0 and self.use_grid_improve:
                main.wait_event(join)
            d.iterate_fused(self.family, d.params, self.use_grid_improve, self.points_hint)
            if self.use_grid_improve:
                fork.record(main)
                with torch.cuda.stream(side):
                    side.wait_event(fork)
                    d.update_map(ALPHA)
                    join.record(side)
            d.finish(BETA)
        if self.use_grid_improve:
            main.wait_event(join)

    def _warm_launches(self):
        per = (1 if self.ns > 0 else 0) + self.dev.update_map_launches
        return 1 + (5 * per if self.use_warmup else 0)

    def _block_launches(self):  # five iterations and the abort test
        return 5 * (3 + (self.dev.update_map_launches if self.use_grid_improve else 0)) + 1

    def _capture(self):
        """Records warm-up + WHILE(block, abort test) without running it."""
        g = torch.cuda.CUDAGraph()
        h = ctypes.c_uint64(0)
        with torch.cuda.graph(g):
            body = L.body_stream(self.dev.device)
            if self._side.cuda_stream in (L.stream_handle(), body.cuda_stream):
                # the map-update stream must be neither capturing stream
                self._side = L.body_stream(self.dev.device, avoid=(body,))
            self._warm_seq()
            L.check(L.lib().tq_capture_while_begin(L.stream_handle(), body.cuda_stream, ctypes.byref(h)),
                    "tq_capture_while_begin")
            try:
                with torch.cuda.stream(body):
                    self._block_seq()
                    self.dev.abort_test(h.value)
            finally:
                L.check(L.lib().tq_capture_while_end(body.cuda_stream), "tq_capture_while_end")
        return g

    def run(self):
        """Warm-up, then blocks until the abort test stops; the results are
        left in the state's host copy (dev.host_*)."""
        self.uses += 1
        d = self.dev
        if self.graph is None and self.uses > 1 and _graphs_enabled():
            torch.cuda.synchronize()
            self.graph = self._capture()
        if self.graph is not None and not FORCE_EAGER[0]:
            self.graph.replay()
            d.read_back()
            L.count_launches(self._warm_launches()
                             + int(d.host_control[L.VC_IT]) // 5 * self._block_launches())
            return
        self._warm_seq()
        while True:
            self._block_seq()
            d.abort_test(0)
            d.read_back()
            if d.host_control[L.VC_STOP]:
                return


def _sum_lr(xs, zero=0.0):
    t = zero
    for x in xs:
        t = t + x
    return t


# Set [True] to run the captured sequences as individual launches (for
# per-kernel instrumentation); graphs stay captured.
FORCE_EAGER = [False]


def _graphs_enabled():
    import os

    return os.environ.get("TORCHQUAD_GB300_CUDA_GRAPHS", "1") != "0"


class VEGAS(BaseIntegrator):
    """VEGAS Enhanced (arXiv:2009.05112) with adaptive map and stratification."""

    def __init__(self):
        super().__init__()

    def integrate(self, fn, dim, N=10000, integration_domain=None, seed=None, rng=None,
                  use_grid_improve=True, eps_rel=0, eps_abs=0, max_iterations=20,
                  use_warmup=True, backend=None, n_intervals=None):
        """Integrate fn with VEGAS+ using about N evaluations.

        Arguments as the reference's VEGAS.integrate; ``n_intervals``
        (extension, default None) overrides the number of map intervals per
        dimension, which the reference fixes to max(2, N_increment // 10)."""
        self._check_inputs(dim=dim, N=N, integration_domain=integration_domain)
        self._dim = dim
        self._nr_of_fevals = 0
        self._max_iterations = max_iterations
        self._eps_rel = eps_rel
        self._eps_abs = eps_abs
        self.use_grid_improve = use_grid_improve
        self.N = N
        self._starting_N = N // (self._max_iterations + 5)
        self._N_increment = N // (self._max_iterations + 5)
        self._fn = fn
        # a domain given as host values goes to the fused kernels as launch
        # arguments; a tensor domain is used where it lives
        domain_values = _host_domain_values(dim, integration_domain, backend)
        if domain_values is not None:
            domain = None
            device = L.require_cuda()
            self.dtype = torch.get_default_dtype()
        else:
            domain = _setup_integration_domain(dim, integration_domain, backend)
            device = domain.device
            self.dtype = domain.dtype
        self.backend = "torch"
        if self.dtype not in (torch.float32, torch.float64):
            raise ValueError(f"unsupported domain dtype {self.dtype}")
        if rng is None:
            rng = RNG(backend="torch", seed=seed)
        elif seed is not None:
            raise ValueError("seed and rng cannot both be passed")
        self.rng = rng

        N_intervals = n_intervals if n_intervals is not None else max(2, self._N_increment // 10)
        n_strat = n_strat_for(self._N_increment, dim)
        self.results = []
        self.sigma2 = []
        self.it = 0

        fused = (
            isinstance(fn, BuiltinIntegrand)
            and type(rng) is RNG
            and fn.dim == dim
            and not (torch.is_grad_enabled()
                     and ((domain is not None and domain.requires_grad) or fn.requires_grad()))
        )
        if fused:
            ns = self._starting_N // 5 if use_warmup else 0
            plan = _FusedPlan.get(
                lambda: VegasDevice(dim, self.dtype, N_intervals, n_strat, device, domain,
                                    stats_slots=max_iterations + 10),
                (str(device), torch.cuda.current_stream().cuda_stream, dim, self.dtype,
                 N_intervals, n_strat), fn.family,
                use_grid_improve, use_warmup, ns, self._N_increment, max_iterations, self)
            self._dev = plan.dev
        else:
            if domain is None:
                domain = torch.tensor(domain_values, dtype=self.dtype).to(device)
            plan = None
            self._dev = VegasDevice(dim, self.dtype, N_intervals, n_strat, device, domain,
                                    stats_slots=max(8, max_iterations + 10))
        self.map = VEGASMap(N_intervals, dim, None, self.dtype, _device_state=self._dev)
        self.strat = VEGASStratification(self._N_increment, dim, rng, None, self.dtype,
                                         _device_state=self._dev)
        if fused:
            return self._integrate_fused(plan, fn, domain, domain_values, use_warmup)

        domain_starts = domain[:, 0]
        domain_sizes = domain[:, 1] - domain_starts
        domain_volume = torch.prod(domain_sizes)

        def transformed_integrand(x):
            return fn(x * domain_sizes + domain_starts) * domain_volume

        self._fn = transformed_integrand
        return self._integrate_materialised(domain, use_warmup)

    # ------------------------------------------------------------ fused
    def _integrate_fused(self, plan, fn, domain, domain_values, use_warmup):
        """The whole run on the device (warm-up, blocks of five iterations,
        the abort test after each block); one read-back at the end gives the
        host the reference's attributes (it, results, sigma2, evaluations,
        _starting_N) and the RNG offset."""
        rng = self.rng
        dev = plan.dev
        # The plan's device state now holds this integrator's map and
        # stratification (as the reference's instances own theirs); no other
        # live integrator is handed this plan while this one holds it.
        plan.owner = weakref.ref(self)
        if domain_values is None:
            dev.set_domain(domain)
        warm_evals = 5 * plan.ns if use_warmup else 0
        dev.dh_pending = False
        run_args = (self._starting_N, self.N, self._N_increment, self._max_iterations, warm_evals,
                    self._eps_rel, self._eps_abs, rng.seed, rng.stream_id, rng.offset, fn.params_numpy(),
                    domain_values)
        self.alpha = ALPHA
        dev.begin_run(*run_args)
        plan.run()
        return self._collect_fused(dev, rng)

    def _collect_fused(self, dev, rng):
        """The reference's attributes from the state's host copy after a
        fused run, and the result."""
        c = dev.host_control
        stop = int(c[L.VC_STOP])
        if stop == 4:
            raise RuntimeError("VEGAS ran out of statistics slots")
        if stop == 5:  # int() of an infinite value in the abort test (vegas.py:186-189)
            raise OverflowError("cannot convert float infinity to integer")
        if stop == 6:
            raise ValueError("cannot convert float NaN to integer")
        self.it = it = int(c[L.VC_IT])
        self._starting_N = int(c[L.VC_NEVALS])
        self._nr_of_fevals = int(c[L.VC_EVALS])
        st = dev.host_stats
        self.results = [float(v) for v in st[it - 5 : it, 0]]
        self.sigma2 = [float(v) for v in st[it - 5 : it, 1]]
        self.map.check_flags(dev.host_flags)
        rng.offset = int(dev.host_rng_offset[0])
        # update_DH leaves dh normalised; done on first access
        # (VEGASStratification.dh)
        dev.dh_pending = True
        return torch.full((), float(self._get_result()), dtype=self.dtype, device=dev.device)

    def _detach_state(self):
        """Move this integrator's map and stratification onto a private copy
        of the shared plan state."""
        snap = self._dev.clone_state()
        self._dev = snap
        self.map._dev = snap
        self.strat._dev = snap

    # ----------------------------------------------------- materialised
    def _integrate_materialised(self, domain, use_warmup):
        if use_warmup:
            self._warmup_grid(5, self._starting_N // 5)
        while True:
            self.it = self.it + 1
            self.results.append(0)
            self.sigma2.append(0)
            self._run_iteration()
            if self._check_abort_conditions():
                break
        res = self._get_result()
        if isinstance(res, torch.Tensor):  # differentiable (see _run_iteration)
            return res.to(self.dtype)
        return torch.tensor(res, dtype=self.dtype, device=domain.device)

    def _warmup_grid(self, warmup_N_it=5, N_samples=1000):
        """Warm up the map: warmup_N_it rounds of N_samples uniform points
        (vegas.py:211-266)."""
        self.alpha = ALPHA
        for _ in range(warmup_N_it):
            yrnd = self.rng.uniform(size=[N_samples, self._dim], dtype=self.dtype)
            yrnd = torch.as_tensor(yrnd).to(self._dev.device, self.dtype) * 0.999999
            x, jac = self.map.get_X_and_Jac(yrnd)
            f_eval = self._eval(x).squeeze()
            jf_vec = f_eval * jac
            jf_vec2 = (jf_vec**2).detach()
            if N_samples > 0:
                self.map.accumulate_weight(yrnd, jf_vec2)
            self.map.update_map()

    def _run_iteration(self):
        """One stratified iteration (vegas.py:268-315)."""
        neval = self.strat.get_NH(self._starting_N)
        y = self.strat.get_Y(neval)
        x, jac = self.map.get_X_and_Jac(y)
        f_eval = self._eval(x).squeeze()
        jf_vec = f_eval * jac
        jf_vec2 = (jf_vec**2).detach()
        if self.use_grid_improve:
            self.map.accumulate_weight(y, jf_vec2)
        self.strat.accumulate_weight(neval, jf_vec)
        slot = self.it - 1
        self.strat.update_DH(slot)  # also the per-iteration result and variance
        if self.use_grid_improve:
            self.map.update_map()
        st = self._dev.stats[slot].cpu()
        res = float(st[0])
        if torch.is_grad_enabled() and jf_vec.requires_grad:
            # The iteration estimate sum_c JF_c V / n_c = sum_i jf_i V / n_c(i)
            # (vegas.py:293-302) as a torch expression for the gradient; its
            # value stays the kernel's compensated fp64 sum.
            w = torch.repeat_interleave(self.strat.V_cubes / neval.to(torch.float64), neval)
            r_t = (jf_vec.to(torch.float64) * w).sum()
            res = res + (r_t - r_t.detach())
        self.results[-1] = res
        self.sigma2[-1] = float(st[1])
        acc = math.sqrt(self.sigma2[-1])
        if float(self.results[-1]) != 0.0:
            acc = acc / abs(float(self.results[-1]))
        return acc

    # ------------------------------------------------- shared host logic
    # The reference keeps results and variances as 0-d tensors of the
    # state's dtype, so the abort test (vegas.py:161-209) and the estimate
    # (:318-362) are computed in that dtype: here as numpy scalars of it
    # (np.float32 / np.float64, every operation rounded once), with Python
    # scalar operands rounded to the dtype first, as torch does.  Sums run
    # left to right from zero, as the reference's sums of tensors do (Python's
    # builtin sum of floats is compensated since 3.12).  x / 0 gives inf or
    # NaN, as tensors do.  tq_vegas_abort_test does the same on the device.
    def _scalar(self):
        return np.float32 if self.dtype == torch.float32 else np.float64

    def _differentiable(self):
        return any(isinstance(r, torch.Tensor) for r in self.results)

    def _check_abort_conditions(self):
        """Every fifth iteration: stop on accuracy, adapt the evaluations per
        iteration, stop on budget/iterations (vegas.py:161-209)."""
        if self.it % 5 > 0:
            return False
        S = self._scalar()
        with np.errstate(all="ignore"):
            res_abs = abs(S(float(self._get_result())))
            err = S(self._get_error())
            chi2 = S(self._get_chisq())
            q = chi2 / S(5.0)
            if (err <= S(self._eps_rel) * res_abs or err <= S(self._eps_abs)) and q < 1.0:
                return True
            if q < 1.0:
                if res_abs == 0.0:
                    self._starting_N += self._N_increment
                else:
                    acc = err / res_abs
                    x = S(self._starting_N) * np.sqrt(acc / S(self._eps_rel + 1e-8))
                    # int() of an infinite / NaN value raises, as in the reference
                    self._starting_N = min(self._starting_N + self._N_increment, int(x))
            elif q > 1.0:
                self._starting_N += self._N_increment
        if self._nr_of_fevals + self._starting_N * 5 > self.N:
            return True
        if self.it + 5 > self._max_iterations:
            return True
        self.results = []
        self.sigma2 = []
        return False

    def _get_result(self):
        """Inverse-variance weighted mean of the iteration results (EQ 30)."""
        if self._differentiable():  # torch expressions carry the gradient
            if any(s == 0.0 for s in self.sigma2):
                return _sum_lr(self.results) / len(self.results)
            num = _sum_lr(r / s for r, s in zip(self.results, self.sigma2))
            den = _sum_lr(1.0 / s for s in self.sigma2)
            return num / den
        S = self._scalar()
        rs = [S(float(r)) for r in self.results]
        ss = [S(float(s)) for s in self.sigma2]
        with np.errstate(all="ignore"):
            if any(s == 0.0 for s in ss):
                return _sum_lr(rs, S(0)) / S(len(rs))
            num = _sum_lr((r / s for r, s in zip(rs, ss)), S(0))
            den = _sum_lr((S(1) / s for s in ss), S(0))
            return num / den

    def _get_error(self):
        """Error estimate from the variances (EQ 31)."""
        S = self._scalar()
        ss = [S(float(s)) for s in self.sigma2]
        with np.errstate(all="ignore"):
            res = _sum_lr((S(1) / s for s in ss if s != 0.0), S(0))
            return ss[0] if res == 0 else S(1) / np.sqrt(res)

    def _get_chisq(self):
        """Chi square of the iteration results (EQ 32)."""
        S = self._scalar()
        I_final = S(float(self._get_result()))
        rs = [S(float(r)) for r in self.results]
        ss = [S(float(s)) for s in self.sigma2]
        chi2 = S(0)
        with np.errstate(all="ignore"):
            for r, s in zip(rs, ss):
                if r != I_final:
                    d = r - I_final
                    chi2 = chi2 + (d * d) / s
        return chi2
