"""VEGAS (VEGAS+ / "VEGAS Enhanced", reference: integration/vegas.py:13-362).

Two drivers with the reference's algorithm and defaults:

* fused — built-in integrand and this package's counter-based RNG: every
  warm-up step and iteration is one sampling kernel (Philox draws,
  stratified points, map transform, integrand, histograms and cube sums in
  registers/shared memory) plus the small get_NH / finish / map-update
  kernels.  The host reads results back only at the every-fifth-iteration
  abort test (vegas.py:170), the only place the reference's control flow
  depends on them.
* materialised — any torch integrand or any ``rng`` object: points are
  written to memory, the integrand runs on them, and the same kernels do the
  map transform, histograms, cube sums and updates.
"""
from __future__ import annotations

import math
import warnings

import torch

from .. import _lib as L
from ..integrands import BuiltinIntegrand
from .base_integrator import BaseIntegrator
from .rng import RNG
from .utils import _setup_integration_domain
from ._vegas_state import VegasDevice, n_strat_for
from .vegas_map import VEGASMap
from .vegas_stratification import VEGASStratification

ALPHA = 0.5  # vegas.py:220
BETA = 0.75  # vegas_stratification.py:13


class _FusedPlan:
    """Device state plus captured CUDA graphs for one fused VEGAS shape.

    The warm-up (state reset + five warm-up sampling/map-update pairs) and a
    block of five stratified iterations (get_NH, fused sampling, finish, map
    update) read every changing input from the state's control block, so
    they are captured once and replayed for every later block and call with
    the same shape.  The first use runs the launches eagerly."""

    _cache = {}
    _MAX = 8

    def __init__(self, dev, family, use_grid_improve, use_warmup, ns):
        self.dev, self.family = dev, family
        self.use_grid_improve, self.use_warmup, self.ns = use_grid_improve, use_warmup, ns
        self.uses = 0
        self.g_warm = None
        self.g_block = None

    @classmethod
    def get(cls, make_dev, shape_key, family, use_grid_improve, use_warmup, ns, max_iterations):
        key = (*shape_key, family, bool(use_grid_improve), bool(use_warmup), ns, max_iterations)
        plan = cls._cache.get(key)
        if plan is None:
            plan = cls(make_dev(), family, use_grid_improve, use_warmup, ns)
            if len(cls._cache) >= cls._MAX:
                cls._cache.pop(next(iter(cls._cache)))
            cls._cache[key] = plan
        return plan

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
        d = self.dev
        for _ in range(5):
            d.get_nh()
            d.iterate_fused(self.family, d.params, self.use_grid_improve)
            if self.use_grid_improve:
                d.finish_update_map(BETA, ALPHA)
            else:
                d.finish(BETA)

    def _capture(self, seq):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            seq()
        return g

    def run_warmup(self):
        self.uses += 1
        if self.g_warm is None and self.uses > 1 and _graphs_enabled():
            torch.cuda.synchronize()
            # capture records the launches without running them
            self.g_warm = self._capture(self._warm_seq)
            self.g_block = self._capture(self._block_seq)
        if self.g_warm is not None and not FORCE_EAGER[0]:
            self.g_warm.replay()
            L.count_launches(1 + (5 * ((1 if self.ns > 0 else 0) + self.dev.update_map_launches)
                                  if self.use_warmup else 0))
        else:
            self._warm_seq()

    def run_block(self):
        if self.g_block is not None and not FORCE_EAGER[0]:
            self.g_block.replay()
            L.count_launches(5 * (3 + (self.dev.finish_update_map_launches if self.use_grid_improve else 1)))
        else:
            self._block_seq()


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
        domain = _setup_integration_domain(dim, integration_domain, backend)
        self.backend = "torch"
        self.dtype = domain.dtype
        if self.dtype not in (torch.float32, torch.float64):
            raise ValueError(f"unsupported domain dtype {self.dtype}")
        if rng is None:
            rng = RNG(backend="torch", seed=seed)
        elif seed is not None:
            raise ValueError("seed and rng cannot both be passed")
        self.rng = rng

        domain_starts = domain[:, 0]
        domain_sizes = domain[:, 1] - domain_starts
        domain_volume = torch.prod(domain_sizes)

        def transformed_integrand(x):
            return fn(x * domain_sizes + domain_starts) * domain_volume

        self._fn = transformed_integrand

        N_intervals = n_intervals if n_intervals is not None else max(2, self._N_increment // 10)
        n_strat = n_strat_for(self._N_increment, dim)
        self.results = []
        self.sigma2 = []
        self.it = 0

        fused = (
            isinstance(fn, BuiltinIntegrand)
            and type(rng) is RNG
            and fn.dim == dim
            and not (torch.is_grad_enabled() and (domain.requires_grad or fn.requires_grad()))
        )
        if fused:
            ns = self._starting_N // 5 if use_warmup else 0
            plan = _FusedPlan.get(
                lambda: VegasDevice(dim, self.dtype, N_intervals, n_strat, domain.device, domain,
                                    stats_slots=max_iterations + 10),
                (str(domain.device), torch.cuda.current_stream().cuda_stream, dim, self.dtype,
                 N_intervals, n_strat), fn.family,
                use_grid_improve, use_warmup, ns, max_iterations)
            self._dev = plan.dev
        else:
            plan = None
            self._dev = VegasDevice(dim, self.dtype, N_intervals, n_strat, domain.device, domain,
                                    stats_slots=max(8, max_iterations + 10))
        self.map = VEGASMap(N_intervals, dim, None, self.dtype, _device_state=self._dev)
        self.strat = VEGASStratification(self._N_increment, dim, rng, None, self.dtype,
                                         _device_state=self._dev)
        if fused:
            return self._integrate_fused(plan, fn, domain, use_warmup)
        return self._integrate_materialised(domain, use_warmup)

    # ------------------------------------------------------------ fused
    def _integrate_fused(self, plan, fn, domain, use_warmup):
        rng = self.rng
        ns = plan.ns
        dev = plan.dev
        dev.set_domain(domain)
        dev.params.copy_(fn.device_params(domain.device))
        dev.rng_offset.fill_(rng.offset)
        dev.set_control(L.TQ_VC_NEVALS | L.TQ_VC_SEED | L.TQ_VC_STREAM, nevals=self._starting_N,
                        seed=rng.seed, sid=rng.stream_id)
        self.alpha = ALPHA
        plan.run_warmup()
        warm_evals = 5 * ns if use_warmup else 0
        self._nr_of_fevals = warm_evals
        while True:
            dev.set_control(L.TQ_VC_NEVALS, nevals=self._starting_N)
            plan.run_block()
            self.it += 5
            stats = dev.stats[: self.it].cpu()  # one host sync per five iterations
            self.map.check_flags()
            self.results = [float(v) for v in stats[self.it - 5 : self.it, 0]]
            self.sigma2 = [float(v) for v in stats[self.it - 5 : self.it, 1]]
            self._nr_of_fevals = warm_evals + int(stats[: self.it, 2].sum())
            if self._check_abort_conditions():
                break
        rng.offset = int(dev.rng_offset.item())
        # leave dh normalised, as update_DH does
        s = dev.scalars[0].to(self.dtype)
        dev.dh.copy_(torch.where(s != 0, dev.dh / s, dev.dh))
        return torch.tensor(self._get_result(), dtype=self.dtype, device=domain.device)

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
    def _check_abort_conditions(self):
        """Every fifth iteration: stop on accuracy, adapt the evaluations per
        iteration, stop on budget/iterations (vegas.py:161-209)."""
        if self.it % 5 > 0:
            return False
        res_abs = abs(float(self._get_result()))
        err = self._get_error()
        chi2 = self._get_chisq()
        if (err <= self._eps_rel * res_abs or err <= self._eps_abs) and chi2 / 5.0 < 1.0:
            return True
        if chi2 / 5.0 < 1.0:
            if res_abs == 0.0:
                self._starting_N += self._N_increment
            else:
                acc = err / res_abs
                self._starting_N = min(
                    self._starting_N + self._N_increment,
                    int(self._starting_N * math.sqrt(acc / (self._eps_rel + 1e-8))),
                )
        elif chi2 / 5.0 > 1.0:
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
        if any(s == 0.0 for s in self.sigma2):
            return sum(self.results) / len(self.results)
        num = sum(r / s for r, s in zip(self.results, self.sigma2))
        den = sum(1.0 / s for s in self.sigma2)
        return num / den

    def _get_error(self):
        """Error estimate from the variances (EQ 31)."""
        res = sum(1.0 / s for s in self.sigma2 if s != 0.0)
        return self.sigma2[0] if res == 0 else 1.0 / math.sqrt(res)

    def _get_chisq(self):
        """Chi square of the iteration results (EQ 32)."""
        I_final = float(self._get_result())
        res = [float(r) for r in self.results]
        return sum(((r - I_final) ** 2 / s for r, s in zip(res, self.sigma2) if r != I_final), 0.0)
