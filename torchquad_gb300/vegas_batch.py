"""Many VEGAS integrals of built-in integrands advanced together.

The reference integrates one VEGAS integral per ``VEGAS().integrate`` call
(vegas.py:100-160).  A :class:`VegasBatch` keeps one resident device state
per integral (adaptive map, stratification, statistics, control block) and
advances all of them at once: each phase of the fused run (state reset and
run inputs, warm-up sampling, warm-up map update, get_NH, stratified
sampling, end of iteration beside the map update, abort test) is one launch
of ``tq_vegas_batch_phase`` for the whole batch, and the iteration loop is a
WHILE node of one captured CUDA graph that repeats blocks of five
iterations while some integral's abort test says go on.  An integral whose
test has stopped it skips the remaining blocks.  Each integral follows the
reference's algorithm exactly as its own ``VEGAS().integrate`` does with the
same random stream (same seed), so results agree with the per-call API up
to the order of floating-point atomic additions.

Shapes are fixed when the batch is made (integrand family, dim, N, dtype,
max_iterations, use_grid_improve, use_warmup); every call may change the
integrand parameters, the domains, the seeds and the accuracy targets.
Maps of at most 1024 intervals per dimension (N up to about 256000 with the
reference's N_increment // 10 intervals).
"""
from __future__ import annotations

import ctypes
import itertools
import warnings

import numpy as np
import torch

from . import _lib as L
from .integrands import BuiltinIntegrand
from .integration.rng import RNG
from .integration.vegas import ALPHA, BETA, _graphs_enabled
from .integration._vegas_state import VegasDevice, n_strat_for
from .integration.vegas_map import _cannot_update_warning

MAX_BATCH_INTERVALS = 1024


def _run_dtype():
    """numpy view of tq_vegas_run (the ctypes mirror's field offsets)."""
    R = L.VegasRun
    fields = [("nevals_exp", "<i8"), ("N", "<i8"), ("N_increment", "<i8"), ("max_iterations", "<i8"),
              ("warm_evals", "<i8"), ("eps_rel", "<f8"), ("eps_abs", "<f8"), ("seed", "<u8"),
              ("stream_id", "<u8"), ("rng_offset", "<u8"), ("n_params", "<i4"), ("n_domain", "<i4"),
              ("params", ("<f8", 2 + 2 * L.TQ_MAX_DIM)), ("domain", ("<f8", 2 * L.TQ_MAX_DIM))]
    return np.dtype({"names": [f for f, _ in fields], "formats": [t for _, t in fields],
                     "offsets": [getattr(R, f).offset for f, _ in fields], "itemsize": ctypes.sizeof(R)})


RUN_DTYPE = _run_dtype()


class VegasBatch:
    """A batch of VEGAS integrals sharing one graph (see module docstring).

    integrands: BuiltinIntegrand per integral (its ``dim`` must match);
    Ns: evaluation budget per integral (the reference's ``N``).  After a
    call, ``it``, ``nr_of_fevals``, ``starting_N_out``, ``results``,
    ``sigma2`` and ``rng_offsets`` hold each integral's counterpart of the
    reference's attributes.  A batch is used from one thread at a time."""

    def __init__(self, integrands, Ns, dtype=torch.float64, max_iterations=20, use_grid_improve=True,
                 use_warmup=True, n_intervals=None, device=None):
        n = len(integrands)
        if n < 1 or len(Ns) != n:
            raise ValueError("VegasBatch needs one N per integrand and at least one integral")
        if dtype not in (torch.float32, torch.float64):
            raise ValueError(f"unsupported dtype {dtype}")
        self.device = device if device is not None else L.require_cuda()
        self.dtype = dtype
        self.n = n
        self.integrands = list(integrands)
        self.max_iterations = int(max_iterations)
        self.use_grid_improve = bool(use_grid_improve)
        self.use_warmup = bool(use_warmup)
        slots = self.max_iterations + 10
        words = VegasDevice.readback_words(slots)
        self._rb = torch.zeros((n, words), dtype=torch.int64, device=self.device)
        self._rb_host = torch.zeros((n, words), dtype=torch.int64, pin_memory=True)
        self.N = np.asarray([int(N) for N in Ns], dtype=np.int64)
        self.starting_N = self.N // (self.max_iterations + 5)
        self.states = []
        items = (L.VegasItem * n)()
        run_size = ctypes.sizeof(L.VegasRun)
        self._runs_host = torch.zeros((n * run_size,), dtype=torch.uint8, pin_memory=True)
        self._runs_dev = torch.zeros((n * run_size,), dtype=torch.uint8, device=self.device)
        self.warm_samples = []
        for i, (fn, N) in enumerate(zip(self.integrands, self.N)):
            if not isinstance(fn, BuiltinIntegrand):
                raise TypeError("VegasBatch integrates built-in integrands (torchquad_gb300.integrands)")
            dim = fn.dim
            if dim < 1 or dim > L.TQ_MAX_DIM:
                raise ValueError(f"VEGAS kernels support 1 <= dim <= {L.TQ_MAX_DIM}, got {dim}")
            n_inc = int(self.starting_N[i])
            B = n_intervals if n_intervals is not None else max(2, n_inc // 10)
            if B > MAX_BATCH_INTERVALS:
                raise ValueError(f"VegasBatch maps have at most {MAX_BATCH_INTERVALS} intervals per "
                                 f"dimension (N = {int(N)} gives {B})")
            dev = VegasDevice(dim, dtype, B, n_strat_for(n_inc, dim), self.device, None, stats_slots=slots,
                              readback=(self._rb[i], self._rb_host[i]))
            self.states.append(dev)
            ns = n_inc // 5 if self.use_warmup else 0
            self.warm_samples.append(ns)
            it = items[i]
            it.st = dev.struct
            it.params = dev.params.data_ptr()
            it.workspace, it.workspace_bytes = dev.ws.data_ptr(), dev.ws.numel()
            it.warm_samples = ns
            it.expected_points = dev.points_hint(n_inc)
            it.family = fn.family
            it.use_grid_improve = int(self.use_grid_improve)
            it.use_warmup = int(self.use_warmup)
        self._items = items
        self.dims = np.asarray([fn.dim for fn in self.integrands], dtype=np.int32)
        # (record, column) of every parameter and every domain bound, in the
        # order of the integrands' flat vectors
        reps_p, reps_d = 2 + 2 * self.dims, 2 * self.dims
        self._p_rows = np.repeat(np.arange(n), reps_p)
        self._p_cols = np.concatenate([np.arange(k) for k in reps_p])
        self._d_rows = np.repeat(np.arange(n), reps_d)
        self._d_cols = np.concatenate([np.arange(k) for k in reps_d])
        self._unit_domains = np.tile([0.0, 1.0], int(self.dims.sum()))
        self.rng_offsets = np.zeros(n, dtype=np.uint64)
        self._runs = self._runs_host.numpy().view(RUN_DTYPE)  # shares the pinned memory
        nbytes = L.lib().tq_vegas_batch_table_size(items, n)
        if nbytes == 0:
            raise ValueError("invalid VEGAS batch (shapes or dtypes)")
        self.table = torch.zeros((int(nbytes),), dtype=torch.uint8, device=self.device)
        self.info = L.VegasBatchInfo()
        L.check(L.lib().tq_vegas_batch_build(items, n, self.table.data_ptr(), self.table.numel(),
                                             ctypes.byref(self.info), L.stream_handle()),
                "tq_vegas_batch_build")
        self.graph = None
        self.calls = 0
        # per-integral outcome of the last call
        self.it = np.zeros(n, dtype=np.int64)
        self.nr_of_fevals = np.zeros(n, dtype=np.int64)
        self.results = None
        self.sigma2 = None

    # ------------------------------------------------------------ launches
    def _phase(self, phase, cond=0):
        L.check(L.lib().tq_vegas_batch_phase(ctypes.byref(self.info), self.table.data_ptr(), phase,
                                             self._runs_dev.data_ptr(), ALPHA, BETA, int(cond),
                                             L.stream_handle()), "tq_vegas_batch_phase")
        L.count_launches(1 if self.info.ctas[phase] > 0 else 0)

    def _warm_seq(self):
        self._phase(L.VB_BEGIN)
        if self.use_warmup:
            for _ in range(5):
                self._phase(L.VB_WARM)
                self._phase(L.VB_MAP)

    def _block_seq(self, cond=0):
        for _ in range(5):
            self._phase(L.VB_NH)
            self._phase(L.VB_SAMPLE)
            self._phase(L.VB_FINISH)
        self._phase(L.VB_ABORT, cond)

    def _active_after_abort(self):
        return int(self.table[8:12].view(torch.int32).item())  # BatchHeader.last_active

    def _capture(self):
        g = torch.cuda.CUDAGraph()
        h = ctypes.c_uint64(0)
        with torch.cuda.graph(g):
            body = L.body_stream(self.device)
            self._warm_seq()
            L.check(L.lib().tq_capture_while_begin(L.stream_handle(), body.cuda_stream, ctypes.byref(h)),
                    "tq_capture_while_begin")
            try:
                with torch.cuda.stream(body):
                    self._block_seq(h.value)
            finally:
                L.check(L.lib().tq_capture_while_end(body.cuda_stream), "tq_capture_while_end")
        return g

    def _launches_per_call(self, blocks):
        c = self.info.ctas
        warm = 1 + (5 * ((c[L.VB_WARM] > 0) + (c[L.VB_MAP] > 0)) if self.use_warmup else 0)
        per_block = 5 * ((c[L.VB_NH] > 0) + (c[L.VB_SAMPLE] > 0) + (c[L.VB_FINISH] > 0)) + 1
        return warm + blocks * per_block

    # ---------------------------------------------------------------- run
    def integrate(self, domains=None, seeds=None, rngs=None, eps_rel=0.0, eps_abs=0.0, params=None):
        """Integrate every integral of the batch; returns a [n] tensor (the
        batch's dtype) of VEGAS results.  domains: per integral [[lo, hi]] *
        dim host values (default the unit cube); seeds (a fresh stream per
        integral, as ``VEGAS().integrate(seed=...)``; default random) or
        rngs (RNG objects whose offsets advance as VEGAS().integrate
        advances them); eps_rel / eps_abs: scalars or one per integral;
        params: optional [n, >= 2 + 2 dim] fp64 parameter rows in place of
        the integrands' current parameters.  The RNG offsets after the run
        are also in ``rng_offsets``."""
        n = self.n
        if domains is not None and len(domains) != n:
            raise ValueError("one domain per integral")
        # the run records (tq_vegas_run), column by column, in the pinned
        # buffer the BEGIN phase reads after one copy
        rec = self._runs
        rec["nevals_exp"] = self.starting_N
        rec["N"] = self.N
        rec["N_increment"] = self.starting_N
        rec["max_iterations"] = self.max_iterations
        rec["warm_evals"] = 5 * np.asarray(self.warm_samples, dtype=np.int64)
        rec["eps_rel"] = np.broadcast_to(np.asarray(eps_rel, dtype=np.float64), (n,))
        rec["eps_abs"] = np.broadcast_to(np.asarray(eps_abs, dtype=np.float64), (n,))
        mask = (1 << 64) - 1
        if rngs is not None:
            if seeds is not None:
                raise ValueError("seed and rng cannot both be passed")
            if len(rngs) != n:
                raise ValueError("one RNG per integral")
            rec["seed"] = np.fromiter((r.seed & mask for r in rngs), dtype=np.uint64, count=n)
            rec["stream_id"] = np.fromiter((r.stream_id & mask for r in rngs), dtype=np.uint64, count=n)
            rec["rng_offset"] = np.fromiter((r.offset & mask for r in rngs), dtype=np.uint64, count=n)
        else:
            if seeds is None:
                seeds = [RNG(seed=None).seed for _ in range(n)]
            seeds = list(seeds)
            if len(seeds) != n:
                raise ValueError("one seed per integral")
            rec["seed"] = np.fromiter((int(x) & mask for x in seeds), dtype=np.uint64, count=n)
            rec["stream_id"] = 0
            rec["rng_offset"] = 0
        rec["n_domain"] = 2 * self.dims
        rec["n_params"] = 2 + 2 * self.dims
        # parameters and domains as flat vectors scattered into the records
        if params is None:
            flat_p = np.concatenate([fn.params_numpy() for fn in self.integrands])
        else:
            pa = np.asarray(params, dtype=np.float64)
            if pa.ndim != 2 or pa.shape[0] != n or pa.shape[1] < int(2 + 2 * self.dims.max()):
                raise ValueError("params must be [n, >= 2 + 2 * max dim] fp64 rows")
            flat_p = pa[self._p_rows, self._p_cols]
        rec["params"][self._p_rows, self._p_cols] = flat_p
        if domains is None:
            flat_d = self._unit_domains
        else:
            for i, dm in enumerate(domains):
                if len(dm) != self.dims[i]:
                    raise ValueError(f"domain {i} has {len(dm)} dimensions, its integrand {self.dims[i]}")
            chain = itertools.chain.from_iterable
            try:
                flat_d = np.fromiter(chain(chain(domains)), dtype=np.float64, count=self._d_rows.size)
            except (TypeError, ValueError) as e:
                raise ValueError("domains must be [[lo, hi]] * dim per integral") from e
        rec["domain"][self._d_rows, self._d_cols] = flat_d
        self._runs_dev.copy_(self._runs_host, non_blocking=True)
        self.calls += 1
        if self.graph is None and self.calls > 1 and _graphs_enabled():
            torch.cuda.current_stream().synchronize()
            self.graph = self._capture()
        if self.graph is not None:
            self.graph.replay()
        else:
            self._warm_seq()
            while True:
                self._block_seq()
                if self._active_after_abort() == 0:
                    break
        self._rb_host.copy_(self._rb, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        out = self._collect()
        if rngs is not None:
            for rng, off in zip(rngs, self.rng_offsets):
                rng.offset = int(off)
        if self.graph is not None:
            L.count_launches(self._launches_per_call(int(self.it.max()) // 5))
        return out

    def _collect(self):
        """The reference's per-integral attributes and results (_get_result,
        EQ 30, in the batch's dtype with left-to-right sums) from the one
        read-back of every state."""
        h = self._rb_host.numpy()
        R = VegasDevice._RB_STATS
        ctl = h[:, :16]
        stop = ctl[:, L.VC_STOP]
        # where a per-call run raises (the reference's int() of a
        # non-finite value in the abort test), the batch raises the same
        # exception, naming the first integral concerned
        for code, exc, msg in ((4, RuntimeError, "VEGAS ran out of statistics slots"),
                               (5, OverflowError, "cannot convert float infinity to integer"),
                               (6, ValueError, "cannot convert float NaN to integer")):
            bad = np.nonzero(stop == code)[0]
            if bad.size:
                raise exc(f"{msg} (integral {int(bad[0])} of the batch)")
        flags = h[:, 16:20].view(np.int32)
        if np.any(flags[:, 2]):
            raise RuntimeError("Could not replace all infinite edges")
        # the reference's warnings (vegas_map.py:187-196, :247-257), one per
        # update of each integral, as the per-call API emits them
        for _ in range(int(flags[:, 0].sum())):
            _cannot_update_warning()
        if np.any(flags[:, 1]):
            warnings.warn("Some calculated VEGASMap edges were infinite", RuntimeWarning)
        self.it = ctl[:, L.VC_IT].copy()
        self.starting_N_out = ctl[:, L.VC_NEVALS].copy()
        self.nr_of_fevals = ctl[:, L.VC_EVALS].copy()
        self.rng_offsets = h[:, 20].view(np.uint64).copy()
        stats = h[:, R:].view(np.float64).reshape(self.n, -1, 4)
        rows = self.it[:, None] - 5 + np.arange(5)[None, :]
        idx = np.arange(self.n)[:, None]
        S = np.float32 if self.dtype == torch.float32 else np.float64
        r = stats[idx, rows, 0].astype(S)
        s = stats[idx, rows, 1].astype(S)
        self.results, self.sigma2 = r, s
        with np.errstate(all="ignore"):
            zero = np.zeros(self.n, dtype=S)
            plain, num, den = zero.copy(), zero.copy(), zero.copy()
            for k in range(5):
                plain = plain + r[:, k]
                num = num + r[:, k] / s[:, k]
                den = den + S(1) / s[:, k]
            res = np.where(np.any(s == 0, axis=1), plain / S(5), num / den)
        return torch.from_numpy(res.astype(S)).to(self.device)


def integrate_vegas_batch(integrands, Ns, domains=None, seeds=None, dtype=torch.float64, max_iterations=20,
                          eps_rel=0.0, eps_abs=0.0, use_grid_improve=True, use_warmup=True):
    """One-shot form of :class:`VegasBatch` (builds the batch, integrates
    once)."""
    vb = VegasBatch(integrands, Ns, dtype=dtype, max_iterations=max_iterations,
                    use_grid_improve=use_grid_improve, use_warmup=use_warmup)
    return vb.integrate(domains=domains, seeds=seeds, eps_rel=eps_rel, eps_abs=eps_abs)


__all__ = ["VegasBatch", "integrate_vegas_batch", "MAX_BATCH_INTERVALS"]
