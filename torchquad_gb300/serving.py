"""Serving: continuous batching of integration requests on one GPU.

Requests (Monte Carlo, VEGAS or Simpson, built-in integrands) arrive at any
time.  A scheduler thread

* admits waiting requests in arrival order while a slot is free and the
  request's device-memory footprint (VEGAS maps and strata dominate) fits
  the HBM budget, and releases both when the request completes;
* launches all newly admitted Simpson requests as one batched grid launch
  per dtype (``tq_batch_grid``; integrand families mixed in one launch);
* advances every active Monte Carlo request by one chunk of its own Philox
  stream per tick (chunks double from ``mc_chunk`` to ``mc_chunk_max``), all
  of them in one launch per dtype (``tq_batch_mc``), stopping a request at
  its N or, with ``mc_early_stop``, at its target relative error;
* runs each VEGAS request on its own stream with its map and stratification
  resident on the device, one block of five iterations at a time (the
  reference's abort test, vegas.py:161-209, decides after each block), so
  the blocks of different requests overlap on the GPU;
* polls completions through CUDA events and pinned-memory copies and never
  blocks on the device.

A request's arithmetic does not depend on the other requests: its draws
come from its own seed, its chunks and tiles are fixed by its own size,
and every reduction sums in a fixed order (VEGAS histogram and cube sums
are fp64 atomics: reproducible to rounding).
"""
from __future__ import annotations

import itertools
import math
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L
from .batch import BatchedGrid
from .integrands import BuiltinIntegrand
from .integration._vegas_state import VegasDevice, n_strat_for
from .integration.vegas import ALPHA, BETA, VEGAS, _graphs_enabled

MC_DESC = np.dtype([("dim", "<i4"), ("family", "<i4"), ("first", "<i8"), ("count", "<i8"), ("seed", "<u8"),
                    ("sid", "<u8"), ("par_off", "<i8"), ("dom_off", "<i8")])
assert MC_DESC.itemsize == 56


@dataclass
class IntegrationRequest:
    method: str  # "montecarlo" | "vegas" | "simpson"
    integrand: BuiltinIntegrand
    N: int
    domain: list
    seed: int = 0
    eps_rel: float = 0.0
    dtype: torch.dtype = torch.float32
    # filled in by the server
    id: int = -1
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    result: float = float("nan")
    error: float = float("nan")
    evals: int = 0
    future: Future = field(default=None, repr=False)

    @property
    def dim(self):
        return self.integrand.dim


def _footprint(req: IntegrationRequest) -> int:
    """Device bytes a request holds while active."""
    s = 4 if req.dtype == torch.float32 else 8
    d = req.dim
    if req.method == "vegas":
        n_inc = req.N // 25
        B = max(2, n_inc // 10)
        nc = n_strat_for(n_inc, d) ** d
        state = d * (2 * B + 1) * s + d * B * 16 + nc * (s + 8 * 5) + 8 * (nc + 1)
        scratch = d * B * 40 + nc * 8 + 4096
        return state + scratch + 64 * 1024
    if req.method == "montecarlo":
        return 64 * 1024
    return 64 * 1024 + 16 * (req.N // 32768 + 1)


def _merge(a, i, s, c):
    """Neumaier-add the compensated pair (s, c) into a[i], a[i+1]."""
    t = a[i] + s
    if abs(a[i]) >= abs(s):
        a[i + 1] += (a[i] - t) + s
    else:
        a[i + 1] += (s - t) + a[i]
    a[i] = t
    a[i + 1] += c


class _VegasSession:
    """One VEGAS request: device state on its own stream, advanced one block
    of five iterations at a time; the host logic is the VEGAS class's."""

    def __init__(self, req, device, stream):
        self.req = req
        self.stream = stream
        dt = req.dtype
        v = VEGAS()
        v._dim = req.dim
        v.dtype = dt
        v._max_iterations = 20
        v._eps_rel, v._eps_abs = req.eps_rel, 0.0
        v.use_grid_improve = True
        v.N = req.N
        v._starting_N = v._N_increment = req.N // 25
        v.results, v.sigma2, v.it = [], [], 0
        self.v = v
        B = max(2, v._N_increment // 10)
        ns = n_strat_for(v._N_increment, req.dim)
        with torch.cuda.stream(stream):
            dom = torch.tensor(req.domain, dtype=dt, device=device)
            self.dev = VegasDevice(req.dim, dt, B, ns, device, dom, stats_slots=32)
            self.params = req.integrand.device_params(device)
            self.dev.set_control(L.TQ_VC_NEVALS | L.TQ_VC_SEED | L.TQ_VC_STREAM, nevals=v._starting_N,
                                 seed=req.seed, sid=0)
        self.host = torch.empty((32 * 4 + 8,), dtype=torch.float64, pin_memory=True)
        self.graph = None
        self.event = None
        self.warm_evals = 5 * (v._starting_N // 5)
        self.started = False

    def launch(self):
        d, v = self.dev, self.v
        with torch.cuda.stream(self.stream):
            if not self.started:
                ns = v._starting_N // 5
                for _ in range(5):
                    if ns > 0:
                        d.warmup_fused(self.req.integrand.family, self.params, ns)
                    d.update_map(ALPHA)
                self.started = True
            else:
                d.set_control(L.TQ_VC_NEVALS, nevals=v._starting_N)
            # The block reads its evaluation count, statistics slot and RNG
            # offset from the control block, so the session captures it once
            # (on its own stream, without a device synchronisation) and
            # replays the graph for every block.
            if self.graph is None and _graphs_enabled():
                g = torch.cuda.CUDAGraph()
                g.capture_begin(capture_error_mode="thread_local")
                try:
                    self._block()
                finally:
                    g.capture_end()
                self.graph = g
            if self.graph is not None:
                self.graph.replay()
                L.count_launches(5 * (3 + d.finish_update_map_launches))
            else:
                self._block()
            v.it += 5
            self.host[: 32 * 4].copy_(d.stats.reshape(-1)[: 32 * 4], non_blocking=True)
            self.event = torch.cuda.Event()
            self.event.record(self.stream)

    def _block(self):
        d = self.dev
        for _ in range(5):
            d.get_nh()
            d.iterate_fused(self.req.integrand.family, self.params, True, d.points_hint(self.v._N_increment))
            d.finish_update_map(BETA, ALPHA)

    def done(self):
        """After the block's event: True if the request is finished."""
        v = self.v
        st = self.host[: 32 * 4].reshape(32, 4)
        v.results = [float(x) for x in st[v.it - 5 : v.it, 0]]
        v.sigma2 = [float(x) for x in st[v.it - 5 : v.it, 1]]
        v._nr_of_fevals = self.warm_evals + int(st[: v.it, 2].sum())
        finished = v._check_abort_conditions() or v.it + 5 > 30
        if finished:
            self.req.result = float(v._get_result())
            self.req.error = float(v._get_error())
            self.req.evals = v._nr_of_fevals
        return finished


class IntegrationServer:
    """Continuous-batching integration server on one CUDA device."""

    def __init__(self, hbm_budget_bytes=None, max_active=64, mc_chunk=1 << 21, mc_chunk_max=1 << 25,
                 mc_tile=1 << 16,
                 grid_tile=1 << 15, device=None, streams=8, mc_early_stop=True):
        self.device = device or L.require_cuda()
        if hbm_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget_bytes = int(free * 0.5)
        self.budget = int(hbm_budget_bytes)
        self.free_bytes = self.budget
        self.max_active = int(max_active)
        self.mc_chunk, self.mc_tile, self.grid_tile = int(mc_chunk), int(mc_tile), int(grid_tile)
        self.mc_chunk_max = max(int(mc_chunk_max), self.mc_chunk)
        # stop a Monte Carlo request at its target relative error (True) or
        # always run it to N, as MonteCarlo.integrate does (False)
        self.mc_early_stop = bool(mc_early_stop)
        self._ids = itertools.count()
        self._pending = deque()
        self._lock = threading.Lock()
        self._wake = threading.Event()
        self._stop = False
        self.completed = []
        self.peak_active = 0
        self._vegas = []  # active sessions
        self._mc = []  # active MC requests (state dicts)
        self._grid_inflight = []  # (event, host tensor, requests)
        self._mc_inflight = None
        self._grid_stream = torch.cuda.Stream(self.device)
        self._mc_stream = torch.cuda.Stream(self.device)
        self._vegas_streams = [torch.cuda.Stream(self.device) for _ in range(max(1, streams))]
        self._stream_rr = itertools.cycle(self._vegas_streams)
        self._thread = None
        self._active = 0
        self.host_launch_s = 0.0  # scheduler time spent issuing device work

    # ---------------------------------------------------------------- API
    def start(self):
        if self._thread is None:
            self._thread = threading.Thread(target=self._loop, name="tq-serving", daemon=True)
            self._thread.start()
        return self

    def stop(self, wait=True):
        self._stop = True
        self._wake.set()
        if wait and self._thread is not None:
            self._thread.join()
            self._thread = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    def submit(self, req: IntegrationRequest) -> Future:
        if req.method not in ("montecarlo", "vegas", "simpson"):
            raise ValueError(f"unknown method {req.method}")
        if not isinstance(req.integrand, BuiltinIntegrand):
            raise ValueError("serving takes built-in integrands")
        if req.dim > L.TQ_MAX_DIM:
            raise ValueError(f"dim must be <= {L.TQ_MAX_DIM}")
        d = np.asarray(req.domain, dtype=np.float64).reshape(req.dim, 2)
        if np.any(d[:, 1] < d[:, 0]):
            raise ValueError("integration_domain has invalid boundary values")
        if _footprint(req) > self.budget:
            raise ValueError("request needs more device memory than the server's HBM budget")
        req.id = next(self._ids)
        req.t_submit = time.perf_counter()
        req.future = Future()
        with self._lock:
            self._pending.append(req)
        self._wake.set()
        return req.future

    def drain(self, timeout=None):
        """Block until every submitted request completed."""
        t0 = time.perf_counter()
        while True:
            with self._lock:
                busy = bool(self._pending) or self._active > 0
            if not busy:
                return
            if timeout is not None and time.perf_counter() - t0 > timeout:
                raise TimeoutError("requests still running")
            time.sleep(0.0005)

    def stats(self):
        lat = np.array([r.t_done - r.t_submit for r in self.completed])
        if lat.size == 0:
            return {}
        span = max(r.t_done for r in self.completed) - min(r.t_submit for r in self.completed)
        return {
            "completed": int(lat.size),
            "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "integrals_per_s": float(lat.size / span) if span > 0 else float("inf"),
            "evals": int(sum(r.evals for r in self.completed)),
            "peak_active": self.peak_active,
            "host_launch_ms": self.host_launch_s * 1e3,
        }

    # ---------------------------------------------------------- scheduler
    def _loop(self):
        torch.cuda.set_device(self.device)
        while True:
            progressed = self._admit()
            progressed |= self._poll()
            progressed |= self._launch()
            with self._lock:
                idle = not self._pending and self._active == 0
            if self._stop and idle:
                return
            if not progressed:
                self._wake.wait(0.0002)
                self._wake.clear()

    def _admit(self):
        new_grid = []
        admitted = False
        while True:
            with self._lock:
                if not self._pending or self._active >= self.max_active:
                    break
                req = self._pending[0]
                fp = _footprint(req)
                if fp > self.free_bytes:
                    break
                self._pending.popleft()
                self.free_bytes -= fp
                self._active += 1
                self.peak_active = max(self.peak_active, self._active)
            req.t_admit = time.perf_counter()
            req._fp = fp
            admitted = True
            if req.method == "vegas":
                self._vegas.append(_VegasSession(req, self.device, next(self._stream_rr)))
            elif req.method == "montecarlo":
                self._mc.append({"req": req, "done_pts": 0, "acc": [0.0, 0.0, 0.0, 0.0],
                                 "next_chunk": self.mc_chunk})
            else:
                new_grid.append(req)
        if new_grid:
            self._launch_grid(new_grid)
        return admitted

    def _finish(self, req):
        req.t_done = time.perf_counter()
        with self._lock:
            self.free_bytes += req._fp
            self._active -= 1
        self.completed.append(req)
        req.future.set_result(req.result)

    def _launch_grid(self, reqs):
        groups = {}
        for r in reqs:
            groups.setdefault(r.dtype, []).append(r)
        for dt, rs in groups.items():
            bg = BatchedGrid(dtype=dt, autotune=False, tile_points=self.grid_tile)
            with torch.cuda.stream(self._grid_stream):
                plan = bg.plan([r.integrand for r in rs], ["simpson"] * len(rs), [r.N for r in rs],
                               [r.domain for r in rs])
                out = bg.run(plan)
                host = torch.empty((len(rs),), dtype=torch.float64, pin_memory=True)
                host.copy_(out.double(), non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(self._grid_stream)
            for r, n in zip(rs, plan.desc_np["total"]):
                r.evals = int(n)
            self._grid_inflight.append((ev, host, rs))

    def _launch(self):
        t0 = time.perf_counter()
        try:
            return self._launch_all()
        finally:
            self.host_launch_s += time.perf_counter() - t0

    def _launch_all(self):
        launched = False
        for s in self._vegas:
            if s.event is None:
                s.launch()
                launched = True
        if self._mc and self._mc_inflight is None:
            self._launch_mc()
            launched = True
        return launched

    def _launch_mc(self):
        groups = {}
        for st in self._mc:
            r = st["req"]
            groups.setdefault(r.dtype, []).append(st)
        inflight = []
        with torch.cuda.stream(self._mc_stream):
            for dt, sts in groups.items():
                m = len(sts)
                desc = np.zeros(m, dtype=MC_DESC)
                par, dom = [], []
                po = do = 0
                for i, st in enumerate(sts):
                    r = st["req"]
                    # a request's chunks double from mc_chunk up to mc_chunk_max:
                    # few ticks for large N, fine steps for the target-error test
                    cnt = min(st["next_chunk"], r.N - st["done_pts"])
                    st["next_chunk"] = min(2 * st["next_chunk"], self.mc_chunk_max)
                    desc[i] = (r.dim, r.integrand.family, st["done_pts"], cnt, r.seed, 0, po, do)
                    st["chunk"] = cnt
                    pv = r.integrand.params_numpy()
                    par.append(pv)
                    dom.append(np.asarray(r.domain, dtype=np.float64).ravel())
                    po += pv.size
                    do += 2 * r.dim
                tiles = (desc["count"] + self.mc_tile - 1) // self.mc_tile
                ts = np.zeros(m + 1, dtype=np.int64)
                np.cumsum(tiles, out=ts[1:])
                npdt = np.float32 if dt == torch.float32 else np.float64
                d_desc = torch.from_numpy(desc.view(np.uint8).copy()).to(self.device, non_blocking=True)
                d_ts = torch.from_numpy(ts).to(self.device, non_blocking=True)
                d_par = torch.from_numpy(np.concatenate(par)).to(self.device, non_blocking=True)
                d_dom = torch.from_numpy(np.concatenate(dom).astype(npdt)).to(self.device, non_blocking=True)
                acc = torch.zeros((m, 4), dtype=torch.float64, device=self.device)
                ws = torch.empty((int(ts[-1]) * 32,), dtype=torch.uint8, device=self.device)
                L.check(L.lib().tq_batch_mc(L.dtype_code(dt), m, d_desc.data_ptr(), d_ts.data_ptr(), int(ts[-1]),
                                            self.mc_tile, d_par.data_ptr(), d_dom.data_ptr(), L.TQ_FN_PER_DESC,
                                            acc.data_ptr(), ws.data_ptr(), ws.numel(), L.stream_handle()),
                        "tq_batch_mc")
                L.count_launches(2)
                host = torch.empty((m, 4), dtype=torch.float64, pin_memory=True)
                host.copy_(acc, non_blocking=True)
                # keep the device buffers alive until the event
                inflight.append((host, sts, (d_desc, d_ts, d_par, d_dom, acc, ws)))
            ev = torch.cuda.Event()
            ev.record(self._mc_stream)
        self._mc_inflight = (ev, inflight)

    def _poll(self):
        progressed = False
        keep = []
        for ev, host, rs in self._grid_inflight:
            if ev.query():
                for r, v in zip(rs, host.tolist()):
                    r.result = v
                    r.error = 0.0
                    self._finish(r)
                progressed = True
            else:
                keep.append((ev, host, rs))
        self._grid_inflight = keep
        if self._mc_inflight is not None and self._mc_inflight[0].query():
            _, inflight = self._mc_inflight
            self._mc_inflight = None
            finished = []
            for host, sts, _bufs in inflight:
                for st, row in zip(sts, host.tolist()):
                    r = st["req"]
                    a = st["acc"]
                    # compensated running sums across chunks, in chunk order
                    _merge(a, 0, row[0], row[1])
                    _merge(a, 2, row[2], row[3])
                    st["done_pts"] += st["chunk"]
                    n = st["done_pts"]
                    vol = float(np.prod(np.diff(np.asarray(r.domain, dtype=np.float64), axis=1)))
                    m1 = (a[0] + a[1]) / n
                    m2 = (a[2] + a[3]) / n
                    r.result = vol * m1
                    r.error = vol * math.sqrt(max(m2 - m1 * m1, 0.0) / n)
                    r.evals = n
                    if n >= r.N or (self.mc_early_stop and r.eps_rel > 0 and n >= 65536
                                    and r.error <= r.eps_rel * abs(r.result)):
                        finished.append(st)
            for st in finished:
                self._mc.remove(st)
                self._finish(st["req"])
            progressed = True
        still = []
        for s in self._vegas:
            if s.event is not None and s.event.query():
                s.event = None
                if s.done():
                    self._finish(s.req)
                    progressed = True
                    continue
                progressed = True
            still.append(s)
        self._vegas = still
        return progressed


def poisson_stream(n, rate, seed=2, dims=(1, 10), n_range=(1e4, 1e8), eps_range=(1e-3, 1e-5),
                   dtype=torch.float32):
    """The serving workload: n requests with exponential inter-arrival times
    at `rate` req/s, methods uniform over {montecarlo, vegas, simpson}, dim
    uniform in dims, N log-uniform in n_range, target relative error
    log-uniform in eps_range, Gaussian-peak or oscillatory integrands with
    seeded parameters.  Returns [(arrival_time_s, IntegrationRequest)]."""
    from .integrands import GaussianPeak, Oscillatory

    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    methods = ["montecarlo", "vegas", "simpson"]
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        meth = methods[int(rng.integers(0, 3))]
        d = int(rng.integers(dims[0], dims[1] + 1))
        N = int(10 ** rng.uniform(math.log10(n_range[0]), math.log10(n_range[1])))
        eps = float(10 ** rng.uniform(math.log10(eps_range[1]), math.log10(eps_range[0])))
        if rng.random() < 0.5:
            f = GaussianPeak(d, a=rng.uniform(0.5, 5.0, d).tolist(), u=rng.uniform(0, 1, d).tolist())
        else:
            f = Oscillatory(d, a=rng.uniform(-3.0, 3.0, d).tolist(), b=float(rng.uniform(0, 1)))
        dom = [[0.0, 1.0]] * d
        out.append((t, IntegrationRequest(meth, f, N, dom, seed=int(rng.integers(0, 2**31)), eps_rel=eps,
                                          dtype=dtype)))
    return out
