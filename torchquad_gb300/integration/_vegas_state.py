"""Device-resident VEGAS state shared by VEGASMap and VEGASStratification.

All arrays live in torch-owned CUDA tensors; ``struct`` is the
``tq_vegas_state`` of include/torchquad_gb300.h pointing at them.  A state
also owns its scratch workspace (its size depends on the state's shape).
"""
from __future__ import annotations

import ctypes
import weakref

import torch

from .. import _lib as L


def n_strat_for(N_increment, dim):
    """vegas_stratification.py:27-28 (at least one step per dimension)."""
    n = int((N_increment / 4.0) ** (1.0 / dim))
    n = 1000 if n > 1000 else n
    return max(1, n)


class VegasDevice:
    def __init__(self, dim, dtype, n_bins, n_strat, device, domain=None, stats_slots=64, readback=None):
        if dim < 1 or dim > L.TQ_MAX_DIM:
            raise ValueError(f"VEGAS kernels support 1 <= dim <= {L.TQ_MAX_DIM}, got {dim}")
        self.dim, self.dtype, self.device = dim, dtype, device
        self.n_bins, self.n_strat = int(n_bins), int(n_strat)
        self.n_cubes = self.n_strat**dim
        f = dict(dtype=dtype, device=device)
        self.x_edges = torch.empty((dim, self.n_bins + 1), **f)
        self.dx_edges = torch.empty((dim, self.n_bins), **f)
        self.weights = torch.zeros((dim, self.n_bins), dtype=torch.float64, device=device)
        self.counts = torch.zeros((dim, self.n_bins), dtype=torch.int64, device=device)
        self.dh = torch.empty((self.n_cubes,), **f)
        self.jf = torch.zeros((self.n_cubes,), dtype=torch.float64, device=device)
        self.jf2 = torch.zeros((self.n_cubes,), dtype=torch.float64, device=device)
        self.neval = torch.zeros((self.n_cubes,), dtype=torch.int64, device=device)
        self.cube_start = torch.zeros((self.n_cubes + 1,), dtype=torch.int64, device=device)
        self.scalars = torch.zeros((4,), dtype=torch.float64, device=device)
        if readback is not None:  # rows of a batch's shared read-back buffers
            self._set_readback(*readback)
        else:
            self._alloc_readback(max(1, stats_slots))
        self.params = torch.zeros((2 + 2 * dim,), dtype=torch.float64, device=device)
        if domain is None:
            domain = torch.tensor([[0.0, 1.0]] * dim, **f)
        # the state's own copy (never an alias of the caller's tensor)
        self.domain = domain.detach().to(device=device, dtype=dtype).clone().contiguous()
        self._domain_src = None
        self.dh_pending = False  # dh awaits update_DH's normalisation (see stratification.dh)
        self._run = L.VegasRun()
        self.struct = L.VegasState()
        self._fill_struct()
        self.ref = ctypes.byref(self.struct)
        nbytes = L.lib().tq_vegas_workspace_size(self.ref)
        if nbytes == 0:
            raise ValueError("invalid VEGAS state shape")
        self.ws = torch.zeros((int(nbytes),), dtype=torch.uint8, device=device)
        L.check(L.lib().tq_vegas_init(self.ref, L.stream_handle()), "tq_vegas_init")
        L.count_launches(1)

    def clone_state(self):
        """A new state of the same shape holding a copy of this one's arrays
        (map, weights, cube sums and counts, dh, statistics, RNG offset,
        domain, parameters): device copies on the current stream."""
        c = VegasDevice(self.dim, self.dtype, self.n_bins, self.n_strat, self.device, self.domain,
                        stats_slots=self.stats.shape[0])
        for name in ("x_edges", "dx_edges", "weights", "counts", "dh", "jf", "jf2", "neval",
                     "cube_start", "scalars", "params", "_rb"):
            getattr(c, name).copy_(getattr(self, name))
        c._rb_host.copy_(self._rb_host)
        c.dh_pending = self.dh_pending
        return c

    def _fill_struct(self):
        s = self.struct
        s.dim = self.dim
        s.dtype = L.dtype_code(self.dtype)
        s.n_bins = self.n_bins
        s.n_strat = self.n_strat
        s.n_cubes = self.n_cubes
        for name in ("x_edges", "dx_edges", "weights", "counts", "dh", "jf", "jf2", "neval",
                     "cube_start", "rng_offset", "stats", "flags", "scalars", "domain", "control"):
            setattr(s, name, getattr(self, name).data_ptr())
        s.n_stat_slots = self.stats.shape[0]

    # Everything the host reads back after a run sits in one int64 buffer, so
    # one copy brings it: control [16], flags [8] (int32), rng_offset [1],
    # padding, stats [slots][4] (fp64).
    _RB_CONTROL, _RB_FLAGS, _RB_OFFSET, _RB_STATS = 0, 16, 20, 24

    @classmethod
    def readback_words(cls, slots):
        """int64 words of the read-back buffer of a state with `slots`
        statistics rows."""
        return cls._RB_STATS + 4 * slots

    def _alloc_readback(self, slots, old=None):
        buf = torch.zeros((self.readback_words(slots),), dtype=torch.int64, device=self.device)
        if old is not None:
            buf[: old.numel()] = old
        self._set_readback(buf, torch.empty(buf.shape, dtype=torch.int64, pin_memory=True))

    def _set_readback(self, buf, host):
        """Device int64 buffer `buf` and its pinned host copy `host` (same
        length) hold control, flags, RNG offset and statistics."""
        slots = (buf.numel() - self._RB_STATS) // 4
        self._rb = buf
        self.control = buf[self._RB_CONTROL:self._RB_FLAGS]
        self.flags = buf[self._RB_FLAGS:self._RB_OFFSET].view(torch.int32)
        self.rng_offset = buf[self._RB_OFFSET:self._RB_OFFSET + 1]
        self.stats = buf[self._RB_STATS:].view(torch.float64).view(slots, 4)
        self._rb_host = host
        h = self._rb_host.numpy()
        self.host_control = h[self._RB_CONTROL:self._RB_FLAGS]
        self.host_flags = h[self._RB_FLAGS:self._RB_OFFSET].view("int32")
        self.host_rng_offset = h[self._RB_OFFSET:self._RB_OFFSET + 1]
        self.host_stats = h[self._RB_STATS:].view("float64").reshape(slots, 4)

    def ensure_slots(self, n):
        if n > self.stats.shape[0]:
            self._alloc_readback(max(n, 2 * self.stats.shape[0]), old=self._rb)
            for name in ("control", "flags", "rng_offset", "stats"):
                setattr(self.struct, name, getattr(self, name).data_ptr())
            self.struct.n_stat_slots = self.stats.shape[0]

    def read_back(self):
        """Copy control, flags, RNG offset and stats to the host (one copy,
        then a wait for the stream); the host_* numpy views then hold them."""
        self._rb_host.copy_(self._rb, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    def set_domain(self, domain):
        """Copy a domain into the state's own buffer (its address stays);
        skipped when it is the tensor copied last time, unchanged since."""
        src = self._domain_src
        if src is not None and src[0]() is domain and src[1] == domain._version:
            return
        self.domain.copy_(domain.detach().to(device=self.device, dtype=self.dtype))
        try:
            self._domain_src = (weakref.ref(domain), domain._version)
        except TypeError:
            self._domain_src = None

    def fill_run(self, nevals, N, n_inc, max_it, warm_evals, eps_rel, eps_abs, seed, sid, offset,
                 params, domain_values=None):
        """The tq_vegas_run struct of a device-side run: control fields, the
        RNG offset, the integrand parameters (fp64 numpy) and, if given, the
        domain as host values ([dim][2] floats)."""
        r = self._run
        r.nevals_exp, r.N, r.N_increment = int(nevals), int(N), int(n_inc)
        r.max_iterations, r.warm_evals = int(max_it), int(warm_evals)
        r.eps_rel, r.eps_abs = float(eps_rel), float(eps_abs)
        mask = (1 << 64) - 1
        r.seed, r.stream_id, r.rng_offset = int(seed) & mask, int(sid) & mask, int(offset) & mask
        n = len(params)
        r.n_params = n
        ctypes.memmove(r.params, params.ctypes.data, 8 * n)
        if domain_values is not None:
            r.n_domain = 2 * self.dim
            k = 0
            for lo, hi in domain_values:
                r.domain[k], r.domain[k + 1] = lo, hi
                k += 2
            self._domain_src = None
        else:
            r.n_domain = 0
        return r

    def begin_run(self, nevals, N, n_inc, max_it, warm_evals, eps_rel, eps_abs, seed, sid, offset,
                  params, domain_values=None):
        """Per-call inputs of a device-side run written by one launch (see
        fill_run)."""
        r = self.fill_run(nevals, N, n_inc, max_it, warm_evals, eps_rel, eps_abs, seed, sid, offset, params,
                          domain_values)
        L.check(L.lib().tq_vegas_begin_run(self.ref, ctypes.byref(r), self.params.data_ptr(),
                                           L.stream_handle()), "tq_vegas_begin_run")
        L.count_launches(1)

    def abort_test(self, cond_handle=0):
        """The every-fifth-iteration abort test on the device (control[11..13],
        control[0]); inside a captured WHILE node, cond_handle stops it."""
        L.check(L.lib().tq_vegas_abort_test(self.ref, int(cond_handle), L.stream_handle()),
                "tq_vegas_abort_test")
        L.count_launches(1)

    def reinit(self):
        self.dh_pending = False
        L.check(L.lib().tq_vegas_init(self.ref, L.stream_handle()), "tq_vegas_init")
        L.count_launches(1)

    def set_control(self, mask, nevals=0, slot=0, normalize=0, seed=0, sid=0):
        L.check(L.lib().tq_vegas_set_control(self.ref, int(mask), int(nevals), int(slot), int(normalize),
                                             int(seed) & ((1 << 64) - 1), int(sid) & ((1 << 64) - 1),
                                             L.stream_handle()), "tq_vegas_set_control")
        L.count_launches(1)

    # ---- thin calls -------------------------------------------------------
    def _ws(self):
        return self.ws.data_ptr(), self.ws.numel()

    def warmup_fused(self, family, params, n_samples):
        p, n = self._ws()
        L.check(L.lib().tq_vegas_warmup_fused(self.ref, family, params.data_ptr(), n_samples, p, n,
                                              L.stream_handle()), "tq_vegas_warmup_fused")
        L.count_launches(1)

    def points_hint(self, n_inc):
        """Points an iteration is sized for (tq_vegas_iterate_fused's
        max_points): N_increment, at least two per cube.  The single-state
        graphs and the batched ones size the sampler alike, so a state gets
        the same CTA split (and the same fp32 partial sums) either way."""
        return max(int(n_inc), 2 * self.n_cubes)

    def iterate_fused(self, family, params, use_grid_improve, max_points=0):
        p, n = self._ws()
        L.check(L.lib().tq_vegas_iterate_fused(self.ref, family, params.data_ptr(),
                                               int(bool(use_grid_improve)), int(max_points), p, n,
                                               L.stream_handle()), "tq_vegas_iterate_fused")
        L.count_launches(1)

    def update_map(self, alpha):
        p, n = self._ws()
        L.check(L.lib().tq_vegas_update_map(self.ref, float(alpha), p, n, L.stream_handle()),
                "tq_vegas_update_map")
        L.count_launches(self.update_map_launches)

    @property
    def update_map_launches(self):
        # maps of more than 1024 intervals per dimension: seven tiled passes
        return 7 if self.n_bins > 1024 else 1

    def smooth(self, alpha):
        out = torch.empty((self.dim, self.n_bins), dtype=self.dtype, device=self.device)
        p, n = self._ws()
        L.check(L.lib().tq_vegas_smooth_weights(self.ref, float(alpha), out.data_ptr(), p, n,
                                                L.stream_handle()), "tq_vegas_smooth_weights")
        L.count_launches(2 if self.n_bins > 1024 else 1)
        return out

    def get_nh(self, nevals_exp=None, normalize=None):
        """get_NH; nevals_exp / normalize, if given, are written to the
        control block first (otherwise the device values are used)."""
        mask = (L.TQ_VC_NEVALS if nevals_exp is not None else 0) | (
            L.TQ_VC_NORMALIZE if normalize is not None else 0)
        if mask:
            self.set_control(mask, nevals=nevals_exp or 0, normalize=int(bool(normalize)))
        self.dh_pending = False  # the device normalises here if control[2] says so
        p, n = self._ws()
        L.check(L.lib().tq_vegas_get_nh(self.ref, p, n, L.stream_handle()), "tq_vegas_get_nh")
        L.count_launches(2)

    def get_nh_split(self):
        """get_NH leaving cube_start split until the next finish (one launch
        instead of two); for the fused get_NH, sampling, finish sequence."""
        self.dh_pending = False
        p, n = self._ws()
        L.check(L.lib().tq_vegas_get_nh_split(self.ref, p, n, L.stream_handle()), "tq_vegas_get_nh_split")
        L.count_launches(1)

    def finish(self, beta, slot=None):
        """finish_iteration into statistics row `slot` (if given, written to
        the control block first; otherwise the device's running slot)."""
        if slot is not None:
            self.ensure_slots(slot + 1)
            self.set_control(L.TQ_VC_SLOT, slot=slot)
        p, n = self._ws()
        L.check(L.lib().tq_vegas_finish_iteration(self.ref, float(beta), p, n, L.stream_handle()),
                "tq_vegas_finish_iteration")
        L.count_launches(1)

    def finish_update_map(self, beta, alpha):
        """finish (running statistics slot) then update_map, one launch for
        maps of at most 1024 intervals per dimension."""
        p, n = self._ws()
        L.check(L.lib().tq_vegas_finish_update_map(self.ref, float(beta), float(alpha), p, n,
                                                   L.stream_handle()), "tq_vegas_finish_update_map")
        L.count_launches(self.finish_update_map_launches)

    @property
    def finish_update_map_launches(self):
        return 1 if self.n_bins <= 1024 else 1 + self.update_map_launches

    def strat_points(self, u):
        y = torch.empty_like(u)
        L.check(L.lib().tq_vegas_strat_points(self.ref, u.data_ptr(), u.shape[0], y.data_ptr(),
                                              L.stream_handle()), "tq_vegas_strat_points")
        L.count_launches(1)
        return y

    def map_points(self, y):
        x = torch.empty_like(y)
        jac = torch.empty((y.shape[0],), dtype=y.dtype, device=y.device)
        L.check(L.lib().tq_vegas_map_points(self.ref, y.data_ptr(), y.shape[0], x.data_ptr(),
                                            jac.data_ptr(), L.stream_handle()), "tq_vegas_map_points")
        L.count_launches(1)
        return x, jac

    def accumulate(self, y, vals, acc_map, stratified):
        p, n = self._ws()
        L.check(L.lib().tq_vegas_accumulate(self.ref, y.data_ptr(), vals.data_ptr(), y.shape[0],
                                            int(acc_map), int(stratified), p, n, L.stream_handle()),
                "tq_vegas_accumulate")
        L.count_launches(1)
