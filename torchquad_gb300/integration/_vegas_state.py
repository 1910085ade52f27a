"""Device-resident VEGAS state shared by VEGASMap and VEGASStratification.

All arrays live in torch-owned CUDA tensors; ``struct`` is the
``tq_vegas_state`` of include/torchquad_gb300.h pointing at them.  A state
also owns its scratch workspace (its size depends on the state's shape).
"""
from __future__ import annotations

import ctypes

import torch

from .. import _lib as L


def n_strat_for(N_increment, dim):
    """vegas_stratification.py:27-28 (at least one step per dimension)."""
    n = int((N_increment / 4.0) ** (1.0 / dim))
    n = 1000 if n > 1000 else n
    return max(1, n)


class VegasDevice:
    def __init__(self, dim, dtype, n_bins, n_strat, device, domain=None, stats_slots=64):
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
        self.rng_offset = torch.zeros((1,), dtype=torch.int64, device=device)
        self.stats = torch.zeros((max(1, stats_slots), 4), dtype=torch.float64, device=device)
        self.flags = torch.zeros((4,), dtype=torch.int32, device=device)
        self.scalars = torch.zeros((4,), dtype=torch.float64, device=device)
        self.control = torch.zeros((8,), dtype=torch.int64, device=device)
        self.params = torch.zeros((2 + 2 * dim,), dtype=torch.float64, device=device)
        if domain is None:
            domain = torch.tensor([[0.0, 1.0]] * dim, **f)
        self.domain = domain.detach().to(device=device, dtype=dtype).contiguous()
        self.struct = L.VegasState()
        self._fill_struct()
        self.ref = ctypes.byref(self.struct)
        nbytes = L.lib().tq_vegas_workspace_size(self.ref)
        if nbytes == 0:
            raise ValueError("invalid VEGAS state shape")
        self.ws = torch.zeros((int(nbytes),), dtype=torch.uint8, device=device)
        L.check(L.lib().tq_vegas_init(self.ref, L.stream_handle()), "tq_vegas_init")
        L.count_launches(1)

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

    def ensure_slots(self, n):
        if n > self.stats.shape[0]:
            new = torch.zeros((max(n, 2 * self.stats.shape[0]), 4), dtype=torch.float64, device=self.device)
            new[: self.stats.shape[0]] = self.stats
            self.stats = new
            self.struct.stats = self.stats.data_ptr()
            self.struct.n_stat_slots = self.stats.shape[0]

    def set_domain(self, domain):
        """Copy a domain into the state's own buffer (its address stays)."""
        self.domain.copy_(domain.detach().to(device=self.device, dtype=self.dtype))

    def reinit(self):
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
        p, n = self._ws()
        L.check(L.lib().tq_vegas_get_nh(self.ref, p, n, L.stream_handle()), "tq_vegas_get_nh")
        L.count_launches(2)

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
