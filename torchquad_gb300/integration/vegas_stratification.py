"""VEGASStratification (reference: integration/vegas_stratification.py:7-165)
on device state: dampened cube probabilities ``dh``, per-cube sums ``JF``,
``JF2`` and the stratified sampling of ``get_Y``."""
from __future__ import annotations

import torch

from .. import _lib as L
from ._vegas_state import VegasDevice, n_strat_for


class VEGASStratification:
    def __init__(self, N_increment, dim, rng, backend=None, dtype=torch.float32, beta=0.75,
                 _device_state=None):
        if backend not in (None, "torch"):
            raise ValueError(f"Unsupported numerical backend: {backend}")
        self.rng = rng
        self.dim = dim
        self.N_strat = n_strat_for(N_increment, dim)  # EQ 41
        self.beta = beta
        self.N_cubes = self.N_strat**self.dim
        self.V_cubes = (1.0 / self.N_strat) ** self.dim
        self.dtype = dtype
        self.backend = "torch"
        self._dev = _device_state or VegasDevice(dim, dtype, 2, self.N_strat, L.require_cuda())
        if self._dev.n_strat != self.N_strat:
            raise ValueError("device state has a different stratification")
        self._nevals = None  # the tensor whose prefix cube_start holds

    @property
    def dh(self):
        d = self._dev
        if d.dh_pending:  # a fused run ended with update_DH's normalisation pending
            d.dh_pending = False
            s = d.scalars[0].to(d.dtype)
            d.dh.copy_(torch.where(s != 0, d.dh / s, d.dh))
            d.control[2] = 0  # normalised: get_NH must not divide again
        return d.dh

    @property
    def JF(self):
        return self._dev.jf

    @property
    def JF2(self):
        return self._dev.jf2

    @property
    def strat_counts(self):
        return self._dev.neval.to(self.dtype)

    def get_NH(self, nevals_exp):
        """Evaluations per cube: max(2, floor(dh * nevals_exp)) (EQ 44)."""
        self._dev.get_nh(nevals_exp, normalize=False)
        self._nevals = self._dev.neval
        return self._dev.neval

    def _sync_prefix(self, nevals):
        if nevals is not self._nevals:
            nevals = nevals.to(self._dev.device, torch.int64)
            self._dev.neval.copy_(nevals)
            self._dev.cube_start[0] = 0
            torch.cumsum(nevals, 0, out=self._dev.cube_start[1:])
            self._nevals = self._dev.neval

    def get_Y(self, nevals):
        """Stratified sample points: for each cube its nevals[c] points
        (cube position + uniform) / N_strat, in cube order."""
        self._sync_prefix(nevals)
        M = int(self._dev.cube_start[-1].item())
        u = self.rng.uniform(size=[M, self.dim], dtype=self.dtype)
        u = torch.as_tensor(u).to(self._dev.device, self.dtype).contiguous()
        return self._dev.strat_points(u)

    def accumulate_weight(self, nevals, weight_all_cubes):
        """JF[c] = sum of the cube's weights, JF2[c] = sum of their squares."""
        self._sync_prefix(nevals)
        self._dev.jf.zero_()
        self._dev.jf2.zero_()
        w = weight_all_cubes.detach().to(self._dev.device, self.dtype).contiguous()
        self._dev.accumulate(w, w, False, True)  # y is not read for the cube sums
        return self._dev.jf, self._dev.jf2

    def update_DH(self, slot=0):
        """Dampened counts dh proportional to the cube variances^beta,
        normalised (EQ 42); also fills the iteration statistics slot."""
        self._dev.finish(self.beta, slot)
        s = self._dev.scalars[0].to(self.dtype)
        self._dev.dh.copy_(torch.where(s != 0, self._dev.dh / s, self._dev.dh))
