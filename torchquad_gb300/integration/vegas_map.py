"""VEGASMap (reference: integration/vegas_map.py:9-261) on device state.

The map arrays (``x_edges`` [dim, B+1], ``dx_edges`` [dim, B]) stay on the
GPU; ``get_X``/``get_Jac`` run the map kernel, ``accumulate_weight`` the
histogram kernel and ``update_map`` the smoothing + edge-update kernel.
The interval weights accumulate in fp64.
"""
from __future__ import annotations

import warnings

import torch

from .. import _lib as L
from ._vegas_state import VegasDevice


def _cannot_update_warning():
    warnings.warn(
        "Cannot update the VEGASMap. This can happen with an integrand which evaluates to zero "
        "everywhere.",
        RuntimeWarning,
    )


class VEGASMap:
    """The adaptive map of VEGAS+ on [0, 1]^dim."""

    def __init__(self, N_intervals, dim, backend=None, dtype=torch.float32, alpha=0.5, _device_state=None):
        if backend not in (None, "torch"):
            raise ValueError(f"Unsupported numerical backend: {backend}")
        self.dim = dim
        self.N_intervals = int(N_intervals)
        self.alpha = alpha
        self.backend = "torch"
        self.dtype = dtype
        self._dev = _device_state or VegasDevice(dim, dtype, N_intervals, 1, L.require_cuda())
        self._flags_seen = 0

    # ---- state views
    @property
    def x_edges(self):
        return self._dev.x_edges

    @property
    def dx_edges(self):
        return self._dev.dx_edges

    @property
    def weights(self):
        return self._dev.weights

    @property
    def counts(self):
        return self._dev.counts

    # ---- reference API
    def get_X(self, y):
        """Mapped points x for y [M, dim] in [0, 1) (EQ 9)."""
        return self._dev.map_points(self._as_state(y))[0]

    def get_Jac(self, y):
        """Jacobian of the map at y (EQ 12)."""
        return self._dev.map_points(self._as_state(y))[1]

    def get_X_and_Jac(self, y):
        return self._dev.map_points(self._as_state(y))

    def _get_interval_ID(self, y):
        return torch.floor(y * float(self.N_intervals)).to(torch.int64)

    def _get_interval_offset(self, y):
        y = y * float(self.N_intervals)
        return y - torch.floor(y)

    def accumulate_weight(self, y, jf_vec2):
        """weights[i, ID_i] += jf_vec2, counts[i, ID_i] += 1 (vegas_map.py:99-111)."""
        self._dev.accumulate(self._as_state(y), self._as_state(jf_vec2.detach()), True, False)

    @staticmethod
    def _smooth_map(weights, counts, alpha):
        """Smoothed, range-compressed weights (EQ 18-22); None if a
        dimension's weights are all zero."""
        dim, B = weights.shape
        dt = weights.dtype if weights.dtype in (torch.float32, torch.float64) else torch.float64
        dev = VegasDevice(dim, dt, B, 1, L.require_cuda())
        dev.weights.copy_(weights.to(dev.device, torch.float64))
        dev.counts.copy_(counts.to(dev.device, torch.int64))
        out = dev.smooth(alpha)
        if int(dev.flags[0].item()) != 0:
            return None
        return out

    def _reset_weight(self):
        self._dev.weights.zero_()
        self._dev.counts.zero_()

    def update_map(self):
        """Update the edges from the accumulated weights (Section II C)."""
        self._dev.update_map(self.alpha)
        self.check_flags()

    def check_flags(self, host_flags=None):
        """Emit the reference's warnings/errors for flags raised on the
        device since the last check (synchronises unless the flags were read
        back already and are passed in)."""
        f = self._dev.flags.cpu() if host_flags is None else host_flags
        if int(f[0]) > self._flags_seen:
            for _ in range(int(f[0]) - self._flags_seen):
                _cannot_update_warning()
            self._flags_seen = int(f[0])
        if int(f[1]):
            warnings.warn("Some calculated VEGASMap edges were infinite", RuntimeWarning)
            self._dev.flags[1] = 0
        if int(f[2]):
            self._dev.flags[2] = 0
            raise RuntimeError("Could not replace all infinite edges")

    def _as_state(self, t):
        t = torch.as_tensor(t)
        if t.device != self._dev.device or t.dtype != self.dtype:
            t = t.to(self._dev.device, self.dtype)
        return t.contiguous()
