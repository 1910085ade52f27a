"""RNG (reference: integration/rng.py:5-152), counter-based.

The reference seeds torch's global generator and calls torch.rand.  This RNG
is a private Philox4x32-10 stream: key = seed, counter = a 64-bit block
offset that ``uniform`` advances by the blocks it consumes (4 fp32 or 2 fp64
values per block).  The same (seed, stream_id, offset) regenerates the same
numbers inside the fused kernels, so fused and materialised paths draw
identical points.  torch's global RNG state is never touched, which is what
the reference's ``torch_save_state=True`` option achieves.
"""
from __future__ import annotations

import math
import secrets

import torch

from .. import _lib as L
from . import _kernels as K


class RNG:
    """A seeded stream of uniform numbers in [0, 1) on the current CUDA device."""

    def __init__(self, backend="torch", seed=None, torch_save_state=False):
        if backend not in (None, "torch"):
            raise ValueError(f"Unsupported numerical backend: {backend}")
        if seed is None:
            seed = secrets.randbits(63)
        self.seed = int(seed) & ((1 << 64) - 1)
        self.stream_id = 0
        self.offset = 0  # Philox blocks consumed so far
        self._torch_save_state = torch_save_state

    @staticmethod
    def blocks_for(numel, dtype) -> int:
        per = 2 if dtype == torch.float64 else 4
        return (int(numel) + per - 1) // per

    def uniform(self, size, dtype):
        """Uniform numbers of shape ``size`` and ``dtype`` in [0, 1)."""
        if dtype not in (torch.float32, torch.float64):
            out = self.uniform(size, torch.float32)
            return out.to(dtype)
        device = L.require_cuda()
        size = [int(s) for s in size]
        out = K.uniform(self.seed, self.stream_id, self.offset, size, dtype, device)
        self.offset += self.blocks_for(math.prod(size), dtype)
        return out

    def reserve(self, numel, dtype) -> int:
        """Advance the stream as ``uniform`` would for ``numel`` values and
        return the block offset they start at (used by the fused kernels)."""
        start = self.offset
        self.offset += self.blocks_for(numel, dtype)
        return start

    def jax_get_key(self):
        raise NotImplementedError("JAX is not a backend of torchquad_gb300")

    def jax_set_key(self, key):
        raise NotImplementedError("JAX is not a backend of torchquad_gb300")
