"""Philox4x32-10 (Salmon et al., SC'11) and the uniform-number layout of
``tq_uniform`` (include/torchquad_gb300.h), vectorised in numpy.  The
reference draws torch.rand (rng.py:120-125); this is the stream the GB300
build draws instead and injects into the reference for parity."""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised bijection on uint32 arrays; returns 4 uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint32) for c in (c0, c1, c2, c3))
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    for _ in range(10):
        p0 = M0 * c0.astype(np.uint64)
        p1 = M1 * c2.astype(np.uint64)
        hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
        lo0 = (p0 & MASK).astype(np.uint32)
        hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
        lo1 = (p1 & MASK).astype(np.uint32)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        with np.errstate(over="ignore"):
            k0 = np.uint32((int(k0) + int(W0)) & 0xFFFFFFFF)
            k1 = np.uint32((int(k1) + int(W1)) & 0xFFFFFFFF)
    return c0, c1, c2, c3


def blocks(seed, stream_id, first_block, nblocks):
    b = np.arange(nblocks, dtype=np.uint64) + np.uint64(first_block)
    lo = (b & MASK).astype(np.uint32)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    s_lo = np.full(nblocks, stream_id & 0xFFFFFFFF, dtype=np.uint32)
    s_hi = np.full(nblocks, (stream_id >> 32) & 0xFFFFFFFF, dtype=np.uint32)
    return philox4x32_10(lo, hi, s_lo, s_hi, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)


def uniform(seed, stream_id, offset, numel, dtype):
    """Exactly the values tq_uniform writes (same counter layout)."""
    if dtype == np.float32:
        nb = (numel + 3) // 4
        r = np.stack(blocks(seed, stream_id, offset, nb), axis=1).reshape(-1)[:numel]
        return ((r >> np.uint32(8)).astype(np.float32) * np.float32(2.0**-24)).astype(np.float32)
    nb = (numel + 1) // 2
    r = np.stack(blocks(seed, stream_id, offset, nb), axis=1).reshape(-1, 2)[:numel]
    x = ((r[:, 1].astype(np.uint64) << np.uint64(32)) | r[:, 0].astype(np.uint64)) >> np.uint64(11)
    return x.astype(np.float64) * 2.0**-53


def blocks_for(numel, dtype):
    per = 2 if dtype == np.float64 else 4
    return (numel + per - 1) // per


class ReplayStream:
    """Counter-based stream with the RNG.uniform interface of the product
    (offset advanced per call), producing numpy arrays."""

    def __init__(self, seed, stream_id=0, offset=0):
        self.seed, self.stream_id, self.offset = seed, stream_id, offset

    def uniform(self, size, dtype):
        n = int(np.prod(size))
        out = uniform(self.seed, self.stream_id, self.offset, n, dtype).reshape(size)
        self.offset += blocks_for(n, dtype)
        return out
