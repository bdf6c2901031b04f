"""Philox4x32-10 counter-based RNG in NumPy (test infrastructure only).

Algorithm: Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
1, 2, 3", SC'11 (Random123).  Ten rounds of the 4x32 Philox bijection with the
published multipliers and Weyl key increments.

The sampling stream used by the MPS sampler is defined as:
    counter = (shot & 0xffffffff, shot >> 32, site, 0)
    key     = (seed & 0xffffffff, seed >> 32)
    u       = (word0 >> 8) * 2**-24          (24-bit uniform in [0, 1))
and a qubit outcome is 1 iff u >= p0 / (p0 + p1) (with the reference's 1e-15
probability floor applied first).  The CUDA sampler implements the same stream.
"""
import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10.  All arguments are uint32 arrays (broadcast)."""
    c0 = np.asarray(c0, dtype=np.uint32)
    c1 = np.asarray(c1, dtype=np.uint32)
    c2 = np.asarray(c2, dtype=np.uint32)
    c3 = np.asarray(c3, dtype=np.uint32)
    k0 = np.asarray(k0, dtype=np.uint32)
    k1 = np.asarray(k1, dtype=np.uint32)
    c0, c1, c2, c3, k0, k1 = np.broadcast_arrays(c0, c1, c2, c3, k0, k1)
    c0, c1, c2, c3 = (x.astype(np.uint32).copy() for x in (c0, c1, c2, c3))
    k0 = k0.astype(np.uint32).copy()
    k1 = k1.astype(np.uint32).copy()
    with np.errstate(over="ignore"):
        for r in range(10):
            if r > 0:
                k0 = (k0 + W0).astype(np.uint32)
                k1 = (k1 + W1).astype(np.uint32)
            p0 = M0 * c0.astype(np.uint64)
            p1 = M1 * c2.astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & MASK).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & MASK).astype(np.uint32)
            c0, c1, c2, c3 = (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0)
    return c0, c1, c2, c3


def sample_uniforms(seed, shots, site):
    """Uniforms u[shot] for one site of the sampling stream (see module doc)."""
    shots = np.asarray(shots, dtype=np.uint64)
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    w0, _, _, _ = philox4x32_10(
        (shots & MASK).astype(np.uint32),
        (shots >> np.uint64(32)).astype(np.uint32),
        np.uint32(site), np.uint32(0),
        np.uint32(seed & 0xFFFFFFFF), np.uint32(seed >> 32))
    return (w0 >> np.uint32(8)).astype(np.float64) * (2.0 ** -24)


def gaussian_pairs(seed, idx, stream):
    """Box-Muller standard normals from Philox words (used for sketch matrices
    and inverse-iteration start vectors in tests)."""
    idx = np.asarray(idx, dtype=np.uint64)
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    w0, w1, _, _ = philox4x32_10(
        (idx & MASK).astype(np.uint32), (idx >> np.uint64(32)).astype(np.uint32),
        np.uint32(stream), np.uint32(0x5EED),
        np.uint32(seed & 0xFFFFFFFF), np.uint32(seed >> 32))
    u1 = ((w0 >> np.uint32(8)).astype(np.float64) + 1.0) * (2.0 ** -24)
    u2 = (w1 >> np.uint32(8)).astype(np.float64) * (2.0 ** -24)
    r = np.sqrt(-2.0 * np.log(u1))
    return r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)
