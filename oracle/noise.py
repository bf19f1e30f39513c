"""ORACLE -- test infrastructure only.

Restatement of the range-noise step for checking rmg_noise_apply: the Philox4x32-10 counter-based
generator (Salmon, Moraes, Dror, Shaw, SC 2011) in numpy integer arithmetic (bit-exact), the
uniform and Box-Muller conversions in binary64, and rmagine's per-element noise arithmetic
(src/rmagine_cuda/src/noise/GaussianNoiseCuda.cu:9-31, RelGaussianNoiseCuda.cu:9-35,
UniformDustNoiseCuda.cu:8-52; CPU twins src/rmagine_core/src/noise/*.cpp).
"""
from __future__ import annotations

import numpy as np

M0, M1, W0, W1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57), np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32 with 10 rounds; all arguments uint32 arrays (broadcast)."""
    c = [np.asarray(x, np.uint32) for x in np.broadcast_arrays(c0, c1, c2, c3)]
    k0 = np.asarray(k0, np.uint32).copy()
    k1 = np.asarray(k1, np.uint32).copy()
    with np.errstate(over="ignore"):
        for r in range(10):
            if r > 0:
                k0 = (k0 + W0).astype(np.uint32)
                k1 = (k1 + W1).astype(np.uint32)
            p0 = M0 * c[0].astype(np.uint64)
            p1 = M1 * c[2].astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & MASK).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & MASK).astype(np.uint32)
            c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
    return c


def blocks(n_blocks, seed, call):
    """Philox blocks for counters (i, call) i < n_blocks: [n_blocks, 4] uint32."""
    i = np.arange(n_blocks, dtype=np.uint64)
    out = philox4x32_10((i & MASK).astype(np.uint32), (i >> np.uint64(32)).astype(np.uint32),
                        np.uint32(call & 0xFFFFFFFF), np.uint32(call >> 32),
                        np.uint32(seed & 0xFFFFFFFF), np.uint32(seed >> 32))
    return np.stack(out, axis=1)


def uniform01(x):
    """Odd multiples of 2^-24 in (0, 1) (exact in binary32)."""
    return (((np.asarray(x, np.uint32) >> np.uint32(8)) | np.uint32(1)).astype(np.float64) * 2.0 ** -24)


def normals(n, seed, call):
    """Standard normals for elements 0..n-1 (4 per Philox block, Box-Muller pairs) in binary64."""
    b = blocks((n + 3) // 4, seed, call)
    u = uniform01(b)
    r0 = np.sqrt(-2.0 * np.log(u[:, 0]))
    r1 = np.sqrt(-2.0 * np.log(u[:, 2]))
    z = np.stack([r0 * np.cos(2 * np.pi * u[:, 1]), r0 * np.sin(2 * np.pi * u[:, 1]),
                  r1 * np.cos(2 * np.pi * u[:, 3]), r1 * np.sin(2 * np.pi * u[:, 3])], axis=1)
    return z.reshape(-1)[:n]


def apply(kind, ranges, seed, call, mean=0.0, stddev=0.0, range_exp=1.0, hit_p=0.0, ret_p=0.0,
          max_range=10000.0):
    """Binary64 restatement; returns (new ranges float64, decided mask for dust)."""
    r = np.asarray(ranges, np.float32).astype(np.float64)
    n = r.size
    if kind in (0, 1):
        z = normals(n, seed, call)
        sd = stddev if kind == 0 else stddev * np.power(np.maximum(r, 0.0), range_exp)
        return np.where(r <= max_range, r + (z * sd + mean), r)
    b = blocks(n, seed, call)
    u = uniform01(b[:, :3])
    rr = np.minimum(r, max_range)
    p_hit = 1.0 - np.power(1.0 - hit_p, rr)
    nr = (u[:, 1].astype(np.float32) * rr.astype(np.float32)).astype(np.float64)
    p_ret = np.power(ret_p, nr)
    take = (u[:, 0] < p_hit) & (u[:, 2] < p_ret)
    return np.where(take, nr, r), (np.abs(u[:, 0] - p_hit), np.abs(u[:, 2] - p_ret))
