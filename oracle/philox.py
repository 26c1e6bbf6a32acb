"""Philox4x32-10 and the canonical normal stream (this project's own RNG).

Philox4x32-10 follows Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
as easy as 1, 2, 3" (SC'11): round (c0..c3) -> (hi(M1 c2) ^ c1 ^ k0,
lo(M1 c2), hi(M0 c0) ^ c3 ^ k1, lo(M0 c0)), key bumped by the Weyl constants
between rounds, ten rounds.  Pinned on the Random123 known-answer vectors in
tests/test_oracle_golden.py.

Canonical stream: the normal for (path n, draw dimension k) comes from
Philox block b = k // 4 (float32; k // 2 for float64) with counter
(b_lo, n_lo, n_hi, b_hi) and key (key0, key1); float32 normals are two
Box–Muller pairs from words (r0, r1) and (r2, r3).
"""

from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = 0x9E3779B9
W1 = 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0: int, k1: int):
    """Vectorised Philox4x32-10 on uint32 arrays; returns four uint32 arrays."""
    c0 = np.asarray(c0, dtype=np.uint64)
    c1 = np.asarray(c1, dtype=np.uint64)
    c2 = np.asarray(c2, dtype=np.uint64)
    c3 = np.asarray(c3, dtype=np.uint64)
    k0 = int(k0) & 0xFFFFFFFF
    k1 = int(k1) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ np.uint64(k0)), lo1, (hi0 ^ c3 ^ np.uint64(k1)), lo0
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return [x.astype(np.uint32) for x in (c0, c1, c2, c3)]


def _u01_oc_f32(r: np.ndarray) -> np.ndarray:
    """(0, 1] float32 built as on the device: (2 - 1.m_hi) - 0.m_lo * 2^-23."""
    r = r.astype(np.uint32)
    hi = ((np.uint32(0x3F800000) | (r >> np.uint32(9))).view(np.float32))
    lo = ((np.uint32(0x3F800000) | ((r << np.uint32(23)) >> np.uint32(9))).view(np.float32)) - np.float32(1)
    base = (np.float32(2) - hi).astype(np.float32)
    return (base.astype(np.float64) - lo.astype(np.float64) * 2.0 ** -23).astype(np.float32)


def _u01_co_f32(r: np.ndarray) -> np.ndarray:
    r = r.astype(np.uint32)
    return ((np.uint32(0x3F800000) | (r >> np.uint32(9))).view(np.float32) - np.float32(1)).astype(np.float32)


def box_muller_f32(a: np.ndarray, b: np.ndarray):
    """Exact-arithmetic model (float64) of the device float32 Box–Muller."""
    u1 = _u01_oc_f32(a).astype(np.float64)
    u2 = _u01_co_f32(b).astype(np.float64)
    rad = np.sqrt(-2.0 * np.log(u1))
    ang = (u2 - 0.5) * 2.0 * np.pi
    return rad * np.cos(ang), rad * np.sin(ang)


def box_muller_f64(r0, r1, r2, r3):
    m1 = (r0.astype(np.uint64) << np.uint64(21)) ^ (r1.astype(np.uint64) >> np.uint64(11))
    m2 = (r2.astype(np.uint64) << np.uint64(21)) ^ (r3.astype(np.uint64) >> np.uint64(11))
    u1 = (m1.astype(np.float64) + 1.0) * 2.0 ** -53
    u2 = m2.astype(np.float64) * 2.0 ** -53
    rad = np.sqrt(-2.0 * np.log(u1))
    return rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)


def normals(paths: np.ndarray, num_dims: int, key0: int, key1: int, dtype=np.float32,
            antithetic_half: int | None = None, path_offset: int = 0) -> np.ndarray:
    """Canonical stream z[p, k] for the given path indices and k < num_dims.

    Returns float64 values (the exact-arithmetic model of the device numbers).
    """
    paths = np.asarray(paths, dtype=np.int64)
    sign = np.ones(paths.shape, dtype=np.float64)
    src = paths.copy()
    if antithetic_half is not None:
        neg = src >= antithetic_half
        src[neg] -= antithetic_half
        sign[neg] = -1.0
    src = src + path_offset
    npb = 4 if dtype == np.float32 else 2
    nblocks = (num_dims + npb - 1) // npb
    out = np.zeros((len(paths), nblocks * npb), dtype=np.float64)
    n_lo = (src & 0xFFFFFFFF).astype(np.uint64)
    n_hi = ((src >> 32) & 0xFFFFFFFF).astype(np.uint64)
    for b in range(nblocks):
        bl = np.full(paths.shape, b & 0xFFFFFFFF, dtype=np.uint64)
        bh = np.full(paths.shape, b >> 32, dtype=np.uint64)
        r0, r1, r2, r3 = philox4x32_10(bl, n_lo, n_hi, bh, key0, key1)
        if npb == 4:
            z0, z1 = box_muller_f32(r0, r1)
            z2, z3 = box_muller_f32(r2, r3)
            out[:, 4 * b:4 * b + 4] = np.stack([z0, z1, z2, z3], axis=1)
        else:
            z0, z1 = box_muller_f64(r0, r1, r2, r3)
            out[:, 2 * b:2 * b + 2] = np.stack([z0, z1], axis=1)
    return out[:, :num_dims] * sign[:, None]


def normal_draws(num_paths: int, num_steps: int, d: int, key0: int, key1: int, dtype=np.float32,
                 antithetic: bool = False) -> np.ndarray:
    """[steps, N, d] draws of the canonical stream (the reference layout of
    generate_mc_normal_draws, tff/models/utils.py:95-127)."""
    half = num_paths // 2 if antithetic else None
    z = normals(np.arange(num_paths), num_steps * d, key0, key1, dtype=dtype, antithetic_half=half)
    return z.reshape(num_paths, num_steps, d).transpose(1, 0, 2)
