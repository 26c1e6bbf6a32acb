"""Sobol sequence restatement (tff/math/random_ops/sobol/sobol_impl.py).

Integers are computed per point by the direct XOR definition instead of the
reference's [nd, n, dim] product tensor (sobol_impl.py:139-157), which gives
the same integers with O(n·dim) memory.
"""

from __future__ import annotations

import math
import os

import numpy as np

DATA_FILE = os.path.join(
    os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
    "tf-quant-finance_gb300", "tqf", "data", "new-joe-kuo-6.21201")


def load_data(path: str = DATA_FILE, max_dims: int | None = None):
    """Parses the Joe–Kuo file (sobol_impl.py:237-261).

    Returns (polynomial coefficients a_k = 2^s + 2a + 1, initial direction
    numbers [18, dims]).
    """
    polys = []
    inits = []
    with open(path) as f:
        next(f)  # header
        for line in f:
            tok = line.split()
            if not tok:
                continue
            s, a = int(tok[1]), int(tok[2])
            polys.append(2 ** s + 2 * a + 1)
            inits.append([int(t) for t in tok[3:]])
            if max_dims is not None and len(polys) >= max_dims:
                break
    init = np.zeros((18, len(polys)), dtype=np.int64)
    for k, ms in enumerate(inits):
        init[: len(ms), k] = ms
    return np.array(polys, dtype=np.int64), init


def compute_direction_numbers(dim: int, path: str = DATA_FILE) -> np.ndarray:
    """m_kj, shape [dim, 32] (sobol_impl.py:171-197), as Python ints in int64."""
    polys, init = load_data(path, max_dims=max(dim - 1, 1))
    m = np.zeros((dim, 32), dtype=np.int64)
    m[0, :] = 1
    for k in range(dim - 1):
        a_k = int(polys[k])
        deg = int(math.floor(math.log2(a_k)))
        m[k + 1, :deg] = init[:deg, k]
        for j in range(deg, 32):
            val = int(m[k + 1, j - deg])
            for i in range(deg):
                if (a_k >> i) & 1:
                    val ^= int(m[k + 1, j - deg + i]) << (deg - i)
            m[k + 1, j] = val & 0xFFFFFFFF
    return m


def num_digits(num_results: int, skip: int) -> int:
    """ceil(log(skip + n + 1) / log 2) in float64 (sobol_impl.py:118-123)."""
    return int(math.ceil(math.log(float(skip + num_results + 1)) / math.log(2.0)))


def sample_int(dim: int, num_results: int, skip: int = 0, nd: int | None = None,
               m: np.ndarray | None = None) -> np.ndarray:
    """Integer Sobol points, indices skip+1 .. skip+n, shape [n, dim] (uint64).

    x(i)_d = XOR_j bit_j(i) * (m_dj << (nd - 1 - j))  (sobol_impl.py:128-157).
    `nd` defaults to the reference's value for this request; chunked callers
    pass the global nd.
    """
    if nd is None:
        nd = num_digits(num_results, skip)
    if m is None:
        m = compute_direction_numbers(dim)
    v = np.zeros((dim, nd), dtype=np.uint64)
    for j in range(nd):
        v[:, j] = (m[:dim, j].astype(np.uint64) << np.uint64(nd - 1 - j)) & np.uint64(0xFFFFFFFFFFFF)
    idx = np.arange(skip + 1, skip + 1 + num_results, dtype=np.uint64)
    out = np.zeros((num_results, dim), dtype=np.uint64)
    for j in range(nd):
        bit = ((idx >> np.uint64(j)) & np.uint64(1)).astype(bool)
        out[bit] ^= v[:, j][None, :]
    return out


def sample(dim: int, num_results: int, skip: int = 0, dtype=np.float32, nd: int | None = None,
           m: np.ndarray | None = None) -> np.ndarray:
    """Float Sobol points: cast(int) / 2^nd in `dtype` (sobol_impl.py:159-167)."""
    if nd is None:
        nd = num_digits(num_results, skip)
    ints = sample_int(dim, num_results, skip, nd=nd, m=m)
    return (ints.astype(dtype) / dtype(2.0 ** nd)).astype(dtype)


def normal_from_uniform(u: np.ndarray) -> np.ndarray:
    """erfinv((u - 0.5) * 2) * sqrt(2) in u's dtype (multivariate_normal.py:420)."""
    from scipy.special import erfinv
    dt = u.dtype.type
    x = (u - dt(0.5)) * dt(2)
    return (erfinv(x.astype(np.float64)).astype(u.dtype) * dt(np.sqrt(2.0))).astype(u.dtype)
