"""Halton sequence, restated in NumPy (test oracle).

Test infrastructure only: the product path never imports this module.

Follows tf_quant_finance/math/random_ops/halton/halton_impl.py:
  sample          halton_impl.py:59-299 (digits by floor division and mod in
                  the output dtype, coefficients / radix / weight summed over
                  the digit positions, optional Owen scrambling + zero
                  correction)
  _randomize      :302-318 (gather from perms[k * sum(p) + offset_d + digit])
  _get_indices    :346-375 (index = sequence index + 1)
  _base_expansion_size, _MAX_SIZES_BY_AXES  :378-533 (floor(log n / log p) + 1
                  of the largest index per dtype: 2^24 - 1 / 2^53 - 1)
The primes are generated here by a sieve (the k-th axis uses the k-th prime).
"""

from __future__ import annotations

import numpy as np

MAX_DIMENSION = 1000
MAX_INDEX = {np.dtype(np.float32): 2 ** 24 - 1, np.dtype(np.float64): 2 ** 53 - 1}
NUM_COEFFS = {np.dtype(np.float32): 24, np.dtype(np.float64): 54}


def primes(n):
    """The first n primes."""
    limit = 16
    while True:
        sieve = np.ones(limit, bool)
        sieve[:2] = False
        for i in range(2, int(limit ** 0.5) + 1):
            if sieve[i]:
                sieve[i * i::i] = False
        p = np.nonzero(sieve)[0]
        if len(p) >= n:
            return p[:n]
        limit *= 2


def max_sizes(dim, dtype):
    """Digit positions per axis: floor(log(max index) / log(p)) + 1 in float64."""
    p = primes(dim).astype(np.int64)
    return (np.floor(np.log(MAX_INDEX[np.dtype(dtype)]) / np.log(p)) + 1).astype(np.int64)


def sample(dim, sequence_indices, dtype, perms=None, zero_correction=None):
    """[n, dim] points; perms [num_coeffs * sum(p)] and zero_correction [dim]
    give the scrambled sequence (randomized=True with randomization_params)."""
    dtype = np.dtype(dtype)
    dt_ = dtype.type
    idx = (np.asarray(sequence_indices, np.int64) + 1).astype(dtype).reshape(-1, 1, 1)
    p_int = primes(dim).astype(np.int64)
    radixes = p_int.astype(dtype).reshape(dim, 1)
    ms = max_sizes(dim, dtype).reshape(dim, 1).astype(dtype)
    max_size = int(ms.max())
    expo = np.tile(np.arange(max_size, dtype=dtype), (dim, 1))
    mask = expo >= ms
    capped = np.where(mask, dt_(0), expo)
    weights = np.round(radixes ** capped).astype(dtype)
    coeffs = np.floor_divide(idx, weights).astype(dtype)
    coeffs = coeffs * (dt_(1) - mask.astype(dtype))
    coeffs = np.mod(coeffs, radixes).astype(dtype)
    if perms is None:
        coeffs = coeffs / radixes
        return np.sum(coeffs / weights, axis=-1).astype(dtype)
    nc = NUM_COEFFS[dtype]
    radix_sum = int(p_int.sum())
    offsets = np.cumsum(np.concatenate([[0], p_int[:-1]])).reshape(-1, 1) + np.arange(nc) * radix_sum
    ci = coeffs.astype(np.int64) + offsets[:, :max_size]
    permuted = np.asarray(perms, np.int64).reshape(-1)[ci].astype(dtype)
    permuted = permuted * (dt_(1) - mask.astype(dtype))
    permuted = permuted / radixes
    base = np.sum(permuted / weights, axis=-1).astype(dtype)
    return (base + np.asarray(zero_correction, dtype).reshape(-1)).astype(dtype)
