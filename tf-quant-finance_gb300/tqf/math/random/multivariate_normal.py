"""RandomType and multivariate normal draws (tff/math/random_ops/multivariate_normal.py).

PSEUDO / STATELESS (and their antithetic variants) draw from this project's
counter-based Philox4x32-10 stream; SOBOL from the Sobol kernels.  The draw
for row n and event dimension k is a pure function of (key, n, k), so draws
of a smaller sample are a prefix of a larger one (the prefix-stability
property tested in multivariate_normal_test.py:366-380).
"""

from __future__ import annotations

import enum
import os

import numpy as np
import torch

from tqf import _lib
from tqf.errors import InvalidArgumentError


@enum.unique
class RandomType(enum.Enum):
    """Types of random number sequences (multivariate_normal.py:27-44)."""

    PSEUDO = 0
    STATELESS = 1
    HALTON = 2
    HALTON_RANDOMIZED = 3
    SOBOL = 4
    PSEUDO_ANTITHETIC = 5
    STATELESS_ANTITHETIC = 6


_ANTITHETIC = (RandomType.PSEUDO_ANTITHETIC, RandomType.STATELESS_ANTITHETIC)
_STATELESS = (RandomType.STATELESS, RandomType.STATELESS_ANTITHETIC)


def is_antithetic(random_type) -> bool:
    return random_type in _ANTITHETIC


def philox_key(random_type, seed) -> tuple[int, int]:
    """Maps the reference's seed conventions onto a Philox key.

    PSEUDO*: a Python int (key = its low/high 32 bits) or None (fresh random
    key).  STATELESS*: an integer pair [a, b] -> key (a, b); missing seed
    raises ValueError as in multivariate_normal.py:265-268.
    """
    if random_type in _STATELESS:
        if seed is None:
            raise ValueError("`seed` should be specified if the `random_type` is `STATELESS` or "
                             "`STATELESS_ANTITHETIC`")
        s = np.asarray(seed.cpu() if isinstance(seed, torch.Tensor) else seed).reshape(-1)
        if s.size != 2:
            raise ValueError(f"STATELESS seed must have shape [2], got {s.shape}")
        return int(s[0]) & 0xFFFFFFFF, int(s[1]) & 0xFFFFFFFF
    if seed is None:
        raw = int.from_bytes(os.urandom(8), "little")
        return raw & 0xFFFFFFFF, raw >> 32
    s = int(np.asarray(seed.cpu() if isinstance(seed, torch.Tensor) else seed).reshape(-1)[0])
    return s & 0xFFFFFFFF, (s >> 32) & 0xFFFFFFFF


def philox_draws(random_type, seed, num_paths: int, path_offset: int = 0) -> _lib.Draws:
    """tqf_draws block for in-kernel generation over `num_paths` paths."""
    k0, k1 = philox_key(random_type, seed)
    d = _lib.Draws()
    d.source = _lib.DRAWS_PHILOX
    d.key0, d.key1 = k0, k1
    d.path_offset = int(path_offset)
    if is_antithetic(random_type):
        if num_paths % 2:
            raise InvalidArgumentError(
                "First dimension of `sample_shape` should be even for PSEUDO_ANTITHETIC random type")
        d.antithetic = 1
        d.antithetic_half = num_paths // 2
    return d


def sobol_draws(num_normal_draws: int, num_time_steps: int, num_paths: int, skip: int = 0,
                device: torch.device | None = None):
    """(tqf_draws, direction numbers to keep alive) for Sobol normals computed
    inside the path kernel: the SOBOL branch of generate_mc_normal_draws
    (tff/models/utils.py:95-127) for `num_paths` paths, point skip + 1 + n,
    dimension step * num_normal_draws + c, nd digits of the whole request."""
    from tqf.math.random import sobol
    device = device or _lib.require_cuda()
    dim = max(int(num_normal_draws) * int(num_time_steps), 1)
    sobol._validate(dim, int(num_paths), int(skip), False)
    v = sobol.device_direction_numbers(dim, device)
    d = _lib.Draws()
    d.source = _lib.DRAWS_SOBOL
    d.ptr = v.data_ptr()
    d.key0 = sobol.num_digits(int(num_paths), int(skip))
    d.key1 = int(num_normal_draws)
    d.path_offset = int(skip)
    return d, v


def memory_draws(draws: torch.Tensor, path_axis: int, step_axis: int) -> _lib.Draws:
    """tqf_draws block reading a 3-D tensor in place (any layout, any strides)."""
    d = _lib.Draws()
    d.source = _lib.DRAWS_MEMORY
    d.ptr = draws.data_ptr()
    st = draws.stride()
    d.stride_path = st[path_axis]
    d.stride_step = st[step_axis]
    d.stride_comp = st[2]
    return d


def philox_normal_draws(random_type, seed, num_normal_draws: int, num_time_steps: int,
                        num_paths: int, dtype: torch.dtype, path_offset: int = 0) -> torch.Tensor:
    """Materialised [steps, N, d] draws of the Philox stream."""
    device = _lib.require_cuda()
    dr = philox_draws(random_type, seed, num_paths, path_offset)
    out = torch.empty((num_time_steps, num_paths, num_normal_draws), dtype=dtype, device=device)
    _lib.call("tqf_philox_normal_draws", dr, num_normal_draws, num_time_steps, num_paths,
              _lib.dtype_code(dtype), out.data_ptr(), _lib.stream_ptr(device))
    return out


def _to_device(x, dtype, device):
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype)
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=device)


def _resolve_dtype(dtype, *tensors):
    if dtype is not None:
        if isinstance(dtype, torch.dtype):
            return dtype
        return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[np.dtype(dtype)]
    for t in tensors:
        if isinstance(t, torch.Tensor) and t.is_floating_point():
            return t.dtype
        if isinstance(t, np.ndarray) and t.dtype.kind == "f":
            return torch.float64 if t.dtype == np.float64 else torch.float32
    return torch.float32


def quasi_layout(points, sample_shape, batch_shape):
    """Arranges low-discrepancy points [n * prod(batch), dim] as sample_shape +
    batch_shape (the last batch axis is the event dimension).

    Element (s, b_1, ..., b_k, c) takes component c of point q, q the C-order
    index of (b_k, ..., b_1, s): the reference reshapes the transposed points
    to reverse(batch_shape) + sample_shape and moves the sample axes to the
    front (multivariate_normal.py:370-416).
    """
    bax = tuple(int(b) for b in batch_shape[:-1])
    dim = int(batch_shape[-1])
    n = int(np.prod(sample_shape)) if len(sample_shape) else 1
    k = len(bax)
    z = points.reshape(tuple(reversed(bax)) + (n, dim))
    z = z.permute((k,) + tuple(range(k - 1, -1, -1)) + (k + 1,))
    return z.reshape(tuple(sample_shape) + tuple(batch_shape))


def multivariate_normal(sample_shape, mean=None, covariance_matrix=None, scale_matrix=None,
                        random_type=None, validate_args=False, seed=None, dtype=None, name=None,
                        **kwargs):
    """Draws from N(mean, scale scale^T) with shape sample_shape + batch + [dim]
    (multivariate_normal.py:47-245)."""
    del name, validate_args
    if covariance_matrix is not None and scale_matrix is not None:
        raise ValueError("Only one of covariance matrix or scale matrix must be specified")
    random_type = RandomType.PSEUDO if random_type is None else random_type
    device = _lib.require_cuda()
    dtype = _resolve_dtype(dtype, mean, scale_matrix, covariance_matrix)
    mean = _to_device(mean, dtype, device)
    scale = _to_device(scale_matrix, dtype, device)
    if covariance_matrix is not None:
        cov = _to_device(covariance_matrix, torch.float64, device)
        scale = torch.linalg.cholesky(cov).to(dtype)
    if mean is None and scale is None:
        raise ValueError("At least one of `mean`, `covariance_matrix` or `scale_matrix` must be given")
    batch_shape = tuple(mean.shape) if mean is not None else tuple(scale.shape[:-1])
    dim = batch_shape[-1]
    sample_shape = tuple(int(s) for s in (np.asarray(sample_shape).reshape(-1)))
    n = int(np.prod(sample_shape)) if sample_shape else 1
    rows = n * int(np.prod(batch_shape[:-1]))
    if random_type in (RandomType.PSEUDO, RandomType.STATELESS) + _ANTITHETIC:
        if is_antithetic(random_type) and (not sample_shape or sample_shape[0] % 2):
            raise InvalidArgumentError(
                "First dimension of `sample_shape` should be even for PSEUDO_ANTITHETIC random type")
        z = philox_normal_draws(random_type, seed, dim, 1, rows, dtype)[0]
        # Antithetic rows [half, 2 half) are the negated rows [0, half), so
        # mean + scale z reproduces concat([m + s, 2 m - (m + s)]).
        z = z.reshape(sample_shape + batch_shape)
    elif random_type in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
        skip = int(kwargs.get("skip", 0) or 0)
        total = n * int(np.prod(batch_shape[:-1]))
        if random_type == RandomType.SOBOL:
            from tqf.math.random import sobol
            points = sobol.sample_normal(dim, total, skip=skip, dtype=dtype)
        else:
            from tqf.math.random import halton
            points, _ = halton.sample(dim, sequence_indices=torch.arange(skip, skip + total),
                                      randomized=random_type == RandomType.HALTON_RANDOMIZED,
                                      randomization_params=kwargs.get("randomization_params"), seed=seed,
                                      dtype=dtype, normal=True)
        z = quasi_layout(points, sample_shape, batch_shape)
    else:
        raise NotImplementedError(f"unsupported random_type {random_type}")
    if scale is not None:
        z = torch.einsum("...ij,...j->...i", scale, z)
    if mean is not None:
        z = mean + z
    return z


__all__ = ["RandomType", "multivariate_normal", "philox_key", "philox_draws", "memory_draws",
           "philox_normal_draws", "is_antithetic", "quasi_layout"]
