"""Halton sequence on the GPU (tff/math/random_ops/halton/halton_impl.py:59-375).

``sample(dim, num_results=None, sequence_indices=None, randomized=True,
randomization_params=None, seed=None, validate_args=False, dtype=None, name=None)``
returns ``(points [n, dim], HaltonParams or None)`` as the reference does.  The
unscrambled sequence is the reference's (digit expansion of index + 1 over
floor(log(max index) / log p) + 1 positions).  Owen scrambling uses
permutations and zero-correction uniforms drawn from this engine's Philox
stream (``tqf_halton_permutations``): a seed reproduces them, but they are not
TensorFlow's ``stateless_random_shuffle`` output, so scrambled points match
the reference in distribution, not bit for bit.  Passing ``randomization_params``
reuses a previous call's permutations exactly, as in the reference.
"""

from __future__ import annotations

import dataclasses
from functools import lru_cache

import numpy as np
import torch

from tqf import _lib
from tqf.errors import InvalidArgumentError

MAX_DIMENSION = 1000
_MAX_INDEX = {torch.float32: 2 ** 24 - 1, torch.float64: 2 ** 53 - 1}
_NUM_COEFFS = {torch.float32: 24, torch.float64: 54}


@dataclasses.dataclass
class HaltonParams:
    """Randomization parameters (halton_impl.py:41-55): perms
    [num_coeffs * sum(primes)] int32 and zero_correction [dim]."""
    perms: torch.Tensor
    zero_correction: torch.Tensor


@lru_cache(maxsize=None)
def _primes(n: int) -> np.ndarray:
    limit = 16
    while True:
        sieve = np.ones(limit, bool)
        sieve[:2] = False
        for i in range(2, int(limit ** 0.5) + 1):
            if sieve[i]:
                sieve[i * i::i] = False
        p = np.nonzero(sieve)[0]
        if len(p) >= n:
            return p[:n].astype(np.int64)
        limit *= 2


def _max_sizes(dim: int, dtype: torch.dtype) -> np.ndarray:
    """floor(log(max index) / log(p)) + 1 in float64 (halton_impl.py:378-400, 530-533)."""
    return (np.floor(np.log(_MAX_INDEX[dtype]) / np.log(_primes(dim))) + 1).astype(np.int32)


@lru_cache(maxsize=None)
def _tables(dim: int, dtype: torch.dtype, device_index: int):
    device = torch.device("cuda", device_index)
    p = _primes(dim)
    offsets = np.concatenate([[0], np.cumsum(p[:-1])]).astype(np.int32)
    return (torch.as_tensor(p.astype(np.int32)).to(device), torch.as_tensor(_max_sizes(dim, dtype)).to(device),
            torch.as_tensor(offsets).to(device), int(p.sum()))


def _torch_dtype(dtype):
    if dtype is None:
        return torch.float32
    if isinstance(dtype, torch.dtype):
        return dtype
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[np.dtype(dtype)]


def _seed_value(seed) -> int:
    if seed is None:
        return int(torch.randint(0, 2 ** 62, (1,)).item())
    a = np.asarray(seed).reshape(-1).astype(np.int64)
    v = 0
    for x in a:
        v = (v * 0x9E3779B97F4A7C15 + int(x) + 0x632BE59BD9B4E019) & ((1 << 64) - 1)
    return v


def make_params(dim: int, seed=None, dtype=None) -> HaltonParams:
    """Owen-scrambling parameters for dim axes from the seed."""
    td = _torch_dtype(dtype)
    device = _lib.require_cuda()
    primes_t, ms_t, off_t, radix_sum = _tables(dim, td, device.index or 0)
    nc = _NUM_COEFFS[td]
    perms = torch.empty(nc * radix_sum, dtype=torch.int32, device=device)
    uni = torch.empty(dim, dtype=torch.float64, device=device)
    _lib.call("tqf_halton_permutations", dim, nc, primes_t.data_ptr(), off_t.data_ptr(), radix_sum,
              _seed_value(seed), perms.data_ptr(), uni.data_ptr(), _lib.stream_ptr(device))
    # zero correction: uniform / p^max_size in the output dtype (halton_impl.py:289-297)
    scale = torch.as_tensor(_primes(dim).astype(np.float64) ** _max_sizes(dim, td).astype(np.float64)).to(device)
    zc = (uni.to(td) / scale.to(td))
    return HaltonParams(perms, zc)


def sample(dim: int, num_results=None, sequence_indices=None, randomized: bool = True, randomization_params=None,
           seed=None, validate_args: bool = False, dtype=None, name=None, normal: bool = False):
    """Returns (points [n, dim], HaltonParams | None).  ``normal`` (extension)
    returns sqrt(2) erfinv(2u - 1) of the points instead (the quasi-normal draws
    of multivariate_normal.py:417-420), fused in the kernel."""
    del name
    if (num_results is None) == (sequence_indices is None):
        raise ValueError("Either `num_results` or `sequence_indices` must be specified but not both.")
    td = _torch_dtype(dtype)
    if validate_args and (dim < 1 or dim > MAX_DIMENSION):
        raise InvalidArgumentError(f"`dim` should be in [1, {MAX_DIMENSION}], got {dim}")
    if dim < 1 or dim > MAX_DIMENSION:
        raise ValueError(f"`dim` should be in [1, {MAX_DIMENSION}], got {dim}")
    device = _lib.require_cuda()
    idx_t = None
    if sequence_indices is not None:
        si = sequence_indices if isinstance(sequence_indices, torch.Tensor) else torch.as_tensor(
            np.asarray(sequence_indices))
        idx_t = si.to(device=device, dtype=torch.int64).reshape(-1).contiguous()
        n = int(idx_t.numel())
        if validate_args and n and int(idx_t.max().item()) + 1 > _MAX_INDEX[td]:
            raise InvalidArgumentError(f"Maximum sequence index exceeded for dtype {td}")
    else:
        n = int(num_results.item() if isinstance(num_results, torch.Tensor) else num_results)
        if validate_args and n > _MAX_INDEX[td]:
            raise InvalidArgumentError(f"Maximum sequence index exceeded for dtype {td}")
    primes_t, ms_t, off_t, radix_sum = _tables(dim, td, device.index or 0)
    params = None
    if randomized:
        params = randomization_params if randomization_params is not None else make_params(dim, seed, td)
        if not isinstance(params, HaltonParams):
            params = HaltonParams(*params)
    out = torch.empty((n, dim), dtype=td, device=device)
    a = _lib.HaltonArgs()
    a.dim = dim
    kinds = {(torch.float32, False): _lib.SOBOL_F32, (torch.float64, False): _lib.SOBOL_F64,
             (torch.float32, True): _lib.SOBOL_NORMAL_F32, (torch.float64, True): _lib.SOBOL_NORMAL_F64}
    a.out_kind = kinds[(td, bool(normal))]
    a.num_results = n
    a.first_index = 0
    a.sequence_indices = idx_t.data_ptr() if idx_t is not None else None
    a.primes, a.max_sizes = primes_t.data_ptr(), ms_t.data_ptr()
    if params is not None:
        perms = params.perms.to(device=device, dtype=torch.int32).contiguous()
        zc = params.zero_correction.to(device=device, dtype=td).contiguous()
        a.perms, a.perm_offsets, a.radix_sum = perms.data_ptr(), off_t.data_ptr(), radix_sum
        a.zero_correction = zc.data_ptr()
    a.out = out.data_ptr()
    _lib.call("tqf_halton_sample", a, _lib.stream_ptr(device))
    return out, (params if randomized else None)


def normal_draws(num_normal_draws: int, num_time_steps: int, num_paths: int, randomized: bool, seed=None,
                 skip: int = 0, dtype=torch.float32):
    """[steps, N, d] quasi-normal draws (tff/models/utils.py:20-128 with HALTON):
    point index skip + path, dimension step * d + c."""
    K = int(num_normal_draws) * int(num_time_steps)
    if K > MAX_DIMENSION:
        raise ValueError(f"Halton draws need num_normal_draws * num_time_steps <= {MAX_DIMENSION}, got {K}")
    pts, _ = sample(K, sequence_indices=torch.arange(int(skip), int(skip) + int(num_paths)), randomized=randomized,
                    seed=seed, dtype=dtype, normal=True)
    return pts.reshape(int(num_paths), int(num_time_steps), int(num_normal_draws)).permute(1, 0, 2).contiguous()


__all__ = ["sample", "HaltonParams", "make_params", "normal_draws"]
