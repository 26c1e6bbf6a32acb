"""Sobol sequence: drop-in for tff.math.random.sobol.sample
(tff/math/random_ops/sobol/sobol_impl.py:39-167).

Points are computed by the ``sobol_rowmajor_kernel`` of libtqf.so in the
reference's natural (non-Gray) order starting at index skip + 1, with the
reference's nd = ceil(log2(skip + n + 1)) integer scaling, so the integers
are bit-identical and the floats equal float(int) / 2^nd.
"""

from __future__ import annotations

import threading

import numpy as np
import torch

from tqf import _lib
from tqf.errors import InvalidArgumentError

_MAX_POSITIVE = 2 ** 31 - 1
_cache_lock = threading.Lock()
_host_table: np.ndarray | None = None
_dev_tables: dict[int, torch.Tensor] = {}


def direction_numbers(dim: int) -> np.ndarray:
    """Host uint32 [dim, 32]: v_dj = m_dj << (31 - j) (sobol_impl.py:171-197)."""
    global _host_table
    with _cache_lock:
        if _host_table is None or _host_table.shape[0] < dim:
            n = max(dim, 1024)
            n = min(n, 21201)
            if dim > 21201:
                raise InvalidArgumentError(f"Sobol dimension {dim} exceeds the 21201 of the Joe–Kuo table")
            out = np.zeros((n, 32), dtype=np.uint32)
            _lib.call("tqf_sobol_direction_numbers", _lib.JOE_KUO_PATH.encode(), n,
                      out.ctypes.data_as(_lib.c_vp))
            _host_table = out
            _dev_tables.clear()
        return _host_table[:dim]


def device_direction_numbers(dim: int, device: torch.device) -> torch.Tensor:
    host = direction_numbers(dim)
    key = device.index if device.index is not None else torch.cuda.current_device()
    with _cache_lock:
        t = _dev_tables.get(key)
        if t is None or t.shape[0] < dim:
            t = torch.from_numpy(np.ascontiguousarray(_host_table)).to(device)
            _dev_tables[key] = t
    return t[:dim]


def num_digits(num_results: int, skip: int) -> int:
    return int(_lib.load().tqf_sobol_num_digits(int(num_results), int(skip)))


def _validate(dim, num_results, skip, validate_args):
    if validate_args:
        if dim < 1:
            raise ValueError(f"Dimension must be greater than zero. Supplied {dim}")
        if num_results <= 0:
            raise InvalidArgumentError("Number of results `num_results` must be greater than zero.")
        # The reference asserts skip > 0 here (sobol_impl.py:96-98), so skip=0
        # is rejected under validate_args; kept for behavioural parity.
        if skip <= 0:
            raise InvalidArgumentError("`skip` must be non-negative.")
        if not (_MAX_POSITIVE - num_results > skip):
            raise InvalidArgumentError(
                f"Skip too large. Should be smaller than {_MAX_POSITIVE} - num_results")
    if dim < 1 or num_results < 1 or skip < 0 or skip + num_results > _MAX_POSITIVE:
        raise InvalidArgumentError(
            f"invalid Sobol request dim={dim}, num_results={num_results}, skip={skip}")


def _as_int(x) -> int:
    if isinstance(x, torch.Tensor):
        return int(x.item())
    return int(np.asarray(x).item()) if not isinstance(x, int) else x


def _launch(dim, num_results, skip, kind, torch_dtype, nd=None, out=None):
    device = _lib.require_cuda()
    nd = num_digits(num_results, skip) if nd is None else int(nd)
    v = device_direction_numbers(dim, device)
    if out is None:
        out = torch.empty((num_results, dim), dtype=torch_dtype, device=device)
    _lib.call("tqf_sobol_sample", v.data_ptr(), dim, num_results, skip, nd, kind, out.data_ptr(),
              _lib.stream_ptr(device))
    return out


def sample(dim: int, num_results, skip=0, validate_args: bool = False, dtype=None, name=None):
    """Returns [num_results, dim] Sobol points (float32 by default) on the GPU."""
    del name
    num_results, skip = _as_int(num_results), _as_int(skip)
    _validate(dim, num_results, skip, validate_args)
    dtype = _torch_dtype(dtype)
    if dtype == torch.float32:
        return _launch(dim, num_results, skip, _lib.SOBOL_F32, torch.float32)
    if dtype == torch.float64:
        return _launch(dim, num_results, skip, _lib.SOBOL_F64, torch.float64)
    if dtype == torch.float16:
        return _launch(dim, num_results, skip, _lib.SOBOL_F32, torch.float32).to(torch.float16)
    raise InvalidArgumentError(f"unsupported Sobol dtype {dtype}")


def sample_uint32(dim: int, num_results, skip=0, nd=None):
    """Integer points at the reference's nd-digit scaling (uint32 bit patterns
    in an int32 tensor), the quantity the reference's float output encodes."""
    num_results, skip = _as_int(num_results), _as_int(skip)
    _validate(dim, num_results, skip, False)
    return _launch(dim, num_results, skip, _lib.SOBOL_U32, torch.int32, nd=nd)


def sample_normal(dim: int, num_results, skip=0, dtype=torch.float32, nd=None, out=None):
    """erfinv((u - 0.5) * 2) * sqrt(2) of the reference floats u
    (tff/math/random_ops/multivariate_normal.py:420), fused in the kernel."""
    num_results, skip = _as_int(num_results), _as_int(skip)
    _validate(dim, num_results, skip, False)
    kind = _lib.SOBOL_NORMAL_F32 if dtype == torch.float32 else _lib.SOBOL_NORMAL_F64
    return _launch(dim, num_results, skip, kind, dtype, nd=nd, out=out)


def sample_centered(dim: int, num_results, skip=0):
    """(int + 0.5) * 2^-nd in float32: strictly inside (0, 1) (opt-in; the
    reference's float can round to exactly 1.0 once nd > 24)."""
    num_results, skip = _as_int(num_results), _as_int(skip)
    _validate(dim, num_results, skip, False)
    return _launch(dim, num_results, skip, _lib.SOBOL_F32_CENTERED, torch.float32)


def normal_draws(num_normal_draws: int, num_time_steps: int, num_paths: int, skip: int = 0,
                 dtype=torch.float32, nd=None):
    """[steps, N, d] normals: point skip+1+n, dimension step*d + c (the SOBOL
    branch of generate_mc_normal_draws, tff/models/utils.py:95-127)."""
    device = _lib.require_cuda()
    dim = num_normal_draws * num_time_steps
    _validate(dim, num_paths, skip, False)
    nd = num_digits(num_paths, skip) if nd is None else int(nd)
    v = device_direction_numbers(dim, device)
    out = torch.empty((num_time_steps, num_paths, num_normal_draws), dtype=dtype, device=device)
    kind = _lib.SOBOL_NORMAL_F32 if dtype == torch.float32 else _lib.SOBOL_NORMAL_F64
    _lib.call("tqf_sobol_normal_draws", v.data_ptr(), num_normal_draws, num_time_steps, num_paths,
              skip, nd, kind, out.data_ptr(), _lib.stream_ptr(device))
    return out


def _torch_dtype(dtype):
    if dtype is None:
        return torch.float32
    if isinstance(dtype, torch.dtype):
        return dtype
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
            np.dtype(np.float16): torch.float16}[np.dtype(dtype)]


__all__ = ["sample", "sample_uint32", "sample_normal", "sample_centered", "normal_draws",
           "direction_numbers", "num_digits"]
