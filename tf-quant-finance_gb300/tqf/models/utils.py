"""Grid construction, draw generation and output-slot planning
(tff/models/utils.py:20-128, 209-320).

Grids are small host-side arrays; they are built with NumPy in the dtype of
the request, reproducing TensorFlow's arithmetic: tf.range(a, b, d) has
ceil((b - a)/d) points a + i*d and tf.linspace(a, b, n) is
[a, a + d, ..., a + (n-2) d, b] with d = (b - a)/(n - 1).
"""

from __future__ import annotations

import collections
import threading

import numpy as np
import torch

from tqf.errors import InvalidArgumentError
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType


def np_dtype(dtype) -> np.dtype:
    if isinstance(dtype, torch.dtype):
        return np.dtype({torch.float32: np.float32, torch.float64: np.float64}[dtype])
    return np.dtype(dtype)


def torch_dtype(dtype) -> torch.dtype:
    if isinstance(dtype, torch.dtype):
        return dtype
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[np.dtype(dtype)]


def to_numpy(x, dtype=None) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    a = np.asarray(x)
    return a.astype(dtype) if dtype is not None else a


def infer_dtype(x) -> np.dtype:
    """TensorFlow's convert_to_tensor dtype: Python floats -> float32."""
    if isinstance(x, torch.Tensor):
        return np_dtype(x.dtype)
    if isinstance(x, np.ndarray) and x.dtype.kind == "f":
        return x.dtype
    if isinstance(x, np.floating):
        return np.dtype(type(x))
    return np.dtype(np.float32)


def tf_range(start, limit, delta, dtype) -> np.ndarray:
    t = np.dtype(dtype).type
    start, limit, delta = t(start), t(limit), t(delta)
    n = int(np.ceil(np.abs((limit - start) / delta)))
    return (start + np.arange(n).astype(dtype) * delta).astype(dtype)


def tf_linspace(start, stop, num, dtype) -> np.ndarray:
    t = np.dtype(dtype).type
    start, stop, num = t(start), t(stop), int(num)
    if num <= 0:
        return np.zeros(0, dtype=dtype)
    if num == 1:
        return np.array([start], dtype=dtype)
    d = (stop - start) / t(num - 1)
    inner = (start + d * np.arange(1, num - 1).astype(dtype)).astype(dtype)
    return np.concatenate([[start], inner, [stop]]).astype(dtype)


def prepare_grid(*, times, time_step, dtype, tolerance=None, num_time_steps=None, times_grid=None):
    """Returns (all_times, keep_mask, time_indices) as NumPy arrays
    (tff/models/utils.py:209-282)."""
    dtype = np_dtype(dtype)
    t = dtype.type
    times = to_numpy(times, dtype).reshape(-1)
    if tolerance is None:
        tolerance = 1e-10 if dtype == np.float64 else 1e-6
    tol = t(tolerance)
    if times_grid is None:
        if num_time_steps is None:
            grid = tf_range(0.0, times[-1], to_numpy(time_step, dtype), dtype)
            all_times = np.sort(np.concatenate([times, grid]), kind="stable").astype(dtype)
            diffs = np.concatenate([[t(1.0)], np.diff(all_times)]).astype(dtype)
            all_times = all_times[diffs > tol]
            ti = np.searchsorted(all_times, times, side="left")
            ti = np.minimum(ti, len(all_times) - 1)
            ti = np.where(all_times[ti] - times > tol, ti - 1, ti)
        else:
            step = t(to_numpy(time_step, dtype))
            uniform = tf_linspace(step, times[-1] - step, max(int(num_time_steps) - len(times), 0), dtype)
            grid = np.sort(np.concatenate([uniform, times]), kind="stable").astype(dtype)
            all_times = np.concatenate([[t(0)], grid]).astype(dtype)
            ti = np.searchsorted(all_times, times, side="left")
    else:
        all_times = to_numpy(times_grid, dtype).reshape(-1)
        ti = np.searchsorted(all_times, times, side="left")
        near = all_times[np.minimum(ti, len(all_times) - 1)] - times
        prev = all_times[np.maximum(ti - 1, 0)] - times
        ti = np.where(np.abs(prev) > np.abs(near), ti, np.maximum(ti - 1, 0))
    ti = ti.astype(np.int32)
    mask = np.zeros(len(all_times), dtype=bool)
    mask[ti] = True
    return all_times, mask, ti


def every_step_layout(step_slot, init_slot: int, steps_exec: int, num_slots: int) -> int:
    """1 if step i records slot base + i for every executed step (base = 1
    after an initial state at slot 0) and the slots end at num_slots: the
    tqf_path_output.every_step declaration that lets the Euler and GBM path
    kernels write rows front to back through their per-warp stager."""
    base = 1 if init_slot >= 0 else 0
    if init_slot not in (-1, 0) or base + int(steps_exec) != int(num_slots):
        return 0
    s = np.asarray(step_slot[:steps_exec]).astype(np.int64)
    return int(bool(np.array_equal(s, base + np.arange(int(steps_exec)))))


def plan_output_slots(keep_mask, num_requested: int, initial_written_count: int):
    """Replays the reference's written_count recursion (euler_sampling.py:424-455;
    heston_model.py:441-446 starts it at 0) on the host.

    Returns (step_slot[steps_exec] int32, init_slot, steps_exec, unwritten):
    step_slot[i] is the slot that finally holds the state after step i (-1 if
    a later step overwrites it), init_slot the slot that keeps the initial
    state (-1 if none), steps_exec the number of steps the loop runs before
    written_count reaches num_requested, and `unwritten` the slots no write
    reaches (left as zeros).
    """
    keep = np.asarray(keep_mask, dtype=bool).reshape(-1)
    steps = max(len(keep) - 1, 0)
    k = int(num_requested)
    # written_count before step i: the start value plus the kept times so far
    wc = int(initial_written_count) + np.concatenate(
        [np.zeros(1, np.int64), np.cumsum(keep[1:steps], dtype=np.int64)])[:steps]
    over = np.flatnonzero(wc >= k)
    n = int(over[0]) if over.size else steps
    wc = wc[:n]
    # a slot is finally held by the last step that writes it
    last = np.ones(n, dtype=bool)
    last[:-1] = wc[1:] != wc[:-1]
    step_slot = np.where(last, wc, -1).astype(np.int32)
    init_slot = -1 if n > 0 and wc[0] == 0 else 0
    written = np.zeros(max(k, 1), dtype=bool)
    written[0] = True
    written[wc[wc < k]] = True
    unwritten = np.flatnonzero(~written[:k]).tolist()
    return step_slot, init_slot, n, unwritten


def generate_mc_normal_draws(num_normal_draws, num_time_steps, num_sample_paths, random_type,
                             batch_shape=None, skip=0, seed=None, dtype=None, name=None):
    """[num_time_steps] + batch_shape + [num_sample_paths, num_normal_draws]
    draws (tff/models/utils.py:20-128).  Sobol dimension of (step i,
    component c) is i * num_normal_draws + c, point index skip + 1 + path."""
    del name
    dtype = torch.float32 if dtype is None else torch_dtype(dtype)
    batch_shape = tuple(int(b) for b in (batch_shape or ()))
    nb = int(np.prod(batch_shape)) if batch_shape else 1
    total = nb * int(num_sample_paths)
    if random_type is None:
        random_type = RandomType.PSEUDO
    shape = (int(num_time_steps),) + batch_shape + (int(num_sample_paths), int(num_normal_draws))
    if random_type == RandomType.SOBOL:
        # The sample shape batch_shape + [num_sample_paths] is flattened in C
        # order: point skip + 1 + b * num_sample_paths + n (utils.py:94-99).
        from tqf.math.random import sobol
        return sobol.normal_draws(int(num_normal_draws), int(num_time_steps), total,
                                  skip=int(skip or 0), dtype=dtype).reshape(shape)
    if random_type in (RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
        from tqf.math.random import halton
        return halton.normal_draws(int(num_normal_draws), int(num_time_steps), total,
                                   randomized=random_type == RandomType.HALTON_RANDOMIZED, seed=seed,
                                   skip=int(skip or 0), dtype=dtype).reshape(shape)
    if mvn.is_antithetic(random_type) and batch_shape:
        # Antithetic samples come first and the batch after (utils.py:98-107):
        # path n of batch entry b is paired with path n + num_sample_paths / 2
        # of the same entry.
        n = int(num_sample_paths)
        if n % 2:
            raise InvalidArgumentError(
                "First dimension of `sample_shape` should be even for PSEUDO_ANTITHETIC random type")
        plain = RandomType.STATELESS if random_type == RandomType.STATELESS_ANTITHETIC else RandomType.PSEUDO
        z = mvn.philox_normal_draws(plain, seed, int(num_normal_draws), int(num_time_steps), nb * (n // 2), dtype)
        z = z.reshape(int(num_time_steps), nb, n // 2, int(num_normal_draws))
        return torch.cat([z, -z], dim=2).reshape(shape)
    draws = mvn.philox_normal_draws(random_type, seed, int(num_normal_draws), int(num_time_steps),
                                    total, dtype)
    return draws.reshape(shape)


_UPLOADS: "collections.OrderedDict[tuple, torch.Tensor]" = collections.OrderedDict()
_UPLOADS_LOCK = threading.Lock()
_UPLOADS_MAX = 256            # arrays kept
_UPLOADS_MAX_BYTES = 1 << 18  # largest array kept


def upload(array, dtype: torch.dtype, device) -> torch.Tensor:
    """Device copy of a small host array that kernels only read (step tables,
    exercise schedules, discount tables, strikes).  Copies are kept by
    content (device, dtype, shape, bytes; at most 256 arrays of at most
    256 KiB, least recently used dropped), so repeated calls with the same
    schedules upload nothing: a pageable host-to-device copy would make the
    host wait for all earlier GPU work before it could prepare the launch.
    Callers must not write to the returned tensor."""
    a = np.ascontiguousarray(array)
    dev = torch.device(device)
    if dev.type != "cuda":
        return torch.tensor(a, dtype=dtype)
    if a.nbytes > _UPLOADS_MAX_BYTES:
        return torch.tensor(a, dtype=dtype).to(dev)
    index = dev.index if dev.index is not None else torch.cuda.current_device()
    key = (index, str(dtype), a.dtype.str, a.shape, a.tobytes())
    with _UPLOADS_LOCK:
        hit = _UPLOADS.get(key)
        if hit is not None:
            _UPLOADS.move_to_end(key)
            return hit
    t = torch.tensor(a, dtype=dtype).to(dev)
    with _UPLOADS_LOCK:
        _UPLOADS[key] = t
        while len(_UPLOADS) > _UPLOADS_MAX:
            _UPLOADS.popitem(last=False)
    return t


def step_times(all_times, steps_exec: int, dtype: torch.dtype, device) -> torch.Tensor:
    """t_1 .. t_steps_exec of a grid as one device tensor, for per-step loops
    that hand each step's time to user callables as a 0-d view (a host
    scalar copied per step would make the host wait for the GPU every step)."""
    return torch.as_tensor(np.asarray(all_times[1:int(steps_exec) + 1]), device=device).to(dtype)


def step_table(rows: np.ndarray, dtype: torch.dtype, device) -> torch.Tensor:
    """Uploads a [steps, cols] host table (16-byte aligned device copy)."""
    return upload(rows, dtype, device)


__all__ = ["prepare_grid", "generate_mc_normal_draws", "plan_output_slots", "tf_range", "tf_linspace", "upload"]
