"""Time-grid construction (tff/models/utils.py:209-320, heston_model.py:575-639).

All arithmetic is done in the caller's dtype, as TensorFlow does it.
tf.range(start, limit, delta) has ceil((limit-start)/delta) points
start + i*delta; tf.linspace(a, b, n) is [a, a + d*1, ..., a + d*(n-2), b]
with d = (b - a)/(n - 1) (TensorFlow's linspace_nd).
"""

from __future__ import annotations

import numpy as np


def tf_range(start, limit, delta, dtype):
    dt = np.dtype(dtype).type
    start, limit, delta = dt(start), dt(limit), dt(delta)
    size = int(np.ceil(np.abs((limit - start) / delta)))
    return (start + np.arange(size).astype(dtype) * delta).astype(dtype)


def tf_linspace(start, stop, num, dtype):
    dt = np.dtype(dtype).type
    start, stop = dt(start), dt(stop)
    num = int(num)
    if num <= 0:
        return np.zeros([0], dtype=dtype)
    if num == 1:
        return np.array([start], dtype=dtype)
    delta = (stop - start) / dt(max(num - 1, 1))
    mid = (start + delta * np.arange(1, num - 1).astype(dtype)).astype(dtype)
    return np.concatenate([[start], mid, [stop]]).astype(dtype)


def prepare_grid(times, time_step, dtype, tolerance=None, num_time_steps=None, times_grid=None):
    """utils.prepare_grid (tff/models/utils.py:209-282).

    Returns (all_times, keep_mask, time_indices).
    """
    dt = np.dtype(dtype).type
    times = np.asarray(times, dtype=dtype)
    if tolerance is None:
        tolerance = 1e-10 if np.dtype(dtype) == np.float64 else 1e-6
    tol = dt(tolerance)
    if times_grid is None:
        if num_time_steps is None:
            grid = tf_range(0.0, times[-1], time_step, dtype)
            all_times = np.sort(np.concatenate([times, grid]).astype(dtype), kind="stable")
            d = np.concatenate([[dt(1.0)], all_times[1:] - all_times[:-1]]).astype(dtype)
            all_times = all_times[d > tol]
            ti = np.searchsorted(all_times, times, side="left").astype(np.int32)
            ti = np.minimum(ti, len(all_times) - 1)
            ti = np.where(all_times[ti] - times > tol, ti - 1, ti).astype(np.int32)
        else:
            uniform = tf_linspace(dt(time_step), times[-1] - dt(time_step),
                                  max(int(num_time_steps) - times.shape[0], 0), dtype)
            grid = np.sort(np.concatenate([uniform, times]).astype(dtype), kind="stable")
            all_times = np.concatenate([[dt(0)], grid]).astype(dtype)
            ti = np.searchsorted(all_times, times, side="left").astype(np.int32)
    else:
        all_times = np.asarray(times_grid, dtype=dtype)
        ti = np.searchsorted(all_times, times, side="left").astype(np.int32)
        ti_c = np.minimum(ti, len(all_times) - 1)
        d1 = all_times[ti_c] - times
        d2 = all_times[np.maximum(ti - 1, 0)] - times
        ti = np.where(np.abs(d2) > np.abs(d1), ti, np.maximum(ti - 1, 0)).astype(np.int32)
    mask = np.zeros(len(all_times), dtype=bool)
    mask[ti] = True
    return all_times, mask, ti


def heston_prepare_grid(times, time_step, dtype, jump_locations=(), num_time_steps=None,
                        times_grid=None):
    """HestonModel._prepare_grid (heston_model.py:575-639): no de-duplication."""
    dt = np.dtype(dtype).type
    times = np.asarray(times, dtype=dtype)
    extra = [np.asarray(j, dtype=dtype).reshape(-1) for j in jump_locations]
    if times_grid is None:
        if time_step is not None and num_time_steps is None:
            grid = tf_range(0.0, times[-1], time_step, dtype)
        else:
            grid = tf_linspace(dt(0.0), times[-1] - dt(time_step), num_time_steps, dtype)
        all_times = np.concatenate([grid, times] + extra).astype(dtype)
        mask = np.concatenate([np.zeros(len(grid), bool), np.ones(len(times), bool)]
                              + [np.zeros(len(e), bool) for e in extra])
        perm = np.argsort(all_times, kind="stable")
        return all_times[perm], mask[perm]
    all_times, mask, _ = prepare_grid(times, time_step, dtype, times_grid=times_grid)
    return all_times, mask


def write_slots(keep_mask, num_requested, initial_written_count):
    """Slot recursion of the reference while-loops (euler_sampling.py:424-455,
    heston_model.py:376-446).

    Returns (step_slot[steps_exec], init_slot, steps_exec, unwritten) where
    step_slot[i] is the slot whose FINAL content is the state after step i
    (-1 if that state is overwritten later), init_slot the slot that keeps the
    initial state (-1 if none) and `unwritten` the slots never written.
    """
    steps = len(keep_mask) - 1
    wc = int(initial_written_count)
    last_writer = {0: -1}  # slot -> step index (-1 = initial state)
    i = 0
    slot_of_step = []
    while i < steps and wc < num_requested:
        slot_of_step.append(wc)
        last_writer[wc] = i
        wc += int(keep_mask[i + 1])
        i += 1
    steps_exec = i
    step_slot = np.full(steps_exec, -1, dtype=np.int32)
    for slot, who in last_writer.items():
        if who >= 0:
            step_slot[who] = slot
    init_slot = 0 if last_writer.get(0, -1) == -1 else -1
    written = set(last_writer.keys())
    unwritten = [s for s in range(num_requested) if s not in written]
    return step_slot, init_slot, steps_exec, unwritten
