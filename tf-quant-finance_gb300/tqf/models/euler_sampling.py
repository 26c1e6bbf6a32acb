"""Euler–Maruyama sampling: drop-in for tff.models.euler_sampling.sample
(tff/models/euler_sampling.py:27-537).

Semantics kept from the reference: the grid (utils.prepare_grid), drift and
volatility evaluated at (t_{i+1}, X_i) (euler_sampling.py:519-529), the
[steps, N, d] draw layout, the written_count / keep_mask recording and the
output shape batch_shape + [num_samples, k, dim].

Execution:
* structured coefficients (tqf.models.coefficients) run the whole loop in
  one fused kernel (``tqf_euler_affine`` / ``tqf_heston_euler``);
* arbitrary torch callables are evaluated once per step by the caller's
  code and the step itself (draws, sqrt dt scaling, B·dW, state update,
  recording) runs in ``tqf_euler_update``; with ``watch_params`` the step is
  wrapped in an autograd Function so gradients reach the parameters and the
  initial state (the role of custom_loops.for_loop, euler_sampling.py:467-510).

``swap_memory`` and ``precompute_normal_draws`` are accepted and ignored:
draws are generated in-kernel from a counter-based stream, so nothing is
precomputed or swapped.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.errors import InvalidArgumentError
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import coefficients as coef
from tqf.models import utils


def _plan(times, time_step, num_time_steps, times_grid, tolerance, dtype, validate_args):
    np_dt = utils.np_dtype(dtype)
    times_np = utils.to_numpy(times, np_dt).reshape(-1)
    if tolerance is None:
        tolerance = 1e-10 if np_dt == np.float64 else 1e-6
    tol = np_dt.type(tolerance)
    if validate_args and np.any(~(times_np[1:] > times_np[:-1] + tol)):
        raise InvalidArgumentError(f"`times` increments should be greater than tolerance {tolerance}")
    if num_time_steps is not None and time_step is not None:
        raise ValueError("When `times_grid` is not supplied only one of either `num_time_steps` or "
                         "`time_step` should be defined but not both.")
    if times_grid is None:
        if time_step is None:
            if num_time_steps is None:
                raise ValueError("When `times_grid` is not supplied, either `num_time_steps` or "
                                 "`time_step` should be defined.")
            time_step = times_np[-1] / np_dt.type(int(num_time_steps))
    else:
        tg = utils.to_numpy(times_grid, np_dt).reshape(-1)
        if validate_args and np.any(~(tg[1:] > tg[:-1] + tol)):
            raise InvalidArgumentError(f"`times_grid` increments should be greater than tolerance {tolerance}")
    all_times, keep, ti = utils.prepare_grid(times=times_np, time_step=time_step, dtype=np_dt,
                                             tolerance=tolerance, num_time_steps=num_time_steps,
                                             times_grid=times_grid)
    return times_np, all_times, keep, ti


def sample(dim, drift_fn, volatility_fn, times, time_step=None, num_time_steps=None,
           num_samples=1, initial_state=None, random_type=None, seed=None, swap_memory=True,
           skip=0, precompute_normal_draws=True, times_grid=None, normal_draws=None,
           watch_params=None, validate_args=False, tolerance=None, dtype=None, name=None):
    """Returns sample paths of shape batch_shape + [num_samples, k, dim]."""
    del swap_memory, precompute_normal_draws, name
    np_dt = utils.np_dtype(dtype) if dtype is not None else utils.infer_dtype(times)
    td = utils.torch_dtype(np_dt)
    times_np, all_times, keep, _ = _plan(times, time_step, num_time_steps, times_grid, tolerance,
                                         np_dt, validate_args)
    num_requested = len(times_np)
    if normal_draws is not None and tuple(normal_draws.shape)[-1] != dim:
        raise ValueError("`dim` should be equal to `normal_draws.shape[2]` but are "
                         f"{dim} and {tuple(normal_draws.shape)[-1]} respectively")
    if validate_args and normal_draws is not None and tuple(normal_draws.shape)[-2] != len(all_times) - 1:
        raise InvalidArgumentError("`num_time_steps` should be equal to `tf.shape(normal_draws)[1]`")
    device = _lib.require_cuda()
    if initial_state is None:
        initial_state = torch.zeros(dim, dtype=td, device=device)
    elif not isinstance(initial_state, torch.Tensor) or not initial_state.requires_grad:
        initial_state = torch.as_tensor(utils.to_numpy(initial_state, np_dt), device=device)
    initial_state = initial_state.to(device=device, dtype=td)
    batch_shape = tuple(initial_state.shape[:-2])
    steps_total = len(all_times) - 1
    draws_t = None
    if normal_draws is not None:
        draws_t = torch.as_tensor(utils.to_numpy(normal_draws, np_dt)) if not isinstance(
            normal_draws, torch.Tensor) else normal_draws
        draws_t = draws_t.to(device=device, dtype=td)
        if draws_t.shape[-1] != dim:
            raise ValueError("`dim` should be equal to `normal_draws.shape[2]` but are "
                             f"{dim} and {draws_t.shape[-1]} respectively")
        if validate_args and draws_t.shape[-2] != steps_total:
            raise InvalidArgumentError("`num_time_steps` should be equal to `tf.shape(normal_draws)[1]`")
        num_samples = int(draws_t.shape[-3])
    num_samples = int(num_samples)
    step_slot, init_slot, steps_exec, unwritten = utils.plan_output_slots(keep, num_requested, int(keep[0]))
    if draws_t is not None and draws_t.shape[-2] < steps_exec:
        raise InvalidArgumentError(
            f"normal_draws cover {draws_t.shape[-2]} time steps, the grid needs {steps_exec}")
    nb = int(np.prod(batch_shape)) if batch_shape else 1
    M = nb * num_samples
    dt = (all_times[1:] - all_times[:-1]).astype(np_dt)
    sqrt_dt = np.sqrt(dt).astype(np_dt)

    # Draw source for the kernels.
    keep_alive = []
    if draws_t is not None:
        flat = draws_t.reshape(M, draws_t.shape[-2], dim)
        keep_alive.append(flat)
        draws = mvn.memory_draws(flat, path_axis=0, step_axis=1)
    else:
        rt = RandomType.PSEUDO if random_type is None else random_type
        quasi = rt in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED)
        if quasi or (mvn.is_antithetic(rt) and batch_shape):
            # materialised in the reference's layout, batch entries flattened
            # into the path axis as the state is
            mat = utils.generate_mc_normal_draws(dim, steps_total, num_samples, rt, batch_shape=batch_shape,
                                                 skip=skip, seed=seed, dtype=td).reshape(steps_total, M, dim)
            keep_alive.append(mat)
            draws = mvn.memory_draws(mat, path_axis=1, step_axis=0)
        else:
            draws = mvn.philox_draws(rt, seed, M)

    out_shape = batch_shape + (num_samples, num_requested, dim)
    alloc = torch.zeros if unwritten else torch.empty
    if watch_params is not None:
        return _generic(dim, drift_fn, volatility_fn, all_times, dt, sqrt_dt, step_slot, init_slot,
                        steps_exec, initial_state, batch_shape, num_samples, M, draws, out_shape,
                        num_requested, td, device, differentiable=True)
    structured = _structured_kind(drift_fn, volatility_fn, dim)
    if structured == "affine" and not initial_state.requires_grad:
        paths = alloc(out_shape, dtype=td, device=device)
        x0 = torch.broadcast_to(initial_state, batch_shape + (num_samples, dim)).reshape(M, dim).contiguous() \
            if (batch_shape or initial_state.dim() > 1) else initial_state.reshape(dim).contiguous()
        rows = np.zeros((steps_exec, 4), dtype=np.float64)
        rows[:, 0] = dt[:steps_exec]
        rows[:, 1] = sqrt_dt[:steps_exec]
        rows[:, 2] = step_slot
        table = utils.step_table(rows, td, device)
        d = drift_fn.m.shape[0]
        t = lambda a: utils.upload(np.asarray(a, np.float64), td, device)  # noqa: E731  (read-only)
        m, Mx, s0, s1, C = t(drift_fn.m), t(drift_fn.M), t(volatility_fn.s0), t(volatility_fn.s1), t(volatility_fn.C)
        if d != dim:
            raise ValueError(f"structured coefficients have dimension {d}, sample() got dim={dim}")
        args = _lib.EulerAffineArgs()
        args.dtype = _lib.dtype_code(td)
        args.dim = dim
        args.num_paths = M
        args.num_steps = steps_exec
        args.x0_per_path = 1 if x0.dim() == 2 else 0
        args.step_table = table.data_ptr() if steps_exec else None
        args.x0 = x0.data_ptr()
        args.drift_m, args.drift_M = m.data_ptr(), Mx.data_ptr()
        args.vol_s0, args.vol_s1, args.vol_C = s0.data_ptr(), s1.data_ptr(), C.data_ptr()
        args.draws = draws
        args.output.ptr = paths.data_ptr()
        args.output.num_slots = num_requested
        args.output.init_slot = init_slot
        args.output.every_step = utils.every_step_layout(step_slot, init_slot, steps_exec, num_requested)
        args.dev_status = _lib.status_buffer(device).data_ptr()
        _lib.call("tqf_euler_affine", args, _lib.stream_ptr(device))
        return paths
    if structured == "heston" and not initial_state.requires_grad and initial_state.numel() == 2:
        from tqf.models import heston_model
        x0 = utils.to_numpy(initial_state.detach(), np.float64).reshape(2)
        paths = alloc(out_shape, dtype=td, device=device)
        heston_model.run_full_truncation(drift_fn.heston, all_times, dt, sqrt_dt, step_slot, init_slot,
                                         steps_exec, x0, M, draws, paths, num_requested, td, device)
        return paths
    return _generic(dim, drift_fn, volatility_fn, all_times, dt, sqrt_dt, step_slot, init_slot,
                    steps_exec, initial_state, batch_shape, num_samples, M, draws, out_shape,
                    num_requested, td, device, differentiable=initial_state.requires_grad)


def _structured_kind(drift_fn, volatility_fn, dim):
    if isinstance(drift_fn, coef.AffineDrift) and isinstance(volatility_fn, coef.ScaledVolatility):
        return "affine"
    h1 = getattr(drift_fn, "heston", None)
    h2 = getattr(volatility_fn, "heston", None)
    if h1 is not None and h1 is h2 and dim == 2:
        return "heston"
    return None


class _EulerStep(torch.autograd.Function):
    """x_next = x + dt a + B (z sqrt dt): forward in tqf_euler_update, backward
    by the chain rule (dx_next/dx = I, /da = dt I, /dB = outer(., dw))."""

    @staticmethod
    def forward(ctx, x, a, B, dw_holder, args_tuple):
        out, dw = _run_update(x, a, B, *args_tuple)
        ctx.save_for_backward(dw)
        ctx.dt = args_tuple[1]
        return out

    @staticmethod
    def backward(ctx, g):
        (dw,) = ctx.saved_tensors
        gx = g
        ga = g * ctx.dt
        gB = g[..., :, None] * dw[..., None, :]
        return gx, ga, gB, None, None


def _run_update(x, a, B, step, dt, sqrt_dt, draws, paths, slot, num_slots, device, need_dw, aux=None):
    M, d = x.shape
    x_next = torch.empty_like(x)
    args = _lib.EulerUpdateArgs()
    args.dtype = _lib.dtype_code(x.dtype)
    args.dim = d
    args.num_paths = M
    args.step = step
    args.out_slot = int(slot)
    args.dt = float(dt)
    args.sqrt_dt = float(sqrt_dt)
    args.x, args.drift, args.vol, args.x_next = x.data_ptr(), a.data_ptr(), B.data_ptr(), x_next.data_ptr()
    args.draws = draws
    args.paths_out = paths.data_ptr() if paths is not None else None
    args.num_slots = num_slots
    _lib.call("tqf_euler_update", args, _lib.stream_ptr(device))
    dw = None
    if need_dw:
        # dw = (x_next - x - dt a) solved through B is ill-posed; instead run the
        # same kernel with a = 0, B = I, x = 0: it returns z sqrt(dt) exactly.
        # (`aux` keeps I and 0 across the steps of one call.)
        aux = {} if aux is None else aux
        if "eye" not in aux:
            aux["eye"] = torch.eye(d, dtype=x.dtype, device=x.device).expand(M, d, d).contiguous()
            aux["zero"] = torch.zeros_like(x)
        eye, zero = aux["eye"], aux["zero"]
        dw = torch.empty_like(x)
        a2 = _lib.EulerUpdateArgs()
        ctypes_copy(args, a2)
        a2.x, a2.drift, a2.vol, a2.x_next = zero.data_ptr(), zero.data_ptr(), eye.data_ptr(), dw.data_ptr()
        a2.paths_out = None
        a2.out_slot = -1
        _lib.call("tqf_euler_update", a2, _lib.stream_ptr(device))
    return x_next, dw


def ctypes_copy(src, dst):
    for name, _ in src._fields_:
        setattr(dst, name, getattr(src, name))


def _generic(dim, drift_fn, volatility_fn, all_times, dt, sqrt_dt, step_slot, init_slot, steps_exec,
             initial_state, batch_shape, num_samples, M, draws, out_shape, num_requested, td,
             device, differentiable):
    """Per-step loop for arbitrary callables (euler_sampling.py:405-464)."""
    x = torch.broadcast_to(initial_state, batch_shape + (num_samples, dim)).reshape(M, dim)
    # the step times on the device in one copy (t_{i+1} as a 0-d view per
    # step): a per-step host scalar copy would wait for the GPU every step
    t_dev = utils.step_times(all_times, steps_exec, td, device)
    if not differentiable:
        x = x.detach().contiguous()
        paths = (torch.zeros if init_slot < 0 else torch.empty)((M, num_requested, dim), dtype=td, device=device)
        if init_slot >= 0:
            paths[:, init_slot] = x
        # one argument block and one stream lookup for the whole loop: per
        # step only the pointers, the step index and its dt change
        args = _lib.EulerUpdateArgs()
        args.dtype = _lib.dtype_code(td)
        args.dim = dim
        args.num_paths = M
        args.draws = draws
        args.paths_out = paths.data_ptr()
        args.num_slots = num_requested
        stream = _lib.stream_ptr(device)
        update = _lib.load().tqf_euler_update
        dts, sdts, slots = [float(v) for v in dt], [float(v) for v in sqrt_dt], [int(v) for v in step_slot]
        ts = t_dev.unbind(0)  # the steps' 0-d time views, made at once
        plain = not batch_shape  # the state is already [num_samples, dim]
        for i in range(steps_exec):
            t = ts[i]
            xs = x if plain else x.reshape(batch_shape + (num_samples, dim))
            a = drift_fn(t, xs)
            if a.shape != (M, dim) or a.dtype != td or not a.is_contiguous():
                a = torch.broadcast_to(a, xs.shape).reshape(M, dim).to(td).contiguous()
            B = volatility_fn(t, xs)
            if B.shape != (M, dim, dim) or B.dtype != td or not B.is_contiguous():
                B = torch.broadcast_to(B, xs.shape + (dim,)).reshape(M, dim, dim).to(td).contiguous()
            if a.device != x.device or B.device != x.device:
                raise ValueError(f"drift_fn and volatility_fn must return tensors on {x.device}")
            x_next = torch.empty_like(x)
            args.step, args.out_slot, args.dt, args.sqrt_dt = i, slots[i], dts[i], sdts[i]
            args.x, args.drift, args.vol, args.x_next = x.data_ptr(), a.data_ptr(), B.data_ptr(), x_next.data_ptr()
            _lib.check(update(args, stream), "tqf_euler_update")
            x = x_next
        return paths.reshape(out_shape)
    # Differentiable route: states kept in the autograd graph.
    x = x.contiguous() if not x.requires_grad else x
    recorded = [None] * num_requested
    if init_slot >= 0:
        recorded[init_slot] = x
    aux = {}
    for i in range(steps_exec):
        t = t_dev[i]
        xs = x.reshape(batch_shape + (num_samples, dim))
        a = torch.broadcast_to(drift_fn(t, xs), xs.shape).reshape(M, dim).to(td).contiguous()
        B = torch.broadcast_to(volatility_fn(t, xs), xs.shape + (dim,)).reshape(M, dim, dim).to(td).contiguous()
        if a.device != x.device or B.device != x.device:
            raise ValueError(f"drift_fn and volatility_fn must return tensors on {x.device}")
        x = _EulerStep.apply(x.contiguous(), a, B, None,
                             (i, dt[i], sqrt_dt[i], draws, None, -1, num_requested, device, True, aux))
        if step_slot[i] >= 0:
            recorded[int(step_slot[i])] = x
    zero = torch.zeros((M, dim), dtype=td, device=device)
    stacked = torch.stack([r if r is not None else zero for r in recorded], dim=1)
    return stacked.reshape(out_shape)


__all__ = ["sample"]
