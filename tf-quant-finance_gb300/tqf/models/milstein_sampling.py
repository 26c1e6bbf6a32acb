"""Milstein sampling on the GPU (tff/models/milstein_sampling.py:35-671).

Signature, grid (utils.prepare_grid), draw layout (dim + 3 dim order normals
per step), evaluation of drift / volatility / its gradient at t_{i+1} and the
recording rule are the reference's.  Structured coefficients
(``coefficients.AffineDrift`` + ``coefficients.ScaledVolatility``: GBM,
arithmetic BM, OU, ...) run the whole loop in one kernel
(``tqf_milstein_affine``) with the exact volatility gradient; any other
callables are evaluated once per step by the caller's torch code (the gradient
by forward-mode AD when ``grad_volatility_fn`` is not given, as the reference
does) and the step runs in ``tqf_milstein_update``.  With ``watch_params``
(or an initial state that requires grad) each step is an autograd Function
whose backward uses the step's dW and Stratonovich integrals, which the
forward kernel writes out: gradients reach the watched parameters through the
drift, the volatility and its gradient, as the reference's custom for_loop
gradient does (milstein_sampling.py:212-215, 389-424).

Extension: ``normal_draws`` ([num_samples, steps, dim + 3 dim order]) supplies
the normals explicitly.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import coefficients as coef
from tqf.models import utils


def num_normal_draws(dim: int, stratonovich_order: int) -> int:
    """Normals per time step (milstein_sampling.py:286-288)."""
    return dim + 3 * dim * stratonovich_order


def sample(*, dim, drift_fn, volatility_fn, times, time_step=None, num_time_steps=None, num_samples=1,
           initial_state=None, grad_volatility_fn=None, random_type=None, seed=None, swap_memory=True, skip=0,
           precompute_normal_draws=True, watch_params=None, stratonovich_order=5, dtype=None, name=None,
           normal_draws=None):
    """Returns sample paths [num_samples, k, dim] by the Milstein method."""
    del swap_memory, precompute_normal_draws, name
    if stratonovich_order <= 0:
        raise ValueError("`stratonovich_order` must be a positive integer.")
    np_dt = utils.np_dtype(dtype) if dtype is not None else utils.infer_dtype(times)
    td = utils.torch_dtype(np_dt)
    times_np = utils.to_numpy(times, np_dt).reshape(-1)
    if num_time_steps is not None and time_step is not None:
        raise ValueError("Only one of either `num_time_steps` or `time_step` should be defined but not both")
    if time_step is None:
        if num_time_steps is None:
            raise ValueError("Either `num_time_steps` or `time_step` should be defined.")
        time_step = times_np[-1] / np_dt.type(int(num_time_steps))
    all_times, keep, _ = utils.prepare_grid(times=times_np, time_step=time_step, dtype=np_dt,
                                            num_time_steps=num_time_steps)
    num_requested = len(times_np)
    device = _lib.require_cuda()
    if initial_state is None:
        initial_state = np.zeros(dim, np_dt)
    if isinstance(initial_state, torch.Tensor) and initial_state.requires_grad:
        x0 = initial_state.to(device=device, dtype=td)
    else:
        x0 = torch.as_tensor(utils.to_numpy(initial_state, np_dt)).to(device)
    differentiable = watch_params is not None or x0.requires_grad
    K = num_normal_draws(dim, stratonovich_order)
    steps_total = len(all_times) - 1
    step_slot, init_slot, steps_exec, unwritten = utils.plan_output_slots(keep, num_requested, int(keep[0]))
    dt = (all_times[1:] - all_times[:-1]).astype(np_dt)
    sqrt_dt = np.sqrt(dt).astype(np_dt)
    keep_alive = []
    if normal_draws is not None:
        dr = normal_draws if isinstance(normal_draws, torch.Tensor) else torch.as_tensor(
            utils.to_numpy(normal_draws, np_dt))
        dr = dr.to(device=device, dtype=td).contiguous()
        if dr.shape[-1] != K:
            raise ValueError(f"normal_draws must have {K} = dim + 3 dim order normals per step, got {dr.shape[-1]}")
        if dr.shape[1] < steps_exec:
            raise ValueError(f"normal_draws cover {dr.shape[1]} steps, the grid needs {steps_exec}")
        num_samples = int(dr.shape[0])
        keep_alive.append(dr)
        draws = mvn.memory_draws(dr, path_axis=0, step_axis=1)
    else:
        rt = RandomType.PSEUDO if random_type is None else random_type
        if rt in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
            sob = utils.generate_mc_normal_draws(K, steps_total, int(num_samples), rt, skip=skip, seed=seed, dtype=td)
            keep_alive.append(sob)
            draws = mvn.memory_draws(sob, path_axis=1, step_axis=0)
        else:
            draws = mvn.philox_draws(rt, seed, int(num_samples))
    N = int(num_samples)
    if differentiable:
        return _differentiable(dim, drift_fn, volatility_fn, grad_volatility_fn, all_times, dt, sqrt_dt, step_slot,
                               init_slot, steps_exec, x0, N, draws, num_requested, int(stratonovich_order), td,
                               device)
    alloc = torch.zeros if unwritten else torch.empty
    paths = alloc((N, num_requested, dim), dtype=td, device=device)
    if isinstance(drift_fn, coef.AffineDrift) and isinstance(volatility_fn, coef.ScaledVolatility) \
            and grad_volatility_fn is None:
        if drift_fn.dim != dim or volatility_fn.dim != dim:
            raise ValueError(f"structured coefficients have dimension {drift_fn.dim}, sample() got dim={dim}")
        x0v = torch.broadcast_to(x0, (N, dim)).contiguous() if x0.dim() > 1 else x0.reshape(dim).contiguous()
        rows = np.zeros((steps_exec, 4), dtype=np.float64)
        rows[:, 0] = dt[:steps_exec]
        rows[:, 1] = sqrt_dt[:steps_exec]
        rows[:, 2] = step_slot
        table = utils.step_table(rows, td, device)
        t = lambda v: torch.as_tensor(np.asarray(v, np.float64), dtype=td).to(device)  # noqa: E731
        m, M, s0, s1, C = (t(drift_fn.m), t(drift_fn.M), t(volatility_fn.s0), t(volatility_fn.s1),
                           t(volatility_fn.C))
        a = _lib.MilsteinAffineArgs()
        a.dtype = _lib.dtype_code(td)
        a.dim = dim
        a.num_paths = N
        a.num_steps = steps_exec
        a.x0_per_path = 1 if x0v.dim() == 2 else 0
        a.order = int(stratonovich_order)
        a.step_table = table.data_ptr() if steps_exec else None
        a.x0 = x0v.data_ptr()
        a.drift_m, a.drift_M = m.data_ptr(), M.data_ptr()
        a.vol_s0, a.vol_s1, a.vol_C = s0.data_ptr(), s1.data_ptr(), C.data_ptr()
        a.draws = draws
        a.output.ptr = paths.data_ptr()
        a.output.num_slots = num_requested
        a.output.init_slot = init_slot
        a.dev_status = _lib.status_buffer(device).data_ptr()
        _lib.call("tqf_milstein_affine", a, _lib.stream_ptr(device))
        return paths
    return _generic(dim, drift_fn, volatility_fn, grad_volatility_fn, all_times, dt, sqrt_dt, step_slot,
                    init_slot, steps_exec, x0, N, draws, paths, num_requested, int(stratonovich_order), td, device)


def _vol_gradient(volatility_fn, grad_volatility_fn, t, x, dim):
    """[N, d(i), d(k), d(j)] = dB_kj / dx_i (milstein_sampling.py:212-227, 649-654)."""
    if grad_volatility_fn is not None:
        if dim == 1:
            g = grad_volatility_fn(t, x, torch.ones_like(x))
            g = g[0] if isinstance(g, (list, tuple)) else g
            return torch.as_tensor(g).reshape(x.shape[0], 1, 1, 1)
        cols = []
        for i in range(dim):
            e = torch.zeros_like(x)
            e[:, i] = 1
            g = grad_volatility_fn(t, x, e)
            g = g[0] if isinstance(g, (list, tuple)) and len(g) == 1 else g
            cols.append(torch.as_tensor(g).reshape(x.shape[0], dim, dim))
        return torch.stack(cols, 1)
    cols = []
    for i in range(dim):
        e = torch.zeros_like(x)
        e[:, i] = 1
        _, g = torch.func.jvp(lambda y: volatility_fn(t, y), (x,), (e,))
        cols.append(torch.broadcast_to(g, (x.shape[0], dim, dim)))
    return torch.stack(cols, 1)


def _run_update(x, a_, B, G, step, dt, sqrt_dt, draws, order, device, paths=None, slot=-1, num_slots=0,
                need_increments=False):
    """One tqf_milstein_update call: (x_next, [N, d + d*d] dW and J or None)."""
    N, dim = x.shape
    x_next = torch.empty_like(x)
    inc = torch.empty((N, dim + dim * dim), dtype=x.dtype, device=x.device) if need_increments else None
    u = _lib.MilsteinUpdateArgs()
    u.dtype = _lib.dtype_code(x.dtype)
    u.dim = dim
    u.num_paths = N
    u.step = step
    u.out_slot = int(slot)
    u.order = order
    u.num_slots = num_slots
    u.dt = float(dt)
    u.sqrt_dt = float(sqrt_dt)
    u.x, u.drift, u.vol, u.grad, u.x_next = x.data_ptr(), a_.data_ptr(), B.data_ptr(), G.data_ptr(), \
        x_next.data_ptr()
    u.draws = draws
    u.paths_out = paths.data_ptr() if paths is not None else None
    u.increments_out = inc.data_ptr() if inc is not None else None
    _lib.call("tqf_milstein_update", u, _lib.stream_ptr(device))
    return x_next, inc


def _coefficients(drift_fn, volatility_fn, grad_volatility_fn, t, x, N, dim, td):
    a_ = torch.broadcast_to(drift_fn(t, x), (N, dim)).to(td).contiguous()
    B = torch.broadcast_to(volatility_fn(t, x), (N, dim, dim)).to(td).contiguous()
    G = _vol_gradient(volatility_fn, grad_volatility_fn, t, x, dim).to(td).contiguous()
    if a_.device != x.device or B.device != x.device or G.device != x.device:
        raise ValueError(f"drift_fn, volatility_fn and grad_volatility_fn must return tensors on {x.device}")
    return a_, B, G


def _generic(dim, drift_fn, volatility_fn, grad_volatility_fn, all_times, dt, sqrt_dt, step_slot, init_slot,
             steps_exec, x0, N, draws, paths, num_requested, order, td, device):
    """Per-step loop for arbitrary callables (milstein_sampling.py:356-424, 596-671)."""
    x = torch.broadcast_to(x0, (N, dim)).to(td).contiguous()
    t_dev = utils.step_times(all_times, steps_exec, td, device)  # one copy, a 0-d view per step
    if init_slot >= 0:
        paths[:, init_slot] = x
    for i in range(steps_exec):
        t = t_dev[i]
        a_, B, G = _coefficients(drift_fn, volatility_fn, grad_volatility_fn, t, x, N, dim, td)
        x, _ = _run_update(x, a_, B, G, i, dt[i], sqrt_dt[i], draws, order, device, paths, int(step_slot[i]),
                           num_requested)
    return paths


class _MilsteinStep(torch.autograd.Function):
    """One Milstein step, forward in tqf_milstein_update, backward by the chain
    rule through the kernel's update (u, h and J as in the kernel):
      d = 1: x' = x + dt a + b dW + b b' q,  q = (dW^2 - dt) / 2;
      d > 1: x'_k = x_k + dt (a_k - u_k) + sum_j B_kj dW_j + h_k,
             u_k = sum_ij G_ikj B_ij,  h_k = sum_im (sum_j G_ikj B_jm) J_im,
    with G_ikj = dB_kj/dx_i and the step's dW, J saved from the forward call."""

    @staticmethod
    def forward(ctx, x, a_, B, G, args_tuple):
        step, dt, sqrt_dt, draws, order, device = args_tuple
        x_next, inc = _run_update(x, a_, B, G, step, dt, sqrt_dt, draws, order, device, need_increments=True)
        ctx.save_for_backward(B, G, inc)
        ctx.dt = float(dt)
        return x_next

    @staticmethod
    def backward(ctx, g):
        B, G, inc = ctx.saved_tensors
        d = g.shape[-1]
        dt = ctx.dt
        dw = inc[:, :d]
        if d == 1:
            q = (dw * dw - dt) / 2
            gB = (g * (dw + G.reshape(-1, 1) * q)).reshape(-1, 1, 1)
            gG = (g * B.reshape(-1, 1) * q).reshape(-1, 1, 1, 1)
        else:
            J = inc[:, d:].reshape(-1, d, d)
            gB = (torch.einsum("nk,nj->nkj", g, dw) - dt * torch.einsum("nk,nikj->nij", g, G)
                  + torch.einsum("nk,nikj,nim->njm", g, G, J))
            R = torch.einsum("nim,njm->nij", J, B) - dt * B  # dx'_k / dG_ikj = g_k R_ij
            gG = torch.einsum("nk,nij->nikj", g, R)
        return g, g * dt, gB, gG, None


def _differentiable(dim, drift_fn, volatility_fn, grad_volatility_fn, all_times, dt, sqrt_dt, step_slot, init_slot,
                    steps_exec, x0, N, draws, num_requested, order, td, device):
    """Per-step loop with the states in the autograd graph (the role of the
    reference's custom for_loop with watch_params)."""
    x = torch.broadcast_to(x0, (N, dim)).to(td).contiguous()
    t_dev = utils.step_times(all_times, steps_exec, td, device)
    recorded = [None] * num_requested
    if init_slot >= 0:
        recorded[init_slot] = x
    for i in range(steps_exec):
        t = t_dev[i]
        a_, B, G = _coefficients(drift_fn, volatility_fn, grad_volatility_fn, t, x, N, dim, td)
        x = _MilsteinStep.apply(x.contiguous(), a_, B, G, (i, dt[i], sqrt_dt[i], draws, order, device))
        if step_slot[i] >= 0:
            recorded[int(step_slot[i])] = x
    zero = torch.zeros((N, dim), dtype=td, device=device)
    return torch.stack([r if r is not None else zero for r in recorded], dim=1)


__all__ = ["sample", "num_normal_draws"]
