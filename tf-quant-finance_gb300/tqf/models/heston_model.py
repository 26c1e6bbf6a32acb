"""Heston model: drop-in for tff.models.HestonModel
(tff/models/heston/heston_model.py:38-639).

``sample_paths`` runs Andersen's QE scheme exactly as the reference does
(QE variance step with psi_c = 1.5, central log-spot step gamma1 = gamma2 =
1/2, no martingale correction, no rate; zero-dt steps skipped but consuming
draws; parameters evaluated at times + min(dt)/2) in the ``tqf_heston_qe``
kernel.  The per-step constants (exp(-kappa dt), the s^2 coefficients,
k0..k4) are computed on the host in float64 from the dtype-rounded
parameters and rounded once to the model dtype.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.errors import InvalidArgumentError
from tqf.math.piecewise import PiecewiseConstantFunc
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import utils
from tqf.models.generic_ito_process import GenericItoProcess

QE_COLS = 12
FT_COLS = 8


def _param_values(param, t, np_dt):
    if isinstance(param, PiecewiseConstantFunc):
        return np.asarray(param(np.asarray(t, dtype=param.dtype())), dtype=np_dt)
    return (np.asarray(param, dtype=np_dt) * np.ones_like(np.asarray(t, dtype=np_dt))).astype(np_dt)


def _scalar(param, t, dtype):
    tt = float(t.item()) if isinstance(t, torch.Tensor) else float(t)
    return float(_param_values(param, np.array([tt]), np.float64)[0])


class HestonModel(GenericItoProcess):
    """dX = -V/2 dt + sqrt(V) dW_X,  dV = kappa (theta - V) dt + xi sqrt(V) dW_V,
    corr(dW_X, dW_V) = rho; state (log-spot X, variance V)."""

    def __init__(self, mean_reversion, theta, volvol, rho, dtype=None, name=None):
        self._name = name or "heston_model"
        np_dt = utils.np_dtype(dtype) if dtype is not None else np.dtype(np.float32)
        self._np_dtype = np_dt

        def conv(p):
            if isinstance(p, PiecewiseConstantFunc):
                return p
            return np_dt.type(utils.to_numpy(p, np_dt))

        self._mean_reversion = conv(mean_reversion)
        self._theta = conv(theta)
        self._volvol = conv(volvol)
        self._rho = conv(rho)

        def _vol_fn(t, x):
            x = torch.as_tensor(x)
            vol = torch.sqrt(torch.abs(x[..., 1]))
            zeros = torch.zeros_like(vol)
            r = _scalar(self._rho, t, np_dt)
            xi = _scalar(self._volvol, t, np_dt)
            col1 = torch.stack([vol, xi * r * vol], -1)
            col2 = torch.stack([zeros, xi * np.sqrt(1 - r ** 2) * vol], -1)
            return torch.stack([col1, col2], -1)

        def _drift_fn(t, x):
            x = torch.as_tensor(x)
            var = x[..., 1]
            k = _scalar(self._mean_reversion, t, np_dt)
            th = _scalar(self._theta, t, np_dt)
            return torch.stack([-var / 2, k * (th - var)], -1)

        super().__init__(2, _drift_fn, _vol_fn, utils.torch_dtype(np_dt), self._name)

    def sample_paths(self, times, initial_state, num_samples=1, random_type=None, seed=None,
                     time_step=None, skip=0, tolerance=1e-6, num_time_steps=None,
                     precompute_normal_draws=True, times_grid=None, normal_draws=None, name=None):
        """Returns [num_samples, k, 2] paths of (log-spot, variance)
        (heston_model.py:177-320)."""
        del precompute_normal_draws, name
        np_dt = self._np_dtype
        td = utils.torch_dtype(np_dt)
        if random_type is None:
            random_type = RandomType.PSEUDO
        times_np = utils.to_numpy(times, np_dt).reshape(-1)
        if times_grid is None and time_step is None and num_time_steps is None:
            raise ValueError("When `times_grid` is not supplied, either `num_time_steps` or "
                             "`time_step` should be defined.")
        if times_grid is None and time_step is not None and num_time_steps is not None:
            raise ValueError("Both `time_step` and `num_time_steps` can not be `None` simultaneously "
                             "when calling sample_paths of HestonModel.")
        device = _lib.require_cuda()
        draws_t = None
        if normal_draws is not None:
            draws_t = normal_draws if isinstance(normal_draws, torch.Tensor) else torch.as_tensor(
                utils.to_numpy(normal_draws, np_dt))
            draws_t = draws_t.to(device=device, dtype=td)
            num_samples = int(draws_t.shape[-3])
        x0 = utils.to_numpy(initial_state, np.float64)
        if x0.size != 2:
            raise NotImplementedError("batched Heston initial states are not supported; pass [log_spot, variance]")
        x0 = x0.reshape(2).astype(np_dt)
        num_requested = len(times_np)
        if times_grid is None:
            if time_step is None:
                if num_time_steps is None:
                    raise ValueError("When `times_grid` is not supplied, either `num_time_steps` or "
                                     "`time_step` should be defined.")
                time_step = times_np[-1] / np_dt.type(int(num_time_steps))
            elif num_time_steps is not None:
                raise ValueError("Both `time_step` and `num_time_steps` can not be `None` simultaneously "
                                 "when calling sample_paths of HestonModel.")
        all_times, keep = self._prepare_grid(times_np, time_step, num_time_steps, times_grid)
        steps_total = len(all_times) - 1
        step_slot, init_slot, steps_exec, unwritten = utils.plan_output_slots(keep, num_requested, 0)
        table = self._qe_table(all_times, tolerance, step_slot, steps_exec)
        keep_alive = []
        if draws_t is not None:
            if draws_t.shape[-2] < steps_exec:
                raise InvalidArgumentError(
                    f"normal_draws cover {draws_t.shape[-2]} time steps, the grid needs {steps_exec}")
            draws = mvn.memory_draws(draws_t, path_axis=0, step_axis=1)
        elif random_type == RandomType.SOBOL:
            # Sobol normals computed inside the kernel, equal to the
            # materialised generate_mc_normal_draws(2, steps_total, ...) bit for bit
            draws, v = mvn.sobol_draws(2, steps_total, int(num_samples), skip, device)
            keep_alive.append(v)
        elif random_type in (RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
            sob = utils.generate_mc_normal_draws(2, steps_total, int(num_samples), random_type, skip=skip, seed=seed,
                                                 dtype=td)
            keep_alive.append(sob)
            draws = mvn.memory_draws(sob, path_axis=1, step_axis=0)
        else:
            draws = mvn.philox_draws(random_type, seed, int(num_samples))
        num_samples = int(num_samples)
        paths = (torch.zeros if unwritten else torch.empty)((num_samples, num_requested, 2), dtype=td, device=device)
        tab = utils.step_table(table, td, device)
        args = _lib.HestonArgs()
        args.dtype = _lib.dtype_code(td)
        args.num_steps = steps_exec
        args.num_paths = num_samples
        args.step_table = tab.data_ptr() if steps_exec else None
        args.x0, args.v0 = float(x0[0]), float(x0[1])
        args.draws = draws
        args.output.ptr = paths.data_ptr()
        args.output.num_slots = num_requested
        args.output.init_slot = init_slot
        args.output.every_step = utils.every_step_layout(step_slot, init_slot, steps_exec, num_requested)
        args.dev_status = _lib.status_buffer(device).data_ptr()
        _lib.call("tqf_heston_qe", args, _lib.stream_ptr(device))
        return paths

    # -- helpers ------------------------------------------------------------
    def _jump_locations(self):
        out = []
        for p in (self._mean_reversion, self._theta, self._volvol, self._rho):
            if isinstance(p, PiecewiseConstantFunc):
                out.append(np.asarray(p.jump_locations(), dtype=self._np_dtype).reshape(-1))
        return out

    def _prepare_grid(self, times, time_step, num_time_steps, times_grid):
        """heston_model.py:575-639: no de-duplication, parameter jumps added."""
        np_dt = self._np_dtype
        t = np_dt.type
        extra = self._jump_locations()
        if times_grid is None:
            if num_time_steps is None:
                grid = utils.tf_range(0.0, times[-1], time_step, np_dt)
            else:
                grid = utils.tf_linspace(t(0.0), times[-1] - t(time_step), int(num_time_steps), np_dt)
            all_times = np.concatenate([grid, times] + extra).astype(np_dt)
            mask = np.concatenate([np.zeros(len(grid), bool), np.ones(len(times), bool)]
                                  + [np.zeros(len(e), bool) for e in extra])
            perm = np.argsort(all_times, kind="stable")
            return all_times[perm], mask[perm]
        all_times, mask, _ = utils.prepare_grid(times=times, time_step=time_step, dtype=np_dt,
                                                times_grid=times_grid)
        return all_times, mask

    def _params_on_grid(self, all_times):
        np_dt = self._np_dtype
        dt = (all_times[1:] - all_times[:-1]).astype(np_dt)
        eval_t = (all_times + np.min(dt) / np_dt.type(2)).astype(np_dt) if len(dt) else all_times
        return dt, [_param_values(p, eval_t, np_dt).astype(np.float64)
                    for p in (self._mean_reversion, self._theta, self._volvol, self._rho)]

    def _qe_table(self, all_times, tolerance, step_slot, steps_exec):
        np_dt = self._np_dtype
        dt, (K, TH, XI, RHO) = self._params_on_grid(all_times)
        n = int(steps_exec)
        h = dt[:n].astype(np.float64)
        k, th, xi, rho = K[:n], TH[:n], XI[:n], RHO[:n]
        E = np.exp(-k * h).astype(np_dt).astype(np.float64)  # e^{-kappa dt} in the model's precision
        rows = np.zeros((n, QE_COLS), dtype=np.float64)
        rows[:, 0] = np.where(dt[:n].astype(np_dt) > np_dt.type(tolerance), 0.0, 1.0)  # 1: state kept
        rows[:, 1] = th
        rows[:, 2] = E
        rows[:, 3] = xi * xi * E * (1.0 - E) / k
        rows[:, 4] = th * xi * xi * ((1.0 - E) * (1.0 - E)) / (2.0 * k)
        rows[:, 5] = -rho * k * th / xi * h
        rows[:, 6] = 0.5 * h * (k * rho / xi - 0.5) - rho / xi
        rows[:, 7] = 0.5 * h * (k * rho / xi - 0.5) + rho / xi
        rows[:, 8] = 0.5 * h * (1.0 - rho * rho)
        rows[:, 9] = 0.5 * h * (1.0 - rho * rho)
        rows[:, 11] = step_slot[:n]
        return rows

    def expected_total_variance(self, future_times, initial_var, name=None):
        """(V0 - theta)(1 - e^{-kappa T})/kappa + theta T (heston_model.py:462-509)."""
        del name
        for p, nm in ((self._mean_reversion, "_mean_reversion"), (self._theta, "_theta")):
            if isinstance(p, PiecewiseConstantFunc):
                raise ValueError(f"Only constant values supported for {nm}")
        t = np.asarray(future_times, dtype=self._np_dtype)
        v0 = np.asarray(initial_var, dtype=self._np_dtype)
        k, th = self._mean_reversion, self._theta
        strength = (1 - np.exp(-k * t)) / k
        return torch.as_tensor(((v0 - th) * strength + th * t).astype(self._np_dtype))


def full_truncation_table(heston, all_times, dt, sqrt_dt, step_slot, steps_exec):
    """[steps, 8] rows (dt/2, sqrt dt, r dt, kappa dt, kappa theta dt, xi rho,
    xi sqrt(1-rho^2), slot) with parameters at t_{i+1} (euler_sampling.py:519)."""
    r, k, th, xirho, xisq = heston.params_at(np.asarray(all_times[1:steps_exec + 1], dtype=np.float64))
    h = np.asarray(dt[:steps_exec], dtype=np.float64)
    rows = np.zeros((steps_exec, FT_COLS), dtype=np.float64)
    rows[:, 0] = 0.5 * h
    rows[:, 1] = sqrt_dt[:steps_exec]
    rows[:, 2], rows[:, 3], rows[:, 4] = r * h, k * h, k * th * h
    rows[:, 5], rows[:, 6] = xirho, xisq
    rows[:, 7] = step_slot
    return rows


def run_full_truncation(heston, all_times, dt, sqrt_dt, step_slot, init_slot, steps_exec, x0, M, draws,
                        paths, num_slots, td, device):
    """Fused full-truncation Euler path simulation into `paths` [M, k, 2]."""
    rows = full_truncation_table(heston, all_times, dt, sqrt_dt, step_slot, steps_exec)
    tab = utils.step_table(rows, td, device)
    args = _lib.HestonArgs()
    args.dtype = _lib.dtype_code(td)
    args.num_steps = steps_exec
    args.num_paths = M
    args.step_table = tab.data_ptr() if steps_exec else None
    args.x0, args.v0 = float(x0[0]), float(x0[1])
    args.draws = draws
    args.output.ptr = paths.data_ptr()
    args.output.num_slots = num_slots
    args.output.init_slot = init_slot
    args.output.every_step = utils.every_step_layout(step_slot, init_slot, steps_exec, num_slots)
    args.dev_status = _lib.status_buffer(device).data_ptr()
    _lib.call("tqf_heston_euler", args, _lib.stream_ptr(device))


__all__ = ["HestonModel", "full_truncation_table", "run_full_truncation"]
