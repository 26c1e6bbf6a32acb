"""Univariate geometric Brownian motion, exact log scheme
(tff/models/geometric_brownian_motion/univariate_geometric_brownian_motion.py:27-330).

dX = mu(t) X dt + sigma(t) X dW with constant or piecewise-constant mu, sigma
and an optional batch of independent processes.  Per interval the reference
forms log increments (int mu - int sigma^2 / 2) + sqrt(int sigma^2) z and their
cumulative sum (:261-318).  Here the per-interval constants are computed on the
host in the process dtype and the path kernel of the correlated GBM
(``tqf_mvgbm_paths`` with one factor, unit drift/volatility multipliers)
accumulates them in registers and writes x0 exp(cumsum) at every requested
time — one launch per batch member, all members on the same draws as in the
reference.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.math import piecewise as pw
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import utils
from tqf.models.ito_process import ItoProcess


class GeometricBrownianMotion(ItoProcess):
    """GeometricBrownianMotion(mean, volatility, dtype=None, name=None)."""

    def __init__(self, mean, volatility, dtype=None, name=None):
        self._name = name or "geometric_brownian_motion"
        # Scalar torch tensors that require grad stay watched: sample_paths
        # returns paths differentiable with respect to them.
        self._watched = {}
        for key, val in (("mean", mean), ("volatility", volatility)):
            if isinstance(val, torch.Tensor) and val.requires_grad:
                if val.numel() != 1:
                    raise NotImplementedError("gradients are supported for scalar mean and volatility")
                self._watched[key] = val
        mean = mean.detach().cpu().numpy() if isinstance(mean, torch.Tensor) else mean
        volatility = volatility.detach().cpu().numpy() if isinstance(volatility, torch.Tensor) else volatility
        self._mean, self._mean_is_constant = pw.convert_to_tensor_or_func(
            mean, dtype=None if dtype is None else utils.np_dtype(dtype))
        if dtype is None:
            dtype = self._mean.dtype() if not self._mean_is_constant else utils.infer_dtype(mean)
        self._np_dtype = utils.np_dtype(dtype)
        if self._mean_is_constant:
            self._mean = np.asarray(self._mean, self._np_dtype)
        self._volatility, self._volatility_is_constant = pw.convert_to_tensor_or_func(volatility,
                                                                                       dtype=self._np_dtype)
        self._dim = 1

    def dim(self):
        return self._dim

    def dtype(self):
        return utils.torch_dtype(self._np_dtype)

    def name(self):
        return self._name

    def drift_fn(self):
        def fn(t, x):
            m = self._mean if self._mean_is_constant else self._mean(utils.to_numpy(t))
            return torch.as_tensor(np.asarray(m), dtype=x.dtype, device=x.device) * x
        return fn

    def volatility_fn(self):
        def fn(t, x):
            v = self._volatility if self._volatility_is_constant else self._volatility(utils.to_numpy(t))
            return (torch.as_tensor(np.asarray(v), dtype=x.dtype, device=x.device) * x)[..., None]
        return fn

    def _integrals(self, t0, t1):
        """(int mu, int sigma^2) over [t0, t1] per batch member: [B, k] each (:230-259)."""
        dt_ = self._np_dtype.type
        if self._mean_is_constant:
            mi = np.asarray(self._mean, self._np_dtype)[..., None] * (t1 - t0)
            mi = mi.reshape(-1, t0.shape[-1]) if mi.ndim > 1 else mi[None]
        else:
            mi = self._mean.integrate(t0, t1)[None]
        if self._volatility_is_constant:
            v = np.asarray(self._volatility, self._np_dtype)
            vi = (v * v)[..., None] * (t1 - t0)
            vi = vi.reshape(-1, t0.shape[-1]) if vi.ndim > 1 else vi[None]
        else:
            sq = pw.PiecewiseConstantFunc(self._volatility.jump_locations(),
                                          self._volatility.values() ** 2, dtype=self._np_dtype)
            vi = sq.integrate(t0, t1)[None]
        B = max(mi.shape[0], vi.shape[0])
        mi = np.broadcast_to(mi, (B, mi.shape[-1])).astype(self._np_dtype)
        vi = np.broadcast_to(vi, (B, vi.shape[-1])).astype(self._np_dtype)
        del dt_
        return mi, vi

    def sample_paths(self, times, initial_state=None, num_samples=1, random_type=None, seed=None, skip=0,
                     normal_draws=None, name=None):
        """Returns [batch..., num_samples, k, 1] (:153-227, 261-318)."""
        del name
        np_dt = self._np_dtype
        td = utils.torch_dtype(np_dt)
        times_np = utils.to_numpy(times, np_dt).reshape(-1)
        k = len(times_np)
        device = _lib.require_cuda()
        keep_alive = []
        if normal_draws is not None:
            dr = normal_draws if isinstance(normal_draws, torch.Tensor) else torch.as_tensor(
                utils.to_numpy(normal_draws, np_dt))
            if dr.shape[-1] != 1:
                raise ValueError(f"`dim` should be equal to `1` but is {dr.shape[-1]}")
            dr = dr.to(device=device, dtype=td).contiguous()
            keep_alive.append(dr)
            num_samples = int(dr.shape[0])
            draws = mvn.memory_draws(dr, path_axis=0, step_axis=1)
        else:
            rt = RandomType.PSEUDO if random_type is None else random_type
            if rt in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
                sob = utils.generate_mc_normal_draws(1, k, int(num_samples), rt, skip=skip, seed=seed, dtype=td)
                keep_alive.append(sob)
                draws = mvn.memory_draws(sob, path_axis=1, step_axis=0)
            else:
                draws = mvn.philox_draws(rt, seed, int(num_samples))
        N = int(num_samples)
        grid = np.concatenate([[np_dt.type(0)], times_np]).astype(np_dt)
        mi, vi = self._integrals(grid[:-1], grid[1:])
        B = mi.shape[0]
        drift_rows = (mi - vi / np_dt.type(2)).astype(np_dt)
        vol_rows = np.sqrt(vi).astype(np_dt)
        x0 = np.ones(1, np_dt) if initial_state is None else utils.to_numpy(initial_state, np_dt)
        x0 = np.broadcast_to(x0.reshape(-1), (B,)) if x0.size in (1, B) else None
        if x0 is None:
            raise ValueError("initial_state must be a scalar or one value per batch member")
        out = torch.empty((B, N, k, 1), dtype=td, device=device)
        ones = torch.ones(1, dtype=td, device=device)
        for b in range(B):
            rows = np.zeros((k, 4), dtype=np.float64)
            rows[:, 0] = drift_rows[b]
            rows[:, 1] = vol_rows[b]
            rows[:, 2] = np.arange(k)
            table = utils.step_table(rows, td, device)
            x0b = torch.full((1,), float(x0[b]), dtype=td, device=device)
            a = _lib.MvgbmArgs()
            a.dtype = _lib.dtype_code(td)
            a.dim = 1
            a.num_paths = N
            a.num_steps = k
            a.x0_per_path = 0
            a.step_table = table.data_ptr()
            a.x0 = x0b.data_ptr()
            a.drift = ones.data_ptr()
            a.vol = ones.data_ptr()
            a.chol = None
            a.draws = draws
            a.output.ptr = out[b].data_ptr()
            a.output.num_slots = k
            a.output.init_slot = -1
            a.output.every_step = 1  # date j records slot j
            a.dev_status = _lib.status_buffer(device).data_ptr()
            a.lz_mode = 1
            _lib.call("tqf_mvgbm_paths", a, _lib.stream_ptr(device))
        shape_b = ()
        if not self._mean_is_constant or not self._volatility_is_constant:
            shape_b = ()
        else:
            sb = np.broadcast_shapes(np.shape(self._mean)[:-1] if np.ndim(self._mean) > 0 else (),
                                     np.shape(self._volatility)[:-1] if np.ndim(self._volatility) > 0 else ())
            shape_b = tuple(sb)
        if not shape_b and B == 1:
            return self._attach_gradient(out[0], times_np, float(x0[0])) if self._watched else out[0]
        return out.reshape(shape_b + (N, k, 1)) if shape_b else out

    def _attach_gradient(self, paths, times_np, x0):
        """Paths as a differentiable function of the watched scalar mean and
        volatility: log x_k = log x0 + (mu - s^2 / 2) t_k + s W_k
        (univariate_geometric_brownian_motion.py:261-318), with the Brownian
        values W_k recovered from the sampled paths.  The values returned are
        the kernel's; only the gradient comes from the expression."""
        td, dev = paths.dtype, paths.device

        def param(key, value):
            if key in self._watched:
                return self._watched[key].to(device=dev, dtype=td).reshape(())
            return torch.tensor(float(np.asarray(value).reshape(-1)[0]), dtype=td, device=dev)

        mu, s = param("mean", self._mean), param("volatility", self._volatility)
        t = torch.as_tensor(times_np, dtype=td, device=dev)[:, None]
        with torch.no_grad():
            drift = (mu - s * s / 2) * t
            w = torch.where(s != 0, (torch.log(paths / x0) - drift) / torch.where(s != 0, s, 1), 0)
        expr = x0 * torch.exp((mu - s * s / 2) * t + s * w)
        return paths + (expr - expr.detach())


__all__ = ["GeometricBrownianMotion"]
