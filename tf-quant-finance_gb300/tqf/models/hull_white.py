"""Vector Hull-White model on the GPU
(tff/models/hull_white/vector_hull_white.py:35-1088, one_factor.py:16-137).

dr = (theta(t) - a(t) r) dt + sigma(t) dW with correlated Brownian motions.
With piecewise-constant volatility / correlation and a constant mean reversion
the reference samples the exact transition (:641-781); so does this module:
the per-step transition constants (decay exp(-a dt), conditional mean
increment, conditional standard deviation, instantaneous forward rate f(0, t),
Cholesky factor of the correlation) are tabulated on the host in the model
dtype with the reference's piecewise integrals (:816-955), and
``tqf_hull_white_paths`` carries each path's state in registers through all
steps.  Time-dependent mean reversion or callable parameters fall back to the
Euler sampler on the model's drift and volatility, as in the reference.

Parameters: scalars / [dim] arrays, or ``PiecewiseConstantFunc`` with shared
(1-D) jump locations and values [n + 1] or [n + 1, dim] ([n + 1, dim, dim] for
the correlation), or per-axis jump locations [dim, n] with values
[dim, n + 1] (mean reversion and volatility; vector_hull_white.py:156-198).
A piecewise mean reversion with jumps samples with the Euler sampler, as the
reference does (:1052-1054).
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.math.piecewise import PiecewiseConstantFunc
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import euler_sampling, utils
from tqf.models.generic_ito_process import GenericItoProcess


class _Param:
    """A parameter as per-axis piecewise-constant functions.

    ``jumps`` keeps the jump locations as given ([n] shared by the axes, or
    [dim, n] per axis, vector_hull_white.py:156-198); ``axis_jumps`` [dim, n]
    and ``axis_values`` [dim, n + 1] hold them per axis (values[i] on
    (jumps[i-1], jumps[i]], left-continuous).  The correlation matrix takes
    shared jumps only, as the reference documents (:176-181)."""

    def __init__(self, p, dim, dtype, name, matrix=False):
        self.name = name
        self.dim = dim
        self.callable = callable(p) and not isinstance(p, PiecewiseConstantFunc)
        self.fn = p if self.callable else None
        self.matrix = matrix
        if self.callable:
            self.jumps = np.zeros(0, dtype)
            self.axis_jumps = np.zeros((dim, 0), dtype)
            return
        if isinstance(p, PiecewiseConstantFunc):
            self.jumps = np.asarray(p.jump_locations(), dtype)
            v = np.asarray(p.values(), dtype)
            if self.jumps.ndim > 2:
                raise ValueError("Batch rank of `jump_locations` should be `1` for all piecewise constant arguments "
                                 f"but {self.jumps.ndim - 1} instead")
            if self.jumps.ndim == 2:
                if self.jumps.shape[0] != dim:
                    raise ValueError(f"Batch shape of `jump_locations` should be either empty or `[{dim}]` but "
                                     f"`[{self.jumps.shape[0]}]` instead")
                if matrix:
                    raise ValueError(f"{name}: jump locations must be shared by the axes (shape [num_jumps])")
                n = self.jumps.shape[1]
                if v.shape[:2] != (dim, n + 1) or v.size != dim * (n + 1):
                    raise ValueError(f"{name}: per-axis values must have shape [{dim}, {n + 1}], got {v.shape}")
                self.axis_jumps = self.jumps
                self.axis_values = v.reshape(dim, n + 1)
                return
        else:
            self.jumps = np.zeros(0, dtype)
            v = np.asarray(p, dtype)[None]
        n = len(self.jumps)
        self.axis_jumps = np.broadcast_to(self.jumps, (dim, n)).astype(dtype)
        if matrix:
            self.values = np.broadcast_to(v, (v.shape[0], dim, dim)).astype(dtype)
        else:
            if v.ndim == 1:
                v = v[:, None]
            if v.shape[-1] not in (1, dim):
                raise ValueError(f"Length of {name} ({v.shape[-1]}) should be the same as `dims`({dim}).")
            self.axis_values = np.ascontiguousarray(np.broadcast_to(v, (v.shape[0], dim)).T).astype(dtype)

    def __call__(self, t):
        """Values at times t (left-continuous): [len(t), dim(, dim)]."""
        t = np.asarray(t, self.axis_jumps.dtype)
        if self.matrix:
            return self.values[np.searchsorted(self.jumps, t, side="left")]
        return self.at(np.broadcast_to(t.reshape(-1), (self.dim, t.size))).T

    def at(self, t):
        """Per-axis values at per-axis times t [dim, m]: [dim, m]."""
        t = np.asarray(t, self.axis_values.dtype)
        return np.stack([self.axis_values[d][np.searchsorted(self.axis_jumps[d], t[d], side="left")]
                         for d in range(self.dim)]).reshape(t.shape)


class VectorHullWhiteModel(GenericItoProcess):
    """VectorHullWhiteModel(dim, mean_reversion, volatility, initial_discount_rate_fn,
    corr_matrix=None, dtype=None, name=None)."""

    def __init__(self, dim, mean_reversion, volatility, initial_discount_rate_fn, corr_matrix=None, dtype=None,
                 name=None):
        self._np_dtype = utils.np_dtype(dtype) if dtype is not None else np.dtype(np.float32)
        npd = self._np_dtype
        self._dim = int(dim)
        self._r_fn = initial_discount_rate_fn
        self._mr = _Param(mean_reversion, self._dim, npd, "mean_reversion")
        self._vol = _Param(volatility, self._dim, npd, "volatility")
        self._corr = None if corr_matrix is None else _Param(corr_matrix, self._dim, npd, "corr_matrix", matrix=True)
        self._generic = (self._mr.callable or self._vol.callable or (self._corr is not None and self._corr.callable)
                         or len(self._mr.jumps) > 0)
        self._mean_reversion = mean_reversion
        self._volatility = volatility
        super().__init__(self._dim, self._drift, self._vol_fn, dtype=utils.torch_dtype(npd),
                         name=name or "hull_white_model")

    # ---- reference accessors --------------------------------------------------
    def mean_reversion(self):
        return self._mean_reversion

    def volatility(self):
        return self._volatility

    def instant_forward_rate(self, t):
        return torch.as_tensor(self._forward(np.asarray(t, np.float64).reshape(-1)))

    # ---- forward curve -----------------------------------------------------------
    def _forward(self, t, derivative=False):
        """f(0, t) = d/dt (r(t) t) (and its derivative) per axis: [len(t), dim] float64.

        The rate function answers input_shape or input_shape + [dim]
        (vector_hull_white.py:208-236).  One that answers [dim] whatever its
        input (a constant curve) is evaluated time by time, on scalars, as the
        reference's sampler does; so is a vector of exactly dim times, where
        the two readings cannot be told apart."""
        t64 = np.asarray(t, np.float64)
        tt = torch.as_tensor(t64, dtype=torch.float64).requires_grad_(True)
        r = torch.as_tensor(self._r_fn(tt), dtype=torch.float64)
        if r.dim() == tt.dim():
            r = r[..., None]
        if tt.dim() == 1 and (tuple(r.shape[:1]) not in ((tt.shape[0],), (1,)) or (tt.shape[0] == self._dim > 1)):
            parts = [self._forward(v.reshape(()), derivative) for v in t64]
            if derivative:
                return (np.stack([p[0] for p in parts]).reshape(len(t64), self._dim),
                        np.stack([p[1] for p in parts]).reshape(len(t64), self._dim))
            return np.stack(parts).reshape(len(t64), self._dim)
        r = torch.broadcast_to(r, tt.shape + (self._dim,))
        f_cols, df_cols = [], []
        for d in range(self._dim):
            y = (r[..., d] * tt).sum()
            (g,) = torch.autograd.grad(y, tt, create_graph=derivative, allow_unused=True)
            g = torch.zeros_like(tt) if g is None else g
            f_cols.append(g.detach())
            if derivative:
                if g.requires_grad:
                    (h,) = torch.autograd.grad(g.sum(), tt, allow_unused=True)
                    h = torch.zeros_like(tt) if h is None else h
                else:
                    h = torch.zeros_like(tt)
                df_cols.append(h.detach())
        f = torch.stack(f_cols, -1).numpy()
        if derivative:
            return f, torch.stack(df_cols, -1).numpy()
        return f

    def _param_at(self, p, t):
        """A parameter at time t; a callable is called with a scalar time, as
        the reference's drift and volatility do (vector_hull_white.py:956-978)."""
        if p.callable:
            tn = np.asarray(t, np.float64)
            v = p.fn(torch.as_tensor(tn.reshape(()) if tn.size == 1 else tn))
            return np.asarray(torch.as_tensor(v).detach().cpu().numpy(), np.float64)
        return p(t)

    # ---- generic (Euler) coefficients (:275-308) -------------------------------
    def _vol_fn(self, t, x):
        tn = np.asarray(utils.to_numpy(t), np.float64).reshape(-1)[:1]
        vol = torch.as_tensor(np.asarray(self._param_at(self._vol, tn)).reshape(-1)[-self._dim:], dtype=x.dtype,
                              device=x.device)
        if self._corr is not None:
            c = np.asarray(self._param_at(self._corr, tn), np.float64).reshape(self._dim, self._dim)
            L = torch.as_tensor(np.linalg.cholesky(c), dtype=x.dtype, device=x.device)
        else:
            L = torch.eye(self._dim, dtype=x.dtype, device=x.device)
        return torch.broadcast_to(vol * L, x.shape[:-1] + (self._dim, self._dim))

    def _drift(self, t, x):
        tn = np.asarray(utils.to_numpy(t), np.float64).reshape(-1)[:1]
        a = np.asarray(self._param_at(self._mr, tn), np.float64).reshape(-1)[-self._dim:]
        s = np.asarray(self._param_at(self._vol, tn), np.float64).reshape(-1)[-self._dim:]
        f, df = self._forward(tn, derivative=True)
        c = df[0] + a * f[0] + s ** 2 / 2 / a * (1 - np.exp(-2 * a * tn[0]))
        at = torch.as_tensor(a, dtype=x.dtype, device=x.device)
        return torch.as_tensor(c, dtype=x.dtype, device=x.device) - at * x

    # ---- exact transition tables (:816-955) -------------------------------------
    def _jumps(self):
        """All parameters' jump locations per axis, sorted: [dim, J] (:816-855)."""
        parts = [self._vol.axis_jumps, self._mr.axis_jumps]
        if self._corr is not None:
            parts.append(np.broadcast_to(self._corr.jumps, (self._dim, len(self._corr.jumps))))
        return np.sort(np.concatenate(parts, axis=1), axis=1).astype(self._np_dtype)

    @staticmethod
    def _search(jl, t):
        """Per-axis searchsorted (left) of t [dim, m] in jl [dim, J]."""
        return np.stack([np.searchsorted(jl[d], t[d], side="left") for d in range(jl.shape[0])])

    def _integrals(self, t):
        """(conditional mean increment, conditional variance) per interval of t: [dim, len(t)-1] each."""
        npd = self._np_dtype
        dim = self._dim
        jl = self._jumps()
        J = jl.shape[1]
        zero = np.zeros((dim, 1), npd)
        jv_vol = self._vol.at(jl) if J else np.zeros((dim, 0), npd)
        jv_mr = self._mr.at(jl) if J else np.zeros((dim, 0), npd)
        knots = np.concatenate([zero, jl[:, :-1]], 1)[:, :J]
        vn = np.concatenate([zero, jl], 1)
        t = np.broadcast_to(np.asarray(t, npd), (dim, len(t)))
        mr_t = self._mr.at(t)
        sig_t = self._vol.at(t)
        ti = self._search(jl, t) if J else np.zeros(t.shape, np.int64)

        def y_int(t0, t1, vol, k):
            return (vol * vol) / (2 * k) * (np.exp(2 * k * t1) - np.exp(2 * k * t0))

        def ex_int(t0, t1, vol, k, y0):
            v = np.exp(k * t1) - np.exp(k * t0) + np.exp(2 * k * t0) * (np.exp(-k * t1) - np.exp(-k * t0))
            return v * vol ** 2 / (2 * k * k) + y0 * (np.exp(-k * t0) - np.exp(-k * t1)) / k

        def gather(a, idx):
            return np.take_along_axis(a, idx, axis=1)

        y_at = np.concatenate([zero, np.cumsum(y_int(knots, jl, jv_vol, jv_mr), 1)], 1)
        ex_at = np.concatenate([zero, np.cumsum(ex_int(knots, jl, jv_vol, jv_mr, y_at[:, :-1]), 1)], 1)
        ex = ex_int(gather(vn, ti), t, sig_t, mr_t, gather(y_at, ti)) + gather(ex_at, ti)
        ex = (ex[:, 1:] - ex[:, :-1]) * np.exp(-mr_t[:, 1:] * t[:, 1:])
        v_at = np.concatenate([zero, np.cumsum(y_int(knots, jl, jv_vol, jv_mr), 1)], 1)
        var = y_int(gather(vn, ti), t, sig_t, mr_t) + gather(v_at, ti)
        var = (var[:, 1:] - var[:, :-1]) * np.exp(-2 * mr_t[:, 1:] * t[:, 1:])
        return ex.astype(npd), var.astype(npd), mr_t.astype(npd)

    def _grid(self, times, times_grid):
        npd = self._np_dtype
        if times_grid is None:
            extra = [self._vol.jumps, self._mr.jumps] + ([self._corr.jumps] if self._corr is not None else [])
            all_times = np.sort(np.concatenate([np.zeros(1, npd), times]
                                               + [np.asarray(e, npd).reshape(-1) for e in extra]))
            idx = np.searchsorted(all_times, times, side="left")
        else:
            all_times = np.asarray(times_grid, npd)
            idx = np.searchsorted(all_times, times, side="left")
            d1 = all_times[np.minimum(idx, len(all_times) - 1)] - times
            d2 = all_times[np.maximum(idx - 1, 0)] - times
            idx = np.where(np.abs(d2) > np.abs(d1), idx, np.maximum(idx - 1, 0))
        keep = np.zeros(len(all_times), bool)
        keep[idx] = True
        return all_times.astype(npd), keep

    # ---- sampling (:319-449) ------------------------------------------------------
    def sample_paths(self, times, num_samples=1, random_type=None, seed=None, skip=0, time_step=None,
                     times_grid=None, normal_draws=None, validate_args=False, name=None):
        """Short-rate paths [num_samples, k, dim]."""
        del name
        npd = self._np_dtype
        td = utils.torch_dtype(npd)
        times = np.asarray(utils.to_numpy(times, npd))
        if times.ndim != 1:
            raise ValueError("`times` should be a rank 1 Tensor. Rank is {} instead.".format(times.ndim))
        if self._generic:
            if time_step is None and times_grid is None:
                raise ValueError("When `mean_reversion` or `volatility` is a time dependent callable, "
                                 "`time_step` or `times_grid` should be supplied.")
            x0 = self._forward(np.zeros(1))[0].astype(npd)
            return euler_sampling.sample(self._dim, self._drift, self._vol_fn, times, time_step=time_step,
                                         num_samples=num_samples, initial_state=x0, random_type=random_type,
                                         seed=seed, skip=skip, times_grid=times_grid, normal_draws=normal_draws,
                                         dtype=npd)
        device = _lib.require_cuda()
        all_times, keep = self._grid(times, times_grid)
        k = len(times)
        dt = (all_times[1:] - all_times[:-1]).astype(npd)
        steps = len(dt)
        step_slot, init_slot, steps_exec, unwritten = utils.plan_output_slots(keep, k, int(keep[0]))
        ex, var, mr_t = self._integrals(all_times)
        decay = np.exp(-mr_t[:, 1:] * dt).astype(npd)  # [dim, steps]
        vx = np.sqrt(np.maximum(var, npd.type(0))).astype(npd)
        vx = np.where(vx > 0, vx, npd.type(0))
        table = np.stack([decay.T, ex.T, vx.T], -1)[:steps_exec]  # [steps, dim, 3]
        f0 = self._forward(all_times[:steps_exec + 1].astype(np.float64)).astype(npd)  # [steps+1, dim]
        keep_alive = []
        chol_t = None
        if self._corr is not None:
            tc = (all_times + np.min(dt) / 2)[:steps_exec] if steps else all_times[:0]
            c = self._corr(tc).astype(np.float64)
            chol_t = torch.as_tensor(np.linalg.cholesky(c).astype(npd)).to(device)
        if normal_draws is not None:
            dr = normal_draws if isinstance(normal_draws, torch.Tensor) else torch.as_tensor(
                utils.to_numpy(normal_draws, npd))
            if dr.shape[-1] != self._dim:
                raise ValueError("`dim` should be equal to `normal_draws.shape[2]`")
            dr = dr.to(device=device, dtype=td).contiguous()
            if validate_args and dr.shape[1] != steps:
                raise ValueError("`tf.shape(normal_draws)[1]` should be equal to the number of all `times` plus "
                                 "the number of all jumps of the piecewise constant parameters.")
            keep_alive.append(dr)
            num_samples = int(dr.shape[0])
            draws = mvn.memory_draws(dr, path_axis=0, step_axis=1)
        else:
            rt = RandomType.PSEUDO if random_type is None else random_type
            if rt in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
                q = utils.generate_mc_normal_draws(self._dim, steps, int(num_samples), rt, skip=skip, seed=seed,
                                                   dtype=td)
                keep_alive.append(q)
                draws = mvn.memory_draws(q, path_axis=1, step_axis=0)
            else:
                draws = mvn.philox_draws(rt, seed, int(num_samples))
        N = int(num_samples)
        out = (torch.zeros if unwritten else torch.empty)((N, k, self._dim), dtype=td, device=device)
        tab_t = torch.as_tensor(np.ascontiguousarray(table)).to(device)
        f0_t = torch.as_tensor(np.ascontiguousarray(f0)).to(device)
        slots_t = torch.as_tensor(np.asarray(step_slot, np.int32)).to(device)
        a = _lib.HullWhiteArgs()
        a.dtype = _lib.dtype_code(td)
        a.dim = self._dim
        a.num_paths = N
        a.num_steps = steps_exec
        a.table = tab_t.data_ptr()
        a.f0 = f0_t.data_ptr()
        a.chol = chol_t.data_ptr() if chol_t is not None else None
        a.slots = slots_t.data_ptr()
        a.draws = draws
        a.output.ptr = out.data_ptr()
        a.output.num_slots = k
        a.output.init_slot = init_slot
        _lib.call("tqf_hull_white_paths", a, _lib.stream_ptr(device))
        return out

    # ---- zero-coupon bonds (:594-639, 783-874) ------------------------------------
    def discount_bond_price(self, short_rate, times, maturities, name=None):
        """P(t, T | r(t)) for short rates of shape batch_shape + [dim]."""
        del name
        npd = self._np_dtype
        sr = torch.as_tensor(short_rate)
        device = sr.device if sr.is_cuda else _lib.require_cuda()
        sr = sr.to(device=device, dtype=utils.torch_dtype(npd))
        t = np.asarray(utils.to_numpy(times), npd)
        T = np.asarray(utils.to_numpy(maturities), npd)
        tf_ = t.reshape(-1)
        # y(t) = exp(-2 a t) int_0^t sigma(u)^2 exp(2 a u) du
        dim = self._dim
        jl = self._jumps()
        J = jl.shape[1]
        zero = np.zeros((dim, 1), npd)
        knots = np.concatenate([zero, jl[:, :-1]], 1)[:, :J]
        jv_vol = self._vol.at(jl) if J else np.zeros((dim, 0), npd)
        jv_mr = self._mr.at(jl) if J else np.zeros((dim, 0), npd)
        yb = jv_vol * jv_vol / (2 * jv_mr) * (np.exp(2 * jv_mr * jl) - np.exp(2 * jv_mr * knots))
        y_at = np.concatenate([zero, np.cumsum(yb, 1)], 1)
        vn = np.concatenate([zero, jl], 1)
        tb = np.broadcast_to(tf_, (dim, tf_.size))
        ti = self._search(jl, tb) if J else np.zeros(tb.shape, np.int64)
        mr_t = self._mr.at(tb)
        sig_t = self._vol.at(tb)
        t0 = np.take_along_axis(vn, ti, 1)
        y = sig_t * sig_t / (2 * mr_t) * (np.exp(2 * mr_t * tf_) - np.exp(2 * mr_t * t0)) + np.take_along_axis(
            y_at, ti, 1)
        y = (np.exp(-2 * mr_t * tf_) * y).T.reshape(t.shape + (dim,))
        mr = mr_t.T.reshape(t.shape + (dim,))
        f0 = self._forward(tf_.astype(np.float64)).reshape(t.shape + (dim,))

        def r_at(x):
            rr = torch.as_tensor(self._r_fn(torch.as_tensor(np.asarray(x, np.float64).reshape(-1))),
                                 dtype=torch.float64).numpy()
            rr = rr.reshape(len(np.asarray(x).reshape(-1)), -1)
            return np.broadcast_to(rr, (rr.shape[0], dim)).reshape(np.shape(x) + (dim,))

        p0t = np.exp(-r_at(t) * t[..., None])
        p0tT = np.exp(-r_at(T) * T[..., None]) / p0t
        g = (1.0 - np.exp(-mr * (T[..., None] - t[..., None]))) / mr
        cst = lambda v: torch.as_tensor(np.asarray(v, npd)).to(device)  # noqa: E731
        x_t = sr - cst(f0)
        return cst(p0tT) * torch.exp(-x_t * cst(g) - 0.5 * cst(y) * cst(g) ** 2)


class HullWhiteModel1F(VectorHullWhiteModel):
    """One-factor Hull-White (one_factor.py:16-137)."""

    def __init__(self, mean_reversion, volatility, initial_discount_rate_fn, dtype=None, name=None):
        super().__init__(1, mean_reversion, volatility, initial_discount_rate_fn, dtype=dtype,
                         name=name or "hull_white_model_1f")


__all__ = ["VectorHullWhiteModel", "HullWhiteModel1F"]
