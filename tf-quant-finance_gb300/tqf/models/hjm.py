"""Gaussian HJM (multi-factor Hull-White) model on the GPU
(tff/models/hjm/gaussian_hjm.py:31-465, quasi_gaussian_hjm.py:366-548).

Factors dx_i = (sum_j y_ij(t) - k_i x_i) dt + sigma_i(t) (L dW)_i, short rate
r = sum_i x_i + f(0, t).  The deterministic state y(t) (piecewise-constant
volatility, closed-form integrals) and the per-step volatility factors are
tabulated on the host; ``tqf_hjm_paths`` runs the reference's Euler scheme on
its grid with the factors in registers and accumulates the short rate and the
discount factor D = prod exp(-r dt) along the way.  Zero-coupon bond curves are
reconstituted from the sampled factors with torch on the device.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.math.piecewise import PiecewiseConstantFunc
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import utils


class GaussianHJM:
    """GaussianHJM(dim, mean_reversion, volatility, initial_discount_rate_fn,
    corr_matrix=None, dtype=None, name=None)."""

    def __init__(self, dim, mean_reversion, volatility, initial_discount_rate_fn, corr_matrix=None, dtype=None,
                 name=None):
        self._name = name or "gaussian_hjm_model"
        self._np_dtype = utils.np_dtype(dtype) if dtype is not None else np.dtype(np.float32)
        npd = self._np_dtype
        self._dim = self._factors = int(dim)
        self._r_fn = initial_discount_rate_fn
        self._mean_reversion = np.asarray(utils.to_numpy(mean_reversion), npd).reshape(self._dim)
        if callable(volatility) and not isinstance(volatility, PiecewiseConstantFunc):
            raise NotImplementedError("callable volatility: the closed-form state y(t) needs piecewise-constant "
                                      "volatility (gaussian_hjm.py:459-465)")
        if isinstance(volatility, PiecewiseConstantFunc):
            jl = np.asarray(volatility.jump_locations(), npd)
            vals = np.asarray(volatility.values(), npd)
            if jl.ndim == 2:
                if not np.all(jl == jl[:1]):
                    raise NotImplementedError("per-factor volatility jumps must coincide")
                jl = jl[0]
                vals = vals.reshape(self._dim, -1)
            else:
                vals = np.broadcast_to(vals.reshape(len(jl) + 1, -1).T, (self._dim, len(jl) + 1))
            self._jumps, self._vol_values = jl, np.ascontiguousarray(vals, npd)
        else:
            v = np.asarray(utils.to_numpy(volatility), npd).reshape(self._dim)
            self._jumps, self._vol_values = np.zeros(0, npd), v[:, None].copy()
        self._volatility = volatility
        rho = np.eye(self._dim) if corr_matrix is None else np.asarray(utils.to_numpy(corr_matrix), np.float64)
        self._rho = rho.astype(npd)
        self._sqrt_rho = np.linalg.cholesky(rho).astype(npd)

    # ---- accessors ------------------------------------------------------------------
    def dim(self):
        return self._dim

    def dtype(self):
        return utils.torch_dtype(self._np_dtype)

    def name(self):
        return self._name

    def mean_reversion(self):
        return self._mean_reversion

    def volatility(self):
        return self._volatility

    def _sigma(self, t):
        idx = np.searchsorted(self._jumps, np.asarray(t, self._np_dtype), side="left")
        return self._vol_values[:, idx]

    def _forward(self, t):
        """f(0, t) = d/dt (r(t) t) in float64 (gaussian_hjm.py:166-179)."""
        tt = torch.as_tensor(np.asarray(t, np.float64)).requires_grad_(True)
        r = torch.as_tensor(self._r_fn(tt), dtype=torch.float64)
        y = torch.broadcast_to(r, tt.shape) * tt
        (g,) = torch.autograd.grad(y.sum(), tt, allow_unused=True)
        return (torch.zeros_like(tt) if g is None else g).detach().numpy()

    def _r(self, t):
        return np.broadcast_to(torch.as_tensor(self._r_fn(torch.as_tensor(np.asarray(t, np.float64))),
                                               dtype=torch.float64).numpy(), np.shape(t))

    def _state_y_np(self, t):
        npd = self._np_dtype
        t = np.asarray(t, npd).reshape(-1)
        k = self._mean_reversion
        mr2 = (k[:, None] + k[None, :])[:, :, None]
        knots = np.concatenate([np.zeros(1, npd), self._jumps])

        def integ(sig, lo, hi):
            s2 = self._rho[:, :, None] * (sig[:, None, :] * sig[None, :, :])
            return s2 / mr2 * (np.exp(mr2 * hi) - np.exp(mr2 * lo))

        J = len(self._jumps)
        between = integ(self._sigma(self._jumps), knots[:-1][None, None, :], self._jumps[None, None, :]) if J else \
            np.zeros((self._dim, self._dim, 0), npd)
        at_knots = np.concatenate([np.zeros((self._dim, self._dim, 1), npd), np.cumsum(between, -1)], -1)
        ti = np.searchsorted(self._jumps, t, side="left")
        v = integ(self._sigma(t), knots[ti][None, None, :], t[None, None, :]) + at_knots[:, :, ti]
        return (np.exp(-mr2 * t) * v).astype(npd)

    def state_y(self, t, name=None):
        """y(t): [dim, dim, num_times] (gaussian_hjm.py:305-360)."""
        del name
        return torch.as_tensor(self._state_y_np(utils.to_numpy(t))).to(_lib.require_cuda())

    def discount_bond_price(self, state, times, maturities, name=None):
        """P(t, T) given the factors x(t): [num_times] (gaussian_hjm.py:362-402)."""
        del name
        npd = self._np_dtype
        device = _lib.require_cuda()
        t = np.asarray(utils.to_numpy(times), npd).reshape(-1)
        T = np.asarray(utils.to_numpy(maturities), npd).reshape(-1)
        y = torch.as_tensor(np.transpose(self._state_y_np(t), (2, 0, 1))).to(device)  # [n, d, d]
        x = torch.as_tensor(np.asarray(utils.to_numpy(state), npd)).to(device).reshape(len(t), self._dim)
        p0tT = np.exp(-self._r(T) * T) / np.exp(-self._r(t) * t)
        g = torch.as_tensor(((1.0 - np.exp(-self._mean_reversion * (T - t)[:, None])) / self._mean_reversion)
                            .astype(npd)).to(device)
        term1 = (x * g).sum(-1)
        term2 = (g * torch.einsum("nij,nj->ni", y, g)).sum(-1)
        return torch.as_tensor(p0tT.astype(npd)).to(device) * torch.exp(-term1 - 0.5 * term2)

    # ---- sampling ---------------------------------------------------------------------
    def sample_paths(self, times, num_samples, time_step=None, num_time_steps=None, random_type=None, seed=None,
                     skip=0, name=None, normal_draws=None):
        """(short rates [N, k], discount factors [N, k], factors x [N, k, dim],
        y [N, k, dim^2]) (gaussian_hjm.py:229-303, 404-457).  ``normal_draws``
        ([N, steps, dim], extension) supplies the Euler increments."""
        del name
        npd = self._np_dtype
        td = utils.torch_dtype(npd)
        times = np.asarray(utils.to_numpy(times), npd)
        if times.ndim != 1:
            raise ValueError("`times` should be a rank 1 Tensor. Rank is {} instead.".format(times.ndim))
        if time_step is None and num_time_steps is None:
            raise ValueError("When `times_grid` is not supplied, either `num_time_steps` or `time_step` should "
                             "be defined.")
        ts = time_step if num_time_steps is None else times[-1] / npd.type(int(num_time_steps))
        all_times, _, ti = utils.prepare_grid(times=times, time_step=npd.type(ts), dtype=npd,
                                              num_time_steps=num_time_steps)
        all_times = np.asarray(all_times, npd)
        ti = np.asarray(ti, np.int64)
        G = len(all_times)
        steps = G - 1
        dt = (all_times[1:] - all_times[:-1]).astype(npd)
        sdt = np.sqrt(dt).astype(npd)
        y = self._state_y_np(all_times)  # [d, d, G]
        sig = self._sigma(all_times)     # [d, G]
        d = self._dim
        table = np.zeros((steps, 2 + d + d * d), npd)
        table[:, 0] = dt
        table[:, 1] = sdt
        table[:, 2:2 + d] = y[:, :, 1:].sum(1).T
        table[:, 2 + d:] = (self._sqrt_rho[None] * sig[:, 1:].T[:, :, None]).reshape(steps, d * d)
        f0 = self._forward(all_times.astype(np.float64)).astype(npd)
        uniq, inverse = np.unique(ti, return_inverse=True)
        grid_slot = -np.ones(G, np.int32)
        grid_slot[uniq] = np.arange(len(uniq), dtype=np.int32)
        device = _lib.require_cuda()
        keep_alive = []
        if normal_draws is not None:
            dr = normal_draws if isinstance(normal_draws, torch.Tensor) else torch.as_tensor(
                utils.to_numpy(normal_draws, npd))
            dr = dr.to(device=device, dtype=td).contiguous()
            keep_alive.append(dr)
            num_samples = int(dr.shape[0])
            draws = mvn.memory_draws(dr, path_axis=0, step_axis=1)
        else:
            rt = RandomType.PSEUDO if random_type is None else random_type
            if rt in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
                q = utils.generate_mc_normal_draws(d, steps, int(num_samples), rt, skip=skip, seed=seed, dtype=td)
                keep_alive.append(q)
                draws = mvn.memory_draws(q, path_axis=1, step_axis=0)
            else:
                draws = mvn.philox_draws(rt, seed, int(num_samples))
        N = int(num_samples)
        U = len(uniq)
        rates = torch.empty((N, U), dtype=td, device=device)
        dfs = torch.empty((N, U), dtype=td, device=device)
        xs = torch.empty((N, U, d), dtype=td, device=device)
        tab_t = torch.as_tensor(np.ascontiguousarray(table)).to(device)
        k_t = torch.as_tensor(self._mean_reversion).to(device)
        f0_t = torch.as_tensor(f0).to(device)
        slot_t = torch.as_tensor(grid_slot).to(device)
        a = _lib.HjmArgs()
        a.dtype = _lib.dtype_code(td)
        a.dim = d
        a.num_paths = N
        a.num_steps = steps
        a.num_slots = U
        a.table = tab_t.data_ptr()
        a.mean_reversion = k_t.data_ptr()
        a.f0 = f0_t.data_ptr()
        a.grid_slot = slot_t.data_ptr()
        a.draws = draws
        a.rate_out, a.df_out, a.x_out = rates.data_ptr(), dfs.data_ptr(), xs.data_ptr()
        _lib.call("tqf_hjm_paths", a, _lib.stream_ptr(device))
        inv = torch.as_tensor(inverse.reshape(-1)).to(device)
        y_req = torch.as_tensor(np.transpose(y, (2, 0, 1))[ti].reshape(len(ti), d * d)).to(device)
        return rates[:, inv], dfs[:, inv], xs[:, inv], y_req.unsqueeze(0).expand(N, len(ti), d * d)

    def sample_discount_curve_paths(self, times, curve_times, num_samples, time_step=None, num_time_steps=None,
                                    random_type=None, seed=None, skip=0, name=None):
        """(bond prices [N, num_curve_nodes, k] for maturities t + curve_times,
        short rates, discount factors) (quasi_gaussian_hjm.py:366-457)."""
        del name
        npd = self._np_dtype
        rates, dfs, x, _ = self.sample_paths(times, num_samples, time_step=time_step, num_time_steps=num_time_steps,
                                             random_type=random_type, seed=seed, skip=skip)
        device = x.device
        t = np.asarray(utils.to_numpy(times), npd).reshape(-1)
        c = np.asarray(utils.to_numpy(curve_times), npd).reshape(-1)
        T = t[None, :] + c[:, None]  # [C, k]
        y = torch.as_tensor(np.transpose(self._state_y_np(t), (2, 0, 1))).to(device)  # [k, d, d]
        p0tT = np.exp(-self._r(T) * T) / np.exp(-self._r(t) * t)[None, :]
        g = (1.0 - np.exp(-self._mean_reversion * (T - t[None, :])[..., None])) / self._mean_reversion  # [C, k, d]
        g_t = torch.as_tensor(g.astype(npd)).to(device)
        term1 = torch.einsum("nkd,ckd->nck", x, g_t)
        term2 = (g_t * torch.einsum("kij,ckj->cki", y, g_t)).sum(-1)  # [C, k]
        bonds = torch.as_tensor(p0tT.astype(npd)).to(device)[None] * torch.exp(-term1 - 0.5 * term2[None])
        return bonds, rates, dfs


__all__ = ["GaussianHJM"]
