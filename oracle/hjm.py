"""Gaussian HJM (Hull-White multi-factor) model, restated in NumPy (test oracle).

Test infrastructure only: the product path never imports this module.

Follows tf_quant_finance/models/hjm/gaussian_hjm.py:
  state_y            :305-360  y_ij(t) = exp(-(k_i + k_j) t) int_0^t rho_ij
                               sigma_i(u) sigma_j(u) exp((k_i + k_j) u) du
                               (piecewise-constant sigma, shared knots)
  drift / volatility :209-227  a(t, x) = sum_j y_ij(t) - k_i x_i,
                               B(t)_rc = L_rc sigma_r(t), L = chol(rho)
  _sample_paths      :404-457  Euler on the grid (utils.prepare_grid), rates
                               sum_k x_k + f0(t), discount factors
                               cumprod(exp(-r_i dt_i)) with 1 first
and quasi_gaussian_hjm.py:515-548 (_bond_reconstitution).
"""

from __future__ import annotations

import numpy as np


class Model:
    def __init__(self, dim, mr, vol_jumps, vol_values, rho, dtype):
        self.dim, self.dtype = dim, np.dtype(dtype)
        self.k = np.asarray(mr, dtype)
        self.jumps = np.asarray(vol_jumps if vol_jumps is not None else [], dtype)
        self.vv = np.asarray(vol_values, dtype).reshape(dim, len(self.jumps) + 1)
        self.rho = np.eye(dim) if rho is None else np.asarray(rho, np.float64)
        self.L = np.linalg.cholesky(self.rho).astype(dtype)
        self.rho = self.rho.astype(dtype)

    def sigma(self, t):
        idx = np.searchsorted(self.jumps, np.asarray(t, self.dtype), side="left")
        return self.vv[:, idx]  # [dim, T]

    def state_y(self, t):
        t = np.asarray(t, self.dtype)
        mr2 = (self.k[:, None] + self.k[None, :])[:, :, None]
        J = len(self.jumps)
        knots = np.concatenate([[0], self.jumps]).astype(self.dtype)

        def integ(sig, lo, hi):
            s2 = self.rho[:, :, None] * (sig[:, None, :] * sig[None, :, :])
            return s2 / mr2 * (np.exp(mr2 * hi) - np.exp(mr2 * lo))

        between = integ(self.sigma(self.jumps), knots[:-1][None, None, :], self.jumps[None, None, :]) if J else \
            np.zeros((self.dim, self.dim, 0), self.dtype)
        at_knots = np.concatenate([np.zeros((self.dim, self.dim, 1), self.dtype), np.cumsum(between, -1)], -1)
        ti = np.searchsorted(self.jumps, t, side="left")
        v = integ(self.sigma(t), knots[ti][None, None, :], t[None, None, :]) + at_knots[:, :, ti]
        return (np.exp(-mr2 * t) * v).astype(self.dtype)

    def bond(self, x_t, times, maturities, r_fn):
        times = np.asarray(times, self.dtype)
        maturities = np.asarray(maturities, self.dtype)
        y = np.transpose(self.state_y(times), (2, 0, 1))  # [T, d, d]
        p0t = np.exp(-r_fn(times) * times)
        p0tT = np.exp(-r_fn(maturities) * maturities) / p0t
        g = (1.0 - np.exp(-self.k * (maturities - times)[:, None])) / self.k  # [T, d]
        term1 = np.sum(np.asarray(x_t) * g, -1)
        term2 = np.sum(g * np.einsum("tij,tj->ti", y, g), -1)
        return p0tT * np.exp(-term1 - 0.5 * term2)

    def sample(self, all_times, time_indices, draws, f0_fn):
        """draws [steps, N, d] -> (rates [N, k], dfs [N, k], x [N, k, d])."""
        dt_ = self.dtype.type
        t = np.asarray(all_times, self.dtype)
        dts = (t[1:] - t[:-1]).astype(self.dtype)
        N = draws.shape[1]
        x = np.zeros((N, self.dim), self.dtype)
        xs = [x]
        y = self.state_y(t)  # [d, d, G]
        sig = self.sigma(t)  # [d, G]
        for i in range(len(dts)):
            c = y[:, :, i + 1].sum(-1)
            drift = c - self.k * x
            B = self.L * sig[:, i + 1][:, None]
            dw = (draws[i].astype(self.dtype) * np.sqrt(dts[i]).astype(self.dtype)).astype(self.dtype)
            x = (x + dts[i] * drift + np.einsum("rc,nc->nr", B, dw)).astype(self.dtype)
            xs.append(x)
        X = np.stack(xs, 1)  # [N, G, d]
        rates = (X.sum(-1) + f0_fn(t)[None, :]).astype(self.dtype)
        disc = np.exp(-rates[:, :-1] * dts).astype(self.dtype)
        df = np.cumprod(np.concatenate([np.ones((N, 1), self.dtype), disc], 1), axis=1).astype(self.dtype)
        ti = np.asarray(time_indices)
        return rates[:, ti], df[:, ti], X[:, ti]
