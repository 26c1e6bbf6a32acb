"""Structured drift / volatility callables that the engine recognises.

Each object is an ordinary ``(t, x) -> tensor`` callable (torch ops, usable
anywhere the reference takes ``drift_fn`` / ``volatility_fn``), and also
carries its parameters so that ``euler_sampling.sample`` can run the whole
time loop in one fused kernel instead of calling it once per step.

* ``AffineDrift``:  a(x) = m + M x
* ``ScaledVolatility``:  B(x)_ij = (s0_i + s1_i x_i) C_ij
  -> ``tqf_euler_affine`` (GBM, arithmetic BM, OU, correlated GBM in levels)
* ``HestonFullTruncation``: drift [r - v+/2, kappa (theta - v+)] and volatility
  [[sqrt v+, 0], [xi rho sqrt v+, xi sqrt(1 - rho^2) sqrt v+]], v+ = max(v, 0)
  -> ``tqf_heston_euler``.  Parameters may be PiecewiseConstantFunc.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf.math.piecewise import PiecewiseConstantFunc


def _arr(x, n=None):
    a = np.asarray(x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else x, dtype=np.float64)
    if n is not None and a.ndim == 0:
        a = np.full(n, float(a))
    return a


class AffineDrift:
    def __init__(self, m, M):
        self.M = _arr(M)
        d = self.M.shape[0]
        self.m = _arr(m, d).reshape(d)
        if self.M.shape != (d, d):
            raise ValueError(f"M must be [{d}, {d}], got {self.M.shape}")
        self.dim = d

    def __call__(self, t, x):
        m = torch.as_tensor(self.m, dtype=x.dtype, device=x.device)
        M = torch.as_tensor(self.M, dtype=x.dtype, device=x.device)
        return m + x @ M.T


class ScaledVolatility:
    def __init__(self, s0, s1, C):
        self.C = _arr(C)
        d = self.C.shape[0]
        self.s0 = _arr(s0, d).reshape(d)
        self.s1 = _arr(s1, d).reshape(d)
        self.dim = d

    def __call__(self, t, x):
        s0 = torch.as_tensor(self.s0, dtype=x.dtype, device=x.device)
        s1 = torch.as_tensor(self.s1, dtype=x.dtype, device=x.device)
        C = torch.as_tensor(self.C, dtype=x.dtype, device=x.device)
        return (s0 + s1 * x)[..., :, None] * C


def gbm(mu, sigma, corr=None):
    """dX_i = mu_i X_i dt + sigma_i X_i (L dW)_i with L = chol(corr)."""
    mu = _arr(mu).reshape(-1)
    sigma = _arr(sigma, mu.size).reshape(-1)
    d = mu.size
    L = np.eye(d) if corr is None else np.linalg.cholesky(_arr(corr))
    return AffineDrift(np.zeros(d), np.diag(mu)), ScaledVolatility(np.zeros(d), sigma, L)


def _param(p, t):
    if isinstance(p, PiecewiseConstantFunc):
        return np.asarray(p(np.asarray(t, dtype=p.dtype())), dtype=np.float64)
    return np.full(np.shape(t), float(_arr(p)), dtype=np.float64)


class HestonFullTruncation:
    """Coefficient pair of the full-truncation Heston model in log-spot form."""

    def __init__(self, r, kappa, theta, xi, rho):
        self.r, self.kappa, self.theta, self.xi, self.rho = r, kappa, theta, xi, rho
        outer = self

        class _Drift:
            heston = outer

            def __call__(self, t, x):
                return outer.drift(t, x)

        class _Vol:
            heston = outer

            def __call__(self, t, x):
                return outer.volatility(t, x)

        self.drift_fn = _Drift()
        self.volatility_fn = _Vol()

    def params_at(self, t):
        """(r, kappa, theta, xi*rho, xi*sqrt(1-rho^2)) at times t (float64)."""
        t = np.asarray(t, dtype=np.float64)
        r, k, th = _param(self.r, t), _param(self.kappa, t), _param(self.theta, t)
        xi, rho = _param(self.xi, t), _param(self.rho, t)
        return r, k, th, xi * rho, xi * np.sqrt(1.0 - rho * rho)

    def _scalars(self, t, like):
        tt = float(t.item()) if isinstance(t, torch.Tensor) else float(t)
        vals = [float(v) for v in self.params_at(np.array(tt))]
        return [torch.as_tensor(v, dtype=like.dtype, device=like.device) for v in vals]

    def drift(self, t, x):
        r, k, th, _, _ = self._scalars(t, x)
        vp = torch.clamp(x[..., 1], min=0)
        return torch.stack([r - 0.5 * vp, k * (th - vp)], -1)

    def volatility(self, t, x):
        _, _, _, xirho, xisq = self._scalars(t, x)
        sq = torch.sqrt(torch.clamp(x[..., 1], min=0))
        z = torch.zeros_like(sq)
        return torch.stack([torch.stack([sq, z], -1), torch.stack([xirho * sq, xisq * sq], -1)], -2)


def heston_full_truncation(r, kappa, theta, xi, rho):
    """Returns (drift_fn, volatility_fn) of the full-truncation Heston model."""
    h = HestonFullTruncation(r, kappa, theta, xi, rho)
    return h.drift_fn, h.volatility_fn


__all__ = ["AffineDrift", "ScaledVolatility", "gbm", "HestonFullTruncation", "heston_full_truncation"]
