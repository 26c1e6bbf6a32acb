"""Multivariate GBM restatement
(tff/models/geometric_brownian_motion/multivariate_geometric_brownian_motion.py:229-281)
and a torch-CPU autograd restatement for pathwise gradients (the quantity
tf.GradientTape returns through the same graph)."""

from __future__ import annotations

import numpy as np


def sample_with_draws(means, vols, corr, times, x0, draws, dtype):
    """draws: [k, N, d] (time-major, as the reference after its transpose).
    Returns [N, k, d]."""
    d_ = np.dtype(dtype).type
    times = np.concatenate([[0], np.asarray(times, dtype=dtype)]).astype(dtype)
    dt = (times[1:] - times[:-1]).astype(dtype)[:, None, None]
    means = np.asarray(means, dtype=dtype)
    vols = np.asarray(vols, dtype=dtype)
    if corr is None:
        incr = draws.astype(dtype)
    else:
        L = np.linalg.cholesky(np.asarray(corr, dtype=np.float64)).astype(dtype)
        incr = np.einsum("ij,knj->kni", L, draws.astype(dtype)).astype(dtype)
    log_inc = ((means - vols ** 2 / d_(2)) * dt + np.sqrt(dt) * vols * incr).astype(dtype)
    cs = np.cumsum(log_inc, axis=0).astype(dtype)
    return (np.asarray(x0, dtype=dtype)[None, None, :] * np.exp(cs)).transpose(1, 0, 2).astype(dtype)


def basket_price_torch(spots, vols, rate, corr, weights, strike, times, draws, is_call=True):
    """Discounted basket option price as a differentiable torch-CPU graph
    (float64); gradients by autograd play the role of the reference's
    GradientTape.  draws: [k, N, d] numpy."""
    import torch
    t = torch.as_tensor(np.concatenate([[0.0], np.asarray(times, np.float64)]))
    dt = (t[1:] - t[:-1])[:, None, None]
    L = torch.as_tensor(np.linalg.cholesky(np.asarray(corr, np.float64)))
    z = torch.as_tensor(draws, dtype=torch.float64)
    incr = torch.einsum("ij,knj->kni", L, z)
    log_inc = (rate - vols ** 2 / 2) * dt + torch.sqrt(dt) * vols * incr
    S_T = spots * torch.exp(log_inc.sum(0))
    B = (S_T * torch.as_tensor(np.asarray(weights, np.float64))).sum(-1)
    pay = torch.clamp(B - strike if is_call else strike - B, min=0)
    T = float(t[-1])
    return torch.exp(-rate * T) * pay.mean()


def univariate_with_draws(mean_int, volsq_int, x0, draws, dtype):
    """Univariate GBM exact scheme (univariate_geometric_brownian_motion.py:261-318):
    x0 exp(cumsum((int mu - int sigma^2 / 2) + sqrt(int sigma^2) z)); draws [N, k]."""
    dt_ = np.dtype(dtype).type
    mean_int = np.asarray(mean_int, dtype)
    volsq_int = np.asarray(volsq_int, dtype)
    inc = ((mean_int - volsq_int / dt_(2)) + np.sqrt(volsq_int) * np.asarray(draws, dtype)).astype(dtype)
    return (dt_(x0) * np.exp(np.cumsum(inc, axis=-1).astype(dtype))).astype(dtype)
