"""Euler–Maruyama restatement (tff/models/euler_sampling.py:335-537).

`sample_with_draws` runs the reference's while-loop semantics (drift and
volatility evaluated at t_{i+1} = times[i+1], dw = draws[i] * sqrt(dt_i),
x += dt_i a + B dw, TensorArray writes at written_count) in the given dtype.
"""

from __future__ import annotations

import numpy as np


def sample_with_draws(drift_fn, volatility_fn, all_times, keep_mask, num_requested_times, x0,
                      draws, dtype):
    """x0: [N, d]; draws: [steps, N, d]. Returns [N, k, d] (k = 1 when
    num_requested_times == 1, as the reference's expand_dims branch)."""
    dt_ = np.dtype(dtype).type
    times = np.asarray(all_times, dtype=dtype)
    dt = (times[1:] - times[:-1]).astype(dtype)
    sqrt_dt = np.sqrt(dt).astype(dtype)
    x = np.array(x0, dtype=dtype)
    steps = len(dt)
    k = int(num_requested_times)
    record = k != 1
    result = np.zeros((k,) + x.shape, dtype=dtype) if record else None
    if record:
        result[0] = x
    wc = int(keep_mask[0])
    i = 0
    while i < steps and wc < k:
        t = times[i + 1]
        dw = (draws[i].astype(dtype) * sqrt_dt[i]).astype(dtype)
        dt_inc = (dt[i] * drift_fn(t, x)).astype(dtype)
        dw_inc = np.einsum("...ij,...j->...i", volatility_fn(t, x), dw).astype(dtype)
        x = (x + dt_inc + dw_inc).astype(dtype)
        if record:
            result[wc] = x
        wc += int(keep_mask[i + 1])
        i += 1
    if not record:
        return x[..., None, :]
    return np.moveaxis(result, 0, -2)


def heston_ft_coefficients(r, kappa, theta, xi, rho, dtype):
    """Full-truncation Heston drift/volatility in the Euler sampler's form:
    state (log-spot, variance), drift [r - v+/2, kappa (theta - v+)], volatility
    [[sqrt v+, 0], [xi rho sqrt v+, xi sqrt(1 - rho^2) sqrt v+]] (the
    HestonModel coefficients, heston_model.py:143-173, with v -> max(v, 0)
    and the rate r in the log-spot drift)."""
    dt_ = np.dtype(dtype).type
    r, kappa, theta, xi, rho = (dt_(v) for v in (r, kappa, theta, xi, rho))
    xirho = dt_(xi * rho)
    xisq = dt_(xi * dt_(np.sqrt(dt_(1) - rho * rho)))

    def drift(t, x):
        vp = np.maximum(x[..., 1], dt_(0))
        return np.stack([r - dt_(0.5) * vp, kappa * (theta - vp)], -1).astype(dtype)

    def vol(t, x):
        vp = np.maximum(x[..., 1], dt_(0))
        sq = np.sqrt(vp)
        z = np.zeros_like(sq)
        row0 = np.stack([sq, z], -1)
        row1 = np.stack([xirho * sq, xisq * sq], -1)
        return np.stack([row0, row1], -2).astype(dtype)

    return drift, vol
