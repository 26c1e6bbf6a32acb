"""Heston restatements.

* `qe_sample_with_draws`: HestonModel._sample_paths with the QE variance step
  and the central log-spot step (heston_model.py:322-460, 522-572), dtype
  arithmetic as in TensorFlow, draws [steps, N, 2] (component 0 -> variance,
  component 1 -> log-spot).  Also reports, per path, whether any step came
  within `near` (relative) of a branch decision (psi vs 1.5, u vs p), where a
  last-ulp difference between two correct implementations can flip the
  branch.
* `drift_fn` / `volatility_fn`: HestonModel coefficients (heston_model.py:143-173).
"""

from __future__ import annotations

import numpy as np
from scipy.special import erf

SQRT_2 = np.sqrt(2.0)


def piecewise_value(jumps, values, x):
    """Left-continuous PiecewiseConstantFunc.__call__ (tff/math/piecewise.py:144-176)."""
    jumps = np.asarray(jumps)
    values = np.asarray(values)
    idx = np.searchsorted(jumps, np.asarray(x), side="left")
    return values[idx]


def param_at(param, t, dtype):
    if isinstance(param, tuple):  # (jumps, values)
        return piecewise_value(np.asarray(param[0], dtype), np.asarray(param[1], dtype), t).astype(dtype)
    return (np.asarray(param, dtype=dtype) * np.ones_like(t, dtype=dtype)).astype(dtype)


def drift_fn(kappa, theta, dtype):
    def f(t, x):
        t = np.asarray([t], dtype=dtype)
        k = param_at(kappa, t, dtype)[0]
        th = param_at(theta, t, dtype)[0]
        var = x[..., 1]
        return np.stack([-var / 2, k * (th - var)], -1).astype(dtype)
    return f


def volatility_fn(volvol, rho, dtype):
    def f(t, x):
        t = np.asarray([t], dtype=dtype)
        r = param_at(rho, t, dtype)[0]
        xi = param_at(volvol, t, dtype)[0]
        vol = np.sqrt(np.abs(x[..., 1]))
        z = np.zeros_like(vol)
        col1 = np.stack([vol, xi * r * vol], -1)
        col2 = np.stack([z, xi * np.sqrt(1 - r ** 2) * vol], -1)
        return np.stack([col1, col2], -1).astype(dtype)
    return f


def _update_variance(kappa, theta, xi, v, dt, z, dtype, near):
    d = np.dtype(dtype).type
    scaled_time = np.exp(-kappa * dt).astype(dtype)
    xi2 = (xi ** 2).astype(dtype)
    m = (theta + (v - theta) * scaled_time).astype(dtype)
    s2 = (v * xi2 * scaled_time / kappa * (d(1) - scaled_time)
          + theta * xi2 / d(2) / kappa * (d(1) - scaled_time) ** 2).astype(dtype)
    psi = (s2 / m ** 2).astype(dtype)
    u = (d(0.5) * (d(1) + erf((z / d(SQRT_2)).astype(np.float64)).astype(dtype))).astype(dtype)
    cond = psi < d(1.5)
    with np.errstate(all="ignore"):
        psi_inv = (d(2) / psi).astype(dtype)
        b2 = (psi_inv - d(1) + np.sqrt(psi_inv * (psi_inv - d(1)))).astype(dtype)
        a = (m / (d(1) + b2)).astype(dtype)
        v_true = (a * (np.sqrt(b2) + z) ** 2).astype(dtype)
        p = ((psi - d(1)) / (psi + d(1))).astype(dtype)
        beta = ((d(1) - p) / m).astype(dtype)
        v_false = (np.where(u > p, np.log(d(1) - p) - np.log(d(1) - u), d(0)) / beta).astype(dtype)
    flag = (np.abs(psi - d(1.5)) <= near * 1.5) | ((~cond) & (np.abs(u - p) <= near))
    return np.where(cond, v_true, v_false).astype(dtype), flag


def _update_log_spot(kappa, theta, xi, rho, v, v_next, x, dt, z, dtype):
    d = np.dtype(dtype).type
    k0 = (-rho * kappa * theta / xi * dt).astype(dtype)
    k1 = (d(0.5) * dt * (kappa * rho / xi - d(0.5)) - rho / xi).astype(dtype)
    k2 = (d(0.5) * dt * (kappa * rho / xi - d(0.5)) + rho / xi).astype(dtype)
    k3 = (d(0.5) * dt * (d(1) - rho ** 2)).astype(dtype)
    k4 = (d(0.5) * dt * (d(1) - rho ** 2)).astype(dtype)
    return (x + k0 + k1 * v + k2 * v_next + np.sqrt(k3 * v + k4 * v_next) * z).astype(dtype)


def qe_sample_with_draws(kappa, theta, xi, rho, all_times, keep_mask, num_requested_times, x0,
                         v0, draws, dtype, tolerance=1e-6, near=0.0):
    """Returns (paths [N, k, 2] (log-spot, variance), near_branch [N] bool).

    kappa/theta/xi/rho: scalars or (jump_locations, values) piecewise tuples.
    draws: [steps, N, 2].
    """
    d = np.dtype(dtype).type
    times = np.asarray(all_times, dtype=dtype)
    dt = (times[1:] - times[:-1]).astype(dtype)
    eval_t = (times + np.min(dt) / d(2)).astype(dtype)
    K = param_at(kappa, eval_t, dtype)
    TH = param_at(theta, eval_t, dtype)
    XI = param_at(xi, eval_t, dtype)
    RHO = param_at(rho, eval_t, dtype)
    N = draws.shape[1]
    x = np.full(N, x0, dtype=dtype)
    v = np.full(N, v0, dtype=dtype)
    k = int(num_requested_times)
    record = k != 1
    res_x = np.zeros((k, N), dtype=dtype)
    res_v = np.zeros((k, N), dtype=dtype)
    if record:
        res_x[0], res_v[0] = x, v
    flags = np.zeros(N, dtype=bool)
    wc = 0  # the reference starts its loop at written_count = 0 (heston_model.py:441-444)
    i = 0
    steps = len(dt)
    while i < steps and wc < k:
        z = draws[i].astype(dtype)
        if dt[i] > d(tolerance):
            v_next, fl = _update_variance(K[i], TH[i], XI[i], v, dt[i], z[:, 0], dtype, near)
            flags |= fl
            x = _update_log_spot(K[i], TH[i], XI[i], RHO[i], v, v_next, x, dt[i], z[:, 1], dtype)
            v = v_next
        if record:
            res_x[wc], res_v[wc] = x, v
        wc += int(keep_mask[i + 1])
        i += 1
    if not record:
        return np.stack([x[:, None], v[:, None]], -1), flags
    return np.stack([res_x.T, res_v.T], -1), flags
