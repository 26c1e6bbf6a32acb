"""Milstein scheme, restated in NumPy (test oracle).

Test infrastructure only: the product path never imports this module.

Follows tf_quant_finance/models/milstein_sampling.py:
  _sample / _while_loop        milstein_sampling.py:258-424 (grid, written_count, records)
  _stratonovich_integral       milstein_sampling.py:481-525
  _milstein_hot                milstein_sampling.py:528-552
  _stratonovich_drift_update   milstein_sampling.py:555-562
  _milstein_1d / _milstein_nd  milstein_sampling.py:565-593
  _milstein_step               milstein_sampling.py:596-671
The formulas are the code's, including its index contractions and scale
factors (e.g. the off-diagonal Stratonovich term uses dt * dW_i dW_j / 2 and
the drift correction has no factor 1/2), since parity is with the reference.

Draws per step: dim + 3 * dim * order normals (utils.generate_mc_normal_draws
with num_normal_draws = dim + 3 dim order): [:dim] the Wiener increments, then
three blocks of dim * order auxiliary normals (mu, zeta, eta), each read as
[dim, order].
"""

from __future__ import annotations

import math

import numpy as np


def num_draws(dim, order):
    return dim + 3 * dim * order


def stratonovich_integral(dt, sqrt_dt, dw, mu, zeta, eta, order, dtype):
    """J[N, dim, dim] (milstein_sampling.py:481-525); mu, zeta, eta: [N, dim, order]."""
    dt_ = np.dtype(dtype).type
    p = order - 1
    sqrt_rho_p = dt_(np.sqrt(dt_(1 / 12 - sum(1 / r ** 2 for r in range(1, order + 1)) / 2 / math.pi ** 2)))
    xi = (dw / sqrt_dt).astype(dtype)
    mup = mu[..., p]
    value = dt * (np.einsum("ni,nj->nij", dw, dw) / dt_(2)
                  + sqrt_rho_p * (np.einsum("ni,nj->nij", mup, xi) - np.einsum("ni,nj->nij", xi, mup)))
    acc = np.zeros_like(value)
    s2 = dt_(np.sqrt(2.0))
    for r in range(1, order + 1):
        z = zeta[..., r - 1]
        e = eta[..., r - 1]
        w = s2 * xi + e
        acc = acc + (np.einsum("ni,nj->nij", z, w) - np.einsum("ni,nj->nij", w, z)) * dt_(1.0 / r)
    value = value + dt * acc / dt_(2 * math.pi)
    return value.astype(dtype)


def milstein_increment_nd(x, drift, vol, grad, dt, sqrt_dt, z, aux, order, dtype):
    """One _milstein_nd step (milstein_sampling.py:577-593).

    vol: [N, d, d] = B; grad: [N, d(i), d(k), d(j)] = dB_kj / dx_i; z: [N, d];
    aux: three [N, d, order] blocks."""
    dw = (z * sqrt_dt).astype(dtype)
    d = x.shape[-1]
    # drift_update[k] = sum_{i,j} dB_kj/dx_i B_ij  (concat(grad_vol, 2) matvec vec(vol))
    drift_update = np.einsum("nikj,nij->nk", grad, vol)
    dt_inc = dt * (drift - drift_update)
    dw_inc = np.einsum("nkj,nj->nk", vol, dw)
    J = stratonovich_integral(dt, sqrt_dt, dw, aux[0], aux[1], aux[2], order, dtype)
    idx = np.arange(d)
    J[:, idx, idx] = dw * dw / np.dtype(dtype).type(2)
    # lbar[s][i][m] = sum_j dB_sj/dx_i B_jm ; hot[s] = sum_{i,m} lbar[s][i][m] J[i][m]
    lbar = np.einsum("nisj,njm->nsim", grad, vol)
    hot = np.einsum("nsim,nim->ns", lbar, J)
    return (x + dt_inc + dw_inc + hot).astype(dtype)


def milstein_increment_1d(x, drift, vol, grad, dt, sqrt_dt, z, dtype):
    """_milstein_1d (milstein_sampling.py:565-574): x + dt a + b dW + b b' (dW^2 - dt) / 2.
    x, drift, vol, grad, z: [N, 1]."""
    dt_ = np.dtype(dtype).type
    dw = (z * sqrt_dt).astype(dtype)
    dt_inc = dt * drift
    dw_inc = vol * dw
    hot = (vol * grad) * (dw * dw - dt) / dt_(2)
    return (x + dt_inc + dw_inc + hot).astype(dtype)


def sample_with_draws(drift_fn, vol_fn, grad_fn, all_times, keep_mask, num_requested_times, x0, draws, order,
                      dtype):
    """draws: [steps, N, dim + 3 dim order].  grad_fn(t, x) -> [N, d(i), d(k), d(j)]
    = dB_kj/dx_i.  Returns [N, k, d] (k = 1 keeps the expand_dims branch)."""
    times = np.asarray(all_times, dtype=dtype)
    dt = (times[1:] - times[:-1]).astype(dtype)
    sqrt_dt = np.sqrt(dt).astype(dtype)
    x = np.array(x0, dtype=dtype)
    d = x.shape[-1]
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
        z = draws[i][:, :d].astype(dtype)
        drift = drift_fn(t, x).astype(dtype)
        vol = vol_fn(t, x).astype(dtype)
        grad = grad_fn(t, x).astype(dtype)
        if d == 1:
            x = milstein_increment_1d(x, drift, vol[..., 0, :], grad[:, 0, 0, :], dt[i], sqrt_dt[i], z, dtype)
        else:
            n = x.shape[0]
            aux = [draws[i][:, d + q * d * order: d + (q + 1) * d * order].reshape(n, d, order).astype(dtype)
                   for q in range(3)]
            x = milstein_increment_nd(x, drift, vol, grad, dt[i], sqrt_dt[i], z, aux, order, dtype)
        if record:
            result[wc] = x
        wc += int(keep_mask[i + 1])
        i += 1
    if not record:
        return x[..., None, :]
    return np.moveaxis(result, 0, -2)


def affine_coefficients(m, M, s0, s1, C, dtype):
    """Structured coefficients a(x) = m + M x, B(x)_kj = (s0_k + s1_k x_k) C_kj and
    their exact gradient dB_kj/dx_i = delta_ik s1_k C_kj."""
    m, M, s0, s1, C = (np.asarray(v, dtype) for v in (m, M, s0, s1, C))
    d = len(m)

    def drift(t, x):
        return (m + x @ M.T).astype(dtype)

    def vol(t, x):
        return ((s0 + s1 * x)[..., :, None] * C).astype(dtype)

    def grad(t, x):
        g = np.zeros((x.shape[0], d, d, d), dtype)
        for i in range(d):
            g[:, i, i, :] = s1[i] * C[i]
        return g

    return drift, vol, grad
