"""Vector Hull-White exact discretisation, restated in NumPy (test oracle).

Test infrastructure only: the product path never imports this module.

Follows tf_quant_finance/models/hull_white/vector_hull_white.py:
  _sample_paths                 :641-781 (loop: x' = exp(-a_{i+1} dt) x + E_i
                                 + sqrt(relu(V_i)) (L_i z); rate = x + f0)
  _bond_reconstitution          :783-814
  _exact_discretization_setup   :816-855 (sorted parameter jumps per axis)
  _compute_yt                   :857-874
  _conditional_mean_x           :876-907
  _y_integral, _ex_integral     :909-923
  _conditional_variance_x, _variance_int :925-955
  _prepare_grid                 :982-1031 (times, 0 and the jumps, sorted)
Parameters are per-axis piecewise-constant functions given as (jumps, values)
with values[i] on (jumps[i-1], jumps[i]] (left-continuous).
"""

from __future__ import annotations

import numpy as np


def pw_eval(jumps, values, t):
    jumps = np.asarray(jumps)
    idx = np.searchsorted(jumps, t, side="left")
    return np.asarray(values)[idx]


class Params:
    """Per-axis piecewise-constant mean reversion / volatility (dtype arrays)."""

    def __init__(self, dim, mr, vol, dtype):
        self.dim, self.dtype = dim, np.dtype(dtype)
        self.mr = [(np.asarray(j, dtype), np.asarray(v, dtype)) for j, v in mr]
        self.vol = [(np.asarray(j, dtype), np.asarray(v, dtype)) for j, v in vol]
        dt = self.dtype.type
        jl = [np.sort(np.concatenate([self.vol[d][0], self.mr[d][0]])) for d in range(dim)]
        J = max(len(x) for x in jl)
        assert all(len(x) == J for x in jl)
        self.jl = np.array(jl, dtype).reshape(dim, J)
        self.jv_vol = np.array([pw_eval(*self.vol[d], self.jl[d]) for d in range(dim)], dtype).reshape(dim, J)
        self.jv_mr = np.array([pw_eval(*self.mr[d], self.jl[d]) for d in range(dim)], dtype).reshape(dim, J)
        zero = np.zeros((dim, 1), dtype)
        self.padded = np.concatenate([zero, self.jl[:, :-1]], 1)[:, :max(J, 1)] if J else zero
        self.vn = np.concatenate([zero, self.jl], 1)
        self.zero = zero
        self._dt = dt

    def at(self, t):
        t = np.asarray(t, self.dtype)
        mr = np.array([pw_eval(*self.mr[d], t) for d in range(self.dim)], self.dtype)
        vol = np.array([pw_eval(*self.vol[d], t) for d in range(self.dim)], self.dtype)
        return mr, vol


def _y_integral(t0, t, vol, k):
    return (vol * vol) / (2 * k) * (np.exp(2 * k * t) - np.exp(2 * k * t0))


def _ex_integral(t0, t, vol, k, y_t0):
    value = (np.exp(k * t) - np.exp(k * t0) + np.exp(2 * k * t0) * (np.exp(-k * t) - np.exp(-k * t0)))
    return value * vol ** 2 / (2 * k * k) + y_t0 * (np.exp(-k * t0) - np.exp(-k * t)) / k


def _variance_int(t0, t, vol, k):
    return vol * vol / (2 * k) * (np.exp(2 * k * t) - np.exp(2 * k * t0))


def _cumsum(x):
    return np.cumsum(x, axis=1)


def _gather(a, idx):
    return np.take_along_axis(a, idx, axis=1)


def conditional_mean_x(p, t, mr_t, sig_t):
    t = np.broadcast_to(np.asarray(t, p.dtype), (p.dim, len(t)))
    ti = np.array([np.searchsorted(p.jl[d], t[d], side="left") for d in range(p.dim)])
    yb = _y_integral(p.padded[:, :p.jl.shape[1]], p.jl, p.jv_vol, p.jv_mr)
    y_at = np.concatenate([p.zero, _cumsum(yb)], 1)
    exb = _ex_integral(p.padded[:, :p.jl.shape[1]], p.jl, p.jv_vol, p.jv_mr, y_at[:, :-1])
    ex_at = np.concatenate([p.zero, _cumsum(exb)], 1)
    c = _gather(y_at, ti)
    ex = _ex_integral(_gather(p.vn, ti), t, sig_t, mr_t, c) + _gather(ex_at, ti)
    return ((ex[:, 1:] - ex[:, :-1]) * np.exp(-np.broadcast_to(mr_t, t.shape)[:, 1:] * t[:, 1:])).astype(p.dtype)


def conditional_variance_x(p, t, mr_t, sig_t):
    t = np.broadcast_to(np.asarray(t, p.dtype), (p.dim, len(t)))
    vb = _variance_int(p.padded[:, :p.jl.shape[1]], p.jl, p.jv_vol, p.jv_mr)
    v_at = np.concatenate([p.zero, _cumsum(vb)], 1)
    ti = np.array([np.searchsorted(p.jl[d], t[d], side="left") for d in range(p.dim)])
    v = _variance_int(_gather(p.vn, ti), t, sig_t, mr_t) + _gather(v_at, ti)
    return ((v[:, 1:] - v[:, :-1]) * np.exp(-2 * np.broadcast_to(mr_t, t.shape)[:, 1:] * t[:, 1:])).astype(p.dtype)


def compute_yt(p, t, mr_t, sig_t):
    t = np.broadcast_to(np.asarray(t, p.dtype), (p.dim, len(t)))
    ti = np.array([np.searchsorted(p.jl[d], t[d], side="left") for d in range(p.dim)])
    yb = _y_integral(p.padded[:, :p.jl.shape[1]], p.jl, p.jv_vol, p.jv_mr)
    y_at = np.concatenate([p.zero, _cumsum(yb)], 1)
    y = _y_integral(_gather(p.vn, ti), t, sig_t, mr_t) + _gather(y_at, ti)
    return np.exp(-2 * mr_t * t) * y


def grid(times, jump_arrays, dtype):
    """all_times = sort([0] + times + jumps), keep = scatter of searchsorted(times)."""
    times = np.asarray(times, dtype)
    extra = [np.asarray(j, dtype).reshape(-1) for j in jump_arrays]
    all_times = np.sort(np.concatenate([np.zeros(1, dtype), times] + extra))
    keep = np.zeros(len(all_times), bool)
    keep[np.searchsorted(all_times, times, side="left")] = True
    return all_times, keep


def sample_with_draws(p, times, jump_arrays, f0_fn, draws, corr=None, dtype=np.float64):
    """Rates [N, k, dim]; draws [steps, N, dim]; f0_fn(t) -> [dim]; corr [dim, dim] or None."""
    dt_ = np.dtype(dtype).type
    all_times, keep = grid(times, jump_arrays, dtype)
    dts = (all_times[1:] - all_times[:-1]).astype(dtype)
    mr, vol = p.at(all_times)
    ex = conditional_mean_x(p, all_times, mr, vol)
    var = conditional_variance_x(p, all_times, mr, vol)
    L = None if corr is None else np.linalg.cholesky(np.asarray(corr, np.float64)).astype(dtype)
    N = draws.shape[1]
    k = len(times)
    x = np.zeros((N, p.dim), dtype)
    record = k != 1
    out = np.zeros((k, N, p.dim), dtype)
    wc = 0
    if record:
        out[0] = x + f0_fn(all_times[0])
    wc += int(keep[0])
    i = 0
    last = x + f0_fn(all_times[0])
    while i < len(dts) and wc < k:
        z = draws[i].astype(dtype)
        if L is not None:
            z = np.einsum("ij,nj->ni", L, z).astype(dtype)
        v = np.sqrt(np.maximum(var[:, i], dt_(0))).astype(dtype)
        v = np.where(v > 0, v, dt_(0))
        x = (np.exp(-mr[:, i + 1] * dts[i]) * x + ex[:, i] + v * z).astype(dtype)
        last = (x + f0_fn(all_times[i + 1])).astype(dtype)
        if record:
            out[wc] = last
        wc += int(keep[i + 1])
        i += 1
    if not record:
        return last[:, None, :]
    return np.transpose(out, (1, 0, 2))


def bond_reconstitution(p, times, maturities, short_rate, f0_fn, r_fn):
    """P(t, T | r(t)) (_bond_reconstitution with y_t from _compute_yt)."""
    times = np.asarray(times, p.dtype)
    maturities = np.asarray(maturities, p.dtype)
    mr, vol = p.at(times)
    y = compute_yt(p, times, mr, vol).T
    mr = mr.T
    x_t = np.asarray(short_rate, p.dtype) - f0_fn(times)
    p0t = np.exp(-r_fn(times)[:, None] * times[:, None])
    p0T = np.exp(-r_fn(maturities)[:, None] * maturities[:, None]) / p0t
    g = (1.0 - np.exp(-mr * (maturities[:, None] - times[:, None]))) / mr
    return p0T * np.exp(-x_t * g - 0.5 * y * g ** 2)
