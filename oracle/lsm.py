"""Longstaff–Schwartz regression Monte Carlo, restated in NumPy (test oracle).

Test infrastructure only: the product path never imports this module.

Follows tf_quant_finance/models/longstaff_schwartz/lsm.py:
  make_polynomial_basis          lsm.py:50-125
  least_square_mc                lsm.py:128-295
  _apply_discount                lsm.py:304-325
  _expected_exercise_fn          lsm.py:328-383 (pseudo-inverse of X'X, lsm.py:372)
  _updated_cashflows_and_values  lsm.py:386-400
  _lsm_loop_body                 lsm.py:403-436
and payoff_utils.py:27-98 (make_basket_put_payoff / _put_valuer).

Arithmetic runs in the dtype of the paths, as in the reference; the
pseudo-inverse cuts singular values at 10 * size * eps(dtype) * max, the
default of tf.linalg.pinv.
"""

import numpy as np


def polynomial_exponents(degree, dim):
    """[(degree+1)^dim, dim] exponent grid in the reference's order: the
    stacked, reshaped np/tf meshgrid with default 'xy' indexing (lsm.py:113-117)."""
    g = np.arange(degree + 1)
    mesh = np.meshgrid(*(dim * [g]))
    return np.stack(mesh, -1).reshape(-1, dim)


def polynomial_basis(sample_paths, time_index, degree):
    """[batch, (degree+1)^dim, num_samples] centred-power design (lsm.py:84-123)."""
    x = np.asarray(sample_paths)
    if x.ndim == 3:
        x = x[None]
    sl = x[:, :, time_index, :][:, :, None, :]  # [B, N, 1, d]
    centred = sl - sl.mean(axis=1, keepdims=True)
    grid = polynomial_exponents(degree, x.shape[-1]).astype(x.dtype)
    expo = np.prod(centred ** grid, axis=-1)  # [B, N, G]
    return np.transpose(expo, (0, 2, 1))


def basket_put_payoff(sample_paths, time_index, strikes):
    """relu(K - mean_d S[n, t, d]) -> [num_samples, batch] (payoff_utils.py:61-98)."""
    x = np.asarray(sample_paths)
    if x.ndim == 3:
        x = x[:, None]
    else:
        x = np.transpose(x, (1, 0, 2, 3))
    avg = x[:, :, time_index, :].mean(axis=-1)
    return np.maximum(np.asarray(strikes, x.dtype) - avg, 0).astype(x.dtype)


def pinv(a):
    """tf.linalg.pinv with its default rcond = 10 * max(m, n) * eps (batched)."""
    u, s, vt = np.linalg.svd(a)
    rcond = 10.0 * max(a.shape[-2:]) * np.finfo(a.dtype).eps
    cutoff = rcond * s.max(axis=-1, keepdims=True)
    s_inv = np.where(s > cutoff, 1.0 / np.where(s > cutoff, s, 1), 0).astype(a.dtype)
    return np.einsum("...ji,...j,...kj->...ik", vt, s_inv, u)


def _discount_table(discount_factors, num_ex, dtype):
    if discount_factors is None:
        d = np.ones(num_ex, dtype)
    else:
        d = np.asarray(discount_factors, dtype)
    if d.ndim == 0:
        d = d.reshape(1, 1, 1)
    elif d.ndim == 1:
        d = d.reshape(1, 1, -1)
    d = np.pad(d, [(0, 0), (0, 0), (1, 0)], constant_values=1)
    return np.transpose(d, (2, 0, 1))  # [E+1, Nd, Bd]


def least_square_mc(sample_paths, exercise_times, strikes, degree, discount_factors=None,
                    num_calibration_samples=None, dtype=None, payoff_fn=None, basis_fn=None):
    """Price of American basket puts [batch] by regression MC (lsm.py:128-295)."""
    x = np.asarray(sample_paths, dtype=dtype)
    dt = x.dtype
    ex = [int(e) for e in np.asarray(exercise_times).reshape(-1)]
    E = len(ex)
    payoff = payoff_fn or (lambda p, t: basket_put_payoff(p, t, strikes))
    basis = basis_fn or (lambda p, t: polynomial_basis(p, t, degree))
    D = _discount_table(discount_factors, E, dt)

    def ratio(i):
        return (D[i + 1] / D[i]).astype(dt)

    cashflow = payoff(x, ex[E - 1])
    values = np.zeros_like(cashflow)
    i = E - 1
    iters = 0
    while i > 0 and iters < x.shape[-2]:
        t = ex[i - 1]
        ev = payoff(x, t)
        cont_value = ratio(i) * (values + cashflow)
        design = basis(x, t)  # [Bp, G, N]
        mask = ev > 0
        design_t = np.transpose(design, (0, 2, 1))  # [Bp, N, G]
        masked = np.where(np.transpose(mask)[..., None], design_t, np.zeros_like(design_t))
        cv = cont_value
        if num_calibration_samples is not None:
            masked = masked[:, :num_calibration_samples]
            cv = cont_value[:num_calibration_samples]
        lhs = np.einsum("bni,bnj->bij", masked, masked)
        rhs = np.einsum("bni,nb->bi", masked, cv)[..., None]
        beta = np.matmul(pinv(lhs), rhs)
        cont = np.matmul(design_t, beta)[..., 0]  # [B, N]
        expected = np.maximum(np.transpose(cont), 0).astype(dt)
        do_update = ev > expected
        upd_values = np.where(do_update, np.zeros_like(cashflow), cashflow + values)
        cashflow = np.where(do_update, ev, np.zeros_like(ev))
        values = ratio(i) * upd_values
        i -= 1
        iters += 1
    present = ratio(0) * (cashflow + values)
    if num_calibration_samples is not None:
        present = present[num_calibration_samples:]
    return present.mean(axis=0)
