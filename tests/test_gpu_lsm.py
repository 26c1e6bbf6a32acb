"""Longstaff–Schwartz regression MC on the GPU against the reference's known
answers (lsm_test.py) and the oracle's restatement."""

import json
import os

import numpy as np
import pytest

from oracle import lsm as olsm

pytestmark = pytest.mark.gpu


def _golden():
    with open(os.path.join(os.path.dirname(__file__), "golden", "lsm_golden.json")) as f:
        return json.load(f)


def _gbm_paths(n, steps, dim=1, seed=0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    dt = 1.0 / steps
    z = rng.standard_normal((n, steps, dim))
    logs = np.cumsum((0.06 - 0.5 * 0.2 ** 2) * dt + 0.2 * np.sqrt(dt) * z, axis=1)
    s = np.concatenate([np.ones((n, 1, dim)), np.exp(logs)], axis=1)
    return s.astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_lsm_reference_known_answers(cuda, dtype):
    from tqf.models import longstaff_schwartz as L
    g = _golden()
    S = np.array(g["samples"])[..., None]
    df = np.exp(-np.cumsum(g["rates"]))
    dfb = np.exp(-np.cumsum(g["batch_rates"], -1))[None]
    tol = g["tolerance"]
    c = g["cases"]
    basis = L.make_polynomial_basis(2)

    def price(paths, ex, strikes, disc, **kw):
        out = L.least_square_mc(paths, ex, L.make_basket_put_payoff(strikes, dtype=dtype), basis,
                                discount_factors=disc, dtype=dtype, **kw)
        return out.cpu().numpy()

    np.testing.assert_allclose(price(S, [3], [1.1], [df[-1]]), c["european_put"]["price"], **tol)
    np.testing.assert_allclose(price(S, [1, 2, 3], [1.1], df), c["american_put"]["price"], **tol)
    np.testing.assert_allclose(price(S, [1, 2, 3], [1.1], df, num_calibration_samples=4),
                               c["american_put_calibration"]["price"], **tol)
    np.testing.assert_allclose(price(S, [1, 2, 3], [1.1, 1.2], dfb), c["american_put_batch_payoff"]["price"], **tol)
    np.testing.assert_allclose(price(np.stack([S, S + 0.1]), [1, 2, 3], [1.1, 1.2], dfb),
                               c["american_put_batch_samples"]["price"], **tol)


def test_lsm_basket_degree_10_two_dims(cuda):
    """121 basis functions on perfectly correlated 2-d paths price as the 1-d
    paths (lsm_test.py:131-160): exercises the rank-deficient pseudo-inverse."""
    from tqf.models import longstaff_schwartz as L
    g = _golden()
    S = np.array(g["samples"])[..., None]
    df = np.exp(-np.cumsum(g["rates"]))
    pay = L.make_basket_put_payoff([1.1, 1.2, 1.3], dtype=np.float64)
    two = L.least_square_mc(np.concatenate([S, S], -1), [1, 2, 3], pay, L.make_polynomial_basis(10),
                            discount_factors=df, dtype=np.float64).cpu().numpy()
    one = L.least_square_mc(S, [1, 2, 3], pay, L.make_polynomial_basis(10), discount_factors=df,
                            dtype=np.float64).cpu().numpy()
    np.testing.assert_allclose(two, one, rtol=1e-4, atol=1e-4)
    want = olsm.least_square_mc(S, [1, 2, 3], [1.1, 1.2, 1.3], 10, discount_factors=df, dtype=np.float64)
    np.testing.assert_allclose(one, want, rtol=1e-9)


@pytest.mark.parametrize("calib", [None, 20000])
def test_lsm_matches_oracle_on_gbm_paths(cuda, calib):
    """50,000 GBM paths, 12 exercise dates, cubic basis, FP64: the GPU price
    equals the restatement's to 1e-9 relative."""
    from tqf.models import longstaff_schwartz as L
    S = _gbm_paths(50000, 12, seed=1)
    ex = list(range(1, 13))
    df = np.exp(-0.06 * np.arange(1, 13) / 12)
    got = L.least_square_mc(S, ex, L.make_basket_put_payoff([1.0, 1.1]), L.make_polynomial_basis(3),
                            discount_factors=df, num_calibration_samples=calib, dtype=np.float64).cpu().numpy()
    want = olsm.least_square_mc(S, ex, [1.0, 1.1], 3, discount_factors=df, num_calibration_samples=calib,
                                dtype=np.float64)
    np.testing.assert_allclose(got, want, rtol=1e-9)


def test_lsm_float32_and_per_path_discount(cuda):
    """Float32 paths and a [N, B, E] discount tensor (stochastic rates).

    In float32 the pseudo-inverse cuts eigenvalues below 10 G eps_f32 x the
    largest (tf.linalg.pinv's default), which drops the smallest directions of
    this 9-function basis: the price moves ~1e-3 from the float64 one, in the
    reference and here alike.  The comparison is with the float32 restatement
    (exercise decisions may flip at exact ties, so 1e-4)."""
    from tqf.models import longstaff_schwartz as L
    S = _gbm_paths(30000, 8, dim=2, seed=2, dtype=np.float32)
    ex = [2, 4, 6, 8]
    rng = np.random.default_rng(3)
    disc = np.exp(-np.cumsum(rng.uniform(0.01, 0.03, (30000, 2, 4)), axis=-1)).astype(np.float32)
    got = L.least_square_mc(S, ex, L.make_basket_put_payoff([1.0, 1.05], dtype=np.float32),
                            L.make_polynomial_basis(2), discount_factors=disc, dtype=np.float32).cpu().numpy()
    want = olsm.least_square_mc(S, ex, [1.0, 1.05], 2, discount_factors=disc, dtype=np.float32)
    np.testing.assert_allclose(got, want, rtol=1e-4)


def test_lsm_explicit_callables_equal_structured(cuda):
    """Arbitrary payoff/basis callables (evaluated by torch each date and fed
    to the same kernels) give the structured path's price; batched paths."""
    from tqf.models import longstaff_schwartz as L
    S = np.stack([_gbm_paths(20000, 6, seed=4), _gbm_paths(20000, 6, seed=5) * 1.02])
    ex = [1, 2, 3, 4, 5, 6]
    df = np.exp(-0.05 * np.arange(1, 7) / 6)
    pay, basis = L.make_basket_put_payoff([1.0, 1.1]), L.make_polynomial_basis(2)
    structured = L.least_square_mc(S, ex, pay, basis, discount_factors=df, dtype=np.float64).cpu().numpy()
    explicit = L.least_square_mc(S, ex, lambda p, t: pay(p, t), lambda p, t: basis(p, t), discount_factors=df,
                                 dtype=np.float64).cpu().numpy()
    np.testing.assert_allclose(explicit, structured, rtol=1e-10)
    want = olsm.least_square_mc(S, ex, [1.0, 1.1], 2, discount_factors=df, dtype=np.float64)
    np.testing.assert_allclose(structured, want, rtol=1e-9)


def test_lsm_american_put_bounds(cuda):
    """1-d American put on GBM: above the European price (Black–Scholes) and
    the immediate exercise value; repeated calls are deterministic."""
    from oracle import closed_form
    from tqf.models import longstaff_schwartz as L
    S = _gbm_paths(200000, 50, seed=6)
    ex = list(range(1, 51))
    df = np.exp(-0.06 * np.arange(1, 51) / 50)
    args = (S, ex, L.make_basket_put_payoff([1.1]), L.make_polynomial_basis(3))
    p1 = L.least_square_mc(*args, discount_factors=df, dtype=np.float64).cpu().numpy()
    p2 = L.least_square_mc(*args, discount_factors=df, dtype=np.float64).cpu().numpy()
    assert p1[0] == p2[0]
    euro = closed_form.black_scholes(1.0, 1.1, 0.06, 0.2, 1.0, is_call=False)
    assert p1[0] > euro and p1[0] > 0.1
    assert p1[0] < euro + 0.03


@pytest.mark.parametrize("dim,degree,calib", [(1, 3, None), (1, 4, 15000), (2, 1, None), (2, 1, 12000)])
def test_lsm_one_launch_loop_matches_oracle(cuda, dim, degree, calib):
    """The one-launch loop (one payoff, d <= 2, <= 5 basis functions: Gram
    pseudo-inverses of every date before the date loop, one barrier per date)
    against the restatement in FP64 to 1e-9, with and without a calibration
    split, and against the float32 restatement in float32 to 2.5e-4: the
    two float32 regressions round differently (sums, the pseudo-inverse's
    cutoff directions), which flips exercise decisions at near-ties;
    measured up to 1.1e-4 on these cases."""
    from tqf import _lib
    from tqf.models import longstaff_schwartz as L
    S = _gbm_paths(40000, 10, dim=dim, seed=11 + dim)
    ex = list(range(1, 11))
    df = np.exp(-0.05 * np.arange(1, 11) / 10)
    pay, basis = L.make_basket_put_payoff([1.05]), L.make_polynomial_basis(degree)
    c0 = _lib.launch_count()
    got = L.least_square_mc(S, ex, pay, basis, discount_factors=df, num_calibration_samples=calib,
                            dtype=np.float64).cpu().numpy()
    assert _lib.launch_count() - c0 == 4  # gather, reduce, scale, loop
    want = olsm.least_square_mc(S, ex, [1.05], degree, discount_factors=df, num_calibration_samples=calib,
                                dtype=np.float64)
    np.testing.assert_allclose(got, want, rtol=1e-9)
    S32 = S.astype(np.float32)
    got32 = L.least_square_mc(S32, ex, L.make_basket_put_payoff([1.05], dtype=np.float32), basis,
                              discount_factors=df, num_calibration_samples=calib, dtype=np.float32).cpu().numpy()
    want32 = olsm.least_square_mc(S32, ex, [1.05], degree, discount_factors=df, num_calibration_samples=calib,
                                  dtype=np.float32)
    np.testing.assert_allclose(got32, want32, rtol=2.5e-4)
