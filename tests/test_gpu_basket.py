"""Correlated GBM paths and the basket pricer against the oracle (GPU)."""

import numpy as np
import pytest
import torch

from oracle import mvgbm as omvgbm

pytestmark = pytest.mark.gpu


def basket_config(d=16, seed=7):
    """16-asset config: vols U[0.1, 0.4], correlation Q diag(lambda) Q^T with a
    random orthogonal Q and lambda ~ U[0.1, 2], renormalised to unit diagonal."""
    rng = np.random.default_rng(seed)
    vols = rng.uniform(0.1, 0.4, d)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    lam = rng.uniform(0.1, 2.0, d)
    c = q @ np.diag(lam) @ q.T
    s = np.sqrt(np.diag(c))
    corr = c / np.outer(s, s)
    return vols, corr


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_mvgbm_paths_match_oracle(cuda, dtype):
    from tqf.models import MultivariateGeometricBrownianMotion
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    d, N = 5, 3000
    vols, corr = basket_config(d)
    times = np.array([0.1, 0.25, 0.5, 1.0], np_dt)
    draws = np.random.default_rng(3).standard_normal((N, 4, d)).astype(np_dt)
    x0 = np.linspace(1.0, 2.0, d).astype(np_dt)
    proc = MultivariateGeometricBrownianMotion(d, means=0.03, volatilities=vols, corr_matrix=corr, dtype=np_dt)
    got = proc.sample_paths(times, initial_state=x0, normal_draws=draws).cpu().numpy()
    want = omvgbm.sample_with_draws(np.full(d, 0.03), vols, corr, times, x0, draws.transpose(1, 0, 2), np_dt)
    rtol = 1e-5 if dtype == torch.float32 else 1e-12
    np.testing.assert_allclose(got, want, rtol=rtol, atol=0)


def test_mvgbm_moments_and_sobol(cuda):
    from tqf.math.random import RandomType
    from tqf.models import MultivariateGeometricBrownianMotion
    proc = MultivariateGeometricBrownianMotion(2, means=1.0, volatilities=[0.1, 0.2],
                                               corr_matrix=[[1, 0.1], [0.1, 1]], dtype=np.float64)
    times = [0.1, 0.2, 1.0]
    for rt, seed in [(RandomType.SOBOL, None), (RandomType.STATELESS, [4, 2])]:
        s = proc.sample_paths(times, initial_state=[1.0, 2.0], random_type=rt, seed=seed,
                              num_samples=100000).cpu().numpy()
        np.testing.assert_allclose(s.mean(0), np.array([1.0, 2.0]) * np.exp(np.array(times))[:, None], rtol=1e-2)


def test_cholesky_on_gpu(cuda):
    from tqf.models.multivariate_gbm import cholesky_f64
    _, corr = basket_config(16)
    L = cholesky_f64(corr, cuda).cpu().numpy()
    np.testing.assert_allclose(L, np.linalg.cholesky(corr), rtol=1e-13, atol=1e-14)
    with pytest.raises(ValueError):
        cholesky_f64(np.array([[1.0, 2.0], [2.0, 1.0]]), cuda)


def test_basket_price_sums_match_oracle_with_same_draws(cuda):
    from tqf.pricing import basket_european_mc
    d, N, steps = 16, 20000, 64
    vols, corr = basket_config(d)
    draws = np.random.default_rng(11).standard_normal((N, steps, d)).astype(np.float32)
    res = basket_european_mc(spots=np.full(d, 100.0), vols=vols, rate=0.02, corr=corr, strike=100.0, expiry=1.0,
                             num_time_steps=steps, num_samples=N, normal_draws=torch.as_tensor(draws).cuda())
    times = np.linspace(0, 1, steps + 1)[1:]
    paths = omvgbm.sample_with_draws(np.full(d, 0.02), vols, corr, times, np.full(d, 100.0),
                                     draws.transpose(1, 0, 2).astype(np.float64), np.float64)
    B = paths[:, -1, :].mean(-1)
    pay = np.maximum(B - 100.0, 0)
    np.testing.assert_allclose(float(res.sums[0]), pay.sum(), rtol=2e-5)
    np.testing.assert_allclose(float(res.sums[1]), (pay * pay).sum(), rtol=5e-5)
    # pathwise Greeks == torch autograd of the restated graph on the same draws
    import torch as th
    spots = th.full((d,), 100.0, dtype=th.float64, requires_grad=True)
    v = th.as_tensor(vols, dtype=th.float64).requires_grad_(True)
    rate = th.tensor(0.02, dtype=th.float64, requires_grad=True)
    p = omvgbm.basket_price_torch(spots, v, rate, corr, np.full(d, 1.0 / d), 100.0, times,
                                  draws.transpose(1, 0, 2).astype(np.float64))
    p.backward()
    np.testing.assert_allclose(res.price, float(p), rtol=2e-5)
    np.testing.assert_allclose(res.delta.numpy(), spots.grad.numpy(), rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(res.vega.numpy(), v.grad.numpy(), rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(res.rho, float(rate.grad), rtol=1e-4)


def test_basket_adjoint_greeks_vs_finite_differences(cuda):
    """Pathwise delta and vega of all 16 assets within 1e-4 (delta absolute,
    vega relative to max(1, |bump|)) of central common-random-number
    bump-and-revalue in float64.  The bumps (1e-5 relative in the spot, 1e-6
    in the volatility) are small enough that few paths cross the strike
    inside a bump, and large enough that the difference quotient's float64
    rounding stays ~1e-9."""
    from tqf.math.random import RandomType
    from tqf.pricing import basket_european_mc
    d = 16
    vols, corr = basket_config(d)
    kw = dict(rate=0.02, corr=corr, strike=100.0, expiry=1.0, num_time_steps=64, num_samples=1 << 20,
              random_type=RandomType.STATELESS, seed=[3, 4], dtype=torch.float64)
    base = basket_european_mc(spots=np.full(d, 100.0), vols=vols, **kw)
    h, hv = 1e-3, 1e-6
    for i in range(d):
        up = np.full(d, 100.0)
        up[i] += h
        dn = np.full(d, 100.0)
        dn[i] -= h
        fd = (basket_european_mc(spots=up, vols=vols, **kw).price - basket_european_mc(spots=dn, vols=vols, **kw).price) / (2 * h)
        assert abs(float(base.delta[i]) - fd) < 1e-4, (i, float(base.delta[i]), fd)
        vu = vols.copy()
        vu[i] += hv
        vd = vols.copy()
        vd[i] -= hv
        fdv = (basket_european_mc(spots=np.full(d, 100.0), vols=vu, **kw).price
               - basket_european_mc(spots=np.full(d, 100.0), vols=vd, **kw).price) / (2 * hv)
        assert abs(float(base.vega[i]) - fdv) < 1e-4 * max(1.0, abs(fdv)), (i, float(base.vega[i]), fdv)


def test_basket_autograd_function(cuda):
    from tqf.math.random import RandomType
    from tqf.pricing import BasketPrice, basket_european_mc
    d = 4
    vols, corr = basket_config(d)
    kw = dict(corr=corr, strike=100.0, expiry=1.0, num_time_steps=16, num_samples=1 << 16,
              random_type=RandomType.STATELESS, seed=[1, 1])
    spots = torch.full((d,), 100.0, dtype=torch.float64, requires_grad=True)
    v = torch.as_tensor(vols).requires_grad_(True)
    r = torch.tensor(0.02, dtype=torch.float64, requires_grad=True)
    price = BasketPrice.apply(spots, v, r, kw)
    price.backward()
    ref = basket_european_mc(spots=np.full(d, 100.0), vols=vols, rate=0.02, **kw)
    np.testing.assert_allclose(spots.grad.numpy(), ref.delta.numpy())
    np.testing.assert_allclose(v.grad.numpy(), ref.vega.numpy())
    np.testing.assert_allclose(float(r.grad), ref.rho)


@pytest.mark.parametrize("N", [3000, 128 * 152 * 8 + 77])
def test_mvgbm_16_factor_tensor_core_lz(cuda, N):
    """16 factors in FP32 take the tensor-core split-BF16 L z path; its paths
    match the oracle and the CUDA-core path within 1e-5 relative (64 steps,
    ragged path count, per-path initial states)."""
    from tqf.models import MultivariateGeometricBrownianMotion
    d = 16
    vols, corr = basket_config(d)
    times = np.linspace(1.0 / 64, 1.0, 64).astype(np.float32)
    draws = np.random.default_rng(11).standard_normal((N, 64, d)).astype(np.float32)
    x0 = np.random.default_rng(12).uniform(50, 150, (N, d)).astype(np.float32)
    proc = MultivariateGeometricBrownianMotion(d, means=0.03, volatilities=vols, corr_matrix=corr, dtype=np.float32)
    tc = proc.sample_paths(times, initial_state=x0, normal_draws=draws, lz_mode=0).cpu().numpy()
    fma = proc.sample_paths(times, initial_state=x0, normal_draws=draws, lz_mode=1).cpu().numpy()
    np.testing.assert_allclose(tc, fma, rtol=1e-5, atol=0)
    if N <= 3000:
        want = omvgbm.sample_with_draws(np.full(d, 0.03), vols, corr, times, np.ones(d, np.float32),
                                        draws.transpose(1, 0, 2), np.float32) * x0[:, None, :]
        np.testing.assert_allclose(tc, want, rtol=1e-5, atol=0)
    # the tensor path is not the CUDA-core path with the products rounded to BF16
    assert np.abs(tc / fma - 1).max() > 0


def test_mvgbm_16_factor_tensor_core_philox(cuda):
    """In-kernel Philox draws: both L z paths agree and the mean is right."""
    from tqf.math.random import RandomType
    from tqf.models import MultivariateGeometricBrownianMotion
    d = 16
    vols, corr = basket_config(d)
    proc = MultivariateGeometricBrownianMotion(d, means=0.01, volatilities=vols, corr_matrix=corr, dtype=np.float32)
    kw = dict(times=np.linspace(1.0 / 32, 1.0, 32), initial_state=np.full(d, 100.0, np.float32),
              num_samples=50000, random_type=RandomType.STATELESS, seed=[1, 2])
    tc = proc.sample_paths(**kw, lz_mode=0).cpu().numpy()
    fma = proc.sample_paths(**kw, lz_mode=1).cpu().numpy()
    np.testing.assert_allclose(tc, fma, rtol=1e-5, atol=0)
    np.testing.assert_allclose(tc[:, -1].mean(0), 100 * np.exp(0.01), rtol=1e-2)
