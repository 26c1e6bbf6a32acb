"""Dimensions above 16 (GPU): the reference's samplers take any dimension
(euler_sampling.py:513-537, multivariate_geometric_brownian_motion.py:229-281,
milstein_sampling.py:35-51).  Here those requests run in the one-warp-per-
path kernels (and, for correlated float32 GBM with 16 < dim <= 64, the
tensor-core L z); paths given identical draws are checked against the oracle
at 1e-5 relative (float32) and 1e-12 (float64), scale-aware as in
test_gpu_paths.py."""

import numpy as np
import pytest
import torch

from oracle import euler as oeuler
from oracle import grids as ogrids

pytestmark = pytest.mark.gpu


def _close(got, want, rtol, scale):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    err = np.abs(got - want) / (np.abs(want) + scale)
    assert np.all(np.isfinite(got)) and float(err.max()) <= rtol, float(err.max())


def _corr(d, seed):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    c = q @ np.diag(rng.uniform(0.1, 2.0, d)) @ q.T
    s = np.sqrt(np.diag(c))
    return c / np.outer(s, s)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("d", [17, 32, 64])
def test_euler_structured_and_callables_any_dim(cuda, dtype, d):
    """Correlated GBM in levels (AffineDrift + ScaledVolatility): the fused
    wide kernel and the per-step callable route (tqf_euler_update) against
    the oracle Euler loop on the same draws, with per-path initial states
    and three recorded times."""
    from tqf.models import coefficients, euler_sampling
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    N, steps = 700, 12
    rng = np.random.default_rng(d)
    mu = rng.uniform(-0.05, 0.05, d)
    sig = rng.uniform(0.1, 0.4, d)
    corr = _corr(d, d + 1)
    drift, vol = coefficients.gbm(mu, sig, corr)
    times = np.array([0.25, 0.5, 1.0], np_dt)
    draws = rng.standard_normal((N, steps, d)).astype(np_dt)
    x0 = rng.uniform(0.5, 2.0, (N, d)).astype(np_dt)
    a = euler_sampling.sample(d, drift, vol, times, num_time_steps=steps, initial_state=x0, normal_draws=draws)
    g = euler_sampling.sample(d, lambda t, x: drift(t, x), lambda t, x: vol(t, x), times, num_time_steps=steps,
                              initial_state=x0, normal_draws=draws)
    all_t, keep, _ = ogrids.prepare_grid(times, times[-1] / np_dt(steps), np_dt, num_time_steps=steps)
    L = np.linalg.cholesky(corr).astype(np_dt)
    want = oeuler.sample_with_draws(lambda t, x: (x * mu.astype(np_dt)).astype(np_dt),
                                    lambda t, x: ((x * sig.astype(np_dt))[..., None] * L).astype(np_dt),
                                    all_t, keep, 3, x0, draws.transpose(1, 0, 2), np_dt)
    rtol = 1e-5 if dtype == torch.float32 else 1e-12
    assert a.shape == (N, 3, d) and g.shape == (N, 3, d)
    _close(a.cpu().numpy(), want, rtol, 1.0)
    _close(g.cpu().numpy(), want, rtol, 1.0)


@pytest.mark.parametrize("d", [20, 100])
def test_euler_wide_in_kernel_draws_equal_materialised(cuda, d):
    """In-kernel Philox draws of the wide kernel are the canonical stream: the
    same paths as with the materialised draws passed explicitly (float64)."""
    from tqf.math.random import RandomType
    from tqf.models import coefficients, euler_sampling, utils
    N, steps = 300, 7
    corr = _corr(d, 3)
    drift, vol = coefficients.gbm(np.full(d, 0.01), np.full(d, 0.2), corr)
    times = np.array([1.0])
    x0 = np.ones(d)
    p = euler_sampling.sample(d, drift, vol, times, num_time_steps=steps, initial_state=x0, num_samples=N,
                              random_type=RandomType.STATELESS, seed=[4, 5], dtype=torch.float64)
    draws = utils.generate_mc_normal_draws(d, steps, N, RandomType.STATELESS, seed=[4, 5], dtype=torch.float64)
    q = euler_sampling.sample(d, drift, vol, times, num_time_steps=steps, initial_state=x0,
                              normal_draws=draws.permute(1, 0, 2), dtype=torch.float64)
    np.testing.assert_allclose(p.cpu().numpy(), q.cpu().numpy(), rtol=1e-13, atol=0)


@pytest.mark.parametrize("dtype,d", [(torch.float32, 17), (torch.float32, 32), (torch.float32, 64),
                                     (torch.float32, 100), (torch.float64, 17), (torch.float64, 64)])
def test_mvgbm_paths_any_dim_match_oracle(cuda, dtype, d):
    """Correlated GBM paths (exact log scheme) for 17..100 factors against the
    oracle given the same draws; float32 with 16 < dim <= 64 takes the
    tensor-core split-BF16 L z (K and N tiled in 16s, zero padding), and
    agrees with the CUDA-core path (lz_mode=1) too."""
    from oracle import mvgbm as omvgbm
    from tqf.models import MultivariateGeometricBrownianMotion
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    N, k = 1000, 9
    rng = np.random.default_rng(d)
    vols = rng.uniform(0.1, 0.4, d)
    corr = _corr(d, d + 7)
    times = np.linspace(1.0 / k, 1.0, k).astype(np_dt)
    draws = rng.standard_normal((N, k, d)).astype(np_dt)
    x0 = rng.uniform(50, 150, (N, d)).astype(np_dt)
    proc = MultivariateGeometricBrownianMotion(d, means=0.03, volatilities=vols, corr_matrix=corr, dtype=np_dt)
    got = proc.sample_paths(times, initial_state=x0, normal_draws=draws).cpu().numpy()
    fma = proc.sample_paths(times, initial_state=x0, normal_draws=draws, lz_mode=1).cpu().numpy()
    want = omvgbm.sample_with_draws(np.full(d, 0.03), vols, corr, times, np.ones(d, np_dt),
                                    draws.transpose(1, 0, 2), np_dt) * x0[:, None, :]
    rtol = 1e-5 if dtype == torch.float32 else 1e-12
    np.testing.assert_allclose(got, want, rtol=rtol, atol=0)
    np.testing.assert_allclose(fma, want, rtol=rtol, atol=0)


def test_cholesky_beyond_64(cuda):
    from tqf.models.multivariate_gbm import cholesky_f64
    c = _corr(100, 5)
    L = cholesky_f64(c, cuda).cpu().numpy()
    np.testing.assert_allclose(L, np.linalg.cholesky(c), rtol=1e-12, atol=1e-13)
    bad = c.copy()
    bad[0, 1] = bad[1, 0] = 2.0
    with pytest.raises(ValueError):
        cholesky_f64(bad, cuda)


@pytest.mark.parametrize("d", [17, 40])
def test_basket_any_dim_sums_and_greeks_match_oracle(cuda, d):
    """The basket pricer for more than 16 assets (one warp per path): payoff
    sums against the oracle paths and the pathwise Greeks against torch
    autograd of the restated graph, on the same draws (float64)."""
    from oracle import mvgbm as omvgbm
    from tqf.pricing import basket_european_mc
    N, steps = 20000, 16
    rng = np.random.default_rng(d)
    vols = rng.uniform(0.1, 0.4, d)
    corr = _corr(d, d + 11)
    draws = rng.standard_normal((N, steps, d))
    res = basket_european_mc(spots=np.full(d, 100.0), vols=vols, rate=0.02, corr=corr, strike=100.0, expiry=1.0,
                             num_time_steps=steps, num_samples=N, normal_draws=torch.as_tensor(draws).cuda(),
                             dtype=torch.float64)
    times = np.linspace(0, 1, steps + 1)[1:]
    paths = omvgbm.sample_with_draws(np.full(d, 0.02), vols, corr, times, np.full(d, 100.0),
                                     draws.transpose(1, 0, 2), np.float64)
    pay = np.maximum(paths[:, -1, :].mean(-1) - 100.0, 0)
    np.testing.assert_allclose(float(res.sums[0]), pay.sum(), rtol=1e-10)
    np.testing.assert_allclose(float(res.sums[1]), (pay * pay).sum(), rtol=1e-10)
    spots = torch.full((d,), 100.0, dtype=torch.float64, requires_grad=True)
    v = torch.as_tensor(vols, dtype=torch.float64).requires_grad_(True)
    rate = torch.tensor(0.02, dtype=torch.float64, requires_grad=True)
    p = omvgbm.basket_price_torch(spots, v, rate, corr, np.full(d, 1.0 / d), 100.0, times, draws.transpose(1, 0, 2))
    p.backward()
    np.testing.assert_allclose(res.price, float(p.detach()), rtol=1e-10)
    np.testing.assert_allclose(res.delta.numpy(), spots.grad.numpy(), rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(res.vega.numpy(), v.grad.numpy(), rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(res.rho, float(rate.grad), rtol=1e-8)


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 1e-5), (np.float64, 1e-12)])
@pytest.mark.parametrize("dim", [10, 17])
def test_milstein_any_dim_matches_oracle(cuda, dtype, rtol, dim):
    """Milstein (Stratonovich order 3) for more than 8 factors, structured
    coefficients (one warp per path) and caller-evaluated callables (the
    update kernel, forward-mode volatility gradient), against the oracle's
    restatement of milstein_sampling.py on the same normals."""
    from oracle import milstein as omil
    from tqf.models import coefficients as coef
    from tqf.models import milstein_sampling, utils
    rng = np.random.default_rng(dim)
    order = 3
    m = rng.uniform(-0.05, 0.05, dim)
    M = np.diag(rng.uniform(0.01, 0.1, dim)) + 0.01 * rng.standard_normal((dim, dim))
    s0 = rng.uniform(0.0, 0.05, dim)
    s1 = rng.uniform(0.1, 0.3, dim)
    C = np.linalg.cholesky(0.5 * np.eye(dim) + 0.5)
    times, time_step, N = [0.25, 0.5], 0.125, 300
    all_times, keep, _ = utils.prepare_grid(times=np.asarray(times, dtype), time_step=dtype(time_step), dtype=dtype)
    steps = len(all_times) - 1
    K = dim + 3 * dim * order
    draws = rng.standard_normal((N, steps, K)).astype(dtype)
    x0 = np.linspace(1.0, 1.5, dim).astype(dtype)
    drift, vol = coef.AffineDrift(m, M), coef.ScaledVolatility(s0, s1, C)
    kw = dict(dim=dim, times=np.asarray(times, dtype), time_step=time_step, initial_state=x0, normal_draws=draws,
              dtype=dtype, stratonovich_order=order)
    got = milstein_sampling.sample(drift_fn=drift, volatility_fn=vol, **kw).cpu().numpy()
    gen = milstein_sampling.sample(drift_fn=lambda t, x: drift(t, x), volatility_fn=lambda t, x: vol(t, x),
                                   **kw).cpu().numpy()
    dfn, vfn, gfn = omil.affine_coefficients(m, M, s0, s1, C, dtype)
    want = omil.sample_with_draws(dfn, vfn, gfn, all_times, keep, len(times), np.broadcast_to(x0, (N, dim)),
                                  draws.transpose(1, 0, 2), order, dtype)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-3)
    np.testing.assert_allclose(gen, want, rtol=rtol, atol=rtol * 1e-3)
