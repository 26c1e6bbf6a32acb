"""Milstein sampler and univariate GBM on the GPU against the oracle's
restatements of milstein_sampling.py and univariate_geometric_brownian_motion.py."""

import numpy as np
import pytest
import torch

from oracle import milstein as omil
from oracle import mvgbm as omvgbm
from tqf.models import utils as mutils

pytestmark = pytest.mark.gpu


def _grid(times, time_step, dtype):
    all_times, keep, _ = mutils.prepare_grid(times=np.asarray(times, dtype), time_step=dtype(time_step),
                                             dtype=np.dtype(dtype))
    return all_times, keep


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 1e-5), (np.float64, 1e-12)])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_milstein_structured_matches_oracle(cuda, dtype, rtol, dim):
    from tqf.models import coefficients as coef
    from tqf.models import milstein_sampling
    rng = np.random.default_rng(dim)
    order = 5
    m = rng.uniform(-0.05, 0.05, dim)
    M = np.diag(rng.uniform(0.01, 0.1, dim)) + 0.01 * rng.standard_normal((dim, dim))
    s0 = rng.uniform(0.0, 0.05, dim)
    s1 = rng.uniform(0.1, 0.3, dim)
    C = np.linalg.cholesky(0.5 * np.eye(dim) + 0.5) if dim > 1 else np.ones((1, 1))
    times, time_step, N = [0.25, 0.5, 1.0], 0.1, 2000
    all_times, keep = _grid(times, time_step, dtype)
    steps = len(all_times) - 1
    K = dim + 3 * dim * order
    draws = rng.standard_normal((N, steps, K)).astype(dtype)
    x0 = np.linspace(1.0, 1.5, dim).astype(dtype)
    got = milstein_sampling.sample(dim=dim, drift_fn=coef.AffineDrift(m, M), volatility_fn=coef.ScaledVolatility(s0, s1, C),
                                   times=np.asarray(times, dtype), time_step=time_step, initial_state=x0,
                                   normal_draws=draws, dtype=dtype).cpu().numpy()
    dfn, vfn, gfn = omil.affine_coefficients(m, M, s0, s1, C, dtype)
    want = omil.sample_with_draws(dfn, vfn, gfn, all_times, keep, len(times), np.broadcast_to(x0, (N, dim)),
                                  draws.transpose(1, 0, 2), order, dtype)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-3)


@pytest.mark.parametrize("dim", [1, 2])
def test_milstein_generic_callables(cuda, dim):
    """Arbitrary callables: per-step torch evaluation (forward-mode gradient, or
    a supplied grad_volatility_fn) and the update kernel equal the fused path."""
    from tqf.models import coefficients as coef
    from tqf.models import milstein_sampling
    dtype = np.float64
    rng = np.random.default_rng(10 + dim)
    m, M = np.full(dim, 0.02), np.diag(np.full(dim, 0.05))
    s0, s1 = np.full(dim, 0.01), np.full(dim, 0.2)
    C = np.linalg.cholesky(0.7 * np.eye(dim) + 0.3) if dim > 1 else np.ones((1, 1))
    drift, vol = coef.AffineDrift(m, M), coef.ScaledVolatility(s0, s1, C)
    times, N = [0.5, 1.0], 1500
    all_times, keep = _grid(times, 0.1, dtype)
    K = dim + 3 * dim * 5
    draws = rng.standard_normal((N, len(all_times) - 1, K))
    kw = dict(dim=dim, times=np.asarray(times), time_step=0.1, initial_state=np.ones(dim), normal_draws=draws,
              dtype=dtype)
    fused = milstein_sampling.sample(drift_fn=drift, volatility_fn=vol, **kw).cpu().numpy()
    generic = milstein_sampling.sample(drift_fn=lambda t, x: drift(t, x), volatility_fn=lambda t, x: vol(t, x),
                                       **kw).cpu().numpy()
    np.testing.assert_allclose(generic, fused, rtol=1e-12, atol=1e-14)

    def grad_fn(t, x, e):
        # directional derivative of B along e: dB_kj = s1_k e_k C_kj
        s1t = torch.as_tensor(s1, dtype=x.dtype, device=x.device)
        Ct = torch.as_tensor(C, dtype=x.dtype, device=x.device)
        return (s1t * e)[..., :, None] * Ct

    with_grad = milstein_sampling.sample(drift_fn=lambda t, x: drift(t, x), volatility_fn=lambda t, x: vol(t, x),
                                         grad_volatility_fn=grad_fn, **kw).cpu().numpy()
    np.testing.assert_allclose(with_grad, fused, rtol=1e-12, atol=1e-14)


def test_milstein_gbm_mean(cuda):
    """GBM by Milstein with in-kernel Philox: E[X_1] = exp(mu) within 4 SE."""
    from tqf.math.random import RandomType
    from tqf.models import coefficients as coef
    from tqf.models import milstein_sampling
    drift, vol = coef.gbm([0.05], [0.3])
    x = milstein_sampling.sample(dim=1, drift_fn=drift, volatility_fn=vol, times=[1.0], time_step=0.02,
                                 num_samples=400000, initial_state=[1.0], random_type=RandomType.STATELESS,
                                 seed=[3, 9], dtype=np.float64).cpu().numpy()[:, -1, 0]
    se = x.std() / np.sqrt(x.size)
    assert abs(x.mean() - np.exp(0.05)) < 4 * se


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 1e-5), (np.float64, 1e-12)])
def test_univariate_gbm_matches_oracle(cuda, dtype, rtol):
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import GeometricBrownianMotion
    times = np.array([0.1, 0.2, 0.6, 1.0], dtype)
    N = 3000
    z = np.random.default_rng(5).standard_normal((N, 4, 1)).astype(dtype)
    dts = np.diff(np.concatenate([[0.0], times])).astype(dtype)
    # constant parameters
    proc = GeometricBrownianMotion(dtype(0.05), dtype(0.3), dtype=dtype)
    got = proc.sample_paths(times, initial_state=dtype(1.5), normal_draws=z).cpu().numpy()
    want = omvgbm.univariate_with_draws(dtype(0.05) * dts, dtype(0.3) * dtype(0.3) * dts, 1.5, z[..., 0], dtype)
    np.testing.assert_allclose(got[..., 0], want, rtol=rtol)
    # piecewise-constant parameters
    mu = PiecewiseConstantFunc([0.3, 0.7], [0.01, 0.05, 0.1], dtype=dtype)
    sig = PiecewiseConstantFunc([0.5], [0.2, 0.4], dtype=dtype)
    proc = GeometricBrownianMotion(mu, sig, dtype=dtype)
    got = proc.sample_paths(times, initial_state=dtype(1.0), normal_draws=z).cpu().numpy()
    t0 = np.concatenate([[0.0], times[:-1]]).astype(dtype)
    sq = PiecewiseConstantFunc([0.5], [0.04, 0.16], dtype=dtype)
    want = omvgbm.univariate_with_draws(mu.integrate(t0, times), sq.integrate(t0, times), 1.0, z[..., 0], dtype)
    np.testing.assert_allclose(got[..., 0], want, rtol=rtol)


def test_univariate_gbm_batch_and_moments(cuda):
    from tqf.math.random import RandomType
    from tqf.models import GeometricBrownianMotion
    proc = GeometricBrownianMotion(np.array([[0.05], [0.1]]), np.array([[0.2], [0.3]]), dtype=np.float64)
    s = proc.sample_paths([0.5, 1.0], initial_state=1.0, num_samples=200000, random_type=RandomType.STATELESS,
                          seed=[1, 2]).cpu().numpy()
    assert s.shape == (2, 200000, 2, 1)
    np.testing.assert_allclose(s[:, :, -1, 0].mean(1), np.exp([0.05, 0.1]), rtol=5e-3)
    sob = GeometricBrownianMotion(0.05, 0.2, dtype=np.float64).sample_paths(
        [1.0], num_samples=100000, random_type=RandomType.SOBOL).cpu().numpy()
    np.testing.assert_allclose(sob[:, -1, 0].mean(), np.exp(0.05), rtol=1e-3)


def test_milstein_time_dependent_1d_mean(cuda):
    """dX = mu sqrt(t) dt + (a t + b) dW: E[X_t] = x0 + 2/3 mu t^1.5; the path with
    t = 0 requested equals the one without it (milstein_sampling_test.py:111-166)."""
    from tqf.math.random import RandomType
    from tqf.models import milstein_sampling
    mu, a, b = 0.2, 0.4, 0.33

    def drift_fn(t, x):
        return mu * torch.sqrt(t) * torch.ones_like(x)

    def vol_fn(t, x):
        return (a * t + b) * torch.ones(x.shape[:-1] + (1, 1), dtype=x.dtype, device=x.device)

    times = np.array([0.0, 0.1, 0.21, 0.32, 0.43, 0.55])
    kw = dict(dim=1, drift_fn=drift_fn, volatility_fn=vol_fn, num_samples=10000, initial_state=np.array([0.1]),
              random_type=RandomType.STATELESS_ANTITHETIC, time_step=0.01, seed=[1, 42], dtype=np.float64)
    paths = milstein_sampling.sample(times=times, **kw).cpu().numpy()
    no_zero = milstein_sampling.sample(times=times[1:], **kw).cpu().numpy()
    assert paths.shape == (10000, 6, 1)
    np.testing.assert_allclose(paths.mean(0).reshape(-1), 0.1 + 2.0 / 3.0 * mu * times ** 1.5, rtol=1e-2, atol=1e-2)
    np.testing.assert_allclose(paths[:, 1:, :], no_zero)


@pytest.mark.parametrize("supply_grad", [False, True])
def test_milstein_sabr_matches_euler_moments(cuda, supply_grad):
    """SABR: Milstein mean / std against Euler's with the reference's tolerance
    (rtol = atol = 0.05, milstein_sampling_test.py:233-322).

    The reference's drift correction (_stratonovich_drift_update, :555-562)
    omits the factor 1/2, so its Milstein variance process drifts like
    v0 exp(-t/2): the mean over the paths sits ~0.014 below Euler's (0.136 vs
    0.150), inside the reference test's atol.  The oracle restatement gives the
    same numbers, so this is the reference's behaviour, reproduced."""
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling, milstein_sampling
    beta, volvol, rho = 0.5, 1.0, 0.2

    def vol_fn(t, x):
        f, v = x[..., 0], x[..., 1]
        fb = torch.where(f > 0, f.clamp(min=0) ** beta, torch.zeros_like(f))
        m11 = v * fb * np.sqrt(1 - rho * rho)
        m12 = v * fb * rho
        m22 = volvol * v
        zero = torch.zeros_like(m11)
        return torch.stack([torch.stack([m11, m12], -1), torch.stack([zero, m22], -1)], -2)

    drift_fn = lambda t, x: torch.zeros_like(x)  # noqa: E731
    grad_fn = None
    if supply_grad:
        def grad_fn(t, x, e):
            return torch.func.jvp(lambda y: vol_fn(t, y), (x,), (e,))[1]
    times = np.array([0.0, 0.1, 0.21, 0.32, 0.43, 0.55])
    x0 = np.array([0.1, 0.2])
    mil = milstein_sampling.sample(dim=2, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, num_samples=20000,
                                   initial_state=x0, grad_volatility_fn=grad_fn,
                                   random_type=RandomType.STATELESS_ANTITHETIC, time_step=0.01, seed=[1, 42],
                                   dtype=np.float64).cpu().numpy()
    eul = euler_sampling.sample(dim=2, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, time_step=0.01,
                                num_samples=20000, initial_state=x0, random_type=RandomType.STATELESS_ANTITHETIC,
                                seed=[1, 42], dtype=np.float64).cpu().numpy()
    np.testing.assert_allclose((mil.mean(), mil.std()), (eul.mean(), eul.std()), rtol=0.05, atol=0.05)
    assert abs(mil[:, -1, 1].mean() - 0.2 * np.exp(-0.55 / 2)) < 0.01  # the reference's v drift


def test_milstein_bsm_matches_euler(cuda):
    """GBM (r x, sigma x): Milstein and Euler moments agree to 1e-3
    (milstein_sampling_test.py:168-223)."""
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling, milstein_sampling
    r, sigma = 0.1, 0.2
    drift_fn = lambda t, x: r * x  # noqa: E731
    vol_fn = lambda t, x: sigma * x[..., None]  # noqa: E731
    times = np.array([0.1, 0.21, 0.32, 0.43, 0.55])
    kw = dict(dim=1, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, num_samples=100000,
              initial_state=np.array([0.1]), random_type=RandomType.STATELESS_ANTITHETIC, time_step=0.01,
              seed=[1, 42], dtype=np.float64)
    mil = milstein_sampling.sample(**kw).cpu().numpy()
    eul = euler_sampling.sample(**kw).cpu().numpy()
    np.testing.assert_allclose((mil.mean(), mil.std()), (eul.mean(), eul.std()), rtol=1e-3, atol=1e-3)
