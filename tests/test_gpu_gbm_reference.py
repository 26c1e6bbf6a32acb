"""The reference's geometric Brownian motion sampling tests (GPU).

Restated from geometric_brownian_motion_test.py with the same parameters,
sizes and tolerances:
* the multivariate log-moments and correlations (:811-859) with Sobol draws
  and with supplied antithetic draws;
* draws whose last dimension does not match the process raise ValueError
  (:953-981);
* the gradient of the sample mean with respect to a watched volatility is
  near zero (:983-1001), and equals central finite differences on common
  random numbers (1e-6 relative).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("supply_draws,dtype", [(False, np.float32), (False, np.float64), (True, np.float64)])
def test_multivariate_sample_mean_and_variance(cuda, supply_draws, dtype):
    from tqf.math.random import RandomType
    from tqf.models import MultivariateGeometricBrownianMotion
    means, vols, corr = 0.05, np.array([0.1, 0.2]), [[1, 0.1], [0.1, 1]]
    process = MultivariateGeometricBrownianMotion(dim=2, means=means, volatilities=vols, corr_matrix=corr,
                                                  dtype=dtype)
    times, initial_state = [0.1, 0.5, 1.0], [1.0, 2.0]
    num_samples, normal_draws = 10000, None
    if supply_draws:
        num_samples = 50000
        half = np.random.default_rng(42).standard_normal((num_samples // 2, 3, 2)).astype(dtype)
        normal_draws = np.concatenate([half, -half], axis=0)
    samples = process.sample_paths(times=times, initial_state=initial_state, random_type=RandomType.SOBOL,
                                   num_samples=num_samples, normal_draws=normal_draws).cpu().numpy()
    log_s = np.log(samples.astype(np.float64))
    mean = log_s.mean(axis=0)
    var = ((log_s - mean) ** 2).mean(axis=0)
    t = np.array(times)[:, None]
    np.testing.assert_allclose(mean, (means - vols ** 2 / 2) * t + np.log(initial_state), atol=1e-3, rtol=1e-3)
    np.testing.assert_allclose(var, vols ** 2 * t, atol=1e-3, rtol=1e-3)
    corr_last = np.corrcoef(samples[:, -1, :].astype(np.float64), rowvar=False)
    np.testing.assert_allclose(corr_last, corr, atol=1e-2, rtol=1e-2)


def test_normal_draws_shape_mismatch(cuda):
    from tqf.models import GeometricBrownianMotion, MultivariateGeometricBrownianMotion
    mv = MultivariateGeometricBrownianMotion(dim=2, means=0.05, volatilities=[0.1, 0.2], dtype=np.float64)
    with pytest.raises(ValueError):
        mv.sample_paths(times=[0.1, 0.5, 1.0], normal_draws=np.random.default_rng(0).standard_normal((100, 3, 3)))
    uv = GeometricBrownianMotion(mean=0.05, volatility=0.1, dtype=np.float64)
    with pytest.raises(ValueError):
        uv.sample_paths(times=[0.1, 0.5, 1.0], normal_draws=np.random.default_rng(0).standard_normal((100, 3, 2)))


def _gbm_mean(volatility, mean=0.05):
    from tqf.math.random import RandomType
    from tqf.models import GeometricBrownianMotion
    process = GeometricBrownianMotion(mean=mean, volatility=volatility, dtype=np.float64)
    samples = process.sample_paths(times=[0.0, 0.1, 0.5, 1.0], num_samples=10_000, seed=[4, 2],
                                   random_type=RandomType.STATELESS_ANTITHETIC)
    return samples.mean()


def test_gbm_normal_draws_gradient(cuda):
    volatility = torch.tensor(0.1, dtype=torch.float64, requires_grad=True)
    (grad,) = torch.autograd.grad(_gbm_mean(volatility), volatility)
    # E[X_t] does not depend on the volatility
    assert abs(float(grad)) < 1e-3
    h = 1e-5
    fd = (float(_gbm_mean(0.1 + h)) - float(_gbm_mean(0.1 - h))) / (2 * h)
    np.testing.assert_allclose(float(grad), fd, rtol=1e-6, atol=1e-9)
    mean = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    (g_mu,) = torch.autograd.grad(_gbm_mean(0.1, mean), mean)
    fd_mu = (float(_gbm_mean(0.1, 0.05 + h)) - float(_gbm_mean(0.1, 0.05 - h))) / (2 * h)
    np.testing.assert_allclose(float(g_mu), fd_mu, rtol=1e-6)
