"""The reference's HestonModel.sample_paths tests (GPU).

Restated from heston_model_test.py with the same parameters, sizes, grids and
tolerances (the draws are this project's own streams, so the checks are
statistical):
* piecewise-constant parameters in float32, float64 and the default dtype
  (:175-219): paths have the requested dtype and shape, and the model's drift
  and volatility at t = 0.1 are the pinned values;
* the QE Monte Carlo price of a call with piecewise mean reversion against
  the semi-analytic Heston price within 0.1 (:270-383), for num_time_steps,
  a times_grid, and a times_grid with supplied antithetic draws.  As in the
  reference the QE scheme carries no rate, so S_T is scaled by e^{rT}.
"""

import numpy as np
import pytest
import torch

from oracle import closed_form

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float32, np.float64, None])
def test_piecewise_and_dtype(cuda, dtype):
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import HestonModel
    process = HestonModel(mean_reversion=PiecewiseConstantFunc([0.5], [1, 1.1], dtype=dtype),
                          theta=PiecewiseConstantFunc([0.5], [1, 0.9], dtype=dtype),
                          volvol=PiecewiseConstantFunc([0.3], [0.1, 0.2], dtype=dtype),
                          rho=PiecewiseConstantFunc([0.5], [0.4, 0.6], dtype=dtype), dtype=dtype)
    initial_state = np.array([np.log(100), 0.045], dtype=dtype)
    paths = process.sample_paths([0.1, 1.0], time_step=0.1, num_samples=100, initial_state=initial_state, seed=None)
    assert tuple(paths.shape) == (100, 2, 2)
    if dtype is not None:
        assert paths.dtype == {np.float32: torch.float32, np.float64: torch.float64}[dtype]
    assert torch.isfinite(paths).all()
    x0 = torch.as_tensor(initial_state.astype(np.float64))
    np.testing.assert_allclose(process.drift_fn()(0.1, x0).numpy(), [-0.0225, 0.955], rtol=1e-6)
    np.testing.assert_allclose(process.volatility_fn()(0.1, x0).numpy(),
                               [[0.21213203, 0.0], [0.00848528, 0.01944222]], rtol=1e-6)


VARIANTS = {
    "SamplePathsWithNumTimeStep": (True, False, False),
    "SamplePathsWithGrid": (False, True, False),
    "SamplePathsWithGridAndDraws": (False, True, True),
}


@pytest.mark.parametrize("case", sorted(VARIANTS))
def test_compare_monte_carlo_to_european_option(cuda, case):
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models import HestonModel
    use_num_time_step, use_time_grid, supply_draws = VARIANTS[case]
    kappa, theta, volvol, rho = 0.3, 0.05, 0.02, 0.1
    maturity, x0, v0, strike, rate = 1.0, 3.0, 0.05, 15, 0.5
    heston = HestonModel(mean_reversion=PiecewiseConstantFunc([0.1, 0.2], [kappa] * 3, dtype=np.float64),
                         theta=theta, volvol=volvol, rho=rho, dtype=np.float64)
    num_samples, time_step, times_grid, num_time_steps, normal_draws = 10000, None, None, None, None
    if use_num_time_step:
        num_time_steps = 100
    else:
        time_step = 0.01
    if use_time_grid:
        times_grid = np.linspace(0.0, 1.0, 101)
    if supply_draws:
        num_samples = 1
        half = np.random.default_rng(142).standard_normal((5000, 100, 2))
        normal_draws = np.concatenate([half, -half], axis=0)
    samples = heston.sample_paths(times=[maturity / 2, maturity], initial_state=np.array([x0, v0]),
                                  time_step=time_step, num_samples=num_samples,
                                  random_type=RandomType.STATELESS_ANTITHETIC, seed=[1, 42],
                                  num_time_steps=num_time_steps, normal_draws=normal_draws, times_grid=times_grid)
    assert tuple(samples.shape) == (10000, 2, 2)
    log_spots = samples[:, -1, 0].cpu().numpy()
    mc = np.exp(-rate * maturity) * np.mean(np.maximum(np.exp(log_spots) * np.exp(rate * maturity) - strike, 0))
    ref = closed_form.heston_price(spot=np.exp(x0), strike=strike, expiry=maturity, rate=rate, v0=v0,
                                   kappa=kappa, theta=theta, xi=volvol, rho=rho)
    np.testing.assert_allclose(mc, ref, atol=0.1, rtol=0.1)


def test_volatility(cuda):
    # :32-49: with a tiny vol of vol the variance stays within 0.005 of theta
    # after the first 50 requested times
    from tqf.models import HestonModel
    process = HestonModel(mean_reversion=1.0, theta=0.05, volvol=0.00001, rho=-0.0, dtype=np.float64)
    times = np.linspace(0.0, 1.0, 365)
    paths = process.sample_paths(times, time_step=0.01, num_samples=2, initial_state=np.array([np.log(100), 0.045]),
                                 seed=None)
    assert np.max(np.abs(paths.cpu().numpy()[..., 1][:, 50:] - 0.05)) < 0.005


def test_state(cuda):
    # :51-77: with a tiny vol of vol the spot is a GBM with volatility sqrt(theta)
    from tqf.models import HestonModel
    process = HestonModel(mean_reversion=1.0, theta=1.0, volvol=0.00001, rho=-0.0, dtype=np.float64)
    times = [0.0, 0.5, 1.0]
    state = process.sample_paths(times, time_step=0.001, num_samples=1000,
                                 initial_state=np.array([np.log(100), 1.0]), seed=None).cpu().numpy()[..., 0]
    np.testing.assert_allclose(state[:, 0], np.log(100), 1e-8)
    for i in (1, 2):
        np.testing.assert_allclose(np.mean(np.exp(state[:, i])), 100, 1.0)
        np.testing.assert_allclose(np.std(np.exp(state[:, 1])), 100 * np.sqrt(np.exp(times[i]) - 1), 2.0)


def test_expected_var_mc(cuda):
    # :97-135: the Monte Carlo integral of the variance over [0, 1] against
    # expected_total_variance within 1%
    from tqf.models import HestonModel
    process = HestonModel(mean_reversion=10.0, theta=0.04, volvol=1.0, rho=-0.5, dtype=np.float64)
    times = np.linspace(0, 1.0, 252)
    paths = process.sample_paths(times, np.array([1.0, 0.1]), time_step=0.1, num_samples=10000,
                                 seed=123).cpu().numpy()
    weights = np.concatenate([[times[0]], np.diff(times)])
    mc = np.mean(np.sum(weights * paths[:, :, 1], axis=1))
    np.testing.assert_allclose(float(process.expected_total_variance(1.0, 0.1)), mc, rtol=0.01)
