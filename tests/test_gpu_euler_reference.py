"""The reference's statistical tests of euler_sampling.sample (GPU).

Restated from euler_sampling_test.py with the same processes, sizes, grids
and tolerances; draws come from this project's streams, so where the
reference fixes a seed the check is statistical, not bit-exact:
* Wiener process dX = dW (:71-133): mean 0 and covariance min(s, t) within
  1e-2 for custom-for-loop / while-loop, time_step / num_time_steps,
  times_grid and times_grid with supplied antithetic draws;
* times_grid running past the last requested time (:135-170);
* the 2-d process dX_i = mu_i sqrt(t) dt + sum_j (a_ij t + b_ij) dW_j, mean
  x0 + 2/3 mu t^1.5 within 1e-2 for PSEUDO, STATELESS, SOBOL and
  HALTON_RANDOMIZED draws (:314-359) and for HALTON draws with skip 100 with
  and without watched parameters (:371-418);
* antithetic means within 5e-3 (:431-481; the reference names its cases
  PSEUDO_ANTITHETIC / STATELESS_ANTITHETIC and its docstring describes
  antithetic draws, which is what runs here);
* output dtypes (:484-500).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

WIENER = {
    "CustomForLoopWithTimeStep": (True, True, False, False),
    "WhileLoopWithTimeStep": (False, True, False, False),
    "CustomForLoopWithNumSteps": (True, False, False, False),
    "WhileLoopWithNumSteps": (False, False, False, False),
    "WhileLoopWithGrid": (False, False, True, False),
    "WhileLoopWithGridAndDraws": (False, False, True, True),
}


def _wiener_fns():
    return (lambda t, x: torch.zeros_like(x)), (lambda t, x: torch.ones_like(x)[..., None])


def _check_wiener(paths, times, num_samples):
    assert tuple(paths.shape) == (num_samples, 3, 1)
    p = paths.detach().cpu().numpy()
    means = p.mean(axis=0).reshape(-1)
    covars = np.cov(p.reshape(num_samples, -1), rowvar=False)
    np.testing.assert_allclose(means, np.zeros(3), rtol=1e-2, atol=1e-2)
    np.testing.assert_allclose(covars, np.minimum(times.reshape(-1, 1), times.reshape(1, -1)), rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("case", sorted(WIENER))
def test_sample_paths_wiener(cuda, case):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    watch, use_time_step, use_grid, supply_draws = WIENER[case]
    drift_fn, vol_fn = _wiener_fns()
    times = np.array([0.1, 0.2, 0.3])
    num_samples = 10000
    time_step, num_time_steps = (0.01, None) if use_time_step else (None, 30)
    times_grid = None
    if use_grid:
        time_step = None
        times_grid = np.linspace(0.0, 0.3, 31)
    normal_draws = None
    if supply_draws:
        num_samples = 1
        half = np.random.default_rng(142).standard_normal((5000, 30, 1))
        normal_draws = np.concatenate([half, -half], axis=0)
    paths = euler_sampling.sample(dim=1, drift_fn=drift_fn, volatility_fn=vol_fn, times=times,
                                  num_samples=num_samples, time_step=time_step, num_time_steps=num_time_steps,
                                  watch_params=[] if watch else None, normal_draws=normal_draws,
                                  times_grid=times_grid, random_type=RandomType.STATELESS_ANTITHETIC,
                                  seed=[1, 42])
    _check_wiener(paths, times, 10000)


def test_times_grid_long(cuda):
    from tqf.models import euler_sampling
    drift_fn, vol_fn = _wiener_fns()
    times = np.array([0.1, 0.2, 0.3])
    half = np.random.default_rng(143).standard_normal((5000, 32, 1))
    paths = euler_sampling.sample(dim=1, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, num_samples=10000,
                                  normal_draws=np.concatenate([half, -half], axis=0),
                                  times_grid=np.linspace(0.0, 0.32, 33), seed=[1, 42])
    _check_wiener(paths, times, 10000)


MU = np.array([0.2, 0.7])
A2 = np.array([[0.4, 0.1], [0.3, 0.2]])
B2 = np.array([[0.33, -0.03], [0.21, 0.5]])
X0 = np.array([0.1, -1.1])


def _expected_2d(times):
    return X0 + (2.0 / 3.0) * MU * np.power(np.reshape(times, [-1, 1]), 1.5)


@pytest.mark.parametrize("rt,seed", [("PSEUDO", 12134), ("STATELESS", [1, 2]), ("SOBOL", None),
                                     ("HALTON_RANDOMIZED", 12134)])
def test_sample_paths_2d(cuda, rt, seed):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling

    def drift_fn(t, x):
        return torch.as_tensor(MU, device=x.device) * torch.sqrt(t) * torch.ones_like(x, dtype=t.dtype)

    def vol_fn(t, x):
        del x
        a, b = (torch.as_tensor(v, device=t.device) for v in (A2, B2))
        return (a * t + b) * torch.ones([2, 2], dtype=t.dtype, device=t.device)

    times = np.array([0.1, 0.21, 0.32, 0.43, 0.55])
    paths = euler_sampling.sample(dim=2, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, num_samples=10000,
                                  initial_state=X0, time_step=0.01, random_type=getattr(RandomType, rt),
                                  seed=seed)
    assert tuple(paths.shape) == (10000, 5, 2)
    np.testing.assert_allclose(paths.cpu().numpy().mean(axis=0), _expected_2d(times), rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("watch", [True, False])
def test_halton_sample_paths_2d(cuda, watch):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    times = np.array([0.1, 0.21, 0.32])
    mu, a, b = (torch.tensor(v, dtype=torch.float64, device=cuda, requires_grad=watch) for v in (MU, A2, B2))

    def drift_fn(t, x):
        return mu * torch.sqrt(t) * torch.ones_like(x, dtype=t.dtype)

    def vol_fn(t, x):
        del x
        return (a * t + b) * torch.ones([2, 2], dtype=t.dtype, device=t.device)

    paths = euler_sampling.sample(dim=2, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, num_samples=10000,
                                  initial_state=X0, random_type=RandomType.HALTON, time_step=0.01, seed=12134,
                                  skip=100, watch_params=[a, b] if watch else None, dtype=torch.float64)
    assert tuple(paths.shape) == (10000, 3, 2)
    np.testing.assert_allclose(paths.detach().cpu().numpy().mean(axis=0), _expected_2d(times), rtol=1e-2,
                               atol=1e-2)


@pytest.mark.parametrize("rt,seed", [("PSEUDO_ANTITHETIC", 12134), ("STATELESS_ANTITHETIC", [0, 12134])])
def test_antithetic_sample_paths_mean_2d(cuda, rt, seed):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling

    def drift_fn(t, x):
        del x
        return torch.as_tensor(MU, device=t.device) * torch.sqrt(t)

    def vol_fn(t, x):
        del x
        a, b = (torch.as_tensor(v, device=t.device) for v in (A2, B2))
        return (a * t + b) * torch.ones([2, 2], dtype=t.dtype, device=t.device)

    times = np.array([0.1, 0.21, 0.32, 0.43, 0.55])
    paths = euler_sampling.sample(dim=2, drift_fn=drift_fn, volatility_fn=vol_fn, times=times, num_samples=5000,
                                  initial_state=X0, random_type=getattr(RandomType, rt), time_step=0.01, seed=seed)
    assert tuple(paths.shape) == (5000, 5, 2)
    np.testing.assert_allclose(paths.cpu().numpy().mean(axis=0), _expected_2d(times), rtol=5e-3, atol=5e-3)


def test_sample_paths_dtypes(cuda):
    from tqf.models import euler_sampling
    for dtype, want in [(np.float32, torch.float32), (np.float64, torch.float64)]:
        paths = euler_sampling.sample(dim=1, drift_fn=lambda t, x: torch.sqrt(t) * torch.ones_like(x, dtype=t.dtype),
                                      volatility_fn=lambda t, x: t * torch.ones([1, 1], dtype=t.dtype,
                                                                                 device=t.device),
                                      times=[0.1, 0.2], num_samples=10, initial_state=[0.1], time_step=0.01,
                                      seed=123, dtype=dtype)
        assert paths.dtype == want and tuple(paths.shape) == (10, 2, 1)
