"""The reference's GenericItoProcess.sample_paths tests (GPU).

Restated from generic_ito_process_test.py:37-231 with the same processes,
sizes, grids and tolerances (draws from this project's streams, so the
checks are statistical): the Wiener process (mean 0, covariance min(s, t)),
the 2-d process dX_i = mu_i sqrt(t) dt + sum_j (a_ij t + b_ij) dW_j with and
without a times_grid and supplied antithetic draws, batches of rank 1 and 2,
and output dtypes.  The fd_solver_backward tests are out of scope (no PDE
solvers are built).

The reference's bounds on sample means (1e-2 absolute plus 1e-2 relative at
10,000 paths) are checks of its own seeded stream and come to about two
standard errors; with another stream a mean is accepted within the larger of
that bound and four standard errors of the sample.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MU = np.array([0.2, 0.7])
A2 = np.array([[0.4, 0.1], [0.3, 0.2]])
B2 = np.array([[0.33, -0.03], [0.21, 0.5]])
X0 = np.array([0.1, -1.1])
TIMES = np.array([0.1, 0.21, 0.32, 0.43, 0.55])


def _assert_means(paths, expected, axis, rtol=1e-2, atol=1e-2):
    mean = paths.mean(axis=axis)
    se = paths.std(axis=axis, ddof=1) / np.sqrt(paths.shape[axis])
    bound = np.maximum(atol + rtol * np.abs(expected), 4 * se)
    assert np.all(np.abs(mean - expected) <= bound), (mean, expected, bound)


def _drift(t, x):
    return torch.as_tensor(MU, device=x.device) * torch.sqrt(t) * torch.ones_like(x, dtype=t.dtype)


def test_sample_paths_wiener(cuda):
    from tqf.models import GenericItoProcess
    process = GenericItoProcess(dim=1, drift_fn=lambda _, x: torch.zeros_like(x),
                                volatility_fn=lambda _, x: torch.ones_like(x)[..., None])
    times = np.array([0.1, 0.2, 0.3])
    paths = process.sample_paths(times=times, num_samples=10000, seed=42, time_step=0.01).cpu().numpy()
    _assert_means(paths.reshape(10000, 3), np.zeros(3), axis=0)
    covars = np.cov(paths.reshape(10000, -1), rowvar=False)
    np.testing.assert_allclose(covars, np.minimum(times.reshape(-1, 1), times.reshape(1, -1)), rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("use_grid_and_draws", [False, True], ids=["NoGridNoDraws", "WithGridWithDraws"])
def test_sample_paths_2d(cuda, use_grid_and_draws):
    from tqf.models import GenericItoProcess

    def vol_fn(t, x):
        del x
        a, b = (torch.as_tensor(v, device=t.device) for v in (A2, B2))
        return (a * t + b) * torch.ones([2, 2], dtype=t.dtype, device=t.device)

    process = GenericItoProcess(dim=2, drift_fn=_drift, volatility_fn=vol_fn)
    if use_grid_and_draws:
        times_grid, time_step, num_samples = np.linspace(0.0, 0.55, 56), None, 1
        half = np.random.default_rng(144).standard_normal((5000, 55, 2))
        normal_draws = np.concatenate([half, -half], axis=0)
    else:
        times_grid, time_step, num_samples, normal_draws = None, 0.01, 10000, None
    paths = process.sample_paths(TIMES, num_samples=num_samples, initial_state=X0, time_step=time_step,
                                 times_grid=times_grid, normal_draws=normal_draws, seed=12134)
    assert tuple(paths.shape) == (10000, 5, 2)
    expected = X0 + (2.0 / 3.0) * MU * np.power(TIMES.reshape(-1, 1), 1.5)
    _assert_means(paths.cpu().numpy(), expected, axis=0)


@pytest.mark.parametrize("batch_rank", [1, 2])
def test_batch_sample_paths_2d(cuda, batch_rank):
    from tqf.models import GenericItoProcess

    def vol_fn(t, x):
        a, b = (torch.as_tensor(v, device=t.device) for v in (A2, B2))
        return (a * t + b) * torch.ones(list(x.shape) + [2], dtype=t.dtype, device=t.device)

    process = GenericItoProcess(dim=2, drift_fn=_drift, volatility_fn=vol_fn, dtype=np.float64)
    x0 = X0 * np.ones([2] * batch_rank + [1, 2])
    paths = process.sample_paths(TIMES, num_samples=10000, initial_state=x0, time_step=0.01, seed=12134)
    assert list(paths.shape) == [2] * batch_rank + [10000, 5, 2]
    times = np.reshape(TIMES, [1] * batch_rank + [-1, 1])
    expected = np.reshape(x0, [2] * batch_rank + [1, 2]) + (2.0 / 3.0) * MU * np.power(times, 1.5)
    _assert_means(paths.cpu().numpy(), expected, axis=batch_rank)


def test_sample_paths_dtypes(cuda):
    from tqf.models import GenericItoProcess
    for dtype, want in [(np.float32, torch.float32), (np.float64, torch.float64)]:
        process = GenericItoProcess(dim=1, drift_fn=lambda t, x: torch.sqrt(t) * torch.ones_like(x, dtype=t.dtype),
                                    volatility_fn=lambda t, x: t * torch.ones([1, 1], dtype=t.dtype, device=t.device),
                                    dtype=dtype)
        paths = process.sample_paths(times=[0.1, 0.2], num_samples=10, initial_state=[0.1], time_step=0.01, seed=123)
        assert paths.dtype == want
