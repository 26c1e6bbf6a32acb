"""The reference's Milstein sampling tests not covered elsewhere (GPU).

Restated from milstein_sampling_test.py with the same process, sizes and
tolerances: the Wiener process dX = dW has mean 0 and covariance min(s, t)
within 1e-2 for the custom for-loop (an empty watch_params list) and the
while loop, with time_step and with num_time_steps (:36-108); output dtypes
(:325-345).  The 1-d, Black-Scholes and SABR cases are in
test_gpu_milstein_gbm.py.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

WIENER = {
    "CustomForLoopWithTimeStep": (True, True),
    "WhileLoopWithTimeStep": (False, True),
    "CustomForLoopWithNumSteps": (True, False),
    "WhileLoopWithNumSteps": (False, False),
}


@pytest.mark.parametrize("case", sorted(WIENER))
def test_sample_paths_wiener(cuda, case):
    from tqf.math.random import RandomType
    from tqf.models import milstein_sampling
    watch, use_time_step = WIENER[case]
    times = np.array([0.1, 0.2, 0.3])
    num_samples = 5000
    paths = milstein_sampling.sample(dim=1, drift_fn=lambda _, x: torch.zeros_like(x),
                                     volatility_fn=lambda _, x: torch.ones_like(x)[..., None], times=times,
                                     num_samples=num_samples, seed=[1, 42],
                                     random_type=RandomType.STATELESS_ANTITHETIC,
                                     time_step=0.02 if use_time_step else None,
                                     num_time_steps=None if use_time_step else 15,
                                     watch_params=[] if watch else None)
    assert tuple(paths.shape) == (num_samples, 3, 1)
    p = paths.cpu().numpy()
    np.testing.assert_allclose(p.mean(axis=0).reshape(-1), np.zeros(3), rtol=1e-2, atol=1e-2)
    np.testing.assert_allclose(np.cov(p.reshape(num_samples, -1), rowvar=False),
                               np.minimum(times.reshape(-1, 1), times.reshape(1, -1)), rtol=1e-2, atol=1e-2)


def test_sample_paths_dtypes(cuda):
    from tqf.models import milstein_sampling
    for dtype, want in [(np.float32, torch.float32), (np.float64, torch.float64)]:
        paths = milstein_sampling.sample(dim=1, drift_fn=lambda t, x: 0.5 * x,
                                         volatility_fn=lambda t, x: 0.5 * x[..., None],
                                         times=[0.1, 0.2], num_samples=10, initial_state=[0.1], time_step=0.01,
                                         seed=123, dtype=dtype)
        assert paths.dtype == want
