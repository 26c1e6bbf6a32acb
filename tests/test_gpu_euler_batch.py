"""euler_sampling.sample with a batch of initial states (GPU).

The reference's 1-d Ito process test (euler_sampling_test.py:172-291):
dX = mu sqrt(t) dt + (a t + b) dW has E[X_t] = x0 + 2/3 mu t^1.5; the sample
means of 10,000 paths must be within 1e-2 of it for plain, batched,
batched-antithetic, batched watch_params and batched supplied draws, and a
run whose times include 0 must equal one without it from the second time on.
Batched draws keep the reference's layouts: quasi-random points are the C
order flattening of batch_shape + [num_samples] (utils.py:94-99) and
antithetic partners are paths n and n + num_samples / 2 of the same batch
entry (utils.py:98-107).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MU, A, B = 0.2, 0.4, 0.33
TIMES = np.array([0.0, 0.1, 0.21, 0.32, 0.43, 0.55])
CASES = {
    "NonBatch": (False, None, False, "STATELESS"),
    "Batch": (True, None, False, "STATELESS"),
    "BatchAntithetic": (True, None, False, "STATELESS_ANTITHETIC"),
    "BatchWithCustomForLoop": (True, [], False, "STATELESS"),
    "BatchWithNormalDraws": (True, None, True, "STATELESS"),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_sample_paths_1d(cuda, case):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    use_batch, watch_params, supply_draws, rt = CASES[case]
    num_samples = 10000

    def drift_fn(t, x):
        return MU * torch.sqrt(t) * torch.ones_like(x, dtype=t.dtype)

    def vol_fn(t, x):
        del x
        shape = [2, 1, 1, 1] if use_batch else [1, 1]
        return (A * t + B) * torch.ones(shape, dtype=t.dtype, device=t.device)

    normal_draws = None
    if supply_draws:
        half = np.random.default_rng(42).standard_normal((2, 5000, 55, 1))
        normal_draws = np.concatenate([half, -half], axis=1)
    x0 = np.array([[[0.1]], [[0.1]]]) if use_batch else np.array([0.1])
    kw = dict(dim=1, drift_fn=drift_fn, volatility_fn=vol_fn, num_samples=num_samples, initial_state=x0,
              random_type=getattr(RandomType, rt), normal_draws=normal_draws, time_step=0.01, seed=[1, 42],
              dtype=torch.float64)
    paths = euler_sampling.sample(times=TIMES, watch_params=watch_params, **kw).detach().cpu().numpy()
    paths_no_zero = euler_sampling.sample(times=TIMES[1:], **kw).cpu().numpy()
    expected_means = 0.1 + (2.0 / 3.0) * MU * np.power(TIMES, 1.5)
    if use_batch:
        assert paths.shape == (2, num_samples, 6, 1)
        means = paths.mean(axis=1).reshape(2, 6)
        np.testing.assert_allclose(means, np.broadcast_to(expected_means, (2, 6)), rtol=1e-2, atol=1e-2)
        assert not np.array_equal(paths[0], paths[1])  # each batch entry has its own draws
    else:
        assert paths.shape == (num_samples, 6, 1)
        np.testing.assert_allclose(paths.mean(axis=0).reshape(-1), expected_means, rtol=1e-2, atol=1e-2)
    np.testing.assert_array_equal(paths[..., 1:, :], paths_no_zero)


@pytest.mark.parametrize("rt", ["SOBOL", "HALTON"])
def test_batched_quasi_random_draws_are_the_flattened_sample(cuda, rt):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    N, nb, d = 1024, 3, 2
    corr = np.linalg.cholesky(np.array([[1.0, 0.5], [0.5, 1.0]]))
    L = torch.from_numpy(corr).to(cuda)
    drift = lambda t, x: 0.03 * x  # noqa: E731
    vol = lambda t, x: (0.25 * x)[..., None] * L  # noqa: E731
    kw = dict(times=[0.5, 1.0], num_time_steps=8, random_type=getattr(RandomType, rt), seed=3,
              dtype=torch.float64)
    batched = euler_sampling.sample(d, drift, vol, num_samples=N, initial_state=np.ones((nb, 1, d)), **kw)
    flat = euler_sampling.sample(d, drift, vol, num_samples=nb * N, initial_state=np.ones(d), **kw)
    assert batched.shape == (nb, N, 2, d)
    np.testing.assert_array_equal(batched.reshape(nb * N, 2, d).cpu().numpy(), flat.cpu().numpy())


def test_batched_antithetic_partners_within_each_entry(cuda):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    N = 512
    paths = euler_sampling.sample(1, lambda t, x: torch.zeros_like(x), lambda t, x: 0.3 * torch.ones_like(x)[..., None],
                                  [0.5, 1.0], num_time_steps=6, num_samples=N, initial_state=np.zeros((2, 1, 1)),
                                  random_type=RandomType.STATELESS_ANTITHETIC, seed=[7, 9],
                                  dtype=torch.float64).cpu().numpy()
    assert paths.shape == (2, N, 2, 1)
    np.testing.assert_array_equal(paths[:, : N // 2], -paths[:, N // 2:])
    assert not np.array_equal(paths[0], paths[1])
    with pytest.raises(ValueError):
        euler_sampling.sample(1, lambda t, x: torch.zeros_like(x), lambda t, x: torch.ones_like(x)[..., None],
                              [1.0], num_time_steps=2, num_samples=N + 1, initial_state=np.zeros((2, 1, 1)),
                              random_type=RandomType.STATELESS_ANTITHETIC, seed=[7, 9], dtype=torch.float64)
