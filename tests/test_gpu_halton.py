"""Halton sequence on the GPU against the oracle restatement of halton_impl.py
and the reference's property tests (halton_test.py)."""

import numpy as np
import pytest

from oracle import halton as ohalton

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 1e-6), (np.float64, 1e-13)])
def test_unscrambled_matches_oracle(cuda, dtype, rtol):
    from tqf.math.random import halton
    dim, n = 40, 3000
    got, params = halton.sample(dim, num_results=n, randomized=False, dtype=dtype)
    assert params is None
    np.testing.assert_allclose(got.cpu().numpy(), ohalton.sample(dim, np.arange(n), dtype), rtol=rtol, atol=1e-30)
    idx = np.array([0, 7, 123456, 2 ** 20 + 5])
    got, _ = halton.sample(dim, sequence_indices=idx, randomized=False, dtype=dtype)
    np.testing.assert_allclose(got.cpu().numpy(), ohalton.sample(dim, idx, dtype), rtol=rtol)
    small, _ = halton.sample(2, num_results=5, randomized=False)
    np.testing.assert_allclose(small.cpu().numpy(), [[1 / 2, 1 / 3], [1 / 4, 2 / 3], [3 / 4, 1 / 9],
                                                     [1 / 8, 4 / 9], [5 / 8, 7 / 9]], rtol=1e-6)


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 1e-6), (np.float64, 1e-13)])
def test_scrambled_matches_oracle_with_same_params(cuda, dtype, rtol):
    from tqf.math.random import halton
    dim, n = 25, 2000
    got, params = halton.sample(dim, num_results=n, seed=1925, dtype=dtype)
    perms = params.perms.cpu().numpy()
    want = ohalton.sample(dim, np.arange(n), dtype, perms=perms, zero_correction=params.zero_correction.cpu().numpy())
    np.testing.assert_allclose(got.cpu().numpy(), want, rtol=rtol)
    # every (digit position, axis) block is a permutation of 0..p-1
    p = ohalton.primes(dim)
    radix_sum = int(p.sum())
    off = np.concatenate([[0], np.cumsum(p[:-1])])
    nc = ohalton.NUM_COEFFS[np.dtype(dtype)]
    for k in (0, nc // 2, nc - 1):
        for d in (0, 3, dim - 1):
            blk = perms[k * radix_sum + off[d]: k * radix_sum + off[d] + p[d]]
            assert sorted(blk.tolist()) == list(range(p[d]))
    u = got.cpu().numpy()
    assert u.min() >= 0 and u.max() < 1


def test_reference_properties(cuda):
    """halton_test.py:205-307: seed determinism, index independence of the
    randomization, batches, reused params, params without randomization."""
    from tqf.math.random import halton
    a, _ = halton.sample(20, num_results=100, seed=1925)
    b, _ = halton.sample(20, num_results=100, seed=1925)
    np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    s1, _ = halton.sample(2, sequence_indices=[0], seed=9427)
    s2, _ = halton.sample(2, sequence_indices=[0, 1000], seed=9427)
    np.testing.assert_allclose(s1.cpu().numpy(), s2.cpu().numpy()[:1], rtol=1e-6)
    full, _ = halton.sample(2, 3, seed=1925)
    parts = [halton.sample(2, sequence_indices=[i], seed=1925)[0].cpu().numpy()[0] for i in range(3)]
    assert set(map(tuple, full.cpu().numpy())) == set(map(tuple, parts))
    s1, params = halton.sample(20, num_results=100, seed=1925)
    s2, _ = halton.sample(20, num_results=100, seed=62278, randomization_params=params)
    np.testing.assert_array_equal(s1.cpu().numpy(), s2.cpu().numpy())
    plain, _ = halton.sample(20, num_results=100, randomized=False)
    withp, _ = halton.sample(20, num_results=100, randomized=False, randomization_params=params)
    np.testing.assert_array_equal(plain.cpu().numpy(), withp.cpu().numpy())
    from tqf import InvalidArgumentError
    with pytest.raises(InvalidArgumentError):
        halton.sample(1, sequence_indices=[2 ** 30], dtype=np.float32, randomized=False, validate_args=True)
    with pytest.raises(InvalidArgumentError):
        halton.sample(1001, num_results=10, randomized=False, validate_args=True)
    with pytest.raises(ValueError):
        halton.sample(2)


def test_integral_and_draws(cuda):
    """Docstring integral (halton_impl.py:100-125) with scrambled points, and
    HALTON / HALTON_RANDOMIZED draws driving the samplers."""
    from tqf.math.random import RandomType, halton
    from tqf.models import coefficients as coef
    from tqf.models import euler_sampling
    dim = 3
    pts, _ = halton.sample(dim, num_results=20000, seed=127, dtype=np.float64)
    powers = np.arange(1.0, dim + 1)
    est = np.mean(np.prod(pts.cpu().numpy() ** powers, axis=-1))
    np.testing.assert_allclose(est, 1.0 / np.prod(powers + 1), rtol=1e-2)
    drift, vol = coef.gbm([0.05], [0.2])
    for rt, seed in [(RandomType.HALTON, None), (RandomType.HALTON_RANDOMIZED, 42)]:
        x = euler_sampling.sample(1, drift, vol, times=[1.0], num_time_steps=20, num_samples=20000,
                                  initial_state=[1.0], random_type=rt, seed=seed, dtype=np.float64).cpu().numpy()
        np.testing.assert_allclose(x[:, -1, 0].mean(), np.exp(0.05), rtol=5e-3)
