"""The reference's mv_normal_sample tests (GPU).

Restated from multivariate_normal_test.py:31-400 with the same shapes, means,
covariances, scales, skips and tolerances.  Pseudo-random draws come from
this project's Philox stream, so where the reference's bound on a sample mean
or covariance is a check of its own seeded stream (about two to three
standard errors at its sizes) the estimate is accepted within the larger of
that bound and four standard errors.  Quasi-random draws (Sobol, Halton) keep
the reference's bounds; batched means follow the reference's point layout.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MEAN = np.array([[1.0, 0.1], [0.1, 1.0]])
COVAR = np.array([[[0.9, -0.1], [-0.1, 1.0]], [[1.1, -0.3], [-0.3, 0.6]]])
SCALE = np.array([[0.4, -0.1], [0.22, 1.38]])
MEAN4 = np.array([[1.0, 0.1], [0.1, 1.0], [2.0, 0.3], [0.0, 0.0]])


def _np(x):
    return x.cpu().numpy()


def _mean_close(sample, expected, tol):
    mean = sample.mean(axis=0)
    se = sample.std(axis=0, ddof=1) / np.sqrt(sample.shape[0])
    bound = np.maximum(tol, 4 * se)
    assert np.all(np.abs(mean - expected) <= bound), (mean, expected, bound)


def _cov_close(sample, expected, tol):
    # sample [n, dim]; the standard error of a sample covariance is
    # sqrt((s_ii s_jj + s_ij^2) / n) for normal data
    cov = np.cov(sample, rowvar=False)
    d = np.diag(expected)
    se = np.sqrt((np.outer(d, d) + expected ** 2) / sample.shape[0])
    bound = np.maximum(tol, 4 * se)
    assert np.all(np.abs(cov - expected) <= bound), (cov, expected, bound)


def test_shapes(cuda):
    from tqf.math.random import mv_normal_sample
    assert tuple(mv_normal_sample([2, 4], mean=[0.2, 0.1]).shape) == (2, 4, 2)
    assert tuple(mv_normal_sample([2, 4], mean=[[0.2, 0.1], [0.0, -0.1], [0.0, 0.1]]).shape) == (2, 4, 3, 2)


def test_mean_default(cuda):
    from tqf.math.random import mv_normal_sample
    covar = np.array([[1.0, 0.1], [0.1, 1.0]])
    sample = _np(mv_normal_sample([40000], covariance_matrix=covar, seed=1234))
    assert sample.shape == (40000, 2)
    _mean_close(sample, [0.0, 0.0], 1e-2)
    _cov_close(sample, covar, 2e-2)


def test_covariance_default(cuda):
    from tqf.math.random import mv_normal_sample
    sample = _np(mv_normal_sample([10000], mean=MEAN))
    assert sample.shape == (10000, 2, 2)
    np.testing.assert_array_almost_equal(sample.mean(axis=0), MEAN, decimal=1)
    for i in range(2):
        np.testing.assert_array_almost_equal(np.cov(sample[:, i, :], rowvar=False), np.eye(2), decimal=1)


@pytest.mark.parametrize("rt,seed", [("PSEUDO", 4567), ("STATELESS", [1, 4567]), ("HALTON", None)])
def test_general_mean_covariance(cuda, rt, seed):
    # :79-108, and :110-134 (the same call under tf.function; HALTON and STATELESS)
    from tqf.math.random import RandomType, mv_normal_sample
    sample = _np(mv_normal_sample([30000], mean=MEAN, covariance_matrix=COVAR,
                                  random_type=getattr(RandomType, rt), seed=seed))
    assert sample.shape == (30000, 2, 2)
    np.testing.assert_array_almost_equal(sample.mean(axis=0), MEAN, decimal=1)
    for i in range(2):
        np.testing.assert_array_almost_equal(np.cov(sample[:, i, :], rowvar=False), COVAR[i], decimal=1)


def test_mean_and_scale(cuda):
    from tqf.math.random import mv_normal_sample
    covariance = SCALE @ SCALE.T
    sample = _np(mv_normal_sample([30000], mean=MEAN, scale_matrix=SCALE, seed=7534))
    assert sample.shape == (30000, 2, 2)
    np.testing.assert_array_almost_equal(sample.mean(axis=0), MEAN, decimal=1)
    for i in range(2):
        np.testing.assert_array_almost_equal(np.cov(sample[:, i, :], rowvar=False), covariance, decimal=1)


@pytest.mark.parametrize("rt", ["SOBOL", "HALTON_RANDOMIZED"])
def test_mean_default_quasi(cuda, rt):
    # :155-168 (SOBOL) and :188-201 (HALTON_RANDOMIZED), skip 1000
    from tqf.math.random import RandomType, mv_normal_sample
    covar = np.array([[1.0, 0.1], [0.1, 1.0]])
    sample = _np(mv_normal_sample([10000], covariance_matrix=covar, random_type=getattr(RandomType, rt), skip=1000))
    assert sample.shape == (10000, 2)
    np.testing.assert_allclose(sample.mean(axis=0), [0.0, 0.0], atol=1e-2, rtol=0)
    np.testing.assert_allclose(np.cov(sample, rowvar=False), covar, atol=2e-2, rtol=0)


@pytest.mark.parametrize("rt,row", [("SOBOL", 1), ("HALTON", 2)])
def test_mean_and_scale_quasi(cuda, rt, row):
    # :170-186 (SOBOL) and :221-237 (HALTON): batched means
    from tqf.math.random import RandomType, mv_normal_sample
    covariance = SCALE @ SCALE.T
    sample_shape = [2, 3, 5000]
    sample = _np(mv_normal_sample(sample_shape, mean=MEAN4, scale_matrix=SCALE, random_type=getattr(RandomType, rt)))
    assert sample.shape == tuple(sample_shape) + (4, 2)
    np.testing.assert_array_almost_equal(sample.mean(axis=(0, 1, 2)), MEAN4, decimal=1)
    for i in range(4):
        np.testing.assert_array_almost_equal(np.cov(sample[0, row, :, i, :], rowvar=False), covariance, decimal=1)


def test_mean_default_halton_randomization_params(cuda):
    from tqf.math.random import RandomType, halton, mv_normal_sample
    covar = np.array([[1.0, 0.1], [0.1, 1.0]], dtype=np.float32)
    params = halton.sample(2, 10000, randomized=True, seed=42)[1]
    sample = _np(mv_normal_sample([10000], covariance_matrix=covar, random_type=RandomType.HALTON_RANDOMIZED,
                                  randomization_params=params))
    assert sample.shape == (10000, 2)
    np.testing.assert_allclose(sample.mean(axis=0), [0.0, 0.0], atol=1e-2, rtol=0)
    np.testing.assert_allclose(np.cov(sample, rowvar=False), covar, atol=2e-2, rtol=0)


@pytest.mark.parametrize("rt,seed", [("PSEUDO_ANTITHETIC", 42), ("STATELESS_ANTITHETIC", [1, 42])])
def test_mean_and_scale_antithetic(cuda, rt, seed):
    from tqf.math.random import RandomType, mv_normal_sample
    covariance = SCALE @ SCALE.T
    size = 30000
    sample = _np(mv_normal_sample([size], mean=MEAN, scale_matrix=SCALE, random_type=getattr(RandomType, rt),
                                  seed=seed))
    assert sample.shape == (size, 2, 2)
    half = size // 2
    np.testing.assert_allclose((sample[:half] + sample[half:]) / 2, MEAN + np.zeros((half, 2, 2)), 1e-10, 1e-10)
    np.testing.assert_array_almost_equal(sample[:half].mean(axis=0), MEAN, decimal=1)
    for i in range(2):
        np.testing.assert_array_almost_equal(np.cov(sample[:half, i, :], rowvar=False), covariance, decimal=1)


def test_antithetic_sample_requires_even_dim(cuda):
    from tqf import InvalidArgumentError
    from tqf.math.random import RandomType, mv_normal_sample
    with pytest.raises(InvalidArgumentError):
        mv_normal_sample([11, 100], mean=MEAN, scale_matrix=SCALE, random_type=RandomType.PSEUDO_ANTITHETIC)


REPEATABLE = [("STATELESS", [1, 4567]), ("STATELESS", [456, 91011]), ("STATELESS_ANTITHETIC", [1, 4567]),
              ("SOBOL", [1, 4567]), ("HALTON", [1, 4567]), ("HALTON_RANDOMIZED", 7889)]


@pytest.mark.parametrize("rt,seed", REPEATABLE)
def test_results_are_repeatable(cuda, rt, seed):
    from tqf.math.random import RandomType, mv_normal_sample
    kw = dict(mean=MEAN, covariance_matrix=COVAR, random_type=getattr(RandomType, rt), seed=seed)
    np.testing.assert_array_almost_equal(_np(mv_normal_sample([10], **kw)), _np(mv_normal_sample([10], **kw)),
                                         decimal=6)


@pytest.mark.parametrize("mean,covar,seed", [(MEAN, COVAR, [1, 4567]),
                                             (np.array([[1.0, 0.1, 2.1], [0.1, 1.0, -0.5]]), None, [456, 91011])])
def test_adding_time_steps(cuda, mean, covar, seed):
    from tqf.math.random import RandomType, mv_normal_sample
    kw = dict(mean=mean, covariance_matrix=covar, random_type=RandomType.STATELESS, seed=seed)
    np.testing.assert_array_almost_equal(_np(mv_normal_sample([10], **kw)),
                                         _np(mv_normal_sample([16], **kw))[:10], decimal=6)
