"""Hull-White short-rate paths on the GPU: exact transition against the
oracle restatement of vector_hull_white.py, the reference's analytic-moment
tests (hull_white_test.py) and its bond-price known values."""

import json
import os

import numpy as np
import pytest
import torch

from oracle import hull_white as ohw

pytestmark = pytest.mark.gpu


def _golden():
    with open(os.path.join(os.path.dirname(__file__), "golden", "hw_golden.json")) as f:
        return json.load(f)


def flat(t):
    return 0.01 * torch.ones_like(t)


def flat2(t):
    return 0.01 * torch.ones(tuple(t.shape) + (2,), dtype=t.dtype)


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 2e-5), (np.float64, 1e-12)])
def test_exact_paths_match_oracle(cuda, dtype, rtol):
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models.hull_white import HullWhiteModel1F, VectorHullWhiteModel
    rng = np.random.default_rng(0)
    # 1-d, piecewise-constant volatility with jumps at 0.1 and 2.0
    vol = PiecewiseConstantFunc([0.1, 2.0], [0.01, 0.02, 0.01], dtype=dtype)
    m = HullWhiteModel1F(0.1, vol, flat, dtype=dtype)
    times = np.array([0.1, 1.0, 2.0, 3.0], dtype)
    all_times, _ = ohw.grid(times, [[0.1, 2.0]], dtype)
    draws = rng.standard_normal((3000, len(all_times) - 1, 1)).astype(dtype)
    got = m.sample_paths(times, normal_draws=draws).cpu().numpy()
    p = ohw.Params(1, [([], [0.1])], [([0.1, 2.0], [0.01, 0.02, 0.01])], dtype)
    want = ohw.sample_with_draws(p, times, [[0.1, 2.0]], lambda t: np.array([0.01], dtype), draws.transpose(1, 0, 2),
                                 dtype=dtype)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-2)
    # 2-d, constant parameters, correlated
    corr = np.array([[1.0, 0.5], [0.5, 1.0]])
    m2 = VectorHullWhiteModel(2, [0.1, 0.05], [0.01, 0.02], flat2, corr_matrix=corr, dtype=dtype)
    times = np.array([0.5, 1.0], dtype)
    draws = rng.standard_normal((2000, 2, 2)).astype(dtype)
    got = m2.sample_paths(times, normal_draws=draws).cpu().numpy()
    p2 = ohw.Params(2, [([], [0.1]), ([], [0.05])], [([], [0.01]), ([], [0.02])], dtype)
    want = ohw.sample_with_draws(p2, times, [], lambda t: np.array([0.01, 0.01], dtype), draws.transpose(1, 0, 2),
                                 corr=corr, dtype=dtype)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-2)


def test_bond_price_known_values(cuda):
    from tqf.models.hull_white import HullWhiteModel1F
    g = _golden()
    m = HullWhiteModel1F(g["mean_reversion"][0], g["volatility"][0], flat, dtype=np.float64)
    b = g["bond"]
    got = m.discount_bond_price(b["short_rate"], b["times"], b["maturities"]).cpu().numpy()
    assert got.shape == (2, 1)
    np.testing.assert_allclose(got.ravel(), b["expected"], atol=b["atol"], rtol=b["rtol"])


def _true_mean(t, a, s, x0=0.01):
    a, s = np.asarray(a), np.asarray(s)
    return 0.01 + s * s / 2 / a ** 2 * (1 - np.exp(-a * t)) ** 2 - 0.01 * np.exp(-a * t) + x0 * np.exp(-a * t)


def _true_var(t, a, s):
    a, s = np.asarray(a), np.asarray(s)
    return s * s / 2 / a * (1 - np.exp(-2 * a * t))


@pytest.mark.parametrize("random_type,seed,dtype", [("STATELESS_ANTITHETIC", [1, 2], np.float32),
                                                     ("HALTON", None, np.float64)])
def test_mean_and_variance_1d(cuda, random_type, seed, dtype):
    """hull_white_test.py:100-138 (rtol = atol = 1e-4)."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hull_white import HullWhiteModel1F
    mr = PiecewiseConstantFunc([], [0.1], dtype=dtype)
    vol = PiecewiseConstantFunc([0.1, 2.0], [0.01, 0.01, 0.01], dtype=dtype)
    m = HullWhiteModel1F(mr, vol, flat, dtype=dtype)
    paths = m.sample_paths([0.1, 0.5, 1.0], num_samples=50000, random_type=getattr(RandomType, random_type),
                           seed=seed, skip=1000000)
    assert paths.dtype == torch.from_numpy(np.zeros(1, dtype)).dtype and tuple(paths.shape) == (50000, 3, 1)
    x = paths.cpu().numpy()[:, -1, :].astype(np.float64)
    np.testing.assert_allclose(x.mean(0), [_true_mean(1.0, 0.1, 0.01)], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(x.var(0), [_true_var(1.0, 0.1, 0.01)], rtol=1e-4, atol=1e-4)


def test_time_dependent_std_and_correlation(cuda):
    """hull_white_test.py:188-214 and :223-270: time-dependent volatility std,
    2-d mean / variance / correlation."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hull_white import HullWhiteModel1F, VectorHullWhiteModel
    vol = PiecewiseConstantFunc([0.1, 2.0], [0.01, 0.02, 0.01], dtype=np.float64)
    m = HullWhiteModel1F(0.1, vol, flat, dtype=np.float64)
    times = np.array([0.1, 1.0, 2.0, 3.0])
    p = m.sample_paths(times, num_samples=500000, random_type=RandomType.STATELESS_ANTITHETIC, seed=[4, 2],
                       skip=1000000).cpu().numpy()
    k, iv, vv = 0.1, np.array([0.0, 0.1, 2.0]), np.array([0.01, 0.02, 0.01])
    want = []
    for tt in times:
        var = 0.0
        for j in range(len(iv)):
            hi = iv[j + 1] if j + 1 < len(iv) else np.inf
            lo = iv[j]
            if tt <= lo:
                break
            up = min(tt, hi)
            var += vv[j] ** 2 / 2 / k * (np.exp(2 * k * up) - np.exp(2 * k * lo))
        want.append(np.exp(-k * tt) * np.sqrt(var))
    np.testing.assert_allclose(p[:, :, 0].std(0), want, rtol=1e-4, atol=1e-4)
    corr = [[1.0, 0.5], [0.5, 1.0]]
    m2 = VectorHullWhiteModel(2, [0.1, 0.05], [0.01, 0.02], flat2, corr_matrix=corr, dtype=np.float64)
    x = m2.sample_paths([0.1, 0.5, 1.0], num_samples=100000, random_type=RandomType.STATELESS_ANTITHETIC,
                        seed=[1, 2]).cpu().numpy()[:, -1, :]
    np.testing.assert_allclose(x.mean(0), _true_mean(1.0, [0.1, 0.05], [0.01, 0.02]), rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(x.var(0), _true_var(1.0, [0.1, 0.05], [0.01, 0.02]), rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(np.corrcoef(x.T), corr, rtol=1e-2, atol=1e-2)


def test_generic_path_time_dependent_mean_reversion(cuda):
    """A callable mean reversion takes the Euler route (time_step required)."""
    from tqf.math.random import RandomType
    from tqf.models.hull_white import HullWhiteModel1F
    mr = lambda t: 0.1 * torch.ones(1, dtype=torch.as_tensor(t).dtype)  # noqa: E731
    m = HullWhiteModel1F(mr, 0.01, flat, dtype=np.float64)
    with pytest.raises(ValueError):
        m.sample_paths([1.0], num_samples=10)
    x = m.sample_paths([0.5, 1.0], num_samples=100000, time_step=0.01, random_type=RandomType.STATELESS_ANTITHETIC,
                       seed=[3, 4]).cpu().numpy()[:, -1, 0]
    np.testing.assert_allclose(x.mean(), _true_mean(1.0, 0.1, 0.01), rtol=1e-3, atol=1e-4)
