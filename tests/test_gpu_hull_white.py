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


@pytest.mark.parametrize("jumps", [[[0.1, 2.0], [0.5, 1.0]], [[0.1, 2.0], [0.1, 2.0]]])
@pytest.mark.parametrize("dtype,rtol", [(np.float32, 2e-5), (np.float64, 1e-12)])
def test_per_axis_volatility_jumps_match_oracle(cuda, dtype, rtol, jumps):
    """Volatility with jump locations per axis ([dim, n], values [dim, n + 1];
    vector_hull_white.py:92-93, 156-198): the per-axis knots of the exact
    transition integrals and the time grid with every axis' jumps merged
    (duplicates kept, :1004-1014) against the oracle."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models.hull_white import VectorHullWhiteModel
    rng = np.random.default_rng(7)
    vals = [[0.01, 0.02, 0.01], [0.01, 0.015, 0.03]]
    vol = PiecewiseConstantFunc(jumps, vals, dtype=dtype)
    corr = np.array([[1.0, 0.1], [0.1, 1.0]])
    m = VectorHullWhiteModel(2, [0.03, 0.02], vol, flat2, corr_matrix=corr, dtype=dtype)
    times = np.array([0.25, 0.75, 1.5, 2.5], dtype)
    all_times, _ = ohw.grid(times, jumps, dtype)
    draws = rng.standard_normal((2000, len(all_times) - 1, 2)).astype(dtype)
    got = m.sample_paths(times, normal_draws=draws).cpu().numpy()
    p = ohw.Params(2, [([], [0.03]), ([], [0.02])], [(jumps[0], vals[0]), (jumps[1], vals[1])], dtype)
    want = ohw.sample_with_draws(p, times, jumps, lambda t: np.array([0.01, 0.01], dtype), draws.transpose(1, 0, 2),
                                 corr=corr, dtype=dtype)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-2)


def test_mean_variance_correlation_piecewise_2d(cuda):
    """hull_white_test.py:223-270: volatility with per-axis jumps
    [[0.1, 0.2, 0.5], [0.1, 2, 3]] (constant values), 50,000 antithetic
    paths; terminal mean and variance within 1e-4, correlation within 1e-2."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hull_white import VectorHullWhiteModel
    vol = PiecewiseConstantFunc([[0.1, 0.2, 0.5], [0.1, 2.0, 3.0]], values=[4 * [0.01], 4 * [0.02]],
                                dtype=np.float64)
    corr = [[1.0, 0.5], [0.5, 1.0]]
    m = VectorHullWhiteModel(2, [0.1, 0.05], vol, flat2, corr_matrix=corr, dtype=np.float64)
    paths = m.sample_paths([0.1, 0.5, 1.0], num_samples=50000, random_type=RandomType.STATELESS_ANTITHETIC,
                           seed=[1, 2])
    assert paths.dtype == torch.float64 and tuple(paths.shape) == (50000, 3, 2)
    x = paths.cpu().numpy()[:, -1, :]
    np.testing.assert_allclose(x.mean(0), _true_mean(1.0, [0.1, 0.05], [0.01, 0.02]), rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(x.var(0), _true_var(1.0, [0.1, 0.05], [0.01, 0.02]), rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(np.corrcoef(x[:, 0], x[:, 1]), corr, rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("supply_draws,supply_grid", [(False, False), (True, False), (True, True)])
def test_mean_variance_correlation_piecewise_constant_2d(cuda, supply_draws, supply_grid):
    """hull_white_test.py:272-342: per-axis volatility jumps 2 x [[0.2, 1]],
    piecewise correlation with jumps [0.5, 2]; generated draws, supplied
    antithetic draws ([N, 9, 2]: the grid holds 0, the three times and all
    six jumps), and supplied draws on a supplied grid ([N, 4, 2]).  The
    supplied normals are seeded torch draws standing in for TensorFlow's
    stateless normals."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hull_white import VectorHullWhiteModel
    vol = PiecewiseConstantFunc(2 * [[0.2, 1.0]], values=np.array(3 * [[0.01, 0.02]]).transpose(), dtype=np.float64)
    want_corr = [[1.0, 0.5], [0.5, 1.0]]
    corr = PiecewiseConstantFunc([0.5, 2.0], values=[want_corr, [[1.0, 0.6], [0.6, 1.0]], [[1.0, 0.9], [0.9, 1.0]]],
                                 dtype=np.float64)
    m = VectorHullWhiteModel(2, [0.1, 0.05], vol, flat2, corr_matrix=corr, dtype=np.float64)
    n = 100000
    draws, grid = None, None
    g = torch.Generator().manual_seed(42)
    if supply_draws:
        steps = 4 if supply_grid else 9
        half = torch.randn(n // 2, steps, 2, dtype=torch.float64, generator=g)
        draws = torch.cat([half, -half], 0).numpy()
    if supply_grid:
        grid = [0.0, 0.1, 0.2, 0.5, 1.0]
    paths = m.sample_paths([0.1, 0.5, 1.0], num_samples=1 if supply_draws else n,
                           random_type=RandomType.STATELESS_ANTITHETIC, seed=[4, 2], normal_draws=draws,
                           times_grid=grid)
    assert paths.dtype == torch.float64 and tuple(paths.shape) == (n, 3, 2)
    p = paths.cpu().numpy()
    np.testing.assert_allclose(np.corrcoef(p[:, 1, 0], p[:, 1, 1]), want_corr, rtol=1e-2, atol=1e-2)
    x = p[:, -1, :]
    np.testing.assert_allclose(x.mean(0), _true_mean(1.0, [0.1, 0.05], [0.01, 0.02]), rtol=1e-3, atol=1e-3)
    np.testing.assert_allclose(x.var(0), _true_var(1.0, [0.1, 0.05], [0.01, 0.02]), rtol=1e-3, atol=1e-3)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_mean_variance_correlation_generic_2d(cuda, dtype):
    """hull_white_test.py:344-386: mean reversion with per-axis jumps
    (Euler route), per-axis volatility jumps, a callable correlation
    [[1, t/2], [t/2, 1]] evaluated at scalar times; 50,000 Sobol paths
    (skip 100,000, time step 0.01); mean and variance within 1e-3."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hull_white import VectorHullWhiteModel
    mr = PiecewiseConstantFunc(2 * [[0.1, 2.0]], values=[3 * [0.1], 3 * [0.1]], dtype=dtype)
    vol = PiecewiseConstantFunc([[0.1, 0.2, 0.5], [0.1, 2.0, 3.0]], values=[4 * [0.01], 4 * [0.02]], dtype=dtype)

    def corr_matrix(t):
        one = torch.ones_like(t)
        row1 = torch.stack([one, 0.5 * t], -1)
        row2 = torch.flip(row1, [0])
        return torch.stack([row1, row2], -1)

    m = VectorHullWhiteModel(2, mr, vol, flat2, corr_matrix=corr_matrix, dtype=dtype)
    assert m._generic
    paths = m.sample_paths([0.1, 0.5], num_samples=50000, random_type=RandomType.SOBOL, skip=100000, time_step=0.01)
    assert paths.dtype == torch.from_numpy(np.zeros(1, dtype)).dtype and tuple(paths.shape) == (50000, 2, 2)
    x = paths.cpu().numpy()[:, -1, :].astype(np.float64)
    np.testing.assert_allclose(x.mean(0), _true_mean(0.5, [0.1, 0.1], [0.01, 0.02]), rtol=1e-3, atol=1e-3)
    np.testing.assert_allclose(x.var(0), _true_var(0.5, [0.1, 0.1], [0.01, 0.02]), rtol=1e-3, atol=1e-3)


def test_per_axis_reference_example(cuda):
    """The reference's class example (vector_hull_white.py:84-115): volatility
    jumps [[0.1, 2], [0.1, 2]], constant correlation, a constant curve given
    as a list, 10,000 Sobol paths.  Terminal means against the model's
    analytic mean f(0, 1) + int_0^1 e^{-a(1-s)} y(s) ds,
    y(s) = int_0^s e^{-2a(s-u)} sigma(u)^2 du, within 2e-5 (a tenth of a
    pseudo-random standard error)."""
    from scipy import integrate
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hull_white import VectorHullWhiteModel
    vol = PiecewiseConstantFunc(jump_locations=[[0.1, 2.0], [0.1, 2.0]],
                                values=[[0.01, 0.02, 0.01], [0.01, 0.015, 0.01]], dtype=np.float64)
    m = VectorHullWhiteModel(2, [0.03, 0.02], vol, lambda *args: [0.01, 0.015],
                             corr_matrix=[[1.0, 0.1], [0.1, 1.0]], dtype=np.float64)
    paths = m.sample_paths(np.linspace(0.0, 1.0, 10), num_samples=10000, random_type=RandomType.SOBOL, seed=[4, 2])
    assert tuple(paths.shape) == (10000, 10, 2)

    def mean(a, s0, s1, f):
        sig = lambda u: s0 if u <= 0.1 else s1  # noqa: E731
        y = lambda s: integrate.quad(lambda u: np.exp(-2 * a * (s - u)) * sig(u) ** 2, 0, s,  # noqa: E731
                                     points=[0.1] if s > 0.1 else None)[0]
        return f + integrate.quad(lambda s: np.exp(-a * (1 - s)) * y(s), 0, 1, points=[0.1])[0]

    want = [mean(0.03, 0.01, 0.02, 0.01), mean(0.02, 0.01, 0.015, 0.015)]
    np.testing.assert_allclose(paths[:, -1, :].mean(0).cpu().numpy(), want, rtol=0, atol=2e-5)
