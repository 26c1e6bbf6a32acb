"""Gaussian HJM on the GPU: Euler factor paths, short rates and discount
factors against the oracle restatement of gaussian_hjm.py, the reference's
statistical tests and its bond-price known values."""

import json
import os

import numpy as np
import pytest
import torch

from oracle import hjm as ohjm

pytestmark = pytest.mark.gpu

FLAT = lambda *args: [0.01]  # noqa: E731  (the reference tests' initial_discount_rate_fn)


def _golden():
    with open(os.path.join(os.path.dirname(__file__), "golden", "hjm_golden.json")) as f:
        return json.load(f)


def test_bond_prices_known_values(cuda):
    from tqf.models.hjm import GaussianHJM
    g = _golden()
    for c in g["cases"]:
        m = GaussianHJM(c["dim"], c["mr"], c["vol"], FLAT, dtype=np.float64)
        t = np.asarray(c["times"])
        got = m.discount_bond_price(g["state"] * np.ones((len(t), c["dim"])), t, t + g["maturity_offset"])
        assert tuple(got.shape) == t.shape
        np.testing.assert_allclose(got.cpu().numpy(), c["expected"], rtol=g["rtol"], atol=g["atol"])


CASES = [
    (1, [0.03], [0.01], None, None, None),
    (2, [0.03, 0.1], [0.005, 0.012], [[1.0, 0.5], [0.5, 1.0]], None, None),
    (2, [0.03, 0.1], None, None, [[0.5, 1.0], [0.5, 1.0]], [[0.005, 0.008, 0.005], [0.005, 0.008, 0.005]]),
]


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 2e-5), (np.float64, 1e-12)])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_paths_match_oracle(cuda, dtype, rtol, case):
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import utils
    from tqf.models.hjm import GaussianHJM
    dim, mr, vol, corr, jumps, values = CASES[case]
    volp = vol if jumps is None else PiecewiseConstantFunc(jumps, values, dtype=dtype)
    m = GaussianHJM(dim, mr, volp, FLAT, corr_matrix=corr, dtype=dtype)
    times = np.array([0.1, 0.5, 1.0, 2.0], dtype)
    all_times, _, ti = utils.prepare_grid(times=times, time_step=dtype(0.1), dtype=np.dtype(dtype))
    draws = np.random.default_rng(case).standard_normal((2000, len(all_times) - 1, dim)).astype(dtype)
    rates, dfs, x, y = m.sample_paths(times, 2000, time_step=0.1, normal_draws=draws)
    om = ohjm.Model(dim, mr, None if jumps is None else jumps[0],
                    np.asarray(vol)[:, None] if jumps is None else values, corr, dtype)
    wr, wd, wx = om.sample(all_times, ti, draws.transpose(1, 0, 2), lambda t: np.full(np.shape(t), 0.01, dtype))
    np.testing.assert_allclose(rates.cpu().numpy(), wr, rtol=rtol, atol=rtol * 1e-2)
    np.testing.assert_allclose(dfs.cpu().numpy(), wd, rtol=rtol)
    np.testing.assert_allclose(x.cpu().numpy(), wx, rtol=rtol, atol=rtol * 1e-2)
    assert tuple(y.shape) == (2000, 4, dim * dim)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_discount_factor_means(cuda, case):
    """E[D(t)] = exp(-0.01 t) within 1e-3 (gaussian_hjm_test.py:62-166)."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models.hjm import GaussianHJM
    dim, mr, vol, corr, jumps, values = CASES[case]
    volp = vol if jumps is None else PiecewiseConstantFunc(jumps, values, dtype=np.float64)
    m = GaussianHJM(dim, mr, volp, FLAT, corr_matrix=corr, dtype=np.float64)
    times = np.array([0.1, 0.5, 1.0, 2.0])
    rates, dfs, _, _ = m.sample_paths(times, 100000, time_step=0.1, random_type=RandomType.STATELESS_ANTITHETIC,
                                      seed=[1, 2], skip=1000000)
    assert tuple(rates.shape) == (100000, 4) and tuple(dfs.shape) == (100000, 4)
    np.testing.assert_allclose(dfs.cpu().numpy().mean(0), np.exp(-0.01 * times), rtol=1e-3, atol=1e-3)


@pytest.mark.parametrize("dim,corr,factor", [(1, None, 1.0), (2, None, np.sqrt(2.0)),
                                             (2, [[1.0, 0.5], [0.5, 1.0]], np.sqrt(3.0))])
def test_zero_coupon_bond_std(cuda, dim, corr, factor):
    """Std of log P(t, t + tau) against the closed form (gaussian_hjm_test.py:193-222)."""
    from tqf.math.random import RandomType
    from tqf.models.hjm import GaussianHJM
    m = GaussianHJM(dim, [0.03] * dim, [0.005] * dim, FLAT, corr_matrix=corr, dtype=np.float64)
    times = np.array([0.1, 0.5, 1.0, 2.0])
    curve = np.array([0.0, 0.5, 1.0, 2.0, 5.0])
    bonds, _, _ = m.sample_discount_curve_paths(times, curve, 100000, time_step=0.1,
                                                random_type=RandomType.STATELESS_ANTITHETIC, seed=[1, 2],
                                                skip=1000000)
    assert tuple(bonds.shape) == (100000, 5, 4)
    std = torch.log(bonds).std(0).cpu().numpy()
    for j, t in enumerate(times):
        tau = curve + t
        e_tau, et = np.exp(-0.03 * tau), np.exp(0.03 * t)
        true = 0.005 / 0.03 * (1.0 - e_tau * et) * np.sqrt((1.0 - 1.0 / et / et) / 0.03 / 2)
        np.testing.assert_allclose(std[:, j], factor * true, rtol=1e-3, atol=1e-3)
