"""Quasi-random draws in the fused pricers (GPU).

random_type SOBOL / HALTON* in the pricing calls generates the reference's
normal draws (generate_mc_normal_draws: dimension step * d + component, point
index skip + 1 + path) on the device and prices with them; the result must
equal pricing with the same draws passed as normal_draws, and differ from the
Philox stream.
"""

import numpy as np
import pytest
import torch

from oracle import closed_form

pytestmark = pytest.mark.gpu

HESTON = dict(expiry=1.0, spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7,
              discount_rate=0.02)


@pytest.mark.parametrize("scheme", ["full_truncation", "qe"])
@pytest.mark.parametrize("rt", ["SOBOL", "HALTON"])
def test_heston_pricing_quasi_random_equals_supplied_draws(cuda, scheme, rt):
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import heston_european_mc
    random_type = getattr(RandomType, rt)
    N, steps = 1 << 14, 32
    strikes = np.array([90.0, 100.0, 110.0])
    kw = dict(strikes=strikes, num_samples=N, num_time_steps=steps, scheme=scheme, **HESTON)
    q = heston_european_mc(random_type=random_type, seed=7, **kw)
    draws = utils.generate_mc_normal_draws(2, steps, N, random_type, seed=7, dtype=torch.float32)
    ref = heston_european_mc(normal_draws=draws.permute(1, 0, 2), **kw)
    np.testing.assert_array_equal(q.price.cpu().numpy(), ref.price.cpu().numpy())
    ph = heston_european_mc(random_type=RandomType.STATELESS, seed=[7, 7], **kw)
    assert not np.array_equal(q.price.cpu().numpy(), ph.price.cpu().numpy())


def test_heston_sobol_price_near_semi_analytic(cuda):
    from tqf.math.random import RandomType
    from tqf.pricing import heston_european_mc
    res = heston_european_mc(strikes=np.array([100.0]), num_samples=1 << 16, num_time_steps=64,
                             random_type=RandomType.SOBOL, **HESTON)
    ref = closed_form.heston_price(spot=100.0, strike=100.0, expiry=1.0, rate=0.02, v0=0.04, kappa=2.0,
                                   theta=0.04, xi=0.3, rho=-0.7)
    # 0.05 covers the full-truncation discretisation bias at 64 steps and the
    # quasi-random integration error of 2^16 points in dimension 128
    assert abs(float(res.price[0]) - ref) < 0.05, (float(res.price[0]), ref)


def test_heston_adjoint_sobol_equals_supplied_draws(cuda):
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import heston_european_mc, heston_european_vjp
    N, steps = 1 << 13, 16
    kw = dict(strikes=np.array([95.0, 105.0]), num_samples=N, num_time_steps=steps, **HESTON)
    base = heston_european_mc(random_type=RandomType.SOBOL, **kw)
    g = heston_european_vjp(np.ones(2), prices=base.price, random_type=RandomType.SOBOL, **kw).cpu().numpy()
    draws = utils.generate_mc_normal_draws(2, steps, N, RandomType.SOBOL, dtype=torch.float32)
    g_ref = heston_european_vjp(np.ones(2), prices=base.price, normal_draws=draws.permute(1, 0, 2),
                                **kw).cpu().numpy()
    np.testing.assert_array_equal(g, g_ref)


def test_basket_sobol_equals_supplied_draws(cuda):
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import basket_european_mc
    d, N, steps = 4, 1 << 13, 8
    corr = 0.5 * np.eye(d) + 0.5
    kw = dict(spots=np.full(d, 100.0), vols=np.linspace(0.1, 0.4, d), rate=0.02, corr=corr, strike=100.0,
              expiry=1.0, num_time_steps=steps, num_samples=N, dtype=torch.float32)
    q = basket_european_mc(random_type=RandomType.SOBOL, **kw)
    draws = utils.generate_mc_normal_draws(d, steps, N, RandomType.SOBOL, dtype=torch.float32)
    ref = basket_european_mc(normal_draws=draws.permute(1, 0, 2), **kw)
    assert q.price == ref.price
    np.testing.assert_array_equal(np.asarray(q.delta.cpu()), np.asarray(ref.delta.cpu()))
