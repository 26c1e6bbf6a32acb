"""Heston pathwise adjoint (replay kernel) against autograd and bump-and-revalue (GPU)."""

import numpy as np
import pytest
import torch

from oracle import heston_grad

pytestmark = pytest.mark.gpu

PARAMS = dict(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7, discount_rate=0.02)
ORDER = ("spot", "variance", "mean_reversion", "theta", "volvol", "rho", "discount_rate")


def test_adjoint_matches_autograd_restatement_on_same_draws(cuda):
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import heston_european_mc, heston_european_vjp
    N, steps = 20000, 32
    strikes = np.array([80.0, 95.0, 100.0, 110.0, 130.0])
    w = np.array([0.3, -1.0, 2.0, 0.5, 1.0])
    draws = utils.generate_mc_normal_draws(2, steps, N, RandomType.STATELESS, seed=[2, 3],
                                           dtype=torch.float64).permute(1, 0, 2).contiguous()
    kw = dict(strikes=strikes, expiry=1.0, num_samples=N, num_time_steps=steps, dtype=torch.float64,
              normal_draws=draws, **PARAMS)
    res = heston_european_mc(**kw)
    grad = heston_european_vjp(w, prices=res.price, **kw).cpu().numpy()
    p_ref, g_ref = heston_grad.price_and_grad([PARAMS[k] for k in ORDER], strikes, w, 1.0, draws.cpu().numpy())
    np.testing.assert_allclose(res.price.cpu().numpy(), p_ref, rtol=1e-10)
    np.testing.assert_allclose(grad, g_ref, rtol=1e-7, atol=1e-9)


def test_float32_adjoint_matches_float64_restatement(cuda):
    """The float32 replay (SFU square roots, float32 tangents) against the
    float64 autograd restatement on the same float32-rounded draws: within
    2e-3 relative (float32 path arithmetic over 32 steps, and the odd path
    whose payoff indicator flips at a strike)."""
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import heston_european_mc, heston_european_vjp
    N, steps = 20000, 32
    strikes = np.array([80.0, 95.0, 100.0, 110.0, 130.0])
    w = np.array([0.3, -1.0, 2.0, 0.5, 1.0])
    draws = utils.generate_mc_normal_draws(2, steps, N, RandomType.STATELESS, seed=[2, 3],
                                           dtype=torch.float32).permute(1, 0, 2).contiguous()
    kw = dict(strikes=strikes, expiry=1.0, num_samples=N, num_time_steps=steps, dtype=torch.float32,
              normal_draws=draws, **PARAMS)
    res = heston_european_mc(**kw)
    grad = heston_european_vjp(w, prices=res.price, **kw).cpu().numpy()
    _, g_ref = heston_grad.price_and_grad([PARAMS[k] for k in ORDER], strikes, w, 1.0,
                                          draws.cpu().numpy().astype(np.float64))
    np.testing.assert_allclose(grad, g_ref, rtol=2e-3, atol=1e-4 * float(np.abs(g_ref).max()))


SCALE = dict(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=0.7, discount_rate=0.02)


@pytest.mark.parametrize("volvol,N,steps,ns", [(0.1, 1 << 19, 64, 1), (0.3, 1 << 19, 64, 1),
                                               (0.3, 1 << 22, 252, 64)])
def test_adjoint_vs_common_random_number_bumps(cuda, volvol, N, steps, ns):
    """Pathwise Greeks vs central bump-and-revalue on the same Philox paths
    (float64), every sensitivity within 1e-4 (delta absolute, the rest
    relative to max(1, |bump|)), at volvol 0.1 and at the headline workload's
    volvol 0.3 (2^22 paths x 252 steps, 64 strikes summed).

    The pathwise derivative is the exact derivative of the discretised
    estimator on these paths, and central differences converge to it as the
    bump shrinks.  With volvol = 0.3 some paths' variance comes close to the
    full truncation max(v, 0), where sqrt(v+) has an unbounded slope: a bump
    of size h moves such a path's result by O(sqrt(h)) rather than O(h), so
    bumps of 1e-4 of the parameter's scale still differ from the pathwise
    value by up to ~1 % (theta, volvol), and the gap closes as h shrinks
    (1e-6: < 2e-4, 1e-7: < 2e-6 relative).  Bumps of 1e-7 of each
    parameter's scale in float64 keep the difference quotient's rounding
    (~1e-16 / 1e-7 of the price) far below the tolerance."""
    from tqf.math.random import RandomType
    from tqf.pricing import heston_european_mc, heston_european_vjp
    params = dict(PARAMS, volvol=volvol)
    kw = dict(strikes=np.linspace(70.0, 130.0, ns) if ns > 1 else np.array([100.0]), expiry=1.0,
              num_samples=N, num_time_steps=steps, dtype=torch.float64, random_type=RandomType.STATELESS,
              seed=[5, 6])
    base = heston_european_mc(**kw, **params)
    grad = heston_european_vjp(np.ones(ns), prices=base.price, **kw, **params).cpu().numpy()
    for i, name in enumerate(ORDER):
        h = 1e-7 * SCALE[name]
        up = dict(params)
        dn = dict(params)
        up[name] += h
        dn[name] -= h
        fd = (float(heston_european_mc(**kw, **up).price.sum()) - float(heston_european_mc(**kw, **dn).price.sum())) / (2 * h)
        tol = 1e-4 if name == "spot" else 1e-4 * max(1.0, abs(fd))
        assert abs(grad[i] - fd) < tol, (name, grad[i], fd)


def test_autograd_function_backward(cuda):
    from tqf.math.random import RandomType
    from tqf.pricing import HestonEuropeanPrice, heston_european_vjp
    kw = dict(strikes=np.array([90.0, 100.0, 110.0]), expiry=1.0, num_samples=1 << 16, num_time_steps=32,
              random_type=RandomType.STATELESS, seed=[9, 9], dtype=torch.float64)
    params = torch.tensor([PARAMS[k] for k in ORDER], dtype=torch.float64, requires_grad=True)
    prices = HestonEuropeanPrice.apply(params, kw)
    prices.sum().backward()
    want = heston_european_vjp(np.ones(3), prices=prices.detach(), **kw, **PARAMS).cpu().numpy()
    np.testing.assert_allclose(params.grad.numpy(), want, rtol=1e-12)
    assert params.grad[0] > 0  # calls: positive delta
