"""Path kernels against the oracle given identical draws (GPU).

Tolerances: float64 paths within 1e-12 relative; float32 within 1e-5
relative (|a - b| <= 1e-5 (|b| + scale), scale = the magnitude of that state
component) — the bar the reference's own float arithmetic sets.
"""

import numpy as np
import pytest
import torch

from oracle import closed_form, euler as oeuler, grids as ogrids, heston as oheston

pytestmark = pytest.mark.gpu


def _close(got, want, rtol, scale):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    err = np.abs(got - want) / (np.abs(want) + scale)
    assert np.all(np.isfinite(got)) and float(err.max()) <= rtol, float(err.max())


def test_gbm_euler_float64_config(cuda):
    """65,536 paths, 100 steps dt=0.01, f64, normal_draws from seed 42."""
    from tqf.models import coefficients, euler_sampling
    from tqf.pricing import european_payoff_stats
    mu, sigma, x0, N = 0.05, 0.2, 100.0, 65536
    draws = np.random.default_rng(42).standard_normal((N, 100, 1))
    drift, vol = coefficients.gbm([mu], [sigma])
    times = np.array([1.0])
    paths = euler_sampling.sample(1, drift, vol, times, time_step=0.01, initial_state=np.array([x0]),
                                  normal_draws=draws, dtype=torch.float64)
    assert paths.shape == (N, 1, 1) and paths.dtype == torch.float64
    all_t, keep, _ = ogrids.prepare_grid(times, 0.01, np.float64)
    want = oeuler.sample_with_draws(lambda t, x: mu * x, lambda t, x: (sigma * x)[..., None],
                                    all_t, keep, 1, np.full((N, 1), x0), draws.transpose(1, 0, 2), np.float64)
    _close(paths.cpu().numpy(), want, 1e-12, 0.0)
    res = european_payoff_stats(paths[:, -1, 0], [100.0], discount=np.exp(-0.05))
    bs = closed_form.black_scholes(100.0, 100.0, 0.05, 0.2, 1.0)
    assert abs(float(res.price[0]) - bs) < 3 * float(res.standard_error[0]) + 0.02


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_generic_callables_match_structured_and_oracle(cuda, dtype):
    from tqf.models import coefficients, euler_sampling
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    N, d = 3000, 3
    rng = np.random.default_rng(0)
    corr = np.array([[1.0, 0.3, 0.1], [0.3, 1.0, -0.2], [0.1, -0.2, 1.0]])
    drift, vol = coefficients.gbm([0.02, 0.05, -0.01], [0.2, 0.3, 0.25], corr)
    times = np.array([0.25, 0.5, 1.0], dtype=np_dt)
    draws = rng.standard_normal((N, 20, d)).astype(np_dt)
    x0 = np.array([1.0, 2.0, 0.5], dtype=np_dt)
    a = euler_sampling.sample(d, drift, vol, times, num_time_steps=20, initial_state=x0, normal_draws=draws)
    g = euler_sampling.sample(d, lambda t, x: drift(t, x), lambda t, x: vol(t, x), times, num_time_steps=20,
                              initial_state=x0, normal_draws=draws)
    all_t, keep, _ = ogrids.prepare_grid(times, times[-1] / np_dt(20), np_dt, num_time_steps=20)
    L = np.linalg.cholesky(corr).astype(np_dt)
    want = oeuler.sample_with_draws(lambda t, x: (x * np.array([0.02, 0.05, -0.01], np_dt)).astype(np_dt),
                                    lambda t, x: ((x * np.array([0.2, 0.3, 0.25], np_dt))[..., None] * L).astype(np_dt),
                                    all_t, keep, 3, np.broadcast_to(x0, (N, d)), draws.transpose(1, 0, 2), np_dt)
    rtol = 1e-5 if dtype == torch.float32 else 1e-12
    assert a.shape == (N, 3, d)
    _close(a.cpu().numpy(), want, rtol, 1.0)
    _close(g.cpu().numpy(), want, rtol, 1.0)


def test_euler_pseudo_random_wiener_statistics(cuda):
    # euler_sampling_test.py:31-133: Wiener process mean 0, cov min(s, t).
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    drift = lambda t, x: torch.zeros_like(x)  # noqa: E731
    vol = lambda t, x: torch.ones(x.shape + (1,), dtype=x.dtype, device=x.device)  # noqa: E731
    times = np.array([0.1, 0.5, 1.0])
    for rt, seed in [(RandomType.PSEUDO, 42), (RandomType.STATELESS, [1, 2]),
                     (RandomType.PSEUDO_ANTITHETIC, 3), (RandomType.SOBOL, None)]:
        p = euler_sampling.sample(1, drift, vol, times, time_step=0.01, num_samples=20000,
                                  random_type=rt, seed=seed, dtype=torch.float64)[..., 0].cpu().numpy()
        np.testing.assert_allclose(p.mean(0), 0.0, atol=2e-2)
        np.testing.assert_allclose(np.cov(p.T), np.minimum.outer(times, times), rtol=3e-2, atol=3e-2)


def test_fused_philox_equals_materialised_draws(cuda):
    from tqf.math.random import RandomType
    from tqf.models import coefficients, euler_sampling, utils
    drift, vol = coefficients.gbm([0.05, 0.01], [0.2, 0.3], [[1, 0.4], [0.4, 1]])
    kw = dict(times=np.array([0.5, 1.0], np.float32), num_time_steps=50, initial_state=np.array([100.0, 50.0], np.float32))
    fused = euler_sampling.sample(2, drift, vol, num_samples=4096, random_type=RandomType.STATELESS, seed=[9, 9], **kw)
    draws = utils.generate_mc_normal_draws(2, 50, 4096, RandomType.STATELESS, seed=[9, 9], dtype=torch.float32)
    mat = euler_sampling.sample(2, drift, vol, normal_draws=draws.permute(1, 0, 2), **kw)
    torch.testing.assert_close(fused, mat, rtol=0, atol=0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_heston_full_truncation_euler_matches_oracle(cuda, dtype):
    """Full truncation max(v, 0) then sqrt amplifies a last-ulp difference in
    v into sqrt(ulp) when v crosses zero; paths whose oracle variance came
    within `kink` of zero are flagged and excluded (and must be rare)."""
    from tqf.models import coefficients, euler_sampling
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    N, steps = 4096, 60
    r, kappa, theta, xi, rho = 0.02, 2.0, 0.04, 0.4, -0.7   # Feller violated: v hits the truncation
    drift, vol = coefficients.heston_full_truncation(r, kappa, theta, xi, rho)
    draws = np.random.default_rng(1).standard_normal((N, steps, 2)).astype(np_dt)
    times = np.array([0.3, 1.0], dtype=np_dt)
    x0 = np.array([np.log(100.0), 0.04], dtype=np_dt)
    got = euler_sampling.sample(2, drift, vol, times, num_time_steps=steps, initial_state=x0, normal_draws=draws)
    all_t, keep, _ = ogrids.prepare_grid(times, times[-1] / np_dt(steps), np_dt, num_time_steps=steps)
    fd, fv = oeuler.heston_ft_coefficients(r, kappa, theta, xi, rho, np_dt)
    min_abs_v = np.full(N, np.inf)
    min_v = np.full(N, np.inf)

    def fd_monitor(t, x):
        np.minimum(min_abs_v, np.abs(x[..., 1]), out=min_abs_v)
        np.minimum(min_v, x[..., 1], out=min_v)
        return fd(t, x)

    want = oeuler.sample_with_draws(fd_monitor, fv, all_t, keep, 2, np.broadcast_to(x0, (N, 2)),
                                    draws.transpose(1, 0, 2), np_dt)
    kink = 1e-4 if dtype == torch.float32 else 1e-12
    ok = min_abs_v > kink
    assert ok.mean() > 0.85
    assert (min_v < 0).sum() > 0  # the truncation is exercised
    rtol = 1e-5 if dtype == torch.float32 else 1e-12
    g = got.cpu().numpy()
    _close(g[ok][..., 0], want[ok][..., 0], rtol, 1.0)
    _close(g[ok][..., 1], want[ok][..., 1], rtol, 0.04)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("grid", ["num_steps", "time_step", "times_grid"])
def test_heston_qe_matches_oracle(cuda, dtype, grid):
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import HestonModel
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    kappa = PiecewiseConstantFunc([0.3], [1.5, 2.5], dtype=np_dt)
    model = HestonModel(kappa, 0.04, 0.6, -0.7, dtype=np_dt)
    times = np.array([0.5, 1.0], dtype=np_dt)
    kw = {"num_steps": dict(num_time_steps=50), "time_step": dict(time_step=0.02),
          "times_grid": dict(times_grid=np.linspace(0.0, 1.0, 51).astype(np_dt))}[grid]
    if grid == "num_steps":
        ts = times[-1] / np_dt(50)
        all_t, keep = ogrids.heston_prepare_grid(times, ts, np_dt, jump_locations=[[0.3]], num_time_steps=50)
    elif grid == "time_step":
        all_t, keep = ogrids.heston_prepare_grid(times, 0.02, np_dt, jump_locations=[[0.3]])
    else:
        all_t, keep = ogrids.heston_prepare_grid(times, None, np_dt, times_grid=kw["times_grid"])
    steps = len(all_t) - 1
    N = 4096
    draws = np.random.default_rng(2).standard_normal((N, steps, 2)).astype(np_dt)
    x0 = np.array([np.log(100.0), 0.04], dtype=np_dt)
    got = model.sample_paths(times, x0, normal_draws=draws, **kw).cpu().numpy()
    want, near = oheston.qe_sample_with_draws(((0.3,), (1.5, 2.5)), 0.04, 0.6, -0.7, all_t, keep, 2, x0[0], x0[1],
                                              draws.transpose(1, 0, 2), np_dt, near=1e-4)
    assert got.shape == (N, 2, 2)
    ok = ~near
    assert ok.mean() > 0.97
    rtol = 1e-5 if dtype == torch.float32 else 1e-12
    _close(got[ok][..., 0], want[ok][..., 0], rtol, 1.0)
    _close(got[ok][..., 1], want[ok][..., 1], rtol, 0.04)


def test_heston_qe_price_vs_semi_analytic(cuda):
    # heston_model_test.py:290-383 configuration (MC vs semi-analytic, 0.1 tolerance)
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.math.random import RandomType
    from tqf.models import HestonModel
    k = PiecewiseConstantFunc([0.1, 0.2], [0.3, 0.3, 0.3], dtype=np.float64)
    model = HestonModel(k, 0.05, 0.02, 0.1, dtype=np.float64)
    samples = model.sample_paths(times=[0.5, 1.0], initial_state=np.array([3.0, 0.05]), time_step=0.01,
                                 num_samples=10000, random_type=RandomType.STATELESS_ANTITHETIC, seed=[1, 42])
    assert samples.shape == (10000, 2, 2)
    log_spots = samples[:, -1, 0].cpu().numpy()
    mc = np.exp(-0.5) * np.mean(np.maximum(np.exp(log_spots) * np.exp(0.5) - 15, 0))
    ref = closed_form.heston_price(spot=np.exp(3.0), strike=15, expiry=1.0, rate=0.5, v0=0.05, kappa=0.3,
                                   theta=0.05, xi=0.02, rho=0.1)
    np.testing.assert_allclose(mc, ref, atol=0.1, rtol=0.1)


@pytest.mark.parametrize("scheme", ["full_truncation", "qe"])
def test_fused_pricing_equals_stored_paths(cuda, scheme):
    """Fused payoff sums == payoff statistics of the same paths stored."""
    from tqf.math.random import RandomType
    from tqf.models import HestonModel, coefficients, euler_sampling, utils
    from tqf.pricing import european_payoff_stats, heston_european_mc
    N, steps, T = 50000, 64, 1.0
    strikes = np.linspace(70, 130, 64)
    kw = dict(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7)
    res = heston_european_mc(strikes=strikes, expiry=T, discount_rate=0.02, num_samples=N, num_time_steps=steps,
                             scheme=scheme, random_type=RandomType.STATELESS, seed=[4, 5], **kw)
    times = np.array([T], np.float32)
    x0 = np.array([np.log(100.0), 0.04], np.float32)
    if scheme == "full_truncation":
        drift, vol = coefficients.heston_full_truncation(0.02, 2.0, 0.04, 0.3, -0.7)
        paths = euler_sampling.sample(2, drift, vol, times, times_grid=np.linspace(0, T, steps + 1).astype(np.float32),
                                      initial_state=x0, num_samples=N, random_type=RandomType.STATELESS, seed=[4, 5])
        scale = 1.0
    else:
        paths = HestonModel(2.0, 0.04, 0.3, -0.7).sample_paths(
            times, x0, num_samples=N, random_type=RandomType.STATELESS, seed=[4, 5],
            times_grid=np.linspace(0, T, steps + 1).astype(np.float32))
        scale = float(np.exp(0.02 * T))
    stored = european_payoff_stats(paths[:, -1, 0], strikes, discount=float(np.exp(-0.02 * T)), log_values=True,
                                   spot_scale=scale)
    torch.testing.assert_close(res.price, stored.price, rtol=1e-6, atol=1e-9)
    torch.testing.assert_close(res.standard_error, stored.standard_error, rtol=1e-5, atol=1e-9)
    ref = np.array([closed_form.heston_price(spot=100.0, strike=k, expiry=T, rate=0.02, v0=0.04, kappa=2.0,
                                             theta=0.04, xi=0.3, rho=-0.7) for k in strikes])
    err = np.abs(res.price.cpu().numpy() - ref) / res.standard_error.cpu().numpy()
    assert np.median(err) < 3.0


def test_fused_pricing_deterministic_and_sharded(cuda):
    from tqf.math.random import RandomType
    from tqf.pricing import heston_european_mc
    kw = dict(strikes=np.linspace(80, 120, 16), expiry=1.0, spot=100.0, variance=0.04, mean_reversion=2.0,
              theta=0.04, volvol=0.3, rho=-0.7, discount_rate=0.02, num_time_steps=32,
              random_type=RandomType.STATELESS, seed=[7, 7])
    a = heston_european_mc(num_samples=100000, **kw)
    b = heston_european_mc(num_samples=100000, **kw)
    torch.testing.assert_close(a.sums, b.sums, rtol=0, atol=0)
    # Two shards of 50,000 paths (path_offset) add up to the whole run.
    s0 = heston_european_mc(num_samples=50000, path_offset=0, **kw)
    s1 = heston_european_mc(num_samples=50000, path_offset=50000, **kw)
    # Payoffs are summed in float32 within 64-path tiles and in float64 across
    # tiles; tile membership depends on the launch shape, so shards agree with
    # the whole run to float32 tile-rounding (~1e-8 relative).
    torch.testing.assert_close(s0.sums + s1.sums, a.sums, rtol=1e-6, atol=1e-6)
