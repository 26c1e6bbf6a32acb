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


def _sobol_ref_draws(steps, N, skip, dtype):
    """Materialised SOBOL normals [steps, N, 2] (generate_mc_normal_draws)."""
    from tqf.math.random import RandomType
    from tqf.models import utils
    return utils.generate_mc_normal_draws(2, steps, N, RandomType.SOBOL, skip=skip, dtype=dtype)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("N,steps,skip", [(100, 5, 0), (3000, 150, 77), (70_000, 70, 2 ** 20 + 5)])
def test_heston_sample_paths_fused_sobol_equals_materialised(cuda, dtype, N, steps, skip):
    """HestonModel.sample_paths with SOBOL computes the normals inside the QE
    kernel (per-window shared tables, point index skip + 1 + n split into
    low bits and 256-blocks).  Paths must equal those from the materialised
    draws of generate_mc_normal_draws bit for bit: nd below 8 (N = 100),
    several windows with a ragged last one (150 steps), tiles that straddle
    two 256-blocks of point indices (skip = 77, 2^20 + 5) and a ragged last
    tile."""
    from tqf.math.random import RandomType
    from tqf.models import HestonModel
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    model = HestonModel(2.0, 0.04, 0.3, -0.7, dtype=np_dt)
    times = np.array([0.25, 0.5, 1.0], np_dt)
    x0 = np.array([np.log(100.0), 0.04], np_dt)
    fused = model.sample_paths(times, x0, num_samples=N, random_type=RandomType.SOBOL, num_time_steps=steps,
                               skip=skip)
    draws = _sobol_ref_draws(steps + len(times) + 1, N, skip, dtype)
    ref = model.sample_paths(times, x0, num_time_steps=steps, normal_draws=draws.permute(1, 0, 2))
    np.testing.assert_array_equal(fused.cpu().numpy(), ref.cpu().numpy())


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_heston_full_truncation_fused_sobol_every_step_equals_materialised(cuda, dtype):
    """The full-truncation kernel with in-kernel Sobol draws and every step
    recorded (staged stores, several Sobol windows) against the same kernel
    reading the materialised draws: equal bit for bit."""
    import math

    import tqf._lib as L
    from tqf.math.random import multivariate_normal as mvn
    from tqf.models import heston_model, utils
    from tqf.models.coefficients import HestonFullTruncation
    N, steps, skip = 5000, 130, 3
    npt = np.float32 if dtype == torch.float32 else np.float64
    t = np.linspace(0.0, 1.0, steps + 1).astype(npt)
    dt = (t[1:] - t[:-1]).astype(npt)
    rows = heston_model.full_truncation_table(HestonFullTruncation(0.02, 2.0, 0.04, 0.3, -0.7), t, dt,
                                              np.sqrt(dt).astype(npt), np.arange(steps, dtype=np.int32), steps)
    table = utils.step_table(rows, dtype, cuda)

    def run(draws):
        out = torch.full((N, steps, 2), float("nan"), dtype=dtype, device=cuda)
        a = L.HestonArgs()
        a.dtype = L.TQF_F32 if dtype == torch.float32 else L.TQF_F64
        a.num_steps, a.num_paths = steps, N
        a.step_table = table.data_ptr()
        a.x0, a.v0 = math.log(100.0), 0.04
        a.draws = draws
        a.output.ptr = out.data_ptr()
        a.output.num_slots = steps
        a.output.init_slot = -1
        a.dev_status = L.status_buffer(cuda).data_ptr()
        L.call("tqf_heston_euler", a, L.stream_ptr())
        L.check_device_status(cuda)
        return out.cpu().numpy()

    sob, keep = mvn.sobol_draws(2, steps, N, skip, cuda)
    mat = _sobol_ref_draws(steps, N, skip, dtype)
    np.testing.assert_array_equal(run(sob), run(mvn.memory_draws(mat, path_axis=1, step_axis=0)))


def test_heston_pricing_fused_sobol_large_matches_materialised(cuda):
    """The headline workload's Sobol variant at 2^20 paths x 252 steps
    (dimension 504): fused prices equal the materialised-draws prices to the
    float64 summation order (the two kernels' persistent grids can differ)."""
    from tqf.math.random import RandomType
    from tqf.pricing import heston_european_mc
    N, steps = 1 << 20, 252
    kw = dict(strikes=np.linspace(70.0, 130.0, 64), num_samples=N, num_time_steps=steps, **HESTON)
    q = heston_european_mc(random_type=RandomType.SOBOL, **kw)
    ref = heston_european_mc(normal_draws=_sobol_ref_draws(steps, N, 0, torch.float32).permute(1, 0, 2), **kw)
    np.testing.assert_allclose(q.price.cpu().numpy(), ref.price.cpu().numpy(), rtol=1e-9, atol=1e-12)


def test_fused_sobol_rejects_bad_requests(cuda):
    import math

    import tqf._lib as L
    from tqf.math.random import multivariate_normal as mvn
    from tqf.models import heston_model, utils
    from tqf.models.coefficients import HestonFullTruncation
    steps, N = 4, 1000
    t = np.linspace(0.0, 1.0, steps + 1).astype(np.float32)
    dt = (t[1:] - t[:-1]).astype(np.float32)
    rows = heston_model.full_truncation_table(HestonFullTruncation(0.02, 2.0, 0.04, 0.3, -0.7), t, dt,
                                              np.sqrt(dt).astype(np.float32), np.full(steps, -1, np.int32), steps)
    table = utils.step_table(rows, torch.float32, cuda)
    d, keep = mvn.sobol_draws(2, steps, N, 0, cuda)
    out = torch.empty((N, 1, 2), device=cuda)
    for field, bad in [("key1", 3), ("key0", 5), ("antithetic", 1)]:
        a = L.HestonArgs()
        a.dtype, a.num_steps, a.num_paths = L.TQF_F32, steps, N
        a.step_table = table.data_ptr()
        a.x0, a.v0 = math.log(100.0), 0.04
        a.draws = d
        setattr(a.draws, field, bad)
        a.output.ptr, a.output.num_slots, a.output.init_slot = out.data_ptr(), 1, -1
        with pytest.raises(ValueError):
            L.call("tqf_heston_euler", a, L.stream_ptr())
