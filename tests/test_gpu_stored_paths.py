"""Stored paths through the coalescing output stagers, against the oracle
given identical draws (GPU).

The path kernels stage recorded states in shared memory and write them out
as whole pieces of each path's output row once a path's row is long enough
(Heston: always; Euler, GBM, Milstein, Hull-White, Gaussian HJM: at least
64 bytes per path).  These cases record many times so that every stager runs several full
flushes and a partial one, with path counts that leave the last CTA round
partly empty, and compare every stored state with the oracle.  Tolerances are
those of the other path tests: 1e-5 relative in float32 and 1e-12 in float64.
"""

import numpy as np
import pytest
import torch

from oracle import euler as oeuler
from oracle import grids as ogrids
from oracle import heston as oheston
from oracle import hjm as ohjm
from oracle import hull_white as ohw
from oracle import milstein as omil
from oracle import mvgbm as omvgbm

pytestmark = pytest.mark.gpu

DTYPES = [(np.float32, 1e-5), (np.float64, 1e-12)]


def _close(got, want, rtol, scale):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    assert got.shape == want.shape, (got.shape, want.shape)
    err = np.abs(got - want) / (np.abs(want) + scale)
    assert np.all(np.isfinite(got)) and float(err.max()) <= rtol, float(err.max())


@pytest.mark.parametrize("dtype,rtol", DTYPES)
@pytest.mark.parametrize("d", [1, 2, 3, 5])
def test_euler_every_step_recorded(cuda, dtype, rtol, d):
    from tqf.models import coefficients, euler_sampling
    N, steps = 1000, 60  # 1000 = 3 x 256 + 232: the last round is partly empty
    rng = np.random.default_rng(d)
    mu = rng.uniform(-0.05, 0.05, d)
    sig = rng.uniform(0.1, 0.3, d)
    corr = 0.6 * np.eye(d) + 0.4
    drift, vol = coefficients.gbm(mu, sig, corr)
    times = (np.arange(0, steps + 1) / steps).astype(dtype)  # t = 0 too: the initial slot
    # the grid merges the requested times with the uniform one (ulp-apart
    # points stay distinct), so the draws are sized from it
    all_t, keep, _ = ogrids.prepare_grid(times, times[-1] / dtype(steps), dtype, num_time_steps=steps)
    draws = rng.standard_normal((N, len(all_t) - 1, d)).astype(dtype)
    x0 = np.linspace(1.0, 2.0, d).astype(dtype)
    got = euler_sampling.sample(d, drift, vol, times, num_time_steps=steps, initial_state=x0,
                                normal_draws=draws).cpu().numpy()
    L = np.linalg.cholesky(corr).astype(dtype)
    want = oeuler.sample_with_draws(lambda t, x: (x * mu.astype(dtype)).astype(dtype),
                                    lambda t, x: ((x * sig.astype(dtype))[..., None] * L).astype(dtype),
                                    all_t, keep, len(times), np.broadcast_to(x0, (N, d)), draws.transpose(1, 0, 2),
                                    dtype)
    assert got.shape == (N, len(times), d)
    _close(got, want, rtol, 1.0)


def test_heston_every_step_recorded_with_duplicate_time(cuda):
    """QE and full-truncation Heston paths with every grid time recorded and
    one requested time repeated (the Heston grid keeps it, so one output slot
    is written twice and the staged run restarts there)."""
    import tqf
    N, steps = 777, 48
    model = tqf.models.HestonModel(2.0, 0.04, 0.3, -0.7)
    x0 = np.array([np.log(100.0), 0.04], np.float32)
    times = np.concatenate([np.arange(1, steps + 1) / steps, [0.5]]).astype(np.float32)
    times.sort()
    all_t, keep = ogrids.heston_prepare_grid(times, times[-1] / np.float32(steps), np.float32,
                                             num_time_steps=steps)
    draws = np.random.default_rng(5).standard_normal((N, len(all_t) - 1, 2)).astype(np.float32)
    got = model.sample_paths(times, x0, num_time_steps=steps, normal_draws=draws).cpu().numpy()
    want, near = oheston.qe_sample_with_draws(2.0, 0.04, 0.3, -0.7, all_t, keep, len(times), x0[0], x0[1],
                                              draws.transpose(1, 0, 2), np.float32, near=1e-4)
    assert got.shape == want.shape == (N, len(times), 2)
    ok = ~near
    err = np.abs(got[ok] - want[ok]) / (np.abs(want[ok]) + np.array([1.0, 0.04]))
    assert err.max() < 1e-5, err.max()
    # full truncation through the Euler sampler (the fused Heston kernel)
    drift, vol = tqf.models.coefficients.heston_full_truncation(0.02, 2.0, 0.04, 0.3, -0.7)
    ft_times = (np.arange(1, steps + 1) / steps).astype(np.float32)
    all_t2, keep2, _ = ogrids.prepare_grid(ft_times, ft_times[-1] / np.float32(steps), np.float32,
                                           num_time_steps=steps)
    d2 = np.ascontiguousarray(draws[:, :len(all_t2) - 1])
    p2 = tqf.models.euler_sampling.sample(2, drift, vol, ft_times, num_time_steps=steps, initial_state=x0,
                                          normal_draws=d2).cpu().numpy()
    fd, fv = oeuler.heston_ft_coefficients(0.02, 2.0, 0.04, 0.3, -0.7, np.float32)
    want2 = oeuler.sample_with_draws(fd, fv, all_t2, keep2, len(ft_times), np.broadcast_to(x0, (N, 2)),
                                     d2.transpose(1, 0, 2), np.float32)
    err = np.abs(p2 - want2) / (np.abs(want2) + np.array([1.0, 0.04]))
    # paths whose variance touches the max(v, 0) kink amplify a last-ulp
    # difference; 99 % of paths must agree to 1e-5 at every recorded time
    assert np.quantile(err.max(axis=(1, 2)), 0.99) < 1e-5


@pytest.mark.parametrize("dtype,rtol", DTYPES)
@pytest.mark.parametrize("d", [1, 2, 5])
def test_gbm_every_date_recorded(cuda, dtype, rtol, d):
    from tqf.models import MultivariateGeometricBrownianMotion
    N, k = 1000, 40
    rng = np.random.default_rng(10 + d)
    vols = rng.uniform(0.1, 0.4, d)
    corr = 0.7 * np.eye(d) + 0.3
    times = (np.arange(1, k + 1) / k).astype(dtype)
    draws = rng.standard_normal((N, k, d)).astype(dtype)
    x0 = np.linspace(1.0, 2.0, d).astype(dtype)
    proc = MultivariateGeometricBrownianMotion(d, means=0.03, volatilities=vols, corr_matrix=corr, dtype=dtype)
    got = proc.sample_paths(times, initial_state=x0, normal_draws=draws).cpu().numpy()
    want = omvgbm.sample_with_draws(np.full(d, 0.03), vols, corr, times, x0, draws.transpose(1, 0, 2), dtype)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=0)


@pytest.mark.parametrize("dtype,rtol", DTYPES)
@pytest.mark.parametrize("dim", [1, 2])
def test_milstein_every_step_recorded(cuda, dtype, rtol, dim):
    from tqf.models import coefficients as coef
    from tqf.models import milstein_sampling
    from tqf.models import utils as mutils
    rng = np.random.default_rng(20 + dim)
    order = 5
    m = rng.uniform(-0.05, 0.05, dim)
    M = np.diag(rng.uniform(0.01, 0.1, dim))
    s0 = rng.uniform(0.0, 0.05, dim)
    s1 = rng.uniform(0.1, 0.3, dim)
    C = np.linalg.cholesky(0.5 * np.eye(dim) + 0.5) if dim > 1 else np.ones((1, 1))
    N, time_step = 300, 0.025  # 300 = 2 x 128 + 44
    times = np.arange(1, 41) * time_step
    all_times, keep, _ = mutils.prepare_grid(times=np.asarray(times, dtype), time_step=dtype(time_step),
                                             dtype=np.dtype(dtype))
    steps = len(all_times) - 1
    draws = rng.standard_normal((N, steps, dim + 3 * dim * order)).astype(dtype)
    x0 = np.linspace(1.0, 1.5, dim).astype(dtype)
    got = milstein_sampling.sample(dim=dim, drift_fn=coef.AffineDrift(m, M), volatility_fn=coef.ScaledVolatility(s0, s1, C),
                                   times=np.asarray(times, dtype), time_step=time_step, initial_state=x0,
                                   normal_draws=draws, dtype=dtype).cpu().numpy()
    dfn, vfn, gfn = omil.affine_coefficients(m, M, s0, s1, C, dtype)
    want = omil.sample_with_draws(dfn, vfn, gfn, all_times, keep, len(times), np.broadcast_to(x0, (N, dim)),
                                  draws.transpose(1, 0, 2), order, dtype)
    assert got.shape == (N, len(times), dim)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-3)


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 2e-5), (np.float64, 1e-12)])
def test_hull_white_every_time_recorded(cuda, dtype, rtol):
    from tqf.models.hull_white import HullWhiteModel1F

    def flat(t):
        return 0.01 * torch.ones_like(t)

    m = HullWhiteModel1F(0.1, 0.01, flat, dtype=dtype)
    times = (np.arange(1, 41) / 20).astype(dtype)  # 40 times to t = 2
    all_times, _ = ohw.grid(times, [], dtype)
    N = 1000
    draws = np.random.default_rng(7).standard_normal((N, len(all_times) - 1, 1)).astype(dtype)
    got = m.sample_paths(times, normal_draws=draws).cpu().numpy()
    p = ohw.Params(1, [([], [0.1])], [([], [0.01])], dtype)
    want = ohw.sample_with_draws(p, times, [], lambda t: np.array([0.01], dtype), draws.transpose(1, 0, 2),
                                 dtype=dtype)
    assert got.shape == (N, len(times), 1)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * 1e-2)


@pytest.mark.parametrize("dtype,rtol", [(np.float32, 2e-5), (np.float64, 1e-12)])
@pytest.mark.parametrize("dim", [1, 2])
def test_gaussian_hjm_every_time_recorded(cuda, dtype, rtol, dim):
    from tqf.models import utils
    from tqf.models.hjm import GaussianHJM
    mr = [0.03, 0.1][:dim]
    vol = [0.005, 0.012][:dim]
    corr = None if dim == 1 else [[1.0, 0.5], [0.5, 1.0]]
    m = GaussianHJM(dim, mr, vol, lambda *args: [0.01], corr_matrix=corr, dtype=dtype)
    times = (np.arange(1, 41) / 20).astype(dtype)  # 40 times to t = 2
    all_times, _, ti = utils.prepare_grid(times=times, time_step=dtype(0.05), dtype=np.dtype(dtype))
    N = 1000
    draws = np.random.default_rng(11).standard_normal((N, len(all_times) - 1, dim)).astype(dtype)
    rates, dfs, x, _ = m.sample_paths(times, N, time_step=0.05, normal_draws=draws)
    om = ohjm.Model(dim, mr, None, np.asarray(vol)[:, None], corr, dtype)
    wr, wd, wx = om.sample(all_times, ti, draws.transpose(1, 0, 2), lambda t: np.full(np.shape(t), 0.01, dtype))
    assert tuple(rates.shape) == (N, len(times)) and tuple(x.shape) == (N, len(times), dim)
    np.testing.assert_allclose(rates.cpu().numpy(), wr, rtol=rtol, atol=rtol * 1e-2)
    np.testing.assert_allclose(dfs.cpu().numpy(), wd, rtol=rtol)
    np.testing.assert_allclose(x.cpu().numpy(), wx, rtol=rtol, atol=rtol * 1e-2)


@pytest.mark.parametrize("dtype,rtol", DTYPES)
@pytest.mark.parametrize("d", [1, 2, 4])
def test_euler_warp_rows_every_step(cuda, dtype, rtol, d):
    """Every grid time recorded (times = times_grid, t = 0 included): the
    kernel gathers 32-word pieces of 32 paths' rows per warp and writes each
    path's piece with one store instruction (72 words per path for d = 1 in
    float32: 2 full pieces and a partial one; pieces end inside a step for
    d = 4 in float32 and every float64 case); 1000 paths leave the last warp
    with 8 paths."""
    from tqf.models import coefficients, euler_sampling
    N, steps = 1000, 71
    rng = np.random.default_rng(20 + d)
    mu = rng.uniform(-0.05, 0.05, d)
    sig = rng.uniform(0.1, 0.3, d)
    corr = 0.6 * np.eye(d) + 0.4
    drift, vol = coefficients.gbm(mu, sig, corr)
    grid = np.linspace(0.0, 1.0, steps + 1).astype(dtype)
    draws = rng.standard_normal((N, steps, d)).astype(dtype)
    x0 = np.linspace(1.0, 2.0, d).astype(dtype)
    got = euler_sampling.sample(d, drift, vol, grid, times_grid=grid, initial_state=x0,
                                normal_draws=draws).cpu().numpy()
    all_t, keep, _ = ogrids.prepare_grid(grid, None, dtype, times_grid=grid)
    L = np.linalg.cholesky(corr).astype(dtype)
    want = oeuler.sample_with_draws(lambda t, x: (x * mu.astype(dtype)).astype(dtype),
                                    lambda t, x: ((x * sig.astype(dtype))[..., None] * L).astype(dtype),
                                    all_t, keep, len(grid), np.broadcast_to(x0, (N, d)), draws.transpose(1, 0, 2),
                                    dtype)
    assert got.shape == (N, steps + 1, d)
    _close(got, want, rtol, 1.0)


def test_heston_every_step_of_times_grid(cuda):
    """QE (HestonModel.sample_paths) and full truncation (euler_sampling with
    the Heston coefficients) with every step of a 72-step times_grid recorded
    (the every-step declaration is set; the Heston kernels keep their
    CTA-cooperative SlotStager), against the oracle."""
    import tqf
    N, steps = 1000, 72
    grid = np.linspace(0.0, 1.0, steps + 1).astype(np.float32)
    x0 = np.array([np.log(100.0), 0.04], np.float32)
    draws = np.random.default_rng(9).standard_normal((N, steps, 2)).astype(np.float32)
    model = tqf.models.HestonModel(2.0, 0.04, 0.3, -0.7)
    got = model.sample_paths(grid[1:], x0, times_grid=grid, normal_draws=draws).cpu().numpy()
    all_t, keep, _ = ogrids.prepare_grid(grid[1:], None, np.float32, times_grid=grid)
    want, near = oheston.qe_sample_with_draws(2.0, 0.04, 0.3, -0.7, all_t, keep, steps, x0[0], x0[1],
                                              draws.transpose(1, 0, 2), np.float32, near=1e-4)
    assert got.shape == want.shape == (N, steps, 2)
    ok = ~near
    err = np.abs(got[ok] - want[ok]) / (np.abs(want[ok]) + np.array([1.0, 0.04]))
    assert err.max() < 1e-5, err.max()
    drift, vol = tqf.models.coefficients.heston_full_truncation(0.02, 2.0, 0.04, 0.3, -0.7)
    p2 = tqf.models.euler_sampling.sample(2, drift, vol, grid[1:], times_grid=grid, initial_state=x0,
                                          normal_draws=draws).cpu().numpy()
    fd, fv = oeuler.heston_ft_coefficients(0.02, 2.0, 0.04, 0.3, -0.7, np.float32)
    want2 = oeuler.sample_with_draws(fd, fv, all_t, keep, steps, np.broadcast_to(x0, (N, 2)),
                                     draws.transpose(1, 0, 2), np.float32)
    err = np.abs(p2 - want2) / (np.abs(want2) + np.array([1.0, 0.04]))
    assert np.quantile(err.max(axis=(1, 2)), 0.99) < 1e-5


def test_every_step_declaration_is_checked(cuda):
    """A path kernel told that every step is recorded in order (the warp-row
    layout) verifies it on its step table: here one date records nothing, so
    the kernel writes no state and reports TQF_E_INVALID in the status word."""
    import tqf._lib as L
    from tqf.math.random import RandomType
    from tqf.math.random import multivariate_normal as mvn
    from tqf.models import utils
    k, N = 8, 300
    rows = np.zeros((k, 4))
    rows[:, 0] = 1.0 / k
    rows[:, 1] = np.sqrt(1.0 / k)
    rows[:, 2] = np.arange(k)
    rows[3, 2] = -1
    table = utils.step_table(rows, torch.float32, cuda)
    one = torch.ones(1, device=cuda)
    out = torch.full((N, k, 1), float("nan"), device=cuda)
    a = L.MvgbmArgs()
    a.dtype, a.dim, a.num_paths, a.num_steps = L.TQF_F32, 1, N, k
    a.step_table = table.data_ptr()
    a.x0 = a.drift = a.vol = one.data_ptr()
    a.chol = None
    a.draws = mvn.philox_draws(RandomType.STATELESS, [1, 2], N)
    a.output.ptr, a.output.num_slots, a.output.init_slot, a.output.every_step = out.data_ptr(), k, -1, 1
    a.dev_status = L.status_buffer(cuda).data_ptr()
    a.lz_mode = 1
    L.call("tqf_mvgbm_paths", a, L.stream_ptr())
    with pytest.raises(RuntimeError):
        L.check_device_status(cuda)
    assert bool(torch.isnan(out).all())
