"""Host-side logic of the drop-in API against the oracle (CPU only)."""

import numpy as np
import pytest
import torch

from oracle import grids as ogrids


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("case", [
    dict(times=[1.0], time_step=0.01),
    dict(times=[0.1, 1.0, 2.0], time_step=0.01),
    dict(times=[0.3, 0.7, 1.0], time_step=0.1),
    dict(times=[0.5, 1.0], num_time_steps=100),
    dict(times=[1.0], num_time_steps=252),
    dict(times=list(np.linspace(1 / 52, 1, 52)), times_grid=np.linspace(0, 1, 253)),
    dict(times=[0.25, 0.5, 0.77], times_grid=np.linspace(0, 1, 11)),
])
def test_prepare_grid_matches_oracle(case, dtype):
    from tqf.models import utils
    times = np.asarray(case["times"], dtype=dtype)
    kw = dict(tolerance=None, num_time_steps=case.get("num_time_steps"), times_grid=case.get("times_grid"))
    step = case.get("time_step")
    if step is None and kw["num_time_steps"] is not None:
        step = times[-1] / dtype(kw["num_time_steps"])
    a = utils.prepare_grid(times=times, time_step=step, dtype=dtype, **kw)
    b = ogrids.prepare_grid(times, step, dtype, **kw)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("seed", range(60))
def test_output_slot_plan_matches_oracle(seed):
    """The vectorised slot plan against the oracle's replay of the
    reference's written_count loop: short and long grids, sparse to dense
    kept times, requests that end the loop early or leave slots unwritten."""
    from tqf.models import utils
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 30)) if seed < 30 else int(rng.integers(30, 700))
    keep = rng.random(n) < rng.choice([0.05, 0.3, 0.5, 1.0])
    k = max(int(keep.sum()), 1) + int(rng.integers(-1, 3))
    k = max(k, 1)
    init = int(rng.integers(0, 2))
    a = utils.plan_output_slots(keep, k, init)
    b = ogrids.write_slots(keep, k, init)
    np.testing.assert_array_equal(a[0], b[0])
    assert a[0].dtype == np.int32
    assert a[1:] == b[1:]


def test_heston_grid_matches_oracle():
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models.heston_model import HestonModel
    k = PiecewiseConstantFunc([0.1, 0.2], [0.3, 0.3, 0.3], dtype=np.float64)
    m = HestonModel(k, 0.05, 0.02, 0.1, dtype=np.float64)
    times = np.array([0.5, 1.0])
    a = m._prepare_grid(times, 0.01, None, None)
    b = ogrids.heston_prepare_grid(times, 0.01, np.float64, jump_locations=[[0.1, 0.2]])
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    m2 = HestonModel(2.0, 0.04, 0.3, -0.7)
    a = m2._prepare_grid(np.array([1.0], np.float32), np.float32(1.0) / np.float32(252), 252, None)
    b = ogrids.heston_prepare_grid(np.array([1.0], np.float32), np.float32(1.0) / np.float32(252), np.float32,
                                   num_time_steps=252)
    np.testing.assert_array_equal(a[0], b[0])
    assert len(a[0]) == 253


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_qe_step_table_rows(dtype):
    """The vectorised QE step table against the row formulas evaluated one
    step at a time (heston_model.py:522-572 constants; the skip flag for
    zero-length steps), on a Heston grid with duplicate times and
    piecewise-constant kappa and rho."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import utils
    from tqf.models.heston_model import HestonModel
    kappa = PiecewiseConstantFunc([0.3, 0.6], [1.5, 2.0, 2.5], dtype=dtype)
    rho = PiecewiseConstantFunc([0.5], [-0.7, -0.4], dtype=dtype)
    m = HestonModel(kappa, 0.04, 0.3, rho, dtype=dtype)
    times = np.array([0.25, 0.5, 1.0], dtype)
    all_times, keep = m._prepare_grid(times, dtype(1.0) / dtype(40), 40, None)
    step_slot, _, steps_exec, _ = utils.plan_output_slots(keep, len(times), 0)
    rows = m._qe_table(all_times, 1e-6, step_slot, steps_exec)
    dt, (K, TH, XI, RHO) = m._params_on_grid(all_times)
    assert rows.shape == (steps_exec, 12) and (rows[:, 0] == 1.0).sum() >= 2  # duplicate times skipped
    for i in range(steps_exec):
        h, k, th, xi, r = float(dt[i]), float(K[i]), float(TH[i]), float(XI[i]), float(RHO[i])
        E = float(dtype(np.exp(-k * h)))
        want = [0.0 if dtype(dt[i]) > dtype(1e-6) else 1.0, th, E, xi * xi * E * (1.0 - E) / k,
                th * xi * xi * (1.0 - E) ** 2 / (2.0 * k), -r * k * th / xi * h,
                0.5 * h * (k * r / xi - 0.5) - r / xi, 0.5 * h * (k * r / xi - 0.5) + r / xi,
                0.5 * h * (1.0 - r * r), 0.5 * h * (1.0 - r * r), 0.0, step_slot[i]]
        np.testing.assert_allclose(rows[i], want, rtol=1e-15, atol=0)


def test_argument_errors_follow_the_reference():
    from tqf import InvalidArgumentError
    from tqf.math.random import sobol
    from tqf.models import euler_sampling, HestonModel
    drift = lambda t, x: x  # noqa: E731
    with pytest.raises(ValueError):  # neither time_step nor num_time_steps
        euler_sampling.sample(1, drift, drift, times=[1.0])
    with pytest.raises(ValueError):  # both
        euler_sampling.sample(1, drift, drift, times=[1.0], time_step=0.1, num_time_steps=10)
    with pytest.raises(InvalidArgumentError):  # times not increasing
        euler_sampling.sample(1, drift, drift, times=[1.0, 0.5], time_step=0.1, validate_args=True)
    with pytest.raises(ValueError):  # dim mismatch with normal_draws
        euler_sampling.sample(2, drift, drift, times=[1.0], time_step=0.1, normal_draws=np.zeros((4, 10, 1)))
    with pytest.raises(InvalidArgumentError):  # draws steps mismatch
        euler_sampling.sample(1, drift, drift, times=[1.0], time_step=0.1, normal_draws=np.zeros((4, 7, 1)),
                              validate_args=True)
    with pytest.raises(ValueError):
        sobol.sample(0, 5, validate_args=True)
    with pytest.raises(InvalidArgumentError):
        sobol.sample(2, 5, skip=-10, validate_args=True)
    with pytest.raises(InvalidArgumentError):
        sobol.sample(2, 0, validate_args=True)
    with pytest.raises(InvalidArgumentError):
        sobol.sample(1, 4, skip=2 ** 31 - 5, validate_args=True)
    m = HestonModel(2.0, 0.04, 0.3, -0.7)
    with pytest.raises(ValueError):
        m.sample_paths([1.0], [0.0, 0.04])
    with pytest.raises(ValueError):
        m.sample_paths([1.0], [0.0, 0.04], time_step=0.1, num_time_steps=10)


def test_piecewise_left_continuous():
    from tqf.math.piecewise import PiecewiseConstantFunc
    f = PiecewiseConstantFunc([0.1, 10], [3, 4, 5], dtype=np.float64)
    np.testing.assert_array_equal(f(np.array([0.0, 0.1, 2.0, 11.0])), [3, 3, 4, 5])


def test_seed_conventions():
    from tqf.math.random.multivariate_normal import RandomType, philox_key
    assert philox_key(RandomType.STATELESS, [3, 4]) == (3, 4)
    assert philox_key(RandomType.PSEUDO, 42) == (42, 0)
    with pytest.raises(ValueError):
        philox_key(RandomType.STATELESS, None)


def test_lsm_host_basis_and_payoff_match_oracle():
    """The drop-in basis and payoff callables (torch, any device) equal the
    oracle's restatement; the exponent grid keeps the reference's order."""
    import torch
    from oracle import lsm as olsm
    from tqf.models.longstaff_schwartz import make_basket_put_payoff, make_polynomial_basis
    from tqf.models.longstaff_schwartz.lsm import _discount_table, polynomial_exponents
    for deg, dim in [(2, 1), (3, 2), (1, 4)]:
        np.testing.assert_array_equal(polynomial_exponents(deg, dim), olsm.polynomial_exponents(deg, dim))
    rng = np.random.default_rng(0)
    x = rng.uniform(0.5, 1.5, (2, 50, 4, 2))
    got = make_polynomial_basis(3)(torch.as_tensor(x), 2).numpy()
    np.testing.assert_allclose(got, olsm.polynomial_basis(x, 2, 3), rtol=1e-12, atol=1e-14)
    pay = make_basket_put_payoff([1.0, 1.1], dtype=np.float64)(torch.as_tensor(x), 1).numpy()
    np.testing.assert_allclose(pay, olsm.basket_put_payoff(x, 1, [1.0, 1.1]), rtol=1e-14)
    d = _discount_table([0.9, 0.8], 2, np.float64)
    assert d.shape == (3, 1, 1) and d[0, 0, 0] == 1.0 and d[2, 0, 0] == 0.8


def test_cv_pipeline_stage_marks():
    """Two pipeline steps strictly inside every interval of at least three
    steps, one for two, none for one; never on a date."""
    from tqf.pricing.neural_cv import stage_marks
    dates = np.array([4, 9, 13, 14, 16, 19])
    m = stage_marks(dates)
    assert m.tolist() == [1, 2, 6, 7, 10, 12, 15, 17, 18]
    assert not set(m.tolist()) & set(dates.tolist())
    # the Asian configuration: 52 dates on 252 steps
    ti = np.round(np.arange(1, 53) * 252 / 52).astype(int)
    m = stage_marks(ti - 1)
    assert len(m) == 2 * 52 and np.all(np.diff(m) > 0)


def test_cv_control_dates_and_marks_around_held_dates():
    """Control dates: every n-th monitoring date counted back from the last;
    the pipeline marks of the longer control intervals avoid the held dates."""
    from tqf.pricing.neural_cv import control_dates, stage_marks
    assert control_dates(52, 1).tolist() == list(range(52))
    assert control_dates(52, 2).tolist() == list(range(1, 52, 2))
    assert control_dates(5, 3).tolist() == [1, 4]
    with pytest.raises(ValueError):
        control_dates(4, 0)
    ti = np.round(np.arange(1, 53) * 252 / 52).astype(int)
    cd = control_dates(52, 2)
    m = stage_marks(ti[cd] - 1, busy=ti - 1)
    assert len(m) == 2 * 26 and np.all(np.diff(m) > 0)
    assert not set(m.tolist()) & set((ti - 1).tolist())
    # a held date at the natural mark moves the mark to the nearest free step
    assert stage_marks([6], busy=[1, 4]).tolist() == [2, 3]


def test_reference_wrong_times_and_sample_shape_mismatch():
    # euler_sampling_test.py:503-572: with validate_args, non-increasing times
    # or times_grid and draws that do not match the grid raise
    # InvalidArgumentError before anything runs.
    from tqf import InvalidArgumentError
    from tqf.models import euler_sampling

    def drift_fn(_, x):
        return x * 0

    def vol_fn(_, x):
        return (x * 0 + 1)[..., None]

    kw = dict(dim=1, drift_fn=drift_fn, volatility_fn=vol_fn, seed=42, validate_args=True, dtype=np.float64)
    with pytest.raises(InvalidArgumentError):  # draws for 5 steps on a 3-point grid
        euler_sampling.sample(times=[0.1, 0.5, 1.0], normal_draws=np.zeros((100, 5, 1)),
                              times_grid=[0.1, 0.5, 1.0], **kw)
    with pytest.raises(InvalidArgumentError):  # times not increasing
        euler_sampling.sample(times=[0.1, 0.5, 2.0, 1.0], time_step=0.01, **kw)
    with pytest.raises(InvalidArgumentError):  # times_grid not increasing
        euler_sampling.sample(times=[0.1, 0.5, 1.0], times_grid=[0.1, 0.5, 1.0, 1.0], **kw)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, None])
def test_heston_model_drift_and_volatility_pinned(dtype):
    # heston_model_test.py:175-219 on the model's own drift_fn / volatility_fn
    # (host torch functions, piecewise-constant parameters read at t = 0.1).
    import torch
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import HestonModel
    process = HestonModel(mean_reversion=PiecewiseConstantFunc([0.5], [1, 1.1], dtype=dtype),
                          theta=PiecewiseConstantFunc([0.5], [1, 0.9], dtype=dtype),
                          volvol=PiecewiseConstantFunc([0.3], [0.1, 0.2], dtype=dtype),
                          rho=PiecewiseConstantFunc([0.5], [0.4, 0.6], dtype=dtype), dtype=dtype)
    x0 = torch.tensor([np.log(100), 0.045], dtype=torch.float64)
    np.testing.assert_allclose(process.drift_fn()(0.1, x0).numpy(), [-0.0225, 0.955], rtol=1e-6)
    np.testing.assert_allclose(process.volatility_fn()(0.1, x0).numpy(),
                               [[0.21213203, 0.0], [0.00848528, 0.01944222]], rtol=1e-6)


@pytest.mark.parametrize("sample_shape,batch_shape", [((7,), (3,)), ((5,), (4, 2)), ((2, 3, 5), (4, 2)),
                                                      ((3,), (2, 3, 2)), ((), (3, 2))])
def test_quasi_random_batch_layout_follows_the_reference(sample_shape, batch_shape):
    # multivariate_normal.py:370-416 restated with NumPy: points [num, dim] ->
    # transpose -> reshape(reverse(batch_shape) + sample_shape) -> sample axes
    # first, batch axes back in order.
    import torch
    from tqf.math.random.multivariate_normal import quasi_layout
    dim = batch_shape[-1]
    num = int(np.prod(sample_shape + batch_shape)) // dim
    points = np.arange(num * dim, dtype=np.float64).reshape(num, dim)
    out_t = tuple(reversed(batch_shape)) + tuple(sample_shape)
    nb, ns = len(batch_shape), len(sample_shape)
    perm = list(range(nb, nb + ns)) + list(range(nb - 1, -1, -1))
    want = np.transpose(points.T.reshape(out_t), perm)
    got = quasi_layout(torch.from_numpy(points), sample_shape, batch_shape).numpy()
    assert got.shape == tuple(sample_shape) + tuple(batch_shape)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("corr", [[[1, 0.1], [0.1, 1]], None])
def test_multivariate_gbm_drift_and_volatility(dtype, corr):
    # geometric_brownian_motion_test.py:174-245 (with and without a correlation matrix)
    import torch
    from tqf.models import ItoProcess, MultivariateGeometricBrownianMotion
    means, vols = [0.05, 0.02], [0.1, 0.2]
    process = MultivariateGeometricBrownianMotion(dim=2, means=means, volatilities=vols, corr_matrix=corr,
                                                  dtype=torch.float64)
    assert isinstance(process, ItoProcess)
    state = np.array([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]], dtype=dtype)
    np.testing.assert_allclose(process.drift_fn()(0.2, state).numpy(), np.array(means) * state,
                               atol=1e-8, rtol=1e-8)
    expected_vol = np.expand_dims(np.array(vols) * state, -1) * np.linalg.cholesky(
        np.eye(2) if corr is None else np.array(corr, np.float64))
    np.testing.assert_allclose(process.volatility_fn()(0.2, state).numpy(), expected_vol, atol=1e-8, rtol=1e-8)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_prepare_grid_reference_cases(dtype):
    # utils_test.py:96-131 on the product's prepare_grid
    from tqf.models import utils
    times = np.linspace(dtype(0.02), dtype(1.0), 50).astype(dtype)
    grid, _, idx = utils.prepare_grid(times=times, time_step=times[-1] / 100, dtype=dtype, num_time_steps=100)
    np.testing.assert_allclose(grid, np.linspace(0, 1, 101, dtype=dtype), rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(idx, [2 * i for i in range(1, 51)])
    times = np.array([0.1, 0.5, 1, 2], dtype=dtype)
    grid, _, idx = utils.prepare_grid(times=times, time_step=np.float64(0.1), dtype=dtype)
    np.testing.assert_allclose(grid, np.linspace(0, 2, 21, dtype=dtype), rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(grid[idx], times, rtol=1e-6, atol=1e-6)


def test_heston_expected_total_variance():
    # heston_model_test.py:79-96, 137-170: scalar and batched closed form;
    # piecewise mean reversion / theta raise ValueError
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models import HestonModel

    def ground(v0, t, k=1.3, th=0.2):
        return (v0 - th) * (1 - np.exp(-k * t)) / k + th * t

    process = HestonModel(mean_reversion=1.3, theta=0.2, volvol=0.01, rho=0.1, dtype=np.float64)
    np.testing.assert_allclose(process.expected_total_variance(1.2, 0.3).numpy(), ground(0.3, 1.2))
    t, v0 = np.array([0.1, 1.0, 2.0]), np.array([0.1, 0.2, 0.3])
    np.testing.assert_allclose(process.expected_total_variance(t, v0).numpy(), ground(v0, t))
    pw = HestonModel(mean_reversion=PiecewiseConstantFunc([0.5], [1, 1.1], dtype=np.float64),
                     theta=PiecewiseConstantFunc([0.5], [1, 0.9], dtype=np.float64), volvol=0.1, rho=0.5,
                     dtype=np.float64)
    with pytest.raises(ValueError):
        pw.expected_total_variance(1.0, 1.0)


def test_hull_white_rejects_bad_jump_batches():
    """hull_white_test.py:388-420: a piecewise parameter's jump locations have
    batch shape [] or [dim]; batch [1] for dim 2, or batch rank 2, raise
    ValueError when the model is built."""
    from tqf.math.piecewise import PiecewiseConstantFunc
    from tqf.models.hull_white import VectorHullWhiteModel

    def rate(t):
        return 0.01 * torch.ones(tuple(t.shape) + (2,), dtype=t.dtype)

    bad_size = PiecewiseConstantFunc([[0.1, 2.0]], values=[3 * [0.1]], dtype=np.float64)
    with pytest.raises(ValueError):
        VectorHullWhiteModel(2, bad_size, [0.01, 0.02], rate, dtype=np.float64)
    bad_rank = PiecewiseConstantFunc([[[0.1, 2.0]]], values=[[3 * [[0.1, 0.05]]]], dtype=np.float64)
    with pytest.raises(ValueError):
        VectorHullWhiteModel(2, bad_rank, [0.01, 0.02], rate, dtype=np.float64)
    # per-axis volatility evaluates per axis; the knots of all parameters are merged per axis
    vol = PiecewiseConstantFunc([[0.1, 2.0], [0.5, 1.0]], [[0.01, 0.02, 0.01], [0.01, 0.015, 0.03]],
                                dtype=np.float64)
    m = VectorHullWhiteModel(2, [0.03, 0.02], vol, rate, dtype=np.float64)
    np.testing.assert_array_equal(m._jumps(), [[0.1, 2.0], [0.5, 1.0]])
    np.testing.assert_array_equal(m._vol(np.array([0.1, 0.7, 3.0])), [[0.01, 0.01], [0.02, 0.015], [0.01, 0.03]])
    # a constant curve given as a list answers the same at every time
    c = VectorHullWhiteModel(2, [0.03, 0.02], vol, lambda *args: [0.01, 0.015], dtype=np.float64)
    np.testing.assert_allclose(c._forward(np.array([0.0, 0.5, 1.0])), [[0.01, 0.015]] * 3, rtol=1e-15)
