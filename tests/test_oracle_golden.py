"""The oracle pinned on the reference's own known-answer tests (CPU)."""

import json
import os

import numpy as np
import pytest

from oracle import closed_form, grids, heston, philox, sobol

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SOBOL_GOLDEN = json.load(open(os.path.join(GOLDEN_DIR, "sobol_golden.json")))
HESTON_GOLDEN = json.load(open(os.path.join(GOLDEN_DIR, "heston_golden.json")))


@pytest.mark.parametrize("dtype", [np.float16, np.float32, np.float64])
def test_sobol_known_values_small_dimension(dtype):
    # sobol_test.py:28-38 — first five points, dimension 2, original order.
    g = SOBOL_GOLDEN["dim2_first5"]
    out = sobol.sample(g["dim"], g["num_results"], dtype=np.float32 if dtype == np.float16 else dtype)
    np.testing.assert_allclose(out.astype(dtype), np.array(g["expected"], dtype=dtype), rtol=1e-6)


def test_sobol_more_known_values_as_set():
    # sobol_test.py:40-81 — 31 points of dimension 5 (listed in Gray-code
    # order, compared as a set, as the reference test does).
    g = SOBOL_GOLDEN["dim5_first31_gray_order"]
    ours = sobol.sample(g["dim"], g["num_results"], dtype=np.float64)
    assert sorted(tuple(r) for r in g["expected"]) == sorted(tuple(r) for r in ours)


def test_sobol_skip():
    # sobol_test.py:83-91
    full = sobol.sample_int(10, 50 + 17, nd=sobol.num_digits(67, 0))
    part = sobol.sample_int(10, 50, skip=17, nd=sobol.num_digits(67, 0))
    np.testing.assert_array_equal(full[17:], part)
    np.testing.assert_allclose(sobol.sample(10, 67)[17:], sobol.sample(10, 50, skip=17))


def test_sobol_large_skip():
    # sobol_test.py:93-98
    g = SOBOL_GOLDEN["large_skip"]
    np.testing.assert_allclose(sobol.sample(g["dim"], g["num_results"], skip=g["skip"]), g["expected"])


def test_sobol_float_rounds_to_one_at_2_pow_26():
    # float32(int)/2^27 for dimension 0, index 2^26 - 1 -> int 2^27 - 2 -> 1.0.
    nd = sobol.num_digits(2 ** 26, 0)
    assert nd == 27
    ints = sobol.sample_int(1, 1, skip=2 ** 26 - 2, nd=nd)
    assert int(ints[0, 0]) == 2 ** 27 - 2
    assert np.float32(ints[0, 0]) / np.float32(2.0 ** 27) == np.float32(1.0)


def test_sobol_num_digits():
    assert sobol.num_digits(5, 0) == 3
    assert sobol.num_digits(3, 2 ** 31 - 5) == 31
    assert sobol.num_digits(2 ** 22, 0) == 23


# Random123 known-answer vectors for philox4x32-10.
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expected", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expected):
    out = philox.philox4x32_10(*[np.array([c], dtype=np.uint64) for c in ctr], *key)
    assert tuple(int(o[0]) for o in out) == expected


def test_philox_normals_moments():
    z = philox.normals(np.arange(20000), 8, 7, 11)
    assert abs(z.mean()) < 0.01
    assert abs(z.std() - 1) < 0.01


def test_heston_drift_and_volatility_pinned():
    # heston_model_test.py:179-219
    g = HESTON_GOLDEN["piecewise_drift_vol"]
    k, th, xi, rho = (tuple(tuple(v) for v in g[n]) for n in ("mean_reversion", "theta", "volvol", "rho"))
    x = np.array([np.log(100), 0.045])
    np.testing.assert_allclose(heston.drift_fn(k, th, np.float64)(g["t"], x), g["drift"])
    np.testing.assert_allclose(heston.volatility_fn(xi, rho, np.float64)(g["t"], x), g["volatility"], rtol=1e-6)


def test_heston_semi_analytic_price_pinned():
    # european_option_test.py:30-53
    g = HESTON_GOLDEN["european_docstring"]
    p = closed_form.heston_price(forward=g["forwards"], strike=g["strikes"], expiry=g["expiries"],
                                 v0=g["variances"], kappa=g["mean_reversion"], theta=g["theta"],
                                 xi=g["volvol"], rho=g["rho"], discount_factor=g["discount_factors"])
    np.testing.assert_allclose(p, g["price"], rtol=1e-5, atol=1e-5)


def test_black_scholes_textbook():
    np.testing.assert_allclose(closed_form.black_scholes(100, 100, 0.05, 0.2, 1.0), 10.450583572185565, rtol=1e-12)
    put = closed_form.black_scholes(100, 100, 0.05, 0.2, 1.0, is_call=False)
    np.testing.assert_allclose(put, 5.573526022256971, rtol=1e-12)


def test_euler_grid_from_time_step():
    # 101 points for times=[1.0], time_step=0.01 (float64)
    t, mask, ti = grids.prepare_grid([1.0], 0.01, np.float64)
    assert len(t) == 101 and mask[-1] and mask.sum() == 1 and ti[0] == 100
    # requested times inside the grid are merged, duplicates removed
    t, mask, ti = grids.prepare_grid([0.1, 1.0, 2.0], 0.01, np.float64)
    assert len(t) == 201 and list(ti) == [10, 100, 200]


def test_euler_grid_from_num_steps_and_times_grid():
    t, mask, ti = grids.prepare_grid([0.5, 1.0], 0.01, np.float32, num_time_steps=100)
    assert len(t) == 101 and t[0] == 0 and list(ti) == [np.searchsorted(t, np.float32(0.5)), 100]
    tg = np.linspace(0, 1, 253)
    t, mask, ti = grids.prepare_grid(np.linspace(1 / 52, 1, 52), None, np.float64, times_grid=tg)
    assert len(t) == 253 and mask.sum() == 52 and ti[-1] == 252


def test_heston_grid_keeps_duplicates():
    t, mask = grids.heston_prepare_grid([0.0, 1.0], 0.25, np.float32)
    assert list(t) == [0.0, 0.0, 0.25, 0.5, 0.75, 1.0]
    assert list(mask) == [False, True, False, False, False, True]


def test_write_slots():
    # times=[0.5, 1.0] on a 4-step grid: states after steps 1 and 3 recorded.
    keep = np.array([False, False, True, False, True])
    step_slot, init_slot, n, unwritten = grids.write_slots(keep, 2, 0)
    assert list(step_slot) == [-1, 0, -1, 1] and init_slot == -1 and n == 4 and not unwritten
    # keep_mask[0] (time 0 requested) keeps the initial state in slot 0.
    keep = np.array([True, False, True])
    step_slot, init_slot, n, unwritten = grids.write_slots(keep, 2, 1)
    assert list(step_slot) == [-1, 1] and init_slot == 0
    # times_grid past the last requested time: the loop stops early.
    keep = np.array([False, True, False, False])
    step_slot, init_slot, n, _ = grids.write_slots(keep, 1, 0)
    assert n == 1 and list(step_slot) == [0]


def _lsm_golden():
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "lsm_golden.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_lsm_oracle_matches_reference_known_answers(dtype):
    """The regression-MC restatement reproduces every price lsm_test.py asserts
    for the Longstaff & Schwartz (2001) 8-path example."""
    from oracle import lsm
    g = _lsm_golden()
    S = np.array(g["samples"])[..., None]
    df = np.exp(-np.cumsum(g["rates"]))
    dfb = np.exp(-np.cumsum(g["batch_rates"], -1))[None]
    tol = g["tolerance"]
    c = g["cases"]
    got = lsm.least_square_mc(S, [3], [1.1], 2, discount_factors=[df[-1]], dtype=dtype)
    np.testing.assert_allclose(got, c["european_put"]["price"], **tol)
    got = lsm.least_square_mc(S, [1, 2, 3], [1.1], 2, discount_factors=df, dtype=dtype)
    np.testing.assert_allclose(got, c["american_put"]["price"], **tol)
    got = lsm.least_square_mc(S, [1, 2, 3], [1.1], 2, discount_factors=df, num_calibration_samples=4, dtype=dtype)
    np.testing.assert_allclose(got, c["american_put_calibration"]["price"], **tol)
    got = lsm.least_square_mc(S, [1, 2, 3], [1.1, 1.2], 2, discount_factors=dfb, dtype=dtype)
    np.testing.assert_allclose(got, c["american_put_batch_payoff"]["price"], **tol)
    got = lsm.least_square_mc(np.stack([S, S + 0.1]), [1, 2, 3], [1.1, 1.2], 2, discount_factors=dfb, dtype=dtype)
    np.testing.assert_allclose(got, c["american_put_batch_samples"]["price"], **tol)
    two = lsm.least_square_mc(np.concatenate([S, S], -1), [1, 2, 3], [1.1, 1.2, 1.3], 10, discount_factors=df,
                              dtype=np.float64)
    one = lsm.least_square_mc(S, [1, 2, 3], [1.1, 1.2, 1.3], 10, discount_factors=df, dtype=np.float64)
    np.testing.assert_allclose(two, one, **tol)
    assert two.shape == (3,)


def test_lsm_basis_docstring_example():
    """make_polynomial_basis(2) on [1, 2, 3, 4] (lsm.py:68-77)."""
    from oracle import lsm
    x = np.array([[1.0], [2.0], [3.0], [4.0]])[:, None, :]
    np.testing.assert_allclose(lsm.polynomial_basis(x, 0, 2)[0],
                               [[1, 1, 1, 1], [-1.5, -0.5, 0.5, 1.5], [2.25, 0.25, 0.25, 2.25]])


def test_halton_oracle_known_values():
    """First five unscrambled points in bases 2 and 3 (halton_test.py:30-37)."""
    from oracle import halton
    expected = np.array([[1 / 2, 1 / 3], [1 / 4, 2 / 3], [3 / 4, 1 / 9], [1 / 8, 4 / 9], [5 / 8, 7 / 9]], np.float32)
    np.testing.assert_allclose(halton.sample(2, np.arange(5), np.float32), expected, rtol=1e-6)
    np.testing.assert_allclose(halton.sample(2, np.arange(5), np.float64), expected.astype(np.float64), rtol=1e-6)
    assert halton.primes(1000)[-1] == 7919 and list(halton.primes(5)) == [2, 3, 5, 7, 11]


def test_qmc_oracle_matches_reference_known_answers():
    """Generating matrices, digital-net and lattice points of the reference's
    qmc tests (sobol_test.py, digital_net_test.py, lattice_rule_test.py)."""
    from oracle import qmc
    with open(os.path.join(os.path.dirname(__file__), "golden", "qmc_golden.json")) as f:
        g = json.load(f)
    tol = dict(rtol=1e-6, atol=1e-6)  # tf.test assertAllClose defaults
    c = g["generating_matrices"]
    np.testing.assert_array_equal(qmc.sobol_generating_matrices(c["dim"], c["num_results"], c["num_digits"]),
                                  c["expected"])
    for key in ("sobol_sample", "sobol_sample_indices", "sobol_sample_tent", "sobol_sample_dtype"):
        c = g[key]
        got = qmc.sobol_sample(c["dim"], c["num_results"], sequence_indices=c.get("sequence_indices"),
                               apply_tent_transform=c.get("tent", False))
        np.testing.assert_allclose(got, c["expected"], **tol)
    for key in ("digital_net", "digital_net_indices", "digital_net_tent"):
        c = g[key]
        gen = qmc.sobol_generating_matrices(c["dim"], c["num_results"], c["num_digits"])
        got = qmc.digital_net_sample(gen, c["num_results"], c["num_digits"], c.get("sequence_indices"),
                                     apply_tent_transform=c.get("tent", False))
        np.testing.assert_allclose(got, c["expected"], **tol)
    gv = g["lattice_generating_vectors"]
    for key, shift in (("lattice", None), ("lattice_indices", None), ("lattice_zero_shift", np.zeros(20)),
                       ("lattice_shift", g["lattice_shift"].get("additive_shift"))):
        c = g[key]
        got = qmc.lattice_rule_sample(gv, c["dim"], c["num_results"], c.get("sequence_indices"), shift)
        np.testing.assert_allclose(got, c["expected"], **tol)
    gen = qmc.sobol_generating_matrices(6, 8, 3)
    np.testing.assert_array_equal(qmc.scramble_generating_matrices(gen, np.full(gen.shape, 4), 3), gen)


def test_hull_white_oracle_bond_prices():
    """P(t, T | r(t)) of hull_white_test.py:465-485 (atol 1e-12 and tf.test's default rtol 1e-6)."""
    from oracle import hull_white as ohw
    with open(os.path.join(os.path.dirname(__file__), "golden", "hw_golden.json")) as f:
        g = json.load(f)
    p = ohw.Params(1, [([], [g["mean_reversion"][0]])], [([], [g["volatility"][0]])], np.float64)
    b = g["bond"]
    got = ohw.bond_reconstitution(p, b["times"], b["maturities"], b["short_rate"],
                                  lambda t: np.full((len(t), 1), g["flat_rate"]),
                                  lambda t: np.full(np.shape(t), g["flat_rate"]))
    np.testing.assert_allclose(got.ravel(), b["expected"], atol=b["atol"], rtol=b["rtol"])


def test_hjm_oracle_bond_prices():
    """Gaussian HJM P(t, t + 1 | x = 0.01) of gaussian_hjm_test.py:224-282."""
    from oracle import hjm
    with open(os.path.join(os.path.dirname(__file__), "golden", "hjm_golden.json")) as f:
        g = json.load(f)
    for c in g["cases"]:
        m = hjm.Model(c["dim"], c["mr"], None, np.asarray(c["vol"])[:, None], None, np.float64)
        t = np.asarray(c["times"])
        got = m.bond(g["state"] * np.ones((len(t), c["dim"])), t, t + g["maturity_offset"],
                     lambda x: np.full(np.shape(x), g["flat_rate"]))
        np.testing.assert_allclose(got, c["expected"], rtol=g["rtol"], atol=g["atol"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_mc_normal_draws_sobol_known_values(dtype):
    # utils_test.py:33-60: generate_mc_normal_draws(2 draws, 3 steps, 4 paths,
    # SOBOL, skip 10) -> [steps, paths, d], dimension step * d + component
    g = SOBOL_GOLDEN["mc_normal_draws_sobol"]
    d, steps, n = g["num_normal_draws"], g["num_time_steps"], g["num_sample_paths"]
    u = sobol.sample(d * steps, n, skip=g["skip"], dtype=dtype)
    z = sobol.normal_from_uniform(u).reshape(n, steps, d).transpose(1, 0, 2)
    np.testing.assert_allclose(z, g["expected"], rtol=g["rtol"], atol=g["atol"])
