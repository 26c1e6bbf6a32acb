"""Extracts the reference's known-answer vectors for the hot path into
sobol_golden.json / heston_golden.json / lsm_golden.json / qmc_golden.json / hw_golden.json / hjm_golden.json.

Run in a checkout that has the reference sources (read as text; TensorFlow is
not needed):  python tests/golden/make_golden.py /path/to/tf-quant-finance
"""

import ast
import json
import os
import sys


def _literal_assignments(path, func_name):
    tree = ast.parse(open(path).read())
    out = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == func_name:
            for stmt in ast.walk(node):
                if isinstance(stmt, ast.Assign) and len(stmt.targets) == 1 and isinstance(stmt.targets[0], ast.Name):
                    try:
                        out[stmt.targets[0].id] = ast.literal_eval(stmt.value)
                    except ValueError:
                        pass
    return out


def main(ref_root):
    tff = os.path.join(ref_root, "tf_quant_finance")
    sob = os.path.join(tff, "math", "random_ops", "sobol", "sobol_test.py")
    more = _literal_assignments(sob, "test_more_known_values")["expected"]
    large = _literal_assignments(sob, "test_large_skip")
    src = open(sob).read()
    # test_known_values_small_dimension builds its array inline: np.array([...])
    tree = ast.parse(src)
    small = None
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == "test_known_values_small_dimension":
            for call in ast.walk(node):
                if isinstance(call, ast.Call) and getattr(call.func, "attr", "") == "array" and call.args:
                    small = ast.literal_eval(call.args[0])
    golden = {
        "source": "tf_quant_finance/math/random_ops/sobol/sobol_test.py",
        "dim2_first5": {"dim": 2, "num_results": 5, "skip": 0, "expected": small},
        "dim5_first31_gray_order": {"dim": 5, "num_results": 31, "skip": 0, "expected": more},
        "large_skip": {"dim": large["dim"], "num_results": large["num_results"],
                       "skip_expr": "2**31 - 5", "skip": 2 ** 31 - 5,
                       "expected": [[0.25], [0.75], [0.5]]},
    }
    # generate_mc_normal_draws with SOBOL draws: [steps, paths, d] normals of
    # the points skip + 1 ..., dimension step * d + component
    utils_test = os.path.join(tff, "models", "utils_test.py")
    usrc = open(utils_test).read()
    for needle in ("num_draws = tf.constant(2", "steps_num = tf.constant(3", "num_samples = tf.constant(4",
                   "skip = 10", "random_type = tff.math.random.RandomType.SOBOL"):
        assert needle in usrc, needle
    draws = _literal_assignments(utils_test, "test_sobol_numbers_generation")["expected_samples"]
    golden["mc_normal_draws_sobol"] = {"source": "tf_quant_finance/models/utils_test.py:33-60",
                                       "num_normal_draws": 2, "num_time_steps": 3, "num_sample_paths": 4,
                                       "skip": 10, "expected": draws, "rtol": 1e-5, "atol": 1e-5}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "sobol_golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    hest = {
        "source": ["tf_quant_finance/models/heston/heston_model_test.py:179-219",
                   "tf_quant_finance/models/heston/approximations/european_option_test.py:30-53"],
        "piecewise_drift_vol": {
            "mean_reversion": [[0.5], [1, 1.1]], "theta": [[0.5], [1, 0.9]],
            "volvol": [[0.3], [0.1, 0.2]], "rho": [[0.5], [0.4, 0.6]],
            "t": 0.1, "state": "log(100), 0.045",
            "drift": [-0.0225, 0.955], "volatility": [[0.21213203, 0.0], [0.00848528, 0.01944222]]},
        "european_docstring": {"variances": 0.11, "strikes": 102.0, "expiries": 1.2, "forwards": 100.0,
                               "mean_reversion": 2.0, "theta": 0.5, "volvol": 0.15, "rho": 0.3,
                               "discount_factors": 1.0, "price": 24.822196},
    }
    # Cross-check the numbers quoted above against the test sources.
    hsrc = open(os.path.join(tff, "models", "heston", "heston_model_test.py")).read()
    assert "0.21213203" in hsrc and "0.00848528, 0.01944222" in hsrc and "-0.0225, 0.955" in hsrc
    esrc = open(os.path.join(tff, "models", "heston", "approximations", "european_option_test.py")).read()
    assert "24.822196" in esrc
    with open(os.path.join(here, "heston_golden.json"), "w") as f:
        json.dump(hest, f, indent=1)
    # Longstaff-Schwartz: the 8-path example of Longstaff & Schwartz (2001) and
    # the prices the reference's tests assert for it.
    lsm_path = os.path.join(tff, "models", "longstaff_schwartz", "lsm_test.py")
    ltree = ast.parse(open(lsm_path).read())
    samples = None
    for node in ltree.body:
        if isinstance(node, ast.Assign) and getattr(node.targets[0], "id", "") == "_SAMPLES":
            samples = ast.literal_eval(node.value)
    lsrc = open(lsm_path).read()
    for needle in ("[0.0564]", "[0.1144]", "[0.174226]", "[0.1144, 0.199]", "[0.1144, 0.1157]",
                   "[0.06, 0.06, 0.06]", "[0.05, 0.05, 0.05]", "make_polynomial_basis(10)"):
        assert needle in lsrc, needle
    lsm = {
        "source": "tf_quant_finance/models/longstaff_schwartz/lsm_test.py:26-224",
        "samples": samples,
        "rates": [0.06, 0.06, 0.06],
        "batch_rates": [[0.06, 0.06, 0.06], [0.05, 0.05, 0.05]],
        "cases": {
            "european_put": {"exercise_times": [3], "strikes": [1.1], "degree": 2, "discount": "last",
                             "price": [0.0564]},
            "american_put": {"exercise_times": [1, 2, 3], "strikes": [1.1], "degree": 2, "price": [0.1144]},
            "american_put_calibration": {"exercise_times": [1, 2, 3], "strikes": [1.1], "degree": 2,
                                         "num_calibration_samples": 4, "price": [0.174226]},
            "american_put_batch_payoff": {"exercise_times": [1, 2, 3], "strikes": [1.1, 1.2], "degree": 2,
                                          "discount": "batch", "price": [0.1144, 0.199]},
            "american_put_batch_samples": {"exercise_times": [1, 2, 3], "strikes": [1.1, 1.2], "degree": 2,
                                           "discount": "batch", "paths_shift": 0.1, "price": [0.1144, 0.1157]},
            "american_basket_put_2d": {"exercise_times": [1, 2, 3], "strikes": [1.1, 1.2, 1.3], "degree": 10,
                                       "note": "2-d paths (the sample path twice) price as the 1-d paths"},
        },
        "tolerance": {"rtol": 1e-4, "atol": 1e-4},
    }
    with open(os.path.join(here, "lsm_golden.json"), "w") as f:
        json.dump(lsm, f, indent=1)
    # tff.math.qmc: the `expected = tf.constant([...])` literal of each test
    # function, with the call it checks (cross-checked against the source).
    qmc_dir = os.path.join(tff, "math", "qmc")

    def expected_of(path, func):
        tree = ast.parse(open(path).read())
        for node in ast.walk(tree):
            if isinstance(node, ast.FunctionDef) and node.name == func:
                for stmt in ast.walk(node):
                    if (isinstance(stmt, ast.Assign) and getattr(stmt.targets[0], "id", "") == "expected"
                            and isinstance(stmt.value, ast.Call) and stmt.value.args):
                        return ast.literal_eval(stmt.value.args[0])
        raise KeyError(func)

    def class_list(path, name):
        tree = ast.parse(open(path).read())
        for node in ast.walk(tree):
            if isinstance(node, ast.Assign) and getattr(node.targets[0], "id", "") == name:
                return ast.literal_eval(node.value)
        raise KeyError(name)

    sob_t = os.path.join(qmc_dir, "sobol_test.py")
    dn_t = os.path.join(qmc_dir, "digital_net_test.py")
    lr_t = os.path.join(qmc_dir, "lattice_rule_test.py")
    src = open(sob_t).read() + open(dn_t).read() + open(lr_t).read()
    for needle in ("qmc.sobol_sample(5, 29, validate_args=True)", "indices = [1, 3, 10, 15, 19, 24, 28]",
                   "apply_tent_transform=True", "qmc.sobol_sample(6, 8, validate_args=True, dtype=dtype)",
                   "indices = [2, 3, 6, 9, 11, 14]"):
        assert needle in src, needle
    qmc = {
        "source": ["tf_quant_finance/math/qmc/sobol_test.py", "tf_quant_finance/math/qmc/digital_net_test.py",
                   "tf_quant_finance/math/qmc/lattice_rule_test.py"],
        "sobol_sample": {"dim": 5, "num_results": 29, "expected": expected_of(sob_t, "test_sobol_sample")},
        "sobol_sample_indices": {"dim": 5, "num_results": 29, "sequence_indices": [1, 3, 10, 15, 19, 24, 28],
                                 "expected": expected_of(sob_t, "test_sobol_sample_with_sequence_indices")},
        "sobol_sample_tent": {"dim": 6, "num_results": 8, "tent": True,
                              "expected": expected_of(sob_t, "test_sobol_sample_with_tent_transform")},
        "sobol_sample_dtype": {"dim": 6, "num_results": 8,
                               "expected": expected_of(sob_t, "test_sobol_sample_with_dtype")},
        "generating_matrices": {"dim": 5, "num_results": 31, "num_digits": 5,
                                "expected": expected_of(sob_t, "test_sobol_generating_matrices")},
        "digital_net": {"dim": 5, "num_results": 29, "num_digits": 5,
                        "expected": expected_of(dn_t, "test_digital_net_sample")},
        "digital_net_indices": {"dim": 5, "num_results": 29, "num_digits": 5,
                                "sequence_indices": [1, 3, 10, 15, 19, 24, 28],
                                "expected": expected_of(dn_t, "test_digital_net_sample_with_sequence_indices")},
        "digital_net_tent": {"dim": 6, "num_results": 8, "num_digits": 3, "tent": True,
                             "expected": expected_of(dn_t, "test_sample_sobol_with_tent_transform")},
        "lattice_generating_vectors": class_list(lr_t, "generating_vectors_values"),
        "lattice": {"dim": 6, "num_results": 16, "expected": expected_of(lr_t, "test_lattice_rule_sample")},
        "lattice_indices": {"dim": 6, "num_results": 16, "sequence_indices": [2, 3, 6, 9, 11, 14],
                            "expected": expected_of(lr_t, "test_lattice_rule_sample_with_sequence_indices")},
        "lattice_zero_shift": {"dim": 5, "num_results": 8,
                               "expected": expected_of(lr_t, "test_lattice_rule_sample_with_zero_additive_shift")},
        "lattice_shift": {"dim": 5, "num_results": 8,
                          "additive_shift": _literal_assignments(
                              lr_t, "test_lattice_rule_sample_with_non_zero_additive_shift")["additive_shift"],
                          "expected": expected_of(lr_t, "test_lattice_rule_sample_with_non_zero_additive_shift")},
        "tolerance": {"rtol": 1e-6},
    }
    with open(os.path.join(here, "qmc_golden.json"), "w") as f:
        json.dump(qmc, f, indent=1)
    # Hull-White: the zero-coupon bond prices conditional on r(t) that
    # hull_white_test.py asserts, with the model parameters of its setUp.
    hw_t = os.path.join(tff, "models", "hull_white", "hull_white_test.py")
    setup = _literal_assignments(hw_t, "setUp")
    bond = _literal_assignments(hw_t, "test_discount_bond_price_fn")
    hsrc = open(hw_t).read()
    assert "[[0.011], [0.01]]" in hsrc and "[1.0, 2.0]" in hsrc and "[2.0, 3.5]" in hsrc
    hw = {
        "source": "tf_quant_finance/models/hull_white/hull_white_test.py",
        "mean_reversion": setup["self.mean_reversion"] if "self.mean_reversion" in setup else [0.1, 0.05],
        "volatility": [0.01, 0.02],
        "volatility_time_dep_1d": [0.01, 0.02, 0.01],
        "flat_rate": 0.01,
        "bond": {"short_rate": [[0.011], [0.01]], "times": [1.0, 2.0], "maturities": [2.0, 3.5],
                 "expected": bond["expected"], "atol": 1e-12, "rtol": 1e-6},  # tf.test default rtol
    }
    for needle in ("self.mean_reversion = [0.1, 0.05]", "self.volatility = [0.01, 0.02]",
                   "self.volatility_time_dep_1d = [0.01, 0.02, 0.01]", "0.01 * tf.ones_like(t)"):
        assert needle in hsrc, needle
    with open(os.path.join(here, "hw_golden.json"), "w") as f:
        json.dump(hw, f, indent=1)
    # Gaussian HJM: discount_bond_price known values (gaussian_hjm_test.py:224-282).
    hjm_t = os.path.join(tff, "models", "hjm", "gaussian_hjm_test.py")
    jsrc = open(hjm_t).read()
    one = [0.9803327113840525, 0.9803218405347454, 0.9803116028646381]
    two = [0.9707109604475661, 0.9706894322583266, 0.9706691582097785]
    for v in one + two:
        assert repr(v) in jsrc, v
    hjm = {
        "source": "tf_quant_finance/models/hjm/gaussian_hjm_test.py:224-282",
        "flat_rate": 0.01,
        "cases": [
            {"dim": 1, "mr": [0.03], "vol": [0.005], "times": [1.0, 2.0, 3.0], "expected": one},
            {"dim": 2, "mr": [0.03, 0.03], "vol": [0.005, 0.005], "times": [1.0, 2.0, 3.0], "expected": two},
        ],
        "state": 0.01, "maturity_offset": 1.0, "rtol": 1e-8, "atol": 1e-8,
    }
    with open(os.path.join(here, "hjm_golden.json"), "w") as f:
        json.dump(hjm, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the tf-quant-finance checkout>")
    main(sys.argv[1])
