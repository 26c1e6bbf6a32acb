"""CPU oracle: a NumPy/SciPy restatement of the reference's hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports, links or
executes this package; only tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, as the
checker or the timed CPU baseline.

TensorFlow is not installable here, so the reference itself cannot run; each
function restates the reference code it cites (paths relative to the
google/tf-quant-finance project root) and is pinned against the reference's
own known-answer tests (tests/test_oracle_golden.py):

* Sobol integers: sobol_test.py:28-98 golden vectors (bit-exact).
* Heston drift/volatility: heston_model_test.py:213-219.
* Heston semi-analytic price: european_option_test.py:53 (24.822196).
* Black–Scholes closed form against textbook values.

Philox4x32-10 / Box–Muller is this project's own random stream (the
reference's TF Philox bit patterns are third-party C++ and unpinned by any
reference test); the oracle restates it and pins it on the Random123
known-answer vectors.
"""
