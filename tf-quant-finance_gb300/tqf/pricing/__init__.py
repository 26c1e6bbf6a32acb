"""Fused Monte Carlo pricing on top of the path kernels.

The reference leaves payoffs and the discounted mean to the caller (e.g. the
Euler notebook, Monte_Carlo_Euler_Scheme.ipynb:235-276, and
heston_model_test.py:349-352).  Here the European payoff over a batch of
strikes and its FP64 cross-path accumulation (sum and sum of squares) run
inside the path kernel, so no path reaches HBM.
"""

from tqf.pricing.european import MonteCarloResult, european_payoff_stats  # noqa: F401
from tqf.pricing.heston import HestonEuropeanPrice, heston_european_mc, heston_european_vjp  # noqa: F401
from tqf.pricing.basket import BasketPrice, basket_european_mc  # noqa: F401
from tqf.pricing.neural_cv import HestonAsianCV, time_to_ci  # noqa: F401

__all__ = ["MonteCarloResult", "european_payoff_stats", "heston_european_mc", "basket_european_mc",
           "BasketPrice", "HestonEuropeanPrice", "heston_european_vjp", "HestonAsianCV", "time_to_ci"]
