"""Longstaff–Schwartz regression Monte Carlo (tff/models/longstaff_schwartz/__init__.py)."""

from tqf.models.longstaff_schwartz.lsm import least_square_mc, make_polynomial_basis  # noqa: F401
from tqf.models.longstaff_schwartz.payoff_utils import make_basket_put_payoff  # noqa: F401

__all__ = ["make_polynomial_basis", "least_square_mc", "make_basket_put_payoff"]
