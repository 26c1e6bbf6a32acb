"""Math namespace: ``random`` (alias of tff.math.random_ops), ``qmc`` and ``piecewise``."""

from tqf.math import piecewise  # noqa: F401
from tqf.math import qmc  # noqa: F401
from tqf.math import random  # noqa: F401
from tqf.math.piecewise import PiecewiseConstantFunc  # noqa: F401

random_ops = random

__all__ = ["piecewise", "qmc", "random", "random_ops", "PiecewiseConstantFunc"]
