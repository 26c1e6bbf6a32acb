"""Random numbers (tff/math/random_ops/__init__.py:17-22)."""

from tqf.math.random import halton  # noqa: F401
from tqf.math.random import sobol  # noqa: F401
from tqf.math.random.multivariate_normal import RandomType  # noqa: F401
from tqf.math.random.multivariate_normal import multivariate_normal as mv_normal_sample  # noqa: F401

__all__ = ["halton", "sobol", "RandomType", "mv_normal_sample"]
