"""Error types mirroring the reference's conventions.

The reference raises ``ValueError`` for inconsistent arguments at trace time
and ``tf.errors.InvalidArgumentError`` for the run-time ``validate_args``
assertions (e.g. tff/models/euler_sampling.py:241-307,
tff/math/random_ops/sobol/sobol_impl.py:85-104).  ``InvalidArgumentError``
subclasses ``ValueError`` so callers catching either keep working.
"""


class InvalidArgumentError(ValueError):
    """A run-time argument check (``validate_args``) failed."""
