"""Abstract Ito process interface (tff/models/ito_process.py:40-112)."""

from __future__ import annotations

import abc


class ItoProcess(abc.ABC):
    """dX = a(t, X) dt + b(t, X) dW with dim-dimensional state."""

    @abc.abstractmethod
    def name(self):
        """The name to give to ops created by this class."""

    @abc.abstractmethod
    def dim(self):
        """The dimension of the process."""

    @abc.abstractmethod
    def dtype(self):
        """The data type of process realizations."""

    @abc.abstractmethod
    def drift_fn(self):
        """Python callable a(t, x)."""

    @abc.abstractmethod
    def volatility_fn(self):
        """Python callable b(t, x)."""

    @abc.abstractmethod
    def sample_paths(self, times, num_samples=1, initial_state=None, random_type=None, seed=None,
                     **kwargs):
        """Returns a sample of paths from the process."""
