"""Ito process from user callables (tff/models/generic_ito_process.py:27-317).

``sample_paths`` forwards to ``euler_sampling.sample`` exactly as the
reference does (generic_ito_process.py:299-317).  The finite-difference PDE
solvers of the reference class are not part of this engine.
"""

from __future__ import annotations

import torch

from tqf.models import euler_sampling
from tqf.models.ito_process import ItoProcess


class GenericItoProcess(ItoProcess):

    def __init__(self, dim, drift_fn, volatility_fn, dtype=None, name=None):
        self._dim = int(dim)
        self._drift_fn = drift_fn
        self._volatility_fn = volatility_fn
        self._dtype = dtype
        self._name = name or "generic_ito_process"

    def dim(self):
        return self._dim

    def dtype(self):
        return self._dtype

    def name(self):
        return self._name

    def drift_fn(self):
        return self._drift_fn

    def volatility_fn(self):
        return self._volatility_fn

    def sample_paths(self, times, num_samples=1, initial_state=None, random_type=None, seed=None,
                     swap_memory=True, name=None, time_step=None, num_time_steps=None, skip=0,
                     precompute_normal_draws=True, times_grid=None, normal_draws=None,
                     watch_params=None, validate_args=False):
        """Returns [batch..., num_samples, k, dim] paths (generic_ito_process.py:187-317)."""
        default_dtype = self._dtype
        if default_dtype is not None and not isinstance(default_dtype, torch.dtype):
            import numpy as np
            default_dtype = {np.dtype(np.float32): torch.float32,
                             np.dtype(np.float64): torch.float64}[np.dtype(default_dtype)]
        return euler_sampling.sample(
            dim=self._dim, drift_fn=self._drift_fn, volatility_fn=self._volatility_fn, times=times,
            time_step=time_step, num_time_steps=num_time_steps, num_samples=num_samples,
            initial_state=initial_state, random_type=random_type, seed=seed,
            swap_memory=swap_memory, skip=skip, precompute_normal_draws=precompute_normal_draws,
            times_grid=times_grid, normal_draws=normal_draws, watch_params=watch_params,
            validate_args=validate_args, dtype=default_dtype, name=name)
