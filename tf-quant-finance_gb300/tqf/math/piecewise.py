"""Batch-free piecewise-constant functions (tff/math/piecewise.py:19-176).

Used by the Heston model for time-dependent parameters; evaluated on the
host into per-step parameter tables before a kernel launch.
"""

from __future__ import annotations

import numpy as np


class PiecewiseConstantFunc:
    """f(x) = values[i] on (jump_locations[i-1], jump_locations[i]] (left-continuous)."""

    def __init__(self, jump_locations, values, dtype=None, name=None):
        self._name = name or "PiecewiseConstantFunc"
        self.is_piecewise_constant = True
        dtype = np.dtype(dtype) if dtype is not None else None
        jl = np.asarray(jump_locations, dtype=dtype)
        self._dtype = dtype or (jl.dtype if jl.dtype.kind == "f" else np.dtype(np.float32))
        self._jump_locations = jl.astype(self._dtype)
        self._values = np.asarray(values, dtype=self._dtype)
        if self._jump_locations.size == 0 and self._jump_locations.ndim == 1 and self._values.ndim == 2 \
                and self._values.shape[-1] == 1 and self._values.shape[0] > 1:
            # [[]] * batch style with values [batch, 1]
            self._jump_locations = np.zeros((self._values.shape[0], 0), self._dtype)
        self._batch_rank = self._jump_locations.ndim - 1
        if self._batch_rank > 1:
            raise NotImplementedError("PiecewiseConstantFunc with batch rank > 1 is not supported")
        if self._batch_rank == 1:
            # batch of functions: jump_locations [B, n], values [B, n + 1] (piecewise.py:19-176)
            if self._values.shape[:1] != self._jump_locations.shape[:1] or \
                    self._values.shape[1] - 1 != self._jump_locations.shape[1]:
                raise ValueError("Batch shapes of `values` and `jump_locations` should be the same and `values` "
                                 "should have one more element per batch member")
        elif self._values.shape[0] - 1 != self._jump_locations.shape[-1]:
            raise ValueError(
                "Event shape of `values` should have one more element than the event shape of "
                f"`jump_locations` but are {self._values.shape[0]} and {self._jump_locations.shape[-1]}")

    def dtype(self):
        return self._dtype

    def values(self):
        return self._values

    def jump_locations(self):
        return self._jump_locations

    def name(self):
        return self._name

    def __call__(self, x, left_continuous=True, name=None):
        x = np.asarray(x, dtype=self._dtype)
        side = "left" if left_continuous else "right"
        if self._batch_rank == 1:
            B = self._jump_locations.shape[0]
            xb = np.broadcast_to(x, (B,) + x.shape[-1:]) if x.ndim <= 1 else x
            idx = np.stack([np.searchsorted(self._jump_locations[b], xb[b], side=side) for b in range(B)])
            return np.take_along_axis(self._values, idx.reshape(B, -1), axis=1).reshape(xb.shape)
        idx = np.searchsorted(self._jump_locations, x, side=side)
        return self._values[idx]

    def integrate(self, x1, x2, name=None):
        """Integral of f over [x1, x2] (piecewise.py:178-208), elementwise."""
        del name
        x1 = np.asarray(x1, dtype=self._dtype)
        x2 = np.asarray(x2, dtype=self._dtype)
        return (self._primitive(x2) - self._primitive(x1)).astype(self._dtype)

    def _primitive(self, x):
        """F(x) = integral of f from the first jump location to x."""
        jl = self._jump_locations.astype(np.float64)
        v = self._values.astype(np.float64)
        x = np.asarray(x, dtype=np.float64)
        # F at each jump location: F(j_0) = 0, F(j_i) = sum_{m=1..i} v_m (j_m - j_{m-1})
        Fj = np.concatenate([[0.0], np.cumsum(v[1:-1] * np.diff(jl))])
        idx = np.searchsorted(jl, x, side="left")  # x in (j_{idx-1}, j_idx]
        below = idx == 0
        i = np.clip(idx - 1, 0, len(jl) - 1)
        out = Fj[i] + v[np.clip(idx, 0, len(v) - 1)] * (x - jl[i])
        return np.where(below, v[0] * (x - jl[0]), out)


def convert_to_tensor_or_func(x, dtype=None, name=None):
    """(x, is_constant): a PiecewiseConstantFunc unchanged, else an array (piecewise.py:421-466)."""
    del name
    if isinstance(x, PiecewiseConstantFunc):
        return x, False
    return np.asarray(x, dtype=dtype), True
