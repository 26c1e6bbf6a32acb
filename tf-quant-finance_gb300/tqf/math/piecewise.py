"""Piecewise-constant functions with batch and event shapes (tff/math/piecewise.py:19-208).

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
        if dtype is None:
            # TensorFlow's conversion: an array keeps its float dtype, Python
            # numbers become float32
            given = getattr(jump_locations, "dtype", None)
            given = np.dtype(str(given).replace("torch.", "")) if given is not None else None
            dtype = given if given is not None and given.kind == "f" else np.dtype(np.float32)
        jl = np.asarray(jump_locations, dtype=dtype)
        self._dtype = dtype
        self._jump_locations = jl.astype(self._dtype)
        self._values = np.asarray(values, dtype=self._dtype)
        if self._jump_locations.size == 0 and self._jump_locations.ndim == 1 and self._values.ndim == 2 \
                and self._values.shape[-1] == 1 and self._values.shape[0] > 1:
            # [[]] * batch style with values [batch, 1]
            self._jump_locations = np.zeros((self._values.shape[0], 0), self._dtype)
        self._batch_shape = self._jump_locations.shape[:-1]
        self._batch_rank = len(self._batch_shape)
        nb = self._batch_rank
        if self._values.shape[:nb] != self._batch_shape:
            raise ValueError("Batch shapes of `values` and `jump_locations` should be the same but are "
                             f"{self._values.shape[:nb]} and {self._batch_shape}")
        if self._values.ndim <= nb or self._values.shape[nb] != self._jump_locations.shape[-1] + 1:
            raise ValueError(
                "Event shape of `values` should have one more element than the event shape of "
                f"`jump_locations` but are {self._values.shape[nb:nb + 1]} and {self._jump_locations.shape[-1:]}")
        # values[..., i, *event] holds on (jump_{i-1}, jump_i]
        self._event_shape = self._values.shape[nb + 1:]

    def dtype(self):
        return self._dtype

    def values(self):
        return self._values

    def jump_locations(self):
        return self._jump_locations

    def name(self):
        return self._name

    def _rows(self, x):
        """(jumps [B, n], values [B, n + 1, *event], x [B, m], output batch shape)."""
        x = np.asarray(x, dtype=self._dtype)
        bs = self._batch_shape
        if bs and x.shape[:-1] != bs:
            x = np.broadcast_to(x, bs + x.shape[-1:])
        B = int(np.prod(bs)) if bs else 1
        n = self._jump_locations.shape[-1]
        jl = self._jump_locations.reshape(B, n)
        v = self._values.reshape((B, n + 1) + self._event_shape)
        xs = x.reshape((B, -1)) if bs else x.reshape(1, -1)
        return jl, v, xs, x.shape

    def __call__(self, x, left_continuous=True, name=None):
        """values[i] on (jump_{i-1}, jump_i] (left-continuous) or on
        [jump_{i-1}, jump_i) (right-continuous), per batch member
        (piecewise.py:144-176); output shape x.shape + event_shape."""
        del name
        side = "left" if left_continuous else "right"
        jl, v, xs, shape = self._rows(x)
        idx = np.stack([np.searchsorted(jl[b], xs[b], side=side) for b in range(jl.shape[0])])
        out = v[np.arange(jl.shape[0])[:, None], idx]
        return out.reshape(shape + self._event_shape).astype(self._dtype)

    def integrate(self, x1, x2, name=None):
        """Integral of f over [x1, x2] per batch member and element
        (piecewise.py:178-208)."""
        del name
        x1 = np.asarray(x1, dtype=self._dtype)
        x2 = np.asarray(x2, dtype=self._dtype)
        x1, x2 = np.broadcast_arrays(x1, x2)
        return (self._primitive(x2) - self._primitive(x1)).astype(self._dtype)

    def _primitive(self, x):
        """F(x) = integral of f from the first jump location to x (float64)."""
        jl, v, xs, shape = self._rows(x)
        jl, v, xs = jl.astype(np.float64), v.astype(np.float64), xs.astype(np.float64)
        ev = (1,) * len(self._event_shape)
        out = []
        for b in range(jl.shape[0]):
            j, vb, xb = jl[b], v[b], xs[b]
            if len(j) == 0:
                out.append(vb[0][None] * xb.reshape((-1,) + ev))
                continue
            # F at the jump locations: F(j_0) = 0, F(j_i) = sum_{m=1..i} v_m (j_m - j_{m-1})
            Fj = np.concatenate([np.zeros((1,) + vb.shape[1:]),
                                 np.cumsum(vb[1:-1] * np.diff(j).reshape((-1,) + ev), axis=0)])
            idx = np.searchsorted(j, xb, side="left")  # x in (j_{idx-1}, j_idx]
            i = np.clip(idx - 1, 0, len(j) - 1)
            dx = (xb - j[i]).reshape((-1,) + ev)
            inside = Fj[i] + vb[np.clip(idx, 0, len(vb) - 1)] * dx
            below = vb[0][None] * (xb - j[0]).reshape((-1,) + ev)
            out.append(np.where((idx == 0).reshape((-1,) + ev), below, inside))
        return np.stack(out).reshape(shape + self._event_shape)


def convert_to_tensor_or_func(x, dtype=None, name=None):
    """(x, is_constant): a PiecewiseConstantFunc unchanged, else an array (piecewise.py:421-466)."""
    del name
    if isinstance(x, PiecewiseConstantFunc):
        return x, False
    return np.asarray(x, dtype=dtype), True
