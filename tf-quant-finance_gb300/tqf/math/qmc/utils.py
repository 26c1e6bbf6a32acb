"""QMC utilities (tff/math/qmc/utils.py:23-158), torch on any device."""

from __future__ import annotations

import numpy as np
import torch


def exp2(value):
    """2 ** value for integer tensors (utils.py:23-54)."""
    v = torch.as_tensor(value)
    return torch.where(v == 0, torch.ones_like(v), torch.bitwise_left_shift(torch.ones_like(v), v))


def log2(value):
    """log(value) / log(2) in the value's float dtype (utils.py:57-77)."""
    v = torch.as_tensor(value)
    return torch.log(v) / torch.log(torch.tensor(2, dtype=v.dtype))


def get_shape(value):
    return tuple(torch.as_tensor(value).shape)


def tent_transform(value):
    """2 v for v < 1/2, else 2 (1 - v) (utils.py:94-117)."""
    v = torch.as_tensor(value)
    return torch.where(v < 0.5, 2 * v, 2 * (1 - v))


def filter_tensor(value, bit_mask, bit_index):
    """value where bit `bit_index` (LSB 0) of bit_mask is set, else 0 (utils.py:120-158)."""
    value, bit_mask, bit_index = (torch.as_tensor(x) for x in (value, bit_mask, bit_index))
    is_set = torch.bitwise_and(torch.bitwise_right_shift(bit_mask, bit_index), 1) == 1
    return torch.where(is_set, value, torch.zeros_like(value))


def log2_f32(x) -> float:
    """float32 log2 as the reference computes num_digits / log_num_results."""
    x = np.float32(x)
    return float(np.float32(np.log(x) / np.log(np.float32(2))))


__all__ = ["exp2", "log2", "get_shape", "tent_transform", "filter_tensor"]
