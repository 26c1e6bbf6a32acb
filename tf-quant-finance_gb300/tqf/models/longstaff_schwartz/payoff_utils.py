"""Basket put payoff for the regression Monte Carlo (payoff_utils.py:27-98)."""

from __future__ import annotations

import numpy as np
import torch

from tqf.models import utils


class BasketPutPayoff:
    """relu(K - mean_d S[..., t, d]) as a callable (payoff_utils.py:61-98).

    ``least_square_mc`` recognises this object and computes the payoff inside
    its kernels; calling it directly evaluates it on the given paths."""

    def __init__(self, strikes, dtype=None):
        np_dt = None if dtype is None else utils.np_dtype(dtype)
        self.strikes = np.asarray(utils.to_numpy(strikes, np_dt)).reshape(-1)
        self.dtype = dtype

    def __call__(self, sample_paths, time_index):
        x = sample_paths if isinstance(sample_paths, torch.Tensor) else torch.as_tensor(np.asarray(sample_paths))
        if x.dim() == 3:
            x = x.unsqueeze(1)  # [N, 1, T, d]
        else:
            x = x.permute(1, 0, 2, 3)  # [N, B, T, d]
        avg = x[:, :, int(time_index), :].mean(dim=-1)
        k = torch.as_tensor(self.strikes, dtype=x.dtype, device=x.device)
        return torch.relu(k - avg)


def make_basket_put_payoff(strikes, dtype=None, name=None):
    """Produces the basket put payoff callable (payoff_utils.py:27-58)."""
    del name
    return BasketPutPayoff(strikes, dtype)


__all__ = ["BasketPutPayoff", "make_basket_put_payoff"]
