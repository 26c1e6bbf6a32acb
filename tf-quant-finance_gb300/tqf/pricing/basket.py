"""Arithmetic-basket European option on correlated GBM with pathwise Greeks
(``tqf_basket_price``): one fused pass gives the price, its standard error,
and the pathwise delta, vega (per asset) and rho, with FP64 accumulation.

``BasketPrice`` exposes the price as a differentiable function of
(spots, vols, rate) through torch.autograd; its backward uses the pathwise
sensitivities the forward kernel accumulated on the same draws.
"""

from __future__ import annotations

import dataclasses

import numpy as np
import torch

from tqf import _lib
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import utils
from tqf.models.multivariate_gbm import cholesky_f64
from tqf.pricing.european import workspace


@dataclasses.dataclass
class BasketResult:
    price: float
    standard_error: float
    delta: torch.Tensor  # [dim]
    vega: torch.Tensor   # [dim]
    rho: float
    sums: torch.Tensor   # raw FP64 sums [2 + 2 dim]


def _run(spots, vols, rate, corr, weights, strike, expiry, num_time_steps, num_samples, random_type, seed,
         dtype, is_call, path_offset, normal_draws):
    device = _lib.require_cuda()
    td = utils.torch_dtype(dtype)
    np_dt = utils.np_dtype(td)
    spots = np.asarray(spots, np.float64).reshape(-1)
    d = spots.size
    vols = np.broadcast_to(np.asarray(vols, np.float64), (d,)).copy()
    weights = np.full(d, 1.0 / d) if weights is None else np.broadcast_to(np.asarray(weights, np.float64), (d,)).copy()
    T, r, steps, N = float(expiry), float(rate), int(num_time_steps), int(num_samples)
    grid = np.linspace(0.0, T, steps + 1).astype(np_dt)
    sdt = np.sqrt((grid[1:] - grid[:-1]).astype(np_dt)).astype(np_dt)
    dev = lambda a: torch.as_tensor(np.asarray(a, np.float64)).to(device, td)  # noqa: E731
    sdt_t, spot_t, vol_t, w_t = dev(sdt), dev(spots), dev(vols), dev(weights)
    drift_t = dev(r - vols ** 2 / 2)
    chol = cholesky_f64(corr, device).to(td) if corr is not None else None
    keep = []
    if normal_draws is not None:
        keep.append(normal_draws)
        draws = mvn.memory_draws(normal_draws, path_axis=0, step_axis=1)
    elif random_type in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
        # quasi-random: [steps, N, d] normal draws (dimension step * d + asset,
        # points path_offset + 1 ...), read in place by the kernel
        q = utils.generate_mc_normal_draws(d, steps, N, random_type, skip=int(path_offset), seed=seed, dtype=td)
        keep.append(q)
        draws = mvn.memory_draws(q, path_axis=1, step_axis=0)
    else:
        draws = mvn.philox_draws(random_type, seed, N, path_offset)
    out = torch.zeros(2 + 2 * d, dtype=torch.float64, device=device)
    nbytes = int(_lib.load().tqf_basket_workspace_bytes(_lib.dtype_code(td), d, N))
    ws = workspace(nbytes, device, "basket")
    a = _lib.BasketArgs()
    a.dtype = _lib.dtype_code(td)
    a.dim = d
    a.num_paths = N
    a.num_steps = steps
    a.is_call = 1 if is_call else 0
    a.sqrt_dt = sdt_t.data_ptr()
    a.total_time = float(np_dt.type(grid[-1]))
    a.strike = float(strike)
    a.spot, a.drift, a.vol, a.weights = spot_t.data_ptr(), drift_t.data_ptr(), vol_t.data_ptr(), w_t.data_ptr()
    a.chol = chol.data_ptr() if chol is not None else None
    a.draws = draws
    a.out = out.data_ptr()
    a.workspace = ws.data_ptr()
    a.workspace_bytes = ws.numel()
    a.dev_status = _lib.status_buffer(device).data_ptr()
    _lib.call("tqf_basket_price", a, _lib.stream_ptr(device))
    return out, spots, vols, T, r, N, d


def basket_european_mc(*, spots, vols, rate, corr, strike, expiry, num_time_steps, num_samples, weights=None,
                       is_call=True, random_type=RandomType.STATELESS, seed=(1, 2), dtype=torch.float32,
                       path_offset=0, normal_draws=None) -> BasketResult:
    out, spots, vols, T, r, N, d = _run(spots, vols, rate, corr, weights, strike, expiry, num_time_steps,
                                        num_samples, random_type, seed, dtype, is_call, path_offset, normal_draws)
    s = out.cpu().numpy()
    disc = np.exp(-r * T)
    mean = s[0] / N
    var = max(s[1] / N - mean * mean, 0.0) * N / max(N - 1, 1)
    g = s[2:2 + d] / N
    gv = s[2 + d:2 + 2 * d] / N
    price = disc * mean
    return BasketResult(price=float(price), standard_error=float(disc * np.sqrt(var / N)),
                        delta=torch.as_tensor(disc * g / spots), vega=torch.as_tensor(disc * gv),
                        rho=float(-T * price + disc * g.sum() * T), sums=out)


class BasketPrice(torch.autograd.Function):
    """price = BasketPrice.apply(spots[d], vols[d], rate[], kwargs) (float64)."""

    @staticmethod
    def forward(ctx, spots, vols, rate, kw):
        res = basket_european_mc(spots=spots.detach().cpu().numpy(), vols=vols.detach().cpu().numpy(),
                                 rate=float(rate), **kw)
        ctx.save_for_backward(res.delta, res.vega, torch.tensor(res.rho, dtype=torch.float64))
        return torch.tensor(res.price, dtype=torch.float64, device=spots.device)

    @staticmethod
    def backward(ctx, g):
        delta, vega, rho = ctx.saved_tensors
        dev = g.device
        return (g * delta.to(dev), g * vega.to(dev), g * rho.to(dev), None)


__all__ = ["basket_european_mc", "BasketPrice", "BasketResult"]
