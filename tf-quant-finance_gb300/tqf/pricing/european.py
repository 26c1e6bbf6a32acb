"""European payoff statistics over stored terminal values (``tqf_european_payoff_sums``)."""

from __future__ import annotations

import dataclasses

import numpy as np
import torch

from tqf import _lib
from tqf.models import utils

_workspaces: dict[tuple[int, str], torch.Tensor] = {}
_ws_bytes: dict[tuple, int] = {}  # workspace sizes per (tag, device, strikes, paths, dtype)


def workspace(nbytes: int, device: torch.device, tag: str) -> torch.Tensor:
    """Reusable device scratch of at least `nbytes` bytes (per device and tag)."""
    idx = device.index if device.index is not None else torch.cuda.current_device()
    key = (idx, tag)
    buf = _workspaces.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)
        _workspaces[key] = buf
    return buf


@dataclasses.dataclass
class MonteCarloResult:
    """Discounted prices and standard errors per strike (FP64, on device)."""

    price: torch.Tensor
    standard_error: torch.Tensor
    sums: torch.Tensor  # [n_strikes, 2] raw (sum, sum of squares) of undiscounted payoffs
    num_paths: int
    discount: float
    stats: "torch.Tensor | None" = None  # [2, n_strikes]: price and standard_error are its rows

    def to_host(self):
        """(price, standard_error) as host arrays, read with one device-to-host copy."""
        if self.stats is not None:
            both = self.stats.cpu().numpy()
            return both[0], both[1]
        return self.price.cpu().numpy(), self.standard_error.cpu().numpy()


def stats_from_sums(sums: torch.Tensor, n: int, discount: float, stream: int | None = None) -> MonteCarloResult:
    """Discounted means and standard errors (unbiased variance) of the
    [n_strikes, 2] payoff sums, in one kernel (tqf_mc_price_stats) on
    `stream` (default: the current stream of the sums' device)."""
    ns = int(sums.shape[0])
    price_se = torch.empty((2, ns), dtype=torch.float64, device=sums.device)
    _lib.call("tqf_mc_price_stats", sums.data_ptr(), ns, int(n), float(discount), price_se.data_ptr(),
              _lib.stream_ptr(sums.device) if stream is None else stream)
    return MonteCarloResult(price=price_se[0], standard_error=price_se[1], sums=sums,
                            num_paths=n, discount=discount, stats=price_se)


def make_payoff(strikes, is_call, dtype, device, num_paths, ws_bytes_fn, tag):
    if isinstance(strikes, torch.Tensor) and strikes.dtype == dtype and not strikes.is_cuda:
        # host tensor in the compute dtype: one copy, asynchronous on the
        # current stream when the tensor is pinned (the caller keeps it
        # unchanged until the stream has passed the call, as for any
        # non-blocking copy), synchronous otherwise (non_blocking has no
        # effect on pageable memory, so no pinned-memory query is needed)
        k = strikes.reshape(-1).to(device, non_blocking=True)
    else:
        k = torch.as_tensor(utils.to_numpy(strikes, np.float64).reshape(-1), dtype=dtype).to(device)
    ns = int(k.numel())
    calls = None
    if is_call is not None:
        calls = torch.as_tensor(np.broadcast_to(np.asarray(is_call, dtype=np.uint8), (ns,)).copy()).to(device)
    out = torch.empty((ns, 2), dtype=torch.float64, device=device)  # written whole by the sum reduction
    # the size depends only on these (ws_bytes_fn is the same function of ns
    # for a given tag, device, path count and dtype)
    idx = device.index if device.index is not None else torch.cuda.current_device()
    wkey = (tag, idx, ns, num_paths, dtype)
    nbytes = _ws_bytes.get(wkey)
    if nbytes is None:
        nbytes = int(ws_bytes_fn(ns))
        _ws_bytes[wkey] = nbytes
    ws = workspace(nbytes, device, tag)
    p = _lib.Payoff()
    p.num_strikes = ns
    p.strikes = k.data_ptr()
    p.is_call = calls.data_ptr() if calls is not None else None
    p.spot_scale = 1.0
    p.out = out.data_ptr()
    p.workspace = ws.data_ptr()
    p.workspace_bytes = ws.numel()
    return p, out, (k, calls, ws)


def european_payoff_stats(values: torch.Tensor, strikes, is_call=None, discount: float = 1.0,
                          log_values: bool = False, spot_scale: float = 1.0) -> MonteCarloResult:
    """Mean discounted max(S - K, 0) (or put) over S = spot_scale * values
    (or spot_scale * exp(values)) with FP64 accumulation."""
    device = _lib.require_cuda()
    v = values.reshape(-1)
    if not v.is_contiguous():
        v = v.contiguous()
    n = int(v.numel())
    p, out, keep = make_payoff(strikes, is_call, v.dtype, device, n,
                               lambda ns: _lib.load().tqf_european_workspace_bytes(n, ns), "european")
    p.spot_scale = float(spot_scale)
    _lib.call("tqf_european_payoff_sums", _lib.dtype_code(v.dtype), v.data_ptr(), 1, n,
              1 if log_values else 0, p, _lib.stream_ptr(device))
    del keep
    return stats_from_sums(out, n, discount)
