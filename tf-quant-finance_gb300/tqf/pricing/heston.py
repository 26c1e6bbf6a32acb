"""Fused Heston European pricing: path simulation, payoff over a strike
batch and FP64 accumulation in one kernel pass.

``scheme="full_truncation"``: log-spot full-truncation Euler with the rate in
the drift (``tqf_heston_euler``), the reference Euler sampler's arithmetic
for the coefficients of ``coefficients.heston_full_truncation``.
``scheme="qe"``: the reference HestonModel QE scheme (``tqf_heston_qe``);
it has no rate term, so S_T = exp(X_T + r T) as in heston_model_test.py:349-352.
Both use a uniform grid of ``num_time_steps`` steps to ``expiry``.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import heston_model
from tqf.models import utils
from tqf.models.coefficients import HestonFullTruncation
from tqf.pricing.european import make_payoff, stats_from_sums

_tables: dict = {}


def _table(key, build, td, device):
    t = _tables.get(key)
    if t is None:
        t = utils.step_table(build(), td, device)
        _tables[key] = t
    return t


_QUASI = (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED)


def _draws(random_type, seed, num_paths, num_steps, path_offset, normal_draws, td, fused_sobol=True):
    """(tqf_draws, tensor to keep alive): caller draws [N, steps, 2] read in
    place; SOBOL computed inside the pricing kernel (dimension step * 2 +
    component, points path_offset + 1 ..., the values of
    generate_mc_normal_draws with skip = path_offset); HALTON* (and SOBOL
    for the adjoint) as [steps, N, 2] normal draws generated on the device;
    otherwise the Philox stream generated inside the kernel."""
    if normal_draws is not None:
        return mvn.memory_draws(normal_draws, path_axis=0, step_axis=1), normal_draws
    if random_type == RandomType.SOBOL and fused_sobol:
        return mvn.sobol_draws(2, num_steps, num_paths, int(path_offset))
    if random_type in _QUASI:
        q = utils.generate_mc_normal_draws(2, num_steps, num_paths, random_type, skip=int(path_offset), seed=seed,
                                           dtype=td)
        return mvn.memory_draws(q, path_axis=1, step_axis=0), q
    return mvn.philox_draws(random_type, seed, num_paths, path_offset), None


def heston_european_mc(*, strikes, expiry, spot, variance, mean_reversion, theta, volvol, rho,
                       discount_rate=0.0, is_call_options=None, num_samples, num_time_steps,
                       scheme="full_truncation", random_type=RandomType.STATELESS, seed=(1, 2),
                       dtype=torch.float32, path_offset=0, normal_draws=None):
    """Returns a MonteCarloResult with per-strike discounted prices and
    standard errors (FP64 on the device).  Strikes given as a pinned host
    tensor in the compute dtype are copied asynchronously on the current
    stream (keep them unchanged until the stream has passed the call)."""
    device = _lib.require_cuda()
    td = utils.torch_dtype(dtype)
    np_dt = utils.np_dtype(td)
    T, r = float(expiry), float(discount_rate)
    steps = int(num_time_steps)
    N = int(num_samples)
    qe = scheme == "qe"
    params = (float(mean_reversion), float(theta), float(volvol), float(rho))

    def grid():  # uniform grid, built only when the step table is not cached
        all_times = np.linspace(0.0, T, steps + 1).astype(np_dt)
        dt = (all_times[1:] - all_times[:-1]).astype(np_dt)
        return all_times, dt, np.sqrt(dt).astype(np_dt), np.full(steps, -1, dtype=np.int32)

    if qe:
        key = ("qe", np_dt.str, T, steps, params, device.index)

        def build():
            all_times, _, _, no_slots = grid()
            return heston_model.HestonModel(*params, dtype=np_dt)._qe_table(all_times, 1e-6, no_slots, steps)

        tab = _table(key, build, td, device)
        x0, scale = float(np.log(spot)), float(np.exp(r * T))
    else:
        key = ("ft", np_dt.str, T, steps, params, r, device.index)

        def build():
            all_times, dt, sqrt_dt, no_slots = grid()
            return heston_model.full_truncation_table(HestonFullTruncation(r, *params), all_times, dt, sqrt_dt,
                                                      no_slots, steps)

        tab = _table(key, build, td, device)
        x0, scale = float(np.log(spot)), 1.0
    draws, draws_keep = _draws(random_type, seed, N, steps, path_offset, normal_draws, td)
    qe_flag = 1 if qe else 0
    p, out, keep = make_payoff(strikes, is_call_options, td, device, N,
                               lambda ns: _lib.load().tqf_heston_workspace_bytes(_lib.dtype_code(td), qe_flag, N, ns),
                               "heston_qe" if qe else "heston_ft")
    p.spot_scale = scale
    args = _lib.HestonArgs()
    args.dtype = _lib.dtype_code(td)
    args.num_steps = steps
    args.num_paths = N
    args.step_table = tab.data_ptr()
    args.x0, args.v0 = x0, float(variance)
    args.draws = draws
    args.payoff = p
    args.dev_status = _lib.status_buffer(device).data_ptr()
    stream = _lib.stream_ptr(device)
    _lib.call("tqf_heston_qe" if qe else "tqf_heston_euler", args, stream)
    del keep, draws_keep
    return stats_from_sums(out, N, float(np.exp(-r * T)), stream)


def heston_european_vjp(grad_prices, *, strikes, expiry, spot, variance, mean_reversion, theta, volvol, rho,
                        discount_rate=0.0, is_call_options=None, num_samples, num_time_steps,
                        random_type=RandomType.STATELESS, seed=(1, 2), dtype=torch.float32, path_offset=0,
                        normal_draws=None, prices=None):
    """Vector-Jacobian product of the full-truncation European prices with
    respect to (spot, variance, mean_reversion, theta, volvol, rho,
    discount_rate), by the replaying pathwise adjoint kernel
    (``tqf_heston_euler_adjoint``).  ``prices`` (the forward result, FP64)
    supplies the discounting term of the rate sensitivity."""
    device = _lib.require_cuda()
    td = utils.torch_dtype(dtype)
    np_dt = utils.np_dtype(td)
    T, r, steps, N = float(expiry), float(discount_rate), int(num_time_steps), int(num_samples)
    all_times = np.linspace(0.0, T, steps + 1).astype(np_dt)
    dt = (all_times[1:] - all_times[:-1]).astype(np_dt)
    sqrt_dt = np.sqrt(dt).astype(np_dt)
    params = (float(mean_reversion), float(theta), float(volvol), float(rho))
    h = HestonFullTruncation(r, *params)
    key = ("ft", np_dt.str, T, steps, params, r, device.index)
    no_slots = np.full(steps, -1, dtype=np.int32)
    tab = _table(key, lambda: heston_model.full_truncation_table(h, all_times, dt, sqrt_dt, no_slots, steps),
                 td, device)
    g = torch.as_tensor(grad_prices, dtype=torch.float64).to(device).reshape(-1)
    disc = float(np.exp(-r * T))
    k = torch.as_tensor(utils.to_numpy(strikes, np.float64).reshape(-1), dtype=td).to(device)
    ns = int(k.numel())
    w = (g * (disc / N)).to(td).contiguous()
    calls = None
    if is_call_options is not None:
        calls = torch.as_tensor(np.broadcast_to(np.asarray(is_call_options, np.uint8), (ns,)).copy()).to(device)
    draws, draws_keep = _draws(random_type, seed, N, steps, path_offset, normal_draws, td, fused_sobol=False)
    out = torch.zeros(7, dtype=torch.float64, device=device)
    from tqf.pricing.european import workspace
    ws = workspace(int(_lib.load().tqf_heston_adjoint_workspace_bytes(N)), device, "heston_adjoint")
    a = _lib.HestonAdjointArgs()
    a.dtype = _lib.dtype_code(td)
    a.num_steps = steps
    a.num_paths = N
    a.step_table = tab.data_ptr()
    a.x0, a.v0 = float(np.log(spot)), float(variance)
    a.kappa, a.theta = float(mean_reversion), float(theta)
    a.xi, a.rho = float(volvol), float(rho)
    a.draws = draws
    a.num_strikes = ns
    a.strikes = k.data_ptr()
    a.is_call = calls.data_ptr() if calls is not None else None
    a.weights = w.data_ptr()
    a.out = out.data_ptr()
    a.workspace = ws.data_ptr()
    a.workspace_bytes = ws.numel()
    a.dev_status = _lib.status_buffer(device).data_ptr()
    _lib.call("tqf_heston_euler_adjoint", a, _lib.stream_ptr(device))
    del draws_keep
    grad = out.clone()
    grad[0] = out[0] / float(spot)  # d/dS0 = (1/S0) d/dlog S0
    if prices is not None:
        grad[6] = out[6] - T * float((g * prices.to(device)).sum())
    return grad


class HestonEuropeanPrice(torch.autograd.Function):
    """prices[n_strikes] = HestonEuropeanPrice.apply(params[7], kwargs) with
    params = (spot, variance, mean_reversion, theta, volvol, rho, rate);
    full-truncation Euler, Philox draws; backward replays the paths."""

    @staticmethod
    def forward(ctx, params, kw):
        p = [float(v) for v in params.detach().cpu()]
        names = ("spot", "variance", "mean_reversion", "theta", "volvol", "rho", "discount_rate")
        args = dict(zip(names, p))
        res = heston_european_mc(**kw, **args, scheme="full_truncation")
        ctx.kw = kw
        ctx.args = args
        ctx.save_for_backward(res.price)
        return res.price.to(params.device)

    @staticmethod
    def backward(ctx, g):
        (prices,) = ctx.saved_tensors
        grad = heston_european_vjp(g, prices=prices, **ctx.kw, **ctx.args)
        return grad.to(g.device), None


__all__ = ["heston_european_mc", "heston_european_vjp", "HestonEuropeanPrice"]
