"""Longstaff–Schwartz regression Monte Carlo on the GPU
(tff/models/longstaff_schwartz/lsm.py:50-436).

``least_square_mc`` keeps the reference's signature and backward loop over
exercise dates.  With the reference's own basis and payoff factories
(``make_polynomial_basis``, ``make_basket_put_payoff``) the whole algorithm is
one native call (``tqf_lsm_price``): a gather pass, then per date one fused
pass over the paths (previous date's exercise update plus this date's masked
FP64 normal equations, the design built per path in the kernel) and one
pseudo-inverse solve.  Any other callables are evaluated by the caller's torch
code once per date and their [N, B] payoffs / [B, G, N] designs are fed to the
same kernels through ``tqf_lsm_pass`` / ``tqf_lsm_solve``.
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.models import utils
from tqf.models.longstaff_schwartz.payoff_utils import BasketPutPayoff


def polynomial_exponents(degree: int, dim: int) -> np.ndarray:
    """[(degree+1)^dim, dim] exponents, in the order of the reference's stacked
    'xy' meshgrid (lsm.py:109-117)."""
    g = np.arange(degree + 1)
    mesh = np.meshgrid(*(dim * [g]))
    return np.stack(mesh, -1).reshape(-1, dim).astype(np.int32)


class PolynomialBasis:
    """Centred tensor-product polynomial basis (lsm.py:50-125) as a callable:
    basis(sample_paths, time_index) -> [batch, (degree+1)^dim, num_samples].

    ``least_square_mc`` recognises this object and builds the design inside
    its kernels; calling it directly evaluates it on the given paths."""

    def __init__(self, degree: int):
        self.degree = int(degree)

    def __call__(self, sample_paths, time_index):
        x = sample_paths if isinstance(sample_paths, torch.Tensor) else torch.as_tensor(np.asarray(sample_paths))
        if x.dim() == 3:
            x = x.unsqueeze(0)
        sl = x[:, :, int(time_index), :].unsqueeze(2)  # [B, N, 1, d]
        centred = sl - sl.mean(dim=1, keepdim=True)
        grid = torch.as_tensor(polynomial_exponents(self.degree, x.shape[-1]), dtype=x.dtype, device=x.device)
        expo = torch.prod(centred ** grid, dim=-1)  # [B, N, G]
        return expo.permute(0, 2, 1)


def make_polynomial_basis(degree):
    """Produces the polynomial basis callable (lsm.py:50-125)."""
    return PolynomialBasis(int(degree))


def _discount_table(discount_factors, num_ex, np_dt):
    """D[E+1, Nd, Bd] with D[0] = 1 (lsm.py:255-272)."""
    if discount_factors is None:
        d = np.ones(num_ex, np_dt)
    else:
        d = utils.to_numpy(discount_factors, np_dt)
    if d.ndim == 0:
        d = d.reshape(1, 1, 1)
    elif d.ndim == 1:
        d = d.reshape(1, 1, -1)
    elif d.ndim == 2:
        raise ValueError("discount_factors of rank 2 are not supported by the reference (lsm.py:262-266); "
                         "pass shape [num_exercise_times] or [num_samples, batch_size, num_exercise_times]")
    d = np.pad(d, [(0, 0), (0, 0), (1, 0)], constant_values=1)
    return np.ascontiguousarray(np.transpose(d, (2, 0, 1)))


def least_square_mc(sample_paths, exercise_times, payoff_fn, basis_fn, discount_factors=None,
                    num_calibration_samples=None, dtype=None, name=None):
    """Values American-style options by regression MC (lsm.py:128-295).

    Returns a tensor of shape [batch_size] (the mean present value per payoff)."""
    del name
    device = _lib.require_cuda()
    if isinstance(sample_paths, torch.Tensor):
        np_dt = utils.np_dtype(dtype) if dtype is not None else utils.np_dtype(sample_paths.dtype)
    else:
        np_dt = utils.np_dtype(dtype) if dtype is not None else utils.infer_dtype(np.asarray(sample_paths))
    td = utils.torch_dtype(np_dt)
    if isinstance(sample_paths, torch.Tensor):
        x = sample_paths.to(device=device, dtype=td)
    else:
        x = torch.as_tensor(utils.to_numpy(sample_paths, np_dt)).to(device)
    if x.dim() not in (3, 4):
        raise ValueError(f"sample_paths must have rank 3 or 4, got shape {tuple(x.shape)}")
    x = x.contiguous()
    ex = [int(e) for e in utils.to_numpy(exercise_times).reshape(-1)]
    E = len(ex)
    if E < 1:
        raise ValueError("exercise_times must not be empty")
    N, T, dim = int(x.shape[-3]), int(x.shape[-2]), int(x.shape[-1])
    if any(e < 0 or e >= T for e in ex):
        raise ValueError(f"exercise_times must lie in [0, {T - 1}]")
    paths_batch = int(x.shape[0]) if x.dim() == 4 else 1
    structured = isinstance(payoff_fn, BasketPutPayoff) and isinstance(basis_fn, PolynomialBasis)

    cache = {}

    def explicit(t):
        if t not in cache:
            ev = payoff_fn(x, t)
            ev = (ev if isinstance(ev, torch.Tensor) else torch.as_tensor(np.asarray(ev)))
            ev = ev.to(device=device, dtype=td)
            if ev.dim() == 1:
                ev = ev.unsqueeze(-1)
            des = basis_fn(x, t)
            des = (des if isinstance(des, torch.Tensor) else torch.as_tensor(np.asarray(des)))
            des = des.to(device=device, dtype=td)
            if des.dim() == 2:
                des = des.unsqueeze(0)
            cache.clear()
            cache[t] = (ev, des)
        return cache[t]

    if structured:
        strikes = basis_strikes = np.asarray(payoff_fn.strikes, np_dt).reshape(-1)
        B = max(len(strikes), paths_batch)
        if len(strikes) not in (1, B) or paths_batch not in (1, B):
            raise ValueError("strikes and the batch of sample_paths must broadcast")
        strikes_t = utils.upload(np.broadcast_to(basis_strikes, (B,)), td, device)
        G = (basis_fn.degree + 1) ** dim
        exps_t = utils.upload(polynomial_exponents(basis_fn.degree, dim), torch.int32, device)
        design_batch = paths_batch
    else:
        ev0, des0 = explicit(ex[E - 1])
        B = int(ev0.shape[1])
        G = int(des0.shape[1])
        design_batch = int(des0.shape[0])
        if design_batch not in (1, B):
            raise ValueError("the basis batch must be 1 or the payoff batch")
        strikes_t = exps_t = None
    if G > 128:
        raise ValueError(f"at most 128 basis functions are supported, got {G}")

    D = _discount_table(discount_factors, E, np_dt)
    if D.shape[0] != E + 1:
        raise ValueError("discount_factors must have one entry per exercise time")
    Nd, Bd = D.shape[1], D.shape[2]
    if Nd not in (1, N) or Bd not in (1, B):
        raise ValueError("discount_factors must broadcast to [num_samples, batch_size, num_exercise_times]")
    D_t = utils.upload(D, td, device)
    ex_t = utils.upload(np.asarray(ex, np.int32), torch.int32, device)
    state = torch.empty((2, B, N), dtype=td, device=device)  # written by the first pass before any read
    out = torch.zeros(B, dtype=torch.float64, device=device)

    a = _lib.LsmArgs()
    a.dtype = _lib.dtype_code(td)
    a.dim = dim
    a.num_paths = N
    a.num_times = T
    a.paths_batch = design_batch if not structured else paths_batch
    a.batch = B
    a.num_basis = G
    a.degree = basis_fn.degree if structured else -1
    a.num_exercise = E
    a.num_calibration = int(num_calibration_samples) if num_calibration_samples is not None else 0
    a.paths = x.data_ptr()
    a.strikes = strikes_t.data_ptr() if strikes_t is not None else None
    a.exponents = exps_t.data_ptr() if exps_t is not None else None
    a.exercise_times = ex_t.data_ptr()
    a.discount = D_t.data_ptr()
    a.disc_stride_e = Nd * Bd
    a.disc_stride_n = Bd if Nd > 1 else 0
    a.disc_stride_b = 1 if Bd > 1 else 0
    a.state = state.data_ptr()
    a.out = out.data_ptr()
    a.dev_status = _lib.status_buffer(device).data_ptr()
    ws = torch.empty(int(_lib.load().tqf_lsm_workspace_bytes(a)), dtype=torch.uint8, device=device)
    a.workspace = ws.data_ptr()
    a.workspace_bytes = ws.numel()
    stream = _lib.stream_ptr(device)
    keep = []

    def run_pass(init=0, upd=0, acc=0, final=0):
        a.init, a.upd_index, a.acc_index, a.final_pass = init, upd, acc, final
        if not structured:
            if init:
                evi, _ = explicit(ex[E - 1])
                a.init_payoff = evi.contiguous().data_ptr()
                keep.append(evi)
            if upd:
                evu, desu = explicit(ex[upd - 1])
                evu, desu = evu.contiguous(), desu.contiguous()
                keep.extend([evu, desu])
                a.upd_payoff, a.upd_design = evu.data_ptr(), desu.data_ptr()
            if acc:
                eva, desa = explicit(ex[acc - 1])
                eva, desa = eva.contiguous(), desa.contiguous()
                keep.extend([eva, desa])
                a.acc_payoff, a.acc_design = eva.data_ptr(), desa.data_ptr()
        _lib.call("tqf_lsm_pass", a, stream)

    if structured:
        _lib.call("tqf_lsm_price", a, stream)  # whole backward loop in one native call
        return out.to(td)
    if E == 1:
        run_pass(init=1, final=1)
    else:
        run_pass(init=1, acc=E - 1)
        _lib.call("tqf_lsm_solve", a, stream)
        for i in range(E - 1, 1, -1):
            run_pass(upd=i, acc=i - 1)
            _lib.call("tqf_lsm_solve", a, stream)
            if len(keep) > 8:
                del keep[:-8]
        run_pass(upd=1, final=1)
    count = N - a.num_calibration if a.num_calibration > 0 else N
    res = (out / count).to(td)
    del keep
    return res


__all__ = ["PolynomialBasis", "make_polynomial_basis", "least_square_mc", "polynomial_exponents"]
