"""Torch-CPU restatement of the control-variate network and its loss, for
checking the kernels: BF16 rounding of the weights, the input features and
the activations as in the kernels, FP32 accumulation, and SiLU evaluated the
way the kernels do in packed BF16 — h = bf16(x)/2, t = bf16(tanh h),
silu = bf16(h + h t) (exact tanh here; the kernels' SFU tanh differs by about
one BF16 ulp).  Gradients pass straight through the roundings with the exact
SiLU derivative.  Loss: mean_p (Y_p - c - sum_k g_pk dS_pk)^2."""

from __future__ import annotations

import torch

H, IN = 64, 16
OFF_W1, OFF_W2 = 0, 64 * 16
OFF_B2 = OFF_W2 + 64 * 64
OFF_W3 = OFF_B2 + 64
OFF_B3 = OFF_W3 + 64
OFF_C = OFF_B3 + 1


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def _silu_bf16(x):
    h = _bf(x) * 0.5
    t = _bf(torch.tanh(h))
    y = _bf(h + h * t)
    exact = torch.nn.functional.silu(x)
    return exact + (y - exact).detach()


def network(params, feats, feat_scale, feat_shift):
    """g for feats [..., >=3] (t, log S, v); params FP32 [5250] (autograd-capable)."""
    w1 = params[OFF_W1:OFF_W2].reshape(H, IN)
    w2 = params[OFF_W2:OFF_B2].reshape(H, H)
    b2 = params[OFF_B2:OFF_W3]
    w3 = params[OFF_W3:OFF_B3]
    b3 = params[OFF_B3]
    f = torch.stack([(feats[..., i] - feat_shift[i]) * feat_scale[i] for i in range(3)], -1)
    x = torch.cat([f, torch.ones_like(f[..., :1]), torch.zeros(f.shape[:-1] + (IN - 4,))], -1)
    # straight-through BF16 rounding: value rounded, gradient passes unchanged
    st = lambda t: t + (_bf(t) - t).detach()  # noqa: E731
    a1 = st(x) @ st(w1).T
    h1 = _silu_bf16(a1)
    a2 = h1 @ st(w2).T + b2
    h2 = _silu_bf16(a2)
    return h2 @ w3 + b3


def loss(params, feats, dS, Y, feat_scale, feat_shift):
    g = network(params, feats, feat_scale, feat_shift)  # [B, D]
    r = Y - params[OFF_C] - (g * dS).sum(-1)
    return (r * r).mean()
