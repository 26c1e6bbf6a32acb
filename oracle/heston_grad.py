"""Torch-CPU autograd restatement of the full-truncation Euler pricer: the
reference Euler sampler (tff/models/euler_sampling.py:513-537) run with the
Heston full-truncation coefficients, differentiated by reverse-mode autograd
(the role tf.GradientTape plays for the reference, via custom_loops.for_loop
when watch_params is given, tff/math/custom_loops.py:20-214)."""

from __future__ import annotations

import numpy as np


def price_and_grad(params, strikes, weights, expiry, draws):
    """params: (spot, v0, kappa, theta, xi, rho, r) floats; draws [N, steps, 2]
    (component 0 drives the log-spot).  Returns (prices [ns], grad [7]) of
    sum_j weights_j price_j."""
    import torch
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    spot, v0, kappa, theta, xi, rho, r = p
    N, steps, _ = draws.shape
    z = torch.as_tensor(draws, dtype=torch.float64)
    t = torch.linspace(0.0, expiry, steps + 1, dtype=torch.float64)
    dt = t[1:] - t[:-1]
    x = torch.log(spot) * torch.ones(N, dtype=torch.float64)
    v = v0 * torch.ones(N, dtype=torch.float64)
    for i in range(steps):
        vp = torch.clamp(v, min=0)
        sq = torch.sqrt(vp)
        dw0 = z[:, i, 0] * torch.sqrt(dt[i])
        dw1 = z[:, i, 1] * torch.sqrt(dt[i])
        x, v = (x + dt[i] * (r - 0.5 * vp) + sq * dw0,
                v + dt[i] * (kappa * (theta - vp)) + xi * rho * sq * dw0 + xi * torch.sqrt(1 - rho * rho) * sq * dw1)
    S = torch.exp(x)
    k = torch.as_tensor(np.asarray(strikes, np.float64))
    prices = torch.exp(-r * expiry) * torch.clamp(S[:, None] - k[None, :], min=0).mean(0)
    (prices * torch.as_tensor(np.asarray(weights, np.float64))).sum().backward()
    return prices.detach().numpy(), p.grad.numpy()
