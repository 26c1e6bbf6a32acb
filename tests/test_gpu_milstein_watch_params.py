"""Milstein sampling with watch_params (GPU): gradients through the per-step
autograd Function (the reference's custom for_loop gradient,
milstein_sampling.py:212-215, 389-424) against a CPU autograd restatement of
the scalar scheme and against central finite differences of the sampler
itself for d = 2 and d = 10 (the one-warp-per-path kernel)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_scalar_gbm_gradients_match_cpu_autograd(cuda):
    """d = 1: x' = x + dt mu x + sigma x dW + sigma^2 x (dW^2 - dt) / 2 with
    dW = z sqrt(dt) from the same explicit normals on the sampler's grid
    (utils.prepare_grid: 10 steps that include t = 0.5), restated in torch on
    the CPU; gradients of a path functional w.r.t. mu, sigma and x0 to 1e-11."""
    from oracle import grids as ogrids
    from tqf.models import milstein_sampling
    N, steps, order = 512, 10, 5
    grid, keep, _ = ogrids.prepare_grid(np.array([0.5, 1.0]), np.float64(0.1), np.float64, num_time_steps=steps)
    assert len(grid) == steps + 1 and keep[5]
    K = milstein_sampling.num_normal_draws(1, order)
    z = torch.randn(N, steps, K, dtype=torch.float64, generator=torch.Generator().manual_seed(3))

    def run(dev, mu, sigma, x0):
        if dev == "gpu":
            paths = milstein_sampling.sample(dim=1, drift_fn=lambda t, x: mu * x,
                                             volatility_fn=lambda t, x: (sigma * x)[..., None], times=[0.5, 1.0],
                                             num_time_steps=steps, initial_state=x0, normal_draws=z.to(cuda),
                                             watch_params=[mu, sigma], dtype=np.float64)
            return paths[:, 1, 0].sum() + 0.5 * paths[:, 0, 0].sum()
        x = x0.expand(N)
        mid = None
        for i in range(steps):
            dt = float(grid[i + 1] - grid[i])
            dw = z[:, i, 0] * dt ** 0.5
            x = x + dt * mu * x + sigma * x * dw + sigma * x * sigma * (dw * dw - dt) / 2
            if i == 4:
                mid = x
        return x.sum() + 0.5 * mid.sum()

    grads = {}
    for dev in ("gpu", "cpu"):
        where = cuda if dev == "gpu" else "cpu"
        mu = torch.tensor(0.05, dtype=torch.float64, device=where, requires_grad=True)
        sigma = torch.tensor(0.3, dtype=torch.float64, device=where, requires_grad=True)
        x0 = torch.tensor([1.2], dtype=torch.float64, device=where, requires_grad=True)
        L = run(dev, mu, sigma, x0)
        L.backward()
        grads[dev] = [float(L.detach()), float(mu.grad), float(sigma.grad), float(x0.grad.sum())]
    np.testing.assert_allclose(grads["gpu"], grads["cpu"], rtol=1e-11)


def _model(dim, kappa, sigma, theta=1.0, rho=0.4):
    c = torch.full((dim, dim), rho, dtype=torch.float64)
    c.fill_diagonal_(1.0)
    C = torch.linalg.cholesky(c).to(kappa.device)

    def drift(t, x):
        return kappa * (theta - x)

    def vol(t, x):
        return sigma * x[..., :, None] * C

    return drift, vol


@pytest.mark.parametrize("dim", [2, 10])
def test_multidimensional_gradients_match_finite_differences(cuda, dim):
    from tqf.models import milstein_sampling
    N, steps, order = 256, 8, 3
    K = milstein_sampling.num_normal_draws(dim, order)
    z = torch.randn(N, steps, K, dtype=torch.float64, generator=torch.Generator().manual_seed(dim)).to(cuda)
    x0 = torch.linspace(0.8, 1.2, dim, dtype=torch.float64)

    def loss(kappa, sigma, init, watch):
        drift, vol = _model(dim, kappa, sigma)
        paths = milstein_sampling.sample(dim=dim, drift_fn=drift, volatility_fn=vol, times=[0.25, 0.5],
                                         num_time_steps=steps, initial_state=init, normal_draws=z,
                                         stratonovich_order=order, watch_params=watch, dtype=np.float64)
        return (paths[:, 1] ** 2).mean() + paths[:, 0].mean(), paths

    kappa = torch.tensor(1.5, dtype=torch.float64, device=cuda, requires_grad=True)
    sigma = torch.tensor(0.4, dtype=torch.float64, device=cuda, requires_grad=True)
    init = x0.clone().to(cuda).requires_grad_(True)
    L, paths_w = loss(kappa, sigma, init, [kappa, sigma])
    L.backward()
    # the differentiable route runs the same update kernel: identical paths
    with torch.no_grad():
        _, paths = loss(kappa.detach(), sigma.detach(), x0.to(cuda), None)
    assert torch.equal(paths_w.detach(), paths)

    def fd(fn, v, h):
        with torch.no_grad():
            return float((fn(v + h) - fn(v - h)) / (2 * h))

    k0, s0 = float(kappa.detach()), float(sigma.detach())
    gk = fd(lambda v: loss(torch.tensor(v, dtype=torch.float64, device=cuda), sigma.detach(), x0.to(cuda), None)[0],
            k0, 1e-5)
    gs = fd(lambda v: loss(kappa.detach(), torch.tensor(v, dtype=torch.float64, device=cuda), x0.to(cuda), None)[0],
            s0, 1e-5)
    e = torch.zeros(dim, dtype=torch.float64)
    e[dim // 2] = 1.0
    gx = fd(lambda v: loss(kappa.detach(), sigma.detach(), (x0 + v * e).to(cuda), None)[0], 0.0, 1e-5)
    np.testing.assert_allclose([float(kappa.grad), float(sigma.grad), float(init.grad[dim // 2])], [gk, gs, gx],
                               rtol=2e-7, atol=1e-10)
