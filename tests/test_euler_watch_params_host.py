"""The watch_params route of euler_sampling.sample (CPU, host logic).

With watch_params the reference runs its accumulating for_loop
(euler_sampling.py:467-510, custom_loops.py:342-424) so that gradients of the
paths with respect to the watched parameters are available.  Here the states
stay in the autograd graph and each step is an autograd Function whose
forward is the device step (tqf_euler_update) and whose backward is the Euler
step's chain rule.  This test replaces the device step with the same update
written in torch on the CPU and checks the graph wiring (recorded slots, the
initial-state slot, drift and volatility callables that close over watched
parameters) and the hand-written backward against plain torch autograd of the
recursion and against the closed-form derivative of a GBM Euler path.
"""

import numpy as np
import torch

STEPS, M = 6, 5


def _z():
    return torch.from_numpy(np.random.default_rng(3).standard_normal((STEPS, M, 2)))


def _fake_run_update(x, a, B, step, dt, sqrt_dt, draws, paths, slot, num_slots, device, need_dw, aux=None):
    # x_next = x + dt a + B (z sqrt dt), the update tqf_euler_update computes
    dw = _z()[step, :, : x.shape[1]].to(x.dtype) * sqrt_dt
    x_next = x + dt * a + torch.einsum("mrc,mc->mr", B, dw)
    if paths is not None and slot >= 0:
        paths[:, slot] = x_next
    return x_next, (dw if need_dw else None)


def _grid():
    all_times = np.linspace(0.0, 1.0, STEPS + 1)
    dt = np.diff(all_times)
    step_slot = np.full(STEPS, -1, np.int64)
    step_slot[1] = 1  # x_2 -> slot 1
    step_slot[STEPS - 1] = 2  # x_6 -> slot 2
    return all_times, dt, np.sqrt(dt), step_slot


def _run(monkeypatch, dim, drift_fn, vol_fn, x0, init_slot):
    import tqf.models.euler_sampling as es
    monkeypatch.setattr(es, "_run_update", _fake_run_update)
    all_times, dt, sqrt_dt, step_slot = _grid()
    return es._generic(dim, drift_fn, vol_fn, all_times, dt, sqrt_dt, step_slot, init_slot, STEPS, x0, (), M,
                       M, None, (M, 3, dim), 3, torch.float64, torch.device("cpu"), differentiable=True)


def _plain(dim, drift_fn, vol_fn, x0, init_slot):
    all_times, dt, sqrt_dt, step_slot = _grid()
    z = _z()
    x = torch.broadcast_to(x0, (M, dim))
    rec = [torch.zeros(M, dim, dtype=torch.float64)] * 3
    if init_slot >= 0:
        rec[init_slot] = x
    for i in range(STEPS):
        t = torch.tensor(all_times[i + 1], dtype=torch.float64)
        a = torch.broadcast_to(drift_fn(t, x), (M, dim))
        B = torch.broadcast_to(vol_fn(t, x), (M, dim, dim))
        x = x + dt[i] * a + torch.einsum("mrc,mc->mr", B, z[i, :, :dim] * sqrt_dt[i])
        if step_slot[i] >= 0:
            rec[int(step_slot[i])] = x
    return torch.stack(rec, 1)


def test_gbm_gradients_match_autograd_and_closed_form(monkeypatch):
    mu = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    sigma = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    x0 = torch.tensor([100.0], dtype=torch.float64, requires_grad=True)
    drift = lambda t, x: mu * x  # noqa: E731
    vol = lambda t, x: (sigma * x)[..., None]  # noqa: E731
    paths = _run(monkeypatch, 1, drift, vol, x0, init_slot=0)
    want = _plain(1, drift, vol, x0, init_slot=0)
    np.testing.assert_allclose(paths.detach().numpy(), want.detach().numpy(), rtol=1e-14)
    np.testing.assert_array_equal(paths[:, 0, 0].detach().numpy(), np.full(M, 100.0))
    g = torch.autograd.grad(paths.sum(), (mu, sigma, x0))
    w = torch.autograd.grad(want.sum(), (mu, sigma, x0))
    for a, b in zip(g, w):
        np.testing.assert_allclose(a.numpy(), b.numpy(), rtol=1e-12)
    # closed form: the Euler GBM path is x0 prod_i (1 + mu dt_i + sigma dw_i)
    _, dt, sqrt_dt, _ = _grid()
    dw = _z()[:, :, 0].numpy() * sqrt_dt[:, None]
    f = 1.0 + 0.05 * dt[:, None] + 0.2 * dw  # [steps, M]
    x_last = 100.0 * f.prod(0)
    np.testing.assert_allclose(paths[:, 2, 0].detach().numpy(), x_last, rtol=1e-13)
    d_sigma_last = x_last * (dw / f).sum(0)
    x_2 = 100.0 * f[:2].prod(0)
    d_sigma = d_sigma_last.sum() + (x_2 * (dw[:2] / f[:2]).sum(0)).sum()
    np.testing.assert_allclose(float(g[1]), d_sigma, rtol=1e-12)


def test_two_factor_state_dependent_volatility(monkeypatch):
    kappa = torch.tensor(1.5, dtype=torch.float64, requires_grad=True)
    xi = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    rho = torch.tensor(-0.6, dtype=torch.float64, requires_grad=True)

    def drift(t, x):
        return torch.stack([-0.5 * x[..., 1], kappa * (0.04 - x[..., 1])], -1)

    def vol(t, x):
        s = torch.sqrt(torch.clamp(x[..., 1], min=0.0))
        z = torch.zeros_like(s)
        row0 = torch.stack([s, z], -1)
        row1 = torch.stack([xi * rho * s, xi * torch.sqrt(1 - rho * rho) * s], -1)
        return torch.stack([row0, row1], -2)

    x0 = torch.tensor([np.log(100.0), 0.04], dtype=torch.float64)
    paths = _run(monkeypatch, 2, drift, vol, x0, init_slot=-1)
    want = _plain(2, drift, vol, x0, init_slot=-1)
    np.testing.assert_allclose(paths.detach().numpy(), want.detach().numpy(), rtol=1e-13, atol=1e-15)
    assert float(paths[:, 0].detach().abs().max()) == 0.0  # slot 0 is never recorded here: it stays zero
    g = torch.autograd.grad((paths[:, 2, 0] ** 2).sum() + paths[:, 1, 1].sum(), (kappa, xi, rho))
    w = torch.autograd.grad((want[:, 2, 0] ** 2).sum() + want[:, 1, 1].sum(), (kappa, xi, rho))
    for a, b in zip(g, w):
        np.testing.assert_allclose(a.numpy(), b.numpy(), rtol=1e-11)
