"""watch_params in euler_sampling.sample (GPU).

With watch_params the reference switches to its accumulating for_loop
(euler_sampling.py:467-510, custom_loops.py:20-214) so that the paths can be
differentiated with respect to the watched parameters; the paths themselves
are unchanged.  Here every step runs in tqf_euler_update and its backward is
the Euler step's chain rule.  The paths must equal those of the plain route
bit for bit, and the gradients must equal torch autograd of the same
recursion on the CPU in float64 given the same normal_draws (1e-9 relative),
or central finite differences with common random numbers for in-kernel
Philox draws (1e-6 relative).
"""

import numpy as np
import pytest
import torch

from oracle import grids as ogrids

pytestmark = pytest.mark.gpu

MU, SIGMA = [0.02, 0.05], [0.2, 0.3]
CORR = np.array([[1.0, 0.4], [0.4, 1.0]])


def _coefficients(mu, sigma, chol):
    return (lambda t, x: mu * x), (lambda t, x: (sigma * x)[..., None] * chol)


def _leaf(values, device):
    return torch.tensor(values, dtype=torch.float64, device=device, requires_grad=True)


def test_gradients_match_autograd_of_the_recursion(cuda):
    from tqf.models import euler_sampling
    N, d, steps = 2000, 2, 10
    times = np.array([0.5, 1.0])
    draws = np.random.default_rng(5).standard_normal((N, steps, d))
    w = torch.from_numpy(np.random.default_rng(6).standard_normal((N, 2, d)))
    chol = np.linalg.cholesky(CORR)
    mu, sigma, x0 = _leaf(MU, cuda), _leaf(SIGMA, cuda), _leaf([1.0, 2.0], cuda)
    drift, vol = _coefficients(mu, sigma, torch.from_numpy(chol).to(cuda))
    kw = dict(num_time_steps=steps, normal_draws=draws, dtype=torch.float64)
    paths = euler_sampling.sample(d, drift, vol, times, initial_state=x0, watch_params=[mu, sigma], **kw)
    plain = euler_sampling.sample(d, drift, vol, times, initial_state=x0.detach(), **kw)
    assert paths.shape == (N, 2, d) and paths.requires_grad
    np.testing.assert_array_equal(paths.detach().cpu().numpy(), plain.cpu().numpy())
    got = torch.autograd.grad((paths * w.to(cuda)).sum(), (mu, sigma, x0))

    # the same recursion in torch on the CPU, float64
    all_t, keep, _ = ogrids.prepare_grid(times, times[-1] / steps, np.float64, num_time_steps=steps)
    cmu, csig, cx0 = _leaf(MU, "cpu"), _leaf(SIGMA, "cpu"), _leaf([1.0, 2.0], "cpu")
    cdrift, cvol = _coefficients(cmu, csig, torch.from_numpy(chol))
    x = torch.broadcast_to(cx0, (N, d))
    rec = []
    for i in range(len(all_t) - 1):
        dt = all_t[i + 1] - all_t[i]
        dw = torch.from_numpy(draws[:, i, :]) * np.sqrt(dt)
        x = x + dt * cdrift(None, x) + torch.einsum("mrc,mc->mr", cvol(None, x), dw)
        if keep[i + 1]:
            rec.append(x)
    want_paths = torch.stack(rec, 1)
    np.testing.assert_allclose(paths.detach().cpu().numpy(), want_paths.detach().numpy(), rtol=1e-12)
    want = torch.autograd.grad((want_paths * w).sum(), (cmu, csig, cx0))
    for g, e in zip(got, want):
        np.testing.assert_allclose(g.cpu().numpy(), e.numpy(), rtol=1e-9)


def test_philox_gradient_matches_finite_differences(cuda):
    from tqf.math.random import RandomType
    from tqf.models import euler_sampling
    N, d, steps = 4096, 2, 8
    times = np.array([1.0])
    chol = torch.from_numpy(np.linalg.cholesky(CORR)).to(cuda)
    kw = dict(num_time_steps=steps, num_samples=N, initial_state=np.array([1.0, 2.0]), seed=[4, 2],
              random_type=RandomType.STATELESS, dtype=torch.float64)

    def run(mu_values, watch):
        mu = _leaf(mu_values, cuda) if watch else torch.tensor(mu_values, dtype=torch.float64, device=cuda)
        drift, vol = _coefficients(mu, torch.tensor(SIGMA, dtype=torch.float64, device=cuda), chol)
        p = euler_sampling.sample(d, drift, vol, times, watch_params=[mu] if watch else None, **kw)
        return mu, p

    mu, paths = run(MU, True)
    np.testing.assert_array_equal(paths.detach().cpu().numpy(), run(MU, False)[1].cpu().numpy())
    (g,) = torch.autograd.grad(paths.sum(), (mu,))
    h = 1e-4
    for j in range(d):
        up, dn = list(MU), list(MU)
        up[j] += h
        dn[j] -= h
        fd = (float(run(up, False)[1].sum()) - float(run(dn, False)[1].sum())) / (2 * h)
        np.testing.assert_allclose(float(g[j]), fd, rtol=1e-6)
