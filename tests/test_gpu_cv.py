"""Neural control variate kernels against the oracle (GPU)."""


import numpy as np
import pytest
import torch

from oracle import euler as oeuler
from oracle import grids as ogrids
from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

KW = dict(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7, rate=0.02, expiry=1.0,
          strike=100.0, num_dates=52, num_time_steps=252)


def _oracle_pilot(cv, N, seed):
    """Same paths as mode 1 from the materialised canonical draws, in float32."""
    from tqf.math.random import RandomType
    from tqf.math.random.multivariate_normal import philox_normal_draws
    f32 = np.float32
    draws = philox_normal_draws(RandomType.STATELESS, list(seed), 2, cv.num_steps, N, torch.float32).cpu().numpy()
    grid = np.linspace(0.0, cv.T, cv.num_steps + 1).astype(f32)
    dates = (np.arange(1, cv.num_dates + 1) * (cv.T / cv.num_dates)).astype(f32)
    _, keep, ti = ogrids.prepare_grid(dates, None, f32, times_grid=grid)
    fd, fv = oeuler.heston_ft_coefficients(cv.rate, cv.kappa, cv.theta, cv.xi, cv.rho, f32)
    min_v = np.full(N, np.inf)

    def fdm(t, x):
        np.minimum(min_v, np.abs(x[..., 1]), out=min_v)
        return fd(t, x)

    x0 = np.tile(np.array([np.log(cv.spot), cv.v0], f32), (N, 1))
    keep_all = np.zeros(cv.num_steps + 1, bool)
    keep_all[ti] = True
    paths = oeuler.sample_with_draws(fdm, fv, grid, keep_all, cv.num_dates, x0, draws, f32).astype(np.float64)
    S = np.exp(paths[..., 0])
    t_d = grid[ti].astype(np.float64)
    disc = np.exp(-cv.rate * t_d)
    prev = np.concatenate([np.full((N, 1), cv.spot), disc[None, :-1] * S[:, :-1]], 1)
    dS = disc[None, :] * S - prev
    Y = np.exp(-cv.rate * float(grid[-1])) * np.maximum(S.mean(1) - cv.strike, 0)
    feats = np.zeros((N, cv.num_dates, 3))
    feats[:, 0] = [0.0, np.log(cv.spot), cv.v0]
    feats[:, 1:, 0] = t_d[None, :-1]
    feats[:, 1:, 1] = paths[:, :-1, 0]
    feats[:, 1:, 2] = paths[:, :-1, 1]
    # control intervals: start features at the previous control date, and the
    # discounted-spot increments summed over the held dates in between
    starts = np.r_[0, cv.control_dates[:-1] + 1]
    return feats[:, starts], np.add.reduceat(dS, starts, axis=1), Y, min_v > 1e-4


@pytest.mark.parametrize("every", [1, 2, 3])
def test_pilot_matches_oracle(cuda, every):
    from tqf.pricing import HestonAsianCV
    cv = HestonAsianCV(**KW, control_every=every)
    assert cv.num_control == len(range(51, -1, -every))
    N, seed = 2048, (5, 9)
    feats, dS, Y = cv.pilot(N, seed=seed)
    of, odS, oY, ok = _oracle_pilot(cv, N, seed)
    assert ok.mean() > 0.95
    f = feats.cpu().numpy()[ok]
    np.testing.assert_allclose(f[..., 0], of[ok][..., 0], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(f[..., 1], of[ok][..., 1], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(f[..., 2], of[ok][..., 2], rtol=1e-4, atol=2e-6)
    np.testing.assert_allclose(dS.cpu().numpy()[ok], odS[ok], rtol=1e-3, atol=5e-3)
    np.testing.assert_allclose(Y.cpu().numpy()[ok], oY[ok], rtol=1e-4, atol=2e-4)


def test_fused_inference_matches_network_restatement(cuda):
    """Mode 2 (network on the tensor cores inside the path kernel) against the
    restated network applied to the same paths' pilot data."""
    from tqf.pricing import HestonAsianCV
    cv = HestonAsianCV(**KW, init_seed=3)
    N, seed = 4096, (7, 1)
    feats, dS, Y = cv.pilot(N, seed=seed)
    est = cv.price(N, control_variate=True, seed=seed)
    params = cv.params.cpu()
    g = omlp.network(params, feats.cpu()[..., :3].double().float(), cv.feat_scale, cv.feat_shift)
    C = (g.double() * dS.cpu().double()).sum(-1)
    np.testing.assert_allclose(est.plain_price, float(Y.double().mean()), rtol=1e-6)
    np.testing.assert_allclose(est.mean_control, float(C.mean()), rtol=2e-2, atol=2e-3 * float(C.abs().mean()))


@pytest.mark.parametrize("every", [1, 2])
def test_fused_inference_per_path_matches_network_restatement(cuda, every):
    """Elementwise: each path's control C = sum_j g_j dS~_j from the fused
    kernel against the restated network applied to the same path's pilot
    features and increments, and each path's payoff Y against the pilot's.
    The kernel's SFU tanh differs from the exact tanh by about one BF16 ulp in
    some activations, so each g moves by a fraction of a percent; a flip in a
    layer-1 activation reaches every layer-2 unit, which makes a few paths'
    errors several times the typical one (measured on GB300 for this case:
    median 0.0023, 99th percentile 0.013, max 0.045 of rms(C_ref)).  Bounds:
    median of |C - C_ref| within 0.005 rms(C_ref), 99th percentile within
    0.02 rms(C_ref), every path within 0.08 rms(C_ref) + 0.01 |C_ref|."""
    from tqf.pricing import HestonAsianCV
    cv = HestonAsianCV(**KW, init_seed=3, control_every=every)
    N, seed = 8192, (7, 1)
    feats, dS, Y = cv.pilot(N, seed=seed)
    pv = torch.empty((N, 2), dtype=torch.float32, device=cuda)
    est = cv.price(N, control_variate=True, seed=seed, path_values=pv)
    pv = pv.cpu().double()
    g = omlp.network(cv.params.cpu(), feats.cpu()[..., :3].float(), cv.feat_scale, cv.feat_shift)
    C_ref = (g.double() * dS.cpu().double()).sum(-1)
    np.testing.assert_allclose(pv[:, 0].numpy(), Y.cpu().double().numpy(), rtol=1e-6, atol=1e-6)
    err = (pv[:, 1] - C_ref).abs()
    rms = float(C_ref.pow(2).mean().sqrt())
    q = [float(torch.quantile(err, p)) / rms for p in (0.5, 0.9, 0.99, 0.999)] + [float(err.max()) / rms]
    assert q[0] <= 0.005 and q[2] <= 0.02, q
    bound = 0.08 * rms + 0.01 * C_ref.abs()
    assert not bool((err > bound).any()), (int((err > bound).sum()), q)
    # the per-path values are the ones the five sums reduce
    np.testing.assert_allclose(est.mean_control, float(pv[:, 1].mean()), rtol=1e-5, atol=1e-7)
    plain = torch.empty((N, 2), dtype=torch.float32, device=cuda)
    cv.price(N, control_variate=False, seed=seed, path_values=plain)
    assert torch.equal(plain[:, 0].cpu().double(), pv[:, 0]) and not bool(plain[:, 1].any())


@pytest.mark.parametrize("every", [1, 2])
def test_train_step_gradient_matches_autograd(cuda, every):
    from tqf.pricing import HestonAsianCV
    cv = HestonAsianCV(**KW, init_seed=11, control_every=every)
    cv.pilot(4096, seed=(2, 2))
    B = 128
    grad, loss = cv.gradient(0, B)
    params = cv.params.cpu().clone().requires_grad_(True)
    feats = cv.feats.cpu()[:B, :, :3]
    L = omlp.loss(params, feats, cv.dS.cpu()[:B], cv.Y.cpu()[:B], cv.feat_scale, cv.feat_shift)
    L.backward()
    ref = params.grad
    got = grad.cpu()
    np.testing.assert_allclose(loss, float(L), rtol=2e-2)
    # Elementwise, per parameter block: |got - ref| <= 0.04 rms(ref block) +
    # 0.02 |ref|.  The kernels' SFU tanh differs from the exact tanh of the
    # restatement by about one BF16 ulp in some activations, which moves
    # elements by up to ~2 % of the block's rms (measured: W1 2.1 %, W2 1.6 %,
    # b2 0.4 %, w3 0.2 %); an element of the wrong sign fails unless it is
    # below ~2 % of the rms.
    blocks = {"W1": (0, 1024), "W2": (1024, 5120), "b2": (5120, 5184), "w3": (5184, 5248), "b3": (5248, 5249),
              "c": (5249, 5250)}
    for name, (a, b) in blocks.items():
        r, gg = ref[a:b].double(), got[a:b].double()
        rms = float(r.pow(2).mean().sqrt())
        bound = 0.04 * rms + 0.02 * r.abs()
        bad = (gg - r).abs() > bound
        assert not bool(bad.any()), (name, int(bad.sum()), float(((gg - r).abs() / rms).max()))


@pytest.mark.parametrize("every", [1, 2])
def test_trained_control_variate_is_unbiased_and_reduces_variance(cuda, every):
    from tqf.pricing import HestonAsianCV
    cv = HestonAsianCV(**KW, control_every=every)
    cv.pilot(1 << 16, seed=(8, 8))
    base = cv.price(1 << 16, control_variate=True, seed=(3, 5))  # untrained network: unbiased, no gain expected
    assert abs(base.mean_control) < 5 * base.se_control
    losses = cv.train(steps=400, batch_paths=2048)
    assert losses[-1] < losses[0]
    est = cv.price(1 << 18, control_variate=True, seed=(13, 17))
    assert abs(est.mean_control) < 5 * est.se_control  # E[C] = 0
    assert est.vrf > 5.0, est.vrf
    assert abs(est.price - est.plain_price) < 5 * est.plain_standard_error


@pytest.mark.parametrize("every", [1, 2])
def test_fused_inference_pipeline_staging_is_exact(cuda, every):
    """The inference pipeline stages run at marked steps or all at the date:
    the same arithmetic either way, so the five sums agree bit for bit."""
    from tqf.pricing import HestonAsianCV
    a = HestonAsianCV(**KW, init_seed=5, control_every=every)
    b = HestonAsianCV(**KW, init_seed=5, pipeline_stages=False, control_every=every)
    ea = a.price(1 << 15, control_variate=True, seed=(4, 4))
    eb = b.price(1 << 15, control_variate=True, seed=(4, 4))
    assert (ea.price, ea.mean_control, ea.var_cv) == (eb.price, eb.mean_control, eb.var_cv)
    assert ea.mean_control != 0.0
