"""In-kernel Philox draws taken a whole block at a time (GPU).

When a step takes exactly 1, 2, 3 or 4 normals of the canonical stream
(draw k = step dim + c of path n, four float32 or two float64 normals per
Philox block), the Euler and exact-GBM path kernels walk groups of steps
that use lcm(dim, normals per block) draws, i.e. whole Philox blocks,
instead of testing every draw against the current block.  The paths must
equal, bit for bit, the same kernels reading the stream's materialised
normals (`generate_mc_normal_draws`, which fills element (step, n, c) from
draw step dim + c of path n): with every step recorded (warp stager) and
with the last time only, with step counts that leave a partial last group,
with antithetic pairs (the sign carried by sqrt(dt)), and for dimensions
that keep the per-draw reader (5, 8) as controls.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _draws(d, steps, n, antithetic, seed, dtype):
    from tqf.math.random import RandomType
    from tqf.models import utils
    rt = RandomType.STATELESS_ANTITHETIC if antithetic else RandomType.STATELESS
    z = utils.generate_mc_normal_draws(d, steps, n, rt, seed=seed, dtype=dtype)
    return rt, z.permute(1, 0, 2)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 8])
@pytest.mark.parametrize("steps", [37, 64])
@pytest.mark.parametrize("every", [True, False])
def test_euler_whole_blocks_equal_materialised(cuda, dtype, d, steps, every):
    from tqf.models import coefficients, euler_sampling
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    rng = np.random.default_rng(100 + d + steps)
    drift, vol = coefficients.gbm(rng.uniform(-0.05, 0.05, d), rng.uniform(0.1, 0.3, d),
                                  0.5 * np.eye(d) + 0.5)
    grid = np.linspace(0.0, 1.0, steps + 1).astype(np_dt)
    times = grid if every else grid[-1:]
    x0 = np.linspace(1.0, 2.0, d).astype(np_dt)
    N = 1000
    for antithetic in (False, True):
        rt, z = _draws(d, steps, N, antithetic, [5, 6], dtype)
        kw = dict(times_grid=grid, initial_state=x0, dtype=dtype)
        fused = euler_sampling.sample(d, drift, vol, times, num_samples=N, random_type=rt, seed=[5, 6], **kw)
        mat = euler_sampling.sample(d, drift, vol, times, normal_draws=z, **kw)
        assert fused.shape == (N, len(times), d)
        torch.testing.assert_close(fused, mat, rtol=0, atol=0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("d", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("k", [1, 37, 64])
def test_exact_gbm_whole_blocks_equal_materialised(cuda, dtype, d, k):
    from tqf.models import MultivariateGeometricBrownianMotion
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    rng = np.random.default_rng(200 + d + k)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    corr = q @ np.diag(rng.uniform(0.5, 1.5, d)) @ q.T
    s = np.sqrt(np.diag(corr))
    corr = corr / s[:, None] / s[None, :]
    proc = MultivariateGeometricBrownianMotion(d, means=rng.uniform(0.0, 0.05, d), volatilities=rng.uniform(0.1, 0.4, d),
                                               corr_matrix=corr, dtype=np_dt)
    times = np.linspace(0.0, 1.0, k + 1)[1:].astype(np_dt)
    N = 1000
    for antithetic in (False, True):
        rt, z = _draws(d, k, N, antithetic, [7, 8], dtype)
        fused = proc.sample_paths(times, initial_state=np.full(d, 100.0, np_dt), num_samples=N, random_type=rt,
                                  seed=[7, 8])
        mat = proc.sample_paths(times, initial_state=np.full(d, 100.0, np_dt), normal_draws=z)
        assert fused.shape == (N, k, d)
        torch.testing.assert_close(fused, mat, rtol=0, atol=0)


def test_univariate_gbm_whole_blocks_equal_materialised(cuda):
    from tqf.models import GeometricBrownianMotion
    proc = GeometricBrownianMotion(0.05, 0.2, dtype=np.float32)
    times = (np.arange(1, 253) / 252).astype(np.float32)
    N = 4100
    rt, z = _draws(1, 252, N, False, [1, 2], torch.float32)
    fused = proc.sample_paths(times, initial_state=100.0, num_samples=N, random_type=rt, seed=[1, 2])
    mat = proc.sample_paths(times, initial_state=100.0, normal_draws=z)
    torch.testing.assert_close(fused, mat, rtol=0, atol=0)


@pytest.mark.parametrize("d", [16, 17, 32, 64])
def test_tensor_core_gbm_whole_blocks_equal_materialised(cuda, d):
    """The tensor-core L z kernel (float32, 16 to 64 factors) takes each
    16-factor column block's draws as 4 whole Philox blocks when the factor
    count is a multiple of 16 (17 keeps the per-draw reader)."""
    from tqf.models import MultivariateGeometricBrownianMotion
    rng = np.random.default_rng(300 + d)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    corr = q @ np.diag(rng.uniform(0.5, 1.5, d)) @ q.T
    s = np.sqrt(np.diag(corr))
    corr = corr / s[:, None] / s[None, :]
    proc = MultivariateGeometricBrownianMotion(d, means=0.03, volatilities=rng.uniform(0.1, 0.4, d), corr_matrix=corr,
                                               dtype=np.float32)
    times = np.linspace(0.0, 1.0, 10)[1:].astype(np.float32)
    N = 1000
    for antithetic in (False, True):
        rt, z = _draws(d, len(times), N, antithetic, [3, 4], torch.float32)
        fused = proc.sample_paths(times, initial_state=np.full(d, 100.0, np.float32), num_samples=N, random_type=rt,
                                  seed=[3, 4], lz_mode=0)
        mat = proc.sample_paths(times, initial_state=np.full(d, 100.0, np.float32), normal_draws=z, lz_mode=0)
        torch.testing.assert_close(fused, mat, rtol=0, atol=0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("d", [3, 4, 8, 16])
def test_basket_pricing_whole_blocks_equal_materialised(cuda, dtype, d):
    """The fused basket pricer (terminal log-spots from w = sum sqrt(dt) z)
    walks whole Philox blocks when the asset count fills its register tile
    (4, 8, 16; 3 keeps the per-draw reader): prices and pathwise Greeks equal
    those from the materialised draws."""
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import basket_european_mc
    N, steps = 1 << 13, 7
    corr = 0.5 * np.eye(d) + 0.5
    kw = dict(spots=np.full(d, 100.0), vols=np.linspace(0.1, 0.4, d), rate=0.02, corr=corr, strike=100.0,
              expiry=1.0, num_time_steps=steps, num_samples=N, dtype=dtype)
    for rt in (RandomType.STATELESS, RandomType.STATELESS_ANTITHETIC):
        q = basket_european_mc(random_type=rt, seed=(5, 9), **kw)
        draws = utils.generate_mc_normal_draws(d, steps, N, rt, seed=(5, 9), dtype=dtype)
        ref = basket_european_mc(normal_draws=draws.permute(1, 0, 2), **kw)
        assert q.price == ref.price
        np.testing.assert_array_equal(np.asarray(q.delta.cpu()), np.asarray(ref.delta.cpu()))
        np.testing.assert_array_equal(np.asarray(q.vega.cpu()), np.asarray(ref.vega.cpu()))
