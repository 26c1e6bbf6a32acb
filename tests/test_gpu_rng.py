"""Sobol and Philox kernels against the oracle (GPU)."""

import numpy as np
import pytest
import torch

from oracle import philox as ophilox
from oracle import sobol as osobol

pytestmark = pytest.mark.gpu


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("dim,n,skip", [(1, 1, 0), (2, 5, 0), (5, 31, 0), (7, 1000, 17), (16, 4099, 0),
                                        (1024, 3000, 0), (13, 2 ** 16, 123), (1, 3, 2 ** 31 - 5),
                                        (504, 4097, 0), (33, 777, 2 ** 20),
                                        # several column slices per row: whole (2048), partial last
                                        # slice (1028), scalar stores (1025, 4099)
                                        (2048, 1500, 0), (1028, 777, 3), (1025, 2000, 5), (4099, 300, 1)])
def test_sobol_integers_bit_exact(cuda, dim, n, skip):
    from tqf.math.random import sobol
    got = _u32(sobol.sample_uint32(dim, n, skip))
    want = osobol.sample_int(dim, n, skip).astype(np.uint32)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_sobol_floats_match_reference_conversion(cuda, dtype):
    from tqf.math.random import sobol
    np_dt = np.float32 if dtype == torch.float32 else np.float64
    for dim, n, skip in [(2, 5, 0), (10, 50, 17), (64, 5000, 3)]:
        got = sobol.sample(dim, n, skip=skip, dtype=dtype).cpu().numpy()
        want = osobol.sample(dim, n, skip=skip, dtype=np_dt)
        np.testing.assert_array_equal(got, want)


def test_sobol_golden_vectors_on_gpu(cuda):
    import json, os
    from tqf.math.random import sobol
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sobol_golden.json")))
    a = g["dim2_first5"]
    np.testing.assert_allclose(sobol.sample(a["dim"], a["num_results"]).cpu().numpy(), a["expected"], rtol=1e-6)
    b = g["dim5_first31_gray_order"]
    got = sobol.sample(b["dim"], b["num_results"], dtype=torch.float64).cpu().numpy()
    assert sorted(map(tuple, got)) == sorted(map(tuple, b["expected"]))
    c = g["large_skip"]
    np.testing.assert_allclose(sobol.sample(c["dim"], c["num_results"], skip=c["skip"]).cpu().numpy(), c["expected"])


def test_sobol_skip_consistency(cuda):
    from tqf.math.random import sobol
    full = sobol.sample(10, 67).cpu().numpy()
    part = sobol.sample(10, 50, skip=17).cpu().numpy()
    np.testing.assert_array_equal(full[17:], part)


def test_sobol_normals_close_to_erfinv(cuda):
    from tqf.math.random import sobol
    got = sobol.sample_normal(12, 5000, skip=5).cpu().numpy()
    u = osobol.sample(12, 5000, skip=5, dtype=np.float32)
    want = osobol.normal_from_uniform(u)
    np.testing.assert_allclose(got, want, rtol=2e-6, atol=2e-6)
    got64 = sobol.sample_normal(12, 5000, skip=5, dtype=torch.float64).cpu().numpy()
    want64 = osobol.normal_from_uniform(osobol.sample(12, 5000, skip=5, dtype=np.float64))
    np.testing.assert_allclose(got64, want64, rtol=1e-13, atol=1e-13)


def test_sobol_normal_f32_every_input_at_20_digits(cuda):
    """Dimension 0 at 2^20 - 1 points (nd = 20) takes every integer 1 ..
    2^20 - 1 once (van der Corput), so the float32 inverse normal is checked
    on every input of that conversion, tails (|x| up to 1 - 2^-19) included:
    within 6e-7 relative of float64 erfinv (erfinvf's documented 2 ulp, the
    rounding of the product by sqrt(2) and of the float32 result), and
    exactly 0 at u = 1/2."""
    from scipy.special import erfinv
    from tqf.math.random import sobol
    n = 2 ** 20 - 1
    got = sobol.sample_normal(1, n).cpu().numpy()[:, 0].astype(np.float64)
    ints = osobol.sample_int(1, n, 0)[:, 0].astype(np.int64)
    assert np.array_equal(np.sort(ints), np.arange(1, n + 1))
    want = erfinv(ints * 2.0 ** -19 - 1.0) * np.sqrt(2.0)
    zero = want == 0
    assert zero.sum() == 1 and got[zero][0] == 0.0
    rel = np.abs(got[~zero] - want[~zero]) / np.abs(want[~zero])
    assert rel.max() < 6e-7, rel.max()
    assert np.array_equal(np.sign(got), np.sign(want))


@pytest.mark.parametrize("dim,n,skip", [(1024, 3000, 7), (1030, 1000, 0)])
def test_sobol_wide_outputs_match_oracle(cuda, dim, n, skip):
    """float32, float32-normal and float64 outputs of wide requests (whole-row
    and half-row CTAs, scalar stores for dim % 4 != 0) against the oracle."""
    from tqf.math.random import sobol
    u32 = osobol.sample(dim, n, skip=skip, dtype=np.float32)
    np.testing.assert_array_equal(sobol.sample(dim, n, skip=skip).cpu().numpy(), u32)
    np.testing.assert_array_equal(sobol.sample(dim, n, skip=skip, dtype=torch.float64).cpu().numpy(),
                                  osobol.sample(dim, n, skip=skip, dtype=np.float64))
    got = sobol.sample_normal(dim, n, skip=skip).cpu().numpy()
    np.testing.assert_allclose(got, osobol.normal_from_uniform(u32), rtol=2e-6, atol=2e-6)


def test_sobol_draw_layout(cuda):
    # [steps, N, d] with Sobol dimension step*d + c and point index skip+1+n.
    from tqf.math.random import sobol
    steps, N, d, skip = 7, 1500, 3, 11
    got = sobol.normal_draws(d, steps, N, skip=skip).cpu().numpy()
    u = osobol.sample(steps * d, N, skip=skip, dtype=np.float32)
    want = osobol.normal_from_uniform(u).reshape(N, steps, d).transpose(1, 0, 2)
    np.testing.assert_allclose(got, want, rtol=2e-6, atol=2e-6)


def test_sobol_full_scale_permutation_property(cuda):
    # n = 2^k - 1 points from index 1: each dimension is a permutation of
    # 1 .. 2^k - 1 (at nd = k digits) — checked by sums (and sums of squares
    # where int64 holds them).
    from tqf.math.random import sobol
    n = 2 ** 24 - 1
    assert sobol.num_digits(n, 0) == 24
    x = sobol.sample_uint32(16, n).to(torch.int64)
    assert torch.all(x.sum(dim=0) == n * (n + 1) // 2)
    n = 2 ** 20 - 1
    x = sobol.sample_uint32(64, n).to(torch.int64)
    assert torch.all(x.sum(dim=0) == n * (n + 1) // 2)
    assert torch.all((x * x).sum(dim=0) == n * (n + 1) * (2 * n + 1) // 6)


@pytest.mark.parametrize("chunk_start", [0, 2 ** 25, 2 ** 26 - 2 ** 20])
def test_sobol_dim1024_2pow26_chunks_bit_exact(cuda, chunk_start):
    """Dimension 1024, 2^26 points (nd = 27 for the whole set), generated in
    chunks of 2^20 points with the global nd, exactly as the throughput
    measurement launches them: 4,096 rows of each chunk (its first, middle and
    last 1,024 rows and 1,024 rows from a seeded random offset) checked bit for
    bit against the oracle's integers, for the uint32 and float32 outputs;
    the inverse-normal output within the float32 erfinv tolerance."""
    import tqf._lib as L
    from tqf.math.random import sobol
    dim, total, chunk = 1024, 2 ** 26, 2 ** 20
    nd = sobol.num_digits(total, 0)
    assert nd == 27
    v = sobol.device_direction_numbers(dim, cuda)
    out = torch.empty((chunk, dim), dtype=torch.int32, device=cuda)
    m = osobol.compute_direction_numbers(dim)
    offs = [0, chunk // 2, chunk - 1024, int(np.random.default_rng(chunk_start + 1).integers(1024, chunk - 2048))]
    want_int = {o: osobol.sample_int(dim, 1024, chunk_start + o, nd=nd, m=m) for o in offs}
    rows = torch.cat([torch.arange(o, o + 1024) for o in offs]).to(cuda)
    for kind in (L.SOBOL_U32, L.SOBOL_F32, L.SOBOL_NORMAL_F32):
        out.fill_(-1)
        L.call("tqf_sobol_sample", v.data_ptr(), dim, chunk, chunk_start, nd, kind, out.data_ptr(), L.stream_ptr())
        got = out.index_select(0, rows).cpu().numpy()
        for i, o in enumerate(offs):
            g = got[i * 1024:(i + 1) * 1024]
            w = want_int[o]
            if kind == L.SOBOL_U32:
                np.testing.assert_array_equal(g.view(np.uint32), w.astype(np.uint32))
            else:
                u = (w.astype(np.float32) / np.float32(2.0 ** nd)).astype(np.float32)
                if kind == L.SOBOL_F32:
                    np.testing.assert_array_equal(g.view(np.float32), u)
                else:
                    np.testing.assert_allclose(g.view(np.float32), osobol.normal_from_uniform(u), rtol=2e-6,
                                               atol=2e-6)


def test_sobol_2pow26_reference_rounding(cuda):
    # At 2^26 points the reference's float32 output reaches exactly 1.0.
    from tqf.math.random import sobol
    x = sobol.sample(1, 4, skip=2 ** 26 - 4)
    nd = sobol.num_digits(4, 2 ** 26 - 4)
    assert nd == 27
    assert float(x.max()) == 1.0
    c = sobol.sample_centered(1, 4, skip=2 ** 26 - 4)
    assert float(c.max()) < 1.0


PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expected", PHILOX_KAT)
def test_philox_kernel_known_answers(cuda, ctr, key, expected):
    import tqf._lib as L
    out = torch.zeros(4, dtype=torch.int32, device=cuda)
    L.call("tqf_philox4x32_10", *ctr, *key, 1, out.data_ptr(), L.stream_ptr())
    assert tuple(int(v) for v in _u32(out)) == expected


def test_philox_kernel_stream_bit_exact(cuda):
    import tqf._lib as L
    out = torch.zeros(4 * 5000, dtype=torch.int32, device=cuda)
    L.call("tqf_philox4x32_10", 7, 8, 9, 10, 11, 12, 5000, out.data_ptr(), L.stream_ptr())
    got = _u32(out).reshape(5000, 4)
    want = ophilox.philox4x32_10((7 + np.arange(5000)).astype(np.uint64), np.full(5000, 8, np.uint64),
                                 np.full(5000, 9, np.uint64), np.full(5000, 10, np.uint64), 11, 12)
    np.testing.assert_array_equal(got, np.stack(want, 1))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("antithetic", [False, True])
def test_philox_normal_draws_match_oracle(cuda, dtype, antithetic):
    from tqf.math.random import RandomType
    from tqf.math.random.multivariate_normal import philox_normal_draws
    rt = RandomType.STATELESS_ANTITHETIC if antithetic else RandomType.STATELESS
    steps, N, d = 9, 2048, 3
    got = philox_normal_draws(rt, [5, 6], d, steps, N, dtype).cpu().numpy()
    want = ophilox.normal_draws(N, steps, d, 5, 6, dtype=np.float32 if dtype == torch.float32 else np.float64,
                                antithetic=antithetic)
    if dtype == torch.float32:
        # Device float32 Box–Muller uses the SFU lg2 (absolute error ~2^-22),
        # so |dz| <= 4e-6 (1 + |z|) + 2.5e-7 / r with r the radius of the pair.
        K = steps * d
        kpad = (K + 3) // 4 * 4
        half = N // 2 if antithetic else None
        full = ophilox.normals(np.arange(N), kpad, 5, 6, antithetic_half=half)
        rad = np.sqrt((full.reshape(N, kpad // 2, 2) ** 2).sum(-1))
        rad = np.repeat(rad, 2, axis=1)[:, :K].reshape(N, steps, d).transpose(1, 0, 2)
        bound = 4e-6 * (1 + np.abs(want)) + 2.5e-7 / rad
        assert np.all(np.abs(got - want) <= bound)
    else:
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def test_draws_prefix_stability_and_moments(cuda):
    from tqf.math.random import RandomType, mv_normal_sample
    a = mv_normal_sample([10], mean=np.zeros(4, np.float32), random_type=RandomType.STATELESS, seed=[1, 2])
    b = mv_normal_sample([16], mean=np.zeros(4, np.float32), random_type=RandomType.STATELESS, seed=[1, 2])
    torch.testing.assert_close(a, b[:10], rtol=0, atol=0)
    z = mv_normal_sample([200000], mean=np.zeros(3, np.float64), random_type=RandomType.PSEUDO, seed=4)
    assert float(z.mean().abs()) < 5e-3 and abs(float(z.std()) - 1) < 5e-3
    cov = np.array([[1.0, 0.5], [0.5, 2.0]])
    z = mv_normal_sample([400000], mean=np.array([1.0, -1.0]), covariance_matrix=cov,
                         random_type=RandomType.STATELESS, seed=[3, 3]).cpu().numpy()
    np.testing.assert_allclose(np.cov(z.T), cov, atol=2e-2)
    np.testing.assert_allclose(z.mean(0), [1.0, -1.0], atol=1e-2)
    s = mv_normal_sample([1000], mean=np.zeros(2), random_type=RandomType.SOBOL, skip=1000)
    assert s.shape == (1000, 2) and abs(float(s.mean())) < 0.02
    z = mv_normal_sample([1000], mean=np.array([2.0, 3.0]), random_type=RandomType.PSEUDO_ANTITHETIC, seed=2)
    torch.testing.assert_close(z[:500] + z[500:], torch.tensor([4.0, 6.0], dtype=z.dtype, device=z.device).expand(500, 2))


def test_sobol_normal_integral_mean_and_var(cuda):
    # sobol_test.py:111-143: importance-sampled mean and standard deviation of
    # N(mu_p, 0.5^2) from N(0, 1) quantiles of 1,000 Sobol points
    from scipy.stats import norm
    from tqf.math.random import sobol
    mu_p, sigma_p = np.array([-1.0, 1.0]), np.array([0.5, 0.5])
    cdf_sample = sobol.sample(2, 1000, dtype=torch.float64).cpu().numpy()
    q_sample = norm.ppf(cdf_sample)
    w = norm.pdf(q_sample, loc=mu_p, scale=sigma_p) / norm.pdf(q_sample)
    e_x = np.mean(q_sample * w, 0)
    stddev = np.sqrt(np.mean(q_sample ** 2 * w - e_x ** 2, 0))
    np.testing.assert_allclose(e_x, mu_p, rtol=0.01)
    np.testing.assert_allclose(stddev, sigma_p, rtol=0.02)


def test_sobol_two_dimensional_projection(cuda):
    # sobol_test.py:145-157: the last two of 170 dimensions are uncorrelated
    from tqf.math.random import sobol
    sample = sobol.sample(170, 1000).cpu().numpy()
    x, y = sample[:, 168], sample[:, 169]
    np.testing.assert_allclose(np.corrcoef(x, y)[1, 0], 0.0, atol=0.05)
    np.testing.assert_allclose((x * y).mean(), 0.25, rtol=0.05)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_mc_normal_draws_sobol_known_values(cuda, dtype):
    # utils_test.py:33-60 on the device generator: [steps, paths, d]
    import json, os
    from tqf.math.random import RandomType
    from tqf.models import utils
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sobol_golden.json")))["mc_normal_draws_sobol"]
    got = utils.generate_mc_normal_draws(num_normal_draws=g["num_normal_draws"], num_time_steps=g["num_time_steps"],
                                         num_sample_paths=g["num_sample_paths"], random_type=RandomType.SOBOL,
                                         dtype=dtype, skip=g["skip"])
    assert tuple(got.shape) == (3, 4, 2) and got.dtype == dtype
    np.testing.assert_allclose(got.cpu().numpy(), g["expected"], rtol=g["rtol"], atol=g["atol"])
