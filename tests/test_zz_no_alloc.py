"""The allocation-free Heston pricing entry point (GPU).

tqf_heston_euler_price_noalloc serves callers that cannot call cudaMalloc: a
host application that owns every device allocation and hands the library
only its inputs and outputs, or a fixed-budget allocator that forbids stray
allocations.  It keeps its per-CTA partial sums in a fixed 2 MiB array inside
libtqf.so.  These tests call it through the C ABI twice in a row and check
both results against the allocating entry point tqf_heston_euler, within the
tolerance the sharded-pricing test uses (float32 tile rounding), for float32
and float64 paths and for in-kernel Philox and in-memory draws.  The file is
named to run last so that a run stopping at the first failure has already
run every other test.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _args(L, dtype, n_paths, table, strikes, out, ws, draws):
    import math

    from tqf.math.random import RandomType
    from tqf.math.random import multivariate_normal as mvn
    a = L.HestonArgs()
    a.dtype = L.TQF_F32 if dtype == torch.float32 else L.TQF_F64
    a.num_steps = table.shape[0]
    a.num_paths = n_paths
    a.step_table = table.data_ptr()
    a.x0, a.v0 = math.log(100.0), 0.04
    if draws is None:
        a.draws = mvn.philox_draws(RandomType.STATELESS, [11, 12], n_paths)
    else:
        a.draws = mvn.memory_draws(draws, path_axis=1, step_axis=0)
    a.payoff.num_strikes = strikes.numel()
    a.payoff.strikes = strikes.data_ptr()
    a.payoff.spot_scale = 1.0
    a.payoff.out = out.data_ptr()
    a.payoff.workspace = ws.data_ptr() if ws is not None else None
    a.payoff.workspace_bytes = ws.numel() if ws is not None else 0
    return a


@pytest.mark.parametrize("dtype,source", [(torch.float32, "philox"), (torch.float64, "philox"),
                                          (torch.float32, "memory")])
def test_noalloc_entry_point_matches_allocating_one_twice(cuda, dtype, source):
    import tqf._lib as L
    from tqf.models import heston_model, utils
    from tqf.models.coefficients import HestonFullTruncation
    n_paths, steps = 300_000, 64
    npt = np.float32 if dtype == torch.float32 else np.float64
    t = np.linspace(0.0, 1.0, steps + 1).astype(npt)
    dt = (t[1:] - t[:-1]).astype(npt)
    rows = heston_model.full_truncation_table(HestonFullTruncation(0.02, 2.0, 0.04, 0.3, -0.7), t, dt,
                                              np.sqrt(dt).astype(npt), np.full(steps, -1, np.int32), steps)
    table = utils.step_table(rows, dtype, cuda)
    strikes = torch.linspace(70.0, 130.0, 64, dtype=dtype, device=cuda)
    draws = None
    if source == "memory":
        g = torch.Generator(device=cuda).manual_seed(5)
        draws = torch.randn((steps, n_paths, 2), generator=g, dtype=dtype, device=cuda)
    stream = L.stream_ptr()
    code = L.TQF_F32 if dtype == torch.float32 else L.TQF_F64

    ref = torch.zeros((64, 2), dtype=torch.float64, device=cuda)
    ws = torch.empty(int(L.load().tqf_heston_workspace_bytes(code, 0, n_paths, 64)), dtype=torch.uint8,
                     device=cuda)
    L.call("tqf_heston_euler", _args(L, dtype, n_paths, table, strikes, ref, ws, draws), stream)

    for _ in range(2):
        out = torch.full((64, 2), float("nan"), dtype=torch.float64, device=cuda)
        L.call("tqf_heston_euler_price_noalloc", _args(L, dtype, n_paths, table, strikes, out, None, draws), stream)
        torch.cuda.synchronize()
        torch.testing.assert_close(out, ref, rtol=1e-6, atol=1e-6)

    too_many = torch.linspace(70.0, 130.0, 65, dtype=dtype, device=cuda)
    with pytest.raises(ValueError):
        out = torch.zeros((65, 2), dtype=torch.float64, device=cuda)
        L.call("tqf_heston_euler_price_noalloc", _args(L, dtype, n_paths, table, too_many, out, None, draws),
               stream)
