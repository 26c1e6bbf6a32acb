"""Path sharding + FP64 all-reduce over a world-size-2 gloo group (CPU).

Each rank prices its shard of a full-truncation Heston run with the oracle
(float64, canonical Philox stream indexed by global path number) and the
shards' sums are combined with tqf.pricing.sharding.allreduce_sums; the result
must equal the single-process sums over all paths.
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

N_TOTAL, STEPS, STRIKES = 1000, 12, np.array([90.0, 100.0, 110.0])


def _sums(paths):
    from oracle import euler as oeuler
    from oracle import philox as ophilox
    draws = ophilox.normals(paths, 2 * STEPS, 3, 4, dtype=np.float64).reshape(len(paths), STEPS, 2)
    drift, vol = oeuler.heston_ft_coefficients(0.02, 2.0, 0.04, 0.3, -0.7, np.float64)
    t = np.linspace(0, 1, STEPS + 1)
    keep = np.zeros(STEPS + 1, bool)
    keep[-1] = True
    x0 = np.tile([np.log(100.0), 0.04], (len(paths), 1))
    out = oeuler.sample_with_draws(drift, vol, t, keep, 1, x0, draws.transpose(1, 0, 2), np.float64)
    pay = np.maximum(np.exp(out[:, 0, 0])[:, None] - STRIKES[None, :], 0)
    return np.stack([pay.sum(0), (pay * pay).sum(0)], 1)


def _worker(rank, world, port, result_q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tf-quant-finance_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from tqf.pricing.sharding import allreduce_sums, shard_range
    off, cnt = shard_range(N_TOTAL, rank, world)
    sums = torch.from_numpy(_sums(np.arange(off, off + cnt)))
    allreduce_sums(sums)
    if rank == 0:
        result_q.put(sums.numpy())
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_shard_ranges_cover_all_paths_once():
    from tqf.pricing.sharding import shard_range, weak_shard
    for n, w in [(10, 3), (1 << 22, 8), (7, 7), (5, 2)]:
        seen = []
        for r in range(w):
            off, cnt = shard_range(n, r, w)
            seen.extend(range(off, off + cnt))
        assert seen == list(range(n))
    assert weak_shard(100, 3) == (300, 100)
    with pytest.raises(ValueError):
        shard_range(10, 3, 3)


def test_two_rank_gloo_allreduce_equals_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = _sums(np.arange(N_TOTAL))
    np.testing.assert_allclose(got, want, rtol=1e-12)
