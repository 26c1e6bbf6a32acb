"""Benchmark: Heston Monte Carlo path-steps/s on one GB300 (or N ranks).

Workload (one "step"): full-truncation Euler Heston in FP32, kappa=2.0,
theta=0.04, xi=0.3, rho=-0.7, v0=0.04, S0=100, r=0.02, 2^22 paths, 252 steps
to T=1, Philox4x32-10 draws generated in-kernel, a batch of 64 European call
strikes uniform in [70, 130] (fixed seed), FP64 cross-path accumulation of
payoff sums and sums of squares — one fused kernel pass plus the fixed-order
partial-sum reduction.  `value` = paths x steps x ranks / max-over-ranks
device time per step.

`--impl reference` times the reference algorithm on the host cores: the
oracle's NumPy restatement of euler_sampling.sample with the same Heston
full-truncation coefficients (TensorFlow itself cannot be installed on
these machines), run on every host core over a bounded path sample.
"""

from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "tf-quant-finance_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Heston path-steps/s"
UNIT = "path-steps/s"
N_PATHS = 1 << 22
N_STEPS = 252
N_STRIKES = 64
PARAMS = dict(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7,
              discount_rate=0.02, expiry=1.0)
# Algorithmic 32-bit lane operations per path-step of the fused kernel,
# counted from the restated math (not from compiled code): Philox4x32-10 half block (40: per round
# 4 multiplies, 2 three-input XORs, 2 key adds; 10 rounds per 2 steps), one
# Box–Muller pair (14: two uniform conversions, lg2, scale, sqrt, angle,
# sin, cos, two products) and the full-truncation step (14: max, sqrt, two
# dW products, 3 ops log-spot, 7 ops variance).
ALU_OPS_PER_PATH_STEP = 40 + 14 + 14
# DRAM bytes (read + write) per launch of the fused kernel: mean of two
# full-size launches (2^22 paths x 252 steps, 64 strikes) captured with
# `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum` (43,776 + 0 and
# 155,392 + 0 bytes): the step table, strikes and parameters; the per-CTA FP64
# partial sums stay in L2 (the ncu summary of this kernel under profiles/).
NCU_TRAFFIC_BYTES = 99584


def strikes():
    return np.sort(np.random.default_rng(2024).uniform(70.0, 130.0, N_STRIKES))


def workload_config(n_paths, n_steps, world):
    return {"workload": f"Heston full-truncation Euler FP32, {n_paths} paths x {n_steps} steps to T=1, "
                        f"Philox4x32-10 in-kernel, 64 European strikes in [70,130], FP64 accumulation",
            "paths_per_rank": n_paths, "time_steps": n_steps, "strikes": N_STRIKES,
            "params": PARAMS, "parallelism": f"path-sharded x{world}" if world > 1 else "single GPU",
            "l2": "L2 flushed (256 MiB write) between timed steps"}


# ---------------------------------------------------------------- CPU side
def _cpu_worker(args):
    n_paths, n_steps, seed = args
    from oracle import euler as oeuler
    p = PARAMS
    dtype = np.float32
    rng = np.random.default_rng(seed)
    drift, vol = oeuler.heston_ft_coefficients(p["discount_rate"], p["mean_reversion"], p["theta"], p["volvol"],
                                               p["rho"], dtype)
    t0 = time.perf_counter()
    all_t = np.linspace(0, p["expiry"], n_steps + 1).astype(dtype)
    keep = np.zeros(n_steps + 1, bool)
    keep[-1] = True
    draws = rng.standard_normal((n_steps, n_paths, 2), dtype=np.float32)
    x0 = np.tile(np.array([np.log(p["spot"]), p["variance"]], dtype), (n_paths, 1))
    out = oeuler.sample_with_draws(drift, vol, all_t, keep, 1, x0, draws, dtype)
    S = np.exp(out[:, 0, 0].astype(np.float64))
    k = strikes()
    pay = np.maximum(S[:, None] - k[None, :], 0.0)
    _ = pay.sum(0), (pay * pay).sum(0)
    return time.perf_counter() - t0, n_paths * n_steps


def cpu_reference_step(pool, cores, paths_per_core, n_steps, seed):
    t0 = time.perf_counter()
    res = pool.map(_cpu_worker, [(paths_per_core, n_steps, seed * 1000 + i) for i in range(cores)])
    wall = time.perf_counter() - t0
    units = sum(r[1] for r in res)
    return units, wall


def run_cpu_baseline(steps, warmup, budget_s=12.0):
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    paths_per_core = 4096
    with ctx.Pool(cores) as pool:
        # calibrate the sample so that one step takes about budget_s / steps,
        # on a warm pool (the first round pays the workers' imports), and
        # never below 8192 paths per worker (pool dispatch stays a small share)
        cpu_reference_step(pool, cores, 512, N_STEPS, 0)
        units, wall = cpu_reference_step(pool, cores, 2048, N_STEPS, 0)
        rate = units / wall
        target = max(budget_s / max(steps + warmup, 1), 0.5)
        paths_per_core = int(max(8192, min(1 << 16, rate * target / (cores * N_STEPS))))
        for w in range(warmup):
            cpu_reference_step(pool, cores, paths_per_core, N_STEPS, 1 + w)
        tot_units, tot_wall = 0, 0.0
        for s in range(steps):
            u, t = cpu_reference_step(pool, cores, paths_per_core, N_STEPS, 100 + s)
            tot_units += u
            tot_wall += t
    return tot_units / tot_wall, cores, paths_per_core, tot_wall / steps


# ---------------------------------------------------------------- GPU side
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [c.strip() for c in line.split(",")]))

    def mark(self, start=True):
        if start:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread is not None:
                self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0, t1 = getattr(self, "t0", 0.0), getattr(self, "t1", float("inf"))
        for ts, r in self.rows:
            if ts < t0 or ts > t1 + 0.25:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fma_peak(torch, L):
    """FP32 FMA lane-ops/s of this GPU (probe kernel, best of 5)."""
    import ctypes
    dev = torch.device("cuda", torch.cuda.current_device())
    out = torch.zeros(1, dtype=torch.float32, device=dev)
    lane_ops = ctypes.c_double(0)
    s = torch.cuda.current_stream()
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        L.call("tqf_fma_peak_probe", 4096, 8, out.data_ptr(), ctypes.byref(lane_ops), s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        best = max(best, lane_ops.value / (e0.elapsed_time(e1) * 1e-3))
    return best


def run_gpu(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    import tqf._lib as L
    from tqf.math.random import RandomType
    from tqf.pricing import heston_european_mc

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n_paths, n_steps = args.paths, args.time_steps
    k = strikes()
    from tqf.pricing.sharding import weak_shard
    offset, _ = weak_shard(n_paths, rank)
    kw = dict(strikes=k, num_samples=n_paths, num_time_steps=n_steps, scheme="full_truncation",
              random_type=RandomType.STATELESS, seed=[20240, 7], path_offset=offset, **PARAMS)

    # Device-resident pieces for the kernel-only timing: everything a step needs
    # is built once; a timed step is the fused kernel + partial-sum reduction.
    import ctypes
    from tqf.models import heston_model
    from tqf.models.coefficients import HestonFullTruncation
    from tqf.models import utils
    from tqf.math.random import multivariate_normal as mvn
    from tqf.pricing.european import make_payoff, stats_from_sums
    p = PARAMS
    all_t = np.linspace(0.0, p["expiry"], n_steps + 1).astype(np.float32)
    dt = (all_t[1:] - all_t[:-1]).astype(np.float32)
    h = HestonFullTruncation(p["discount_rate"], p["mean_reversion"], p["theta"], p["volvol"], p["rho"])
    rows = heston_model.full_truncation_table(h, all_t, dt, np.sqrt(dt).astype(np.float32),
                                              np.full(n_steps, -1, np.int32), n_steps)
    table = utils.step_table(rows, torch.float32, dev)
    pay, out, keep = make_payoff(k, None, torch.float32, dev, n_paths,
                                 lambda ns: L.load().tqf_heston_workspace_bytes(0, 0, n_paths, ns), "bench")
    hargs = L.HestonArgs()
    hargs.dtype = L.TQF_F32
    hargs.num_steps = n_steps
    hargs.num_paths = n_paths
    hargs.step_table = table.data_ptr()
    hargs.x0, hargs.v0 = math.log(p["spot"]), p["variance"]
    hargs.draws = mvn.philox_draws(RandomType.STATELESS, [20240, 7], n_paths, offset)
    hargs.payoff = pay
    hargs.dev_status = L.status_buffer(dev).data_ptr()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def kernel_step():
        L.call("tqf_heston_euler", hargs, stream.cuda_stream)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        kernel_step()
        flush.fill_(1)
    barrier()
    launches0 = L.launch_count()
    times_ms = []
    with ClockSampler(local_rank) as clocks:
        time.sleep(1.0)  # let the sampler start before the timed region
        clocks.mark(True)
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            kernel_step()
            e1.record(stream)
            flush.fill_(1)  # evict L2 between timed steps (outside the events)
            times_ms.append((e0, e1))
        barrier()
        wall = time.perf_counter() - t_wall0
        clocks.mark(False)
    launches = L.launch_count() - launches0
    per_step = [a.elapsed_time(b) for a, b in times_ms]
    ms = sum(per_step) / len(per_step)
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    L.check_device_status(dev)
    res = stats_from_sums(out, n_paths, math.exp(-p["discount_rate"] * p["expiry"]))
    value = n_paths * n_steps * world / (ms * 1e-3)

    # The dominant kernel's own duration: the fused path kernel alone
    # (payoff.out = NULL leaves the partial sums in the workspace and skips
    # the reduction launch), timed by events on the launching stream.
    kargs = L.HestonArgs()
    ctypes.memmove(ctypes.byref(kargs), ctypes.byref(hargs), ctypes.sizeof(L.HestonArgs))
    kargs.payoff.out = None
    hk = []
    for _ in range(max(3, min(args.steps, 10))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.call("tqf_heston_euler", kargs, stream.cuda_stream)
        e1.record(stream)
        flush.fill_(1)
        hk.append((e0, e1))
    torch.cuda.synchronize()
    step_ms = sum(a.elapsed_time(b) for a, b in hk) / len(hk)

    # End to end through the public API with host buffers: strikes from pinned
    # host memory, results read back each step.
    k_host = torch.from_numpy(k.astype(np.float32)).pin_memory()
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = heston_european_mc(**{**kw, "strikes": k_host})
        price, se = r.to_host()  # one device-to-host copy of the [2, 64] results
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_s = sum(e2e_times) / len(e2e_times)
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
        from tqf.pricing.sharding import allreduce_sums
        allreduce_sums(out)  # the one exchange step: FP64 payoff sums

    peaks, peak_kind = measured_peaks()
    fp32_peak = fma_peak(torch, L)
    alg_ops = ALU_OPS_PER_PATH_STEP * n_paths * n_steps
    achieved = alg_ops / (step_ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox draws, fixed strikes)",
        "config": workload_config(n_paths, n_steps, world),
        "e2e": {"value": n_paths * n_steps * world / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(k.size * 4), "d2h_bytes_per_step": int(2 * k.size * 8),
                "api": "tqf.pricing.heston_european_mc (host strikes -> device prices)"},
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fp32_peak / 1e12,
                     "unit": "T lane-op/s", "frac": achieved / fp32_peak, "traffic": NCU_TRAFFIC_BYTES,
                     "kernel": "heston_kernel<float, FT, PHILOX, store=0, price=1>",
                     "kernel_ms": step_ms, "alg_ops_per_path_step": ALU_OPS_PER_PATH_STEP,
                     "peak_source": "tqf_fma_peak_probe measured live (FP32 FMA lane-ops/s)",
                     "hbm_peak_gbs": peaks.get("hbm_gbs"), "hbm_peak_kind": peak_kind},
        "gpu_launches": int(launches),
        "wall_s_timed_region": wall,
        "clocks": clocks.summary(),
        "result_check": {"atm_call_price": float(res.price[int(np.argmin(np.abs(k - 100)))]),
                         "strike": float(k[int(np.argmin(np.abs(k - 100)))]),
                         "se": float(res.standard_error[int(np.argmin(np.abs(k - 100)))])},
    }
    return line


def run_neural_cv(pilot_paths=1 << 20, train_steps=600, eval_paths=1 << 26, batch_paths=1024, lr=3e-3,
                  control_every=2):
    """Config C5: Heston arithmetic-Asian call (52 dates, K=100) — pilot paths,
    600 Adam steps (lr 3e-3, 1,024-path minibatches) on the tcgen05 training
    kernels, then fused CV pricing vs plain MC on the same evaluation paths;
    the network's position is rebalanced at every second monitoring date
    (26 evaluations per path).  Time to a 1e-4 relative 95% CI for both (GPU
    seconds, CUDA events), with and without pilot and training."""
    import torch
    from tqf.pricing import HestonAsianCV, time_to_ci
    cv = HestonAsianCV(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7, rate=0.02,
                       expiry=1.0, strike=100.0, num_dates=52, num_time_steps=252, control_every=control_every)
    cv.pilot(pilot_paths, seed=(977, 5))
    cv.price(1 << 16, control_variate=False, seed=(1, 1))  # warm-up of both pricing kernels
    cv.price(1 << 16, control_variate=True, seed=(1, 1))
    losses = cv.train(steps=train_steps, batch_paths=batch_paths, lr=lr)
    plain = cv.price(eval_paths, control_variate=False, seed=(31, 41))
    est = cv.price(eval_paths, control_variate=True, seed=(31, 41))
    t_plain = time_to_ci(plain)
    t_cv = time_to_ci(est)
    setup = cv.pilot_seconds + cv.train_seconds
    torch.cuda.synchronize()
    return {
        "config": "Heston FT-Euler FP32, 252 steps, arithmetic Asian 52 dates, K=100; MLP 3-64-64-1 SiLU BF16, "
                  f"control rebalanced every {control_every} dates ({cv.num_control} evaluations per path), "
                  f"{pilot_paths} pilot paths, {train_steps} Adam steps (lr {lr}) x {batch_paths} paths, "
                  f"{eval_paths} eval paths",
        "price_cv": est.price, "se_cv": est.standard_error, "price_plain": plain.price, "se_plain": plain.standard_error,
        "vrf": est.vrf, "bias_in_se": (est.price - plain.price) / plain.standard_error,
        "mean_control_in_se": est.mean_control / est.se_control,
        "eval_seconds_plain": plain.seconds, "eval_seconds_cv": est.seconds,
        "cost_ratio_cv_over_plain": est.seconds / plain.seconds,
        "pilot_seconds": cv.pilot_seconds, "train_seconds": cv.train_seconds,
        "loss_first_last": [losses[0], losses[-1]],
        "time_to_1e-4_ci_plain_s": t_plain["seconds"], "time_to_1e-4_ci_cv_s": t_cv["seconds"],
        "time_to_1e-4_ci_cv_incl_training_s": t_cv["seconds"] + setup,
        "speedup_vs_plain": t_plain["seconds"] / t_cv["seconds"],
        "speedup_vs_plain_incl_training": t_plain["seconds"] / (t_cv["seconds"] + setup),
        "as_configured": _neural_cv_as_configured(pilot_paths, eval_paths, t_plain["seconds"], plain.price,
                                                  plain.standard_error),
    }


def _neural_cv_as_configured(pilot_paths, eval_paths, t_plain_s, price_plain, se_plain):
    """The C5 configuration as written (network rebalanced at every one of the
    52 dates, 2,000 Adam steps at lr 1e-3 on 512-path minibatches), on the
    same evaluation paths as the default leg, whose plain-MC run it shares."""
    import torch
    from tqf.pricing import HestonAsianCV, time_to_ci
    cv = HestonAsianCV(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7, rate=0.02,
                       expiry=1.0, strike=100.0, num_dates=52, num_time_steps=252, control_every=1)
    cv.pilot(pilot_paths, seed=(977, 5))
    cv.price(1 << 16, control_variate=True, seed=(1, 1))
    cv.train(steps=2000, batch_paths=512, lr=1e-3)
    est = cv.price(eval_paths, control_variate=True, seed=(31, 41))
    torch.cuda.synchronize()
    t_cv = time_to_ci(est)["seconds"]
    setup = cv.pilot_seconds + cv.train_seconds
    return {"config": "control at every date (52 evaluations per path), 2000 Adam steps (lr 0.001) x 512 paths",
            "vrf": est.vrf, "bias_in_se": (est.price - price_plain) / se_plain,
            "eval_seconds_cv": est.seconds, "pilot_seconds": cv.pilot_seconds, "train_seconds": cv.train_seconds,
            "time_to_1e-4_ci_cv_s": t_cv, "time_to_1e-4_ci_cv_incl_training_s": t_cv + setup,
            "speedup_vs_plain": t_plain_s / t_cv, "speedup_vs_plain_incl_training": t_plain_s / (t_cv + setup)}


def run_sobol(dim=1024, total_points=1 << 26, chunk=1 << 20, timed_chunks=8):
    """Config C2: Sobol dim 1024, 2^26 points (nd = 27 for the whole set),
    generated in chunks of 2^20 points (4 GiB each) into one reused buffer,
    for the uint32, float32 and float32 inverse-normal outputs.  Timed chunks
    are spread over the index range (chunk c * total/(timed*chunk)); each is
    written once, larger than L2.  Roofline: 4 B written per element against
    the measured copy bandwidth, and against the write-only bandwidth of a
    fill of the same buffer measured here."""
    import torch
    from tqf import _lib
    from tqf.math.random import sobol
    dev = torch.device("cuda", torch.cuda.current_device())
    nd = sobol.num_digits(total_points, 0)
    v = sobol.device_direction_numbers(dim, dev)
    out = torch.empty((chunk, dim), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    spacing = total_points // (timed_chunks * chunk)
    peaks, peak_src = measured_peaks()
    peak = peaks.get("hbm_gbs")
    res = {"config": f"dim {dim}, {total_points} points, nd {nd}, chunks of {chunk} points, "
                     f"{timed_chunks} chunks timed (every {spacing}th)"}
    # write-only ceiling of this GPU: torch's fill of the same 4 GiB buffer
    # (the measured copy bandwidth counts read + write bytes)
    fill_ms = []
    for j in range(8):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out.fill_(j)
        e1.record(stream)
        e1.synchronize()
        if j >= 3:
            fill_ms.append(e0.elapsed_time(e1))
    fill_gbs = chunk * dim * 4 / (sorted(fill_ms)[len(fill_ms) // 2] / 1e3) / 1e9
    res["write_fill_gbs"] = fill_gbs
    for kind, tag in [(_lib.SOBOL_U32, "u32"), (_lib.SOBOL_F32, "f32"), (_lib.SOBOL_NORMAL_F32, "normal_f32")]:
        def launch(c):
            _lib.call("tqf_sobol_sample", v.data_ptr(), dim, chunk, c * chunk, nd, kind, out.data_ptr(),
                      stream.cuda_stream)
        for c in range(2):
            launch(c)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * timed_chunks)]
        for j in range(timed_chunks):
            ev[2 * j].record(stream)
            launch(j * spacing)
            ev[2 * j + 1].record(stream)
        torch.cuda.synchronize()
        ms = [ev[2 * j].elapsed_time(ev[2 * j + 1]) for j in range(timed_chunks)]
        sec = sum(ms) / 1e3 / timed_chunks
        gbs = chunk * dim * 4 / sec / 1e9
        res[tag] = {"seconds_per_chunk": sec, "points_per_s": chunk / sec, "write_gbs": gbs,
                    "frac_of_hbm": gbs / peak, "peak_source": peak_src, "frac_of_write_fill": gbs / fill_gbs,
                    "full_set_seconds": sec * total_points / chunk}
    del out
    torch.cuda.empty_cache()
    return res


def run_lsm(n_paths=1 << 20, n_dates=50, degree=3, reps=5, cpu_paths=1 << 15):
    """Longstaff–Schwartz American put (K = 1.1, r = 6 %, sigma = 0.2, T = 1)
    on GBM paths from this engine's sampler: N paths x 50 exercise dates,
    float32, centred cubic basis.  Time of least_square_mc through the public
    API (the gather, then the whole backward loop in one cooperative kernel;
    paths resident) from CUDA events; the oracle's NumPy restatement timed on
    a path sample beside it."""
    import torch
    from tqf.math.random import RandomType
    from tqf.models import MultivariateGeometricBrownianMotion
    from tqf.models import longstaff_schwartz as L
    from oracle import lsm as olsm  # CPU baseline only
    proc = MultivariateGeometricBrownianMotion(1, means=0.06, volatilities=[0.2], dtype=np.float32)
    times = np.linspace(1.0 / n_dates, 1.0, n_dates)
    paths = proc.sample_paths(times, initial_state=[1.0], num_samples=n_paths, random_type=RandomType.STATELESS,
                              seed=[7, 8])
    ex = list(range(n_dates))
    df = np.exp(-0.06 * times)
    pay, basis = L.make_basket_put_payoff([1.1], dtype=np.float32), L.make_polynomial_basis(degree)
    price = None
    for _ in range(2):
        price = L.least_square_mc(paths, ex, pay, basis, discount_factors=df, dtype=np.float32)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        price = L.least_square_mc(paths, ex, pay, basis, discount_factors=df, dtype=np.float32)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / reps / 1e3
    from tqf import _lib
    c0 = _lib.launch_count()
    L.least_square_mc(paths, ex, pay, basis, discount_factors=df, dtype=np.float32)
    launches = _lib.launch_count() - c0
    torch.cuda.synchronize()
    sample = paths[:cpu_paths].cpu().numpy()
    t0 = time.perf_counter()
    cpu_price = olsm.least_square_mc(sample, ex, [1.1], degree, discount_factors=df, dtype=np.float32)
    cpu_sec = time.perf_counter() - t0
    return {"config": f"American put K=1.1 on GBM (r 0.06, vol 0.2, T 1), {n_paths} paths x {n_dates} exercise dates, "
                      f"float32, degree-{degree} basis",
            "price": float(price.cpu().numpy()[0]), "seconds": sec,
            "path_dates_per_s": n_paths * n_dates / sec,
            "launches_per_call": launches,
            "cpu_baseline": {"path_dates_per_s": cpu_paths * n_dates / cpu_sec, "cores": 1, "kind": "port",
                             "sample": f"oracle NumPy restatement, {cpu_paths} paths, price {float(cpu_price[0]):.5f}"}}


def run_basket(paths_n=1 << 22, price_paths=1 << 22, n_steps=64, reps=10):
    """Config C4: 16-asset correlated GBM (FP32, 64 steps, in-kernel Philox).
    (1) sample_paths writing every date, [paths, 64, 16] float32, with L z on
    the tensor cores (split BF16, three products) and on CUDA cores; (2) the
    fused basket call pricer with pathwise delta/vega (L applied once per path
    to w = sum sqrt(dt) z).  Device time from CUDA events, mean of `reps`."""
    import torch
    from tqf.math.random import RandomType
    from tqf.models import MultivariateGeometricBrownianMotion
    from tqf.pricing import basket_european_mc
    d = 16
    rng = np.random.default_rng(7)
    vols = rng.uniform(0.1, 0.4, d)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    c = q @ np.diag(rng.uniform(0.1, 2.0, d)) @ q.T
    s = np.sqrt(np.diag(c))
    corr = c / np.outer(s, s)
    proc = MultivariateGeometricBrownianMotion(d, means=0.02, volatilities=vols, corr_matrix=corr, dtype=np.float32)
    times = np.linspace(1.0 / n_steps, 1.0, n_steps)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3

    res = {"config": f"16 assets, vols U[0.1,0.4], random-orthogonal correlation, {n_steps} steps, FP32, Philox"}
    bytes_out = paths_n * n_steps * d * 4
    for mode, tag in [(0, "tensor_core_lz"), (1, "cuda_core_lz")]:
        launch, out = proc.paths_launcher(times, initial_state=np.full(d, 100.0, np.float32), num_samples=paths_n,
                                          random_type=RandomType.STATELESS, seed=[3, 4], lz_mode=mode)
        sec = timed(launch)
        res[f"paths_{tag}"] = {"paths": paths_n, "seconds": sec, "path_steps_per_s": paths_n * n_steps / sec,
                               "store_gbs": bytes_out / sec / 1e9}
        del out
    torch.cuda.empty_cache()
    kw = dict(spots=np.full(d, 100.0), vols=vols, rate=0.02, corr=corr, strike=100.0, expiry=1.0,
              num_time_steps=n_steps, num_samples=price_paths, dtype=torch.float32)
    basket_european_mc(**kw, seed=(5, 6))
    t0 = time.perf_counter()
    b = basket_european_mc(**kw, seed=(5, 6))
    sec = time.perf_counter() - t0
    res["basket_price"] = {"paths": price_paths, "price": b.price, "se": b.standard_error,
                           "wall_seconds_incl_host": sec, "path_steps_per_s": price_paths * n_steps / sec}
    # 64 assets: L z on the tensor cores with K and N tiled in 16s (four
    # K = 16 instructions per product) against the one-warp-per-path CUDA-core
    # kernel; [2^20, 64, 64] float32 output (17.2 GB written per call).
    d64, p64 = 64, paths_n // 4
    rng = np.random.default_rng(64)
    vols64 = rng.uniform(0.1, 0.4, d64)
    q, _ = np.linalg.qr(rng.standard_normal((d64, d64)))
    c = q @ np.diag(rng.uniform(0.1, 2.0, d64)) @ q.T
    s = np.sqrt(np.diag(c))
    proc64 = MultivariateGeometricBrownianMotion(d64, means=0.02, volatilities=vols64, corr_matrix=c / np.outer(s, s),
                                                 dtype=np.float32)
    bytes64 = p64 * n_steps * d64 * 4
    res["assets64"] = {"config": f"64 assets, {p64} paths x {n_steps} dates, FP32, Philox"}
    for mode, tag in [(0, "tensor_core_lz"), (1, "cuda_core_lz")]:
        launch, out = proc64.paths_launcher(times, initial_state=np.full(d64, 100.0, np.float32), num_samples=p64,
                                            random_type=RandomType.STATELESS, seed=[3, 4], lz_mode=mode)
        sec = timed(launch)
        res["assets64"][f"paths_{tag}"] = {"seconds": sec, "path_steps_per_s": p64 * n_steps / sec,
                                           "store_gbs": bytes64 / sec / 1e9}
        del out
    torch.cuda.empty_cache()
    return res


def run_stored_paths(n_paths=N_PATHS, n_steps=N_STEPS, reps=5):
    """Path sampling with every step recorded (the drop-in sample_paths /
    euler_sampling.sample outputs, [N, 252, d] float32): Heston QE and
    full-truncation Euler, GBM through euler_sampling (d = 1, 2, 3) and the
    exact GBM sampler; the same calls recording only t = T show the cost of
    the stores.  Median of `reps` calls through the public API, CUDA events;
    write GB/s counts the output bytes."""
    import torch
    import tqf
    from tqf.math.random import RandomType
    from tqf.models import coefficients as co

    def timed(fn):
        out = fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
            del out
        return sorted(ts)[len(ts) // 2]

    N = n_paths
    times = (np.arange(1, n_steps + 1, dtype=np.float64) / n_steps).astype(np.float32)
    last = np.array([1.0], np.float32)
    rnd = dict(num_samples=N, random_type=RandomType.STATELESS, seed=[1, 2])
    x0h = np.array([np.log(100.0), 0.04], np.float32)
    heston = tqf.models.HestonModel(2.0, 0.04, 0.3, -0.7)
    ft_drift, ft_vol = co.heston_full_truncation(0.02, 2.0, 0.04, 0.3, -0.7)
    cases = {
        "heston_qe": (2, lambda t: heston.sample_paths(t, x0h, num_time_steps=n_steps, **rnd)),
        "heston_ft_euler": (2, lambda t: tqf.models.euler_sampling.sample(2, ft_drift, ft_vol, t, num_time_steps=n_steps,
                                                                          initial_state=x0h, **rnd)),
    }
    for d in (1, 2, 3):
        drift, vol = co.gbm(np.full(d, 0.05, np.float32), np.full(d, 0.2, np.float32),
                            (0.5 * np.eye(d) + 0.5).astype(np.float32))
        cases[f"gbm_euler_d{d}"] = (d, (lambda dr, vo, dd: lambda t: tqf.models.euler_sampling.sample(
            dd, dr, vo, t, num_time_steps=n_steps, initial_state=np.full(dd, 100.0, np.float32), **rnd))(drift, vol, d))
    gbm = tqf.models.GeometricBrownianMotion(0.05, 0.2, dtype=np.float32)
    cases["gbm_exact"] = (1, lambda t: gbm.sample_paths(t, initial_state=100.0, **rnd))
    res = {"config": f"{N} paths x {n_steps} steps, float32, every step recorded vs t = T only, Philox draws"}
    for name, (d, fn) in cases.items():
        t_all = timed(lambda: fn(times))
        t_last = timed(lambda: fn(last))
        gb = N * n_steps * d * 4 / 1e9
        res[name] = {"all_steps_ms": t_all * 1e3, "last_only_ms": t_last * 1e3, "output_gb": gb,
                     "write_gbs": gb / t_all}
    return res


def run_heston_sobol(n_paths=N_PATHS, n_steps=N_STEPS, reps=5):
    """The Heston pricing workload with Sobol draws (the quasi-random variant
    of the headline config: dimension 2 x 252 = 504, points 1 .. 2^22).
    Fused: the normals are computed inside the pricing kernel from per-window
    shared-memory tables (no draw buffer).  Materialised (for comparison): the
    draws are generated on the device ([252, 2^22, 2] float32, 8.5 GB) and
    read in place by the same kernel.  Median of `reps` calls through the
    public API, CUDA events, draw generation included; the two prices agree
    to the float64 summation order."""
    import torch
    from tqf.math.random import RandomType
    from tqf.models import utils
    from tqf.pricing import heston_european_mc
    kw = dict(strikes=strikes(), expiry=1.0, spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3,
              rho=-0.7, discount_rate=0.02, num_samples=n_paths, num_time_steps=n_steps)

    def timed(fn):
        res = fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return sorted(ts)[len(ts) // 2], res

    sec, res = timed(lambda: heston_european_mc(random_type=RandomType.SOBOL, **kw))

    def materialised():
        d = utils.generate_mc_normal_draws(2, n_steps, n_paths, RandomType.SOBOL, dtype=torch.float32)
        return heston_european_mc(normal_draws=d.permute(1, 0, 2), **kw)

    sec_m, res_m = timed(materialised)
    torch.cuda.empty_cache()
    k = strikes()
    j = int(np.argmin(np.abs(k - 100.0)))
    return {"config": f"Heston FT-Euler FP32, {n_paths} paths x {n_steps} steps, 64 strikes, Sobol dim {2 * n_steps}",
            "seconds": sec, "path_steps_per_s": n_paths * n_steps / sec,
            "materialised_seconds": sec_m, "materialised_draw_bytes": n_paths * n_steps * 2 * 4,
            "max_rel_price_diff_fused_vs_materialised": float(
                ((res.price - res_m.price).abs() / res_m.price.abs().clamp_min(1e-12)).max()),
            "atm_call_price": float(res.price[j]), "strike": float(k[j])}


def run_euler_call_f64(reps=5):
    """The workload of the reference's only published timing for this path: a
    European call under Black-Scholes by the Euler scheme through
    GenericItoProcess.sample_paths, float64, 200,000 paths (PSEUDO_ANTITHETIC)
    x 100 steps to T = 1, priced at 3 strikes (synthetic parameters: S0 = 700,
    sigma = 0.25, r = 0.01, strikes 600 / 650 / 680).  Timed through the
    public API with CUDA events, sampling plus payoff reduction: once with the
    drift and volatility as plain Python callables (one step kernel per time
    step, the callables evaluated by torch), once with the structured GBM
    coefficients (one fused kernel for the whole loop)."""
    import torch
    from tqf.math.random import RandomType
    from tqf.models import GenericItoProcess, coefficients
    from tqf.pricing import european_payoff_stats
    s0, sigma, r, n = 700.0, 0.25, 0.01, 200_000
    k = np.array([600.0, 650.0, 680.0])

    def price(drift, vol):
        proc = GenericItoProcess(1, drift, vol, dtype=np.float64)
        paths = proc.sample_paths([1.0], num_samples=n, initial_state=np.array([s0]), time_step=0.01,
                                  random_type=RandomType.PSEUDO_ANTITHETIC, seed=42)
        return european_payoff_stats(paths[:, -1, 0], k, discount=float(np.exp(-r)))

    callables = (lambda t, x: r * x, lambda t, x: (sigma * x)[..., None])
    structured = coefficients.gbm([r], [sigma])
    out = {"config": "GBM Euler f64, 200000 paths (antithetic) x 100 steps, 3 strikes; sample_paths + payoff"}
    for name, (drift, vol) in (("callables", callables), ("structured", structured)):
        res = price(drift, vol)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = price(drift, vol)
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        sec = sorted(ts)[len(ts) // 2]
        out[name] = {"seconds": sec, "path_steps_per_s": n * 100 / sec,
                     "prices": [float(x) for x in res.price.cpu()]}
    bs = [float(closed_form_bs(s0, kk, r, sigma, 1.0)) for kk in k]
    out["black_scholes"] = bs
    # the reference's published wall times for this workload (TensorFlow on a
    # Colab CPU, core count not stated): graph mode and with XLA
    out["published_tf_cpu_seconds"] = {"graph": 2.162, "xla": 0.715}
    for name in ("callables", "structured"):
        out[name]["speedup_vs_published_tf_cpu"] = {m: t / out[name]["seconds"]
                                                    for m, t in out["published_tf_cpu_seconds"].items()}
    return out


def closed_form_bs(s, k, r, v, t):
    from math import erf, exp, log, sqrt
    d1 = (log(s / k) + (r + 0.5 * v * v) * t) / (v * sqrt(t))
    n = lambda x: 0.5 * (1.0 + erf(x / sqrt(2.0)))  # noqa: E731
    return s * n(d1) - k * exp(-r * t) * n(d1 - v * sqrt(t))


def run_greeks(n_paths=N_PATHS, n_steps=N_STEPS, reps=5):
    """Pathwise adjoint Greeks on the headline workload: the 7 sensitivities
    (spot, variance, mean reversion, theta, vol of vol, rho, rate) of the sum
    of the 64 strikes' prices, from the replaying adjoint kernel
    (tqf_heston_euler_adjoint: paths regenerated from their Philox counters,
    tangents carried forward, nothing stored), timed against one forward
    pricing of the same paths; central bump-and-revalue would take 14
    pricings.  Median of `reps` calls through the public API, CUDA events."""
    import torch
    from tqf.math.random import RandomType
    from tqf.pricing import heston_european_mc, heston_european_vjp
    k = strikes()
    params = dict(spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7,
                  discount_rate=0.02)
    kw = dict(strikes=k, expiry=1.0, num_samples=n_paths, num_time_steps=n_steps,
              random_type=RandomType.STATELESS, seed=(3, 4))
    g = np.ones(len(k))

    def timed(fn):
        out = fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return sorted(ts)[len(ts) // 2], out

    fwd_s, res = timed(lambda: heston_european_mc(**kw, **params))
    adj_s, grad = timed(lambda: heston_european_vjp(g, prices=res.price, **kw, **params))
    names = ("spot", "variance", "mean_reversion", "theta", "volvol", "rho", "discount_rate")
    return {"config": f"Heston FT-Euler FP32, {n_paths} paths x {n_steps} steps, 64 strikes, d(sum of prices)/d(7 params)",
            "forward_seconds": fwd_s, "adjoint_seconds": adj_s, "adjoint_over_forward": adj_s / fwd_s,
            "bump_and_revalue_seconds_est": 14 * fwd_s, "speedup_vs_bumps": 14 * fwd_s / adj_s,
            "adjoint_path_steps_per_s": n_paths * n_steps / adj_s,
            "sensitivities": {n: float(v) for n, v in zip(names, grad.cpu().numpy())}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["tqf", "reference"], default="tqf")
    ap.add_argument("--paths", type=int, default=N_PATHS)
    ap.add_argument("--time-steps", type=int, default=N_STEPS)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-neural-cv", action="store_true")
    ap.add_argument("--cv-only", action="store_true", help="run only the neural-CV measurement (small sizes ok)")
    ap.add_argument("--cv-eval-paths", type=int, default=1 << 26)
    ap.add_argument("--cv-train-steps", type=int, default=600)
    ap.add_argument("--cv-batch", type=int, default=1024, help="pilot paths per Adam step")
    ap.add_argument("--cv-lr", type=float, default=3e-3, help="Adam learning rate of the control-variate network")
    ap.add_argument("--cv-every", type=int, default=2, help="rebalance the control every n-th monitoring date")
    ap.add_argument("--no-basket", action="store_true")
    ap.add_argument("--basket-only", action="store_true", help="run only the 16-asset basket measurement")
    ap.add_argument("--basket-paths", type=int, default=1 << 22)
    ap.add_argument("--no-sobol", action="store_true")
    ap.add_argument("--no-lsm", action="store_true")
    ap.add_argument("--no-greeks", action="store_true")
    ap.add_argument("--no-heston-sobol", action="store_true")
    ap.add_argument("--heston-sobol-only", action="store_true",
                    help="run only the Heston pricing measurement with Sobol draws")
    ap.add_argument("--no-euler-call", action="store_true")
    ap.add_argument("--euler-call-only", action="store_true", help="run only the float64 Euler call measurement")
    ap.add_argument("--no-stored-paths", action="store_true")
    ap.add_argument("--stored-paths-only", action="store_true", help="run only the stored-path measurement")
    ap.add_argument("--greeks-only", action="store_true", help="run only the adjoint-Greeks measurement")
    ap.add_argument("--lsm-only", action="store_true", help="run only the Longstaff-Schwartz measurement")
    ap.add_argument("--lsm-paths", type=int, default=1 << 20)
    ap.add_argument("--sobol-only", action="store_true", help="run only the Sobol dim-1024 measurement")
    ap.add_argument("--sobol-chunk", type=int, default=1 << 20, help="points per Sobol launch")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "tqf" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        rate, cores, ppc, step_s = run_cpu_baseline(args.steps, args.warmup, args.cpu_budget)
        sample = f"oracle full-truncation Euler (numpy f32) {cores} procs x {ppc} paths x {N_STEPS} steps per step, incl. RNG + 64-strike payoff"
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.paths, args.time_steps, 1),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    if args.lsm_only:
        print(json.dumps({"lsm": run_lsm(n_paths=args.lsm_paths)}))
        return
    if args.euler_call_only:
        print(json.dumps({"euler_call_f64": run_euler_call_f64()}))
        return
    if args.stored_paths_only:
        print(json.dumps({"stored_paths": run_stored_paths(n_paths=args.paths)}))
        return
    if args.greeks_only:
        print(json.dumps({"greeks": run_greeks(n_paths=args.paths)}))
        return
    if args.sobol_only:
        print(json.dumps({"sobol": run_sobol(chunk=args.sobol_chunk)}))
        return
    if args.heston_sobol_only:
        print(json.dumps({"heston_sobol": run_heston_sobol(n_paths=args.paths)}))
        return
    if args.basket_only:
        print(json.dumps({"basket": run_basket(paths_n=args.basket_paths)}))
        return
    if args.cv_only:
        print(json.dumps({"neural_cv": run_neural_cv(eval_paths=args.cv_eval_paths, train_steps=args.cv_train_steps,
                                                  batch_paths=args.cv_batch, lr=args.cv_lr,
                                                  control_every=args.cv_every)}))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # CPU sample first (spawned workers, before any CUDA context exists).
        rate, cores, ppc, _ = run_cpu_baseline(2, 1, args.cpu_budget)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"oracle full-truncation Euler (numpy f32), {cores} procs x {ppc} paths x {N_STEPS} steps, 2 timed rounds, incl. RNG + 64-strike payoff"}
    line = run_gpu(args, rank, world, local_rank)
    if rank == 0 and world == 1 and not args.no_neural_cv:
        line["neural_cv"] = run_neural_cv(eval_paths=args.cv_eval_paths, train_steps=args.cv_train_steps,
                                                  batch_paths=args.cv_batch, lr=args.cv_lr,
                                                  control_every=args.cv_every)
    if rank == 0 and world == 1 and not args.no_basket:
        line["basket"] = run_basket(paths_n=args.basket_paths)
    if rank == 0 and world == 1 and not args.no_sobol:
        line["sobol"] = run_sobol()
    if rank == 0 and world == 1 and not args.no_lsm:
        line["lsm"] = run_lsm(n_paths=args.lsm_paths)
    if rank == 0 and world == 1 and not args.no_greeks:
        line["greeks"] = run_greeks(n_paths=args.paths)
    if rank == 0 and world == 1 and not args.no_heston_sobol:
        line["heston_sobol"] = run_heston_sobol(n_paths=args.paths)
    if rank == 0 and world == 1 and not args.no_euler_call:
        line["euler_call_f64"] = run_euler_call_f64()
    if rank == 0 and world == 1 and not args.no_stored_paths:
        line["stored_paths"] = run_stored_paths(n_paths=args.paths)
    if rank == 0:
        line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
