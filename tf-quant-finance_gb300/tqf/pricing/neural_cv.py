"""Neural martingale control variate for the Heston arithmetic-Asian call.

Pipeline, all on the GPU through libtqf.so:

1. ``pilot``: full-truncation Euler paths (``tqf_heston_asian`` mode 1) give,
   per path and control interval j, the start features (t_j, log S_j, v_j),
   the discounted-spot increment dS~_j and the discounted payoff Y.  The
   control dates are every ``control_every``-th monitoring date counted back
   from the last; the network's position is held over the dates in between.
2. ``train``: the MLP g (3 -> 64 -> 64 -> 1, SiLU, BF16 weights, FP32
   accumulation) minimises mean_p (Y_p - c - sum_k g_pk dS~_pk)^2 with Adam
   (``tqf_mlp_train_step`` on tcgen05 tensor cores + ``tqf_mlp_adam``).
3. ``price``: fresh paths with the network fused into the path kernel
   (mode 2) return the sums of Y, C = sum_k g_k dS~_k and their squares and
   cross product; the estimator is mean(Y - C), unbiased because
   E[S~_{i+1} | F_i] = S~_i under the log-Euler step.  Mode 0 is plain MC.

The monitoring dates are snapped to the simulation grid exactly as
``euler_sampling.sample(times_grid=...)`` snaps requested times
(tff/models/utils.py:261-271).
"""

from __future__ import annotations

import ctypes
import dataclasses
import math
import time

import numpy as np
import torch

from tqf import _lib
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import heston_model, utils
from tqf.models.coefficients import HestonFullTruncation
from tqf.pricing.european import workspace

H = 64
IN = 16
OFF_W1, OFF_W2 = 0, 64 * 16
OFF_B2 = OFF_W2 + 64 * 64
OFF_W3 = OFF_B2 + 64
OFF_B3 = OFF_W3 + 64
OFF_C = OFF_B3 + 1
NUM_PARAMS = OFF_C + 1


@dataclasses.dataclass
class AsianEstimate:
    price: float
    standard_error: float
    plain_price: float
    plain_standard_error: float
    var_plain: float
    var_cv: float
    vrf: float
    num_paths: int
    seconds: float  # GPU time of the pricing pass (CUDA events)
    mean_control: float = 0.0  # mean of C (zero in expectation)
    se_control: float = 0.0


def stage_marks(date_steps, busy=()) -> np.ndarray:
    """Steps at which the fused inference advances its network pipeline.

    The evaluation for control interval j starts after step date_steps[j-1]
    (before step 0 for j = 0) and must be complete after step date_steps[j];
    its two middle stages run at the free steps strictly inside the interval
    nearest a third and two thirds of the way between.  ``busy`` steps (the
    other monitoring dates) carry a date slot and are never marked; without a
    free step the kernel runs the stage at the date."""
    busy = set(int(b) for b in np.asarray(busy, dtype=np.int64).reshape(-1).tolist())
    marks = []
    prev = -1
    for s in np.asarray(date_steps, dtype=np.int64).tolist():
        gap = s - prev
        free = [m for m in range(prev + 1, s) if m not in busy]
        chosen = []
        for target in (prev + gap / 3.0, prev + 2.0 * gap / 3.0):
            cands = [m for m in free if not chosen or m > chosen[-1]]
            if cands:
                chosen.append(min(cands, key=lambda m: (abs(m - target), m)))
        marks += chosen
        prev = s
    return np.asarray(marks, dtype=np.int64)


def control_dates(num_dates: int, every: int) -> np.ndarray:
    """Indices of the monitoring dates that end a control interval: every
    ``every``-th date counted back from the last (which always ends one)."""
    if every < 1:
        raise ValueError("control_every must be >= 1")
    k = np.arange(num_dates)
    return k[(num_dates - 1 - k) % every == 0]


def _bf16_bits(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.bfloat16).view(torch.int16)


class HestonAsianCV:
    """Heston (full-truncation Euler, FP32) arithmetic-Asian call with a neural
    martingale control variate."""

    def __init__(self, *, spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04, volvol=0.3, rho=-0.7,
                 rate=0.02, expiry=1.0, strike=100.0, num_dates=52, num_time_steps=252, init_seed=0,
                 pipeline_stages=True, control_every=1):
        self.device = _lib.require_cuda()
        d = self.device
        self.spot, self.v0, self.kappa, self.theta, self.xi, self.rho = spot, variance, mean_reversion, theta, volvol, rho
        self.rate, self.T, self.strike = rate, expiry, strike
        self.num_steps, self.num_dates = int(num_time_steps), int(num_dates)
        f32 = np.float32
        grid = np.linspace(0.0, expiry, self.num_steps + 1).astype(f32)
        dates = (np.arange(1, self.num_dates + 1) * (expiry / self.num_dates)).astype(f32)
        _, keep, ti = utils.prepare_grid(times=dates, time_step=None, dtype=f32, times_grid=grid)
        if len(set(ti.tolist())) != self.num_dates or ti.min() < 1:
            raise ValueError("monitoring dates must map to distinct grid points after t = 0")
        slots = np.full(self.num_steps, -1, np.int32)
        slots[ti - 1] = np.arange(self.num_dates)  # state after step i is at grid point i + 1
        self.control_every = int(control_every)
        self.control_dates = control_dates(self.num_dates, self.control_every)
        self.num_control = len(self.control_dates)
        if pipeline_stages:
            slots[stage_marks(ti[self.control_dates] - 1, busy=ti - 1)] = -2
        dt = (grid[1:] - grid[:-1]).astype(f32)
        coef = HestonFullTruncation(rate, mean_reversion, theta, volvol, rho)
        rows = heston_model.full_truncation_table(coef, grid, dt, np.sqrt(dt).astype(f32), slots, self.num_steps)
        self.step_table = utils.step_table(rows, torch.float32, d)
        t_dates = grid[ti].astype(np.float64)
        dtab = np.zeros((self.num_dates, 4), np.float32)
        dtab[:, 0] = t_dates
        dtab[:, 1] = np.exp(-rate * t_dates)
        dtab[:, 2] = 1.0  # hold the network's position over the date ...
        dtab[self.control_dates, 2] = 0.0  # ... except at the control dates
        self.date_table = torch.as_tensor(dtab).to(d)
        self.dates = t_dates
        self.discount_T = float(np.exp(-rate * float(grid[-1])))
        # feature normalisation: t / T, (log S - log S0) / sqrt(theta T), (v - theta) / (xi sqrt(theta / 2 kappa))
        self.feat_shift = [0.0, math.log(spot), theta]
        self.feat_scale = [1.0 / expiry, 1.0 / math.sqrt(theta * expiry),
                           1.0 / max(volvol * math.sqrt(theta / (2 * mean_reversion)), 1e-6)]
        # one training CTA holds whole paths (all their control intervals) in one 128-row tile
        self.train_paths_per_cta = max(1, 128 // self.num_control)
        self._init_params(init_seed)
        self.loss_history: list[float] = []
        self.train_seconds = 0.0
        self.pilot_seconds = 0.0

    # ---- parameters --------------------------------------------------------------
    def _init_params(self, seed):
        g = torch.Generator().manual_seed(seed)
        u = lambda shape, fan_in: (torch.rand(shape, generator=g) * 2 - 1) / math.sqrt(fan_in)  # noqa: E731
        p = torch.zeros(NUM_PARAMS, dtype=torch.float32)
        w1 = torch.zeros(H, IN)
        w1[:, :3] = u((H, 3), 3)
        w1[:, 3] = u((H,), 3)  # layer-1 bias lives in column 3
        p[OFF_W1:OFF_W2] = w1.reshape(-1)
        p[OFF_W2:OFF_B2] = u((H, H), H).reshape(-1)
        p[OFF_B2:OFF_W3] = u((H,), H)
        p[OFF_W3:OFF_B3] = u((H,), H)
        p[OFF_B3] = float(u((1,), H)[0])
        self.set_params(p)

    def set_params(self, p: torch.Tensor):
        d = self.device
        self.params = p.detach().to(torch.float32).clone().to(d)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.w1_bf16 = _bf16_bits(self.params[OFF_W1:OFF_W2]).contiguous()
        self.w2_bf16 = _bf16_bits(self.params[OFF_W2:OFF_B2]).contiguous()
        self.adam_t = 0

    def _mlp_struct(self):
        """Inference weights: W2 stays on the device (tensor-core operand);
        the small layers are copied to the host once and passed by value."""
        p = self.params.detach().cpu().numpy()
        hw = _lib.MlpHostWeights()
        w1 = p[OFF_W1:OFF_W2].reshape(H, IN)
        hwv = np.ctypeslib.as_array(hw.w1)
        hwv[:] = w1[:, :4]
        np.ctypeslib.as_array(hw.b2)[:] = p[OFF_B2:OFF_W3]
        np.ctypeslib.as_array(hw.w3)[:] = p[OFF_W3:OFF_B3]
        hw.b3 = float(p[OFF_B3])
        self._host_weights = hw  # kept alive for the call
        w = _lib.MlpWeights()
        w.w2_bf16 = self.w2_bf16.data_ptr()
        w.host = ctypes.pointer(hw)
        for i in range(3):
            w.feat_scale[i] = self.feat_scale[i]
            w.feat_shift[i] = self.feat_shift[i]
        return w

    def _args(self, mode, num_paths, seed, path_offset):
        a = _lib.HestonAsianArgs()
        a.mode = mode
        a.num_steps = self.num_steps
        a.num_paths = int(num_paths)
        a.step_table = self.step_table.data_ptr()
        a.num_dates = self.num_dates
        a.date_table = self.date_table.data_ptr()
        a.x0, a.v0 = math.log(self.spot), float(self.v0)
        a.strike = float(self.strike)
        a.discount_T = self.discount_T
        a.draws = mvn.philox_draws(RandomType.STATELESS, seed, int(num_paths), path_offset)
        a.dev_status = _lib.status_buffer(self.device).data_ptr()
        return a

    # ---- stages ------------------------------------------------------------------
    def pilot(self, num_paths=1 << 20, seed=(977, 5)):
        d = self.device
        D = self.num_control
        # date-major storage (coalesced stores in the path kernel); the
        # attributes are [N, D, ...] views of it
        self._feats_dm = torch.empty((D, num_paths, 4), dtype=torch.float32, device=d)
        self._dS_dm = torch.empty((D, num_paths), dtype=torch.float32, device=d)
        self.feats = self._feats_dm.permute(1, 0, 2)
        self.dS = self._dS_dm.t()
        self.Y = torch.empty((num_paths,), dtype=torch.float32, device=d)
        a = self._args(1, num_paths, seed, 0)
        a.pilot_feats, a.pilot_dS, a.pilot_Y = self._feats_dm.data_ptr(), self._dS_dm.data_ptr(), self.Y.data_ptr()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        _lib.call("tqf_heston_asian", a, s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        self.pilot_seconds = e0.elapsed_time(e1) * 1e-3
        self.num_pilot = int(num_paths)
        return self.feats, self.dS, self.Y

    def _train_args(self, path_begin, batch_paths, partials):
        t = _lib.MlpTrainArgs()
        t.num_dates = self.num_control
        t.batch_paths = int(batch_paths)
        t.paths_per_cta = self.train_paths_per_cta
        t.path_begin = int(path_begin)
        t.pilot_paths = self.num_pilot
        t.feats, t.dS, t.Y = self._feats_dm.data_ptr(), self._dS_dm.data_ptr(), self.Y.data_ptr()
        t.params = self.params.data_ptr()
        t.w1_bf16, t.w2_bf16 = self.w1_bf16.data_ptr(), self.w2_bf16.data_ptr()
        for i in range(3):
            t.feat_scale[i] = self.feat_scale[i]
            t.feat_shift[i] = self.feat_shift[i]
        t.grad_partials = partials.data_ptr()
        t.dev_status = _lib.status_buffer(self.device).data_ptr()
        return t

    def gradient(self, path_begin, batch_paths):
        """(grad [NUM_PARAMS], loss) of one minibatch (for tests)."""
        if batch_paths % self.train_paths_per_cta:
            raise ValueError(f"batch_paths must be a multiple of {self.train_paths_per_cta}")
        n_cta = batch_paths // self.train_paths_per_cta
        partials = torch.zeros((n_cta, NUM_PARAMS + 2), dtype=torch.float32, device=self.device)
        _lib.call("tqf_mlp_train_step", self._train_args(path_begin, batch_paths, partials), _lib.stream_ptr())
        s = partials.sum(0)
        return s[:NUM_PARAMS], float(s[NUM_PARAMS])

    def train(self, steps=2000, batch_paths=512, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, graph=True,
              init_intercept=True):
        """Adam on minibatches of pilot paths taken in order (wrapping).  The
        2 x steps kernel launches are captured once into a CUDA graph and
        replayed (graph=True) so that host launch overhead stays out of the
        loop; each kernel is a programmatic dependent launch, so the next one
        starts its independent prologue while the previous one finishes.
        ``train_seconds`` is the GPU time of the replay.  Before the first
        step the loss offset c starts at the pilot mean of Y
        (init_intercept), so that the residuals start centred."""
        if batch_paths % self.train_paths_per_cta:
            raise ValueError(f"batch_paths must be a multiple of {self.train_paths_per_cta}")
        d = self.device
        if init_intercept and self.adam_t == 0:
            self.params[OFF_C] = self.Y[: self.num_pilot].double().mean().float()
        n_cta = batch_paths // self.train_paths_per_cta
        partials = torch.zeros((n_cta, NUM_PARAMS + 2), dtype=torch.float32, device=d)
        losses = torch.zeros(steps, dtype=torch.float32, device=d)
        lib = _lib.load()
        span = self.num_pilot - batch_paths
        step_args, adam_args = [], []
        for k in range(steps):
            begin = (k * batch_paths) % max(span, 1)
            step_args.append(self._train_args(begin, batch_paths, partials))
            self.adam_t += 1
            adam = _lib.MlpAdamArgs()
            adam.params, adam.m, adam.v = self.params.data_ptr(), self.m.data_ptr(), self.v.data_ptr()
            adam.grad_partials = partials.data_ptr()
            adam.num_partials = n_cta
            adam.w1_bf16, adam.w2_bf16 = self.w1_bf16.data_ptr(), self.w2_bf16.data_ptr()
            adam.lr, adam.beta1, adam.beta2, adam.eps = lr, beta1, beta2, eps
            adam.bias1 = 1.0 - beta1 ** self.adam_t
            adam.bias2 = 1.0 - beta2 ** self.adam_t
            adam.loss_out = losses[k:].data_ptr()
            adam_args.append(adam)

        def launch_all(stream_ptr):
            for ta, aa in zip(step_args, adam_args):
                _lib.check(lib.tqf_mlp_train_step(ta, stream_ptr), "tqf_mlp_train_step")
                _lib.check(lib.tqf_mlp_adam(aa, stream_ptr), "tqf_mlp_adam")

        if graph:
            # load both kernels before capture without touching the model state
            self.gradient(0, batch_paths)
            scratch = torch.zeros_like(self.params)
            warm = _lib.MlpAdamArgs()
            warm.params, warm.m, warm.v = scratch.data_ptr(), scratch.data_ptr(), scratch.data_ptr()
            w1s, w2s = torch.zeros_like(self.w1_bf16), torch.zeros_like(self.w2_bf16)
            warm.grad_partials, warm.num_partials = partials.data_ptr(), n_cta
            warm.w1_bf16, warm.w2_bf16 = w1s.data_ptr(), w2s.data_ptr()
            warm.lr, warm.beta1, warm.beta2, warm.eps, warm.bias1, warm.bias2 = 0.0, 0.9, 0.999, 1e-8, 1.0, 1.0
            _lib.check(lib.tqf_mlp_adam(warm, _lib.stream_ptr()), "tqf_mlp_adam")
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                launch_all(torch.cuda.current_stream().cuda_stream)
            s = torch.cuda.current_stream()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            g.replay()
            e1.record(s)
            e1.synchronize()
            del g
        else:
            s = torch.cuda.current_stream()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            launch_all(s.cuda_stream)
            e1.record(s)
            e1.synchronize()
        self.train_seconds = e0.elapsed_time(e1) * 1e-3
        _lib.check_device_status(d)
        self.loss_history = losses.cpu().tolist()
        return self.loss_history

    def price(self, num_paths, control_variate=True, seed=(31, 41), path_offset=0, path_values=None) -> AsianEstimate:
        """Fresh paths: plain MC (control_variate=False) or the fused control
        variate.  ``path_values`` (optional float32 [num_paths, 2] device
        tensor) receives each path's (Y, C)."""
        d = self.device
        mode = 2 if control_variate else 0
        out = torch.zeros(5, dtype=torch.float64, device=d)
        ws = workspace(int(_lib.load().tqf_heston_asian_workspace_bytes(mode, int(num_paths), self.num_steps)), d,
                       f"asian{mode}")
        a = self._args(mode, num_paths, seed, path_offset)
        if control_variate:
            a.mlp = self._mlp_struct()
        a.out = out.data_ptr()
        if path_values is not None:
            if (path_values.dtype != torch.float32 or tuple(path_values.shape) != (int(num_paths), 2)
                    or not path_values.is_contiguous() or path_values.device != d):
                raise ValueError("path_values must be a contiguous float32 [num_paths, 2] tensor on the device")
            a.path_values = path_values.data_ptr()
        a.workspace = ws.data_ptr()
        a.workspace_bytes = ws.numel()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        _lib.call("tqf_heston_asian", a, s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        _lib.check_device_status(d)
        sec = e0.elapsed_time(e1) * 1e-3
        sy, syy, sc, scc, syc = (float(x) for x in out.cpu())
        n = float(num_paths)
        my, mc = sy / n, sc / n
        var_y = max(syy / n - my * my, 0.0) * n / (n - 1)
        var_c = max(scc / n - mc * mc, 0.0) * n / (n - 1)
        cov = (syc / n - my * mc) * n / (n - 1)
        var_cv = max(var_y + var_c - 2 * cov, 0.0) if control_variate else var_y
        est = my - mc if control_variate else my
        return AsianEstimate(price=est, standard_error=math.sqrt(var_cv / n), plain_price=my,
                             plain_standard_error=math.sqrt(var_y / n), var_plain=var_y, var_cv=var_cv,
                             vrf=var_y / var_cv if var_cv > 0 else float("inf"), num_paths=int(num_paths),
                             seconds=sec, mean_control=mc, se_control=math.sqrt(var_c / n))


def time_to_ci(estimate: AsianEstimate, rel_halfwidth=1e-4, z=1.96) -> dict:
    """Paths and GPU seconds needed for a 95% CI half-width of rel_halfwidth x price,
    extrapolated from one run (cost linear in paths, variance ~ 1 / paths)."""
    target_se = rel_halfwidth * abs(estimate.price) / z
    se = estimate.standard_error
    n_req = estimate.num_paths * (se / target_se) ** 2
    return {"paths": n_req, "seconds": estimate.seconds * n_req / estimate.num_paths}


__all__ = ["HestonAsianCV", "AsianEstimate", "time_to_ci", "stage_marks", "control_dates"]
