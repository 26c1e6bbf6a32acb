"""ctypes binding of libtqf.so (the C ABI declared in include/tqf.h).

The library is the only compute path: if it is missing, or no CUDA device is
present, every entry point raises instead of falling back to the CPU.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

from tqf.errors import InvalidArgumentError

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libtqf.so")
DATA_DIR = os.path.join(_HERE, "data")
JOE_KUO_PATH = os.path.join(DATA_DIR, "new-joe-kuo-6.21201")

TQF_OK = 0
TQF_E_INVALID = -1
TQF_E_CUDA = -2
TQF_E_UNSUPPORTED = -3
TQF_E_TIMEOUT = -4
TQF_E_IO = -5

TQF_F32 = 0
TQF_F64 = 1
DRAWS_MEMORY = 0
DRAWS_PHILOX = 1
DRAWS_SOBOL = 2

SOBOL_U32 = 0
SOBOL_F32 = 1
SOBOL_F64 = 2
SOBOL_NORMAL_F32 = 3
SOBOL_NORMAL_F64 = 4
SOBOL_F32_CENTERED = 5

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_u32 = ctypes.c_uint32
c_vp = ctypes.c_void_p


class Draws(ctypes.Structure):
    _fields_ = [
        ("source", c_i32),
        ("antithetic", c_i32),
        ("ptr", c_vp),
        ("stride_step", c_i64),
        ("stride_path", c_i64),
        ("stride_comp", c_i64),
        ("key0", c_u32),
        ("key1", c_u32),
        ("path_offset", c_i64),
        ("antithetic_half", c_i64),
    ]


class PathOutput(ctypes.Structure):
    _fields_ = [("ptr", c_vp), ("num_slots", c_i32), ("init_slot", c_i32), ("every_step", c_i32), ("pad0", c_i32)]


class Payoff(ctypes.Structure):
    _fields_ = [
        ("num_strikes", c_i32),
        ("pad0", c_i32),
        ("strikes", c_vp),
        ("is_call", c_vp),
        ("spot_scale", ctypes.c_double),
        ("out", c_vp),
        ("workspace", c_vp),
        ("workspace_bytes", ctypes.c_size_t),
    ]


class EulerAffineArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_steps", c_i32),
        ("x0_per_path", c_i32),
        ("step_table", c_vp),
        ("x0", c_vp),
        ("drift_m", c_vp),
        ("drift_M", c_vp),
        ("vol_s0", c_vp),
        ("vol_s1", c_vp),
        ("vol_C", c_vp),
        ("draws", Draws),
        ("output", PathOutput),
        ("dev_status", c_vp),
    ]


class HaltonArgs(ctypes.Structure):
    _fields_ = [
        ("dim", c_i32),
        ("out_kind", c_i32),
        ("num_results", c_i64),
        ("first_index", c_i64),
        ("sequence_indices", c_vp),
        ("primes", c_vp),
        ("max_sizes", c_vp),
        ("perms", c_vp),
        ("perm_offsets", c_vp),
        ("radix_sum", c_i32),
        ("pad0", c_i32),
        ("zero_correction", c_vp),
        ("out", c_vp),
    ]


class DigitalNetArgs(ctypes.Structure):
    _fields_ = [
        ("dim", c_i32),
        ("log_num_results", c_i32),
        ("num_digits", c_i32),
        ("out_kind", c_i32),
        ("tent", c_i32),
        ("int_bits", c_i32),
        ("count", c_i64),
        ("sequence_indices", c_vp),
        ("matrices", c_vp),
        ("digital_shift", c_vp),
        ("out", c_vp),
    ]


class LatticeArgs(ctypes.Structure):
    _fields_ = [
        ("dim", c_i32),
        ("out_kind", c_i32),
        ("tent", c_i32),
        ("int_bits", c_i32),
        ("num_results", c_i64),
        ("count", c_i64),
        ("sequence_indices", c_vp),
        ("generating_vectors", c_vp),
        ("additive_shift", c_vp),
        ("out", c_vp),
    ]


class HullWhiteArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_steps", c_i32),
        ("pad0", c_i32),
        ("table", c_vp),
        ("f0", c_vp),
        ("chol", c_vp),
        ("slots", c_vp),
        ("draws", Draws),
        ("output", PathOutput),
    ]


class HjmArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_steps", c_i32),
        ("num_slots", c_i32),
        ("table", c_vp),
        ("mean_reversion", c_vp),
        ("f0", c_vp),
        ("grid_slot", c_vp),
        ("draws", Draws),
        ("rate_out", c_vp),
        ("df_out", c_vp),
        ("x_out", c_vp),
    ]


class MilsteinAffineArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_steps", c_i32),
        ("x0_per_path", c_i32),
        ("order", c_i32),
        ("pad0", c_i32),
        ("step_table", c_vp),
        ("x0", c_vp),
        ("drift_m", c_vp),
        ("drift_M", c_vp),
        ("vol_s0", c_vp),
        ("vol_s1", c_vp),
        ("vol_C", c_vp),
        ("draws", Draws),
        ("output", PathOutput),
        ("dev_status", c_vp),
    ]


class MilsteinUpdateArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("step", c_i32),
        ("out_slot", c_i32),
        ("order", c_i32),
        ("num_slots", c_i32),
        ("dt", ctypes.c_double),
        ("sqrt_dt", ctypes.c_double),
        ("x", c_vp),
        ("drift", c_vp),
        ("vol", c_vp),
        ("grad", c_vp),
        ("x_next", c_vp),
        ("draws", Draws),
        ("paths_out", c_vp),
        ("increments_out", c_vp),
    ]


class EulerUpdateArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("step", c_i32),
        ("out_slot", c_i32),
        ("dt", ctypes.c_double),
        ("sqrt_dt", ctypes.c_double),
        ("x", c_vp),
        ("drift", c_vp),
        ("vol", c_vp),
        ("x_next", c_vp),
        ("draws", Draws),
        ("paths_out", c_vp),
        ("num_slots", c_i32),
        ("pad0", c_i32),
    ]


class HestonArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("num_steps", c_i32),
        ("num_paths", c_i64),
        ("step_table", c_vp),
        ("x0", ctypes.c_double),
        ("v0", ctypes.c_double),
        ("draws", Draws),
        ("output", PathOutput),
        ("payoff", Payoff),
        ("dev_status", c_vp),
    ]


class HestonAdjointArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("num_steps", c_i32),
        ("num_paths", c_i64),
        ("step_table", c_vp),
        ("x0", ctypes.c_double),
        ("v0", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("theta", ctypes.c_double),
        ("xi", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("draws", Draws),
        ("num_strikes", c_i32),
        ("pad0", c_i32),
        ("strikes", c_vp),
        ("is_call", c_vp),
        ("weights", c_vp),
        ("out", c_vp),
        ("workspace", c_vp),
        ("workspace_bytes", ctypes.c_size_t),
        ("dev_status", c_vp),
    ]


class MvgbmArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_steps", c_i32),
        ("x0_per_path", c_i32),
        ("step_table", c_vp),
        ("x0", c_vp),
        ("drift", c_vp),
        ("vol", c_vp),
        ("chol", c_vp),
        ("draws", Draws),
        ("output", PathOutput),
        ("dev_status", c_vp),
        ("lz_mode", c_i32),
        ("pad0", c_i32),
    ]


class LsmArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_times", c_i32),
        ("paths_batch", c_i32),
        ("batch", c_i32),
        ("num_basis", c_i32),
        ("degree", c_i32),
        ("num_exercise", c_i32),
        ("num_calibration", c_i64),
        ("paths", c_vp),
        ("strikes", c_vp),
        ("exponents", c_vp),
        ("exercise_times", c_vp),
        ("discount", c_vp),
        ("disc_stride_e", c_i64),
        ("disc_stride_n", c_i64),
        ("disc_stride_b", c_i64),
        ("state", c_vp),
        ("init", c_i32),
        ("upd_index", c_i32),
        ("acc_index", c_i32),
        ("final_pass", c_i32),
        ("init_payoff", c_vp),
        ("upd_payoff", c_vp),
        ("upd_design", c_vp),
        ("acc_payoff", c_vp),
        ("acc_design", c_vp),
        ("out", c_vp),
        ("workspace", c_vp),
        ("workspace_bytes", ctypes.c_size_t),
        ("dev_status", c_vp),
    ]


class BasketArgs(ctypes.Structure):
    _fields_ = [
        ("dtype", c_i32),
        ("dim", c_i32),
        ("num_paths", c_i64),
        ("num_steps", c_i32),
        ("is_call", c_i32),
        ("sqrt_dt", c_vp),
        ("total_time", ctypes.c_double),
        ("strike", ctypes.c_double),
        ("spot", c_vp),
        ("drift", c_vp),
        ("vol", c_vp),
        ("chol", c_vp),
        ("weights", c_vp),
        ("draws", Draws),
        ("out", c_vp),
        ("workspace", c_vp),
        ("workspace_bytes", ctypes.c_size_t),
        ("dev_status", c_vp),
    ]


class MlpHostWeights(ctypes.Structure):
    _fields_ = [
        ("w1", (ctypes.c_float * 4) * 64),
        ("b2", ctypes.c_float * 64),
        ("w3", ctypes.c_float * 64),
        ("b3", ctypes.c_float),
    ]


class MlpWeights(ctypes.Structure):
    _fields_ = [
        ("w2_bf16", c_vp),
        ("host", ctypes.POINTER(MlpHostWeights)),
        ("feat_scale", ctypes.c_float * 3),
        ("feat_shift", ctypes.c_float * 3),
    ]


class HestonAsianArgs(ctypes.Structure):
    _fields_ = [
        ("mode", c_i32),
        ("num_steps", c_i32),
        ("num_paths", c_i64),
        ("step_table", c_vp),
        ("num_dates", c_i32),
        ("pad0", c_i32),
        ("date_table", c_vp),
        ("x0", ctypes.c_double),
        ("v0", ctypes.c_double),
        ("strike", ctypes.c_double),
        ("discount_T", ctypes.c_double),
        ("draws", Draws),
        ("mlp", MlpWeights),
        ("pilot_feats", c_vp),
        ("pilot_dS", c_vp),
        ("pilot_Y", c_vp),
        ("out", c_vp),
        ("workspace", c_vp),
        ("workspace_bytes", ctypes.c_size_t),
        ("dev_status", c_vp),
        ("path_values", c_vp),
    ]


class MlpTrainArgs(ctypes.Structure):
    _fields_ = [
        ("num_dates", c_i32),
        ("batch_paths", c_i32),
        ("paths_per_cta", c_i32),
        ("pad0", c_i32),
        ("path_begin", c_i64),
        ("pilot_paths", c_i64),
        ("feats", c_vp),
        ("dS", c_vp),
        ("Y", c_vp),
        ("params", c_vp),
        ("w1_bf16", c_vp),
        ("w2_bf16", c_vp),
        ("feat_scale", ctypes.c_float * 3),
        ("feat_shift", ctypes.c_float * 3),
        ("grad_partials", c_vp),
        ("dev_status", c_vp),
    ]


class MlpAdamArgs(ctypes.Structure):
    _fields_ = [
        ("params", c_vp),
        ("m", c_vp),
        ("v", c_vp),
        ("grad_partials", c_vp),
        ("num_partials", c_i32),
        ("pad0", c_i32),
        ("w1_bf16", c_vp),
        ("w2_bf16", c_vp),
        ("lr", ctypes.c_float),
        ("beta1", ctypes.c_float),
        ("beta2", ctypes.c_float),
        ("eps", ctypes.c_float),
        ("bias1", ctypes.c_float),
        ("bias2", ctypes.c_float),
        ("loss_out", c_vp),
    ]


# name -> (restype, argtypes)
_SIGNATURES = {
    "tqf_abi_version": (ctypes.c_int, []),
    "tqf_last_error": (ctypes.c_char_p, []),
    "tqf_launch_count": (ctypes.c_uint64, []),
    "tqf_sobol_direction_numbers": (ctypes.c_int, [ctypes.c_char_p, c_i32, c_vp]),
    "tqf_sobol_num_digits": (c_i32, [c_i64, c_i64]),
    "tqf_sobol_sample": (ctypes.c_int, [c_vp, c_i32, c_i64, c_i64, c_i32, c_i32, c_vp, c_vp]),
    "tqf_sobol_normal_draws": (ctypes.c_int, [c_vp, c_i32, c_i32, c_i64, c_i64, c_i32, c_i32, c_vp, c_vp]),
    "tqf_philox4x32_10": (ctypes.c_int, [c_u32, c_u32, c_u32, c_u32, c_u32, c_u32, c_i64, c_vp, c_vp]),
    "tqf_philox_normal_draws": (ctypes.c_int, [ctypes.POINTER(Draws), c_i32, c_i32, c_i64, c_i32, c_vp, c_vp]),
    "tqf_euler_affine": (ctypes.c_int, [ctypes.POINTER(EulerAffineArgs), c_vp]),
    "tqf_euler_update": (ctypes.c_int, [ctypes.POINTER(EulerUpdateArgs), c_vp]),
    "tqf_milstein_affine": (ctypes.c_int, [ctypes.POINTER(MilsteinAffineArgs), c_vp]),
    "tqf_halton_sample": (ctypes.c_int, [ctypes.POINTER(HaltonArgs), c_vp]),
    "tqf_hull_white_paths": (ctypes.c_int, [ctypes.POINTER(HullWhiteArgs), c_vp]),
    "tqf_hjm_paths": (ctypes.c_int, [ctypes.POINTER(HjmArgs), c_vp]),
    "tqf_digital_net_sample": (ctypes.c_int, [ctypes.POINTER(DigitalNetArgs), c_vp]),
    "tqf_lattice_rule_sample": (ctypes.c_int, [ctypes.POINTER(LatticeArgs), c_vp]),
    "tqf_halton_permutations": (ctypes.c_int, [c_i32, c_i32, c_vp, c_vp, c_i32, ctypes.c_uint64, c_vp, c_vp, c_vp]),
    "tqf_milstein_update": (ctypes.c_int, [ctypes.POINTER(MilsteinUpdateArgs), c_vp]),
    "tqf_heston_euler": (ctypes.c_int, [ctypes.POINTER(HestonArgs), c_vp]),
    "tqf_heston_qe": (ctypes.c_int, [ctypes.POINTER(HestonArgs), c_vp]),
    "tqf_heston_euler_price_noalloc": (ctypes.c_int, [ctypes.POINTER(HestonArgs), c_vp]),
    "tqf_heston_workspace_bytes": (ctypes.c_size_t, [c_i32, c_i32, c_i64, c_i32]),
    "tqf_european_payoff_sums": (ctypes.c_int, [c_i32, c_vp, c_i64, c_i64, c_i32, ctypes.POINTER(Payoff), c_vp]),
    "tqf_european_workspace_bytes": (ctypes.c_size_t, [c_i64, c_i32]),
    "tqf_mc_price_stats": (ctypes.c_int, [c_vp, c_i32, c_i64, ctypes.c_double, c_vp, c_vp]),
    "tqf_heston_euler_adjoint": (ctypes.c_int, [ctypes.POINTER(HestonAdjointArgs), c_vp]),
    "tqf_heston_adjoint_workspace_bytes": (ctypes.c_size_t, [c_i64]),
    "tqf_cholesky_f64": (ctypes.c_int, [c_vp, c_i32, c_vp, c_vp, c_vp]),
    "tqf_mvgbm_paths": (ctypes.c_int, [ctypes.POINTER(MvgbmArgs), c_vp]),
    "tqf_lsm_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(LsmArgs)]),
    "tqf_lsm_gather": (ctypes.c_int, [ctypes.POINTER(LsmArgs), c_vp]),
    "tqf_lsm_price": (ctypes.c_int, [ctypes.POINTER(LsmArgs), c_vp]),
    "tqf_lsm_pass": (ctypes.c_int, [ctypes.POINTER(LsmArgs), c_vp]),
    "tqf_lsm_solve": (ctypes.c_int, [ctypes.POINTER(LsmArgs), c_vp]),
    "tqf_basket_price": (ctypes.c_int, [ctypes.POINTER(BasketArgs), c_vp]),
    "tqf_basket_workspace_bytes": (ctypes.c_size_t, [c_i32, c_i32, c_i64]),
    "tqf_tc_selftest": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp]),
    "tqf_heston_asian": (ctypes.c_int, [ctypes.POINTER(HestonAsianArgs), c_vp]),
    "tqf_heston_asian_workspace_bytes": (ctypes.c_size_t, [c_i32, c_i64, c_i32]),
    "tqf_heston_asian_occupancy": (ctypes.c_int, [c_i32, c_i32]),
    "tqf_mlp_num_params": (ctypes.c_int, []),
    "tqf_mlp_train_step": (ctypes.c_int, [ctypes.POINTER(MlpTrainArgs), c_vp]),
    "tqf_mlp_adam": (ctypes.c_int, [ctypes.POINTER(MlpAdamArgs), c_vp]),
    "tqf_fma_peak_probe": (ctypes.c_int, [c_i32, c_i32, c_vp, ctypes.POINTER(ctypes.c_double), c_vp]),
}

_lock = threading.Lock()
_lib = None


def load() -> ctypes.CDLL:
    """Loads libtqf.so (built by ``csrc/build.py``); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libtqf.so not found at {LIB_PATH}: build the CUDA kernels first "
                "(python tf-quant-finance_gb300/csrc/build.py)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def last_error() -> str:
    msg = load().tqf_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str) -> None:
    if rc == TQF_OK:
        return
    msg = last_error()
    if rc == TQF_E_INVALID:
        raise InvalidArgumentError(f"{what}: {msg}")
    if rc == TQF_E_UNSUPPORTED:
        raise NotImplementedError(f"{what}: {msg}")
    raise RuntimeError(f"{what} failed (status {rc}): {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def launch_count() -> int:
    return int(load().tqf_launch_count())


_cuda_checked = False


def require_cuda() -> torch.device:
    global _cuda_checked
    if not _cuda_checked:
        if not torch.cuda.is_available():
            raise RuntimeError("tqf runs on a CUDA device (sm_103a); none is available")
        load()
        _cuda_checked = True
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.float32:
        return TQF_F32
    if dtype == torch.float64:
        return TQF_F64
    raise InvalidArgumentError(f"tqf kernels compute in float32 or float64, got {dtype}")


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


_status_cache: dict[int, torch.Tensor] = {}


def status_buffer(device: torch.device) -> torch.Tensor:
    """A per-device int32 that kernels set when a bounded wait runs out."""
    idx = device.index if device.index is not None else torch.cuda.current_device()
    buf = _status_cache.get(idx)
    if buf is None:
        buf = torch.zeros(1, dtype=torch.int32, device=device)
        _status_cache[idx] = buf
    return buf


def check_device_status(device: torch.device) -> None:
    """Raises if a kernel recorded a device-side error (synchronises): a
    timed-out bounded wait (TQF_E_TIMEOUT), or an every-step output layout
    declared by the caller that the step table contradicts (TQF_E_INVALID)."""
    buf = status_buffer(device)
    v = int(buf.item())
    if v != 0:
        buf.zero_()
        why = {TQF_E_TIMEOUT: "bounded wait timed out",
               TQF_E_INVALID: "the every-step output declaration does not match the step table"}.get(v, "error")
        raise RuntimeError(f"tqf kernel reported device status {v} ({why})")
