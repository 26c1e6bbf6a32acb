"""Randomized QMC point sets on the GPU (tff/math/qmc/__init__.py).

Digital nets (Sobol generating matrices, Owen-type linear matrix scrambling,
digital shifts) and rank-1 lattice rules, with the reference's signatures and
index-0 convention.  Points are produced by the ``tqf_digital_net_sample`` and
``tqf_lattice_rule_sample`` kernels; the small generating-matrix tables are
built on the host.  The random scrambling matrices / shifts / vectors come from
this engine's Philox stream (a seed reproduces them; they are not
TensorFlow's stateless_uniform values).
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.errors import InvalidArgumentError
from tqf.math.qmc import utils
from tqf.math.qmc.utils import log2_f32

_JOE_KUO = None


def _joe_kuo(max_dims: int):
    """(polynomial 2^s + 2a + 1, initial direction numbers m_1..m_s) of the
    Joe-Kuo dimensions 2, 3, ... (the file shipped for the Sobol sampler)."""
    global _JOE_KUO
    if _JOE_KUO is None or len(_JOE_KUO[0]) < max_dims:
        polys, inits = [], []
        with open(_lib.JOE_KUO_PATH) as f:
            next(f)
            for line in f:
                tok = line.split()
                if not tok:
                    continue
                s, a = int(tok[1]), int(tok[2])
                polys.append((1 << s) + 2 * a + 1)
                inits.append([int(t) for t in tok[3:]])
                if len(polys) >= max(max_dims, 1):
                    break
        _JOE_KUO = (polys, inits)
    return _JOE_KUO


def _int_dtype(dtype):
    if dtype is None:
        return torch.int32
    if isinstance(dtype, torch.dtype):
        return dtype
    return {np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64}[np.dtype(dtype)]


def _real_dtype(dtype):
    if dtype is None:
        return torch.float32
    if isinstance(dtype, torch.dtype):
        return dtype
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[np.dtype(dtype)]


def _as_int(x) -> int:
    return int(x.item()) if isinstance(x, torch.Tensor) else int(x)


def sobol_generating_matrices(dim, num_results, num_digits, validate_args=False, dtype=None, name=None):
    """[dim, ceil(log2 num_results)] Sobol generating matrices, column c of
    axis d as an integer with num_digits bits (sobol.py:132-395): the identity
    for the first axis, then direction numbers m_k << (num_digits - 1 - k) and
    the primitive-polynomial recurrence
      M[k] = (M[k-s] >> s) ^ XOR_{b < s} bit_b(poly) M[k-s+b],  k >= s."""
    del name
    dim, num_results, num_digits = _as_int(dim), _as_int(num_results), _as_int(num_digits)
    if validate_args and (dim <= 0 or num_results <= 0 or num_digits <= 0):
        raise InvalidArgumentError("dim, num_results and num_digits must be positive")
    log_n = int(np.ceil(log2_f32(num_results)))
    if validate_args and log_n >= 32:
        raise InvalidArgumentError("log2(num_results) must be less than 32")
    out = np.zeros((dim, log_n), np.int64)
    for c in range(log_n):
        out[0, c] = (1 << (num_digits - 1 - c)) if num_digits - 1 - c >= 0 else 0
    polys, inits = _joe_kuo(dim - 1)
    for j in range(dim - 1):
        poly, ms = polys[j], inits[j]
        s = poly.bit_length() - 1
        row = out[j + 1]
        for c in range(min(s, log_n)):
            sh = num_digits - 1 - c
            row[c] = (ms[c] << sh) if sh >= 0 else 0
        for k in range(s, log_n):
            v = row[k - s] >> s
            for b in range(s):
                if (poly >> b) & 1:
                    v ^= row[k - s + b]
            row[k] = v
    return torch.as_tensor(out, dtype=_int_dtype(dtype)).to(_lib.require_cuda())


def scramble_generating_matrices(generating_matrices, scrambling_matrices, num_digits, validate_args=False,
                                 dtype=None, name=None):
    """Linear matrix scrambling (digital_net.py:422-527): column c becomes
    XOR over shifts t < num_digits with bit (num_digits-1-t) of M[c] set of
    (S[t] >> t)."""
    del name, validate_args
    gm = torch.as_tensor(generating_matrices)
    dtype = _int_dtype(dtype) if dtype is not None else gm.dtype
    g = gm.detach().cpu().numpy().astype(np.int64)
    s = torch.as_tensor(scrambling_matrices).detach().cpu().numpy().astype(np.int64)
    nd = _as_int(num_digits)
    out = np.zeros_like(g)
    for t in range(nd):
        col = (s[:, t:t + 1] >> t)
        out ^= np.where(((g >> (nd - 1 - t)) & 1) == 1, col, 0)
    return torch.as_tensor(out, dtype=dtype).to(_lib.require_cuda())


def _uniform_u32(count: int, seed, salt: int) -> np.ndarray:
    """count uint32 values of Philox4x32-10 with key = seed (this engine's stream)."""
    device = _lib.require_cuda()
    a = np.asarray(seed if seed is not None else torch.randint(0, 2 ** 31, (2,)).tolist()).reshape(-1)
    k0, k1 = int(a[0]) & 0xFFFFFFFF, int(a[1] if a.size > 1 else 0) & 0xFFFFFFFF
    blocks = (count + 3) // 4
    out = torch.empty(4 * blocks, dtype=torch.int32, device=device)
    _lib.call("tqf_philox4x32_10", 0, salt, 0x51A1, 0, k0, k1, blocks, out.data_ptr(), _lib.stream_ptr(device))
    return out.cpu().numpy().view(np.uint32)[:count]


def _random_ints(shape, num_digits, seed, dtype, salt):
    """Uniform integers in [2^(nd-1), 2^nd) (digital_net.py:155-202)."""
    nd = _as_int(num_digits)
    n = int(np.prod(shape))
    lo, span = 1 << (nd - 1), 1 << (nd - 1)
    u = _uniform_u32(2 * n, seed, salt).astype(np.uint64)
    r = ((u[0::2] << np.uint64(32)) | u[1::2]) % np.uint64(span)
    return torch.as_tensor((lo + r.astype(np.int64)).reshape(shape), dtype=_int_dtype(dtype)).to(_lib.require_cuda())


def random_scrambling_matrices(dim, num_digits, seed, validate_args=False, dtype=None, name=None):
    """[dim, num_digits] uniform integers in [2^(nd-1), 2^nd) (digital_net.py:98-152)."""
    del name, validate_args
    return _random_ints((_as_int(dim), _as_int(num_digits)), num_digits, seed, dtype, salt=1)


def random_digital_shift(dim, num_digits, seed, validate_args=False, dtype=None, name=None):
    """[dim] uniform integers in [2^(nd-1), 2^nd) (digital_net.py:45-95)."""
    del name, validate_args
    return _random_ints((_as_int(dim),), num_digits, seed, dtype, salt=2)


def random_scrambling_vectors(dim, seed, validate_args=False, dtype=None, name=None):
    """[dim] uniforms in [0, 1) (lattice_rule.py:40-96)."""
    del name
    dim = _as_int(dim)
    if validate_args and dim <= 0:
        raise InvalidArgumentError("dim must be positive")
    td = _real_dtype(dtype)
    u = _uniform_u32(2 * dim, seed, salt=3).astype(np.float64)
    v = u[0::2] * 2.0 ** -32 + u[1::2] * 2.0 ** -64  # [0, 1) in float64
    np_t = np.float32 if td == torch.float32 else np.float64
    v = np.minimum(v.astype(np_t), np.nextafter(np_t(1), np_t(0)))  # stays below 1 after rounding
    return torch.as_tensor(v, dtype=td).to(_lib.require_cuda())


def digital_net_sample(generating_matrices, num_results, num_digits, sequence_indices=None,
                       scrambling_matrices=None, digital_shift=None, apply_tent_transform=False,
                       validate_args=False, dtype=None, name=None):
    """[n, dim] points of the digital net (digital_net.py:205-419)."""
    del name
    device = _lib.require_cuda()
    gm = torch.as_tensor(generating_matrices).to(device)
    num_results, num_digits = _as_int(num_results), _as_int(num_digits)
    if validate_args:
        if gm.dim() != 2:
            raise InvalidArgumentError("generating_matrices must have rank 2")
        if num_results <= 0 or num_digits <= 0:
            raise InvalidArgumentError("num_results and num_digits must be positive")
    if scrambling_matrices is not None:
        gm = scramble_generating_matrices(gm, scrambling_matrices, num_digits, dtype=gm.dtype)
    int_bits = 64 if gm.dtype == torch.int64 else 32
    gm = gm.to(torch.int64 if int_bits == 64 else torch.int32).contiguous()
    dim = int(gm.shape[0])
    log_n = int(np.ceil(log2_f32(num_results)))
    idx = None
    count = num_results
    if sequence_indices is not None:
        idx = torch.as_tensor(sequence_indices).to(device=device, dtype=torch.int64).reshape(-1).contiguous()
        count = int(idx.numel())
        if validate_args and count and int(idx.max().item()) >= num_results:
            raise InvalidArgumentError("values in sequence_indices must be less than num_results")
    shift = None
    if digital_shift is not None:
        shift = torch.as_tensor(digital_shift).to(device=device, dtype=gm.dtype).reshape(-1).contiguous()
        if validate_args and shift.numel() != dim:
            raise InvalidArgumentError("digital_shift must have size tf.shape(generating_matrices)[0]")
    td = _real_dtype(dtype)
    out = torch.empty((count, dim), dtype=td, device=device)
    a = _lib.DigitalNetArgs()
    a.dim, a.log_num_results, a.num_digits = dim, min(log_n, int(gm.shape[1])), num_digits
    a.out_kind = _lib.SOBOL_F32 if td == torch.float32 else _lib.SOBOL_F64
    a.tent = 1 if apply_tent_transform else 0
    a.int_bits = int_bits
    a.count = count
    a.sequence_indices = idx.data_ptr() if idx is not None else None
    a.matrices = gm.data_ptr()
    a.digital_shift = shift.data_ptr() if shift is not None else None
    a.out = out.data_ptr()
    _lib.call("tqf_digital_net_sample", a, _lib.stream_ptr(device))
    return out


def sobol_sample(dim, num_results, sequence_indices=None, digital_shift=None, scrambling_matrices=None,
                 apply_tent_transform=False, validate_args=False, dtype=None, name=None):
    """[n, dim] Sobol points from index 0, num_digits = ceil(log2 n) (sobol.py:32-130)."""
    del name
    num_results = _as_int(num_results)
    nd = int(np.ceil(log2_f32(num_results)))
    gm = sobol_generating_matrices(dim, num_results, nd, validate_args=validate_args, dtype=torch.int32)
    if scrambling_matrices is not None:
        gm = scramble_generating_matrices(gm, scrambling_matrices, nd)
    return digital_net_sample(gm, num_results, nd, sequence_indices=sequence_indices, digital_shift=digital_shift,
                              apply_tent_transform=apply_tent_transform, validate_args=validate_args, dtype=dtype)


def lattice_rule_sample(generating_vectors, dim, num_results, sequence_indices=None, additive_shift=None,
                        apply_tent_transform=False, validate_args=False, dtype=None, name=None):
    """[n, dim] rank-1 lattice points frac(i * frac(g / n) + shift) (lattice_rule.py:99-229)."""
    del name
    device = _lib.require_cuda()
    gv = torch.as_tensor(generating_vectors).to(device)
    dim, num_results = _as_int(dim), _as_int(num_results)
    if validate_args:
        if gv.dim() != 1:
            raise InvalidArgumentError("generating_vectors must have rank 1")
        if dim > gv.numel():
            raise InvalidArgumentError("dim must not exceed the size of generating_vectors")
        if num_results <= 0:
            raise InvalidArgumentError("num_results must be positive")
    int_bits = 64 if gv.dtype == torch.int64 else 32
    gv = gv.to(torch.int64 if int_bits == 64 else torch.int32).contiguous()
    td = _real_dtype(dtype)
    idx = None
    count = num_results
    if sequence_indices is not None:
        idx = torch.as_tensor(sequence_indices).to(device=device, dtype=torch.int64).reshape(-1).contiguous()
        count = int(idx.numel())
    shift = None
    if additive_shift is not None:
        shift = torch.as_tensor(additive_shift).to(device=device, dtype=td).reshape(-1).contiguous()
    out = torch.empty((count, dim), dtype=td, device=device)
    a = _lib.LatticeArgs()
    a.dim = dim
    a.out_kind = _lib.SOBOL_F32 if td == torch.float32 else _lib.SOBOL_F64
    a.tent = 1 if apply_tent_transform else 0
    a.int_bits = int_bits
    a.num_results = num_results
    a.count = count
    a.sequence_indices = idx.data_ptr() if idx is not None else None
    a.generating_vectors = gv.data_ptr()
    a.additive_shift = shift.data_ptr() if shift is not None else None
    a.out = out.data_ptr()
    _lib.call("tqf_lattice_rule_sample", a, _lib.stream_ptr(device))
    return out


__all__ = ["digital_net_sample", "lattice_rule_sample", "random_digital_shift", "random_scrambling_matrices",
           "random_scrambling_vectors", "scramble_generating_matrices", "sobol_generating_matrices",
           "sobol_sample", "utils"]
