"""tff.math.qmc restated in NumPy (test oracle).

Test infrastructure only: the product path never imports this module.

Follows tf_quant_finance/math/qmc/:
  sobol.py:32-130        sobol_sample (num_digits = ceil(log2 n) in float32)
  sobol.py:132-218       sobol_generating_matrices (identity row, then the
                         Joe-Kuo dimensions)
  sobol.py:246-395       _sobol_generating_matrices (direction numbers
                         shifted to num_digits, then the while-loop
                         recurrence over columns)
  digital_net.py:205-419 digital_net_sample (XOR of the matrix columns of the
                         set index bits, digital shift, / 2^num_digits)
  digital_net.py:422-527 scramble_generating_matrices
  lattice_rule.py:99-229 lattice_rule_sample
  utils.py:94-158        tent_transform, filter_tensor
Indices start at 0 (unlike sobol_impl.py's skip + 1).
"""

from __future__ import annotations

import numpy as np

from oracle import sobol as osobol


def log2_f32(x):
    x = np.float32(x)
    return np.float32(np.log(x) / np.log(np.float32(2)))


def _filter(value, mask, bit):
    """value where bit `bit` of mask is set, else 0 (utils.filter_tensor)."""
    bit = np.asarray(bit)
    is_set = np.where(bit >= 0, (np.right_shift(mask, np.maximum(bit, 0)) & 1) == 1, False)
    return np.where(is_set, value, 0)


def sobol_generating_matrices(dim, num_results, num_digits, dtype=np.int32):
    log_n = int(np.ceil(log2_f32(num_results)))
    cols = np.arange(log_n)
    identity = np.left_shift(np.ones(log_n, np.int64), num_digits - 1 - cols)
    if dim == 1:
        return identity[None].astype(dtype)
    polys, init = osobol.load_data(max_dims=dim - 1)
    directions = np.zeros((max(log_n, init.shape[0]), dim - 1), np.int64)
    directions[: init.shape[0]] = init[:, : dim - 1]
    directions = directions[:log_n].T  # [dim-1, log_n]
    poly = polys[: dim - 1].reshape(-1, 1)
    degree = np.floor(np.log(poly.astype(np.float32)) / np.log(np.float32(2))).astype(np.int64)
    m = np.left_shift(directions, (num_digits - 1 - cols)[None, :])
    idx = cols[None, :]
    for column in range(log_n - 1):
        cv = m[:, column: column + 1]
        upd = (np.maximum(degree, column + 1) <= idx) & (idx <= column + degree)
        base = np.where(idx == column + degree, np.right_shift(cv, degree), m)
        new = np.bitwise_xor(base, _filter(cv, poly, column + degree - idx))
        m = np.where(upd, new, m)
    return np.concatenate([identity[None], m], 0).astype(dtype)


def scramble_generating_matrices(gen, scr, num_digits):
    gen = np.asarray(gen, np.int64)
    scr = np.asarray(scr, np.int64)
    out = np.zeros_like(gen)
    for shift in range(num_digits):
        col = np.right_shift(scr[:, shift: shift + 1], shift)
        out = np.bitwise_xor(out, _filter(col, gen, num_digits - 1 - shift))
    return out


def digital_net_sample(gen, num_results, num_digits, sequence_indices=None, digital_shift=None,
                       apply_tent_transform=False, dtype=np.float32):
    gen = np.asarray(gen, np.int64)
    dim = gen.shape[0]
    log_n = int(np.ceil(log2_f32(num_results)))
    idx = np.arange(num_results) if sequence_indices is None else np.asarray(sequence_indices, np.int64)
    pts = np.broadcast_to(np.zeros(dim, np.int64) if digital_shift is None else np.asarray(digital_shift, np.int64),
                          (len(idx), dim)).copy()
    for b in range(log_n):
        pts = np.bitwise_xor(pts, _filter(gen[None, :, b], idx[:, None], b))
    dt_ = np.dtype(dtype).type
    out = (pts.astype(dtype) / dt_(2 ** num_digits)).astype(dtype)
    return tent(out) if apply_tent_transform else out


def sobol_sample(dim, num_results, sequence_indices=None, digital_shift=None, scrambling_matrices=None,
                 apply_tent_transform=False, dtype=np.float32):
    nd = int(np.ceil(log2_f32(num_results)))
    gen = sobol_generating_matrices(dim, num_results, nd)
    if scrambling_matrices is not None:
        gen = scramble_generating_matrices(gen, scrambling_matrices, nd)
    return digital_net_sample(gen, num_results, nd, sequence_indices, digital_shift, apply_tent_transform, dtype)


def tent(v):
    return np.where(v < 0.5, 2 * v, 2 * (1 - v)).astype(v.dtype)


def lattice_rule_sample(gen_vectors, dim, num_results, sequence_indices=None, additive_shift=None,
                        apply_tent_transform=False, dtype=np.float32):
    dt_ = np.dtype(dtype).type
    idx = np.arange(num_results) if sequence_indices is None else np.asarray(sequence_indices)
    scaled = (np.asarray(gen_vectors[:dim]).astype(dtype) / dt_(num_results)).astype(dtype)
    pts = (idx.astype(dtype)[:, None] * np.mod(scaled, dt_(1))[None, :]).astype(dtype)
    if additive_shift is not None:
        pts = (pts + np.asarray(additive_shift, dtype)[:dim]).astype(dtype)
    pts = np.mod(pts, dt_(1)).astype(dtype)
    return tent(pts) if apply_tent_transform else pts
