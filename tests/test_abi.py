"""libtqf.so loads on the CPU host and exports every symbol include/tqf.h declares."""

import os
import re

import numpy as np

from oracle import sobol as osobol

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "tqf.h")).read()
    return sorted(set(re.findall(r"TQF_API\s+[\w\s\*]+?\b(tqf_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    assert "tqf_heston_euler" in names and "tqf_sobol_sample" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    import tqf._lib as L
    lib = L.load()
    for name in _declared():
        assert hasattr(lib, name), name
    # and the Python binding covers all of them
    assert set(_declared()) <= set(L.exported_symbols())


def test_abi_version_and_error_string():
    import tqf._lib as L
    lib = L.load()
    assert lib.tqf_abi_version() >= 100
    assert isinstance(L.last_error(), str)


def test_direction_numbers_match_oracle():
    import tqf._lib as L
    dim = 300
    out = np.zeros((dim, 32), dtype=np.uint32)
    L.call("tqf_sobol_direction_numbers", L.JOE_KUO_PATH.encode(), dim, out.ctypes.data_as(L.c_vp))
    m = osobol.compute_direction_numbers(dim)
    for j in range(31):
        expect = ((m[:, j].astype(np.uint64) << np.uint64(31 - j)) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        np.testing.assert_array_equal(out[:, j], expect)


def test_direction_numbers_reject_bad_requests():
    import pytest
    import tqf._lib as L
    out = np.zeros((4, 32), dtype=np.uint32)
    with pytest.raises(ValueError):
        L.call("tqf_sobol_direction_numbers", L.JOE_KUO_PATH.encode(), 0, out.ctypes.data_as(L.c_vp))
    with pytest.raises(RuntimeError):
        L.call("tqf_sobol_direction_numbers", b"/nonexistent/file", 4, out.ctypes.data_as(L.c_vp))


def test_num_digits_matches_oracle():
    import tqf._lib as L
    lib = L.load()
    for n, skip in [(5, 0), (2 ** 22, 0), (2 ** 26, 0), (3, 2 ** 31 - 5), (1, 0), (2 ** 20 - 1, 0)]:
        assert lib.tqf_sobol_num_digits(n, skip) == osobol.num_digits(n, skip)


def test_entry_points_reject_null_arguments_without_a_gpu():
    # Argument validation happens on the host before any CUDA call.
    import pytest
    import tqf._lib as L
    with pytest.raises(ValueError):
        L.call("tqf_sobol_sample", None, 2, 5, 0, 3, L.SOBOL_F32, None, None)
    args = L.HestonArgs()
    args.dtype = 7
    with pytest.raises(ValueError):
        L.call("tqf_heston_euler", args, None)
    eargs = L.EulerAffineArgs()
    eargs.dtype = L.TQF_F32
    eargs.dim = 40
    with pytest.raises(ValueError):
        L.call("tqf_euler_affine", eargs, None)


# Entry points whose work is host-only (file parsing, sizes, version, error text).
_HOST_ONLY = {"tqf_abi_version", "tqf_last_error", "tqf_launch_count", "tqf_sobol_direction_numbers",
              "tqf_sobol_num_digits", "tqf_mlp_num_params", "tqf_heston_asian_occupancy"}


def _compute_entry_points():
    import ctypes
    import tqf._lib as L
    for name, (res, args) in L._SIGNATURES.items():
        if name not in _HOST_ONLY and res is ctypes.c_int:
            yield name, args


def test_every_compute_entry_point_rejects_null_pointers_on_the_host():
    # Every pointer null, every size 1: each entry point must answer
    # TQF_E_INVALID with a message naming itself, before any CUDA call (this
    # host has no GPU, so a call that reached CUDA would answer TQF_E_CUDA).
    import ctypes
    import tqf._lib as L
    lib = L.load()
    names = []
    for name, args in _compute_entry_points():
        vals = [1 if t in (L.c_i32, L.c_i64, L.c_u32, ctypes.c_uint64) else 1.0 if t is ctypes.c_double else None
                for t in args]
        assert getattr(lib, name)(*vals) == L.TQF_E_INVALID, name
        assert L.last_error().startswith(name + ":"), (name, L.last_error())
        names.append(name)
    assert len(names) >= 30


def test_every_args_struct_entry_point_rejects_a_zeroed_struct():
    # A zero-initialised argument struct has no sizes and no buffers: each
    # entry point taking one must reject it on the host.
    import ctypes
    import tqf._lib as L
    lib = L.load()
    count = 0
    for name, args in _compute_entry_points():
        target = getattr(args[0], "_type_", None)
        if len(args) != 2 or not (isinstance(target, type) and issubclass(target, ctypes.Structure)):
            continue
        zero = args[0]._type_()
        assert getattr(lib, name)(ctypes.byref(zero), None) == L.TQF_E_INVALID, name
        assert L.last_error().startswith(name + ":"), (name, L.last_error())
        count += 1
    assert count >= 20
