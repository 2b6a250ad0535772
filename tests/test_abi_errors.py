"""CPU: the C ABI rejects bad arguments before it touches the device.

Each call below fails (or, for empty inputs, succeeds) in the entry point's
host-side checks, so it runs without a GPU; the status is FGB_BAD_ARG and
``fgb_last_error()`` names the problem."""
import ctypes as C

import pytest

from fluxpy_gb300 import _lib
from fluxpy_gb300.compressed_form_factors import fgb_op_desc


@pytest.fixture(scope="module")
def lib():
    return _lib.lib()


def _rejects(lib, st, *words):
    assert st == _lib.FGB_BAD_ARG
    msg = lib.fgb_last_error().decode()
    for w in words:
        assert w in msg, msg


def test_column_reductions_check_sizes(lib):
    for fn in ("fgb_colmax_absdiff", "fgb_residual"):
        f = getattr(lib, fn)
        extra = (None, None) if fn == "fgb_residual" else ()
        # Y, B, [E, R,] N, K, colmax, stream
        _rejects(lib, f(None, None, *extra, -1, 4, None, None), "bad sizes")
        _rejects(lib, f(None, None, *extra, 10, 0, None, None), "bad sizes")
        # one word per column in shared memory: at most 8,192 columns
        _rejects(lib, f(None, None, *extra, 10, 8193, None, None), "8192")
        # nothing to reduce: no launch
        assert f(None, None, *extra, 0, 16, None, None) == _lib.FGB_OK
    _rejects(lib, lib.fgb_axpy_cols(None, None, None, 10, 0, None), "bad sizes")
    _rejects(lib, lib.fgb_scale_rows_bf16(None, None, 1.0, None, -5, 8, None), "bad sizes")
    assert lib.fgb_scale_rows_bf16(None, None, 1.0, None, 0, 8, None) == _lib.FGB_OK


def test_tensor_core_products_check_operands(lib):
    d = fgb_op_desc()
    d.num_zrows = 4
    flags = C.c_uint(0)
    pd, pf = C.byref(d), C.byref(flags)
    a16, b16 = 0x10000, 0x20000          # aligned addresses (never dereferenced)
    # phase A: desc, vt_hi, vt_lo, X_hi, X_lo, Z, K, zero_z, flags, stream
    _rejects(lib, lib.fgb_tc_phase_a(None, a16, None, b16, None, None, 16, 1, pf, None),
             "null operator")
    for K in (0, 4, 12):
        _rejects(lib, lib.fgb_tc_phase_a(pd, a16, None, b16, None, None, K, 1, pf, None),
                 "multiple of 8")
    _rejects(lib, lib.fgb_tc_phase_a(pd, a16, a16, b16, None, None, 16, 1, pf, None), "pairs")
    _rejects(lib, lib.fgb_tc_phase_a(pd, a16 + 8, None, b16, None, None, 16, 1, pf, None),
             "16-byte aligned")
    # phase B: desc, w_hi, w_lo, X_hi, X_lo, Z_hi, Z_lo, Y, K, add, alpha, flags, stream
    _rejects(lib, lib.fgb_tc_phase_b(pd, a16, None, b16, None, b16, None, None, 20, None, 1.0,
                                     pf, None), "multiple of 8")
    # split operands come in pairs; Z's pair is needed only when there are Z rows
    _rejects(lib, lib.fgb_tc_phase_b(pd, a16, a16, b16, b16, b16, None, None, 16, None, 1.0,
                                     pf, None), "pairs")
    _rejects(lib, lib.fgb_tc_phase_b(pd, a16, None, b16, None, b16 + 4, None, None, 16, None,
                                     1.0, pf, None), "16-byte aligned")
    _rejects(lib, lib.fgb_tc_phase_b(pd, a16, None, b16, None, b16, None, None, 16, None, 1.0,
                                     None, None), "flags")


def test_conduction_checks_grid(lib):
    P = None
    for fn in ("fgb_conduction_q_f64", "fgb_conduction_q_f32"):
        f = getattr(lib, fn)
        _rejects(lib, f(-1, 10, P, 1.0, P, P, P, P, P, P, P, P, P, None, None), "num_faces")
        for nz in (1, 256):
            _rejects(lib, f(4, nz, P, 1.0, P, P, P, P, P, P, P, P, P, None, None),
                     f"got {nz}")
        # no facets: nothing to do
        assert f(0, 10, P, 1.0, P, P, P, P, P, P, P, P, P, None, None) == _lib.FGB_OK


def test_scene_and_compression_entry_points_check_arguments(lib):
    flags = C.c_uint(0)
    pf = C.byref(flags)
    _rejects(lib, lib.fgb_facet_geometry_f64(None, -1, None, 4, None, None, None, pf, None),
             "negative sizes")
    assert lib.fgb_facet_geometry_f64(None, 0, None, 0, None, None, None, pf, None) == _lib.FGB_OK
    h = C.c_void_p()
    _rejects(lib, lib.fgb_bvh_build_f64(None, 3, None, -1, 0, C.byref(h), pf, None),
             "bad arguments")
    _rejects(lib, lib.fgb_bvh_build_f64(None, 3, None, 1, 0, None, pf, None), "bad arguments")
    # an empty scene: a handle with no primitives, no device memory
    assert lib.fgb_bvh_build_f64(None, 0, None, 0, 0, C.byref(h), pf, None) == _lib.FGB_OK
    n, nbytes = C.c_longlong(-1), C.c_longlong(-1)
    assert lib.fgb_bvh_info(h, C.byref(n), C.byref(nbytes)) == _lib.FGB_OK
    assert n.value == 0 and nbytes.value == 0
    assert lib.fgb_bvh_free(h) == _lib.FGB_OK
    _rejects(lib, lib.fgb_bvh_info(None, C.byref(n), None), "null bvh")
    _rejects(lib, lib.fgb_visibility_f64(None, None, 4, None, 2, None, 2, 1, 0, None, None, pf,
                                         None), "null BVH")
    _rejects(lib, lib.fgb_ff_triangles_f64(None, None, -1, None, pf, None), "n must be >= 0")
    _rejects(lib, lib.fgb_ff_triangles_f64(None, None, 3, None, pf, None), "null pointer")
    assert lib.fgb_ff_triangles_f64(None, None, 0, None, pf, None) == _lib.FGB_OK
    # ACA scratch: ranks up to 128, block sides below 2^31, an output word
    per = C.c_longlong(0)
    for r, m, n_ in ((0, 64, 64), (129, 64, 64), (8, 0, 64), (8, 64, 1 << 31)):
        _rejects(lib, lib.fgb_aca_scratch_floats(r, m, n_, C.byref(per)), "bad ACA sizes")
    _rejects(lib, lib.fgb_aca_scratch_floats(8, 64, 32, None), "null output")
    assert lib.fgb_aca_scratch_floats(8, 64, 32, C.byref(per)) == _lib.FGB_OK
    assert per.value == 8 * (64 + 32) + 2 * (64 + 32)
    _rejects(lib, lib.fgb_split_bf16(None, None, None, -1, None), "bad arguments")
    _rejects(lib, lib.fgb_retile_panel_bf16_n(0x10000, 4, None, None, 64, 0x20000, None),
             "128 or 256")
