"""ctypes binding of libfluxgb.so (the C ABI declared in include/fluxgb.h).

The product path has no CPU fallback: importing a module that needs the
library raises if ``libfluxgb.so`` has not been built, and every call raises
if no CUDA device is present.  Status codes map to the reference's exception
types (RuntimeError / ValueError), with the C-side message attached.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import torch

LIB_PATH = Path(__file__).resolve().parent / "libfluxgb.so"

FGB_OK = 0
FGB_BAD_ARG = 1
FGB_NONFINITE = 2
FGB_NEGATIVE = 3
FGB_ZERO_PIVOT = 4
FGB_NO_CONVERGENCE = 5
FGB_DEVICE_TIMEOUT = 6
FGB_CUDA_ERR = 7
FGB_NO_MEMORY = 8
FGB_TOO_LARGE = 9

FLAG_NONFINITE_IN = 1 << 0
FLAG_NEGATIVE_IN = 1 << 1
FLAG_NONFINITE_OUT = 1 << 2
FLAG_NEGATIVE_OUT = 1 << 3
FLAG_ZERO_PIVOT = 1 << 4
FLAG_PREDCORR_MAX = 1 << 5
FLAG_STACK_OVERFLOW = 1 << 6
FLAG_INDEX_RANGE = 1 << 7
FLAG_RANK_CAP = 1 << 8
FLAG_DEVICE_TIMEOUT = 1 << 9
FLAG_NO_CONVERGE = 1 << 10

P = C.c_void_p
I32 = C.c_int
I64 = C.c_longlong
F64 = C.c_double
F32 = C.c_float
U32P = C.c_void_p

# name -> argument types (all return int status unless listed in _RESTYPES)
SIGNATURES: dict[str, list] = {
    "fgb_last_error": [],
    "fgb_version": [],
    "fgb_launch_count": [],
    # conduction (a14)
    "fgb_conduction_q_f64": [I32, I32, P, F64, P, P, P, P, P, P, P, P, P, U32P, P],
    "fgb_conduction_q_f32": [I32, I32, P, F32, P, P, P, P, P, P, P, P, P, U32P, P],
    "fgb_conduction_t_f64": [I32, I32, P, F64, P, P, P, P, P, P, P, P, U32P, P],
    "fgb_conduction_q_ti_f64": [I32, I32, P, F64, P, P, P, P, P, I64, P, P, P, U32P, P],
    "fgb_conduction_q_adjoint_f64": [I32, I32, P, F64, P, P, P, P, I64, P, P, P, P, P, P, P,
                                     P, P, U32P, P],
    # facet geometry (a1)
    "fgb_facet_geometry_f64": [P, I64, P, I64, P, P, P, U32P, P],
    "fgb_facet_geometry_f32": [P, I64, P, I64, P, P, P, U32P, P],
    # LBVH (a2)
    "fgb_bvh_build_f64": [P, I64, P, I64, I32, P, U32P, P],
    "fgb_bvh_build_f32": [P, I64, P, I64, I32, P, U32P, P],
    "fgb_bvh_free": [P],
    "fgb_bvh_info": [P, P, P],
    # ray queries (a3, a4)
    "fgb_visibility_f64": [P, P, I64, P, I64, P, I64, I32, I32, P, P, U32P, P],
    "fgb_visibility_f32": [P, P, I64, P, I64, P, I64, I32, I32, P, P, U32P, P],
    "fgb_occluded_f64": [P, P, P, I64, P, I64, P, I64, I32, I32, P, U32P, P],
    "fgb_occluded_f32": [P, P, P, I64, P, I64, P, I64, I32, I32, P, U32P, P],
    "fgb_direct_irradiance_f64": [P, P, P, I64, P, I64, P, I32, P, U32P, P],
    "fgb_direct_irradiance_f64_to_f32": [P, P, P, I64, P, I64, P, I32, P, U32P, P],
    "fgb_direct_irradiance_f32": [P, P, P, I64, P, I64, P, I32, P, U32P, P],
    "fgb_intersect1_f64": [P, P, P, I64, P, P, U32P, P],
    # form-factor pair kernel (a5)
    "fgb_ff_count_f64": [P, P, P, P, P, P, P, P, P, P, P, P, I64, I64, F64, I32, P, P, P, U32P, P],
    "fgb_ff_count_f32": [P, P, P, P, P, P, P, P, P, P, P, P, I64, I64, F32, I32, P, P, P, U32P, P],
    "fgb_ff_fill_f64": [P, P, P, P, P, P, P, P, P, P, P, I64, I64, P, P, P, P, P],
    "fgb_ff_fill_f32": [P, P, P, P, P, P, P, P, P, P, P, I64, I64, P, P, P, P, P],
    "fgb_ff_fill_f64_to_f32": [P, P, P, P, P, P, P, P, P, P, P, I64, I64, P, P, P, P, P],
    "fgb_nf_pair_masks": [P, P, P, I64, I64, P, P, P, P, P, P, P, P, P],
    "fgb_nf_enumerate": [P, P, P, I64, P, P, P, P, P, P],
    "fgb_nf_fill_f32_f32": [P, P, I64, P, P, P, P, P, P, P, P, P, P, P, I64, P, P],
    "fgb_nf_fill_f32_bf16": [P, P, I64, P, P, P, P, P, P, P, P, P, P, P, I64, P, P],
    "fgb_nf_fill_f64_f64": [P, P, I64, P, P, P, P, P, P, P, P, P, P, P, I64, P, P],
    "fgb_nf_fill_f64_f32": [P, P, I64, P, P, P, P, P, P, P, P, P, P, P, I64, P, P],
    "fgb_nf_fill_f64_bf16": [P, P, I64, P, P, P, P, P, P, P, P, P, P, P, I64, P, P],
    # compression (a6-a8)
    "fgb_aca_scratch_floats": [I32, I64, I64, P],
    "fgb_aca_f64": [P, P, P, P, P, I64, P, P, P, P, I64, I64, F64, I32, F32, I32, I32, I64, P,
                    P, I32, P, I64, P, P, P, P, U32P, P],
    "fgb_aca_f64_static": [P, P, P, P, P, I64, P, P, P, P, I64, I64, F64, I32, F32, I32, I32,
                           I64, I32, P, I64, P, P, P, U32P, P],
    "fgb_recompress_f32": [P, P, P, P, P, I64, F32, P, I64, P, P, P, P, U32P, P],
    # exact triangle-triangle view factor (view_factor_narayanaswamy.c)
    "fgb_ff_triangles_f64": [P, P, I64, P, U32P, P],
    "fgb_ff_adjacent_fix_f64": [P, P, P, P, I64, P, P, P, P, U32P, P],
    # block matvec (a9)
    "fgb_build_panel_f32_f32": [P, I64, P, P, P, P, P, I64, P, P],
    "fgb_build_panel_f32_bf16": [P, I64, P, P, P, P, P, I64, P, P],
    "fgb_build_panel_f64_f64": [P, I64, P, P, P, P, P, I64, P, P],
    "fgb_build_panel_f64_f32": [P, I64, P, P, P, P, P, I64, P, P],
    "fgb_build_panel_f64_bf16": [P, I64, P, P, P, P, P, I64, P, P],
    "fgb_build_vpanel_f32_f32": [P, I64, P, P, P, P, P],
    "fgb_build_vpanel_f32_bf16": [P, I64, P, P, P, P, P],
    "fgb_build_vpanel_f64_f64": [P, I64, P, P, P, P, P],
    "fgb_build_vpanel_f64_f32": [P, I64, P, P, P, P, P],
    "fgb_build_vpanel_f64_bf16": [P, I64, P, P, P, P, P],
    "fgb_matvec_f32": [P, P, P, P, P, P, P, F32, I32, P],
    "fgb_matvec_f64": [P, P, P, P, P, P, P, F64, I32, P],
    "fgb_matvec_f32_f64": [P, P, P, P, P, P, P, F64, I32, P],
    "fgb_rmatvec_f64": [P, P, P, P, P, U32P, P],
    "fgb_rmatvec_f32_f64": [P, P, P, P, P, U32P, P],
    "fgb_matmat_f32_f64": [P, P, P, P, P, P, I32, P, F64, I32, P],
    "fgb_matmat_f32": [P, P, P, P, P, P, I32, P, F32, I32, I32, P],
    "fgb_matmat_bf16": [P, P, P, P, P, P, P, I32, P, F32, I32, I32, P],
    "fgb_tc_phase_a": [P, P, P, P, P, P, I32, I32, P, P],
    "fgb_tc_phase_a_bf16": [P, P, P, P, P, P, P, I32, P, P],
    "fgb_tc_phase_b": [P, P, P, P, P, P, P, P, I32, P, F32, P, P],
    "fgb_tc_phase_b_tma": [P, P, P, P, P, P, I32, P, F32, P, P],
    "fgb_split_bf16": [P, P, P, I64, P],
    "fgb_retile_panel_bf16": [P, I64, P, P, P, P],
    "fgb_retile_panel_bf16_n": [P, I64, P, P, I32, P, P],
    "fgb_retile_panel_split_bf16": [P, I64, P, P, P, P, P],
    "fgb_vpanel_transpose_bf16": [P, P, P, P, P, I64, P, P, P],
    # solve (a10-a12)
    "fgb_scale_rows_f32": [P, P, F32, P, I64, I32, P],
    "fgb_scale_rows_bf16": [P, P, F32, P, I64, I32, P],
    "fgb_colmax_absdiff": [P, P, I64, I32, P, P],
    "fgb_residual": [P, P, P, P, I64, I32, P, P],
    "fgb_axpy_cols": [P, P, P, I64, I32, P],
    "fgb_gather_rows_f32": [P, P, P, I64, I32, P],
    "fgb_gather_rows_f64": [P, P, P, I64, I32, P],
    "fgb_csr_spmm_f64": [P, P, P, I64, P, I32, P, P, F64, P],
    "fgb_csr_spmm_f32": [P, P, P, I64, P, I32, P, P, F32, P],
}
_RESTYPES = {"fgb_last_error": C.c_char_p, "fgb_version": C.c_char_p,
             "fgb_launch_count": C.c_longlong}

_lock = threading.Lock()
_lib = None


class FluxGBError(RuntimeError):
    """Failure reported by libfluxgb with a status code."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def lib():
    """Load libfluxgb.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        handle = C.CDLL(str(LIB_PATH))
        for name, argtypes in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, C.c_int)
        _lib = handle
    return _lib


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("fluxpy_gb300 needs a CUDA device (GB300); no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def last_error() -> str:
    return lib().fgb_last_error().decode()


def check(status: int, what: str = "") -> None:
    if status == FGB_OK:
        return
    msg = last_error()
    if what:
        msg = f"{what}: {msg}"
    if status == FGB_BAD_ARG:
        raise ValueError(msg)
    raise FluxGBError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def launch_count() -> int:
    """Kernels launched by libfluxgb in this process so far."""
    return int(lib().fgb_launch_count())


def loaded_library_path() -> str:
    lib()
    return str(LIB_PATH)
