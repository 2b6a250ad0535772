"""Exact view factor between two planar triangles on the GPU: drop-in for
``flux.view_factor`` (src/flux/view_factor/view_factor.pyx, whose
``ff_narayanaswamy(V1, V2)`` calls view_factor_narayanaswamy.c:338).

``ff_narayanaswamy(V1, V2)`` returns the view factor of triangle V1 (3 x 3,
one vertex per row) towards V2 as a float, like the reference;
``ff_triangles(T1, T2)`` evaluates n pairs (n x 3 x 3 each) in one launch
(libfluxgb ``fgb_ff_triangles_f64``, one pair per thread, FP64).
``get_form_factor_matrix(..., exact_adjacent=True)`` uses the same kernel
as a near-field correction (``fgb_ff_adjacent_fix_f64``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def ff_triangles(T1, T2):
    """View factors of the triangles T1[q] towards T2[q] (arrays n x 3 x 3,
    or device tensors); FP64; a host array for host input."""
    dev = _lib.require_cuda()
    host = not isinstance(T1, torch.Tensor)
    a = torch.as_tensor(np.asarray(T1, np.float64) if host else T1, device=dev).to(torch.float64)
    b = torch.as_tensor(np.asarray(T2, np.float64) if host else T2, device=dev).to(torch.float64)
    if a.ndim == 2:
        a, b = a[None], b[None]
    if a.shape != b.shape or a.shape[1:] != (3, 3):
        raise ValueError("triangles should be arrays of shape (n, 3, 3)")
    a, b = a.contiguous(), b.contiguous()
    n = a.shape[0]
    out = torch.empty(n, dtype=torch.float64, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("fgb_ff_triangles_f64", _lib.ptr(a), _lib.ptr(b), n, _lib.ptr(out),
              _lib.ptr(flags), _lib.stream_handle())
    if int(flags.item()) & _lib.FLAG_NONFINITE_OUT:
        raise RuntimeError("Unknown error occured.")   # the reference asserts !isnan
    return out.cpu().numpy() if host else out


def ff_narayanaswamy(V1, V2):
    """View factor of triangle V1 towards triangle V2 (3 x 3 arrays)."""
    V1 = np.asarray(V1, np.float64)
    V2 = np.asarray(V2, np.float64)
    if V1.shape != (3, 3) or V2.shape != (3, 3):
        raise ValueError("V1 and V2 should be 3 x 3 arrays of triangle vertices")
    return float(ff_triangles(V1[None], V2[None])[0])
