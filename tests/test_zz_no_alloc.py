"""GPU: fgb_aca_f64_static (the ACA kernel with its scratch and work queue in
the library's static device memory, no allocation) against fgb_aca_f64 with
caller-provided scratch, on the same blocks, for two calls in a row (the
second call must see a fresh work queue)."""
import ctypes as C

import numpy as np
import pytest
import torch

from fluxpy_gb300 import _lib, config, shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import ClusterTree

pytestmark = pytest.mark.gpu

RMAX, NSAMPLE, EXACT_MAX, NUM_CTAS, TOL = 32, 512, 4096, 8, 1e-5


def _case():
    V, F = terrain.fbm_terrain(n=24, seed=3, n_craters=2)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    tree = ClusterTree(sm.P, 3, leaf_size=64)
    nodes = [i for i in range(tree.num_nodes) if tree.level[i] == 2 and tree.size[i] > 0]
    pairs = [(i, j) for i in nodes for j in nodes if i != j][:96]
    r0 = np.array([tree.start[i] for i, _ in pairs], np.int32)
    m = np.array([tree.size[i] for i, _ in pairs], np.int32)
    c0 = np.array([tree.start[j] for _, j in pairs], np.int32)
    n = np.array([tree.size[j] for _, j in pairs], np.int32)
    dev = torch.device("cuda")
    blocks = {k: torch.as_tensor(v, device=dev) for k, v in
              dict(r0=r0, m=m, c0=c0, n=n).items()}
    perm = torch.as_tensor(tree.perm, device=dev)
    cap_k = np.minimum(RMAX, np.maximum(1, (m.astype(np.int64) * n) // (2 * (m.astype(np.int64) + n))))
    capacity = int((cap_k * (m.astype(np.int64) + n)).sum())
    return sm, perm, blocks, (int(m.max()), int(n.max())), capacity, (m, n)


def _outputs(nb, capacity):
    dev = torch.device("cuda")
    return dict(pool=torch.full((capacity,), float("nan"), device=dev),
                used=torch.zeros(1, dtype=torch.int64, device=dev),
                rank=torch.full((nb,), -9, dtype=torch.int32, device=dev),
                off=torch.full((nb,), -9, dtype=torch.int64, device=dev),
                flags=torch.zeros(1, dtype=torch.int32, device=dev))


def _common_args(sm, perm, blocks, mn_max):
    P, N, A = sm.device_geometry()
    nb = blocks["r0"].numel()
    return [sm.bvh.handle, _lib.ptr(P), _lib.ptr(N), _lib.ptr(A), _lib.ptr(perm), nb,
            _lib.ptr(blocks["r0"]), _lib.ptr(blocks["m"]), _lib.ptr(blocks["c0"]),
            _lib.ptr(blocks["n"]), mn_max[0], mn_max[1], float(config.DEFAULT_EPS),
            sm.semantics, TOL, RMAX, NSAMPLE, EXACT_MAX]


def test_static_scratch_aca_matches_caller_scratch():
    sm, perm, blocks, mn_max, capacity, (m, n) = _case()
    nb = blocks["r0"].numel()
    st = _lib.stream_handle()
    common = _common_args(sm, perm, blocks, mn_max)
    # the existing entry point with caller scratch
    per_cta = C.c_longlong()
    _lib.call("fgb_aca_scratch_floats", RMAX, mn_max[0], mn_max[1], C.byref(per_cta))
    scratch = torch.empty(NUM_CTAS * per_cta.value, dtype=torch.float32, device="cuda")
    dense = torch.empty(NUM_CTAS * EXACT_MAX, dtype=torch.float32, device="cuda")
    queue = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref = _outputs(nb, capacity)
    _lib.call("fgb_aca_f64", *common, _lib.ptr(dense), _lib.ptr(scratch), NUM_CTAS,
              _lib.ptr(ref["pool"]), capacity, _lib.ptr(ref["used"]), _lib.ptr(ref["rank"]),
              _lib.ptr(ref["off"]), _lib.ptr(queue), _lib.ptr(ref["flags"]), st)
    torch.cuda.synchronize()
    rank_ref = ref["rank"].cpu().numpy()
    off_ref = ref["off"].cpu().numpy()
    pool_ref = ref["pool"].cpu().numpy()
    assert (rank_ref != -9).all() and (rank_ref > 0).any()
    # the static-scratch entry point, twice in a row on the same stream
    for call in range(2):
        out = _outputs(nb, capacity)
        _lib.call("fgb_aca_f64_static", *common, NUM_CTAS, _lib.ptr(out["pool"]), capacity,
                  _lib.ptr(out["used"]), _lib.ptr(out["rank"]), _lib.ptr(out["off"]),
                  _lib.ptr(out["flags"]), st)
        torch.cuda.synchronize()
        rank = out["rank"].cpu().numpy()
        off = out["off"].cpu().numpy()
        pool = out["pool"].cpu().numpy()
        assert np.array_equal(rank, rank_ref), call
        assert int(out["flags"].item()) == int(ref["flags"].item())
        assert int(out["used"].item()) == int(ref["used"].item())
        # pool offsets depend on completion order; the factors do not
        for b in np.flatnonzero(rank_ref > 0):
            k = int(rank_ref[b])
            size = k * (int(m[b]) + int(n[b]))
            a = pool_ref[off_ref[b]:off_ref[b] + size]
            c = pool[off[b]:off[b] + size]
            assert np.array_equal(a, c), (call, b)


def test_static_scratch_aca_rejects_oversize():
    sm, perm, blocks, mn_max, capacity, _ = _case()
    nb = blocks["r0"].numel()
    out = _outputs(nb, capacity)
    common = _common_args(sm, perm, blocks, mn_max)
    common[-1] = 1 << 22                           # exact_max: 4 Mi floats per CTA
    with pytest.raises(ValueError, match="static scratch"):
        _lib.call("fgb_aca_f64_static", *common, 64, _lib.ptr(out["pool"]), capacity,
                  _lib.ptr(out["used"]), _lib.ptr(out["rank"]), _lib.ptr(out["off"]),
                  _lib.ptr(out["flags"]), _lib.stream_handle())
    # sizes whose product would wrap around a signed 64-bit count are
    # rejected too (each term is bounded before it is combined)
    for exact_max, ctas in ((1 << 62, 64), ((1 << 63) - 1, 1), (1 << 40, 1 << 30)):
        common[-1] = exact_max
        with pytest.raises(ValueError, match="static scratch"):
            _lib.call("fgb_aca_f64_static", *common, ctas, _lib.ptr(out["pool"]), capacity,
                      _lib.ptr(out["used"]), _lib.ptr(out["rank"]), _lib.ptr(out["off"]),
                      _lib.ptr(out["flags"]), _lib.stream_handle())
    # nothing ran: the outputs are untouched
    torch.cuda.synchronize()
    assert (out["rank"].cpu().numpy() == -9).all()
