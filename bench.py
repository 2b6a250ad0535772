#!/usr/bin/env python
"""Benchmark: sun-direction radiosity solves per second at 522,242 facets.

Workload (one "step"): the right-placement radiosity solve
B = E + F (rho B) for 1,024 sun directions at once on a 512 x 512 fBm terrain
with 30 power-law craters (522,242 facets), compressed form-factor operator
(octree, ACA tolerance 1e-5, 64-facet leaves), albedo 0.12, every column
driven to max|E - (B - F rho B)| <= 1e-5 max|E| by BF16 tensor-core Jacobi
sweeps inside FP32 iterative refinement.  E (2.1 GB) and the operator are
far larger than the 129 MB L2, so no flush is needed between steps.

Printed (one JSON line, rank 0): value = whole-job solves/s; e2e = the same
through the public API solve_radiosity(..., method='batched-bf16') with a
pinned host E and a host result; roofline of the dominant kernel; the plain
FP32 GPU path (batched FP32 Jacobi, and single right-hand side); the
residual in FP64 arithmetic and the compression error against exactly
assembled rows; the CPU baseline (the oracle's restatement of the
reference's Jacobi solve with a scipy CSR operator on a bounded sample).

--impl reference prints the CPU reference arm instead (rank 0 only).
Multi-GPU (torchrun): every rank solves its own 1,024 directions on its own
replica of the operator (the solve does not shard); value sums the ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "sun-direction solves/s @520k facets: BF16+refine vs plain FP32, err≤1e-5"
RHO = 0.12
F0 = 1365.0
RTOL = 1e-5
# Stored entries (low-rank factors + exact leaves) of the compressed
# operator of the 522,242-facet terrain (octree, tolerance 1e-5, 64-facet
# leaves) as the GPU arm builds it; the CPU reference arm scales its sample
# rate by this count.  The GPU arm's line reports the count it builds.
OPERATOR_ENTRIES_522K = 11404279888


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--grid", type=int, default=512, help="terrain grid (512 -> 522,242 facets)")
    p.add_argument("--rhs", type=int, default=1024)
    p.add_argument("--tol", type=float, default=1e-5)
    p.add_argument("--no-extras", action="store_true", help="skip FP32/e2e/error/CPU legs")
    p.add_argument("--plain-tiles", default="auto", choices=["auto", "64", "128", "256"],
                   help="phase-B tile rows of the plain BF16 product (auto: autotuned)")
    p.add_argument("--split-plan", default="auto",
                   choices=["auto", "a64-b64", "a128-b64", "a64-b128", "a128-b128"],
                   help="phase-A slice / phase-B tile rows of the split product (auto: autotuned)")
    p.add_argument("--facets", type=int, default=522242,
                   help="facets of the conduction workload")
    p.add_argument("--conduction-spinup", type=int, default=300,
                   help="spin-up steps of the conduction workload's diurnal regime")
    p.add_argument("--workload", default="terrain",
                   choices=["terrain", "craters64", "adjoint", "conduction"],
                   help="terrain: the headline solve (default); craters64: 64 uneven crater "
                        "meshes, coupled time-dependent model; adjoint: misfit gradient of the "
                        "coupled model on a 200k-facet terrain; conduction: the 1-D "
                        "conduction step alone (FP32 and FP64, 41 nodes)")
    p.add_argument("--adjoint-steps", type=int, default=500,
                   help="time steps of the adjoint workload")
    p.add_argument("--adjoint-fd-steps", type=int, default=50,
                   help="time steps of the model checked by central differences")
    p.add_argument("--adjoint-fd-facets", type=int, default=32,
                   help="random facets per field checked by central differences")
    p.add_argument("--adjoint-grid", type=int, default=317,
                   help="terrain grid of the adjoint workload (317 -> 199,712 facets)")
    return p.parse_args()


# ------------------------------------------------------------- clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------- CPU baseline --
def _cpu_sample():
    """The CPU baseline's sample: a 64 x 64 fBm terrain (7,938 facets), its
    exact sparse form factors from the oracle's CPU ray caster, and the
    insolation of 64 sun directions."""
    from oracle import vis
    from fluxpy_gb300 import terrain
    V, F = terrain.fbm_terrain(n=64, seed=1, n_craters=4)
    P, N, A = vis.geometry(V, F)
    scene = vis.Scene(V, F)
    FFc = scene.ff_csr(P, N, A)
    dirs = terrain.random_sun_directions(64, seed=2)
    occ = scene.occluded(P, N, np.arange(F.shape[0]), dirs)
    E = np.where(~occ, F0 * np.maximum(0, N @ dirs.T), 0.0)
    return FFc, E


_SAMPLE_FILE = None


def _cpu_sample_file():
    """The sample written once per process to a temporary .npz (CSR arrays
    and E), so that the baseline's worker processes only load it."""
    global _SAMPLE_FILE
    if _SAMPLE_FILE is None:
        import tempfile
        FFc, E = _cpu_sample()
        fd, path = tempfile.mkstemp(suffix=".npz", prefix="fluxgb_cpu_sample_")
        os.close(fd)
        np.savez(path, data=FFc.data, indices=FFc.indices, indptr=FFc.indptr,
                 shape=np.array(FFc.shape), E=E)
        import atexit
        atexit.register(lambda: os.path.exists(path) and os.remove(path))
        _SAMPLE_FILE = path
    return _SAMPLE_FILE


def _cpu_solver_worker(job):
    """One host process of the CPU baseline: Jacobi solves of its share of
    the directions for ``seconds``, each to the GPU arm's stopping test
    (update <= RTOL max|E| of its column); returns (solves, seconds taken,
    nnz, N, Jacobi iterations summed)."""
    k, workers, seconds, path = job
    import scipy.sparse
    from oracle import solve as osolve
    z = np.load(path)
    FFc = scipy.sparse.csr_matrix((z["data"], z["indices"], z["indptr"]),
                                  shape=tuple(z["shape"]))
    E = z["E"]
    cols = list(range(k, E.shape[1], workers)) or [0]
    done = iters = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        e = E[:, cols[done % len(cols)]]
        _, it = osolve.solve_radiosity(FFc, e, RHO, tol=RTOL * float(np.abs(e).max()))
        iters += it
        done += 1
    return done, time.perf_counter() - t0, int(FFc.nnz), int(FFc.shape[0]), iters


def cpu_baseline(full_operator_entries=None, seconds=12.0, workers=None, entries_source=""):
    """The oracle's restatement of the reference's Jacobi solve
    (src/flux/solve.py:36-45) with the exact sparse form-factor matrix of the
    7,938-facet sample (_cpu_sample), one direction per solve as the
    reference does, each to the GPU arm's stopping test (relative update
    RTOL), on every host core: one process per core (spawned, so it is safe
    after CUDA initialisation), each solving its own directions.
    solves/s = the sum of the processes' rates, scaled to the full workload
    by the ratio of operator entries (matvec cost is proportional to them;
    the sample and the full workload need about the same Jacobi iterations
    at this albedo)."""
    import multiprocessing as mp
    workers = workers or (os.cpu_count() or 1)
    path = _cpu_sample_file()
    jobs = [(k, workers, seconds, path) for k in range(workers)]
    if workers > 1:
        # one single-threaded process per core (numpy / scipy loops here are
        # single-threaded; BLAS is not used by the CSR products)
        env = {"OMP_NUM_THREADS": "1", "OPENBLAS_NUM_THREADS": "1"}
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            with mp.get_context("spawn").Pool(workers) as pool:
                res = pool.map(_cpu_solver_worker, jobs)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    else:
        res = [_cpu_solver_worker(jobs[0])]
    rate = sum(r[0] / r[1] for r in res)
    done = sum(r[0] for r in res)
    iters = sum(r[4] for r in res) / max(done, 1)
    entries, nf = res[0][2], res[0][3]
    scale = entries / full_operator_entries if full_operator_entries else 1.0
    return {"value": rate * scale, "unit": "solves/s", "cores": workers, "kind": "port",
            "sample": (f"oracle Jacobi (numpy/scipy CSR, reference solve.py:36-45) on a 64x64 "
                       f"terrain ({nf} facets, {entries} nonzeros), one direction per solve to "
                       f"update <= {RTOL:g} max|E| ({iters:.1f} Jacobi iterations on average), "
                       f"{workers} processes x {seconds:.0f} s, {done} solves = {rate:.2f} "
                       f"solves/s, scaled by operator entries {entries}/"
                       f"{full_operator_entries} ({entries_source}) to the 522k-facet operator "
                       f"(extrapolation)"),
            "measured_solves_per_s_at_sample": rate, "sample_jacobi_iterations": iters,
            "scale": scale}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # stored entries of the 522k-facet compressed operator (a GPU build of
    # this workload, which this CPU-only process does not repeat; the GPU
    # arm's line reports its own in-process count beside its baseline)
    entries = OPERATOR_ENTRIES_522K
    src = "stored entries of the GPU build of this workload"
    t0 = time.perf_counter()
    reps = []
    for _ in range(max(1, args.warmup)):
        cpu_baseline(entries, seconds=2.0, entries_source=src)
    for _ in range(max(1, args.steps)):
        reps.append(cpu_baseline(entries, seconds=10.0, entries_source=src))
    v = float(np.mean([r["value"] for r in reps]))
    base = reps[-1]
    base["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * (time.perf_counter() - t0) / max(1, args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _config(args, 522242), "cpu_baseline": base,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------ replicas --
# N > 1 runs N independent replicas, one per GPU: each rank solves its own
# sun directions on its own copy of the operator (the solve has no
# cross-rank exchange); the job's time is the slowest rank's.
def replica_directions(terrain, rhs, rank):
    """The sun directions of one rank: seed 2 for rank 0 (the workload's
    own), 2 + rank for the others, so the replicas solve different columns."""
    return terrain.random_sun_directions(rhs, seed=2 + rank)


def job_time_ms(ms_local, dist, device):
    """Max over ranks of the timed region (identity without a process group)."""
    if dist is None:
        return float(ms_local)
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, steps, ms_total):
    """Whole-job throughput: the units all ranks processed over the job's time."""
    return world * units_per_rank * steps / (ms_total / 1000.0)


def _config(args, nfacets):
    return {"workload": (f"fBm terrain {args.grid}x{args.grid} + 30 craters ({nfacets} facets), "
                         f"{args.rhs} sun directions (elev 1-30 deg, seed 2), rho {RHO}, "
                         f"compressed FF (octree, ACA tol {args.tol}, leaf 64)"),
            "facets": nfacets, "rhs": args.rhs, "rtol": 1e-5,
            "l2": "inputs larger than L2 (E 2.1 GB, operator > 1 GB); no flush",
            "parallelism": f"replicas x{args.gpus}"}


# ------------------------------------------------ other workloads --
def _events_ms(fn, reps=5):
    import torch
    s = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(reps):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def craters_cpu_baseline(sizes, seconds=8.0):
    """The reference's ThermalModel step (model.py:44-69, 218-224: two sparse
    form-factor products and conductionQ for every facet, restated by the
    oracle: scipy CSR and oracle/pcc_oracle.c) on one host core, timed on the
    4.2k-facet spherical crater with its exact form factors and a 41-node
    grid.  Extrapolated to the batch of meshes with ``sizes`` facets by the
    cost model  step = sum_i (N_i c_cond + 2 nnz_i c_mv),  nnz_i = d N_i^2
    (d: the sample's fraction of visible pairs; the bowls are the same
    shape, so d does not depend on the facet count)."""
    from oracle import pcc as opcc
    from oracle import vis
    from fluxpy_gb300 import terrain
    from fluxpy_gb300.thermal import setgrid
    V, F = terrain.spherical_crater(n_points=2000, seed=0)
    P, N, A = vis.geometry(V, F)
    FFc = vis.Scene(V, F).ff_csr(P, N, A)
    n = F.shape[0]
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    T = np.full((n, z.size), 200.0)
    ti, rhoc = np.linspace(55.0, 400.0, z.size), np.full(z.size, 1.2e6)
    em, Fg = np.full(n, 0.95), np.full(n, 0.005)
    rng = np.random.default_rng(0)
    Q = rng.uniform(0, 600, n)
    x = rng.uniform(0, 600, n)
    # conduction: c_cond per facet-step
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds / 2:
        opcc.step_q(z, 8504.0, Q, Q, T, ti, rhoc, em, Fg)
        reps += 1
    c_cond = (time.perf_counter() - t0) / (reps * n)
    # products: c_mv per stored entry
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds / 2:
        FFc @ x
        reps += 1
    c_mv = (time.perf_counter() - t0) / (reps * FFc.nnz)
    d = FFc.nnz / float(n) ** 2
    sizes = np.asarray(sizes, np.float64)
    step_s = float(np.sum(sizes * c_cond + 2 * d * sizes**2 * c_mv))
    return {"value": float(sizes.sum()) / step_s, "unit": "facet-steps/s", "cores": 1,
            "kind": "port",
            "sample": (f"oracle conductionQ (C) and scipy CSR products on the {n}-facet "
                       f"spherical crater ({FFc.nnz} nonzeros): {c_cond * 1e6:.2f} us per "
                       f"facet-step, {c_mv * 1e9:.2f} ns per nonzero; extrapolated to the "
                       f"batch with nnz = {d:.4f} N^2 per mesh (cost model)"),
            "sample_facet_steps_per_s": 1.0 / (c_cond + 2 * FFc.nnz * c_mv / n)}


def adjoint_cpu_baseline(seconds=8.0):
    """The oracle's forward model and hand-written gradient of the coupled
    misfit (oracle/adjoint.py, FP64, dense form factors) on one host core, on
    a 24 x 24 fBm terrain sample (1,058 facets) for 8 steps; facet-steps/s
    of the gradient at the sample's size (no extrapolation)."""
    from oracle import adjoint as oadj
    from oracle import vis
    from fluxpy_gb300 import terrain
    from fluxpy_gb300.thermal import setgrid
    V, F = terrain.fbm_terrain(n=24, seed=4, n_craters=2)
    P, Nn, Ar = vis.geometry(V, F)
    FF = vis.Scene(V, F).ff_csr(P, Nn, Ar)
    n = F.shape[0]
    S = 8
    rng = np.random.default_rng(4)
    dirs = terrain.random_sun_directions(S + 1, seed=2, elev=(5, 40))
    E = np.stack([F0 * np.maximum(0, Nn @ dd) for dd in dirs], 1)
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    args = (rng.uniform(0.07, 0.2, n), rng.uniform(0.9, 0.98, n), rng.uniform(40, 120, n), z,
            np.full(z.size, 1.2e6), 3600.0, np.full((n, z.size), 220.0), np.full(n, 0.005),
            rng.uniform(150, 300, (n, S)))
    reps, t0 = 0, time.perf_counter()
    while reps == 0 or time.perf_counter() - t0 < seconds:
        oadj.coupled_gradient(FF, E, *args)
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    return {"value": n * S / dt, "unit": "facet-steps/s (forward + reverse)", "cores": 1,
            "kind": "port",
            "sample": (f"oracle coupled_gradient (numpy, FP64, sparse exact F) on a "
                       f"{n}-facet fBm terrain, {S} steps, 40 layers: {dt:.2f} s per "
                       f"gradient; at the sample's size, not extrapolated")}


def run_craters64(args):
    """64 independent crater meshes of 2k-60k facets (log-uniform sizes,
    seed 3), each a spherical bowl (depth/diameter 0.2) triangulated from
    random points, FP32 compressed operators (octree, ACA tol 1e-5, leaf 64);
    the coupled time-dependent model of ThermalModel (lagged reflected and
    infrared fluxes, 2 products per step) with PCC conduction on 40 layers
    graded 2 mm -> 1 m, ti 55 -> 400, for 2 lunar days at 300 steps per day,
    all meshes in one batch (one launch per kernel per step), the step pair
    replayed from a CUDA graph.  Metric: facet-steps/s."""
    import torch
    from fluxpy_gb300 import _lib, shape, terrain
    from fluxpy_gb300.batch import MultiMeshThermalModel
    from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                      FormFactorOctreeBlock)
    from fluxpy_gb300.thermal import setgrid
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(2000), np.log(60000), 64)).astype(np.int64)
    t0 = time.perf_counter()
    ops = []
    for i, nf in enumerate(sizes):
        g = max(10, int(np.sqrt(nf) / 3))
        npts = int(max(50, (nf - 4 * (g - 1)) // 2))
        V, F = terrain.spherical_crater(n_points=npts, seed=1000 + i, boundary_grid=g)
        sm = shape.EmbreeTrimeshShapeModel(V, F)
        ops.append(CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, leaf_size=64,
                                              RootBlock=FormFactorOctreeBlock,
                                              dtype=np.float32))
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    period = 29.53 * 86400.0
    per_day = 300
    S = 2 * per_day
    t = np.arange(S + 1) * (period / per_day)
    h = 2 * np.pi * t / period
    lat = np.deg2rad(45.0)
    D = np.column_stack([-np.sin(h), -np.sin(lat) * np.cos(h), np.cos(lat) * np.cos(h)])
    F0s = np.where(D[:, 2] > 0, F0, 0.0)
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    ti = np.linspace(55.0, 400.0, z.size)
    kw = dict(rho=RHO, z=z, ti=ti, rhoc=np.full(z.size, 1.2e6), emiss=0.95, Fgeotherm=0.005,
              T0=200.0)
    warm = 4
    res = {}
    for graph in (True, False):
        m = MultiMeshThermalModel(ops, t, D, F0s, use_graph=graph, **kw)
        m.run(warm)
        torch.cuda.synchronize()
        clocks = ClockSampler(0)
        clocks.start()
        l0 = _lib.launch_count()
        s = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        m.run()
        b.record(s)
        torch.cuda.synchronize()
        clk = clocks.stop()
        m.check_errors()
        ms = a.elapsed_time(b)
        res[graph] = dict(ms=ms, steps=S - warm, clocks=clk,
                          launches=_lib.launch_count() - l0, model=m)
    m = res[True]["model"]
    op = m.op
    steps = res[True]["steps"]
    nf_tot = op.num_faces
    value = nf_tot * steps / (res[True]["ms"] / 1000.0)
    u = torch.ones(op.num_rows, dtype=torch.float32, device="cuda")
    prod_ms = _events_ms(lambda: op.matvec_cluster(u, out=m._y, z=m._zs))
    cond_ms = _events_ms(lambda: _lib.call(
        "fgb_conduction_q_f32", op.num_rows, m.nz, _lib.ptr(m.z), float(m.dts[0]),
        _lib.ptr(m._Q[0]), _lib.ptr(m._Q[1]), _lib.ptr(m._T[0]), _lib.ptr(m._T[1]),
        _lib.ptr(m.ti), _lib.ptr(m.rhoc), _lib.ptr(m.emiss), _lib.ptr(m.Fg), _lib.ptr(m._Fsurf),
        _lib.ptr(m.flags), _lib.stream_handle()))
    op_bytes = op.nbytes
    hbm = _measured_hbm()
    prod_gbs = (op_bytes + 8 * op.num_rows + 4 * op.num_zrows) / (prod_ms / 1e3) / 1e9
    w = z.size
    cond_gbs = op.num_rows * (2 * w * 4 + 5 * 4) / (cond_ms / 1e3) / 1e9
    Ts = m.surface_temperature()
    line = {
        "metric": "facet-steps/s, 64 uneven crater meshes, coupled radiosity + conduction",
        "value": value, "unit": "facet-steps/s", "n_gpus": 1, "steps": steps, "warmup": warm,
        "ms_per_step": res[True]["ms"] / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "64 crater meshes 2k-60k facets (log-uniform, seed 3), "
                               "2 lunar days x 300 steps, 40 layers 2 mm-1 m, ti 55-400",
                   "facets": nf_tot, "meshes": 64, "rows_padded": op.num_rows,
                   "l2": "operator and state larger than L2; no flush"},
        # graph replays launch the captured kernels without passing the host
        # counter: the eager run's count is the same set of launches
        "clocks": res[True]["clocks"], "gpu_launches": int(res[False]["launches"]),
        "graph_replays": steps // 2,
        "eager": {"ms_per_step": res[False]["ms"] / steps,
                  "facet_steps_per_s": nf_tot * steps / (res[False]["ms"] / 1000.0),
                  "gpu_launches": int(res[False]["launches"])},
        "kernel_ms": {"merged_product": prod_ms, "conduction_step": cond_ms},
        "roofline": {"product": {"bound": "hbm", "achieved": prod_gbs, "peak": hbm,
                                 "unit": "GB/s", "frac": prod_gbs / hbm},
                     "conduction": {"bound": "hbm", "achieved": cond_gbs, "peak": hbm,
                                    "unit": "GB/s", "frac": cond_gbs / hbm}},
        "operator_bytes": int(op_bytes), "build_s": build_s,
        "surface_T_range_K": [float(Ts.min().item()), float(Ts.max().item())],
        "cpu_baseline": craters_cpu_baseline(sizes),
    }
    print(json.dumps(line))


def run_adjoint(args):
    """Gradient of the coupled radiosity + conduction misfit with respect to
    per-facet albedo, emissivity and thermal inertia (fluxpy_gb300.adjoint) on
    an fBm terrain (seed 4; grid 317 -> 199,712 facets), compressed operator
    (octree, tolerance 1e-5, leaf 64) stored in FP32 and applied in FP64
    arithmetic (K columns at once; F^T through the transposed operator),
    many-column solves refined with FP32 sweeps, 40 conduction layers,
    synthetic observations from perturbed fields (albedo 0.07-0.2,
    emissivity 0.9-0.98, thermal inertia 40-120), 500 steps with a
    checkpoint every 25.  Times one forward pass and one forward + reverse
    sweep; checks the gradient by central differences of the same model on
    32 random facets per field (over the first fd-steps steps)."""
    import torch
    from fluxpy_gb300 import _lib, shape, terrain
    from fluxpy_gb300.adjoint import ThermalMisfit
    from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                      FormFactorOctreeBlock)
    from fluxpy_gb300.thermal import setgrid
    t0 = time.perf_counter()
    V, F = terrain.fbm_terrain(n=args.adjoint_grid, seed=4)
    sm = shape.EmbreeTrimeshShapeModel(V, F)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, leaf_size=64,
                                    RootBlock=FormFactorOctreeBlock, dtype=np.float32)
    FF.transposed()
    FF.offload_pool()
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    N = sm.num_faces
    S = args.adjoint_steps
    period = 29.53 * 86400.0
    t = np.arange(S + 1) * (period / 300)
    h = 2 * np.pi * t / period - np.pi / 3
    lat = np.deg2rad(30.0)
    D = np.column_stack([-np.sin(h), -np.sin(lat) * np.cos(h), np.cos(lat) * np.cos(h)])
    F0s = np.where(D[:, 2] > 0, F0, 0.0)
    E = sm.get_direct_irradiance_batch(F0s, D, out_dtype=torch.float64)
    rng = np.random.default_rng(4)
    true = dict(rho=rng.uniform(0.07, 0.2, N), emiss=rng.uniform(0.9, 0.98, N),
                ti=rng.uniform(40, 120, N))
    guess = dict(rho=np.full(N, 0.12), emiss=np.full(N, 0.94), ti=np.full(N, 80.0))
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])

    def model(E_, steps):
        return ThermalMisfit(FF, E_, z, np.full(z.size, 1.2e6), period / 300,
                             np.full((N, z.size), 220.0), np.full(N, 0.005),
                             np.zeros((N, steps)), checkpoint_every=25, tol=1e-12)
    m = model(E, S)
    m.Tobs = m.surface_temperatures(**true)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    clocks = ClockSampler(0)
    clocks.start()
    l0 = _lib.launch_count()
    ev[0].record(s)
    L0 = m.value(**guess)
    ev[1].record(s)
    ev[2].record(s)
    L, grho, gem, gti = m.value_and_grad(**guess)
    ev[3].record(s)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = _lib.launch_count() - l0
    fwd_ms = ev[0].elapsed_time(ev[1])
    grad_ms = ev[2].elapsed_time(ev[3])
    fd = adjoint_fd_check(model, E, true, guess, N, args.adjoint_fd_steps, args.adjoint_fd_facets)
    line = {
        "metric": "misfit gradient (albedo, emissivity, thermal inertia) of the coupled model",
        "value": N * S / (grad_ms / 1000.0), "unit": "facet-steps/s (forward + reverse)",
        "n_gpus": 1, "steps": S, "warmup": 0, "ms_per_step": grad_ms / S,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"fBm terrain {args.adjoint_grid}x{args.adjoint_grid} (seed 4), "
                               f"{N} facets, {S} steps, 40 layers, checkpoint every 25",
                   "facets": N},
        "clocks": clk, "gpu_launches": int(launches),
        "forward_ms": fwd_ms, "forward_and_gradient_ms": grad_ms,
        "gradient_over_forward": grad_ms / fwd_ms,
        "misfit": float(L.item()), "misfit_forward_only": float(L0.item()),
        "grad_norms": {"rho": float(grho.norm().item()), "emiss": float(gem.norm().item()),
                       "ti": float(gti.norm().item())},
        "finite_differences": fd,
        "build_s": build_s, "operator_device_bytes": int(FF.device_nbytes),
        "cpu_baseline": adjoint_cpu_baseline(),
    }
    print(json.dumps(line))


def adjoint_fd_check(model, E, true, guess, N, steps, nfacets):
    """Central differences of the misfit over the first `steps` steps
    (checkpoints every 25, so several segments) on `nfacets` random facets
    per field, against the hand-written gradient of the same model; step
    1e-4 of the parameter (relative)."""
    if nfacets <= 0:
        return None
    m = model(E[:, :steps + 1].contiguous(), steps)
    m.Tobs = m.surface_temperatures(**true)
    L, grho, gem, gti = m.value_and_grad(**guess)
    grads = {"rho": grho.cpu().numpy(), "emiss": gem.cpu().numpy(), "ti": gti.cpu().numpy()}
    rng = np.random.default_rng(32)
    facets = rng.choice(N, nfacets, replace=False)
    out = {"steps": steps, "facets": int(nfacets), "rel_step": 1e-4}
    for key in ("rho", "emiss", "ti"):
        errs = []
        for i in facets:
            x = guess[key]
            h = 1e-4 * x[i]
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            Lp = m.value(**{**guess, key: xp}).item()
            Lm = m.value(**{**guess, key: xm}).item()
            fdv = (Lp - Lm) / (2 * h)
            errs.append(abs(fdv - grads[key][i]) / max(abs(fdv), 1e-300))
        out[key] = {"max_rel_err": float(np.max(errs)), "median_rel_err": float(np.median(errs))}
    return out


def run_conduction(args):
    """The PCC 1-D conduction step (PccThermalModel1D.step,
    thermal.pyx:249-261 -> conductionQ.c:10-186) for --facets facets on the
    41-node grid of the thermal configuration (setgrid(40, 1.0817, 1.0)),
    FP32 and FP64, timed with CUDA events.  Two regimes:
      diurnal    the time step of the thermal configuration (a lunar day in
                 300 steps), absorbed flux A_f max(0, cos(2 pi n / 300 +
                 phi_f)) per facet, after one day of spin-up: the state a
                 time-dependent model steps through (few predictor-corrector
                 redos);
      cold_start every profile at 250 K and a random flux each step, one
                 hour steps: most facets redo the linearisation several times.
    Metric: facet-steps/s (diurnal, FP32); roofline: the algorithmic bytes
    (profile read + write, Qprev, X, emiss, Fgeotherm, Fsurf) against the
    measured HBM bandwidth."""
    import torch
    from fluxpy_gb300 import _lib
    from fluxpy_gb300.thermal import PccThermalModel1D, setgrid
    nf = args.facets
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    rng = np.random.default_rng(3)
    ti = np.linspace(55.0, 400.0, z.size)
    rhoc = np.full(z.size, 1.2e6)
    hbm = _measured_hbm()
    dev = torch.device("cuda")
    steps = max(args.steps, 20)
    day = 300
    amp = rng.uniform(0, 1000, nf)
    phase = rng.uniform(0, 2 * np.pi, nf)

    def forcing(n, tdt):
        x = amp * np.maximum(0.0, np.cos(2 * np.pi * n / day + phase))
        return torch.as_tensor(x, device=dev, dtype=tdt)

    def timed(dt, regime):
        tdt = torch.float64 if dt == np.float64 else torch.float32
        if regime == "diurnal":
            m = PccThermalModel1D(z, np.full((nf, z.size), 250.0), ti, rhoc, np.full(nf, 0.95),
                                  np.full(nf, 0.005), forcing(0, tdt).cpu().numpy().astype(np.float64),
                                  np.full(nf, 250.0), dtype=dt)
            step_dt = 29.53 * 86400.0 / day
            spin = args.conduction_spinup
            xs = [forcing(n, tdt) for n in range(1, spin + steps + 1)]
            for n in range(spin):
                m.step(step_dt, xs[n], check=False)
            run = xs[spin:]
        else:
            m = PccThermalModel1D(z, np.full((nf, z.size), 250.0), ti, rhoc, np.full(nf, 0.95),
                                  np.full(nf, 0.005), rng.uniform(0, 400, nf), np.full(nf, 250.0),
                                  dtype=dt)
            step_dt = 3600.0
            run = [torch.as_tensor(rng.uniform(0, 400, nf), device=dev, dtype=tdt)
                   for _ in range(steps + 3)]
            for n in range(3):
                m.step(step_dt, run[n], check=False)
            run = run[3:]
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = _lib.launch_count()
        a.record(s)
        for x in run:
            m.step(step_dt, x, check=False)
        b.record(s)
        torch.cuda.synchronize()
        m.check_errors()
        ms = a.elapsed_time(b) / len(run)
        isz = np.dtype(dt).itemsize
        per = 2 * z.size * isz + 5 * isz
        gbs = nf * per / (ms * 1e-3) / 1e9
        del m
        return {"facet_steps_per_s": nf / (ms * 1e-3), "ms_per_step": ms,
                "bytes_per_facet_step": per, "achieved_gbs": gbs, "frac": gbs / hbm,
                "launches": int(_lib.launch_count() - l0), "steps": len(run)}

    clocks = ClockSampler(0)
    clocks.start()
    out = {f"{name}_{regime}": timed(dt, regime)
           for regime in ("diurnal", "cold_start")
           for name, dt in (("fp32", np.float32), ("fp64", np.float64))}
    clk = clocks.stop()
    from oracle import pcc as opcc
    ns = 4096
    Ts = np.full((ns, z.size), 250.0)
    Q = rng.uniform(0, 400, ns)
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < 3.0:
        opcc.step_q(z, 3600.0, Q, Q, Ts, ti, rhoc, np.full(ns, 0.95), np.full(ns, 0.005))
        reps += 1
    cpu = ns * reps / (time.perf_counter() - t0)
    f32 = out["fp32_diurnal"]
    line = {"metric": "conduction facet-steps/s (41 nodes)", "value": f32["facet_steps_per_s"],
            "unit": "facet-steps/s", "n_gpus": 1, "steps": f32["steps"],
            "warmup": args.conduction_spinup,
            "ms_per_step": f32["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": f"PCC conduction step, {nf} facets, 41-node grid "
                                   "(2 mm - 1 m), ti 55-400, diurnal forcing, 300 steps per "
                                   f"lunar day after {args.conduction_spinup} spin-up steps",
                       "facets": nf,
                       "l2": "profiles larger than L2 at the default size; no flush"},
            "clocks": clk, "gpu_launches": f32["launches"],
            "roofline": {"bound": "hbm", "achieved": f32["achieved_gbs"], "peak": hbm,
                         "unit": "GB/s", "frac": f32["frac"], "traffic": None},
            "regimes": out,
            "cpu_baseline": {"value": cpu, "unit": "facet-steps/s", "cores": 1, "kind": "port",
                             "sample": f"oracle conductionQ (C), {ns} facets x {reps} steps"}}
    print(json.dumps(line))


def _measured_hbm():
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except Exception:
        return 6800.0


# ------------------------------------------------------------- GPU arm --
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "craters64":
        run_craters64(args)
        return
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "conduction":
        run_conduction(args)
        return
    # the operator and the solver's buffers take most of the device: let the
    # caching allocator grow segments instead of fragmenting
    os.environ.setdefault("PYTORCH_CUDA_ALLOC_CONF", "expandable_segments:True")
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    from fluxpy_gb300 import _lib, shape, terrain
    from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                      FormFactorOctreeBlock)
    from fluxpy_gb300.form_factors import get_form_factor_matrix
    from fluxpy_gb300.solve import solve_radiosity, solve_radiosity_batched
    dev = torch.device("cuda", torch.cuda.current_device())
    t_setup = time.perf_counter()
    V, F = terrain.fbm_terrain(n=args.grid, seed=1)
    sm = shape.EmbreeTrimeshShapeModel(V, F)
    FF = CompressedFormFactorMatrix(sm, tol=args.tol, min_size=4096, leaf_size=64,
                                    RootBlock=FormFactorOctreeBlock, dtype=np.float32)
    # build the FP32 panels and the tensor-core operands, then move the
    # block pool and the exact-leaf CSR (not used by the products) to host
    FF.offload_pool()
    FF.tc_operands(split=True)
    # kernel layouts of the BF16 / split products: timed on this operator
    tune = FF.autotune_products(args.rhs)
    if args.plain_tiles != "auto":
        FF.product_plan()["plain"] = "b" + args.plain_tiles
    if args.split_plan != "auto":
        FF.product_plan()["split"] = args.split_plan
    nf = sm.num_faces
    dirs = replica_directions(terrain, args.rhs, rank)
    E = sm.get_direct_irradiance_batch(F0, dirs, out_dtype=torch.float32)
    Ep = FF.permute(E).contiguous()
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    # device memory held by the operator, its tensor-core operands and E
    setup_bytes = int(torch.cuda.memory_allocated())

    def step():
        st = {}
        B = solve_radiosity_batched(FF, Ep, RHO, rtol=1e-5, precision="bf16-refine",
                                    E_is_permuted=True, return_permuted=True, stats=st)
        return B, st

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    stream = torch.cuda.current_stream()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches0 = _lib.launch_count()
    torch.cuda.synchronize()
    # an NVTX range marks the timed steps (profilers can filter on it)
    torch.cuda.nvtx.range_push("timed_steps")
    ev0.record(stream)
    stats = []
    marks = []
    for _ in range(args.steps):
        B, st = step()
        stats.append(st)
        marks.append(torch.cuda.Event(enable_timing=True))
        marks[-1].record(stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    step_ms = [a.elapsed_time(b) for a, b in zip([ev0] + marks[:-1], marks)]
    launches = _lib.launch_count() - launches0
    clk = clocks.stop()
    ms_total = job_time_ms(ev0.elapsed_time(ev1), dist, dev)
    if dist:
        dist.barrier()
    ms_step = ms_total / args.steps
    value = job_rate(args.rhs, world, args.steps, ms_total)

    extras = {}
    if rank == 0 and not args.no_extras:
        extras = measure_extras(args, FF, sm, E, Ep, B, stats, dev)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic", "config": _config(args, nf), "clocks": clk,
        "gpu_launches": int(launches),
        "ms_each_step": [round(t, 2) for t in step_ms],
        "solver": {"outer": [s["outer"] for s in stats], "bf16_matmats": stats[-1]["bf16_matmats"],
                   "split_bf16_matmats": stats[-1].get("split_matmats", 0),
                   "fp32_matmats": stats[-1]["fp32_matmats"], "chunks": stats[-1].get("chunks", 1),
                   "residual_checked": stats[-1].get("residual")},
        "setup_s": setup_s, "device_bytes_after_setup": setup_bytes, "build": {k: (round(v, 3) if isinstance(v, float) else v)
                                      for k, v in FF.stats.items() if k != "autotune"},
        "near_edge_pairs": int(FF.stats.get("near_edge_pairs", 0)),
        "near_edge_note": ("visible pairs of the exact leaves whose ray passed within 1e-6 "
                           "(relative) of a triangle edge, decided in FP64 and counted"),
        "operator_entries": int(FF.stats["operator_entries"]),
        "autotune_ms": tune,
        "product_plan": dict(FF.product_plan()),
    }
    line.update(extras)
    fp = extras.get("fp32_plain")
    if fp:
        line["speedup_vs_fp32_plain"] = {
            "batched": (value / world) / fp["batched_solves_per_s"],
            "single_rhs": (value / world) / fp["single_rhs_solves_per_s"]}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def operator_work(FF):
    """Stored entries of the operator's leaves, from its block list: the U
    (sum r m) and V (sum r n) factors of the low-rank blocks and the
    nonzeros of the exact leaves."""
    from fluxpy_gb300.compressed_form_factors import LEAF_LOWRANK
    tree = FF._tree
    lr = (FF._kind == LEAF_LOWRANK) & (FF._rank > 0)
    r = FF._rank[lr].astype(np.int64)
    return {"lowrank_u_entries": int(np.sum(r * tree.size[FF._rows[lr]])),
            "lowrank_v_entries": int(np.sum(r * tree.size[FF._cols[lr]])),
            "exact_nnz": int(FF.stats.get("exact_nnz", 0)),
            "lowrank_blocks": int(lr.sum())}


# DRAM traffic of one phase-B launch (tc_gather_gemm, plain BF16, 128-row
# tiles) from a small-case ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum, -c 1); the full-size figure scales it by the
# executed panel weights times the columns (units of work).  The small case
# keeps more of its gathered source rows in L2 than the full size does, so
# the scaled figure is a lower bound.
TRAFFIC_CAPTURE = {"kernel": "phaseB_tc", "tile_rows": 128, "panel_rows": 2006912,
                   "columns": 1024, "dram_bytes": 1124346000 + 122825472,
                   "source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum (1 pass) of one "
                              "tc_gather_gemm<1, 0, 128> launch on the 128x128 terrain (32,258 "
                              "facets, 2,006,912 panel rows, 1,024 columns), scaled by panel rows "
                              "x columns; a lower bound at full size, where fewer gathered "
                              "sources stay in L2")}


def scaled_dram_traffic(kernel, FF, K, tile_rows):
    """The capture's DRAM bytes scaled to this launch (None when the timed
    kernel or its tile layout is not the one captured)."""
    c = TRAFFIC_CAPTURE
    if kernel != c["kernel"] or tile_rows != c["tile_rows"] or not c["dram_bytes"]:
        return None
    rows = int(FF.stats.get(f"panel_rows_{tile_rows}", 0))
    return c["dram_bytes"] * (rows * K) / (c["panel_rows"] * c["columns"])


def fp64_solve_permuted(FF, Ep_cols, tol=1e-13, max_iter=200, rho=RHO):
    """Right-placement Jacobi of the compressed operator in FP64 arithmetic
    (the FP32-stored operator, K = 1 products), per column, to a relative
    update of tol: the FP64 solution of the stored system."""
    import torch
    cols = []
    for q in range(Ep_cols.shape[1]):
        e = Ep_cols[:, q].double().contiguous()
        b = e.clone()
        thr = tol * float(e.abs().max())
        for _ in range(max_iter):
            b1 = FF.matvec_permuted((rho * b).contiguous(), "fp32-fp64", add=e)
            done = float((b1 - b).abs().max()) <= thr
            b = b1
            if done:
                break
        cols.append(b)
    return torch.stack(cols, 1)


def measure_errors(FF, sm, Ep, B, dev, nrows=256, ncols=32):
    """Errors of the many-direction solve against FP64 references:
    - compression: |(F~ - F) x| on nrows random rows of the exactly assembled
      FP64 form factors, relative to max|F x| (x uniform in [0, 1]);
    - residual of the computed B with the exact FP64 rows, per column
      relative to max|E|, on ncols columns;
    - solution: |B - B64| / max|B64| with B64 the FP64 solve of the stored
      system (all rows), and on the sampled rows the residual of B64 with the
      exact rows (the compression's share of the error);
    - the residual of B in FP64 arithmetic on the stored operator."""
    import torch
    from fluxpy_gb300.form_factors import get_form_factor_matrix
    N, K = Ep.shape
    rng = np.random.default_rng(0)
    rows = np.sort(rng.choice(N, nrows, replace=False))
    facet_rows = FF._tree.perm[rows]
    Fx = get_form_factor_matrix(sm, facet_rows)          # exact FP64 rows (all columns)
    x = rng.uniform(0, 1, N)
    y_exact = Fx @ x
    y_c = FF @ x
    comp = float(np.max(np.abs(y_c[facet_rows] - y_exact)) / np.max(np.abs(y_exact)))
    cols = torch.as_tensor(np.linspace(0, K - 1, ncols).astype(np.int64), device=dev)
    Bp = B[:, cols].double().contiguous()
    Epc = Ep[:, cols].double().contiguous()
    res_stored = []
    for q in range(ncols):
        y = FF.matvec_permuted((RHO * Bp[:, q]).contiguous(), "fp32-fp64")
        r = Epc[:, q] - (Bp[:, q] - y)
        res_stored.append(float(r.abs().max() / Epc[:, q].abs().max()))
    B64 = fp64_solve_permuted(FF, Epc)
    sol = ((Bp - B64).abs().amax(0) / B64.abs().amax(0)).cpu().numpy()
    # residuals with the exact rows (facet order)
    Bf = FF.unpermute(Bp).cpu().numpy()
    B64f = FF.unpermute(B64).cpu().numpy()
    Ef = FF.unpermute(Epc).cpu().numpy()
    emax = np.maximum(np.abs(Ef).max(0), 1e-30)
    r_B = Ef[facet_rows] - (Bf[facet_rows] - Fx @ (RHO * Bf))
    r_64 = Ef[facet_rows] - (B64f[facet_rows] - Fx @ (RHO * B64f))
    return {"compression_rel_err_sampled_rows": comp, "rows": nrows, "columns": ncols,
            "residual_vs_exact_rows": float(np.max(np.abs(r_B).max(0) / emax)),
            "solution_rel_err_vs_fp64_solve": float(sol.max()),
            "fp64_solve_residual_vs_exact_rows": float(np.max(np.abs(r_64).max(0) / emax)),
            "residual_rel_fp64_stored_operator": max(res_stored),
            "note": ("rows: random rows of the uncompressed form factors assembled exactly in "
                     "FP64; compression: |(F~ - F) x| / max|F x| on them; residual_vs_exact_"
                     "rows: max|E - (B - rho F B)| / max|E| with those rows, per column; "
                     "solution: max|B - B64| / max|B64| per column, B64 the FP64 Jacobi solve "
                     "(1e-13) of the stored operator; its residual with the exact rows shows the "
                     "compression's part")}


def measure_single_direction(FF, sm, dev, elev=5.0, azim=0.0):
    """One sun direction (elevation 5 degrees): the plain FP32 Jacobi with
    the K = 1 kernels to a relative update of RTOL, timed (CUDA events), and
    its error against the FP64 solve of the stored operator."""
    import torch
    from fluxpy_gb300 import terrain
    d = terrain.sun_directions([elev], [azim])
    E1 = sm.get_direct_irradiance_batch(F0, d, out_dtype=torch.float32)
    e = FF.permute(E1[:, 0]).contiguous()
    tol = RTOL * float(e.abs().max())

    def solve():
        b = e.clone()
        for it in range(1, 200):
            b1 = FF.matvec_permuted(RHO * b, "fp32", add=e)
            if float((b1 - b).abs().max()) <= tol:
                return b, it
            b = b1
        return b, it
    solve()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    a.record(s)
    for _ in range(reps):
        b, its = solve()
    z.record(s)
    torch.cuda.synchronize()
    ms = a.elapsed_time(z) / reps
    b64 = fp64_solve_permuted(FF, e.reshape(-1, 1))[:, 0]
    err = float((b.double() - b64).abs().max() / b64.abs().max())
    r = e.double() - (b.double() - FF.matvec_permuted((RHO * b.double()).contiguous(),
                                                      "fp32-fp64"))
    return {"elevation_deg": elev, "azimuth_deg": azim, "solves_per_s": 1000.0 / ms,
            "ms_per_solve": ms, "jacobi_iterations": its,
            "rel_err_vs_fp64_solve": err,
            "residual_rel_fp64": float(r.abs().max() / e.abs().max())}


def measure_steady_state(FF, E):
    """compute_steady_state_temp (model.py:8-42 semantics) for all K
    directions at once through the BF16+refine solver (visible solve, one
    K-column product, infrared solve with rho = 1), timed with CUDA events
    after one untimed call; emissivity 0.95."""
    import torch
    from fluxpy_gb300.model import compute_steady_state_temp
    compute_steady_state_temp(FF, E, RHO, 0.95, method="batched-bf16")
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    T = compute_steady_state_temp(FF, E, RHO, 0.95, method="batched-bf16")
    z.record(s)
    torch.cuda.synchronize()
    ms = a.elapsed_time(z)
    K = E.shape[1]
    # against FP64 arithmetic on the stored operator for 8 directions: the
    # visible and infrared Jacobi solves to 1e-13, the infrared product
    from scipy.constants import Stefan_Boltzmann as sig
    cols = list(range(0, K, max(1, K // 8)))[:8]
    Ep8 = FF.permute(E[:, cols].double())
    B64 = fp64_solve_permuted(FF, Ep8).clamp_min(0)
    IR = torch.stack([FF.matvec_permuted(((1 - RHO) * B64[:, q]).contiguous(), "fp32-fp64")
                      for q in range(len(cols))], 1)
    Q64 = fp64_solve_permuted(FF, IR, max_iter=1000, rho=1.0).clamp_min(0)
    T64 = FF.unpermute(((((1 - RHO) * B64 + 0.95 * Q64) / (0.95 * sig)) ** 0.25))
    dT = (T[cols, :].double().T - T64).abs()
    return {"directions": K, "ms": ms, "directions_per_s": K / (ms / 1000.0),
            "T_range_K": [float(T.min().item()), float(T.max().item())],
            "T_err_vs_fp64_K": {"columns": len(cols), "max": float(dT.max().item()),
                                "median": float(dT.median().item())},
            "note": "visible solve, infrared product (split-BF16 tensor cores) and infrared "
                    "solve (rho = 1), each column to a relative residual 1e-5, BF16+refine; "
                    "T_err against FP64 solves of the stored operator"}


def measure_extras(args, FF, sm, E, Ep, B, stats, dev):
    import ctypes as C
    import torch
    from fluxpy_gb300 import _lib
    from fluxpy_gb300.form_factors import get_form_factor_matrix
    from fluxpy_gb300.solve import solve_radiosity, solve_radiosity_batched
    out = {}
    N, K_all = Ep.shape
    stream = torch.cuda.current_stream()
    # ---- e2e through the public API with host buffers, first (the same
    # device memory state as the timed steps): pinned host E in, B out into
    # a pinned host buffer allocated once
    K = K_all
    E_host = torch.empty((N, K), dtype=torch.float32, pin_memory=True)
    E_host.copy_(E.cpu())
    B_host = torch.empty((N, K), dtype=torch.float32, pin_memory=True)
    solve_radiosity(FF, E_host, RHO, method="batched-bf16", out=B_host)
    torch.cuda.synchronize()
    reps = max(1, min(3, args.steps))
    t0 = time.perf_counter()
    for _ in range(reps):
        Bh, _ = solve_radiosity(FF, E_host, RHO, method="batched-bf16", out=B_host)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / reps
    out["e2e"] = {"value": K / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": N * K * 4,
                  "d2h_bytes_per_step": N * K * 4, "ms_per_step": t_e2e * 1e3,
                  "note": "solve_radiosity(FF, E_host, 0.12, method='batched-bf16', out=B_host),"
                          " pinned host buffers; B is copied to B_host on a side stream while"
                          " the last residual check runs"}
    del E_host, B_host, Bh
    torch.cuda.empty_cache()
    # ---- dominant kernels, timed alone with CUDA events, on the column
    # block the solver works on (it solves the 1,024 columns in blocks that
    # fit in memory)
    from fluxpy_gb300.solve import _auto_chunk
    K = min(K_all, _auto_chunk(FF, N, K_all, fp32_z=False))
    zr = max(FF._num_zrows, 1)
    Ek = Ep[:, :K].contiguous()
    X32 = (RHO * Ek).contiguous()
    # sources stacked as [Z; X] (hi and lo parts), as the solver keeps them
    nz = int(FF._num_zrows)
    sh = torch.zeros((nz + N, K), dtype=torch.bfloat16, device=dev)
    sl = torch.zeros_like(sh)
    zh, xh = sh[:nz], sh[nz:]
    zl, xl = sl[:nz], sl[nz:]
    Y = torch.empty_like(Ek)
    tc = FF.tc_operands(split=True)
    panel_f, vpanel_f = FF.panels("fp32")
    flags = FF.device_flags()
    desc = C.byref(FF._desc)
    st = _lib.stream_handle
    _lib.call("fgb_split_bf16", _lib.ptr(X32), _lib.ptr(xh), _lib.ptr(xl), N * K, st())

    def t_events(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    def tc_a(split, rows64=True):
        # phase A as the solver runs it: whole-group work items, Z written
        # directly as BF16 (hi, and lo for the split product, on 64-row work
        # slices)
        dsc = FF._desc_tc64 if split and rows64 else FF._desc_tc
        _lib.call("fgb_tc_phase_a_bf16", C.byref(dsc), _lib.ptr(tc["vt_hi"]),
                  _lib.ptr(tc["vt_lo"]) if split else None, _lib.ptr(xh),
                  _lib.ptr(xl) if split else None, _lib.ptr(zh), _lib.ptr(zl) if split else None,
                  K, _lib.ptr(flags), st())

    plain_plan = FF.product_plan()["plain"]
    plain_rows = {"b128": 128, "b256": 256}.get(plain_plan, 64)

    split_plan = FF.product_plan()["split"]
    split_rows = 128 if split_plan.endswith("b128") else 64

    def tc_b(split, rows=None):
        # the layouts the autotuner chose, as the solver runs them: plain
        # products on 128- or 256-row tiles, split ones on 64- or 128-row
        # tiles
        rows = (split_rows if split else plain_rows) if rows is None else rows
        if split and rows == 128:
            _lib.call("fgb_tc_phase_b", C.byref(FF._desc128), _lib.ptr(tc["w128"]),
                      _lib.ptr(FF._split128_lo()), _lib.ptr(xh), _lib.ptr(xl), _lib.ptr(zh),
                      _lib.ptr(zl), _lib.ptr(Y), K, _lib.ptr(Ek), 1.0, _lib.ptr(flags), st())
            return
        if rows in (128, 256) and not split:
            dsc, w = ((FF._desc128, tc["w128"]) if rows == 128 else
                      (FF._desc256, FF.tc_operands256()["w256"]))
            _lib.call("fgb_tc_phase_b", C.byref(dsc), _lib.ptr(w), None,
                      _lib.ptr(xh), None, _lib.ptr(zh), None, _lib.ptr(Y), K, _lib.ptr(Ek), 1.0,
                      _lib.ptr(flags), st())
            return
        _lib.call("fgb_tc_phase_b", desc, _lib.ptr(tc["w_hi"]),
                  _lib.ptr(tc["w_lo"]) if split else None, _lib.ptr(xh),
                  _lib.ptr(xl) if split else None, _lib.ptr(zh), _lib.ptr(zl) if split else None,
                  _lib.ptr(Y), K, _lib.ptr(Ek), 1.0, _lib.ptr(flags), st())

    def tc_b_tma():
        _lib.call("fgb_tc_phase_b_tma", desc, _lib.ptr(tc["w_hi"]), None, _lib.ptr(sh), None,
                  _lib.ptr(Y), K, _lib.ptr(Ek), 1.0, _lib.ptr(flags), st())

    def f32(phases):
        _lib.call("fgb_matmat_f32", desc, _lib.ptr(panel_f), _lib.ptr(vpanel_f), _lib.ptr(X32),
                  _lib.ptr(Z32), _lib.ptr(Y), K, None, 1.0, int(FF._needs_zero_z), phases, st())

    a_rows64 = split_plan.startswith("a64")
    ms = {"phaseA_tc": t_events(lambda: tc_a(False)), "phaseB_tc": t_events(lambda: tc_b(False)),
          "phaseA_tc_split": t_events(lambda: tc_a(True, rows64=a_rows64)),
          "phaseB_tc_split": t_events(lambda: tc_b(True))}
    ms_split_other = t_events(lambda: tc_b(True, rows=192 - split_rows), 3)
    if split_rows == 64:
        FF.tc_operands().pop("w128_lo", None)    # built for this comparison only
        torch.cuda.empty_cache()
    ms_tma = t_events(tc_b_tma, 3)
    ms_a_other = t_events(lambda: tc_a(True, rows64=not a_rows64), 3)
    ms_b64 = t_events(lambda: tc_b(False, rows=64), 3)
    ms_bwide = {r: t_events(lambda: tc_b(False, rows=r), 3) for r in (128, 256)
                if r != plain_rows and (r == 128 or "w256" in FF.tc_operands())}
    # the FP32 kernels write Z in FP32 (the BF16 sources are not needed)
    del xh, xl, zh, zl, sh, sl
    Z32 = torch.zeros((zr, K), dtype=torch.float32, device=dev)
    ms["phaseA_f32"] = t_events(lambda: f32(1), 3)
    ms["phaseB_f32"] = t_events(lambda: f32(2), 3)
    FF.check_device_flags()
    # algorithmic work per launch, from the operator's own blocks: phase B
    # applies the U factors of the low-rank blocks (sum r m weights) and the
    # exact leaves (nnz values + a column index each), phase A the V factors
    # (sum r n); flops 2 per stored entry and right-hand side (x3 for the
    # split products); every source row read once, outputs written once.
    # The executed work counts the padded panel weights instead.
    alg = operator_work(FF)
    U_, V_, nnz = alg["lowrank_u_entries"], alg["lowrank_v_entries"], alg["exact_nnz"]
    zrows = int(FF._num_zrows)
    rows_plain = int(FF.stats.get(f"panel_rows_{plain_rows}", FF._panel_rows))
    work = {   # (algorithmic bytes, algorithmic flops, executed flops)
        "phaseA_tc": (2 * V_ + 2 * K * N + 2 * K * zrows, 2.0 * V_ * K,
                      2.0 * int(FF._vpanel_size) * K),
        "phaseB_tc": (2 * U_ + 6 * nnz + 2 * K * (zrows + N) + 8 * K * N, 2.0 * (U_ + nnz) * K,
                      2.0 * rows_plain * plain_rows * K),
        "phaseA_tc_split": (4 * V_ + 4 * K * N + 4 * K * zrows, 6.0 * V_ * K,
                            6.0 * int(FF._vpanel_size) * K),
        "phaseB_tc_split": (4 * U_ + 8 * nnz + 4 * K * (zrows + N) + 8 * K * N,
                            6.0 * (U_ + nnz) * K,
                            6.0 * int(FF.stats.get(f"panel_rows_{split_rows}", FF._panel_rows))
                            * split_rows * K),
        "phaseA_f32": (4 * V_ + 4 * K * N + 4 * K * zrows, 2.0 * V_ * K,
                       2.0 * int(FF._vpanel_size) * K),
        "phaseB_f32": (4 * U_ + 8 * nnz + 4 * K * (zrows + N) + 8 * K * N, 2.0 * (U_ + nnz) * K,
                       2.0 * int(FF._panel_rows) * 64 * K)}
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    tf = float(peaks.get("bf16_tflops", 1900.0))
    src = "measured" if pk.exists() else "fallback"
    s_last = stats[-1]
    nb, ns, nf = (s_last.get("bf16_matmats", 0), s_last.get("split_matmats", 0),
                  s_last.get("fp32_matmats", 0))
    per_step = {"phaseA_tc": ms["phaseA_tc"] * nb, "phaseB_tc": ms["phaseB_tc"] * nb,
                "phaseA_tc_split": ms["phaseA_tc_split"] * ns,
                "phaseB_tc_split": ms["phaseB_tc_split"] * ns,
                "phaseA_f32": ms["phaseA_f32"] * nf, "phaseB_f32": ms["phaseB_f32"] * nf}
    dom = max(per_step, key=per_step.get)
    t_ms = ms[dom]
    byts, fl, fl_exec = work[dom]
    gbs = byts / (t_ms * 1e-3) / 1e9
    tfl = fl / (t_ms * 1e-3) / 1e12
    # the roofline's bound: arithmetic intensity against the ridge point of
    # the measured peaks
    ai = fl / byts
    ridge = tf * 1e12 / (hbm * 1e9)
    traffic = scaled_dram_traffic(dom, FF, K, plain_rows)
    common = {"kernel": dom, "traffic": traffic, "traffic_source": TRAFFIC_CAPTURE["source"],
              "peak_source": src, "algorithmic_flops": fl, "algorithmic_bytes": byts,
              "executed_flops": fl_exec, "executed_tflops": fl_exec / (t_ms * 1e-3) / 1e12,
              "arithmetic_intensity": ai, "ridge_flop_per_byte": ridge,
              "ms_per_launch": t_ms, "hbm_gbs_algorithmic": gbs, "hbm_peak": hbm,
              "tflops_algorithmic": tfl, "bf16_peak": tf,
              "frac_of_tensor_peak": tfl / tf, "frac_of_hbm_peak": gbs / hbm}
    if "tc" in dom and ai >= ridge:
        out["roofline"] = {"bound": "tensor", "achieved": tfl, "peak": tf, "unit": "TFLOP/s",
                           "frac": tfl / tf, **common}
    else:
        out["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                           "frac": gbs / hbm, **common}
    out["kernel_ms"] = {"columns": K, **ms, "phaseB_tc_tma_gather_variant": ms_tma,
                        "phaseB_tc_tile_rows": plain_rows,
                        "phaseB_tc_64row_tiles": ms_b64,
                        **{f"phaseB_tc_{r}row_tiles": v for r, v in ms_bwide.items()},
                        "phaseB_tc_split_tile_rows": split_rows,
                        f"phaseB_tc_split_{192 - split_rows}row_tiles": ms_split_other,
                        "phaseA_tc_split_slice_rows": 64 if a_rows64 else 128,
                        f"phaseA_tc_split_{128 if a_rows64 else 64}row_slices": ms_a_other,
                        "per_step_ms": per_step,
                        "tflops_algorithmic": {k: work[k][1] / (ms[k] * 1e-3) / 1e12 for k in ms},
                        "tflops_executed": {k: work[k][2] / (ms[k] * 1e-3) / 1e12 for k in ms}}
    del X32, Z32, Y, Ek
    torch.cuda.empty_cache()
    K = K_all
    # ---- plain FP32 GPU paths
    st = {}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    solve_radiosity_batched(FF, Ep, RHO, precision="fp32", E_is_permuted=True,
                            return_permuted=True, stats=st)
    torch.cuda.synchronize()
    t_fp32 = time.perf_counter() - t0
    ncol = 8
    t0 = time.perf_counter()
    iters = []
    for c in range(ncol):
        e = Ep[:, c].contiguous()
        b = e.clone()
        tol = 1e-5 * float(e.abs().max())
        for it in range(1, 200):
            b1 = FF.matvec_permuted(RHO * b, "fp32", add=e)
            if float((b1 - b).abs().max()) <= tol:
                break
            b = b1
        iters.append(it)
    torch.cuda.synchronize()
    t_single = (time.perf_counter() - t0) / ncol
    value_fp32_batched = K / t_fp32
    out["fp32_plain"] = {"batched_solves_per_s": value_fp32_batched, "batched_iterations": st["outer"],
                         "single_rhs_solves_per_s": 1.0 / t_single,
                         "single_rhs_iterations": iters}
    # ---- errors against FP64: 256 exactly assembled rows of the
    # uncompressed form factors (FP64 pair kernel), 32 columns
    out["error"] = measure_errors(FF, sm, Ep, B, dev)
    # ---- config 2: one FP32 right-hand side (sun at 5 degrees elevation),
    # plain FP32 Jacobi with the K = 1 kernels, against FP64
    out["single_direction"] = measure_single_direction(FF, sm, dev)
    # ---- steady-state temperature of every direction (visible and
    # infrared solves, compute_steady_state_temp with the batched solver)
    try:
        out["steady_state"] = measure_steady_state(FF, E)
    except Exception as e:  # secondary measurements must not break the line
        out["steady_state"] = {"error": str(e)}
    # ---- the other hot-path kernels on the same terrain
    try:
        out["other_paths"] = measure_other_paths(FF, sm, dev, hbm)
    except Exception as e:  # secondary measurements must not break the line
        out["other_paths"] = {"error": str(e)}
    # ---- CPU baseline (oracle port, bounded sample)
    try:
        out["cpu_baseline"] = cpu_baseline(int(FF.stats["operator_entries"]),
                                           entries_source="this run's operator")
    except Exception as e:  # the checker must not break the GPU measurement
        out["cpu_baseline"] = {"value": None, "error": str(e)}
    return out


def measure_other_paths(FF, sm, dev, hbm):
    """Insolation rays/s, pair-kernel pairs/s (from the operator build) and
    the 1-D conduction step (facet-steps/s, against HBM bandwidth) on the
    bench terrain; the conduction CPU rate is the oracle's restatement of
    the reference's serial conductionQ loop on a sample of facets."""
    import torch
    from fluxpy_gb300 import terrain
    from fluxpy_gb300.thermal import PccThermalModel1D, setgrid
    stream = torch.cuda.current_stream()
    out = {}
    nf = sm.num_faces
    # insolation: one ray per facet and direction
    dirs = terrain.random_sun_directions(256, seed=5)
    sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float32)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float32)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    out["insolation"] = {"rays_per_s": nf * 256 / (ms * 1e-3), "directions": 256, "ms": ms}
    st = FF.stats
    if st.get("exact_s"):
        out["pair_kernel"] = {"kept_pairs_per_s": st["kept_pairs"] / st["exact_s"],
                              "kept_pairs": st["kept_pairs"], "s": st["exact_s"],
                              "note": "visibility ray + form factor per kept pair (count and "
                                      "fill passes), from the operator build"}
    # conduction: 41-node grid (setgrid(40, 1.0817, 1.0) as in the thermal
    # configuration), every facet of the terrain
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    rng = np.random.default_rng(3)
    ti = np.linspace(55.0, 400.0, z.size)
    rhoc = np.full(z.size, 1.2e6)
    emiss = np.full(nf, 0.95)
    Fg = np.full(nf, 0.005)
    Q0 = rng.uniform(0, 400, nf)
    Ts = np.full(nf, 250.0)
    cond = {}
    for dt_name, dt in (("fp64", np.float64), ("fp32", np.float32)):
        m = PccThermalModel1D(z, np.full((nf, z.size), 250.0), ti, rhoc, emiss, Fg, Q0, Ts,
                              dtype=dt)
        X = torch.as_tensor(rng.uniform(0, 400, nf), device=dev,
                            dtype=torch.float64 if dt == np.float64 else torch.float32)
        for _ in range(3):
            m.step(3600.0, X, check=False)
        torch.cuda.synchronize()
        a.record(stream)
        nsteps = 20
        for _ in range(nsteps):
            m.step(3600.0, X, check=False)
        b.record(stream)
        torch.cuda.synchronize()
        m.check_errors()
        ms = a.elapsed_time(b) / nsteps
        isz = 8 if dt == np.float64 else 4
        per = 2 * z.size * isz + 5 * isz      # T read + write, Qprev, X, emiss, Fgeotherm, Fsurf
        gbs = nf * per / (ms * 1e-3) / 1e9
        cond[dt_name] = {"facet_steps_per_s": nf / (ms * 1e-3), "ms_per_step": ms,
                         "bytes_per_facet_step": per, "achieved_gbs": gbs, "hbm_peak": hbm,
                         "frac": gbs / hbm}
        del m
    try:
        from oracle import pcc as opcc
        ns = 4096
        T = np.full((ns, z.size), 250.0)
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 2.0:
            opcc.step_q(z, 3600.0, Q0[:ns], Q0[:ns], T, ti, rhoc, emiss[:ns], Fg[:ns])
            reps += 1
        rate = ns * reps / (time.perf_counter() - t0)
        cond["cpu_oracle"] = {"facet_steps_per_s": rate, "cores": 1,
                              "sample": f"{ns} facets x {reps} steps, serial C loop"}
    except Exception as e:
        cond["cpu_oracle"] = {"error": str(e)}
    out["conduction"] = cond
    return out


if __name__ == "__main__":
    main()
