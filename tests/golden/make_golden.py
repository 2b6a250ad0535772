"""Generate the golden fixtures under tests/golden/ from the reference tree.

Run where the fluxpy reference is checked out (read-only), with
FLUXPY_REFERENCE naming that checkout:

    FLUXPY_REFERENCE=<checkout> python tests/golden/make_golden.py [section ...]

Sections:
  pcc      the reference's PCC golden files
           (tests/data/thermal/pcc_thermal_model_1d/{Tsurface,Tprofile}_conductionQ,
           written by the reference's own PCC code) parsed into
           pcc_conductionQ.npz.
  spheres  the reference's sphere meshes (tests/data/icosa_sphere*.npz,
           used by tests/test_shape.py / test_form_factors.py there) copied
           as V/F arrays into spheres.npz.
  tree     the block-tree introspection of the reference's compressed
           matrices at tol = 0 (compressed_form_factors.py:808-847:
           get_blocks_at_depth, get_row_inds_at_depth, get_row_blocks,
           get_col_inds_for_row, depth, nbytes) on the stretched octree
           sphere and the quadtree crater at depths 1-3, into tree.npz.
  vf       triangle pairs and the reference's exact view factor between
           them (src/flux/view_factor/view_factor_narayanaswamy.c, compiled
           under oracle/_ref by oracle/build.py): separated, edge- and
           vertex-sharing (from a terrain mesh) and parallel-edge pairs,
           into viewfactor.npz.
  cpuarm   the CPU baseline's 7,938-facet sample (64 x 64 fBm terrain, seed 1)
           through the reference's own form factors, insolation and Jacobi
           solves (tolerance 1e-5 max|E|): F's pattern (digest), F x and row
           sums, E of 8 directions (sums and maxima; 2 in full), their
           iteration counts and 2 solutions,
           into cpuarm.npz, with the time per solve of the reference's solve
           and of the oracle's on this machine.
  thermal  the helpers at the end of src/flux/thermal.pyx (setgrid,
           flux_noatm, analytT_; plain Python, run from the source text) on
           fixed inputs, into thermal_helpers.npz.
  ffref    form-factor matrices and steady-state solves computed by the
           reference's Python code (src/flux/form_factors.py,
           compressed_form_factors.py, solve.py, model.py), imported from the
           reference tree with the runtime shims its code needs under numpy 2
           and scipy 1.18, with visibility from the oracle's CPU ray caster
           plugged into the reference's backend seam
           (TrimeshShapeModel._get_visibility / _is_occluded).
The GPU machines have no reference tree; the tests read only these files.
"""
from __future__ import annotations

import csv
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _reference_root() -> Path:
    root = os.environ.get("FLUXPY_REFERENCE")
    if not root:
        sys.exit("make_golden.py: set FLUXPY_REFERENCE to the fluxpy reference checkout")
    path = Path(root)
    if not (path / "src" / "flux").is_dir():
        sys.exit(f"make_golden.py: FLUXPY_REFERENCE={root} holds no src/flux tree")
    return path


REF = _reference_root() if __name__ == "__main__" else None


def make_pcc():
    d = REF / "tests" / "data" / "thermal" / "pcc_thermal_model_1d"
    out = []
    for name in ("Tprofile_conductionQ", "Tsurface_conductionQ"):
        rows = []
        with open(d / name) as f:
            for row in csv.reader(f, delimiter=" ", quoting=csv.QUOTE_NONNUMERIC):
                rows.append([x for x in row if x != ""])
        out.append(np.array(rows, dtype=np.float64))
    np.savez_compressed(HERE / "pcc_conductionQ.npz", Tprofile=out[0], Tsurface=out[1])
    print("pcc:", out[0].shape, out[1].shape)


def make_spheres():
    arrs = {}
    for name in ("icosa_sphere", "icosa_sphere_5"):
        z = np.load(REF / "tests" / "data" / f"{name}.npz")
        arrs[f"{name}_V"] = z["V"]
        arrs[f"{name}_F"] = z["F"]
    np.savez_compressed(HERE / "spheres.npz", **arrs)
    print("spheres:", {k: v.shape for k, v in arrs.items()})


def import_reference():
    """Import the reference package from its source tree with the runtime
    shims its code needs here (numpy 2.x, scipy 1.18): the removed
    np.product alias, the cached_property package (stdlib equivalent), and
    the LinearOperator attributes that scipy now expects from subclasses that
    never call LinearOperator.__init__.  flux.thermal (Cython) is not built:
    a placeholder module satisfies flux.model's import."""
    import functools
    import types

    import scipy.sparse.linalg as sla
    np.product = np.prod
    sys.modules.setdefault("cached_property",
                           types.SimpleNamespace(cached_property=functools.cached_property))
    try:
        import scipy._external.array_api_compat.numpy as npc
        sla.LinearOperator._xp = npc
    except Exception:
        pass
    sla.LinearOperator.ndim = 2
    thermal = types.ModuleType("flux.thermal")
    thermal.PccThermalModel1D = None
    sys.modules["flux.thermal"] = thermal
    sys.path.insert(0, str(REF / "src"))
    import flux.compressed_form_factors as cff
    import flux.form_factors as ff
    import flux.model as model
    import flux.shape as shape
    import flux.solve as solve
    return shape, ff, cff, solve, model


def oracle_shape_class(shape_mod, sem):
    """A reference TrimeshShapeModel whose ray queries come from the oracle's
    CPU ray caster (plugged into the reference's backend seam)."""
    sys.path.insert(0, str(HERE.parent.parent))
    from oracle import vis

    class OracleShape(shape_mod.TrimeshShapeModel):
        def _make_scene(self):
            self._scene = vis.Scene(self.V, self.F)

        def _get_visibility(self, I, J):
            return self._scene.visibility(self.P, np.asarray(I, np.int64), np.asarray(J, np.int64),
                                          sem=sem)

        def _is_occluded(self, I, D):
            return self._scene.occluded(self.P, self.N, np.asarray(I, np.int64), D, sem=sem)

    return OracleShape


def make_ffref():
    """Reference Python form factors, compressed matrices and solves."""
    shape, ff, cff, solve, model = import_reference()
    sys.path.insert(0, str(HERE.parent.parent))
    from fluxpy_gb300 import terrain
    out = {}
    Shape = oracle_shape_class(shape, 0)
    # (1) inward sphere, all pairs visible (tests/test_form_factors.py:18-38)
    z = np.load(REF / "tests" / "data" / "icosa_sphere_5.npz")
    V, F = z["V"], z["F"]
    sm = Shape(V, F)
    sm.N[(sm.P * sm.N).sum(1) > 0] *= -1
    A = ff.get_form_factor_matrix(sm)
    S = A[0::4]  # every 4th row keeps the fixture small
    out.update(sphere_V=V, sphere_F=F, sphere_N=sm.N, sphere_data=S.data,
               sphere_indices=S.indices, sphere_indptr=S.indptr, sphere_nnz=A.nnz)
    # (2) the spherical crater with occlusion, Embree semantics
    V, F = terrain.spherical_crater()
    sm = Shape(V, F)
    A = ff.get_form_factor_matrix(sm)
    S = A[0::16]  # every 16th row keeps the fixture small
    out.update(crater_V=V, crater_F=F, crater_data=S.data, crater_indices=S.indices,
               crater_indptr=S.indptr, crater_nnz=A.nnz, crater_rowsum=np.asarray(A.sum(1)).ravel())
    # (3) solves on the crater (rho 0.12, emissivity 0.95, F0 1365, sun at
    # 10 degrees elevation, azimuth 0), reference Jacobi
    e0 = np.deg2rad(10.0)
    dsun = np.array([np.cos(e0), 0.0, np.sin(e0)])
    E = sm.get_direct_irradiance(1365.0, dsun)
    B, niter = solve.solve_radiosity(A, E, 0.12, "right", "jacobi")
    T = model.compute_steady_state_temp(A, E, 0.12, 0.95)
    out.update(crater_E=E, crater_B=B, crater_niter=niter, crater_T=T)
    # multi-column visible solve (E.ndim == 2 path of compute_steady_state_temp)
    dirs = terrain.sun_directions([10.0, 20.0, 5.0], [0.0, 90.0, 200.0])
    E2 = np.column_stack([sm.get_direct_irradiance(1365.0, d) for d in dirs])
    B2, niter2 = solve.solve_radiosity(A, E2, 0.12, "right", "jacobi")
    T2 = model.compute_steady_state_temp(A, E2, 0.12, 0.95)
    out.update(crater_E2=E2, crater_B2=B2, crater_niter2=niter2, crater_T2=T2)
    # (4) compressed matrices at tol=0 (tests/test_compressed_form_factors.py)
    rng = np.random.default_rng(7)
    zs = np.load(REF / "tests" / "data" / "icosa_sphere.npz")
    Vs = zs["V"] * rng.random(3)
    sms = Shape(Vs, zs["F"])
    sms.N[(sms.P * sms.N).sum(1) > 0] *= -1
    C = cff.CompressedFormFactorMatrix(sms, tol=0, max_depth=1, force_max_depth=True,
                                       RootBlock=cff.FormFactorOctreeBlock)
    x = rng.standard_normal(sms.num_faces)
    out.update(octsphere_V=Vs, octsphere_F=zs["F"], octsphere_N=sms.N, octsphere_x=x,
               octsphere_y=C @ x,
               octsphere_types=np.array([type(b).__name__ for b in C._root._blocks.ravel()]),
               octsphere_rows=np.array([len(r) for r in C._root._row_block_inds]))
    for depth in (1, 2, 3):
        Cq = cff.CompressedFormFactorMatrix(sm, tol=0, max_depth=depth, force_max_depth=False,
                                            RootBlock=cff.FormFactorQuadtreeBlock, min_size=4096)
        out[f"crater_quad{depth}_y"] = Cq @ E
        out[f"crater_quad{depth}_depth"] = Cq.depth
    np.savez_compressed(HERE / "ffref.npz", **out)
    print("ffref:", {k: getattr(v, "shape", v) for k, v in out.items()})


def _record_tree(out, p, C, rows):
    """The reference operator C's introspection answers under prefix p."""
    out[f"{p}_depth"] = C.depth
    out[f"{p}_nbytes"] = C.nbytes
    out[f"{p}_root_types"] = np.array([type(b).__name__ for b in C._root._blocks.ravel()])
    out[f"{p}_root_nbytes"] = np.array([b.nbytes for b in C._root._blocks.ravel()], np.int64)
    for d in range(C.depth + 1):
        try:
            blocks = list(C.get_blocks_at_depth(d))
        except Exception as e:
            # recorded as the exception's type (the reference's leaves lack
            # _get_blocks_at_depth, so its traversal fails at any leaf below
            # the root)
            out[f"{p}_bad{d}_error"] = np.array(type(e).__name__)
            blocks = None
        if blocks is not None:
            out[f"{p}_bad{d}_types"] = np.array([type(b).__name__ for b in blocks])
            out[f"{p}_bad{d}_shapes"] = np.array([b.shape for b in blocks],
                                                 np.int64).reshape(-1, 2)
            out[f"{p}_bad{d}_nbytes"] = np.array([b.nbytes for b in blocks], np.int64)
        sets = list(C.get_row_inds_at_depth(d))
        out[f"{p}_rid{d}"] = np.concatenate(sets).astype(np.int64)
        out[f"{p}_rid{d}_len"] = np.array([len(x) for x in sets], np.int64)
    out[f"{p}_rows"] = np.asarray(rows, np.int64)
    for i, r in enumerate(rows):
        blocks = list(C.get_row_blocks(int(r)))
        out[f"{p}_rb{i}_types"] = np.array([type(b).__name__ for b in blocks])
        out[f"{p}_rb{i}_shapes"] = np.array([b.shape for b in blocks], np.int64).reshape(-1, 2)
        sets = list(C.get_col_inds_for_row(int(r)))
        out[f"{p}_ci{i}"] = np.concatenate(sets).astype(np.int64)
        out[f"{p}_ci{i}_len"] = np.array([len(x) for x in sets], np.int64)


def make_tree():
    """Block-tree introspection of the reference's compressed matrices."""
    shape, ff, cff, solve, model = import_reference()
    sys.path.insert(0, str(HERE.parent.parent))
    from fluxpy_gb300 import terrain
    Shape = oracle_shape_class(shape, 0)
    out = {}
    # the stretched sphere of tests/test_compressed_form_factors.py:25-76
    ref = np.load(HERE / "ffref.npz")
    sms = Shape(ref["octsphere_V"], ref["octsphere_F"])
    sms.N[:] = ref["octsphere_N"]
    C = cff.CompressedFormFactorMatrix(sms, tol=0, max_depth=1, force_max_depth=True,
                                       RootBlock=cff.FormFactorOctreeBlock)
    _record_tree(out, "octsphere", C, [0, 17, 160, sms.num_faces - 1])
    V, F = terrain.spherical_crater()
    sm = Shape(V, F)
    for depth in (1, 2, 3):
        Cq = cff.CompressedFormFactorMatrix(sm, tol=0, max_depth=depth, force_max_depth=False,
                                            RootBlock=cff.FormFactorQuadtreeBlock, min_size=4096)
        _record_tree(out, f"crater_quad{depth}", Cq, [0, 1234, 2500, sm.num_faces - 1])
    np.savez_compressed(HERE / "tree.npz", **out)
    print("tree:", len(out), "arrays")


def make_vf():
    """The reference's exact triangle-triangle view factors."""
    sys.path.insert(0, str(HERE.parent.parent))
    from oracle import viewfactor as ovf
    from fluxpy_gb300 import terrain
    if ovf.ff_ref(np.eye(3), np.eye(3) + 1) is None:
        sys.exit("make_golden.py vf: build oracle/_ref first (python oracle/build.py)")
    rng = np.random.default_rng(11)
    T1, T2 = [], []
    # separated pairs: a triangle near z = 0 facing up, one near z = 1 facing down
    for _ in range(150):
        a = rng.uniform(-0.5, 0.5, (3, 3)) * [1, 1, 0.1]
        b = rng.uniform(-0.5, 0.5, (3, 3)) * [1, 1, 0.1] + [rng.uniform(-1, 1), 0, 1]
        if np.cross(a[1] - a[0], a[2] - a[0])[2] < 0:
            a = a[[0, 2, 1]]
        if np.cross(b[1] - b[0], b[2] - b[0])[2] > 0:
            b = b[[0, 2, 1]]
        T1.append(a)
        T2.append(b)
    # facets of a terrain that share an edge or a vertex
    V, F = terrain.fbm_terrain(n=12, seed=7, n_craters=1)
    shared = []
    for i in range(F.shape[0]):
        for j in range(F.shape[0]):
            k = np.intersect1d(F[i], F[j]).size
            if i != j and k in (1, 2):
                shared.append((i, j, k))
    pick = rng.choice(len(shared), 200, replace=False)
    for q in pick:
        i, j, _ = shared[q]
        T1.append(V[F[i]])
        T2.append(V[F[j]])
    # parallel edges: a triangle and a translated copy
    for _ in range(50):
        a = rng.uniform(-0.5, 0.5, (3, 3))
        T1.append(a)
        T2.append(a + rng.uniform(-1, 1, 3) + [0, 0, 2])
    T1 = np.array(T1, np.float64)
    T2 = np.array(T2, np.float64)
    Fv = np.array([ovf.ff_ref(a, b) for a, b in zip(T1, T2)])
    kind = np.array(["separated"] * 150 + ["shared_" + str(shared[q][2]) for q in pick] +
                    ["parallel"] * 50)
    np.savez_compressed(HERE / "viewfactor.npz", T1=T1, T2=T2, F=Fv, kind=kind)
    print("vf:", T1.shape, float(Fv.min()), float(Fv.max()))


def _digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_cpuarm():
    """The CPU baseline's sample computed by the reference's own Python code:
    its form factors (src/flux/form_factors.py:11-72, oracle visibility in
    the backend seam), insolation (shape.py:181-244) and Jacobi solves
    (solve.py:36-45, one direction per solve, stopping at an update of
    1e-5 max|E|), with the time each solve took here beside the oracle's
    restatement of the same solve on the same operator."""
    import time
    shape, ff, cff, solve, model = import_reference()
    sys.path.insert(0, str(HERE.parent.parent))
    from fluxpy_gb300 import terrain
    from oracle import solve as osolve
    Shape = oracle_shape_class(shape, 0)
    V, F = terrain.fbm_terrain(n=64, seed=1, n_craters=4)
    sm = Shape(V, F)
    A = ff.get_form_factor_matrix(sm).tocsr()
    dirs = terrain.random_sun_directions(64, seed=2)
    cols = list(range(0, 64, 8))
    E = np.column_stack([sm.get_direct_irradiance(1365.0, dirs[c]) for c in cols])
    niter, Bs, t_ref, t_orc = [], [], 0.0, 0.0
    for k in range(len(cols)):
        e = np.ascontiguousarray(E[:, k])
        tol = 1e-5 * float(np.abs(e).max())
        t0 = time.perf_counter()
        B, it = solve.solve_radiosity(A, e, 0.12, "right", "jacobi", tol=tol)
        t_ref += time.perf_counter() - t0
        t0 = time.perf_counter()
        Bo, ito = osolve.solve_radiosity(A, e, 0.12, tol=tol)
        t_orc += time.perf_counter() - t0
        assert ito == it and np.array_equal(Bo, B)
        niter.append(it)
        Bs.append(B)
    # the operator's pattern by digest, its values through a product with a
    # fixed vector and the row sums; B of three of the directions in full
    x = np.random.default_rng(0).uniform(0, 1, F.shape[0])
    out = dict(num_faces=F.shape[0], nnz=A.nnz,
               pattern_digest=_digest(A.indptr.astype(np.int64), A.indices.astype(np.int64)),
               x=x, Ax=A @ x, rowsum=np.asarray(A.sum(1)).ravel(), cols=np.array(cols),
               dirs=dirs, E_sum=E.sum(0), E_max=E.max(0), niter=np.array(niter),
               full_cols=np.array([0, 7]), E=E[:, [0, 7]], B=np.column_stack([Bs[0], Bs[7]]),
               seconds_reference=t_ref, seconds_oracle=t_orc)
    np.savez_compressed(HERE / "cpuarm.npz", **out)
    print("cpuarm:", F.shape[0], "facets", A.nnz, "nnz, niter", niter,
          f"reference {t_ref / len(cols) * 1e3:.1f} ms/solve, oracle {t_orc / len(cols) * 1e3:.1f}")


def thermal_helper_cases():
    """Inputs of the thermal.pyx helper goldens (shared with the test)."""
    grids = [(20, 1.08, 0.5), (40, 1.0817, 1.0), (60, 1.05, 1.0), (10, 1.0, 0.3),
             (5, 0.9, 2.0), (2, 1.2, 0.1), (3, 1.5, 0.2)]
    ha = np.linspace(-np.pi, np.pi, 13)
    flux = [(R, decl, lat, h, slope, az)
            for R in (1.0, 1.52) for decl in (-0.4, 0.0, 0.2)
            for lat in (-1.2, -0.3, 0.05, 0.5, 1.4) for h in ha
            for slope in (0.0, 0.3) for az in (0.0, 2.0)]
    analyt = dict(z=np.linspace(0.0, 0.5, 7), T0=250.0, rhoc=1.2e6, ti=100.0, P=86400.0,
                  dt=3600.0)
    return grids, np.array(flux), analyt


def make_thermal():
    """setgrid, flux_noatm and analytT_ as the reference defines them at the
    end of src/flux/thermal.pyx (plain Python after the Cython class, so
    they run here without building the extension)."""
    src = (REF / "src" / "flux" / "thermal.pyx").read_text()
    ns = {"np": np}
    exec(compile(src[src.index("\ndef setgrid("):], "thermal.pyx", "exec"), ns)
    grids, flux, analyt = thermal_helper_cases()
    z = [ns["setgrid"](*g) for g in grids]
    F = np.array([ns["flux_noatm"](*row) for row in flux])
    T = ns["analytT_"](**analyt)
    np.savez_compressed(HERE / "thermal_helpers.npz", setgrid=np.concatenate(z),
                        setgrid_len=np.array([len(a) for a in z]), flux_noatm=F, analytT=T)
    print("thermal:", len(z), "grids,", F.size, "fluxes, analytT", T.shape)


SECTIONS = {"pcc": make_pcc, "spheres": make_spheres, "ffref": make_ffref, "tree": make_tree,
            "vf": make_vf, "cpuarm": make_cpuarm, "thermal": make_thermal}

if __name__ == "__main__":
    todo = sys.argv[1:] or list(SECTIONS)
    for s in todo:
        SECTIONS[s]()
