/*
 * fluxgb — C ABI of the GB300 (sm_103a) radiosity / thermal hot path.
 *
 * Conventions
 *   - Every function returns an fgb_status (0 = FGB_OK). On failure the
 *     message is available from fgb_last_error() on the same host thread.
 *   - All array arguments are DEVICE pointers (allocated by the caller, e.g.
 *     as torch tensors or with cudaMalloc), C-contiguous, with the element
 *     type in the function name.  Sizes are plain integers.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream).  Calls are asynchronous with respect to the host unless the
 *     comment says otherwise; device-side error flags are OR-ed into a
 *     caller-provided `unsigned* flags` word (FGB_FLAG_*) that the caller
 *     reads after synchronising.
 *   - No torch or C++ types cross this boundary.
 *
 * Each declaration names the reference interface it replaces
 * (paths inside the fluxpy source tree, file:line).
 */
#ifndef FLUXGB_H
#define FLUXGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum fgb_status {
  FGB_OK = 0,
  FGB_BAD_ARG = 1,        /* invalid size / argument (reference: ValueError) */
  FGB_NONFINITE = 2,      /* non-finite input or output (RuntimeError)       */
  FGB_NEGATIVE = 3,       /* negative flux / temperature (RuntimeError)      */
  FGB_ZERO_PIVOT = 4,     /* tridiagonal zero pivot (tridag.c:14-26 exit(1)) */
  FGB_NO_CONVERGENCE = 5, /* iteration cap reached (solve.py has no cap)     */
  FGB_DEVICE_TIMEOUT = 6, /* a bounded device-side wait gave up              */
  FGB_CUDA_ERR = 7,       /* CUDA runtime error                              */
  FGB_NO_MEMORY = 8,      /* device allocation failed                        */
  FGB_TOO_LARGE = 9       /* request exceeds a documented fixed capacity     */
};

/* device-side flag bits (OR-ed into *flags) */
#define FGB_FLAG_NONFINITE_IN   (1u << 0)
#define FGB_FLAG_NEGATIVE_IN    (1u << 1)
#define FGB_FLAG_NONFINITE_OUT  (1u << 2)
#define FGB_FLAG_NEGATIVE_OUT   (1u << 3)
#define FGB_FLAG_ZERO_PIVOT     (1u << 4)
#define FGB_FLAG_PREDCORR_MAX   (1u << 5) /* conductionQ.c:173 warning      */
#define FGB_FLAG_STACK_OVERFLOW (1u << 6) /* BVH traversal stack exhausted  */
#define FGB_FLAG_INDEX_RANGE    (1u << 7)
#define FGB_FLAG_RANK_CAP       (1u << 8) /* ACA reached its rank cap       */
#define FGB_FLAG_DEVICE_TIMEOUT (1u << 9) /* a bounded device-side wait ran out */
#define FGB_FLAG_NO_CONVERGE    (1u << 10) /* a Jacobi eigen solve hit its sweep cap */

/* Message of the last failed call on this host thread ("" if none). */
const char* fgb_last_error(void);
/* Library version string. */
const char* fgb_version(void);
/* Number of kernels this library has launched in the process so far. */
long long fgb_launch_count(void);

/* ------------------------------------------------ 1-D conduction (a14) */
/*
 * One Crank-Nicolson step of the radiative-flux boundary problem for every
 * facet.  Replaces the per-facet loop over
 *   void conductionQ(int nz, double z[], double dt, double Qn, double Qnp1,
 *                    double T[], double ti[], double rhoc[], double emiss,
 *                    double Fgeotherm, double *Fsurf)
 * (src/flux/pcc/thrmlLib.h:3-4, src/flux/pcc/conductionQ.c:10) as driven by
 * PccThermalModel1D.step (src/flux/thermal.pyx:249-261).
 *   z[0..nz], ti[0..nz], rhoc[0..nz]  per-layer, shared by all facets
 *   Qn, Qnp1, emiss, Fgeotherm, Fsurf[num_faces]
 *   T_in, T_out[num_faces * (nz+1)]   row-major; may alias (in place)
 */
int fgb_conduction_q_f64(int num_faces, int nz, const double* z, double dt,
                         const double* Qn, const double* Qnp1, const double* T_in,
                         double* T_out, const double* ti, const double* rhoc,
                         const double* emiss, const double* Fgeotherm, double* Fsurf,
                         unsigned* flags, void* stream);
/* Same in FP32 (used by the FP32 time-stepping driver): the same equations,
 * eliminated from the bottom up, so that the predictor-corrector redos of
 * the radiative boundary re-solve only the surface row (the same solution in
 * exact arithmetic; results within FP32 rounding of the FP64 entry point). */
int fgb_conduction_q_f32(int num_faces, int nz, const float* z, float dt, const float* Qn,
                         const float* Qnp1, const float* T_in, float* T_out,
                         const float* ti, const float* rhoc, const float* emiss,
                         const float* Fgeotherm, float* Fsurf, unsigned* flags,
                         void* stream);
/*
 * Prescribed-surface-temperature step.  Replaces the per-facet loop over
 *   void conductionT(int nz, double z[], double dt, double T[], double Tsurf,
 *                    double Tsurfp1, double ti[], double rhoc[],
 *                    double Fgeotherm, double *Fsurf)
 * (src/flux/pcc/thrmlLib.h:6-8, conductionT.c:4; thermal.pyx:275-286).
 */
int fgb_conduction_t_f64(int num_faces, int nz, const double* z, double dt,
                         const double* Tsurf, const double* Tsurfp1, const double* T_in,
                         double* T_out, const double* ti, const double* rhoc,
                         const double* Fgeotherm, double* Fsurf, unsigned* flags,
                         void* stream);

/*
 * conductionQ (src/flux/pcc/conductionQ.c:10-186) for every facet with the
 * thermal inertia given per facet and layer: ti is num_faces x (nz+1) with
 * row stride ti_ld = nz + 1, or one shared profile with ti_ld = 0 (then the
 * result is bit-identical to fgb_conduction_q_f64).  The reference takes one
 * ti profile for all facets (thermal.pyx:89-156); per-facet thermal inertia
 * is what the differentiable model fits.  nz <= 127.  No Fsurf output.
 */
int fgb_conduction_q_ti_f64(int num_faces, int nz, const double* z, double dt,
                            const double* Qn, const double* Qnp1, const double* T_in,
                            double* T_out, const double* ti, long long ti_ld,
                            const double* rhoc, const double* emiss, const double* Fgeotherm,
                            unsigned* flags, void* stream);
/*
 * Reverse-mode derivative of fgb_conduction_q_ti_f64 (no reference
 * counterpart: the reference has no derivatives).  Given the cotangent
 * gT_out of the new profiles (num_faces x (nz+1)), writes the cotangents of
 * the pre-step profiles gT_in (may alias gT_out), of Qn and Qnp1, and ADDS
 * those of emiss (num_faces) and of ti (num_faces x (nz+1), row stride
 * nz+1, column 0 untouched) into gemiss and gti.  The step's
 * predictor-corrector passes are replayed and differentiated exactly.
 */
int fgb_conduction_q_adjoint_f64(int num_faces, int nz, const double* z, double dt,
                                 const double* Qn, const double* Qnp1, const double* T_in,
                                 const double* ti, long long ti_ld, const double* rhoc,
                                 const double* emiss, const double* Fgeotherm,
                                 const double* gT_out, double* gT_in, double* gQn,
                                 double* gQnp1, double* gemiss, double* gti, unsigned* flags,
                                 void* stream);

/* ---------------------------------------------- facet geometry (a1) */
/*
 * Centroids P (nf x 3), unit normals N (nf x 3) and areas A (nf) of a mesh
 * with vertices V (nv x 3) and faces F (nf x 3, int64), bit-identical to
 * numpy's get_centroids / get_surface_normals_and_face_areas
 * (src/flux/shape.py:16-45) as called by TrimeshShapeModel.__init__
 * (shape.py:92-106).  Any of P, N, A may be NULL.
 */
int fgb_facet_geometry_f64(const double* V, long long nv, const long long* F, long long nf,
                           double* P, double* N, double* A, unsigned* flags, void* stream);
int fgb_facet_geometry_f32(const float* V, long long nv, const long long* F, long long nf,
                           float* P, float* N, float* A, unsigned* flags, void* stream);

/* ------------------------------------------------------- LBVH (a2) */
/*
 * Build a linear BVH over the triangles (FP32 vertices as Embree stores
 * them; keep_f64 also keeps FP64 vertices for CGAL semantics).  Replaces
 * EmbreeTrimeshShapeModel._make_scene (src/flux/shape.py:296-344) and
 *   void cgal_aabb_init_from_trimesh(cgal_aabb *aabb, size_t num_points,
 *        double (*points)[3], size_t num_faces, size_t (*faces)[3])
 * (src/flux/cgal/aabb_wrapper.h:8-10).  *out_bvh receives an opaque handle
 * owned by the library (device memory), released by fgb_bvh_free
 * (cgal_aabb_dealloc, aabb_wrapper.h:11).  Synchronous allocation; the build
 * itself runs on `stream`.
 */
int fgb_bvh_build_f64(const double* V, long long nv, const long long* F, long long nf,
                      int keep_f64, void** out_bvh, unsigned* flags, void* stream);
int fgb_bvh_build_f32(const float* V, long long nv, const long long* F, long long nf,
                      int keep_f64, void** out_bvh, unsigned* flags, void* stream);
int fgb_bvh_free(void* bvh);
int fgb_bvh_info(const void* bvh, long long* num_prims, long long* bytes);

/* ------------------------------------------- ray queries (a3, a4) */
/* semantics: 0 = Embree backend (shape.py:349-421), 1 = CGAL backend
 * (aabb_wrapper.cpp:64-108). */
/*
 * Pair visibility.  paired == 0: vis[p*n+q] for (I[p], J[q]) (m x n), as
 * TrimeshShapeModel.get_visibility / _get_visibility (shape.py:138-163,
 * 272-281, 349-398) and
 *   bool cgal_aabb_test_face_to_face_vis(cgal_aabb const *aabb, size_t i, size_t j)
 * (aabb_wrapper.h:12).  paired != 0: vis[k] for (I[k], J[k]).  near_edge
 * (optional) flags rays that passed within 1e-6 (relative) of an edge.
 */
int fgb_visibility_f64(const void* bvh, const double* P, long long num_faces, const long long* I,
                       long long m, const long long* J, long long n, int paired, int semantics,
                       unsigned char* vis, unsigned char* near_edge, unsigned* flags, void* stream);
int fgb_visibility_f32(const void* bvh, const float* P, long long num_faces, const long long* I,
                       long long m, const long long* J, long long n, int paired, int semantics,
                       unsigned char* vis, unsigned char* near_edge, unsigned* flags, void* stream);
/*
 * Sun occlusion of facets I along directions D.  per_facet == 0: D holds
 * ndirs directions and occluded[p*ndirs+k] is written; per_facet != 0: D is
 * m x 3, one direction per facet.  Replaces TrimeshShapeModel.is_occluded
 * (shape.py:181-188, 283-292, 400-421) and
 *   bool cgal_aabb_ray_from_centroid_is_occluded(cgal_aabb const *aabb, size_t i, double d[3])
 * (aabb_wrapper.h:13-14).
 */
int fgb_occluded_f64(const void* bvh, const double* P, const double* N, long long num_faces,
                     const long long* I, long long m, const double* D, long long ndirs,
                     int per_facet, int semantics, unsigned char* occluded, unsigned* flags,
                     void* stream);
int fgb_occluded_f32(const void* bvh, const float* P, const float* N, long long num_faces,
                     const long long* I, long long m, const float* D, long long ndirs,
                     int per_facet, int semantics, unsigned char* occluded, unsigned* flags,
                     void* stream);
/*
 * Direct irradiance for K sun directions: E[i*K+k] = F0[k] max(0, N_i.d_k)
 * if facet i sees the sun along d_k, else 0 — get_direct_irradiance
 * (shape.py:190-226) for every column at once.
 */
int fgb_direct_irradiance_f64(const void* bvh, const double* P, const double* N,
                              long long num_faces, const double* D, long long K, const double* F0,
                              int semantics, double* E, unsigned* flags, void* stream);
int fgb_direct_irradiance_f64_to_f32(const void* bvh, const double* P, const double* N,
                                     long long num_faces, const double* D, long long K,
                                     const double* F0, int semantics, float* E, unsigned* flags,
                                     void* stream);
int fgb_direct_irradiance_f32(const void* bvh, const float* P, const float* N, long long num_faces,
                              const float* D, long long K, const float* F0, int semantics,
                              float* E, unsigned* flags, void* stream);
/*
 * First intersection of FP64 rays (X[p], D[p]): hit[p] = facet id or -1,
 * xt[p] = hit point.  Replaces
 *   bool cgal_aabb_intersect1(cgal_aabb const *aabb, double const x[3],
 *        double const d[3], size_t *i, double xt[3])
 * (aabb_wrapper.h:15-16; CgalTrimeshShapeModel._intersect1, shape.py:269).
 * Needs a BVH built with keep_f64.
 */
int fgb_intersect1_f64(const void* bvh, const double* X, const double* D, long long m,
                       long long* hit, double* xt, unsigned* flags, void* stream);

/* --------------------------------------- form-factor pair kernel (a5) */
/*
 * Two-pass CSR assembly of form factors for a list of tiles (tile t: rows
 * I[row0[t] .. +nrows[t]), columns J[col0[t] .. +ncols[t])).  Replaces the
 * row loop of get_form_factor_matrix (src/flux/form_factors.py:11-72).
 *   word_off[T+1]: exclusive prefix of nrows*ceil(ncols/32); row_off[T+1]:
 *   exclusive prefix of nrows.
 * fgb_ff_count_*: bits[total_words] (visible-and-kept bitmask),
 *   row_counts[total_rows] (must be zeroed), stats[0] += kept pairs,
 *   stats[1] += near-edge pairs.
 * The caller scans row_counts into indptr[total_rows+1] (int64), then
 * fgb_ff_fill_* writes indices (column position within the tile, int32) and
 * data.
 */
int fgb_ff_count_f64(const void* bvh, const double* P, const double* N, const double* A,
                     const long long* I, const long long* J, const long long* row0,
                     const long long* nrows, const long long* col0, const long long* ncols,
                     const long long* word_off, const long long* row_off, long long num_tiles,
                     long long total_words, double eps, int semantics, unsigned* bits,
                     int* row_counts, unsigned long long* stats, unsigned* flags, void* stream);
int fgb_ff_count_f32(const void* bvh, const float* P, const float* N, const float* A,
                     const long long* I, const long long* J, const long long* row0,
                     const long long* nrows, const long long* col0, const long long* ncols,
                     const long long* word_off, const long long* row_off, long long num_tiles,
                     long long total_words, float eps, int semantics, unsigned* bits,
                     int* row_counts, unsigned long long* stats, unsigned* flags, void* stream);
int fgb_ff_fill_f64(const double* P, const double* N, const double* A, const long long* I,
                    const long long* J, const long long* row0, const long long* nrows,
                    const long long* col0, const long long* ncols, const long long* word_off,
                    const long long* row_off, long long num_tiles, long long total_rows,
                    const unsigned* bits, const long long* indptr, int* indices, double* data,
                    void* stream);
int fgb_ff_fill_f64_to_f32(const double* P, const double* N, const double* A, const long long* I,
                           const long long* J, const long long* row0, const long long* nrows,
                           const long long* col0, const long long* ncols,
                           const long long* word_off, const long long* row_off,
                           long long num_tiles, long long total_rows, const unsigned* bits,
                           const long long* indptr, int* indices, float* data, void* stream);
int fgb_ff_fill_f32(const float* P, const float* N, const float* A, const long long* I,
                    const long long* J, const long long* row0, const long long* nrows,
                    const long long* col0, const long long* ncols, const long long* word_off,
                    const long long* row_off, long long num_tiles, long long total_rows,
                    const unsigned* bits, const long long* indptr, int* indices, float* data,
                    void* stream);

/* ------------------------------------------- compression (a6-a8) */
/*
 * Batched adaptive cross approximation of admissible blocks.  Replaces the
 * rank estimation of the reference's compressed matrix,
 *   estimate_rank(spmat, tol, max_nbytes=None, k0=40) / sparse_svd(spmat, k)
 * (src/flux/linalg.py:8-51) called from FormFactorBlockMatrix._get_svd_block
 * (src/flux/compressed_form_factors.py:388-405), which needs every entry of
 * the block; ACA evaluates O(k (m+n)) entries (with their rays).
 * Block b covers cluster-order rows [r0, r0+m) and columns [c0, c0+n); perm
 * maps cluster order to facet ids.  Outputs rank_out[b] (-1: did not
 * converge under its cap, -2: pool full) and off_out[b]: offset in `pool`
 * of U^T (k x m) followed by V^T (k x n).  scratch: num_ctas *
 * fgb_aca_scratch_floats(...) floats; queue: one zeroed int.  Blocks with
 * m*n <= exact_max are evaluated in full into dense_scratch (num_ctas *
 * exact_max floats) and approximated with full pivoting on the exact
 * residual; larger blocks use partial pivoting with the residual norm
 * estimated from nsample random entries.
 */
int fgb_aca_scratch_floats(int rmax, long long mmax, long long nmax, long long* per_cta);
int fgb_aca_f64(const void* bvh, const double* P, const double* N, const double* A,
                const long long* perm, long long nblocks, const int* r0, const int* m,
                const int* c0, const int* n, long long mmax, long long nmax, double eps,
                int semantics, float tol, int rmax, int nsample, long long exact_max,
                float* dense_scratch, float* scratch, int num_ctas,
                float* pool, long long pool_capacity, unsigned long long* pool_used,
                int* rank_out, long long* off_out, int* queue, unsigned* flags, void* stream);
/*
 * fgb_aca_f64 without caller-provided scratch (no reference counterpart),
 * for callers that cannot allocate device memory: a host whose memory is
 * managed by its own pool or fixed budget, or code that issues the call
 * inside a region where cudaMalloc is not allowed or too slow.  The factor
 * scratch, the dense-block scratch and the work queue live in the
 * library's static device memory (32 MiB of floats per device).  The first
 * call on a device looks up its address with cudaGetSymbolAddress; make
 * that first call before any stream capture.  The address is kept for the
 * life of the CUDA context it was looked up in: after cudaDeviceReset the
 * next call (the first one in the new context) looks it up again.  The call
 * allocates nothing.
 * A call whose num_ctas * (fgb_aca_scratch_floats(...) + exact_max) floats
 * exceed that returns FGB_BAD_ARG with the sizes in fgb_last_error().  The
 * queue is zeroed by the call (cudaMemsetAsync on `stream`); *pool_used
 * must be zero on entry, as for fgb_aca_f64.  The static scratch is shared
 * by every call on a device and keeps the last call's contents: calls that
 * overlap on the GPU race, so issue them on one stream or synchronise
 * between streams / host threads.
 */
int fgb_aca_f64_static(const void* bvh, const double* P, const double* N, const double* A,
                       const long long* perm, long long nblocks, const int* r0, const int* m,
                       const int* c0, const int* n, long long mmax, long long nmax, double eps,
                       int semantics, float tol, int rmax, int nsample, long long exact_max,
                       int num_ctas, float* pool, long long pool_capacity,
                       unsigned long long* pool_used, int* rank_out, long long* off_out,
                       unsigned* flags, void* stream);
/*
 * Rank truncation of low-rank factors in FP64, replacing the reference's SVD
 * truncation of a block (src/flux/linalg.py:20-51, estimate_rank, applied by
 * FormFactor2dTreeBlock._get_svd_block, compressed_form_factors.py:388-405:
 * keep the singular values with sigma_i / sigma_0 > tol).
 * Block b holds U^T (k x m) then V^T (k x n) at pool_in + off_in[b], FP32,
 * k = rank_in[b].  The singular values of U V^T come from the FP64 Gram
 * matrices of U and V (Jacobi eigen-decompositions, no block formed); the
 * truncated factors U'^T (r x m) then V'^T (r x n) (U' orthogonal columns
 * scaled by sigma, V' orthonormal) are written to pool_out at off_out[b]
 * (bump allocator *pool_used, zero on entry; pool_capacity floats), with
 * r in rank_out[b].  Blocks of rank 0 or 1 are copied, blocks of rank above
 * 64 copied with FGB_FLAG_INDEX_RANGE, negative ranks passed through.  A full
 * pool gives rank -2 and FGB_FLAG_RANK_CAP; an eigen solve that hit its sweep
 * cap sets FGB_FLAG_NO_CONVERGE.  queue: two zeroed ints.
 */
int fgb_recompress_f32(const float* pool_in, const long long* off_in, const int* rank_in,
                       const int* m, const int* n, long long nblocks, float tol, float* pool_out,
                       long long pool_capacity, unsigned long long* pool_used, int* rank_out,
                       long long* off_out, int* queue, unsigned* flags, void* stream);

/* ------------------------------------- exact triangle view factor (f4) */
/*
 * View factor of triangle tri1[q] towards tri2[q] for q < n (each 3 x 3
 * FP64, one vertex per row), the closed form of Narayanaswamy (2015) for two
 * mutually visible planar triangles.  Replaces
 *   double ff_narayanaswamy_impl(double const tri1[3][3], double const tri2[3][3])
 * (src/flux/view_factor/view_factor.h:3, view_factor_narayanaswamy.c:338),
 * bound as flux.view_factor.ff_narayanaswamy (view_factor.pyx:5-7).  A
 * non-finite result sets FGB_FLAG_NONFINITE_OUT (the reference asserts).
 */
int fgb_ff_triangles_f64(const double* tri1, const double* tri2, long long n, double* out,
                         unsigned* flags, void* stream);
/*
 * Near-field correction of a form-factor CSR (an addition; the reference
 * keeps the midpoint rule of form_factors.py:62-64 for every pair): row r
 * is facet rows[r], entry e of it is facet cols[indices[e]] (indptr int64,
 * indices int32); entries whose two facets share a vertex (V: vertices x 3
 * FP64, F: faces x 3 int64) are replaced by the exact view factor.  The
 * number of replaced entries is added to *fixed.
 */
int fgb_ff_adjacent_fix_f64(const double* V, const long long* F, const long long* rows,
                            const long long* cols, long long nrows, const long long* indptr,
                            const int* indices, double* data, unsigned long long* fixed,
                            unsigned* flags, void* stream);

/* ----------------------------------------------- block matvec (a9) */
/*
 * Flat description of a compressed operator in cluster order (device
 * arrays; layout in fluxpy_gb300/csrc/matvec.cu):
 *   phase A groups g (low-rank blocks sharing a column range): g_c0, g_n,
 *     g_kz (stacked rank), g_ldv (panel row stride, n rounded up to 8),
 *     g_voff (panel offset), g_z0 (first Z row); work items a_grp, a_j0,
 *     a_j1, a_excl (1: the item covers its whole group);
 *   phase B row tiles of 64 rows: t_p0[num_tiles+1] panel-row offsets (each
 *     tile a multiple of 64 rows), src[row] = source row (< num_zrows: a row
 *     of Z; else a row of X at src - num_zrows);
 *   tensor-core phase A: the transposed BF16 phase-A panel holds group g as
 *     n x g_kzp (g_kz rounded up to 128) at g_vtoff, element (r, j) at
 *     g_vtoff + j g_kzp + r; a_woff[num_items + 1]: first work slice of each
 *     item, num_work = a_woff[num_items].  The CUDA-core kernels take 64-row
 *     slices (ceil(g_kz / 64) per item); the tensor-core phase A takes
 *     128-row slices (g_kzp / 128 per item): it is called with a descriptor
 *     whose a_woff / num_work count those.
 */
struct fgb_op_desc {
  const int* g_c0;
  const int* g_n;
  const int* g_kz;
  const int* g_ldv;
  const long long* g_voff;
  const long long* g_z0;
  const int* a_grp;
  const int* a_j0;
  const int* a_j1;
  const unsigned char* a_excl;
  long long num_items;
  const long long* t_p0;
  const int* src;
  long long num_tiles;
  long long N;
  long long num_zrows;
  int max_group_tiles; /* max over groups of ceil(g_kz / 64) */
  const int* g_kzp;
  const long long* g_vtoff;
  const long long* a_woff;
  long long num_work;   /* a_woff[num_items] */
  long long panel_rows; /* t_p0[num_tiles] */
  int tile_rows;        /* rows per phase-B tile: 64 (every kernel), or 128
                           or 256 (tensor-core BF16 phase B only; 256: plain
                           products); 0 means 64 */
  int slice_rows;       /* rows per tensor-core phase-A work slice (a_woff
                           counts slices of this height): 128, or 64 for the
                           split products of fgb_tc_phase_a_bf16; 0 means 128 */
  const int* a_witem;   /* optional, num_work entries: the item of each
                           tensor-core phase-A work slice (the i with
                           a_woff[i] <= slice < a_woff[i+1]); null: found by
                           binary search over a_woff */
  const int* tile_order; /* optional, num_tiles entries (tensor-core phase B):
                           the order in which the CTAs take the tiles (a
                           permutation of 0 .. num_tiles - 1); null: in
                           order */
};
/*
 * y = F x (or y = add + alpha F x), vectors in cluster order.  Replaces
 * CompressedFormFactorMatrix._matmat (src/flux/compressed_form_factors.py:805)
 * and the recursive FormFactorBlockMatrix._matmat (:407-414) with its leaf
 * products (dense :175, CSR :193, SVD :247-251).  panel / vpanel: the
 * phase-B and phase-A panels in the function's precision; z: num_zrows
 * scratch (zeroed here when zero_z != 0, needed when some a_excl == 0).
 */
int fgb_matvec_f32(const struct fgb_op_desc* d, const float* panel, const float* vpanel,
                   const float* x, float* z, float* y, const float* add, float alpha, int zero_z,
                   void* stream);
int fgb_matvec_f64(const struct fgb_op_desc* d, const double* panel, const double* vpanel,
                   const double* x, double* z, double* y, const double* add, double alpha,
                   int zero_z, void* stream);
/* FP32 panels with FP64 vectors and FP64 accumulation (residual checks of the
 * stored FP32 operator in FP64 arithmetic). */
int fgb_matvec_f32_f64(const struct fgb_op_desc* d, const float* panel, const float* vpanel,
                       const double* x, double* z, double* y, const double* add, double alpha,
                       int zero_z, void* stream);
/*
 * Transpose product y -> F^T y of the compressed operator in cluster order
 * (the x @ F of CompressedKernelMatrix._rmatvec,
 * src/flux/compressed_form_factors.py:904-913; the reference computes it for
 * sparse / dense F only).  FP64 vectors and accumulation, panels in FP64 or
 * FP32 (64-row phase-B panel).  work: num_zrows + N doubles, zeroed here;
 * the result is work[num_zrows .. num_zrows + N).  Sums are formed with FP64
 * atomics, so the last bits may differ between calls.
 */
int fgb_rmatvec_f64(const struct fgb_op_desc* d, const double* panel, const double* vpanel,
                    const double* y, double* work, unsigned* flags, void* stream);
int fgb_rmatvec_f32_f64(const struct fgb_op_desc* d, const float* panel, const float* vpanel,
                        const double* y, double* work, unsigned* flags, void* stream);
/* K right-hand sides (X, Y, add: N x K row-major; Z: num_zrows x K):
 * FP32 CUDA cores ...  phases: 1 = phase A only, 2 = phase B only, 3 = both. */
int fgb_matmat_f32(const struct fgb_op_desc* d, const float* panel, const float* vpanel,
                   const float* X, float* Z, float* Y, int K, const float* add, float alpha,
                   int zero_z, int phases, void* stream);
/* ... the FP32-stored operator (64-row panel) in FP64 arithmetic: X, Z, Y,
 * add FP64 (FP64 residuals of K columns; both phases). */
int fgb_matmat_f32_f64(const struct fgb_op_desc* d, const float* panel, const float* vpanel,
                       const double* X, double* Z, double* Y, int K, const double* add,
                       double alpha, int zero_z, void* stream);
/* ... and BF16 tensor cores with FP32 accumulation (X, panels bf16, K % 8 == 0;
 * Zb: num_zrows x K bf16 scratch). */
int fgb_matmat_bf16(const struct fgb_op_desc* d, const void* panel, const void* vpanel,
                    const void* X, float* Z, void* Zb, float* Y, int K, const float* add,
                    float alpha, int zero_z, int phases, void* stream);
/*
 * The two phases on the tcgen05 tensor cores (TMEM accumulators, FP32), BF16
 * operands, K % 8 == 0, all matrices row stride K.  With the *_lo operands
 * NULL the product is the plain BF16 one; with them, every FP32 operand is
 * given as hi = bf16(v), lo = bf16(v - hi) and the product is
 * hi.hi + hi.lo + lo.hi ("split BF16": relative error per product term
 * about 2^-16 instead of 2^-8).  Bounded device waits: a wait that runs out
 * sets FGB_FLAG_DEVICE_TIMEOUT in *flags.
 *   phase A: Z = Vg^T-panel x X rows (Z FP32, num_zrows x K; items that do
 *            not cover their group accumulate atomically into a zeroed Z);
 *   phase B: Y = add + alpha * (panel rows x gathered [Z; X] rows).
 */
int fgb_tc_phase_a(const struct fgb_op_desc* d, const void* vt_hi, const void* vt_lo,
                   const void* X_hi, const void* X_lo, float* Z, int K, int zero_z,
                   unsigned* flags, void* stream);
/* Phase A writing Z directly as BF16 (Z_hi = bf16(z), and with the split
 * operands Z_lo = bf16(z - Z_hi)), num_zrows x K each: for a descriptor whose
 * work items all cover their whole group (a_excl == 1; an item that does not
 * is skipped and flagged FGB_FLAG_INDEX_RANGE).  Split products may take
 * 64-row work slices (slice_rows = 64: two CTAs per SM). */
int fgb_tc_phase_a_bf16(const struct fgb_op_desc* d, const void* vt_hi, const void* vt_lo,
                        const void* X_hi, const void* X_lo, void* Z_hi, void* Z_lo, int K,
                        unsigned* flags, void* stream);
int fgb_tc_phase_b(const struct fgb_op_desc* d, const void* w_hi, const void* w_lo,
                   const void* X_hi, const void* X_lo, const void* Z_hi, const void* Z_lo,
                   float* Y, int K, const float* add, float alpha, unsigned* flags,
                   void* stream);
/* Phase B with the sources stacked in one (num_zrows + N) x K tensor S = [Z; X]
 * (and S_lo for split products), rows gathered by TMA (tile::gather4, four
 * 128-byte lines per request) in a warp-specialised kernel.  Same results as
 * fgb_tc_phase_b for plain products (split ones drain their FP32 windows
 * after 64 rows instead of 256: equal to FP32 rounding); slower on GB300 for
 * these 128-byte row pieces than the cp.async gathers (per-request cost),
 * kept as the TMA variant. */
int fgb_tc_phase_b_tma(const struct fgb_op_desc* d, const void* w_hi, const void* w_lo,
                       const void* S_hi, const void* S_lo, float* Y, int K, const float* add,
                       float alpha, unsigned* flags, void* stream);
/* 128-row phase-B panel (BF16) from the 64-row FP32 one: old row r goes to
 * half half[r] (0/1) of new row new_row[r] (skipped when < 0); panel128 must
 * be zeroed.  With a descriptor of tile_rows = 128, fgb_tc_phase_b computes
 * 128 output rows per CTA, so each gathered source row feeds twice the
 * flops. */
int fgb_retile_panel_bf16(const float* panel64, long long num_rows, const long long* new_row,
                          const unsigned char* half, void* panel128, void* stream);
/* The same for tiles of `width` rows (128 or 256): old row r goes to part
 * part[r] (its 64-row tile's position in the wider tile) of new row
 * new_row[r]; out (width BF16 weights per row) must be zeroed.  A descriptor
 * with tile_rows = 256 gives fgb_tc_phase_b's plain product 256 output rows
 * per CTA (MMA N = 256). */
int fgb_retile_panel_bf16_n(const float* panel64, long long num_rows, const long long* new_row,
                            const unsigned char* part, int width, void* out, void* stream);
/* The same for split products: hi128 = bf16(w), lo128 = bf16(w - hi), both
 * zeroed by the caller (fgb_tc_phase_b takes them with tile_rows = 128). */
int fgb_retile_panel_split_bf16(const float* panel64, long long num_rows,
                                const long long* new_row, const unsigned char* half,
                                void* hi128, void* lo128, void* stream);
/* hi = bf16(in), lo = bf16(in - hi) elementwise (lo may be NULL). */
int fgb_split_bf16(const float* in, void* hi, void* lo, long long n, void* stream);
/* Transposed BF16 phase-A panel from the FP32 one (layouts in fgb_op_desc);
 * tiles: (group, 64-row slice, 64-column block) triples, num_tiles of them. */
int fgb_vpanel_transpose_bf16(const struct fgb_op_desc* d, const float* vpanel,
                              const int* tile_g, const int* tile_s, const int* tile_j,
                              long long num_tiles, void* vt_hi, void* vt_lo, void* stream);
/*
 * Panel construction (setup).  Phase B: pairs q (tile, contributing block)
 * with pair_p0 (first panel row, sorted), pair_w (pool offset of the block's
 * weight row 0), pair_m (weight row length = block rows), pair_shift (tile
 * first row - block first row), pair_k (weight rows; panel rows beyond it
 * are zero padding).  Phase A: one stacked row per (row_src pool offset,
 * row_dst panel offset, row_n length).  Suffix: pool type _ panel type.
 */
int fgb_build_panel_f32_f32(const float* pool, long long num_rows, const long long* pair_p0,
                          const long long* pair_w, const int* pair_m, const long long* pair_shift,
                          const int* pair_k, long long num_pairs, void* panel, void* stream);
int fgb_build_panel_f32_bf16(const float* pool, long long num_rows, const long long* pair_p0,
                          const long long* pair_w, const int* pair_m, const long long* pair_shift,
                          const int* pair_k, long long num_pairs, void* panel, void* stream);
int fgb_build_panel_f64_f64(const double* pool, long long num_rows, const long long* pair_p0,
                          const long long* pair_w, const int* pair_m, const long long* pair_shift,
                          const int* pair_k, long long num_pairs, void* panel, void* stream);
int fgb_build_panel_f64_f32(const double* pool, long long num_rows, const long long* pair_p0,
                          const long long* pair_w, const int* pair_m, const long long* pair_shift,
                          const int* pair_k, long long num_pairs, void* panel, void* stream);
int fgb_build_panel_f64_bf16(const double* pool, long long num_rows, const long long* pair_p0,
                          const long long* pair_w, const int* pair_m, const long long* pair_shift,
                          const int* pair_k, long long num_pairs, void* panel, void* stream);
int fgb_build_vpanel_f32_f32(const float* pool, long long num_rows, const long long* row_src,
                           const long long* row_dst, const int* row_n, void* vpanel, void* stream);
int fgb_build_vpanel_f32_bf16(const float* pool, long long num_rows, const long long* row_src,
                           const long long* row_dst, const int* row_n, void* vpanel, void* stream);
int fgb_build_vpanel_f64_f64(const double* pool, long long num_rows, const long long* row_src,
                           const long long* row_dst, const int* row_n, void* vpanel, void* stream);
int fgb_build_vpanel_f64_f32(const double* pool, long long num_rows, const long long* row_src,
                           const long long* row_dst, const int* row_n, void* vpanel, void* stream);
int fgb_build_vpanel_f64_bf16(const double* pool, long long num_rows, const long long* row_src,
                           const long long* row_dst, const int* row_n, void* vpanel, void* stream);


/* ------------------------------------------ near-field panels (a7, a9) */
/*
 * Column-compacted phase-B panel rows of the exact leaves, built from the
 * pair kernel's bitmask and CSR (fgb_ff_count_* / fgb_ff_fill_*) — the exact
 * counterpart of the reference's dense / CSR leaf blocks
 * (src/flux/compressed_form_factors.py:151-229, chosen at :330-341).  Pair p
 * = (64-row tile starting at pair_t0[p], exact leaf pair_q[p]); leaves give
 * their first cluster row, rows, mask words per row and offsets into the
 * bitmask / CSR.  fgb_nf_pair_masks ORs the tile's row masks (count[p] must
 * be zeroed); fgb_nf_enumerate writes one (pair, column) descriptor per set
 * bit from desc_off[p]; fgb_nf_fill_* writes 64 weights per descriptor at
 * panel row desc_row[d].
 */
int fgb_nf_pair_masks(const int* pair_q, const long long* pair_t0, const long long* pair_moff,
                      long long num_pairs, long long total_words, const long long* leaf_r0,
                      const int* leaf_m, const int* leaf_wpr, const long long* leaf_word_off,
                      const long long* leaf_row_off, const unsigned* bits, unsigned* mask,
                      int* count, void* stream);
int fgb_nf_enumerate(const int* pair_q, const long long* pair_t0, const long long* pair_moff,
                     long long num_pairs, const int* leaf_wpr, const unsigned* mask,
                     const long long* desc_off, int* desc_pair, int* desc_col, void* stream);
int fgb_nf_fill_f32_f32(const int* pair_q, const long long* pair_t0, long long num_pairs,
                        const long long* leaf_r0, const int* leaf_m, const int* leaf_wpr,
                        const long long* leaf_word_off, const long long* leaf_row_off,
                        const unsigned* bits, const long long* indptr, const float* data,
                        const int* desc_pair, const int* desc_col, const long long* desc_row,
                        long long num_desc, void* panel, void* stream);
int fgb_nf_fill_f32_bf16(const int* pair_q, const long long* pair_t0, long long num_pairs,
                        const long long* leaf_r0, const int* leaf_m, const int* leaf_wpr,
                        const long long* leaf_word_off, const long long* leaf_row_off,
                        const unsigned* bits, const long long* indptr, const float* data,
                        const int* desc_pair, const int* desc_col, const long long* desc_row,
                        long long num_desc, void* panel, void* stream);
int fgb_nf_fill_f64_f64(const int* pair_q, const long long* pair_t0, long long num_pairs,
                        const long long* leaf_r0, const int* leaf_m, const int* leaf_wpr,
                        const long long* leaf_word_off, const long long* leaf_row_off,
                        const unsigned* bits, const long long* indptr, const double* data,
                        const int* desc_pair, const int* desc_col, const long long* desc_row,
                        long long num_desc, void* panel, void* stream);
int fgb_nf_fill_f64_f32(const int* pair_q, const long long* pair_t0, long long num_pairs,
                        const long long* leaf_r0, const int* leaf_m, const int* leaf_wpr,
                        const long long* leaf_word_off, const long long* leaf_row_off,
                        const unsigned* bits, const long long* indptr, const double* data,
                        const int* desc_pair, const int* desc_col, const long long* desc_row,
                        long long num_desc, void* panel, void* stream);
int fgb_nf_fill_f64_bf16(const int* pair_q, const long long* pair_t0, long long num_pairs,
                        const long long* leaf_r0, const int* leaf_m, const int* leaf_wpr,
                        const long long* leaf_word_off, const long long* leaf_row_off,
                        const unsigned* bits, const long long* indptr, const double* data,
                        const int* desc_pair, const int* desc_col, const long long* desc_row,
                        long long num_desc, void* panel, void* stream);

/* --------------------------------------------- solve kernels (a10-a12) */
/*
 * Element-wise pieces of solve_radiosity (src/flux/solve.py:4-45) for N x K
 * FP32 blocks: X = rho .* B (rho per row, or rho_scalar when rho == NULL),
 * column maxima of |Y - B| (Jacobi stopping test, solve.py:42) and of the
 * refinement residual R = E - B + Y, B += D, and row gathers between facet
 * order and cluster order.  colmax holds IEEE bits of non-negative floats.
 */
int fgb_scale_rows_f32(const float* B, const float* rho, float rho_scalar, float* X, long long N,
                       int K, void* stream);
int fgb_scale_rows_bf16(const float* B, const float* rho, float rho_scalar, void* X, long long N,
                        int K, void* stream);
/* colmax[c] = max(colmax[c], max_i |Y - B|) per column (B may be NULL: |Y|). */
int fgb_colmax_absdiff(const float* Y, const float* B, long long N, int K, unsigned* colmax,
                       void* stream);
int fgb_residual(const float* Y, const float* B, const float* E, float* R, long long N, int K,
                 unsigned* colmax, void* stream);
int fgb_axpy_cols(float* B, const float* D, const unsigned char* mask, long long N, int K,
                  void* stream);
int fgb_gather_rows_f32(const float* in, const long long* idx, float* out, long long N, int K,
                        void* stream);
int fgb_gather_rows_f64(const double* in, const long long* idx, double* out, long long N, int K,
                        void* stream);
/*
 * Y = add + alpha * A X for a CSR matrix A (int64 indptr, int32 indices) and
 * X, Y: n x K row-major — the product with the uncompressed matrix of
 * get_form_factor_matrix (src/flux/form_factors.py:72) inside
 * solve_radiosity / compute_steady_state_temp (src/flux/model.py:16).
 */
int fgb_csr_spmm_f64(const long long* indptr, const int* indices, const double* data, long long m,
                     const double* X, int K, double* Y, const double* add, double alpha,
                     void* stream);
int fgb_csr_spmm_f32(const long long* indptr, const int* indices, const float* data, long long m,
                     const float* X, int K, float* Y, const float* add, float alpha, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FLUXGB_H */
