// Ray-query entry points: pair visibility, sun occlusion, direct irradiance
// and first intersection.  They replace the reference's
//   TrimeshShapeModel.get_visibility / _get_visibility  (src/flux/shape.py:138-170, 272-281, 349-398)
//   TrimeshShapeModel.is_occluded / _is_occluded        (shape.py:181-188, 283-292, 400-421)
//   TrimeshShapeModel.get_direct_irradiance             (shape.py:190-244)
//   CgalTrimeshShapeModel.intersect1                     (shape.py:269-270, aabb_wrapper.cpp:110-129)
// One thread per ray; predicates in visibility.cuh.
#include "common.cuh"
#include "visibility.cuh"

namespace fgb {
BvhView view_of(const void* handle);

namespace {

template <class R>
__global__ void visibility_kernel(BvhView b, const R* __restrict__ P, long long num_faces,
                                  const long long* __restrict__ I, long long m,
                                  const long long* __restrict__ J, long long n, int paired, int sem,
                                  unsigned char* __restrict__ vis,
                                  unsigned char* __restrict__ near_edge,
                                  unsigned* __restrict__ flags) {
  long long total = paired ? m : m * n;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    long long i = paired ? I[q] : I[q / n];
    long long j = paired ? J[q] : J[q % n];
    if (i < 0 || j < 0 || i >= num_faces || j >= num_faces) {
      atomicOr(flags, kFlagIndexRange);
      vis[q] = 0;
      continue;
    }
    bool ne = false, of = false;
    bool v = pair_visible<R>(b, P, (int)i, (int)j, sem, &ne, &of);
    if (of) atomicOr(flags, kFlagStackOverflow);
    vis[q] = v ? 1 : 0;
    if (near_edge) near_edge[q] = ne ? 1 : 0;
  }
}

template <class R>
__global__ void occluded_kernel(BvhView b, const R* __restrict__ P, const R* __restrict__ N,
                                long long num_faces, const long long* __restrict__ I, long long m,
                                const R* __restrict__ D, long long ndirs, int per_facet, int sem,
                                unsigned char* __restrict__ occ, unsigned* __restrict__ flags) {
  long long total = per_facet ? m : m * ndirs;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    long long p = per_facet ? q : q / ndirs;
    long long k = per_facet ? q : q % ndirs;
    long long i = I[p];
    if (i < 0 || i >= num_faces) {
      atomicOr(flags, kFlagIndexRange);
      occ[q] = 0;
      continue;
    }
    R dir[3] = {D[3 * k], D[3 * k + 1], D[3 * k + 2]};
    bool of = false;
    bool o = sun_occluded<R>(b, P, N, (int)i, dir, sem, &of);
    if (of) atomicOr(flags, kFlagStackOverflow);
    occ[q] = o ? 1 : 0;
  }
}

// E[i, k] = F0[k] * max(0, N_i . d_k) if facet i sees the sun along d_k,
// else 0 (shape.py:224-226 for each direction).  Direction-major thread
// order: a warp traces one direction from 32 neighbouring facets.
template <class R, class RO>
__global__ void irradiance_kernel(BvhView b, const R* __restrict__ P, const R* __restrict__ N,
                                  long long num_faces, const R* __restrict__ D, long long K,
                                  const R* __restrict__ F0, int sem, RO* __restrict__ E,
                                  unsigned* __restrict__ flags) {
  long long total = num_faces * K;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    long long k = q / num_faces;
    long long i = q % num_faces;
    R dir[3] = {D[3 * k], D[3 * k + 1], D[3 * k + 2]};
    // N[I] @ Dsun: BLAS-free dot, same order as the FF numerator
    R nd = dot3(N[3 * i], N[3 * i + 1], N[3 * i + 2], dir[0], dir[1], dir[2]);
    R e = R(0);
    if (nd > R(0)) {
      bool of = false;
      bool o = sun_occluded<R>(b, P, N, (int)i, dir, sem, &of);
      if (of) atomicOr(flags, kFlagStackOverflow);
      if (!o) e = fmul(F0[k], nd);
    }
    E[i * K + k] = (RO)e;
  }
}

// Closest hit of FP64 rays (x_p, d_p), no face skipped (aabb_wrapper.cpp:110-129).
__global__ void intersect1_kernel(BvhView b, const double* __restrict__ X, const double* __restrict__ Dd,
                                  long long m, long long* __restrict__ hit, double* __restrict__ xt,
                                  unsigned* __restrict__ flags) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < m;
       q += (long long)gridDim.x * blockDim.x) {
    Ray64 r;
    make_ray64(r, X + 3 * q, Dd + 3 * q);
    double t;
    bool of = false;
    int h = first_hit64(b, r, -1, -1, INFINITY, false, &t, &of);
    if (of) atomicOr(flags, kFlagStackOverflow);
    hit[q] = h;
    for (int k = 0; k < 3; k++) xt[3 * q + k] = h >= 0 ? fadd(r.o[k], fmul(t, r.d[k])) : NAN;
  }
}

int check_bvh(const void* bvh, int sem) {
  if (!bvh) { set_error("null BVH handle"); return FGB_BAD_ARG; }
  if (sem != kSemEmbree && sem != kSemCgal) { set_error("unknown semantics %d", sem); return FGB_BAD_ARG; }
  if (sem == kSemCgal && view_of(bvh).tris64 == nullptr && view_of(bvh).num_prims > 0) {
    set_error("CGAL semantics need a BVH built with keep_f64");
    return FGB_BAD_ARG;
  }
  return FGB_OK;
}

template <class R>
int visibility(const void* bvh, const R* P, long long num_faces, const long long* I, long long m,
               const long long* J, long long n, int paired, int sem, unsigned char* vis,
               unsigned char* near_edge, unsigned* flags, void* stream) {
  int st = check_bvh(bvh, sem);
  if (st) return st;
  if (m < 0 || n < 0 || (paired && m != n)) { set_error("bad sizes"); return FGB_BAD_ARG; }
  long long total = paired ? m : m * n;
  if (total == 0) return FGB_OK;
  visibility_kernel<R><<<grid_for(total, 128, 152LL * 64), 128, 0, as_stream(stream)>>>(
      view_of(bvh), P, num_faces, I, m, J, n, paired, sem, vis, near_edge, flags);
  FGB_LAUNCH_CHECK("visibility_kernel");
  return FGB_OK;
}

template <class R>
int occluded(const void* bvh, const R* P, const R* N, long long num_faces, const long long* I,
             long long m, const R* D, long long ndirs, int per_facet, int sem, unsigned char* occ,
             unsigned* flags, void* stream) {
  int st = check_bvh(bvh, sem);
  if (st) return st;
  long long total = per_facet ? m : m * ndirs;
  if (total == 0) return FGB_OK;
  occluded_kernel<R><<<grid_for(total, 128, 152LL * 64), 128, 0, as_stream(stream)>>>(
      view_of(bvh), P, N, num_faces, I, m, D, ndirs, per_facet, sem, occ, flags);
  FGB_LAUNCH_CHECK("occluded_kernel");
  return FGB_OK;
}

template <class R, class RO>
int irradiance(const void* bvh, const R* P, const R* N, long long num_faces, const R* D,
               long long K, const R* F0, int sem, RO* E, unsigned* flags, void* stream) {
  int st = check_bvh(bvh, sem);
  if (st) return st;
  long long total = num_faces * K;
  if (total == 0) return FGB_OK;
  irradiance_kernel<R, RO><<<grid_for(total, 128, 152LL * 64), 128, 0, as_stream(stream)>>>(
      view_of(bvh), P, N, num_faces, D, K, F0, sem, E, flags);
  FGB_LAUNCH_CHECK("irradiance_kernel");
  return FGB_OK;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_visibility_f64(const void* bvh, const double* P, long long num_faces, const long long* I,
                       long long m, const long long* J, long long n, int paired, int semantics,
                       unsigned char* vis, unsigned char* near_edge, unsigned* flags, void* stream) {
  return fgb::visibility<double>(bvh, P, num_faces, I, m, J, n, paired, semantics, vis, near_edge,
                                 flags, stream);
}

int fgb_visibility_f32(const void* bvh, const float* P, long long num_faces, const long long* I,
                       long long m, const long long* J, long long n, int paired, int semantics,
                       unsigned char* vis, unsigned char* near_edge, unsigned* flags, void* stream) {
  return fgb::visibility<float>(bvh, P, num_faces, I, m, J, n, paired, semantics, vis, near_edge,
                                flags, stream);
}

int fgb_occluded_f64(const void* bvh, const double* P, const double* N, long long num_faces,
                     const long long* I, long long m, const double* D, long long ndirs,
                     int per_facet, int semantics, unsigned char* occluded, unsigned* flags,
                     void* stream) {
  return fgb::occluded<double>(bvh, P, N, num_faces, I, m, D, ndirs, per_facet, semantics,
                               occluded, flags, stream);
}

int fgb_occluded_f32(const void* bvh, const float* P, const float* N, long long num_faces,
                     const long long* I, long long m, const float* D, long long ndirs,
                     int per_facet, int semantics, unsigned char* occluded, unsigned* flags,
                     void* stream) {
  return fgb::occluded<float>(bvh, P, N, num_faces, I, m, D, ndirs, per_facet, semantics, occluded,
                              flags, stream);
}

int fgb_direct_irradiance_f64(const void* bvh, const double* P, const double* N,
                              long long num_faces, const double* D, long long K, const double* F0,
                              int semantics, double* E, unsigned* flags, void* stream) {
  return fgb::irradiance<double, double>(bvh, P, N, num_faces, D, K, F0, semantics, E, flags,
                                         stream);
}

int fgb_direct_irradiance_f64_to_f32(const void* bvh, const double* P, const double* N,
                                     long long num_faces, const double* D, long long K,
                                     const double* F0, int semantics, float* E, unsigned* flags,
                                     void* stream) {
  return fgb::irradiance<double, float>(bvh, P, N, num_faces, D, K, F0, semantics, E, flags,
                                        stream);
}

int fgb_direct_irradiance_f32(const void* bvh, const float* P, const float* N, long long num_faces,
                              const float* D, long long K, const float* F0, int semantics,
                              float* E, unsigned* flags, void* stream) {
  return fgb::irradiance<float, float>(bvh, P, N, num_faces, D, K, F0, semantics, E, flags,
                                       stream);
}

int fgb_intersect1_f64(const void* bvh, const double* X, const double* D, long long m,
                       long long* hit, double* xt, unsigned* flags, void* stream) {
  int st = fgb::check_bvh(bvh, fgb::kSemCgal);
  if (st) return st;
  if (m <= 0) return FGB_OK;
  fgb::intersect1_kernel<<<fgb::grid_for(m, 128), 128, 0, fgb::as_stream(stream)>>>(
      fgb::view_of(bvh), X, D, m, hit, xt, flags);
  FGB_LAUNCH_CHECK("intersect1_kernel");
  return FGB_OK;
}

}  // extern "C"
