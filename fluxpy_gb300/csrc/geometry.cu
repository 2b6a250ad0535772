// Facet geometry: centroids, unit normals, areas.
//
// Restates get_centroids / get_cross_products /
// get_surface_normals_and_face_areas (src/flux/shape.py:16-45) with the same
// per-element operation order as numpy, so results are bit-identical:
//   P = ((v0 + v1) + v2) / 3           (V[F].mean(axis=1))
//   C = (v1-v0) x (v2-v0)              (np.cross, no FMA)
//   |C| = sqrt((c0^2 + c1^2) + c2^2)
//   N = C / |C|,  A = |C| / 2
#include "common.cuh"
#include "fparith.cuh"

namespace fgb {
namespace {

template <class R, class IDX>
__global__ void facet_geometry_kernel(const R* __restrict__ V, long long nv,
                                      const IDX* __restrict__ F, long long nf,
                                      R* __restrict__ P, R* __restrict__ N, R* __restrict__ A,
                                      unsigned* __restrict__ flags) {
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
       f += (long long)gridDim.x * blockDim.x) {
    long long i0 = (long long)F[3 * f], i1 = (long long)F[3 * f + 1], i2 = (long long)F[3 * f + 2];
    if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= nv || i1 >= nv || i2 >= nv) {
      atomicOr(flags, kFlagIndexRange);
      continue;
    }
    R a[3], b[3], c[3];
    for (int k = 0; k < 3; k++) {
      a[k] = V[3 * i0 + k];
      b[k] = V[3 * i1 + k];
      c[k] = V[3 * i2 + k];
    }
    if (P) {
      for (int k = 0; k < 3; k++) P[3 * f + k] = fdiv(fadd(fadd(a[k], b[k]), c[k]), R(3));
    }
    R e1[3], e2[3];
    for (int k = 0; k < 3; k++) {
      e1[k] = fsub(b[k], a[k]);
      e2[k] = fsub(c[k], a[k]);
    }
    R cx = fsub(fmul(e1[1], e2[2]), fmul(e1[2], e2[1]));
    R cy = fsub(fmul(e1[2], e2[0]), fmul(e1[0], e2[2]));
    R cz = fsub(fmul(e1[0], e2[1]), fmul(e1[1], e2[0]));
    R nrm = fsqrt(fadd(fadd(fmul(cx, cx), fmul(cy, cy)), fmul(cz, cz)));
    if (N) {
      N[3 * f] = fdiv(cx, nrm);
      N[3 * f + 1] = fdiv(cy, nrm);
      N[3 * f + 2] = fdiv(cz, nrm);
    }
    if (A) A[f] = fdiv(nrm, R(2));
  }
}

template <class R>
int launch_geometry(const R* V, long long nv, const long long* F, long long nf, R* P, R* N, R* A,
                    unsigned* flags, void* stream) {
  if (nv < 0 || nf < 0) { set_error("negative sizes"); return FGB_BAD_ARG; }
  if (nf == 0) return FGB_OK;
  cudaStream_t s = as_stream(stream);
  facet_geometry_kernel<R, long long><<<grid_for(nf, 256), 256, 0, s>>>(V, nv, F, nf, P, N, A, flags);
  FGB_LAUNCH_CHECK("facet_geometry_kernel");
  return FGB_OK;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_facet_geometry_f64(const double* V, long long nv, const long long* F, long long nf,
                           double* P, double* N, double* A, unsigned* flags, void* stream) {
  return fgb::launch_geometry<double>(V, nv, F, nf, P, N, A, flags, stream);
}

int fgb_facet_geometry_f32(const float* V, long long nv, const long long* F, long long nf,
                           float* P, float* N, float* A, unsigned* flags, void* stream) {
  return fgb::launch_geometry<float>(V, nv, F, nf, P, N, A, flags, stream);
}

}  // extern "C"
