// Visibility predicates with the semantics of the reference's two ray-tracing
// backends, evaluated on the LBVH (bvh.cuh).
//
// Embree semantics (EmbreeTrimeshShapeModel, src/flux/shape.py:349-421):
//   pair (i, j): D = P_j - P_i in the shape dtype; if |D| <= eps the pair is
//   forced visible (shape.py:360-361, 392); otherwise the FP32 ray starts at
//   P_i + eps * D/|D| with direction D/|D| (shape.py:380-381) and the pair is
//   visible iff its closest hit is facet j (shape.py:393-396).  Here: j's hit
//   distance t_j is computed with the watertight test, and the pair is
//   visible iff j is hit and no other facet is hit at t in (0, t_j).
//   sun (i, d): origin P_i + eps * N_i, occluded iff any hit
//   (shape.py:410-421).  eps = 1e3 * finfo(float32).resolution, which under
//   numpy 2 evaluates in float32 to 0.0010000000474974513.
// CGAL semantics (CgalTrimeshShapeModel, src/flux/cgal/aabb_wrapper.cpp:64-108):
//   rays in FP64 from the mesh centroid of face i with direction
//   centroid_j - centroid_i, face i skipped; visible iff the first hit is j
//   (no hit: not visible); i == j is not visible (aabb.pyx:58-70).  Sun: any
//   hit with face i skipped.
#pragma once
#include "bvh.cuh"

namespace fgb {

enum : int { kSemEmbree = 0, kSemCgal = 1 };

template <class R> struct EmbreeEps;
template <> struct EmbreeEps<double> { static constexpr double v = 0.0010000000474974513; };
template <> struct EmbreeEps<float> { static constexpr float v = 0.001f; };

__device__ __forceinline__ void tri_centroid64(const BvhView& b, int facet, double* c) {
  const double* v = b.tris64 + 9 * (size_t)b.slot_of[facet];
  for (int k = 0; k < 3; k++) c[k] = fdiv(fadd(fadd(v[k], v[3 + k]), v[6 + k]), 3.0);
}

template <class R>
__device__ __forceinline__ bool pair_visible_embree(const BvhView& b, const R* __restrict__ P, int i,
                                                    int j, bool* near_edge, bool* overflow) {
  const R eps = EmbreeEps<R>::v;
  R pi[3] = {P[3 * i], P[3 * i + 1], P[3 * i + 2]};
  R d[3] = {fsub(P[3 * j], pi[0]), fsub(P[3 * j + 1], pi[1]), fsub(P[3 * j + 2], pi[2])};
  R dn = fsqrt(fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2])));
  if (!(dn > eps)) return true;
  R dh[3], org[3];
  for (int k = 0; k < 3; k++) {
    dh[k] = fdiv(d[k], dn);
    org[k] = fadd(pi[k], fmul(eps, dh[k]));
  }
  Ray r;
  make_ray(r, (float)org[0], (float)org[1], (float)org[2], (float)dh[0], (float)dh[1],
           (float)dh[2]);
  int sj = b.slot_of[j];
  float v0[3], v1[3], v2[3];
  int prim;
  load_tri(b, sj, v0, v1, v2, &prim);
  TriHit hj = tri_test(r, v0, v1, v2, INFINITY);
  if (!hj.hit) return false;
  return any_hit(b, r, hj.t, j, -1, near_edge, overflow) == 0;
}

__device__ __forceinline__ bool pair_visible_cgal(const BvhView& b, int i, int j, bool* overflow) {
  if (i == j) return false;
  double ci[3], cj[3], d[3];
  tri_centroid64(b, i, ci);
  tri_centroid64(b, j, cj);
  for (int k = 0; k < 3; k++) d[k] = fsub(cj[k], ci[k]);
  Ray64 r;
  make_ray64(r, ci, d);
  double tj;
  if (!tri_test64(r, b.tris64 + 9 * (size_t)b.slot_of[j], INFINITY, &tj)) return false;
  double t;
  return first_hit64(b, r, i, j, tj, true, &t, overflow) < 0;
}

template <class R>
__device__ __forceinline__ bool pair_visible(const BvhView& b, const R* __restrict__ P, int i, int j,
                                             int sem, bool* near_edge, bool* overflow) {
  if (sem == kSemCgal) return pair_visible_cgal(b, i, j, overflow);
  return pair_visible_embree<R>(b, P, i, j, near_edge, overflow);
}

// Sun occlusion of facet i along direction dir (3 values of the shape dtype).
template <class R>
__device__ __forceinline__ bool sun_occluded(const BvhView& b, const R* __restrict__ P,
                                             const R* __restrict__ N, int i, const R* dir, int sem,
                                             bool* overflow) {
  if (sem == kSemCgal) {
    double ci[3], d[3] = {(double)dir[0], (double)dir[1], (double)dir[2]};
    tri_centroid64(b, i, ci);
    Ray64 r;
    make_ray64(r, ci, d);
    double t;
    return first_hit64(b, r, i, -1, INFINITY, true, &t, overflow) >= 0;
  }
  const R eps = EmbreeEps<R>::v;
  R org[3];
  for (int k = 0; k < 3; k++) org[k] = fadd(P[3 * i + k], fmul(eps, N[3 * i + k]));
  Ray r;
  make_ray(r, (float)org[0], (float)org[1], (float)org[2], (float)dir[0], (float)dir[1],
           (float)dir[2]);
  bool ne = false;
  return any_hit(b, r, INFINITY, -1, -1, &ne, overflow) != 0;
}

}  // namespace fgb
