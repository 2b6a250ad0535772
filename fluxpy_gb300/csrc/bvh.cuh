// Device view of the linear BVH (LBVH) over the triangles of a shape model,
// and the ray queries that replace Embree's intersect1M / occluded1M
// (src/flux/shape.py:375-421) and CGAL's AABB first_intersection
// (src/flux/cgal/aabb_wrapper.cpp:64-129).
//
// Layout (all in HBM, built by lbvh.cu):
//   nodes  : 4 x float4 per internal node i (0 <= i < n-1):
//            [0] = left child box lo (xyz) | left child index (w, int bits)
//            [1] = left child box hi (xyz) | unused
//            [2] = right child box lo       | right child index
//            [3] = right child box hi       | unused
//            child index >= 0: internal node; < 0: leaf ~k (k = sorted slot)
//   tris   : 3 x float4 per sorted slot: v0, v1, v2 (FP32, as Embree's
//            float32 vertex buffer, shape.py:316-323); v0.w = original
//            facet id (int bits)
//   tris64 : 9 doubles per sorted slot (FP64 vertices), for CGAL semantics
//   slot_of: facet id -> sorted slot
//
// Ray/triangle test: the watertight algorithm of Woop, Benthin & Wald,
// "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013, with the
// double-precision fallback for edge functions that evaluate to zero.  All
// arithmetic goes through the _rn intrinsics so the CPU oracle (same steps in
// C, -ffp-contract=off) produces identical decisions.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "fparith.cuh"

namespace fgb {

struct BvhView {
  const float4* nodes;
  const float4* tris;
  const double* tris64;
  const int* slot_of;  // facet id -> sorted slot
  int num_prims;
};

constexpr int kStackSize = 96;

// Relative edge margin below which a tested triangle counts as "near edge"
// for the ray (pairs reported, not changed).
constexpr float kNearEdgeRel = 1e-6f;

struct Ray {
  float o[3];
  float d[3];
  float inv[3];
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

__device__ __forceinline__ void make_ray(Ray& r, float ox, float oy, float oz, float dx, float dy,
                                         float dz) {
  r.o[0] = ox; r.o[1] = oy; r.o[2] = oz;
  r.d[0] = dx; r.d[1] = dy; r.d[2] = dz;
  for (int k = 0; k < 3; k++) r.inv[k] = fdiv(1.0f, r.d[k]);
  float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > (kz == 0 ? ax : ay)) kz = 2;
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (r.d[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = fdiv(r.d[kx], r.d[kz]);
  r.Sy = fdiv(r.d[ky], r.d[kz]);
  r.Sz = fdiv(1.0f, r.d[kz]);
}

// Conservative slab test (Ize, "Robust BVH Ray Traversal", JCGT 2013):
// tmax is inflated by 1 + 2*gamma(3) so rounding never culls a true hit.
__device__ __forceinline__ bool ray_box(const Ray& r, float4 lo, float4 hi, float tmax_limit) {
  float t0x = (lo.x - r.o[0]) * r.inv[0], t1x = (hi.x - r.o[0]) * r.inv[0];
  float t0y = (lo.y - r.o[1]) * r.inv[1], t1y = (hi.y - r.o[1]) * r.inv[1];
  float t0z = (lo.z - r.o[2]) * r.inv[2], t1z = (hi.z - r.o[2]) * r.inv[2];
  float tnx = fminf(t0x, t1x), tfx = fmaxf(t0x, t1x);
  float tny = fminf(t0y, t1y), tfy = fmaxf(t0y, t1y);
  float tnz = fminf(t0z, t1z), tfz = fmaxf(t0z, t1z);
  // NaN (0 * inf) slabs: fminf/fmaxf drop NaN operands, keeping the test conservative.
  float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
  float tf = fminf(fminf(tfx, tfy), tfz) * 1.0000004f;
  return tn <= tf && tn <= tmax_limit * 1.0000004f;
}

struct TriHit {
  bool hit;
  float t;       // valid when hit
  bool near_edge;
};

// Edge functions in double, for the zero case (Woop et al. section 3).
__device__ __forceinline__ void edge_fns_f64(float Ax, float Ay, float Bx, float By, float Cx,
                                             float Cy, float& U, float& V, float& W) {
  double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
  U = (float)__dsub_rn(CxBy, CyBx);
  double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
  V = (float)__dsub_rn(AxCy, AyCx);
  double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
  W = (float)__dsub_rn(BxAy, ByAx);
}

// Watertight FP32 test.  Reports a hit with t in (0, tmax) (tmax exclusive).
// near_edge is set when the ray meets the triangle's plane inside (0, tmax]
// within kNearEdgeRel (relative to the edge-function sum) of its boundary.
__device__ __forceinline__ TriHit tri_test(const Ray& r, const float* v0, const float* v1,
                                           const float* v2, float tmax) {
  TriHit h{false, 0.0f, false};
  const int kx = r.kx, ky = r.ky, kz = r.kz;
  float A[3], B[3], C[3];
  for (int k = 0; k < 3; k++) {
    A[k] = fsub(v0[k], r.o[k]);
    B[k] = fsub(v1[k], r.o[k]);
    C[k] = fsub(v2[k], r.o[k]);
  }
  float Ax = fsub(A[kx], fmul(r.Sx, A[kz]));
  float Ay = fsub(A[ky], fmul(r.Sy, A[kz]));
  float Bx = fsub(B[kx], fmul(r.Sx, B[kz]));
  float By = fsub(B[ky], fmul(r.Sy, B[kz]));
  float Cx = fsub(C[kx], fmul(r.Sx, C[kz]));
  float Cy = fsub(C[ky], fmul(r.Sy, C[kz]));
  float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
  float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
  float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) edge_fns_f64(Ax, Ay, Bx, By, Cx, Cy, U, V, W);
  bool outside = (U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f);
  float det = fadd(fadd(U, V), W);
  if (det == 0.0f) return h;
  // edge margin relative to |det| (det > 0: inside means U,V,W >= 0)
  float sU = det > 0.0f ? U : -U, sV = det > 0.0f ? V : -V, sW = det > 0.0f ? W : -W;
  float lim = fmul(kNearEdgeRel, fabsf(det));
  bool near;
  if (!outside) near = fminf(fminf(sU, sV), sW) < lim;
  else near = fmaxf(fmaxf(-sU, -sV), -sW) < lim;
  if (outside && !near) return h;
  float Az = fmul(r.Sz, A[kz]);
  float Bz = fmul(r.Sz, B[kz]);
  float Cz = fmul(r.Sz, C[kz]);
  float T = fadd(fadd(fmul(U, Az), fmul(V, Bz)), fmul(W, Cz));
  float t = fdiv(T, det);
  if (near && t > 0.0f && t <= tmax) h.near_edge = true;
  if (outside) return h;
  if (!(t > 0.0f && t < tmax)) return h;
  h.hit = true;
  h.t = t;
  return h;
}

__device__ __forceinline__ void load_tri(const BvhView& b, int slot, float* v0, float* v1,
                                         float* v2, int* prim) {
  float4 a = __ldg(&b.tris[3 * slot]);
  float4 c = __ldg(&b.tris[3 * slot + 1]);
  float4 e = __ldg(&b.tris[3 * slot + 2]);
  v0[0] = a.x; v0[1] = a.y; v0[2] = a.z;
  v1[0] = c.x; v1[1] = c.y; v1[2] = c.z;
  v2[0] = e.x; v2[1] = e.y; v2[2] = e.z;
  *prim = __float_as_int(a.w);
}

// Any hit with t in (0, tmax), skipping facets skip0 / skip1 (-1 = none).
// Returns 1 if occluded, 0 if not; sets *near_edge; on stack overflow sets
// *overflow and reports occluded.
__device__ __forceinline__ int any_hit(const BvhView& b, const Ray& r, float tmax, int skip0,
                                       int skip1, bool* near_edge, bool* overflow) {
  if (b.num_prims <= 0) return 0;
  int stack[kStackSize];
  int sp = 0;
  int node = (b.num_prims == 1) ? ~0 : 0;
  while (true) {
    if (node < 0) {
      int slot = ~node;
      float v0[3], v1[3], v2[3];
      int prim;
      load_tri(b, slot, v0, v1, v2, &prim);
      if (prim != skip0 && prim != skip1) {
        TriHit h = tri_test(r, v0, v1, v2, tmax);
        if (h.near_edge) *near_edge = true;
        if (h.hit) return 1;
      }
      if (sp == 0) return 0;
      node = stack[--sp];
      continue;
    }
    const float4* nd = b.nodes + 4 * (size_t)node;
    float4 ll = __ldg(nd), lh = __ldg(nd + 1), rl = __ldg(nd + 2), rh = __ldg(nd + 3);
    bool hl = ray_box(r, ll, lh, tmax);
    bool hr = ray_box(r, rl, rh, tmax);
    int cl = __float_as_int(ll.w), cr = __float_as_int(rl.w);
    if (hl && hr) {
      if (sp >= kStackSize) { *overflow = true; return 1; }
      stack[sp++] = cr;
      node = cl;
    } else if (hl) {
      node = cl;
    } else if (hr) {
      node = cr;
    } else {
      if (sp == 0) return 0;
      node = stack[--sp];
    }
  }
}

// Closest hit with t in (0, +inf), skipping facet `skip` (-1 = none).
// Returns the facet id or -1.  Ties in t keep the first found.
__device__ __forceinline__ int closest_hit(const BvhView& b, const Ray& r, int skip, float* t_out,
                                           bool* overflow) {
  if (b.num_prims <= 0) return -1;
  int stack[kStackSize];
  int sp = 0;
  int node = (b.num_prims == 1) ? ~0 : 0;
  float best = INFINITY;
  int best_prim = -1;
  while (true) {
    if (node < 0) {
      int slot = ~node;
      float v0[3], v1[3], v2[3];
      int prim;
      load_tri(b, slot, v0, v1, v2, &prim);
      if (prim != skip) {
        TriHit h = tri_test(r, v0, v1, v2, best);
        if (h.hit && (h.t < best)) { best = h.t; best_prim = prim; }
      }
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    const float4* nd = b.nodes + 4 * (size_t)node;
    float4 ll = __ldg(nd), lh = __ldg(nd + 1), rl = __ldg(nd + 2), rh = __ldg(nd + 3);
    bool hl = ray_box(r, ll, lh, best);
    bool hr = ray_box(r, rl, rh, best);
    int cl = __float_as_int(ll.w), cr = __float_as_int(rl.w);
    if (hl && hr) {
      if (sp >= kStackSize) { *overflow = true; break; }
      stack[sp++] = cr;
      node = cl;
    } else if (hl) {
      node = cl;
    } else if (hr) {
      node = cr;
    } else {
      if (sp == 0) break;
      node = stack[--sp];
    }
  }
  *t_out = best;
  return best_prim;
}

// ---------------------------------------------------------------- FP64 ----
// CGAL semantics (aabb_wrapper.cpp:64-108): rays in double from the centroid,
// skip the source face, first intersection.  Boxes are tested in FP32 on a
// ray rounded outward-safe (conservative slab test); triangles in FP64 with
// the same watertight algorithm.

struct Ray64 {
  double o[3], d[3];
  int kx, ky, kz;
  double Sx, Sy, Sz;
};

__device__ __forceinline__ void make_ray64(Ray64& r, const double* o, const double* d) {
  for (int k = 0; k < 3; k++) { r.o[k] = o[k]; r.d[k] = d[k]; }
  double ax = fabs(d[0]), ay = fabs(d[1]), az = fabs(d[2]);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > (kz == 0 ? ax : ay)) kz = 2;
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (r.d[kz] < 0.0) { int t = kx; kx = ky; ky = t; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = fdiv(r.d[kx], r.d[kz]);
  r.Sy = fdiv(r.d[ky], r.d[kz]);
  r.Sz = fdiv(1.0, r.d[kz]);
}

// FP64 watertight test, t in (0, tmax).
__device__ __forceinline__ bool tri_test64(const Ray64& r, const double* v, double tmax, double* t_out) {
  const int kx = r.kx, ky = r.ky, kz = r.kz;
  double A[3], B[3], C[3];
  for (int k = 0; k < 3; k++) {
    A[k] = fsub(v[k], r.o[k]);
    B[k] = fsub(v[3 + k], r.o[k]);
    C[k] = fsub(v[6 + k], r.o[k]);
  }
  double Ax = fsub(A[kx], fmul(r.Sx, A[kz]));
  double Ay = fsub(A[ky], fmul(r.Sy, A[kz]));
  double Bx = fsub(B[kx], fmul(r.Sx, B[kz]));
  double By = fsub(B[ky], fmul(r.Sy, B[kz]));
  double Cx = fsub(C[kx], fmul(r.Sx, C[kz]));
  double Cy = fsub(C[ky], fmul(r.Sy, C[kz]));
  double U = fsub(fmul(Cx, By), fmul(Cy, Bx));
  double V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
  double W = fsub(fmul(Bx, Ay), fmul(By, Ax));
  if ((U < 0.0 || V < 0.0 || W < 0.0) && (U > 0.0 || V > 0.0 || W > 0.0)) return false;
  double det = fadd(fadd(U, V), W);
  if (det == 0.0) return false;
  double T = fadd(fadd(fmul(U, fmul(r.Sz, A[kz])), fmul(V, fmul(r.Sz, B[kz]))),
                  fmul(W, fmul(r.Sz, C[kz])));
  double t = fdiv(T, det);
  if (!(t > 0.0 && t < tmax)) return false;
  *t_out = t;
  return true;
}

// Conservative FP32 box test for an FP64 ray: origin/direction rounded to
// float, boxes inflated by a relative 1e-6 and the slab interval by 1e-5.
__device__ __forceinline__ bool ray64_box(const float* o, const float* inv, float4 lo, float4 hi,
                                          float tmax_f) {
  float lx = lo.x - 1e-6f * fabsf(lo.x) - 1e-30f, ly = lo.y - 1e-6f * fabsf(lo.y) - 1e-30f,
        lz = lo.z - 1e-6f * fabsf(lo.z) - 1e-30f;
  float hx = hi.x + 1e-6f * fabsf(hi.x) + 1e-30f, hy = hi.y + 1e-6f * fabsf(hi.y) + 1e-30f,
        hz = hi.z + 1e-6f * fabsf(hi.z) + 1e-30f;
  float t0x = (lx - o[0]) * inv[0], t1x = (hx - o[0]) * inv[0];
  float t0y = (ly - o[1]) * inv[1], t1y = (hy - o[1]) * inv[1];
  float t0z = (lz - o[2]) * inv[2], t1z = (hz - o[2]) * inv[2];
  float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), 0.0f));
  float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
  tf = tf * 1.00001f + 1e-30f;
  return tn <= tf && tn <= tmax_f;
}

// First hit of an FP64 ray with t in (0, tmax), skipping skip0 / skip1;
// any_only stops at the first hit found.  Returns the facet id or -1.
__device__ __forceinline__ int first_hit64(const BvhView& b, const Ray64& r, int skip0, int skip1,
                                           double tmax, bool any_only, double* t_out,
                                           bool* overflow) {
  if (b.num_prims <= 0) return -1;
  float o[3], inv[3];
  for (int k = 0; k < 3; k++) {
    o[k] = (float)r.o[k];
    inv[k] = (float)(1.0 / r.d[k]);
  }
  int stack[kStackSize];
  int sp = 0;
  int node = (b.num_prims == 1) ? ~0 : 0;
  double best = tmax;
  int best_prim = -1;
  while (true) {
    if (node < 0) {
      int slot = ~node;
      float4 a = __ldg(&b.tris[3 * slot]);
      int prim = __float_as_int(a.w);
      if (prim != skip0 && prim != skip1) {
        double t;
        if (tri_test64(r, b.tris64 + 9 * (size_t)slot, best, &t)) {
          best = t;
          best_prim = prim;
          if (any_only) break;
        }
      }
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    const float4* nd = b.nodes + 4 * (size_t)node;
    float4 ll = __ldg(nd), lh = __ldg(nd + 1), rl = __ldg(nd + 2), rh = __ldg(nd + 3);
    float tb = isinf(best) ? INFINITY : (float)best * 1.0001f + 1e-30f;
    bool hl = ray64_box(o, inv, ll, lh, tb);
    bool hr = ray64_box(o, inv, rl, rh, tb);
    int cl = __float_as_int(ll.w), cr = __float_as_int(rl.w);
    if (hl && hr) {
      if (sp >= kStackSize) { *overflow = true; break; }
      stack[sp++] = cr;
      node = cl;
    } else if (hl) {
      node = cl;
    } else if (hr) {
      node = cr;
    } else {
      if (sp == 0) break;
      node = stack[--sp];
    }
  }
  *t_out = best;
  return best_prim;
}

}  // namespace fgb
