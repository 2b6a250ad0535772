// Linear BVH built on the device, replacing Embree's scene build
// (src/flux/shape.py:296-344) and CGAL's AABB tree
// (src/flux/cgal/aabb_wrapper.cpp:40-57).
//
// Steps (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012):
//   1. per-triangle FP32 vertices (Embree stores float32 vertices,
//      shape.py:316-323), AABB centroid, scene bounds of the centroids;
//   2. 63-bit Morton codes (21 bits per axis);
//   3. radix sort of (code, facet id) with CUB;
//   4. internal nodes from the sorted codes (ties broken by slot index);
//   5. bottom-up refit with one atomic arrival counter per node.
// Leaves hold one triangle.  Layout is documented in bvh.cuh.
#include "common.cuh"
#include "bvh.cuh"

#include <cub/cub.cuh>

struct fgb_bvh_impl {
  float4* nodes = nullptr;
  float4* tris = nullptr;
  double* tris64 = nullptr;
  int* slot_of = nullptr;
  long long num_prims = 0;
  size_t bytes = 0;
};

namespace fgb {

BvhView view_of(const void* handle) {
  const fgb_bvh_impl* h = static_cast<const fgb_bvh_impl*>(handle);
  BvhView v;
  v.nodes = h->nodes;
  v.tris = h->tris;
  v.tris64 = h->tris64;
  v.slot_of = h->slot_of;
  v.num_prims = (int)h->num_prims;
  return v;
}

namespace {

__device__ __forceinline__ unsigned long long expand21(unsigned long long v) {
  v &= 0x1fffffULL;
  v = (v | (v << 32)) & 0x1f00000000ffffULL;
  v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
  v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}

// Order-preserving float <-> uint mapping for atomic min/max.
__device__ __forceinline__ unsigned f2u(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float u2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

template <class R>
__global__ void tri_bounds_kernel(const R* __restrict__ V, long long nv, const long long* __restrict__ F,
                                  long long nf, float4* __restrict__ tri_tmp,
                                  unsigned* __restrict__ scene, unsigned* __restrict__ flags) {
  // scene: [minx, miny, minz, maxx, maxy, maxz] of AABB centroids (ordered uints)
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
       f += (long long)gridDim.x * blockDim.x) {
    long long id[3] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]};
    float v[3][3];
    for (int a = 0; a < 3; a++) {
      long long i = id[a];
      if (i < 0 || i >= nv) { atomicOr(flags, kFlagIndexRange); i = 0; }
      for (int k = 0; k < 3; k++) v[a][k] = (float)V[3 * i + k];
    }
    tri_tmp[3 * f] = make_float4(v[0][0], v[0][1], v[0][2], __int_as_float((int)f));
    tri_tmp[3 * f + 1] = make_float4(v[1][0], v[1][1], v[1][2], 0.f);
    tri_tmp[3 * f + 2] = make_float4(v[2][0], v[2][1], v[2][2], 0.f);
    for (int k = 0; k < 3; k++) {
      float mn = fminf(fminf(v[0][k], v[1][k]), v[2][k]);
      float mx = fmaxf(fmaxf(v[0][k], v[1][k]), v[2][k]);
      float c = 0.5f * (mn + mx);
      lo[k] = fminf(lo[k], c);
      hi[k] = fmaxf(hi[k], c);
    }
  }
  for (int k = 0; k < 3; k++) {
    for (int off = 16; off > 0; off >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; k++) {
      atomicMin(&scene[k], f2u(lo[k]));
      atomicMax(&scene[3 + k], f2u(hi[k]));
    }
  }
}

__global__ void morton_kernel(const float4* __restrict__ tri_tmp, long long nf,
                              const unsigned* __restrict__ scene,
                              unsigned long long* __restrict__ codes, int* __restrict__ ids) {
  float lo[3], ext[3];
  for (int k = 0; k < 3; k++) {
    lo[k] = u2f(scene[k]);
    float e = u2f(scene[3 + k]) - lo[k];
    ext[k] = e > 0.f ? e : 1.f;
  }
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
       f += (long long)gridDim.x * blockDim.x) {
    float4 a = tri_tmp[3 * f], b = tri_tmp[3 * f + 1], c = tri_tmp[3 * f + 2];
    float va[3] = {a.x, a.y, a.z}, vb[3] = {b.x, b.y, b.z}, vc[3] = {c.x, c.y, c.z};
    unsigned long long q[3];
    for (int k = 0; k < 3; k++) {
      float mn = fminf(fminf(va[k], vb[k]), vc[k]);
      float mx = fmaxf(fmaxf(va[k], vb[k]), vc[k]);
      float u = (0.5f * (mn + mx) - lo[k]) / ext[k];
      u = fminf(fmaxf(u, 0.f), 1.f);
      q[k] = (unsigned long long)fminf(u * 2097152.f, 2097151.f);
    }
    codes[f] = (expand21(q[0]) << 2) | (expand21(q[1]) << 1) | expand21(q[2]);
    ids[f] = (int)f;
  }
}

template <class R>
__global__ void gather_tris_kernel(const float4* __restrict__ tri_tmp, const int* __restrict__ ids,
                                   long long nf, float4* __restrict__ tris,
                                   const R* __restrict__ V, const long long* __restrict__ F,
                                   double* __restrict__ tris64, int* __restrict__ slot_of) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nf;
       s += (long long)gridDim.x * blockDim.x) {
    int f = ids[s];
    slot_of[f] = (int)s;
    tris[3 * s] = tri_tmp[3 * (long long)f];
    tris[3 * s + 1] = tri_tmp[3 * (long long)f + 1];
    tris[3 * s + 2] = tri_tmp[3 * (long long)f + 2];
    if (tris64) {
      for (int a = 0; a < 3; a++) {
        long long i = F[3 * (long long)f + a];
        for (int k = 0; k < 3; k++) tris64[9 * s + 3 * a + k] = (double)V[3 * i + k];
      }
    }
  }
}

__device__ __forceinline__ int delta(const unsigned long long* __restrict__ codes, long long n,
                                     long long i, long long j) {
  if (j < 0 || j >= n) return -1;
  unsigned long long a = codes[i], b = codes[j];
  if (a == b) return 64 + __clz((int)((unsigned)i ^ (unsigned)j));
  return __clzll((long long)(a ^ b));
}

__global__ void karras_kernel(const unsigned long long* __restrict__ codes, long long n,
                              float4* __restrict__ nodes, int* __restrict__ parent,
                              int* __restrict__ leaf_parent) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n - 1;
       i += (long long)gridDim.x * blockDim.x) {
    int dl = delta(codes, n, i, i - 1), dr = delta(codes, n, i, i + 1);
    int d = (dr - dl) > 0 ? 1 : -1;
    int dmin = delta(codes, n, i, i - d);
    long long lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    long long l = 0;
    for (long long t = lmax >> 1; t >= 1; t >>= 1)
      if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    long long j = i + l * d;
    int dnode = delta(codes, n, i, j);
    long long s = 0, t = l;
    do {
      t = (t + 1) >> 1;
      if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    long long gamma = i + s * d + (d < 0 ? -1 : 0);
    long long lo = i < j ? i : j, hi = i < j ? j : i;
    int left = (lo == gamma) ? ~(int)gamma : (int)gamma;
    int right = (hi == gamma + 1) ? ~(int)(gamma + 1) : (int)(gamma + 1);
    float4* nd = nodes + 4 * i;
    nd[0].w = __int_as_float(left);
    nd[2].w = __int_as_float(right);
    if (left < 0) leaf_parent[~left] = (int)i; else parent[left] = (int)i;
    if (right < 0) leaf_parent[~right] = (int)i; else parent[right] = (int)i;
  }
}

__device__ __forceinline__ void write_child_box(float4* nd, bool is_left, float lo0, float lo1,
                                                float lo2, float hi0, float hi1, float hi2) {
  float4* lo = nd + (is_left ? 0 : 2);
  float4* hi = nd + (is_left ? 1 : 3);
  // keep .w (child index) of the lo slot
  __stcg(&lo->x, lo0); __stcg(&lo->y, lo1); __stcg(&lo->z, lo2);
  __stcg(&hi->x, hi0); __stcg(&hi->y, hi1); __stcg(&hi->z, hi2);
}

__global__ void refit_kernel(const float4* __restrict__ tris, long long n, float4* nodes,
                             const int* __restrict__ parent, const int* __restrict__ leaf_parent,
                             int* __restrict__ arrivals) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    float4 a = tris[3 * s], b = tris[3 * s + 1], c = tris[3 * s + 2];
    float lo[3] = {fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z)};
    float hi[3] = {fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z)};
    int child = ~(int)s;
    int p = leaf_parent[s];
    while (p >= 0) {
      float4* nd = nodes + 4 * (long long)p;
      bool is_left = __float_as_int(__ldcg(&nd[0].w)) == child;
      write_child_box(nd, is_left, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]);
      __threadfence();
      if (atomicAdd(&arrivals[p], 1) == 0) break;
      __threadfence();
      float4 ll = __ldcg(nd), lh = __ldcg(nd + 1), rl = __ldcg(nd + 2), rh = __ldcg(nd + 3);
      lo[0] = fminf(ll.x, rl.x); lo[1] = fminf(ll.y, rl.y); lo[2] = fminf(ll.z, rl.z);
      hi[0] = fmaxf(lh.x, rh.x); hi[1] = fmaxf(lh.y, rh.y); hi[2] = fmaxf(lh.z, rh.z);
      child = p;
      p = parent[p];
    }
  }
}

__global__ void init_scene_kernel(unsigned* scene) {
  if (threadIdx.x < 3) scene[threadIdx.x] = 0xffffffffu;
  else if (threadIdx.x < 6) scene[threadIdx.x] = 0u;
}

template <class R>
int build(const R* V, long long nv, const long long* F, long long nf, int keep_f64, void** out,
          unsigned* flags, void* stream) {
  if (nf < 0 || nv < 0 || !out) { set_error("bad arguments"); return FGB_BAD_ARG; }
  if (nf >= (1LL << 31) - 1) { set_error("too many facets for 32-bit slots"); return FGB_TOO_LARGE; }
  cudaStream_t s = as_stream(stream);
  fgb_bvh_impl* h = new fgb_bvh_impl();
  h->num_prims = nf;
  *out = h;
  if (nf == 0) return FGB_OK;
  long long ni = nf > 1 ? nf - 1 : 1;
  size_t bytes_nodes = sizeof(float4) * 4 * (size_t)ni;
  size_t bytes_tris = sizeof(float4) * 3 * (size_t)nf;
  FGB_CUDA_TRY(cudaMalloc(&h->nodes, bytes_nodes));
  FGB_CUDA_TRY(cudaMalloc(&h->tris, bytes_tris));
  FGB_CUDA_TRY(cudaMalloc(&h->slot_of, sizeof(int) * (size_t)nf));
  h->bytes = bytes_nodes + bytes_tris + sizeof(int) * (size_t)nf;
  if (keep_f64) {
    FGB_CUDA_TRY(cudaMalloc(&h->tris64, sizeof(double) * 9 * (size_t)nf));
    h->bytes += sizeof(double) * 9 * (size_t)nf;
  }
  float4* tri_tmp = nullptr;
  unsigned* scene = nullptr;
  unsigned long long *codes = nullptr, *codes_sorted = nullptr;
  int *ids = nullptr, *ids_sorted = nullptr, *parent = nullptr, *leaf_parent = nullptr,
      *arrivals = nullptr;
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
  int st = FGB_OK;
#define TRY(x) do { st = (x); if (st) goto done; } while (0)
  TRY(scratch_alloc(&tri_tmp, 3 * (size_t)nf, s));
  TRY(scratch_alloc(&scene, 6, s));
  TRY(scratch_alloc(&codes, nf, s));
  TRY(scratch_alloc(&codes_sorted, nf, s));
  TRY(scratch_alloc(&ids, nf, s));
  TRY(scratch_alloc(&ids_sorted, nf, s));
  TRY(scratch_alloc(&parent, ni, s));
  TRY(scratch_alloc(&leaf_parent, nf, s));
  TRY(scratch_alloc(&arrivals, ni, s));
  init_scene_kernel<<<1, 32, 0, s>>>(scene);
  tri_bounds_kernel<R><<<grid_for(nf, 256), 256, 0, s>>>(V, nv, F, nf, tri_tmp, scene, flags);
  morton_kernel<<<grid_for(nf, 256), 256, 0, s>>>(tri_tmp, nf, scene, codes, ids);
  cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, codes, codes_sorted, ids, ids_sorted,
                                  (int)nf, 0, 63, s);
  TRY(scratch_alloc((char**)&cub_tmp, cub_bytes, s));
  cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, codes, codes_sorted, ids, ids_sorted,
                                  (int)nf, 0, 63, s);
  gather_tris_kernel<R><<<grid_for(nf, 256), 256, 0, s>>>(tri_tmp, ids_sorted, nf, h->tris, V, F,
                                                          h->tris64, h->slot_of);
  if (nf > 1) {
    cudaMemsetAsync(parent, 0xff, sizeof(int) * ni, s);
    cudaMemsetAsync(arrivals, 0, sizeof(int) * ni, s);
    karras_kernel<<<grid_for(ni, 256), 256, 0, s>>>(codes_sorted, nf, h->nodes, parent, leaf_parent);
    refit_kernel<<<grid_for(nf, 256), 256, 0, s>>>(h->tris, nf, h->nodes, parent, leaf_parent, arrivals);
  }
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_status(e, "lbvh build");
  }
done:
#undef TRY
  scratch_free(tri_tmp, s);
  scratch_free(scene, s);
  scratch_free(codes, s);
  scratch_free(codes_sorted, s);
  scratch_free(ids, s);
  scratch_free(ids_sorted, s);
  scratch_free(parent, s);
  scratch_free(leaf_parent, s);
  scratch_free(arrivals, s);
  scratch_free(cub_tmp, s);
  return st;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_bvh_build_f64(const double* V, long long nv, const long long* F, long long nf, int keep_f64,
                      void** out_bvh, unsigned* flags, void* stream) {
  return fgb::build<double>(V, nv, F, nf, keep_f64, out_bvh, flags, stream);
}

int fgb_bvh_build_f32(const float* V, long long nv, const long long* F, long long nf, int keep_f64,
                      void** out_bvh, unsigned* flags, void* stream) {
  return fgb::build<float>(V, nv, F, nf, keep_f64, out_bvh, flags, stream);
}

int fgb_bvh_free(void* bvh) {
  if (!bvh) return FGB_OK;
  fgb_bvh_impl* h = static_cast<fgb_bvh_impl*>(bvh);
  cudaFree(h->nodes);
  cudaFree(h->tris);
  cudaFree(h->tris64);
  cudaFree(h->slot_of);
  delete h;
  return FGB_OK;
}

int fgb_bvh_info(const void* bvh, long long* num_prims, long long* bytes) {
  if (!bvh) { fgb::set_error("null bvh"); return FGB_BAD_ARG; }
  const fgb_bvh_impl* h = static_cast<const fgb_bvh_impl*>(bvh);
  if (num_prims) *num_prims = h->num_prims;
  if (bytes) *bytes = (long long)h->bytes;
  return FGB_OK;
}

}  // extern "C"
