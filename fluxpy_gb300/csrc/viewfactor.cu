// Exact view factor between two planar triangles, one pair per thread, FP64.
//
// Replaces the reference's ff_narayanaswamy_impl
// (src/flux/view_factor/view_factor_narayanaswamy.c:338-494, bound as
// flux.view_factor.ff_narayanaswamy by view_factor.pyx), which evaluates the
// closed form of Narayanaswamy, "An analytic expression for radiation view
// factor between two arbitrarily oriented planar polygons", Int. J. Heat
// Mass Transfer 91 (2015) 841-847.  The method: by Stokes' theorem the
// double area integral of cos(t1) cos(t2) / (pi r^2) becomes a double contour
// integral over the two boundaries, a sum over pairs of edges (one of each
// triangle) of
//     (u . v) [G(s_j, l_q) - G(s_i, l_q) - G(s_j, l_p) + G(s_i, l_p)]
// where u, v are the edge directions, s and l the endpoints' coordinates
// along the two edge lines measured from the lines' closest points, and G
// the antiderivative of the method (Eq. 22b for skew lines, with the
// imaginary part of the dilogarithm written through the Clausen function,
// Eq. 24 and Eq. 26; Eq. 23 for parallel lines).  Area A's view factor of B
// is |sum| / (4 pi area_A).
//
// As in the reference, a vertex of B closer than 0.5e-13 to an endpoint of
// A's edge is moved by 1e-13 along (1, 1, 1) for that edge pair (shared
// vertices make G singular), the logarithms are regularised by 1e-13, and
// lines are parallel when 1 - (u . v)^2 <= 1e-13.  The Clausen function uses
// the method's Chebyshev expansion (its published coefficients), evaluated
// here by the three-term recurrence of the odd Chebyshev polynomials.
//
// The near-field correction (fgb_ff_adjacent_fix_f64) applies it to the
// entries of a form-factor CSR whose two facets share a vertex, where the
// midpoint rule of get_form_factor_matrix (1 / r^2 at the centroids) is
// least accurate.
#include "common.cuh"

namespace fgb {
namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTiny = 1e-13;
constexpr double kCoincident = 0.5e-13;

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double len(D3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ D3 unit(D3 a) { return (1.0 / len(a)) * a; }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Clausen's function Cl_2(theta) for theta >= 0: the closed part plus the
// Chebyshev series in x = theta / pi - 1 (odd polynomials T_1 ... T_13).
__device__ double clausen(double theta) {
  constexpr double kB[7] = {1.865555351433979e-1, 6.269948963579612e-2, 3.139559104552675e-4,
                            3.916780537368088e-6, 6.499672439854756e-8, 1.238143696612060e-9,
                            5.586505893753557e-13};
  theta = fmod(theta, 2.0 * kPi);
  const double x = theta / kPi - 1.0;
  // odd Chebyshev polynomials: T_{k+2} = 2 (2 x^2 - 1) T_k - T_{k-2}, T_{-1} = T_1 = x
  const double c = 2.0 * (2.0 * x * x - 1.0);
  double t_prev = x, t = x;
  double series = kB[0] * t;
#pragma unroll
  for (int k = 1; k < 7; k++) {
    const double t_next = c * t - t_prev;
    t_prev = t;
    t = t_next;
    series += kB[k] * t;
  }
  const double two_pi = 2.0 * kPi;
  return (theta - kPi) * (2.0 + log(kPi * kPi / 2.0)) +
         (two_pi - theta) * log((two_pi - theta) * (1.0 - kTiny) + kTiny) -
         theta * log(theta * (1.0 - kTiny) + kTiny) + series;
}

// Im Li_2(r e^{i phi}) for r >= 0 (Eq. 24 of the method).
__device__ double im_dilog(double r, double phi) {
  if (!(r > kTiny)) return r * sin(phi);
  const double omega = atan2(r * sin(phi), 1.0 - r * cos(phi));
  return 0.5 * (clausen(2.0 * phi) + clausen(2.0 * omega) - clausen(2.0 * omega + 2.0 * phi)) +
         log(r) * omega;
}

// Antiderivative for skew edge lines at distance d, angle alpha (Eq. 22b).
__device__ double g_skew(double s, double l, double alpha, double ca, double sa, double d) {
  const double s2 = s * s, l2 = l * l, d2 = d * d, sa2 = sa * sa;
  const double ws = sqrt(s2 + d2 / sa2);
  const double ps = sqrt(l2 + d2 / sa2);
  const double wd = fabs(s + ws) > 0.0 ? s + ws : kTiny;
  const double pd = fabs(l + ps) > 0.0 ? l + ps : kTiny;
  const double logs = (0.5 * ca * (s2 + l2) - s * l) * log(s2 + l2 - 2.0 * s * l * ca + d2);
  const double at1 = s * sa * ws * atan2(sqrt(s2 * sa2 + d2), l - s * ca);
  const double at2 = l * sa * ps * atan2(sqrt(l2 * sa2 + d2), s - l * ca);
  const double dil = im_dilog(wd / pd, alpha) + im_dilog(pd / wd, alpha) -
                     2.0 * im_dilog((wd - 2.0 * s) / pd, kPi - alpha);
  return logs + at1 + at2 + s * l + 0.5 * (d2 / sa) * dil;
}

// Antiderivative for parallel edge lines at distance d (Eq. 23).
__device__ double g_parallel(double s, double l, double d) {
  if (d == 0.0) d = kTiny;
  const double sl = s - l, d2 = d * d;
  double c = sl / sqrt(s * s + l * l - 2.0 * s * l + d2);
  c = fmin(1.0, fmax(-1.0, c));
  return 0.5 * (sl * sl - d2) * log(sl * sl + d2) - 2.0 * sl * d * acos(c) + s * l;
}

// The contribution of edge a0->a1 of triangle A and edge b0->b1 of B.
__device__ double edge_pair(D3 a0, D3 a1, D3 b0, D3 b1) {
  // closest points of the two lines (a0 + s u, b0 + t v, u and v unit)
  D3 u = unit(a1 - a0), v = unit(b1 - b0);
  const D3 w = a0 - b0;
  const double uv = dot(u, v), uw = dot(u, w), vw = dot(v, w);
  const double den = 1.0 - uv * uv;
  const bool skew = den > kTiny;
  double s0, t0;
  if (skew) {
    s0 = (uv * vw - uw) / den;
    t0 = (vw - uv * uw) / den;
  } else {
    s0 = 0.0;
    t0 = vw;
  }
  const D3 sorg = a0 + s0 * u, torg = b0 + t0 * v;
  const D3 gap = w + s0 * u - t0 * v;
  const double dmin = sqrt(fmax(0.0, dot(gap, gap)));
  // coordinates along each line measured from its closest point, pointing
  // towards the farther endpoint
  const D3 sh = unit(fabs(s0) < len(a1 - sorg) ? a1 - sorg : a0 - sorg);
  D3 th = unit(fabs(t0) < len(b1 - torg) ? b1 - torg : b0 - torg);
  if (!skew) th = sh;
  const double si = dot(a0, sh) - dot(sorg, sh), sj = dot(a1, sh) - dot(sorg, sh);
  const double lp = dot(b0, th) - dot(torg, th), lq = dot(b1, th) - dot(torg, th);
  const double ca = dot(sh, th);
  if (skew) {
    const double alpha = acos(ca);
    const double sa = sin(alpha);
    return ca * (g_skew(sj, lq, alpha, ca, sa, dmin) - g_skew(si, lq, alpha, ca, sa, dmin) -
                 g_skew(sj, lp, alpha, ca, sa, dmin) + g_skew(si, lp, alpha, ca, sa, dmin));
  }
  return ca * (g_parallel(sj, lq, dmin) - g_parallel(si, lq, dmin) - g_parallel(sj, lp, dmin) +
               g_parallel(si, lp, dmin));
}

// View factor of triangle A (vertices a[3]) towards triangle B.
__device__ double tri_view_factor(const D3* a, const D3* b, bool* nonfinite) {
  const double area_a = 0.5 * len(cross(a[1] - a[0], a[2] - a[0]));
  double sum = 0.0;
  for (int p = 0; p < 3; p++) {
    for (int i = 0; i < 3; i++) {
      const D3 ai = a[i], aj = a[(i + 1) % 3];
      D3 bp = b[p], bq = b[(p + 1) % 3];
      const D3 nudge = {kTiny, kTiny, kTiny};
      if (len(ai - bp) < kCoincident || len(aj - bp) < kCoincident)
        bp = bp + nudge;
      else if (len(ai - bq) < kCoincident || len(aj - bq) < kCoincident)
        bq = bq + nudge;
      sum += edge_pair(ai, aj, bp, bq);
    }
  }
  const double F = fabs(sum) / (4.0 * kPi * area_a);
  if (!isfinite(F)) *nonfinite = true;
  return F;
}

__device__ __forceinline__ D3 load3(const double* p) { return {p[0], p[1], p[2]}; }

__global__ void view_factor_kernel(const double* __restrict__ tri1,
                                   const double* __restrict__ tri2, long long n,
                                   double* __restrict__ out, unsigned* flags) {
  bool bad = false;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    D3 a[3], b[3];
    for (int k = 0; k < 3; k++) {
      a[k] = load3(tri1 + 9 * q + 3 * k);
      b[k] = load3(tri2 + 9 * q + 3 * k);
    }
    out[q] = tri_view_factor(a, b, &bad);
  }
  if (bad) atomicOr(flags, kFlagNonfiniteOut);
}

// Entries of a CSR over facet pairs (row r is facet rows[r], entry e is
// facet cols[indices[e]]) whose facets share a vertex get the exact value.
__global__ void adjacent_fix_kernel(const double* __restrict__ V, const long long* __restrict__ F,
                                    const long long* __restrict__ rows,
                                    const long long* __restrict__ cols, long long nrows,
                                    const long long* __restrict__ indptr,
                                    const int* __restrict__ indices, double* __restrict__ data,
                                    unsigned long long* __restrict__ fixed, unsigned* flags) {
  bool bad = false;
  unsigned long long count = 0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nrows;
       r += (long long)gridDim.x * blockDim.x) {
    const long long fi = rows[r];
    const long long vi0 = F[3 * fi], vi1 = F[3 * fi + 1], vi2 = F[3 * fi + 2];
    for (long long e = indptr[r]; e < indptr[r + 1]; e++) {
      const long long fj = cols[indices[e]];
      const long long vj0 = F[3 * fj], vj1 = F[3 * fj + 1], vj2 = F[3 * fj + 2];
      const bool shared = vj0 == vi0 || vj0 == vi1 || vj0 == vi2 || vj1 == vi0 ||
                          vj1 == vi1 || vj1 == vi2 || vj2 == vi0 || vj2 == vi1 || vj2 == vi2;
      if (!shared || fj == fi) continue;
      const D3 a[3] = {load3(V + 3 * vi0), load3(V + 3 * vi1), load3(V + 3 * vi2)};
      const D3 b[3] = {load3(V + 3 * vj0), load3(V + 3 * vj1), load3(V + 3 * vj2)};
      data[e] = tri_view_factor(a, b, &bad);
      count++;
    }
  }
  if (count) atomicAdd(fixed, count);
  if (bad) atomicOr(flags, kFlagNonfiniteOut);
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_ff_triangles_f64(const double* tri1, const double* tri2, long long n, double* out,
                         unsigned* flags, void* stream) {
  if (n < 0) { fgb::set_error("n must be >= 0"); return FGB_BAD_ARG; }
  if (n == 0) return FGB_OK;
  if (!tri1 || !tri2 || !out || !flags) { fgb::set_error("null pointer"); return FGB_BAD_ARG; }
  fgb::view_factor_kernel<<<fgb::grid_for(n, 128, 152LL * 64), 128, 0, fgb::as_stream(stream)>>>(
      tri1, tri2, n, out, flags);
  FGB_LAUNCH_CHECK("view_factor_kernel");
  return FGB_OK;
}

int fgb_ff_adjacent_fix_f64(const double* V, const long long* F, const long long* rows,
                            const long long* cols, long long nrows, const long long* indptr,
                            const int* indices, double* data, unsigned long long* fixed,
                            unsigned* flags, void* stream) {
  if (nrows < 0) { fgb::set_error("nrows must be >= 0"); return FGB_BAD_ARG; }
  if (nrows == 0) return FGB_OK;
  if (!V || !F || !rows || !cols || !indptr || !indices || !data || !fixed || !flags) {
    fgb::set_error("null pointer");
    return FGB_BAD_ARG;
  }
  fgb::adjacent_fix_kernel<<<fgb::grid_for(nrows, 128, 152LL * 64), 128, 0,
                             fgb::as_stream(stream)>>>(V, F, rows, cols, nrows, indptr, indices,
                                                        data, fixed, flags);
  FGB_LAUNCH_CHECK("adjacent_fix_kernel");
  return FGB_OK;
}

}  // extern "C"
