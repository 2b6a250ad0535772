// One form-factor entry, as get_form_factor_matrix defines it
// (src/flux/form_factors.py:46-64):
//   num = max(0, N_i.(P_j - P_i)) * max(0, P_i.N_j - N_j.P_j)
//   kept when i != j and |num| > eps (eps = 1e-5 absolute, config.py:2)
//   visible per the backend semantics (visibility.cuh)
//   F_ij = num * A_j / (pi * |P_i - P_j|^4)      (s == 0 -> F = 0)
// Dot products are summed left to right with the _rn intrinsics; the CPU
// oracle uses the same order, so entries are bit-identical to it.
#pragma once
#include "visibility.cuh"

namespace fgb {

template <class R>
__device__ __forceinline__ R ff_num(const R* __restrict__ P, const R* __restrict__ N, long long i,
                                    long long j) {
  R d0 = fsub(P[3 * j], P[3 * i]), d1 = fsub(P[3 * j + 1], P[3 * i + 1]),
    d2 = fsub(P[3 * j + 2], P[3 * i + 2]);
  R a = dot3(N[3 * i], N[3 * i + 1], N[3 * i + 2], d0, d1, d2);
  R pn = dot3(P[3 * i], P[3 * i + 1], P[3 * i + 2], N[3 * j], N[3 * j + 1], N[3 * j + 2]);
  R np_ = dot3(N[3 * j], N[3 * j + 1], N[3 * j + 2], P[3 * j], P[3 * j + 1], P[3 * j + 2]);
  R b = fsub(pn, np_);
  if (a < R(0)) a = R(0);
  if (b < R(0)) b = R(0);
  return fmul(a, b);
}

template <class R> struct PiConst;
template <> struct PiConst<double> { static constexpr double v = 3.141592653589793; };
template <> struct PiConst<float> { static constexpr float v = 3.14159265358979f; };

template <class R>
__device__ __forceinline__ R ff_value(const R* __restrict__ P, const R* __restrict__ A, long long i,
                                      long long j, R num) {
  R e0 = fsub(P[3 * i], P[3 * j]), e1 = fsub(P[3 * i + 1], P[3 * j + 1]),
    e2 = fsub(P[3 * i + 2], P[3 * j + 2]);
  R sq = fadd(fadd(fmul(e0, e0), fmul(e1, e1)), fmul(e2, e2));
  R s = fmul(PiConst<R>::v, fmul(sq, sq));
  if (s == R(0)) return R(0);
  return fdiv(fmul(num, A[j]), s);
}

// Full entry with visibility.  *kept: passed the orientation threshold;
// *near_edge: the visibility ray passed within the near-edge margin.
template <class R>
__device__ __forceinline__ R ff_entry(const BvhView& b, const R* __restrict__ P, const R* __restrict__ N,
                                      const R* __restrict__ A, long long i, long long j, R eps,
                                      int sem, bool* kept, bool* near_edge, bool* overflow) {
  *kept = false;
  if (i == j) return R(0);
  R num = ff_num(P, N, i, j);
  if (!(fabs(num) > eps)) return R(0);
  *kept = true;
  if (!pair_visible<R>(b, P, (int)i, (int)j, sem, near_edge, overflow)) return R(0);
  return ff_value(P, A, i, j, num);
}

}  // namespace fgb
