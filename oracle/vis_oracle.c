/*
 * ORACLE (test infrastructure only; never linked into the product library).
 *
 * CPU restatement of the reference's ray-cast visibility and form-factor
 * assembly:
 *   Embree backend   src/flux/shape.py:349-421 (pair visibility: forced
 *                    visible within eps, origin offset eps along the unit
 *                    direction, closest hit must be j; sun: origin offset
 *                    eps along N, any hit occludes)
 *   CGAL backend     src/flux/cgal/aabb_wrapper.cpp:64-108 with the loops of
 *                    src/flux/cgal/aabb.pyx:58-87 (FP64 rays from the face
 *                    centroid, source face skipped, first hit must be j)
 *   form factors     src/flux/form_factors.py:11-72
 * The visibility backends themselves (Embree 3.13.2 via python-embree, CGAL
 * 5.3) are third-party and absent; their published semantics are restated
 * with the watertight ray/triangle test of Woop, Benthin & Wald (JCGT 2013)
 * in FP32 (Embree stores float32 vertices, shape.py:316-323) or FP64 (CGAL).
 * Occlusion decisions do not depend on traversal order, so this simple
 * median-split BVH gives the same answers as any other BVH.
 * Compiled with -ffp-contract=off; every expression is evaluated in the same
 * order as the GPU kernels (fluxpy_gb300/csrc/bvh.cuh, visibility.cuh,
 * formfactor.cu), which makes the two bit-identical.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EMBREE_EPS_F64 0.0010000000474974513
#define NEAR_EDGE_REL 1e-6f
#define LEAF_SIZE 4

typedef struct {
  float lo[3], hi[3];
  int left, right; /* children, or -1 */
  int start, count; /* leaf range in order[] when count > 0 */
} bnode;

typedef struct {
  int nf;
  float *v32;   /* nf x 9 */
  double *v64;  /* nf x 9 */
  int *order;
  bnode *nodes;
  int num_nodes;
} obvh;

static void tri_box(const obvh *b, int f, float *lo, float *hi) {
  const float *v = b->v32 + 9 * (size_t)f;
  for (int k = 0; k < 3; k++) {
    float a = v[k], c = v[3 + k], d = v[6 + k];
    lo[k] = fminf(fminf(a, c), d);
    hi[k] = fmaxf(fmaxf(a, c), d);
  }
}

static int cmp_axis;
static const obvh *cmp_bvh;
static float centroid(const obvh *b, int f, int k) {
  const float *v = b->v32 + 9 * (size_t)f;
  return (v[k] + v[3 + k] + v[6 + k]) / 3.0f;
}
static int cmp_fn(const void *x, const void *y) {
  float a = centroid(cmp_bvh, *(const int *)x, cmp_axis), c = centroid(cmp_bvh, *(const int *)y, cmp_axis);
  return (a < c) ? -1 : (a > c) ? 1 : 0;
}

static int build_rec(obvh *b, int start, int count) {
  int id = b->num_nodes++;
  bnode *n = &b->nodes[id];
  for (int k = 0; k < 3; k++) { n->lo[k] = INFINITY; n->hi[k] = -INFINITY; }
  for (int q = start; q < start + count; q++) {
    float lo[3], hi[3];
    tri_box(b, b->order[q], lo, hi);
    for (int k = 0; k < 3; k++) {
      if (lo[k] < n->lo[k]) n->lo[k] = lo[k];
      if (hi[k] > n->hi[k]) n->hi[k] = hi[k];
    }
  }
  if (count <= LEAF_SIZE) {
    n->left = n->right = -1;
    n->start = start;
    n->count = count;
    return id;
  }
  int axis = 0;
  float ext = n->hi[0] - n->lo[0];
  for (int k = 1; k < 3; k++) if (n->hi[k] - n->lo[k] > ext) { ext = n->hi[k] - n->lo[k]; axis = k; }
  cmp_axis = axis;
  cmp_bvh = b;
  qsort(b->order + start, count, sizeof(int), cmp_fn);
  int half = count / 2;
  n->count = 0;
  int l = build_rec(b, start, half);
  int r = build_rec(b, start + half, count - half);
  b->nodes[id].left = l;
  b->nodes[id].right = r;
  return id;
}

void *oracle_bvh_build(const double *V, long long nv, const long long *F, long long nf) {
  obvh *b = calloc(1, sizeof(obvh));
  b->nf = (int)nf;
  b->v32 = malloc(sizeof(float) * 9 * (size_t)(nf ? nf : 1));
  b->v64 = malloc(sizeof(double) * 9 * (size_t)(nf ? nf : 1));
  b->order = malloc(sizeof(int) * (size_t)(nf ? nf : 1));
  for (long long f = 0; f < nf; f++) {
    for (int a = 0; a < 3; a++) {
      long long i = F[3 * f + a];
      if (i < 0 || i >= nv) i = 0;
      for (int k = 0; k < 3; k++) {
        b->v64[9 * f + 3 * a + k] = V[3 * i + k];
        b->v32[9 * f + 3 * a + k] = (float)V[3 * i + k];
      }
    }
    b->order[f] = (int)f;
  }
  b->nodes = malloc(sizeof(bnode) * (size_t)(2 * nf + 1));
  b->num_nodes = 0;
  if (nf > 0) build_rec(b, 0, (int)nf);
  return b;
}

void oracle_bvh_free(void *h) {
  obvh *b = h;
  if (!b) return;
  free(b->v32);
  free(b->v64);
  free(b->order);
  free(b->nodes);
  free(b);
}

/* ------------------------------------------------------------ FP32 rays -- */
typedef struct {
  float o[3], d[3], inv[3];
  int kx, ky, kz;
  float Sx, Sy, Sz;
} ray32;

static void make_ray(ray32 *r, const float *o, const float *d) {
  for (int k = 0; k < 3; k++) { r->o[k] = o[k]; r->d[k] = d[k]; r->inv[k] = 1.0f / d[k]; }
  float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > (kz == 0 ? ax : ay)) kz = 2;
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (d[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
  r->kx = kx; r->ky = ky; r->kz = kz;
  r->Sx = d[kx] / d[kz];
  r->Sy = d[ky] / d[kz];
  r->Sz = 1.0f / d[kz];
}

static int box_hit(const ray32 *r, const float *lo, const float *hi, float tmax) {
  float tn = 0.0f, tf = INFINITY;
  for (int k = 0; k < 3; k++) {
    float t0 = (lo[k] - r->o[k]) * r->inv[k], t1 = (hi[k] - r->o[k]) * r->inv[k];
    float a = fminf(t0, t1), c = fmaxf(t0, t1);
    if (a == a && a > tn) tn = a;
    if (c == c && c < tf) tf = c;
  }
  tf *= 1.0000004f;
  return tn <= tf && tn <= tmax * 1.0000004f;
}

typedef struct { int hit; float t; int near_edge; } trihit;

static trihit tri_test(const ray32 *r, const float *v, float tmax) {
  trihit h = {0, 0.0f, 0};
  int kx = r->kx, ky = r->ky, kz = r->kz;
  float A[3], B[3], C[3];
  for (int k = 0; k < 3; k++) {
    A[k] = v[k] - r->o[k];
    B[k] = v[3 + k] - r->o[k];
    C[k] = v[6 + k] - r->o[k];
  }
  float Ax = A[kx] - r->Sx * A[kz];
  float Ay = A[ky] - r->Sy * A[kz];
  float Bx = B[kx] - r->Sx * B[kz];
  float By = B[ky] - r->Sy * B[kz];
  float Cx = C[kx] - r->Sx * C[kz];
  float Cy = C[ky] - r->Sy * C[kz];
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  int outside = (U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f);
  float det = U + V + W;
  if (det == 0.0f) return h;
  float sU = det > 0.0f ? U : -U, sV = det > 0.0f ? V : -V, sW = det > 0.0f ? W : -W;
  float lim = NEAR_EDGE_REL * fabsf(det);
  int near;
  if (!outside) near = fminf(fminf(sU, sV), sW) < lim;
  else near = fmaxf(fmaxf(-sU, -sV), -sW) < lim;
  if (outside && !near) return h;
  float Az = r->Sz * A[kz], Bz = r->Sz * B[kz], Cz = r->Sz * C[kz];
  float T = U * Az + V * Bz + W * Cz;
  float t = T / det;
  if (near && t > 0.0f && t <= tmax) h.near_edge = 1;
  if (outside) return h;
  if (!(t > 0.0f && t < tmax)) return h;
  h.hit = 1;
  h.t = t;
  return h;
}

/* any hit with t in (0, tmax), skipping two facets */
static int any_hit(const obvh *b, const ray32 *r, float tmax, int s0, int s1, int *near_edge) {
  if (b->nf <= 0) return 0;
  int stack[256];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const bnode *n = &b->nodes[stack[--sp]];
    if (!box_hit(r, n->lo, n->hi, tmax)) continue;
    if (n->count > 0) {
      for (int q = n->start; q < n->start + n->count; q++) {
        int f = b->order[q];
        if (f == s0 || f == s1) continue;
        trihit h = tri_test(r, b->v32 + 9 * (size_t)f, tmax);
        if (h.near_edge) *near_edge = 1;
        if (h.hit) return 1;
      }
    } else {
      stack[sp++] = n->right;
      stack[sp++] = n->left;
    }
  }
  return 0;
}

/* ------------------------------------------------------------ FP64 rays -- */
typedef struct {
  double o[3], d[3];
  int kx, ky, kz;
  double Sx, Sy, Sz;
} ray64;

static void make_ray64(ray64 *r, const double *o, const double *d) {
  for (int k = 0; k < 3; k++) { r->o[k] = o[k]; r->d[k] = d[k]; }
  double ax = fabs(d[0]), ay = fabs(d[1]), az = fabs(d[2]);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > (kz == 0 ? ax : ay)) kz = 2;
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (d[kz] < 0.0) { int t = kx; kx = ky; ky = t; }
  r->kx = kx; r->ky = ky; r->kz = kz;
  r->Sx = d[kx] / d[kz];
  r->Sy = d[ky] / d[kz];
  r->Sz = 1.0 / d[kz];
}

static int tri_test64(const ray64 *r, const double *v, double tmax, double *t_out) {
  int kx = r->kx, ky = r->ky, kz = r->kz;
  double A[3], B[3], C[3];
  for (int k = 0; k < 3; k++) {
    A[k] = v[k] - r->o[k];
    B[k] = v[3 + k] - r->o[k];
    C[k] = v[6 + k] - r->o[k];
  }
  double Ax = A[kx] - r->Sx * A[kz], Ay = A[ky] - r->Sy * A[kz];
  double Bx = B[kx] - r->Sx * B[kz], By = B[ky] - r->Sy * B[kz];
  double Cx = C[kx] - r->Sx * C[kz], Cy = C[ky] - r->Sy * C[kz];
  double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if ((U < 0.0 || V < 0.0 || W < 0.0) && (U > 0.0 || V > 0.0 || W > 0.0)) return 0;
  double det = U + V + W;
  if (det == 0.0) return 0;
  double T = U * (r->Sz * A[kz]) + V * (r->Sz * B[kz]) + W * (r->Sz * C[kz]);
  double t = T / det;
  if (!(t > 0.0 && t < tmax)) return 0;
  *t_out = t;
  return 1;
}

static int box_hit64(const ray64 *r, const float *lo, const float *hi, double tmax) {
  double tn = 0.0, tf = INFINITY;
  for (int k = 0; k < 3; k++) {
    double l = (double)lo[k] - 1e-6 * fabs((double)lo[k]) - 1e-30;
    double h = (double)hi[k] + 1e-6 * fabs((double)hi[k]) + 1e-30;
    double inv = 1.0 / r->d[k];
    double t0 = (l - r->o[k]) * inv, t1 = (h - r->o[k]) * inv;
    double a = fmin(t0, t1), c = fmax(t0, t1);
    if (a == a && a > tn) tn = a;
    if (c == c && c < tf) tf = c;
  }
  tf = tf * 1.00001 + 1e-30;
  return tn <= tf && tn <= tmax * 1.0001 + 1e-30;
}

static int first_hit64(const obvh *b, const ray64 *r, int s0, int s1, double tmax, int any_only,
                       double *t_out) {
  if (b->nf <= 0) return -1;
  int stack[256];
  int sp = 0;
  stack[sp++] = 0;
  double best = tmax;
  int best_f = -1;
  while (sp) {
    const bnode *n = &b->nodes[stack[--sp]];
    if (!box_hit64(r, n->lo, n->hi, best)) continue;
    if (n->count > 0) {
      for (int q = n->start; q < n->start + n->count; q++) {
        int f = b->order[q];
        if (f == s0 || f == s1) continue;
        double t;
        if (tri_test64(r, b->v64 + 9 * (size_t)f, best, &t)) {
          best = t;
          best_f = f;
          if (any_only) { *t_out = best; return best_f; }
        }
      }
    } else {
      stack[sp++] = n->right;
      stack[sp++] = n->left;
    }
  }
  *t_out = best;
  return best_f;
}

static void centroid64(const obvh *b, int f, double *c) {
  const double *v = b->v64 + 9 * (size_t)f;
  for (int k = 0; k < 3; k++) c[k] = (v[k] + v[3 + k] + v[6 + k]) / 3.0;
}

/* ------------------------------------------------------ predicates ------- */
static int pair_visible(const obvh *b, const double *P, int i, int j, int sem, int *near_edge) {
  if (sem == 1) {
    if (i == j) return 0;
    double ci[3], cj[3], d[3];
    centroid64(b, i, ci);
    centroid64(b, j, cj);
    for (int k = 0; k < 3; k++) d[k] = cj[k] - ci[k];
    ray64 r;
    make_ray64(&r, ci, d);
    double tj, t;
    if (!tri_test64(&r, b->v64 + 9 * (size_t)j, INFINITY, &tj)) return 0;
    return first_hit64(b, &r, i, j, tj, 1, &t) < 0;
  }
  const double eps = EMBREE_EPS_F64;
  double pi[3] = {P[3 * i], P[3 * i + 1], P[3 * i + 2]};
  double d[3] = {P[3 * j] - pi[0], P[3 * j + 1] - pi[1], P[3 * j + 2] - pi[2]};
  double dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (!(dn > eps)) return 1;
  float o[3], dir[3];
  for (int k = 0; k < 3; k++) {
    double dh = d[k] / dn;
    o[k] = (float)(pi[k] + eps * dh);
    dir[k] = (float)dh;
  }
  ray32 r;
  make_ray(&r, o, dir);
  trihit hj = tri_test(&r, b->v32 + 9 * (size_t)j, INFINITY);
  if (!hj.hit) return 0;
  return any_hit(b, &r, hj.t, j, -1, near_edge) == 0;
}

static int sun_occluded(const obvh *b, const double *P, const double *N, int i, const double *D,
                        int sem) {
  if (sem == 1) {
    double ci[3];
    centroid64(b, i, ci);
    ray64 r;
    make_ray64(&r, ci, D);
    double t;
    return first_hit64(b, &r, i, -1, INFINITY, 1, &t) >= 0;
  }
  float o[3], dir[3];
  for (int k = 0; k < 3; k++) {
    o[k] = (float)(P[3 * i + k] + EMBREE_EPS_F64 * N[3 * i + k]);
    dir[k] = (float)D[k];
  }
  ray32 r;
  make_ray(&r, o, dir);
  int ne = 0;
  return any_hit(b, &r, INFINITY, -1, -1, &ne) != 0;
}

/* vis[p*n+q] for (I[p], J[q]) (or vis[p] for pairs when paired). */
void oracle_visibility(void *h, const double *P, const long long *I, long long m,
                       const long long *J, long long n, int paired, int sem, uint8_t *vis,
                       uint8_t *near_edge) {
  const obvh *b = h;
  long long total = paired ? m : m * n;
#pragma omp parallel for schedule(dynamic, 256)
  for (long long q = 0; q < total; q++) {
    long long i = paired ? I[q] : I[q / n];
    long long j = paired ? J[q] : J[q % n];
    int ne = 0;
    vis[q] = (uint8_t)pair_visible(b, P, (int)i, (int)j, sem, &ne);
    if (near_edge) near_edge[q] = (uint8_t)ne;
  }
}

void oracle_occluded(void *h, const double *P, const double *N, const long long *I, long long m,
                     const double *D, long long ndirs, int per_facet, int sem, uint8_t *occ) {
  const obvh *b = h;
  long long total = per_facet ? m : m * ndirs;
#pragma omp parallel for schedule(dynamic, 256)
  for (long long q = 0; q < total; q++) {
    long long p = per_facet ? q : q / ndirs;
    long long k = per_facet ? q : q % ndirs;
    occ[q] = (uint8_t)sun_occluded(b, P, N, (int)I[p], D + 3 * k, sem);
  }
}

/* ---------------------------------------------------- form factors ------- */
/* Numerator of get_form_factor_matrix (form_factors.py:46-47):
 *   max(0, N_i.(P_j - P_i)) * max(0, P_i.N_j - N_j.P_j)
 * dot products summed left to right. */
static double ff_num(const double *P, const double *N, long long i, long long j) {
  double d0 = P[3 * j] - P[3 * i], d1 = P[3 * j + 1] - P[3 * i + 1], d2 = P[3 * j + 2] - P[3 * i + 2];
  double a = N[3 * i] * d0 + N[3 * i + 1] * d1 + N[3 * i + 2] * d2;
  double pn = P[3 * i] * N[3 * j] + P[3 * i + 1] * N[3 * j + 1] + P[3 * i + 2] * N[3 * j + 2];
  double np = N[3 * j] * P[3 * j] + N[3 * j + 1] * P[3 * j + 1] + N[3 * j + 2] * P[3 * j + 2];
  double bb = pn - np;
  if (a < 0.0) a = 0.0;
  if (bb < 0.0) bb = 0.0;
  return a * bb;
}

static double ff_value(const double *P, const double *A, long long i, long long j, double num) {
  double e0 = P[3 * i] - P[3 * j], e1 = P[3 * i + 1] - P[3 * j + 1], e2 = P[3 * i + 2] - P[3 * j + 2];
  double sq = e0 * e0 + e1 * e1 + e2 * e2;
  double s = 3.141592653589793 * (sq * sq);
  if (s == 0.0) s = INFINITY;
  return num * A[j] / s;
}

/* Dense form-factor block F[p*n+q] = F(I[p], J[q]) and per-pair flags:
 * kept[p*n+q] = 1 when the pair passed the orientation threshold and went
 * to the visibility test (bit 0), visible (bit 1), near edge (bit 2). */
void oracle_ff_dense(void *h, const double *P, const double *N, const double *A,
                     const long long *I, long long m, const long long *J, long long n, double eps,
                     int sem, double *Fout, uint8_t *info) {
  const obvh *b = h;
#pragma omp parallel for schedule(dynamic, 4)
  for (long long p = 0; p < m; p++) {
    long long i = I[p];
    for (long long q = 0; q < n; q++) {
      long long j = J[q];
      double num = (i == j) ? 0.0 : ff_num(P, N, i, j);
      double v = 0.0;
      uint8_t fl = 0;
      if (fabs(num) > eps) {
        int ne = 0;
        fl |= 1;
        if (pair_visible(b, P, (int)i, (int)j, sem, &ne)) {
          fl |= 2;
          v = ff_value(P, A, i, j, num);
        }
        if (ne) fl |= 4;
      }
      Fout[p * n + q] = v;
      if (info) info[p * n + q] = fl;
    }
  }
}

/* Exact rows of the form-factor matrix for sampled rows I (all columns
 * 0..nf-1), written densely: out[p*nf + j]. */
void oracle_ff_rows(void *h, const double *P, const double *N, const double *A,
                    const long long *I, long long m, double eps, int sem, double *out) {
  const obvh *b = h;
  long long nf = b->nf;
#pragma omp parallel for schedule(dynamic, 1024)
  for (long long q = 0; q < m * nf; q++) {
    long long i = I[q / nf], j = q % nf;
    double num = (i == j) ? 0.0 : ff_num(P, N, i, j);
    double v = 0.0;
    if (fabs(num) > eps) {
      int ne = 0;
      if (pair_visible(b, P, (int)i, (int)j, sem, &ne)) v = ff_value(P, A, i, j, num);
    }
    out[q] = v;
  }
}
