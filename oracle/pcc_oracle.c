/*
 * ORACLE (test infrastructure only; never linked into the product library).
 *
 * CPU restatement of the reference's per-facet 1-D conduction step:
 *   conductionQ  src/flux/pcc/conductionQ.c:10-186
 *   conductionT  src/flux/pcc/conductionT.c:4-88
 *   tridag       src/flux/pcc/tridag.c:5-34
 * and of the facet loop in PccThermalModel1D.step (src/flux/thermal.pyx:236-299).
 *
 * Differences from the reference, none of which change results:
 *   - workspaces come from the caller-sized stack buffers instead of malloc;
 *   - a zero pivot returns 4 instead of calling exit(1) (tridag.c:14-26);
 *   - the "consider taking shorter time steps" print (conductionQ.c:173) is
 *     reported through *warn instead of stdout.
 * Arithmetic follows the reference's order of operations; compiled with
 * -ffp-contract=off so results do not depend on FMA contraction.
 *
 * Pinned against the reference's golden files
 * tests/data/thermal/pcc_thermal_model_1d/{Tsurface,Tprofile}_conductionQ
 * (tests/test_pcc_oracle.py) and against the reference C sources compiled
 * into oracle/_ref when they are available.
 */
#include <math.h>
#include <stddef.h>

#define SIGSB 5.6704e-8

/* Thomas algorithm on 1-based arrays a,b,c,r of length n+1 (tridag.c:5-34). */
static int thomas(const double *a, const double *b, const double *c, const double *r,
                  double *u, double *gam, int n) {
  double bet = b[1];
  if (bet == 0.0) return 4;
  u[1] = r[1] / bet;
  for (int j = 2; j <= n; j++) {
    gam[j] = c[j - 1] / bet;
    bet = b[j] - a[j] * gam[j];
    if (bet == 0.0) return 4;
    u[j] = (r[j] - a[j] * u[j - 1]) / bet;
  }
  for (int j = n - 1; j >= 1; j--) u[j] -= gam[j + 1] * u[j + 1];
  return 0;
}

int oracle_conduction_q(int nz, const double *z, double dt, double Qn, double Qnp1,
                        double *T, const double *ti, const double *rhoc, double emiss,
                        double Fgeotherm, double *Fsurf, int *warn) {
  double k[nz + 1], alpha[nz + 1], gamma_[nz + 1];
  double a[nz + 1], b[nz + 1], c[nz + 1], r[nz + 1], Told[nz + 1], gam[nz + 1];
  for (int i = 1; i <= nz; i++) k[i] = ti[i] * ti[i] / rhoc[i];
  double dz = 2. * z[1];
  double beta = dt / rhoc[1] / (2. * dz * dz);
  alpha[1] = beta * k[2];
  gamma_[1] = beta * k[1];
  for (int i = 2; i < nz; i++) {
    double buf = dt / (z[i + 1] - z[i - 1]);
    alpha[i] = 2 * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    gamma_[i] = 2 * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  double buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
  gamma_[nz] = k[nz] * buf / (2 * rhoc[nz]);
  alpha[nz] = 0.0;
  double k1 = k[1] / dz;
  for (int i = 1; i <= nz; i++) {
    a[i] = -gamma_[i];
    b[i] = 1. + alpha[i] + gamma_[i];
    c[i] = -alpha[i];
  }
  b[nz] = 1. + gamma_[nz];

  double Tr = T[0];
  int iter = 0;
  for (int i = 1; i <= nz; i++) Told[i] = T[i];
  for (;;) {
    double arad = -3 * emiss * SIGSB * Tr * Tr * Tr * Tr;
    double brad = 2 * emiss * SIGSB * Tr * Tr * Tr;
    double ann = (Qn - arad) / (k1 + brad);
    double annp1 = (Qnp1 - arad) / (k1 + brad);
    double bn = (k1 - brad) / (k1 + brad);
    b[1] = 1. + alpha[1] + gamma_[1] - gamma_[1] * bn;
    r[1] = gamma_[1] * (annp1 + ann) + (1. - alpha[1] - gamma_[1] + gamma_[1] * bn) * T[1] +
           alpha[1] * T[2];
    for (int i = 2; i < nz; i++)
      r[i] = gamma_[i] * T[i - 1] + (1 - alpha[i] - gamma_[i]) * T[i] + alpha[i] * T[i + 1];
    r[nz] = gamma_[nz] * T[nz - 1] + (1. - gamma_[nz]) * T[nz] +
            dt / rhoc[nz] * Fgeotherm / (z[nz] - z[nz - 1]);
    int st = thomas(a, b, c, r, T, gam, nz);
    if (st) return st;
    T[0] = 0.5 * (annp1 + bn * T[1] + T[1]);
    if ((T[0] > 1.2 * Tr || T[0] < 0.8 * Tr) && iter < 10) {
      iter++;
      Tr = sqrt(Tr * T[0]);
      for (int i = 1; i <= nz; i++) T[i] = Told[i];
      continue;
    }
    break;
  }
  if (warn) *warn = iter >= 9;
  *Fsurf = -k[1] * (T[1] - T[0]) / z[1];
  return 0;
}

int oracle_conduction_t(int nz, const double *z, double dt, double *T, double Tsurf,
                        double Tsurfp1, const double *ti, const double *rhoc, double Fgeotherm,
                        double *Fsurf) {
  double k[nz + 1], alpha[nz + 1], gamma_[nz + 1];
  double a[nz + 1], b[nz + 1], c[nz + 1], r[nz + 1], gam[nz + 1];
  for (int i = 1; i <= nz; i++) k[i] = ti[i] * ti[i] / rhoc[i];
  alpha[1] = k[2] * dt / rhoc[1] / (z[2] - z[1]) / z[2];
  gamma_[1] = k[1] * dt / rhoc[1] / z[1] / z[2];
  for (int i = 2; i < nz; i++) {
    double buf = dt / (z[i + 1] - z[i - 1]);
    alpha[i] = 2 * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    gamma_[i] = 2 * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  double buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
  gamma_[nz] = k[nz] * buf / (rhoc[nz] + rhoc[nz]);
  alpha[nz] = 0.0;
  for (int i = 1; i <= nz; i++) {
    a[i] = -gamma_[i];
    b[i] = 1. + alpha[i] + gamma_[i];
    c[i] = -alpha[i];
  }
  b[nz] = 1. + gamma_[nz];
  r[1] = alpha[1] * T[2] + (1. - alpha[1] - gamma_[1]) * T[1] + gamma_[1] * (Tsurf + Tsurfp1);
  for (int i = 2; i < nz; i++)
    r[i] = gamma_[i] * T[i - 1] + (1. - alpha[i] - gamma_[i]) * T[i] + alpha[i] * T[i + 1];
  r[nz] = gamma_[nz] * T[nz - 1] + (1. - gamma_[nz]) * T[nz] +
          dt / rhoc[nz] * Fgeotherm / (z[nz] - z[nz - 1]);
  int st = thomas(a, b, c, r, T, gam, nz);
  if (st) return st;
  *Fsurf = -k[1] * (T[1] - Tsurfp1) / z[1];
  return 0;
}

/* The facet loop of PccThermalModel1D.step, bcond 'Q' (thermal.pyx:249-261):
 * T is num_faces x (nz+1) row-major, updated in place. Returns the first
 * nonzero status. */
int oracle_pcc_step_q(int num_faces, int nz, const double *z, double dt, const double *Qprev,
                      const double *X, double *T, const double *ti, const double *rhoc,
                      const double *emiss, const double *Fgeotherm, double *Fsurf) {
  for (int i = 0; i < num_faces; i++) {
    int st = oracle_conduction_q(nz, z, dt, Qprev[i], X[i], T + (size_t)i * (nz + 1), ti, rhoc,
                                 emiss[i], Fgeotherm[i], Fsurf + i, NULL);
    if (st) return st;
  }
  return 0;
}

int oracle_pcc_step_t(int num_faces, int nz, const double *z, double dt, const double *Tsprev,
                      const double *X, double *T, const double *ti, const double *rhoc,
                      const double *Fgeotherm, double *Fsurf) {
  for (int i = 0; i < num_faces; i++) {
    int st = oracle_conduction_t(nz, z, dt, T + (size_t)i * (nz + 1), Tsprev[i], X[i], ti, rhoc,
                                 Fgeotherm[i], Fsurf + i);
    if (st) return st;
  }
  return 0;
}
