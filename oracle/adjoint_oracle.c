/*
 * adjoint_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain serial FP64 restatement of the parameter gradients the library's
 * adjoint kernels compute, over the reference's own pair enumeration (the
 * half box pairs of eamForce, src-flat/eam.c:484-549, and the id-ordered
 * pairs of ljForce, src-flat/ljForce.c:151-215).  It checks the GPU
 * gradients; finite differences of the oracle's energies (comd_oracle.c)
 * check it.  The reference has no gradients, so nothing here is "the
 * reference's arithmetic"; the definitions follow the same formulas as the
 * library (U = total energy, f the reference's forces, lambda_i =
 * 2 (f_i - target_i), D = sum_i lambda_i . grad_i U):
 *   dU/dc^phi_k = sum_{i<j} B_k(r_ij)         dD/dc^phi_k = sum_{i<j} v_ij B'_k(r_ij)
 *   dU/dc^rho_k = sum_{i<j} (F'_i+F'_j) B_k(r_ij)
 *   dD/dc^rho_k = sum_{i<j} [(F'_i+F'_j) v_ij B'_k(r_ij) + (X_i+X_j) B_k(r_ij)]
 *   dU/dc^F_k   = sum_i B_k(rho_i)            dD/dc^F_k   = sum_i W_i B'_k(rho_i)
 * with v_ij = (lambda_i - lambda_j).(r_i - r_j)/r_ij, W_i = sum_j v_ij rho'(r_ij)
 * (embedding pairs, r2 < rc2), X_i = F''(rho_i) W_i, B_k the Chebyshev basis
 * of eamCheb (k = 0 halved) and B'_k = T'_k(y) 2/(b-a).  For EAM f = +grad U,
 * so dL/dc = dD/dc; for LJ f = -grad U, so dL/dtheta = -dD/dtheta.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "comdgb_simflat.h"

#define MAXAT COMDGB_MAXATOMS
#define NNBR COMDGB_NUMNEIGHBORS

int orc_eam_force(simflat_t *s, int use_cheby);
int orc_lj_force(simflat_t *s);
int orc_neighbor_boxes(const simflat_t *s, int b, int *nbrs);
double orc_cheb_eval(const potentialarray_t *c, double x);
int orc_get_periodic(void);

/* minimum-image box offset, src-flat/eam.c:494-502 */
static void box_off(const simflat_t *s, int ib, int jb, double *d) {
  for (int j = 0; j < 3; j++) {
    d[j] = s->dcenter[ib][j] - s->dcenter[jb][j];
    if (orc_get_periodic()) {
      if (d[j] < -0.5 * s->bounds[j]) d[j] += s->bounds[j];
      else if (d[j] > 0.5 * s->bounds[j]) d[j] -= s->bounds[j];
    }
  }
}

/* chder / genDer, src-flat/cheby.c:180-270 */
static void derive(double a, double b, const double *c, double *cd, int n) {
  cd[n - 1] = 0.0;
  cd[n - 2] = 2.0 * (n - 1) * c[n - 1];
  for (int j = n - 2; j > 0; j--) cd[j - 1] = cd[j + 1] + 2 * (j)*c[j];
  double con = 2.0 / (b - a);
  for (int j = 0; j < n; j++) cd[j] = cd[j] * con;
}

/* replace the base series phi, rho, F (coef[n*q + k]) and derive the
 * derivative series as setChebPot does (cheby.c:99-121) */
void orc_cheb_set(eam_cheby_t *ch, const double *coef, const double *x0, const double *xn) {
  potentialarray_t *base[3] = {ch->phi, ch->rho, ch->f};
  potentialarray_t *der[3] = {ch->dphi, ch->drho, ch->df};
  for (int q = 0; q < 3; q++) {
    int n = base[q]->n;
    memcpy(base[q]->values, coef + (size_t)q * n, sizeof(double) * n);
    base[q]->x0 = der[q]->x0 = x0[q];
    base[q]->xn = der[q]->xn = xn[q];
    derive(x0[q], xn[q], base[q]->values, der[q]->values, n);
  }
}

/* y of x on [a, b] after the clamp, T_k(y), T'_k(y) (k < n) */
static void basis(const potentialarray_t *c, double x, int n, double *t, double *tp, double *sc) {
  double a = c->x0, b = c->xn;
  if (x < a) x = a;
  double y = (2.0 * x - a - b) / (b - a);
  *sc = 2.0 / (b - a);
  double t0 = 1.0, t1 = y, u0 = 1.0, u1 = 2.0 * y;
  t[0] = 1.0;
  tp[0] = 0.0;
  for (int k = 1; k < n; k++) {
    t[k] = t1;
    tp[k] = k * u0;
    double t2 = 2.0 * y * t1 - t0, u2 = 2.0 * y * u1 - u0;
    t0 = t1;
    t1 = t2;
    u0 = u1;
    u1 = u2;
  }
}

/* second-derivative series value of a clamped series (0 below a) */
static double dd_eval(const potentialarray_t *d, double x) {
  double cd[64];
  int n = d->n;
  if (x < d->x0) return 0.0;
  derive(d->x0, d->xn, d->values, cd, n);
  potentialarray_t t = *d;
  t.values = cd;
  return orc_cheb_eval(&t, x);
}

/* EAM Chebyshev: *energy, gu[3n] = dU/dc and, with target (3 per atom id),
 * *loss and gl[3n] = dL/dc.  Returns 0 or the force call's error. */
int orc_eam_cheb_grad(simflat_t *s, const double *target, double *energy, double *gu,
                      double *loss, double *gl) {
  int rc = orc_eam_force(s, 1);
  if (rc) return rc;
  const eampotential_t *pot = (const eampotential_t *)s->pot;
  const eam_cheby_t *ch = s->ch_pot;
  const int n = ch->phi->n;
  const double rcut2 = pot->cutoff * pot->cutoff;
  const size_t ns = (size_t)s->nboxes * MAXAT;
  double *lam = calloc(ns * 3, sizeof(double)), *W = calloc(ns, sizeof(double));
  double *X = calloc(ns, sizeof(double));
  double tp_[64], t_[64], tq[64], tqp[64], sc, sq;
  int nbrs[NNBR];
  *energy = s->e;
  memset(gu, 0, sizeof(double) * 3 * n);
  if (gl) memset(gl, 0, sizeof(double) * 3 * n);
  double L = 0.0;
  for (int ib = 0; ib < s->nboxes; ib++)
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++)
      if (target) {
        const double *t = target + 3 * (size_t)s->id[io];
        for (int k = 0; k < 3; k++) {
          double d = s->f[io][k] - t[k];
          lam[3 * io + k] = 2.0 * d;
          L += d * d;
        }
      }
  if (loss) *loss = L;
  /* W over the embedding pairs, then X */
  for (int pass = 0; pass < 2; pass++)
    for (int ib = 0; ib < s->nboxes; ib++) {
      int ni = s->natoms[ib], nn = orc_neighbor_boxes(s, ib, nbrs);
      for (int q = 0; q < nn; q++) {
        int jb = nbrs[q];
        if (jb < 0) break;
        if (jb < ib) continue;
        double drbox[3];
        box_off(s, ib, jb, drbox);
        for (int ii = 0, io = MAXAT * ib; ii < ni; ii++, io++)
          for (int ij = 0, jo = MAXAT * jb; ij < s->natoms[jb]; ij++, jo++) {
            if (ib == jb && ij <= ii) continue;
            double dr[3], r2 = 0.0;
            for (int k = 0; k < 3; k++) {
              dr[k] = drbox[k] + s->r[io][k] - s->r[jo][k];
              r2 += dr[k] * dr[k];
            }
            if (r2 > rcut2) continue;
            double r = sqrt(r2), v = 0.0;
            for (int k = 0; k < 3; k++) v += (lam[3 * io + k] - lam[3 * jo + k]) * dr[k];
            v /= r;
            if (pass == 0) {
              if (r2 < rcut2) {
                double rp = orc_cheb_eval(ch->drho, r);
                W[io] += v * rp;
                W[jo] += v * rp;
              }
              continue;
            }
            double fs = s->fi[io] + s->fi[jo];
            basis(ch->phi, r, n, t_, tp_, &sc);
            basis(ch->rho, r, n, tq, tqp, &sq);
            for (int k = 0; k < n; k++) {
              double bp = k ? t_[k] : 0.5, bq = k ? tq[k] : 0.5;
              gu[k] += bp;
              gu[n + k] += fs * bq;
              if (gl) {
                gl[k] += v * sc * tp_[k];
                gl[n + k] += (r2 < rcut2 ? fs * v * sq * tqp[k] : 0.0) + (X[io] + X[jo]) * bq;
              }
            }
          }
      }
      if (pass == 0 && ib == s->nboxes - 1)
        for (int b = 0; b < s->nboxes; b++)
          for (int i = 0, o = MAXAT * b; i < s->natoms[b]; i++, o++)
            X[o] = dd_eval(ch->df, s->rho[o]) * W[o];
    }
  for (int ib = 0; ib < s->nboxes; ib++)
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++) {
      basis(ch->f, s->rho[io], n, t_, tp_, &sc);
      for (int k = 0; k < n; k++) {
        gu[2 * n + k] += k ? t_[k] : 0.5;
        if (gl) gl[2 * n + k] += W[io] * sc * tp_[k];
      }
    }
  free(lam);
  free(W);
  free(X);
  return 0;
}

/* LJ: *energy, gu[2] = dU/d(eps, sigma) and, with target, *loss and gl[2] */
int orc_lj_grad(simflat_t *s, const double *target, double *energy, double *gu, double *loss,
                double *gl) {
  int rc = orc_lj_force(s);
  if (rc) return rc;
  const ljpotential_t *pot = (const ljpotential_t *)s->pot;
  const double eps = pot->epsilon, sg = pot->sigma, r2cut = pot->cutoff * pot->cutoff;
  const size_t ns = (size_t)s->nboxes * MAXAT;
  double *lam = calloc(ns * 3, sizeof(double));
  double L = 0.0, ge = 0.0, gs = 0.0, de = 0.0, ds = 0.0;
  int nbrs[NNBR];
  *energy = s->e;
  for (int ib = 0; ib < s->nboxes; ib++)
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++)
      if (target) {
        const double *t = target + 3 * (size_t)s->id[io];
        for (int k = 0; k < 3; k++) {
          double d = s->f[io][k] - t[k];
          lam[3 * io + k] = 2.0 * d;
          L += d * d;
        }
      }
  for (int ib = 0; ib < s->nboxes; ib++) {
    int ni = s->natoms[ib], nn = orc_neighbor_boxes(s, ib, nbrs);
    for (int q = 0; q < nn; q++) {
      int jb = nbrs[q];
      if (jb < 0) break;
      double drbox[3];
      box_off(s, ib, jb, drbox);
      for (int ii = 0, io = MAXAT * ib; ii < ni; ii++, io++)
        for (int ij = 0, jo = MAXAT * jb; ij < s->natoms[jb]; ij++, jo++) {
          if (s->id[jo] <= s->id[io]) continue;
          double dr[3], r2 = 0.0;
          for (int k = 0; k < 3; k++) {
            dr[k] = drbox[k] + s->r[io][k] - s->r[jo][k];
            r2 += dr[k] * dr[k];
          }
          if (r2 > r2cut) continue;
          double r = sqrt(r2), s2 = sg * sg / r2, s6 = s2 * s2 * s2, s12 = s6 * s6, v = 0.0;
          for (int k = 0; k < 3; k++) v += (lam[3 * io + k] - lam[3 * jo + k]) * dr[k];
          v /= r;
          ge += 4.0 * (s12 - s6);
          gs += 4.0 * eps * (12.0 * s12 - 6.0 * s6) / sg;
          de += v * 4.0 * (-12.0 * s12 + 6.0 * s6) / r;
          ds += v * 4.0 * eps * (-144.0 * s12 + 36.0 * s6) / (sg * r);
        }
    }
  }
  gu[0] = ge;
  gu[1] = gs;
  if (loss) *loss = L;
  if (gl) {
    gl[0] = -de;
    gl[1] = -ds;
  }
  free(lam);
  return 0;
}
