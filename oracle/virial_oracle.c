/*
 * virial_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain serial FP64 restatement of the virial tensor, kinetic tensor and
 * per-atom stress that the library's virial kernel computes.  The reference
 * reports a single scalar (s->stress: x-x of the embedding term only in
 * eamForce, src-flat/eam.c:649; x-x with the kinetic term counted once per
 * neighbour box in LJ, src-flat/ljForce.c:175,210), so nothing here is the
 * reference's arithmetic: the definitions are the physical ones, over the
 * reference's own half-pair enumeration (src-flat/eam.c:484-549,
 * src-flat/ljForce.c:151-215).  Finite differences of the oracle's energy
 * under homogeneous strain check them (tests/test_virial.py):
 * W_aa = -dU/d(eps_aa).
 *
 * For a pair within the cutoff, F_ij = g dr_ij is the force on atom i from
 * atom j (dr_ij = r_i - r_j):
 *   EAM  g = -(phi'(r) [r2 <= rc2] + (F'_i + F'_j) rho'(r) [r2 < rc2]) / r
 *        (eamForce adds +grad U into f: eam.c:533-535, 644-647)
 *   LJ   g = 4 eps sigma^6 r^-8 (12 sigma^6 r^-6 - 6)  (ljForce.c:205-209)
 * W = sum over pairs of dr (x) F; each atom of a pair gets half of it.
 * K = sum over atoms of p (x) p / M, M = mass x amu_to_m_e (the mass of
 * advancePositions, timestep.c:90).  Per-atom stress x volume:
 * -(p (x) p / M + w_i).  Voigt order xx yy zz yz xz xy.
 *
 * Call after a force call (orc_force) on the same state: the EAM terms use
 * s->fi = F'(rho).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "comdgb_seed.h"
#include "comdgb_simflat.h"

#define MAXAT COMDGB_MAXATOMS
#define NNBR COMDGB_NUMNEIGHBORS

enum { V_EAM_TABLE = 0, V_EAM_CHEBY = 1, V_LJ = 2 };

int orc_neighbor_boxes(const simflat_t *s, int b, int *nbrs);
double orc_cheb_eval(const potentialarray_t *c, double x);
void orc_table_eval(const potentialarray_t *a, double r, double *value, double *deriv);
int orc_get_periodic(void);
int orc_alloc_domains(simflat_t *s);
int orc_put_atom(simflat_t *s, int id, int itype, double mass, double x, double y, double z,
                 double px, double py, double pz);
void orc_sim_free(simflat_t *s);

static void box_off(const simflat_t *s, int ib, int jb, double *d) {
  for (int j = 0; j < 3; j++) {
    d[j] = s->dcenter[ib][j] - s->dcenter[jb][j];
    if (orc_get_periodic()) {
      if (d[j] < -0.5 * s->bounds[j]) d[j] += s->bounds[j];
      else if (d[j] > 0.5 * s->bounds[j]) d[j] -= s->bounds[j];
    }
  }
}

static void add_pair(double *w, double *aw_i, double *aw_j, double g, const double *dr) {
  const double c[6] = {g * dr[0] * dr[0], g * dr[1] * dr[1], g * dr[2] * dr[2],
                       g * dr[1] * dr[2], g * dr[0] * dr[2], g * dr[0] * dr[1]};
  for (int q = 0; q < 6; q++) {
    w[q] += c[q];
    if (aw_i) {
      aw_i[q] += 0.5 * c[q];
      aw_j[q] += 0.5 * c[q];
    }
  }
}

/* w[6], k[6]; atom (optional): 6 doubles per slot, -(K_i + w_i), empty
 * slots 0.  Returns 0, or -20 for a Chebyshev kind without s->ch_pot. */
int orc_virial(const simflat_t *s, int kind, double *w, double *k, double *atom) {
  const int ns = s->nboxes * MAXAT;
  double *aw = atom;
  memset(w, 0, 6 * sizeof(double));
  memset(k, 0, 6 * sizeof(double));
  if (aw) memset(aw, 0, (size_t)ns * 6 * sizeof(double));
  int nbrs[NNBR];
  const eampotential_t *ep = (const eampotential_t *)s->pot;
  const ljpotential_t *lp = (const ljpotential_t *)s->pot;
  const eam_cheby_t *ch = s->ch_pot;
  if (kind == V_EAM_CHEBY && !ch) return -20;
  const double rc = kind == V_LJ ? lp->cutoff : ep->cutoff, rc2 = rc * rc;
  double s6 = 0.0;
  if (kind == V_LJ) s6 = pow(lp->sigma, 6.0);
  for (int ib = 0; ib < s->nboxes; ib++) {
    const int ni = s->natoms[ib];
    const int nn = orc_neighbor_boxes(s, ib, nbrs);
    for (int q = 0; q < nn; q++) {
      const int jb = nbrs[q];
      if (jb < 0) break;
      if (jb < ib) continue;
      double drbox[3];
      box_off(s, ib, jb, drbox);
      const int nj = s->natoms[jb];
      for (int ii = 0, io = MAXAT * ib; ii < ni; ii++, io++) {
        for (int ij = 0, jo = MAXAT * jb; ij < nj; ij++, jo++) {
          if (ib == jb && ij <= ii) continue;
          double dr[3], r2 = 0.0;
          for (int m = 0; m < 3; m++) {
            dr[m] = drbox[m] + s->r[io][m] - s->r[jo][m];
            r2 += dr[m] * dr[m];
          }
          if (r2 > rc2) continue;
          double g;
          if (kind == V_LJ) {
            const double ir2 = 1.0 / r2, r6 = ir2 * ir2 * ir2;
            g = 4.0 * lp->epsilon * s6 * r6 * ir2 * (12.0 * s6 * r6 - 6.0);
          } else {
            const double r = sqrt(r2);
            double v, dphi, drho = 0.0;
            if (kind == V_EAM_CHEBY) {
              dphi = orc_cheb_eval(ch->dphi, r);
              if (r2 < rc2) drho = orc_cheb_eval(ch->drho, r);
            } else {
              orc_table_eval(ep->phi, r, &v, &dphi);
              if (r2 < rc2) orc_table_eval(ep->rho, r, &v, &drho);
            }
            g = -(dphi + (s->fi[io] + s->fi[jo]) * drho) / r;
          }
          add_pair(w, aw ? aw + 6 * io : NULL, aw ? aw + 6 * jo : NULL, g, dr);
        }
      }
    }
  }
  const double rmass = COMDGB_AMU_TO_ME * s->pot->mass;
  for (int ib = 0; ib < s->nboxes; ib++)
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++) {
      const double *p = s->p[io];
      const double c[6] = {p[0] * p[0] / rmass, p[1] * p[1] / rmass, p[2] * p[2] / rmass,
                           p[1] * p[2] / rmass, p[0] * p[2] / rmass, p[0] * p[1] / rmass};
      for (int q = 0; q < 6; q++) {
        k[q] += c[q];
        if (aw) aw[6 * io + q] = -(aw[6 * io + q] + c[q]);
      }
    }
  return 0;
}

/* A copy of s under the homogeneous strain x_a -> scale[a] x_a: bounds and
 * every world position (box corner + box-relative r) scaled, atoms put in
 * slot order (ids, types, masses and momenta kept) into the grid
 * allocDomains makes for the new bounds.  NULL on failure. */
simflat_t *orc_strained(const simflat_t *s, const double *scale) {
  simflat_t *t = (simflat_t *)calloc(1, sizeof(simflat_t));
  if (!t) return NULL;
  t->pot = s->pot;
  t->ch_pot = s->ch_pot;
  t->bf = s->bf;
  t->defgrad = s->defgrad;
  for (int m = 0; m < 3; m++) t->bounds[m] = s->bounds[m] * scale[m];
  if (orc_alloc_domains(t)) {
    orc_sim_free(t);
    return NULL;
  }
  for (int ib = 0; ib < s->nboxes; ib++)
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++) {
      double x[3];
      for (int m = 0; m < 3; m++) x[m] = (s->dcenter[ib][m] + s->r[io][m]) * scale[m];
      if (orc_put_atom(t, s->id[io], s->iType[io], s->mass[io], x[0], x[1], x[2], s->p[io][0],
                       s->p[io][1], s->p[io][2])) {
        orc_sim_free(t);
        return NULL;
      }
    }
  return t;
}
