/*
 * centro_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain serial restatement of the centrosymmetry parameter of the in-situ
 * visualiser (AtomVisualize::computeCentrosymmetry,
 * src-viz/AtomVisualize.c:399-672), the oracle of the library's
 * centrosymmetry kernel.  It follows the routine's loops step for step.
 * The visualiser as a whole cannot be compiled without its VTK and OpenGL
 * headers, so oracle/Makefile compiles that one routine's text inside
 * oracle/centro_ref_shim.cpp, and the tests pin this restatement against
 * it bit for bit (and against fixtures it generated); known answers of the
 * physics (perfect lattice, vacancy neighbours) are a second check.
 *
 * Per atom: up to 12 nearest candidates, scanned from the atom's own box
 * (box-relative differences, :421-447) and then the 26 adjacent boxes in
 * x-outer, z-inner order, wrapped once per axis with a periodic offset held
 * in a float (:458-505).  Candidate j goes to the next free entry while
 * fewer than 12 are held; after that it replaces the first entry of largest
 * r^2 unless its own r^2 is larger.  With fewer than 12 neighbours the value
 * is 1000.  Otherwise (the default build, :560-664) it is the minimum over
 * all 10395 ways of pairing the 12 vectors of the sum of |r_a + r_b|^2,
 * accumulated in a float over the pairs in the order of their lower index;
 * or (APPROX_CENTROSYM, :528-557) the greedy pairing: each unpaired vector
 * in turn with the unpaired later vector of least |r_j + r_k|^2 (a vector
 * with r^2 = 0 counts as paired).
 */
#include <stdint.h>
#include <string.h>

#include "comdgb_simflat.h"

#define MAXAT COMDGB_MAXATOMS

typedef struct {
  double r[3], rsq;
} cand_t;

static void offer(cand_t *nl, int *nb, double dx, double dy, double dz) {
  const double rsq = dx * dx + dy * dy + dz * dz;
  int i1;
  if (*nb < 12) {
    i1 = (*nb)++;
  } else {
    int kmax = 0;
    double rmax = nl[0].rsq;
    for (int k = 1; k < 12; k++)
      if (nl[k].rsq > rmax) {
        kmax = k;
        rmax = nl[k].rsq;
      }
    if (rsq > rmax) return;
    i1 = kmax;
  }
  nl[i1].rsq = rsq;
  nl[i1].r[0] = dx;
  nl[i1].r[1] = dy;
  nl[i1].r[2] = dz;
}

static double pair_term(const cand_t *a, const cand_t *b) {
  return (a->r[0] + b->r[0]) * (a->r[0] + b->r[0]) + (a->r[1] + b->r[1]) * (a->r[1] + b->r[1]) +
         (a->r[2] + b->r[2]) * (a->r[2] + b->r[2]);
}

/* all pairings of the unpaired entries, the lowest unpaired entry first:
 * the float accumulator as the visualiser's testCentro */
static void pairings(const cand_t *nl, int *used, float acc, double *best) {
  int n = 0;
  while (n < 12 && used[n]) n++;
  if (n == 12) {
    if (acc < *best) *best = acc;
    return;
  }
  used[n] = 1;
  for (int p = n + 1; p < 12; p++) {
    if (used[p]) continue;
    used[p] = 1;
    float next = acc;
    next += pair_term(&nl[n], &nl[p]);
    pairings(nl, used, next, best);
    used[p] = 0;
  }
  used[n] = 0;
}

static double greedy(cand_t *nl) {
  double c = 0.0;
  for (int j = 0; j < 11; j++) {
    if (!(nl[j].rsq > 0.0)) continue;
    double summin = 1000.0;
    int kmin = -1;
    for (int k = j + 1; k < 12; k++) {
      if (!(nl[k].rsq > 0.0)) continue;
      const double sum = pair_term(&nl[j], &nl[k]);
      if (sum < summin) {
        kmin = k;
        summin = sum;
      }
    }
    c += summin;
    nl[j].rsq = -1.0;
    if (kmin >= 0) nl[kmin].rsq = -1.0;
  }
  return c;
}

/* centro: one double per slot (occupied slots written); *cmin / *cmax the
 * range over atoms (minCentro from 1000, maxCentro from 0, :667-676) */
void orc_centro(const simflat_t *s, int approx, double *centro, double *cmin, double *cmax) {
  const int nx = s->nbx[0], ny = s->nbx[1], nz = s->nbx[2];
  for (int ib = 0; ib < s->nboxes; ib++) {
    if (!s->natoms[ib]) continue;
    const int bz = ib / (nx * ny), by = (ib - bz * nx * ny) / nx, bx = ib - bz * nx * ny - by * nx;
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++) {
      cand_t nl[12];
      int nb = 0;
      for (int jj = 0, jo = MAXAT * ib; jj < s->natoms[ib]; jj++, jo++) {
        if (jo == io) continue;
        offer(nl, &nb, s->r[jo][0] - s->r[io][0], s->r[jo][1] - s->r[io][1],
              s->r[jo][2] - s->r[io][2]);
      }
      for (int cx = bx - 1; cx <= bx + 1; cx++)
        for (int cy = by - 1; cy <= by + 1; cy++)
          for (int cz = bz - 1; cz <= bz + 1; cz++) {
            if (cx == bx && cy == by && cz == bz) continue;
            float ox = 0.0f, oy = 0.0f, oz = 0.0f;
            int qx = cx, qy = cy, qz = cz;
            if (qx < 0) { qx = nx - 1; ox = (float)-s->bounds[0]; }
            if (qx >= nx) { qx = 0; ox = (float)s->bounds[0]; }
            if (qy < 0) { qy = ny - 1; oy = (float)-s->bounds[1]; }
            if (qy >= ny) { qy = 0; oy = (float)s->bounds[1]; }
            if (qz < 0) { qz = nz - 1; oz = (float)-s->bounds[2]; }
            if (qz >= nz) { qz = 0; oz = (float)s->bounds[2]; }
            const int b2 = qz * nx * ny + qy * nx + qx;
            for (int jj = 0, jo = MAXAT * b2; jj < s->natoms[b2]; jj++, jo++) {
              const double dx = (ox + s->dcenter[b2][0] + s->r[jo][0]) -
                                (s->dcenter[ib][0] + s->r[io][0]);
              const double dy = (oy + s->dcenter[b2][1] + s->r[jo][1]) -
                                (s->dcenter[ib][1] + s->r[io][1]);
              const double dz = (oz + s->dcenter[b2][2] + s->r[jo][2]) -
                                (s->dcenter[ib][2] + s->r[io][2]);
              offer(nl, &nb, dx, dy, dz);
            }
          }
      double c = 1000.0;
      if (nb >= 12) {
        if (approx) {
          c = greedy(nl);
        } else {
          int used[12] = {0};
          pairings(nl, used, 0.0f, &c);
        }
      }
      centro[io] = c;
    }
  }
  double lo = 1000.0, hi = 0.0;
  for (int ib = 0; ib < s->nboxes; ib++)
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++) {
      if (centro[io] < lo) lo = centro[io];
      if (centro[io] > hi) hi = centro[io];
    }
  if (cmin) *cmin = lo;
  if (cmax) *cmax = hi;
}
