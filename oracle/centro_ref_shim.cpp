/*
 * centro_ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference visualiser's own centrosymmetry routine
 * (AtomVisualize::computeCentrosymmetry, src-viz/AtomVisualize.c:399-672)
 * without its graphics.  oracle/Makefile copies the text of that one
 * function from the reference tree into oracle/_ref/centro_body.inc (never
 * into the repository) and compiles this file around it:
 *   * the reference's pmdTypes.h gives real_t, real3 and MAXATOMS; the
 *     neighbour record the routine keeps 12 of is declared here with the
 *     members of the reference's Neighbor (pmdTypes.h:84-89, compiled only
 *     with USE_IN_SITU_VIZ, which would also pull in the GLUT headers);
 *   * the routine reads only nboxes, nbx, bounds, dcenter, natoms, r and
 *     writes centro, so `simflat_t` is mapped, for that text alone, onto a
 *     view struct holding exactly those members, filled from a caller's
 *     slot arrays;
 *   * the class has just the members the routine touches (minCentro,
 *     maxCentro).
 * Built twice: as written (the exact minimum over pairings) and with
 * -DAPPROX_CENTROSYM (the reference's greedy pairing).  The tests use it to
 * pin oracle/centro_oracle.c and the GPU kernel to the reference itself.
 */
#include <cstdio>
#include <iostream>

#include "pmdTypes.h"

namespace {

struct Neighbor {
  real3 r;
  real_t rsq;
  int index;
};
typedef Neighbor Neighbor12[12];

struct CentroView {
  int nboxes;
  int nbx[3];
  real3 bounds;
  real3 *dcenter;
  int *natoms;
  real3 *r;
  real_t *centro;
};

class AtomVisualize {
 public:
  static void computeCentrosymmetry(CentroView *atoms);
  static float minCentro;
  static float maxCentro;
};

float AtomVisualize::minCentro = 0.0f;
float AtomVisualize::maxCentro = 0.0f;

#define simflat_t CentroView
#include "centro_body.inc"
#undef simflat_t

// (pmdTypes.h declares a global `AtomVisualize` too: call from inside)
void run(CentroView *v, float *minmax) {
  AtomVisualize::computeCentrosymmetry(v);
  minmax[0] = AtomVisualize::minCentro;
  minmax[1] = AtomVisualize::maxCentro;
}

}  // namespace

/* The reference routine over a caller's slot arrays (slot = box * MAXATOMS +
 * k): dcenter [nboxes][3], natoms [nboxes], r [nboxes * MAXATOMS][3] as the
 * reference stores them; centro [nboxes * MAXATOMS] receives the values of
 * the occupied slots.  minmax gets the routine's minCentro and maxCentro
 * (the latter clamped to 100 as the routine does).  Returns MAXATOMS so the
 * caller can check the slot stride. */
extern "C" int refc_centro(int nboxes, const int *nbx, const double *bounds, double *dcenter,
                           int *natoms, double *r, double *centro, float *minmax) {
  CentroView v;
  v.nboxes = nboxes;
  for (int i = 0; i < 3; i++) {
    v.nbx[i] = nbx[i];
    v.bounds[i] = bounds[i];
  }
  v.dcenter = reinterpret_cast<real3 *>(dcenter);
  v.natoms = natoms;
  v.r = reinterpret_cast<real3 *>(r);
  v.centro = centro;
  run(&v, minmax);
  return MAXATOMS;
}
