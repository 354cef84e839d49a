/*
 * comdgb_simflat.h -- host data model shared with CoMD src-flat (double build).
 *
 * These structs are the drop-in boundary: a host program that built its
 * simulation with CoMD's own setup code (create_fcc_lattice, fromFileGzip,
 * setEamPot, setChebPot) hands the same pointers to the GB300 library.  The
 * field order and types therefore match, member for member, the -DDOUBLE
 * build of:
 *   simflat_t            src-flat/include/pmdTypes.h:104-141
 *   pmd_base_potential_t src-flat/include/pmdTypes.h:74-79
 *   potentialarray_t     src-flat/include/eamTypes.h:68-74
 *   eampotential_t       src-flat/include/eamTypes.h:92-101
 *   eam_cheby_t          src-flat/include/eamTypes.h:104-114
 *   ljpotential_t        src-flat/include/ljTypes.h:72-81
 * real_t is double here (the reference's -DDOUBLE oracle build); the
 * reference's default -DSINGLE layout is not supported by this library.
 *
 * In a translation unit of the reference itself, include comdgb.h after the
 * reference's pmd.h: the structs are then the reference's own definitions
 * (its include guards are tested below) and this header adds none of its
 * own.  That needs the reference's double layout (-DDOUBLE) and a simflat_t
 * without the in-situ visualiser's extra member (USE_IN_SITU_VIZ); either
 * mismatch stops the compile here.
 */
#ifndef COMDGB_SIMFLAT_H
#define COMDGB_SIMFLAT_H

/* the reference's headers already seen (pmdTypes.h, eamTypes.h, ljTypes.h) */
#if defined(__PMDTYPES_H_) || defined(__EAM_TYPES_H_) || defined(_LJTYPES_H_)
#if defined(SINGLE)
#error "libcomdgb takes the reference's double layout: build the reference with -DDOUBLE"
#endif
#if defined(__PMDTYPES_H_) && defined(USE_IN_SITU_VIZ)
#error "libcomdgb takes simflat_t without the visualiser's centro member (USE_IN_SITU_VIZ)"
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* per-box slot capacity, src-flat/include/pmdTypes.h:57 */
#define COMDGB_MAXATOMS 64
/* 3x3x3 link-cell stencil, src-flat/include/domains.h:60 */
#define COMDGB_NUMNEIGHBORS 27

typedef double comdgb_real_t;
typedef comdgb_real_t comdgb_real3[3];
typedef comdgb_real_t comdgb_real4[4];

#ifndef __PMDTYPES_H_
typedef struct pmd_base_potential_t {
  comdgb_real_t cutoff;          /* Angstrom */
  comdgb_real_t mass;            /* amu */
  int (*force)(void *s);         /* the force routine; takes simflat_t* */
  void (*destroy)(void *pot);
} pmd_base_potential_t;
#endif

#ifndef __EAM_TYPES_H_
/* Tabulated function.  values[-1], values[n] and values[n+1] are guard
 * cells; x0 is already shifted by one interval (eam.c:130-153). */
typedef struct potentialarray_t {
  int n;
  comdgb_real_t x0;
  comdgb_real_t xn;
  comdgb_real_t invDx;
  comdgb_real_t *values;
} potentialarray_t;

typedef struct eampotential_t {
  comdgb_real_t cutoff;
  comdgb_real_t mass;
  int (*force)(void *s);
  void (*destroy)(void **pot);
  potentialarray_t *phi;
  potentialarray_t *rho;
  potentialarray_t *f;
  comdgb_real_t lat;
} eampotential_t;

/* Chebyshev series: values[] holds n coefficients on [x0, xn]. */
typedef struct eam_cheby_t {
  comdgb_real_t cutoff;
  comdgb_real_t mass;
  potentialarray_t *phi;
  potentialarray_t *rho;
  potentialarray_t *f;
  potentialarray_t *dphi;
  potentialarray_t *drho;
  potentialarray_t *df;
  comdgb_real_t lat;
} eam_cheby_t;
#endif

#ifndef _LJTYPES_H_
typedef struct ljpotential_t {
  comdgb_real_t cutoff;
  comdgb_real_t mass;
  int (*force)(void *s);
  void (*destroy)(void **pot);
  comdgb_real_t sigma;
  comdgb_real_t epsilon;
} ljpotential_t;
#endif

#ifndef __PMDTYPES_H_
/* Flat link-cell simulation: slot = box*64 + k for k < natoms[box]. */
typedef struct simflat_t {
  int stateflag;
  int nbx[3];
  int nboxes;
  int ntot;
  comdgb_real3 bounds;
  comdgb_real3 boxsize;
  comdgb_real3 *dcenter;       /* lower corner of each box */
  int *natoms;
  int *id;
  int *iType;
  comdgb_real_t *mass;
  comdgb_real3 *r;             /* box-relative positions */
  comdgb_real3 *p;             /* momenta */
  comdgb_real4 *f;             /* fx, fy, fz, per-atom energy */
  comdgb_real_t *rho;
  comdgb_real_t *fi;
  comdgb_real_t e;
  int nAtoms;
  pmd_base_potential_t *pot;
  char *comment;
  comdgb_real_t stress;
  comdgb_real_t defgrad;
  comdgb_real_t bf;
  eam_cheby_t *ch_pot;
} simflat_t;
#endif

#ifdef __cplusplus
}
#endif

#endif /* COMDGB_SIMFLAT_H */
