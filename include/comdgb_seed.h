/*
 * comdgb_seed.h -- seeded synthetic inputs for the CoMD timestep.
 *
 * The reference builds a perfect, motionless FCC lattice
 * (src-flat/ic_fcc.c:63-141 zeroes p; src-flat/mycommand.c:149 parses a
 * temperature it never uses).  The workloads this library is measured on
 * need displaced atoms and thermal momenta, so every harness (the GPU
 * library's builder, the CPU oracle, the harness around the compiled
 * reference) applies the same deterministic perturbation to an already
 * binned simflat_t and then calls reBoxAll once, as initSimFromCmdLine does
 * (src-flat/docompute.c:157).
 *
 * Random numbers: SplitMix64 keyed by (seed, atom id, stream), so the result
 * does not depend on the slot an atom occupies.  Gaussians by Box-Muller.
 * Units are the reference's: Angstrom, Hartree, electron masses and the
 * time unit t0 = A*sqrt(me/Ha) (src-flat/timestep.c:90,126).
 */
#ifndef COMDGB_SEED_H
#define COMDGB_SEED_H

#include <stdint.h>
#include <math.h>
#include "comdgb_simflat.h"

#ifdef __cplusplus
extern "C" {
#endif

/* amu -> electron masses, src-flat/include/constants.h:65 */
#define COMDGB_AMU_TO_ME 1822.83
/* Boltzmann constant in Hartree per kelvin */
#define COMDGB_KB_HA_PER_K 3.166811563e-6
/* 1 eV in Hartree */
#define COMDGB_EV_TO_HA (1.0 / 27.211386245988)

enum {
  COMDGB_DISP_NONE = 0,
  COMDGB_DISP_UNIFORM = 1,   /* each component uniform in [-amp, +amp) */
  COMDGB_DISP_GAUSSIAN = 2   /* each component normal with sigma = amp */
};

static inline uint64_t comdgb_splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* uniform double in [0, 1) for (seed, id, stream) */
static inline double comdgb_uniform(uint64_t seed, int64_t id, int stream) {
  uint64_t key = comdgb_splitmix64((uint64_t)id * 16u + (uint64_t)stream);
  uint64_t bits = comdgb_splitmix64(seed ^ key);
  return (double)(bits >> 11) * (1.0 / 9007199254740992.0);
}

/* standard normal for (seed, id, stream pair 2s, 2s+1) */
static inline double comdgb_normal(uint64_t seed, int64_t id, int s) {
  double u1 = comdgb_uniform(seed, id, 2 * s);
  double u2 = comdgb_uniform(seed, id, 2 * s + 1);
  return sqrt(-2.0 * log(1.0 - u1)) * cos(6.283185307179586 * u2);
}

/*
 * Displace every atom by a seeded amount and give it seeded thermal
 * momenta p = sqrt(M kB T) N(0,1) with M = mass_amu * 1822.83, then remove
 * the centre-of-mass momentum (summed in slot order).  Positions stay
 * box-relative; atoms that leave their box are moved by the caller's
 * reBoxAll.  Streams: 0..2 displacement, 3..5 momenta.
 */
static inline void comdgb_seed_apply(simflat_t *s, uint64_t seed, int disp_kind,
                                     double disp_amp, double temperature_k,
                                     double mass_amu) {
  double pscale = (temperature_k > 0.0)
                      ? sqrt(mass_amu * COMDGB_AMU_TO_ME * COMDGB_KB_HA_PER_K * temperature_k)
                      : 0.0;
  double psum[3] = {0.0, 0.0, 0.0};
  long nat = 0;
  int b, k, m;
  for (b = 0; b < s->nboxes; b++) {
    for (k = 0; k < s->natoms[b]; k++) {
      int slot = b * COMDGB_MAXATOMS + k;
      int64_t id = s->id[slot];
      for (m = 0; m < 3; m++) {
        double d = 0.0;
        if (disp_kind == COMDGB_DISP_UNIFORM)
          d = disp_amp * (2.0 * comdgb_uniform(seed, id, m) - 1.0);
        else if (disp_kind == COMDGB_DISP_GAUSSIAN)
          d = disp_amp * comdgb_normal(seed, id, m);
        s->r[slot][m] += d;
        if (pscale > 0.0) {
          s->p[slot][m] = pscale * comdgb_normal(seed, id, 3 + m);
          psum[m] += s->p[slot][m];
        }
      }
      nat++;
    }
  }
  if (pscale > 0.0 && nat > 0) {
    for (m = 0; m < 3; m++) psum[m] /= (double)nat;
    for (b = 0; b < s->nboxes; b++)
      for (k = 0; k < s->natoms[b]; k++)
        for (m = 0; m < 3; m++) s->p[b * COMDGB_MAXATOMS + k][m] -= psum[m];
  }
}

#ifdef __cplusplus
}
#endif

#endif /* COMDGB_SEED_H */
