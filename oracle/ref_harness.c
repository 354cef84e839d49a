/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A thin C driver around the reference CoMD src-flat, compiled from the
 * reference's own sources by oracle/Makefile into oracle/_ref/.  It calls
 * the reference's setup and timestep routines directly (no main(), no
 * do_compute_work printing loop) so tests can pin the oracle against the
 * reference bit for bit, and bench.py can time the reference's CPU path.
 * This file is compiled against the reference headers (real_t = double).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pmd.h"
#include "cheby.h"
#include "ic_fcc.h"
#include "read.h"

extern int PERIODIC;
extern void reBoxAll(simflat_t *s);
extern struct pmd_base_potential_t *setEamPot(char *dir, char *file);
extern ljpotential_t *getLJPot();

/* implemented in ref_seed.c against the library's layout-identical header */
extern void refh_seed_apply_impl(void *s, uint64_t seed, int kind, double amp, double temp_k,
                                 double mass_amu);

int refh_is_cheby(void) {
#ifdef USE_CHEBY
  return 1;
#else
  return 0;
#endif
}

void refh_set_periodic(int p) { PERIODIC = p; }

void *refh_eam_load(const char *dir, const char *name) {
  return setEamPot((char *)dir, (char *)name);
}

void *refh_lj_make(double sigma, double epsilon, double cutoff, double mass) {
  ljpotential_t *p = getLJPot();
  p->sigma = sigma;
  p->epsilon = epsilon;
  p->cutoff = cutoff;
  p->mass = mass;
  return p;
}

/* create_fcc_lattice with an explicit command_t; the Chebyshev series are
 * generated for EAM as initSimFromCmdLine does (src-flat/docompute.c:140) */
void *refh_fcc(int nx, int ny, int nz, double lat, double defgrad, double bf, void *pot,
               int is_eam) {
  command_t cmd;
  memset(&cmd, 0, sizeof cmd);
  cmd.nx = nx;
  cmd.ny = ny;
  cmd.nz = nz;
  cmd.lat = lat;
  cmd.defgrad = defgrad;
  cmd.bf = bf;
  cmd.doeam = is_eam;
  simflat_t *s = create_fcc_lattice(cmd, (struct pmd_base_potential_t *)pot);
  if (is_eam) s->ch_pot = setChebPot((eampotential_t *)pot, 32);
  return s;
}

/* the reference's own clsman reader (fromFileASCII -> fromFileGzip in a
 * GZIPSUPPORT build), then setChebPot for EAM as initSimFromCmdLine does */
void *refh_read_clsman(const char *path, double bf, void *pot, int is_eam) {
  command_t cmd;
  memset(&cmd, 0, sizeof cmd);
  strncpy(cmd.filename, path, sizeof cmd.filename - 1);
  cmd.bf = bf;
  cmd.doeam = is_eam;
  simflat_t *s = fromFileASCII(cmd, (struct pmd_base_potential_t *)pot);
  if (s && is_eam) s->ch_pot = setChebPot((eampotential_t *)pot, 32);
  return s;
}

/* the reference's FileAtom reader (read.c:248-315, fixed bounds) */
void *refh_read_tim(const char *path, double bf, void *pot) {
  command_t cmd;
  memset(&cmd, 0, sizeof cmd);
  strncpy(cmd.filename, path, sizeof cmd.filename - 1);
  cmd.bf = bf;
  return fromFileTim(cmd, (struct pmd_base_potential_t *)pot);
}

/* the reference's clsman writers (write.c:112-167 binary, :175-220 gzip
 * text) and its debug print (write.c:89-110) into a file */
extern void writeClsman(simflat_t *s, char *fname);
extern void gzASCIIWrite(simflat_t *s, char *fname);
extern void printIt(simflat_t *s, FILE *fp);

/* the simulation's comment line (gzASCIIWrite writes it verbatim) */
void refh_set_comment(void *s, const char *text) {
  simflat_t *q = (simflat_t *)s;
  strncpy(q->comment, text, 1023);
}

void refh_write_clsman(void *s, const char *path) { writeClsman((simflat_t *)s, (char *)path); }

void refh_gz_ascii_write(void *s, const char *path) {
  gzASCIIWrite((simflat_t *)s, (char *)path);
}

int refh_print_it(void *s, const char *path) {
  FILE *fp = fopen(path, "w");
  if (!fp) return -1;
  printIt((simflat_t *)s, fp);
  fclose(fp);
  return 0;
}

void refh_seed_apply(void *s, uint64_t seed, int kind, double amp, double temp_k,
                     double mass_amu) {
  refh_seed_apply_impl(s, seed, kind, amp, temp_k, mass_amu);
}

void refh_rebox(void *s) { reBoxAll((simflat_t *)s); }

int refh_force(void *s) { return computeForce((simflat_t *)s); }

double refh_ntimesteps(int n, void *s, double dt) {
  return nTimeSteps(n, (simflat_t *)s, (real_t)dt);
}
