/*
 * comdgb_run.c -- a C host for libcomdgb that runs the reference's own
 * driver loop: the set-up of initSimFromCmdLine (src-flat/docompute.c:68-163)
 * and the timestep loop of do_compute_work (src-flat/docompute.c:166-218),
 * with the potential's force pointer set to comdgb_force
 * (src-flat/include/pmdTypes.h:77, src-flat/timestep.c:110-112) and
 * nTimeSteps replaced by comdgb_nTimeSteps (src-flat/timestep.c:114-140).
 *
 * It is also the worked example of the drop-in boundary: everything the
 * loop touches is the reference's data model (include/comdgb_simflat.h) and
 * the calls a maintainer adds to the reference's own host.
 *
 * Flags as the reference's command line (src-flat/mycommand.c:108-161):
 *   -e        EAM (else LJ with getLJPot's parameters, ljForce.c:75-86)
 *   -p NAME   potential name (default ag)     -d DIR  potential directory
 *   -f FILE   clsman structure file (else an FCC lattice)
 *   -x/-y/-z N  unit cells (default 20)        -b BF   box factor (default 1)
 *   -s DG     deformation gradient along x    -o      not periodic
 *   -t T      temperature of seeded momenta in K (the reference parses it
 *             and uses it nowhere; here it seeds comdgb_seed)
 * and the library's own:
 *   -c        EAM by the Chebyshev series (the reference's -DUSE_CHEBY build)
 *   -m        mixed precision (default FP64)
 *   -S SEED   seed of the displacements and momenta (default 1)
 *   -a AMP    Gaussian displacement in Angstrom (default 0)
 *   -n N      iterations (default 20)          -k K    steps per iteration (10)
 *   -G DEV    CUDA device                      -l      lazy mode
 * Output: the reference's per-iteration lines (energy, virial stress and
 * microseconds per atom and force call), then one line
 *   "comdgb_run: iterations N steps K atoms A final_energy E"
 * and the run as one JSON record (atoms, steps, atom-steps/s over the
 * comdgb_nTimeSteps calls, final energy and stress).
 * Exit status 0, or the library's negative error code as 1 with a message.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "comdgb.h"

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static int fail(const char *what, int code) {
  char msg[512];
  comdgb_last_error(msg, (int)sizeof msg);
  fprintf(stderr, "comdgb_run: %s failed (%d): %s\n", what, code, msg);
  return 1;
}

typedef struct {
  int eam, cheby, mixed, periodic, nx, ny, nz, niter, nsteps, device, lazy;
  double bf, defgrad, temp, amp;
  uint64_t seed;
  char potname[256], potdir[1024], filename[1024];
} run_opts;

static int parse(int argc, char **argv, run_opts *r) {
  memset(r, 0, sizeof *r);
  strcpy(r->potname, "ag");
  strcpy(r->potdir, "pots");
  r->periodic = 1;
  r->nx = r->ny = r->nz = 20;
  r->bf = 1.0;
  r->defgrad = 1.0;
  r->seed = 1;
  r->niter = 20;
  r->nsteps = 10;
  int c;
  while ((c = getopt(argc, argv, "ep:d:f:x:y:z:b:s:ot:cmS:a:n:k:G:lh")) != -1) {
    switch (c) {
      case 'e': r->eam = 1; break;
      case 'p': snprintf(r->potname, sizeof r->potname, "%s", optarg); break;
      case 'd': snprintf(r->potdir, sizeof r->potdir, "%s", optarg); break;
      case 'f': snprintf(r->filename, sizeof r->filename, "%s", optarg); break;
      case 'x': r->nx = atoi(optarg); break;
      case 'y': r->ny = atoi(optarg); break;
      case 'z': r->nz = atoi(optarg); break;
      case 'b': r->bf = atof(optarg); break;
      case 's': r->defgrad = atof(optarg); break;
      case 'o': r->periodic = 0; break;
      case 't': r->temp = atof(optarg); break;
      case 'c': r->cheby = 1; break;
      case 'm': r->mixed = 1; break;
      case 'S': r->seed = strtoull(optarg, NULL, 10); break;
      case 'a': r->amp = atof(optarg); break;
      case 'n': r->niter = atoi(optarg); break;
      case 'k': r->nsteps = atoi(optarg); break;
      case 'G': r->device = atoi(optarg); break;
      case 'l': r->lazy = 1; break;
      default:
        fprintf(stderr, "usage: %s [-e] [-p name] [-d dir] [-f file] [-x n -y n -z n] [-b bf] "
                        "[-s defgrad] [-o] [-t K] [-c] [-m] [-S seed] [-a amp] [-n iter] "
                        "[-k steps] [-G dev] [-l]\n", argv[0]);
        return -1;
    }
  }
  return 0;
}

int main(int argc, char **argv) {
  run_opts ro;
  if (parse(argc, argv, &ro)) return 2;
  printf("    Double Precision=true (library: %s)\n", comdgb_version());

  /* the potential (initSimFromCmdLine, docompute.c:81-119) */
  eampotential_t *eam = NULL;
  ljpotential_t *lj = NULL;
  pmd_base_potential_t *pot;
  double lat;
  if (ro.eam) {
    eam = comdgb_eam_read(ro.potdir, ro.potname);
    if (!eam) return fail("comdgb_eam_read", COMDGB_ERR_IO);
    pot = (pmd_base_potential_t *)eam;
    lat = eam->lat;
  } else {
    lj = comdgb_lj_make(1.53, 0.0085, 3.0 * 1.53, 1.0);
    if (!lj) return fail("comdgb_lj_make", COMDGB_ERR_NOMEM);
    pot = (pmd_base_potential_t *)lj;
    lat = 1.122462048 * lj->cutoff;
  }

  /* the structure: a file or the FCC lattice (docompute.c:121-130) */
  int st = 0;
  simflat_t *sim;
  if (ro.filename[0])
    sim = comdgb_read_clsman(ro.filename, pot, ro.bf, ro.device, &st);
  else
    sim = comdgb_fcc(ro.nx, ro.ny, ro.nz, lat, ro.defgrad, ro.bf, pot, &st);
  if (!sim) return fail("structure set-up", st);
  if (ro.temp > 0.0 || ro.amp > 0.0)
    comdgb_seed(sim, ro.seed, ro.amp > 0.0 ? 2 : 0, ro.amp, ro.temp, pot->mass);

  /* setChebPot (docompute.c:132-135), fitted on the GPU */
  eam_cheby_t *ch = NULL;
  if (ro.eam) {
    ch = comdgb_cheb_make(eam, 32, ro.device);
    if (!ch) return fail("comdgb_cheb_make", COMDGB_ERR_CUDA);
    sim->ch_pot = ch;
  }
  printf("    total atoms is: %d\n", sim->ntot);

  /* the initial reBoxAll (docompute.c:159) */
  int rc = comdgb_rebox_host(sim, ro.periodic, ro.device);
  if (rc) return fail("comdgb_rebox_host", rc);

  /* the drop-in: the simulation mirrored on the GPU, computeForce through
   * the potential's own force pointer */
  comdgb_opts o;
  comdgb_default_opts(&o);
  o.potential = !ro.eam ? COMDGB_POT_LJ : ro.cheby ? COMDGB_POT_EAM_CHEBY : COMDGB_POT_EAM_TABLE;
  o.precision = ro.mixed ? COMDGB_PREC_MIXED : COMDGB_PREC_FP64;
  o.periodic = ro.periodic;
  o.device = ro.device;
  o.cheby_from_host = ro.eam ? 1 : 0;
  rc = comdgb_attach(sim, &o);
  if (rc) return fail("comdgb_attach", rc);
  if (ro.lazy && (rc = comdgb_set_lazy(sim, 1))) return fail("comdgb_set_lazy", rc);
  sim->pot->force = comdgb_force;
  printf("Initialization finished\n");

  /* do_compute_work (docompute.c:166-218) */
  const double dt = 1.0e-15;
  printf("Starting simulation\n");
  double ts = now_s();
  rc = sim->pot->force(sim); /* computeForce, timestep.c:110-112 */
  double te = now_s();
  if (rc) return fail("computeForce", rc);
  printf("Starting timesteps\n");
  double steps_s = 0.0; /* host time inside comdgb_nTimeSteps */
  int iter;
  for (iter = 0; iter < ro.niter; iter++) {
    const double ns = iter == 0 ? 1.0 : (double)(1 + ro.nsteps);
    printf(" %3d %30.20g computed in %.3fs (%8.4f us/atom for %d atoms)\n", iter * ro.nsteps,
           sim->e, te - ts, 1.0e6 * (te - ts) / ns / (double)sim->ntot, sim->ntot);
    printf("Virial stress = %.17g\n", sim->stress);
    ts = now_s();
    const double eone = comdgb_nTimeSteps(ro.nsteps, sim, dt);
    te = now_s();
    steps_s += te - ts;
    if (eone != eone) return fail("comdgb_nTimeSteps", COMDGB_ERR_CUDA);
  }
  printf(" %3d %30.20g computed in %.3fs (%8.4f us/atom for %d atoms)\n", iter * ro.nsteps,
         sim->e, te - ts, 1.0e6 * (te - ts) / (double)(ro.nsteps + 1) / (double)sim->ntot,
         sim->ntot);
  printf("Virial stress = %.17g\n", sim->stress);
  printf("comdgb_run: iterations %d steps %d atoms %d final_energy %.17g\n", ro.niter,
         ro.nsteps, sim->ntot, sim->e);
  /* the same run as one JSON record: atom-steps/s over the nTimeSteps calls
   * (host clock, each call with its trailing force call and copies) */
  const double atom_steps = (double)sim->ntot * (double)ro.niter * (double)ro.nsteps;
  printf("{\"comdgb_run\": {\"atoms\": %d, \"iterations\": %d, \"steps_per_call\": %d, "
         "\"potential\": \"%s\", \"precision\": \"%s\", \"lazy\": %d, "
         "\"seconds_in_nTimeSteps\": %.6f, \"atom_steps_per_s\": %.6g, "
         "\"final_energy\": %.17g, \"final_stress\": %.17g}}\n",
         sim->ntot, ro.niter, ro.nsteps,
         !ro.eam ? "lj" : ro.cheby ? "eam_cheby" : "eam_table", ro.mixed ? "mixed" : "fp64",
         ro.lazy, steps_s, steps_s > 0.0 ? atom_steps / steps_s : 0.0, sim->e, sim->stress);

  rc = comdgb_detach(sim); /* brings the state home (lazy mode) */
  if (rc) return fail("comdgb_detach", rc);
  comdgb_sim_free_host(sim);
  if (ch) comdgb_cheb_free(ch);
  if (eam) comdgb_eam_free(eam);
  if (lj) comdgb_lj_free(lj);
  return 0;
}
