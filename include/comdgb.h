/*
 * comdgb.h -- C ABI of libcomdgb.so, the GB300 (sm_103a) implementation of
 * CoMD's force-and-integrate timestep.
 *
 * Two ways in:
 *  1. Drop-in on a host simflat_t (the reference's own data model,
 *     include/comdgb_simflat.h).  comdgb_attach() mirrors the simulation
 *     on the GPU; comdgb_force() has the signature of the potential's force
 *     pointer (src-flat/include/pmdTypes.h:77) so `s->pot->force =
 *     comdgb_force` makes the reference's computeForce
 *     (src-flat/timestep.c:110-112) run on the GPU; comdgb_nTimeSteps()
 *     replaces nTimeSteps (src-flat/timestep.c:114-140).  The host simflat_t
 *     stays the source of truth: every such call copies the host state to
 *     the GPU and the results back.
 *  2. Device-resident handles (comdgb_sim_*) for callers that keep the
 *     state on the GPU between calls and read it back only when asked.
 *
 * Every function returns 0 or a negative COMDGB_ERR_* code (the reference
 * exit()s instead); comdgb_last_error() gives the message.  All functions
 * are host functions; one library instance drives one GPU per handle.
 */
#ifndef COMDGB_H
#define COMDGB_H

#include <stddef.h>
#include <stdio.h>
#include <stdint.h>

#include "comdgb_simflat.h"

#ifdef __cplusplus
extern "C" {
#endif

/* potential kinds */
enum {
  COMDGB_POT_EAM_TABLE = 0, /* eamForce with eamInterpolateDeriv, src-flat/eam.c:438-660 */
  COMDGB_POT_EAM_CHEBY = 1, /* eamForce built with -DUSE_CHEBY, src-flat/cheby.c:276-310 */
  COMDGB_POT_LJ = 2         /* LJ, src-flat/ljForce.c:89-224 */
};

/* arithmetic of the force kernels (integration is always FP64) */
enum {
  COMDGB_PREC_FP64 = 0,  /* every pair term in double precision; the Verlet
                            half steps round as the reference does */
  COMDGB_PREC_MIXED = 1  /* FP32 pair terms on box-relative coordinates,
                            Kahan-compensated FP32 per-atom sums, FP64 totals;
                            FP64 Verlet half steps as fused multiply-adds,
                            p - dt*f and r + p*(dt/M) */
};

/* error codes; -11 and -3 keep the reference's abort codes */
enum {
  COMDGB_OK = 0,
  COMDGB_ERR_ARG = -1,
  COMDGB_ERR_NOBOX = -3,        /* "Need at least one cutoff wide domain" domains.c:180 */
  COMDGB_ERR_MAXATOMS = -11,    /* "Increase maxatoms" domains.c:229 */
  COMDGB_ERR_BOXRANGE = -12,    /* an atom's box index fell outside the grid */
  COMDGB_ERR_CUDA = -30,
  COMDGB_ERR_NOMEM = -31,
  COMDGB_ERR_NOTATTACHED = -32,
  COMDGB_ERR_IO = -33,
  COMDGB_ERR_UNSUPPORTED = -34,
  COMDGB_ERR_NONFINITE = -35    /* NaN/Inf in the total energy */
};

typedef struct comdgb_opts {
  int potential;   /* COMDGB_POT_* */
  int precision;   /* COMDGB_PREC_* */
  int periodic;    /* 1: periodic boundaries (reference default PERIODIC=1) */
  int device;      /* CUDA device ordinal */
  int n_cheby;     /* Chebyshev terms; only 32 is supported (NUM_CHEBY, docompute.c:56) */
  int cheby_from_host; /* 1: take the series from s->ch_pot; 0: fit them on the GPU */
  int list_mode;       /* COMDGB_LIST_AUTO (default) or COMDGB_LIST_PER_STEP */
  double skin;         /* persistent-list skin in Angstrom (default 0.5; at most the
                          boxes' width minus the cutoff) */
} comdgb_opts;

/* Neighbour lists.  AUTO keeps lists across steps (cutoff rc + skin, keyed
 * by atom id, rebuilt when an atom has moved more than skin/2) whenever the
 * grid allows it: periodic, at least 3 boxes per axis, boxes at least
 * rc + 0.1 A wide and ids 0..ntot-1; otherwise, and with PER_STEP, the list
 * is rebuilt from the link cells at every force call.  Both give the same
 * set of pairs within rc. */
enum { COMDGB_LIST_AUTO = 0, COMDGB_LIST_PER_STEP = 1 };

/* fills o with the reference defaults (EAM table, FP64, periodic, device 0) */
void comdgb_default_opts(comdgb_opts *o);

/* ---------------- drop-in API on a host simflat_t ---------------- */

/* Mirror s on the GPU.  s->pot must be an eampotential_t (EAM kinds) or an
 * ljpotential_t (LJ); for COMDGB_POT_EAM_CHEBY with cheby_from_host, s->ch_pot
 * must be set (setChebPot, src-flat/cheby.c:99-121). */
int comdgb_attach(simflat_t *s, const comdgb_opts *o);
/* Drop-in for the potential's force pointer (pmdTypes.h:77): copies the host
 * slot arrays up, computes, writes f, rho, fi, e and stress back into s. */
int comdgb_force(void *s);
/* Drop-in for nTimeSteps (timestep.c:114-140): n velocity-Verlet steps and a
 * final force call on the GPU; dt in seconds; returns s->e (NaN on error,
 * see comdgb_last_error). */
double comdgb_nTimeSteps(int n, simflat_t *s, double dt);
/* Drop-in for reBoxAll (domains.c:347-389) on the GPU. */
int comdgb_reBoxAll(simflat_t *s);
/* Releases the mirror; in lazy mode the host first gets the device state. */
int comdgb_detach(simflat_t *s);
/* Lazy mode (off by default).  The drop-in calls above keep the state on the
 * GPU between calls and write back only s->e and s->stress.  The host's slot
 * arrays are brought up to date by comdgb_sync_to_host (and by
 * comdgb_detach, or by leaving lazy mode).  After the host changes them,
 * comdgb_sync_to_device makes the GPU take them.  With lazy mode off, every
 * call copies the state up and its results back. */
int comdgb_set_lazy(simflat_t *s, int lazy);
int comdgb_sync_to_host(simflat_t *s);
int comdgb_sync_to_device(simflat_t *s);
/* Bytes copied host -> device and device -> host for s since it was
 * attached.  The attached arrays are registered.  Uploads and downloads of
 * f, rho and fi are kernels that read or write the occupied slots only
 * (the slots of the ntot atoms, after natoms).  The state after nTimeSteps
 * streams back by the copy engines while the trailing force call runs, as
 * 2D copies of each box's slots up to the largest occupancy (so do all
 * copies where registration fails).  A force call or nTimeSteps does not
 * upload f, rho and fi (it computes them before reading them). */
int comdgb_transfer_bytes(simflat_t *s, long long *h2d, long long *d2h);

/* ---------------- device-resident handles ---------------- */

typedef struct comdgb_sim comdgb_sim;

/* Creates a GPU simulation from a host simflat_t (copied; s is not kept). */
int comdgb_sim_create(const simflat_t *s, const comdgb_opts *o, comdgb_sim **out);
void comdgb_sim_destroy(comdgb_sim *h);
/* copy the host simulation's slot arrays to the GPU / the GPU's back */
int comdgb_sim_upload(comdgb_sim *h, const simflat_t *s);
int comdgb_sim_download(comdgb_sim *h, simflat_t *s);
/* one force evaluation on the GPU state (results stay on the GPU) */
int comdgb_sim_force(comdgb_sim *h);
/* n steps + final force on the GPU state; dt in seconds; captured in a
 * CUDA graph after the first call with the same dt */
int comdgb_sim_steps(comdgb_sim *h, int n, double dt);
/* reBoxAll (domains.c:347-389) on the GPU state */
int comdgb_sim_rebox(comdgb_sim *h);
/* advanceVelocity (timestep.c:62-74): p -= dt f; dt in the reference's
 * internal time unit (seconds * 0.529/2.418e-17, timestep.c:126) */
int comdgb_sim_advance_velocity(comdgb_sim *h, double dt);
/* advancePositions (timestep.c:76-108): r += dt p / (1822.83 m), then reBoxAll */
int comdgb_sim_advance_positions(comdgb_sim *h, double dt);
/* totals of the last force call: energy, stress (reference definitions) */
int comdgb_sim_energy(comdgb_sim *h, double *e, double *stress);
/* kinetic energy sum p^2/2M on the GPU */
int comdgb_sim_kinetic(comdgb_sim *h, double *ek);
/* device-side counters: unique in-cutoff pairs of the last force call */
int comdgb_sim_pair_count(comdgb_sim *h, long long *pairs);
/* waits for the handle's queued GPU work (COMDGB_ERR_CUDA if it failed) */
int comdgb_sim_synchronize(comdgb_sim *h);

/* Timed run for benchmarks: `n` steps (graph replays), events recorded on
 * the library's stream; step_ms[0..n-1] gets each step's device time,
 * step_ms[n] the span from the first step's start to the last step's end,
 * and kernel_ms[k] the average device time of kernel group k of a step
 * (names via comdgb_kernel_name).  Returns the number of groups per step.
 * With the rebox merged (comdgb_sim_set_merge_rebox) the steps run as an
 * opening part, n-1 middle parts and a closing part: step_ms[0..n-2] and
 * kernel_ms are the middle parts', step_ms[n-1] the opening and closing
 * parts' together, step_ms[n] the span of all of them. */
int comdgb_sim_timed_steps(comdgb_sim *h, int n, double dt, float *step_ms,
                           float *kernel_ms, int max_kernels);
const char *comdgb_kernel_name(comdgb_sim *h, int k);
/* nTimeSteps(n, ., dt) with the n steps captured as ONE CUDA graph (captured
 * at the first call for this n and dt, then replayed), launched once; *ms
 * (optional) = that launch's device time.  Ends with the force call. */
int comdgb_sim_graph_steps(comdgb_sim *h, int n, double dt, float *ms);
/* kernels a sequence of n steps launches (after a step has run): n times
 * the step graph's, or with the rebox merged the opening part's, n-1 middle
 * parts' and the closing part's.  In force order (mixed precision with skin
 * lists) a step part's rebuild section -- classify, rebin, compact, list
 * build -- is the body of a conditional graph node and launches only in
 * steps that rebuild the lists: comdgb_sim_rebuild_launches gives its
 * kernels, to be added once per rebuild (comdgb_sim_list_info counts them). */
int comdgb_sim_step_launches(comdgb_sim *h, int n, long long *launches);
int comdgb_sim_rebuild_launches(comdgb_sim *h, int *kernels);
/* kernels launched per replay of the captured step graph / force graph
 * (with the rebox merged: per middle part) */
int comdgb_sim_graph_kernels(comdgb_sim *h, int *per_step, int *per_force);
/* Launch shapes of the mixed-precision force-order kernels, for autotuning
 * (0 keeps the default): the skin-list build's threads per box -- the
 * threads per cell -- (64, 128 or 256; default 128) and atoms tested per
 * candidate load (2, 4 or 8; default 4), and pass 2's threads per CTA (128,
 * 256 or 512; default 512).  Results do not depend on them (the lists and
 * every per-atom sum keep their order); the graphs are recaptured. */
int comdgb_sim_set_launch(comdgb_sim *h, int build_threads, int build_atoms, int pass2_threads);
/* Mixed precision only (its default): a sequence of steps reboxes once per
 * step instead of after each position half step (timestep.c:129-132 with
 * reBoxAll at the end of advancePositions, timestep.c:106).  The closing
 * half step of one step and the opening one of the next become one position
 * update, r + p*(dt/M), and one rebox follows; with skin lists in force
 * order that rebox (and the atom list) waits until a list rebuild is due,
 * the force passes reading no layout in between.  The last step of a call
 * still ends with its own rebox.  The positions differ from the unmerged ones by
 * roundings, and atoms may sit in other slots of their boxes.  0 restores
 * the reference's two reboxes per step (FP64 always has them). */
int comdgb_sim_set_merge_rebox(comdgb_sim *h, int on);
/* Mixed precision, EAM Chebyshev: whether the pair functions come from the
 * FP32 cubic segment table in r^2 fitted to the FP64 series (on = 1, the
 * default) or from the reference's 32-term series evaluated in FP32 for
 * every pair (0; no counterpart needed in the reference, whose FP64 path
 * always sums the series, cheby.c:276-310).  Other potentials and FP64
 * ignore it.  The graphs are recaptured. */
int comdgb_sim_set_pair_table(comdgb_sim *h, int on);
/* Neighbour-list capacity in use (entries per atom), at most the capacity
 * allocated at creation (0 restores it); no counterpart in the reference,
 * whose loops have no lists.  Atoms with more neighbours than the capacity
 * are computed by scanning their 27 neighbour boxes instead, with the same
 * results up to roundings, so a lower capacity exercises that path.  Lists
 * in use are rebuilt at the next force call; the graphs are recaptured. */
int comdgb_sim_set_list_capacity(comdgb_sim *h, int cap);
/* list mode in use (1 persistent, 0 per step), its skin, and the number of
 * persistent-list builds since the last upload */
int comdgb_sim_list_info(comdgb_sim *h, int *persistent, double *skin, long long *builds);
/* measured FP32 FMA throughput of the device (TFLOP/s, FMA = 2 flops); the
 * peak the mixed-precision force kernels are compared against */
int comdgb_fp32_fma_peak(int device, double *tflops);
/* y[i] = x[i] rounded to FP32 (nearest, ties to even) by the integer routine
 * the mixed-precision kernels use for positions; runs on the host */
int comdgb_round_f32(const double *x, float *y, long n);

/* ---------------- batched replicas ---------------- */
/* n independent simulations (uneven sizes allowed) with one potential (that
 * of sims[0]) and the same options, advanced together: every kernel of a
 * step runs once over all replicas' boxes and atoms, each replica on its own
 * box grid and rebinned exactly as reBoxAll rebins it alone.  The handle
 * takes every comdgb_sim_* call (energy: the sum over replicas); uploads and
 * downloads go per replica. */
int comdgb_batch_create(const simflat_t *const *sims, int n, const comdgb_opts *o,
                        comdgb_sim **out);
/* the number of replicas; replica r's host state to the GPU (s must have
 * the replica's grid) and back */
int comdgb_batch_replicas(comdgb_sim *h);
int comdgb_batch_upload(comdgb_sim *h, int r, const simflat_t *s);
int comdgb_batch_download(comdgb_sim *h, int r, simflat_t *s);
/* per-replica total energy and scalar stress of the last force call */
int comdgb_batch_energies(comdgb_sim *h, double *e, double *stress);

/* Batch autotuner.  No counterpart in the reference (one system, no
 * tunable launches).  Times every (box factor, skin) candidate as a batch of
 * the replicas rebinned at that box factor (`steps` steps as one CUDA graph
 * after a warm-up replay), then at the best pair the list build's threads
 * per box (64, 128, 256) and atoms per candidate load (2, 4, 8), then the
 * force pass's threads per CTA (128, 256, 512).  nbf = 0: the replicas' own
 * box factor; nskin = 0: o->skin.  Box factors at which a box of some
 * replica would pass 64 atoms are skipped.  cache_path (NULL: none) is a
 * text file keyed by the GPU, the replicas' sizes and bounds, the options
 * and the candidates: a system tuned before returns at once with
 * from_cache = 1; a new result is appended.  The caller adopts the box
 * factor by building its replicas at it (comdgb_rebin_host does that for a
 * host simflat_t), the skin through comdgb_opts.skin, and the launch shapes
 * with comdgb_sim_apply_tune. */
typedef struct comdgb_tune {
  double box_factor;
  double skin;
  int build_threads, build_atoms, pass2_threads;
  double ms_per_step;  /* measured for the choice (the cached value when from_cache) */
  int from_cache;
} comdgb_tune;
int comdgb_batch_autotune(const simflat_t *const *sims, int n, const comdgb_opts *o,
                          const double *box_factors, int nbf, const double *skins, int nskin,
                          int steps, double dt, const char *cache_path, comdgb_tune *out);
int comdgb_sim_apply_tune(comdgb_sim *h, const comdgb_tune *t);
/* A new host simflat_t with the atoms of s binned at box factor bf
 * (allocDomains then one putAtomInBox per atom in id order, domains.c:155-200,
 * 237-291); COMDGB_ERR_MAXATOMS in *status when a box would pass 64 atoms.
 * Free with comdgb_sim_free_host. */
simflat_t *comdgb_rebin_host(const simflat_t *s, double bf, int *status);

/* Launch-structure probes (no counterpart in the reference): the cost of one
 * kernel node of a CUDA graph whose kernel does nothing (4 CTAs of 256
 * threads per SM, as the step's stood-down launches), and of one grid-wide
 * barrier inside a cooperative kernel of every resident CTA (what a
 * persistent step kernel would pay between phases).  Microseconds. */
int comdgb_graph_node_cost(int device, double *us_per_node);
int comdgb_grid_barrier_cost(int device, double *us_per_barrier);

/* ---------------- gradients and adjoint (FP64 simulations) ---------------- */
/* Parameters.  EAM Chebyshev: the base series phi, rho, F -- coef[32*q + k],
 * q = 0 phi, 1 rho, 2 F, on [x0[q], xn[q]] -- whose derivative series follow
 * as genDer derives them (cheby.c:219-270).  LJ: (epsilon, sigma) at the
 * fixed cutoff.  The gradient calls compute the forces first (FP64). */
int comdgb_sim_set_cheby(comdgb_sim *h, const double *coef, const double *x0, const double *xn);
int comdgb_sim_get_cheby(comdgb_sim *h, double *coef, double *x0, double *xn);
int comdgb_sim_set_lj(comdgb_sim *h, double epsilon, double sigma);
/* total energy U at the current positions and dU/d(parameters): 96 values
 * (EAM Chebyshev, coef order) or 2 (LJ: epsilon, sigma) */
int comdgb_sim_energy_grad(comdgb_sim *h, double *energy, double *grad);
/* force-matching loss L = sum_i |f_i - target[id_i]|^2 (target: 3 doubles per
 * atom id, host memory; f as the reference defines it) and dL/d(parameters) */
int comdgb_sim_force_loss_grad(comdgb_sim *h, const double *target, double *loss, double *grad);
/* J = U after n velocity-Verlet steps of dt seconds from the current state and
 * dJ/d(parameters) (EAM Chebyshev), by the reverse of the loop with the state
 * checkpointed every `every` steps and the steps in between recomputed; the
 * state is left as after the n steps */
int comdgb_sim_traj_energy_grad(comdgb_sim *h, int n, double dt, int every, double *j,
                                double *grad);

/* ---------------- virial tensor and per-atom stress ---------------- */
/* The reference reports one scalar, s->stress (eam.c:649: x-x of the
 * embedding term only; ljForce.c:175,210: x-x with the kinetic term added
 * once per neighbour box); force calls keep that value as it is.  These
 * calls give the physical tensors next to it.  Voigt order xx yy zz yz xz
 * xy, energy units (Hartree; lengths in Angstrom):
 *   w = sum over pairs of dr_ij (x) F_ij   F_ij the force on i from j,
 *                                          dr_ij = r_i - r_j
 *   k = sum over atoms of p (x) p / M      M = mass x amu_to_m_e
 * The pressure tensor is (k + w) / volume.  comdgb_sim_virial runs a force
 * call on the current state, then the virial of every replica, and reports
 * replica 0 (a batch: comdgb_batch_virial for the others). */
int comdgb_sim_virial(comdgb_sim *h, double w[6], double k[6], double *volume);
/* replica r's tensors and volume from the last comdgb_sim_virial call */
int comdgb_batch_virial(comdgb_sim *h, int r, double w[6], double k[6], double *volume);
/* per-atom stress x volume from the last comdgb_sim_virial call,
 * -(p (x) p / M + 1/2 sum_j dr_ij (x) F_ij), in replica r's slot layout:
 * out[6 * (box * 64 + i) + c] for the replica's boxes (empty slots 0) */
int comdgb_sim_atom_stress(comdgb_sim *h, int r, double *out);

/* ---------------- centrosymmetry ---------------- */
/* The visualiser's centrosymmetry parameter (src-viz/AtomVisualize.c:399-672)
 * of every atom of replica r, from the 12 nearest candidates in the 27
 * boxes around its own: the least sum of |r_a + r_b|^2 over the pairings of
 * the 12 (approx = 0, the default build) or the greedy pairing
 * (approx = 1, APPROX_CENTROSYM); 1000 for fewer than 12 candidates.
 * out (optional): one double per slot of the replica's boxes (empty slots
 * 0), the layout of the visualiser's sim->centro; *cmin / *cmax (optional):
 * the range over the replica's atoms (minCentro, maxCentro before the
 * visualiser clamps the latter to 100). */
int comdgb_sim_centrosymmetry(comdgb_sim *h, int r, int approx, double *out, double *cmin,
                              double *cmax);

/* ---------------- host-side setup (reference setup routines) ---------------- */

/* setEamPot / eamReadASCII (eam.c:102-109, 347-398): reads <dir>/<name>.{phi,rho,f,doc} */
eampotential_t *comdgb_eam_read(const char *dir, const char *name);
void comdgb_eam_free(eampotential_t *p);
/* setChebPot (cheby.c:99-121), the series fitted in FP64 on the GPU */
eam_cheby_t *comdgb_cheb_make(const eampotential_t *p, int n, int device);
void comdgb_cheb_free(eam_cheby_t *c);
/* an LJ potential (getLJPot, ljForce.c:75-86, with caller parameters) */
ljpotential_t *comdgb_lj_make(double sigma, double epsilon, double cutoff, double mass);
void comdgb_lj_free(ljpotential_t *p);
/* create_fcc_lattice (ic_fcc.c:63-141) into a new host simflat_t */
simflat_t *comdgb_fcc(int nx, int ny, int nz, double lat, double defgrad, double bf,
                      pmd_base_potential_t *pot, int *status);
/* fromFileGzip / fromFileASCII (read.c:155-241): a clsman file (gzip when
 * the library was built with zlib, else plain text; COMDGB_ERR_UNSUPPORTED
 * for gzip without zlib) into a new host simflat_t: allocDomains' grid for
 * box factor bf, atom i with id i, type 0 and the potential's mass, binned as
 * successive putAtomInBox calls on the GPU `device` (device < 0: on the
 * host).  The caller reboxes, as initSimFromCmdLine does. */
simflat_t *comdgb_read_clsman(const char *path, pmd_base_potential_t *pot, double bf, int device,
                              int *status);

/* fromFileTim (read.c:248-315): a raw array of FileAtom records (five native
 * floats x, y, z, bond order, centrosymmetry) into a new host simflat_t; the
 * reference's fixed bounds (327.424 x 354.446877 x 3007.581486 A, rounded to
 * float as the reference holds them) unless
 * `bounds` is given; atom i: id i, type 1, the potential's mass, zero
 * momenta; binned on the GPU `device` (device < 0: on the host). */
simflat_t *comdgb_read_tim(const char *path, pmd_base_potential_t *pot, double bf,
                           const double *bounds, int device, int *status);

/* ---------------- clsman output (write.c) ---------------- */
enum {
  COMDGB_CLSMAN_BINARY = 0,  /* writeClsman (write.c:112-167), byte for byte */
  COMDGB_CLSMAN_TEXT_GZ = 1, /* gzASCIIWrite (write.c:175-220); gzip members, one per chunk */
  COMDGB_CLSMAN_TEXT = 2     /* the same text, uncompressed (fromFileASCII reads it) */
};
/* replica r's atoms in id order, gathered on the device (getRL, write.c:58-87):
 * out[6 * id + 0..2] = box corner + r (write.c:157), [3..5] = p; ids must be
 * 0..ntot-1, each once (else COMDGB_ERR_ARG, nothing written) */
int comdgb_sim_gather(comdgb_sim *h, int r, double *out);
/* replica r's current state to `path` in `format`; `comment` is the text
 * file's comment line (a newline is added when it has none; NULL: empty) */
int comdgb_sim_write_clsman(comdgb_sim *h, int r, const char *path, int format,
                            const char *comment);
/* drop-ins for writeClsman(s, fname) and gzASCIIWrite(s, fname): a simflat_t
 * attached in lazy mode is gathered on the device (it holds the current
 * state), any other on the host */
int comdgb_writeClsman(simflat_t *s, const char *fname);
int comdgb_gzASCIIWrite(simflat_t *s, const char *fname);
/* printIt (write.c:89-110): the atoms with id < 10, box by box */
void comdgb_printIt(const simflat_t *s, FILE *fp);
/* seeded displacement / momenta (include/comdgb_seed.h) followed by nothing;
 * the caller reboxes */
void comdgb_seed(simflat_t *s, uint64_t seed, int disp_kind, double amp, double temp_k,
                 double mass_amu);
/* frees a host simflat_t made by comdgb_fcc, comdgb_read_clsman,
 * comdgb_read_tim or comdgb_rebin_host (not its potential) */
void comdgb_sim_free_host(simflat_t *s);
/* reBoxAll on the host simflat_t via the GPU (upload, rebox, download) */
int comdgb_rebox_host(simflat_t *s, int periodic, int device);

/* Bin atoms given in id order by their world coordinates on the GPU, with
 * the slot order of n successive putAtomInBox calls (domains.c:237-291).
 * s must have its domains allocated (nbx, boxsize, dcenter, arrays) and no
 * atoms; fills natoms, id, iType, mass, r, p, ntot. */
int comdgb_put_atoms(simflat_t *s, int n, const double *xyz, const double *pxyz,
                     const int *ids, const int *itypes, const double *masses, int device);

/* Allocation-free binning.  No counterpart in the reference: it is
 * comdgb_put_atoms for callers that cannot allocate device memory while
 * they run (an engine owning all GPU memory through its own arena,
 * latency-critical loops where cudaMalloc's implicit synchronisation would
 * stall the GPU).  All arrays are device pointers in the reference's slot
 * layout (r and p as real3 rows, slot = box*64 + k); dcenter is nbx product
 * x 3 doubles.  The result equals comdgb_put_atoms: n putAtomInBox calls in
 * array order; an atom whose coordinates are not finite, or that lies more
 * than one period outside, gives COMDGB_ERR_BOXRANGE, a box of more than 64
 * atoms COMDGB_ERR_MAXATOMS.  Scratch is a library-owned device array of
 * COMDGB_NOALLOC_MAX_BOXES*64 ints (4 MiB per device, held until the
 * process exits); larger grids are rejected with COMDGB_ERR_ARG.  The first
 * call on a device looks up that array's address (cudaGetSymbolAddress) --
 * make it before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race.  The call makes `device` current for its work
 * and restores the caller's current device; it synchronises `stream` (a
 * cudaStream_t, NULL = default) to report errors. */
#define COMDGB_NOALLOC_MAX_BOXES 16384
int comdgb_put_atoms_noalloc(const int nbx[3], const double bounds[3], const double boxsize[3],
                             const double *dcenter, int n, const double *xyz, const double *pxyz,
                             const int *ids, const int *itypes, const double *masses,
                             int *natoms, int *id, int *itype, double *mass, double *r, double *p,
                             int device, void *stream);

/* The message of the last failing call made by the calling thread (each
 * thread has its own), copied into buf and truncated to len - 1 characters
 * (buf may be NULL); returns the message's full length. */
int comdgb_last_error(char *buf, int len);
/* "comdgb <version> sm_103a" */
const char *comdgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* COMDGB_H */
