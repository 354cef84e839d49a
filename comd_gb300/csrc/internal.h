// internal.h -- launchers shared between the kernel translation units and the
// host API (api.cu).  All launches go to the caller's stream.
#pragma once

#include "common.cuh"
#include "force_kernels.cuh"

namespace cg {

// rebin scratch (one set per simulation)
struct RebinWork {
  uint32_t *depmask;    // [2*nboxes] departure bits of slots 0-31 / 32-63
  int *arr_lo, *arr_hi; // [nboxes] arrivals from lower / higher boxes (same
                        // allocation as depmask, cleared with it: 4*nboxes words)
  int *n_lo;            // [nboxes] arrivals from lower-index boxes
  int *final_len;       // [nboxes] occupancy after the box's own scan
  uint8_t *final_src;   // [nboxes*64] slot t <- old slot (<64) or placeholder 64+p
  uint8_t *dep_rank;    // [nboxes*64] departure rank of a departing old slot
  int *arr_list;        // [2*nboxes*64] old slots of the arrivals of a box
                        // from lower / higher boxes, in claim order
  Slots stage;          // full records of departing atoms, indexed by old slot
  Persist pl;           // id-keyed persistent lists: displacement check
  ForceOrder fo;        // force order: positions to track (fo.of_id null: none)
  SlotMap map;          // slot maps the rebin keeps
};

// ---- md_kernels.cu ----
// packed box coordinates (g.boxc must point at boxc) and the stencil table
void launch_entry_table(const Geom &g, const double *dcenter, EntryTab et, int *boxc,
                        cudaStream_t st);
double mass_reciprocal(double rmass);
// The Verlet and classify kernels run one thread per atom of the compacted
// atom list atom_slot (which must match the current layout).
// r += dt*p/rmass (and optionally the classify step of reBoxAll)
// use_delta: add the increments the previous step's last half step left in
// f.xyz when the status word says they are there (step graphs only)
void launch_advance_positions(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt,
                              double rmass, bool mixed, bool classify, const RebinWork &w,
                              int *status, cudaStream_t st, bool use_delta = false);
// p -= dt_v*f; r += dt_r*p/rmass; classify (the FP32 copy is not refreshed);
// FP64 leaves the position increments in f.xyz and says so in the status word
// write32: also the FP32 copies and the force-order tracking (the closing
// part of a merged mixed-precision sequence)
void launch_advance_vp(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                       double dt_r, double rmass, bool mixed, const RebinWork &w, int *status,
                       cudaStream_t st, bool write32 = false);
// merged rebox (mixed precision): p -= dt_v*f, then the closing position
// half step of one step and the opening one of the next with no rebox
// between them (one update r += p*(2*dt_r/rmass)), the FP32 copy, the list
// tracking and classify
void launch_advance_vpp(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                        double dt_r, double rmass, bool mixed, const RebinWork &w, int *status,
                        cudaStream_t st, bool classify = true);
// p -= dt_v*f only (advanceVelocity)
void launch_advance_velocity(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                             cudaStream_t st);
// classify only (reBoxAll without a position update); only_if (optional):
// the status words of a force-order simulation whose rebox waits for list
// rebuilds: nothing is classified unless a rebuild is due (ST_REBUILD)
void launch_classify(const Geom &g, Slots s, const int *atom_slot, int ntot, bool mixed,
                     const RebinWork &w, int *status, cudaStream_t st,
                     const int *only_if = nullptr);
// plan + apply + serial fallback; must follow a classify launch.  only_if
// (optional) as above; while it stands the launches down they do nothing
// (the atoms stay in the boxes they had, their box-relative positions as
// the half steps left them)
void launch_rebin_finish(const Geom &g, Slots s, bool mixed, const RebinWork &w, int *status,
                         cudaStream_t st, const int *only_if = nullptr);
// the atom list of the layout; only_if as above (the layout did not change)
void launch_compact(const Geom &g, const int *natoms, int *box_start, int *atom_slot, int ntot,
                    int *partials, int npart, cudaStream_t st, const int *only_if = nullptr);
int compact_partials(int nboxes);
void launch_reduce(const ForceArgs &A, double *partials, long long *ipartials, int npart,
                   double *out, long long *iout, cudaStream_t st);
int reduce_partials(int ntot);
void launch_kinetic(const Geom &g, Slots s, const int *atom_slot, int ntot, double rmass,
                    double *partials, int npart, double *out, cudaStream_t st);
void launch_unpack3(const double *src3, d4 *dst, long n, cudaStream_t st);
void launch_add_offset(int *v, long n, int off, cudaStream_t st);
// per replica: out[2r] energy sum, out[2r+1] stress sum
void launch_rep_reduce(const ForceArgs &A, double *out, cudaStream_t st);
void launch_pack3(const d4 *src, double *dst3, long n, cudaStream_t st);
// A host simflat_t's registered slot arrays as the device addresses them
// (r, p: 3 doubles per slot; f: 4).
struct HostSlots {
  int *id, *itype;
  double *mass, *r, *p, *f, *rho, *fi;
};
// Transfers of the occupied slots only (k < natoms[b]; the device natoms
// must hold the layout), one warp per box, the kernel reading or writing
// host memory directly in whole lines: no staging copy, no bytes for empty
// slots.
// upload: id, itype, mass, r, p (and f, rho, fi when forces)
void launch_zc_upload(const HostSlots &hs, Slots s, int nboxes, bool forces, cudaStream_t st);
// download of the state (id, itype, mass, r, p) or of the force results
// (f, rho, fi)
void launch_zc_download(const HostSlots &hs, Slots s, int nboxes, bool state, bool forces,
                        cudaStream_t st, int max_blocks = 0);
void launch_pos32(const Geom &g, Slots s, cudaStream_t st, const int *only_if_overflow = nullptr);
void launch_bin_atoms(const Geom &g, const double *dcenter, Slots s, int n, const double *xyz,
                      const double *pxyz, const int *ids, const int *types, const double *masses,
                      int *tmp_index, int *status, cudaStream_t st);
void launch_cheb_fit(const double *table_v, double x0, double xn, double invdx, int n_terms,
                     double *coef, double *dcoef, cudaStream_t st);

// persistent lists: id -> slot map of the current layout (ids must be
// 0..ntot-1; a duplicate or out-of-range id sets ST_ERROR to -1), and the
// end of a (possible) rebuild
void launch_slot_of(const Geom &g, Slots s, Persist pl, int ntot, int *status, cudaStream_t st);
void launch_rebuild_done(int *status, cudaStream_t st);
// launch_rebuild_done, then sets `cond` to whether a current list overflowed
void launch_rebuild_done_cond(int *status, cudaGraphConditionalHandle cond, cudaStream_t st);
// sets the conditional node `cond` to whether status word `word` is set
void launch_status_cond(cudaGraphConditionalHandle cond, const int *status, int word,
                        cudaStream_t st);
void launch_skin_check(const Geom &g, Slots s, Persist pl, bool mixed, int *status,
                       cudaStream_t st);
void launch_fo_track(const Geom &g, Slots s, const ForceOrder &fo, const int *atom_slot,
                     int ntot, int *status, cudaStream_t st);
// after an upload that keeps the lists: force-order slots of the new layout
void launch_fo_reslot(const Geom &g, Slots s, const ForceOrder &fo, int ntot, cudaStream_t st);

// Launch shapes of the mixed-precision force-order kernels (results do not
// depend on them): the list build's threads per box and atoms tested per
// candidate load, pass 2's threads per CTA and its grid cap (0: the resident
// CTAs of the default shape)
struct Tune {
  int build_threads = 128, build_atoms = 4;
  int pass2_threads = 512, pass2_blocks = 0;  // force pass: 2 CTAs of 512 per SM
  int pass2_blocks_fast = 0;  // the same for the force pass without energies (OBS = false)
};

// ---- force_fp64.cu (T = double) / force_mixed.cu (T = float) ----
template <class T>
cudaError_t prepare_force_kernels();
template <class T>
void launch_nbr_build(const ForceArgs &A, T rc2, cudaStream_t st, const Tune *tune = nullptr);
template <class T, int EVAL>
void launch_eam_pass1(const ForceArgs &A, const EamPot<T, EVAL> &P, cudaStream_t st);
template <class T, int EVAL>
void launch_eam_pass2(const ForceArgs &A, const EamPot<T, EVAL> &P, cudaStream_t st);
template <class T>
void launch_lj(const ForceArgs &A, const LjPot<T> &P, cudaStream_t st);
// force order (mixed precision only, force_mixed.cu); pass 0 or 1.  obs:
// the caller can read this force call's energies, stress, rho and F' (else
// forces only: the force calls inside a step sequence)
template <int EVAL>
void launch_fo_eam(const ForceArgs &A, const EamPot<float, EVAL> &P, int pass, cudaStream_t st,
                   const Tune *tune = nullptr, bool obs = true);
// resident-CTA grid cap of pass 2 at `threads` per CTA (SMs x CTAs per SM),
// with or without energies; call outside stream capture
int fo_pass2_blocks(int eval, bool multi, int threads, bool obs = true);
void launch_fo_lj(const ForceArgs &A, const LjPot<float> &P, cudaStream_t st, bool obs = true);

}  // namespace cg
