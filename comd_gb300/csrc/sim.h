// sim.h -- the device simulation object behind the C ABI handle and the
// host helpers shared by the API translation units (api.cu, adjoint.cu).
#pragma once

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "comdgb.h"
#include "internal.h"

namespace cgapi {

// records the message for comdgb_last_error and returns code
int set_err(int code, const char *fmt, ...);

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return set_err(COMDGB_ERR_CUDA, "%s failed: %s (%s:%d)", #call,                   \
                     cudaGetErrorString(e_), __FILE__, __LINE__);                       \
  } while (0)

// bohr_per_atu_to_A_per_s (constants.h:61) and amu_to_m_e (constants.h:65)
constexpr double kBohrPerAtu = (double)0.529 / (double)2.418e-17;
constexpr double kAmuToMe = 1822.83;

template <class T>
T *dalloc(size_t n, int *err) {
  void *p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
    *err = 1;
    return nullptr;
  }
  return (T *)p;
}

}  // namespace cgapi

using cg::d4;

struct comdgb_sim {
  int device = 0;
  int sms = 0;  // streaming multiprocessors of the device
  comdgb_opts opts{};
  bool mixed = false;
  cudaStream_t stream = nullptr;
  cg::Geom g{};
  // replicas (a plain simulation is one): grids, first atom of each (+ total)
  int nrep = 1;
  std::vector<cg::RepGeo> reps;
  std::vector<int> atom0;
  std::vector<double> volumes;
  cg::RepGeo *rep_d = nullptr;
  double *rep_out = nullptr;                 // [2*nrep] energy, stress sums (batch)
  std::vector<double> rep_e, rep_stress;     // per replica, after a force call
  int ntot = 0, nslots = 0;
  double rmass = 1.0, cutoff = 0.0;
  double volume = 1.0;
  std::vector<void *> allocs;
  cg::Slots s{};
  cg::RebinWork w{};
  cg::Persist pl{};        // persistent lists (all null when lists are rebuilt each step)
  cg::ForceOrder fo{};     // mixed precision: persistent lists in force order
  double skin = 0.0;
  cg::EntryTab et{};
  double *dcenter = nullptr;
  int *boxc = nullptr;
  int *box_start = nullptr, *atom_slot = nullptr, *cpart = nullptr;
  int ncpart = 0;
  uint16_t *nbr = nullptr;
  int *nbr_n = nullptr;
  int cap = 0;
  // list capacities as allocated (comdgb_sim_set_list_capacity may lower the
  // capacity in use): per-step, id-keyed and force-order lists
  int cap_alloc = 0, pl_vcap_alloc = 0, fo_vcap_alloc = 0;
  double *atom_stress = nullptr;
  double *rpart = nullptr;
  long long *ripart = nullptr;
  int nrpart = 0;
  double *d_out = nullptr;     // [0] energy sum [1] stress sum [2] kinetic
  long long *d_iout = nullptr; // [0] directed pair count
  int *status = nullptr;
  double *stage3 = nullptr;    // real3 staging for host transfers
  int *bin_tmp = nullptr;
  // potentials
  cg::EamPot<double, cg::EVAL_TABLE> eam64t{};
  cg::EamPot<double, cg::EVAL_CHEBY> eam64c{};
  cg::EamPot<float, cg::EVAL_TABLE> eam32t{};
  cg::EamPot<float, cg::EVAL_CHEBY> eam32c{};
  cg::LjPot<double> lj64{};
  cg::LjPot<float> lj32{};
  double lj_eps = 0, lj_s6 = 0, lj_sigma = 0;
  // EAM Chebyshev: the installed FP64 series (0 phi, 1 rho, 2 F, 3-5 their
  // derivatives) and the FP32 pair-table lower end
  double cheb_coef[6][CG_NCHEB] = {};
  double cheb_a[6] = {}, cheb_b[6] = {};
  double pair_lo = 0.0;
  float4 *seg_buf = nullptr;
  // the FP32 pair segment table as built (seg_built) and whether the mixed
  // Chebyshev evaluator uses it (comdgb_sim_set_pair_table)
  cg::PairSeg seg_built{};
  bool pair_table_off = false;
  // adjoint scratch, allocated on first use (adjoint.cu)
  struct Adj {
    d4 *lam = nullptr;
    double *w = nullptr, *x = nullptr, *loss = nullptr, *partial = nullptr, *out = nullptr;
    double *target = nullptr, *rb = nullptr, *pb = nullptr, *u = nullptr, *hv = nullptr;
    int nblk = 0;
    std::vector<void *> snaps;  // Snapshot* (checkpoints, mid-step states, final)
  } adj;
  // virial (virial.cu): per-slot virial / per-atom stress, partial sums,
  // per-replica sums (device) and their host copy, W then K per replica
  double *vir_slot = nullptr, *vir_part = nullptr, *vir_out = nullptr;
  std::vector<double> vir_sums;
  // centrosymmetry (centro.cu): one value per slot, then the range of the
  // last replica asked for
  double *centro = nullptr;
  cg::Tune tune;  // launch shapes of the force-order kernels (comdgb_sim_set_launch)
  // graphs
  // merge_rebox (mixed precision): a sequence of steps reboxes once per step
  // -- the closing position half step of a step and the opening one of the
  // next run back to back -- instead of after each half step; part_exec
  // holds the opening, middle and closing parts of such a sequence
  bool merge_rebox = false;
  cudaGraphExec_t part_exec[3] = {nullptr, nullptr, nullptr};
  cudaGraphExec_t step_exec = nullptr;
  cudaGraphExec_t force_exec = nullptr;
  // the force call that ends a merged mixed-precision sequence: the closing
  // part has already written the FP32 copies and the force-order tracking
  cudaGraphExec_t force_exec_tracked = nullptr;
  // the same writing f, rho and F' straight into the attached host arrays
  cudaGraphExec_t force_exec_host = nullptr;
  double graph_dt = NAN;
  // n steps captured as one graph (comdgb_sim_graph_steps)
  cudaGraphExec_t loop_exec = nullptr;
  int loop_n = 0;
  double loop_dt = NAN;
  // timing graph (event record nodes between kernel groups)
  cudaGraphExec_t timed_exec = nullptr;
  cudaGraph_t timed_graph = nullptr;
  double timed_dt = NAN;
  std::vector<cudaGraphNode_t> timed_nodes;  // event record nodes, group order
  std::vector<cudaEvent_t> timed_cap_events;
  int step_kernels = 0, force_kernels = 0;  // kernel nodes per captured graph
  int part_kernels[3] = {0, 0, 0};           // opening, middle, closing parts
  // force order: the rebuild section of a step (classify, rebin, compact,
  // list build) is the body of a conditional graph node, captured on
  // cond_stream; its kernel nodes run only in steps that rebuild
  cudaStream_t cond_stream = nullptr;
  int rebuild_kernels = 0;
  int overflow_kernels = 0;  // the slot-order copy's refresh after a list overflow
  std::string trace_note;    // phases of the last drop-in call (COMDGB_TRACE_CALLS)
  // host last results
  double e = 0.0, stress = 0.0;
  simflat_t *host = nullptr;   // drop-in owner (attach)
  bool host_pinned = false;
  // the owner's registered slot arrays as the device addresses them: its
  // transfers move the occupied slots only, by kernels (zc)
  cg::HostSlots hs{};
  bool zc = false;
  void *pinned[9] = {};  // the host arrays registered at attach (natoms .. fi)
  // drop-in lazy mode: the device keeps the state between calls (dev_valid:
  // it holds the current state; host_stale: the host's arrays are older)
  bool lazy = false, dev_valid = false, host_stale = false;
  long long xfer_h2d = 0, xfer_d2h = 0;  // bytes copied by uploads / downloads
  bool lists_built = false;  // persistent lists exist (a force call completed)
  // drop-in nTimeSteps: the state download overlaps the trailing force call
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_state = nullptr;
};


namespace cgapi {

template <class T>
T *track(comdgb_sim *h, T *p) {
  h->allocs.push_back((void *)p);
  return p;
}
cg::ForceArgs force_args(comdgb_sim *h);
comdgb_sim *find_attached(const void *s);  // the handle of an attached simflat_t
int do_force(comdgb_sim *h);       // force call (graph), energy and stress to the host
int check_status(comdgb_sim *h);
double cheb_host(const double *c, double a, double b, double x);  // eamCheb on the host
void drop_graphs(comdgb_sim *h);  // after a change of potential parameters
void install_lj(comdgb_sim *h, double eps, double sigma, double cutoff);
// after a state replacement: id maps, list rebuild due, compacted atom list
int relist(comdgb_sim *h);
// a velocity-Verlet step as separate launches around the caller's force call
int step_first_half(comdgb_sim *h, double dt_atu);
int step_second_half(comdgb_sim *h, double dt_atu);
// device copy of the slot state; snapshot_copy(save) stores, (!save) restores
struct Snapshot {
  int *natoms = nullptr, *id = nullptr, *itype = nullptr;
  double *mass = nullptr;
  d4 *r = nullptr, *p = nullptr;
};
int snapshot_alloc(comdgb_sim *h, Snapshot *q);
int snapshot_copy(comdgb_sim *h, const Snapshot &q, bool save);
// series order 0 phi, 1 rho, 2 F, 3 dphi, 4 drho, 5 dF: install on the device
// (FP64 and FP32 forms, pair segment table) and drop the captured graphs
int install_cheby(comdgb_sim *h, const double coef[6][CG_NCHEB], const double a[6],
                  const double b[6]);

}  // namespace cgapi
