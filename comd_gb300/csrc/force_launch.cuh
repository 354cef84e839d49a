// force_launch.cuh -- launchers of the force kernels for one arithmetic type
// FT (included once by force_fp64.cu and once by force_mixed.cu).
#include "internal.h"

namespace cg {

static size_t nbr_build_smem() {
  return sizeof(FT) == 8 ? (size_t)NB_MAXC * (3 * sizeof(double) + sizeof(uint16_t)) : 0;
}

// resident CTAs per SM of the EAM pass kernels ([pass][eval]) and the SM
// count, found before any launch or stream capture
static int g_pass_per_sm[2][2];
// force order: [without, with energies][pass 1, pass 2, LJ][eval]
static int g_fo_per_sm[2][3][2];
static int g_num_sms = 1;
// resident CTAs per SM of the FP32 list builds: force order [64, 128, 256
// threads][2, 4, 8 atoms per load], per-step and id-keyed lists
static int g_build_per_sm[3][3], g_build_step_per_sm = 1, g_build_id_per_sm = 1;

template <class K>
static cudaError_t pass_occupancy(K kernel, size_t smem, int *out, int threads = PASS_THREADS) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kernel, threads, smem);
  if (*out < 1) *out = 1;
  return e;
}

static size_t pass_smem(int pass, int eval) {
  if (sizeof(FT) != 4 || eval != EVAL_CHEBY) return 0;
  return sizeof(float4) * (pass == 0 ? 2 : 1) * SEG_N;
}

// force order: the density pass stages its rho table (SEG1_N cubics, in
// RHO_COPIES copies), the force pass its derivative cubics (2 SEG2_N, in
// FORCE_COPIES copies) and, summing energies (obs), the phi cubics (SEG_N)
static size_t fo_pass_smem(int pass, int eval, bool obs = true) {
  if (sizeof(FT) != 4 || eval != EVAL_CHEBY) return 0;
  if (pass == 0) return sizeof(float4) * SEG1_N * RHO_COPIES;
  return sizeof(float4) * (2 * SEG2_N * FORCE_COPIES + (obs ? SEG_N : 0));
}

#if COMDGB_FT_FLOAT
// resident CTAs per SM of the force-order builds with NT threads, for 2, 4
// and 8 atoms per load
template <int NT>
static cudaError_t build_occupancy_nt(int *out) {
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &out[0], nbr_build32_kernel<LIST_FO, NT, 2>, NT, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&out[1], nbr_build32_kernel<LIST_FO, NT, 4>,
                                                      NT, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&out[2], nbr_build32_kernel<LIST_FO, NT, 8>,
                                                      NT, 0);
  for (int i = 0; i < 3; i++) out[i] = out[i] < 1 ? 1 : out[i];
  return e;
}
#endif

#if COMDGB_FT_FLOAT
// resident CTAs per SM of the force-order passes with or without energies
// (g_fo_per_sm[OBS]); every variant's shared-memory limit set
template <bool OBS>
static cudaError_t fo_occupancy() {
  int dummy = 0;
  int(&o)[3][2] = g_fo_per_sm[OBS];
  const size_t s0 = fo_pass_smem(0, EVAL_CHEBY), s1 = fo_pass_smem(1, EVAL_CHEBY, OBS);
  cudaError_t e = pass_occupancy(fo_eam_pass1_kernel<EVAL_TABLE, false, OBS>, 0,
                                 &o[0][EVAL_TABLE], FO1_THREADS);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass1_kernel<EVAL_CHEBY, false, OBS>, s0, &o[0][EVAL_CHEBY],
                       FO1_THREADS);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass2_kernel<EVAL_TABLE, false, OBS>, 0, &o[1][EVAL_TABLE],
                       FO2_MAX_THREADS);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass2_kernel<EVAL_CHEBY, false, OBS>, s1, &o[1][EVAL_CHEBY],
                       FO2_MAX_THREADS);
  if (e == cudaSuccess) e = pass_occupancy(fo_lj_kernel<false, OBS>, 0, &o[2][0]);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass1_kernel<EVAL_TABLE, true, OBS>, 0, &dummy, FO1_THREADS);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass1_kernel<EVAL_CHEBY, true, OBS>, s0, &dummy, FO1_THREADS);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass2_kernel<EVAL_TABLE, true, OBS>, 0, &dummy, FO2_MAX_THREADS);
  if (e == cudaSuccess)
    e = pass_occupancy(fo_eam_pass2_kernel<EVAL_CHEBY, true, OBS>, s1, &dummy, FO2_MAX_THREADS);
  if (e == cudaSuccess) e = pass_occupancy(fo_lj_kernel<true, OBS>, 0, &dummy);
  return e;
}
#endif

// grid of a list build: one CTA per box, capped at the resident CTAs
static int build_grid(int nboxes, int per_sm) {
  const long cap = (long)g_num_sms * per_sm;
  return nboxes < cap ? nboxes : (int)cap;
}

// called on the current device before any launch or stream capture
template <>
cudaError_t prepare_force_kernels<FT>() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = pass_occupancy(eam_pass1_kernel<FT, EVAL_TABLE>, pass_smem(0, EVAL_TABLE),
                       &g_pass_per_sm[0][EVAL_TABLE]);
  if (e == cudaSuccess)
    e = pass_occupancy(eam_pass1_kernel<FT, EVAL_CHEBY>, pass_smem(0, EVAL_CHEBY),
                       &g_pass_per_sm[0][EVAL_CHEBY]);
  if (e == cudaSuccess)
    e = pass_occupancy(eam_pass2_kernel<FT, EVAL_TABLE>, pass_smem(1, EVAL_TABLE),
                       &g_pass_per_sm[1][EVAL_TABLE]);
  if (e == cudaSuccess)
    e = pass_occupancy(eam_pass2_kernel<FT, EVAL_CHEBY>, pass_smem(1, EVAL_CHEBY),
                       &g_pass_per_sm[1][EVAL_CHEBY]);
  if (e != cudaSuccess) return e;
#if COMDGB_FT_FLOAT
  {
    // resident CTAs of the single-replica variants (the batch variants take
    // the same grids; they are grid-stride loops)
    e = fo_occupancy<false>();
    if (e == cudaSuccess) e = fo_occupancy<true>();
    if (e == cudaSuccess) e = build_occupancy_nt<64>(g_build_per_sm[0]);
    if (e == cudaSuccess) e = build_occupancy_nt<128>(g_build_per_sm[1]);
    if (e == cudaSuccess) e = build_occupancy_nt<256>(g_build_per_sm[2]);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &g_build_step_per_sm, nbr_build32_kernel<LIST_STEP>, NB_THREADS, 0);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &g_build_id_per_sm, nbr_build32_kernel<LIST_ID>, NB_THREADS, 0);
    g_build_step_per_sm = g_build_step_per_sm < 1 ? 1 : g_build_step_per_sm;
    g_build_id_per_sm = g_build_id_per_sm < 1 ? 1 : g_build_id_per_sm;
    return e;
  }
#endif
  e = cudaFuncSetAttribute(nbr_build64_kernel<LIST_STEP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)nbr_build_smem());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(nbr_build64_kernel<LIST_ID>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nbr_build_smem());
}

// grid of a pass: every atom one thread, capped at the resident CTAs
static int pass_grid(int pass, int eval, int ntot, bool fo = false,
                     int threads = PASS_THREADS, bool obs = true) {
  long need = (ntot + threads - 1) / threads;
  long cap = (long)g_num_sms * (fo ? g_fo_per_sm[obs][pass][eval] : g_pass_per_sm[pass][eval]);
  return (int)(need < cap ? need : cap);
}

#if COMDGB_FT_FLOAT
// the force-order build at the tuned shape (threads per box x atoms per load)
template <int NT>
static void launch_fo_build_nt(const ForceArgs &A, float rc2, int na, cudaStream_t st) {
  const int *per_sm = g_build_per_sm[NT == 64 ? 0 : NT == 128 ? 1 : 2];
  if (na == 2)
    nbr_build32_kernel<LIST_FO, NT, 2><<<build_grid(A.g.nboxes, per_sm[0]), NT, 0, st>>>(A, rc2);
  else if (na == 8)
    nbr_build32_kernel<LIST_FO, NT, 8><<<build_grid(A.g.nboxes, per_sm[2]), NT, 0, st>>>(A, rc2);
  else
    nbr_build32_kernel<LIST_FO, NT, 4><<<build_grid(A.g.nboxes, per_sm[1]), NT, 0, st>>>(A, rc2);
}
static void launch_fo_build(const ForceArgs &A, float rc2, cudaStream_t st, const Tune *t) {
  const int nt = t ? t->build_threads : NB_THREADS, na = t ? t->build_atoms : NB_ATOMS;
  if (nt == 64) launch_fo_build_nt<64>(A, rc2, na, st);
  else if (nt == 256) launch_fo_build_nt<256>(A, rc2, na, st);
  else launch_fo_build_nt<128>(A, rc2, na, st);
}
#endif

template <>
void launch_nbr_build<FT>(const ForceArgs &A, FT rc2, cudaStream_t st, const Tune *tune) {
  (void)tune;
  if (sizeof(FT) == 4) {
#if COMDGB_FT_FLOAT
    if (A.fo.list) {
      launch_fo_build(A, (float)rc2, st, tune);
      return;
    }
#endif
    if (A.pl.vlist)
      nbr_build32_kernel<LIST_ID><<<build_grid(A.g.nboxes, g_build_id_per_sm), NB_THREADS, 0,
                                    st>>>(A, (float)rc2);
    else
      nbr_build32_kernel<LIST_STEP><<<build_grid(A.g.nboxes, g_build_step_per_sm), NB_THREADS,
                                      0, st>>>(A, (float)rc2);
  } else {
    if (A.pl.vlist)
      nbr_build64_kernel<LIST_ID><<<A.g.nboxes, NB_THREADS, nbr_build_smem(), st>>>(A, (double)rc2);
    else
      nbr_build64_kernel<LIST_STEP><<<A.g.nboxes, NB_THREADS, nbr_build_smem(), st>>>(A,
                                                                                  (double)rc2);
  }
}

#if COMDGB_FT_FLOAT
template <int EVAL, bool OBS>
static void launch_fo_eam_obs(const ForceArgs &A, const EamPot<float, EVAL> &P, int pass,
                              cudaStream_t st, const Tune *tune) {
  const size_t smem = P.seg.n > 0 ? fo_pass_smem(pass, EVAL, OBS) : 0;
  const bool multi = A.g.nrep > 1;
  if (pass == 0) {
    const int g0 = pass_grid(0, EVAL, A.ntot, true, FO1_THREADS, OBS);
    if (multi) fo_eam_pass1_kernel<EVAL, true, OBS><<<g0, FO1_THREADS, smem, st>>>(A, P);
    else fo_eam_pass1_kernel<EVAL, false, OBS><<<g0, FO1_THREADS, smem, st>>>(A, P);
  } else {
    const int threads = tune ? tune->pass2_threads : FO2_MAX_THREADS;
    const int tuned = tune ? (OBS ? tune->pass2_blocks : tune->pass2_blocks_fast) : 0;
    int g1;
    if (tuned > 0) {
      const long need = ((long)A.ntot + threads - 1) / threads;
      g1 = (int)(need < tuned ? need : tuned);
    } else {
      g1 = pass_grid(1, EVAL, A.ntot, true, threads, OBS);
    }
    if (multi) fo_eam_pass2_kernel<EVAL, true, OBS><<<g1, threads, smem, st>>>(A, P);
    else fo_eam_pass2_kernel<EVAL, false, OBS><<<g1, threads, smem, st>>>(A, P);
  }
}

template <int EVAL>
void launch_fo_eam(const ForceArgs &A, const EamPot<float, EVAL> &P, int pass, cudaStream_t st,
                   const Tune *tune, bool obs) {
  if (A.ntot <= 0) return;
  if (obs) launch_fo_eam_obs<EVAL, true>(A, P, pass, st, tune);
  else launch_fo_eam_obs<EVAL, false>(A, P, pass, st, tune);
}
template void launch_fo_eam<EVAL_TABLE>(const ForceArgs &, const EamPot<float, EVAL_TABLE> &,
                                        int, cudaStream_t, const Tune *, bool);
template void launch_fo_eam<EVAL_CHEBY>(const ForceArgs &, const EamPot<float, EVAL_CHEBY> &,
                                        int, cudaStream_t, const Tune *, bool);

template <int EVAL, bool OBS>
static int fo_pass2_per_sm(bool multi, int threads) {
  int per_sm = 0;
  const size_t smem = fo_pass_smem(1, EVAL, OBS);
  const cudaError_t e =
      multi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                  &per_sm, fo_eam_pass2_kernel<EVAL, true, OBS>, threads, smem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                  &per_sm, fo_eam_pass2_kernel<EVAL, false, OBS>, threads, smem);
  return e != cudaSuccess || per_sm < 1 ? 1 : per_sm;
}

int fo_pass2_blocks(int eval, bool multi, int threads, bool obs) {
  int per_sm;
  if (eval == EVAL_CHEBY)
    per_sm = obs ? fo_pass2_per_sm<EVAL_CHEBY, true>(multi, threads)
                 : fo_pass2_per_sm<EVAL_CHEBY, false>(multi, threads);
  else
    per_sm = obs ? fo_pass2_per_sm<EVAL_TABLE, true>(multi, threads)
                 : fo_pass2_per_sm<EVAL_TABLE, false>(multi, threads);
  return per_sm * g_num_sms;
}

void launch_fo_lj(const ForceArgs &A, const LjPot<float> &P, cudaStream_t st, bool obs) {
  if (A.ntot <= 0) return;
  const int grid = pass_grid(2, 0, A.ntot, true, PASS_THREADS, obs);
  const bool multi = A.g.nrep > 1;
  if (obs) {
    if (multi) fo_lj_kernel<true, true><<<grid, PASS_THREADS, 0, st>>>(A, P);
    else fo_lj_kernel<false, true><<<grid, PASS_THREADS, 0, st>>>(A, P);
  } else {
    if (multi) fo_lj_kernel<true, false><<<grid, PASS_THREADS, 0, st>>>(A, P);
    else fo_lj_kernel<false, false><<<grid, PASS_THREADS, 0, st>>>(A, P);
  }
}
#endif

template <>
void launch_eam_pass1<FT, EVAL_TABLE>(const ForceArgs &A, const EamPot<FT, EVAL_TABLE> &P,
                                      cudaStream_t st) {
  if (A.ntot <= 0) return;
  const size_t smem = P.seg.n > 0 ? pass_smem(0, EVAL_TABLE) : 0;
  eam_pass1_kernel<FT, EVAL_TABLE><<<pass_grid(0, EVAL_TABLE, A.ntot), PASS_THREADS, smem, st>>>(A, P);
}
template <>
void launch_eam_pass1<FT, EVAL_CHEBY>(const ForceArgs &A, const EamPot<FT, EVAL_CHEBY> &P,
                                      cudaStream_t st) {
  if (A.ntot <= 0) return;
  const size_t smem = P.seg.n > 0 ? pass_smem(0, EVAL_CHEBY) : 0;
  eam_pass1_kernel<FT, EVAL_CHEBY><<<pass_grid(0, EVAL_CHEBY, A.ntot), PASS_THREADS, smem, st>>>(A, P);
}
template <>
void launch_eam_pass2<FT, EVAL_TABLE>(const ForceArgs &A, const EamPot<FT, EVAL_TABLE> &P,
                                      cudaStream_t st) {
  if (A.ntot <= 0) return;
  const size_t smem = P.seg.n > 0 ? pass_smem(1, EVAL_TABLE) : 0;
  eam_pass2_kernel<FT, EVAL_TABLE><<<pass_grid(1, EVAL_TABLE, A.ntot), PASS_THREADS, smem, st>>>(A, P);
}
template <>
void launch_eam_pass2<FT, EVAL_CHEBY>(const ForceArgs &A, const EamPot<FT, EVAL_CHEBY> &P,
                                      cudaStream_t st) {
  if (A.ntot <= 0) return;
  const size_t smem = P.seg.n > 0 ? pass_smem(1, EVAL_CHEBY) : 0;
  eam_pass2_kernel<FT, EVAL_CHEBY><<<pass_grid(1, EVAL_CHEBY, A.ntot), PASS_THREADS, smem, st>>>(A, P);
}
template <>
void launch_lj<FT>(const ForceArgs &A, const LjPot<FT> &P, cudaStream_t st) {
  if (A.ntot > 0) lj_pass_kernel<FT><<<(A.ntot + 127) / 128, 128, 0, st>>>(A, P);
}

}  // namespace cg
