// force_launch.cuh -- launchers of the force kernels for one arithmetic type
// FT (included once by force_fp64.cu and once by force_mixed.cu).
#include "internal.h"

namespace cg {

static size_t nbr_build_smem() {
  return sizeof(FT) == 8 ? (size_t)NB_MAXC * (3 * sizeof(double) + sizeof(uint16_t)) : 0;
}

// called on the current device before any launch or stream capture
template <>
cudaError_t prepare_nbr_build<FT>() {
  if (sizeof(FT) == 4) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(nbr_build64_kernel<false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)nbr_build_smem());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(nbr_build64_kernel<true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nbr_build_smem());
}

template <>
void launch_nbr_build<FT>(const ForceArgs &A, FT rc2, cudaStream_t st) {
  const bool persist = A.pl.vlist != nullptr;
  if (sizeof(FT) == 4) {
    if (persist) nbr_build32_kernel<true><<<A.g.nboxes, NB_THREADS, 0, st>>>(A, (float)rc2);
    else nbr_build32_kernel<false><<<A.g.nboxes, NB_THREADS, 0, st>>>(A, (float)rc2);
  } else {
    if (persist)
      nbr_build64_kernel<true><<<A.g.nboxes, NB_THREADS, nbr_build_smem(), st>>>(A, (double)rc2);
    else
      nbr_build64_kernel<false><<<A.g.nboxes, NB_THREADS, nbr_build_smem(), st>>>(A, (double)rc2);
  }
}

template <>
void launch_eam_pass1<FT, EVAL_TABLE>(const ForceArgs &A, const EamPot<FT, EVAL_TABLE> &P,
                                      cudaStream_t st) {
  if (A.ntot > 0) eam_pass1_kernel<FT, EVAL_TABLE><<<(A.ntot + 127) / 128, 128, 0, st>>>(A, P);
}
template <>
void launch_eam_pass1<FT, EVAL_CHEBY>(const ForceArgs &A, const EamPot<FT, EVAL_CHEBY> &P,
                                      cudaStream_t st) {
  if (A.ntot > 0) eam_pass1_kernel<FT, EVAL_CHEBY><<<(A.ntot + 127) / 128, 128, 0, st>>>(A, P);
}
template <>
void launch_eam_pass2<FT, EVAL_TABLE>(const ForceArgs &A, const EamPot<FT, EVAL_TABLE> &P,
                                      cudaStream_t st) {
  if (A.ntot > 0) eam_pass2_kernel<FT, EVAL_TABLE><<<(A.ntot + 127) / 128, 128, 0, st>>>(A, P);
}
template <>
void launch_eam_pass2<FT, EVAL_CHEBY>(const ForceArgs &A, const EamPot<FT, EVAL_CHEBY> &P,
                                      cudaStream_t st) {
  if (A.ntot > 0) eam_pass2_kernel<FT, EVAL_CHEBY><<<(A.ntot + 127) / 128, 128, 0, st>>>(A, P);
}
template <>
void launch_lj<FT>(const ForceArgs &A, const LjPot<FT> &P, cudaStream_t st) {
  if (A.ntot > 0) lj_pass_kernel<FT><<<(A.ntot + 127) / 128, 128, 0, st>>>(A, P);
}

}  // namespace cg
