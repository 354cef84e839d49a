// force_launch.cuh -- launchers of the force kernels for one arithmetic type
// FT (included once by force_fp64.cu and once by force_mixed.cu).
#include "internal.h"

namespace cg {

static size_t nbr_build_smem() {
  return (size_t)CG_NNBR * CG_MAXATOMS * (3 * sizeof(FT) + sizeof(uint16_t));
}

// called on the current device before any launch or stream capture
template <>
cudaError_t prepare_nbr_build<FT>() {
  return cudaFuncSetAttribute(nbr_build_kernel<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)nbr_build_smem());
}

template <>
void launch_nbr_build<FT>(const ForceArgs &A, FT rc2, cudaStream_t st) {
  nbr_build_kernel<FT><<<A.g.nboxes, 128, nbr_build_smem(), st>>>(A, rc2);
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
