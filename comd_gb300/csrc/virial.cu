// virial.cu -- full virial tensor, kinetic tensor and per-atom stress of the
// current configuration.  The force passes keep the reference's scalar
// stress as it is (eam.c:649: x-x of the embedding term only; ljForce.c:175,
// 210: x-x with the kinetic term counted once per neighbour box); this is the
// physical tensor next to it, computed on request, off the timestep.
//
// For a pair within the cutoff, F_ij = g dr_ij is the force on atom i from
// atom j, dr_ij = r_i - r_j:
//   EAM  g = -(phi'(r) [r2 <= rc2] + (F'_i + F'_j) rho'(r) [r2 < rc2]) / r
//        (the reference's f is +grad U: eam.c:533-535, 644-647)
//   LJ   g = 4 eps sigma^6 r^-8 (12 sigma^6 r^-6 - 6)   (ljForce.c:205-209)
// Per atom w_i = 1/2 sum_j g dr (x) dr over its neighbour list (each pair
// split evenly between its two atoms); W = sum_i w_i is the sum over pairs of
// dr (x) F.  K = sum_i p (x) p / M with M the mass in electron masses
// (advancePositions, timestep.c:90).  The pressure tensor is (K + W) / V; the
// per-atom stress (stress x volume) is -(p (x) p / M + w_i).  Components in
// Voigt order xx yy zz yz xz xy.
//
// The pair walk is the one of the last force call, in that call's precision:
// the per-step list (FP64, or FP32 with per-step lists) or the force-order
// list (mixed precision), with F' from that call.  Per-atom sums are
// compensated in FP32 and plain in FP64; the sums over atoms are FP64 in a
// fixed order (deterministic).
#include "sim.h"

using namespace cg;
using namespace cgapi;

namespace {

constexpr int VIR_THREADS = 256;
constexpr int VIR_PARTS = 64;  // partial sums per replica

template <class T>
struct VirAcc {
  typename PrecT<T>::Acc c[6];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int q = 0; q < 6; q++) c[q].zero();
  }
  // half of g dr (x) dr
  __device__ __forceinline__ void add(T g, T dx, T dy, T dz) {
    const T hx = T(0.5) * g * dx, hy = T(0.5) * g * dy, hz = T(0.5) * g * dz;
    c[0].add(hx * dx);
    c[1].add(hy * dy);
    c[2].add(hz * dz);
    c[3].add(hy * dz);
    c[4].add(hx * dz);
    c[5].add(hx * dy);
  }
  __device__ __forceinline__ void store(double *out) const {
#pragma unroll
    for (int q = 0; q < 6; q++) out[q] = c[q].value();
  }
};

// EAM pair terms of one atom: sm holds the pair segment table (phi cubics,
// then rho cubics) when the potential uses it; pairs below the table come
// from the series in a second sweep, as in the force passes
template <class T, int EVAL, class V>
__device__ __forceinline__ void eam_virial_sum(const EamPot<T, EVAL> &P, const float4 *sm,
                                               T fii, VirAcc<T> &acc, V &&visit) {
  const T rc2 = P.rc2;
  const float4 *smr = uses_seg(P) ? sm + P.seg.n : sm;
  bool low = false;
  visit([&](T fj, T dx, T dy, T dz, T r2) {
    if (r2 > rc2) return;
    T phi, w, rho, wr = T(0);
    if (!eam_pair_w(P, sm, r2, phi, w, rho)) {
      low = true;
      return;
    }
    if (r2 < rc2) eam_embed_w(P, smr, r2, fii + fj, wr);
    acc.add(-(w + wr), dx, dy, dz);
  });
  if (low)
    visit([&](T fj, T dx, T dy, T dz, T r2) {
      if (r2 > rc2 || !below_seg(P, r2)) return;
      T phi, w, rho;
      pair_w_series(P, r2, phi, w, rho);
      const T wr = r2 < rc2 ? embed_w_series(P, r2, fii + fj) : T(0);
      acc.add(-(w + wr), dx, dy, dz);
    });
}

// out: 6 doubles per slot.  FO: force-order list (mixed precision).
template <class T, int EVAL, bool FO>
__global__ void __launch_bounds__(VIR_THREADS)
    eam_virial_kernel(ForceArgs A, const __grid_constant__ EamPot<T, EVAL> P, double *out) {
  extern __shared__ float4 seg_sm[];
  if (uses_seg(P)) stage_seg(seg_sm, P.seg.p1, 2 * P.seg.n);
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    VirAcc<T> acc;
    acc.zero();
    int slot;
    if constexpr (FO) {
      slot = A.fo.slot[a];
      const float4 pi = A.fo.pf[a];
      eam_virial_sum(P, seg_sm, pi.w, acc,
                     [&](auto &&fn) { fo_for_each<true, true>(A, a, slot, pi, P.rc2, fn); });
    } else {
      slot = A.atom_slot[a];
      const int b = slot >> 6, i = slot & 63;
      T xi, yi, zi;
      PrecT<T>::pos(A.s, slot, xi, yi, zi);
      eam_virial_sum(P, seg_sm, PrecT<T>::fi(A.s, slot), acc, [&](auto &&fn) {
        for_each_neighbor<T, true>(A, a, b, i, xi, yi, zi, P.rc2,
                                   [&](int js, T dx, T dy, T dz, T r2) {
                                     fn(PrecT<T>::fi(A.s, js), dx, dy, dz, r2);
                                   });
      });
    }
    acc.store(out + 6 * (size_t)slot);
  }
}

template <class T, bool FO>
__global__ void __launch_bounds__(VIR_THREADS) lj_virial_kernel(ForceArgs A, LjPot<T> P,
                                                                double *out) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    VirAcc<T> acc;
    acc.zero();
    const T s12 = P.s6x12, c4 = P.eps4s6, rc2 = P.rc2;
    auto fn = [&](T, T dx, T dy, T dz, T r2) {
      if (r2 > rc2) return;
      const T ir2 = T(1.0) / r2;
      const T r6 = ir2 * ir2 * ir2;
      acc.add(c4 * r6 * ir2 * (s12 * r6 - T(6.0)), dx, dy, dz);
    };
    int slot;
    if constexpr (FO) {
      slot = A.fo.slot[a];
      fo_for_each<false, true>(A, a, slot, A.fo.pos[a], (float)rc2, fn);
    } else {
      slot = A.atom_slot[a];
      const int b = slot >> 6, i = slot & 63;
      T xi, yi, zi;
      PrecT<T>::pos(A.s, slot, xi, yi, zi);
      for_each_neighbor<T, false>(A, a, b, i, xi, yi, zi, rc2,
                                  [&](int, T dx, T dy, T dz, T r2) { fn(T(0), dx, dy, dz, r2); });
    }
    acc.store(out + 6 * (size_t)slot);
  }
}

// Per replica r (blockIdx.y), part x (blockIdx.x) of its compact atoms:
// adds the kinetic tensor, turns the per-slot virial into the per-atom
// stress -(K_i + w_i) in place, and writes the part's 12 sums (W, K) to
// part[(r * gridDim.x + x) * 12 + c] (fixed order within the CTA).
__global__ void __launch_bounds__(VIR_THREADS)
    virial_reduce_kernel(Geom g, Slots s, const int *atom_slot, double rmass, double *w,
                         double *part) {
  __shared__ double red[VIR_THREADS];
  const RepGeo &R = g.rep[blockIdx.y];
  double acc[12];
#pragma unroll
  for (int c = 0; c < 12; c++) acc[c] = 0.0;
  for (int a = R.a0 + blockIdx.x * blockDim.x + threadIdx.x; a < R.a0 + R.na;
       a += gridDim.x * blockDim.x) {
    const int slot = atom_slot[a];
    const d4 p = s.p[slot];
    const double k[6] = {p.x * p.x / rmass, p.y * p.y / rmass, p.z * p.z / rmass,
                         p.y * p.z / rmass, p.x * p.z / rmass, p.x * p.y / rmass};
    double *ws = w + 6 * (size_t)slot;
#pragma unroll
    for (int c = 0; c < 6; c++) {
      const double v = ws[c];
      acc[c] += v;
      acc[6 + c] += k[c];
      ws[c] = -(v + k[c]);
    }
  }
  for (int c = 0; c < 12; c++) {
    red[threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = VIR_THREADS / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 12 + c] = red[0];
    __syncthreads();
  }
}

// out[12 r + c] = sum over the parts of replica r, in part order
__global__ void virial_final_kernel(const double *part, int nparts, double *out) {
  const int r = blockIdx.x, c = threadIdx.x;
  if (c >= 12) return;
  double v = 0.0;
  for (int x = 0; x < nparts; x++) v += part[((size_t)r * nparts + x) * 12 + c];
  out[12 * r + c] = v;
}

size_t eam_virial_smem(const comdgb_sim *h) {
  return (h->mixed && h->opts.potential == COMDGB_POT_EAM_CHEBY && h->eam32c.seg.n > 0)
             ? sizeof(float4) * 2 * (size_t)h->eam32c.seg.n
             : 0;
}

template <class K>
int allow_smem(K kernel, size_t smem) {
  if (smem) CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  return 0;
}

// the per-slot virial of the state the last force call saw
int launch_virial(comdgb_sim *h, double *out) {
  const ForceArgs A = force_args(h);
  cudaStream_t st = h->stream;
  const int pot = h->opts.potential;
  int dev_sms = 1;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, h->device));
  long need = ((long)h->ntot + VIR_THREADS - 1) / VIR_THREADS;
  const int grid = (int)(need < 4L * dev_sms ? (need > 0 ? need : 1) : 4L * dev_sms);
  const size_t smem = eam_virial_smem(h);
  const bool fo = h->fo.list != nullptr;
  if (pot == COMDGB_POT_LJ) {
    if (fo) lj_virial_kernel<float, true><<<grid, VIR_THREADS, 0, st>>>(A, h->lj32, out);
    else if (h->mixed) lj_virial_kernel<float, false><<<grid, VIR_THREADS, 0, st>>>(A, h->lj32, out);
    else lj_virial_kernel<double, false><<<grid, VIR_THREADS, 0, st>>>(A, h->lj64, out);
  } else if (pot == COMDGB_POT_EAM_TABLE) {
    if (fo)
      eam_virial_kernel<float, EVAL_TABLE, true><<<grid, VIR_THREADS, 0, st>>>(A, h->eam32t, out);
    else if (h->mixed)
      eam_virial_kernel<float, EVAL_TABLE, false><<<grid, VIR_THREADS, 0, st>>>(A, h->eam32t, out);
    else
      eam_virial_kernel<double, EVAL_TABLE, false><<<grid, VIR_THREADS, 0, st>>>(A, h->eam64t, out);
  } else {
    int rc;
    if (fo) {
      if ((rc = allow_smem(eam_virial_kernel<float, EVAL_CHEBY, true>, smem))) return rc;
      eam_virial_kernel<float, EVAL_CHEBY, true><<<grid, VIR_THREADS, smem, st>>>(A, h->eam32c,
                                                                                  out);
    } else if (h->mixed) {
      if ((rc = allow_smem(eam_virial_kernel<float, EVAL_CHEBY, false>, smem))) return rc;
      eam_virial_kernel<float, EVAL_CHEBY, false><<<grid, VIR_THREADS, smem, st>>>(A, h->eam32c,
                                                                                   out);
    } else {
      eam_virial_kernel<double, EVAL_CHEBY, false><<<grid, VIR_THREADS, 0, st>>>(A, h->eam64c,
                                                                                 out);
    }
  }
  CK(cudaGetLastError());
  return 0;
}

int check_handle(comdgb_sim *h) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (h->opts.potential < 0) return set_err(COMDGB_ERR_ARG, "simulation has no potential");
  CK(cudaSetDevice(h->device));
  return 0;
}

}  // namespace

namespace cgapi {

// force call, per-slot virial, kinetic tensor and per-replica sums:
// h->vir_sums[12 r + c] (W then K) on the host
int compute_virial(comdgb_sim *h) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = do_force(h))) return rc;
  int err = 0;
  if (!h->vir_slot) {
    h->vir_slot = track(h, dalloc<double>(6 * (size_t)h->nslots, &err));
    h->vir_part = track(h, dalloc<double>((size_t)h->nrep * VIR_PARTS * 12, &err));
    h->vir_out = track(h, dalloc<double>((size_t)h->nrep * 12, &err));
    if (err) return set_err(COMDGB_ERR_NOMEM, "virial scratch allocation failed");
  }
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(h->vir_slot, 0, sizeof(double) * 6 * (size_t)h->nslots, st));
  if ((rc = launch_virial(h, h->vir_slot))) return rc;
  virial_reduce_kernel<<<dim3(VIR_PARTS, h->nrep), VIR_THREADS, 0, st>>>(
      h->g, h->s, h->atom_slot, h->rmass, h->vir_slot, h->vir_part);
  virial_final_kernel<<<h->nrep, 32, 0, st>>>(h->vir_part, VIR_PARTS, h->vir_out);
  CK(cudaGetLastError());
  h->vir_sums.resize(12 * (size_t)h->nrep);
  CK(cudaMemcpyAsync(h->vir_sums.data(), h->vir_out, sizeof(double) * h->vir_sums.size(),
                     cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return check_status(h);
}

}  // namespace cgapi

extern "C" {

int comdgb_sim_virial(comdgb_sim *h, double *w, double *k, double *volume) {
  return comdgb_batch_virial(h, -1, w, k, volume);
}

int comdgb_batch_virial(comdgb_sim *h, int r, double *w, double *k, double *volume) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (r >= h->nrep) return set_err(COMDGB_ERR_ARG, "replica %d of %d", r, h->nrep);
  if (r < 0) {  // compute, then report replica 0
    if ((rc = compute_virial(h))) return rc;
    r = 0;
  } else if (h->vir_sums.size() != 12 * (size_t)h->nrep) {
    return set_err(COMDGB_ERR_ARG, "no virial computed yet (comdgb_sim_virial)");
  }
  const double *v = h->vir_sums.data() + 12 * (size_t)r;
  for (int c = 0; c < 6; c++) {
    if (w) w[c] = v[c];
    if (k) k[c] = v[6 + c];
  }
  if (volume) *volume = r < (int)h->volumes.size() ? h->volumes[r] : h->volume;
  return 0;
}

int comdgb_sim_atom_stress(comdgb_sim *h, int r, double *out) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!out) return set_err(COMDGB_ERR_ARG, "null argument");
  if (r < 0 || r >= h->nrep) return set_err(COMDGB_ERR_ARG, "replica %d of %d", r, h->nrep);
  if (!h->vir_slot || h->vir_sums.empty())
    return set_err(COMDGB_ERR_ARG, "no virial computed yet (comdgb_sim_virial)");
  const RepGeo &R = h->reps[r];
  CK(cudaMemcpyAsync(out, h->vir_slot + 6 * (size_t)R.box0 * CG_MAXATOMS,
                     sizeof(double) * 6 * (size_t)R.nb * CG_MAXATOMS, cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

}  // extern "C"
