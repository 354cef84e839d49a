// md_kernels.cu -- integration, link-cell rebinning, initial binning, stencil
// table, atom compaction, reductions and the Chebyshev fit.
//
// Built with -fmad=false: the FP64 integrator must reproduce the
// reference's separately rounded multiply and add (timestep.c:71,104) so
// that, given the same forces, positions and momenta are bit-identical and
// the rebinning decisions agree with reBoxAll.
#include <cstdio>
#include <cstring>

#include <algorithm>

#include "binning.cuh"
#include "internal.h"

namespace cg {

// ---------------------------------------------------------------------------
// stencil table: getNeighborBoxes (domains.c:391-430) + min-image drbox
// (eam.c:494-502), one thread per box
// ---------------------------------------------------------------------------
__global__ void entry_table_kernel(Geom g, const double *dcenter, EntryTab et) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nboxes) return;
  int base = b * CG_NNBR;
  int cnt = 0;
  const RepGeo &R = rep_of(g, b);
  if (R.nb == 1) {
    et.box[base] = b;
    et.dr64[base] = d4{0.0, 0.0, 0.0, 0.0};
    et.dr32[2 * base] = make_float4(0.f, 0.f, 0.f, 0.f);
    et.dr32[2 * base + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    et.n[b] = 1;
    return;
  }
  int ix[3];
  box_ixyz(R, b, ix);
  for (int i = ix[0] - 1; i <= ix[0] + 1; i++)
    for (int j = ix[1] - 1; j <= ix[1] + 1; j++)
      for (int k = ix[2] - 1; k <= ix[2] + 1; k++) {
        int t[3] = {i, j, k};
        int nb = box_from_ixyz(R, g.periodic, t);
        if (nb < 0) continue;
        double dr[3];
        for (int d = 0; d < 3; d++) {
          dr[d] = dcenter[3 * b + d] - dcenter[3 * nb + d];
          if (g.periodic) {
            if (dr[d] < -0.5 * R.bounds[d]) dr[d] += R.bounds[d];
            else if (dr[d] > 0.5 * R.bounds[d]) dr[d] -= R.bounds[d];
          }
        }
        et.box[base + cnt] = nb;
        et.dr64[base + cnt] = d4{dr[0], dr[1], dr[2], 0.0};
        float hi[3];
        for (int d = 0; d < 3; d++) hi[d] = (float)dr[d];
        et.dr32[2 * (base + cnt)] = make_float4(hi[0], hi[1], hi[2], 0.f);
        et.dr32[2 * (base + cnt) + 1] =
            make_float4((float)(dr[0] - (double)hi[0]), (float)(dr[1] - (double)hi[1]),
                        (float)(dr[2] - (double)hi[2]), 0.f);
        cnt++;
      }
  for (int e = cnt; e < CG_NNBR; e++) et.box[base + e] = -1;
  et.n[b] = cnt;
}

__global__ void box_coord_kernel(Geom g, int *boxc) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nboxes) return;
  int ix[3];
  box_ixyz(rep_of(g, b), b, ix);
  boxc[b] = ix[0] | (ix[1] << 10) | (ix[2] << 20);
}

void launch_entry_table(const Geom &g, const double *dcenter, EntryTab et, int *boxc,
                        cudaStream_t st) {
  box_coord_kernel<<<(g.nboxes + 127) / 128, 128, 0, st>>>(g, boxc);
  entry_table_kernel<<<(g.nboxes + 127) / 128, 128, 0, st>>>(g, dcenter, et);
}

// ---------------------------------------------------------------------------
// reBoxAll, parallel form (domains.c:347-389).
//
// The reference scans boxes in ascending order with swap-remove.  Box j's
// scan list is its own atoms followed by the arrivals from lower-index boxes
// (in source order, then in each source's departure order); arrivals from
// higher-index boxes are appended after the scan.  Which atoms leave a box,
// and for where, depends only on each atom's own position, so:
//   classify  per slot: destination (+-1 box per axis, periodic wrap) and
//             the moved position; departing records copied to a stage, their
//             old slots listed at the destination (lower / higher sources).
//   plan      per box: replay the swap-remove scan with placeholders for
//             the lower arrivals -> each departure's rank and the box's
//             arrangement after its scan.
//   apply     per box: move stayers, sort the box's arrival lists by
//             (source box, departure rank), place the lower arrivals into
//             their placeholders and append the higher ones.
// If an arrival from a lower box would itself leave again when rescanned
// (a move of more than one box per axis, or r+boxsize rounding to boxsize),
// the plan is invalid and a serial replay of reBoxAll runs instead.
// ---------------------------------------------------------------------------

// move one atom's record; with persistent lists also re-point its id
__device__ __forceinline__ void copy_record(const Slots &dst, int ds, const Slots &src, int ss,
                                            bool mixed, const SlotMap &map) {
  map.moved(src.id[ss], ds);
  dst.id[ds] = src.id[ss];
  dst.itype[ds] = src.itype[ss];
  dst.mass[ds] = src.mass[ss];
  dst.r[ds] = src.r[ss];
  dst.p[ds] = src.p[ss];
  dst.f[ds] = src.f[ss];
  dst.rho[ds] = src.rho[ss];
  dst.fi[ds] = src.fi[ss];
  if (mixed) dst.pos32[ds] = src.pos32[ss];
}

// classify one atom; r is its (possibly just advanced) position.  A
// departing atom sets its bit in depmask (cleared before the launch), records
// its destination and copies its record, with the moved position, to the stage.
__device__ __forceinline__ void classify_atom(const Geom &g, const Slots &s, int slot, d4 r,
                                              bool mixed, const RebinWork &w, int *status) {
  const int b = slot >> 6;
  const RepGeo &R = rep_of(g, b);
  int ixo[3], ixn[3];
  const int sd[3] = {side_of(r.x, R.boxsize[0]), side_of(r.y, R.boxsize[1]),
                      side_of(r.z, R.boxsize[2])};
  if ((sd[0] | sd[1] | sd[2]) == 0) return;  // stays (the common case: no FP64 work)
  box_ixyz_tab(g, b, ixo);
  double rn[3] = {r.x, r.y, r.z};
  for (int k = 0; k < 3; k++) {
    ixn[k] = ixo[k] + sd[k];
    if (sd[k] < 0) rn[k] += R.boxsize[k];
    else if (sd[k] > 0) rn[k] -= R.boxsize[k];
  }
  const int jb = box_from_ixyz(R, g.periodic, ixn);
  if (jb < 0 || jb == b) return;
  atomicOr(w.depmask + (slot >> 5), 1u << (slot & 31));
  // the destination's arrival lists (lower / higher source box), in claim
  // order; 64 or more arrivals overflow the box, which the plan reports
  const bool from_lo = b < jb;
  const int k = atomicAdd(from_lo ? w.arr_lo + jb : w.arr_hi + jb, 1);
  if (k < CG_MAXATOMS)
    w.arr_list[(from_lo ? 0 : (size_t)g.nboxes * CG_MAXATOMS) + (size_t)jb * CG_MAXATOMS + k] =
        slot;
  Slots st = w.stage;
  st.id[slot] = s.id[slot];
  st.itype[slot] = s.itype[slot];
  st.mass[slot] = s.mass[slot];
  st.r[slot] = d4{rn[0], rn[1], rn[2], 0.0};
  st.p[slot] = s.p[slot];
  st.f[slot] = s.f[slot];
  st.rho[slot] = s.rho[slot];
  st.fi[slot] = s.fi[slot];
  if (mixed) st.pos32[slot] = centred32(R, rn[0], rn[1], rn[2]);
  if (jb > b) {
    // re-examined in jb's scan: must stay there
    int ix2[3], ix3[3];
    box_ixyz_tab(g, jb, ix2);
    for (int k = 0; k < 3; k++) {
      if (rn[k] < 0.0) ix3[k] = ix2[k] - 1;
      else if (rn[k] >= R.boxsize[k]) ix3[k] = ix2[k] + 1;
      else ix3[k] = ix2[k];
    }
    const int jb2 = box_from_ixyz(R, g.periodic, ix3);
    if (jb2 >= 0 && jb2 != jb) atomicExch(status + ST_REBIN_SERIAL, 1);
  }
}

// how a half step divides by the (constant) mass.  FP64 follows the
// reference's roundings: (dt*p)/rmass by Markstein's correctly rounded
// division (INT_MARK, rinv = RN(1/rmass)) or by IEEE division (INT_IEEE).
// Mixed precision, whose forces are FP32 anyway, spends the scarce FP64
// issue slots once per component (INT_FMA): p - dt*f and r + p*(dt/rmass)
// as one fused multiply-add each, with dt/rmass rounded once on the host.
enum { INT_IEEE = 0, INT_MARK = 1, INT_FMA = 2 };
template <int MODE>
__device__ __forceinline__ double div_mass(double a, double rmass, double rinv) {
  return MODE == INT_MARK ? div_markstein(a, rmass, rinv) : a / rmass;
}

// fo_track_at for atom id (before the first build, no force-order number:
// a rebuild is due anyway)
__device__ __forceinline__ void fo_track(const Geom &g, const ForceOrder &fo, int b, int id,
                                         const d4 &r, float4 p32, int *status) {
  const int af = fo.of_id[id];
  if (af >= 0) fo_track_at(g, fo, b, af, r, p32, status);
}

// delta: the two position half steps around a step boundary add the same
// increment RN(RN(dt/2 * p) / rmass) -- p does not change in between -- so
// the one that ends a step (DELTA_STORE) leaves it in f.xyz, which is dead
// until the next force computation overwrites it, and the one that starts
// the next step (DELTA_USE) adds it instead of recomputing it when the
// status word ST_DELTA says f.xyz holds it (set after DELTA_STORE, cleared
// by every force computation and upload).  Bit for bit the same positions.
enum { DELTA_NONE = 0, DELTA_STORE = 1, DELTA_USE = 2 };

// INT_FMA: rinv is the drift coefficient, dt_r/rmass or (twice) 2*dt_r/rmass
template <bool POS, bool VEL, int MODE>
__global__ void __launch_bounds__(256) advance_kernel(Geom g, Slots s, const int *atom_slot,
                                                      int ntot, double dt_v, double dt_r,
                                                      double rmass, double rinv, bool mixed,
                                                      bool write32, bool classify, int delta,
                                                      bool twice, bool lazy32, RebinWork w,
                                                      int *status) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= ntot) return;
  const int slot = atom_slot[a];
  const int b = slot >> 6;
  d4 r = s.r[slot];
  if (MODE == INT_FMA && (POS || VEL)) {
    d4 p = s.p[slot];
    if (VEL) {
      // force order: the forces of the last force call are the FP32 records
      // (the slot arrays' f holds them only after a force call the caller reads)
      const int af = w.fo.force ? w.fo.of_id[s.id[slot]] : -1;
      d4 f;
      if (af >= 0) {
        const float4 f32 = w.fo.force[af];
        f.x = f32.x;
        f.y = f32.y;
        f.z = f32.z;
      } else {
        f = s.f[slot];
      }
      p.x = fma(-dt_v, f.x, p.x);
      p.y = fma(-dt_v, f.y, p.y);
      p.z = fma(-dt_v, f.z, p.z);
      s.p[slot] = p;
    }
    if (POS) {
      r.x = fma(p.x, rinv, r.x);
      r.y = fma(p.y, rinv, r.y);
      r.z = fma(p.z, rinv, r.z);
      s.r[slot] = r;
    }
  } else if (POS && !VEL && delta == DELTA_USE && *(volatile const int *)(status + ST_DELTA)) {
    const d4 dl = s.f[slot];
    r.x = r.x + dl.x;
    r.y = r.y + dl.y;
    r.z = r.z + dl.z;
    s.r[slot] = r;
  } else if (POS || VEL) {
    d4 p = s.p[slot];
    d4 f;
    if (VEL) {
      // advanceVelocity, timestep.c:71
      f = s.f[slot];
      p.x = p.x - dt_v * f.x;
      p.y = p.y - dt_v * f.y;
      p.z = p.z - dt_v * f.z;
      s.p[slot] = p;
    }
    if (POS) {
      // advancePositions, timestep.c:104: r + (dt*p)/rmass
      const double ix = div_mass<MODE>(dt_r * p.x, rmass, rinv);
      const double iy = div_mass<MODE>(dt_r * p.y, rmass, rinv);
      const double iz = div_mass<MODE>(dt_r * p.z, rmass, rinv);
      r.x = r.x + ix;
      r.y = r.y + iy;
      r.z = r.z + iz;
      if (twice) {
        // the closing half step of one step and the opening one of the next
        r.x = r.x + ix;
        r.y = r.y + iy;
        r.z = r.z + iz;
      }
      s.r[slot] = r;
      if (VEL && delta == DELTA_STORE) {
        f.x = ix;
        f.y = iy;
        f.z = iz;
        s.f[slot] = f;
      }
    }
  }
  if (POS) {
    if (mixed && write32) {
      const float4 p32 = centred32(rep_of(g, b), r.x, r.y, r.z);
      // lazy32: between list rebuilds only the stencil scan of an overflowed
      // list reads the slot-order copy (the classification before a rebuild
      // rewrites it for every atom)
      if (!lazy32 || *(volatile const int *)(status + ST_NBR_OVERFLOW)) s.pos32[slot] = p32;
      if (w.fo.of_id) fo_track(g, w.fo, b, s.id[slot], r, p32, status);
    }
    if ((!VEL || twice) && w.pl.rref) {
      // persistent lists: the half step before a force call decides
      // whether the lists are rebuilt (an atom moved more than skin/2)
      if (persist_stale(g, b, r, w.pl.rref[s.id[slot]], w.pl.half_skin2))
        atomicExch(status + ST_REBUILD, 1);
    }
  }
  if (classify) classify_atom(g, s, slot, r, mixed, w, status);
}

static unsigned slot_blocks(const Geom &g) {
  long nslots = (long)g.nboxes * CG_MAXATOMS;
  return (unsigned)((nslots + 255) / 256);
}

static unsigned atom_blocks(int ntot) { return (unsigned)((ntot + 255) / 256); }

// y = RN(1/b) when Markstein's division is exact for b, else 0 (IEEE path)
double mass_reciprocal(double rmass) {
  uint64_t bits;
  memcpy(&bits, &rmass, sizeof bits);
  const uint64_t mant = bits & ((1ull << 52) - 1);
  if (mant == (1ull << 52) - 1 || !(rmass > 0.0)) return 0.0;
  return 1.0 / rmass;
}

// the advance kernel for the integration mode of the simulation: mixed
// precision INT_FMA (rinv becomes the drift coefficient c), FP64 Markstein's
// division where it is exact for rmass, else IEEE division
template <bool POS, bool VEL>
static void launch_advance(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                           double dt_r, double c, double rmass, bool mixed, bool write32,
                           bool classify, int delta, bool twice, const RebinWork &w, int *status,
                           cudaStream_t st, bool lazy32 = false) {
  if (ntot <= 0) return;
  const unsigned nb = atom_blocks(ntot);
  const double rinv = mass_reciprocal(rmass);
  if (mixed && POS)
    advance_kernel<POS, VEL, INT_FMA><<<nb, 256, 0, st>>>(g, s, atom_slot, ntot, dt_v, dt_r,
                                                          rmass, c, mixed, write32, classify,
                                                          DELTA_NONE, twice, lazy32, w, status);
  else if (rinv != 0.0)
    advance_kernel<POS, VEL, INT_MARK><<<nb, 256, 0, st>>>(g, s, atom_slot, ntot, dt_v, dt_r,
                                                           rmass, rinv, mixed, write32, classify,
                                                           delta, twice, false, w, status);
  else
    advance_kernel<POS, VEL, INT_IEEE><<<nb, 256, 0, st>>>(g, s, atom_slot, ntot, dt_v, dt_r,
                                                           rmass, rinv, mixed, write32, classify,
                                                           delta, twice, false, w, status);
}

void launch_advance_positions(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt,
                              double rmass, bool mixed, bool classify, const RebinWork &w,
                              int *status, cudaStream_t st, bool use_delta) {
  if (classify) cudaMemsetAsync(w.depmask, 0, sizeof(uint32_t) * 4 * (size_t)g.nboxes, st);
  launch_advance<true, false>(g, s, atom_slot, ntot, 0.0, dt, dt / rmass, rmass, mixed, true,
                              classify, use_delta ? DELTA_USE : DELTA_NONE, false, w, status, st,
                              !classify && w.fo.of_id);
}

void launch_advance_vp(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                       double dt_r, double rmass, bool mixed, const RebinWork &w, int *status,
                       cudaStream_t st, bool write32) {
  cudaMemsetAsync(w.depmask, 0, sizeof(uint32_t) * 4 * (size_t)g.nboxes, st);
  launch_advance<true, true>(g, s, atom_slot, ntot, dt_v, dt_r, dt_r / rmass, rmass, mixed,
                             write32, true, DELTA_STORE, false, w, status, st);
  // FP64: f.xyz now holds the increments (the next position half step
  // reuses them); mixed precision does not keep them
  if (!mixed) cudaMemsetAsync(status + ST_DELTA, 0x01, 1, st);
}

void launch_advance_vpp(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                        double dt_r, double rmass, bool mixed, const RebinWork &w, int *status,
                        cudaStream_t st, bool classify) {
  if (classify) cudaMemsetAsync(w.depmask, 0, sizeof(uint32_t) * 4 * (size_t)g.nboxes, st);
  // mixed precision: one multiply-add by 2*dt_r/rmass for the two half steps
  launch_advance<true, true>(g, s, atom_slot, ntot, dt_v, dt_r, 2.0 * dt_r / rmass, rmass, mixed,
                             true, classify, DELTA_NONE, true, w, status, st,
                             !classify && w.fo.of_id);
}

void launch_advance_velocity(const Geom &g, Slots s, const int *atom_slot, int ntot, double dt_v,
                             cudaStream_t st) {
  RebinWork none{};
  if (ntot > 0)
    advance_kernel<false, true, INT_IEEE><<<atom_blocks(ntot), 256, 0, st>>>(
        g, s, atom_slot, ntot, dt_v, 0.0, 1.0, 0.0, false, false, false, DELTA_NONE, false, false,
        none, nullptr);
}

// only_if (optional): the status words of a force-order simulation whose
// rebox waits for list rebuilds; the launch does nothing unless a rebuild is
// due (ST_REBUILD).  Between rebuilds atoms may sit up to skin/2 outside
// their boxes; the skin is at most the box width minus the cutoff, so
// in-cutoff pairs stay within adjacent boxes and an overflowed atom's
// stencil scan still sees all of them.
__device__ __forceinline__ bool stood_down(const int *only_if) {
  return only_if && !*(volatile const int *)(only_if + ST_REBUILD);
}

// classify only, grid-stride over the atoms (a stood-down launch costs one
// check per CTA)
__global__ void __launch_bounds__(256) classify_kernel(Geom g, Slots s, const int *atom_slot,
                                                       int ntot, bool mixed, RebinWork w,
                                                       int *status, const int *only_if) {
  if (stood_down(only_if)) return;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < ntot; a += gridDim.x * blockDim.x) {
    const int slot = atom_slot[a];
    const d4 r = s.r[slot];
    if (mixed) s.pos32[slot] = centred32(rep_of(g, slot >> 6), r.x, r.y, r.z);
    classify_atom(g, s, slot, r, mixed, w, status);
  }
}

void launch_classify(const Geom &g, Slots s, const int *atom_slot, int ntot, bool mixed,
                     const RebinWork &w, int *status, cudaStream_t st, const int *only_if) {
  cudaMemsetAsync(w.depmask, 0, sizeof(uint32_t) * 4 * (size_t)g.nboxes, st);
  if (ntot > 0) {
    const unsigned nb = std::min(atom_blocks(ntot), 4096u);
    classify_kernel<<<nb, 256, 0, st>>>(g, s, atom_slot, ntot, mixed, w, status, only_if);
  }
}

__device__ __forceinline__ unsigned long long box_mask(const RebinWork &w, int b) {
  return (unsigned long long)w.depmask[2 * b] | ((unsigned long long)w.depmask[2 * b + 1] << 32);
}

__device__ __forceinline__ void set_error(int *status, int code) {
  atomicCAS(status + ST_ERROR, 0, code);
}

__global__ void rebin_plan_kernel(Geom g, Slots s, RebinWork w, int *status, const int *only_if) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nboxes || stood_down(only_if)) return;
  if (*(volatile int *)(status + ST_REBIN_SERIAL)) return;
  const unsigned long long mask = box_mask(w, b);
  const int n = s.natoms[b];
  const int n_lo = w.arr_lo[b];  // counted by the classify step
  w.n_lo[b] = n_lo;
  if (mask == 0ull && n_lo == 0) {
    w.final_len[b] = n;
    return;
  }
  int L = n + n_lo;
  if (n_lo > 0 && L >= CG_MAXATOMS) {  // moveAtom aborts at 64 (domains.c:229)
    set_error(status, -11);
    w.final_len[b] = 0;
    return;
  }
  uint8_t arr[CG_MAXATOMS];
  for (int t = 0; t < n; t++) arr[t] = (uint8_t)t;
  for (int t = 0; t < n_lo; t++) arr[n + t] = (uint8_t)(CG_MAXATOMS + t);
  int i = 0, d = 0;
  uint8_t *rank = w.dep_rank + (size_t)b * CG_MAXATOMS;
  while (i < L) {
    int e = arr[i];
    if (e < CG_MAXATOMS && ((mask >> e) & 1ull)) {
      rank[e] = (uint8_t)d++;
      arr[i] = arr[--L];
    } else {
      i++;
    }
  }
  uint8_t *fs = w.final_src + (size_t)b * CG_MAXATOMS;
  for (int t = 0; t < L; t++) fs[t] = arr[t];
  w.final_len[b] = L;
}

// the n (< 64) arrivals listed at list (old slots) in the order the
// reference's scans take them: by source box, then by departure rank there
__device__ __forceinline__ void sorted_arrivals(const RebinWork &w, const int *list, int n,
                                                int *src_of) {
  int key[CG_MAXATOMS];
  for (int t = 0; t < n; t++) {
    const int slot = list[t];
    const int kk = ((slot >> 6) << 6) | w.dep_rank[slot];  // source box, rank
    int q = t;
    while (q > 0 && key[q - 1] > kk) {
      key[q] = key[q - 1];
      src_of[q] = src_of[q - 1];
      q--;
    }
    key[q] = kk;
    src_of[q] = slot;
  }
}

__device__ void rebin_serial(const Geom &g, const Slots &s, bool mixed, int *status,
                             const SlotMap &slot_of);

// the plan stood down (a move of more than one box): thread 0 replays
// reBoxAll serially instead
__global__ void rebin_apply_kernel(Geom g, Slots s, bool mixed, RebinWork w, int *status,
                                   const int *only_if) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (stood_down(only_if)) return;
  if (*(volatile int *)(status + ST_REBIN_SERIAL)) {
    if (b == 0) rebin_serial(g, s, mixed, status, w.map);
    return;
  }
  if (b >= g.nboxes) return;
  if (*(volatile int *)(status + ST_ERROR)) return;
  const unsigned long long mask = box_mask(w, b);
  const int n_lo = w.n_lo[b];
  const int n_hi = w.arr_hi[b];  // counted by the classify step
  if (mask == 0ull && n_lo == 0 && n_hi == 0) return;
  const int L = w.final_len[b];
  if (n_hi > 0 && L + n_hi >= CG_MAXATOMS) {
    set_error(status, -11);
    return;
  }
  const int base = b * CG_MAXATOMS;
  const uint8_t *fs = w.final_src + (size_t)b * CG_MAXATOMS;
  // 1. stayers moved into holes (sources >= L, destinations < L)
  if (mask != 0ull)
    for (int t = 0; t < L; t++) {
      int e = fs[t];
      if (e < CG_MAXATOMS && e != t)
        copy_record(s, base + t, s, base + e, mixed, w.map);
    }
  int src_of[CG_MAXATOMS];
  // 2. lower arrivals into their placeholders, in (source, departure) order
  if (n_lo > 0) {
    sorted_arrivals(w, w.arr_list + base, n_lo, src_of);
    for (int t = 0; t < L; t++) {
      int e = fs[t];
      if (e >= CG_MAXATOMS)
        copy_record(s, base + t, w.stage, src_of[e - CG_MAXATOMS], mixed, w.map);
    }
  }
  // 3. higher arrivals appended, in (source, departure) order
  if (n_hi > 0) {
    sorted_arrivals(w, w.arr_list + (size_t)g.nboxes * CG_MAXATOMS + base, n_hi, src_of);
    for (int h = 0; h < n_hi; h++)
      copy_record(s, base + L + h, w.stage, src_of[h], mixed, w.map);
  }
  s.natoms[b] = L + n_hi;
}

// reBoxAll replayed serially on the device (used only when the parallel plan
// cannot reproduce it); the reference algorithm, statement for statement
__device__ void rebin_serial(const Geom &g, const Slots &s, bool mixed, int *status,
                             const SlotMap &slot_of) {
  status[ST_SERIAL_RUNS] += 1;
  for (int b = 0; b < g.nboxes; b++) {
    const RepGeo &R = rep_of(g, b);
    int ixo[3];
    box_ixyz(R, b, ixo);
    int i = 0;
    while (i < s.natoms[b]) {
      int off = b * CG_MAXATOMS + i;
      d4 r = s.r[off];
      double rc[3] = {r.x, r.y, r.z}, rn[3] = {r.x, r.y, r.z};
      int ixn[3];
      for (int k = 0; k < 3; k++) {
        if (rc[k] < 0.0) {
          ixn[k] = ixo[k] - 1;
          rn[k] += R.boxsize[k];
        } else if (rc[k] >= R.boxsize[k]) {
          ixn[k] = ixo[k] + 1;
          rn[k] -= R.boxsize[k];
        } else {
          ixn[k] = ixo[k];
        }
      }
      int jb = box_from_ixyz(R, g.periodic, ixn);
      if (jb < 0 || jb == b) {
        i++;
        continue;
      }
      s.r[off] = d4{rn[0], rn[1], rn[2], 0.0};
      if (mixed) s.pos32[off] = centred32(R, rn[0], rn[1], rn[2]);
      int nj = s.natoms[jb];
      if (nj >= CG_MAXATOMS - 1) {  // reaching 64 aborts (domains.c:229)
        set_error(status, -11);
        return;
      }
      copy_record(s, jb * CG_MAXATOMS + nj, s, off, mixed, slot_of);
      s.natoms[jb] = nj + 1;
      int ni = s.natoms[b] - 1;
      s.natoms[b] = ni;
      // the box's last atom fills the hole; when the departed atom was the
      // last one the reference's copy is onto itself, a no-op that must not
      // re-point the departed atom's id at its old slot
      if (ni && off != b * CG_MAXATOMS + ni)
        copy_record(s, off, s, b * CG_MAXATOMS + ni, mixed, slot_of);
    }
  }
}

void launch_rebin_finish(const Geom &g, Slots s, bool mixed, const RebinWork &w, int *status,
                         cudaStream_t st, const int *only_if) {
  unsigned nb = (unsigned)((g.nboxes + 127) / 128);
  rebin_plan_kernel<<<nb, 128, 0, st>>>(g, s, w, status, only_if);
  rebin_apply_kernel<<<nb, 128, 0, st>>>(g, s, mixed, w, status, only_if);
}

// ---------------------------------------------------------------------------
// persistent lists: id -> slot map, end of a rebuild
// ---------------------------------------------------------------------------
__global__ void slot_of_kernel(Geom g, Slots s, Persist pl, int ntot, int *status) {
  const long slot = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= (long)g.nboxes * CG_MAXATOMS) return;
  const int b = (int)(slot >> 6), k = (int)(slot & 63);
  if (k >= s.natoms[b]) return;
  const int id = s.id[slot];
  if (id < 0 || id >= ntot) {
    set_error(status, -1);
    return;
  }
  if (atomicExch(pl.slot_of + id, (int)slot) != -1) set_error(status, -1);
}

void launch_slot_of(const Geom &g, Slots s, Persist pl, int ntot, int *status, cudaStream_t st) {
  cudaMemsetAsync(pl.slot_of, 0xff, sizeof(int) * (size_t)ntot, st);
  slot_of_kernel<<<slot_blocks(g), 256, 0, st>>>(g, s, pl, ntot, status);
}

__global__ void rebuild_done_kernel(int *status) {
  if (status[ST_REBUILD]) {
    status[ST_REBUILDS] += 1;
    status[ST_REBUILD] = 0;
    // the overflows of the lists just built are those of the current lists
    status[ST_NBR_OVERFLOW] = status[ST_OVF_BUILD];
    status[ST_OVF_BUILD] = 0;
  }
}

// Force order after a host upload that keeps the lists: every atom's slot
// in the uploaded layout, by id
__global__ void fo_reslot_kernel(Geom g, Slots s, ForceOrder fo, int ntot) {
  const long slot = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= (long)g.nboxes * CG_MAXATOMS) return;
  const int b = (int)(slot >> 6), k = (int)(slot & 63);
  if (k >= s.natoms[b]) return;
  const int id = s.id[slot];
  if (id < 0 || id >= ntot) return;  // the id -> slot map reports it
  const int a = fo.of_id[id];
  if (a >= 0) fo.slot[a] = (int)slot;
}

void launch_fo_reslot(const Geom &g, Slots s, const ForceOrder &fo, int ntot, cudaStream_t st) {
  fo_reslot_kernel<<<slot_blocks(g), 256, 0, st>>>(g, s, fo, ntot);
}

// Force order, standalone force calls: every atom's force-order position
// from its refreshed FP32 position, and the rebuild test
__global__ void __launch_bounds__(256) fo_track_kernel(Geom g, Slots s, ForceOrder fo,
                                                       const int *atom_slot, int ntot,
                                                       int *status) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= ntot) return;
  const int slot = atom_slot[a];
  fo_track(g, fo, slot >> 6, s.id[slot], s.r[slot], s.pos32[slot], status);
}

void launch_fo_track(const Geom &g, Slots s, const ForceOrder &fo, const int *atom_slot,
                     int ntot, int *status, cudaStream_t st) {
  if (ntot > 0)
    fo_track_kernel<<<atom_blocks(ntot), 256, 0, st>>>(g, s, fo, atom_slot, ntot, status);
}

// skin test of every atom (standalone force calls: positions may have moved
// since the last half step that tested them)
__global__ void skin_check_kernel(Geom g, Slots s, Persist pl, bool mixed, int *status) {
  const long slot = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= (long)g.nboxes * CG_MAXATOMS) return;
  const int b = (int)(slot >> 6), k = (int)(slot & 63);
  if (k >= s.natoms[b]) return;
  if (persist_stale(g, b, s.r[slot], pl.rref[s.id[slot]], pl.half_skin2))
    atomicExch(status + ST_REBUILD, 1);
}

void launch_skin_check(const Geom &g, Slots s, Persist pl, bool mixed, int *status,
                       cudaStream_t st) {
  skin_check_kernel<<<slot_blocks(g), 256, 0, st>>>(g, s, pl, mixed, status);
}

void launch_rebuild_done(int *status, cudaStream_t st) {
  rebuild_done_kernel<<<1, 1, 0, st>>>(status);
}

// rebuild_done_kernel, then the condition of a conditional graph node: some
// list of the current lists overflowed
__global__ void rebuild_done_cond_kernel(int *status, cudaGraphConditionalHandle cond) {
  if (status[ST_REBUILD]) {
    status[ST_REBUILDS] += 1;
    status[ST_REBUILD] = 0;
    status[ST_NBR_OVERFLOW] = status[ST_OVF_BUILD];
    status[ST_OVF_BUILD] = 0;
  }
  cudaGraphSetConditional(cond, status[ST_NBR_OVERFLOW] != 0 ? 1u : 0u);
}
void launch_rebuild_done_cond(int *status, cudaGraphConditionalHandle cond, cudaStream_t st) {
  rebuild_done_cond_kernel<<<1, 1, 0, st>>>(status, cond);
}

// the condition of a conditional graph node: status word `word` is set
__global__ void status_cond_kernel(cudaGraphConditionalHandle cond, const int *status, int word) {
  cudaGraphSetConditional(cond, *(volatile const int *)(status + word) != 0 ? 1u : 0u);
}
void launch_status_cond(cudaGraphConditionalHandle cond, const int *status, int word,
                        cudaStream_t st) {
  status_cond_kernel<<<1, 1, 0, st>>>(cond, status, word);
}

// ---------------------------------------------------------------------------
// compaction: box_start = exclusive scan of natoms; atom_slot[a] = slot
// ---------------------------------------------------------------------------
#define CP_THREADS 256
#ifndef COMDGB_CP_PER
#define COMDGB_CP_PER 1  // boxes per thread in the compaction scans (1: 20 us at 110,592 boxes, 2: 27, 4: 37)
#endif
#define CP_PER COMDGB_CP_PER
#define CP_CHUNK (CP_THREADS * CP_PER)

int compact_partials(int nboxes) { return (nboxes + CP_CHUNK - 1) / CP_CHUNK; }

__device__ __forceinline__ int block_excl_scan(int v, int *sh, int &total) {
  // sh has CP_THREADS/32 ints
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = lane < CP_THREADS / 32 ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < CP_THREADS / 32) sh[lane] = t;
  }
  __syncthreads();
  total = sh[CP_THREADS / 32 - 1];
  int pre = wid > 0 ? sh[wid - 1] : 0;
  __syncthreads();
  return pre + x - v;
}

__global__ void __launch_bounds__(CP_THREADS) compact_sum_kernel(const int *natoms, int nboxes,
                                                                 int *partials,
                                                                 const int *only_if) {
  __shared__ int sh[CP_THREADS / 32];
  if (stood_down(only_if)) return;
  int base = blockIdx.x * CP_CHUNK + threadIdx.x * CP_PER;
  int v = 0;
  for (int q = 0; q < CP_PER; q++)
    if (base + q < nboxes) v += natoms[base + q];
  int total;
  block_excl_scan(v, sh, total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void __launch_bounds__(CP_THREADS) compact_scan_partials_kernel(int *partials,
                                                                           int npart,
                                                                           const int *only_if) {
  if (stood_down(only_if)) return;
  __shared__ int sh[CP_THREADS / 32];
  int carry = 0;
  for (int base = 0; base < npart; base += CP_THREADS) {
    int idx = base + threadIdx.x;
    int v = idx < npart ? partials[idx] : 0;
    int total;
    int ex = block_excl_scan(v, sh, total);
    if (idx < npart) partials[idx] = carry + ex;
    carry += total;
  }
}

// box offsets from the block's scan, then each warp writes whole boxes'
// atom entries (coalesced)
__global__ void __launch_bounds__(CP_THREADS) compact_write_kernel(const int *natoms, int nboxes,
                                                                   const int *partials,
                                                                   int *box_start,
                                                                   int *atom_slot, int ntot,
                                                                   const int *only_if) {
  __shared__ int sh[CP_THREADS / 32];
  __shared__ int s_off[CP_CHUNK], s_n[CP_CHUNK];
  if (stood_down(only_if)) return;
  const int b0 = blockIdx.x * CP_CHUNK;
  int loc[CP_PER];
  int v = 0;
  for (int q = 0; q < CP_PER; q++) {
    const int b = b0 + threadIdx.x * CP_PER + q;
    loc[q] = b < nboxes ? natoms[b] : 0;
    v += loc[q];
  }
  int total;
  int off = block_excl_scan(v, sh, total) + partials[blockIdx.x];
  for (int q = 0; q < CP_PER; q++) {
    const int i = threadIdx.x * CP_PER + q, b = b0 + i;
    s_off[i] = off;
    s_n[i] = loc[q];
    if (b < nboxes) {
      box_start[b] = off;
      if (b == nboxes - 1) box_start[nboxes] = off + loc[q];
    }
    off += loc[q];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, nbk = min(CP_CHUNK, nboxes - b0);
  for (int i = threadIdx.x >> 5; i < nbk; i += CP_THREADS / 32) {
    const int o = s_off[i], n = s_n[i], base = (b0 + i) * CG_MAXATOMS;
    // the counts sum to ntot unless a reported overflow left them inconsistent
    for (int k = lane; k < n; k += 32)
      if (o + k < ntot) atom_slot[o + k] = base + k;
  }
}

void launch_compact(const Geom &g, const int *natoms, int *box_start, int *atom_slot, int ntot,
                    int *partials, int npart, cudaStream_t st, const int *only_if) {
  compact_sum_kernel<<<npart, CP_THREADS, 0, st>>>(natoms, g.nboxes, partials, only_if);
  compact_scan_partials_kernel<<<1, CP_THREADS, 0, st>>>(partials, npart, only_if);
  compact_write_kernel<<<npart, CP_THREADS, 0, st>>>(natoms, g.nboxes, partials, box_start,
                                                     atom_slot, ntot, only_if);
}

// ids of a replica's slots, offset by its first atom
__global__ void add_offset_kernel(int *v, long n, int off) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) v[q] += off;
}
void launch_add_offset(int *v, long n, int off, cudaStream_t st) {
  if (n > 0) add_offset_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(v, n, off);
}

// ---------------------------------------------------------------------------
// deterministic reductions: energy (sum of f[3]), stress share, pair count
// ---------------------------------------------------------------------------
#define RD_THREADS 256
#define RD_PER 16

int reduce_partials(int ntot) {
  int n = (ntot + RD_THREADS * RD_PER - 1) / (RD_THREADS * RD_PER);
  return n < 1 ? 1 : n;
}

__device__ __forceinline__ double block_sum_d(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
  __syncthreads();
  return t;
}

__device__ __forceinline__ long long block_sum_l(long long v, long long *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  long long t = 0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(RD_THREADS) reduce_force_kernel(ForceArgs A, double *partials,
                                                                  long long *ipartials) {
  __shared__ double shd[RD_THREADS / 32];
  __shared__ long long shl[RD_THREADS / 32];
  int base = blockIdx.x * RD_THREADS * RD_PER;
  double e = 0.0, sx = 0.0;
  long long np = 0;
  for (int q = 0; q < RD_PER; q++) {
    int a = base + q * RD_THREADS + threadIdx.x;
    if (a < A.ntot) {
      e += A.s.f[A.atom_slot[a]].w;
      sx += A.atom_stress[a];
      np += A.nbr_n[a];
    }
  }
  e = block_sum_d(e, shd);
  sx = block_sum_d(sx, shd);
  np = block_sum_l(np, shl);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = e;
    partials[2 * blockIdx.x + 1] = sx;
    ipartials[blockIdx.x] = np;
  }
}

// The block partials summed by one CTA in a fixed order (thread t sums
// partials t, t + RD_THREADS, ... in turn, then the block tree), so every
// run gives the same bits.  (One thread summing them serially took 150 us
// for the ~1000 partials of 4 M atoms.)
__global__ void __launch_bounds__(RD_THREADS) reduce_final_kernel(const double *partials,
                                                                  const long long *ipartials,
                                                                  int npart, double *out,
                                                                  long long *iout) {
  __shared__ double shd[RD_THREADS / 32];
  __shared__ long long shl[RD_THREADS / 32];
  double e = 0.0, sx = 0.0;
  long long np = 0;
  for (int q = threadIdx.x; q < npart; q += RD_THREADS) {
    e += partials[2 * q];
    sx += partials[2 * q + 1];
    np += ipartials[q];
  }
  e = block_sum_d(e, shd);
  sx = block_sum_d(sx, shd);
  np = block_sum_l(np, shl);
  if (threadIdx.x == 0) {
    out[0] = e;
    out[1] = sx;
    iout[0] = np;
  }
}

void launch_reduce(const ForceArgs &A, double *partials, long long *ipartials, int npart,
                   double *out, long long *iout, cudaStream_t st) {
  reduce_force_kernel<<<npart, RD_THREADS, 0, st>>>(A, partials, ipartials);
  reduce_final_kernel<<<1, RD_THREADS, 0, st>>>(partials, ipartials, npart, out, iout);
}

// per replica (one block each, fixed order): energy sum f.w and stress share
__global__ void __launch_bounds__(RD_THREADS) rep_reduce_kernel(ForceArgs A, double *out) {
  __shared__ double shd[RD_THREADS / 32];
  const RepGeo &R = A.g.rep[blockIdx.x];
  double e = 0.0, sx = 0.0;
  for (int a = R.a0 + threadIdx.x; a < R.a0 + R.na; a += RD_THREADS) {
    e += A.s.f[A.atom_slot[a]].w;
    sx += A.atom_stress[a];
  }
  e = block_sum_d(e, shd);
  sx = block_sum_d(sx, shd);
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = e;
    out[2 * blockIdx.x + 1] = sx;
  }
}

void launch_rep_reduce(const ForceArgs &A, double *out, cudaStream_t st) {
  rep_reduce_kernel<<<A.g.nrep, RD_THREADS, 0, st>>>(A, out);
}

__global__ void __launch_bounds__(RD_THREADS) kinetic_kernel(Slots s, const int *atom_slot,
                                                             int ntot, double *partials) {
  __shared__ double shd[RD_THREADS / 32];
  int base = blockIdx.x * RD_THREADS * RD_PER;
  double ek = 0.0;
  for (int q = 0; q < RD_PER; q++) {
    int a = base + q * RD_THREADS + threadIdx.x;
    if (a < ntot) {
      d4 p = s.p[atom_slot[a]];
      ek += p.x * p.x + p.y * p.y + p.z * p.z;
    }
  }
  ek = block_sum_d(ek, shd);
  if (threadIdx.x == 0) partials[blockIdx.x] = ek;
}

// (the partials summed as in reduce_final_kernel)
__global__ void __launch_bounds__(RD_THREADS) kinetic_final_kernel(const double *partials,
                                                                   int npart, double rmass,
                                                                   double *out) {
  __shared__ double shd[RD_THREADS / 32];
  double ek = 0.0;
  for (int q = threadIdx.x; q < npart; q += RD_THREADS) ek += partials[q];
  ek = block_sum_d(ek, shd);
  if (threadIdx.x == 0) out[0] = ek / (2.0 * rmass);
}

void launch_kinetic(const Geom &g, Slots s, const int *atom_slot, int ntot, double rmass,
                    double *partials, int npart, double *out, cudaStream_t st) {
  (void)g;
  kinetic_kernel<<<npart, RD_THREADS, 0, st>>>(s, atom_slot, ntot, partials);
  kinetic_final_kernel<<<1, RD_THREADS, 0, st>>>(partials, npart, rmass, out);
}

// ---------------------------------------------------------------------------
// host layout (real3, 24-byte stride) <-> device double4
// ---------------------------------------------------------------------------
__global__ void unpack3_kernel(const double *src3, d4 *dst, long n) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[i] = d4{src3[3 * i], src3[3 * i + 1], src3[3 * i + 2], 0.0};
}

__global__ void pack3_kernel(const d4 *src, double *dst3, long n) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  d4 v = src[i];
  dst3[3 * i] = v.x;
  dst3[3 * i + 1] = v.y;
  dst3[3 * i + 2] = v.z;
}

// One warp per box.  Host memory is written and read in whole lines: the
// lanes walk each array's occupied range element by element (3 or 4 doubles
// per slot for r, p, f), so one warp instruction covers 256 contiguous bytes
// of the host array; the device side gathers or scatters the components of
// the 32-byte records.
__device__ __forceinline__ int zc_box(int nboxes, int &lane) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  lane = threadIdx.x & 31;
  const long b = t >> 5;
  if (b >= nboxes) return -1;
  return (int)b;
}

__global__ void zc_upload_kernel(HostSlots hs, Slots s, int nboxes, bool forces) {
  int lane;
  const int b = zc_box(nboxes, lane);
  if (b < 0) return;
  const int n = min(max(s.natoms[b], 0), CG_MAXATOMS);
  const long base = (long)b * CG_MAXATOMS;
  for (int k = lane; k < n; k += 32) {
    s.id[base + k] = hs.id[base + k];
    s.itype[base + k] = hs.itype[base + k];
    s.mass[base + k] = hs.mass[base + k];
  }
  double *rd = reinterpret_cast<double *>(s.r + base), *pd = reinterpret_cast<double *>(s.p + base);
  const double *rh = hs.r + 3 * base, *ph = hs.p + 3 * base;
  for (int q = lane; q < 3 * n; q += 32) {
    const int k = q / 3, c = q - 3 * k;
    rd[4 * k + c] = rh[q];
    pd[4 * k + c] = ph[q];
  }
  for (int k = lane; k < n; k += 32) {
    rd[4 * k + 3] = 0.0;
    pd[4 * k + 3] = 0.0;
  }
  if (forces) {
    double *fd = reinterpret_cast<double *>(s.f + base);
    const double *fh = hs.f + 4 * base;
    for (int q = lane; q < 4 * n; q += 32) fd[q] = fh[q];
    for (int k = lane; k < n; k += 32) {
      s.rho[base + k] = hs.rho[base + k];
      s.fi[base + k] = hs.fi[base + k];
    }
  }
}

__device__ __forceinline__ void zc_download_box(const HostSlots &hs, const Slots &s, int b,
                                                int lane, bool state, bool forces) {
  const int n = min(max(s.natoms[b], 0), CG_MAXATOMS);
  const long base = (long)b * CG_MAXATOMS;
  if (state) {
    for (int k = lane; k < n; k += 32) {
      hs.id[base + k] = s.id[base + k];
      hs.itype[base + k] = s.itype[base + k];
      hs.mass[base + k] = s.mass[base + k];
    }
    const double *rd = reinterpret_cast<const double *>(s.r + base);
    const double *pd = reinterpret_cast<const double *>(s.p + base);
    double *rh = hs.r + 3 * base, *ph = hs.p + 3 * base;
    for (int q = lane; q < 3 * n; q += 32) {
      const int k = q / 3, c = q - 3 * k;
      rh[q] = rd[4 * k + c];
      ph[q] = pd[4 * k + c];
    }
  }
  if (forces) {
    const double *fd = reinterpret_cast<const double *>(s.f + base);
    double *fh = hs.f + 4 * base;
    for (int q = lane; q < 4 * n; q += 32) fh[q] = fd[q];
    for (int k = lane; k < n; k += 32) {
      hs.rho[base + k] = s.rho[base + k];
      hs.fi[base + k] = s.fi[base + k];
    }
  }
}

// (a warp per box, grid-stride over the boxes: a small grid runs beside
// other kernels)
__global__ void zc_download_kernel(HostSlots hs, Slots s, int nboxes, bool state, bool forces) {
  const int lane = threadIdx.x & 31;
  const long w0 = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nw = ((long)gridDim.x * blockDim.x) >> 5;
  for (long bb = w0; bb < nboxes; bb += nw) zc_download_box(hs, s, (int)bb, lane, state, forces);
}

static unsigned zc_blocks(int nboxes) {
  return (unsigned)(((long)nboxes * 32 + 255) / 256);  // one warp per box
}

void launch_zc_upload(const HostSlots &hs, Slots s, int nboxes, bool forces, cudaStream_t st) {
  if (nboxes > 0) zc_upload_kernel<<<zc_blocks(nboxes), 256, 0, st>>>(hs, s, nboxes, forces);
}

void launch_zc_download(const HostSlots &hs, Slots s, int nboxes, bool state, bool forces,
                        cudaStream_t st, int max_blocks) {
  unsigned nb = zc_blocks(nboxes);
  if (max_blocks > 0 && nb > (unsigned)max_blocks) nb = (unsigned)max_blocks;
  if (nboxes > 0) zc_download_kernel<<<nb, 256, 0, st>>>(hs, s, nboxes, state, forces);
}

void launch_unpack3(const double *src3, d4 *dst, long n, cudaStream_t st) {
  if (n > 0) unpack3_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src3, dst, n);
}

void launch_pack3(const d4 *src, double *dst3, long n, cudaStream_t st) {
  if (n > 0) pack3_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst3, n);
}

// only_if_overflow (optional): status words; nothing unless some list
// overflowed (ST_NBR_OVERFLOW), the one case the slot-order copy is read
__global__ void pos32_kernel(Geom g, Slots s, const int *only_if_overflow) {
  long slot = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= (long)g.nboxes * CG_MAXATOMS) return;
  if (only_if_overflow && !*(volatile const int *)(only_if_overflow + ST_NBR_OVERFLOW)) return;
  d4 r = s.r[slot];
  s.pos32[slot] = centred32(rep_of(g, (int)(slot >> 6)), r.x, r.y, r.z);
}

void launch_pos32(const Geom &g, Slots s, cudaStream_t st, const int *only_if_overflow) {
  pos32_kernel<<<slot_blocks(g), 256, 0, st>>>(g, s, only_if_overflow);
}

// ---------------------------------------------------------------------------
// initial binning: n putAtomInBox calls (domains.c:237-291) as a counting
// sort that keeps call order within each box
// ---------------------------------------------------------------------------
// (one replica: the initial binning of a single simulation; the bodies are
// shared with the allocation-free entry point, binning.cuh)
__device__ __forceinline__ BinGrid bin_grid(const Geom &g) {
  const RepGeo &R = g.rep[0];
  BinGrid b;
  for (int m = 0; m < 3; m++) {
    b.nbx[m] = R.nbx[m];
    b.bounds[m] = R.bounds[m];
    b.boxsize[m] = R.boxsize[m];
  }
  b.nboxes = g.nboxes;
  return b;
}

__global__ void bin_count_kernel(Geom g, Slots s, int n, const double *xyz, int *tmp_index,
                                 int *status) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int err = bin_count_atom(bin_grid(g), t, xyz, s.natoms, tmp_index);
  if (err) set_error(status, err);
}

__global__ void bin_place_kernel(Geom g, const double *dcenter, Slots s, int n,
                                 const double *xyz, const double *pxyz, const int *ids,
                                 const int *types, const double *masses, int *tmp_index,
                                 int *status) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nboxes) return;
  if (*(volatile int *)(status + ST_ERROR)) return;
  int nb = s.natoms[b];
  if (nb > CG_MAXATOMS) return;  // reported by bin_count_kernel
  int *ix = tmp_index + b * CG_MAXATOMS;
  bin_sort_box(ix, nb);
  const BinGrid bg = bin_grid(g);
  for (int k = 0; k < nb; k++) {
    int t = ix[k];
    int slot = b * CG_MAXATOMS + k;
    double w[3];
    bool ok;
    bin_world_box(bg, xyz + 3 * (long)t, w, ok);
    s.id[slot] = ids[t];
    s.itype[slot] = types[t];
    s.mass[slot] = masses[t];
    s.r[slot] = d4{w[0] - dcenter[3 * b], w[1] - dcenter[3 * b + 1], w[2] - dcenter[3 * b + 2],
                   0.0};
    s.p[slot] = d4{pxyz[3 * (long)t], pxyz[3 * (long)t + 1], pxyz[3 * (long)t + 2], 0.0};
    s.f[slot] = d4{0.0, 0.0, 0.0, 0.0};
    s.rho[slot] = 0.0;
    s.fi[slot] = 0.0;
  }
}

void launch_bin_atoms(const Geom &g, const double *dcenter, Slots s, int n, const double *xyz,
                      const double *pxyz, const int *ids, const int *types, const double *masses,
                      int *tmp_index, int *status, cudaStream_t st) {
  cudaMemsetAsync(s.natoms, 0, sizeof(int) * g.nboxes, st);
  if (n > 0) bin_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(g, s, n, xyz, tmp_index, status);
  bin_place_kernel<<<(g.nboxes + 127) / 128, 128, 0, st>>>(g, dcenter, s, n, xyz, pxyz, ids,
                                                           types, masses, tmp_index, status);
}

// ---------------------------------------------------------------------------
// Chebyshev fit in FP64 (genCheb/genDer, cheby.c:125-179, 219-270), one
// block of n threads per series
// ---------------------------------------------------------------------------
__global__ void cheb_fit_kernel(const double *v, double x0, double xn, double invdx, int n,
                                double *coef, double *dcoef) {
  __shared__ double fk[64];
  __shared__ double c[64];
  const double PI = 3.141592653589793;
  int k = threadIdx.x;
  double a = x0, b = xn;
  double bma = 0.5 * (b - a), bpa = 0.5 * (b + a);
  if (k < n) {
    double y = cos(PI * (k + 0.5) / n);
    // eamInterpolateDerivlocal (cheby.c:15-60): table value, >1e10 -> 0
    double r = y * bma + bpa;
    if (r < x0) r = x0;
    else if (r > xn) r = xn;
    r = (r - x0) * invdx;
    double fl = floor(r);
    int i1 = (int)fl;
    r = r - fl;
    double gi = v[i1 + 1] - v[i1 - 1];
    double val = v[i1] + 0.5 * r * (r * (v[i1 + 1] + v[i1 - 1] - 2.0 * v[i1]) + gi);
    if (val > 1.0e10) val = 0.0;
    fk[k] = val;
  }
  __syncthreads();
  if (k < n) {
    double fac = 2.0 / n, sum = 0.0;
    for (int q = 0; q < n; q++) sum += fk[q] * cos(PI * k * (q + 0.5) / n);
    c[k] = fac * sum;
    coef[k] = c[k];
  }
  __syncthreads();
  if (k == 0) {
    double cd[64];
    cd[n - 1] = 0.0;
    cd[n - 2] = 2.0 * (n - 1) * c[n - 1];
    for (int j = n - 2; j > 0; j--) cd[j - 1] = cd[j + 1] + 2 * (j)*c[j];
    double con = 2.0 / (b - a);
    for (int j = 0; j < n; j++) dcoef[j] = cd[j] * con;
  }
}

void launch_cheb_fit(const double *table_v, double x0, double xn, double invdx, int n_terms,
                     double *coef, double *dcoef, cudaStream_t st) {
  cheb_fit_kernel<<<1, 64, 0, st>>>(table_v, x0, xn, invdx, n_terms, coef, dcoef);
}

}  // namespace cg
