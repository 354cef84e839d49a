// force_kernels.cuh -- link-cell force kernels, templated on the pair
// arithmetic type T (double: the plain FP64 kernels; float: mixed precision).
//
// Work decomposition (full pairs: every atom sums over all its neighbours,
// so per-atom sums need no atomics and are deterministic):
//   nbr_build   one CTA per box.  The box's stencil entries (27 neighbour
//               boxes with the reference's multiplicity) are staged from HBM
//               into shared memory; each warp takes one atom of the box and
//               tests 32 candidates per iteration, compacting hits with a
//               ballot into the atom's neighbour list (uint16 codes: entry
//               index << 6 | slot).  Cutoff test as pass 1 of eamForce:
//               r2 <= rc2 (eam.c:521, ljForce.c:193).
//   eam_pass1   one thread per atom over its list: pair phi, phi', rho
//               (eam.c:484-549), then F(rho) and F'(rho) fused in
//               (eam.c:576-594).
//   eam_pass2   one thread per atom: (F'_i + F'_j) rho'(r) dr/r and the
//               x-x stress (eam.c:595-653), r2 < rc2.
//   lj_pass     one thread per atom: the 12-6 terms of ljForce.c:151-215.
// Atoms whose neighbour count exceeds the list capacity fall back to a
// direct scan of their stencil, so results never depend on the capacity.
#pragma once

#include "common.cuh"

namespace cg {

enum { EVAL_TABLE = 0, EVAL_CHEBY = 1 };
constexpr int PASS_THREADS = 256;  // CTA size of the EAM passes

struct ForceArgs {
  Geom g;
  Slots s;
  EntryTab et;
  const int *atom_slot;  // [ntot] slot of the a-th atom (box order)
  const int *box_start;  // [nboxes+1] first atom index of each box
  int ntot;
  uint16_t *nbr;         // [ntot*cap]
  int *nbr_n;            // [ntot] true neighbour count
  int cap;
  double *atom_stress;   // [ntot] per-atom share of the scalar stress
  int *status;
  Persist pl;            // persistent lists keyed by id (FP64)
  ForceOrder fo;         // persistent lists in force order (mixed; fo.list != nullptr)
  // force order, a step sequence: the velocity-Verlet coefficients of the
  // update the force pass makes when ST_FUSE is set (p -= vv_dt f, r += vv_c p)
  double vv_dt, vv_c;
  // force order, a force call whose results go straight to an attached host
  // simflat_t (device pointers of its registered f, rho, fi; slot-indexed),
  // or null
  double *host_f, *host_rho, *host_fi;
};

// Stencil entry of box jb seen from box b when both stencils are the full
// 27 boxes in getNeighborBoxes order (periodic, nbx >= 3): (dx+1)*9 +
// (dy+1)*3 + (dz+1) with the minimum-image box difference; -1 when the boxes
// are not neighbours (then the atoms are farther apart than a box, i.e.
// beyond the cutoff).
__device__ __forceinline__ int stencil_entry(const Geom &g, int b, int jb) {
  const int ci = __ldg(g.boxc + b), cj = __ldg(g.boxc + jb);
  const RepGeo &R = rep_of(g, b);
  int e = 0;
#pragma unroll
  for (int ax = 0; ax < 3; ax++) {
    int d = ((cj >> (10 * ax)) & 1023) - ((ci >> (10 * ax)) & 1023);
    if (d > 1) d -= R.nbx[ax];
    else if (d < -1) d += R.nbx[ax];
    if (d > 1 || d < -1) return -1;
    e = e * 3 + d + 1;
  }
  return e;
}

// Box offset of a stencil entry: FP64 value, or FP32 hi + lo parts.
template <class T>
struct BoxOff;
template <>
struct BoxOff<double> {
  double x, y, z;
};
template <>
struct BoxOff<float> {
  float x, y, z, lx, ly, lz;
};

template <class T>
struct PrecT;

template <>
struct PrecT<double> {
  typedef DSum Acc;
  static __device__ __forceinline__ void pos(const Slots &s, int slot, double &x, double &y,
                                             double &z) {
    d4 v = s.r[slot];
    x = v.x; y = v.y; z = v.z;
  }
  static __device__ __forceinline__ BoxOff<double> drbox(const EntryTab &et, int idx) {
    d4 v = et.dr64[idx];
    return BoxOff<double>{v.x, v.y, v.z};
  }
  static __device__ __forceinline__ double fi(const Slots &s, int slot) { return s.fi[slot]; }
};

template <>
struct PrecT<float> {
  // every per-atom sum Kahan-compensated: forces, energy, density, stress
  typedef KSum Acc;
  static __device__ __forceinline__ void pos(const Slots &s, int slot, float &x, float &y,
                                             float &z) {
    float4 v = __ldg(s.pos32 + slot);
    x = v.x; y = v.y; z = v.z;
  }
  static __device__ __forceinline__ BoxOff<float> drbox(const EntryTab &et, int idx) {
    float4 h = __ldg(et.dr32 + 2 * idx), l = __ldg(et.dr32 + 2 * idx + 1);
    return BoxOff<float>{h.x, h.y, h.z, l.x, l.y, l.z};
  }
  static __device__ __forceinline__ float fi(const Slots &s, int slot) {
    return __ldg(s.fi32 + slot);
  }
};

// FP64: dr = drbox + r_i - r_j and r2 accumulated in the reference's order
__device__ __forceinline__ double pair_r2(const BoxOff<double> &o, double xi, double yi,
                                          double zi, double xj, double yj, double zj, double &dx,
                                          double &dy, double &dz) {
  dx = (o.x + xi) - xj;
  dy = (o.y + yi) - yj;
  dz = (o.z + zi) - zj;
  double r2 = dx * dx;
  r2 = r2 + dy * dy;
  r2 = r2 + dz * dz;
  return r2;
}

// FP32: coordinates are relative to the box centre (|x| <= boxsize/2) and
// the box offset is added as hi + lo, so dr carries only its own rounding
__device__ __forceinline__ float pair_r2(const BoxOff<float> &o, float xi, float yi, float zi,
                                         float xj, float yj, float zj, float &dx, float &dy,
                                         float &dz) {
  dx = ((xi - xj) + o.x) + o.lx;
  dy = ((yi - yj) + o.y) + o.ly;
  dz = ((zi - zj) + o.z) + o.lz;
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// Visit every stencil candidate of atom (b, i) directly (overflow path).
// fn(j_slot, dx, dy, dz, r2) is called for candidates with r2 <= rc2.
template <class T, class F>
__device__ void scan_stencil(const ForceArgs &A, int b, int i, T xi, T yi, T zi, T rc2, F &&fn) {
  int ne = A.et.n[b];
  for (int e = 0; e < ne; e++) {
    int jb = A.et.box[b * CG_NNBR + e];
    BoxOff<T> bo = PrecT<T>::drbox(A.et, b * CG_NNBR + e);
    int nj = A.s.natoms[jb];
    for (int k = 0; k < nj; k++) {
      if (jb == b && k == i) continue;
      int js = jb * CG_MAXATOMS + k;
      T xj, yj, zj, dx, dy, dz;
      PrecT<T>::pos(A.s, js, xj, yj, zj);
      T r2 = pair_r2(bo, xi, yi, zi, xj, yj, zj, dx, dy, dz);
      if (r2 > rc2) continue;
      fn(js, dx, dy, dz, r2);
    }
  }
}

// Persistent list of atom (b, i): neighbour ids, looked up in their current
// slots; the pair's box offset is the stencil entry of the two current boxes,
// so dr is formed exactly as with the per-step list.
// With `a` >= 0 the pairs within rc2 are also written, as slot codes, to the
// per-step list of compact atom a (for the passes that follow).
template <class T, class F>
__device__ __forceinline__ void for_each_persistent(const ForceArgs &A, int a, int b, int i, T xi,
                                                    T yi, T zi, T rc2, F &&fn) {
  const int idi = A.s.id[b * CG_MAXATOMS + i];
  const int n = A.pl.vcount[idi];
  if (n > A.pl.vcap) {
    scan_stencil<T>(A, b, i, xi, yi, zi, rc2, fn);
    if (a >= 0) A.nbr_n[a] = A.cap + 1;  // later passes scan the stencil too
    return;
  }
  uint16_t *emit = a >= 0 ? A.nbr + (size_t)a * A.cap : nullptr;
  int cnt = 0;
  const int *lst = A.pl.vlist + (size_t)idi * A.pl.vcap;
#pragma unroll 1
  for (int t = 0; t < n; t++) {
    const int js = __ldg(A.pl.slot_of + __ldg(lst + t));
    const int e = stencil_entry(A.g, b, js >> 6);
    if (e < 0) continue;
    T xj, yj, zj, dx, dy, dz;
    BoxOff<T> bo = PrecT<T>::drbox(A.et, b * CG_NNBR + e);
    PrecT<T>::pos(A.s, js, xj, yj, zj);
    T r2 = pair_r2(bo, xi, yi, zi, xj, yj, zj, dx, dy, dz);
    if (emit && r2 <= rc2) {
      if (cnt < A.cap) emit[cnt] = (uint16_t)((e << 6) | (js & 63));
      cnt++;
    }
    fn(js, dx, dy, dz, r2);
  }
  if (a >= 0) {
    A.nbr_n[a] = cnt;
    if (cnt > A.cap) atomicAdd(A.status + ST_NBR_OVERFLOW, 1);
  }
}

// Visit the atom's neighbour list (or its stencil when the list overflowed).
// The first pass of a force call with persistent lists (PERSIST_FIRST)
// walks the skin list instead and leaves the exact per-step list behind.
// VEC: read eight codes per 16-byte load and unroll over them (light
// passes: independent gathers in flight); otherwise one copy of the pair
// code in the loop (heavy passes: instruction cache).
template <class T, bool VEC = false, bool PERSIST_FIRST = false, class F>
__device__ __forceinline__ void for_each_neighbor(const ForceArgs &A, int a, int b, int i, T xi,
                                                  T yi, T zi, T rc2, F &&fn) {
  if (PERSIST_FIRST && A.pl.vlist) {
    for_each_persistent<T>(A, a, b, i, xi, yi, zi, rc2, fn);
    return;
  }
  const int n = A.nbr_n[a];
  if (n > A.cap) {
    scan_stencil<T>(A, b, i, xi, yi, zi, rc2, fn);
    return;
  }
  const int ebase = b * CG_NNBR;
  auto visit = [&](uint32_t code) {
    const int e = code >> 6, k = code & 63;
    const int js = __ldg(A.et.box + ebase + e) * CG_MAXATOMS + k;
    T xj, yj, zj, dx, dy, dz;
    BoxOff<T> bo = PrecT<T>::drbox(A.et, ebase + e);
    PrecT<T>::pos(A.s, js, xj, yj, zj);
    T r2 = pair_r2(bo, xi, yi, zi, xj, yj, zj, dx, dy, dz);
    fn(js, dx, dy, dz, r2);
  };
  if (VEC) {
    const uint16_t *lst = A.nbr + (size_t)a * A.cap;
    for (int t0 = 0; t0 < n; t0 += 8) {
      const uint4 pk = *reinterpret_cast<const uint4 *>(lst + t0);
      const uint32_t w[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (t0 + u < n) visit((w[u >> 1] >> ((u & 1) * 16)) & 0xffffu);
    }
  } else {
    const uint32_t *lst = reinterpret_cast<const uint32_t *>(A.nbr + (size_t)a * A.cap);
#pragma unroll 1
    for (int t = 0; t < n; t++) visit((__ldg(lst + (t >> 1)) >> ((t & 1) * 16)) & 0xffffu);
  }
}

// ---------------------------------------------------------------------------
// neighbour-list build: one CTA per box, one warp per atom of the box
// ---------------------------------------------------------------------------
#define NB_THREADS 128
#define NB_MAXC (CG_NNBR * CG_MAXATOMS)

// stencil entries of box b: boxes, box offsets and candidate offsets (warp 0)
template <class T>
__device__ __forceinline__ int stage_entries(const ForceArgs &A, int b, int *s_box, int *s_off,
                                             BoxOff<T> *s_dr) {
  const int ne = A.et.n[b];
  if (threadIdx.x < 32) {
    const int e = threadIdx.x;
    int n = 0;
    if (e < ne) {
      int jb = A.et.box[b * CG_NNBR + e];
      s_box[e] = jb;
      s_dr[e] = PrecT<T>::drbox(A.et, b * CG_NNBR + e);
      n = min(A.s.natoms[jb], CG_MAXATOMS);  // (more only in a reported overflow)
    }
    int x = n;  // inclusive warp scan
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (e >= o) x += y;
    }
    if (e < ne) s_off[e + 1] = x;
    if (e == 0) s_off[0] = 0;
  }
  __syncthreads();
  return ne;
}

// FP32 lists: the staged entries sorted by neighbour box (ties by entry),
// so that every list comes out in ascending neighbour slot -- atoms in force
// order are in box order, and lanes of a warp then walk the position array
// together.  s_code keeps each entry's stencil index (the passes take the
// box offset from it); s_off is rebuilt in the new order.
__device__ __forceinline__ void order_entries_by_box(int ne, int *s_box, int *s_off,
                                                     BoxOff<float> *s_dr, int *s_code) {
  if (threadIdx.x < 32) {
    const int e = threadIdx.x;
    const int jb = e < ne ? s_box[e] : 0x7fffffff;
    BoxOff<float> dr{};
    int n = 0;
    if (e < ne) {
      dr = s_dr[e];
      n = s_off[e + 1] - s_off[e];
    }
    int rank = 0;
    for (int q = 0; q < ne; q++) {
      const int jq = __shfl_sync(0xffffffffu, jb, q);
      rank += (jq < jb) || (jq == jb && q < e);
    }
    // n of the entry at each rank, for the new prefix
    int x = 0;
    for (int q = 0; q < ne; q++) {
      const int rq = __shfl_sync(0xffffffffu, rank, q);
      const int nq = __shfl_sync(0xffffffffu, n, q);
      if (rq == e) x = nq;
    }
    __syncwarp();
    if (e < ne) {
      s_box[rank] = jb;
      s_dr[rank] = dr;
      s_code[rank] = e;
    }
    for (int o = 1; o < 32; o <<= 1) {  // inclusive scan over ranks
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (e >= o) x += y;
    }
    if (e < ne) s_off[e + 1] = x;
    if (e == 0) s_off[0] = 0;
  }
  __syncthreads();
}

// force-order entry code of stencil entry e = (dx+1)*9 + (dy+1)*3 + (dz+1)
// (periodic, nbx >= 3): the three box differences as 2-bit fields d+1 at
// bits 0, 2 and 4
__device__ __forceinline__ int fo_code(int e) {
  return (e / 9) | (((e / 3) % 3) << 2) | ((e % 3) << 4);
}

__device__ __forceinline__ int entry_of(const int *s_off, int ne, int c) {
  int lo = 0, hi = ne - 1;  // last e with s_off[e] <= c
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (s_off[mid] <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// FP32: candidates staged as (x - drbox, y - drbox, z - drbox, code) in the
// centre box's frame, padded to whole 32-candidate chunks with far-away
// sentinels.  Each warp takes two atoms per candidate load and parks every
// chunk's ballot in warp-private shared memory; the warp then writes each
// atom's list cooperatively (one mask word per lane, prefix sum of the
// popcounts, each lane emits its own bits).  The cutoff of the build is
// widened by a hair so the list is a superset of the pairs the passes accept
// with their exact dr.
#define NB_CHUNKS (NB_MAXC / 32)  // 54
#define NB_ATOMS 4                 // atoms tested per candidate load
// Modes: LIST_STEP writes the per-step list (uint16 codes); LIST_ID (runs
// only when a rebuild is due) writes neighbour ids into the atom's id-keyed
// row and records its position; LIST_FO (also only when due) writes the
// transposed force-order list and the atom's force-order record.
enum { LIST_STEP = 0, LIST_ID = 1, LIST_FO = 2 };

template <int MODE>
__device__ __forceinline__ bool build_skipped(const ForceArgs &A) {
  return MODE != LIST_STEP && !*(volatile const int *)(A.status + ST_REBUILD);
}

// row of atom i of box b: list storage, count slot and capacity
template <int MODE>
__device__ __forceinline__ int build_row(const ForceArgs &A, int b, int i) {
  const int slot = b * CG_MAXATOMS + i;
  if (MODE == LIST_ID) {
    const int idi = A.s.id[slot];
    A.pl.rref[idi] = world64(A.g, b, A.s.r[slot]);
    return idi;
  }
  const int a = A.box_start[b] + i;
  if (MODE == LIST_FO) {
    const float4 p = A.s.pos32[slot];
    const int id = A.s.id[slot];
    A.fo.ref[a] = make_float4(p.x, p.y, p.z, __int_as_float(b));
    A.fo.id[a] = id;
    A.fo.of_id[id] = a;
    A.fo.slot[a] = slot;
    A.fo.pos[a] = p;
  }
  return a;
}

template <int MODE>
__device__ __forceinline__ void build_store(const ForceArgs &A, int row, int h, int value) {
  if (MODE == LIST_ID) A.pl.vlist[(size_t)row * A.pl.vcap + h] = value;
  else if (MODE == LIST_FO)
    A.fo.list[((size_t)(row >> 5) * A.fo.vcap + h) * 32 + (row & 31)] = (uint32_t)value;
  else A.nbr[(size_t)row * A.cap + h] = (uint16_t)value;
}

template <int MODE>
__device__ __forceinline__ int build_cap(const ForceArgs &A) {
  return MODE == LIST_ID ? A.pl.vcap : MODE == LIST_FO ? A.fo.vcap : A.cap;
}

template <int MODE>
__device__ __forceinline__ void build_count(const ForceArgs &A, int row, int total) {
  if (MODE == LIST_ID) A.pl.vcount[row] = total;
  else if (MODE == LIST_FO) A.fo.n[row] = total;
  else A.nbr_n[row] = total;
  // persistent lists: counted for the lists being built (rebuild_done makes
  // it the current lists' count)
  if (total > build_cap<MODE>(A))
    atomicAdd(A.status + (MODE == LIST_STEP ? ST_NBR_OVERFLOW : ST_OVF_BUILD), 1);
}

// the lists of the atoms of box b (not empty): NT threads (the CTA), NA
// atoms tested per candidate load, the shared arrays of the kernel
template <int MODE, int NT, int NA>
__device__ __forceinline__ void build_box32(const ForceArgs &A, float rc2, int b, float4 *cand,
                                            uint32_t (*s_mask)[NA][NB_CHUNKS], int *s_box,
                                            int *s_off, int *s_code, BoxOff<float> *s_dr) {
  const int ni = A.s.natoms[b];
  const int ne = stage_entries<float>(A, b, s_box, s_off, s_dr);
  if (MODE != LIST_ID) order_entries_by_box(ne, s_box, s_off, s_dr, s_code);
  const int ncand = s_off[ne];
  const int nchunk = (ncand + 31) >> 5;
  for (int c = threadIdx.x; c < (nchunk << 5); c += NT) {
    if (c < ncand) {
      int e = entry_of(s_off, ne, c);
      int k = c - s_off[e];
      float4 q = __ldg(A.s.pos32 + s_box[e] * CG_MAXATOMS + k);
      BoxOff<float> o = s_dr[e];
      // force order: with periodic nbx >= 3 the entry index is the code
      const int tag = MODE == LIST_ID   ? A.s.id[s_box[e] * CG_MAXATOMS + k]
                      : MODE == LIST_FO ? (int)(((unsigned)(A.box_start[s_box[e]] + k) << 6) |
                                                fo_code(s_code[e]))
                                        : ((s_code[e] << 6) | k);
      // negated, so the test below is one packed add per axis: pa + (-c)
      // rounds exactly as pa - c
      cand[c] = make_float4(-((q.x - o.x) - o.lx), -((q.y - o.y) - o.ly), -((q.z - o.z) - o.lz),
                            __int_as_float(tag));
    } else {
      cand[c] = make_float4(-1e18f, -1e18f, -1e18f, 0.f);
    }
  }
  __syncthreads();
  const float rc2b = rc2 * (1.0f + 4e-6f);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  static_assert(NA % 2 == 0, "atoms are tested in pairs");
  for (int i0 = NA * warp; i0 < ni; i0 += NA * (NT / 32)) {
    const int na = min(NA, ni - i0);
    // the atoms in pairs, one per half of the packed FP32x2 operations (two
    // pair tests per instruction; r^2 = dx*dx, + dy*dy, + dz*dz rounded as
    // fmaf(dz, dz, fmaf(dy, dy, dx * dx)))
    float2 px[NA / 2], py[NA / 2], pz[NA / 2];
#pragma unroll
    for (int u = 0; u < NA / 2; u++) {
      const float4 a0 = __ldg(A.s.pos32 + b * CG_MAXATOMS + i0 + (2 * u < na ? 2 * u : 0));
      const float4 a1 = __ldg(A.s.pos32 + b * CG_MAXATOMS + i0 + (2 * u + 1 < na ? 2 * u + 1 : 0));
      px[u] = make_float2(a0.x, a1.x);
      py[u] = make_float2(a0.y, a1.y);
      pz[u] = make_float2(a0.z, a1.z);
    }
    for (int q = 0; q < nchunk; q++) {
      const float4 cq = cand[(q << 5) + lane];
      const float2 cx = make_float2(cq.x, cq.x), cy = make_float2(cq.y, cq.y),
                   cz = make_float2(cq.z, cq.z);
#pragma unroll
      for (int u = 0; u < NA / 2; u++) {
        const float2 dx = __fadd2_rn(px[u], cx), dy = __fadd2_rn(py[u], cy),
                     dz = __fadd2_rn(pz[u], cz);
        float2 r2 = __fmul2_rn(dx, dx);
        r2 = __ffma2_rn(dy, dy, r2);
        r2 = __ffma2_rn(dz, dz, r2);
        const uint32_t m0 = __ballot_sync(0xffffffffu, r2.x <= rc2b);
        const uint32_t m1 = __ballot_sync(0xffffffffu, r2.y <= rc2b);
        if (lane == 0) {
          s_mask[warp][2 * u][q] = m0;
          s_mask[warp][2 * u + 1][q] = m1;
        }
      }
    }
    __syncwarp();
    // the atom itself sits in every stencil entry of its own box (one entry
    // unless nbx < 3): clear those bits
    if (lane < na)
      for (int e = 0; e < ne; e++)
        if (s_box[e] == b) {
          const int c = s_off[e] + i0 + lane;
          s_mask[warp][lane][c >> 5] &= ~(1u << (c & 31));
        }
    __syncwarp();
    for (int t = 0; t < na; t++) {
      const uint32_t *ms = s_mask[warp][t];
      if (MODE != LIST_ID && A.box_start[b] + i0 + t >= A.ntot) break;  // only after an overflow
      const int row = (lane == 0) ? build_row<MODE>(A, b, i0 + t) : 0;
      const int a = __shfl_sync(0xffffffffu, row, 0);
      const int cap = build_cap<MODE>(A);
      // chunk words in candidate order: word w is held by lane w & 31 (w < 32
      // in `lo`, w >= 32 in `hi`); inclusive prefix of the hit counts
      const uint32_t lo = lane < nchunk ? ms[lane] : 0u;
      const uint32_t hi = lane + 32 < nchunk ? ms[lane + 32] : 0u;
      int xl = __popc(lo), xh = __popc(hi);
      for (int o = 1; o < 32; o <<= 1) {
        const int yl = __shfl_up_sync(0xffffffffu, xl, o);
        const int yh = __shfl_up_sync(0xffffffffu, xh, o);
        if (lane >= o) {
          xl += yl;
          xh += yh;
        }
      }
      const int tot_lo = __shfl_sync(0xffffffffu, xl, 31);
      const int total = tot_lo + __shfl_sync(0xffffffffu, xh, 31);
      // one hit per lane per round: find its word by binary search over the
      // prefix, then its bit with fns
      for (int h0 = 0; h0 < total; h0 += 32) {
        const int h = h0 + lane;
        const bool second = h >= tot_lo;
        const int hh = second ? h - tot_lo : h;
        int l = 0;
        for (int step = 16; step > 0; step >>= 1) {
          const int vl = __shfl_sync(0xffffffffu, xl, l + step - 1);
          const int vh = __shfl_sync(0xffffffffu, xh, l + step - 1);
          if ((second ? vh : vl) <= hh) l += step;
        }
        const int prev_l = __shfl_sync(0xffffffffu, xl, (l + 31) & 31);
        const int prev_h = __shfl_sync(0xffffffffu, xh, (l + 31) & 31);
        const uint32_t wl = __shfl_sync(0xffffffffu, lo, l);
        const uint32_t wh = __shfl_sync(0xffffffffu, hi, l);
        if (h < total && h < cap) {
          const int before = l ? (second ? prev_h : prev_l) : 0;
          const uint32_t word = second ? wh : wl;
          const unsigned bit = __fns(word, 0, hh - before + 1);
          const int c = ((second ? l + 32 : l) << 5) + (int)(bit & 31u);
          if (bit < 32u && c < (nchunk << 5))
            build_store<MODE>(A, a, h, __float_as_int(cand[c].w));
        }
      }
      if (lane == 0) build_count<MODE>(A, a, total);
    }
    __syncwarp();
  }
}

// NT threads per CTA, NA atoms tested per candidate load.  A grid-stride
// loop over the boxes, the grid sized to the resident CTAs: a launch with no
// rebuild due (most steps, with skin lists) costs one check per resident
// CTA instead of one CTA per box.
template <int MODE, int NT = NB_THREADS, int NA = NB_ATOMS>
static __global__ void __launch_bounds__(NT) nbr_build32_kernel(ForceArgs A, float rc2) {
  __shared__ __align__(16) float4 cand[NB_MAXC];
  __shared__ uint32_t s_mask[NT / 32][NA][NB_CHUNKS];
  __shared__ int s_box[CG_NNBR], s_off[CG_NNBR + 1], s_code[CG_NNBR];
  __shared__ BoxOff<float> s_dr[CG_NNBR];
  if (build_skipped<MODE>(A)) return;
  for (int b = blockIdx.x; b < A.g.nboxes; b += gridDim.x) {
    if (A.s.natoms[b] == 0) continue;
    build_box32<MODE, NT, NA>(A, rc2, b, cand, s_mask, s_box, s_off, s_code, s_dr);
    __syncthreads();  // the next box restages the shared arrays
  }
}

// FP64: the reference's dr = (drbox + r_i) - r_j, operation by operation
template <int MODE>
static __global__ void __launch_bounds__(NB_THREADS) nbr_build64_kernel(ForceArgs A, double rc2) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *cx = reinterpret_cast<double *>(smem_raw);
  double *cy = cx + NB_MAXC;
  double *cz = cy + NB_MAXC;
  uint16_t *cc = reinterpret_cast<uint16_t *>(cz + NB_MAXC);
  __shared__ int s_box[CG_NNBR], s_off[CG_NNBR + 1];
  __shared__ BoxOff<double> s_dr[CG_NNBR];
  if (build_skipped<MODE>(A)) return;
  const int b = blockIdx.x;
  const int ni = A.s.natoms[b];
  if (ni == 0) return;
  const int ne = stage_entries<double>(A, b, s_box, s_off, s_dr);
  const int ncand = s_off[ne];
  for (int c = threadIdx.x; c < ncand; c += NB_THREADS) {
    int e = entry_of(s_off, ne, c);
    int k = c - s_off[e];
    d4 q = A.s.r[s_box[e] * CG_MAXATOMS + k];
    cx[c] = q.x;
    cy[c] = q.y;
    cz[c] = q.z;
    cc[c] = (uint16_t)((e << 6) | k);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int i = warp; i < ni; i += NB_THREADS / 32) {
    double xi, yi, zi;
    PrecT<double>::pos(A.s, b * CG_MAXATOMS + i, xi, yi, zi);
    if (MODE != LIST_ID && A.box_start[b] + i >= A.ntot) break;  // only after an overflow
    const int row = (lane == 0) ? build_row<MODE>(A, b, i) : 0;
    const int a = __shfl_sync(0xffffffffu, row, 0);
    const int cap = build_cap<MODE>(A);
    int cnt = 0;
    for (int c0 = 0; c0 < ncand; c0 += 32) {
      const int c = c0 + lane;
      bool hit = false;
      uint16_t code = 0;
      if (c < ncand) {
        code = cc[c];
        int e = code >> 6, k = code & 63;
        double dx, dy, dz;
        double r2 = pair_r2(s_dr[e], xi, yi, zi, cx[c], cy[c], cz[c], dx, dy, dz);
        hit = (r2 <= rc2) && !(s_box[e] == b && k == i);
      }
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      const int pos = cnt + __popc(m & lt);
      if (hit && pos < cap)
        build_store<MODE>(A, a, pos,
                             MODE == LIST_ID ? A.s.id[s_box[code >> 6] * CG_MAXATOMS + (code & 63)]
                                     : (int)code);
      cnt += __popc(m);
    }
    if (lane == 0) build_count<MODE>(A, a, cnt);
  }
}

// ---------------------------------------------------------------------------
// EAM pass 1 (+ embedding): phi, phi', rho per pair; F, F' per atom
// ---------------------------------------------------------------------------
template <class T, int EVAL>
struct EamPot {
  Table<T> phi, rho, f;
  Cheb<T> ch;
  ChebLow32 chlo;  // FP32 only
  PairSeg seg;     // FP32 Chebyshev only
  T rc2;
};

template <int EVAL>
__device__ __forceinline__ double cheb_series(const EamPot<double, EVAL> &P, int s, double x) {
  return cheb_eval64(P.ch.c[s], P.ch.a[s], P.ch.b[s], x);
}
// the reference coefficients for arguments below the re-expansion interval
// (never taken in practice; kept out of line so it costs no code in the loop)
static __device__ __noinline__ float cheb_low32(const ChebLow32 &L, int s, float x) {
  return cheb_eval32(L.c[s], L.a[s], L.ys[s], L.yo[s], x);
}

template <int EVAL>
__device__ __forceinline__ float cheb_series(const EamPot<float, EVAL> &P, int s, float x) {
  if (x >= P.chlo.lo[s]) return cheb_eval32(P.ch.c[s], P.ch.a[s], P.ch.ys[s], P.ch.yo[s], x);
  return cheb_low32(P.chlo, s, x);
}

// r and 1/r from r^2: FP64 as the reference (sqrt, then divide); FP32 from
// rsqrt refined by one Newton step (about 1 ulp)
__device__ __forceinline__ void r_and_inv(double r2, double &r, double &inv) {
  r = sqrt(r2);
  inv = 1.0 / r;
}
__device__ __forceinline__ void r_and_inv(float r2, float &r, float &inv) {
  float y = rsqrtf(r2);
  y = y * fmaf(-0.5f * r2, y * y, 1.5f);
  inv = y;
  r = r2 * y;
}

// phi, phi' and rho of one pair distance from the FP32 series: the three
// re-expanded series share the interval [lo, rc] and so one T_k recurrence
template <int EVAL>
__device__ __forceinline__ void cheb_pair32(const EamPot<float, EVAL> &P, float r, float &phi,
                                            float &dphi, float &rho) {
  if (P.chlo.pair_shared && r >= P.chlo.lo[0]) {
    cheb3_eval32(P.ch.c[0], P.ch.c[3], P.ch.c[1], P.ch.a[0], P.ch.ys[0], P.ch.yo[0], r, phi,
                 dphi, rho);
  } else if (!P.chlo.pair_shared) {
    phi = cheb_series(P, 0, r);
    dphi = cheb_series(P, 3, r);
    rho = cheb_series(P, 1, r);
  } else {
    phi = cheb_low32(P.chlo, 0, r);
    dphi = cheb_low32(P.chlo, 3, r);
    rho = cheb_low32(P.chlo, 1, r);
  }
}
template <int EVAL>
__device__ __forceinline__ void cheb_pair32(const EamPot<double, EVAL> &, double, double &,
                                            double &, double &) {}

template <class T, int EVAL>
__device__ __forceinline__ void eam_pair_terms(const EamPot<T, EVAL> &P, T r, T &phi, T &dphi,
                                               T &rho) {
  if (EVAL == EVAL_CHEBY && sizeof(T) == 4) {
    cheb_pair32(P, r, phi, dphi, rho);
  } else if (EVAL == EVAL_CHEBY) {
    phi = cheb_series(P, 0, r);
    dphi = cheb_series(P, 3, r);
    rho = cheb_series(P, 1, r);
  } else {
    T drho;
    table_eval(P.phi, r, phi, dphi);
    table_eval(P.rho, r, rho, drho);
  }
}

template <class T, int EVAL>
__device__ __forceinline__ void eam_embed(const EamPot<T, EVAL> &P, T rho, T &F, T &dF) {
  if (EVAL == EVAL_CHEBY) {
    F = cheb_series(P, 2, rho);
    dF = cheb_series(P, 5, rho);
  } else {
    table_eval(P.f, rho, F, dF);
  }
}

template <class T, int EVAL>
__device__ __forceinline__ T eam_drho(const EamPot<T, EVAL> &P, T r) {
  if (EVAL == EVAL_CHEBY) return cheb_series(P, 4, r);
  T v, d;
  table_eval(P.rho, r, v, d);
  return d;
}

// Pair terms of one distance: phi, w = phi'(r)/r and rho.  The FP32
// Chebyshev path reads them from the segment table in shared memory (sm)
// and returns false for a distance below the table (or with no table): the
// caller then takes that pair from the series in a second, rare sweep, so
// the pair loop itself holds no call.
template <class T, int EVAL>
__device__ __forceinline__ bool eam_pair_w(const EamPot<T, EVAL> &P, const float4 *, T r2,
                                           T &phi, T &w, T &rho) {
  T r, inv_r, dphi;
  r_and_inv(r2, r, inv_r);
  eam_pair_terms<T, EVAL>(P, r, phi, dphi, rho);
  w = dphi * inv_r;
  return true;
}
static __device__ __forceinline__ bool eam_pair_w(const EamPot<float, EVAL_CHEBY> &P,
                                                  const float4 *sm, float r2, float &phi,
                                                  float &w, float &rho) {
  const float u = (r2 - P.seg.s_lo) * P.seg.inv_h;
  if (!(u >= 0.f)) return false;
  const int k = min((int)u, P.seg.n - 1);
  const float t = u - (float)k;
  const float4 cp = sm[k], cr = sm[P.seg.n + k];
  phi = seg_cubic(cp, t);
  w = P.seg.dscale * seg_dcubic(cp, t);
  rho = seg_cubic(cr, t);
  return true;
}
// the series for a pair below the table (FP32 Chebyshev only)
template <class T, int EVAL>
__device__ __forceinline__ void pair_w_series(const EamPot<T, EVAL> &, T, T &, T &, T &) {}
static __device__ __noinline__ void pair_w_series(const EamPot<float, EVAL_CHEBY> &P, float r2,
                                                  float &phi, float &w, float &rho) {
  float r, inv_r, dphi;
  r_and_inv(r2, r, inv_r);
  cheb_pair32(P, r, phi, dphi, rho);
  w = dphi * inv_r;
}
template <class T, int EVAL>
__device__ __forceinline__ bool below_seg(const EamPot<T, EVAL> &, T) {
  return false;
}
static __device__ __forceinline__ bool below_seg(const EamPot<float, EVAL_CHEBY> &P, float r2) {
  return !((r2 - P.seg.s_lo) * P.seg.inv_h >= 0.f);
}

// wr = (F'_i + F'_j) rho'(r) / r for one pair (fsum = F'_i + F'_j); the FP32
// Chebyshev path reads rho's cubic (sm holds the rho half of the table).
// false: below the table, as eam_pair_w.
template <class T, int EVAL>
__device__ __forceinline__ bool eam_embed_w(const EamPot<T, EVAL> &P, const float4 *, T r2,
                                            T fsum, T &wr) {
  T r, inv_r;
  r_and_inv(r2, r, inv_r);
  wr = fsum * eam_drho<T, EVAL>(P, r) * inv_r;
  return true;
}
static __device__ __forceinline__ bool eam_embed_w(const EamPot<float, EVAL_CHEBY> &P,
                                                   const float4 *sm, float r2, float fsum,
                                                   float &wr) {
  const float u = (r2 - P.seg.s_lo) * P.seg.inv_h;
  if (!(u >= 0.f)) return false;
  const int k = min((int)u, P.seg.n - 1);
  wr = fsum * (P.seg.dscale * seg_dcubic(sm[k], u - (float)k));
  return true;
}
template <class T, int EVAL>
__device__ __forceinline__ T embed_w_series(const EamPot<T, EVAL> &, T, T) {
  return T(0);
}
static __device__ __noinline__ float embed_w_series(const EamPot<float, EVAL_CHEBY> &P, float r2,
                                                    float fsum) {
  float r, inv_r;
  r_and_inv(r2, r, inv_r);
  return fsum * (cheb_series(P, 4, r) * inv_r);
}

template <class T, int EVAL>
__device__ __forceinline__ bool uses_seg(const EamPot<T, EVAL> &P) {
  return sizeof(T) == 4 && EVAL == EVAL_CHEBY && P.seg.n > 0;
}

// the segment table (nrec float4 from src) into shared memory, once per CTA
__device__ __forceinline__ void stage_seg(float4 *sm, const float4 *src, int nrec) {
  for (int q = threadIdx.x; q < nrec; q += blockDim.x) sm[q] = __ldg(src + q);
  __syncthreads();
}

// the density pass's rho table (nrec cubics from src) as RHO_COPIES
// interleaved copies: record q of the shared array is segment q / RHO_COPIES
__device__ __forceinline__ void stage_rho_copies(float4 *sm, const float4 *src, int nrec) {
  for (int q = threadIdx.x; q < nrec * RHO_COPIES; q += blockDim.x)
    sm[q] = __ldg(src + q / RHO_COPIES);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// EAM pass 1: density, pair energy and pair force of one atom.  `visit`
// runs the atom's neighbour traversal with a pair functor.
// ---------------------------------------------------------------------------
template <class T>
struct Pass1Acc {
  typename PrecT<T>::Acc fx, fy, fz, ep, rh;
  int cnt;
  __device__ __forceinline__ void zero() {
    fx.zero(); fy.zero(); fz.zero(); ep.zero(); rh.zero();
    cnt = 0;
  }
  __device__ __forceinline__ void add(T phi, T w, T rho, T dx, T dy, T dz) {
    fx.add(w * dx);
    fy.add(w * dy);
    fz.add(w * dz);
    ep.add(phi / T(2.0));
    rh.add(rho);
  }
};

template <class T, int EVAL, class V>
__device__ __forceinline__ void eam_pass1_sum(const EamPot<T, EVAL> &P, const float4 *sm,
                                              Pass1Acc<T> &acc, V &&visit) {
  const T rc2 = P.rc2;
  bool low = false;
  visit([&](T, T dx, T dy, T dz, T r2) {
    if (r2 > rc2) return;
    acc.cnt++;
    T phi, w, rho;
    if (!eam_pair_w(P, sm, r2, phi, w, rho)) {
      low = true;
      return;
    }
    acc.add(phi, w, rho, dx, dy, dz);
  });
  if (low)  // pairs below the table: the series, in a second sweep
    visit([&](T, T dx, T dy, T dz, T r2) {
      if (r2 > rc2 || !below_seg(P, r2)) return;
      T phi, w, rho;
      pair_w_series(P, r2, phi, w, rho);
      acc.add(phi, w, rho, dx, dy, dz);
    });
}

// per-atom results of pass 1: F and F' fused in (eam.c:576-594)
template <class T, int EVAL>
__device__ __forceinline__ float eam_pass1_store(const ForceArgs &A, const EamPot<T, EVAL> &P,
                                                 Pass1Acc<T> &acc, int slot) {
  double rho_i = acc.rh.value();
  T F, dF;
  eam_embed<T, EVAL>(P, (T)rho_i, F, dF);
  d4 fo;
  fo.x = acc.fx.value();
  fo.y = acc.fy.value();
  fo.z = acc.fz.value();
  fo.w = acc.ep.value() + (double)F;
  A.s.f[slot] = fo;
  A.s.rho[slot] = rho_i;
  A.s.fi[slot] = (double)dF;
  if (sizeof(T) == 4) A.s.fi32[slot] = (float)dF;
  return (float)dF;
}

// grid-stride over the compact atoms; the grid is sized to the resident CTAs
// so each CTA stages the segment table once
template <class T, int EVAL>
__global__ void __launch_bounds__(PASS_THREADS)
    eam_pass1_kernel(ForceArgs A, const __grid_constant__ EamPot<T, EVAL> P) {
  extern __shared__ float4 seg_sm[];
  if (uses_seg(P)) stage_seg(seg_sm, P.seg.p1, 2 * P.seg.n);
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.atom_slot[a];
    const int b = slot >> 6, i = slot & 63;
    T xi, yi, zi;
    PrecT<T>::pos(A.s, slot, xi, yi, zi);
    Pass1Acc<T> acc;
    acc.zero();
    eam_pass1_sum(P, seg_sm, acc, [&](auto &&fn) {
      for_each_neighbor<T, false, true>(A, a, b, i, xi, yi, zi, P.rc2,
                                        [&](int, T dx, T dy, T dz, T r2) { fn(T(0), dx, dy, dz, r2); });
    });
    eam_pass1_store(A, P, acc, slot);
  }
}

// ---------------------------------------------------------------------------
// EAM pass 2: embedding force and stress
// ---------------------------------------------------------------------------
template <class T>
struct Pass2Acc {
  typename PrecT<T>::Acc fx, fy, fz, sx;
  __device__ __forceinline__ void zero() { fx.zero(); fy.zero(); fz.zero(); sx.zero(); }
  __device__ __forceinline__ void add(T wr, T dx, T dy, T dz) {
    fx.add(wr * dx);
    fy.add(wr * dy);
    fz.add(wr * dz);
    sx.add(wr * dx * dx);
  }
};

// visit(fn) calls fn(F'_j, dx, dy, dz, r2) per neighbour
template <class T, int EVAL, class V>
__device__ __forceinline__ void eam_pass2_sum(const EamPot<T, EVAL> &P, const float4 *sm, T fii,
                                              Pass2Acc<T> &acc, V &&visit) {
  const T rc2 = P.rc2;
  bool low = false;
  visit([&](T fj, T dx, T dy, T dz, T r2) {
    if (r2 >= rc2) return;
    T wr;
    if (!eam_embed_w(P, sm, r2, fii + fj, wr)) {
      low = true;
      return;
    }
    acc.add(wr, dx, dy, dz);
  });
  if (low)
    visit([&](T fj, T dx, T dy, T dz, T r2) {
      if (r2 >= rc2 || !below_seg(P, r2)) return;
      acc.add(embed_w_series(P, r2, fii + fj), dx, dy, dz);
    });
}

template <class T>
__device__ __forceinline__ void eam_pass2_store(const ForceArgs &A, Pass2Acc<T> &acc, int slot,
                                                int a) {
  d4 fo = A.s.f[slot];
  fo.x += acc.fx.value();
  fo.y += acc.fy.value();
  fo.z += acc.fz.value();
  A.s.f[slot] = fo;
  A.atom_stress[a] = acc.sx.value();
}

template <class T, int EVAL>
__global__ void __launch_bounds__(PASS_THREADS)
    eam_pass2_kernel(ForceArgs A, const __grid_constant__ EamPot<T, EVAL> P) {
  extern __shared__ float4 seg_sm[];
  if (uses_seg(P)) stage_seg(seg_sm, P.seg.p1 + P.seg.n, P.seg.n);
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.atom_slot[a];
    const int b = slot >> 6, i = slot & 63;
    T xi, yi, zi;
    PrecT<T>::pos(A.s, slot, xi, yi, zi);
    Pass2Acc<T> acc;
    acc.zero();
    eam_pass2_sum(P, seg_sm, PrecT<T>::fi(A.s, slot), acc, [&](auto &&fn) {
      for_each_neighbor<T, true>(A, a, b, i, xi, yi, zi, P.rc2,
                                 [&](int js, T dx, T dy, T dz, T r2) {
                                   fn(PrecT<T>::fi(A.s, js), dx, dy, dz, r2);
                                 });
    });
    eam_pass2_store(A, acc, slot, a);
  }
}

// ---------------------------------------------------------------------------
// Force-order passes (mixed precision, persistent lists)
// ---------------------------------------------------------------------------
constexpr int FO1_THREADS = 512;  // pass 1 (density): 2 CTAs of 64 registers per SM

// list lines fetched ahead, unroll of the list walk and pass 2's register
// cap (chosen by measurement; -D overrides for sweeps).  Pass 2 (the force
// pass, five compensated sums) runs with CTAs of 128 to 512 threads; its
// register count follows the cap, not the CTA size.
#ifndef COMDGB_FO_PREFETCH
#define COMDGB_FO_PREFETCH 4
#endif
#ifndef COMDGB_FO1_UNROLL
#define COMDGB_FO1_UNROLL 4  // pass 1 (and LJ)
#endif
#ifndef COMDGB_FO2_UNROLL
#define COMDGB_FO2_UNROLL 2  // pass 2
#endif
#ifndef COMDGB_FO2F_MAXNREG  // the force pass without energies (OBS = false)
#define COMDGB_FO2F_MAXNREG 64
#endif
#ifndef COMDGB_FO2_MAXNREG
#define COMDGB_FO2_MAXNREG 64
#endif
// 1: the density pass writes the entries within the cutoff (the cut list)
// and the force pass walks them; 0: the force pass walks the skin list
#ifndef COMDGB_FO_CUT
#define COMDGB_FO_CUT 1
#endif
constexpr int FO_PREFETCH = COMDGB_FO_PREFETCH;
constexpr int FO1_UNROLL = COMDGB_FO1_UNROLL, FO2_UNROLL = COMDGB_FO2_UNROLL;

__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// The box sizes of the pair offsets of force-order atom `slot`'s replica:
// FP32 hi + lo, the y and z ones pre-scaled by 1/4 and 1/16 (their code
// fields are read in place, x 4 and x 16, exactly).  MULTI: a batch of
// replicas (the box size comes from the atom's replica); else replica 0's
// sizes are kernel-parameter constants (no registers held).
struct FoFrame {
  float hx, hy, hz, lx, ly, lz;
};
template <bool MULTI>
__device__ __forceinline__ FoFrame fo_frame(const ForceArgs &A, int slot) {
  FoFrame f{A.g.hi0[0], A.g.hi0[1], A.g.hi0[2], A.g.lo0[0], A.g.lo0[1], A.g.lo0[2]};
  if (MULTI) {
    const RepGeo &R = rep_of(A.g, slot >> 6);
    f = FoFrame{R.hi[0], R.hi[1], R.hi[2], R.lo[0], R.lo[1], R.lo[2]};
  }
  f.hy *= 0.25f, f.ly *= 0.25f, f.hz *= 0.0625f, f.lz *= 0.0625f;
  return f;
}

// dr of list entry p = j << 6 | (dz+1) << 4 | (dy+1) << 2 | (dx+1) between
// the atom at pi and its neighbour at q: (pi - q) - d * boxsize.  A field
// f * 2^s in place, OR-ed into the bits of 2^23, is the float 2^23 + f *
// 2^s: subtracted from 2^23 + 2^s it gives -d * 2^s exactly.
__device__ __forceinline__ float fo_dr(const FoFrame &f, uint32_t p, float4 pi, float4 q,
                                       float &dx, float &dy, float &dz) {
  const float ex = 8388609.0f - __int_as_float(0x4B000000 | (int)(p & 0x3u));
  const float ey = 8388612.0f - __int_as_float(0x4B000000 | (int)(p & 0xCu));
  const float ez = 8388624.0f - __int_as_float(0x4B000000 | (int)(p & 0x30u));
  dx = fmaf(ex, f.lx, fmaf(ex, f.hx, pi.x - q.x));
  dy = fmaf(ey, f.ly, fmaf(ey, f.hy, pi.y - q.y));
  dz = fmaf(ez, f.lz, fmaf(ez, f.hz, pi.z - q.z));
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// the transposed row of force-order atom a in a list of capacity vcap
__device__ __forceinline__ size_t fo_row(int a, int vcap) {
  return (size_t)(a >> 5) * vcap * 32 + (a & 31);
}

// Visit n entries of the list `lst` (a force-order list: skin or cut) of
// force-order atom a at FP32 position pi: fn(fj, dx, dy, dz, r2) for every
// entry; with NEED_FI positions come from fo.pf and fj is F'(rho_j) (its w),
// else fj is unspecified.  n > vcap (the skin list overflowed): the stencil
// of the atom's current slot is scanned instead.
template <bool NEED_FI, bool MULTI, int UNROLL, class F>
__device__ __forceinline__ void fo_walk(const ForceArgs &A, const uint32_t *list, int n, int a,
                                        int slot, float4 pi, float rc2, F &&fn) {
  if (n > A.fo.vcap) {
    const float4 p = __ldg(A.s.pos32 + slot);
    scan_stencil<float>(A, slot >> 6, slot & 63, p.x, p.y, p.z, rc2,
                        [&](int js, float dx, float dy, float dz, float r2) {
                          fn(NEED_FI ? __ldg(A.s.fi32 + js) : 0.f, dx, dy, dz, r2);
                        });
    return;
  }
  const FoFrame fr = fo_frame<MULTI>(A, slot);
  const uint32_t *lst = list + fo_row(a, A.fo.vcap);
  const float4 *pj = NEED_FI ? A.fo.pf : A.fo.pos;
  // the warp's list lines stream from HBM: pull line t + FO_PREFETCH into L1
  // while line t is used (within this atom's list only)
#pragma unroll UNROLL
  for (int t = 0; t < n; t++) {
    if (t + FO_PREFETCH < n) prefetch_l1(lst + (size_t)(t + FO_PREFETCH) * 32);
    const uint32_t p = __ldg(lst + (size_t)t * 32);
    const float4 q = __ldg(pj + (p >> 6));
    float dx, dy, dz;
    const float r2 = fo_dr(fr, p, pi, q, dx, dy, dz);
    fn(q.w, dx, dy, dz, r2);
  }
}

// the skin list of force-order atom a
template <bool NEED_FI, bool MULTI, int UNROLL = FO2_UNROLL, class F>
__device__ __forceinline__ void fo_for_each(const ForceArgs &A, int a, int slot, float4 pi,
                                            float rc2, F &&fn) {
  fo_walk<NEED_FI, MULTI, UNROLL>(A, A.fo.list, A.fo.n[a], a, slot, pi, rc2, fn);
}

// ---------------------------------------------------------------------------
// Force-order EAM (mixed precision, persistent lists): the density pass with
// the embedding fused in, then the force pass.  The reference's pass 1
// (eam.c:484-549) computes phi, phi' and rho per pair and pass 3
// (eam.c:595-653) rho'; here the density pass needs rho alone, and the
// force pass takes phi (the pair energy), phi' and rho' together, so every
// per-atom force component is one compensated sum.  The pass criteria stay
// the reference's: phi, phi' and rho for r^2 <= rc^2, the embedding force
// and stress for r^2 < rc^2.
// ---------------------------------------------------------------------------

// rho(r) of one pair distance: the rho cubics of the FP32 pair table (sm),
// or the table evaluator.  false: below the pair table (the series, in a
// second sweep)
template <int EVAL>
__device__ __forceinline__ bool fo_rho(const EamPot<float, EVAL> &P, const float4 *, float r2,
                                       float &rho) {
  float r, inv_r, v, d;
  r_and_inv(r2, r, inv_r);
  if (EVAL == EVAL_CHEBY) {
    rho = cheb_series(P, 1, r);
  } else {
    table_eval(P.rho, r, v, d);
    rho = v;
  }
  return true;
}
// (sm: this lane's copy of the density pass's rho table, n1 segments
// RHO_COPIES records apart; the same lower end s_lo, so "below the table"
// is below_seg's test)
static __device__ __forceinline__ bool fo_rho(const EamPot<float, EVAL_CHEBY> &P,
                                              const float4 *sm, float r2, float &rho) {
  const float u = (r2 - P.seg.s_lo) * P.seg.inv_h1;
  if (!(u >= 0.f)) return false;
  const int k = min((int)u, P.seg.n1 - 1);
  rho = seg_cubic(sm[k * RHO_COPIES], u - (float)k);
  return true;
}
template <int EVAL>
__device__ __forceinline__ float fo_rho_series(const EamPot<float, EVAL> &, float) {
  return 0.f;
}
static __device__ __noinline__ float fo_rho_series(const EamPot<float, EVAL_CHEBY> &P, float r2) {
  float r, inv_r;
  r_and_inv(r2, r, inv_r);
  return cheb_series(P, 1, r);
}

// phi (OBS only), phi'(r)/r and rho'(r)/r of one pair distance: the force
// pass's tables (staged by stage_force_table: sm this lane's copy of the
// derivative cubics, phi_sm the phi cubics), or the table evaluator.
// false: below the pair table
template <bool OBS, int EVAL>
__device__ __forceinline__ bool fo_pair(const EamPot<float, EVAL> &P, const float4 *,
                                        const float4 *, float r2, float &phi, float &wphi,
                                        float &wrho) {
  float r, inv_r, dphi, v, drho;
  r_and_inv(r2, r, inv_r);
  if (EVAL == EVAL_CHEBY) {
    phi = cheb_series(P, 0, r);
    dphi = cheb_series(P, 3, r);
    drho = cheb_series(P, 4, r);
  } else {
    table_eval(P.phi, r, phi, dphi);
    table_eval(P.rho, r, v, drho);
  }
  wphi = dphi * inv_r;
  wrho = drho * inv_r;
  return true;
}
// (two conflict-free 16-byte shared loads per pair, the phi cubic a third
// only when the energy is summed)
template <bool OBS>
static __device__ __forceinline__ bool fo_pair(const EamPot<float, EVAL_CHEBY> &P,
                                               const float4 *sm, const float4 *phi_sm, float r2,
                                               float &phi, float &wphi, float &wrho) {
  const float d = r2 - P.seg.s_lo;
  float u = d * P.seg.inv_h2;
  if (!(u >= 0.f)) return false;
  if (COMDGB_SEG2_RUNS > 1 && u >= (float)P.seg.n2a)
    u = fmaf(r2 - P.seg.s2b, P.seg.inv_h2b, (float)P.seg.n2a);
  const int k = min((int)u, P.seg.n2 - 1);
  const float t = u - (float)k;
  wphi = seg_cubic(sm[(2 * k) * FORCE_COPIES], t);
  wrho = seg_cubic(sm[(2 * k + 1) * FORCE_COPIES], t);
  if (OBS) {
    const float u1 = d * P.seg.inv_h;
    const int k1 = min((int)u1, P.seg.n - 1);
    phi = seg_cubic(phi_sm[k1], u1 - (float)k1);
  }
  return true;
}

// the force pass's tables into shared memory, once per CTA: FORCE_COPIES
// interleaved copies of the derivative cubics (2 n2 records each), then
// with OBS the phi cubics (n records)
template <bool OBS>
__device__ __forceinline__ void stage_force_table(float4 *sm, const PairSeg &S) {
  const int m = 2 * S.n2 * FORCE_COPIES;
  for (int q = threadIdx.x; q < m; q += blockDim.x) sm[q] = __ldg(S.dcub + q / FORCE_COPIES);
  if (OBS)
    for (int q = threadIdx.x; q < S.n; q += blockDim.x) sm[m + q] = __ldg(S.p1 + q);
  __syncthreads();
}
// the series for a pair below the table (FP32 Chebyshev only)
template <int EVAL>
__device__ __forceinline__ void fo_pair_series(const EamPot<float, EVAL> &, float, float &,
                                               float &, float &) {}
static __device__ __noinline__ void fo_pair_series(const EamPot<float, EVAL_CHEBY> &P, float r2,
                                                   float &phi, float &wphi, float &wrho) {
  float r, inv_r, dphi, rho;
  r_and_inv(r2, r, inv_r);
  cheb_pair32(P, r, phi, dphi, rho);
  wphi = dphi * inv_r;
  wrho = cheb_series(P, 4, r) * inv_r;
}

// per-atom results of the density pass: F and F' fused in (eam.c:576-594)
template <int EVAL, bool OBS>
__device__ __forceinline__ void fo_density_store(const ForceArgs &A,
                                                 const EamPot<float, EVAL> &P, const KSum &rh,
                                                 int a, int slot, float4 pi, int cnt, int ncut) {
  const double rho_i = rh.value();
  float F, dF;
  eam_embed<float, EVAL>(P, (float)rho_i, F, dF);
  if (OBS) {  // the host-visible rho, F' and the embedding energy
    A.s.rho[slot] = rho_i;
    A.s.fi[slot] = (double)dF;
    A.fo.emb[a] = F;
    if (A.host_rho) {
      A.host_rho[slot] = rho_i;
      A.host_fi[slot] = (double)dF;
    }
  }
  A.s.fi32[slot] = dF;
  A.fo.pf[a] = make_float4(pi.x, pi.y, pi.z, dF);
  A.fo.ncut[a] = ncut;
  A.nbr_n[a] = cnt;
}

#ifdef COMDGB_FO1_MAXNREG  // sweep variant: a register cap instead of the launch bound
#define FO1_BOUNDS __maxnreg__(COMDGB_FO1_MAXNREG)
#else
#define FO1_BOUNDS __launch_bounds__(FO1_THREADS, 2)
#endif

// Density pass: rho_i = sum of rho(r_ij) over the skin list within the
// cutoff, F(rho_i) and F'(rho_i); the entries within the cutoff are written
// to the cut list for the force pass.  OBS: a force call whose results the
// caller can read (see the force pass); otherwise only what the force pass
// needs is stored.
template <int EVAL, bool MULTI, bool OBS>
__global__ void FO1_BOUNDS
    fo_eam_pass1_kernel(ForceArgs A, const __grid_constant__ EamPot<float, EVAL> P) {
  extern __shared__ float4 seg_sm[];
  if (uses_seg(P)) stage_rho_copies(seg_sm, P.seg.rho1, P.seg.n1);  // the rho cubics
  const float4 *rho_sm = seg_sm + (threadIdx.x & (RHO_COPIES - 1));  // this lane's copy
  const float rc2 = P.rc2;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.fo.slot[a];
    const float4 pi = A.fo.pos[a];
    const int n = A.fo.n[a];
    KSum rh;
    rh.zero();
    int cnt = 0;
    if (n > A.fo.vcap) {  // overflowed skin list: the stencil, no cut list
      fo_walk<false, MULTI, 1>(A, A.fo.list, n, a, slot, pi, rc2,
                               [&](float, float, float, float, float r2) {
                                 if (r2 > rc2) return;
                                 cnt++;
                                 float rho;
                                 if (!fo_rho(P, rho_sm, r2, rho)) rho = fo_rho_series(P, r2);
                                 rh.add(rho);
                               });
      fo_density_store<EVAL, OBS>(A, P, rh, a, slot, pi, cnt, A.fo.vcap + 1);
      continue;
    }
    const FoFrame fr = fo_frame<MULTI>(A, slot);
    const size_t row = fo_row(a, A.fo.vcap);
    const uint32_t *lst = A.fo.list + row;
    uint32_t *cut = A.fo.cut + row;
    bool low = false;
#pragma unroll FO1_UNROLL
    for (int t = 0; t < n; t++) {
      if (t + FO_PREFETCH < n) prefetch_l1(lst + (size_t)(t + FO_PREFETCH) * 32);
      const uint32_t p = __ldg(lst + (size_t)t * 32);
      const float4 q = __ldg(A.fo.pos + (p >> 6));
      float dx, dy, dz;
      const float r2 = fo_dr(fr, p, pi, q, dx, dy, dz);
      if (r2 > rc2) continue;
      if (COMDGB_FO_CUT) cut[(size_t)cnt * 32] = p;
      cnt++;
      float rho;
      if (fo_rho(P, rho_sm, r2, rho)) rh.add(rho);
      else low = true;
    }
    if (low)  // pairs below the table: the series, in a second sweep
      fo_walk<false, MULTI, 1>(A, A.fo.list, n, a, slot, pi, rc2,
                               [&](float, float, float, float, float r2) {
                                 if (r2 <= rc2 && below_seg(P, r2)) rh.add(fo_rho_series(P, r2));
                               });
    fo_density_store<EVAL, OBS>(A, P, rh, a, slot, pi, cnt, cnt);
  }
}

// force pass: the per-atom sums
// (OBS: also the pair energy and the embedding stress)
template <bool OBS>
struct ForceSums {
  KSum fx, fy, fz, ep, sx;
  __device__ __forceinline__ void zero() {
    fx.zero(); fy.zero(); fz.zero();
    if (OBS) {
      ep.zero();
      sx.zero();
    }
  }
  // phi and w = phi'/r for r^2 <= rc^2; we = (F'_i + F'_j) rho'/r, zero
  // unless r^2 < rc^2
  __device__ __forceinline__ void add(float phi, float wphi, float we, float dx, float dy,
                                      float dz) {
    const float w = wphi + we;
    fx.add(w * dx);
    fy.add(w * dy);
    fz.add(w * dz);
    if (OBS) {
      ep.add(phi);
      sx.add(we * dx * dx);
    }
  }
};

constexpr int FO2_MAX_THREADS = 512;  // the force pass runs with 128, 256 (default) or 512

// the force of slot into the attached host array (real4 per slot)
__device__ __forceinline__ void fo_host_f(const ForceArgs &A, int slot, const d4 &f) {
  double *h = A.host_f + 4 * (size_t)slot;
  h[0] = f.x;
  h[1] = f.y;
  h[2] = f.z;
  h[3] = f.w;
}

// The end of a force-order force call inside a step sequence: with ST_FUSE
// set (fuse), atom a's velocity step with the force just summed and the two
// position half steps around the step boundary, as one multiply-add each
// (the arithmetic of the mixed-precision middle-part update), and its
// tracking record; else its FP32 force record for the velocity step that
// follows.  Safe inside the pass: the other atoms of the pass read the
// positions the density pass stored (pf), never r, p, fo.pos or pos32.
__device__ __forceinline__ void fo_force_end(const ForceArgs &A, int a, int slot, bool fuse,
                                             float fx, float fy, float fz) {
  if (!fuse) {
    A.fo.force[a] = make_float4(fx, fy, fz, 0.f);
    return;
  }
  d4 p = A.s.p[slot];
  p.x = fma(-A.vv_dt, (double)fx, p.x);
  p.y = fma(-A.vv_dt, (double)fy, p.y);
  p.z = fma(-A.vv_dt, (double)fz, p.z);
  A.s.p[slot] = p;
  d4 r = A.s.r[slot];
  r.x = fma(p.x, A.vv_c, r.x);
  r.y = fma(p.y, A.vv_c, r.y);
  r.z = fma(p.z, A.vv_c, r.z);
  A.s.r[slot] = r;
  const int b = slot >> 6;
  fo_track_at(A.g, A.fo, b, a, r, centred32(rep_of(A.g, b), r.x, r.y, r.z), A.status);
}

// Force pass: f_i = sum over the cut list of (phi'(r) + (F'_i + F'_j)
// rho'(r)) dr/r, the per-atom energy 1/2 sum phi + F(rho_i) and the
// embedding x-x stress (eam.c:534-545, 644-649; f is +grad U as in the
// reference).
// Every force call ends with fo_force_end: the FP32 force record in force
// order, or inside a step sequence (ST_FUSE) the next step's velocity and
// position update made right here.  OBS: also the slot arrays' f with the
// per-atom energy, and the stress -- a force call whose results the caller
// can read (a force call, the one ending nTimeSteps).  The force calls
// inside a step sequence are not OBS: the next force call overwrites their
// energies and stress before anything can read them (the reference's
// nTimeSteps ends with its own computeForce, timestep.c:137).
template <int EVAL, bool MULTI, bool OBS>
__global__ void __maxnreg__(OBS ? COMDGB_FO2_MAXNREG : COMDGB_FO2F_MAXNREG)
    fo_eam_pass2_kernel(ForceArgs A, const __grid_constant__ EamPot<float, EVAL> P) {
  extern __shared__ float4 seg_sm[];
  if (uses_seg(P)) stage_force_table<OBS>(seg_sm, P.seg);
  const float4 *dcub_sm = seg_sm + (threadIdx.x & (FORCE_COPIES - 1));  // this lane's copy
  const float4 *phi_sm = seg_sm + 2 * SEG2_N * FORCE_COPIES;
  const float rc2 = P.rc2;
  const bool fuse = !OBS && *(volatile const int *)(A.status + ST_FUSE);
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.fo.slot[a];
    const float4 pi = A.fo.pf[a];
    const float fii = pi.w;
    const int n = COMDGB_FO_CUT ? A.fo.ncut[a] : A.fo.n[a];
    ForceSums<OBS> acc;
    acc.zero();
    bool low = false;
    auto walk = [&](auto &&fn) {
      fo_walk<true, MULTI, FO2_UNROLL>(A, COMDGB_FO_CUT ? A.fo.cut : A.fo.list, n, a, slot, pi,
                                       rc2, fn);
    };
    walk([&](float fj, float dx, float dy, float dz, float r2) {
      if (r2 > rc2) return;
      float phi, wphi, wrho;
      if (!fo_pair<OBS>(P, dcub_sm, phi_sm, r2, phi, wphi, wrho)) {
        low = true;
        return;
      }
      const float we = r2 < rc2 ? (fii + fj) * wrho : 0.f;
      acc.add(phi, wphi, we, dx, dy, dz);
    });
    if (low)  // pairs below the table: the series, in a second sweep
      walk([&](float fj, float dx, float dy, float dz, float r2) {
        if (r2 > rc2 || !below_seg(P, r2)) return;
        float phi, wphi, wrho;
        fo_pair_series(P, r2, phi, wphi, wrho);
        const float we = r2 < rc2 ? (fii + fj) * wrho : 0.f;
        acc.add(phi, wphi, we, dx, dy, dz);
      });
    const float fx = acc.fx.valuef(), fy = acc.fy.valuef(), fz = acc.fz.valuef();
    fo_force_end(A, a, slot, fuse, fx, fy, fz);
    if (OBS) {
      d4 fo;
      fo.x = fx;
      fo.y = fy;
      fo.z = fz;
      fo.w = 0.5 * acc.ep.value() + (double)__ldg(A.fo.emb + a);
      A.s.f[slot] = fo;
      A.atom_stress[a] = acc.sx.value();
      if (A.host_f) fo_host_f(A, slot, fo);
    }
  }
}

// ---------------------------------------------------------------------------
// LJ: ljForce.c:151-215 as full pairs; the kinetic stress term is added once
// per (atom, non-empty neighbour box) as at ljForce.c:175
// ---------------------------------------------------------------------------
template <class T>
struct LjPot {
  T s6, s6x12, eps4s6, rc2;  // sigma^6, 12*sigma^6, 4*eps*sigma^6, rc^2
};

template <class T>
__global__ void __launch_bounds__(128) lj_pass_kernel(ForceArgs A, LjPot<T> P) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A.ntot) return;
  const int slot = A.atom_slot[a];
  const int b = slot >> 6, i = slot & 63;
  T xi, yi, zi;
  PrecT<T>::pos(A.s, slot, xi, yi, zi);
  typename PrecT<T>::Acc fx, fy, fz, ep, sx;
  fx.zero(); fy.zero(); fz.zero(); ep.zero(); sx.zero();
  const T s6 = P.s6, s12 = P.s6x12, c4 = P.eps4s6;
  const T rc2 = P.rc2;
  auto fn = [&](int js, T dx, T dy, T dz, T r2) {
    if (r2 > rc2) return;
    T ir2 = T(1.0) / r2;
    T r6 = ir2 * ir2 * ir2;
    ep.add(T(0.5) * r6 * (s6 * r6 - T(1.0)));
    T fr = c4 * r6 * ir2 * (s12 * r6 - T(6.0));
    fx.add(dx * fr);
    fy.add(dy * fr);
    fz.add(dz * fr);
    sx.add(fr * dx * dx);
  };
  for_each_neighbor<T, false, true>(A, a, b, i, xi, yi, zi, rc2, fn);
  // kinetic term: -p_x^2/m per non-empty stencil entry
  int ne = A.et.n[b], nonempty = 0;
  for (int e = 0; e < ne; e++) nonempty += A.s.natoms[A.et.box[b * CG_NNBR + e]] > 0;
  d4 p = A.s.p[slot];
  double kin = __ddiv_rn(__dmul_rn(p.x, p.x), A.s.mass[slot]);
  d4 fo;
  fo.x = fx.value();
  fo.y = fy.value();
  fo.z = fz.value();
  fo.w = ep.value();
  A.s.f[slot] = fo;
  A.atom_stress[a] = sx.value() - (double)nonempty * kin;
}

// LJ in force order (mixed precision, persistent lists)
// (OBS as in the EAM force pass: energy and stress only where readable)
template <bool MULTI, bool OBS>
__global__ void __launch_bounds__(PASS_THREADS) fo_lj_kernel(ForceArgs A, LjPot<float> P) {
  const float s6 = P.s6, s12 = P.s6x12, c4 = P.eps4s6, rc2 = P.rc2;
  const bool fuse = !OBS && *(volatile const int *)(A.status + ST_FUSE);
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.fo.slot[a];
    const int b = slot >> 6;
    KSum fx, fy, fz, ep, sx;
    fx.zero(); fy.zero(); fz.zero(); ep.zero(); sx.zero();
    int cnt = 0;
    auto fn = [&](float, float dx, float dy, float dz, float r2) {
      if (r2 > rc2) return;
      cnt++;
      float ir2 = 1.0f / r2;
      float r6 = ir2 * ir2 * ir2;
      if (OBS) ep.add(0.5f * r6 * (s6 * r6 - 1.0f));
      float fr = c4 * r6 * ir2 * (s12 * r6 - 6.0f);
      fx.add(dx * fr);
      fy.add(dy * fr);
      fz.add(dz * fr);
      if (OBS) sx.add(fr * dx * dx);
    };
    fo_for_each<false, MULTI, FO1_UNROLL>(A, a, slot, A.fo.pos[a], rc2, fn);
    fo_force_end(A, a, slot, fuse, fx.valuef(), fy.valuef(), fz.valuef());
    if (OBS) {
      d4 fo;
      fo.x = fx.value();
      fo.y = fy.value();
      fo.z = fz.value();
      fo.w = ep.value();
      A.s.f[slot] = fo;
      if (A.host_f) fo_host_f(A, slot, fo);
      int ne = A.et.n[b], nonempty = 0;
      for (int e = 0; e < ne; e++) nonempty += A.s.natoms[A.et.box[b * CG_NNBR + e]] > 0;
      d4 p = A.s.p[slot];
      double kin = __ddiv_rn(__dmul_rn(p.x, p.x), A.s.mass[slot]);
      A.atom_stress[a] = sx.value() - (double)nonempty * kin;
    }
    A.nbr_n[a] = cnt;
  }
}

}  // namespace cg
