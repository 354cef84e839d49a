// common.cuh -- device data layout and shared device helpers of libcomdgb.
//
// HBM layout (one GPU, structure of arrays over the reference's slots
// slot = box*64 + k, src-flat/include/pmdTypes.h:100):
//   r, p, f   double4 per slot (x, y, z, -) / (fx, fy, fz, e): one aligned
//             32-byte access per atom for gathers and the Verlet kernel
//   rho, fi, mass  double per slot;  id, itype  int per slot
//   pos32     float4 per slot: FP32 copy of the box-relative position
//             (mixed precision); fi32 float per slot: F'(rho) in FP32
//   natoms    int per box
// Per-box link-cell stencil ("entry table"), built once: for each box the
// up to 27 neighbour box ids in getNeighborBoxes order (domains.c:391-430)
// with multiplicity, and the minimum-image box offsets drbox
// (eam.c:494-502) in FP64 and FP32.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#define CG_MAXATOMS 64
#define CG_NNBR 27
#define CG_NCHEB 32

namespace cg {

// 32-byte aligned double4 (CUDA 13 deprecates the 16-byte aligned one)
typedef double4_32a d4;

// The box grid of one replica (one reference simflat_t).  A simulation is
// one replica; a batch packs several, each with its own grid, one after the
// other in the global box, slot and atom numbering.
struct RepGeo {
  int nbx[3];
  int box0;            // first global box of the replica
  int nb;              // boxes of the replica
  int a0, na;          // first atom (compacted order) and atoms of the replica
  int pad;
  double bounds[3], boxsize[3];
  double half[3];      // boxsize / 2: the box centre of the FP32 positions
  float hi[3], lo[3];  // boxsize as FP32 hi + lo
};

struct Geom {
  int nboxes;            // all replicas
  int periodic;
  int nrep;
  const RepGeo *rep;     // [nrep]
  const int *box_rep;    // [nboxes] replica of each box (null: one replica)
  const int *boxc;       // [nboxes] packed box coordinates (within the replica) ix | iy << 10 | iz << 20
  float hi0[3], lo0[3];  // replica 0's boxsize as FP32 hi + lo (kernel-parameter copies)
};

// the grid of the replica box b belongs to
__device__ __forceinline__ const RepGeo &rep_of(const Geom &g, int b) {
  return g.rep[g.box_rep ? __ldg(g.box_rep + b) : 0];
}

// RN(x) to FP32 from the IEEE bits with integer operations (the FP64 pipe of
// this part issues two operations per SM per clock); results that are not
// normal FP32 numbers take the hardware conversion.
__host__ __device__ __forceinline__ float d2f_rn(double x) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof b);
#endif
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (e <= 0 || e >= 255) return (float)x;
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 of 52 bits
  const unsigned rest = lo & 0x1fffffffu;                    // the 29 dropped bits
  unsigned f = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) f += 1u;  // ties to even
#ifdef __CUDA_ARCH__
  return __uint_as_float(f);
#else
  float y;
  memcpy(&y, &f, sizeof y);
  return y;
#endif
}

// FP32 position relative to the box centre, RN(x - boxsize/2): one FP64
// subtraction and the integer rounding per coordinate
__device__ __forceinline__ float4 centred32(const RepGeo &R, double x, double y, double z) {
  return make_float4(d2f_rn(x - R.half[0]), d2f_rn(y - R.half[1]), d2f_rn(z - R.half[2]), 0.f);
}

// which side of [0, hi) x lies on (-1: x < 0, +1: x >= hi, 0: inside or NaN)
// for a finite hi > 0, by integer compares of the IEEE bits
__device__ __forceinline__ int side_of(double x, double hi) {
  const long long b = __double_as_longlong(x);
  const long long inf = 0x7ff0000000000000LL;
  if (b < 0) return (b != (long long)0x8000000000000000ULL && (b & 0x7fffffffffffffffLL) <= inf) ? -1 : 0;
  return (b >= __double_as_longlong(hi) && b <= inf) ? 1 : 0;
}

// box coordinates from the packed table (avoids integer division)
__device__ __forceinline__ void box_ixyz_tab(const Geom &g, int b, int *ix) {
  int c = __ldg(g.boxc + b);
  ix[0] = c & 1023;
  ix[1] = (c >> 10) & 1023;
  ix[2] = (c >> 20) & 1023;
}

// RN(a / b) from y = RN(1/b) with two fused multiply-adds (Markstein): the
// residual a - b*q is exact and q + r*y rounds to the correctly rounded
// quotient.  Used only when b's significand is not all ones (checked on
// the host); the integrator's result equals a division a / b bit for bit.
__device__ __forceinline__ double div_markstein(double a, double b, double y) {
  double q = __dmul_rn(a, y);
  double r = __fma_rn(-q, b, a);
  return __fma_rn(r, y, q);
}

struct Slots {
  int *natoms;
  int *id;
  int *itype;
  double *mass;
  d4 *r;
  d4 *p;
  d4 *f;
  double *rho;
  double *fi;
  float4 *pos32;
  float *fi32;
};

struct EntryTab {
  int *n;          // [nboxes] number of valid entries
  int *box;        // [nboxes*27] neighbour box id
  d4 *dr64;     // [nboxes*27] drbox (x, y, z, 0)
  float4 *dr32;    // [nboxes*27] drbox rounded to FP32
};

// device status words
enum {
  ST_ERROR = 0,       // first error code (COMDGB_ERR_*), 0 if none
  ST_REBIN_SERIAL = 1,// set when the parallel rebin cannot reproduce reBoxAll
  ST_NBR_OVERFLOW = 2,// atoms whose neighbour list overflowed (handled); with
                      // persistent lists: the overflows of the current lists
  ST_SERIAL_RUNS = 3, // number of serial rebin fallbacks taken
  ST_REBUILD = 4,     // persistent lists: an atom moved more than skin/2
  ST_REBUILDS = 5,    // persistent lists: number of list builds
  ST_DELTA = 6,       // f.xyz holds the half-step position increments (see advance_kernel)
  ST_OVF_BUILD = 7,   // persistent lists: overflows counted by the build in progress
  ST_FUSE = 8,        // force order: the force pass also makes the next step's velocity
                      // step and both position half steps (see fo_eam_pass2_kernel)
  ST_COUNT = 9
};

// Persistent (skin) neighbour lists, keyed by atom id: built with cutoff
// rc + skin, rebuilt when an atom has moved more than skin/2 since the last
// build.  Every member is null when lists are rebuilt each step.
struct Persist {
  int *vlist;        // [ntot*vcap] neighbour ids of atom id
  int *vcount;       // [ntot] true neighbour count
  int vcap;
  int *slot_of;      // [ntot] current slot of atom id (kept by the rebin)
  d4 *rref;          // [ntot] position (world frame, FP64) at the last build
  double half_skin2; // (skin/2 - 2e-4 A)^2
};

// Force order (mixed precision with persistent lists): each list build
// numbers the atoms in the box order of that moment, a = box_start[b] + k,
// and the passes work in that numbering until the next build.  The list of
// atom a is stored transposed per warp of 32 atoms -- entry t of atom a at
// ((a / 32) * vcap + t) * 32 + a % 32, so the 32 lanes of a warp read entry
// t as one 128-byte line -- each entry (neighbour number << 6) | code, the
// code the neighbour's build box relative to a's as three 2-bit fields
// (dx+1) | (dy+1) << 2 | (dz+1) << 4 (so at most 2^26 atoms).  Positions are FP32 relative to the centre of the atom's build
// box, refreshed every step from the FP64 slot data, so a pair's dr is
// (pos_a - pos_j) - d * boxsize with d the code's box difference.
struct ForceOrder {
  uint32_t *list;
  int *n;            // [ntot] list length (> vcap: overflowed, the stencil is scanned)
  int vcap;
  int *id;           // [ntot] atom id of a
  int *of_id;        // [ntot] force-order number of atom id (-1 before the first build)
  float4 *ref;       // [ntot] FP32 position at the build (build-box centred); w = build box
  float4 *pos;       // [ntot] FP32 position relative to the build box centre
  int *slot;         // [ntot] current slot of a (kept by the rebin)
  float4 *pf;        // [ntot] EAM: pos with w = F'(rho) of a (written by pass 1 for pass 2)
  float half_skin2;    // rebuild when an atom moved more than this squared
  // EAM: the pairs of this force call.  The density pass (pass 1) walks the
  // skin list and writes the entries within the cutoff, in the list's
  // transposed layout, for the force pass (pass 2).
  uint32_t *cut;     // [rows*vcap] entries with r^2 <= rc^2
  int *ncut;         // [ntot] their count (> vcap: the skin list overflowed)
  float *emb;        // [ntot] F(rho) of a, from pass 1 (the per-atom energy's embedding part)
  // the force of a from every force-order force call, as the FP32 value its
  // compensated sum gives (the FP64 f of the slot arrays holds the same
  // values, written only by the force calls whose results the caller reads);
  // the velocity steps of a step sequence read it
  float4 *force;     // [ntot] xyz
};

// Force order: the FP32 position of force-order atom af (now in box b at
// box-relative FP64 position r, FP32 centred position p32) relative to its
// build box centre -- p32 itself while the atom is in its build box, else
// RN(r - boxsize/2 + (b - build box) * boxsize), one rounding either way --
// and the rebuild test on its displacement since the build.
__device__ __forceinline__ void fo_track_at(const Geom &g, const ForceOrder &fo, int b, int af,
                                            const d4 &r, float4 p32, int *status) {
  const float4 q = fo.ref[af];
  const RepGeo &R = rep_of(g, b);
  int ixn[3], ixb[3];
  box_ixyz_tab(g, b, ixn);
  box_ixyz_tab(g, __float_as_int(q.w), ixb);
  const double rv[3] = {r.x, r.y, r.z};
  const float qv[3] = {q.x, q.y, q.z};
  float pv[3] = {p32.x, p32.y, p32.z}, d2 = 0.f;
  bool far = false;
  for (int k = 0; k < 3; k++) {
    int db = ixn[k] - ixb[k];
    if (g.periodic) {
      if (db > 1) db -= R.nbx[k];
      else if (db < -1) db += R.nbx[k];
    }
    far |= db > 1 || db < -1;
    // more than a box width outside its box (only a runaway step does that):
    // the box-centred FP32 position says so without FP64 work
    far |= !(fabsf(pv[k]) <= 1.5f * R.hi[k]);
    if (db != 0) pv[k] = d2f_rn(fma((double)db, R.boxsize[k], rv[k] - R.half[k]));
    const float d = pv[k] - qv[k];
    d2 = fmaf(d, d, d2);
  }
  if (far || !(d2 <= fo.half_skin2)) atomicExch(status + ST_REBUILD, 1);
  fo.pos[af] = make_float4(pv[0], pv[1], pv[2], 0.f);
}
// the slot of an atom moved by the rebin, in the maps the list mode keeps
struct SlotMap {
  int *slot_of;        // by id (id-keyed persistent lists) or null
  const int *fo_of_id; // force order: id -> a, or null
  int *fo_slot;        // force order: a -> slot
  __device__ __forceinline__ void moved(int id, int ds) const {
    if (slot_of) slot_of[id] = ds;
    if (fo_slot) {
      const int a = fo_of_id[id];
      if (a >= 0) fo_slot[a] = ds;
    }
  }
};

// world-frame position in FP32 from the FP32 box-centred position (mixed
// precision) or from the FP64 box-relative one; good to ~1e-4 A, used only
// for the skin test
// FP64 world position of the atom in slot r of box b: the box corner plus
// the box-relative position
__device__ __forceinline__ d4 world64(const Geom &g, int b, const d4 &r) {
  const RepGeo &R = rep_of(g, b);
  int ix[3];
  box_ixyz_tab(g, b, ix);
  d4 w;
  w.x = R.boxsize[0] * (double)ix[0] + r.x;
  w.y = R.boxsize[1] * (double)ix[1] + r.y;
  w.z = R.boxsize[2] * (double)ix[2] + r.z;
  w.w = 0.0;
  return w;
}

// Persistent lists of an atom at box-relative r in box b are stale when it
// moved more than skin/2 since the build (FP64 minimum-image distance to
// its build position ref), when that distance is not a number, or when the
// atom sits more than a box width outside its box -- a state only a runaway
// step makes, in which a distance measured through one periodic image says
// nothing.
__device__ __forceinline__ bool persist_stale(const Geom &g, int b, const d4 &r, const d4 &ref,
                                              double half_skin2) {
  const RepGeo &R = rep_of(g, b);
  const double rv[3] = {r.x, r.y, r.z};
  for (int k = 0; k < 3; k++)
    if (!(rv[k] >= -R.boxsize[k] && rv[k] <= 2.0 * R.boxsize[k])) return true;
  const d4 w = world64(g, b, r);
  double d[3] = {w.x - ref.x, w.y - ref.y, w.z - ref.z}, s2 = 0.0;
  for (int k = 0; k < 3; k++) {
    const double L = R.bounds[k];
    if (d[k] > 0.5 * L) d[k] -= L;
    else if (d[k] < -0.5 * L) d[k] += L;
    s2 += d[k] * d[k];
  }
  return !(s2 <= half_skin2);
}

// tabulated function (potentialarray_t): v points at element 0, guards at
// v[-1], v[n], v[n+1]
template <class T>
struct Table {
  const T *v;
  T x0, xn, invDx;
  int n;
  // FP32 path: per interval i, two float4 (c0, c1, c2, d0) (d1, 0, 0, 0)
  // computed in FP64 from v[i-1..i+2] so no FP32 differences of nearby table
  // values are formed: value = c0 + u(c1 + u c2), deriv = d0 + u d1
  const float4 *seg;
};

// Chebyshev series of the reference: 0 phi, 1 rho, 2 F, 3 dphi, 4 drho, 5 dF
template <class T>
struct Cheb {
  T c[6][CG_NCHEB];
  T a[6], b[6];
  T ys[6], yo[6];  // y = x*ys + yo (FP32 path)
};

// FP32 path: the pair series (phi, rho, dphi, drho) are the same degree-31
// polynomials re-expanded in FP64 on the sub-interval [lo, xn] where pair
// distances occur (Cheb<float> then holds those coefficients); arguments
// below lo use the reference's own coefficients kept here.
struct ChebLow32 {
  float c[6][CG_NCHEB];
  float a[6], ys[6], yo[6];
  float lo[6];
  int pair_shared;  // phi, rho, dphi re-expanded on one interval (same y)
};

// The pair functions of an EAM Chebyshev potential as piecewise cubics in
// s = r^2 for the FP32 path: n equal segments from s_lo, u = (s - s_lo) *
// inv_h, segment k = floor(u), t = u - k.  p1[k] holds the monomial
// coefficients (c0, c1, c2, c3) in t of phi on segment k, p1[n + k] those of
// rho: cubic Hermite interpolants of the FP64 series (value and derivative
// at both segment ends).  The reference's derivative series are the exact
// derivatives of its phi and rho series (genDer), so phi'(r)/r = 2 dphi/ds
// = dscale * dphi/dt with dscale = 2 * inv_h, and likewise rho'(r)/r.
// s < s_lo (and n == 0: no table) takes the series instead.
// The force-order density pass reads rho alone, no derivative: it has its
// own rho table of SEG1_N segments over the same range (rho1, inv_h1; the
// cubic's error at 512 segments is 4e-9 of rho's maximum, at 256 segments
// 6e-8, FP32's own rounding).
#ifndef COMDGB_SEG_N
#define COMDGB_SEG_N 2048
#endif
#ifndef COMDGB_SEG1_N
#define COMDGB_SEG1_N 512
#endif
constexpr int SEG_N = COMDGB_SEG_N;    // segments of the table
constexpr int SEG1_N = COMDGB_SEG1_N;  // segments of the density pass's rho table
static_assert(SEG_N % 2 == 0, "the float2 derivative records pair up into float4");
// The density pass keeps RHO_COPIES copies of its rho table in shared
// memory, interleaved record by record (segment k of copy c at k *
// RHO_COPIES + c), and lane l reads copy l % RHO_COPIES.  A warp's 16-byte
// shared loads are served a quarter-warp (8 lanes, 128 bytes, all 32 banks)
// at a time; with 8 copies the 8 lanes of a quarter read 8 different
// 16-byte bank groups whatever segments they look up, so the lookup takes
// its minimum of 4 wavefronts instead of about 10 for random segments of
// one copy.  The price is shared memory taken from the L1 cache: 64 KB a
// CTA at 8 copies.  (At 4M atoms, EAM Cu: 0.588 ms a pass with 8 copies,
// 0.610 with 4, 0.614 with 2, 0.625 with one.)
#ifndef COMDGB_RHO_COPIES
#define COMDGB_RHO_COPIES 8
#endif
constexpr int RHO_COPIES = COMDGB_RHO_COPIES;
static_assert(RHO_COPIES == 1 || RHO_COPIES == 2 || RHO_COPIES == 4 || RHO_COPIES == 8,
              "copies of the rho table: 1, 2, 4 or 8");
// The force-order force pass reads the derivatives alone (and phi when it
// sums energies): SEG2_N segments over the same range in two uniform runs,
// n2a of width 1/inv_h2 from s_lo to s2b and the rest of width 1/inv_h2b
// from s2b to rc^2 (u = (s - s_lo) inv_h2, or n2a + (s - s2b) inv_h2b past
// n2a).  On segment k phi'(r)/r = dcub[2k] and rho'(r)/r = dcub[2k + 1] as
// cubics in t = u - k, each interpolating the reference's derivative
// series D(r)/r at t = 0, 1/3, 2/3 and 1, rounded once from FP64.  The
// interpolation error falls off steeply with r (for EAM Cu at 256 uniform
// segments, 1.3e-7 of the largest magnitude at 2.0 A, 5e-9 at 2.5 A, below
// 2e-10 past 3 A; FP32 rounding alone gives 6e-8).  By default the table
// is one uniform run (n2a = n2); COMDGB_SEG2_RUNS=2 makes the first run
// finer, with s2b and n2a picked by the host for the smallest error (EAM
// Cu: 3.4e-9 everywhere), at one compare and one FMA more per pair (2.7 %
// of the force pass).  Its shared memory holds FORCE_COPIES
// interleaved copies, as the density pass's rho table: record (2k + h) *
// FORCE_COPIES + c is cubic h of segment k in copy c, so a pair's two
// lookups take 4 wavefronts each.
#ifndef COMDGB_SEG2_N
#define COMDGB_SEG2_N 256
#endif
#ifndef COMDGB_FORCE_COPIES
#define COMDGB_FORCE_COPIES 8
#endif
#ifndef COMDGB_SEG2_RUNS  // 1: one uniform run, 2: a finer first run
#define COMDGB_SEG2_RUNS 1
#endif
static_assert(COMDGB_SEG2_RUNS == 1 || COMDGB_SEG2_RUNS == 2, "one or two runs of segments");
constexpr int SEG2_N = COMDGB_SEG2_N;
constexpr int FORCE_COPIES = COMDGB_FORCE_COPIES;
static_assert(FORCE_COPIES == 1 || FORCE_COPIES == 2 || FORCE_COPIES == 4 || FORCE_COPIES == 8,
              "copies of the force pass's table: 1, 2, 4 or 8");
struct PairSeg {
  const float4 *p1;
  float s_lo, inv_h, dscale;
  int n;
  const float4 *rho1;  // [n1] rho cubics for the density pass
  float inv_h1;
  int n1;
  const float4 *dcub;  // [2 * n2] phi'(r)/r and rho'(r)/r cubics for the force pass
  float inv_h2, s2b, inv_h2b;
  int n2a, n2;
};

__device__ __forceinline__ float seg_cubic(float4 c, float t) {
  return fmaf(fmaf(fmaf(c.w, t, c.z), t, c.y), t, c.x);
}
// d/dt of the cubic
__device__ __forceinline__ float seg_dcubic(float4 c, float t) {
  return fmaf(fmaf(3.0f * c.w, t, 2.0f * c.z), t, c.y);
}

// coordinates of global box b within its replica's grid R
__host__ __device__ inline void box_ixyz(const RepGeo &R, int b, int *ix) {
  const int l = b - R.box0;
  ix[0] = l % R.nbx[0];
  ix[1] = (l / R.nbx[0]) % R.nbx[1];
  ix[2] = (l / R.nbx[0] / R.nbx[1]) % R.nbx[2];
}

// getIBoxFromIxyz3NP (domains.c:297-325): -1 outside a non-periodic grid,
// else wrap by one period; the global box of the replica's coordinates ix
__host__ __device__ inline int box_from_ixyz(const RepGeo &R, int periodic, int *ix) {
  if (!periodic)
    for (int j = 0; j < 3; j++)
      if (ix[j] < 0 || ix[j] >= R.nbx[j]) return -1;
  for (int j = 0; j < 3; j++) {
    if (ix[j] < 0) ix[j] += R.nbx[j];
    else if (ix[j] >= R.nbx[j]) ix[j] -= R.nbx[j];
  }
  return R.box0 + ix[0] + ix[1] * R.nbx[0] + ix[2] * R.nbx[0] * R.nbx[1];
}

// Kahan-compensated FP32 accumulator
struct KSum {
  float s, c;
  __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  // combined in FP32 (one conversion, no FP64 subtraction: FP64 issue slots
  // are scarce on this GPU); the result is good to half an FP32 ulp
  __device__ __forceinline__ double value() const { return (double)__fsub_rn(s, c); }
  __device__ __forceinline__ float valuef() const { return __fsub_rn(s, c); }
};

struct DSum {
  double s;
  __device__ __forceinline__ void zero() { s = 0.0; }
  __device__ __forceinline__ void add(double x) { s = __dadd_rn(s, x); }
  __device__ __forceinline__ double value() const { return s; }
};

// eamInterpolateDeriv (eam.c:401-434), same operation order
template <class T>
__device__ __forceinline__ void table_eval(const Table<T> &a, T r, T &value, T &deriv) {
  if (r < a.x0) r = a.x0;
  else if (r > a.xn) r = a.xn;
  r = (r - a.x0) * a.invDx;
  T fl = floor(r);
  int i1 = (int)fl;
  r = r - fl;
  // a NaN argument must not index outside the table (valid r gives 0..n-1)
  i1 = i1 < 0 ? 0 : (i1 > a.n - 1 ? a.n - 1 : i1);
  const T *v = a.v;
  T vm = __ldg(v + i1 - 1), v0 = __ldg(v + i1), v1 = __ldg(v + i1 + 1), v2 = __ldg(v + i1 + 2);
  T gi = v1 - vm;
  T gi1 = v2 - v0;
  value = v0 + T(0.5) * r * (r * (v1 + vm - T(2.0) * v0) + gi);
  deriv = (i1 <= 0) ? T(0) : T(0.5) * (gi + r * (gi1 - gi)) * a.invDx;
}

// FP32 table lookup from the per-interval coefficients (same function)
__device__ __forceinline__ void table_eval(const Table<float> &a, float r, float &value,
                                           float &deriv) {
  if (r < a.x0) r = a.x0;
  else if (r > a.xn) r = a.xn;
  float t = (r - a.x0) * a.invDx;
  float fl = floorf(t);
  int i1 = (int)fl;
  i1 = i1 < 0 ? 0 : (i1 > a.n - 1 ? a.n - 1 : i1);
  float u = t - fl;
  float4 s0 = __ldg(a.seg + 2 * i1);
  float d1 = __ldg(reinterpret_cast<const float *>(a.seg + 2 * i1 + 1));
  value = fmaf(u, fmaf(u, s0.z, s0.y), s0.x);
  deriv = fmaf(u, d1, s0.w);
}

// eamCheb (cheby.c:276-310) in FP64: Clenshaw, lower clamp only
__device__ __forceinline__ double cheb_eval64(const double *c, double a, double b, double x) {
  if (x < a) x = a;
  double d = 0.0, dd = 0.0, sv;
  double y = __ddiv_rn(__dsub_rn(__dsub_rn(__dmul_rn(2.0, x), a), b), __dsub_rn(b, a));
  double y2 = __dmul_rn(2.0, y);
#pragma unroll
  for (int j = CG_NCHEB - 1; j > 0; j--) {
    sv = d;
    d = __dadd_rn(__dsub_rn(__dmul_rn(y2, d), dd), c[j]);
    dd = sv;
  }
  return __dadd_rn(__dsub_rn(__dmul_rn(y, d), dd), __dmul_rn(0.5, c[0]));
}

// the same series in FP32 with y from a fused multiply-add
__device__ __forceinline__ float cheb_eval32(const float *c, float a, float ys, float yo,
                                             float x) {
  if (x < a) x = a;
  float y = fmaf(x, ys, yo);
  float y2 = 2.0f * y;
  float d = 0.f, dd = 0.f;
#pragma unroll
  for (int j = CG_NCHEB - 1; j > 0; j--) {
    float sv = d;
    d = fmaf(y2, d, c[j] - dd);
    dd = sv;
  }
  return fmaf(y, d, 0.5f * c[0] - dd);
}

// Three series on the same interval at one argument: the Chebyshev
// polynomials T_k(y) from their three-term recurrence (shared by the three
// sums), then sum c_k T_k with c_0 halved -- the same value as three
// Clenshaw sums for two thirds of the FP32 operations.  Forward recurrence
// and Clenshaw have the same FP32 accuracy for |y| <= 1 on these series.
__device__ __forceinline__ void cheb3_eval32(const float *c0, const float *c1, const float *c2,
                                             float a, float ys, float yo, float x, float &s0,
                                             float &s1, float &s2) {
  if (x < a) x = a;
  const float y = fmaf(x, ys, yo);
  const float y2 = 2.0f * y;
  float tm = 1.0f, t = y;
  s0 = fmaf(c0[1], y, 0.5f * c0[0]);
  s1 = fmaf(c1[1], y, 0.5f * c1[0]);
  s2 = fmaf(c2[1], y, 0.5f * c2[0]);
#pragma unroll
  for (int k = 2; k < CG_NCHEB; k++) {
    const float tn = fmaf(y2, t, -tm);
    tm = t;
    t = tn;
    s0 = fmaf(c0[k], t, s0);
    s1 = fmaf(c1[k], t, s1);
    s2 = fmaf(c2[k], t, s2);
  }
}

}  // namespace cg
