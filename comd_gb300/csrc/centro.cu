// centro.cu -- centrosymmetry parameter of every atom
// (AtomVisualize::computeCentrosymmetry, src-viz/AtomVisualize.c:399-672), a
// headless kernel over the link cells.
//
// One thread per atom of the compacted atom list (64 per CTA).  The
// neighbour scan visits the atom's own box (box-relative differences), then
// the 26 adjacent boxes in x-outer, z-inner order, wrapped once per axis with
// the periodic offset rounded to float (AtomVisualize.c:458-505), and keeps
// up to 12 candidates: the next free entry while fewer than 12 are held, then
// the first entry of largest r^2 is replaced unless the candidate's r^2 is
// larger.  All of it in FP64 with the reference's operation order (this
// translation unit is built without FMA contraction); r^2 values are
// compared as the integer images of non-negative doubles.
//
// The parameter is the minimum over the 10395 pairings of the 12 vectors of
// the sum of |r_a + r_b|^2, accumulated in a float over the pairs in the
// order of their lower index (testCentro, :560-664).  The 66 pair terms are
// rounded to FP32 once; a depth-first search over the pairings (the lowest
// unpaired vector paired first, as the visualiser's loops pair them) finds
// the least plain-FP32 sum, cutting every branch whose partial sum already
// reaches the best complete one (partial sums of non-negative terms never
// decrease, so the cut loses nothing; the greedy pairing gives the first
// bound).  A second search visits the pairings whose FP32 sum lies within
// 4e-6 of that least and sums them exactly as testCentro does (double terms,
// each partial sum rounded to float).  Both sums round at most six float
// additions of non-negative terms, so each is within 12 units of 2^-24 of
// the exact sum: a pairing outside the window cannot be the reference's
// minimum, and the result is the reference's value bit for bit.
// APPROX_CENTROSYM's greedy pairing (:528-557) is the `approx` variant.
#include "sim.h"

using namespace cg;
using namespace cgapi;

namespace {

constexpr int NPAIR = 66;
constexpr int CT = 64;  // threads (atoms) per CTA

// index of the pair a < b among the 66, row by row
__device__ __forceinline__ int pidx(int a, int b) { return 11 * a - (a * (a - 1)) / 2 + b - a - 1; }

__device__ __forceinline__ long long key(double rsq) { return __double_as_longlong(rsq); }

// |a + b|^2 of two held vectors, the reference's order
__device__ __forceinline__ double pair_term(const double (*v)[3][CT], int a, int b, int t) {
  const double x = __dadd_rn(v[a][0][t], v[b][0][t]);
  const double y = __dadd_rn(v[a][1][t], v[b][1][t]);
  const double z = __dadd_rn(v[a][2][t], v[b][2][t]);
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// Depth-first over the pairings: the lowest unpaired entry is paired next,
// with its partners in index order.  A branch whose partial FP32 sum reaches
// `bound` (STRICT) or exceeds it is cut.  leaf(sum, nn, pp) gets every
// pairing kept; its pairs are (nn[l], pp[l]), l = 0..5, lower index first.
template <bool STRICT, class Leaf>
__device__ __forceinline__ void pairing_dfs(const float (*p)[CT], int t, const float &bound,
                                            Leaf &&leaf) {
  int nn[6], pp[6];
  float acc[6];
  int used = 1, lvl = 0;
  nn[0] = 0;
  pp[0] = 0;
  acc[0] = 0.0f;
  while (true) {
    int q = pp[lvl] + 1;
    while (q < 12 && (used >> q & 1)) q++;
    if (q >= 12) {  // this level's partners are done
      used &= ~(1 << nn[lvl]);
      if (lvl == 0) break;
      lvl--;
      used &= ~(1 << pp[lvl]);
      continue;
    }
    pp[lvl] = q;
    const float a = __fadd_rn(acc[lvl], p[pidx(nn[lvl], q)][t]);
    if (STRICT ? a >= bound : a > bound) continue;
    if (lvl == 5) {
      leaf(a, nn, pp);
      continue;
    }
    used |= 1 << q;
    lvl++;
    acc[lvl] = a;
    const int n = __ffs(~used) - 1;
    nn[lvl] = n;
    pp[lvl] = n;
    used |= 1 << n;
  }
}

__global__ void __launch_bounds__(CT) centro_kernel(Geom g, Slots s, const double *dcenter,
                                                    const int *atom_slot, int ntot, int approx,
                                                    double *out) {
  // per thread (column t): held vectors, their r^2 (integer images) and the
  // pair terms rounded to FP32.  Warps run the scan and the pairing phases
  // at different times with no barrier between them, so no array is shared
  // between the phases.
  __shared__ double v[12][3][CT];
  __shared__ long long vk[12][CT];
  __shared__ float p32[NPAIR][CT];
  const int t = threadIdx.x;
  const int a = blockIdx.x * CT + t;
  if (a >= ntot) return;
  const int io = atom_slot[a];
  const int b = io >> 6, i = io & 63;
  const int ni = s.natoms[b];
  const RepGeo &R = rep_of(g, b);
  const int nx = R.nbx[0], ny = R.nbx[1], nz = R.nbx[2];
  const int lb = b - R.box0;
  const int bz = lb / (nx * ny), by = (lb - bz * nx * ny) / nx, bx = lb - bz * nx * ny - by * nx;
  const d4 ri = s.r[io];
  int nb = 0, kmax = 0;
  long long rmax = 0;
  auto offer = [&](double dx, double dy, double dz) {
    const double rsq =
        __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const long long kk = key(rsq);
    int i1;
    if (nb < 12) {
      i1 = nb++;
    } else {
      if (kk > rmax) return;
      i1 = kmax;
    }
    v[i1][0][t] = dx;
    v[i1][1][t] = dy;
    v[i1][2][t] = dz;
    vk[i1][t] = kk;
    if (nb == 12) {  // first entry of largest r^2
      kmax = 0;
      rmax = vk[0][t];
      for (int k = 1; k < 12; k++)
        if (vk[k][t] > rmax) {
          kmax = k;
          rmax = vk[k][t];
        }
    }
  };
  // own box: box-relative differences
  for (int j = 0; j < ni; j++) {
    if (j == i) continue;
    const d4 rj = s.r[b * CG_MAXATOMS + j];
    offer(__dsub_rn(rj.x, ri.x), __dsub_rn(rj.y, ri.y), __dsub_rn(rj.z, ri.z));
  }
  const double cxi = __dadd_rn(dcenter[3 * b + 0], ri.x);
  const double cyi = __dadd_rn(dcenter[3 * b + 1], ri.y);
  const double czi = __dadd_rn(dcenter[3 * b + 2], ri.z);
  for (int cx = bx - 1; cx <= bx + 1; cx++)
    for (int cy = by - 1; cy <= by + 1; cy++)
      for (int cz = bz - 1; cz <= bz + 1; cz++) {
        if (cx == bx && cy == by && cz == bz) continue;
        float ox = 0.0f, oy = 0.0f, oz = 0.0f;
        int qx = cx, qy = cy, qz = cz;
        if (qx < 0) { qx = nx - 1; ox = __double2float_rn(-R.bounds[0]); }
        if (qx >= nx) { qx = 0; ox = __double2float_rn(R.bounds[0]); }
        if (qy < 0) { qy = ny - 1; oy = __double2float_rn(-R.bounds[1]); }
        if (qy >= ny) { qy = 0; oy = __double2float_rn(R.bounds[1]); }
        if (qz < 0) { qz = nz - 1; oz = __double2float_rn(-R.bounds[2]); }
        if (qz >= nz) { qz = 0; oz = __double2float_rn(R.bounds[2]); }
        const int b2 = R.box0 + qz * nx * ny + qy * nx + qx;
        const double ex = __dadd_rn((double)ox, dcenter[3 * b2 + 0]);
        const double ey = __dadd_rn((double)oy, dcenter[3 * b2 + 1]);
        const double ez = __dadd_rn((double)oz, dcenter[3 * b2 + 2]);
        const int nj = s.natoms[b2];
        for (int j = 0; j < nj; j++) {
          const d4 rj = s.r[b2 * CG_MAXATOMS + j];
          offer(__dsub_rn(__dadd_rn(ex, rj.x), cxi), __dsub_rn(__dadd_rn(ey, rj.y), cyi),
                __dsub_rn(__dadd_rn(ez, rj.z), czi));
        }
      }
  double c = 1000.0;
  if (nb >= 12) {
    if (approx) {
      // greedy pairing; a vector with r^2 = 0 counts as paired
      int paired = 0;
      for (int q = 0; q < 12; q++) paired |= (vk[q][t] > 0 ? 0 : 1) << q;
      c = 0.0;
      for (int j = 0; j < 11; j++) {
        if (paired >> j & 1) continue;
        double summin = 1000.0;
        int kmin = -1;
        for (int k = j + 1; k < 12; k++) {
          if (paired >> k & 1) continue;
          const double sum = pair_term(v, j, k, t);
          if (sum < summin) {
            kmin = k;
            summin = sum;
          }
        }
        c = __dadd_rn(c, summin);
        paired |= 1 << j;
        if (kmin >= 0) paired |= 1 << kmin;
      }
    } else {
      for (int x = 0, k = 0; x < 12; x++)
        for (int y = x + 1; y < 12; y++, k++) p32[k][t] = __double2float_rn(pair_term(v, x, y, t));
      // first bound: the greedy pairing's FP32 sum (a complete pairing)
      float best = 0.0f;
      for (int used = 0, step = 0; step < 6; step++) {
        const int n = __ffs(~used) - 1;
        used |= 1 << n;
        int qb = -1;
        float pb = 0.0f;
        for (int q = n + 1; q < 12; q++)
          if (!(used >> q & 1) && (qb < 0 || p32[pidx(n, q)][t] < pb)) {
            qb = q;
            pb = p32[pidx(n, q)][t];
          }
        used |= 1 << qb;
        best = __fadd_rn(best, pb);
      }
      pairing_dfs<true>(p32, t, best, [&](float sum, const int *, const int *) { best = sum; });
      const float window = __fadd_rn(best, __fmul_rn(best, 4e-6f)) + 1e-37f;
      pairing_dfs<false>(p32, t, window, [&](float, const int *nn, const int *pp) {
        float e = 0.0f;  // testCentro
        for (int l = 0; l < 6; l++)
          e = __double2float_rn(__dadd_rn((double)e, pair_term(v, nn[l], pp[l], t)));
        if ((double)e < c) c = (double)e;
      });
    }
  }
  out[io] = c;
}

// min / max over the replica's atoms (minCentro from 1000, maxCentro from 0)
__global__ void centro_range_kernel(Geom g, const int *natoms, const double *c, int r,
                                    double *range) {
  __shared__ double lo_s[256], hi_s[256];
  const RepGeo &R = g.rep[r];
  double lo = 1000.0, hi = 0.0;
  for (int b = R.box0 + threadIdx.x; b < R.box0 + R.nb; b += blockDim.x)
    for (int i = 0; i < natoms[b]; i++) {
      const double x = c[b * CG_MAXATOMS + i];
      lo = x < lo ? x : lo;
      hi = x > hi ? x : hi;
    }
  lo_s[threadIdx.x] = lo;
  hi_s[threadIdx.x] = hi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      lo_s[threadIdx.x] = fmin(lo_s[threadIdx.x], lo_s[threadIdx.x + o]);
      hi_s[threadIdx.x] = fmax(hi_s[threadIdx.x], hi_s[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    range[0] = lo_s[0];
    range[1] = hi_s[0];
  }
}

}  // namespace

extern "C" {

int comdgb_sim_centrosymmetry(comdgb_sim *h, int r, int approx, double *out, double *cmin,
                              double *cmax) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (r < 0 || r >= h->nrep) return set_err(COMDGB_ERR_ARG, "replica %d of %d", r, h->nrep);
  CK(cudaSetDevice(h->device));
  int err = 0;
  if (!h->centro) {
    h->centro = track(h, dalloc<double>((size_t)h->nslots + 2, &err));
    if (err) return set_err(COMDGB_ERR_NOMEM, "centrosymmetry buffer");
  }
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(h->centro, 0, sizeof(double) * (size_t)h->nslots, st));  // empty slots 0
  // the atom list of the current layout
  launch_compact(h->g, h->s.natoms, h->box_start, h->atom_slot, h->ntot, h->cpart, h->ncpart, st);
  if (h->ntot > 0)
    centro_kernel<<<(h->ntot + CT - 1) / CT, CT, 0, st>>>(h->g, h->s, h->dcenter, h->atom_slot,
                                                           h->ntot, approx, h->centro);
  centro_range_kernel<<<1, 256, 0, st>>>(h->g, h->s.natoms, h->centro, r,
                                         h->centro + h->nslots);
  CK(cudaGetLastError());
  const RepGeo &R = h->reps[r];
  if (out)
    CK(cudaMemcpyAsync(out, h->centro + (size_t)R.box0 * CG_MAXATOMS,
                       sizeof(double) * (size_t)R.nb * CG_MAXATOMS, cudaMemcpyDeviceToHost, st));
  double range[2];
  CK(cudaMemcpyAsync(range, h->centro + h->nslots, sizeof range, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (cmin) *cmin = range[0];
  if (cmax) *cmax = range[1];
  return 0;
}

}  // extern "C"
