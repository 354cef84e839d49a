// adjoint.cu -- gradients of the EAM Chebyshev and LJ potentials with respect
// to their parameters, and the adjoint of the velocity-Verlet loop (FP64).
//
// Parameters: EAM Chebyshev -- the base series c = (phi, rho, F), 3 x 32
// coefficients on their [a, b]; the derivative series follow from them by the
// reference's genDer (cheby.c:219-270), so they are not free parameters.
// LJ -- (epsilon, sigma) at fixed cutoff.  eamCheb (cheby.c:276-310) is
// sum'_k c_k T_k(y), y = (2x - a - b)/(b - a), x clamped below at a, with the
// k = 0 term halved; its derivative in c_k is the basis B_k(y) and d/dx of
// that is B'_k = T'_k(y) * 2/(b - a) (0 below a, where eamCheb is clamped).
//
// With U the total energy, f the reference's forces (EAM f = +grad U,
// eam.c:438-660; LJ f = -grad U, ljForce.c:89-224) and a vector lambda per
// atom, D = sum_i lambda_i . grad_i U.  The force-matching loss
// L = sum_i |f_i - t_i|^2 has dL/dc = +/- dD/dc at lambda = 2 (f - t) (fixed),
// and one reverse velocity-Verlet step needs the same dD/dc at lambda = the
// force adjoint, plus the Hessian-vector product H lambda = grad_r D.
// For EAM, with v_ij = (lambda_i - lambda_j) . (r_i - r_j)/r_ij (symmetric),
// W_i = sum_j v_ij rho'(r_ij) and X_i = F''(rho_i) W_i:
//   D = sum_{i<j} v_ij phi'(r_ij) + sum_i F'(rho_i) W_i
//   dU/dc^phi_k = sum_{i<j} B_k(r_ij)        dD/dc^phi_k = sum_{i<j} v_ij B'_k(r_ij)
//   dU/dc^rho_k = sum_{i<j} (F'_i + F'_j) B_k(r_ij)
//   dD/dc^rho_k = sum_{i<j} [(F'_i + F'_j) v_ij B'_k(r_ij) + (X_i + X_j) B_k(r_ij)]
//   dU/dc^F_k   = sum_i B_k(rho_i)           dD/dc^F_k   = sum_i W_i B'_k(rho_i)
// Unique pairs are the list entries with slot_j > slot_i (duplicate stencil
// entries of small grids are separate terms, as in the reference's sums).
// Sums over atoms and pairs are per CTA in fixed order, then over CTAs in a
// fixed order: results are deterministic.
#include <algorithm>
#include <cstring>

#include "sim.h"

using namespace cg;
using namespace cgapi;

namespace {

constexpr int NC = CG_NCHEB;
constexpr int ADJ_THREADS = 64;  // CTA of the basis-sum kernels
constexpr int NQ = 6;            // sums per coefficient index: see adj_basis_kernel

// the FP64 series of the simulation and their second derivatives
struct ChebSet {
  double c[9][NC];  // 0 phi 1 rho 2 F 3 dphi 4 drho 5 dF 6 d2phi 7 d2rho 8 d2F
  double a[9], b[9];
};

// eamCheb (cheby.c:276-310), the reference's operation order
__device__ __forceinline__ double cheb_val(const ChebSet &S, int q, double x) {
  const double a = S.a[q], b = S.b[q];
  if (x < a) x = a;
  const double y = (2.0 * x - a - b) / (b - a), y2 = 2.0 * y;
  double d = 0.0, dd = 0.0;
  for (int j = NC - 1; j > 0; j--) {
    const double sv = d;
    d = y2 * d - dd + S.c[q][j];
    dd = sv;
  }
  return y * d - dd + 0.5 * S.c[q][0];
}

// x-derivative of a clamped series: 0 below a.  (The reference's forces use
// the derivative series at the clamped argument, eamCheb(dphi, r) -- which
// cheb_val gives -- so D differentiates those values in c, while its
// position derivatives below a are 0.)
__device__ __forceinline__ double cheb_der(const ChebSet &S, int qd, int q, double x) {
  return x < S.a[q] ? 0.0 : cheb_val(S, qd, x);
}

struct Lam {
  const d4 *lam;    // [nslots] lambda by slot
  const double *x;  // [nslots] X = F'' W by slot (EAM)
};

// lambda per slot: 2 (f - target[id]) (loss), or u[id] (given vector)
__global__ void adj_lambda_kernel(Slots s, const int *atom_slot, int ntot, const double *target,
                                  const double *u, d4 *lam, double *loss) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= ntot) return;
  const int slot = atom_slot[a];
  const int id = s.id[slot];
  d4 l;
  l.x = l.y = l.z = l.w = 0.0;
  if ((unsigned)id >= (unsigned)ntot) {  // ids must be 0..ntot-1
    lam[slot] = l;
    if (target) loss[a] = 0.0;
    return;
  }
  if (target) {
    const d4 f = s.f[slot];
    const double dx = f.x - target[3 * (size_t)id], dy = f.y - target[3 * (size_t)id + 1],
                 dz = f.z - target[3 * (size_t)id + 2];
    l.x = 2.0 * dx;
    l.y = 2.0 * dy;
    l.z = 2.0 * dz;
    loss[a] = dx * dx + dy * dy + dz * dz;
  } else {
    l.x = u[3 * (size_t)id];
    l.y = u[3 * (size_t)id + 1];
    l.z = u[3 * (size_t)id + 2];
  }
  lam[slot] = l;
}

// W_i = sum_j v_ij rho'(r_ij) over the embedding-force pairs (r2 < rc2,
// eam.c:612) and X_i = F''(rho_i) W_i, per slot
__global__ void adj_w_kernel(ForceArgs A, const __grid_constant__ ChebSet S, double rc2,
                             const d4 *lam, double *wout, double *xout) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A.ntot) return;
  const int slot = A.atom_slot[a];
  const int b = slot >> 6, i = slot & 63;
  double xi, yi, zi;
  PrecT<double>::pos(A.s, slot, xi, yi, zi);
  const d4 li = lam[slot];
  double W = 0.0;
  for_each_neighbor<double, true>(A, a, b, i, xi, yi, zi, rc2,
                                  [&](int js, double dx, double dy, double dz, double r2) {
                                    if (r2 >= rc2) return;
                                    const double r = sqrt(r2);
                                    const d4 lj = lam[js];
                                    const double v = ((li.x - lj.x) * dx + (li.y - lj.y) * dy +
                                                      (li.z - lj.z) * dz) / r;
                                    W += v * cheb_val(S, 4, r);
                                  });
  wout[slot] = W;
  xout[slot] = cheb_der(S, 8, 2, A.s.rho[slot]) * W;
}

// y of x on [a, b] after the clamp at a, and 2/(b - a)
__device__ __forceinline__ void cheb_y(const ChebSet &S, int q, double x, double &y, double &sc) {
  const double a = S.a[q], b = S.b[q];
  if (x < a) x = a;
  y = (2.0 * x - a - b) / (b - a);
  sc = 2.0 / (b - a);
}

// Per-CTA basis sums, row q*NC + k of acc (one column per thread):
//   0 dU/dc^phi   1 dD/dc^phi   2 dU/dc^rho   3 dD/dc^rho   4 dU/dc^F   5 dD/dc^F
// lam / x may be null (energy only).  Writes the CTA's NQ*NC row sums.
__global__ void __launch_bounds__(ADJ_THREADS)
    adj_basis_kernel(ForceArgs A, const __grid_constant__ ChebSet S, double rc2, Lam L,
                     const double *wsl, double *partial) {
  extern __shared__ double acc[];  // [NQ*NC][ADJ_THREADS]
  const int tid = threadIdx.x;
  for (int r = 0; r < NQ * NC; r++) acc[r * ADJ_THREADS + tid] = 0.0;
  const bool same = S.a[0] == S.a[1] && S.b[0] == S.b[1];
  for (int a = blockIdx.x * blockDim.x + tid; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.atom_slot[a];
    const int b = slot >> 6, i = slot & 63;
    double xi, yi, zi;
    PrecT<double>::pos(A.s, slot, xi, yi, zi);
    const double fpi = A.s.fi[slot];
    const double Xi = L.x ? L.x[slot] : 0.0, Wi = wsl ? wsl[slot] : 0.0;
    d4 li;
    li.x = li.y = li.z = 0.0;
    if (L.lam) li = L.lam[slot];
    {  // F(rho_i) terms
      double y, sc;
      cheb_y(S, 2, A.s.rho[slot], y, sc);
      double t0 = 1.0, t1 = y, u0 = 1.0, u1 = 2.0 * y;
      acc[(4 * NC + 0) * ADJ_THREADS + tid] += 0.5;
      for (int k = 1; k < NC; k++) {
        // t1 = T_k, u0 = U_{k-1}
        acc[(4 * NC + k) * ADJ_THREADS + tid] += t1;
        acc[(5 * NC + k) * ADJ_THREADS + tid] += Wi * sc * (double)k * u0;
        const double t2 = 2.0 * y * t1 - t0, u2 = 2.0 * y * u1 - u0;
        t0 = t1;
        t1 = t2;
        u0 = u1;
        u1 = u2;
      }
    }
    for_each_neighbor<double, true>(
        A, a, b, i, xi, yi, zi, rc2, [&](int js, double dx, double dy, double dz, double r2) {
          if (js <= slot || r2 > rc2) return;
          const double r = sqrt(r2);
          double v = 0.0;
          if (L.lam) {
            const d4 lj = L.lam[js];
            v = ((li.x - lj.x) * dx + (li.y - lj.y) * dy + (li.z - lj.z) * dz) / r;
          }
          const double fsum = fpi + A.s.fi[js];
          const double ap = v;                                 // x B'_k / sc
          const double ar = r2 < rc2 ? fsum * v : 0.0;         // x B'_k / sc
          const double br = L.x ? Xi + L.x[js] : 0.0;          // x B_k
          double yp, sp, yr, sr;
          cheb_y(S, 0, r, yp, sp);
          cheb_y(S, 1, r, yr, sr);
          // phi series
          {
            double t0 = 1.0, t1 = yp, u0 = 1.0, u1 = 2.0 * yp;
            acc[(0 * NC + 0) * ADJ_THREADS + tid] += 0.5;
            for (int k = 1; k < NC; k++) {
              acc[(0 * NC + k) * ADJ_THREADS + tid] += t1;
              acc[(1 * NC + k) * ADJ_THREADS + tid] += ap * sp * (double)k * u0;
              if (same) {
                acc[(2 * NC + k) * ADJ_THREADS + tid] += fsum * t1;
                acc[(3 * NC + k) * ADJ_THREADS + tid] += ar * sr * (double)k * u0 + br * t1;
              }
              const double t2 = 2.0 * yp * t1 - t0, u2 = 2.0 * yp * u1 - u0;
              t0 = t1;
              t1 = t2;
              u0 = u1;
              u1 = u2;
            }
          }
          acc[(2 * NC + 0) * ADJ_THREADS + tid] += 0.5 * fsum;
          acc[(3 * NC + 0) * ADJ_THREADS + tid] += 0.5 * br;
          if (!same) {
            double t0 = 1.0, t1 = yr, u0 = 1.0, u1 = 2.0 * yr;
            for (int k = 1; k < NC; k++) {
              acc[(2 * NC + k) * ADJ_THREADS + tid] += fsum * t1;
              acc[(3 * NC + k) * ADJ_THREADS + tid] += ar * sr * (double)k * u0 + br * t1;
              const double t2 = 2.0 * yr * t1 - t0, u2 = 2.0 * yr * u1 - u0;
              t0 = t1;
              t1 = t2;
              u0 = u1;
              u1 = u2;
            }
          }
        });
  }
  __syncthreads();
  for (int r = tid; r < NQ * NC; r += ADJ_THREADS) {
    double t = 0.0;
    for (int c = 0; c < ADJ_THREADS; c++) t += acc[r * ADJ_THREADS + c];
    partial[(size_t)blockIdx.x * NQ * NC + r] = t;
  }
}

// out[r] = sum over n partial rows (fixed order)
__global__ void adj_sum_kernel(const double *partial, int n, int width, double *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= width) return;
  double t = 0.0;
  for (int q = 0; q < n; q++) t += partial[(size_t)q * width + r];
  out[r] = t;
}

// LJ (ljForce.c:151-215, U = 4 eps sum_{i<j} (s^12 - s^6), s = sigma/r, no
// shift at the cutoff; f = -grad U): per-CTA sums of dU/deps, dU/dsigma and
// of sum_{i<j} v_ij dV'(r_ij)/d(eps, sigma) (V' = dU_pair/dr), so that
// dL/d(eps, sigma) = -(the last two) for lambda = 2 (f - t)
__global__ void __launch_bounds__(128) adj_lj_kernel(ForceArgs A, double eps, double sigma,
                                                     double rc2, const d4 *lam, double *partial) {
  __shared__ double sh[4][128];
  double ge = 0.0, gs = 0.0, de = 0.0, ds = 0.0;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.ntot; a += gridDim.x * blockDim.x) {
    const int slot = A.atom_slot[a];
    const int b = slot >> 6, i = slot & 63;
    double xi, yi, zi;
    PrecT<double>::pos(A.s, slot, xi, yi, zi);
    d4 li;
    li.x = li.y = li.z = 0.0;
    if (lam) li = lam[slot];
    for_each_neighbor<double, true>(
        A, a, b, i, xi, yi, zi, rc2, [&](int js, double dx, double dy, double dz, double r2) {
          if (js <= slot || r2 > rc2) return;
          const double r = sqrt(r2);
          const double s2 = sigma * sigma / r2, s6 = s2 * s2 * s2, s12 = s6 * s6;
          ge += 4.0 * (s12 - s6);
          gs += 4.0 * eps * (12.0 * s12 - 6.0 * s6) / sigma;
          if (lam) {
            const d4 lj = lam[js];
            const double v = ((li.x - lj.x) * dx + (li.y - lj.y) * dy + (li.z - lj.z) * dz) / r;
            de += v * 4.0 * (-12.0 * s12 + 6.0 * s6) / r;
            ds += v * 4.0 * eps * (-144.0 * s12 + 36.0 * s6) / (sigma * r);
          }
        });
  }
  sh[0][threadIdx.x] = ge;
  sh[1][threadIdx.x] = gs;
  sh[2][threadIdx.x] = de;
  sh[3][threadIdx.x] = ds;
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int c = 0; c < 128; c++) t += sh[threadIdx.x][c];
    partial[blockIdx.x * 4 + threadIdx.x] = t;
  }
}

// EAM Hessian-vector product, (H u)_k = grad_k sum_i u_i . f_i (f the
// reference's forces), per atom over its full list: for each pair (k, j),
// rhat = (r_k - r_j)/r, du = u_k - u_j, v = du . rhat,
//   g  = phi'(r) + (F'_k + F'_j) rho'(r)      (embedding part for r2 < rc2)
//   g' = phi''(r) + (F'_k + F'_j) rho''(r)
//   += g (du - v rhat)/r + v g' rhat + (X_k + X_j) d rho/dr rhat
// with X = F'' W (adj_w_kernel at lambda = u).  Written by atom id.
__global__ void adj_hvp_kernel(ForceArgs A, const __grid_constant__ ChebSet S, double rc2,
                               const d4 *u, const double *X, double *hv) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A.ntot) return;
  const int slot = A.atom_slot[a];
  const int b = slot >> 6, i = slot & 63;
  double xi, yi, zi;
  PrecT<double>::pos(A.s, slot, xi, yi, zi);
  const d4 uk = u[slot];
  const double Fk = A.s.fi[slot], Xk = X[slot];
  double hx = 0.0, hy = 0.0, hz = 0.0;
  for_each_neighbor<double, true>(
      A, a, b, i, xi, yi, zi, rc2, [&](int js, double dx, double dy, double dz, double r2) {
        if (r2 > rc2) return;
        const double r = sqrt(r2), ir = 1.0 / r;
        const double ex = dx * ir, ey = dy * ir, ez = dz * ir;
        const d4 uj = u[js];
        const double ux = uk.x - uj.x, uy = uk.y - uj.y, uz = uk.z - uj.z;
        const double v = ux * ex + uy * ey + uz * ez;
        const double fs = Fk + A.s.fi[js];
        const bool emb = r2 < rc2;
        const double g = cheb_val(S, 3, r) + (emb ? fs * cheb_val(S, 4, r) : 0.0);
        const double gp = cheb_der(S, 6, 0, r) + (emb ? fs * cheb_der(S, 7, 1, r) : 0.0);
        const double c = (Xk + X[js]) * cheb_der(S, 4, 1, r) + v * gp - g * v * ir;
        hx += g * ux * ir + c * ex;
        hy += g * uy * ir + c * ey;
        hz += g * uz * ir + c * ez;
      });
  const int id = A.s.id[slot];
  if ((unsigned)id >= (unsigned)A.ntot) return;
  hv[3 * (size_t)id] = hx;
  hv[3 * (size_t)id + 1] = hy;
  hv[3 * (size_t)id + 2] = hz;
}

// per-id vectors: y = a*x + y (n triples)
__global__ void adj_axpy_kernel(double a, const double *x, double *y, long n) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) y[q] = a * x[q] + y[q];
}
// y = a*x
__global__ void adj_scale_kernel(double a, const double *x, double *y, long n) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) y[q] = a * x[q];
}
// v[3 id] = f[slot] (the EAM force is grad U)
__global__ void adj_force_by_id_kernel(Slots s, const int *atom_slot, int ntot, double *v) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= ntot) return;
  const int slot = atom_slot[a];
  const int id = s.id[slot];
  if ((unsigned)id >= (unsigned)ntot) return;
  const d4 f = s.f[slot];
  v[3 * (size_t)id] = f.x;
  v[3 * (size_t)id + 1] = f.y;
  v[3 * (size_t)id + 2] = f.z;
}
// per-block sums of x[0..n) (fixed order)
__global__ void adj_block_sum_kernel(const double *x, int n, double *partial) {
  __shared__ double sh[256];
  double t = 0.0;
  for (int q = blockIdx.x * 256 + threadIdx.x; q < n; q += gridDim.x * 256) t += x[q];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

// chder / genDer (cheby.c:180-270): derivative coefficients of an n-term
// series on [a, b], the reference's recurrence and scaling
void cheb_derive(double a, double b, const double *c, double *cd, int n) {
  cd[n - 1] = 0.0;
  cd[n - 2] = 2.0 * (n - 1) * c[n - 1];
  for (int j = n - 2; j > 0; j--) cd[j - 1] = cd[j + 1] + 2 * (j)*c[j];
  const double con = 2.0 / (b - a);
  for (int j = 0; j < n; j++) cd[j] = cd[j] * con;
}

ChebSet cheb_set(const comdgb_sim *h) {
  ChebSet S{};
  for (int q = 0; q < 6; q++) {
    memcpy(S.c[q], h->cheb_coef[q], sizeof S.c[q]);
    S.a[q] = h->cheb_a[q];
    S.b[q] = h->cheb_b[q];
  }
  for (int q = 6; q < 9; q++) {
    cheb_derive(S.a[q - 3], S.b[q - 3], S.c[q - 3], S.c[q], NC);
    S.a[q] = S.a[q - 3];
    S.b[q] = S.b[q - 3];
  }
  return S;
}

typedef comdgb_sim::Adj Work;

// the handle's adjoint scratch (allocated once)
int work(comdgb_sim *h, Work *&Wp) {
  Work &W = h->adj;
  Wp = &W;
  if (W.lam) return 0;
  int err = 0;
  size_t ns = (size_t)h->nslots, nv = 3 * (size_t)h->ntot + 3;
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  W.nblk = std::max(1, std::min(2 * nsm, (h->ntot + ADJ_THREADS - 1) / ADJ_THREADS));
  W.lam = track(h, dalloc<d4>(ns, &err));
  W.w = track(h, dalloc<double>(ns, &err));
  W.x = track(h, dalloc<double>(ns, &err));
  W.loss = track(h, dalloc<double>((size_t)h->ntot + 1, &err));
  W.partial = track(h, dalloc<double>((size_t)W.nblk * NQ * NC + 4096, &err));
  W.out = track(h, dalloc<double>(NQ * NC + 8, &err));
  W.target = track(h, dalloc<double>(nv, &err));
  W.rb = track(h, dalloc<double>(nv, &err));
  W.pb = track(h, dalloc<double>(nv, &err));
  W.u = track(h, dalloc<double>(nv, &err));
  W.hv = track(h, dalloc<double>(nv, &err));
  if (err) {
    W.lam = nullptr;
    return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed for adjoint scratch");
  }
  CK(cudaFuncSetAttribute(adj_basis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)(sizeof(double) * NQ * NC * ADJ_THREADS)));
  return 0;
}

// snapshot i of the handle's pool (grown on demand)
int snap(comdgb_sim *h, size_t i, Snapshot *&q) {
  while (h->adj.snaps.size() <= i) {
    Snapshot *n = new Snapshot();
    int rc = snapshot_alloc(h, n);
    if (rc) {
      delete n;
      return rc;
    }
    h->adj.snaps.push_back(n);
  }
  q = (Snapshot *)h->adj.snaps[i];
  return 0;
}

int need_fp64(comdgb_sim *h) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (h->mixed) return set_err(COMDGB_ERR_UNSUPPORTED, "gradients need an FP64 simulation");
  if (h->opts.potential != COMDGB_POT_EAM_CHEBY && h->opts.potential != COMDGB_POT_LJ)
    return set_err(COMDGB_ERR_UNSUPPORTED, "gradients are for EAM Chebyshev or LJ potentials");
  CK(cudaSetDevice(h->device));
  return 0;
}

unsigned blocks(long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// sum of W.loss[0..ntot) to the host
int loss_sum(comdgb_sim *h, Work &W, double *loss) {
  const int nb = std::min(1024, (int)blocks(h->ntot));
  adj_block_sum_kernel<<<nb, 256, 0, h->stream>>>(W.loss, h->ntot, W.partial);
  adj_sum_kernel<<<1, 32, 0, h->stream>>>(W.partial, nb, 1, W.out);
  CK(cudaMemcpyAsync(loss, W.out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

// EAM Chebyshev basis sums at the current forces and per-step list: rows
// 0..5 (see adj_basis_kernel) into out[6*NC] on the host.  lam/x/w null:
// energy rows only.
int eam_rows(comdgb_sim *h, Work &W, const ChebSet &S, bool with_lam, double *rows) {
  ForceArgs A = force_args(h);
  const double rc2 = h->eam64c.rc2;
  Lam L{with_lam ? W.lam : nullptr, with_lam ? W.x : nullptr};
  adj_basis_kernel<<<W.nblk, ADJ_THREADS, sizeof(double) * NQ * NC * ADJ_THREADS, h->stream>>>(
      A, S, rc2, L, with_lam ? W.w : nullptr, W.partial);
  adj_sum_kernel<<<blocks(NQ * NC, 64), 64, 0, h->stream>>>(W.partial, W.nblk, NQ * NC, W.out);
  CK(cudaMemcpyAsync(rows, W.out, sizeof(double) * NQ * NC, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return check_status(h);
}

// lambda (from target forces by id, or a per-id vector u) and, for EAM, W and X
int set_lambda(comdgb_sim *h, Work &W, const ChebSet &S, const double *d_target,
               const double *d_u) {
  adj_lambda_kernel<<<blocks(h->ntot), 256, 0, h->stream>>>(h->s, h->atom_slot, h->ntot, d_target,
                                                           d_u, W.lam, W.loss);
  if (h->opts.potential == COMDGB_POT_EAM_CHEBY)
    adj_w_kernel<<<blocks(h->ntot, 128), 128, 0, h->stream>>>(force_args(h), S, h->eam64c.rc2,
                                                              W.lam, W.w, W.x);
  CK(cudaGetLastError());
  return 0;
}

// LJ sums: out[0..3] = dU/deps, dU/dsigma, sum v dV'/deps, sum v dV'/dsigma
int lj_sums(comdgb_sim *h, Work &W, bool with_lam, double *out4) {
  const int nb = std::min(W.nblk, 1024);
  adj_lj_kernel<<<nb, 128, 0, h->stream>>>(force_args(h), h->lj_eps, h->lj_sigma, h->lj64.rc2,
                                           with_lam ? W.lam : nullptr, W.partial);
  adj_sum_kernel<<<1, 32, 0, h->stream>>>(W.partial, nb, 4, W.out);
  CK(cudaMemcpyAsync(out4, W.out, sizeof(double) * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return check_status(h);
}

// a force call whose lists are built from the current state (so forces are
// a function of the state alone, whatever the history of list builds)
int force_fresh(comdgb_sim *h) {
  if (h->pl.slot_of) CK(cudaMemsetAsync(h->status + ST_REBUILD, 0x01, 1, h->stream));
  return do_force(h);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int comdgb_sim_set_cheby(comdgb_sim *h, const double *coef, const double *x0, const double *xn) {
  if (!h || !coef || !x0 || !xn) return set_err(COMDGB_ERR_ARG, "null argument");
  if (h->opts.potential != COMDGB_POT_EAM_CHEBY)
    return set_err(COMDGB_ERR_UNSUPPORTED, "not an EAM Chebyshev simulation");
  CK(cudaSetDevice(h->device));
  double c6[6][NC], a[6], b[6];
  for (int q = 0; q < 3; q++) {
    if (!(xn[q] > x0[q])) return set_err(COMDGB_ERR_ARG, "series %d: empty interval", q);
    memcpy(c6[q], coef + (size_t)q * NC, sizeof c6[q]);
    a[q] = a[q + 3] = x0[q];
    b[q] = b[q + 3] = xn[q];
    cheb_derive(a[q], b[q], c6[q], c6[q + 3], NC);
  }
  return install_cheby(h, c6, a, b);
}

int comdgb_sim_get_cheby(comdgb_sim *h, double *coef, double *x0, double *xn) {
  if (!h || !coef || !x0 || !xn) return set_err(COMDGB_ERR_ARG, "null argument");
  if (h->opts.potential != COMDGB_POT_EAM_CHEBY)
    return set_err(COMDGB_ERR_UNSUPPORTED, "not an EAM Chebyshev simulation");
  for (int q = 0; q < 3; q++) {
    memcpy(coef + (size_t)q * NC, h->cheb_coef[q], sizeof(double) * NC);
    x0[q] = h->cheb_a[q];
    xn[q] = h->cheb_b[q];
  }
  return 0;
}

int comdgb_sim_set_lj(comdgb_sim *h, double epsilon, double sigma) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (h->opts.potential != COMDGB_POT_LJ)
    return set_err(COMDGB_ERR_UNSUPPORTED, "not an LJ simulation");
  if (!(sigma > 0.0)) return set_err(COMDGB_ERR_ARG, "sigma must be positive");
  install_lj(h, epsilon, sigma, h->cutoff);
  return 0;
}

int comdgb_sim_energy_grad(comdgb_sim *h, double *energy, double *grad) {
  int rc = need_fp64(h);
  if (rc) return rc;
  if (!grad) return set_err(COMDGB_ERR_ARG, "null argument");
  Work *Wp;
  if ((rc = work(h, Wp)) || (rc = force_fresh(h))) return rc;
  Work &W = *Wp;
  if (energy) *energy = h->e;
  if (h->opts.potential == COMDGB_POT_LJ) {
    double o[4];
    if ((rc = lj_sums(h, W, false, o))) return rc;
    grad[0] = o[0];
    grad[1] = o[1];
    return 0;
  }
  double rows[NQ * NC];
  if ((rc = eam_rows(h, W, cheb_set(h), false, rows))) return rc;
  for (int q = 0; q < 3; q++)
    for (int k = 0; k < NC; k++) grad[q * NC + k] = rows[(2 * q) * NC + k];
  return 0;
}

int comdgb_sim_force_loss_grad(comdgb_sim *h, const double *target, double *loss, double *grad) {
  int rc = need_fp64(h);
  if (rc) return rc;
  if (!target || !grad) return set_err(COMDGB_ERR_ARG, "null argument");
  Work *Wp;
  if ((rc = work(h, Wp)) || (rc = force_fresh(h))) return rc;
  Work &W = *Wp;
  double *d_t = W.target;
  CK(cudaMemcpyAsync(d_t, target, sizeof(double) * 3 * h->ntot, cudaMemcpyHostToDevice,
                     h->stream));
  const ChebSet S = h->opts.potential == COMDGB_POT_EAM_CHEBY ? cheb_set(h) : ChebSet{};
  if ((rc = set_lambda(h, W, S, d_t, nullptr))) return rc;
  double l = 0.0;
  if ((rc = loss_sum(h, W, &l))) return rc;
  if (loss) *loss = l;
  if (h->opts.potential == COMDGB_POT_LJ) {
    double o[4];
    if ((rc = lj_sums(h, W, true, o))) return rc;
    grad[0] = -o[2];  // f = -grad U
    grad[1] = -o[3];
    return 0;
  }
  double rows[NQ * NC];
  if ((rc = eam_rows(h, W, S, true, rows))) return rc;
  for (int q = 0; q < 3; q++)
    for (int k = 0; k < NC; k++) grad[q * NC + k] = rows[(2 * q + 1) * NC + k];
  return 0;
}

// Reverse velocity Verlet.  Forward: x_{n+1} = Phi(x_n) with r_a = r_n + c p_n,
// p_{n+1} = p_n - dt f(r_a), r_{n+1} = r_a + c p_{n+1}, c = (dt/2)/M.  Given
// the adjoints (rb, pb) of step n+1:  pb += c rb;  u = -dt pb;  rb += H(r_a) u;
// cbar += d(u . f(r_a))/dc;  pb += c rb.  Start: rb = grad U(r_N) (= f for
// EAM), pb = 0, cbar = dU/dc at r_N.  Adjoint vectors are kept by atom id (the
// rebox permutes slots, not atoms).
int comdgb_sim_traj_energy_grad(comdgb_sim *h, int n, double dt, int every, double *j,
                                double *grad) {
  int rc = need_fp64(h);
  if (rc) return rc;
  if (h->opts.potential != COMDGB_POT_EAM_CHEBY)
    return set_err(COMDGB_ERR_UNSUPPORTED, "the trajectory adjoint is for EAM Chebyshev");
  if (n < 1 || every < 1 || !grad) return set_err(COMDGB_ERR_ARG, "bad argument");
  const double dt_atu = dt * kBohrPerAtu;
  const double c = (dt_atu / 2.0) / h->rmass;
  const long nv = 3L * h->ntot;
  Work *Wp;
  if ((rc = work(h, Wp))) return rc;
  Work &W = *Wp;
  double *rb = W.rb, *pb = W.pb, *u = W.u, *hv = W.hv;
  const int nseg = (n + every - 1) / every;
  std::vector<Snapshot *> ck((size_t)nseg), mid((size_t)every);
  Snapshot *fin = nullptr;
  size_t si = 0;
  for (auto &q : ck)
    if ((rc = snap(h, si++, q))) return rc;
  for (auto &q : mid)
    if ((rc = snap(h, si++, q))) return rc;
  if ((rc = snap(h, si++, fin))) return rc;
  const ChebSet S = cheb_set(h);
  // forward, keeping the state at the start of every segment
  for (int t = 0; t < n; t++) {
    if (t % every == 0 && (rc = snapshot_copy(h, *ck[t / every], true))) return rc;
    if ((rc = step_first_half(h, dt_atu)) || (rc = force_fresh(h)) ||
        (rc = step_second_half(h, dt_atu)))
      return rc;
  }
  if ((rc = force_fresh(h))) return rc;
  if (j) *j = h->e;
  if ((rc = snapshot_copy(h, *fin, true))) return rc;
  double rows[NQ * NC], cbar[3 * NC];
  if ((rc = eam_rows(h, W, S, false, rows))) return rc;
  for (int q = 0; q < 3; q++)
    for (int k = 0; k < NC; k++) cbar[q * NC + k] = rows[(2 * q) * NC + k];
  adj_force_by_id_kernel<<<blocks(h->ntot), 256, 0, h->stream>>>(h->s, h->atom_slot, h->ntot, rb);
  CK(cudaMemsetAsync(pb, 0, sizeof(double) * nv, h->stream));
  // backward, segment by segment: recompute the segment's mid-step states
  for (int sgm = nseg - 1; sgm >= 0; sgm--) {
    const int t0 = sgm * every, m = std::min(every, n - t0);
    if ((rc = snapshot_copy(h, *ck[sgm], false))) return rc;
    for (int t = 0; t < m; t++) {
      if ((rc = step_first_half(h, dt_atu)) || (rc = snapshot_copy(h, *mid[t], true)) ||
          (rc = force_fresh(h)) || (rc = step_second_half(h, dt_atu)))
        return rc;
    }
    for (int t = m - 1; t >= 0; t--) {
      if ((rc = snapshot_copy(h, *mid[t], false)) || (rc = force_fresh(h))) return rc;
      adj_axpy_kernel<<<blocks(nv), 256, 0, h->stream>>>(c, rb, pb, nv);
      adj_scale_kernel<<<blocks(nv), 256, 0, h->stream>>>(-dt_atu, pb, u, nv);
      if ((rc = set_lambda(h, W, S, nullptr, u))) return rc;
      adj_hvp_kernel<<<blocks(h->ntot, 128), 128, 0, h->stream>>>(force_args(h), S,
                                                                 h->eam64c.rc2, W.lam, W.x, hv);
      if ((rc = eam_rows(h, W, S, true, rows))) return rc;
      for (int q = 0; q < 3; q++)
        for (int k = 0; k < NC; k++) cbar[q * NC + k] += rows[(2 * q + 1) * NC + k];
      adj_axpy_kernel<<<blocks(nv), 256, 0, h->stream>>>(1.0, hv, rb, nv);
      adj_axpy_kernel<<<blocks(nv), 256, 0, h->stream>>>(c, rb, pb, nv);
    }
  }
  CK(cudaGetLastError());
  for (int q = 0; q < 3 * NC; q++) grad[q] = cbar[q];
  if ((rc = snapshot_copy(h, *fin, false))) return rc;
  return force_fresh(h);
}

}  // extern "C"
