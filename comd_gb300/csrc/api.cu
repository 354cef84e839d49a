// api.cu -- the C ABI of libcomdgb: device mirror of a simflat_t, the force
// call, the velocity-Verlet loop (captured in CUDA graphs) and the drop-in
// wrappers keyed by the caller's simflat_t pointer.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "sim.h"

using namespace cg;
using namespace cgapi;

namespace cgapi {

thread_local char g_err[512] = "";
std::mutex g_reg_mu;

int set_err(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

enum KernelGroup {
  KG_ADV_POS = 0,
  KG_REBIN1,
  KG_COMPACT,
  KG_NBR,
  KG_PASS1,
  KG_PASS2,
  KG_ADV_VP,
  KG_REBIN2,
  KG_COUNT
};
const char *kGroupName[KG_COUNT] = {"advance_positions+classify", "rebin_plan_apply",
                                    "compact_atoms",              "nbr_build",
                                    "force_pass1",                "force_pass2",
                                    "advance_velocity_positions+classify",
                                    "rebin_plan_apply_2"};
// parts of a step (enqueue_step)
enum { PART_NONE = -1, PART_OPEN = 0, PART_MID = 1, PART_CLOSE = 2, PART_FULL = 3 };
// the middle part of a step sequence with the rebox merged
enum { KGM_ADV_VPP, KGM_REBIN, KGM_COMPACT, KGM_NBR, KGM_PASS1, KGM_PASS2, KGM_COUNT };
const char *kGroupNameMerged[KGM_COUNT] = {"advance_velocity_positions+classify",
                                           "rebin_plan_apply", "compact_atoms", "nbr_build",
                                           "force_pass1", "force_pass2"};
// the middle part of a force-order sequence: the rebuild section (classify,
// rebin, compact, list build) is one conditional graph node, and the force
// pass ends with the velocity-Verlet update of the step boundary
enum { KGF_REBUILD, KGF_PASS1, KGF_PASS2, KGF_COUNT };
const char *kGroupNameFo[KGF_COUNT] = {"rebuild_if_due", "force_pass1",
                                       "force_pass2+advance_velocity_positions"};

}  // namespace

namespace cgapi {

std::vector<comdgb_sim *> g_attached;

ForceArgs force_args(comdgb_sim *h) {
  ForceArgs A;
  A.g = h->g;
  A.s = h->s;
  A.et = h->et;
  A.atom_slot = h->atom_slot;
  A.box_start = h->box_start;
  A.ntot = h->ntot;
  A.nbr = h->nbr;
  A.nbr_n = h->nbr_n;
  A.cap = h->cap;
  A.atom_stress = h->atom_stress;
  A.status = h->status;
  A.pl = h->pl;
  A.fo = h->fo;
  A.vv_dt = A.vv_c = 0.0;
  A.host_f = A.host_rho = A.host_fi = nullptr;
  return A;
}

int alloc_slots(comdgb_sim *h, Slots &s, bool with_natoms, int *err) {
  size_t ns = (size_t)h->nslots;
  s.natoms = with_natoms ? track(h, dalloc<int>(h->g.nboxes, err)) : nullptr;
  s.id = track(h, dalloc<int>(ns, err));
  s.itype = track(h, dalloc<int>(ns, err));
  s.mass = track(h, dalloc<double>(ns, err));
  s.r = track(h, dalloc<d4>(ns, err));
  s.p = track(h, dalloc<d4>(ns, err));
  s.f = track(h, dalloc<d4>(ns, err));
  s.rho = track(h, dalloc<double>(ns, err));
  s.fi = track(h, dalloc<double>(ns, err));
  s.pos32 = track(h, dalloc<float4>(ns, err));
  s.fi32 = with_natoms ? track(h, dalloc<float>(ns, err)) : nullptr;
  return *err;
}

void free_all(comdgb_sim *h) {
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->ev_state) cudaEventDestroy(h->ev_state);
  if (h->loop_exec) cudaGraphExecDestroy(h->loop_exec);
  if (h->step_exec) cudaGraphExecDestroy(h->step_exec);
  if (h->force_exec) cudaGraphExecDestroy(h->force_exec);
  if (h->force_exec_tracked) cudaGraphExecDestroy(h->force_exec_tracked);
  if (h->force_exec_host) cudaGraphExecDestroy(h->force_exec_host);
  if (h->timed_exec) cudaGraphExecDestroy(h->timed_exec);
  if (h->timed_graph) cudaGraphDestroy(h->timed_graph);
  for (cudaGraphExec_t &x : h->part_exec)
    if (x) cudaGraphExecDestroy(x);
  for (cudaEvent_t e : h->timed_cap_events) cudaEventDestroy(e);
  for (void *p : h->allocs)
    if (p) cudaFree(p);
  h->allocs.clear();
  for (void *q : h->adj.snaps) delete (Snapshot *)q;  // their device arrays were in allocs
  h->adj.snaps.clear();
  if (h->cond_stream) cudaStreamDestroy(h->cond_stream);
  if (h->stream) cudaStreamDestroy(h->stream);
}

int neighbor_capacity(const simflat_t *s, double rc) {
  double vol = s->bounds[0] * s->bounds[1] * s->bounds[2];
  double dens = vol > 0 ? (double)s->ntot / vol : 0.0;
  double expect = 4.18879020478639 * rc * rc * rc * dens;
  int cap = (int)(1.4 * expect) + 24;
  cap = (cap + 7) & ~7;
  if (cap < 32) cap = 32;
  if (cap > CG_NNBR * CG_MAXATOMS) cap = CG_NNBR * CG_MAXATOMS;
  return cap;
}

template <class T>
Table<T> upload_table(comdgb_sim *h, const potentialarray_t *a, int *err) {
  int n = a->n;
  std::vector<T> v(n + 3);
  for (int i = -1; i <= n + 1; i++) v[i + 1] = (T)a->values[i];
  T *d = track(h, dalloc<T>(n + 3, err));
  Table<T> t{};
  if (*err) return t;
  cudaMemcpy(d, v.data(), sizeof(T) * (n + 3), cudaMemcpyHostToDevice);
  t.v = d + 1;
  t.x0 = (T)a->x0;
  t.xn = (T)a->xn;
  t.invDx = (T)a->invDx;
  t.n = n;
  t.seg = nullptr;
  if (sizeof(T) == 4) {
    // per-interval coefficients of eamInterpolateDeriv (eam.c:422-431) in FP64
    const double *w = a->values;
    std::vector<float4> seg(2 * (size_t)n);
    for (int i = 0; i < n; i++) {
      double gi = w[i + 1] - w[i - 1], gi1 = w[i + 2] - w[i];
      double c1 = 0.5 * gi, c2 = 0.5 * (w[i + 1] + w[i - 1] - 2.0 * w[i]);
      double d0 = i <= 0 ? 0.0 : 0.5 * gi * a->invDx;
      double d1 = i <= 0 ? 0.0 : 0.5 * (gi1 - gi) * a->invDx;
      seg[2 * i] = make_float4((float)w[i], (float)c1, (float)c2, (float)d0);
      seg[2 * i + 1] = make_float4((float)d1, 0.f, 0.f, 0.f);
    }
    float4 *ds = track(h, dalloc<float4>(2 * (size_t)n, err));
    if (*err) return t;
    cudaMemcpy(ds, seg.data(), sizeof(float4) * 2 * n, cudaMemcpyHostToDevice);
    t.seg = ds;
  }
  return t;
}

// eamCheb (cheby.c:276-310) on the host, FP64
double cheb_host(const double *c, double a, double b, double x) {
  if (x < a) x = a;
  double d = 0.0, dd = 0.0, y = (2.0 * x - a - b) / (b - a), y2 = 2.0 * y;
  for (int j = CG_NCHEB - 1; j > 0; j--) {
    double sv = d;
    d = y2 * d - dd + c[j];
    dd = sv;
  }
  return y * d - dd + 0.5 * c[0];
}

// The degree-31 polynomial of series c on [a, b] written in the Chebyshev
// basis of [lo, b]: sampled at the 32 Chebyshev nodes of [lo, b] (exact for
// a degree-31 polynomial) and transformed back.  Identical function to
// ~1e-14 relative; in FP32 its Clenshaw sum no longer cancels the large
// coefficients that the repulsive core near a puts into the series.
void cheb_reexpand(const double *c, double a, double b, double lo, double *out) {
  const double PI = 3.141592653589793;
  double fk[CG_NCHEB];
  for (int k = 0; k < CG_NCHEB; k++) {
    double y = cos(PI * (k + 0.5) / CG_NCHEB);
    fk[k] = cheb_host(c, a, b, y * 0.5 * (b - lo) + 0.5 * (b + lo));
  }
  for (int j = 0; j < CG_NCHEB; j++) {
    double sum = 0.0;
    for (int k = 0; k < CG_NCHEB; k++) sum += fk[k] * cos(PI * j * (k + 0.5) / CG_NCHEB);
    out[j] = 2.0 / CG_NCHEB * sum;
  }
}

// series order: 0 phi, 1 rho, 2 F, 3 dphi, 4 drho, 5 dF.  pair_lo: lower end
// of the re-expansion interval of the pair series (FP32 path)
void fill_cheb(Cheb<double> &c64, Cheb<float> &c32, ChebLow32 &lo32,
               const double coef[6][CG_NCHEB], const double a[6], const double b[6],
               double pair_lo) {
  for (int s = 0; s < 6; s++) {
    for (int j = 0; j < CG_NCHEB; j++) {
      c64.c[s][j] = coef[s][j];
      lo32.c[s][j] = (float)coef[s][j];
    }
    c64.a[s] = a[s];
    c64.b[s] = b[s];
    c64.ys[s] = 2.0 / (b[s] - a[s]);
    c64.yo[s] = -(a[s] + b[s]) / (b[s] - a[s]);
    lo32.a[s] = (float)a[s];
    lo32.ys[s] = (float)c64.ys[s];
    lo32.yo[s] = (float)c64.yo[s];
    bool pair = (s == 0 || s == 1 || s == 3 || s == 4);
    double lo = (pair && pair_lo > a[s] && pair_lo < b[s]) ? pair_lo : a[s];
    double re[CG_NCHEB];
    if (lo > a[s]) cheb_reexpand(coef[s], a[s], b[s], lo, re);
    for (int j = 0; j < CG_NCHEB; j++) c32.c[s][j] = (float)(lo > a[s] ? re[j] : coef[s][j]);
    c32.a[s] = (float)lo;
    c32.b[s] = (float)b[s];
    c32.ys[s] = (float)(2.0 / (b[s] - lo));
    c32.yo[s] = (float)(-(lo + b[s]) / (b[s] - lo));
    lo32.lo[s] = lo > a[s] ? (float)lo : -3.0e38f;
  }
  // one recurrence serves phi, rho and dphi only if they share the interval
  lo32.pair_shared = 1;
  for (int s : {1, 3})
    if (c32.a[s] != c32.a[0] || c32.ys[s] != c32.ys[0] || c32.yo[s] != c32.yo[0] ||
        lo32.lo[s] != lo32.lo[0])
      lo32.pair_shared = 0;
}

// Segment table of the FP32 pair path (PairSeg): phi and rho of the FP64
// series as cubic Hermite interpolants in s = r^2 on [lo^2, rc^2], lo =
// max(pair_lo, series lower ends); the end slopes come from the derivative
// series (d/dt = h * D(r) / (2 r)).  Checked at 9 points per segment: values
// to 1e-7 and slopes (dscale * d/dt against D(r)/r) to 1e-6 of the
// function's largest magnitude on the interval -- so derivative series that
// are not the derivatives of phi and rho drop the table (series path).
// Returns 0, or -1 when device memory ran out.
// no table: every pair distance lies below s_lo, so the kernels take the
// series for every pair and never index the (absent) table
PairSeg no_pair_seg() {
  return PairSeg{nullptr, 3.0e38f, 1.0f, 2.0f, 0, nullptr, 1.0f, 0, nullptr, 1.0f, 3.0e38f, 1.0f, 0, 0};
}

int build_pair_seg(comdgb_sim *h, const double coef[6][CG_NCHEB], const double a[6],
                   const double b[6], double pair_lo, double rc, PairSeg *out) {
  *out = no_pair_seg();
  double lo = pair_lo;
  for (int s : {0, 1, 3, 4}) lo = std::max(lo, a[s]);
  if (!(lo > 0.0 && lo < rc)) return 0;
  const int n = SEG_N;
  const float s_lo = (float)(lo * lo);
  const float inv_h = (float)(n / (rc * rc - (double)s_lo));
  const float dscale = 2.0f * inv_h;
  const double hs = 1.0 / (double)inv_h;
  // q = 0: phi (series 0, derivative 3); q = 1: rho (series 1, derivative 4)
  auto val = [&](int q, double s) {
    return q == 0 ? cheb_host(coef[0], a[0], b[0], sqrt(s)) : cheb_host(coef[1], a[1], b[1], sqrt(s));
  };
  auto der = [&](int q, double s) {  // D(r) / r
    double r = sqrt(s);
    return (q == 0 ? cheb_host(coef[3], a[3], b[3], r) : cheb_host(coef[4], a[4], b[4], r)) / r;
  };
  std::vector<float4> p1((size_t)2 * n);
  for (int q = 0; q < 2; q++) {
    double fmax = 0, gmax = 0, ferr = 0, gerr = 0;
    double f0 = val(q, (double)s_lo), m0 = 0.5 * hs * der(q, (double)s_lo);
    for (int k = 0; k < n; k++) {
      const double s1 = (double)s_lo + (k + 1) * hs;
      const double f1 = val(q, s1), m1 = 0.5 * hs * der(q, s1);
      const double c0 = f0, c1 = m0, c2 = 3.0 * (f1 - f0) - 2.0 * m0 - m1,
                   c3 = 2.0 * (f0 - f1) + m0 + m1;
      p1[(size_t)q * n + k] = make_float4((float)c0, (float)c1, (float)c2, (float)c3);
      for (int e = 0; e <= 8; e++) {
        const double t = e / 8.0, s = (double)s_lo + (k + t) * hs;
        const double fv = val(q, s), gv = der(q, s);
        const double pv = ((c3 * t + c2) * t + c1) * t + c0;
        const double pd = (double)dscale * ((3.0 * c3 * t + 2.0 * c2) * t + c1);
        fmax = std::max(fmax, fabs(fv));
        gmax = std::max(gmax, fabs(gv));
        ferr = std::max(ferr, fabs(pv - fv));
        gerr = std::max(gerr, fabs(pd - gv));
      }
      f0 = f1;
      m0 = m1;
    }
    if (!(ferr <= 1e-7 * fmax) || !(gerr <= 1e-6 * gmax)) return 0;
  }
  // the density pass's rho table: n1 segments, values checked as above
  const int n1 = SEG1_N;
  const float inv_h1 = (float)(n1 / (rc * rc - (double)s_lo));
  const double hs1 = 1.0 / (double)inv_h1;
  {
    double fmax = 0, ferr = 0;
    double f0 = val(1, (double)s_lo), m0 = 0.5 * hs1 * der(1, (double)s_lo);
    for (int k = 0; k < n1; k++) {
      const double s1 = (double)s_lo + (k + 1) * hs1;
      const double f1 = val(1, s1), m1 = 0.5 * hs1 * der(1, s1);
      const double c0 = f0, c1 = m0, c2 = 3.0 * (f1 - f0) - 2.0 * m0 - m1,
                   c3 = 2.0 * (f0 - f1) + m0 + m1;
      p1.push_back(make_float4((float)c0, (float)c1, (float)c2, (float)c3));
      for (int e = 0; e <= 8; e++) {
        const double t = e / 8.0, s = (double)s_lo + (k + t) * hs1;
        const double fv = val(1, s), pv = ((c3 * t + c2) * t + c1) * t + c0;
        fmax = std::max(fmax, fabs(fv));
        ferr = std::max(ferr, fabs(pv - fv));
      }
      f0 = f1;
      m0 = m1;
    }
    if (!(ferr <= 1e-7 * fmax)) return 0;
  }
  // the force pass's derivative cubics: n2 segments in two uniform runs (n2a
  // from s_lo to s2b, the rest from s2b to rc^2), on each D(r)/r of phi and
  // of rho interpolated at t = 0, 1/3, 2/3, 1 (Newton's forward differences
  // in x = 3t).  The split is the candidate with the smallest interpolation
  // error relative to each function's largest magnitude, probed where the
  // error term t (t - 1/3) (t - 2/3) (t - 1) peaks; the table is then
  // checked at 9 points per segment to 1e-6 of that magnitude.
  const int n2 = SEG2_N;
  const double span = rc * rc - (double)s_lo;
  struct Split {
    float inv_a, s_b, inv_b;
    int na;
  };
  auto make_split = [&](double frac, int na) {
    Split sp;
    sp.na = na;
    sp.inv_a = (float)(na / (span * frac));
    sp.s_b = (float)((double)s_lo + na / (double)sp.inv_a);
    sp.inv_b = (float)((n2 - na) / (rc * rc - (double)sp.s_b));
    return sp;
  };
  auto seg_of = [&](const Split &sp, int k, double &s0, double &hh) {
    if (k < sp.na) {
      hh = 1.0 / (double)sp.inv_a;
      s0 = (double)s_lo + k * hh;
    } else {
      hh = 1.0 / (double)sp.inv_b;
      s0 = (double)sp.s_b + (k - sp.na) * hh;
    }
  };
  auto dcubic = [&](int q, double s0, double hh, double c[4]) {
    double g[4];
    for (int i = 0; i < 4; i++) g[i] = der(q, s0 + (i / 3.0) * hh);
    const double d1 = g[1] - g[0], d2 = g[2] - 2.0 * g[1] + g[0],
                 d3 = g[3] - 3.0 * g[2] + 3.0 * g[1] - g[0];
    c[0] = g[0];
    c[1] = 3.0 * (d1 - 0.5 * d2 + d3 / 3.0);
    c[2] = 4.5 * (d2 - d3);
    c[3] = 4.5 * d3;
  };
  auto cubic_at = [](const double c[4], double t) {
    return ((c[3] * t + c[2]) * t + c[1]) * t + c[0];
  };
  double gm[2] = {0.0, 0.0};
  for (int q = 0; q < 2; q++)
    for (int i = 0; i <= 4 * n2; i++)
      gm[q] = std::max(gm[q], fabs(der(q, (double)s_lo + span * i / (4.0 * n2))));
  if (!(gm[0] > 0.0 && gm[1] > 0.0)) return 0;
  auto split_err = [&](const Split &sp, const double *ts, int nt) {
    double e = 0.0;
    for (int q = 0; q < 2; q++)
      for (int k = 0; k < n2; k++) {
        double s0, hh, c[4];
        seg_of(sp, k, s0, hh);
        dcubic(q, s0, hh, c);
        for (int i = 0; i < nt; i++)
          e = std::max(e, fabs(cubic_at(c, ts[i]) - der(q, s0 + ts[i] * hh)) / gm[q]);
      }
    return e;
  };
  const double probe[3] = {0.12, 0.5, 0.88};
  Split best = make_split(0.5, n2 / 2);
  if (COMDGB_SEG2_RUNS == 1) {  // one run: the kernel ignores the split
    best.inv_b = best.inv_a;
    best.s_b = 3.0e38f;
    best.na = n2;
  }
  double best_err = split_err(best, probe, 3);
  if (COMDGB_SEG2_RUNS > 1)
    for (double frac : {0.1, 0.15, 0.2, 0.25, 0.3, 0.35, 0.4})
      for (int j = 2; j <= 7; j++) {
        const Split sp = make_split(frac, n2 * j / 8);
        const double e = split_err(sp, probe, 3);
        if (e < best_err) {
          best_err = e;
          best = sp;
        }
      }
  const size_t off2 = p1.size();
  p1.resize(off2 + 2 * (size_t)n2);
  for (int q = 0; q < 2; q++) {
    double gerr = 0;
    for (int k = 0; k < n2; k++) {
      double s0, hh, c[4];
      seg_of(best, k, s0, hh);
      dcubic(q, s0, hh, c);
      p1[off2 + 2 * (size_t)k + q] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
      for (int e = 0; e <= 8; e++)
        gerr = std::max(gerr, fabs(cubic_at(c, e / 8.0) - der(q, s0 + (e / 8.0) * hh)));
    }
    if (!(gerr <= 1e-6 * gm[q])) return 0;
  }
  int err = 0;
  float4 *d1 = h->seg_buf ? h->seg_buf : track(h, dalloc<float4>(p1.size(), &err));
  if (err) return -1;
  h->seg_buf = d1;
  if (cudaMemcpy(d1, p1.data(), sizeof(float4) * p1.size(), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return -1;
  *out = PairSeg{d1, s_lo, inv_h, dscale, n, d1 + 2 * (size_t)n, inv_h1, n1,
                 d1 + off2, best.inv_a, best.s_b, best.inv_b, best.na, n2};
  return 0;
}

int fit_cheb_gpu(comdgb_sim *h, const eampotential_t *pot, double coef[6][CG_NCHEB],
                 double a[6], double b[6]) {
  int err = 0;
  const potentialarray_t *tabs[3] = {pot->phi, pot->rho, pot->f};
  double *d = dalloc<double>(2 * CG_NCHEB * 3, &err);
  if (err) return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed for Chebyshev fit");
  std::vector<double *> tmp;
  for (int q = 0; q < 3; q++) {
    const potentialarray_t *t = tabs[q];
    double *tv = dalloc<double>(t->n + 3, &err);
    if (err) return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed for Chebyshev fit");
    tmp.push_back(tv);
    cudaMemcpyAsync(tv, t->values - 1, sizeof(double) * (t->n + 3), cudaMemcpyHostToDevice,
                    h->stream);
    launch_cheb_fit(tv + 1, t->x0, t->xn, t->invDx, CG_NCHEB, d + q * CG_NCHEB,
                    d + (3 + q) * CG_NCHEB, h->stream);
    a[q] = a[q + 3] = t->x0;
    b[q] = b[q + 3] = t->xn;
  }
  std::vector<double> hbuf(6 * CG_NCHEB);
  CK(cudaMemcpyAsync(hbuf.data(), d, sizeof(double) * 6 * CG_NCHEB, cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int q = 0; q < 6; q++)
    for (int j = 0; j < CG_NCHEB; j++) coef[q][j] = hbuf[q * CG_NCHEB + j];
  cudaFree(d);
  for (double *p : tmp) cudaFree(p);
  return 0;
}

int setup_potential(comdgb_sim *h, const simflat_t *s) {
  int err = 0;
  const comdgb_opts &o = h->opts;
  if (o.potential < 0) return 0;  // binning-only simulation
  if (!s->pot) return set_err(COMDGB_ERR_ARG, "simflat_t has no potential");
  h->cutoff = s->pot->cutoff;
  h->rmass = (double)(kAmuToMe * (double)s->pot->mass);
  if (o.potential == COMDGB_POT_LJ) {
    const ljpotential_t *lp = (const ljpotential_t *)s->pot;
    install_lj(h, lp->epsilon, lp->sigma, lp->cutoff);
    return 0;
  }
  const eampotential_t *ep = (const eampotential_t *)s->pot;
  if (!ep->phi || !ep->rho || !ep->f) return set_err(COMDGB_ERR_ARG, "EAM tables missing");
  double rc2 = h->cutoff * h->cutoff;
  if (o.potential == COMDGB_POT_EAM_TABLE) {
    h->eam64t.phi = upload_table<double>(h, ep->phi, &err);
    h->eam64t.rho = upload_table<double>(h, ep->rho, &err);
    h->eam64t.f = upload_table<double>(h, ep->f, &err);
    h->eam64t.rc2 = rc2;
    h->eam32t.phi = upload_table<float>(h, ep->phi, &err);
    h->eam32t.rho = upload_table<float>(h, ep->rho, &err);
    h->eam32t.f = upload_table<float>(h, ep->f, &err);
    h->eam32t.rc2 = (float)rc2;
    if (err) return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed for EAM tables");
    return 0;
  }
  if (o.potential != COMDGB_POT_EAM_CHEBY)
    return set_err(COMDGB_ERR_ARG, "unknown potential kind %d", o.potential);
  if (o.n_cheby != CG_NCHEB)
    return set_err(COMDGB_ERR_UNSUPPORTED, "only %d Chebyshev terms are supported", CG_NCHEB);
  double coef[6][CG_NCHEB], a[6], b[6];
  if (o.cheby_from_host) {
    const eam_cheby_t *ch = s->ch_pot;
    if (!ch) return set_err(COMDGB_ERR_ARG, "cheby_from_host set but s->ch_pot is NULL");
    const potentialarray_t *ser[6] = {ch->phi, ch->rho, ch->f, ch->dphi, ch->drho, ch->df};
    for (int q = 0; q < 6; q++) {
      if (!ser[q] || ser[q]->n != CG_NCHEB)
        return set_err(COMDGB_ERR_UNSUPPORTED, "Chebyshev series %d must have %d terms", q,
                       CG_NCHEB);
      for (int j = 0; j < CG_NCHEB; j++) coef[q][j] = ser[q]->values[j];
      a[q] = ser[q]->x0;
      b[q] = ser[q]->xn;
    }
  } else {
    int rc = fit_cheb_gpu(h, ep, coef, a, b);
    if (rc) return rc;
  }
  h->pair_lo = ep->lat > 0 ? 0.75 * ep->lat / sqrt(2.0) : 0.0;
  h->eam64c.rc2 = rc2;
  h->eam32c.rc2 = (float)rc2;
  return install_cheby(h, coef, a, b);
}

}  // namespace cgapi

// the captured graphs hold the potentials by value
void cgapi::drop_graphs(comdgb_sim *h) {
  if (h->loop_exec) cudaGraphExecDestroy(h->loop_exec);
  h->loop_exec = nullptr;
  if (h->step_exec) cudaGraphExecDestroy(h->step_exec);
  if (h->force_exec) cudaGraphExecDestroy(h->force_exec);
  if (h->force_exec_tracked) cudaGraphExecDestroy(h->force_exec_tracked);
  if (h->force_exec_host) cudaGraphExecDestroy(h->force_exec_host);
  if (h->timed_exec) cudaGraphExecDestroy(h->timed_exec);
  if (h->timed_graph) cudaGraphDestroy(h->timed_graph);
  h->step_exec = h->force_exec = h->force_exec_tracked = h->force_exec_host = h->timed_exec =
      nullptr;
  h->timed_graph = nullptr;
  for (cudaGraphExec_t &x : h->part_exec) {
    if (x) cudaGraphExecDestroy(x);
    x = nullptr;
  }
}

// ljForce.c:75-86 parameters (sigma^6 forms of the pair terms)
void cgapi::install_lj(comdgb_sim *h, double eps, double sigma, double cutoff) {
  const double s6 = sigma * sigma * sigma * sigma * sigma * sigma;
  h->lj_eps = eps;
  h->lj_sigma = sigma;
  h->lj_s6 = s6;
  h->lj64 = LjPot<double>{s6, 12.0 * s6, 4.0 * eps * s6, cutoff * cutoff};
  h->lj32 = LjPot<float>{(float)s6, (float)(12.0 * s6), (float)(4.0 * eps * s6),
                         (float)(cutoff * cutoff)};
  drop_graphs(h);
}

// series order 0 phi, 1 rho, 2 F, 3 dphi, 4 drho, 5 dF.  Pair distances below
// 0.75 of the nearest-neighbour distance of the potential's lattice
// (h->pair_lo) take the reference coefficients in FP32 (never in practice).
int cgapi::install_cheby(comdgb_sim *h, const double coef[6][CG_NCHEB], const double a[6],
                         const double b[6]) {
  fill_cheb(h->eam64c.ch, h->eam32c.ch, h->eam32c.chlo, coef, a, b, h->pair_lo);
  if (build_pair_seg(h, coef, a, b, h->pair_lo, h->cutoff, &h->seg_built))
    return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed for the pair segment table");
  h->eam32c.seg = h->pair_table_off ? no_pair_seg() : h->seg_built;
  for (int q = 0; q < 6; q++) {
    for (int j = 0; j < CG_NCHEB; j++) h->cheb_coef[q][j] = coef[q][j];
    h->cheb_a[q] = a[q];
    h->cheb_b[q] = b[q];
  }
  drop_graphs(h);
  return 0;
}

namespace cgapi {

int read_status(comdgb_sim *h, int *st) {
  CK(cudaMemcpyAsync(st, h->status, sizeof(int) * ST_COUNT, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int check_status(comdgb_sim *h) {
  int st[ST_COUNT];
  int rc = read_status(h, st);
  if (rc) return rc;
  if (st[ST_ERROR] == COMDGB_ERR_MAXATOMS)
    return set_err(COMDGB_ERR_MAXATOMS, "Increase maxatoms: a box reached %d atoms",
                   CG_MAXATOMS);
  if (st[ST_ERROR] == COMDGB_ERR_BOXRANGE)
    return set_err(COMDGB_ERR_BOXRANGE, "an atom's box index fell outside the grid");
  if (st[ST_ERROR] == COMDGB_ERR_ARG)
    return set_err(COMDGB_ERR_ARG, "atom ids must be 0..ntot-1, each once (persistent lists)");
  if (st[ST_ERROR]) return set_err(st[ST_ERROR], "device error %d", st[ST_ERROR]);
  return 0;
}

// ---- kernel groups of one step --------------------------------------------

// groups of the graph comdgb_sim_timed_steps times: a whole step, the
// middle part of a merged sequence, or that of a force-order sequence
int group_count(const comdgb_sim *h) {
  if (!h->merge_rebox) return KG_COUNT;
  return h->fo.list ? KGF_COUNT : KGM_COUNT;
}

// lazy: the rebox only when a list rebuild is due (see enqueue_step)
void enqueue_classify_finish(comdgb_sim *h, bool lazy = false) {
  launch_rebin_finish(h->g, h->s, h->mixed, h->w, h->status, h->stream,
                      lazy ? h->status : nullptr);
}

void enqueue_force_parts(comdgb_sim *h, cudaEvent_t *ev, int &evi, bool obs = true,
                         bool host_out = false) {
  // ev (optional) records after each group: compact, nbr, pass1, pass2.
  // obs = false: a force call inside a step sequence, whose energies, stress,
  // rho and F' the next force call overwrites before the caller can read
  // them (the force-order passes then compute forces only).  host_out: the
  // force-order passes also write f, rho and F' into the attached host
  // arrays (zero-copy), so no download follows the call.
  ForceArgs A = force_args(h);
  if (host_out && h->fo.list) {
    A.host_f = h->hs.f;
    A.host_rho = h->hs.rho;
    A.host_fi = h->hs.fi;
  }
  cudaStream_t st = h->stream;
  cudaMemsetAsync(h->status + ST_DELTA, 0, sizeof(int), st);  // f is about to hold forces
  launch_compact(h->g, h->s.natoms, h->box_start, h->atom_slot, h->ntot, h->cpart, h->ncpart,
                 st);
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
  const int pot = h->opts.potential;
  // persistent lists are built with rc + skin, and only when a rebuild is due
  const double rcl = h->cutoff + h->skin;
  if (h->fo.list) {
    // force order (positions were placed by the half step before, or by
    // fo_track): the list build if due, then the passes
    launch_nbr_build<float>(A, (float)(rcl * rcl), st, &h->tune);
    launch_rebuild_done(h->status, st);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    if (pot == COMDGB_POT_LJ) {
      launch_fo_lj(A, h->lj32, st, obs);
      if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    } else if (pot == COMDGB_POT_EAM_TABLE) {
      launch_fo_eam<EVAL_TABLE>(A, h->eam32t, 0, st, &h->tune, obs);
      if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
      launch_fo_eam<EVAL_TABLE>(A, h->eam32t, 1, st, &h->tune, obs);
    } else {
      launch_fo_eam<EVAL_CHEBY>(A, h->eam32c, 0, st, &h->tune, obs);
      if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
      launch_fo_eam<EVAL_CHEBY>(A, h->eam32c, 1, st, &h->tune, obs);
    }
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    return;
  }
  if (h->mixed) {
    float rc2 = h->pl.vlist ? (float)(rcl * rcl)
                            : (pot == COMDGB_POT_LJ ? h->lj32.rc2 : (float)(h->cutoff * h->cutoff));
    launch_nbr_build<float>(A, rc2, st);
  } else {
    double rc2 = h->pl.vlist ? rcl * rcl
                             : (pot == COMDGB_POT_LJ ? h->lj64.rc2 : h->cutoff * h->cutoff);
    launch_nbr_build<double>(A, rc2, st);
  }
  if (h->pl.vlist) launch_rebuild_done(h->status, st);
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
  if (pot == COMDGB_POT_LJ) {
    if (h->mixed) launch_lj<float>(A, h->lj32, st);
    else launch_lj<double>(A, h->lj64, st);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    return;
  }
  if (pot == COMDGB_POT_EAM_TABLE) {
    if (h->mixed) launch_eam_pass1<float, EVAL_TABLE>(A, h->eam32t, st);
    else launch_eam_pass1<double, EVAL_TABLE>(A, h->eam64t, st);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    if (h->mixed) launch_eam_pass2<float, EVAL_TABLE>(A, h->eam32t, st);
    else launch_eam_pass2<double, EVAL_TABLE>(A, h->eam64t, st);
  } else {
    if (h->mixed) launch_eam_pass1<float, EVAL_CHEBY>(A, h->eam32c, st);
    else launch_eam_pass1<double, EVAL_CHEBY>(A, h->eam64c, st);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    if (h->mixed) launch_eam_pass2<float, EVAL_CHEBY>(A, h->eam32c, st);
    else launch_eam_pass2<double, EVAL_CHEBY>(A, h->eam64c, st);
  }
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
}

int count_kernel_nodes(cudaGraph_t graph);

// Under stream capture of h->stream: a kernel that sets a new conditional
// handle to "status word `word` is set" (word < 0: the end of a possible
// rebuild and "a current list overflowed", rebuild_done_cond_kernel), then
// an IF node after it whose body is captured on h->cond_stream until
// cond_end.  Returns that stream, or nullptr when h->stream is not capturing
// or the node cannot be made (the caller then enqueues the body on
// h->stream, where its kernels stand down by themselves; with word < 0 it
// also launches rebuild_done itself).
cudaStream_t cond_begin(comdgb_sim *h, int word) {
  // COMDGB_GRAPH_CONDITIONALS=0: no conditional nodes (the sections stand
  // down by themselves instead).  ncu profiles no kernel of a graph that
  // holds a conditional node, so the launch lists are taken with this set.
  static const bool off = [] {
    const char *e = getenv("COMDGB_GRAPH_CONDITIONALS");
    return e && e[0] == '0';
  }();
  if (off) return nullptr;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  if (!h->cond_stream ||
      cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, &graph, &deps, nullptr, &nd) !=
          cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return nullptr;
  cudaGraphConditionalHandle cond;
  if (cudaGraphConditionalHandleCreate(&cond, graph, 0, cudaGraphCondAssignDefault) !=
      cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (word < 0) launch_rebuild_done_cond(h->status, cond, h->stream);
  else launch_status_cond(cond, h->status, word, h->stream);
  if (cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, &graph, &deps, nullptr, &nd) !=
      cudaSuccess)
    return nullptr;
  std::vector<cudaGraphNode_t> dv(deps, deps + nd);
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = cond;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, graph, dv.data(), nullptr, dv.size(), &p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;  // the handle stays unused
  }
  if (cudaStreamUpdateCaptureDependencies(h->stream, &node, nullptr, 1,
                                          cudaStreamSetCaptureDependencies) != cudaSuccess ||
      cudaStreamBeginCaptureToGraph(h->cond_stream, p.conditional.phGraph_out[0], nullptr,
                                    nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return nullptr;  // (an error the end of the capture of h->stream reports)
  return h->cond_stream;
}

// ends the body's capture; its kernel nodes
int cond_end(comdgb_sim *h) {
  cudaGraph_t body = nullptr;
  if (cudaStreamEndCapture(h->cond_stream, &body) == cudaSuccess && body)
    return count_kernel_nodes(body);
  return 0;
}

// Inside a force-order step sequence the force pass makes the next step's
// velocity step and position half steps (ST_FUSE), except in the sequence's
// last force call: the closing part makes that step's own.  n steps: set
// before the opening part, cleared before the last middle part.
void set_fuse(comdgb_sim *h, bool on, cudaStream_t st = nullptr) {
  if (h->fo.list)
    cudaMemsetAsync(h->status + ST_FUSE, on ? 1 : 0, sizeof(int), st ? st : h->stream);
}

// The force call of a force-order step part (OPEN or MID, mixed precision):
// the rebuild section -- classify, rebin, compact and the list build, all
// needed only when an atom moved more than skin/2 since the build -- as the
// body of a conditional node; the slot-order FP32 copy refreshed (another
// conditional node) when a list overflowed, since only the stencil scan of
// an overflowed list reads it and the fused update does not keep it; then
// the passes without energies, the force pass with the update of the step
// boundary when ST_FUSE is set (dt_atu: the step).  ev: events after the
// rebuild section and after each pass.
void enqueue_fo_step_force(comdgb_sim *h, double dt_atu, cudaEvent_t *ev, int &evi) {
  ForceArgs A = force_args(h);
  A.vv_dt = dt_atu;
  const double dt_r = dt_atu / 2.0;
  A.vv_c = 2.0 * dt_r / h->rmass;  // both half steps, as one multiply-add
  cudaStream_t st = h->stream;
  cudaStream_t bs = cond_begin(h, ST_REBUILD);
  cudaStream_t rs = bs ? bs : st;
  cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), rs);
  launch_classify(h->g, h->s, h->atom_slot, h->ntot, h->mixed, h->w, h->status, rs, h->status);
  launch_rebin_finish(h->g, h->s, h->mixed, h->w, h->status, rs, h->status);
  launch_compact(h->g, h->s.natoms, h->box_start, h->atom_slot, h->ntot, h->cpart, h->ncpart,
                 rs, h->status);
  const double rcl = h->cutoff + h->skin;
  launch_nbr_build<float>(A, (float)(rcl * rcl), rs, &h->tune);
  if (bs) h->rebuild_kernels = cond_end(h);
  // (mixed precision keeps no position increments in f: ST_DELTA stays 0)
  cudaStream_t os = cond_begin(h, -1);
  if (!os) launch_rebuild_done(h->status, st);
  launch_pos32(h->g, h->s, os ? os : st, h->status);
  if (os) h->overflow_kernels = cond_end(h);
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
  const int pot = h->opts.potential;
  if (pot == COMDGB_POT_LJ) {
    launch_fo_lj(A, h->lj32, st, false);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
  } else if (pot == COMDGB_POT_EAM_TABLE) {
    launch_fo_eam<EVAL_TABLE>(A, h->eam32t, 0, st, &h->tune, false);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    launch_fo_eam<EVAL_TABLE>(A, h->eam32t, 1, st, &h->tune, false);
  } else {
    launch_fo_eam<EVAL_CHEBY>(A, h->eam32c, 0, st, &h->tune, false);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    launch_fo_eam<EVAL_CHEBY>(A, h->eam32c, 1, st, &h->tune, false);
  }
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
}

void enqueue_reduce(comdgb_sim *h) {
  ForceArgs A = force_args(h);
  launch_reduce(A, h->rpart, h->ripart, h->nrpart, h->d_out, h->d_iout, h->stream);
  if (h->nrep > 1) launch_rep_reduce(A, h->rep_out, h->stream);
}

// atom list (atom -> slot) of the current layout
void enqueue_compact(comdgb_sim *h) {
  launch_compact(h->g, h->s.natoms, h->box_start, h->atom_slot, h->ntot, h->cpart, h->ncpart,
                 h->stream);
}

void enqueue_rebox(comdgb_sim *h) {
  cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), h->stream);
  launch_classify(h->g, h->s, h->atom_slot, h->ntot, h->mixed, h->w, h->status, h->stream);
  enqueue_classify_finish(h);
  enqueue_compact(h);
}

// one velocity-Verlet step (timestep.c:129-132); ev: optional group events.
// part: the whole step (PART_FULL), or with the rebox merged one of
// PART_OPEN (position half step, rebox, force), PART_MID (velocity step, the
// closing position half step and the opening one of the next step, one
// rebox, force) and PART_CLOSE (velocity step, position half step, rebox):
// n steps are OPEN, n-1 MID, CLOSE.
// Force order (mixed precision, skin lists) reads no layout between list
// builds -- the passes walk the lists with positions relative to the build
// boxes -- so the OPEN and MID parts rebox (and recompact) only when a
// rebuild is due; until then atoms keep their boxes and slots, a little
// outside them.  The CLOSE part always reboxes, so a call ends boxed.
void enqueue_step(comdgb_sim *h, double dt_atu, cudaEvent_t *ev, int part) {
  int evi = 0;
  cudaStream_t st = h->stream;
  const bool lazy = h->fo.list && (part == PART_OPEN || part == PART_MID);
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
  if (lazy) {
    // force order: the opening position half step; a middle part's update
    // was made by the force pass before it (ST_FUSE); the classification,
    // rebox and list build only when a rebuild is due
    if (part == PART_OPEN)
      launch_advance_positions(h->g, h->s, h->atom_slot, h->ntot, dt_atu / 2.0, h->rmass,
                               h->mixed, false, h->w, h->status, st, true);
    enqueue_fo_step_force(h, dt_atu, ev, evi);
    return;
  }
  if (part != PART_CLOSE) {
    // the atom list is the one made after the previous rebin
    cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), st);
    if (part == PART_MID)
      launch_advance_vpp(h->g, h->s, h->atom_slot, h->ntot, dt_atu, dt_atu / 2.0, h->rmass,
                         h->mixed, h->w, h->status, st, true);
    else
      launch_advance_positions(h->g, h->s, h->atom_slot, h->ntot, dt_atu / 2.0, h->rmass,
                               h->mixed, true, h->w, h->status, st, true);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    enqueue_classify_finish(h);
    if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
    // inside the sequence (OPEN, MID): the CLOSE part and the force call
    // that ends nTimeSteps follow, so nothing reads this call's energies
    enqueue_force_parts(h, ev, evi, part == PART_FULL);  // the atom list of the new layout
    if (part != PART_FULL) return;
  }
  cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), st);
  // the closing part writes the FP32 copies and the force-order tracking for
  // the force call that ends the sequence
  launch_advance_vp(h->g, h->s, h->atom_slot, h->ntot, dt_atu, dt_atu / 2.0, h->rmass, h->mixed,
                    h->w, h->status, st, h->mixed && part == PART_CLOSE);
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
  enqueue_classify_finish(h);
  enqueue_compact(h);
  if (ev) cudaEventRecordWithFlags(ev[evi++], st, cudaEventRecordExternal);
}

int count_kernel_nodes(cudaGraph_t graph) {
  size_t nn = 0;
  if (cudaGraphGetNodes(graph, nullptr, &nn) != cudaSuccess) return -1;
  std::vector<cudaGraphNode_t> nodes(nn);
  if (cudaGraphGetNodes(graph, nodes.data(), &nn) != cudaSuccess) return -1;
  int k = 0;
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

// part: the step part to capture, or PART_NONE; force: then a force call
// (tracked: after a closing part, which wrote the FP32 copies and the
// force-order tracking itself)
int capture(comdgb_sim *h, cudaGraphExec_t *exec, double dt_atu, int part, bool force,
            bool tracked = false, bool host_out = false) {
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const bool step = part != PART_NONE;
  if (step) enqueue_step(h, dt_atu, nullptr, part);
  if (force) {
    int evi = 0;
    // the last half step of a step leaves the FP32 copy stale (unless the
    // closing part of a merged sequence wrote it)
    if (h->mixed && !tracked) launch_pos32(h->g, h->s, h->stream);
    if (h->pl.vlist) launch_skin_check(h->g, h->s, h->pl, h->mixed, h->status, h->stream);
    if (h->fo.list && !tracked)
      launch_fo_track(h->g, h->s, h->fo, h->atom_slot, h->ntot, h->status, h->stream);
    enqueue_force_parts(h, nullptr, evi, true, host_out);
    enqueue_reduce(h);
  }
  CK(cudaStreamEndCapture(h->stream, &graph));
  if (part == PART_FULL || part == PART_MID) h->step_kernels = count_kernel_nodes(graph);
  if (part >= PART_OPEN && part <= PART_CLOSE) h->part_kernels[part] = count_kernel_nodes(graph);
  if (force) h->force_kernels = count_kernel_nodes(graph);
  if (*exec) cudaGraphExecDestroy(*exec);
  cudaError_t e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  // on the device now, conditional bodies included, not at a first launch
  if (e == cudaSuccess) e = cudaGraphUpload(*exec, h->stream);
  if (e != cudaSuccess)
    return set_err(COMDGB_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  return 0;
}

int finish_force(comdgb_sim *h) {
  double out[2];
  long long iout;
  CK(cudaMemcpyAsync(out, h->d_out, sizeof(double) * 2, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(&iout, h->d_iout, sizeof(long long), cudaMemcpyDeviceToHost, h->stream));
  int rc = check_status(h);
  if (rc) return rc;
  (void)iout;
  const double escale = h->opts.potential == COMDGB_POT_LJ ? 4.0 * h->lj_eps * h->lj_s6 : 1.0;
  h->e = h->opts.potential == COMDGB_POT_LJ ? out[0] * escale : out[0];
  h->stress = out[1] / h->volume;
  if (h->nrep > 1) {
    std::vector<double> ro(2 * (size_t)h->nrep);
    CK(cudaMemcpy(ro.data(), h->rep_out, sizeof(double) * ro.size(), cudaMemcpyDeviceToHost));
    h->rep_e.resize(h->nrep);
    h->rep_stress.resize(h->nrep);
    for (int r = 0; r < h->nrep; r++) {
      h->rep_e[r] = h->opts.potential == COMDGB_POT_LJ ? ro[2 * r] * escale : ro[2 * r];
      h->rep_stress[r] = ro[2 * r + 1] / h->volumes[r];
    }
  }
  if (!std::isfinite(h->e)) return set_err(COMDGB_ERR_NONFINITE, "total energy is %g", h->e);
  h->lists_built = h->pl.slot_of != nullptr;  // a force call builds them when due
  return 0;
}

// the force call graph; after_steps: the one that ends a step sequence
// (with the rebox merged in mixed precision the closing part already wrote
// the FP32 copies and the tracking, so that graph skips them)
// host_out: the force-order passes write f, rho and F' straight into the
// attached host arrays (only with `tracked`, in force order)
int force_graph(comdgb_sim *h, bool after_steps, cudaGraphExec_t *out, bool host_out = false) {
  const bool tracked = after_steps && h->merge_rebox && h->mixed;
  host_out = host_out && tracked && h->fo.list;
  cudaGraphExec_t *exec = host_out  ? &h->force_exec_host
                          : tracked ? &h->force_exec_tracked
                                    : &h->force_exec;
  if (!*exec) {
    int rc = capture(h, exec, 0.0, PART_NONE, true, tracked, host_out);
    if (rc) return rc;
  }
  *out = *exec;
  return 0;
}

int do_force_ex(comdgb_sim *h, bool after_steps) {
  if (h->opts.potential < 0) return set_err(COMDGB_ERR_ARG, "simulation has no potential");
  cudaGraphExec_t exec = nullptr;
  int rc = force_graph(h, after_steps, &exec);
  if (rc) return rc;
  CK(cudaGraphLaunch(exec, h->stream));
  return finish_force(h);
}

int do_force(comdgb_sim *h) { return do_force_ex(h, false); }

// n steps as one captured graph (captured once per n and dt), launched once
// between two events; *ms = the graph's device time.  Then the force call
// that ends nTimeSteps.
int do_steps_graph(comdgb_sim *h, int n, double dt, float *ms) {
  if (h->opts.potential < 0) return set_err(COMDGB_ERR_ARG, "simulation has no potential");
  const double dt_atu = dt * kBohrPerAtu;
  if (!h->loop_exec || h->loop_n != n || h->loop_dt != dt_atu) {
    if (h->loop_exec) cudaGraphExecDestroy(h->loop_exec);
    h->loop_exec = nullptr;
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    if (!h->merge_rebox)
      for (int i = 0; i < n; i++) enqueue_step(h, dt_atu, nullptr, PART_FULL);
    else if (n > 0) {
      set_fuse(h, n > 1);
      enqueue_step(h, dt_atu, nullptr, PART_OPEN);
      for (int i = 1; i < n; i++) {
        if (i == n - 1) set_fuse(h, false);
        enqueue_step(h, dt_atu, nullptr, PART_MID);
      }
      enqueue_step(h, dt_atu, nullptr, PART_CLOSE);
    }
    CK(cudaStreamEndCapture(h->stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&h->loop_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e == cudaSuccess) e = cudaGraphUpload(h->loop_exec, h->stream);
    if (e != cudaSuccess)
      return set_err(COMDGB_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    h->loop_n = n;
    h->loop_dt = dt_atu;
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, h->stream));
  CK(cudaGraphLaunch(h->loop_exec, h->stream));
  CK(cudaEventRecord(e1, h->stream));
  CK(cudaEventSynchronize(e1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t;
  int rc = check_status(h);
  return rc ? rc : do_force_ex(h, n > 0);
}

// the step graphs for dt_atu: one step, or the three parts with the rebox
// merged
int ensure_step_graphs(comdgb_sim *h, double dt_atu) {
  const bool have = h->merge_rebox ? h->part_exec[0] && h->part_exec[1] && h->part_exec[2]
                                   : h->step_exec != nullptr;
  if (have && h->graph_dt == dt_atu) return 0;
  int rc = 0;
  if (h->merge_rebox)
    for (int p = 0; p < 3 && !rc; p++) rc = capture(h, &h->part_exec[p], dt_atu, PART_OPEN + p, false);
  else
    rc = capture(h, &h->step_exec, dt_atu, PART_FULL, false);
  if (!rc) h->graph_dt = dt_atu;
  return rc;
}

// n steps on stream st from the graphs ensure_step_graphs made
int launch_steps(comdgb_sim *h, int n, cudaStream_t st) {
  if (n <= 0) return 0;
  if (!h->merge_rebox) {
    for (int i = 0; i < n; i++) CK(cudaGraphLaunch(h->step_exec, st));
    return 0;
  }
  set_fuse(h, n > 1, st);
  CK(cudaGraphLaunch(h->part_exec[0], st));
  for (int i = 1; i < n; i++) {
    if (i == n - 1) set_fuse(h, false, st);
    CK(cudaGraphLaunch(h->part_exec[1], st));
  }
  CK(cudaGraphLaunch(h->part_exec[2], st));
  return 0;
}

int do_steps(comdgb_sim *h, int n, double dt) {
  if (h->opts.potential < 0) return set_err(COMDGB_ERR_ARG, "simulation has no potential");
  double dt_atu = dt * kBohrPerAtu;  // timestep.c:126
  if (n > 0) {
    int rc = ensure_step_graphs(h, dt_atu);
    if (!rc) rc = launch_steps(h, n, h->stream);
    if (rc) return rc;
  }
  return do_force_ex(h, n > 0);
}

// ---- host transfers ---------------------------------------------------------

// the host arrays of replica r into its box and slot range (ids offset by
// the replica's first atom)
// Host <-> device copies of slot arrays: a 2D copy with the 64-slot pitch
// moves only the first w slots of every box (w = the largest box
// occupancy), one plain copy when w = 64.  Slots past a box's occupancy are
// never read.  Returns the bytes moved in *bytes.
static cudaError_t slots_copy(void *dst, const void *src, size_t elem, size_t nb, int w,
                              cudaMemcpyKind kind, cudaStream_t st, size_t *bytes) {
  const size_t pitch = elem * CG_MAXATOMS;
  if (w <= 0) {
    *bytes = 0;
    return cudaSuccess;
  }
  if (w >= CG_MAXATOMS) {
    *bytes = pitch * nb;
    return cudaMemcpyAsync(dst, src, pitch * nb, kind, st);
  }
  *bytes = elem * (size_t)w * nb;
  return cudaMemcpy2DAsync(dst, pitch, src, pitch, elem * (size_t)w, nb, kind, st);
}

static int max_occupancy(const int *natoms, size_t nb) {
  int w = 0;
  for (size_t b = 0; b < nb; b++) w = natoms[b] > w ? natoms[b] : w;
  return w;
}

// a slots_copy call on stream st, its bytes added to h->counter
#define CKX(dst, src, elem, nb, w, kind, counter, st)                             \
  do {                                                                            \
    size_t moved_ = 0;                                                            \
    CK(slots_copy(dst, src, elem, nb, w, kind, st, &moved_));                     \
    h->counter += (long long)moved_;                                              \
  } while (0)

// forces: also f, rho and fi (a force call or nTimeSteps recomputes them
// before reading them; reBoxAll and the handle API carry them)
// the attached owner's arrays move by the zero-copy kernels (one replica),
// as long as they are still the arrays registered at attach
bool zero_copy(const comdgb_sim *h, const simflat_t *s) {
  if (!h->zc || h->nrep != 1 || s != h->host) return false;
  const void *now[9] = {s->natoms, s->id, s->iType, s->mass, s->r, s->p, s->f, s->rho, s->fi};
  for (int i = 0; i < 9; i++)
    if (now[i] != h->pinned[i]) return false;
  return true;
}

// bytes per occupied slot: id, itype, mass, r, p / f, rho, fi
constexpr long long kStateBytes = 4 + 4 + 8 + 24 + 24, kForceBytes = 32 + 8 + 8;

int upload_rep(comdgb_sim *h, int r, const simflat_t *s, bool forces = true) {
  cudaStream_t st = h->stream;
  const RepGeo &R = h->reps[r];
  if (s->nboxes != R.nb) return set_err(COMDGB_ERR_ARG, "box count changed");
  if (s->ntot != h->atom0[r + 1] - h->atom0[r]) return set_err(COMDGB_ERR_ARG, "atom count changed");
  const size_t nb = (size_t)R.nb, ns = nb * CG_MAXATOMS, b0 = (size_t)R.box0;
  const size_t s0 = b0 * CG_MAXATOMS, NS = (size_t)h->nslots;
  const cudaMemcpyKind H2D = cudaMemcpyHostToDevice;
  CK(cudaMemcpyAsync(h->s.natoms + b0, s->natoms, nb * sizeof(int), H2D, st));
  h->xfer_h2d += (long long)(nb * sizeof(int));
  if (zero_copy(h, s)) {
    launch_zc_upload(h->hs, h->s, (int)nb, forces, st);
    h->xfer_h2d += (long long)s->ntot * (kStateBytes + (forces ? kForceBytes : 0));
    return 0;
  }
  const int w = max_occupancy(s->natoms, nb);
  CKX(h->s.id + s0, s->id, sizeof(int), nb, w, H2D, xfer_h2d, st);
  if (h->atom0[r]) launch_add_offset(h->s.id + s0, (long)ns, h->atom0[r], st);
  CKX(h->s.itype + s0, s->iType, sizeof(int), nb, w, H2D, xfer_h2d, st);
  CKX(h->s.mass + s0, s->mass, sizeof(double), nb, w, H2D, xfer_h2d, st);
  CKX(h->stage3 + 3 * s0, s->r, 3 * sizeof(double), nb, w, H2D, xfer_h2d, st);
  launch_unpack3(h->stage3 + 3 * s0, h->s.r + s0, (long)ns, st);
  CKX(h->stage3 + 3 * (NS + s0), s->p, 3 * sizeof(double), nb, w, H2D, xfer_h2d, st);
  launch_unpack3(h->stage3 + 3 * (NS + s0), h->s.p + s0, (long)ns, st);
  if (forces) {
    CKX(h->s.f + s0, s->f, 4 * sizeof(double), nb, w, H2D, xfer_h2d, st);
    CKX(h->s.rho + s0, s->rho, sizeof(double), nb, w, H2D, xfer_h2d, st);
    CKX(h->s.fi + s0, s->fi, sizeof(double), nb, w, H2D, xfer_h2d, st);
  }
  return 0;
}

// After the uploads: FP32 copies, status, id maps, atom list.  Persistent
// lists built by an earlier force call stay: they are keyed by atom id (or
// by force-order number, which the id keeps), the maps are redone for the
// uploaded layout, and the skin tests of the next step or force call rebuild
// them if any atom moved more than skin/2 from its build position -- as
// after any step.  Before the first force call a build is due anyway.
int upload_done(comdgb_sim *h) {
  cudaStream_t st = h->stream;
  if (h->mixed) launch_pos32(h->g, h->s, st);
  CK(cudaMemsetAsync(h->status, 0, sizeof(int) * ST_COUNT, st));
  if (h->pl.slot_of) {
    launch_slot_of(h->g, h->s, h->pl, h->ntot, h->status, st);
    if (h->lists_built) {
      if (h->fo.of_id) launch_fo_reslot(h->g, h->s, h->fo, h->ntot, st);
    } else {
      if (h->fo.of_id)
        CK(cudaMemsetAsync(h->fo.of_id, 0xff, sizeof(int) * ((size_t)h->ntot + 1), st));
      CK(cudaMemsetAsync(h->status + ST_REBUILD, 0x01, 1, st));
    }
  }
  enqueue_compact(h);
  CK(cudaGetLastError());
  return 0;
}

int upload(comdgb_sim *h, const simflat_t *s, bool forces = true) {
  if (h->nrep != 1) return set_err(COMDGB_ERR_ARG, "a batch takes comdgb_batch_upload");
  int rc = upload_rep(h, 0, s, forces);
  return rc ? rc : upload_done(h);
}

// After the slot state was replaced on the device: id -> slot maps and a
// list rebuild at the next force call; f holds no position increments.
int relist(comdgb_sim *h) {
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(h->status + ST_DELTA, 0, sizeof(int), st));
  if (h->pl.slot_of) {
    launch_slot_of(h->g, h->s, h->pl, h->ntot, h->status, st);
    if (h->fo.of_id)
      CK(cudaMemsetAsync(h->fo.of_id, 0xff, sizeof(int) * ((size_t)h->ntot + 1), st));
    CK(cudaMemsetAsync(h->status + ST_REBUILD, 0x01, 1, st));
  }
  enqueue_compact(h);
  CK(cudaGetLastError());
  return 0;
}

// a velocity-Verlet step (timestep.c:129-132) as separate launches: the first
// position half step and its rebox, then (after the caller's force call) the
// velocity step, the second position half step and its rebox
int step_first_half(comdgb_sim *h, double dt_atu) {
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), st));
  launch_advance_positions(h->g, h->s, h->atom_slot, h->ntot, dt_atu / 2.0, h->rmass, h->mixed,
                           true, h->w, h->status, st, false);
  enqueue_classify_finish(h);
  enqueue_compact(h);
  CK(cudaGetLastError());
  return check_status(h);
}
int step_second_half(comdgb_sim *h, double dt_atu) {
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), st));
  launch_advance_vp(h->g, h->s, h->atom_slot, h->ntot, dt_atu, dt_atu / 2.0, h->rmass, h->mixed,
                    h->w, h->status, st);
  CK(cudaMemsetAsync(h->status + ST_DELTA, 0, sizeof(int), st));  // not kept across calls
  enqueue_classify_finish(h);
  enqueue_compact(h);
  CK(cudaGetLastError());
  return check_status(h);
}

// a device copy of the slot state (natoms, id, itype, mass, r, p)
int snapshot_alloc(comdgb_sim *h, Snapshot *q) {
  int err = 0;
  size_t ns = (size_t)h->nslots, nb = (size_t)h->g.nboxes;
  q->natoms = track(h, dalloc<int>(nb, &err));
  q->id = track(h, dalloc<int>(ns, &err));
  q->itype = track(h, dalloc<int>(ns, &err));
  q->mass = track(h, dalloc<double>(ns, &err));
  q->r = track(h, dalloc<d4>(ns, &err));
  q->p = track(h, dalloc<d4>(ns, &err));
  return err ? set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed for a state snapshot") : 0;
}
int snapshot_copy(comdgb_sim *h, const Snapshot &q, bool save) {
  size_t ns = (size_t)h->nslots, nb = (size_t)h->g.nboxes;
  cudaStream_t st = h->stream;
  auto cp = [&](void *dev, void *snap, size_t bytes) {
    return save ? cudaMemcpyAsync(snap, dev, bytes, cudaMemcpyDeviceToDevice, st)
                : cudaMemcpyAsync(dev, snap, bytes, cudaMemcpyDeviceToDevice, st);
  };
  CK(cp(h->s.natoms, q.natoms, nb * sizeof(int)));
  CK(cp(h->s.id, q.id, ns * sizeof(int)));
  CK(cp(h->s.itype, q.itype, ns * sizeof(int)));
  CK(cp(h->s.mass, q.mass, ns * sizeof(double)));
  CK(cp(h->s.r, q.r, ns * sizeof(d4)));
  CK(cp(h->s.p, q.p, ns * sizeof(d4)));
  if (save) return 0;
  if (h->mixed) launch_pos32(h->g, h->s, st);
  return relist(h);
}

// f, rho, fi (and e, stress) of replica r
// w: the largest box occupancy of the replica's current layout (-1: read it)
static int replica_width(comdgb_sim *h, int r, int w) {
  if (w >= 0) return w;
  const RepGeo &R = h->reps[r];
  std::vector<int> n((size_t)R.nb);
  if (cudaMemcpyAsync(n.data(), h->s.natoms + R.box0, sizeof(int) * n.size(),
                      cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return CG_MAXATOMS;
  return max_occupancy(n.data(), n.size());
}

// written: the force call already wrote f, rho and F' into the host arrays
int download_forces_rep(comdgb_sim *h, int r, simflat_t *s, int w = -1, bool written = false) {
  cudaStream_t st = h->stream;
  const RepGeo &R = h->reps[r];
  const size_t nb = (size_t)R.nb, s0 = (size_t)R.box0 * CG_MAXATOMS;
  if (written) {
    h->xfer_d2h += (long long)h->ntot * kForceBytes;
  } else if (zero_copy(h, s)) {
    launch_zc_download(h->hs, h->s, (int)nb, false, true, st);
    h->xfer_d2h += (long long)h->ntot * kForceBytes;
  } else {
    w = replica_width(h, r, w);
    const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
    CKX(s->f, h->s.f + s0, 4 * sizeof(double), nb, w, D2H, xfer_d2h, st);
    CKX(s->rho, h->s.rho + s0, sizeof(double), nb, w, D2H, xfer_d2h, st);
    CKX(s->fi, h->s.fi + s0, sizeof(double), nb, w, D2H, xfer_d2h, st);
  }
  CK(cudaStreamSynchronize(st));
  if (h->nrep == 1) {
    s->e = h->e;
    s->stress = h->stress;
  } else {
    s->e = r < (int)h->rep_e.size() ? h->rep_e[r] : 0.0;
    s->stress = r < (int)h->rep_stress.size() ? h->rep_stress[r] : 0.0;
  }
  return 0;
}

int download_rep(comdgb_sim *h, int r, simflat_t *s) {
  cudaStream_t st = h->stream;
  const RepGeo &R = h->reps[r];
  if (s->nboxes != R.nb) return set_err(COMDGB_ERR_ARG, "box count differs");
  const size_t nb = (size_t)R.nb, ns = nb * CG_MAXATOMS, b0 = (size_t)R.box0;
  const size_t s0 = b0 * CG_MAXATOMS, NS = (size_t)h->nslots;
  const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
  CK(cudaMemcpyAsync(s->natoms, h->s.natoms + b0, nb * sizeof(int), D2H, st));
  h->xfer_d2h += (long long)(nb * sizeof(int));
  if (zero_copy(h, s)) {
    launch_zc_download(h->hs, h->s, (int)nb, true, false, st);
    h->xfer_d2h += (long long)h->ntot * kStateBytes;
    return download_forces_rep(h, r, s, -1);
  }
  CK(cudaStreamSynchronize(st));
  const int w = max_occupancy(s->natoms, nb);
  CKX(s->id, h->s.id + s0, sizeof(int), nb, w, D2H, xfer_d2h, st);
  CKX(s->iType, h->s.itype + s0, sizeof(int), nb, w, D2H, xfer_d2h, st);
  CKX(s->mass, h->s.mass + s0, sizeof(double), nb, w, D2H, xfer_d2h, st);
  launch_pack3(h->s.r + s0, h->stage3 + 3 * s0, (long)ns, st);
  CKX(s->r, h->stage3 + 3 * s0, 3 * sizeof(double), nb, w, D2H, xfer_d2h, st);
  launch_pack3(h->s.p + s0, h->stage3 + 3 * (NS + s0), (long)ns, st);
  CKX(s->p, h->stage3 + 3 * (NS + s0), 3 * sizeof(double), nb, w, D2H, xfer_d2h, st);
  int rc = download_forces_rep(h, r, s, w);
  if (rc) return rc;
  const int off = h->atom0[r];
  if (off)
    for (size_t b = 0; b < nb; b++)
      for (int k = 0; k < s->natoms[b]; k++) s->id[b * CG_MAXATOMS + k] -= off;
  return 0;
}

int download_forces(comdgb_sim *h, simflat_t *s) { return download_forces_rep(h, 0, s, -1); }

// nTimeSteps(n) with all results copied back (one replica).  After the last
// step the layout, ids, types, masses, r and p are final: they stream to the
// host by the copy engines on a second stream while the trailing force call
// runs on the first (a kernel there would wait for the force kernels' SMs);
// f, rho and fi follow the force call.
int steps_and_download(comdgb_sim *h, int n, double dt, simflat_t *s) {
  if (h->nrep != 1) return set_err(COMDGB_ERR_ARG, "a batch takes comdgb_batch_download");
  if (h->opts.potential < 0) return set_err(COMDGB_ERR_ARG, "simulation has no potential");
  if (s->nboxes != h->reps[0].nb) return set_err(COMDGB_ERR_ARG, "box count differs");
  if (!h->copy_stream) {
    CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->ev_state, cudaEventDisableTiming));
  }
  const double dt_atu = dt * kBohrPerAtu;  // timestep.c:126
  if (n > 0) {
    int rc = ensure_step_graphs(h, dt_atu);
    if (rc) return rc;
  }
  // the attached arrays registered at attach: the results of the trailing
  // force call go to them from the passes themselves (force order)
  const bool zc = zero_copy(h, s);
  const bool host_out = zc && n > 0 && h->merge_rebox && h->mixed && h->fo.list;
  cudaGraphExec_t force_exec = nullptr;
  {
    int rc = force_graph(h, n > 0, &force_exec, host_out);
    if (rc) return rc;
  }
  cudaStream_t st = h->stream, cs = h->copy_stream;
  {
    int rc = launch_steps(h, n, st);
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev_state, st));
  CK(cudaStreamWaitEvent(cs, h->ev_state, 0));
  const size_t nb = (size_t)h->reps[0].nb, ns = nb * CG_MAXATOMS, NS = (size_t)h->nslots;
  CK(cudaMemcpyAsync(s->natoms, h->s.natoms, nb * sizeof(int), cudaMemcpyDeviceToHost, cs));
  h->xfer_d2h += (long long)(nb * sizeof(int));
  // the attached arrays: the state of the occupied slots by the zero-copy
  // kernel on the copy stream, beside the trailing force call (it needs few
  // of the SMs the L1-bound passes leave, and moves 64 bytes per atom where
  // the 2D copies move 96 per slot up to the fullest box's occupancy)
  if (zc) {
    // (one CTA per SM: the download is bound by the host link, not the SMs)
    launch_zc_download(h->hs, h->s, (int)nb, true, false, cs, h->sms);
    h->xfer_d2h += (long long)h->ntot * kStateBytes;
  }
  CK(cudaGraphLaunch(force_exec, st));  // the trailing force call (timestep.c:139)
  const auto ta = std::chrono::steady_clock::now();
  CK(cudaStreamSynchronize(cs));
  const auto tb = std::chrono::steady_clock::now();
  const int w = max_occupancy(s->natoms, nb);
  if (!zc) {
    const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
    CKX(s->id, h->s.id, sizeof(int), nb, w, D2H, xfer_d2h, cs);
    CKX(s->iType, h->s.itype, sizeof(int), nb, w, D2H, xfer_d2h, cs);
    CKX(s->mass, h->s.mass, sizeof(double), nb, w, D2H, xfer_d2h, cs);
    launch_pack3(h->s.r, h->stage3, (long)ns, cs);
    CKX(s->r, h->stage3, 3 * sizeof(double), nb, w, D2H, xfer_d2h, cs);
    launch_pack3(h->s.p, h->stage3 + 3 * NS, (long)ns, cs);
    CKX(s->p, h->stage3 + 3 * NS, 3 * sizeof(double), nb, w, D2H, xfer_d2h, cs);
  }
  int rc = finish_force(h);
  const auto tc = std::chrono::steady_clock::now();
  if (!rc) rc = download_forces_rep(h, 0, s, w, host_out);
  const auto td = std::chrono::steady_clock::now();
  const cudaError_t e = cudaStreamSynchronize(cs);
  const auto te = std::chrono::steady_clock::now();
  {
    const auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
    char buf[160];
    snprintf(buf, sizeof buf, " (steps %.2f, force %.2f, forces down %.2f, state down %.2f)",
             ms(ta, tb), ms(tb, tc), ms(tc, td), ms(td, te));
    h->trace_note = buf;
  }
  if (!rc && e != cudaSuccess)
    rc = set_err(COMDGB_ERR_CUDA, "state download: %s", cudaGetErrorString(e));
  return rc;
}
int download(comdgb_sim *h, simflat_t *s) {
  if (h->nrep != 1) return set_err(COMDGB_ERR_ARG, "a batch takes comdgb_batch_download");
  return download_rep(h, 0, s);
}

// Persistent lists need the full 27-box stencil of distinct boxes (periodic,
// nbx >= 3), boxes at least rc + skin wide (so a list pair is always in
// neighbouring boxes) and ids 0..ntot-1 (they key the lists).
bool use_persistent_lists(comdgb_sim *h, const simflat_t *const *sims, int nrep,
                          const comdgb_opts *o) {
  if (o->potential < 0 || o->list_mode == COMDGB_LIST_PER_STEP || !o->periodic) return false;
  double bmin = 1e300;
  for (int r = 0; r < nrep; r++) {
    const simflat_t *s = sims[r];
    for (int j = 0; j < 3; j++) {
      if (s->nbx[j] < 3) return false;
      bmin = std::min(bmin, s->boxsize[j]);
    }
    std::vector<char> seen((size_t)s->ntot, 0);
    for (int b = 0; b < s->nboxes; b++)
      for (int k = 0; k < s->natoms[b]; k++) {
        int id = s->id[b * CG_MAXATOMS + k];
        if (id < 0 || id >= s->ntot || seen[id]) return false;
        seen[id] = 1;
      }
  }
  double skin = o->skin > 0.0 ? o->skin : 0.5;
  skin = std::min(skin, bmin - h->cutoff);
  if (!(skin >= 0.1)) return false;
  h->skin = skin;
  return true;
}

// One simulation of nrep replicas (nrep = 1: a plain simulation).  Replica r
// owns global boxes [box0_r, box0_r + nboxes_r), the slots of those boxes and
// atoms [atom0_r, atom0_r + ntot_r) of the compacted order; its ids are
// offset by atom0_r on the device.  All replicas use the potential of the
// first.
int create(const simflat_t *const *sims, int nrep, const comdgb_opts *o, comdgb_sim **out) {
  *out = nullptr;
  if (!sims || !o || nrep < 1) return set_err(COMDGB_ERR_ARG, "null argument");
  long nbt = 0, ntt = 0;
  for (int r = 0; r < nrep; r++) {
    const simflat_t *q = sims[r];
    if (!q) return set_err(COMDGB_ERR_ARG, "null replica %d", r);
    if (q->nboxes < 1 || !q->natoms || !q->r)
      return set_err(COMDGB_ERR_ARG, "simflat_t has no allocated domains");
    for (int j = 0; j < 3; j++) {
      if (q->nbx[j] > 1023) return set_err(COMDGB_ERR_UNSUPPORTED, "more than 1023 boxes per axis");
      // the stencils index boxes by nbx, the arrays hold nboxes: they must agree
      if (q->nbx[j] < 1 || !(q->boxsize[j] > 0.0) || !(q->bounds[j] > 0.0) ||
          !std::isfinite(q->boxsize[j]) || !std::isfinite(q->bounds[j]))
        return set_err(COMDGB_ERR_ARG, "replica %d: box grid (nbx, boxsize, bounds) not set", r);
    }
    if ((long)q->nbx[0] * q->nbx[1] * q->nbx[2] != q->nboxes)
      return set_err(COMDGB_ERR_ARG, "replica %d: nboxes %d is not nbx[0]*nbx[1]*nbx[2]", r,
                     q->nboxes);
    if (r > 0 && q->pot != sims[0]->pot &&
        (!q->pot || !sims[0]->pot || q->pot->cutoff != sims[0]->pot->cutoff))
      return set_err(COMDGB_ERR_ARG, "replica %d has another potential", r);
    nbt += q->nboxes;
    ntt += q->ntot;
  }
  if (nbt * CG_MAXATOMS >= (1L << 31) || ntt >= (1L << 31))
    return set_err(COMDGB_ERR_UNSUPPORTED, "too many boxes");
  const simflat_t *s = sims[0];
  comdgb_sim *h = new comdgb_sim();
  h->opts = *o;
  h->device = o->device;
  h->mixed = o->precision == COMDGB_PREC_MIXED;
  h->merge_rebox = h->mixed;
  cudaError_t ce = cudaSetDevice(o->device);
  if (ce != cudaSuccess) {
    delete h;
    return set_err(COMDGB_ERR_CUDA, "cudaSetDevice(%d): %s", o->device, cudaGetErrorString(ce));
  }
  cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, o->device);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->cond_stream, cudaStreamNonBlocking) != cudaSuccess) {
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return set_err(COMDGB_ERR_CUDA, "cudaStreamCreate failed");
  }
  h->nrep = nrep;
  h->reps.resize(nrep);
  h->atom0.assign(nrep + 1, 0);
  h->volumes.assign(nrep, 0.0);
  int box0 = 0;
  for (int r = 0; r < nrep; r++) {
    const simflat_t *q = sims[r];
    RepGeo &R = h->reps[r];
    R = RepGeo{};
    for (int j = 0; j < 3; j++) {
      R.nbx[j] = q->nbx[j];
      R.bounds[j] = q->bounds[j];
      R.boxsize[j] = q->boxsize[j];
      R.half[j] = 0.5 * q->boxsize[j];
      R.hi[j] = (float)q->boxsize[j];
      R.lo[j] = (float)(q->boxsize[j] - (double)R.hi[j]);
    }
    R.box0 = box0;
    R.nb = q->nboxes;
    box0 += q->nboxes;
    h->atom0[r + 1] = h->atom0[r] + q->ntot;
    R.a0 = h->atom0[r];
    R.na = q->ntot;
    h->volumes[r] = q->bounds[0] * q->bounds[1] * q->bounds[2];
  }
  h->g.nboxes = (int)nbt;
  h->g.periodic = o->periodic;
  h->g.nrep = nrep;
  for (int j = 0; j < 3; j++) {
    h->g.hi0[j] = h->reps[0].hi[j];
    h->g.lo0[j] = h->reps[0].lo[j];
  }
  h->ntot = (int)ntt;
  h->nslots = (int)nbt * CG_MAXATOMS;
  h->volume = h->volumes[0];
  int err = 0;
  size_t nb = (size_t)nbt, ns = (size_t)h->nslots;
  h->rep_d = track(h, dalloc<RepGeo>(nrep, &err));
  h->g.rep = h->rep_d;
  h->g.box_rep = nullptr;
  if (nrep > 1) {
    int *br = track(h, dalloc<int>(nb, &err));
    std::vector<int> hb(nb);
    for (int r = 0; r < nrep; r++)
      for (int b = 0; b < h->reps[r].nb; b++) hb[h->reps[r].box0 + b] = r;
    if (br) cudaMemcpy(br, hb.data(), nb * sizeof(int), cudaMemcpyHostToDevice);
    h->g.box_rep = br;
    h->rep_out = track(h, dalloc<double>(2 * (size_t)nrep, &err));
  }
  if (h->rep_d)
    cudaMemcpy(h->rep_d, h->reps.data(), sizeof(RepGeo) * nrep, cudaMemcpyHostToDevice);
  alloc_slots(h, h->s, true, &err);
  alloc_slots(h, h->w.stage, false, &err);
  h->w.depmask = track(h, dalloc<uint32_t>(4 * nb, &err));
  h->w.arr_lo = reinterpret_cast<int *>(h->w.depmask + 2 * nb);
  h->w.arr_hi = h->w.arr_lo + nb;
  h->w.n_lo = track(h, dalloc<int>(nb, &err));
  h->w.final_len = track(h, dalloc<int>(nb, &err));
  h->w.final_src = track(h, dalloc<uint8_t>(ns, &err));
  h->w.dep_rank = track(h, dalloc<uint8_t>(ns, &err));
  h->w.arr_list = track(h, dalloc<int>(2 * ns, &err));
  h->et.n = track(h, dalloc<int>(nb, &err));
  h->et.box = track(h, dalloc<int>(nb * CG_NNBR, &err));
  h->et.dr64 = track(h, dalloc<d4>(nb * CG_NNBR, &err));
  h->et.dr32 = track(h, dalloc<float4>(2 * nb * CG_NNBR, &err));
  h->dcenter = track(h, dalloc<double>(nb * 3, &err));
  h->boxc = track(h, dalloc<int>(nb, &err));
  h->g.boxc = h->boxc;
  h->box_start = track(h, dalloc<int>(nb + 1, &err));
  h->atom_slot = track(h, dalloc<int>((size_t)h->ntot + 1, &err));
  h->ncpart = compact_partials((int)nbt);
  h->cpart = track(h, dalloc<int>(h->ncpart, &err));
  double rc = s->pot ? s->pot->cutoff : 1.0;
  h->cap = 0;
  for (int r = 0; r < nrep; r++) h->cap = std::max(h->cap, neighbor_capacity(sims[r], rc));
  h->cutoff = rc;
  if (use_persistent_lists(h, sims, nrep, o)) {
    int vcap = 0;
    for (int r = 0; r < nrep; r++)
      vcap = std::max(vcap, neighbor_capacity(sims[r], rc + h->skin));
    const size_t n1 = (size_t)h->ntot + 1;
    h->pl.slot_of = track(h, dalloc<int>(n1, &err));
    if (h->mixed && h->ntot < (1 << 26)) {  // entries hold the neighbour in 26 bits
      // force order: rows padded to whole warps of 32 atoms
      const size_t rows = ((size_t)h->ntot + 31) / 32 * 32;
      h->fo.vcap = vcap;
      h->fo.list = track(h, dalloc<uint32_t>(rows * vcap, &err));
      h->fo.n = track(h, dalloc<int>(n1, &err));
      h->fo.id = track(h, dalloc<int>(n1, &err));
      h->fo.of_id = track(h, dalloc<int>(n1, &err));
      h->fo.ref = track(h, dalloc<float4>(n1, &err));
      h->fo.pos = track(h, dalloc<float4>(n1, &err));
      h->fo.slot = track(h, dalloc<int>(n1, &err));
      h->fo.pf = track(h, dalloc<float4>(n1, &err));
      h->fo.cut = track(h, dalloc<uint32_t>(rows * vcap, &err));
      h->fo.ncut = track(h, dalloc<int>(n1, &err));
      h->fo.emb = track(h, dalloc<float>(n1, &err));
      h->fo.force = track(h, dalloc<float4>(n1, &err));
      const double hs = 0.5 * h->skin - 1e-5;  // FP32 displacements err by < 1e-6 A
      h->fo.half_skin2 = (float)(hs * hs);
    } else {
      h->pl.vcap = vcap;
      h->pl.vlist = track(h, dalloc<int>((size_t)h->ntot * vcap + 4, &err));
      h->pl.vcount = track(h, dalloc<int>(n1, &err));
      h->pl.rref = track(h, dalloc<d4>(n1, &err));
      const double hs = 0.5 * h->skin - 2e-4;
      h->pl.half_skin2 = hs * hs;
    }
    h->w.pl = h->pl;
    if (h->fo.list) {
      h->w.fo = h->fo;
      h->w.map = SlotMap{nullptr, h->fo.of_id, h->fo.slot};
    } else {
      h->w.map = SlotMap{h->pl.slot_of, nullptr, nullptr};
    }
  }
  h->cap_alloc = h->cap;
  h->pl_vcap_alloc = h->pl.vcap;
  h->fo_vcap_alloc = h->fo.vcap;
  // per-step list: built each step, or (persistent lists) left by pass 1
  // (the force-order passes keep their own lists and never read this one)
  h->nbr = track(h, dalloc<uint16_t>((h->fo.list ? 0 : (size_t)h->ntot * h->cap) + 8, &err));
  h->nbr_n = track(h, dalloc<int>((size_t)h->ntot + 1, &err));
  h->atom_stress = track(h, dalloc<double>((size_t)h->ntot + 1, &err));
  h->nrpart = reduce_partials(h->ntot);
  h->rpart = track(h, dalloc<double>(2 * (size_t)h->nrpart, &err));
  h->ripart = track(h, dalloc<long long>(h->nrpart, &err));
  h->d_out = track(h, dalloc<double>(4, &err));
  h->d_iout = track(h, dalloc<long long>(2, &err));
  h->status = track(h, dalloc<int>(ST_COUNT, &err));
  h->stage3 = track(h, dalloc<double>(ns * 6, &err));
  if (err) {
    free_all(h);
    delete h;
    return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed (%zu slots)", ns);
  }
  if (prepare_force_kernels<double>() != cudaSuccess || prepare_force_kernels<float>() != cudaSuccess)
    err = 1;
  cudaMemsetAsync(h->nbr_n, 0, sizeof(int) * ((size_t)h->ntot + 1), h->stream);
  cudaMemsetAsync(h->atom_stress, 0, sizeof(double) * ((size_t)h->ntot + 1), h->stream);
  for (int r = 0; r < nrep; r++)
    cudaMemcpyAsync(h->dcenter + 3 * (size_t)h->reps[r].box0, sims[r]->dcenter,
                    (size_t)h->reps[r].nb * 3 * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  launch_entry_table(h->g, h->dcenter, h->et, h->boxc, h->stream);
  int rc2 = setup_potential(h, s);
  for (int r = 0; r < nrep && !rc2; r++) rc2 = upload_rep(h, r, sims[r]);
  if (!rc2) rc2 = upload_done(h);
  if (!rc2) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc2 = set_err(COMDGB_ERR_CUDA, "setup: %s", cudaGetErrorString(e));
  }
  if (rc2) {
    free_all(h);
    delete h;
    return rc2;
  }
  *out = h;
  return 0;
}

int create(const simflat_t *s, const comdgb_opts *o, comdgb_sim **out) {
  return create(&s, 1, o, out);
}

comdgb_sim *find_attached(const void *s) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  for (comdgb_sim *h : g_attached)
    if (h->host == s) return h;
  return nullptr;
}

void pin_host(comdgb_sim *h, simflat_t *s) {
  size_t ns = (size_t)h->nslots, nb = (size_t)h->g.nboxes;
  struct {
    void *p;
    size_t n;
  } regs[] = {{s->natoms, nb * 4},     {s->id, ns * 4}, {s->iType, ns * 4}, {s->mass, ns * 8},
              {s->r, ns * 24},         {s->p, ns * 24}, {s->f, ns * 32},    {s->rho, ns * 8},
              {s->fi, ns * 8}};
  bool ok = true, done[9] = {};
  for (int i = 0; i < 9; i++) {
    done[i] = cudaHostRegister(regs[i].p, regs[i].n, cudaHostRegisterDefault) == cudaSuccess;
    ok &= done[i];
  }
  cudaGetLastError();
  h->host_pinned = ok;
  for (int i = 0; i < 9; i++) {
    if (!ok && done[i]) cudaHostUnregister(regs[i].p);  // all or none stay registered
    h->pinned[i] = ok ? regs[i].p : nullptr;
  }
  cudaGetLastError();
  // device addresses of the registered arrays (registration maps them)
  void *dp[9] = {};
  bool mapped = ok;
  for (int i = 1; i < 9 && mapped; i++)
    mapped = cudaHostGetDevicePointer(&dp[i], regs[i].p, 0) == cudaSuccess && dp[i];
  cudaGetLastError();
  if (mapped)
    h->hs = HostSlots{(int *)dp[1],    (int *)dp[2],    (double *)dp[3],
                      (double *)dp[4], (double *)dp[5], (double *)dp[6],
                      (double *)dp[7], (double *)dp[8]};
  h->zc = mapped && h->nrep == 1;
}

void unpin_host(comdgb_sim *h, simflat_t *s) {
  (void)s;
  h->zc = false;
  if (!h->host_pinned) return;
  for (void *p : h->pinned)  // the arrays registered at attach
    if (p) cudaHostUnregister(p);
  cudaGetLastError();
  h->host_pinned = false;
}

}  // namespace

// FP32 FMA throughput probe: 8 independent FMA chains per thread
__global__ void fma_probe_kernel(float *out, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = threadIdx.x * 1e-3f + q;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = fmaf(x[q], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  if (s == 1.2345f) out[0] = s;  // keeps the chains live; practically never stores
}

// message for comdgb_last_error from other translation units (C and C++;
// not exported from the library)
extern "C" __attribute__((visibility("hidden"))) int comdgb_internal_set_error(int code,
                                                                                const char *msg) {
  return set_err(code, "%s", msg);
}

// ============================================================================
// exported C ABI
// ============================================================================
extern "C" {

void comdgb_default_opts(comdgb_opts *o) {
  o->potential = COMDGB_POT_EAM_TABLE;
  o->precision = COMDGB_PREC_FP64;
  o->periodic = 1;
  o->device = 0;
  o->n_cheby = CG_NCHEB;
  o->cheby_from_host = 0;
  o->list_mode = COMDGB_LIST_AUTO;
  o->skin = 0.5;
}

int comdgb_round_f32(const double *x, float *y, long n) {
  if ((!x || !y) && n > 0) return set_err(COMDGB_ERR_ARG, "null argument");
  for (long i = 0; i < n; i++) y[i] = d2f_rn(x[i]);
  return 0;
}

int comdgb_fp32_fma_peak(int device, double *tflops) {
  if (!tflops) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(device));
  int nsm = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  float *out = nullptr;
  CK(cudaMalloc(&out, sizeof(float)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 512, blocks = nsm * 4, iters = 4096;
  double best = 0.0;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0);
    fma_probe_kernel<<<blocks, threads>>>(out, iters, 0.9999f, 1e-6f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
    if (ms > 0 && rep > 0) best = fmax(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  CK(cudaGetLastError());
  *tflops = best;
  return 0;
}

int comdgb_last_error(char *buf, int len) {
  if (buf && len > 0) snprintf(buf, (size_t)len, "%s", g_err);
  return (int)strlen(g_err);
}

const char *comdgb_version(void) { return "comdgb 0.1 sm_103a"; }

int comdgb_sim_create(const simflat_t *s, const comdgb_opts *o, comdgb_sim **out) {
  return create(s, o, out);
}

// ---------------------------------------------------------------- batches

int comdgb_batch_create(const simflat_t *const *sims, int n, const comdgb_opts *o,
                        comdgb_sim **out) {
  if (!out) return set_err(COMDGB_ERR_ARG, "null argument");
  return create(sims, n, o, out);
}

int comdgb_batch_replicas(comdgb_sim *h) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  return h->nrep;
}

int comdgb_batch_upload(comdgb_sim *h, int r, const simflat_t *s) {
  if (!h || !s || r < 0 || r >= h->nrep) return set_err(COMDGB_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  int rc = upload_rep(h, r, s);
  if (!rc) rc = upload_done(h);
  if (!rc) CK(cudaStreamSynchronize(h->stream));
  return rc ? rc : check_status(h);
}

int comdgb_batch_download(comdgb_sim *h, int r, simflat_t *s) {
  if (!h || !s || r < 0 || r >= h->nrep) return set_err(COMDGB_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  return download_rep(h, r, s);
}

int comdgb_batch_energies(comdgb_sim *h, double *e, double *stress) {
  if (!h || !e) return set_err(COMDGB_ERR_ARG, "null argument");
  for (int r = 0; r < h->nrep; r++) {
    const bool one = h->nrep == 1;
    e[r] = one ? h->e : (r < (int)h->rep_e.size() ? h->rep_e[r] : 0.0);
    if (stress) stress[r] = one ? h->stress : (r < (int)h->rep_stress.size() ? h->rep_stress[r] : 0.0);
  }
  return 0;
}

void comdgb_sim_destroy(comdgb_sim *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

int comdgb_sim_upload(comdgb_sim *h, const simflat_t *s) {
  if (!h || !s) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  int rc = upload(h, s);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int comdgb_sim_download(comdgb_sim *h, simflat_t *s) {
  if (!h || !s) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  return download(h, s);
}

int comdgb_sim_force(comdgb_sim *h) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  return do_force(h);
}

int comdgb_sim_steps(comdgb_sim *h, int n, double dt) {
  if (!h || n < 0) return set_err(COMDGB_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  return do_steps(h, n, dt);
}

int comdgb_sim_graph_steps(comdgb_sim *h, int n, double dt, float *ms) {
  if (!h || n < 1) return set_err(COMDGB_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  return do_steps_graph(h, n, dt, ms);
}

int comdgb_sim_rebox(comdgb_sim *h) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  enqueue_rebox(h);
  CK(cudaGetLastError());
  return check_status(h);
}

int comdgb_sim_advance_velocity(comdgb_sim *h, double dt) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  launch_advance_velocity(h->g, h->s, h->atom_slot, h->ntot, dt, h->stream);
  CK(cudaGetLastError());
  return check_status(h);
}

int comdgb_sim_advance_positions(comdgb_sim *h, double dt) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  cudaMemsetAsync(h->status + ST_REBIN_SERIAL, 0, sizeof(int), h->stream);
  launch_advance_positions(h->g, h->s, h->atom_slot, h->ntot, dt, h->rmass, h->mixed, true, h->w,
                           h->status, h->stream);
  enqueue_classify_finish(h);
  enqueue_compact(h);
  CK(cudaGetLastError());
  return check_status(h);
}

int comdgb_sim_energy(comdgb_sim *h, double *e, double *stress) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (e) *e = h->e;
  if (stress) *stress = h->stress;
  return 0;
}

int comdgb_sim_kinetic(comdgb_sim *h, double *ek) {
  if (!h || !ek) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  launch_compact(h->g, h->s.natoms, h->box_start, h->atom_slot, h->ntot, h->cpart, h->ncpart,
                 h->stream);
  launch_kinetic(h->g, h->s, h->atom_slot, h->ntot, h->rmass, h->rpart, h->nrpart, h->d_out + 2,
                 h->stream);
  CK(cudaMemcpyAsync(ek, h->d_out + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int comdgb_sim_set_launch(comdgb_sim *h, int build_threads, int build_atoms, int pass2_threads) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (build_threads == 0) build_threads = 128;
  if (build_atoms == 0) build_atoms = 4;
  if (pass2_threads == 0) pass2_threads = 512;
  if ((build_threads != 64 && build_threads != 128 && build_threads != 256) ||
      (build_atoms != 2 && build_atoms != 4 && build_atoms != 8) ||
      (pass2_threads != 128 && pass2_threads != 256 && pass2_threads != 512))
    return set_err(COMDGB_ERR_ARG, "launch shape %d/%d/%d: build threads 64, 128 or 256, "
                   "atoms per load 2, 4 or 8, pass 2 threads 128, 256 or 512",
                   build_threads, build_atoms, pass2_threads);
  CK(cudaSetDevice(h->device));
  h->tune.build_threads = build_threads;
  h->tune.build_atoms = build_atoms;
  h->tune.pass2_threads = pass2_threads;
  const bool fo_eam = h->mixed && h->opts.potential != COMDGB_POT_LJ;
  const int eval = h->opts.potential == COMDGB_POT_EAM_CHEBY ? EVAL_CHEBY : EVAL_TABLE;
  h->tune.pass2_blocks = fo_eam ? fo_pass2_blocks(eval, h->nrep > 1, pass2_threads, true) : 0;
  h->tune.pass2_blocks_fast =
      fo_eam ? fo_pass2_blocks(eval, h->nrep > 1, pass2_threads, false) : 0;
  CK(cudaGetLastError());
  drop_graphs(h);  // recaptured with the new shapes at the next call
  return 0;
}

int comdgb_sim_set_pair_table(comdgb_sim *h, int on) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  h->pair_table_off = !on;
  h->eam32c.seg = h->pair_table_off ? no_pair_seg() : h->seg_built;
  drop_graphs(h);  // the captured kernels hold the table by value
  return 0;
}

int comdgb_sim_set_list_capacity(comdgb_sim *h, int cap) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  const bool fo = h->fo.list != nullptr, pl = h->pl.vlist != nullptr;
  const int alloc = fo ? h->fo_vcap_alloc : pl ? h->pl_vcap_alloc : h->cap_alloc;
  if (cap == 0) cap = alloc;
  if (cap < 1 || cap > alloc)
    return set_err(COMDGB_ERR_ARG, "list capacity %d: 1..%d (0 restores %d)", cap, alloc, alloc);
  CK(cudaSetDevice(h->device));
  if (fo) {
    h->fo.vcap = cap;
    h->w.fo = h->fo;
  } else if (pl) {
    h->pl.vcap = cap;
    h->w.pl = h->pl;
  } else {
    h->cap = cap;
  }
  // the lists in use were laid out for the old capacity: rebuild them
  if (fo || pl) CK(cudaMemsetAsync(h->status + ST_REBUILD, 0x01, 1, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  drop_graphs(h);  // the captured kernels hold the capacity by value
  return 0;
}

int comdgb_sim_list_info(comdgb_sim *h, int *persistent, double *skin, long long *builds) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  const bool pers = h->pl.vlist || h->fo.list;
  if (persistent) *persistent = pers;
  if (skin) *skin = pers ? h->skin : 0.0;
  if (builds) {
    int st[ST_COUNT];
    int rc = read_status(h, st);
    if (rc) return rc;
    *builds = st[ST_REBUILDS];
  }
  return 0;
}

int comdgb_sim_pair_count(comdgb_sim *h, long long *pairs) {
  if (!h || !pairs) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  long long v = 0;
  CK(cudaMemcpyAsync(&v, h->d_iout, sizeof(long long), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  *pairs = v / 2;
  return 0;
}

int comdgb_sim_synchronize(comdgb_sim *h) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int comdgb_sim_graph_kernels(comdgb_sim *h, int *per_step, int *per_force) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (per_step) *per_step = h->step_kernels;
  if (per_force) *per_force = h->force_kernels;
  return 0;
}

int comdgb_sim_step_launches(comdgb_sim *h, int n, long long *launches) {
  if (!h || !launches || n < 0) return set_err(COMDGB_ERR_ARG, "bad argument");
  if (n == 0) {
    *launches = 0;
  } else if (h->merge_rebox) {
    if (!h->part_exec[0]) return set_err(COMDGB_ERR_ARG, "no step has run yet");
    *launches = h->part_kernels[0] + (long long)(n - 1) * h->part_kernels[1] + h->part_kernels[2];
  } else {
    if (!h->step_exec) return set_err(COMDGB_ERR_ARG, "no step has run yet");
    *launches = (long long)n * h->step_kernels;
  }
  return 0;
}

int comdgb_sim_rebuild_launches(comdgb_sim *h, int *kernels) {
  if (!h || !kernels) return set_err(COMDGB_ERR_ARG, "bad argument");
  *kernels = h->rebuild_kernels;
  return 0;
}

const char *comdgb_kernel_name(comdgb_sim *h, int k) {
  if (!h || k < 0 || k >= group_count(h)) return "";
  if (h->merge_rebox) return h->fo.list ? kGroupNameFo[k] : kGroupNameMerged[k];
  return kGroupName[k];
}

int comdgb_sim_set_merge_rebox(comdgb_sim *h, int on) {
  if (!h) return set_err(COMDGB_ERR_ARG, "null handle");
  if (on && !h->mixed) return set_err(COMDGB_ERR_ARG, "the rebox is merged in mixed precision only");
  if ((bool)on != h->merge_rebox) {
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->stream));
    drop_graphs(h);
    h->merge_rebox = on != 0;
  }
  return 0;
}

int comdgb_sim_timed_steps(comdgb_sim *h, int n, double dt, float *step_ms, float *kernel_ms,
                           int max_kernels) {
  if (!h || n <= 0) return set_err(COMDGB_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  double dt_atu = dt * kBohrPerAtu;
  const bool merged = h->merge_rebox;
  // events around the groups of the timed graph: one whole step, or the
  // middle part of a merged sequence (n steps: the opening part, n-1 middle
  // parts, the closing part; the span covers all three)
  const int NG = group_count(h), NE = NG + 1;
  if (merged) {
    int rc = ensure_step_graphs(h, dt_atu);
    if (rc) return rc;
  }
  const int nt = merged ? n - 1 : n;  // launches of the timed graph
  if (!h->timed_exec || h->timed_dt != dt_atu || (int)h->timed_cap_events.size() != NE) {
    for (cudaEvent_t e : h->timed_cap_events) cudaEventDestroy(e);
    h->timed_cap_events.assign(NE, nullptr);
    for (int i = 0; i < NE; i++) CK(cudaEventCreate(&h->timed_cap_events[i]));
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(h, dt_atu, h->timed_cap_events.data(), merged ? PART_MID : PART_FULL);
    CK(cudaStreamEndCapture(h->stream, &graph));
    size_t nn = 0;
    CK(cudaGraphGetNodes(graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
    if (h->timed_exec) cudaGraphExecDestroy(h->timed_exec);
    if (h->timed_graph) cudaGraphDestroy(h->timed_graph);
    h->timed_graph = graph;  // node handles below belong to it
    CK(cudaGraphInstantiate(&h->timed_exec, graph, 0));
    CK(cudaGraphUpload(h->timed_exec, h->stream));
    // map each capture event to its record node in the instantiated graph
    h->timed_nodes.assign(NE, nullptr);
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType t;
      CK(cudaGraphNodeGetType(nd, &t));
      if (t != cudaGraphNodeTypeEventRecord) continue;
      cudaEvent_t ev;
      CK(cudaGraphEventRecordNodeGetEvent(nd, &ev));
      for (int i = 0; i < NE; i++)
        if (h->timed_cap_events[i] == ev) h->timed_nodes[i] = nd;
    }
    h->timed_dt = dt_atu;
  }
  std::vector<cudaEvent_t> evs((size_t)nt * NE);
  for (auto &e : evs) CK(cudaEventCreate(&e));
  cudaEvent_t span0, span1;  // around everything
  CK(cudaEventCreate(&span0));
  CK(cudaEventCreate(&span1));
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaEventRecord(span0, h->stream));
  if (merged) {
    set_fuse(h, n > 1);
    CK(cudaGraphLaunch(h->part_exec[PART_OPEN], h->stream));
  }
  for (int s = 0; s < nt; s++) {
    for (int i = 0; i < NE; i++)
      if (h->timed_nodes[i])
        CK(cudaGraphExecEventRecordNodeSetEvent(h->timed_exec, h->timed_nodes[i],
                                                evs[(size_t)s * NE + i]));
    if (merged && s == nt - 1) set_fuse(h, false);
    CK(cudaGraphLaunch(h->timed_exec, h->stream));
  }
  if (merged) CK(cudaGraphLaunch(h->part_exec[PART_CLOSE], h->stream));
  CK(cudaEventRecord(span1, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  std::vector<double> ksum(NG, 0.0);
  float span = 0.f, timed = 0.f;
  CK(cudaEventElapsedTime(&span, span0, span1));
  cudaEventDestroy(span0);
  cudaEventDestroy(span1);
  if (step_ms) step_ms[n] = span;
  for (int s = 0; s < nt; s++) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, evs[(size_t)s * NE], evs[(size_t)s * NE + NG]));
    if (step_ms) step_ms[s] = ms;
    timed += ms;
    for (int k = 0; k < NG; k++) {
      float km = 0.f;
      CK(cudaEventElapsedTime(&km, evs[(size_t)s * NE + k], evs[(size_t)s * NE + k + 1]));
      ksum[k] += km;
    }
  }
  // merged: the last entry is the opening and closing parts together
  if (merged && step_ms) step_ms[n - 1] = span - timed;
  for (auto &e : evs) cudaEventDestroy(e);
  if (kernel_ms)
    for (int k = 0; k < NG && k < max_kernels; k++)
      kernel_ms[k] = nt > 0 ? (float)(ksum[k] / nt) : 0.f;
  int rc = check_status(h);
  if (rc) return rc;
  // forces of the final positions, as nTimeSteps ends (timestep.c:137)
  rc = do_force_ex(h, true);
  if (rc) return rc;
  return NG;
}

// ---------------------------------------------------------------- drop-in

int comdgb_attach(simflat_t *s, const comdgb_opts *o) {
  if (!s || !o) return set_err(COMDGB_ERR_ARG, "null argument");
  if (find_attached(s)) return set_err(COMDGB_ERR_ARG, "simflat_t already attached");
  comdgb_sim *h = nullptr;
  int rc = create(s, o, &h);
  if (rc) return rc;
  h->host = s;
  pin_host(h, s);
  std::lock_guard<std::mutex> lk(g_reg_mu);
  g_attached.push_back(h);
  return 0;
}

int comdgb_detach(simflat_t *s) {
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  cudaSetDevice(h->device);
  // lazy mode: the host gets the device state before the mirror goes away
  const int rc = h->host_stale ? download(h, s) : 0;
  {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    for (size_t i = 0; i < g_attached.size(); i++)
      if (g_attached[i] == h) {
        g_attached.erase(g_attached.begin() + i);
        break;
      }
  }
  unpin_host(h, s);
  comdgb_sim_destroy(h);
  return rc;
}

// Before a drop-in call: the device state is current (eager mode uploads
// every call; lazy mode only while the host holds the newer state).
// forces: the call reads f, rho and fi as input (reBoxAll carries them; a
// force call and nTimeSteps compute them before reading them)
static int drop_in_enter(comdgb_sim *h, simflat_t *s, bool forces) {
  CK(cudaSetDevice(h->device));
  if (h->lazy && h->dev_valid) return 0;
  int rc = upload(h, s, forces);
  if (!rc) h->dev_valid = true;
  return rc;
}

// After it: eager mode copies the results back (`full`: the whole state,
// else the force outputs); lazy mode only e and stress, and marks the
// host's arrays stale until comdgb_sync_to_host.
static int drop_in_leave(comdgb_sim *h, simflat_t *s, bool full) {
  if (h->lazy) {
    s->e = h->e;
    s->stress = h->stress;
    h->host_stale = true;
    return 0;
  }
  return full ? download(h, s) : download_forces(h, s);
}

int comdgb_force(void *sv) {
  simflat_t *s = (simflat_t *)sv;
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  int rc = drop_in_enter(h, s, false);
  if (!rc) rc = do_force(h);
  if (!rc) rc = drop_in_leave(h, s, false);
  return rc;
}

double comdgb_nTimeSteps(int n, simflat_t *s, double dt) {
  comdgb_sim *h = find_attached(s);
  if (!h) {
    set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
    return NAN;
  }
  // COMDGB_TRACE_CALLS=1: the host time of the call's phases on stderr
  static const bool trace = [] {
    const char *e = getenv("COMDGB_TRACE_CALLS");
    return e && e[0] == '1';
  }();
  const auto t0 = std::chrono::steady_clock::now();
  int rc = drop_in_enter(h, s, false);
  const auto t1 = std::chrono::steady_clock::now();
  if (!rc) rc = h->lazy ? do_steps(h, n, dt) : steps_and_download(h, n, dt, s);
  if (!rc && h->lazy) rc = drop_in_leave(h, s, true);
  if (trace) {
    const auto t2 = std::chrono::steady_clock::now();
    const auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
    fprintf(stderr, "comdgb_nTimeSteps(%d): upload %.2f ms, steps to download %.2f ms%s\n", n,
            ms(t0, t1), ms(t1, t2), h->trace_note.c_str());
  }
  return rc ? NAN : s->e;
}

int comdgb_reBoxAll(simflat_t *s) {
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  int rc = drop_in_enter(h, s, true);
  if (!rc) {
    enqueue_rebox(h);
    rc = check_status(h);
  }
  if (!rc) rc = drop_in_leave(h, s, true);
  return rc;
}

int comdgb_set_lazy(simflat_t *s, int lazy) {
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  CK(cudaSetDevice(h->device));
  if (!lazy && h->host_stale) {  // leaving lazy mode: the host gets the state
    int rc = download(h, s);
    if (rc) return rc;
    h->host_stale = false;
  }
  h->lazy = lazy != 0;
  return 0;
}

int comdgb_transfer_bytes(simflat_t *s, long long *h2d, long long *d2h) {
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  if (h2d) *h2d = h->xfer_h2d;
  if (d2h) *d2h = h->xfer_d2h;
  return 0;
}

int comdgb_sync_to_host(simflat_t *s) {
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  CK(cudaSetDevice(h->device));
  if (!h->dev_valid) return 0;  // nothing ran on the device yet
  int rc = download(h, s);
  if (!rc) h->host_stale = false;
  return rc;
}

int comdgb_sync_to_device(simflat_t *s) {
  comdgb_sim *h = find_attached(s);
  if (!h) return set_err(COMDGB_ERR_NOTATTACHED, "simflat_t is not attached");
  CK(cudaSetDevice(h->device));
  int rc = upload(h, s);
  if (!rc) {
    h->dev_valid = true;
    h->host_stale = false;
  }
  return rc;
}

int comdgb_rebox_host(simflat_t *s, int periodic, int device) {
  comdgb_opts o;
  comdgb_default_opts(&o);
  o.potential = -1;
  o.periodic = periodic;
  o.device = device;
  comdgb_sim *h = nullptr;
  int rc = create(s, &o, &h);
  if (rc) return rc;
  enqueue_rebox(h);
  rc = check_status(h);
  if (!rc) rc = download(h, s);
  comdgb_sim_destroy(h);
  return rc;
}

int comdgb_put_atoms(simflat_t *s, int n, const double *xyz, const double *pxyz,
                     const int *ids, const int *itypes, const double *masses, int device) {
  if (!s || n < 0 || (n > 0 && (!xyz || !pxyz || !ids || !itypes || !masses)))
    return set_err(COMDGB_ERR_ARG, "bad argument");
  comdgb_opts o;
  comdgb_default_opts(&o);
  o.potential = -1;
  o.device = device;
  comdgb_sim *h = nullptr;
  int saved = s->ntot;
  s->ntot = 0;
  int rc = create(s, &o, &h);
  s->ntot = saved;
  if (rc) return rc;
  int err = 0;
  double *dxyz = dalloc<double>((size_t)n * 3, &err), *dp = dalloc<double>((size_t)n * 3, &err);
  double *dm = dalloc<double>(n, &err);
  int *did = dalloc<int>(n, &err), *dty = dalloc<int>(n, &err);
  int *tmp = dalloc<int>((size_t)h->nslots, &err);
  if (err) rc = set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed");
  cudaStream_t st = h->stream;
  if (!rc && n > 0) {
    cudaMemcpyAsync(dxyz, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dp, pxyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dm, masses, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(did, ids, sizeof(int) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dty, itypes, sizeof(int) * n, cudaMemcpyHostToDevice, st);
  }
  if (!rc) {
    launch_bin_atoms(h->g, h->dcenter, h->s, n, dxyz, dp, did, dty, dm, tmp, h->status, st);
    rc = check_status(h);
  }
  if (!rc) {
    h->ntot = n;
    rc = download(h, s);
    s->ntot = n;
  }
  cudaFree(dxyz);
  cudaFree(dp);
  cudaFree(dm);
  cudaFree(did);
  cudaFree(dty);
  cudaFree(tmp);
  comdgb_sim_destroy(h);
  return rc;
}

eam_cheby_t *comdgb_cheb_make(const eampotential_t *p, int n, int device) {
  if (!p || n != CG_NCHEB) {
    set_err(COMDGB_ERR_UNSUPPORTED, "only %d Chebyshev terms are supported", CG_NCHEB);
    return nullptr;
  }
  cudaError_t ce = cudaSetDevice(device);
  comdgb_sim tmp;
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    set_err(COMDGB_ERR_CUDA, "comdgb_cheb_make on device %d: %s", device, cudaGetErrorString(ce));
    return nullptr;
  }
  double coef[6][CG_NCHEB], a[6], b[6];
  int rc = fit_cheb_gpu(&tmp, p, coef, a, b);
  cudaStreamDestroy(tmp.stream);
  tmp.stream = nullptr;
  if (rc) return nullptr;
  eam_cheby_t *c = (eam_cheby_t *)calloc(1, sizeof(eam_cheby_t));
  if (!c) {
    set_err(COMDGB_ERR_NOMEM, "comdgb_cheb_make: out of host memory");
    return nullptr;
  }
  c->cutoff = p->cutoff;
  c->mass = p->mass;
  c->lat = p->lat;
  potentialarray_t **ser[6] = {&c->phi, &c->rho, &c->f, &c->dphi, &c->drho, &c->df};
  for (int q = 0; q < 6; q++) {
    potentialarray_t *pa = (potentialarray_t *)calloc(1, sizeof(potentialarray_t));
    double *v = (double *)malloc(sizeof(double) * n);
    if (!pa || !v) {
      free(pa);
      free(v);
      comdgb_cheb_free(c);
      set_err(COMDGB_ERR_NOMEM, "comdgb_cheb_make: out of host memory");
      return nullptr;
    }
    pa->n = n;
    pa->x0 = a[q];
    pa->xn = b[q];
    pa->invDx = q >= 3 ? 1.0 : 0.0;
    pa->values = v;
    for (int j = 0; j < n; j++) pa->values[j] = coef[q][j];
    *ser[q] = pa;
  }
  return c;
}

void comdgb_cheb_free(eam_cheby_t *c) {
  if (!c) return;
  potentialarray_t *ser[6] = {c->phi, c->rho, c->f, c->dphi, c->drho, c->df};
  for (potentialarray_t *pa : ser)
    if (pa) {
      free(pa->values);
      free(pa);
    }
  free(c);
}

}  // extern "C"
