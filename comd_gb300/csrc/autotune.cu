// autotune.cu -- the batch autotuner: box factor, persistent-list skin and
// the launch shapes of the force-order kernels, chosen by timing every
// candidate on the batch itself, with a cache file so that a system seen
// before on the same GPU is not timed again.  No counterpart in the
// reference (one system, serial loops, no tunable launches).
//
// Search: every (box factor, skin) candidate as a batch of the caller's
// replicas rebinned at that box factor (comdgb_rebin_host), `steps` steps as
// one CUDA graph after a warm-up replay; then at the best pair the list
// build's threads per box (64, 128, 256) and atoms per candidate load (2, 4,
// 8), then the force pass's threads per CTA (128, 256, 512).  Box factors
// at which a box of some replica would pass 64 atoms are skipped (the
// reference aborts there).  No shape or skin changes a result beyond
// summation order; the box factor changes the grid, and with it the
// reference's stress quirks, so the caller decides whether to adopt it.
//
// Cache: a text file, one line per tuned system, "key<TAB>bf skin bt ba pt
// ms"; the key holds the GPU's name and SM count, the replica count, the
// total atom count, the potential and precision, and a hash of every
// replica's size and bounds, of the options and of the candidate lists.
// The last line with the key wins; new results are appended.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sim.h"

using namespace cgapi;

namespace {

uint64_t fnv(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = (const unsigned char *)p;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

std::string tune_key(const simflat_t *const *sims, int n, const comdgb_opts *o,
                     const double *bfs, int nbf, const double *skins, int nskin, int steps) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, o->device);
  uint64_t h = 1469598103934665603ull;
  long long atoms = 0;
  for (int r = 0; r < n; r++) {
    const simflat_t *s = sims[r];
    atoms += s->ntot;
    h = fnv(h, &s->ntot, sizeof s->ntot);
    h = fnv(h, s->bounds, sizeof s->bounds);
    h = fnv(h, &s->defgrad, sizeof s->defgrad);
  }
  const int opt[4] = {o->potential, o->precision, o->periodic, o->list_mode};
  h = fnv(h, opt, sizeof opt);
  h = fnv(h, bfs, sizeof(double) * (size_t)nbf);
  h = fnv(h, skins, sizeof(double) * (size_t)nskin);
  h = fnv(h, &steps, sizeof steps);
  char name[256];
  snprintf(name, sizeof name, "%s", prop.name);
  for (char *c = name; *c; c++)
    if (*c == ' ' || *c == '\t') *c = '_';
  char key[512];
  snprintf(key, sizeof key, "comdgb-tune-1 gpu=%s sm=%d reps=%d atoms=%lld pot=%d prec=%d h=%016llx",
           name, prop.multiProcessorCount, n, atoms, o->potential, o->precision,
           (unsigned long long)h);
  return key;
}

bool cache_lookup(const char *path, const std::string &key, comdgb_tune *t) {
  if (!path || !*path) return false;
  FILE *f = fopen(path, "r");
  if (!f) return false;
  bool found = false;
  char line[1024];
  while (fgets(line, sizeof line, f)) {
    char *tab = strchr(line, '\t');
    if (!tab) continue;
    *tab = 0;
    if (key != line) continue;
    comdgb_tune v{};
    // a line that does not parse, or holds values comdgb_sim_set_launch
    // would refuse (an edited or damaged file), is skipped: the system is
    // tuned again
    if (sscanf(tab + 1, "%lf %lf %d %d %d %lf", &v.box_factor, &v.skin, &v.build_threads,
               &v.build_atoms, &v.pass2_threads, &v.ms_per_step) == 6 &&
        v.box_factor > 0.0 && std::isfinite(v.box_factor) && v.skin > 0.0 &&
        std::isfinite(v.skin) &&
        (v.build_threads == 64 || v.build_threads == 128 || v.build_threads == 256) &&
        (v.build_atoms == 2 || v.build_atoms == 4 || v.build_atoms == 8) &&
        (v.pass2_threads == 128 || v.pass2_threads == 256 || v.pass2_threads == 512)) {
      *t = v;
      found = true;
    }
  }
  fclose(f);
  return found;
}

void cache_store(const char *path, const std::string &key, const comdgb_tune &t) {
  if (!path || !*path) return;
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s\t%.17g %.17g %d %d %d %.9g\n", key.c_str(), t.box_factor, t.skin,
          t.build_threads, t.build_atoms, t.pass2_threads, t.ms_per_step);
  fclose(f);
}

// ms per step of `steps` steps as one graph (after a warm-up replay) of a
// batch of `reps` with options o and launch shapes (0: default); < 0: the
// error code
double time_batch(const std::vector<const simflat_t *> &reps, const comdgb_opts &o, int bt, int ba,
                  int pt, int steps, double dt) {
  comdgb_sim *h = nullptr;
  int rc = comdgb_batch_create(reps.data(), (int)reps.size(), &o, &h);
  if (rc) return rc;
  float ms = 0.f;
  if (bt || ba || pt) rc = comdgb_sim_set_launch(h, bt, ba, pt);
  if (!rc) rc = comdgb_sim_graph_steps(h, steps, dt, &ms);
  if (!rc) rc = comdgb_sim_graph_steps(h, steps, dt, &ms);
  comdgb_sim_destroy(h);
  return rc ? (double)rc : (double)ms / steps;
}

}  // namespace

extern "C" int comdgb_batch_autotune(const simflat_t *const *sims, int n, const comdgb_opts *o,
                                     const double *box_factors, int nbf, const double *skins,
                                     int nskin, int steps, double dt, const char *cache_path,
                                     comdgb_tune *out) {
  if (!sims || n < 1 || !o || !out || nbf < 0 || nskin < 0 || (nbf && !box_factors) ||
      (nskin && !skins) || steps < 1)
    return set_err(COMDGB_ERR_ARG, "comdgb_batch_autotune: bad arguments");
  for (int r = 0; r < n; r++)
    if (!sims[r] || !sims[r]->pot) return set_err(COMDGB_ERR_ARG, "replica %d has no potential", r);
  CK(cudaSetDevice(o->device));
  const double own_bf = sims[0]->bf == 0.0 ? 1.0 : sims[0]->bf;
  const std::vector<double> bf_c = nbf ? std::vector<double>(box_factors, box_factors + nbf)
                                       : std::vector<double>{own_bf};
  const std::vector<double> skin_c = nskin ? std::vector<double>(skins, skins + nskin)
                                           : std::vector<double>{o->skin > 0.0 ? o->skin : 0.5};
  const std::string key = tune_key(sims, n, o, bf_c.data(), (int)bf_c.size(), skin_c.data(),
                                   (int)skin_c.size(), steps);
  comdgb_tune best{};
  if (cache_lookup(cache_path, key, &best)) {
    best.from_cache = 1;
    *out = best;
    return 0;
  }
  best.ms_per_step = INFINITY;
  std::vector<simflat_t *> owned;
  auto free_owned = [&]() {
    for (simflat_t *s : owned) comdgb_sim_free_host(s);
    owned.clear();
  };
  // the replicas at box factor bf (the caller's own at their own factor);
  // false when a box would pass 64 atoms
  auto replicas_at = [&](double bf, std::vector<const simflat_t *> &reps) -> int {
    reps.clear();
    free_owned();
    for (int r = 0; r < n; r++) {
      const double rbf = sims[r]->bf == 0.0 ? 1.0 : sims[r]->bf;
      if (rbf == bf) {
        reps.push_back(sims[r]);
        continue;
      }
      int st = 0;
      simflat_t *c = comdgb_rebin_host(sims[r], bf, &st);
      if (!c) return st;
      owned.push_back(c);
      reps.push_back(c);
    }
    return 0;
  };
  std::vector<const simflat_t *> reps;
  for (double bf : bf_c) {
    const int st = replicas_at(bf, reps);
    if (st == COMDGB_ERR_MAXATOMS || st == COMDGB_ERR_NOBOX) continue;  // not a valid grid
    if (st) {
      free_owned();
      return set_err(st, "comdgb_batch_autotune: rebinning at box factor %g failed", bf);
    }
    for (double skin : skin_c) {
      comdgb_opts oc = *o;
      oc.skin = skin;
      const double ms = time_batch(reps, oc, 0, 0, 0, steps, dt);
      if (ms < 0) {
        free_owned();
        return (int)ms;
      }
      if (ms < best.ms_per_step) {
        best.box_factor = bf;
        best.skin = skin;
        best.ms_per_step = ms;
      }
    }
  }
  if (!std::isfinite(best.ms_per_step)) {
    free_owned();
    return set_err(COMDGB_ERR_ARG,
                   "comdgb_batch_autotune: no box factor keeps every box within 64 atoms");
  }
  // launch shapes at the best box factor and skin
  int rc = replicas_at(best.box_factor, reps);
  if (rc) {
    free_owned();
    return set_err(rc, "comdgb_batch_autotune: rebinning failed");
  }
  comdgb_opts ob = *o;
  ob.skin = best.skin;
  best.build_threads = 128;
  best.build_atoms = 4;
  best.pass2_threads = 512;
  double best_shape = INFINITY;
  for (int bt : {64, 128, 256})
    for (int ba : {2, 4, 8}) {
      const double ms = time_batch(reps, ob, bt, ba, 512, steps, dt);
      if (ms < 0) {
        free_owned();
        return (int)ms;
      }
      if (ms < best_shape) {
        best_shape = ms;
        best.build_threads = bt;
        best.build_atoms = ba;
      }
    }
  for (int pt : {128, 256}) {
    const double ms = time_batch(reps, ob, best.build_threads, best.build_atoms, pt, steps, dt);
    if (ms < 0) {
      free_owned();
      return (int)ms;
    }
    if (ms < best_shape) {
      best_shape = ms;
      best.pass2_threads = pt;
    }
  }
  free_owned();
  best.ms_per_step = best_shape;
  best.from_cache = 0;
  cache_store(cache_path, key, best);
  *out = best;
  return 0;
}

extern "C" int comdgb_sim_apply_tune(comdgb_sim *h, const comdgb_tune *t) {
  if (!h || !t) return set_err(COMDGB_ERR_ARG, "comdgb_sim_apply_tune: null argument");
  return comdgb_sim_set_launch(h, t->build_threads, t->build_atoms, t->pass2_threads);
}
