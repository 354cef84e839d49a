// binning.cuh -- the per-atom and per-box bodies of the device binning
// (n putAtomInBox calls, src-flat/domains.c:237-291, as a counting sort that
// keeps call order within each box).  Shared by comdgb_put_atoms
// (md_kernels.cu) and comdgb_put_atoms_noalloc (noalloc.cu), so the two
// entry points give the same slot order by construction.
#pragma once

#include "common.cuh"

namespace cg {

// one replica's box grid as the binning sees it
struct BinGrid {
  int nbx[3];
  int nboxes;
  double bounds[3], boxsize[3];
};

// Wrap once into the primary period and find the box (domains.c:255-269,
// getBoxIDWorldCoords domains.c:71-82).  ok is false when the wrapped
// coordinate is not in [0, bounds) -- an atom more than one period outside,
// or a NaN or infinite coordinate -- or its box index falls outside the grid.
__device__ __forceinline__ int bin_world_box(const BinGrid &g, const double *in, double *w,
                                             bool &ok) {
  int ib[3];
  ok = true;
  for (int m = 0; m < 3; m++) {
    double x = in[m];
    if (x < 0.0) x += g.bounds[m];
    else if (x >= g.bounds[m]) x -= g.bounds[m];
    w[m] = x;
    if (!(x >= 0.0 && x < g.bounds[m])) ok = false;
    ib[m] = ok ? (int)floor(x / g.boxsize[m]) : 0;
    if (ib[m] < 0 || ib[m] >= g.nbx[m]) ok = false;
  }
  return ok ? ib[0] + g.nbx[0] * ib[1] + g.nbx[0] * g.nbx[1] * ib[2] : 0;
}

// Count step for input atom t: claims a place in its box and records t
// there (index[box*64 + place]).  Returns 0, COMDGB_ERR_BOXRANGE (-12) or
// COMDGB_ERR_MAXATOMS (-11).
__device__ __forceinline__ int bin_count_atom(const BinGrid &g, int t, const double *xyz,
                                              int *natoms, int *index) {
  double w[3];
  bool ok;
  const int b = bin_world_box(g, xyz + 3 * (long)t, w, ok);
  if (!ok) return -12;
  const int pos = atomicAdd(natoms + b, 1);
  if (pos >= CG_MAXATOMS) return -11;
  index[b * CG_MAXATOMS + pos] = t;
  return 0;
}

// Per-box step: the nb (<= 64) recorded input indexes ix[] sorted
// ascending, which is the order of the reference's calls.
__device__ __forceinline__ void bin_sort_box(int *ix, int nb) {
  for (int i = 1; i < nb; i++) {  // insertion sort
    const int v = ix[i];
    int j = i - 1;
    while (j >= 0 && ix[j] > v) {
      ix[j + 1] = ix[j];
      j--;
    }
    ix[j + 1] = v;
  }
}

}  // namespace cg
