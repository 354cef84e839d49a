// noalloc.cu -- an allocation-free variant of the device binning
// (putAtomInBox as a counting sort, src-flat/domains.c:237-291).
//
// Who needs it: callers that must not allocate device memory while they run
// -- an engine that owns all GPU memory through its own arena and forbids
// allocations after start-up, and tight loops where cudaMalloc's implicit
// synchronisation would stall the GPU.  comdgb_put_atoms allocates its
// temporaries; this entry point takes every input and output as a device
// pointer and keeps its scratch (one index per slot plus a status word) in a
// file-scope device array that exists from the moment the library's code is
// loaded on a device until the process exits.  The count and place bodies
// are the ones comdgb_put_atoms runs (binning.cuh).
//
// Limits and rules (also in include/comdgb.h):
//  * at most COMDGB_NOALLOC_MAX_BOXES boxes (16,384 boxes = 1,048,576 slots,
//    4 MiB of scratch per device); larger grids are rejected with an error;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that
//    first call before any stream capture;
//  * the call makes `device` current for its work and restores the caller's
//    current device before it returns;
//  * every call shares the one array, so calls whose work overlaps on the
//    GPU (different streams or host threads without ordering) race; the
//    array keeps the previous call's contents, so each call clears the
//    status word it reads and writes every index before it reads it;
//  * the call reads its status back and synchronises `stream` to report
//    errors.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "comdgb.h"
#include "binning.cuh"

// records the message that comdgb_last_error() returns (api.cu)
extern "C" int comdgb_internal_set_error(int code, const char *msg);

namespace {

constexpr int kMaxSlots = COMDGB_NOALLOC_MAX_BOXES * CG_MAXATOMS;
constexpr int kStatusWords = 64;  // one 256-byte block after the indices

// scratch: [0, kMaxSlots) input index per slot; [kMaxSlots] error status
static __device__ __align__(256) int g_bin_scratch[kMaxSlots + kStatusWords];

std::mutex g_mu;
int *g_scratch_ptr[64];  // device address of g_bin_scratch per device ordinal

int fail(int code, const char *msg) { return comdgb_internal_set_error(code, msg); }

using cg::BinGrid;

__global__ void na_count_kernel(BinGrid g, int n, const double *xyz, int *natoms, int *scratch) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int err = cg::bin_count_atom(g, t, xyz, natoms, scratch);
  if (err) atomicCAS(scratch + kMaxSlots, 0, err);
}

__global__ void na_place_kernel(BinGrid g, const double *dcenter, int n, const double *xyz,
                                const double *pxyz, const int *ids, const int *types,
                                const double *masses, const int *natoms, int *id, int *itype,
                                double *mass, double *r, double *p, int *scratch) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nboxes) return;
  if (*(volatile int *)(scratch + kMaxSlots)) return;
  int nb = natoms[b];
  if (nb > CG_MAXATOMS) return;
  int *ix = scratch + b * CG_MAXATOMS;
  cg::bin_sort_box(ix, nb);
  for (int k = 0; k < nb; k++) {
    int t = ix[k];
    long slot = (long)b * CG_MAXATOMS + k;
    double w[3];
    bool ok;
    cg::bin_world_box(g, xyz + 3 * (long)t, w, ok);
    id[slot] = ids[t];
    itype[slot] = types[t];
    mass[slot] = masses[t];
    for (int m = 0; m < 3; m++) {
      r[3 * slot + m] = w[m] - dcenter[3 * b + m];
      p[3 * slot + m] = pxyz[3 * (long)t + m];
    }
  }
}

// device address of the scratch array on `device` (looked up once)
int scratch_for(int device, int **out) {
  if (device < 0 || device >= 64) return fail(COMDGB_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[device]) {
    int *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_bin_scratch);
    if (e != cudaSuccess) {
      char m[200];
      snprintf(m, sizeof m, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return fail(COMDGB_ERR_CUDA, m);
    }
    g_scratch_ptr[device] = ptr;
  }
  *out = g_scratch_ptr[device];
  return 0;
}

// the work of one call on the current device (see comdgb_put_atoms_noalloc)
int put_atoms_noalloc(const BinGrid &g, int device, const double *dcenter, int n,
                      const double *xyz, const double *pxyz, const int *ids, const int *itypes,
                      const double *masses, int *natoms, int *id, int *itype, double *mass,
                      double *r, double *p, cudaStream_t st) {
  int *scratch = nullptr;
  int rc = scratch_for(device, &scratch);
  if (rc) return rc;
  // outputs that are accumulated and the status word start at zero
  cudaError_t e = cudaMemsetAsync(natoms, 0, sizeof(int) * (size_t)g.nboxes, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch + kMaxSlots, 0, sizeof(int), st);
  if (e != cudaSuccess) return fail(COMDGB_ERR_CUDA, cudaGetErrorString(e));
  if (n > 0) na_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(g, n, xyz, natoms, scratch);
  na_place_kernel<<<(g.nboxes + 127) / 128, 128, 0, st>>>(g, dcenter, n, xyz, pxyz, ids, itypes,
                                                          masses, natoms, id, itype, mass, r, p,
                                                          scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(COMDGB_ERR_CUDA, cudaGetErrorString(e));
  int status = 0;
  e = cudaMemcpyAsync(&status, scratch + kMaxSlots, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(COMDGB_ERR_CUDA, cudaGetErrorString(e));
  if (status == COMDGB_ERR_MAXATOMS)
    return fail(status, "comdgb_put_atoms_noalloc: a box received more than 64 atoms");
  if (status) return fail(status, "comdgb_put_atoms_noalloc: an atom's box fell outside the grid");
  return 0;
}

}  // namespace

extern "C" int comdgb_put_atoms_noalloc(const int nbx[3], const double bounds[3],
                                        const double boxsize[3], const double *dcenter, int n,
                                        const double *xyz, const double *pxyz, const int *ids,
                                        const int *itypes, const double *masses, int *natoms,
                                        int *id, int *itype, double *mass, double *r,
                                        double *p, int device, void *stream) {
  if (!nbx || !bounds || !boxsize || !dcenter || !natoms || !id || !itype || !mass || !r || !p ||
      n < 0 || (n > 0 && (!xyz || !pxyz || !ids || !itypes || !masses)))
    return fail(COMDGB_ERR_ARG, "comdgb_put_atoms_noalloc: null pointer or negative count");
  BinGrid g;
  long nboxes = 1;
  for (int j = 0; j < 3; j++) {
    if (nbx[j] < 1) return fail(COMDGB_ERR_ARG, "comdgb_put_atoms_noalloc: nbx < 1");
    if (!(std::isfinite(bounds[j]) && bounds[j] > 0.0 && std::isfinite(boxsize[j]) &&
          boxsize[j] > 0.0))
      return fail(COMDGB_ERR_ARG,
                  "comdgb_put_atoms_noalloc: bounds and boxsize must be finite and positive");
    g.nbx[j] = nbx[j];
    g.bounds[j] = bounds[j];
    g.boxsize[j] = boxsize[j];
    nboxes *= nbx[j];  // checked after every factor: at most 16,384 * (2^31 - 1)
    if (nboxes > COMDGB_NOALLOC_MAX_BOXES) {
      char m[240];
      snprintf(m, sizeof m,
               "comdgb_put_atoms_noalloc: a grid of %d x %d x %d boxes exceeds the "
               "allocation-free limit of %d boxes",
               nbx[0], nbx[1], nbx[2], COMDGB_NOALLOC_MAX_BOXES);
      return fail(COMDGB_ERR_ARG, m);
    }
  }
  g.nboxes = (int)nboxes;
  int prev = 0;
  cudaError_t e = cudaGetDevice(&prev);
  if (e == cudaSuccess) e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(COMDGB_ERR_CUDA, cudaGetErrorString(e));
  const int rc = put_atoms_noalloc(g, device, dcenter, n, xyz, pxyz, ids, itypes, masses, natoms,
                                   id, itype, mass, r, p, (cudaStream_t)stream);
  e = cudaSetDevice(prev);  // the caller's current device, on every return path
  if (rc) return rc;
  if (e != cudaSuccess) return fail(COMDGB_ERR_CUDA, cudaGetErrorString(e));
  return 0;
}
