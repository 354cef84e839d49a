// clsman_io.cu -- clsman output (write.c:112-220).  The state is gathered
// into atom-id order on the device (replacing getRL, write.c:58-87: one
// thread per atom scatters its world position and momentum to row id), then
// the host writes the reference's formats byte for byte:
//   writeClsman  (write.c:112-167)  binary records: [12] ntot 0 0 [12] 0 0,
//                [24] bounds [24], [52 n] per atom x y z 1 px py pz [52 n]
//   gzASCIIWrite (write.c:175-220)  text: "ntot 0", the comment line, the
//                bounds "%.8lf" x 3, per atom "%.8lf" x 3 " 1 " "%.8lf" x 3
// Text lines are formatted by several host threads; a gzip file is written
// as one gzip member per thread's chunk (a concatenation of members is one
// valid gzip file: zlib's gzread and Python's gzip read it whole).
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#ifdef COMDGB_HAVE_ZLIB
#include <zlib.h>
#endif

#include "sim.h"

using namespace cg;
using namespace cgapi;

namespace {

// Replica atoms [a0, a0 + na) of the compact order; device ids id0 + 0..na-1.
// out[6 * lid + 0..2] = box corner + r (write.c:157, one FP64 add),
// [3..5] = p.  bad counts ids out of range or seen twice.
__global__ void gather_by_id_kernel(Slots s, const double *dcenter, const int *atom_slot, int a0,
                                    int na, int id0, double *out, int *seen, int *bad) {
  for (int a = a0 + blockIdx.x * blockDim.x + threadIdx.x; a < a0 + na;
       a += gridDim.x * blockDim.x) {
    const int slot = atom_slot[a];
    const int b = slot >> 6;
    const int lid = s.id[slot] - id0;
    if (lid < 0 || lid >= na || atomicAdd(seen + lid, 1) != 0) {
      atomicAdd(bad, 1);
      continue;
    }
    const d4 r = s.r[slot], p = s.p[slot];
    double *o = out + 6 * (size_t)lid;
    o[0] = __dadd_rn(dcenter[3 * b + 0], r.x);
    o[1] = __dadd_rn(dcenter[3 * b + 1], r.y);
    o[2] = __dadd_rn(dcenter[3 * b + 2], r.z);
    o[3] = p.x;
    o[4] = p.y;
    o[5] = p.z;
  }
}

int device_gather(comdgb_sim *h, int r, double *host_out) {
  if (r < 0 || r >= h->nrep) return set_err(COMDGB_ERR_ARG, "replica %d of %d", r, h->nrep);
  CK(cudaSetDevice(h->device));
  const RepGeo &R = h->reps[r];
  const int na = R.na;
  if (na == 0) return 0;
  int err = 0;
  double *d_out = dalloc<double>(6 * (size_t)na, &err);
  int *d_seen = dalloc<int>((size_t)na + 1, &err);
  if (err) {
    cudaFree(d_out);
    cudaFree(d_seen);
    return set_err(COMDGB_ERR_NOMEM, "gather buffers (%d atoms)", na);
  }
  cudaStream_t st = h->stream;
  int bad = 0;
  cudaError_t e = cudaMemsetAsync(d_seen, 0, sizeof(int) * ((size_t)na + 1), st);
  if (e == cudaSuccess) {
    // the atom list must be the current layout's
    launch_compact(h->g, h->s.natoms, h->box_start, h->atom_slot, h->ntot, h->cpart, h->ncpart,
                   st);
    int dev_sms = 1;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, h->device);
    const long need = ((long)na + 255) / 256;
    const int grid = (int)(need < 8L * dev_sms ? need : 8L * dev_sms);
    gather_by_id_kernel<<<grid, 256, 0, st>>>(h->s, h->dcenter, h->atom_slot, R.a0, na,
                                              h->atom0[r], d_out, d_seen, d_seen + na);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host_out, d_out, sizeof(double) * 6 * (size_t)na, cudaMemcpyDeviceToHost,
                        st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&bad, d_seen + na, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_out);
  cudaFree(d_seen);
  if (e != cudaSuccess) return set_err(COMDGB_ERR_CUDA, "gather: %s", cudaGetErrorString(e));
  if (bad)
    return set_err(COMDGB_ERR_ARG, "%d atom(s) with an id outside 0..%d or seen twice", bad,
                   na - 1);
  return 0;
}

// getRL's order on the host (a simflat_t that is not attached)
int host_gather(const simflat_t *s, double *out) {
  const int n = s->ntot;
  std::vector<char> seen((size_t)n, 0);
  for (int b = 0; b < s->nboxes; b++)
    for (int i = 0; i < s->natoms[b]; i++) {
      const int slot = b * CG_MAXATOMS + i;
      const int id = s->id[slot];
      if (id < 0 || id >= n || seen[id])
        return set_err(COMDGB_ERR_ARG, "atom id %d outside 0..%d or seen twice", id, n - 1);
      seen[id] = 1;
      double *o = out + 6 * (size_t)id;
      for (int k = 0; k < 3; k++) {
        o[k] = s->dcenter[b][k] + s->r[slot][k];
        o[3 + k] = s->p[slot][k];
      }
    }
  for (int i = 0; i < n; i++)
    if (!seen[i]) return set_err(COMDGB_ERR_ARG, "atom id %d missing", i);
  return 0;
}

template <class T>
void put(std::string &b, T v) {
  b.append(reinterpret_cast<const char *>(&v), sizeof v);
}

// writeClsman's byte image (native byte order, packed records)
std::string binary_image(const double bounds[3], const double *v, int n) {
  std::string b;
  b.reserve(60 + 52 * (size_t)n + 8);
  const int head[7] = {3 * (int)sizeof(int), n, 0, 0, 3 * (int)sizeof(int), 0, 0};
  for (int q = 0; q < 7; q++) put(b, head[q]);
  put(b, 3 * (int)sizeof(double));
  for (int q = 0; q < 3; q++) put(b, bounds[q]);
  put(b, 3 * (int)sizeof(double));
  // the record length as the reference's int expression computes it
  const int rec = (int)(unsigned)((size_t)n * (6 * sizeof(double) + sizeof(int)));
  put(b, rec);
  const int jtype = 1;
  for (int i = 0; i < n; i++) {
    const double *o = v + 6 * (size_t)i;
    for (int q = 0; q < 3; q++) put(b, o[q]);
    put(b, jtype);
    for (int q = 3; q < 6; q++) put(b, o[q]);
  }
  put(b, rec);
  return b;
}

std::string text_header(int n, const char *comment, const double bounds[3]) {
  char line[256];
  std::string t;
  snprintf(line, sizeof line, "%d 0\n", n);
  t += line;
  // the comment verbatim, as the reader keeps it (its newline included); a
  // missing newline is added so that the file reads back
  std::string c = comment ? comment : "";
  if (c.empty() || c.back() != '\n') c += '\n';
  t += c;
  snprintf(line, sizeof line, "%.8lf %.8lf %.8lf\n", bounds[0], bounds[1], bounds[2]);
  t += line;
  return t;
}

void text_lines(const double *v, int i0, int i1, std::string &t) {
  char line[512];
  for (int i = i0; i < i1; i++) {
    const double *o = v + 6 * (size_t)i;
    const int len = snprintf(line, sizeof line, "%.8lf %.8lf %.8lf %d %.8lf %.8lf %.8lf\n", o[0],
                             o[1], o[2], 1, o[3], o[4], o[5]);
    t.append(line, (size_t)len);
  }
}

int n_threads(int n) {
  unsigned hw = std::thread::hardware_concurrency();
  int t = (int)(hw ? (hw < 32 ? hw : 32) : 4);
  const int by_size = (n + 16383) / 16384;
  return t < by_size ? t : (by_size > 0 ? by_size : 1);
}

#ifdef COMDGB_HAVE_ZLIB
// one gzip member of `in` (level 6, gzopen's "wb" default)
bool gzip_member(const std::string &in, std::string &out) {
  z_stream z;
  memset(&z, 0, sizeof z);
  if (deflateInit2(&z, 6, Z_DEFLATED, 15 + 16, 8, Z_DEFAULT_STRATEGY) != Z_OK) return false;
  out.resize(deflateBound(&z, (uLong)in.size()) + 64);
  z.next_in = (Bytef *)in.data();
  z.avail_in = (uInt)in.size();
  z.next_out = (Bytef *)&out[0];
  z.avail_out = (uInt)out.size();
  const int rc = deflate(&z, Z_FINISH);
  out.resize(z.total_out);
  deflateEnd(&z);
  return rc == Z_STREAM_END;
}
#endif

int write_bytes(const char *path, const std::vector<const std::string *> &parts) {
  FILE *fp = fopen(path, "wb");
  if (!fp) return set_err(COMDGB_ERR_IO, "cannot open %s for writing", path);
  bool ok = true;
  for (const std::string *p : parts)
    if (!p->empty() && fwrite(p->data(), 1, p->size(), fp) != p->size()) ok = false;
  if (fclose(fp) != 0) ok = false;
  if (!ok) return set_err(COMDGB_ERR_IO, "write to %s failed", path);
  return 0;
}

// write the gathered atoms (v: 6 per atom in id order) in `format`
int write_atoms(const char *path, int format, const char *comment, const double bounds[3],
                const double *v, int n) {
  if (!path) return set_err(COMDGB_ERR_ARG, "null path");
  if (format == COMDGB_CLSMAN_BINARY) {
    const std::string img = binary_image(bounds, v, n);
    return write_bytes(path, {&img});
  }
  if (format != COMDGB_CLSMAN_TEXT && format != COMDGB_CLSMAN_TEXT_GZ)
    return set_err(COMDGB_ERR_ARG, "unknown clsman format %d", format);
#ifndef COMDGB_HAVE_ZLIB
  if (format == COMDGB_CLSMAN_TEXT_GZ)
    return set_err(COMDGB_ERR_UNSUPPORTED, "gzip output needs the library built with zlib");
#endif
  const bool gz = format == COMDGB_CLSMAN_TEXT_GZ;
  const int nt = n_threads(n);
  // chunk 0 is the header; chunks 1..nt the atom lines
  std::vector<std::string> text((size_t)nt + 1), packed((size_t)nt + 1);
  text[0] = text_header(n, comment, bounds);
  std::vector<char> ok((size_t)nt + 1, 1);
  auto work = [&](int c) {
    if (c > 0) {
      const int i0 = (int)((long)n * (c - 1) / nt), i1 = (int)((long)n * c / nt);
      text[c].reserve((size_t)(i1 - i0) * 96);
      text_lines(v, i0, i1, text[c]);
    }
#ifdef COMDGB_HAVE_ZLIB
    if (gz) {
      ok[c] = gzip_member(text[c], packed[c]);
      std::string().swap(text[c]);
    }
#endif
  };
  std::vector<std::thread> pool;
  for (int c = 1; c <= nt; c++) pool.emplace_back(work, c);
  work(0);
  for (std::thread &t : pool) t.join();
  for (char k : ok)
    if (!k) return set_err(COMDGB_ERR_IO, "gzip compression failed");
  std::vector<const std::string *> parts;
  for (int c = 0; c <= nt; c++) parts.push_back(gz ? &packed[c] : &text[c]);
  return write_bytes(path, parts);
}

}  // namespace

extern "C" {

int comdgb_sim_gather(comdgb_sim *h, int r, double *out) {
  if (!h || !out) return set_err(COMDGB_ERR_ARG, "null argument");
  return device_gather(h, r, out);
}

int comdgb_sim_write_clsman(comdgb_sim *h, int r, const char *path, int format,
                            const char *comment) {
  if (!h || !path) return set_err(COMDGB_ERR_ARG, "null argument");
  if (r < 0 || r >= h->nrep) return set_err(COMDGB_ERR_ARG, "replica %d of %d", r, h->nrep);
  std::vector<double> v(6 * (size_t)h->reps[r].na + 6);
  int rc = device_gather(h, r, v.data());
  if (rc) return rc;
  return write_atoms(path, format, comment, h->reps[r].bounds, v.data(), h->reps[r].na);
}

// the drop-ins: a simflat_t attached in lazy mode (the device holds the
// current state) is gathered on the device, any other on the host
static int write_simflat(simflat_t *s, const char *fname, int format) {
  if (!s || !fname) return set_err(COMDGB_ERR_ARG, "null argument");
  comdgb_sim *h = find_attached(s);
  if (h && h->lazy) return comdgb_sim_write_clsman(h, 0, fname, format, s->comment);
  std::vector<double> v(6 * (size_t)s->ntot + 6);
  int rc = host_gather(s, v.data());
  if (rc) return rc;
  return write_atoms(fname, format, s->comment, s->bounds, v.data(), s->ntot);
}

int comdgb_writeClsman(simflat_t *s, const char *fname) {
  return write_simflat(s, fname, COMDGB_CLSMAN_BINARY);
}

int comdgb_gzASCIIWrite(simflat_t *s, const char *fname) {
  return write_simflat(s, fname, COMDGB_CLSMAN_TEXT_GZ);
}

}  // extern "C"
