/*
 * host_setup.c -- host-side setup routines of libcomdgb (plain C): reading
 * the EAM tables, the FCC lattice generator, seeded perturbation and the
 * host simflat_t allocation.  They build the same structures as the
 * reference's setup code so a caller without the reference can drive the
 * GPU path; none of them is on the timed path.
 */
#define _POSIX_C_SOURCE 200112L
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef COMDGB_HAVE_ZLIB
#include <zlib.h>
#endif

#include "comdgb.h"
#include "comdgb_seed.h"

static void *zalloc(size_t n) {
  void *p = NULL;
  size_t padded = (n + 127) & ~(size_t)127;
  if (padded == 0) padded = 128;
  if (posix_memalign(&p, 128, padded)) return NULL;
  memset(p, 0, padded);
  return p;
}

/* the message comdgb_last_error() returns (api.cu) */
int comdgb_internal_set_error(int code, const char *msg);

/* records why a host set-up call failed: the call, the file when there is
 * one, and the meaning of the code */
static int host_err(int code, const char *call, const char *path) {
  const char *why;
  switch (code) {
    case COMDGB_ERR_ARG:
      why = "bad argument, or a grid whose slot indexes do not fit an int";
      break;
    case COMDGB_ERR_NOBOX:
      why = "Need at least one cutoff wide domain (bounds below the cutoff)";
      break;
    case COMDGB_ERR_MAXATOMS:
      why = "Increase maxatoms (a box would hold more than 64 atoms)";
      break;
    case COMDGB_ERR_BOXRANGE:
      why = "an atom's coordinate is not finite or lies more than one period outside";
      break;
    case COMDGB_ERR_NOMEM:
      why = "out of host memory";
      break;
    case COMDGB_ERR_IO:
      why = "cannot open the file, or it is short or malformed";
      break;
    case COMDGB_ERR_UNSUPPORTED:
      why = "gzip input needs the library built with zlib";
      break;
    default:
      why = "failed";
      break;
  }
  char m[512];
  snprintf(m, sizeof m, "%s%s%.300s: %s", call, path ? " " : "", path ? path : "", why);
  return comdgb_internal_set_error(code, m);
}

static int read_be_or_le(FILE *fp, void *dst, int size, int swap) {
  unsigned char b[8];
  if (fread(b, (size_t)size, 1, fp) != 1) return 0;
  unsigned char *d = (unsigned char *)dst;
  for (int i = 0; i < size; i++) d[i] = swap ? b[size - 1 - i] : b[i];
  return 1;
}

/* Fortran-record table file: [36][n x0 xn invDx iflo ifhi][36][8n][values][8n]
 * (getPotentialArrayFromBinaryFile, eam.c:156-249).  Byte order is detected
 * from the first record length.  Guard cells: values[-1] = iflo ? v[0] : 0,
 * values[n] = values[n+1] = ifhi ? v[n-1] : 0; x0 is moved up one interval
 * (allocPotentialArray, eam.c:130-153). */
static potentialarray_t *read_table(const char *path) {
  FILE *fp = fopen(path, "rb");
  if (!fp) return NULL;
  unsigned char head[4];
  if (fread(head, 4, 1, fp) != 1) { fclose(fp); return NULL; }
  int le = head[0] | (head[1] << 8) | (head[2] << 16) | (head[3] << 24);
  int swap = le > 4096;
  int n = 0, iflo = 0, ifhi = 0, rec = 0;
  double x0 = 0, xn = 0, invdx = 0;
  int ok = read_be_or_le(fp, &n, 4, swap) && read_be_or_le(fp, &x0, 8, swap) &&
           read_be_or_le(fp, &xn, 8, swap) && read_be_or_le(fp, &invdx, 8, swap) &&
           read_be_or_le(fp, &iflo, 4, swap) && read_be_or_le(fp, &ifhi, 4, swap) &&
           read_be_or_le(fp, &rec, 4, swap) && read_be_or_le(fp, &rec, 4, swap);
  /* a table the interpolation can index: n points on x0 < xn with a finite,
   * positive 1/dx (the reference reads these fields unchecked) */
  if (!ok || n <= 0 || n > (1 << 26) || rec != n * 8 || !isfinite(x0) || !isfinite(xn) ||
      !(xn > x0) || !isfinite(invdx) || !(invdx > 0.0)) {
    fclose(fp);
    return NULL;
  }
  potentialarray_t *a = (potentialarray_t *)zalloc(sizeof *a);
  double *buf = (double *)zalloc((size_t)(n + 3) * sizeof(double));
  if (!a || !buf) { free(a); free(buf); fclose(fp); return NULL; }
  a->values = buf + 1;
  for (int i = 0; i < n; i++)
    if (!read_be_or_le(fp, a->values + i, 8, swap)) { free(buf); free(a); fclose(fp); return NULL; }
  fclose(fp);
  a->n = n;
  a->invDx = invdx;
  a->xn = xn;
  a->x0 = x0 + (xn - x0) / (double)n;
  a->values[-1] = iflo ? a->values[0] : 0.0;
  a->values[n] = ifhi ? a->values[n - 1] : 0.0;
  a->values[n + 1] = a->values[n];
  return a;
}

static void free_table(potentialarray_t *a) {
  if (!a) return;
  free(a->values - 1);
  free(a);
}

static double doc_line_value(const char *path, int line) {
  FILE *fp = fopen(path, "r");
  if (!fp) return -1.0;
  char buf[4096];
  double v = -1.0;
  int l = 0;
  while (l < line && fgets(buf, sizeof buf, fp)) l++;
  if (l == line && sscanf(buf, "%lf", &v) != 1) v = -1.0;
  fclose(fp);
  return v;
}

eampotential_t *comdgb_eam_read(const char *dir, const char *name) {
  char path[4096];
  eampotential_t *p = (eampotential_t *)zalloc(sizeof *p);
  if (!p) return NULL;
  static const char *ext[3] = {"phi", "rho", "f"};
  potentialarray_t **tab[3] = {&p->phi, &p->rho, &p->f};
  for (int q = 0; q < 3; q++) {
    snprintf(path, sizeof path, "%s/%s.%s", dir, name, ext[q]);
    *tab[q] = read_table(path);
    if (!*tab[q]) {
      host_err(COMDGB_ERR_IO, "comdgb_eam_read", path);
      comdgb_eam_free(p);
      return NULL;
    }
  }
  snprintf(path, sizeof path, "%s/%s.doc", dir, name);
  p->mass = doc_line_value(path, 2); /* mass in amu, second line */
  p->lat = doc_line_value(path, 3);  /* lattice constant, third line */
  if (p->mass < 0.0) {
    host_err(COMDGB_ERR_IO, "comdgb_eam_read", path);
    comdgb_eam_free(p);
    return NULL;
  }
  p->cutoff = p->phi->xn; /* eam.c:392 */
  return p;
}

void comdgb_eam_free(eampotential_t *p) {
  if (!p) return;
  free_table(p->phi);
  free_table(p->rho);
  free_table(p->f);
  free(p);
}

ljpotential_t *comdgb_lj_make(double sigma, double epsilon, double cutoff, double mass) {
  ljpotential_t *p = (ljpotential_t *)zalloc(sizeof *p);
  if (!p) return NULL;
  p->sigma = sigma;
  p->epsilon = epsilon;
  p->cutoff = cutoff;
  p->mass = mass;
  return p;
}

void comdgb_lj_free(ljpotential_t *p) { free(p); }

void comdgb_sim_free_host(simflat_t *s) {
  if (!s) return;
  free(s->dcenter);
  free(s->natoms);
  free(s->id);
  free(s->iType);
  free(s->mass);
  free(s->r);
  free(s->p);
  free(s->f);
  free(s->rho);
  free(s->fi);
  free(s->comment);
  free(s);
}

/* allocDomains (domains.c:155-200) */
static int alloc_domains(simflat_t *s) {
  double strain[3] = {s->defgrad == 0.0 ? 1.0 : s->defgrad, 1.0, 1.0};
  double bf = s->bf == 0.0 ? 1.0 : s->bf;
  /* slot indexes (box * 64 + k) are int, as in the reference: a grid of
   * more boxes than that allows (or a non-finite extent) is an argument
   * error here, where the reference's int conversion would be undefined */
  const long long max_boxes = 0x7fffffffLL / COMDGB_MAXATOMS;
  long long nboxes = 1;
  for (int j = 0; j < 3; j++) {
    const double q = floor(s->bounds[j] / (s->pot->cutoff * bf * strain[j]));
    if (q != q || q > (double)max_boxes) return COMDGB_ERR_ARG;
    if (q < 1.0) return COMDGB_ERR_NOBOX;
    s->nbx[j] = (int)q;
    nboxes *= s->nbx[j];
    if (nboxes > max_boxes) return COMDGB_ERR_ARG;
    s->boxsize[j] = s->bounds[j] / (double)s->nbx[j];
  }
  s->nboxes = (int)nboxes;
  size_t nb = (size_t)s->nboxes, ns = nb * COMDGB_MAXATOMS;
  s->dcenter = (comdgb_real3 *)zalloc(nb * sizeof(comdgb_real3));
  s->natoms = (int *)zalloc(nb * sizeof(int));
  s->id = (int *)zalloc(ns * sizeof(int));
  s->iType = (int *)zalloc(ns * sizeof(int));
  s->mass = (double *)zalloc(ns * sizeof(double));
  s->r = (comdgb_real3 *)zalloc(ns * sizeof(comdgb_real3));
  s->p = (comdgb_real3 *)zalloc(ns * sizeof(comdgb_real3));
  s->f = (comdgb_real4 *)zalloc(ns * sizeof(comdgb_real4));
  s->rho = (double *)zalloc(ns * sizeof(double));
  s->fi = (double *)zalloc(ns * sizeof(double));
  if (!s->dcenter || !s->natoms || !s->id || !s->iType || !s->mass || !s->r || !s->p ||
      !s->f || !s->rho || !s->fi)
    return COMDGB_ERR_NOMEM;
  s->stateflag = 1;
  for (int b = 0; b < s->nboxes; b++) {
    int ib[3] = {b % s->nbx[0], (b / s->nbx[0]) % s->nbx[1], b / s->nbx[0] / s->nbx[1]};
    for (int j = 0; j < 3; j++) s->dcenter[b][j] = s->boxsize[j] * (double)ib[j];
  }
  return 0;
}

/* putAtomInBox (domains.c:237-291) for one atom at world position x with
 * momenta p (NULL: zero).  A coordinate that is not in [0, bounds) after
 * one wrap -- more than a period outside, NaN or infinite -- is
 * COMDGB_ERR_BOXRANGE, as in the device binning (binning.cuh): the
 * conversion of floor(NaN) to int differs between hosts. */
static int put_atom(simflat_t *s, int id, int itype, double mass, const double *x,
                    const double *p) {
  double w[3];
  int ib[3];
  for (int m = 0; m < 3; m++) {
    w[m] = x[m];
    if (w[m] < 0.0) w[m] += s->bounds[m];
    else if (w[m] >= s->bounds[m]) w[m] -= s->bounds[m];
    if (!(w[m] >= 0.0 && w[m] < s->bounds[m])) return COMDGB_ERR_BOXRANGE;
    ib[m] = (int)floor(w[m] / s->boxsize[m]);
    if (ib[m] < 0 || ib[m] >= s->nbx[m]) return COMDGB_ERR_BOXRANGE;
  }
  int b = ib[0] + s->nbx[0] * ib[1] + s->nbx[0] * s->nbx[1] * ib[2];
  if (s->natoms[b] >= COMDGB_MAXATOMS) return COMDGB_ERR_MAXATOMS;
  int off = b * COMDGB_MAXATOMS + s->natoms[b]++;
  s->ntot++;
  s->id[off] = id;
  s->iType[off] = itype;
  s->mass[off] = mass;
  for (int m = 0; m < 3; m++) {
    s->r[off][m] = w[m] - s->dcenter[b][m];
    s->p[off][m] = p ? p[m] : 0.0;
  }
  return 0;
}

/* create_fcc_lattice (ic_fcc.c:63-141): walk the half-lattice points with
 * running counters and keep those with odd index sum; ids in walk order */
simflat_t *comdgb_fcc(int nx, int ny, int nz, double lat, double defgrad, double bf,
                      pmd_base_potential_t *pot, int *status) {
  int st = 0;
  simflat_t *s = (simflat_t *)zalloc(sizeof *s);
  if (!s) { if (status) *status = COMDGB_ERR_NOMEM; return NULL; }
  s->pot = pot;
  s->comment = (char *)zalloc(1024);
  s->defgrad = defgrad;
  s->bf = bf;
  s->bounds[0] = nx * lat * defgrad;
  s->bounds[1] = ny * lat;
  s->bounds[2] = nz * lat;
  st = alloc_domains(s);
  if (!st) {
    double half = lat / 2.0, pt[3];
    int ci = 0, cj = 0, ck = 0, nid = 0;
    for (pt[2] = lat / 4.0; pt[2] < s->bounds[2] && !st; pt[2] += half, ck++)
      for (pt[1] = lat / 4.0; pt[1] < s->bounds[1] && !st; pt[1] += half, cj++)
        for (pt[0] = lat * defgrad / 4.0; pt[0] < s->bounds[0] && !st;
             pt[0] += half * defgrad, ci++)
          if ((ci + cj + ck) % 2) st = put_atom(s, nid++, 1, pot->mass, pt, NULL);
  }
  if (status) *status = st;
  if (st) {
    host_err(st, "comdgb_fcc", NULL);
    comdgb_sim_free_host(s);
    return NULL;
  }
  return s;
}

/* A copy of s with its atoms binned on a grid of box factor bf
 * (allocDomains, domains.c:155-200, then putAtomInBox, domains.c:237-291,
 * once per atom in id order at its world position, box corner + r); ids,
 * types, masses and momenta are kept, forces zero.  Fails with
 * COMDGB_ERR_MAXATOMS when a box of the new grid would pass 64 atoms. */
simflat_t *comdgb_rebin_host(const simflat_t *src, double bf, int *status) {
  int st = 0;
  if (!src || !src->pot || !(bf > 0.0)) {
    if (status) *status = host_err(COMDGB_ERR_ARG, "comdgb_rebin_host", NULL);
    return NULL;
  }
  simflat_t *s = (simflat_t *)zalloc(sizeof *s);
  if (!s) { if (status) *status = COMDGB_ERR_NOMEM; return NULL; }
  s->pot = src->pot;
  s->comment = (char *)zalloc(1024);
  s->defgrad = src->defgrad;
  s->bf = bf;
  s->ch_pot = src->ch_pot;
  for (int j = 0; j < 3; j++) s->bounds[j] = src->bounds[j];
  st = s->comment ? alloc_domains(s) : COMDGB_ERR_NOMEM;
  /* slot of every id in the source */
  int *slot_of = st ? NULL : (int *)malloc(sizeof(int) * (size_t)(src->ntot > 0 ? src->ntot : 1));
  if (!st && !slot_of) st = COMDGB_ERR_NOMEM;
  if (!st) {
    for (int i = 0; i < src->ntot; i++) slot_of[i] = -1;
    for (int b = 0; b < src->nboxes && !st; b++)
      for (int k = 0; k < src->natoms[b]; k++) {
        const int off = b * COMDGB_MAXATOMS + k, id = src->id[off];
        if (id < 0 || id >= src->ntot || slot_of[id] >= 0) {
          st = COMDGB_ERR_ARG;  /* ids must be 0..ntot-1, each once */
          break;
        }
        slot_of[id] = off;
      }
    for (int id = 0; id < src->ntot && !st; id++) {
      const int off = slot_of[id];
      if (off < 0) { st = COMDGB_ERR_ARG; break; }
      const int b = off / COMDGB_MAXATOMS;
      double x[3];
      for (int m = 0; m < 3; m++) x[m] = src->dcenter[b][m] + src->r[off][m];
      st = put_atom(s, id, src->iType[off], src->mass[off], x, src->p[off]);
    }
  }
  free(slot_of);
  if (status) *status = st;
  if (st) {
    host_err(st, "comdgb_rebin_host", NULL);
    comdgb_sim_free_host(s);
    return NULL;
  }
  return s;
}

/* The whole file into memory (gzip through zlib when the library was built
 * with it); NUL-terminated.  Returns NULL on failure with *st set. */
static char *read_all(const char *path, int *st) {
  FILE *fp = fopen(path, "rb");
  if (!fp) {
    *st = COMDGB_ERR_IO;
    return NULL;
  }
  unsigned char magic[2] = {0, 0};
  size_t got = fread(magic, 1, 2, fp);
  fclose(fp);
  int gz = got == 2 && magic[0] == 0x1f && magic[1] == 0x8b;
  size_t cap = 1 << 20, len = 0;
  char *buf = (char *)malloc(cap + 1);
  if (!buf) {
    *st = COMDGB_ERR_NOMEM;
    return NULL;
  }
  if (gz) {
#ifdef COMDGB_HAVE_ZLIB
    gzFile g = gzopen(path, "rb");
    if (!g) {
      free(buf);
      *st = COMDGB_ERR_IO;
      return NULL;
    }
    for (;;) {
      if (len == cap) {
        char *nb = (char *)realloc(buf, 2 * cap + 1);
        if (!nb) {
          gzclose(g);
          free(buf);
          *st = COMDGB_ERR_NOMEM;
          return NULL;
        }
        buf = nb;
        cap *= 2;
      }
      int n = gzread(g, buf + len, (unsigned)(cap - len));
      if (n <= 0) break;
      len += (size_t)n;
    }
    gzclose(g);
#else
    free(buf);
    *st = COMDGB_ERR_UNSUPPORTED;  /* built without zlib: pass the decompressed text */
    return NULL;
#endif
  } else {
    fp = fopen(path, "rb");
    if (!fp) {
      free(buf);
      *st = COMDGB_ERR_IO;
      return NULL;
    }
    for (;;) {
      if (len == cap) {
        char *nb = (char *)realloc(buf, 2 * cap + 1);
        if (!nb) {
          fclose(fp);
          free(buf);
          *st = COMDGB_ERR_NOMEM;
          return NULL;
        }
        buf = nb;
        cap *= 2;
      }
      size_t n = fread(buf + len, 1, cap - len, fp);
      if (n == 0) break;
      len += n;
    }
    fclose(fp);
  }
  buf[len] = 0;
  return buf;
}

/* next line of the buffer, as gzgets reads it: *len = its length with the
 * '\n'.  The line is cut off with a NUL in place of the '\n' (the buffer is
 * ours), so that sscanf sees one line and not the rest of the file: glibc's
 * sscanf measures its whole input string on every call. */
static char *next_line(char **cur, size_t *len) {
  char *l = *cur;
  if (!*l) return NULL;
  char *e = strchr(l, '\n');
  if (e) {
    *e = 0;
    *cur = e + 1;
    if (len) *len = (size_t)(e - l) + 1;
  } else {
    *cur = l + strlen(l);
    if (len) *len = (size_t)(*cur - l);
  }
  return l;
}

/* The atom lines of a clsman file, parsed by up to 16 threads: each takes a
 * contiguous range of lines (already cut off with NULs) and reads them with
 * the reference's format. */
struct clsman_job {
  char **lines;
  double *xyz, *pxyz;
  int lo, hi, bad;
};

static void *clsman_parse(void *arg) {
  struct clsman_job *j = (struct clsman_job *)arg;
  for (int i = j->lo; i < j->hi && !j->bad; i++) {
    int itype = 0;
    double *x = j->xyz + 3 * (size_t)i, *p = j->pxyz + 3 * (size_t)i;
    if (sscanf(j->lines[i], "%lg %lg %lg %d %lg %lg %lg", &x[0], &x[1], &x[2], &itype, &p[0],
               &p[1], &p[2]) != 7)
      j->bad = 1;
  }
  return NULL;
}

static int clsman_parse_all(char **lines, int natoms, double *xyz, double *pxyz) {
  int nt = natoms / 8192;
  nt = nt < 1 ? 1 : nt > 16 ? 16 : nt;
  struct clsman_job job[16];
  pthread_t tid[16];
  int started[16] = {0};
  for (int t = 0; t < nt; t++) {
    job[t] = (struct clsman_job){lines, xyz, pxyz, (int)((long)natoms * t / nt),
                                 (int)((long)natoms * (t + 1) / nt), 0};
    started[t] = t > 0 && pthread_create(&tid[t], NULL, clsman_parse, &job[t]) == 0;
  }
  for (int t = 0; t < nt; t++)
    if (!started[t]) clsman_parse(&job[t]);  /* range 0, or a thread that did not start */
  int bad = 0;
  for (int t = 0; t < nt; t++) {
    if (started[t]) pthread_join(tid[t], NULL);
    bad |= job[t].bad;
  }
  return bad ? COMDGB_ERR_IO : 0;
}

/* fromFileGzip / fromFileASCII (read.c:155-241): a clsman file -- "natoms
 * nmove", a comment line, the periodic bounds, then one line "x y z itype px
 * py pz" per atom -- into a new simflat_t with allocDomains' grid for box
 * factor bf; atom i gets id i, type 0 and the potential's mass, placed as n
 * successive putAtomInBox calls (on the GPU `device`, or on the host for
 * device < 0). */
simflat_t *comdgb_read_clsman(const char *path, pmd_base_potential_t *pot, double bf, int device,
                              int *status) {
  int st = 0, from_gpu = 0;
  simflat_t *s = NULL;
  double *xyz = NULL, *pxyz = NULL, *masses = NULL;
  int *ids = NULL, *types = NULL;
  char **lines = NULL;
  if (!path || !pot) {
    if (status) *status = host_err(COMDGB_ERR_ARG, "comdgb_read", path);
    return NULL;
  }
  char *buf = read_all(path, &st);
  if (!buf) goto done;
  char *cur = buf, *l;
  size_t llen = 0;
  int natoms = 0, nmove = 0;
  if (!(l = next_line(&cur, NULL)) || sscanf(l, "%d%d", &natoms, &nmove) < 1 || natoms < 0) {
    st = COMDGB_ERR_IO;
    goto done;
  }
  s = (simflat_t *)zalloc(sizeof *s);
  if (!s) {
    st = COMDGB_ERR_NOMEM;
    goto done;
  }
  s->pot = pot;
  s->bf = bf;
  s->defgrad = 0.0; /* blankSimulation's; allocDomains then takes strain 1 */
  s->comment = (char *)zalloc(1024);
  if ((l = next_line(&cur, &llen)) && s->comment) {
    /* the comment as the reference keeps it: the line with its '\n' */
    size_t n = llen < 1023 ? llen : 1023;
    memcpy(s->comment, l, n);
    if (n && l[n - 1] == 0) s->comment[n - 1] = '\n';
  }
  if (!(l = next_line(&cur, NULL)) ||
      sscanf(l, "%lg %lg %lg", &s->bounds[0], &s->bounds[1], &s->bounds[2]) != 3) {
    st = COMDGB_ERR_IO;
    goto done;
  }
  /* every atom line holds seven numbers: a count the rest of the file
   * cannot hold is an I/O error before anything is allocated for it */
  if ((size_t)natoms > strlen(cur) / 2 + 1) {
    st = COMDGB_ERR_IO;
    goto done;
  }
  if ((st = alloc_domains(s))) goto done;
  size_t n = (size_t)natoms;
  xyz = (double *)malloc(3 * n * sizeof(double) + 8);
  pxyz = (double *)malloc(3 * n * sizeof(double) + 8);
  masses = (double *)malloc(n * sizeof(double) + 8);
  ids = (int *)malloc(n * sizeof(int) + 4);
  types = (int *)malloc(n * sizeof(int) + 4);
  lines = (char **)malloc(n * sizeof(char *) + 8);
  if (!xyz || !pxyz || !masses || !ids || !types || !lines) {
    st = COMDGB_ERR_NOMEM;
    goto done;
  }
  for (int i = 0; i < natoms; i++) {
    if (!(lines[i] = next_line(&cur, NULL))) {
      st = COMDGB_ERR_IO;
      goto done;
    }
    ids[i] = i;
    types[i] = 0; /* read.c:236: putAtomInBox(s, i, 1, 0, mass, ...) */
    masses[i] = pot->mass;
  }
  if ((st = clsman_parse_all(lines, natoms, xyz, pxyz))) goto done;
  if (device >= 0) {
    st = comdgb_put_atoms(s, natoms, xyz, pxyz, ids, types, masses, device);
    from_gpu = st != 0;  /* comdgb_put_atoms recorded its own message */
  } else {
    for (int i = 0; i < natoms && !st; i++)
      st = put_atom(s, ids[i], types[i], masses[i], xyz + 3 * (size_t)i, pxyz + 3 * (size_t)i);
  }
done:
  free(buf);
  free(lines);
  free(xyz);
  free(pxyz);
  free(masses);
  free(ids);
  free(types);
  if (status) *status = st;
  if (st && !from_gpu) host_err(st, "comdgb_read_clsman", path);
  if (st && s) {
    comdgb_sim_free_host(s);
    s = NULL;
  }
  return s;
}

/* printIt (write.c:89-110): box, id + 1, box-relative position, momentum
 * and force of the atoms with id < 10, in slot order */
void comdgb_printIt(const simflat_t *s, FILE *fp) {
  for (int b = 0; b < s->nboxes; b++)
    for (int i = 0, o = b * COMDGB_MAXATOMS; i < s->natoms[b]; i++, o++)
      if (s->id[o] < 10)
        fprintf(fp,
                "%02d, %02d, X=(%+020.12e %+020.12e %+020.12e) 1 "
                "P=(%+020.12e %+020.12e %+020.12e) F=(%+020.12e %+020.12e %+020.12e)\n",
                b, s->id[o] + 1, s->r[o][0], s->r[o][1], s->r[o][2], s->p[o][0], s->p[o][1],
                s->p[o][2], s->f[o][0], s->f[o][1], s->f[o][2]);
}

/* fromFileTim (read.c:248-315): a raw array of the visualiser's FileAtom
 * records (five native floats: x, y, z, bond order, centrosymmetry; the
 * file size gives the count) into a new simflat_t.  The reference fixes the
 * bounds to 327.424 x 354.446877 x 3007.581486 A rounded to float (its
 * :274, 287-289, one data set's); bounds != NULL replaces them.  Atom i gets id i, type 1 (:300),
 * the potential's mass and zero momenta, binned as successive putAtomInBox
 * calls on the GPU `device` (device < 0: on the host). */
simflat_t *comdgb_read_tim(const char *path, pmd_base_potential_t *pot, double bf,
                           const double *bounds, int device, int *status) {
  static const double kTimBounds[3] = {327.42399999999997817, 354.44687726089500757,
                                       3007.58148577889733133};
  int st = 0, from_gpu = 0;
  simflat_t *s = NULL;
  float *rec = NULL;
  double *xyz = NULL, *pxyz = NULL, *masses = NULL;
  int *ids = NULL, *types = NULL;
  long n = 0;
  if (!path || !pot) {
    if (status) *status = host_err(COMDGB_ERR_ARG, "comdgb_read", path);
    return NULL;
  }
  FILE *fp = fopen(path, "rb");
  if (!fp) {
    st = COMDGB_ERR_IO;
    goto done;
  }
  if (fseek(fp, 0, SEEK_END) == 0) n = ftell(fp) / (long)(5 * sizeof(float));
  rewind(fp);
  if (n > 0x7fffffffL) {  /* atom ids and counts are int */
    fclose(fp);
    st = COMDGB_ERR_ARG;
    goto done;
  }
  rec = (float *)malloc((size_t)n * 5 * sizeof(float) + 4);
  if (!rec || fread(rec, 5 * sizeof(float), (size_t)n, fp) != (size_t)n) {
    fclose(fp);
    st = rec ? COMDGB_ERR_IO : COMDGB_ERR_NOMEM;
    goto done;
  }
  fclose(fp);
  s = (simflat_t *)zalloc(sizeof *s);
  if (!s) {
    st = COMDGB_ERR_NOMEM;
    goto done;
  }
  s->pot = pot;
  s->bf = bf;
  s->defgrad = 0.0; /* blankSimulation's; allocDomains then takes strain 1 */
  s->comment = (char *)zalloc(1024);
  /* the reference holds its fixed bounds in floats (read.c:274, 287-289) */
  for (int m = 0; m < 3; m++) s->bounds[m] = bounds ? bounds[m] : (double)(float)kTimBounds[m];
  if ((st = alloc_domains(s))) goto done;
  xyz = (double *)malloc(3 * (size_t)n * sizeof(double) + 8);
  pxyz = (double *)calloc(3 * (size_t)n + 1, sizeof(double));
  masses = (double *)malloc((size_t)n * sizeof(double) + 8);
  ids = (int *)malloc((size_t)n * sizeof(int) + 4);
  types = (int *)malloc((size_t)n * sizeof(int) + 4);
  if (!xyz || !pxyz || !masses || !ids || !types) {
    st = COMDGB_ERR_NOMEM;
    goto done;
  }
  for (long i = 0; i < n; i++) {
    for (int m = 0; m < 3; m++) xyz[3 * i + m] = (double)rec[5 * i + m];
    ids[i] = (int)i;
    types[i] = 1;
    masses[i] = pot->mass;
  }
  if (device >= 0) {
    st = comdgb_put_atoms(s, (int)n, xyz, pxyz, ids, types, masses, device);
    from_gpu = st != 0;  /* comdgb_put_atoms recorded its own message */
  } else {
    for (long i = 0; i < n && !st; i++)
      st = put_atom(s, ids[i], types[i], masses[i], xyz + 3 * i, NULL);
  }
done:
  free(rec);
  free(xyz);
  free(pxyz);
  free(masses);
  free(ids);
  free(types);
  if (status) *status = st;
  if (st && !from_gpu) host_err(st, "comdgb_read_tim", path);
  if (st && s) {
    comdgb_sim_free_host(s);
    s = NULL;
  }
  return s;
}

void comdgb_seed(simflat_t *s, uint64_t seed, int disp_kind, double amp, double temp_k,
                 double mass_amu) {
  comdgb_seed_apply(s, seed, disp_kind, amp, temp_k, mass_amu);
}
