/*
 * comd_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement, in plain serial C with double precision, of CoMD's
 * force-and-integrate timestep (src-flat).  It is the oracle of the GB300
 * library's tests: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it, and never as the thing measured on the GPU or
 * shipped.
 *
 * Every function follows the reference loop for loop and operation for
 * operation (same evaluation order, no FMA contraction: build with
 * -ffp-contract=off), so for the same input it reproduces the reference's
 * double-precision results bit for bit.  That claim is pinned by the tests
 * against the reference itself, compiled from its sources into oracle/_ref
 * (see oracle/Makefile), and against the known answers of the reference's
 * own runs recorded under tests/golden/.
 *
 * Differences from the reference, all outside the arithmetic:
 *  - errors are returned as the reference's exit codes instead of exit()
 *    (e.g. -11 "Increase maxatoms", src-flat/domains.c:229);
 *  - the neighbour-box list is returned in a caller buffer instead of a
 *    static one (src-flat/domains.c:391-430);
 *  - the potential kind is a runtime argument instead of -DUSE_CHEBY.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "comdgb_simflat.h"
#include "comdgb_seed.h"

#define MAXAT COMDGB_MAXATOMS
#define NNBR COMDGB_NUMNEIGHBORS

enum { ORC_EAM_TABLE = 0, ORC_EAM_CHEBY = 1, ORC_LJ = 2 };

static int orc_periodic = 1; /* src-flat/mycommand.c:67 PERIODIC */

void orc_set_periodic(int p) { orc_periodic = p; }
int orc_get_periodic(void) { return orc_periodic; }

static void *orc_calloc(size_t n) {
  void *p = NULL;
  size_t padded = (n + 15) & ~(size_t)15;
  if (padded == 0) padded = 16;
  if (posix_memalign(&p, 128, padded)) return NULL;
  memset(p, 0, padded);
  return p;
}

/* ------------------------------------------------------------------ */
/* potential tables: src-flat/eam.c:130-249, 290-329, 347-398          */
/* ------------------------------------------------------------------ */

static void swap_bytes(void *p, int nelem, int esize, int doswap) {
  if (!doswap) return;
  unsigned char *c = (unsigned char *)p;
  for (int i = 0; i < nelem; i++, c += esize)
    for (int a = 0, b = esize - 1; a < b; a++, b--) {
      unsigned char t = c[a];
      c[a] = c[b];
      c[b] = t;
    }
}

/* allocPotentialArray, src-flat/eam.c:130-153: one guard below, two above,
 * x0 moved up by one interval */
static potentialarray_t *table_alloc(int n, double x0, double xn, double invdx) {
  potentialarray_t *a = (potentialarray_t *)orc_calloc(sizeof(potentialarray_t));
  if (!a) return NULL;
  double *v = (double *)orc_calloc((size_t)(n + 3) * sizeof(double));
  if (!v) { free(a); return NULL; }
  a->values = v + 1;
  a->n = n;
  a->invDx = invdx;
  a->xn = xn;
  a->x0 = x0 + (xn - x0) / (double)n;
  return a;
}

void orc_table_free(potentialarray_t *a) {
  if (!a) return;
  if (a->values) free(a->values - 1);
  free(a);
}

/* getPotentialArrayFromBinaryFile, src-flat/eam.c:156-249 */
static potentialarray_t *table_read(const char *path) {
  FILE *fp = fopen(path, "rb");
  if (!fp) return NULL;
  int rec = 0, n = 0, iflo = 0, ifhi = 0;
  double x0 = 0, xn = 0, invdx = 0;
  int ok = 1;
  ok &= fread(&rec, 4, 1, fp) == 1;
  int sw = rec > 4096;
  ok &= fread(&n, 4, 1, fp) == 1;
  swap_bytes(&n, 1, 4, sw);
  ok &= fread(&x0, 8, 1, fp) == 1;
  swap_bytes(&x0, 1, 8, sw);
  ok &= fread(&xn, 8, 1, fp) == 1;
  swap_bytes(&xn, 1, 8, sw);
  ok &= fread(&invdx, 8, 1, fp) == 1;
  swap_bytes(&invdx, 1, 8, sw);
  ok &= fread(&iflo, 4, 1, fp) == 1;
  swap_bytes(&iflo, 1, 4, sw);
  ok &= fread(&ifhi, 4, 1, fp) == 1;
  swap_bytes(&ifhi, 1, 4, sw);
  ok &= fread(&rec, 4, 1, fp) == 1; /* trailer of record 1 */
  ok &= fread(&rec, 4, 1, fp) == 1; /* header of record 2 */
  swap_bytes(&rec, 1, 4, sw);
  if (!ok || n <= 0 || rec != n * 8) { fclose(fp); return NULL; }
  potentialarray_t *a = table_alloc(n, x0, xn, invdx);
  if (!a) { fclose(fp); return NULL; }
  double *raw = (double *)malloc((size_t)n * 8);
  if (!raw || fread(raw, 8, (size_t)n, fp) != (size_t)n) {
    free(raw); orc_table_free(a); fclose(fp); return NULL;
  }
  swap_bytes(raw, n, 8, sw);
  for (int i = 0; i < n; i++) a->values[i] = raw[i];
  free(raw);
  double lo = iflo == 0 ? 0.0 : a->values[0];
  double hi = ifhi == 0 ? 0.0 : a->values[n - 1];
  a->values[-1] = lo;
  a->values[n] = hi;
  a->values[n + 1] = hi;
  fclose(fp);
  return a;
}

/* getMassFromFile / getLatFromFile, src-flat/eam.c:290-329: value on
 * line 2 / line 3 of the .doc file */
static double doc_value(const char *path, int line) {
  FILE *fp = fopen(path, "r");
  if (!fp) return -1.0;
  char buf[4096];
  double v = -1.0;
  for (int i = 0; i < line; i++)
    if (!fgets(buf, sizeof buf, fp)) { fclose(fp); return -1.0; }
  if (sscanf(buf, "%lf", &v) != 1) v = -1.0;
  fclose(fp);
  return v;
}

void orc_eam_free(eampotential_t *p) {
  if (!p) return;
  orc_table_free(p->phi);
  orc_table_free(p->rho);
  orc_table_free(p->f);
  free(p);
}

/* eamReadASCII, src-flat/eam.c:347-398; cutoff = phi.xn (:392) */
eampotential_t *orc_eam_read(const char *dir, const char *name) {
  char path[4096];
  eampotential_t *p = (eampotential_t *)orc_calloc(sizeof(eampotential_t));
  if (!p) return NULL;
  snprintf(path, sizeof path, "%s/%s.phi", dir, name);
  p->phi = table_read(path);
  snprintf(path, sizeof path, "%s/%s.rho", dir, name);
  p->rho = table_read(path);
  snprintf(path, sizeof path, "%s/%s.f", dir, name);
  p->f = table_read(path);
  snprintf(path, sizeof path, "%s/%s.doc", dir, name);
  p->mass = doc_value(path, 2);
  p->lat = doc_value(path, 3);
  if (p->mass < 0.0 || !p->phi || !p->rho || !p->f) { orc_eam_free(p); return NULL; }
  p->cutoff = p->phi->xn;
  return p;
}

/* eamInterpolateDeriv, src-flat/eam.c:401-434: 3-point quadratic with
 * guard cells; derivative is zero for the first interval */
void orc_table_eval(const potentialarray_t *a, double r, double *value, double *deriv) {
  if (r < a->x0) r = a->x0;
  else if (r > a->xn) r = a->xn;
  r = (r - a->x0) * a->invDx;
  int i1 = (int)floor(r);
  r = r - floor(r);
  const double *v = a->values;
  double gi = v[i1 + 1] - v[i1 - 1];
  double gi1 = v[i1 + 2] - v[i1];
  *value = v[i1] + 0.5 * r * (r * (v[i1 + 1] + v[i1 - 1] - 2.0 * v[i1]) + gi);
  if (i1 <= 0) *deriv = 0.0;
  else *deriv = 0.5 * (gi + r * (gi1 - gi)) * a->invDx;
}

/* ------------------------------------------------------------------ */
/* Chebyshev series: src-flat/cheby.c:15-60, 99-179, 219-310           */
/* ------------------------------------------------------------------ */

#define ORC_PI 3.141592653589793

/* eamInterpolateDerivlocal, src-flat/cheby.c:15-60: the table evaluator
 * with values above 1e10 (the F table's 1e60 sentinel) replaced by 0 */
static double table_sample(const potentialarray_t *a, double r) {
  double x0 = a->x0, xn = a->xn, invdx = a->invDx;
  if (r < x0) r = x0;
  else if (r > xn) r = xn;
  r = (r - x0) * invdx;
  int i1 = (int)floor(r);
  r = r - floor(r);
  const double *v = a->values;
  double gi = v[i1 + 1] - v[i1 - 1];
  double value = v[i1] + 0.5 * r * (r * (v[i1 + 1] + v[i1 - 1] - 2.0 * v[i1]) + gi);
  if (value > 1.0e10) value = 0.0;
  return value;
}

/* genCheb, src-flat/cheby.c:125-179: n coefficients from samples at the
 * Chebyshev nodes of [x0, xn] */
static potentialarray_t *cheb_fit(const potentialarray_t *t, int n) {
  potentialarray_t *c = (potentialarray_t *)orc_calloc(sizeof(potentialarray_t));
  c->x0 = t->x0;
  c->xn = t->xn;
  c->n = n;
  c->values = (double *)orc_calloc((size_t)n * sizeof(double));
  double a = t->x0, b = t->xn;
  double bma = 0.5 * (b - a), bpa = 0.5 * (b + a);
  double *fk = (double *)malloc((size_t)n * sizeof(double));
  for (int k = 0; k < n; k++) {
    double y = cos(ORC_PI * (k + 0.5) / n);
    fk[k] = table_sample(t, y * bma + bpa);
  }
  double fac = 2.0 / n;
  for (int j = 0; j < n; j++) {
    double sum = 0.0;
    for (int k = 0; k < n; k++) sum += fk[k] * cos(ORC_PI * j * (k + 0.5) / n);
    c->values[j] = fac * sum;
  }
  free(fk);
  return c;
}

/* genDer, src-flat/cheby.c:219-270: derivative series by the downward
 * recurrence c'_{j-1} = c'_{j+1} + 2j c_j, scaled by 2/(b-a) */
static potentialarray_t *cheb_deriv(const potentialarray_t *c) {
  int n = c->n;
  potentialarray_t *d = (potentialarray_t *)orc_calloc(sizeof(potentialarray_t));
  d->x0 = c->x0;
  d->xn = c->xn;
  d->invDx = 1.0;
  d->n = n;
  d->values = (double *)orc_calloc((size_t)n * sizeof(double));
  double *cd = d->values;
  const double *cc = c->values;
  cd[n - 1] = 0.0;
  cd[n - 2] = 2.0 * (n - 1) * cc[n - 1];
  for (int j = n - 2; j > 0; j--) cd[j - 1] = cd[j + 1] + 2 * (j)*cc[j];
  double con = 2.0 / (c->xn - c->x0);
  for (int j = 0; j < n; j++) cd[j] = cd[j] * con;
  return d;
}

/* setChebPot, src-flat/cheby.c:99-121 */
eam_cheby_t *orc_cheb_make(const eampotential_t *p, int n) {
  eam_cheby_t *c = (eam_cheby_t *)orc_calloc(sizeof(eam_cheby_t));
  c->cutoff = p->cutoff;
  c->mass = p->mass;
  c->lat = p->lat;
  c->phi = cheb_fit(p->phi, n);
  c->dphi = cheb_deriv(c->phi);
  c->rho = cheb_fit(p->rho, n);
  c->drho = cheb_deriv(c->rho);
  c->f = cheb_fit(p->f, n);
  c->df = cheb_deriv(c->f);
  return c;
}

static void cheb_series_free(potentialarray_t *c) {
  if (!c) return;
  free(c->values);
  free(c);
}

void orc_cheb_free(eam_cheby_t *c) {
  if (!c) return;
  cheb_series_free(c->phi);
  cheb_series_free(c->rho);
  cheb_series_free(c->f);
  cheb_series_free(c->dphi);
  cheb_series_free(c->drho);
  cheb_series_free(c->df);
  free(c);
}

/* eamCheb, src-flat/cheby.c:276-310: Clenshaw sum; x is clamped from below
 * only (the upper clamp at :293 is a no-op in the reference) */
double orc_cheb_eval(const potentialarray_t *c, double x) {
  double a = c->x0, b = c->xn;
  const double *cf = c->values;
  int m = c->n;
  if (x < a) x = a;
  double d = 0.0, dd = 0.0, sv;
  double y = (2.0 * x - a - b) / (b - a);
  double y2 = 2.0 * y;
  for (int j = m - 1; j > 0; j--) {
    sv = d;
    d = y2 * d - dd + cf[j];
    dd = sv;
  }
  return y * d - dd + 0.5 * cf[0];
}

/* ------------------------------------------------------------------ */
/* link cells: src-flat/domains.c                                      */
/* ------------------------------------------------------------------ */

void orc_sim_free(simflat_t *s) {
  if (!s) return;
  free(s->dcenter); free(s->natoms); free(s->id); free(s->iType);
  free(s->mass); free(s->r); free(s->p); free(s->f); free(s->rho); free(s->fi);
  free(s->comment);
  free(s);
}

/* allocDomains, src-flat/domains.c:155-200: nbx = floor(L/(rc*bf*strain))
 * with the x-strain equal to the deformation gradient; dcenter is the box's
 * lower corner.  Returns 3 (the reference's abort code) if a dimension has
 * no box. */
int orc_alloc_domains(simflat_t *s) {
  double strain[3] = {s->defgrad, 1.0, 1.0};
  if (strain[0] == 0.0) strain[0] = 1.0;
  double bf = s->bf;
  if (bf == 0.0) bf = 1.0;
  s->nboxes = 1;
  for (int j = 0; j < 3; j++) {
    s->nbx[j] = (int)floor(s->bounds[j] / (s->pot->cutoff * bf * strain[j]));
    if (s->nbx[j] < 1) return 3;
    s->nboxes = s->nboxes * s->nbx[j];
    s->boxsize[j] = s->bounds[j] / (double)s->nbx[j];
  }
  size_t nb = (size_t)s->nboxes, ns = nb * MAXAT;
  s->dcenter = (comdgb_real3 *)orc_calloc(nb * sizeof(comdgb_real3));
  s->natoms = (int *)orc_calloc(nb * sizeof(int));
  s->id = (int *)orc_calloc(ns * sizeof(int));
  s->iType = (int *)orc_calloc(ns * sizeof(int));
  s->mass = (double *)orc_calloc(ns * sizeof(double));
  s->r = (comdgb_real3 *)orc_calloc(ns * sizeof(comdgb_real3));
  s->p = (comdgb_real3 *)orc_calloc(ns * sizeof(comdgb_real3));
  s->f = (comdgb_real4 *)orc_calloc(ns * sizeof(comdgb_real4));
  s->fi = (double *)orc_calloc(ns * sizeof(double));
  s->rho = (double *)orc_calloc(ns * sizeof(double));
  if (!s->dcenter || !s->natoms || !s->id || !s->iType || !s->mass || !s->r ||
      !s->p || !s->f || !s->fi || !s->rho)
    return 4;
  s->stateflag |= 1;
  for (int b = 0; b < s->nboxes; b++) {
    int ib[3] = {b % s->nbx[0], (b / s->nbx[0]) % s->nbx[1], b / s->nbx[0] / s->nbx[1]};
    for (int j = 0; j < 3; j++) s->dcenter[b][j] = s->boxsize[j] * (double)ib[j];
  }
  return 0;
}

/* putAtomInBox, src-flat/domains.c:237-291 with getBoxIDWorldCoords
 * (:71-82): wrap once into the primary period, box from floor(x/boxsize),
 * append.  The reference has no overflow check; this returns -11 when the
 * box is full and -12 when the box index is out of range. */
int orc_put_atom(simflat_t *s, int id, int itype, double mass, double x, double y,
                 double z, double px, double py, double pz) {
  double xyz[3] = {x, y, z};
  for (int m = 0; m < 3; m++) {
    if (xyz[m] < 0.0) xyz[m] += s->bounds[m];
    else if (xyz[m] >= s->bounds[m]) xyz[m] -= s->bounds[m];
  }
  int ib[3];
  for (int m = 0; m < 3; m++) ib[m] = (int)(floor(xyz[m] / s->boxsize[m]));
  for (int m = 0; m < 3; m++)
    if (ib[m] < 0 || ib[m] >= s->nbx[m]) return -12;
  int b = ib[0] + s->nbx[0] * ib[1] + s->nbx[0] * s->nbx[1] * ib[2];
  if (s->natoms[b] >= MAXAT) return -11;
  int off = b * MAXAT + s->natoms[b];
  s->ntot++;
  s->natoms[b]++;
  s->id[off] = id;
  s->iType[off] = itype;
  s->mass[off] = mass;
  for (int m = 0; m < 3; m++) s->r[off][m] = (double)(xyz[m] - s->dcenter[b][m]);
  s->p[off][0] = px;
  s->p[off][1] = py;
  s->p[off][2] = pz;
  s->f[off][0] = 0.0;
  s->f[off][1] = 0.0;
  s->f[off][2] = 0.0;
  return 0;
}

/* create_fcc_lattice, src-flat/ic_fcc.c:63-141: the half-lattice walk
 * (counters i, j, k never reset) keeps points with i+j+k odd; generation
 * order is the atom id order. */
simflat_t *orc_fcc(int nx, int ny, int nz, double lat, double defgrad, double bf,
                   pmd_base_potential_t *pot, int *status) {
  simflat_t *s = (simflat_t *)orc_calloc(sizeof(simflat_t));
  *status = 0;
  s->pot = pot;
  s->comment = (char *)orc_calloc(1024);
  double halflat = lat / 2.0;
  s->defgrad = defgrad;
  s->bounds[0] = nx * lat * defgrad;
  s->bounds[1] = ny * lat;
  s->bounds[2] = nz * lat;
  s->bf = bf;
  int rc = orc_alloc_domains(s);
  if (rc) { *status = rc; orc_sim_free(s); return NULL; }
  int i = 0, j = 0, k = 0, n = 0;
  double z = lat / 4.0;
  while (z < s->bounds[2]) {
    double y = lat / 4.0;
    while (y < s->bounds[1]) {
      double x = lat * defgrad / 4.0;
      while (x < s->bounds[0]) {
        if ((i + j + k) % 2) {
          rc = orc_put_atom(s, n++, 1, pot->mass, x, y, z, 0, 0, 0);
          if (rc) { *status = rc; orc_sim_free(s); return NULL; }
        }
        x += halflat * defgrad;
        i++;
      }
      y += halflat;
      j++;
    }
    z += halflat;
    k++;
  }
  return s;
}

/* deep copy (test helper) */
simflat_t *orc_sim_clone(const simflat_t *a) {
  simflat_t *s = (simflat_t *)orc_calloc(sizeof(simflat_t));
  *s = *a;
  size_t nb = (size_t)a->nboxes, ns = nb * MAXAT;
#define DUP(field, bytes)                       \
  s->field = orc_calloc(bytes);                 \
  memcpy(s->field, a->field, bytes);
  DUP(dcenter, nb * sizeof(comdgb_real3));
  DUP(natoms, nb * sizeof(int));
  DUP(id, ns * sizeof(int));
  DUP(iType, ns * sizeof(int));
  DUP(mass, ns * sizeof(double));
  DUP(r, ns * sizeof(comdgb_real3));
  DUP(p, ns * sizeof(comdgb_real3));
  DUP(f, ns * sizeof(comdgb_real4));
  DUP(rho, ns * sizeof(double));
  DUP(fi, ns * sizeof(double));
#undef DUP
  s->comment = (char *)orc_calloc(1024);
  if (a->comment) memcpy(s->comment, a->comment, 1024);
  return s;
}

/* copyAtom, src-flat/domains.c:209-222 */
static void copy_atom(simflat_t *s, int ia, int ib, int ja, int jb) {
  int io = MAXAT * ib + ia, jo = MAXAT * jb + ja;
  s->id[jo] = s->id[io];
  s->iType[jo] = s->iType[io];
  s->mass[jo] = s->mass[io];
  memcpy(s->r[jo], s->r[io], sizeof(comdgb_real3));
  memcpy(s->f[jo], s->f[io], sizeof(comdgb_real4));
  memcpy(s->p[jo], s->p[io], sizeof(comdgb_real3));
  s->fi[jo] = s->fi[io];
  s->rho[jo] = s->rho[io];
}

/* moveAtom, src-flat/domains.c:224-236: append to jbox, abort when it
 * reaches MAXATOMS, then fill the hole with ibox's last atom */
static int move_atom(simflat_t *s, int i, int ib, int jb) {
  int nj = s->natoms[jb];
  copy_atom(s, i, ib, nj, jb);
  s->natoms[jb]++;
  if (s->natoms[jb] >= MAXAT) return -11;
  s->natoms[ib]--;
  int ni = s->natoms[ib];
  if (ni) copy_atom(s, ni, ib, i, ib);
  return 0;
}

/* getIBoxFromIxyz3 / getIBoxFromIxyz3NP, src-flat/domains.c:297-325 */
static int box_from_ixyz(const simflat_t *s, int *ix) {
  if (!orc_periodic)
    for (int j = 0; j < 3; j++)
      if (ix[j] < 0 || ix[j] >= s->nbx[j]) return -1;
  for (int j = 0; j < 3; j++) {
    if (ix[j] < 0) ix[j] += s->nbx[j];
    else if (ix[j] >= s->nbx[j]) ix[j] -= s->nbx[j];
  }
  return ix[0] + ix[1] * s->nbx[0] + ix[2] * s->nbx[0] * s->nbx[1];
}

/* getIxyz3, src-flat/domains.c:332-337 */
static void box_ixyz(const simflat_t *s, int b, int *ix) {
  ix[0] = b % s->nbx[0];
  ix[1] = (b / s->nbx[0]) % s->nbx[1];
  ix[2] = (b / s->nbx[0] / s->nbx[1]) % s->nbx[2];
}

/* reBoxAll, src-flat/domains.c:347-389: boxes in ascending order, each
 * scanned with swap-remove; an atom leaves by at most one box per axis */
int orc_rebox_all(simflat_t *s) {
  for (int b = 0; b < s->nboxes; b++) {
    int ixo[3];
    box_ixyz(s, b, ixo);
    int i = 0, off = b * MAXAT;
    while (i < s->natoms[b]) {
      int ixn[3];
      double rn[3];
      memcpy(rn, s->r[off], sizeof rn);
      for (int k = 0; k < 3; k++) {
        if (s->r[off][k] < 0.0) {
          ixn[k] = ixo[k] - 1;
          rn[k] += s->boxsize[k];
        } else if (s->r[off][k] >= s->boxsize[k]) {
          ixn[k] = ixo[k] + 1;
          rn[k] -= s->boxsize[k];
        } else {
          ixn[k] = ixo[k];
        }
      }
      int jb = box_from_ixyz(s, ixn);
      if (jb < 0 || jb == b) {
        i++;
        off++;
      } else {
        memcpy(s->r[off], rn, sizeof rn);
        int rc = move_atom(s, i, b, jb);
        if (rc) return rc;
      }
    }
  }
  return 0;
}

/* getNeighborBoxes, src-flat/domains.c:391-430: ids in x-outer, y, z-inner
 * order including the box itself; invalid (non-periodic) ids are dropped;
 * a single-box system has the one entry 0.  Returns the count. */
int orc_neighbor_boxes(const simflat_t *s, int b, int *nbrs) {
  for (int q = 0; q < NNBR; q++) nbrs[q] = -1;
  if (s->nboxes == 1) {
    nbrs[0] = 0;
    return 1;
  }
  int ix[3];
  box_ixyz(s, b, ix);
  int cnt = 0;
  for (int i = ix[0] - 1; i <= ix[0] + 1; i++)
    for (int j = ix[1] - 1; j <= ix[1] + 1; j++)
      for (int k = ix[2] - 1; k <= ix[2] + 1; k++) {
        int t[3] = {i, j, k};
        int nb = box_from_ixyz(s, t);
        nbrs[cnt] = nb;
        if (nb >= 0) cnt++;
      }
  return cnt;
}

/* minimum-image box offset, src-flat/eam.c:494-502 */
static void box_offset(const simflat_t *s, int ib, int jb, double *drbox) {
  for (int j = 0; j < 3; j++) {
    drbox[j] = s->dcenter[ib][j] - s->dcenter[jb][j];
    if (orc_periodic) {
      if (drbox[j] < -0.5 * s->bounds[j]) drbox[j] += s->bounds[j];
      else if (drbox[j] > 0.5 * s->bounds[j]) drbox[j] -= s->bounds[j];
    }
  }
}

/* fromFileGzip (src-flat/read.c:155-241) on an uncompressed clsman file:
 * "natoms nmove", a comment line, the bounds, then "x y z itype px py pz"
 * per atom; atom i goes in by putAtomInBox(s, i, 1, 0, mass, ...), line by
 * line as gzgets reads it */
simflat_t *orc_read_clsman(const char *path, pmd_base_potential_t *pot, double bf,
                           int *status) {
  char line[16348];
  *status = 0;
  FILE *fp = fopen(path, "r");
  if (!fp) {
    *status = -3; /* "Input file does not exist", docompute.c:126 */
    return NULL;
  }
  simflat_t *s = (simflat_t *)orc_calloc(sizeof(simflat_t));
  s->pot = pot;
  s->bf = bf;
  s->comment = (char *)orc_calloc(1024);
  int natoms = 0, nmove = 0, rc = 0;
  if (!fgets(line, sizeof line, fp) || sscanf(line, "%d%d", &natoms, &nmove) < 1) rc = -33;
  if (!rc && fgets(line, sizeof line, fp)) {
    size_t n = strlen(line);
    memcpy(s->comment, line, n < 1023 ? n : 1023);
  }
  if (!rc && (!fgets(line, sizeof line, fp) ||
              sscanf(line, "%lg %lg %lg", s->bounds, s->bounds + 1, s->bounds + 2) != 3))
    rc = -33;
  if (!rc) rc = orc_alloc_domains(s);
  for (int i = 0; i < natoms && !rc; i++) {
    double x, y, z, px, py, pz;
    int itype;
    if (!fgets(line, sizeof line, fp) ||
        sscanf(line, "%lg %lg %lg %d %lg %lg %lg", &x, &y, &z, &itype, &px, &py, &pz) != 7) {
      rc = -33;
      break;
    }
    rc = orc_put_atom(s, i, 0, pot->mass, x, y, z, px, py, pz);
  }
  fclose(fp);
  if (rc) {
    *status = rc;
    orc_sim_free(s);
    return NULL;
  }
  return s;
}

/* ------------------------------------------------------------------ */
/* forces                                                              */
/* ------------------------------------------------------------------ */

/* eamForce, src-flat/eam.c:438-660.  f holds +grad U; f[3] the per-atom
 * energy; stress is the x-x embedding term only, divided by the volume. */
int orc_eam_force(simflat_t *s, int use_cheby) {
  const eampotential_t *pot = (const eampotential_t *)s->pot;
  const eam_cheby_t *ch = s->ch_pot;
  if (use_cheby && !ch) return -20;
  double rcut2 = pot->cutoff * pot->cutoff;
  double etot = 0.0;
  size_t ns = (size_t)s->nboxes * MAXAT;
  memset(s->f, 0, ns * sizeof(comdgb_real4));
  memset(s->fi, 0, ns * sizeof(double));
  memset(s->rho, 0, ns * sizeof(double));
  s->stress = 0.0;
  int nbrs[NNBR];

  /* pass 1: pair energy, pair force and density over half box pairs */
  for (int ib = 0; ib < s->nboxes; ib++) {
    int ni = s->natoms[ib];
    int nn = orc_neighbor_boxes(s, ib, nbrs);
    for (int q = 0; q < nn; q++) {
      int jb = nbrs[q];
      if (jb < 0) break;
      if (jb < ib) continue;
      double drbox[3];
      box_offset(s, ib, jb, drbox);
      int nj = s->natoms[jb];
      for (int ii = 0, io = MAXAT * ib; ii < ni; ii++, io++) {
        for (int ij = 0, jo = MAXAT * jb; ij < nj; ij++, jo++) {
          if (ib == jb && ij <= ii) continue;
          double dr[3], r2 = 0.0;
          for (int k = 0; k < 3; k++) {
            dr[k] = drbox[k] + s->r[io][k] - s->r[jo][k];
            r2 += dr[k] * dr[k];
          }
          if (r2 > rcut2) continue;
          double r = sqrt(r2), phiv, dphi, rhov, drho;
          if (use_cheby) {
            phiv = orc_cheb_eval(ch->phi, r);
            dphi = orc_cheb_eval(ch->dphi, r);
            rhov = orc_cheb_eval(ch->rho, r);
            drho = orc_cheb_eval(ch->drho, r);
          } else {
            orc_table_eval(pot->phi, r, &phiv, &dphi);
            orc_table_eval(pot->rho, r, &rhov, &drho);
          }
          (void)drho;
          for (int k = 0; k < 3; k++) {
            s->f[io][k] += dphi * dr[k] / r;
            s->f[jo][k] -= dphi * dr[k] / r;
          }
          etot += phiv;
          s->f[io][3] += phiv / 2.0;
          s->f[jo][3] += phiv / 2.0;
          s->rho[io] += rhov;
          s->rho[jo] += rhov;
        }
      }
    }
  }

  /* pass 2: embedding energy F(rho) and F'(rho) per atom */
  for (int ib = 0; ib < s->nboxes; ib++) {
    for (int ii = 0, io = MAXAT * ib; ii < s->natoms[ib]; ii++, io++) {
      double fv, fp;
      if (use_cheby) {
        fv = orc_cheb_eval(ch->f, s->rho[io]);
        fp = orc_cheb_eval(ch->df, s->rho[io]);
      } else {
        orc_table_eval(pot->f, s->rho[io], &fv, &fp);
      }
      s->fi[io] = fp;
      etot += fv;
      s->f[io][3] += fv;
    }
  }

  /* pass 3: embedding force (F'_i + F'_j) rho'(r) dr/r and the stress */
  for (int ib = 0; ib < s->nboxes; ib++) {
    int ni = s->natoms[ib];
    orc_neighbor_boxes(s, ib, nbrs);
    for (int ii = 0, io = MAXAT * ib; ii < ni; ii++, io++) {
      for (int q = 0; q < NNBR; q++) {
        int jb = nbrs[q];
        if (jb < 0) break;
        if (jb < ib) continue;
        double drbox[3];
        box_offset(s, ib, jb, drbox);
        int nj = s->natoms[jb];
        for (int ij = 0, jo = MAXAT * jb; ij < nj; ij++, jo++) {
          if (ib == jb && ij <= ii) continue;
          double dr[3], r2 = 0.0;
          for (int k = 0; k < 3; k++) {
            dr[k] = drbox[k] + s->r[io][k] - s->r[jo][k];
            r2 += dr[k] * dr[k];
          }
          if (r2 >= rcut2) continue;
          double r = sqrt(r2), rhov, drho;
          if (use_cheby) drho = orc_cheb_eval(ch->drho, r);
          else orc_table_eval(pot->rho, r, &rhov, &drho);
          for (int k = 0; k < 3; k++) {
            s->f[io][k] += (s->fi[io] + s->fi[jo]) * drho * dr[k] / r;
            s->f[jo][k] -= (s->fi[io] + s->fi[jo]) * drho * dr[k] / r;
          }
          s->stress += 2.0 * (s->fi[io] + s->fi[jo]) * drho * dr[0] / r * dr[0];
        }
      }
    }
  }
  s->e = etot;
  s->stress = s->stress / (s->bounds[0] * s->bounds[1] * s->bounds[2]);
  return 0;
}

/* LJ, src-flat/ljForce.c:89-224.  f holds the physical force -grad U;
 * f[3] is the unscaled half pair sum r^-6(s6 r^-6 - 1)/2; the stress adds
 * -p_x^2/m once per (atom, non-empty neighbour box). */
int orc_lj_force(simflat_t *s) {
  const ljpotential_t *pot = (const ljpotential_t *)s->pot;
  double sigma = pot->sigma, epsilon = pot->epsilon, rcut = pot->cutoff;
  double r2cut = rcut * rcut;
  double etot = 0.0;
  s->e = 0.0;
  memset(s->f, 0, (size_t)s->nboxes * MAXAT * sizeof(comdgb_real4));
  double s6 = sigma * sigma * sigma * sigma * sigma * sigma;
  s->stress = 0.0;
  int nbrs[NNBR];
  for (int ib = 0; ib < s->nboxes; ib++) {
    int ni = s->natoms[ib];
    if (!ni) continue;
    int nn = orc_neighbor_boxes(s, ib, nbrs);
    for (int q = 0; q < nn; q++) {
      int jb = nbrs[q];
      if (jb < 0) break;
      double drbox[3];
      box_offset(s, ib, jb, drbox);
      int nj = s->natoms[jb];
      if (!nj) continue;
      for (int ii = 0, io = ib * MAXAT; ii < ni; ii++, io++) {
        s->stress -= s->p[io][0] * s->p[io][0] / s->mass[io];
        int idi = s->id[io];
        for (int ij = 0, jo = MAXAT * jb; ij < nj; ij++, jo++) {
          int idj = s->id[jo];
          if (idj <= idi) continue;
          double dr[3], r2 = 0.0;
          for (int m = 0; m < 3; m++) {
            dr[m] = drbox[m] + s->r[io][m] - s->r[jo][m];
            r2 += dr[m] * dr[m];
          }
          if (r2 > r2cut) continue;
          r2 = 1.0 / r2;
          double r6 = r2 * r2 * r2;
          s->f[io][3] += 0.5 * r6 * (s6 * r6 - 1.0);
          s->f[jo][3] += 0.5 * r6 * (s6 * r6 - 1.0);
          etot += r6 * (s6 * r6 - 1.0);
          double fr = 4.0 * epsilon * s6 * r6 * r2 * (12.0 * s6 * r6 - 6.0);
          for (int m = 0; m < 3; m++) {
            s->f[io][m] += dr[m] * fr;
            s->f[jo][m] -= dr[m] * fr;
          }
          s->stress += 2.0 * fr * dr[0] * dr[0];
        }
      }
    }
  }
  etot = etot * 4.0 * epsilon * s6;
  s->e = etot;
  s->stress = s->stress / (s->bounds[0] * s->bounds[1] * s->bounds[2]);
  return 0;
}

int orc_force(simflat_t *s, int kind) {
  if (kind == ORC_LJ) return orc_lj_force(s);
  return orc_eam_force(s, kind == ORC_EAM_CHEBY);
}

/* ------------------------------------------------------------------ */
/* velocity Verlet: src-flat/timestep.c:62-140                         */
/* ------------------------------------------------------------------ */

/* s -> (0.529/2.418e-17), src-flat/include/constants.h:61 */
static const double orc_bohr_per_atu = (double)0.529 / (double)2.418e-17;

/* advanceVelocity, src-flat/timestep.c:62-74 */
void orc_advance_velocity(simflat_t *s, double dt) {
  for (int b = 0; b < s->nboxes; b++)
    for (int ii = 0, o = MAXAT * b; ii < s->natoms[b]; ii++, o++)
      for (int k = 0; k < 3; k++) s->p[o][k] -= dt * s->f[o][k];
}

/* advancePositions, src-flat/timestep.c:76-108, without the reBoxAll */
void orc_advance_positions(simflat_t *s, double dt) {
  double rmass = (double)(COMDGB_AMU_TO_ME * (double)s->pot->mass);
  for (int b = 0; b < s->nboxes; b++) {
    if (!s->natoms[b]) continue;
    for (int ii = 0, o = MAXAT * b; ii < s->natoms[b]; ii++, o++)
      for (int k = 0; k < 3; k++) s->r[o][k] += dt * s->p[o][k] / rmass;
  }
}

/* nTimeSteps, src-flat/timestep.c:114-140: n x {r += dt/2 p/M; reBoxAll;
 * F; p -= dt f; r += dt/2 p/M; reBoxAll} and a final force call.  dt is
 * in seconds.  Returns 0 or the first error code; the energy is s->e. */
int orc_ntimesteps(int n, simflat_t *s, double dt, int kind) {
  int rc;
  dt = dt * orc_bohr_per_atu;
  for (int i = 0; i < n; i++) {
    orc_advance_positions(s, dt / 2.0);
    if ((rc = orc_rebox_all(s))) return rc;
    if ((rc = orc_force(s, kind))) return rc;
    orc_advance_velocity(s, dt);
    orc_advance_positions(s, dt / 2.0);
    if ((rc = orc_rebox_all(s))) return rc;
  }
  return orc_force(s, kind);
}

/* ------------------------------------------------------------------ */
/* harness helpers                                                     */
/* ------------------------------------------------------------------ */

void orc_seed_apply(simflat_t *s, uint64_t seed, int disp_kind, double amp, double temp_k,
                    double mass_amu) {
  comdgb_seed_apply(s, seed, disp_kind, amp, temp_k, mass_amu);
}

/* kinetic energy sum p^2/(2M) with M = pot mass in electron masses */
double orc_kinetic(const simflat_t *s) {
  double rmass = COMDGB_AMU_TO_ME * s->pot->mass, ek = 0.0;
  for (int b = 0; b < s->nboxes; b++)
    for (int ii = 0, o = MAXAT * b; ii < s->natoms[b]; ii++, o++)
      for (int k = 0; k < 3; k++) ek += s->p[o][k] * s->p[o][k];
  return ek / (2.0 * rmass);
}

/* potential structs owned by the oracle for tests */
ljpotential_t *orc_lj_make(double sigma, double epsilon, double cutoff, double mass) {
  ljpotential_t *p = (ljpotential_t *)orc_calloc(sizeof(ljpotential_t));
  p->sigma = sigma;
  p->epsilon = epsilon;
  p->cutoff = cutoff;
  p->mass = mass;
  return p;
}

void orc_free(void *p) { free(p); }
