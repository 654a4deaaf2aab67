/*
 * CPU oracle: plain-C restatement of the BSAM 1.2 FAS V-cycle.
 * TEST INFRASTRUCTURE ONLY -- see bsam_oracle.h for scope and parity status
 * (pinned to the reference's own outputs, run by oracle/fortran_exec.py).
 *
 * Every routine cites the reference routine it restates (file:line, paths
 * within the reference project).  Evaluation order of each floating-point
 * expression follows the Fortran source left to right; build with
 * -ffp-contract=off so that no multiply-add is fused.
 */
#include "bsam_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXDEPTH 10 /* nodeinfodef.f90:62 */
#define INTERNALBC 999 /* nodeinfodef.f90:59 */
#define NLEV (2 * MAXDEPTH + 1)

/* C/F interpolation weights, boundary.f90:54-63 */
static const double A1 = -01.0 / 05.0;
static const double A2 = 02.0 / 03.0;
static const double A3 = 08.0 / 15.0;
static const double B1 = 05.0 / 32.0;
static const double B2 = 15.0 / 16.0;
static const double B3 = -03.0 / 32.0;
static const double C1 = 09.0 / 16.0;
static const double C2 = 03.0 / 16.0;
static const double C3 = 03.0 / 16.0;
static const double C4 = 01.0 / 16.0;

typedef struct {
  int level, id, parent_id, parent;
  int mx[3], mglobal[3][2], mbounds[3][2], mthbc[6];
  double dx[3], xlower[3];
  int cmx[3];
  int qlo[3], qn[3]; /* q, qold: ghosted */
  int clo[3], cn[3]; /* qc: ghosted, coarse */
  int fn[3];         /* f, rf, ftmp: interior, lower bound 1 */
  double *q, *qold, *qc, *f, *rf, *ftmp;
} OPatch;

struct bsamo_hier {
  int ndims, nrvars, mbc, problem;
  double dt, eps, eps2, gamma, lambda, czero;
  double cpress; /* growth plugin: pressure source coefficient */
  double qpo[10];
  int np, cap;
  OPatch* p;
  int committed;
  int lev_n[NLEV];
  int* lev_list[NLEV];
  int periodic, nperoff, peroffidx[13];
  int mxmax[MAXDEPTH + 1][3];
  int minlevel_present, maxlevel_present;
  double integral[2];
  int has_root_xupper; /* built by bsamo_build_uniform: the root's xupper */
  double root_xupper[3];
};

/* ------------------------------------------------------------------ */
/* indexing                                                            */

static inline size_t iq(const OPatch* p, int i, int j, int k, int v) {
  return (((size_t)v * p->qn[2] + (size_t)(k - p->qlo[2])) * p->qn[1] +
          (size_t)(j - p->qlo[1])) * p->qn[0] + (size_t)(i - p->qlo[0]);
}
static inline size_t ic(const OPatch* p, int i, int j, int k, int v) {
  return (((size_t)v * p->cn[2] + (size_t)(k - p->clo[2])) * p->cn[1] +
          (size_t)(j - p->clo[1])) * p->cn[0] + (size_t)(i - p->clo[0]);
}
static inline size_t iff(const OPatch* p, int i, int j, int k, int v) {
  return (((size_t)v * p->fn[2] + (size_t)(k - 1)) * p->fn[1] +
          (size_t)(j - 1)) * p->fn[0] + (size_t)(i - 1);
}
#define Q(p, i, j, k, v) ((p)->q[iq((p), (i), (j), (k), (v))])
#define QO(p, i, j, k, v) ((p)->qold[iq((p), (i), (j), (k), (v))])
#define QC(p, i, j, k, v) ((p)->qc[ic((p), (i), (j), (k), (v))])
#define FF(p, i, j, k, v) ((p)->f[iff((p), (i), (j), (k), (v))])
#define RF(p, i, j, k, v) ((p)->rf[iff((p), (i), (j), (k), (v))])
#define FT(p, i, j, k, v) ((p)->ftmp[iff((p), (i), (j), (k), (v))])

static OPatch* find_patch(const bsamo_hier* h, int id) {
  for (int n = 0; n < h->np; n++)
    if (h->p[n].id == id) return &h->p[n];
  return NULL;
}
static OPatch* parent_of(bsamo_hier* h, const OPatch* p) {
  return p->parent >= 0 ? &h->p[p->parent] : NULL;
}
static int nlev(const bsamo_hier* h, int level) {
  if (level < -MAXDEPTH || level > MAXDEPTH) return 0;
  return h->lev_n[level + MAXDEPTH];
}
/* The n-th patch of a level in the reference's visiting order:
 * ApplyOnLevel walks a level from its youngest node to its eldest
 * (treeops.f90:536-550; CreateChild makes each new node the youngest of
 * its level, :349-395), i.e. the reverse of the order of creation that
 * lev_list keeps. */
static int lev_index(const bsamo_hier* h, int level, int n) {
  return h->lev_list[level + MAXDEPTH][h->lev_n[level + MAXDEPTH] - 1 - n];
}
static OPatch* lev_patch(bsamo_hier* h, int level, int n) {
  return &h->p[lev_index(h, level, n)];
}
static inline int imod(int a, int b) { int r = a % b; return r < 0 ? r + b : r; }

/* ------------------------------------------------------------------ */
/* construction                                                        */

int bsamo_create(int ndims, int nrvars, int mbc, int problem,
                 const double* params, int nparams, const double* qpo,
                 bsamo_hier** out) {
  if (!out) return -1;
  if (ndims < 2 || ndims > 3) return -2;
  if (nrvars < 1 || nrvars > 10) return -2;
  if (mbc < 1 || mbc > 2) return -2; /* RootInit, bsamroutines.f90:305-308 */
  if (problem != BSAMO_PROBLEM_CH && problem != BSAMO_PROBLEM_BIOGROWTH &&
      problem != BSAMO_PROBLEM_GROWTH)
    return -2;
  if (nparams < 2) return -2;
  if ((problem == BSAMO_PROBLEM_GROWTH) != (nrvars == 3)) return -2;
  if (problem == BSAMO_PROBLEM_GROWTH && nparams < 6) return -2;
  bsamo_hier* h = (bsamo_hier*)calloc(1, sizeof(*h));
  h->ndims = ndims;
  h->nrvars = nrvars;
  h->mbc = mbc;
  h->problem = problem;
  h->dt = params[0];
  h->eps = params[1];
  h->eps2 = h->eps * h->eps; /* SetProb, CH/problem.f90:32 */
  h->gamma = nparams > 2 ? params[2] : 0.0;
  h->lambda = nparams > 3 ? params[3] : 0.0;
  h->czero = nparams > 4 ? params[4] : 0.0;
  h->cpress = nparams > 5 ? params[5] : 0.0;
  for (int v = 0; v < 10; v++) h->qpo[v] = (qpo && v < nrvars) ? qpo[v] : 0.0;
  *out = h;
  return 0;
}

int bsamo_destroy(bsamo_hier* h) {
  if (!h) return 0;
  for (int n = 0; n < h->np; n++) {
    OPatch* p = &h->p[n];
    free(p->q); free(p->qold); free(p->qc); free(p->f); free(p->rf);
    free(p->ftmp);
  }
  for (int l = 0; l < NLEV; l++) free(h->lev_list[l]);
  free(h->p);
  free(h);
  return 0;
}

int bsamo_patch_add(bsamo_hier* h, int level, int id, int parent_id,
                    const int mx[3], const int mglobal[6],
                    const int mbounds[6], const int mthbc[6],
                    const double dx[3], const double xlower[3]) {
  if (!h || h->committed) return -1;
  if (level < -MAXDEPTH || level > MAXDEPTH) return -2;
  if (find_patch(h, id)) return -2;
  if (h->np == h->cap) {
    h->cap = h->cap ? 2 * h->cap : 16;
    h->p = (OPatch*)realloc(h->p, sizeof(OPatch) * h->cap);
  }
  OPatch* p = &h->p[h->np++];
  memset(p, 0, sizeof(*p));
  p->level = level;
  p->id = id;
  p->parent_id = parent_id;
  p->parent = -1;
  for (int d = 0; d < 3; d++) {
    p->mx[d] = d < h->ndims ? mx[d] : 1;
    p->mglobal[d][0] = d < h->ndims ? mglobal[2 * d] : 1;
    p->mglobal[d][1] = d < h->ndims ? mglobal[2 * d + 1] : 1;
    p->mbounds[d][0] = d < h->ndims ? mbounds[2 * d] : 1;
    p->mbounds[d][1] = d < h->ndims ? mbounds[2 * d + 1] : 1;
    p->dx[d] = d < h->ndims ? dx[d] : 0.0;
    p->xlower[d] = d < h->ndims ? xlower[d] : 0.0;
  }
  for (int f = 0; f < 6; f++) p->mthbc[f] = f < 2 * h->ndims ? mthbc[f] : 10;
  return 0;
}

/* RootInit (bsamroutines.f90:226-440) and InitSeed (:443-510).  Patch ids:
 * root = 0, level l < 0 has id = -l. */
int bsamo_build_uniform(bsamo_hier* h, const int mx[3], int minlevel,
                        const int mthbc[6], const double xlower[3],
                        const double xupper[3]) {
  if (!h || h->committed || h->np) return -1;
  int nd = h->ndims;
  int cmx[3] = {1, 1, 1}, mg[6] = {1, 1, 1, 1, 1, 1}, mb[6] = {1, 1, 1, 1, 1, 1};
  double dx[3] = {0, 0, 0}, xl[3] = {0, 0, 0};
  for (int d = 0; d < nd; d++) {
    if (mx[d] <= 0 || mx[d] % 2) return -2; /* :345-359 */
    cmx[d] = mx[d];
    mg[2 * d + 1] = mx[d];
    dx[d] = (xupper[d] - xlower[d]) / (double)mx[d]; /* :388 */
    xl[d] = xlower[d];
  }
  for (int d = 1; d < nd; d++)
    if (fabs(dx[0] - dx[d]) > 1.0e-10) return -2; /* :390-395 */
  /* root mbounds are set to (1, mx/2) by InitSeed of level -1 (:482) */
  for (int d = 0; d < nd; d++) {
    mb[2 * d] = 1;
    mb[2 * d + 1] = minlevel < 0 ? mx[d] / 2 : mx[d];
  }
  int rc = bsamo_patch_add(h, 0, 0, minlevel < 0 ? 1 : -1, cmx, mg, mb, mthbc,
                           dx, xl);
  if (rc) return rc;
  h->has_root_xupper = 1;
  for (int d = 0; d < 3; d++) h->root_xupper[d] = d < nd ? xupper[d] : 0.0;
  for (int l = -1; l >= minlevel; l--) {
    int nmx[3] = {1, 1, 1}, nmg[6] = {1, 1, 1, 1, 1, 1}, nmb[6] = {1, 1, 1, 1, 1, 1};
    double ndx[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) {
      if (cmx[d] % 2) return -3; /* :472-475 */
      nmx[d] = cmx[d] / 2;
      ndx[d] = dx[d] * 2.0; /* :478 */
      nmg[2 * d] = 1;
      nmg[2 * d + 1] = mg[2 * d + 1] / 2; /* :480 */
      nmb[2 * d] = 1;
      nmb[2 * d + 1] = l > minlevel ? nmx[d] / 2 : nmx[d];
      if (nmx[d] != nmg[2 * d + 1]) return -3; /* :486 */
    }
    rc = bsamo_patch_add(h, l, -l, l > minlevel ? -l + 1 : -1, nmx, nmg, nmb,
                         mthbc, ndx, xl);
    if (rc) return rc;
    memcpy(cmx, nmx, sizeof(cmx));
    memcpy(mg, nmg, sizeof(mg));
    memcpy(dx, ndx, sizeof(dx));
  }
  return 0;
}

/* PeriodicSetup, boundary.f90:805-872 */
static void periodic_setup(bsamo_hier* h, const int mthbc_in[6]) {
  int m[6];
  for (int f = 0; f < 6; f++) m[f] = 10;
  for (int f = 0; f < 2 * h->ndims; f++) m[f] = mthbc_in[f];
  static const int i13[13] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13};
  static const int i1245[4] = {1, 2, 4, 5};
  static const int i1389[4] = {1, 3, 8, 9};
  static const int i2367[4] = {2, 3, 6, 7};
  h->periodic = 1;
  const int* src = NULL;
  int n = 0;
  if (m[0] == 2) {
    if (m[2] == 2) {
      if (m[4] == 2) { src = i13; n = 13; } else { src = i1245; n = 4; }
    } else {
      if (m[4] == 2) { src = i1389; n = 4; } else { static const int a[1] = {1}; src = a; n = 1; }
    }
  } else {
    if (m[2] == 2) {
      if (m[4] == 2) { src = i2367; n = 4; } else { static const int a[1] = {2}; src = a; n = 1; }
    } else {
      if (m[4] == 2) { static const int a[1] = {3}; src = a; n = 1; } else { h->periodic = 0; }
    }
  }
  h->nperoff = n;
  for (int i = 0; i < n; i++) h->peroffidx[i] = src[i];
}

int bsamo_commit(bsamo_hier* h) {
  if (!h || h->committed) return -1;
  OPatch* root = NULL;
  for (int n = 0; n < h->np; n++)
    if (h->p[n].level == 0) { root = &h->p[n]; break; }
  if (!root) return -2;
  h->minlevel_present = 0;
  h->maxlevel_present = 0;
  for (int n = 0; n < h->np; n++) {
    OPatch* p = &h->p[n];
    if (p->level < h->minlevel_present) h->minlevel_present = p->level;
    if (p->level > h->maxlevel_present) h->maxlevel_present = p->level;
    if (p->parent_id >= 0) {
      OPatch* par = find_patch(h, p->parent_id);
      if (!par || par->level != p->level - 1) return -3;
      p->parent = (int)(par - h->p);
    }
    for (int f = 0; f < 2 * h->ndims; f++)
      if (p->mthbc[f] != 2 && p->mthbc[f] != 10 && p->mthbc[f] != INTERNALBC)
        return -4;
    for (int d = 0; d < 3; d++) {
      int used = d < h->ndims;
      p->cmx[d] = (used && p->mx[d] % 2 == 0) ? p->mx[d] / 2 : 1; /* bsamstorage.f90:67-73 */
      p->qlo[d] = used ? 1 - h->mbc : 1;
      p->qn[d] = used ? p->mx[d] + 2 * h->mbc : 1;
      p->clo[d] = used ? 1 - h->mbc : 1;
      p->cn[d] = used ? p->cmx[d] + 2 * h->mbc : 1;
      p->fn[d] = used ? p->mx[d] : 1;
    }
    size_t nq = (size_t)p->qn[0] * p->qn[1] * p->qn[2] * h->nrvars;
    size_t nc = (size_t)p->cn[0] * p->cn[1] * p->cn[2] * h->nrvars;
    size_t nf = (size_t)p->fn[0] * p->fn[1] * p->fn[2] * h->nrvars;
    p->q = (double*)calloc(nq, sizeof(double)); /* zero fill, bsamstorage.f90:136-140 */
    p->qold = (double*)calloc(nq, sizeof(double));
    p->qc = (double*)calloc(nc, sizeof(double));
    p->f = (double*)calloc(nf, sizeof(double));
    p->rf = (double*)calloc(nf, sizeof(double));
    p->ftmp = (double*)calloc(nf, sizeof(double));
  }
  for (int l = 0; l < NLEV; l++) {
    h->lev_n[l] = 0;
    free(h->lev_list[l]);
    h->lev_list[l] = (int*)malloc(sizeof(int) * (h->np + 1));
  }
  for (int n = 0; n < h->np; n++) {
    int l = h->p[n].level + MAXDEPTH;
    h->lev_list[l][h->lev_n[l]++] = n;
  }
  /* mxmax, bsamroutines.f90:397-401 */
  for (int l = 0; l <= MAXDEPTH; l++)
    for (int d = 0; d < 3; d++)
      h->mxmax[l][d] = d < h->ndims ? root->mx[d] << l : 1;
  periodic_setup(h, root->mthbc);
  h->committed = 1;
  return 0;
}

int bsamo_num_patches(const bsamo_hier* h) { return h ? h->np : -1; }

int bsamo_patch_info(const bsamo_hier* h, int index, int* out, double* dxl) {
  if (!h || index < 0 || index >= h->np) return -1;
  const OPatch* p = &h->p[index];
  out[0] = p->level; out[1] = p->id; out[2] = p->parent_id;
  for (int d = 0; d < 3; d++) {
    out[3 + d] = p->mx[d];
    out[6 + 2 * d] = p->mglobal[d][0];
    out[7 + 2 * d] = p->mglobal[d][1];
    out[12 + 2 * d] = p->mbounds[d][0];
    out[13 + 2 * d] = p->mbounds[d][1];
  }
  for (int f = 0; f < 6; f++) out[18 + f] = p->mthbc[f];
  if (dxl)
    for (int d = 0; d < 3; d++) { dxl[d] = p->dx[d]; dxl[3 + d] = p->xlower[d]; }
  return 0;
}

static double* field_ptr(const OPatch* p, int field, size_t* n, int nrvars) {
  size_t nq = (size_t)p->qn[0] * p->qn[1] * p->qn[2] * nrvars;
  size_t nc = (size_t)p->cn[0] * p->cn[1] * p->cn[2] * nrvars;
  size_t nf = (size_t)p->fn[0] * p->fn[1] * p->fn[2] * nrvars;
  switch (field) {
    case BSAMO_FIELD_Q: *n = nq; return p->q;
    case BSAMO_FIELD_QOLD: *n = nq; return p->qold;
    case BSAMO_FIELD_QC: *n = nc; return p->qc;
    case BSAMO_FIELD_F: *n = nf; return p->f;
    case BSAMO_FIELD_RF: *n = nf; return p->rf;
    case BSAMO_FIELD_FTMP: *n = nf; return p->ftmp;
  }
  *n = 0;
  return NULL;
}

size_t bsamo_field_size(const bsamo_hier* h, int id, int field) {
  if (!h || !h->committed) return 0;
  const OPatch* p = find_patch(h, id);
  if (!p) return 0;
  size_t n;
  field_ptr(p, field, &n, h->nrvars);
  return n;
}

int bsamo_put_field(bsamo_hier* h, int id, int field, const double* a, size_t n) {
  if (!h || !h->committed) return -1;
  OPatch* p = find_patch(h, id);
  if (!p) return -2;
  size_t nn;
  double* d = field_ptr(p, field, &nn, h->nrvars);
  if (!d || nn != n) return -3;
  memcpy(d, a, n * sizeof(double));
  return 0;
}

int bsamo_get_field(const bsamo_hier* h, int id, int field, double* a, size_t n) {
  if (!h || !h->committed) return -1;
  const OPatch* p = find_patch(h, id);
  if (!p) return -2;
  size_t nn;
  double* d = field_ptr(p, field, &nn, h->nrvars);
  if (!d || nn != n) return -3;
  memcpy(a, d, n * sizeof(double));
  return 0;
}

/* ------------------------------------------------------------------ */
/* grid utilities (LIBRARY/gridutilities.f90)                           */

static inline double cube(double c) { return c * c * c; } /* CH/problem.f90:918-928 */
static inline double sqr(double c) { return c * c; }      /* :931-941 */

/* ULap2D, gridutilities.f90:50-72, on plane v of a ghosted q-like array */
static inline double ulap2(const OPatch* p, const double* a, int i, int j, int v,
                           int coarse) {
  size_t (*ix)(const OPatch*, int, int, int, int) = coarse ? ic : iq;
  return a[ix(p, i + 1, j, 1, v)] + a[ix(p, i - 1, j, 1, v)] +
         a[ix(p, i, j + 1, 1, v)] + a[ix(p, i, j - 1, 1, v)] -
         4.0 * a[ix(p, i, j, 1, v)];
}
/* ULap3D, gridutilities.f90:372-399 */
static inline double ulap3(const OPatch* p, const double* a, int i, int j, int k,
                           int v, int coarse) {
  size_t (*ix)(const OPatch*, int, int, int, int) = coarse ? ic : iq;
  return a[ix(p, i + 1, j, k, v)] + a[ix(p, i - 1, j, k, v)] +
         a[ix(p, i, j + 1, k, v)] + a[ix(p, i, j - 1, k, v)] +
         a[ix(p, i, j, k + 1, v)] + a[ix(p, i, j, k - 1, v)] -
         6.0 * a[ix(p, i, j, k, v)];
}

/* ------------------------------------------------------------------ */
/* problem plugins                                                     */

/* Growth / Uptake, BioGrowth/problem.f90:743-766 */
static inline double growth(const bsamo_hier* h, double p) {
  return h->gamma * 0.5 * (p + 1.0);
}
static inline double uptake(const bsamo_hier* h, double p) {
  return h->lambda * 0.5 * (p + 1.0);
}

/* RelaxGrid2D, CH/problem.f90:318-369 */
static void relax_ch2d(const bsamo_hier* h, OPatch* p, int ipass) {
  double hh = p->dx[0];
  double h2 = hh * hh;
  double tmp1 = h->dt / h2, tmp2 = h->eps2 / h2, tmp3 = 4.0 * h->eps2 / h2;
  double a12 = 4.0 * tmp1;
  for (int j = 1; j <= p->mx[1]; j++)
    for (int i = 1 + imod(j + ipass, 2); i <= p->mx[0]; i += 2) {
      double a21 = -3.0 * sqr(Q(p, i, j, 1, 0)) - tmp3;
      double b1 = FF(p, i, j, 1, 0) +
                  tmp1 * (Q(p, i - 1, j, 1, 1) + Q(p, i + 1, j, 1, 1) +
                          Q(p, i, j - 1, 1, 1) + Q(p, i, j + 1, 1, 1));
      double b2 = FF(p, i, j, 1, 1) -
                  tmp2 * (Q(p, i + 1, j, 1, 0) + Q(p, i - 1, j, 1, 0) +
                          Q(p, i, j + 1, 1, 0) + Q(p, i, j - 1, 1, 0)) -
                  2.0 * cube(Q(p, i, j, 1, 0));
      double det = 1.0 - a12 * a21;
      Q(p, i, j, 1, 0) = (b1 - a12 * b2) / det;
      Q(p, i, j, 1, 1) = (b2 - a21 * b1) / det;
    }
}

/* RelaxGrid3D, CH/problem.f90:554-614 */
static void relax_ch3d(const bsamo_hier* h, OPatch* p, int ipass) {
  double hh = p->dx[0];
  double h2 = hh * hh;
  double tmp1 = h->dt / h2, tmp2 = h->eps2 / h2, tmp3 = 6.0 * h->eps2 / h2;
  double a12 = 6.0 * tmp1;
  for (int k = 1; k <= p->mx[2]; k++)
    for (int j = 1; j <= p->mx[1]; j++)
      for (int i = 1 + imod(k + j + ipass, 2); i <= p->mx[0]; i += 2) {
        double a21 = -3.0 * sqr(Q(p, i, j, k, 0)) - tmp3;
        double b1 = FF(p, i, j, k, 0) +
                    tmp1 * (Q(p, i - 1, j, k, 1) + Q(p, i + 1, j, k, 1) +
                            Q(p, i, j - 1, k, 1) + Q(p, i, j + 1, k, 1) +
                            Q(p, i, j, k - 1, 1) + Q(p, i, j, k + 1, 1));
        double b2 = FF(p, i, j, k, 1) -
                    tmp2 * (Q(p, i + 1, j, k, 0) + Q(p, i - 1, j, k, 0) +
                            Q(p, i, j + 1, k, 0) + Q(p, i, j - 1, k, 0) +
                            Q(p, i, j, k + 1, 0) + Q(p, i, j, k - 1, 0)) -
                    2.0 * cube(Q(p, i, j, k, 0));
        double det = 1.0 - a12 * a21;
        Q(p, i, j, k, 0) = (b1 - a12 * b2) / det;
        Q(p, i, j, k, 1) = (b2 - a21 * b1) / det;
      }
}

/* RelaxGrid2D, BioGrowth/problem.f90:255-296 */
static void relax_bio2d(const bsamo_hier* h, OPatch* p, int ipass) {
  double hh = p->dx[0];
  double h2 = hh * hh;
  double dt = h->dt;
  double tmp1 = dt * h->eps2 / h2, tmp3 = 1.0 / h2;
  for (int j = 1; j <= p->mx[1]; j++)
    for (int i = 1 + imod(j + ipass, 2); i <= p->mx[0]; i += 2) {
      double tmp2 = 4.0 * tmp1 + 1.0 + dt * sqr(Q(p, i, j, 1, 0));
      Q(p, i, j, 1, 0) =
          (FF(p, i, j, 1, 0) +
           dt * growth(h, QO(p, i, j, 1, 0)) * (Q(p, i, j, 1, 1) - h->czero) +
           tmp1 * (Q(p, i - 1, j, 1, 0) + Q(p, i + 1, j, 1, 0) +
                   Q(p, i, j - 1, 1, 0) + Q(p, i, j + 1, 1, 0))) / tmp2;
      double tmp4 = 4.0 * tmp3 + uptake(h, QO(p, i, j, 1, 0));
      Q(p, i, j, 1, 1) =
          (FF(p, i, j, 1, 1) +
           tmp3 * (Q(p, i + 1, j, 1, 1) + Q(p, i - 1, j, 1, 1) +
                   Q(p, i, j + 1, 1, 1) + Q(p, i, j - 1, 1, 1))) / tmp4;
    }
}

/* Growth plugin (no reference counterpart): phi and n as BioGrowth's
 * RelaxGrid2D with 2*ndims neighbours, then p = (f3 + Sum p_nb/h^2 +
 * cpress*phi*n) / (2*ndims/h^2) from the updated phi and n. */
static void relax_growth(const bsamo_hier* h, OPatch* p, int ipass) {
  double hh = p->dx[0];
  double h2 = hh * hh;
  double dt = h->dt;
  int nd = h->ndims;
  double kk = 2.0 * nd;
  double tmp1 = dt * h->eps2 / h2, tmp3 = 1.0 / h2;
  double c2 = kk * tmp1 + 1.0, c3 = kk * tmp3;
  int kmx = nd == 3 ? p->mx[2] : 1;
  for (int k = 1; k <= kmx; k++)
    for (int j = 1; j <= p->mx[1]; j++)
      for (int i = 1 + imod((nd == 3 ? k : 0) + j + ipass, 2); i <= p->mx[0]; i += 2) {
        double phi = Q(p, i, j, k, 0), ol = QO(p, i, j, k, 0);
        double tmp2 = c2 + dt * sqr(phi);
        double s0 = Q(p, i - 1, j, k, 0) + Q(p, i + 1, j, k, 0) + Q(p, i, j - 1, k, 0) + Q(p, i, j + 1, k, 0);
        double s1 = Q(p, i + 1, j, k, 1) + Q(p, i - 1, j, k, 1) + Q(p, i, j + 1, k, 1) + Q(p, i, j - 1, k, 1);
        double s2 = Q(p, i + 1, j, k, 2) + Q(p, i - 1, j, k, 2) + Q(p, i, j + 1, k, 2) + Q(p, i, j - 1, k, 2);
        if (nd == 3) {
          s0 = s0 + Q(p, i, j, k - 1, 0) + Q(p, i, j, k + 1, 0);
          s1 = s1 + Q(p, i, j, k + 1, 1) + Q(p, i, j, k - 1, 1);
          s2 = s2 + Q(p, i, j, k + 1, 2) + Q(p, i, j, k - 1, 2);
        }
        double np = (FF(p, i, j, k, 0) + dt * growth(h, ol) * (Q(p, i, j, k, 1) - h->czero) + tmp1 * s0) / tmp2;
        double tmp4 = c3 + uptake(h, ol);
        double nn = (FF(p, i, j, k, 1) + tmp3 * s1) / tmp4;
        Q(p, i, j, k, 0) = np;
        Q(p, i, j, k, 1) = nn;
        Q(p, i, j, k, 2) = (FF(p, i, j, k, 2) + tmp3 * s2 + h->cpress * np * nn) / c3;
      }
}

/* RelaxGrid3D, BioGrowth/problem.f90:445-478 (zero stub) */
static void relax_bio3d(const bsamo_hier* h, OPatch* p, int ipass) {
  (void)h;
  for (int k = 1; k <= p->mx[2]; k++)
    for (int j = 1; j <= p->mx[1]; j++)
      for (int i = 1 + imod(k + j + ipass, 2); i <= p->mx[0]; i += 2) {
        Q(p, i, j, k, 0) = 0.0;
        Q(p, i, j, k, 1) = 0.0;
      }
}

/* Operator2D/3D of the plugin evaluated on a ghosted array `a` described by
 * patch `p` (coarse=1 selects the qc extents), with qold `ao` (may equal
 * NULL when the plugin does not read qold at these cells), spacing hh; the
 * result for interior cell (i,j,k) of variable v. */
typedef struct {
  const OPatch* p;
  const double* a;
  int coarse;
  /* qold view: patch + offset mapping from (i,j,k) of `a` to qold indices */
  const OPatch* po;
  const double* ao;
  int ooff[3];
  double hh;
} OpView;

static inline double opA(const OpView* w, int i, int j, int k, int v) {
  return w->a[(w->coarse ? ic : iq)(w->p, i, j, k, v)];
}
static inline double opO(const OpView* w, int i, int j, int k, int v) {
  return w->ao[iq(w->po, i + w->ooff[0], j + w->ooff[1], k + w->ooff[2], v)];
}

/* Operator2D CH/problem.f90:393-422, Operator3D :638-669,
 * Operator2D BioGrowth/problem.f90:320-353, Operator3D :518-520 (zero) */
static void op_eval(const bsamo_hier* h, const OpView* w, int i, int j, int k,
                    double* out) {
  double h2 = w->hh * w->hh;
  if (h->problem == BSAMO_PROBLEM_CH) {
    double tmp1 = h->dt / h2, tmp2 = h->eps2 / h2;
    if (h->ndims == 2) {
      out[0] = opA(w, i, j, 1, 0) - tmp1 * ulap2(w->p, w->a, i, j, 1, w->coarse);
      out[1] = opA(w, i, j, 1, 1) - cube(opA(w, i, j, 1, 0)) +
               tmp2 * ulap2(w->p, w->a, i, j, 0, w->coarse);
    } else {
      out[0] = opA(w, i, j, k, 0) - tmp1 * ulap3(w->p, w->a, i, j, k, 1, w->coarse);
      out[1] = opA(w, i, j, k, 1) - cube(opA(w, i, j, k, 0)) +
               tmp2 * ulap3(w->p, w->a, i, j, k, 0, w->coarse);
    }
  } else if (h->problem == BSAMO_PROBLEM_GROWTH) {
    double dt = h->dt;
    double tmp1 = dt * h->eps2 / h2, tmp3 = 1.0 / h2;
    int kk = h->ndims == 3 ? k : 1;
    double l0, l1, l2;
    if (h->ndims == 2) {
      l0 = ulap2(w->p, w->a, i, j, 0, w->coarse);
      l1 = ulap2(w->p, w->a, i, j, 1, w->coarse);
      l2 = ulap2(w->p, w->a, i, j, 2, w->coarse);
    } else {
      l0 = ulap3(w->p, w->a, i, j, k, 0, w->coarse);
      l1 = ulap3(w->p, w->a, i, j, k, 1, w->coarse);
      l2 = ulap3(w->p, w->a, i, j, k, 2, w->coarse);
    }
    double a0 = opA(w, i, j, kk, 0), a1 = opA(w, i, j, kk, 1), o0 = opO(w, i, j, kk, 0);
    out[0] = a0 - tmp1 * l0 + dt * cube(a0) - dt * growth(h, o0) * (a1 - h->czero);
    out[1] = -tmp3 * l1 + uptake(h, o0) * a1;
    out[2] = -tmp3 * l2 - h->cpress * a0 * a1;
  } else {
    if (h->ndims == 2) {
      double dt = h->dt;
      double tmp1 = dt * h->eps2 / h2, tmp3 = 1.0 / h2;
      out[0] = opA(w, i, j, 1, 0) - tmp1 * ulap2(w->p, w->a, i, j, 0, w->coarse) +
               dt * cube(opA(w, i, j, 1, 0)) -
               dt * growth(h, opO(w, i, j, 1, 0)) * (opA(w, i, j, 1, 1) - h->czero);
      out[1] = -tmp3 * ulap2(w->p, w->a, i, j, 1, w->coarse) +
               uptake(h, opO(w, i, j, 1, 0)) * opA(w, i, j, 1, 1);
    } else {
      out[0] = 0.0;
      out[1] = 0.0;
    }
  }
}

/* Source2D/3D + SourceUpdate2D/3D (CH :425-476 / :672-721, BioGrowth
 * :356-405): value of the source at interior cell for variable v. */
static inline double source_val(const bsamo_hier* h, const OPatch* p, int i,
                                int j, int k, int v) {
  if (h->problem == BSAMO_PROBLEM_CH) {
    return v == 0 ? QO(p, i, j, k, 0) : -QO(p, i, j, k, 0);
  }
  if (h->problem == BSAMO_PROBLEM_GROWTH || h->ndims == 2)
    return v == 0 ? (1.0 + h->dt) * QO(p, i, j, k, 0) : 0.0;
  return 0.0;
}

/* UserBC2D/3D (CH :770-881, BioGrowth :623-736) on face `bc` (1..2*ndims) */
static void user_bc(const bsamo_hier* h, OPatch* p, int bc) {
  int nd = h->ndims, mbc = h->mbc, ll = 1 - mbc;
  int ul[3];
  for (int d = 0; d < 3; d++) ul[d] = p->mx[d] + mbc;
  int kl = nd == 3 ? ll : 1, ku = nd == 3 ? ul[2] : 1;
  for (int v = 0; v < h->nrvars; v++) {
    /* per variable: reflect (0), Dirichlet 2-q (1) or Dirichlet -q (2) */
    int dir;
    if (h->problem == BSAMO_PROBLEM_CH) dir = nd == 3 ? 1 : 0;
    else if (h->problem == BSAMO_PROBLEM_GROWTH) dir = v;
    else dir = nd == 3 ? 1 : (v == 1);
    for (int ibc = 1; ibc <= mbc; ibc++) {
      int d = (bc - 1) / 2, hi = (bc - 1) % 2;
      int gdst = hi ? p->mx[d] + ibc : 1 - ibc;
      int gsrc = hi ? p->mx[d] - ibc + 1 : ibc;
      if (d == 0) {
        for (int k = kl; k <= ku; k++)
          for (int j = ll; j <= ul[1]; j++) {
            double s = Q(p, gsrc, j, k, v);
            Q(p, gdst, j, k, v) = dir == 1 ? 2.0 - s : (dir == 2 ? -s : s);
          }
      } else if (d == 1) {
        for (int k = kl; k <= ku; k++)
          for (int i = ll; i <= ul[0]; i++) {
            double s = Q(p, i, gsrc, k, v);
            Q(p, i, gdst, k, v) = dir == 1 ? 2.0 - s : (dir == 2 ? -s : s);
          }
      } else {
        for (int j = ll; j <= ul[1]; j++)
          for (int i = ll; i <= ul[0]; i++) {
            double s = Q(p, i, j, gsrc, v);
            Q(p, i, j, gdst, v) = dir == 1 ? 2.0 - s : (dir == 2 ? -s : s);
          }
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* boundary.f90                                                        */

/* Interpolate2D, boundary.f90:143-333.  qf = child q, qc = parent q. */
static void interpolate2d(const bsamo_hier* h, OPatch* f, const OPatch* c,
                          int ipass) {
  int mx1 = f->mx[0], mx2 = f->mx[1];
  int mb11 = f->mbounds[0][0], mb12 = f->mbounds[0][1];
  int mb21 = f->mbounds[1][0], mb22 = f->mbounds[1][1];
  const int* m = f->mthbc;
#define QF(i, j) Q(f, i, j, 1, v)
#define QCC(i, j) Q(c, i, j, 1, v)
  for (int v = 0; v < h->nrvars; v++) {
    if (ipass == 1 || ipass == 0) { /* red corners :158-168 */
      QF(mx1 + 1, mx2 + 1) = A1 * QF(mx1 - 1, mx2 - 1) + A2 * QF(mx1, mx2) +
                             A3 * QCC(mb12 + 1, mb22 + 1);
      QF(0, 0) = A1 * QF(2, 2) + A2 * QF(1, 1) + A3 * QCC(mb11 - 1, mb21 - 1);
    }
    if (ipass == 2 || ipass == 0) { /* black corners :171-181 */
      QF(mx1 + 1, 0) = A1 * QF(mx1 - 1, 2) + A2 * QF(mx1, 1) +
                       A3 * QCC(mb12 + 1, mb21 - 1);
      QF(0, mx2 + 1) = A1 * QF(2, mx2 - 1) + A2 * QF(1, mx2) +
                       A3 * QCC(mb11 - 1, mb22 + 1);
    }
  }
  for (int v = 0; v < h->nrvars; v++) {
    if (m[0] == 2 || m[0] == INTERNALBC) { /* face 1 :185-216 */
      if (ipass == 1 || ipass == 0) {
        for (int j = 2, n = 0; j <= mx2 - 2; j += 2, n++)
          QF(0, j) = A1 * QF(2, j + 2) + A2 * QF(1, j + 1) + A3 * QCC(mb11 - 1, mb21 + n);
        QF(0, mx2) = A1 * QF(2, mx2) + A2 * QF(1, mx2) +
                     A3 * (B1 * QCC(mb11 - 1, mb22 + 1) + B2 * QCC(mb11 - 1, mb22) +
                           B3 * QCC(mb11 - 1, mb22 - 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int j = 3, n = 0; j <= mx2 - 1; j += 2, n++)
          QF(0, j) = A1 * QF(2, j - 2) + A2 * QF(1, j - 1) + A3 * QCC(mb11 - 1, mb21 + 1 + n);
        QF(0, 1) = A1 * QF(2, 1) + A2 * QF(1, 1) +
                   A3 * (B1 * QCC(mb11 - 1, mb21 - 1) + B2 * QCC(mb11 - 1, mb21) +
                         B3 * QCC(mb11 - 1, mb21 + 1));
      }
    }
    if (m[1] == 2 || m[1] == INTERNALBC) { /* face 2 :222-257 */
      if (ipass == 1 || ipass == 0) {
        for (int j = 3, n = 0; j <= mx2 - 1; j += 2, n++)
          QF(mx1 + 1, j) = A1 * QF(mx1 - 1, j - 2) + A2 * QF(mx1, j - 1) +
                           A3 * QCC(mb12 + 1, mb21 + 1 + n);
        QF(mx1 + 1, 1) = A1 * QF(mx1 - 1, 1) + A2 * QF(mx1, 1) +
                         A3 * (B1 * QCC(mb12 + 1, mb21 - 1) + B2 * QCC(mb12 + 1, mb21) +
                               B3 * QCC(mb12 + 1, mb21 + 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int j = 2, n = 0; j <= mx2 - 2; j += 2, n++)
          QF(mx1 + 1, j) = A1 * QF(mx1 - 1, j + 2) + A2 * QF(mx1, j + 1) +
                           A3 * QCC(mb12 + 1, mb21 + n);
        QF(mx1 + 1, mx2) = A1 * QF(mx1 - 1, mx2) + A2 * QF(mx1, mx2) +
                           A3 * (B1 * QCC(mb12 + 1, mb22 + 1) + B2 * QCC(mb12 + 1, mb22) +
                                 B3 * QCC(mb12 + 1, mb22 - 1));
      }
    }
    if (m[2] == 2 || m[2] == INTERNALBC) { /* face 3 :259-294 */
      if (ipass == 1 || ipass == 0) {
        for (int i = 2, n = 0; i <= mx1 - 2; i += 2, n++)
          QF(i, 0) = A1 * QF(i + 2, 2) + A2 * QF(i + 1, 1) + A3 * QCC(mb11 + n, mb21 - 1);
        QF(mx1, 0) = A1 * QF(mx1, 2) + A2 * QF(mx1, 1) +
                     A3 * (B1 * QCC(mb12 + 1, mb21 - 1) + B2 * QCC(mb12, mb21 - 1) +
                           B3 * QCC(mb12 - 1, mb21 - 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int i = 3, n = 0; i <= mx1 - 1; i += 2, n++)
          QF(i, 0) = A1 * QF(i - 2, 2) + A2 * QF(i - 1, 1) + A3 * QCC(mb11 + 1 + n, mb21 - 1);
        QF(1, 0) = A1 * QF(1, 2) + A2 * QF(1, 1) +
                   A3 * (B1 * QCC(mb11 - 1, mb21 - 1) + B2 * QCC(mb11, mb21 - 1) +
                         B3 * QCC(mb11 + 1, mb21 - 1));
      }
    }
    if (m[3] == 2 || m[3] == INTERNALBC) { /* face 4 :296-331 */
      if (ipass == 1 || ipass == 0) {
        for (int i = 3, n = 0; i <= mx1 - 1; i += 2, n++)
          QF(i, mx2 + 1) = A1 * QF(i - 2, mx2 - 1) + A2 * QF(i - 1, mx2) +
                           A3 * QCC(mb11 + 1 + n, mb22 + 1);
        QF(1, mx2 + 1) = A1 * QF(1, mx2 - 1) + A2 * QF(1, mx2) +
                         A3 * (B1 * QCC(mb11 - 1, mb22 + 1) + B2 * QCC(mb11, mb22 + 1) +
                               B3 * QCC(mb11 + 1, mb22 + 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int i = 2, n = 0; i <= mx1 - 2; i += 2, n++)
          QF(i, mx2 + 1) = A1 * QF(i + 2, mx2 - 1) + A2 * QF(i + 1, mx2) +
                           A3 * QCC(mb11 + n, mb22 + 1);
        QF(mx1, mx2 + 1) = A1 * QF(mx1, mx2 - 1) + A2 * QF(mx1, mx2) +
                           A3 * (B1 * QCC(mb12 + 1, mb22 + 1) + B2 * QCC(mb12, mb22 + 1) +
                                 B3 * QCC(mb12 - 1, mb22 + 1));
      }
    }
  }
#undef QF
#undef QCC
}

/* ---- Interpolate3D, boundary.f90:1048-1550 ---------------------------- */

/* GetFaceIndex, boundary.f90:1018-1045: for dimension d and parity 1 (low) or
 * 2 (high): [0] ghost index, [1] second fine cell, [2] first fine cell,
 * [3] coarse cell beyond the patch, [4] coarse cell at the patch edge. */
static void face_index(const OPatch* f, int d, int parity, int fi[5]) {
  if (parity == 1) {
    fi[0] = 0; fi[1] = 2; fi[2] = 1;
    fi[3] = f->mbounds[d][0] - 1; fi[4] = f->mbounds[d][0];
  } else {
    fi[0] = f->mx[d] + 1; fi[1] = f->mx[d] - 1; fi[2] = f->mx[d];
    fi[3] = f->mbounds[d][1] + 1; fi[4] = f->mbounds[d][1];
  }
}

/* one interpolated ghost value, all variables:
 * q(g) = a1*q(s1) + a2*q(s2) + a3*coarse, coarse one of
 *   kind 0: qc(c[0]);  kind 1: b1*qc(c[0]) + b2*qc(c[1]) + b3*qc(c[2]);
 *   kind 2: c1*qc(c[0]) + c2*qc(c[1]) + c3*qc(c[2]) + c4*qc(c[3]) */
static void cf3_put(const bsamo_hier* h, OPatch* f, const OPatch* pc, const int g[3], const int s1[3],
                    const int s2[3], int kind, int c[4][3]) {
  for (int v = 0; v < h->nrvars; v++) {
    double co;
    if (kind == 0) co = Q(pc, c[0][0], c[0][1], c[0][2], v);
    else if (kind == 1)
      co = B1 * Q(pc, c[0][0], c[0][1], c[0][2], v) + B2 * Q(pc, c[1][0], c[1][1], c[1][2], v) +
           B3 * Q(pc, c[2][0], c[2][1], c[2][2], v);
    else
      co = C1 * Q(pc, c[0][0], c[0][1], c[0][2], v) + C2 * Q(pc, c[1][0], c[1][1], c[1][2], v) +
           C3 * Q(pc, c[2][0], c[2][1], c[2][2], v) + C4 * Q(pc, c[3][0], c[3][1], c[3][2], v);
    Q(f, g[0], g[1], g[2], v) = A1 * Q(f, s1[0], s1[1], s1[2], v) + A2 * Q(f, s2[0], s2[1], s2[2], v) + A3 * co;
  }
}

static int cf_face(int m) { return m == 2 || m == INTERNALBC; }

/* An edge with dimensions d1, d2 fixed at the faces given by fa, fb (face
 * index arrays) and dimension t running; the four statements of each edge
 * block (boundary.f90:1096-1126 and the two groups after it). */
static void cf3_edge(const bsamo_hier* h, OPatch* f, const OPatch* pc, int d1, const int* fa, int d2,
                     const int* fb, int t) {
  int mx = f->mx[t], lo = f->mbounds[t][0], hi = f->mbounds[t][1];
  int g[3], s1[3], s2[3], c[4][3];
  g[d1] = fa[0]; s1[d1] = fa[1]; s2[d1] = fa[2];
  g[d2] = fb[0]; s1[d2] = fb[1]; s2[d2] = fb[2];
  for (int x = 0; x < 4; x++) { c[x][d1] = fa[3]; c[x][d2] = fb[3]; }
  for (int i = 3, n = 0; i <= mx - 1; i += 2, n++) { /* 3:mx-1:2 */
    g[t] = i; s1[t] = i - 2; s2[t] = i - 1; c[0][t] = lo + 1 + n;
    cf3_put(h, f, pc, g, s1, s2, 0, c);
  }
  g[t] = 1; s1[t] = 1; s2[t] = 1;
  c[0][t] = lo - 1; c[1][t] = lo; c[2][t] = lo + 1;
  cf3_put(h, f, pc, g, s1, s2, 1, c);
  for (int i = 2, n = 0; i <= mx - 2; i += 2, n++) { /* 2:mx-2:2 */
    g[t] = i; s1[t] = i + 2; s2[t] = i + 1; c[0][t] = lo + n;
    cf3_put(h, f, pc, g, s1, s2, 0, c);
  }
  g[t] = mx; s1[t] = mx; s2[t] = mx;
  c[0][t] = hi + 1; c[1][t] = hi; c[2][t] = hi - 1;
  cf3_put(h, f, pc, g, s1, s2, 1, c);
}

/* The tangential classes of one face (normal n fixed by fn, tangential
 * dimensions t1 < t2), boundary.f90:1209-1335 and its two analogues.
 * cls 0: yellow (t1, t2 even) with its edge rows; 1: blue (odd, odd);
 * 2: green (t1 odd, t2 even); 3: red (t1 even, t2 odd). */
static void cf3_face_class(const bsamo_hier* h, OPatch* f, const OPatch* pc, int n, const int* fn, int t1, int t2,
                           int cls) {
  int m1 = f->mx[t1], m2 = f->mx[t2];
  int l1 = f->mbounds[t1][0], h1 = f->mbounds[t1][1], l2 = f->mbounds[t2][0], h2 = f->mbounds[t2][1];
  int g[3], s1[3], s2[3], c[4][3];
  g[n] = fn[0]; s1[n] = fn[1]; s2[n] = fn[2];
  for (int x = 0; x < 4; x++) c[x][n] = fn[3];
  /* direction of the diagonal in t1 and t2: +1 for even classes, -1 for odd */
  int e1 = (cls == 0 || cls == 3), e2 = (cls == 0 || cls == 2);
  int a1lo = e1 ? 2 : 3, a1hi = e1 ? m1 - 2 : m1 - 1, a2lo = e2 ? 2 : 3, a2hi = e2 ? m2 - 2 : m2 - 1;
  int d1 = e1 ? 1 : -1, d2 = e2 ? 1 : -1;
  /* bulk: both coordinates in the strided ranges */
  for (int j = a2lo; j <= a2hi; j += 2)
    for (int i = a1lo; i <= a1hi; i += 2) {
      g[t1] = i; g[t2] = j;
      s1[t1] = i + 2 * d1; s1[t2] = j + 2 * d2;
      s2[t1] = i + d1; s2[t2] = j + d2;
      c[0][t1] = e1 ? l1 + i / 2 - 1 : l1 + (i - 1) / 2;
      c[0][t2] = e2 ? l2 + j / 2 - 1 : l2 + (j - 1) / 2;
      cf3_put(h, f, pc, g, s1, s2, 0, c);
    }
  /* edge row with t1 at its end (even class: t1 = m1, odd class: t1 = 1),
   * t2 in its strided range; coarse b-combination along t1 */
  for (int j = a2lo; j <= a2hi; j += 2) {
    int i = e1 ? m1 : 1;
    g[t1] = i; g[t2] = j;
    s1[t1] = i; s1[t2] = j + 2 * d2;
    s2[t1] = i; s2[t2] = j + d2;
    int ct2 = e2 ? l2 + j / 2 - 1 : l2 + (j - 1) / 2;
    for (int x = 0; x < 3; x++) c[x][t2] = ct2;
    if (e1) { c[0][t1] = h1 + 1; c[1][t1] = h1; c[2][t1] = h1 - 1; }
    else { c[0][t1] = l1 - 1; c[1][t1] = l1; c[2][t1] = l1 + 1; }
    cf3_put(h, f, pc, g, s1, s2, 1, c);
  }
  /* edge row with t2 at its end, t1 in its strided range; b along t2 */
  for (int i = a1lo; i <= a1hi; i += 2) {
    int j = e2 ? m2 : 1;
    g[t1] = i; g[t2] = j;
    s1[t1] = i + 2 * d1; s1[t2] = j;
    s2[t1] = i + d1; s2[t2] = j;
    int ct1 = e1 ? l1 + i / 2 - 1 : l1 + (i - 1) / 2;
    for (int x = 0; x < 3; x++) c[x][t1] = ct1;
    if (e2) { c[0][t2] = h2 + 1; c[1][t2] = h2; c[2][t2] = h2 - 1; }
    else { c[0][t2] = l2 - 1; c[1][t2] = l2; c[2][t2] = l2 + 1; }
    cf3_put(h, f, pc, g, s1, s2, 1, c);
  }
}

/* grey corner cells of a face, boundary.f90:1322-1333 and analogues */
static void cf3_face_grey(const bsamo_hier* h, OPatch* f, const OPatch* pc, int n, const int* fn, int t1, int t2) {
  for (int p1 = 1; p1 <= 2; p1++) {
    int fa[5];
    face_index(f, t1, p1, fa);
    for (int p2 = 1; p2 <= 2; p2++) {
      int fb[5];
      face_index(f, t2, p2, fb);
      int g[3], s1[3], s2[3], c[4][3];
      g[n] = fn[0]; s1[n] = fn[1]; s2[n] = fn[2];
      g[t1] = s1[t1] = s2[t1] = fa[2];
      g[t2] = s1[t2] = s2[t2] = fb[2];
      for (int x = 0; x < 4; x++) c[x][n] = fn[3];
      c[0][t1] = fa[4]; c[0][t2] = fb[4];
      c[1][t1] = fa[3]; c[1][t2] = fb[4];
      c[2][t1] = fa[4]; c[2][t2] = fb[3];
      c[3][t1] = fa[3]; c[3][t2] = fb[3];
      cf3_put(h, f, pc, g, s1, s2, 2, c);
    }
  }
}

static void interpolate3d(const bsamo_hier* h, OPatch* f, const OPatch* pc, int ipass) {
  const int* m = f->mthbc;
  int fa[5], fb[5], fcc[5];
  /* (1) corners */
  for (int p1 = 1; p1 <= 2; p1++) {
    if (!cf_face(m[p1 - 1]) && ipass == 1) continue;
    face_index(f, 0, p1, fa);
    for (int p2 = 1; p2 <= 2; p2++) {
      if (!cf_face(m[p2 + 1]) && ipass == 1) continue;
      face_index(f, 1, p2, fb);
      for (int p3 = 1; p3 <= 2; p3++) {
        if (!cf_face(m[p3 + 3]) && ipass == 1) continue;
        face_index(f, 2, p3, fcc);
        int g[3] = {fa[0], fb[0], fcc[0]}, s1[3] = {fa[1], fb[1], fcc[1]}, s2[3] = {fa[2], fb[2], fcc[2]};
        int c[4][3] = {{fa[3], fb[3], fcc[3]}};
        cf3_put(h, f, pc, g, s1, s2, 0, c);
      }
    }
  }
  /* (2) edges 1-4: dimensions 1 and 3 fixed; the face-5/6 test of the
   * reference compares with 99, not 999 (boundary.f90:1104) */
  for (int p1 = 1; p1 <= 2; p1++) {
    if (!cf_face(m[p1 - 1]) && ipass == 1) continue;
    face_index(f, 0, p1, fa);
    for (int p3 = 1; p3 <= 2; p3++) {
      if (m[p3 + 3] != 2 && m[p3 + 3] != 99 && ipass == 1) continue;
      face_index(f, 2, p3, fcc);
      cf3_edge(h, f, pc, 0, fa, 2, fcc, 1);
    }
  }
  /* edges 5-8: dimensions 1 and 2 fixed */
  for (int p1 = 1; p1 <= 2; p1++) {
    if (!cf_face(m[p1 - 1]) && ipass == 1) continue;
    face_index(f, 0, p1, fa);
    for (int p2 = 1; p2 <= 2; p2++) {
      if (!cf_face(m[p2 + 1]) && ipass == 1) continue;
      face_index(f, 1, p2, fb);
      cf3_edge(h, f, pc, 0, fa, 1, fb, 2);
    }
  }
  /* edges 9-12: dimensions 2 and 3 fixed */
  for (int p2 = 1; p2 <= 2; p2++) {
    if (!cf_face(m[p2 + 1]) && ipass == 1) continue;
    face_index(f, 1, p2, fb);
    for (int p3 = 1; p3 <= 2; p3++) {
      if (!cf_face(m[p3 + 3]) && ipass == 1) continue;
      face_index(f, 2, p3, fcc);
      cf3_edge(h, f, pc, 1, fb, 2, fcc, 0);
    }
  }
  /* (3) faces, normal dimension n with tangential dimensions (t1, t2) */
  static const int T[3][2] = {{1, 2}, {0, 2}, {0, 1}};
  for (int n = 0; n < 3; n++)
    for (int par = 1; par <= 2; par++) {
      if (!cf_face(m[2 * n + par - 1])) continue;
      int fn[5];
      face_index(f, n, par, fn);
      if (ipass == 0 || (par + ipass) % 2 == 0) {
        cf3_face_class(h, f, pc, n, fn, T[n][0], T[n][1], 0);
        cf3_face_class(h, f, pc, n, fn, T[n][0], T[n][1], 1);
      }
      if (ipass == 0 || (par + ipass) % 2 == 1) {
        cf3_face_class(h, f, pc, n, fn, T[n][0], T[n][1], 2);
        cf3_face_class(h, f, pc, n, fn, T[n][0], T[n][1], 3);
      }
      cf3_face_grey(h, f, pc, n, fn, T[n][0], T[n][1]);
    }
}

/* GhostOverlap, boundary.f90:359-431 (the level-landscape part, :434-475, is
 * only used while the mesh is being built and is not restated). */
static void ghost_overlap(const bsamo_hier* h, OPatch* g1, OPatch* g2,
                          const int* off) {
  int nd = h->ndims, mbc = h->mbc;
  int mg1[3][2], mg2[3][2], ovg[3][2], ovg1[3][2], ovg2[3][2];
  for (int n = 0; n < 3; n++) {
    mg1[n][0] = mg1[n][1] = mg2[n][0] = mg2[n][1] = 1;
    ovg[n][0] = ovg[n][1] = ovg1[n][0] = ovg1[n][1] = ovg2[n][0] = ovg2[n][1] = 1;
  }
  for (int n = 0; n < nd; n++) {
    mg1[n][0] = g1->mglobal[n][0];
    mg1[n][1] = g1->mglobal[n][1];
    mg2[n][0] = g2->mglobal[n][0] + (off ? off[n] : 0);
    mg2[n][1] = g2->mglobal[n][1] + (off ? off[n] : 0);
  }
  for (int n = 0; n < nd; n++) {
    ovg[n][0] = mg1[n][0] - mbc > mg2[n][0] - mbc ? mg1[n][0] - mbc : mg2[n][0] - mbc;
    ovg[n][1] = mg1[n][1] + mbc < mg2[n][1] + mbc ? mg1[n][1] + mbc : mg2[n][1] + mbc;
  }
  for (int n = 0; n < nd; n++)
    if (ovg[n][1] - ovg[n][0] < 0) return;
  for (int n = 0; n < nd; n++) {
    ovg1[n][0] = ovg[n][0] > mg2[n][0] ? ovg[n][0] : mg2[n][0];
    ovg1[n][1] = ovg[n][1] < mg2[n][1] ? ovg[n][1] : mg2[n][1];
    ovg2[n][0] = ovg[n][0] > mg1[n][0] ? ovg[n][0] : mg1[n][0];
    ovg2[n][1] = ovg[n][1] < mg1[n][1] ? ovg[n][1] : mg1[n][1];
  }
  /* grid2 interior -> grid1 (:412-420) */
  int ml1[3][2], ml2[3][2];
  for (int n = 0; n < 3; n++) ml1[n][0] = ml1[n][1] = ml2[n][0] = ml2[n][1] = 1;
  for (int n = 0; n < nd; n++) {
    ml1[n][0] = ovg1[n][0] - mg1[n][0] + 1;
    ml1[n][1] = ovg1[n][1] - mg1[n][0] + 1;
    ml2[n][0] = ovg1[n][0] - mg2[n][0] + 1;
    ml2[n][1] = ovg1[n][1] - mg2[n][0] + 1;
  }
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 0; k <= ml1[2][1] - ml1[2][0]; k++)
      for (int j = 0; j <= ml1[1][1] - ml1[1][0]; j++)
        for (int i = 0; i <= ml1[0][1] - ml1[0][0]; i++)
          Q(g1, ml1[0][0] + i, ml1[1][0] + j, ml1[2][0] + k, v) =
              Q(g2, ml2[0][0] + i, ml2[1][0] + j, ml2[2][0] + k, v);
  /* grid1 interior -> grid2 (:422-430) */
  for (int n = 0; n < nd; n++) {
    ml1[n][0] = ovg2[n][0] - mg1[n][0] + 1;
    ml1[n][1] = ovg2[n][1] - mg1[n][0] + 1;
    ml2[n][0] = ovg2[n][0] - mg2[n][0] + 1;
    ml2[n][1] = ovg2[n][1] - mg2[n][0] + 1;
  }
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 0; k <= ml2[2][1] - ml2[2][0]; k++)
      for (int j = 0; j <= ml2[1][1] - ml2[1][0]; j++)
        for (int i = 0; i <= ml2[0][1] - ml2[0][0]; i++)
          Q(g2, ml2[0][0] + i, ml2[1][0] + j, ml2[2][0] + k, v) =
              Q(g1, ml1[0][0] + i, ml1[1][0] + j, ml1[2][0] + k, v);
}

/* SelfPeriodicBC, boundary.f90:480-577 */
static void self_periodic(const bsamo_hier* h, OPatch* p) {
  int mbc = h->mbc, nd = h->ndims;
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = d < nd ? 1 - mbc : 1;
    hi[d] = d < nd ? p->mx[d] + mbc : 1;
  }
  if (p->mthbc[0] == 2 && p->mthbc[1] == 2) {
    for (int ibc = 1; ibc <= mbc; ibc++)
      for (int v = 0; v < h->nrvars; v++) {
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            Q(p, p->mx[0] + ibc, j, k, v) = Q(p, ibc, j, k, v) + h->qpo[v];
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            Q(p, 1 - ibc, j, k, v) = Q(p, p->mx[0] + 1 - ibc, j, k, v) - h->qpo[v];
      }
  }
  if (p->mthbc[2] == 2 && p->mthbc[3] == 2) {
    for (int ibc = 1; ibc <= mbc; ibc++)
      for (int v = 0; v < h->nrvars; v++) {
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int i = lo[0]; i <= hi[0]; i++)
            Q(p, i, p->mx[1] + ibc, k, v) = Q(p, i, ibc, k, v);
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int i = lo[0]; i <= hi[0]; i++)
            Q(p, i, 1 - ibc, k, v) = Q(p, i, p->mx[1] + 1 - ibc, k, v);
      }
  }
  if (nd == 3 && p->mthbc[4] == 2 && p->mthbc[5] == 2) {
    for (int ibc = 1; ibc <= mbc; ibc++)
      for (int v = 0; v < h->nrvars; v++) {
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++)
            Q(p, i, j, p->mx[2] + ibc, v) = Q(p, i, j, ibc, v);
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++)
            Q(p, i, j, 1 - ibc, v) = Q(p, i, j, p->mx[2] + 1 - ibc, v);
      }
  }
}

/* GetPeriodicOffsets, boundary.f90:875-954 */
static void periodic_offsets(const bsamo_hier* h, int level, int poff[13][3]) {
  const int* mm = h->mxmax[level];
  for (int o = 0; o < h->nperoff; o++) {
    int a = 0, b = 0, c = 0;
    switch (h->peroffidx[o]) {
      case 1: a = mm[0]; break;
      case 2: b = mm[1]; break;
      case 3: c = mm[2]; break;
      case 4: a = mm[0]; b = mm[1]; break;
      case 5: a = -mm[0]; b = mm[1]; break;
      case 6: b = mm[1]; c = mm[2]; break;
      case 7: b = mm[1]; c = -mm[2]; break;
      case 8: a = mm[0]; c = mm[2]; break;
      case 9: a = -mm[0]; c = mm[2]; break;
      case 10: a = mm[0]; b = mm[1]; c = mm[2]; break;
      case 11: a = mm[0]; b = mm[1]; c = -mm[2]; break;
      case 12: a = -mm[0]; b = mm[1]; c = mm[2]; break;
      case 13: a = mm[0]; b = -mm[1]; c = mm[2]; break;
    }
    poff[o][0] = a; poff[o][1] = b; poff[o][2] = c;
  }
}

/* SetPhysicalBC2D/3D, boundary.f90:614-802 */
static void set_physical_bc(const bsamo_hier* h, OPatch* p) {
  for (int face = 1; face <= 2 * h->ndims; face++)
    if (p->mthbc[face - 1] == 10) user_bc(h, p, face);
}

/* SetGhost, boundary.f90:67-97 */
static void set_ghost(bsamo_hier* h, int level, int ipass) {
  int n = nlev(h, level);
  if (level > 0) {
    for (int a = 0; a < n; a++) { /* InterpolateCoarseFine :100-140 */
      OPatch* p = lev_patch(h, level, a);
      OPatch* c = parent_of(h, p);
      if (h->ndims == 2) interpolate2d(h, p, c, ipass);
      else interpolate3d(h, p, c, ipass);
    }
    for (int a = 0; a < n; a++) /* ApplyOnLevelPairs(TransferBC) */
      for (int b = a + 1; b < n; b++)
        ghost_overlap(h, lev_patch(h, level, a), lev_patch(h, level, b), NULL);
  }
  if (h->periodic) {
    for (int a = 0; a < n; a++) self_periodic(h, lev_patch(h, level, a));
    if (level > 0) { /* TransferPeriodicBC :580-611 */
      int poff[13][3];
      periodic_offsets(h, level, poff);
      for (int a = 0; a < n; a++)
        for (int b = a + 1; b < n; b++)
          for (int pol = -1; pol <= 1; pol += 2)
            for (int o = 0; o < h->nperoff; o++) {
              int off[3] = {pol * poff[o][0], pol * poff[o][1], pol * poff[o][2]};
              ghost_overlap(h, lev_patch(h, level, a), lev_patch(h, level, b), off);
            }
    }
  }
  for (int a = 0; a < n; a++) set_physical_bc(h, lev_patch(h, level, a));
}

/* GetCoarseGhostPoints, boundary.f90:957-1015 */
static void get_coarse_ghost_points(const bsamo_hier* h, OPatch* p) {
  OPatch* par = &((bsamo_hier*)h)->p[p->parent];
  int nd = h->ndims;
  int il[3] = {1, 1, 1}, ih[3] = {1, 1, 1}, jl[3] = {1, 1, 1}, jh[3] = {1, 1, 1};
  int mb[3][2];
  for (int d = 0; d < 3; d++) { mb[d][0] = mb[d][1] = 1; }
  for (int d = 0; d < nd; d++) {
    il[d] = 0; ih[d] = p->cmx[d] + 1;
    mb[d][0] = p->mbounds[d][0]; mb[d][1] = p->mbounds[d][1];
    jl[d] = mb[d][0] - 1; jh[d] = mb[d][1] + 1;
  }
  for (int v = 0; v < h->nrvars; v++) {
    /* face 1 and 2 */
    for (int k = il[2]; k <= ih[2]; k++)
      for (int j = il[1]; j <= ih[1]; j++) {
        QC(p, il[0], j, k, v) = Q(par, jl[0], jl[1] + (j - il[1]), jl[2] + (k - il[2]), v);
      }
    for (int k = il[2]; k <= ih[2]; k++)
      for (int j = il[1]; j <= ih[1]; j++) {
        QC(p, ih[0], j, k, v) = Q(par, jh[0], jl[1] + (j - il[1]), jl[2] + (k - il[2]), v);
      }
    /* face 3 and 4 */
    for (int k = il[2]; k <= ih[2]; k++)
      for (int i = 1; i <= p->cmx[0]; i++)
        QC(p, i, il[1], k, v) = Q(par, mb[0][0] + i - 1, jl[1], jl[2] + (k - il[2]), v);
    for (int k = il[2]; k <= ih[2]; k++)
      for (int i = 1; i <= p->cmx[0]; i++)
        QC(p, i, ih[1], k, v) = Q(par, mb[0][0] + i - 1, jh[1], jl[2] + (k - il[2]), v);
    if (nd >= 3) { /* face 5 and 6 */
      for (int j = 1; j <= p->cmx[1]; j++)
        for (int i = 1; i <= p->cmx[0]; i++)
          QC(p, i, j, il[2], v) = Q(par, mb[0][0] + i - 1, mb[1][0] + j - 1, jl[2], v);
      for (int j = 1; j <= p->cmx[1]; j++)
        for (int i = 1; i <= p->cmx[0]; i++)
          QC(p, i, j, ih[2], v) = Q(par, mb[0][0] + i - 1, mb[1][0] + j - 1, jh[2], v);
    }
  }
}

/* ------------------------------------------------------------------ */
/* afasroutines.f90                                                     */

static void relax_patch(const bsamo_hier* h, OPatch* p, int ipass) {
  /* RelaxPatch, afasroutines.f90:560-607 */
  if (h->problem == BSAMO_PROBLEM_CH) {
    if (h->ndims == 2) relax_ch2d(h, p, ipass); else relax_ch3d(h, p, ipass);
  } else if (h->problem == BSAMO_PROBLEM_BIOGROWTH) {
    if (h->ndims == 2) relax_bio2d(h, p, ipass); else relax_bio3d(h, p, ipass);
  } else {
    relax_growth(h, p, ipass);
  }
}

int bsamo_relax_level_color(bsamo_hier* h, int level, int ipass) {
  if (!h || !h->committed) return -1;
  for (int a = 0; a < nlev(h, level); a++) relax_patch(h, lev_patch(h, level, a), ipass);
  return 0;
}

int bsamo_set_ghost(bsamo_hier* h, int level, int ipass) {
  if (!h || !h->committed) return -1;
  set_ghost(h, level, ipass);
  return 0;
}

/* LevelRelax, afasroutines.f90:532-557 */
static void level_relax(bsamo_hier* h, int level, int nsmooth) {
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int rb = 1; rb <= 2; rb++) {
      for (int a = 0; a < nlev(h, level); a++) relax_patch(h, lev_patch(h, level, a), rb);
      set_ghost(h, level, rb);
    }
}

int bsamo_level_relax(bsamo_hier* h, int level, int nsmooth) {
  if (!h || !h->committed) return -1;
  level_relax(h, level, nsmooth);
  return 0;
}

/* Residual, afasroutines.f90:817-857: rf = f - Operator(q) */
static void residual(const bsamo_hier* h, OPatch* p) {
  OpView w = {p, p->q, 0, p, p->qold, {0, 0, 0}, p->dx[0]};
  double out[3];
  int kmx = h->ndims == 3 ? p->mx[2] : 1;
  for (int k = 1; k <= kmx; k++)
    for (int j = 1; j <= p->mx[1]; j++)
      for (int i = 1; i <= p->mx[0]; i++) {
        op_eval(h, &w, i, j, k, out);
        for (int v = 0; v < h->nrvars; v++) RF(p, i, j, k, v) = FF(p, i, j, k, v) - out[v];
      }
}

/* Restriction2D/3D, gridutilities.f90:103-126, :437-466, of an interior
 * array accessor. */
typedef double (*Getter)(const OPatch*, int, int, int, int);
static double get_q(const OPatch* p, int i, int j, int k, int v) { return Q(p, i, j, k, v); }
static double get_f(const OPatch* p, int i, int j, int k, int v) { return FF(p, i, j, k, v); }
static double get_rf(const OPatch* p, int i, int j, int k, int v) { return RF(p, i, j, k, v); }

static inline double restrict_at(const bsamo_hier* h, const OPatch* p, Getter g,
                                 int ci, int cj, int ck, int v) {
  int i = 2 * ci, j = 2 * cj;
  if (h->ndims == 2)
    return 0.25 * (g(p, i, j, 1, v) + g(p, i - 1, j, 1, v) + g(p, i, j - 1, 1, v) +
                   g(p, i - 1, j - 1, 1, v));
  int k = 2 * ck;
  return 0.125 * (g(p, i, j, k, v) + g(p, i - 1, j, k, v) + g(p, i, j - 1, k, v) +
                  g(p, i - 1, j - 1, k, v) + g(p, i, j, k - 1, v) +
                  g(p, i - 1, j, k - 1, v) + g(p, i, j - 1, k - 1, v) +
                  g(p, i - 1, j - 1, k - 1, v));
}

/* RestrictSolution, afasroutines.f90:610-652 */
static void restrict_solution(bsamo_hier* h, OPatch* p) {
  OPatch* par = parent_of(h, p);
  int kc = h->ndims == 3 ? p->cmx[2] : 1;
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 1; k <= kc; k++)
      for (int j = 1; j <= p->cmx[1]; j++)
        for (int i = 1; i <= p->cmx[0]; i++)
          QC(p, i, j, k, v) = restrict_at(h, p, get_q, i, j, k, v);
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 1; k <= kc; k++)
      for (int j = 1; j <= p->cmx[1]; j++)
        for (int i = 1; i <= p->cmx[0]; i++)
          Q(par, p->mbounds[0][0] + i - 1, p->mbounds[1][0] + j - 1,
            h->ndims == 3 ? p->mbounds[2][0] + k - 1 : 1, v) = QC(p, i, j, k, v);
}

/* CoarseLoadingFunction, afasroutines.f90:673-736 */
static void coarse_loading(bsamo_hier* h, OPatch* p) {
  OPatch* par = parent_of(h, p);
  double ch = par->dx[0];
  residual(h, p);
  /* qold of the parent offset so that qc index (i,j,k) maps to parent
   * index mb-1+i (the section parent%qold(mb-1:mb+1)) */
  OpView w = {p, p->qc, 1, par, par->qold,
              {p->mbounds[0][0] - 1, p->mbounds[1][0] - 1,
               h->ndims == 3 ? p->mbounds[2][0] - 1 : 0}, ch};
  double out[3];
  int kc = h->ndims == 3 ? p->cmx[2] : 1;
  for (int k = 1; k <= kc; k++)
    for (int j = 1; j <= p->cmx[1]; j++)
      for (int i = 1; i <= p->cmx[0]; i++) {
        op_eval(h, &w, i, j, k, out);
        for (int v = 0; v < h->nrvars; v++)
          FF(par, p->mbounds[0][0] + i - 1, p->mbounds[1][0] + j - 1,
             h->ndims == 3 ? p->mbounds[2][0] + k - 1 : 1, v) =
              restrict_at(h, p, get_rf, i, j, k, v) + out[v];
      }
}

/* CorrectFine, afasroutines.f90:860-980: qc(1-mbc:cmx+mbc) = parent%q -
 * qc, then q(1-mbc:mx+mbc) += P(qc) with BiLinProlongationP1/P2
 * (gridutilities.f90:156-239) or TriLinProlongationP1/P2 (:510-625).  P2 is
 * P1's stencil over one more layer: fine cell 2c takes 3 a(c) + a(c+1) and
 * fine cell 2c+1 takes a(c) + 3 a(c+1) in each direction, x first, then y
 * (and z), dividing by 16 (64) in the last direction.  P2 writes the odd
 * cells' sum as 3 a(c+1) + a(c), the same IEEE sum.  The second ring of qc
 * is written only here and by InitFields, so it carries the previous
 * correction into the next (as the reference's does). */
static void correct_fine(bsamo_hier* h, OPatch* p) {
  OPatch* par = parent_of(h, p);
  int nd = h->ndims, mbc = h->mbc, L = 1 - mbc;
  int c0 = p->cmx[0], c1 = p->cmx[1], c2 = nd == 3 ? p->cmx[2] : 1;
  int mb0 = p->mbounds[0][0], mb1 = p->mbounds[1][0], mb2 = nd == 3 ? p->mbounds[2][0] : 1;
  int klo = nd == 3 ? L : 1, khi = nd == 3 ? c2 + mbc : 1;
  for (int v = 0; v < h->nrvars; v++)
    for (int k = klo; k <= khi; k++)
      for (int j = L; j <= c1 + mbc; j++)
        for (int i = L; i <= c0 + mbc; i++)
          QC(p, i, j, k, v) =
              Q(par, mb0 - 1 + i, mb1 - 1 + j, nd == 3 ? mb2 - 1 + k : 1, v) - QC(p, i, j, k, v);
  int m0 = p->mx[0], m1 = p->mx[1];
  /* fine and coarse extents of the prolongation's arrays, index L first */
  int fn0 = m0 + 2 * mbc, fn1 = m1 + 2 * mbc, cn1 = c1 + 2 * mbc, cn2 = nd == 3 ? c2 + 2 * mbc : 1;
  /* fine index f -> its lower coarse index c (f = 2c or 2c+1) */
#define CLO(f) (((f) - ((f) & 1)) / 2)
  if (nd == 2) {
    double* b = (double*)malloc(sizeof(double) * (size_t)fn0 * cn1);
#define B(i, j) b[(size_t)((j) - L) * fn0 + ((i) - L)]
    for (int v = 0; v < h->nrvars; v++) {
      for (int cj = L; cj <= c1 + mbc; cj++)
        for (int i = L; i <= m0 + mbc; i++) {
          int c = CLO(i);
          B(i, cj) = (i & 1) ? QC(p, c, cj, 1, v) + 3.0 * QC(p, c + 1, cj, 1, v)
                             : 3.0 * QC(p, c, cj, 1, v) + QC(p, c + 1, cj, 1, v);
        }
      for (int j = L; j <= m1 + mbc; j++)
        for (int i = L; i <= m0 + mbc; i++) {
          int c = CLO(j);
          double pv = (j & 1) ? (B(i, c) + 3.0 * B(i, c + 1)) / 16.0 : (3.0 * B(i, c) + B(i, c + 1)) / 16.0;
          Q(p, i, j, 1, v) = Q(p, i, j, 1, v) + pv;
        }
    }
#undef B
    free(b);
  } else {
    int m2 = p->mx[2];
    double* b = (double*)malloc(sizeof(double) * (size_t)fn0 * cn1 * cn2);
    double* cc = (double*)malloc(sizeof(double) * (size_t)fn0 * fn1 * cn2);
#define B(i, j, k) b[((size_t)((k) - L) * cn1 + ((j) - L)) * fn0 + ((i) - L)]
#define CC(i, j, k) cc[((size_t)((k) - L) * fn1 + ((j) - L)) * fn0 + ((i) - L)]
    for (int v = 0; v < h->nrvars; v++) {
      for (int ck = L; ck <= c2 + mbc; ck++)
        for (int cj = L; cj <= c1 + mbc; cj++)
          for (int i = L; i <= m0 + mbc; i++) {
            int c = CLO(i);
            B(i, cj, ck) = (i & 1) ? QC(p, c, cj, ck, v) + 3.0 * QC(p, c + 1, cj, ck, v)
                                   : 3.0 * QC(p, c, cj, ck, v) + QC(p, c + 1, cj, ck, v);
          }
      for (int ck = L; ck <= c2 + mbc; ck++)
        for (int j = L; j <= m1 + mbc; j++)
          for (int i = L; i <= m0 + mbc; i++) {
            int c = CLO(j);
            CC(i, j, ck) = (j & 1) ? B(i, c, ck) + 3.0 * B(i, c + 1, ck) : 3.0 * B(i, c, ck) + B(i, c + 1, ck);
          }
      for (int k = L; k <= m2 + mbc; k++)
        for (int j = L; j <= m1 + mbc; j++)
          for (int i = L; i <= m0 + mbc; i++) {
            int c = CLO(k);
            double pv = (k & 1) ? (CC(i, j, c) + 3.0 * CC(i, j, c + 1)) / 64.0
                                : (3.0 * CC(i, j, c) + CC(i, j, c + 1)) / 64.0;
            Q(p, i, j, k, v) = Q(p, i, j, k, v) + pv;
          }
    }
#undef B
#undef CC
    free(b);
    free(cc);
  }
#undef CLO
}

/* AFASVcycle, afasroutines.f90:495-529 */
static void afas_vcycle(bsamo_hier* h, int level, int minlevel, int nsmooth) {
  level_relax(h, level, nsmooth);
  if (level > minlevel) {
    int n = nlev(h, level);
    for (int a = 0; a < n; a++) restrict_solution(h, lev_patch(h, level, a));
    set_ghost(h, level - 1, 0);
    for (int a = 0; a < n; a++) get_coarse_ghost_points(h, lev_patch(h, level, a));
    for (int a = 0; a < n; a++) coarse_loading(h, lev_patch(h, level, a));
    afas_vcycle(h, level - 1, minlevel, nsmooth);
    for (int a = 0; a < n; a++) correct_fine(h, lev_patch(h, level, a));
    set_ghost(h, level, 0);
    level_relax(h, level, nsmooth);
  }
}

int bsamo_vcycle(bsamo_hier* h, int level, int minlevel, int nsmooth) {
  if (!h || !h->committed) return -1;
  afas_vcycle(h, level, minlevel, nsmooth);
  return 0;
}

/* ApplyOnLevel(level, CorrectFine) alone (afasroutines.f90:518) */
int bsamo_correct_fine(bsamo_hier* h, int level) {
  if (!h || !h->committed || level < -MAXDEPTH || level > MAXDEPTH) return -1;
  for (int n = 0; n < nlev(h, level); n++)
    if (lev_patch(h, level, n)->parent < 0) return -1;
  for (int n = 0; n < nlev(h, level); n++) correct_fine(h, lev_patch(h, level, n));
  return 0;
}

static void get_source(bsamo_hier* h, OPatch* p);
static void update_source(bsamo_hier* h, OPatch* p);
static void fill_down_level(bsamo_hier* h, OPatch* p, int field);
/* one per-patch operation on every patch of a level (ApplyOnLevel,
 * treeops.f90:515-552): 1 RestrictSolution, 2 GetCoarseGhostPoints,
 * 3 CoarseLoadingFunction, 4 GetSourceFunction, 5 UpdateSourceFunction,
 * 6 FillDownLevel(source), 7 FillDownLevel(solution) */
int bsamo_level_op(bsamo_hier* h, int level, int which) {
  if (!h || !h->committed || level < -MAXDEPTH || level > MAXDEPTH || which < 1 || which > 7) return -1;
  if (which != 4 && which != 5)
    for (int n = 0; n < nlev(h, level); n++)
      if (lev_patch(h, level, n)->parent < 0) return -1;
  for (int n = 0; n < nlev(h, level); n++) {
    OPatch* p = lev_patch(h, level, n);
    switch (which) {
      case 1: restrict_solution(h, p); break;
      case 2: get_coarse_ghost_points(h, p); break;
      case 3: coarse_loading(h, p); break;
      case 4: get_source(h, p); break;
      case 5: update_source(h, p); break;
      default: fill_down_level(h, p, which == 6 ? 1 : 2); break;
    }
  }
  return 0;
}

static void prolong_mc(int nd, int mbc, const double* a, const int cmx[3], double* out);
/* one variable of P1MC / P2MC (InitFields' prolongation) alone */
int bsamo_prolong_mc(int nd, int mbc, const double* a, const int cmx[3], double* out) {
  if ((nd != 2 && nd != 3) || mbc < 1 || mbc > 2 || !a || !cmx || !out) return -1;
  prolong_mc(nd, mbc, a, cmx, out);
  return 0;
}

/* FillDown / FillDownLevel, afasroutines.f90:236-327 (1 = source, 2 = q) */
/* FillDownLevel, afasroutines.f90:262-327: parent f (field 1) or q (2)
 * under the patch = Restriction of the patch's */
static void fill_down_level(bsamo_hier* h, OPatch* p, int field) {
  OPatch* par = parent_of(h, p);
  int kc = h->ndims == 3 ? p->cmx[2] : 1;
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 1; k <= kc; k++)
      for (int j = 1; j <= p->cmx[1]; j++)
        for (int i = 1; i <= p->cmx[0]; i++) {
          int pi = p->mbounds[0][0] + i - 1, pj = p->mbounds[1][0] + j - 1;
          int pk = h->ndims == 3 ? p->mbounds[2][0] + k - 1 : 1;
          if (field == 1) FF(par, pi, pj, pk, v) = restrict_at(h, p, get_f, i, j, k, v);
          else Q(par, pi, pj, pk, v) = restrict_at(h, p, get_q, i, j, k, v);
        }
}

static void fill_down(bsamo_hier* h, int field, int finest, int minlevel) {
  for (int level = finest; level >= minlevel + 1; level--) {
    for (int a = 0; a < nlev(h, level); a++) fill_down_level(h, lev_patch(h, level, a), field);
    if (field == 2) set_ghost(h, level - 1, 0);
  }
}

int bsamo_fill_down(bsamo_hier* h, int field, int finestlevel, int minlevel) {
  if (!h || !h->committed || (field != 1 && field != 2)) return -1;
  fill_down(h, field, finestlevel, minlevel);
  return 0;
}

/* CopyQToQold, bsamroutines.f90:592-605 */
int bsamo_copy_q_to_qold(bsamo_hier* h, int minlevel, int finestlevel) {
  if (!h || !h->committed) return -1;
  for (int level = minlevel; level <= finestlevel; level++)
    for (int a = 0; a < nlev(h, level); a++) {
      OPatch* p = lev_patch(h, level, a);
      size_t nq = (size_t)p->qn[0] * p->qn[1] * p->qn[2] * h->nrvars;
      memcpy(p->qold, p->q, nq * sizeof(double));
    }
  return 0;
}

/* GetSourceFunction (:330-381) then UpdateSourceFunction (:438-492) */
static void get_source(bsamo_hier* h, OPatch* p) {
  int kmx = h->ndims == 3 ? p->mx[2] : 1;
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 1; k <= kmx; k++)
      for (int j = 1; j <= p->mx[1]; j++)
        for (int i = 1; i <= p->mx[0]; i++) FT(p, i, j, k, v) = source_val(h, p, i, j, k, v);
}
static void update_source(bsamo_hier* h, OPatch* p) {
  int kmx = h->ndims == 3 ? p->mx[2] : 1;
  for (int v = 0; v < h->nrvars; v++)
    for (int k = 1; k <= kmx; k++)
      for (int j = 1; j <= p->mx[1]; j++)
        for (int i = 1; i <= p->mx[0]; i++) FF(p, i, j, k, v) = FT(p, i, j, k, v) + 0.0;
}

/* ErrorAFAS, afasroutines.f90:113-160, with L2Error (:163-189) and
 * L2ComponentErrors (:192-219) */
static double error_afas(bsamo_hier* h, int level, int errortype) {
  if (errortype == 1) {
    h->integral[0] = 0.0;
    h->integral[1] = 0.0;
    for (int a = 0; a < nlev(h, level); a++) {
      OPatch* p = lev_patch(h, level, a);
      residual(h, p);
      double s = 0.0; /* SquareSum in array-element order */
      size_t nf = (size_t)p->fn[0] * p->fn[1] * p->fn[2] * h->nrvars;
      for (size_t n = 0; n < nf; n++) s = s + p->rf[n] * p->rf[n];
      h->integral[0] = s + h->integral[0];
      h->integral[1] = (double)(h->nrvars * p->mx[0] * p->mx[1] * p->mx[2]) + h->integral[1];
    }
    return sqrt(h->integral[0] / h->integral[1]);
  }
  double comp[10] = {0};
  h->integral[1] = 0.0;
  for (int a = 0; a < nlev(h, level); a++) {
    OPatch* p = lev_patch(h, level, a);
    residual(h, p);
    size_t nc = (size_t)p->fn[0] * p->fn[1] * p->fn[2];
    for (int v = 0; v < h->nrvars; v++) {
      double s = 0.0;
      for (size_t n = 0; n < nc; n++) s = s + p->rf[v * nc + n] * p->rf[v * nc + n];
      comp[v] = s + comp[v];
    }
    h->integral[1] = (double)(p->mx[0] * p->mx[1] * p->mx[2]) + h->integral[1];
  }
  double mx = 0.0;
  for (int v = 0; v < h->nrvars; v++) {
    double e = sqrt(comp[v] / h->integral[1]);
    if (v == 0 || e > mx) mx = e;
  }
  return mx;
}

int bsamo_residual_norm(bsamo_hier* h, int level, int errortype, double* out) {
  if (!h || !h->committed || !out) return -1;
  *out = error_afas(h, level, errortype);
  return 0;
}

/* MultigridIterations, afasroutines.f90:48-110 (the plugins' aux updates
 * are empty for maux = 0 and are skipped) */
int bsamo_multigrid_iterations(bsamo_hier* h, int finest, int minlevel,
                               int nsmooth, int maxvcycles, double qerrortol,
                               int updateauxfreq, int errortype,
                               int* ncycles, double* residuals) {
  if (!h || !h->committed) return -1;
  (void)updateauxfreq;
  fill_down(h, 2, finest, minlevel);
  for (int level = finest; level >= 0; level--)
    for (int a = 0; a < nlev(h, level); a++) get_source(h, lev_patch(h, level, a));
  for (int level = finest; level >= 0; level--)
    for (int a = 0; a < nlev(h, level); a++) update_source(h, lev_patch(h, level, a));
  fill_down(h, 1, finest, minlevel);
  int it;
  for (it = 1; it <= maxvcycles; it++) {
    afas_vcycle(h, finest, minlevel, nsmooth);
    fill_down(h, 2, finest, minlevel);
    for (int level = finest; level >= 0; level--)
      for (int a = 0; a < nlev(h, level); a++) update_source(h, lev_patch(h, level, a));
    fill_down(h, 1, finest, minlevel);
    double r = error_afas(h, finest, errortype);
    if (residuals) residuals[it - 1] = r;
    if (r < qerrortol) break;
  }
  if (ncycles) *ncycles = it > maxvcycles ? maxvcycles : it;
  return 0;
}

int bsamo_time_step(bsamo_hier* h, int first, int finest, int minlevel,
                    int nsmooth, int maxvcycles, double qerrortol,
                    int updateauxfreq, int errortype, int* ncycles,
                    double* residuals) {
  if (!h || !h->committed) return -1;
  for (int level = 0; level <= finest; level++) set_ghost(h, level, 0);
  if (first) fill_down(h, 2, finest, minlevel);
  bsamo_copy_q_to_qold(h, minlevel, finest);
  return bsamo_multigrid_iterations(h, finest, minlevel, nsmooth, maxvcycles,
                                    qerrortol, updateauxfreq, errortype,
                                    ncycles, residuals);
}

/* splitmix64 (Steele, Lea, Flood 2014) on seed ^ (gidx * golden gamma) */
double bsamo_uniform_pm1(unsigned long long seed, unsigned long long gidx) {
  uint64_t z = (uint64_t)seed ^ ((uint64_t)gidx * 0x9E3779B97F4A7C15ULL);
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

/* ------------------------------------------------------------------ */
/* AMR regrid (bsamroutines.f90:657-689, :966-1951)                    */

/* a patch added to a committed hierarchy, fields allocated (zero) */
static int add_live_patch(bsamo_hier* h, int level, int id, int parent, const int mx[3], const int mg[3][2],
                          const int mb[3][2], const int thbc[6], const double dx[3], const double xl[3]) {
  if (h->np == h->cap) {
    h->cap = h->cap ? 2 * h->cap : 16;
    h->p = (OPatch*)realloc(h->p, sizeof(OPatch) * h->cap);
  }
  int n = h->np++;
  OPatch* p = &h->p[n];
  memset(p, 0, sizeof(*p));
  p->level = level;
  p->id = id;
  p->parent = parent;
  p->parent_id = parent >= 0 ? h->p[parent].id : -1;
  for (int d = 0; d < 3; d++) {
    int used = d < h->ndims;
    p->mx[d] = mx[d];
    p->mglobal[d][0] = mg[d][0];
    p->mglobal[d][1] = mg[d][1];
    p->mbounds[d][0] = mb[d][0];
    p->mbounds[d][1] = mb[d][1];
    p->dx[d] = dx[d];
    p->xlower[d] = xl[d];
    p->cmx[d] = (used && p->mx[d] % 2 == 0) ? p->mx[d] / 2 : 1;
    p->qlo[d] = used ? 1 - h->mbc : 1;
    p->qn[d] = used ? p->mx[d] + 2 * h->mbc : 1;
    p->clo[d] = used ? 1 - h->mbc : 1;
    p->cn[d] = used ? p->cmx[d] + 2 * h->mbc : 1;
    p->fn[d] = used ? p->mx[d] : 1;
  }
  for (int f = 0; f < 6; f++) p->mthbc[f] = thbc[f];
  size_t nq = (size_t)p->qn[0] * p->qn[1] * p->qn[2] * h->nrvars;
  size_t nc = (size_t)p->cn[0] * p->cn[1] * p->cn[2] * h->nrvars;
  size_t nf = (size_t)p->fn[0] * p->fn[1] * p->fn[2] * h->nrvars;
  p->q = (double*)calloc(nq, sizeof(double));
  p->qold = (double*)calloc(nq, sizeof(double));
  p->qc = (double*)calloc(nc, sizeof(double));
  p->f = (double*)calloc(nf, sizeof(double));
  p->rf = (double*)calloc(nf, sizeof(double));
  p->ftmp = (double*)calloc(nf, sizeof(double));
  int l = level + MAXDEPTH;
  h->lev_list[l] = (int*)realloc(h->lev_list[l], sizeof(int) * (h->lev_n[l] + 1));
  h->lev_list[l][h->lev_n[l]++] = n;
  if (level > h->maxlevel_present) h->maxlevel_present = level;
  return n;
}

static inline size_t fidx(const OPatch* p, int i, int j, int k) {
  return ((size_t)(k - 1) * p->mx[1] + (size_t)(j - 1)) * p->mx[0] + (size_t)(i - 1);
}

/* SetErrFlagsUser2D/3D (CH/problem.f90:248-308) or the gradient rule */
static void tag_patch(const bsamo_hier* h, const OPatch* p, const bsamo_regrid_params* prm, int* fl) {
  double tol = prm->qtolerance[p->level];
  int nd = h->ndims;
  for (int k = 1; k <= p->mx[2]; k++)
    for (int j = 1; j <= p->mx[1]; j++)
      for (int i = 1; i <= p->mx[0]; i++) {
        int t;
        if (prm->tagging == BSAMO_TAG_CH) {
          double s = fabs(Q(p, i + 1, j, k, 0) - 2.0 * Q(p, i, j, k, 0) + Q(p, i - 1, j, k, 0)) +
                     fabs(Q(p, i, j + 1, k, 0) - 2.0 * Q(p, i, j, k, 0) + Q(p, i, j - 1, k, 0));
          if (nd == 3) s = s + fabs(Q(p, i, j, k + 1, 0) - 2.0 * Q(p, i, j, k, 0) + Q(p, i, j, k - 1, 0));
          t = s > (nd == 3 ? 3.0 : 2.0) * tol;
        } else {
          double gx = (Q(p, i + 1, j, k, 0) - Q(p, i - 1, j, k, 0)) * 0.5;
          double gy = (Q(p, i, j + 1, k, 0) - Q(p, i, j - 1, k, 0)) * 0.5;
          double g = gx * gx + gy * gy;
          if (nd == 3) {
            double gz = (Q(p, i, j, k + 1, 0) - Q(p, i, j, k - 1, 0)) * 0.5;
            g = g + gz * gz;
          }
          t = g > tol * tol;
        }
        fl[fidx(p, i, j, k)] = t;
      }
}

typedef struct {
  int n, cap;
  int (*c)[3];
} TagList;

/* BufferAndList, bsamroutines.f90:1206-1247 */
static void buffer_and_list(const bsamo_hier* h, const OPatch* p, int ib, int* fl, TagList* tl) {
  size_t n = (size_t)p->mx[0] * p->mx[1] * p->mx[2];
  int* tmp = (int*)malloc(sizeof(int) * n);
  memcpy(tmp, fl, sizeof(int) * n);
  for (int k = 1; k <= p->mx[2]; k++)
    for (int j = 1; j <= p->mx[1]; j++)
      for (int i = 1; i <= p->mx[0]; i++) {
        if (tmp[fidx(p, i, j, k)] != 1) continue;
        int idx[3] = {i, j, k}, lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1}, out = 0;
        for (int d = 0; d < h->ndims; d++) {
          lo[d] = idx[d] - ib;
          hi[d] = idx[d] + ib;
        }
        for (int d = 0; d < 3; d++)
          if (lo[d] < 1 || hi[d] > p->mx[d]) out = 1;
        if (out) { /* AddTaggedCellToList, :1250-1264 */
          if (tl->n == tl->cap) {
            tl->cap = tl->cap ? 2 * tl->cap : 64;
            tl->c = realloc(tl->c, sizeof(*tl->c) * tl->cap);
          }
          for (int d = 0; d < 3; d++) tl->c[tl->n][d] = d < h->ndims ? idx[d] + p->mglobal[d][0] - 1 : 1;
          tl->n++;
        } else {
          for (int c = lo[2]; c <= hi[2]; c++)
            for (int b = lo[1]; b <= hi[1]; b++)
              for (int a = lo[0]; a <= hi[0]; a++) fl[fidx(p, a, b, c)] = 1;
        }
      }
  free(tmp);
}

/* BufferTaggedCells, bsamroutines.f90:1311-1349 */
static void buffer_tagged(const bsamo_hier* h, const OPatch* p, const int tag[3], int ib, int* fl) {
  int lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1};
  for (int d = 0; d < h->ndims; d++) {
    lo[d] = tag[d] - ib > p->mglobal[d][0] ? tag[d] - ib : p->mglobal[d][0];
    hi[d] = tag[d] + ib < p->mglobal[d][1] ? tag[d] + ib : p->mglobal[d][1];
    if (hi[d] < lo[d]) return;
    lo[d] = lo[d] - p->mglobal[d][0] + 1;
    hi[d] = hi[d] - p->mglobal[d][0] + 1;
  }
  for (int c = lo[2]; c <= hi[2]; c++)
    for (int b = lo[1]; b <= hi[1]; b++)
      for (int a = lo[0]; a <= hi[0]; a++) fl[fidx(p, a, b, c)] = 1;
}

/* GetSignatures, :1608-1632; signature of dimension n over box mb */
static void signatures(const OPatch* p, const int* fl, int mb[3][2], int nd, int* sig /* [3][maxm+1] */, int maxm) {
  for (int n = 0; n < nd; n++)
    for (int i = mb[n][0]; i <= mb[n][1]; i++) {
      int lo[3], hi[3], s = 0;
      for (int d = 0; d < 3; d++) { lo[d] = mb[d][0]; hi[d] = mb[d][1]; }
      lo[n] = hi[n] = i;
      for (int c = lo[2]; c <= hi[2]; c++)
        for (int b = lo[1]; b <= hi[1]; b++)
          for (int a = lo[0]; a <= hi[0]; a++) s += fl[fidx(p, a, b, c)];
      sig[n * (maxm + 2) + i] = s;
    }
}

/* GridFlagRatio, :1635-1660 */
static double flag_ratio(const OPatch* p, const int* fl, int mb[3][2], int nd) {
  double total = 1.0;
  for (int d = 0; d < nd; d++) total = total * (double)(mb[d][1] - mb[d][0] + 1);
  for (int d = nd; d < 3; d++) mb[d][0] = mb[d][1] = 1;
  double flagged = 0.0;
  long long s = 0;
  for (int c = mb[2][0]; c <= mb[2][1]; c++)
    for (int b = mb[1][0]; b <= mb[1][1]; b++)
      for (int a = mb[0][0]; a <= mb[0][1]; a++) s += fl[fidx(p, a, b, c)];
  flagged = (double)s;
  return flagged / total;
}

#define MAXSUBGRIDS 1024 /* nodeinfodef.f90:62 */

/* NewSubGrids, :1408-1605 (modified Berger-Rigoutsos).  Returns the number
 * of subgrids written to sub[][3][2] (parent index space), or -1 on the
 * reference's error stops. */
static int new_sub_grids(const bsamo_hier* h, const OPatch* p, const int* fl, const bsamo_regrid_params* prm,
                         int (*sub)[3][2]) {
  int nd = h->ndims, level = p->level;
  double desfill = prm->desiredfillratio[level];
  int mgp = prm->minimumgridpoints[level];
  if (mgp < 4 || mgp % 2) return -1;
  int mb[3][2];
  for (int d = 0; d < 3; d++) { mb[d][0] = 1; mb[d][1] = d < nd ? p->mx[d] : 1; }
  if (flag_ratio(p, fl, mb, nd) < 1.0e-10) return 0;
  int maxm = 0;
  for (int d = 0; d < nd; d++) if (p->mx[d] > maxm) maxm = p->mx[d];
  int* sig = (int*)calloc((size_t)3 * (maxm + 2), sizeof(int));
  int* dds = (int*)calloc((size_t)3 * (maxm + 2), sizeof(int));
  static char cansplit[MAXSUBGRIDS + 1];
  int ngrid = 1;
  for (int g = 0; g <= MAXSUBGRIDS; g++) cansplit[g] = 1;
  memcpy(sub[0], mb, sizeof(mb));
  int igrid = 1;
  while (ngrid < MAXSUBGRIDS && igrid <= ngrid) {
    int (*b)[2] = sub[igrid - 1];
    int npass = 0;
    while (cansplit[igrid] && npass < 15) {
      npass++;
      signatures(p, fl, b, nd, sig, maxm);
      for (int n = 0; n < nd; n++) { /* trim unflagged edges */
        int* sg = sig + n * (maxm + 2);
        int i1 = b[n][0], i2 = b[n][1];
        while (sg[i1] == 0 && i1 < b[n][1] && i2 - i1 + 1 > mgp) i1++;
        while (sg[i2] == 0 && i2 > b[n][0] && i2 - i1 + 1 > mgp) i2--;
        b[n][0] = i1 - imod(i1 + 1, 2);
        b[n][1] = i2 + imod(i2, 2);
      }
      double fill = flag_ratio(p, fl, b, nd);
      if (fill < desfill) {
        signatures(p, fl, b, nd, sig, maxm);
        int isplit[3] = {0, 0, 0}, have = 0;
        for (int n = 0; n < nd && !have; n++) { /* holes */
          int* sg = sig + n * (maxm + 2);
          int i1 = b[n][0], i2 = b[n][1];
          for (int i = i1 + mgp - 1; i <= i2 - mgp; i += 2) {
            int m = i - i1 + 1 < i2 - i ? i - i1 + 1 : i2 - i;
            if (sg[i] == 0 && m >= mgp) {
              isplit[n] = i;
              have = 1;
              break;
            }
          }
        }
        if (!have) { /* inflection points */
          for (int n = 0; n < nd; n++) {
            int *sg = sig + n * (maxm + 2), *dd = dds + n * (maxm + 2);
            for (int i = b[n][0] + 1; i <= b[n][1] - 1; i++) dd[i] = sg[i - 1] - 2 * sg[i] + sg[i + 1];
          }
          int inflect = 0, dist0 = 0;
          for (int n = 0; n < nd; n++) {
            int* dd = dds + n * (maxm + 2);
            int i1 = b[n][0], i2 = b[n][1];
            for (int i = i1 + mgp; i <= i2 - mgp + 1; i += 2) {
              int del = abs(dd[i] - dd[i - 1]);
              if (del > inflect) {
                inflect = del;
                isplit[0] = isplit[1] = isplit[2] = 0;
                isplit[n] = i - 1;
                have = 1;
                dist0 = i - i1 < i2 - i + 1 ? i - i1 : i2 - i + 1;
              } else if (del == inflect && inflect > 0) {
                int dist1 = i - i1 < i2 - i + 1 ? i - i1 : i2 - i + 1;
                if (dist1 > dist0) {
                  isplit[0] = isplit[1] = isplit[2] = 0;
                  isplit[n] = i - 1;
                  have = 1;
                  dist0 = dist1;
                }
              }
            }
          }
        }
        if (have) {
          for (int n = 0; n < nd; n++) {
            int m = b[n][1] - isplit[n] < isplit[n] - b[n][0] + 1 ? b[n][1] - isplit[n] : isplit[n] - b[n][0] + 1;
            if (isplit[n] > 0 && m >= mgp) {
              ngrid++;
              cansplit[ngrid] = 1;
              memcpy(sub[ngrid - 1], b, sizeof(int) * 6);
              sub[ngrid - 1][n][0] = isplit[n] + 1;
              b[n][1] = isplit[n];
              break;
            }
          }
        } else {
          cansplit[igrid] = 0;
        }
      } else {
        cansplit[igrid] = 0;
      }
    }
    igrid++;
  }
  free(sig);
  free(dds);
  for (int g = 0; g < ngrid; g++)
    for (int n = 0; n < nd; n++) { /* the reference's checks, :1565-1595 */
      int len = sub[g][n][1] - sub[g][n][0] + 1;
      if (len < mgp || len % 2 || sub[g][n][0] % 2 == 0 || sub[g][n][1] % 2 == 1) return -1;
    }
  return ngrid;
}

/* Patches longer than maxside child cells (maxside/2 parent cells) are cut
 * into nearly equal even pieces along that dimension (not a reference
 * feature: it bounds the patch size for the batched kernels). */
/* NewSubGrids alone on a flag field of one patch (level 0, mbounds the
 * whole patch): the boxes (lo, hi per dimension) in the order it makes
 * them, at most cap; returns their number or a negative status */
int bsamo_new_sub_grids(int nd, const int mx[3], const int* flags, double desfill, int mgp, int* out, int cap) {
  if ((nd != 2 && nd != 3) || !mx || !flags || !out || cap < 0) return -1;
  bsamo_hier hh;
  memset(&hh, 0, sizeof(hh));
  hh.ndims = nd;
  OPatch p;
  memset(&p, 0, sizeof(p));
  for (int d = 0; d < 3; d++) {
    p.mx[d] = d < nd ? mx[d] : 1;
    p.mglobal[d][0] = 1;
    p.mglobal[d][1] = p.mx[d];
  }
  bsamo_regrid_params prm;
  memset(&prm, 0, sizeof(prm));
  prm.desiredfillratio[0] = desfill;
  prm.minimumgridpoints[0] = mgp;
  int (*sub)[3][2] = malloc(sizeof(*sub) * MAXSUBGRIDS);
  int ng = new_sub_grids(&hh, &p, flags, &prm, sub);
  for (int g = 0; g < ng && g < cap; g++)
    for (int d = 0; d < 3; d++) {
      out[6 * g + 2 * d] = sub[g][d][0];
      out[6 * g + 2 * d + 1] = sub[g][d][1];
    }
  free(sub);
  return ng;
}

static int split_long(int nd, int maxside, int (*sub)[3][2], int ng, int cap) {
  if (maxside <= 0) return ng;
  int P = maxside / 2;
  for (int g = 0; g < ng; g++)
    for (int n = 0; n < nd; n++) {
      int len = sub[g][n][1] - sub[g][n][0] + 1;
      if (len <= P) continue;
      int pieces = (len + P - 1) / P;
      int lo = sub[g][n][0];
      for (int k = 0; k < pieces; k++) {
        /* even lengths, the remainder spread from the first piece on */
        int half = len / 2, base = half / pieces, extra = half % pieces;
        int plen = 2 * (base + (k < extra ? 1 : 0));
        int (*t)[2];
        if (k == 0) t = sub[g];
        else {
          if (ng == cap) return -1;
          memcpy(sub[ng], sub[g], sizeof(int) * 6);
          t = sub[ng++];
        }
        t[n][0] = lo;
        t[n][1] = lo + plen - 1;
        lo += plen;
      }
    }
  return ng;
}

/* BiLin/TriLinProlongationP1MC and P2MC (gridutilities.f90:242-369,
 * :628-829): a is the coarse block with mbc ghost layers (cmx+2 mbc per
 * dimension, index 1-mbc first), out the fine block with mbc ghost layers.
 * The prolongation is CorrectFine's (P2: one more layer); the mass
 * correction of each coarse interior cell goes to its 2^d fine cells. */
static void prolong_mc(int nd, int mbc, const double* a, const int cmx[3], double* out) {
  int L = 1 - mbc;
  int cn0 = cmx[0] + 2 * mbc, cn1 = cmx[1] + 2 * mbc, cn2 = nd == 3 ? cmx[2] + 2 * mbc : 1;
  int fn0 = 2 * cmx[0] + 2 * mbc, fn1 = 2 * cmx[1] + 2 * mbc, fn2 = nd == 3 ? 2 * cmx[2] + 2 * mbc : 1;
  int kL = nd == 3 ? L : 0;
#define A(i, j, k) a[((size_t)((k) - kL) * cn1 + ((j) - L)) * cn0 + ((i) - L)]
#define O(i, j, k) out[((size_t)((k) - kL) * fn1 + ((j) - L)) * fn0 + ((i) - L)]
#define CLO(f) (((f) - ((f) & 1)) / 2)
  double* b = (double*)malloc(sizeof(double) * fn0 * cn1 * cn2);
#define Bx(i, j, k) b[((size_t)((k) - kL) * cn1 + ((j) - L)) * fn0 + ((i) - L)]
  for (int k = kL; k < kL + cn2; k++)
    for (int j = L; j < L + cn1; j++)
      for (int i = L; i < L + fn0; i++) {
        int c = CLO(i);
        Bx(i, j, k) = (i & 1) ? A(c, j, k) + 3.0 * A(c + 1, j, k) : 3.0 * A(c, j, k) + A(c + 1, j, k);
      }
  if (nd == 2) {
    for (int j = L; j < L + fn1; j++)
      for (int i = L; i < L + fn0; i++) {
        int c = CLO(j);
        O(i, j, 0) = (j & 1) ? (Bx(i, c, 0) + 3.0 * Bx(i, c + 1, 0)) / 16.0 : (3.0 * Bx(i, c, 0) + Bx(i, c + 1, 0)) / 16.0;
      }
    for (int J = 1; J <= cmx[1]; J++)
      for (int I = 1; I <= cmx[0]; I++) {
        double cor = A(I, J, 0) - 0.25 * (O(2 * I, 2 * J, 0) + O(2 * I - 1, 2 * J, 0) + O(2 * I, 2 * J - 1, 0) +
                                          O(2 * I - 1, 2 * J - 1, 0));
        O(2 * I, 2 * J, 0) = O(2 * I, 2 * J, 0) + cor;
        O(2 * I - 1, 2 * J, 0) = O(2 * I - 1, 2 * J, 0) + cor;
        O(2 * I, 2 * J - 1, 0) = O(2 * I, 2 * J - 1, 0) + cor;
        O(2 * I - 1, 2 * J - 1, 0) = O(2 * I - 1, 2 * J - 1, 0) + cor;
      }
  } else {
    double* c = (double*)malloc(sizeof(double) * fn0 * fn1 * cn2);
#define Cy(i, j, k) c[((size_t)((k) - kL) * fn1 + ((j) - L)) * fn0 + ((i) - L)]
    for (int k = kL; k < kL + cn2; k++)
      for (int j = L; j < L + fn1; j++)
        for (int i = L; i < L + fn0; i++) {
          int cj = CLO(j);
          Cy(i, j, k) = (j & 1) ? Bx(i, cj, k) + 3.0 * Bx(i, cj + 1, k) : 3.0 * Bx(i, cj, k) + Bx(i, cj + 1, k);
        }
    for (int k = L; k < L + fn2; k++)
      for (int j = L; j < L + fn1; j++)
        for (int i = L; i < L + fn0; i++) {
          int ck = CLO(k);
          O(i, j, k) = (k & 1) ? (Cy(i, j, ck) + 3.0 * Cy(i, j, ck + 1)) / 64.0
                               : (3.0 * Cy(i, j, ck) + Cy(i, j, ck + 1)) / 64.0;
        }
    for (int K = 1; K <= cmx[2]; K++)
      for (int J = 1; J <= cmx[1]; J++)
        for (int I = 1; I <= cmx[0]; I++) {
          double cor = A(I, J, K) -
                       0.125 * (O(2 * I, 2 * J, 2 * K) + O(2 * I - 1, 2 * J, 2 * K) + O(2 * I, 2 * J - 1, 2 * K) +
                                O(2 * I - 1, 2 * J - 1, 2 * K) + O(2 * I, 2 * J, 2 * K - 1) +
                                O(2 * I - 1, 2 * J, 2 * K - 1) + O(2 * I, 2 * J - 1, 2 * K - 1) +
                                O(2 * I - 1, 2 * J - 1, 2 * K - 1));
          for (int dk = 0; dk < 2; dk++)
            for (int dj = 0; dj < 2; dj++)
              for (int di = 0; di < 2; di++)
                O(2 * I - di, 2 * J - dj, 2 * K - dk) = O(2 * I - di, 2 * J - dj, 2 * K - dk) + cor;
        }
    free(c);
#undef Cy
  }
  free(b);
#undef A
#undef O
#undef Bx
#undef CLO
}

/* MakeNewGrid (:1663-1784) + InitFields (:1787-1856); returns the index */
static int make_new_grid(bsamo_hier* h, int pidx, int mbp[3][2], int id, const bsamo_regrid_params* prm,
                         bsamo_qinit_fn qinit, void* user) {
  int nd = h->ndims;
  int mx[3] = {1, 1, 1}, mg[3][2], mb[3][2], thbc[6];
  double dx[3] = {0, 0, 0}, xl[3] = {0, 0, 0};
  const OPatch* par = &h->p[pidx];
  for (int d = 0; d < 3; d++) {
    mg[d][0] = mg[d][1] = mb[d][0] = mb[d][1] = 1;
    if (d >= nd) continue;
    mx[d] = (mbp[d][1] - mbp[d][0] + 1) * 2;
    mb[d][0] = mbp[d][0];
    mb[d][1] = mbp[d][1];
    int g0 = par->mglobal[d][0] + mbp[d][0] - 1;
    int g1 = g0 + mbp[d][1] - mbp[d][0];
    mg[d][0] = (g0 - 1) * 2 + 1;
    mg[d][1] = g1 * 2;
    xl[d] = (double)(mbp[d][0] - 1) * par->dx[d] + par->xlower[d];
    dx[d] = par->dx[d] / 2.0;
  }
  for (int f = 0; f < 6; f++) thbc[f] = f < 2 * nd ? INTERNALBC : 10;
  for (int n = 0; n < nd; n++) {
    if (par->mthbc[2 * n] < INTERNALBC && mb[n][0] == 1) thbc[2 * n] = par->mthbc[2 * n];
    if (par->mthbc[2 * n + 1] < INTERNALBC && mb[n][1] == par->mx[n]) thbc[2 * n + 1] = par->mthbc[2 * n + 1];
  }
  int c = add_live_patch(h, par->level + 1, id, pidx, mx, mg, mb, thbc, dx, xl);
  OPatch* ch = &h->p[c];
  par = &h->p[pidx];
  if (prm->initial) {
    qinit(user, ch->level, ch->mx, ch->dx, ch->xlower, ch->q);
  } else {
    /* child%qc(1-mbc:cmx+mbc) = parent%q(mb-mbc:mb+mbc), then
     * child%q(1-mbc:mx+mbc) = P1MC / P2MC(child%qc) (:1815-1850) */
    int mbc = h->mbc;
    int cmx[3] = {ch->cmx[0], ch->cmx[1], nd == 3 ? ch->cmx[2] : 0};
    size_t nc = (size_t)ch->cn[0] * ch->cn[1] * ch->cn[2];
    size_t nfine = (size_t)ch->qn[0] * ch->qn[1] * ch->qn[2];
    for (int v = 0; v < h->nrvars; v++) {
      int k0 = nd == 3 ? 1 - mbc : 1, k1 = nd == 3 ? cmx[2] + mbc : 1;
      for (int k = k0; k <= k1; k++)
        for (int j = 1 - mbc; j <= cmx[1] + mbc; j++)
          for (int i = 1 - mbc; i <= cmx[0] + mbc; i++)
            QC(ch, i, j, k, v) = Q(par, mb[0][0] - 1 + i, mb[1][0] - 1 + j, nd == 3 ? mb[2][0] - 1 + k : 1, v);
      prolong_mc(nd, mbc, ch->qc + v * nc, cmx, ch->q + v * nfine);
    }
  }
  /* child%rf = parent%rf = child%f = parent%f = 0 (:1773-1776); SetSrc is
   * empty for CH; child%qold = child%q (:1782) */
  size_t nf = (size_t)ch->fn[0] * ch->fn[1] * ch->fn[2] * h->nrvars;
  size_t npf = (size_t)par->fn[0] * par->fn[1] * par->fn[2] * h->nrvars;
  memset(ch->f, 0, nf * sizeof(double));
  memset(ch->rf, 0, nf * sizeof(double));
  memset(par->f, 0, npf * sizeof(double));
  memset(par->rf, 0, npf * sizeof(double));
  memcpy(ch->qold, ch->q, sizeof(double) * (size_t)ch->qn[0] * ch->qn[1] * ch->qn[2] * h->nrvars);
  return c;
}

/* TransferOverlap (:1919-1951): interior q values of src onto dst */
static void transfer_overlap(const bsamo_hier* h, const OPatch* src, OPatch* dst) {
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = src->mglobal[d][0] > dst->mglobal[d][0] ? src->mglobal[d][0] : dst->mglobal[d][0];
    hi[d] = src->mglobal[d][1] < dst->mglobal[d][1] ? src->mglobal[d][1] : dst->mglobal[d][1];
    if (hi[d] < lo[d]) return;
  }
  for (int v = 0; v < h->nrvars; v++)
    for (int k = lo[2]; k <= hi[2]; k++)
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++)
          Q(dst, i - dst->mglobal[0][0] + 1, j - dst->mglobal[1][0] + 1, k - dst->mglobal[2][0] + 1, v) =
              Q(src, i - src->mglobal[0][0] + 1, j - src->mglobal[1][0] + 1, k - src->mglobal[2][0] + 1, v);
}

int bsamo_regrid(const bsamo_hier* old, const bsamo_regrid_params* prm, bsamo_qinit_fn qinit, void* user,
                 bsamo_hier** out) {
  if (!old || !old->committed || !prm || !out) return -1;
  if (prm->maxlevel < 0 || prm->maxlevel > MAXDEPTH || (prm->initial && !qinit)) return -2;
  double params[6] = {old->dt, old->eps, old->gamma, old->lambda, old->czero, old->cpress};
  bsamo_hier* h = NULL;
  int rc = bsamo_create(old->ndims, old->nrvars, old->mbc, old->problem, params, 6, old->qpo, &h);
  if (rc) return rc;
  h->has_root_xupper = old->has_root_xupper;
  memcpy(h->root_xupper, old->root_xupper, sizeof(h->root_xupper));
  for (int n = 0; n < old->np; n++) { /* the root and the levels below persist */
    const OPatch* p = &old->p[n];
    if (p->level > 0) continue;
    int mg[6], mb[6];
    for (int d = 0; d < 3; d++) {
      mg[2 * d] = p->mglobal[d][0]; mg[2 * d + 1] = p->mglobal[d][1];
      mb[2 * d] = p->mbounds[d][0]; mb[2 * d + 1] = p->mbounds[d][1];
    }
    bsamo_patch_add(h, p->level, p->id, p->parent_id, p->mx, mg, mb, p->mthbc, p->dx, p->xlower);
  }
  if ((rc = bsamo_commit(h))) { bsamo_destroy(h); return rc; }
  for (int n = 0; n < h->np; n++) {
    OPatch* p = &h->p[n];
    const OPatch* o = find_patch(old, p->id);
    size_t nq = (size_t)p->qn[0] * p->qn[1] * p->qn[2] * h->nrvars;
    size_t nc = (size_t)p->cn[0] * p->cn[1] * p->cn[2] * h->nrvars;
    size_t nf = (size_t)p->fn[0] * p->fn[1] * p->fn[2] * h->nrvars;
    memcpy(p->q, o->q, nq * sizeof(double));
    memcpy(p->qold, o->qold, nq * sizeof(double));
    memcpy(p->qc, o->qc, nc * sizeof(double));
    memcpy(p->f, o->f, nf * sizeof(double));
    memcpy(p->rf, o->rf, nf * sizeof(double));
    memcpy(p->ftmp, o->ftmp, nf * sizeof(double));
  }
  int next_id = prm->first_id;
  int (*sub)[3][2] = malloc(sizeof(*sub) * 4 * MAXSUBGRIDS);
  int level;
  for (level = 0; level < prm->maxlevel && nlev(h, level) > 0; level++) { /* AMR(level), :966-991 */
    set_ghost(h, level, 0);
    int np = nlev(h, level);
    int** fl = (int**)calloc(np, sizeof(int*));
    TagList tl = {0, 0, NULL};
    int ib = prm->ibuffer[level];
    for (int a = 0; a < np; a++) { /* ErrFlag, :1059-1131 */
      OPatch* p = lev_patch(h, level, a);
      fl[a] = (int*)calloc((size_t)p->mx[0] * p->mx[1] * p->mx[2], sizeof(int));
      tag_patch(h, p, prm, fl[a]);
      if (ib > 0) buffer_and_list(h, p, ib, fl[a], &tl);
    }
    if (tl.n > 0) { /* InflateEdgeTags, :1267-1308 */
      int poff[13][3];
      if (h->periodic) periodic_offsets(h, level, poff);
      for (int t = tl.n - 1; t >= 0; t--) {
        for (int a = 0; a < np; a++) buffer_tagged(h, lev_patch(h, level, a), tl.c[t], ib, fl[a]);
        if (h->periodic)
          for (int pol = -1; pol <= 1; pol += 2)
            for (int o = 0; o < h->nperoff; o++) {
              int c[3];
              for (int d = 0; d < 3; d++) c[d] = tl.c[t][d] + pol * poff[o][d];
              for (int a = 0; a < np; a++) buffer_tagged(h, lev_patch(h, level, a), c, ib, fl[a]);
            }
      }
    }
    free(tl.c);
    int first_new = h->np;
    for (int a = 0; a < np && rc == 0; a++) { /* GridAdapt -> RefineGrid, :1366-1405 */
      int pidx = lev_index(h, level, a);
      int ng = new_sub_grids(h, &h->p[pidx], fl[a], prm, sub);
      if (ng < 0) { rc = -5; break; }
      ng = split_long(h->ndims, prm->maxside, sub, ng, 4 * MAXSUBGRIDS);
      if (ng < 0) { rc = -5; break; }
      for (int g = 0; g < ng; g++) make_new_grid(h, pidx, sub[g], next_id++, prm, qinit, user);
    }
    for (int a = 0; a < np; a++) free(fl[a]);
    free(fl);
    if (rc) break;
    /* TransferValues (:1859-1951): previous level-(l+1) grids onto new ones */
    for (int c = first_new; c < h->np; c++)
      for (int n = 0; n < old->np; n++)
        if (old->p[n].level == level + 1) transfer_overlap(h, &old->p[n], &h->p[c]);
  }
  free(sub);
  if (rc) { bsamo_destroy(h); return rc; }
  if (nlev(h, level) > 0) set_ghost(h, level, 0); /* AMR(finest) */
  *out = h;
  return 0;
}

/* ------------------------------------------------------------------ */
/* after-step statistics, frame files and restart                      */

/* one F25.12 field (the edit descriptor of every real in WriteQ,
 * bsaminputoutput.f90:72, :106-120, :147): the C library's correctly rounded
 * fixed notation, a field of 25 asterisks when the number needs more than
 * 25 characters, NaN and Infinity right-justified. */
void bsamo_format_f25_12(double x, char out[26]) {
  char b[64];
  int n;
  if (isnan(x))
    n = snprintf(b, sizeof b, "%25s", "NaN");
  else if (isinf(x))
    n = snprintf(b, sizeof b, "%25s", x < 0 ? "-Infinity" : "Infinity");
  else
    n = snprintf(b, sizeof b, "%25.12f", x);
  if (n > 25) {
    memset(b, '*', 25);
    b[25] = 0;
  }
  memcpy(out, b, 26);
}

static void put_f25(FILE* f, double x) {
  char b[26];
  bsamo_format_f25_12(x, b);
  fputs(b, f);
}

/* xupper of a patch: the root's as given to RootInit (bsamroutines.f90:
 * 267-413) for levels <= 0 of a hierarchy built by bsamo_build_uniform;
 * MakeNewGrid's mbounds(2)*parent%dx + parent%xlower (:1752) for a patch
 * with a parent above the root; otherwise xlower + mx*dx. */
static double xupper_of(const bsamo_hier* h, const OPatch* p, int d) {
  if (p->level <= 0 && h->has_root_xupper) return h->root_xupper[d];
  if (p->level > 0 && p->parent >= 0) {
    const OPatch* q = &h->p[p->parent];
    return (double)p->mbounds[d][1] * q->dx[d] + q->xlower[d];
  }
  return p->xlower[d] + (double)p->mx[d] * p->dx[d];
}

/* Ff (CH/problem.f90:901-915) */
static inline double ff_energy(double c) {
  double c2 = c * c;
  return c2 * (c2 - 2.0) / 4.0;
}

/* SUM of variable 1 over m0 x m1 x m2 cells of p starting after (i0,j0,k0) */
static double sum_var1(const OPatch* p, int i0, int j0, int k0, int m0, int m1, int m2) {
  double s = 0.0;
  for (int k = 1; k <= m2; k++)
    for (int j = 1; j <= m1; j++)
      for (int i = 1; i <= m0; i++) s = s + Q(p, i0 + i, j0 + j, k0 + k, 0);
  return s;
}

/* Energy2D (CH/problem.f90:518-547) of variable 1 on the block
 * c(0:m0+1, 0:m1+1) = q(i0:i0+m0+1, j0:j0+m1+1) of p, spacing hh */
static double energy2d(const bsamo_hier* h, const OPatch* p, int i0, int j0, int m0, int m1, double hh) {
#define CE(i, j) Q(p, i0 + (i), j0 + (j), 1, 0)
  double h2 = hh * hh;
  double sf = 0.0, sg = 0.0;
  for (int j = 1; j <= m1; j++)
    for (int i = 1; i <= m0; i++) sf = sf + ff_energy(CE(i, j));
  for (int j = 1; j <= m1; j++)
    for (int i = 1; i <= m0; i++) {
      double a = CE(i + 1, j) - CE(i, j), b = CE(i, j) - CE(i - 1, j);
      double c = CE(i, j + 1) - CE(i, j), d = CE(i, j) - CE(i, j - 1);
      sg = sg + (((a * a + b * b) + c * c) + d * d);
    }
  double tmp = h->eps2 / h2 / 4.0;
  return h2 * (sf + tmp * sg);
#undef CE
}

/* AfterStepStatistics + GetMeshSize over levels finest..0 (bsamroutines.f90:
 * 763-775, :846-868, :918-963) with the plugins' AfterStep2D/3D:
 * CH 2D integral of phi and Energy2D (CH/problem.f90:149-183), CH 3D the
 * integral of phi (:186-215), BioGrowth 2D the integral of phi
 * (BioGrowth/problem.f90:107-136), BioGrowth 3D nothing (:139-152).  A level
 * > 0 patch subtracts the same quantity of its parent's cells under it (the
 * parent's q over mbounds).  The growth plugin, which has no reference
 * counterpart, reports the integral of phi as CH in 3D. */
int bsamo_after_step_stats(const bsamo_hier* h, int finest, double integral[2], long long* meshsize) {
  if (!h || !h->committed || !integral) return -1;
  int nd = h->ndims;
  int mass = !(h->problem == BSAMO_PROBLEM_BIOGROWTH && nd == 3);
  int energy = h->problem == BSAMO_PROBLEM_CH && nd == 2;
  double r1 = 0.0, r2 = 0.0;
  long long ms = 0;
  for (int level = finest; level >= 0; level--)
    for (int a = 0; a < nlev(h, level); a++) {
      const OPatch* p = &h->p[lev_index(h, level, a)];
      double hh = p->dx[0], ch = hh * 2.0;
      double hd = nd == 2 ? hh * hh : hh * hh * hh;
      double chd = nd == 2 ? ch * ch : ch * ch * ch;
      long long pm = 1, pc = 1;
      for (int d = 0; d < nd; d++) {
        pm *= p->mx[d];
        pc *= p->mx[d] / 2;
      }
      if (level == 0) {
        if (mass) r1 = r1 + hd * sum_var1(p, 0, 0, 0, p->mx[0], p->mx[1], p->mx[2]);
        if (energy) r2 = r2 + energy2d(h, p, 0, 0, p->mx[0], p->mx[1], hh);
        ms += pm;
      } else {
        if (p->parent < 0) return -3;
        const OPatch* q = &h->p[p->parent];
        int i0 = p->mbounds[0][0] - 1, j0 = p->mbounds[1][0] - 1, k0 = nd == 3 ? p->mbounds[2][0] - 1 : 0;
        if (mass)
          r1 = r1 + hd * sum_var1(p, 0, 0, 0, p->mx[0], p->mx[1], p->mx[2]) -
               chd * sum_var1(q, i0, j0, k0, p->cmx[0], p->cmx[1], p->cmx[2]);
        if (energy)
          r2 = r2 + energy2d(h, p, 0, 0, p->mx[0], p->mx[1], hh) - energy2d(h, q, i0, j0, p->cmx[0], p->cmx[1], ch);
        ms += pm - pc;
      }
    }
  integral[0] = r1;
  integral[1] = r2;
  if (meshsize) *meshsize = ms;
  return 0;
}

/* one patch block of a frame file: OutputQ (bsaminputoutput.f90:85-129),
 * WriteQ2D/3D (:132-181).  q is the ghosted Fortran-layout array. */
static void write_block(FILE* f, int nd, int nv, int level, const double* dx, const double* xl, const double* xu,
                        const int* mx, const int mg[3][2], const double* q) {
  fputs("  \n", f); /* WRITE(54,*) ' ': list-directed, a leading blank then ' ' */
  fprintf(f, "%3d %3d %3d %3d\n", level, nd, 2, nv);
  const double* rows[3] = {dx, xl, xu};
  for (int r = 0; r < 3; r++) {
    for (int d = 0; d < nd; d++) {
      if (d) fputc(' ', f);
      put_f25(f, rows[r][d]);
    }
    fputc('\n', f);
  }
  for (int d = 0; d < nd; d++) fprintf(f, d ? " %8d" : "%8d", mx[d]);
  fputc('\n', f);
  for (int d = 0; d < nd; d++) fprintf(f, d ? " %8d %8d" : "%8d %8d", mg[d][0], mg[d][1]);
  fputc('\n', f);
  int qn0 = mx[0] + 2, qn1 = mx[1] + 2, qn2 = nd == 3 ? mx[2] + 2 : 1;
  size_t plane = (size_t)qn0 * qn1 * qn2;
  for (int k = 0; k < qn2; k++)
    for (int j = 0; j < qn1; j++)
      for (int i = 0; i < qn0; i++) {
        size_t c = ((size_t)k * qn1 + j) * qn0 + i;
        for (int v = 0; v < nv; v++) { /* 10(F25.12,2X): no blanks after the last value */
          if (v) fputs("  ", f);
          put_f25(f, q[v * plane + c]);
        }
        fputc('\n', f);
      }
}

/* WriteQ (bsaminputoutput.f90:60-82): time, finest level, then every patch
 * of levels 0..finest in visiting order */
int bsamo_write_q(const bsamo_hier* h, const char* path, double time, int finest) {
  if (!h || !h->committed || !path || finest < 0 || finest > MAXDEPTH) return -1;
  FILE* f = fopen(path, "w");
  if (!f) return -8;
  put_f25(f, time);
  fprintf(f, "\n%3d\n", finest);
  for (int level = 0; level <= finest; level++)
    for (int a = 0; a < nlev(h, level); a++) {
      const OPatch* p = &h->p[lev_index(h, level, a)];
      double xu[3];
      int mg[3][2];
      for (int d = 0; d < 3; d++) {
        xu[d] = xupper_of(h, p, d);
        mg[d][0] = p->mglobal[d][0];
        mg[d][1] = p->mglobal[d][1];
      }
      /* q(0:mx+1) (OutputQ, :114-126), whatever mbc is */
      size_t cells = (size_t)(p->mx[0] + 2) * (p->mx[1] + 2) * (h->ndims == 3 ? p->mx[2] + 2 : 1), t = 0;
      double* qb = (double*)malloc(sizeof(double) * cells * h->nrvars);
      for (int v = 0; v < h->nrvars; v++)
        for (int k = h->ndims == 3 ? 0 : 1; k <= (h->ndims == 3 ? p->mx[2] + 1 : 1); k++)
          for (int j = 0; j <= p->mx[1] + 1; j++)
            for (int i = 0; i <= p->mx[0] + 1; i++) qb[t++] = Q(p, i, j, k, v);
      write_block(f, h->ndims, h->nrvars, p->level, p->dx, p->xlower, xu, p->mx, mg, qb);
      free(qb);
    }
  return fclose(f) ? -8 : 0;
}

/* WriteUniformMeshQ (bsaminputoutput.f90:446-572): the root's q prolonged
 * level by level with the mass-corrected bilinear/trilinear operator
 * (gridutilities.f90 BiLinProlongationP1MC / TriLinProlongationP1MC) over the
 * whole domain, each level's patches (ghost layers included) copied over it
 * in visiting order (CopyPatchToUniformGrid), written as one level-0 patch
 * at the finest spacing. */
int bsamo_write_uniform_q(const bsamo_hier* h, const char* path, double time, int finest) {
  if (!h || !h->committed || !path || finest < 0 || finest > MAXDEPTH) return -1;
  if (nlev(h, 0) < 1) return -1;
  int nd = h->ndims, nv = h->nrvars;
  const OPatch* r = &h->p[h->lev_list[MAXDEPTH][0]];
  int n[3] = {r->mx[0], r->mx[1], nd == 3 ? r->mx[2] : 1};
  double dx[3] = {r->dx[0], r->dx[1], r->dx[2]};
  size_t sz = (size_t)(n[0] + 2) * (n[1] + 2) * (nd == 3 ? n[2] + 2 : 1);
  double* u = (double*)malloc(sizeof(double) * sz * nv);
  /* the root's q(0:mx+1): the uniform grids keep one ghost layer whatever
   * mbc is (bsaminputoutput.f90:476-480) */
  {
    size_t t = 0;
    for (int v = 0; v < nv; v++)
      for (int k = nd == 3 ? 0 : 1; k <= (nd == 3 ? n[2] + 1 : 1); k++)
        for (int j = 0; j <= n[1] + 1; j++)
          for (int i = 0; i <= n[0] + 1; i++) u[t++] = Q(r, i, j, k, v);
  }
  for (int level = 1; level <= finest; level++) {
    int nf[3] = {2 * n[0], 2 * n[1], nd == 3 ? 2 * n[2] : 1};
    size_t szf = (size_t)(nf[0] + 2) * (nf[1] + 2) * (nd == 3 ? nf[2] + 2 : 1);
    double* uf = (double*)malloc(sizeof(double) * szf * nv);
    int cmx[3] = {n[0], n[1], nd == 3 ? n[2] : 0};
    for (int v = 0; v < nv; v++) prolong_mc(nd, 1, u + v * sz, cmx, uf + v * szf);
    for (int d = 0; d < nd; d++) dx[d] = dx[d] / 2.0;
    for (int a = 0; a < nlev(h, level); a++) { /* CopyPatchToUniformGrid */
      const OPatch* p = &h->p[lev_index(h, level, a)];
      int k0 = nd == 3 ? p->mglobal[2][0] - 1 : 0;
      int kh = nd == 3 ? p->mx[2] + 1 : 0;
      for (int v = 0; v < nv; v++)  /* q(0:mx+1) (:566-570) */
        for (int k = 0; k <= kh; k++)
          for (int j = 0; j <= p->mx[1] + 1; j++)
            for (int i = 0; i <= p->mx[0] + 1; i++)
              uf[v * szf + ((size_t)(k0 + k) * (nf[1] + 2) + (p->mglobal[1][0] - 1 + j)) * (nf[0] + 2) +
                 (p->mglobal[0][0] - 1 + i)] = Q(p, i, j, nd == 3 ? k : 1, v);
    }
    free(u);
    u = uf;
    sz = szf;
    memcpy(n, nf, sizeof(n));
  }
  FILE* f = fopen(path, "w");
  if (!f) {
    free(u);
    return -8;
  }
  put_f25(f, time);
  fprintf(f, "\n%3d\n", 0);
  double xu[3];
  int mg[3][2];
  for (int d = 0; d < 3; d++) {
    xu[d] = xupper_of(h, r, d);
    mg[d][0] = 1;
    mg[d][1] = n[d];
  }
  write_block(f, nd, nv, 0, dx, r->xlower, xu, n, mg, u);
  free(u);
  return fclose(f) ? -8 : 0;
}

/* ---- ReadQ (bsaminputoutput.f90:184-443) ---- */

typedef struct {
  char* buf;
  size_t nlines;
  char** line;
  size_t* len;
} Lines;

static int read_lines(const char* path, Lines* L) {
  memset(L, 0, sizeof(*L));
  FILE* f = fopen(path, "rb");
  if (!f) return -8;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  L->buf = (char*)malloc((size_t)sz + 1);
  if (sz > 0 && fread(L->buf, 1, (size_t)sz, f) != (size_t)sz) {
    fclose(f);
    return -8;
  }
  fclose(f);
  L->buf[sz] = 0;
  size_t cap = 0;
  for (long i = 0; i < sz;) {
    long e = i;
    while (e < sz && L->buf[e] != '\n') e++;
    if (L->nlines == cap) {
      cap = cap ? 2 * cap : 1024;
      L->line = (char**)realloc(L->line, sizeof(char*) * cap);
      L->len = (size_t*)realloc(L->len, sizeof(size_t) * cap);
    }
    size_t n = (size_t)(e - i);
    if (n && L->buf[i + n - 1] == '\r') n--;
    L->line[L->nlines] = L->buf + i;
    L->len[L->nlines++] = n;
    L->buf[e < sz ? e : sz] = 0;
    i = e + 1;
  }
  return 0;
}

static void free_lines(Lines* L) {
  free(L->buf);
  free(L->line);
  free(L->len);
}

/* the characters [col, col+w) of a record, blank-padded (PAD='YES') */
static void field_of(const Lines* L, size_t ln, int col, int w, char* out) {
  for (int c = 0; c < w; c++) out[c] = (size_t)(col + c) < L->len[ln] ? L->line[ln][col + c] : ' ';
  out[w] = 0;
}

/* Iw input: a blank field is 0 */
static int read_int(const Lines* L, size_t ln, int col, int w, int* v) {
  char b[32], *e;
  field_of(L, ln, col, w, b);
  long x = strtol(b, &e, 10);
  while (*e == ' ') e++;
  if (*e) return -8;
  *v = (int)x;
  return 0;
}

/* F25.12 input of a field written by F25.12 output (a decimal point is
 * required; a blank field is 0) */
static int read_real(const Lines* L, size_t ln, int col, double* v) {
  char b[32], *e;
  field_of(L, ln, col, 25, b);
  int blank = 1, point = 0;
  for (int c = 0; c < 25; c++) {
    if (b[c] != ' ') blank = 0;
    if (b[c] == '.') point = 1;
  }
  if (blank) {
    *v = 0.0;
    return 0;
  }
  if (!point) return -8;
  *v = strtod(b, &e);
  while (*e == ' ') e++;
  return *e ? -8 : 0;
}

/* Restart from a frame file.  `root` is a committed hierarchy with the
 * run's root grid and the levels below it (RootInit); the result copies it,
 * replaces the root's q (ghost layers included) by the file's and adds the
 * file's refinement patches with ids first_id, first_id + 1, ...  The checks
 * of the root block are ReadQ's (:296-336, including its one-sided dx test).
 * Unlike ReadQ, whose restart patches all hang off the youngest patch of
 * the level below (:246, "the usual parent-child relationship is broken"),
 * each patch gets the patch of the level below that contains it as parent,
 * with mbounds and mthbc as MakeNewGrid would set them; qold = q.  The
 * restart patches only feed TransferValues of the first regrid, so the
 * regrid result does not depend on that choice. */
int bsamo_read_q(const bsamo_hier* root, const char* path, int first_id, double* time, bsamo_hier** out) {
  if (!root || !root->committed || !path || !out) return -1;
  Lines L;
  int rc = read_lines(path, &L);
  if (rc) {
    free_lines(&L);
    return rc;
  }
  double params[6] = {root->dt, root->eps, root->gamma, root->lambda, root->czero, root->cpress};
  bsamo_hier* h = NULL;
  if ((rc = bsamo_create(root->ndims, root->nrvars, root->mbc, root->problem, params, 6, root->qpo, &h))) {
    free_lines(&L);
    return rc;
  }
  h->has_root_xupper = root->has_root_xupper;
  memcpy(h->root_xupper, root->root_xupper, sizeof(h->root_xupper));
  for (int n = 0; n < root->np; n++) {
    const OPatch* p = &root->p[n];
    if (p->level > 0) continue;
    int mg[6], mb[6];
    for (int d = 0; d < 3; d++) {
      mg[2 * d] = p->mglobal[d][0]; mg[2 * d + 1] = p->mglobal[d][1];
      mb[2 * d] = p->mbounds[d][0]; mb[2 * d + 1] = p->mbounds[d][1];
    }
    bsamo_patch_add(h, p->level, p->id, p->parent_id, p->mx, mg, mb, p->mthbc, p->dx, p->xlower);
  }
  if ((rc = bsamo_commit(h))) goto fail;
  for (int n = 0; n < h->np; n++) {
    OPatch* p = &h->p[n];
    const OPatch* o = find_patch(root, p->id);
    size_t nq = (size_t)p->qn[0] * p->qn[1] * p->qn[2] * h->nrvars;
    size_t nc = (size_t)p->cn[0] * p->cn[1] * p->cn[2] * h->nrvars;
    size_t nf = (size_t)p->fn[0] * p->fn[1] * p->fn[2] * h->nrvars;
    memcpy(p->q, o->q, nq * sizeof(double));
    memcpy(p->qold, o->qold, nq * sizeof(double));
    memcpy(p->qc, o->qc, nc * sizeof(double));
    memcpy(p->f, o->f, nf * sizeof(double));
    memcpy(p->rf, o->rf, nf * sizeof(double));
    memcpy(p->ftmp, o->ftmp, nf * sizeof(double));
  }
  rc = -8;
  int nd = h->ndims, finest, r0 = h->lev_list[MAXDEPTH][0];
  double t;
  if (L.nlines < 2 || read_real(&L, 0, 0, &t) || read_int(&L, 1, 0, 3, &finest)) goto fail;
  if (finest < 0 || finest > MAXDEPTH) goto fail;
  size_t ln = 2;
  int next_id = first_id;
  for (int lvl = 0; lvl <= finest; lvl++) {
    for (;;) {
      if (ln >= L.nlines) goto done; /* READ(54,'(A1)',IOSTAT=ioerror); ioerror < 0 */
      int level, rnd, ratio, nv;
      if (ln + 1 >= L.nlines) goto fail;
      if (read_int(&L, ln + 1, 0, 3, &level) || read_int(&L, ln + 1, 4, 3, &rnd) ||
          read_int(&L, ln + 1, 8, 3, &ratio) || read_int(&L, ln + 1, 12, 3, &nv))
        goto fail;
      if (level != lvl) break; /* BACKSPACE twice, next level */
      ln += 2;
      if (rnd != nd || ratio != 2 || nv != h->nrvars || ln + 5 > L.nlines) goto fail;
      double dx[3] = {0, 0, 0}, xl[3] = {0, 0, 0}, xu[3] = {0, 0, 0};
      int mx[3] = {1, 1, 1}, mg[3][2] = {{1, 1}, {1, 1}, {1, 1}};
      for (int d = 0; d < nd; d++)
        if (read_real(&L, ln, 26 * d, &dx[d]) || read_real(&L, ln + 1, 26 * d, &xl[d]) ||
            read_real(&L, ln + 2, 26 * d, &xu[d]) || read_int(&L, ln + 3, 9 * d, 8, &mx[d]) ||
            read_int(&L, ln + 4, 18 * d, 8, &mg[d][0]) || read_int(&L, ln + 4, 18 * d + 9, 8, &mg[d][1]))
          goto fail;
      ln += 5;
      OPatch* tgt;
      if (level == 0) {
        tgt = &h->p[r0];
        for (int d = 0; d < nd; d++) {
          const double small = 1.0e-08;
          if (dx[d] - tgt->dx[d] > small) goto fail;
          if (fabs(xl[d] - tgt->xlower[d]) > small) goto fail;
          if (fabs(xu[d] - xupper_of(h, tgt, d)) > small) goto fail;
          if (mx[d] != tgt->mx[d] || mg[d][0] != 1 || mg[d][1] != tgt->mx[d]) goto fail;
        }
      } else {
        int par = -1, mb[3][2] = {{1, 1}, {1, 1}, {1, 1}}, thbc[6];
        for (int d = 0; d < nd; d++)
          if (mx[d] < 2 || mg[d][0] % 2 != 1 || mg[d][1] % 2 != 0 || mg[d][1] - mg[d][0] + 1 != mx[d]) goto fail;
        for (int a = 0; a < nlev(h, level - 1) && par < 0; a++) {
          int c = lev_index(h, level - 1, a), in = 1;
          const OPatch* q = &h->p[c];
          for (int d = 0; d < nd; d++)
            if ((mg[d][0] + 1) / 2 < q->mglobal[d][0] || mg[d][1] / 2 > q->mglobal[d][1]) in = 0;
          if (in) par = c;
        }
        if (par < 0) goto fail;
        const OPatch* q = &h->p[par];
        for (int d = 0; d < nd; d++) {
          mb[d][0] = (mg[d][0] + 1) / 2 - q->mglobal[d][0] + 1;
          mb[d][1] = mg[d][1] / 2 - q->mglobal[d][0] + 1;
        }
        for (int f = 0; f < 6; f++) thbc[f] = f < 2 * nd ? INTERNALBC : 10;
        for (int e = 0; e < nd; e++) {
          if (q->mthbc[2 * e] < INTERNALBC && mb[e][0] == 1) thbc[2 * e] = q->mthbc[2 * e];
          if (q->mthbc[2 * e + 1] < INTERNALBC && mb[e][1] == q->mx[e]) thbc[2 * e + 1] = q->mthbc[2 * e + 1];
        }
        int c = add_live_patch(h, level, next_id++, par, mx, mg, mb, thbc, dx, xl);
        tgt = &h->p[c];
      }
      /* q(0:mx+1) (ReadQ2D/3D, :392-440), whatever mbc is */
      size_t plane = (size_t)tgt->qn[0] * tgt->qn[1] * tgt->qn[2];
      size_t cells = (size_t)(tgt->mx[0] + 2) * (tgt->mx[1] + 2) * (nd == 3 ? tgt->mx[2] + 2 : 1);
      if (ln + cells > L.nlines) goto fail;
      int k0 = nd == 3 ? 0 : 1, k1 = nd == 3 ? tgt->mx[2] + 1 : 1;
      for (int k = k0; k <= k1; k++)
        for (int j = 0; j <= tgt->mx[1] + 1; j++)
          for (int i = 0; i <= tgt->mx[0] + 1; i++, ln++)
            for (int v = 0; v < nv; v++)
              if (read_real(&L, ln, 27 * v, &Q(tgt, i, j, k, v))) goto fail;
      if (level > 0) memcpy(tgt->qold, tgt->q, sizeof(double) * plane * nv);
    }
  }
done:
  free_lines(&L);
  if (time) *time = t;
  *out = h;
  return 0;
fail:
  free_lines(&L);
  bsamo_destroy(h);
  return rc ? rc : -8;
}

/* one record of OUT/stats.dat: WRITE(65,'(3(F25.12),1x,I8)') currenttime,
 * integralresult(1:2), totalmeshsize (bsamroutines.f90:771-775) */
int bsamo_format_stats_line(double time, const double integral[2], long long meshsize, char* out, size_t n) {
  char a[26], b[26], c[26], m[16];
  bsamo_format_f25_12(time, a);
  bsamo_format_f25_12(integral[0], b);
  bsamo_format_f25_12(integral[1], c);
  if (meshsize < -9999999LL || meshsize > 99999999LL)
    strcpy(m, "********");
  else
    snprintf(m, sizeof m, "%8lld", meshsize);
  int k = snprintf(out, n, "%s%s%s %s\n", a, b, c, m);
  return k < 0 || (size_t)k >= n ? -1 : 0;
}
