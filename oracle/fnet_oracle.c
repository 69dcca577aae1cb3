/*
 * ORACLE — test infrastructure only (see fnet_oracle.h).  FP64 CPU restatement of
 * Fortnet's hot path.  Compiled with -ffp-contract=off so that every floating-point
 * operation is a separately rounded IEEE operation, as in the reference's x86-64 build,
 * and so that the result is the same on x86-64 and aarch64 hosts.
 *
 * Reference file paths below are relative to the Fortnet source tree.
 */
#include "fnet_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846 /* lib_dftbp/constants.F90:15 */
#define GOLDEN_MEAN_P1 1.6180339887498949 /* lib_dftbp/constants.F90:131 */
#define DP_EPS 2.220446049250313e-16 /* epsilon(1.0_dp) */

/* ====================================================================================
 * RANLUX, luxury level 0..4 — restates lib_dftbp/ranlux.F90:150-360 (James/Luescher).
 * Arrays are kept 1-based (index 0 unused) to follow the published algorithm literally.
 * ==================================================================================== */
typedef struct {
  int next[25];
  int luxlev, nskip, in24, i24, j24;
  int iseeds[25];
  int icarry;
  double twom24, twom12;
} ranlux_t;

static const int NDSKIP[5] = {0, 24, 73, 199, 365};
#define ITWO24 (1 << 24)
#define ICONS 2147483563
#define MASKLO (ITWO24 - 1)
#define MASKHI (~MASKLO)

void *orc_ranlux_new(int32_t luxlev, int32_t seed) {
  ranlux_t *r = (ranlux_t *)calloc(1, sizeof(ranlux_t));
  int jseed = 314159265;
  r->luxlev = 3;
  if (luxlev >= 0 && luxlev <= 4) r->luxlev = luxlev;
  if (seed > 0) jseed = seed;
  r->nskip = NDSKIP[r->luxlev];
  r->in24 = 0;
  r->twom24 = 1.0;
  for (int ii = 1; ii <= 24; ii++) {
    r->twom24 = r->twom24 * 0.5;
    int kk = jseed / 53668;
    jseed = 40014 * (jseed - kk * 53668) - kk * 12211;
    if (jseed < 0) jseed = jseed + ICONS;
    r->iseeds[ii] = jseed % ITWO24;
    r->next[ii] = ii - 1;
  }
  r->twom12 = r->twom24 * 4096.0;
  r->next[1] = 24;
  r->i24 = 24;
  r->j24 = 10;
  r->icarry = 0;
  if ((r->iseeds[24] & MASKHI) != 0) r->icarry = 1;
  return r;
}

static void ranlux_step(ranlux_t *r, int *out_iuni) {
  int iuni = r->iseeds[r->j24] - r->iseeds[r->i24] - r->icarry;
  if ((iuni & MASKHI) != 0) {
    iuni = iuni & MASKLO;
    r->icarry = 1;
  } else {
    r->icarry = 0;
  }
  r->iseeds[r->i24] = iuni;
  r->i24 = r->next[r->i24];
  r->j24 = r->next[r->j24];
  *out_iuni = iuni;
}

void orc_ranlux_get(void *h, double *out, int64_t n) {
  ranlux_t *r = (ranlux_t *)h;
  for (int64_t iv = 0; iv < n; iv++) {
    int iuni;
    ranlux_step(r, &iuni);
    double uni = (double)iuni * r->twom24;
    if (uni < r->twom12) {
      uni = uni + ((double)r->iseeds[r->j24] * r->twom24) * r->twom24;
      if (uni <= 0.0) uni = r->twom24 * r->twom24;
    }
    out[iv] = uni;
    r->in24 = r->in24 + 1;
    if (r->in24 == 24) {
      r->in24 = 0;
      for (int isk = 0; isk < r->nskip; isk++) ranlux_step(r, &iuni);
    }
  }
}

void orc_ranlux_free(void *h) { free(h); }

/* normalXavier2d (lib_common/random.F90:122-181): gain 1, min 0.1, column-major fill. */
static void normal_xavier(ranlux_t *r, double *arr, int64_t n, int n_last, int n_current) {
  orc_ranlux_get(r, arr, n);
  double var = 1.0 * 1.0 * 2.0 / (double)(n_last + n_current);
  double bound = sqrt(-2.0 * var * log(0.1 * sqrt(2.0 * ORC_PI * var)));
  for (int64_t i = 0; i < n; i++) {
    double x = (arr[i] - 0.5) * 2.0 * bound;
    arr[i] = exp(-0.5 * (x * x) / var) / sqrt(2.0 * ORC_PI * var);
  }
}

/* ---- parameter vector layout of one sub-network (network.F90:397-427, H10) ---- */
static void layout(const orc_net *net, int64_t *woff, int64_t *boff, int64_t *np) {
  int L = net->nlayer;
  int64_t ind = 0;
  for (int l = 0; l < L; l++) {
    woff[l] = ind;
    ind += (int64_t)net->dims[l] * (l < L - 1 ? net->dims[l + 1] : 1);
  }
  for (int l = 0; l < L; l++) {
    boff[l] = ind;
    ind += net->dims[l];
  }
  *np = ind;
}

int64_t orc_nparams(const orc_net *net) {
  int64_t woff[64], boff[64], np;
  layout(net, woff, boff, &np);
  return np;
}

/* TBpnn_init -> TNetwork_init -> initLayers -> TLayer_init draw order
 * (bpnn.F90:133-136, network.F90:110-120, layer.F90:72-86). */
void orc_init_bpnn_params(void *h, const orc_net *net, int32_t nspecies, double *params) {
  ranlux_t *r = (ranlux_t *)h;
  int64_t woff[64], boff[64], np;
  layout(net, woff, boff, &np);
  int L = net->nlayer;
  for (int s = 0; s < nspecies; s++) {
    double *p = params + (int64_t)s * np;
    for (int l = 0; l < L; l++) {
      int ncur = net->dims[l];
      int nnext = (l < L - 1) ? net->dims[l + 1] : 1;
      normal_xavier(r, p + woff[l], (int64_t)ncur * nnext, nnext, ncur);
      for (int i = 0; i < ncur; i++) p[boff[l] + i] = 0.0;
    }
    for (int i = 0; i < net->dims[L - 1]; i++) p[woff[L - 1] + i] = 0.0;
  }
}

void orc_knuth_shuffle(void *h, int32_t *arr, int32_t n) {
  ranlux_t *r = (ranlux_t *)h;
  for (int ii = n; ii >= 2; ii--) {
    double rnd;
    orc_ranlux_get(r, &rnd, 1);
    int rndpos = (int)(rnd * ii) + 1;
    int tmp = arr[rndpos - 1];
    arr[rndpos - 1] = arr[ii - 1];
    arr[ii - 1] = tmp;
  }
}

/* ====================================================================================
 * Geometry: recVecs2p (fnetdata.F90:1141-1148, simplealgebra.F90:41-125)
 * ==================================================================================== */
int orc_recvecs2p(const double *L, double *R) {
#define M(i, j) L[((i)-1) + 3 * ((j)-1)]
  double tmp = M(1, 1) * (M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3));
  tmp = tmp - M(1, 2) * (M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3));
  tmp = tmp + M(1, 3) * (M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2));
  double det = tmp;
  if (fabs(det) < 1e-12) return -1;
  double inv[9];
#define INV(i, j) inv[((i)-1) + 3 * ((j)-1)]
  INV(1, 1) = -(M(2, 3) * M(3, 2)) + M(2, 2) * M(3, 3);
  INV(2, 1) = M(2, 3) * M(3, 1) - M(2, 1) * M(3, 3);
  INV(3, 1) = -(M(2, 2) * M(3, 1)) + M(2, 1) * M(3, 2);
  INV(1, 2) = M(1, 3) * M(3, 2) - M(1, 2) * M(3, 3);
  INV(2, 2) = -(M(1, 3) * M(3, 1)) + M(1, 1) * M(3, 3);
  INV(3, 2) = M(1, 2) * M(3, 1) - M(1, 1) * M(3, 2);
  INV(1, 3) = -(M(1, 3) * M(2, 2)) + M(1, 2) * M(2, 3);
  INV(2, 3) = M(1, 3) * M(2, 1) - M(1, 1) * M(2, 3);
  INV(3, 3) = -(M(1, 2) * M(2, 1)) + M(1, 1) * M(2, 2);
  for (int k = 0; k < 9; k++) inv[k] = inv[k] / det;
  /* reshape(..., order=[2,1]) == transpose */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i + 3 * j] = inv[j + 3 * i];
#undef M
#undef INV
  return 0;
}

/* ====================================================================================
 * Neighbour iteration — restates TNeighIterator_getNextNeighbours (dynneighlist.F90:233-320)
 * over TLatPointIter (latpointiter.F90:62-253, getRanges 226-253), for the atoms sel[] of a
 * (possibly species-reduced) geometry, centre atom sel[ic].  Entries come out in the
 * iterator's order: central cell ic+1..nsel-1,0..ic-1, then every lattice point in
 * (n1 outer, n3 inner) order with atoms ic, ic+1, ... (cyclic).
 * ==================================================================================== */
typedef struct {
  int64_t n, cap;
  int32_t *j;      /* original atom index (0-based, within the structure) */
  int32_t *shift;  /* 3 per entry */
  double *crd;     /* 3 per entry: image coordinates */
  double *d2;      /* squared distance */
  double *dist;    /* sqrt(d2) */
} nblist;

static void nb_reset(nblist *l) { l->n = 0; }
static void nb_free(nblist *l) {
  free(l->j); free(l->shift); free(l->crd); free(l->d2); free(l->dist);
  memset(l, 0, sizeof(*l));
}
static void nb_push(nblist *l, int32_t j, const int *sh, const double *xyz, double d2) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 256;
    l->j = (int32_t *)realloc(l->j, l->cap * sizeof(int32_t));
    l->shift = (int32_t *)realloc(l->shift, 3 * l->cap * sizeof(int32_t));
    l->crd = (double *)realloc(l->crd, 3 * l->cap * sizeof(double));
    l->d2 = (double *)realloc(l->d2, l->cap * sizeof(double));
    l->dist = (double *)realloc(l->dist, l->cap * sizeof(double));
  }
  int64_t k = l->n++;
  l->j[k] = j;
  for (int c = 0; c < 3; c++) {
    l->shift[3 * k + c] = sh[c];
    l->crd[3 * k + c] = xyz[c];
  }
  l->d2[k] = d2;
  l->dist[k] = sqrt(d2);
}

typedef struct {
  int natom;
  int periodic;
  const double *coords; /* natom*3 */
  const double *L;      /* 9 */
  double R[9];
} geo_t;

static inline void nb_test(const geo_t *g, const double *ci, int j, const double *cv,
                           const int *sh, double rc2, nblist *out) {
  double nc[3], d[3];
  for (int c = 0; c < 3; c++) nc[c] = g->coords[3 * j + c] + cv[c];
  for (int c = 0; c < 3; c++) d[c] = ci[c] - nc[c];
  double dist2 = d[0] * d[0];
  dist2 = dist2 + d[1] * d[1];
  dist2 = dist2 + d[2] * d[2];
  if (dist2 <= rc2) nb_push(out, j, sh, nc, dist2);
}

static void lattice_ranges(const geo_t *g, double rcut, int *lo, int *hi) {
  for (int ii = 0; ii < 3; ii++) {
    const double *col = g->R + 3 * ii;
    double s = col[0] * col[0];
    s = s + col[1] * col[1];
    s = s + col[2] * col[2];
    int itmp = (int)floor(rcut * sqrt(s));
    lo[ii] = -(itmp + 1);
    hi[ii] = itmp + 1;
  }
}

static void nb_build(const geo_t *g, const int32_t *sel, int nsel, int ic, double rcut,
                     nblist *out) {
  nb_reset(out);
  double rc2 = rcut * rcut;
  const double *ci = g->coords + 3 * sel[ic];
  double zero[3] = {0.0, 0.0, 0.0};
  int sh0[3] = {0, 0, 0};
  for (int t = 1; t < nsel; t++) nb_test(g, ci, sel[(ic + t) % nsel], zero, sh0, rc2, out);
  if (!g->periodic) return;
  int lo[3], hi[3];
  lattice_ranges(g, rcut, lo, hi);
  for (int n1 = lo[0]; n1 <= hi[0]; n1++)
    for (int n2 = lo[1]; n2 <= hi[1]; n2++)
      for (int n3 = lo[2]; n3 <= hi[2]; n3++) {
        if (n1 == 0 && n2 == 0 && n3 == 0) continue;
        int sh[3] = {n1, n2, n3};
        double cv[3];
        for (int c = 0; c < 3; c++) {
          double v = g->L[c + 0] * (double)n1;
          v = v + g->L[c + 3] * (double)n2;
          v = v + g->L[c + 6] * (double)n3;
          cv[c] = v;
        }
        for (int t = 0; t < nsel; t++) nb_test(g, ci, sel[(ic + t) % nsel], cv, sh, rc2, out);
      }
}

static int geo_of(const orc_batch *b, int s, geo_t *g) {
  int64_t a0 = b->atom_offsets[s];
  g->natom = (int)(b->atom_offsets[s + 1] - a0);
  g->periodic = b->periodic ? b->periodic[s] : 0;
  g->coords = b->coords + 3 * a0;
  g->L = b->latvecs ? b->latvecs + 9 * (int64_t)s : NULL;
  if (g->periodic) return orc_recvecs2p(g->L, g->R);
  return 0;
}

/* ---- thread pool helper: contiguous block split like getStartAndEndIndex ---- */
typedef struct {
  int start, end;
  void *ctx;
  int (*fn)(void *ctx, int s, void *scratch);
  int rc;
} job_t;

static void block_range(int n, int nth, int rank, int *s, int *e) {
  /* parallel.F90:23-56: the remainder goes to the last ranks */
  int base = n / nth, rem = n % nth;
  int first_big = nth - rem;
  if (rank < first_big) {
    *s = rank * base;
    *e = *s + base;
  } else {
    *s = first_big * base + (rank - first_big) * (base + 1);
    *e = *s + base + 1;
  }
}

/* ====================================================================================
 * Cutoff functions and G1..G5 (acsf.F90:1159-1492)
 * ==================================================================================== */
static inline double cutoff_wo(double rr, double id1, double id2, double rcut) {
  return 0.5 * id1 * id2 * (cos(ORC_PI * rr / rcut) + 1.0);
}
static inline double cutoff_chk(double rr, double id1, double id2, double rcut) {
  return rr > rcut ? 0.0 : 0.5 * id1 * id2 * (cos(ORC_PI * rr / rcut) + 1.0);
}
static inline double dfcutoff_wo(double rr, double id1, double id2, double rcut) {
  /* deriv = 1: (pi/rcut)**1 * cos(pi*rr/rcut + 0.5*1*pi) */
  return 0.5 * id1 * id2 * (ORC_PI / rcut) * cos((ORC_PI * rr / rcut) + 0.5 * 1.0 * ORC_PI);
}
static inline double norm2v(const double *v) {
  /* norm2 intrinsic; the reference's compiler uses a scaled sum, equal to rounding level */
  return sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
}

typedef struct {
  int n;
  const double *crd, *dist;
  const double *ids; /* atom ids of the neighbours */
  const int32_t *idx;
} glist;

static double gval(const orc_gfunc *gf, const double *ci, double atomId, const glist *l1,
                   const glist *l2) {
  double s = 0.0;
  switch (gf->type) {
    case 1:
      for (int k = 0; k < l1->n; k++) s = s + cutoff_chk(l1->dist[k], atomId, l1->ids[k], gf->rcut);
      return s;
    case 2:
      for (int k = 0; k < l1->n; k++) {
        double r = l1->dist[k];
        s = s + exp(-(gf->eta * ((r - gf->rs) * (r - gf->rs)))) *
                    cutoff_chk(r, atomId, l1->ids[k], gf->rcut);
      }
      return s;
    case 3:
      for (int k = 0; k < l1->n; k++) {
        double r = l1->dist[k];
        s = s + cos(gf->kappa * r) * cutoff_chk(r, atomId, l1->ids[k], gf->rcut);
      }
      return s;
    case 4:
    case 5: {
      if (l1->n == 0 && l2->n == 0) return 0.0;
      for (int jj = 0; jj < l1->n; jj++) {
        const double *cj = l1->crd + 3 * jj;
        double rj = l1->dist[jj];
        for (int kk = 0; kk < l2->n; kk++) {
          const double *ck = l2->crd + 3 * kk;
          double rk = l2->dist[kk];
          double vj[3] = {cj[0] - ci[0], cj[1] - ci[1], cj[2] - ci[2]};
          double vk[3] = {ck[0] - ci[0], ck[1] - ci[1], ck[2] - ci[2]};
          double dot = vj[0] * vk[0];
          dot = dot + vj[1] * vk[1];
          dot = dot + vj[2] * vk[2];
          double theta = acos(dot / (rj * rk + 1e-13));
          double ang = pow(1.0 + gf->lambda * cos(theta), gf->xi);
          if (gf->type == 5) {
            s = s + ang * exp(-(gf->eta * (rj * rj + rk * rk))) *
                        cutoff_wo(rj, atomId, l1->ids[jj], gf->rcut) *
                        cutoff_wo(rk, atomId, l2->ids[kk], gf->rcut);
          } else {
            double vjk[3] = {cj[0] - ck[0], cj[1] - ck[1], cj[2] - ck[2]};
            double djk = norm2v(vjk);
            s = s + ang * exp(-(gf->eta * (rj * rj + rk * rk + djk * djk))) *
                        cutoff_wo(rj, atomId, l1->ids[jj], gf->rcut) *
                        cutoff_wo(rk, atomId, l2->ids[kk], gf->rcut) *
                        cutoff_chk(djk, l1->ids[jj], l2->ids[kk], gf->rcut);
          }
        }
      }
      return s * pow(2.0, 1.0 - gf->xi);
    }
  }
  return NAN;
}

/* ---- per-(atom, G) neighbour lists (buildGFunctionNeighborlists, acsf.F90:943-1066) ---- */
typedef struct {
  nblist full;          /* mode 1: one unrestricted list per atom */
  nblist a, b;          /* the function's lists 1 and 2 */
  int32_t *sel;         /* reduced geometry atom indices */
  double *ids1, *ids2;  /* atom ids of list entries */
  int32_t *idx1, *idx2; /* original indices of list entries */
  int64_t cap_ids;
} gwork;

static void gwork_free(gwork *w) {
  nb_free(&w->full); nb_free(&w->a); nb_free(&w->b);
  free(w->sel); free(w->ids1); free(w->ids2); free(w->idx1); free(w->idx2);
  memset(w, 0, sizeof(*w));
}

static void ensure_ids(gwork *w, int64_t n) {
  if (n <= w->cap_ids) return;
  w->cap_ids = n + 256;
  w->ids1 = (double *)realloc(w->ids1, w->cap_ids * sizeof(double));
  w->ids2 = (double *)realloc(w->ids2, w->cap_ids * sizeof(double));
  w->idx1 = (int32_t *)realloc(w->idx1, w->cap_ids * sizeof(int32_t));
  w->idx2 = (int32_t *)realloc(w->idx2, w->cap_ids * sizeof(int32_t));
}

/* Species-reduced list of atom i for atomic number z (z == 0: no reduction), mode 0. */
static void list_for_species(const geo_t *g, const int32_t *atnum, int i, int z, double rcut,
                             gwork *w, nblist *out) {
  int nsel = 0, ic = 0;
  for (int a = 0; a < g->natom; a++) {
    if (a == i) {
      ic = nsel;
      w->sel[nsel++] = a;
    } else if (z == 0 || atnum[a] == z) {
      w->sel[nsel++] = a;
    }
  }
  nb_build(g, w->sel, nsel, ic, rcut, out);
}

/* Same list obtained by filtering the unrestricted list (mode 1). */
static void filter_species(const nblist *full, const int32_t *atnum, int i, int z, nblist *out) {
  nb_reset(out);
  for (int64_t k = 0; k < full->n; k++) {
    int j = full->j[k];
    if (z == 0 || j == i || atnum[j] == z)
      nb_push(out, j, full->shift + 3 * k, full->crd + 3 * k, full->d2[k]);
  }
}

typedef struct {
  glist l1, l2;
  double atomId;
} gctx;

/* Builds lists 1 and 2 of (atom i, function gf); returns 0 on success. */
static void build_glists(const geo_t *g, const int32_t *atnum, const double *ext, int next,
                         int i, const orc_gfunc *gf, int mode, double full_rcut, gwork *w,
                         gctx *out) {
  int resolved = !(gf->z1 == 0 && gf->z2 == 0);
  int z1 = resolved ? gf->z1 : 0;
  int z2 = resolved ? gf->z2 : 0;
  int angular = gf->type >= 4;
  (void)full_rcut;
  if (mode == 0) {
    list_for_species(g, atnum, i, z1, gf->rcut, w, &w->a);
    if (resolved && angular) list_for_species(g, atnum, i, z2, gf->rcut, w, &w->b);
  } else {
    filter_species(&w->full, atnum, i, z1, &w->a);
    if (resolved && angular) filter_species(&w->full, atnum, i, z2, &w->b);
  }
  const nblist *A = &w->a;
  const nblist *B = (resolved && angular) ? &w->b : &w->a;
  ensure_ids(w, (A->n > B->n ? A->n : B->n) + 1);
  for (int64_t k = 0; k < A->n; k++) {
    w->idx1[k] = A->j[k];
    w->ids1[k] = gf->atomid > 0 ? ext[(int64_t)A->j[k] * next + (gf->atomid - 1)] : 1.0;
  }
  for (int64_t k = 0; k < B->n; k++) {
    w->idx2[k] = B->j[k];
    w->ids2[k] = gf->atomid > 0 ? ext[(int64_t)B->j[k] * next + (gf->atomid - 1)] : 1.0;
  }
  out->l1 = (glist){(int)A->n, A->crd, A->dist, w->ids1, w->idx1};
  out->l2 = (glist){(int)B->n, B->crd, B->dist, w->ids2, w->idx2};
  out->atomId = gf->atomid > 0 ? ext[(int64_t)i * next + (gf->atomid - 1)] : 1.0;
}

typedef struct {
  const orc_batch *b;
  const orc_gfunc *g;
  int ng, mode;
  double *vals;
} acsf_job;

static int acsf_struct(void *vctx, int s, void *scratch) {
  acsf_job *J = (acsf_job *)vctx;
  gwork *w = (gwork *)scratch;
  geo_t geo;
  if (geo_of(J->b, s, &geo)) return -1;
  int64_t a0 = J->b->atom_offsets[s];
  const int32_t *atnum = J->b->atnum + a0;
  const double *ext = J->b->ext ? J->b->ext + a0 * J->b->next : NULL;
  w->sel = (int32_t *)realloc(w->sel, (geo.natom + 1) * sizeof(int32_t));
  for (int i = 0; i < geo.natom; i++) {
    const double *ci = geo.coords + 3 * i;
    if (J->mode == 1) {
      /* all functions of one run share the cutoff in mode 1 (checked by the caller) */
      for (int a = 0; a < geo.natom; a++) w->sel[a] = a;
      nb_build(&geo, w->sel, geo.natom, i, J->g[0].rcut, &w->full);
    }
    for (int k = 0; k < J->ng; k++) {
      gctx c;
      build_glists(&geo, atnum, ext, J->b->next, i, &J->g[k], J->mode, 0.0, w, &c);
      J->vals[(a0 + i) * J->ng + k] = gval(&J->g[k], ci, c.atomId, &c.l1, &c.l2);
    }
  }
  return 0;
}

typedef struct {
  job_t job;
  void *scratch;
} worker_t;

static void *worker_main(void *arg) {
  worker_t *w = (worker_t *)arg;
  for (int s = w->job.start; s < w->job.end && w->job.rc == 0; s++)
    w->job.rc = w->job.fn(w->job.ctx, s, w->scratch);
  return NULL;
}

static int run_blocks(int nstruct, int nthreads, void *ctx,
                      int (*fn)(void *, int, void *), size_t scratch_size,
                      void (*scratch_free)(void *)) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > nstruct) nthreads = nstruct > 0 ? nstruct : 1;
  worker_t *ws = (worker_t *)calloc(nthreads, sizeof(worker_t));
  pthread_t *th = (pthread_t *)calloc(nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; t++) {
    block_range(nstruct, nthreads, t, &ws[t].job.start, &ws[t].job.end);
    ws[t].job.ctx = ctx;
    ws[t].job.fn = fn;
    ws[t].scratch = calloc(1, scratch_size);
  }
  if (nthreads == 1) {
    worker_main(&ws[0]);
  } else {
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, worker_main, &ws[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  }
  int rc = 0;
  for (int t = 0; t < nthreads; t++) {
    if (ws[t].job.rc) rc = ws[t].job.rc;
    if (scratch_free) scratch_free(ws[t].scratch);
    free(ws[t].scratch);
  }
  free(ws);
  free(th);
  return rc;
}

static void gwork_free_v(void *p) { gwork_free((gwork *)p); }

int orc_acsf(const orc_batch *b, const orc_gfunc *g, int32_t ng, int32_t mode, double *vals,
             int32_t nthreads) {
  if (mode == 1)
    for (int k = 1; k < ng; k++)
      if (g[k].rcut != g[0].rcut) return -2;
  acsf_job J = {b, g, ng, mode, vals};
  return run_blocks(b->nstruct, nthreads, &J, acsf_struct, sizeof(gwork), gwork_free_v);
}

/* ---- full neighbour lists (for pair-set comparisons) ---- */
typedef struct {
  const orc_batch *b;
  double rcut;
  int64_t *counts;
  const int64_t *offsets;
  int32_t *oj, *osh;
  double *od2;
} nbjob;

static int nb_struct(void *vctx, int s, void *scratch) {
  nbjob *J = (nbjob *)vctx;
  nblist *l = (nblist *)scratch;
  geo_t geo;
  if (geo_of(J->b, s, &geo)) return -1;
  int64_t a0 = J->b->atom_offsets[s];
  int32_t *sel = (int32_t *)malloc((geo.natom + 1) * sizeof(int32_t));
  for (int a = 0; a < geo.natom; a++) sel[a] = a;
  for (int i = 0; i < geo.natom; i++) {
    nb_build(&geo, sel, geo.natom, i, J->rcut, l);
    J->counts[a0 + i] = l->n;
    if (J->oj) {
      int64_t o = J->offsets[a0 + i];
      for (int64_t k = 0; k < l->n; k++) {
        J->oj[o + k] = l->j[k];
        for (int c = 0; c < 3; c++) J->osh[3 * (o + k) + c] = l->shift[3 * k + c];
        J->od2[o + k] = l->d2[k];
      }
    }
  }
  free(sel);
  return 0;
}

static void nb_free_v(void *p) { nb_free((nblist *)p); }

int orc_neighbours(const orc_batch *b, double rcut, int64_t *counts, const int64_t *offsets,
                   int32_t *out_j, int32_t *out_shift, double *out_d2, int32_t nthreads) {
  nbjob J = {b, rcut, counts, offsets, out_j, out_shift, out_d2};
  return run_blocks(b->nstruct, nthreads, &J, nb_struct, sizeof(nblist), nb_free_v);
}

/* ====================================================================================
 * dG/dR — gFuncGrad (acsf.F90:1496-1670), T_matr (1674-1697), iGeoAcsfGrad (870-939)
 * ==================================================================================== */
static void t_matr(const double *u, double nrm, double *T /* col-major 3x3 */) {
  for (int k = 0; k < 9; k++) T[k] = 0.0;
  for (int i = 0; i < 3; i++) {
    T[i + 3 * i] = 1.0 - u[i] * u[i];
    for (int j = i + 1; j < 3; j++) {
      T[i + 3 * j] = -u[i] * u[j];
      T[j + 3 * i] = T[i + 3 * j];
    }
  }
  for (int k = 0; k < 9; k++) T[k] = T[k] / nrm;
}

static void gemv3(const double *T, const double *x, double *y) {
  /* reference BLAS dgemv 'N': column-wise accumulation */
  y[0] = y[1] = y[2] = 0.0;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) y[i] = y[i] + x[j] * T[i + 3 * j];
}

static void gfunc_grad(const orc_gfunc *gf, const double *ci, double atomId, const glist *l1,
                       const glist *l2, double *grad /* 3*n1 */) {
  int n1 = l1->n, n2 = l2->n;
  double rcut = gf->rcut, eta = gf->eta, lam = gf->lambda, xi = gf->xi;
  for (int k = 0; k < 3 * n1; k++) grad[k] = 0.0;
  if (gf->type <= 3) {
    for (int j = 0; j < n1; j++) {
      double r = l1->dist[j];
      double f;
      if (gf->type == 1) {
        f = dfcutoff_wo(r, atomId, l1->ids[j], rcut);
      } else if (gf->type == 2) {
        f = (dfcutoff_wo(r, atomId, l1->ids[j], rcut) -
             cutoff_wo(r, atomId, l1->ids[j], rcut) * 2.0 * eta * (r - gf->rs)) *
            exp(-(eta * ((r - gf->rs) * (r - gf->rs))));
      } else {
        f = (cos(gf->kappa * r) * dfcutoff_wo(r, atomId, l1->ids[j], rcut) -
             sin(gf->kappa * r) * cutoff_wo(r, atomId, l1->ids[j], rcut) * gf->kappa);
      }
      for (int c = 0; c < 3; c++) grad[3 * j + c] = f * (l1->crd[3 * j + c] - ci[c]) / r;
    }
    return;
  }
  double *u2 = (double *)malloc((3 * (size_t)n2 + 3) * sizeof(double));
  double *sq2 = (double *)malloc(((size_t)n2 + 1) * sizeof(double));
  double *fc2 = (double *)malloc(((size_t)n2 + 1) * sizeof(double));
  for (int j = 0; j < n2; j++) {
    for (int c = 0; c < 3; c++) u2[3 * j + c] = (l2->crd[3 * j + c] - ci[c]) / l2->dist[j];
    sq2[j] = l2->dist[j] * l2->dist[j];
    fc2[j] = 0.0;
    if (l2->dist[j] > rcut) continue;
    fc2[j] = cutoff_wo(l2->dist[j], atomId, l2->ids[j], rcut);
  }
  double T[9], tmp[3];
  if (gf->z1 == gf->z2) {
    for (int k = 0; k < n1; k++) {
      t_matr(u2 + 3 * k, l1->dist[k], T);
      for (int q = 0; q < 9; q++) T[q] = T[q] * lam * xi;
      double dfc_ik = -2.0 * eta * l1->dist[k] * fc2[k] +
                      dfcutoff_wo(l1->dist[k], atomId, l1->ids[k], rcut);
      double pref = 1.0;
      if (gf->type == 4) pref = l1->ids[k] * l2->ids[k];
      double f0 = pow(1.0 + lam, xi) * fc2[k] * dfc_ik * exp(-(2.0 * eta * sq2[k]));
      for (int c = 0; c < 3; c++) grad[3 * k + c] = grad[3 * k + c] + f0 * u2[3 * k + c] * pref;
      for (int j = 0; j < n2; j++) {
        if (j == k) continue;
        const double *uj = u2 + 3 * j, *uk = u2 + 3 * k;
        double dot = uj[0] * uk[0];
        dot = dot + uj[1] * uk[1];
        dot = dot + uj[2] * uk[2];
        double a = 1.0 + lam * dot;
        if (gf->type == 5) {
          gemv3(T, uj, tmp);
          double f = fc2[j] * exp(-(eta * (sq2[k] + sq2[j]))) * pow(a, xi - 1.0);
          for (int c = 0; c < 3; c++)
            grad[3 * k + c] = grad[3 * k + c] + f * (fc2[k] * tmp[c] + a * dfc_ik * uk[c]);
          continue;
        }
        double ujk[3];
        for (int c = 0; c < 3; c++) ujk[c] = l1->crd[3 * k + c] - l2->crd[3 * j + c];
        double djk = norm2v(ujk);
        if (djk > rcut) continue;
        for (int c = 0; c < 3; c++) ujk[c] = ujk[c] / djk;
        double fc_jk = cutoff_wo(djk, l1->ids[k], l2->ids[j], rcut);
        double dfc_jk = -2.0 * eta * djk * fc_jk + dfcutoff_wo(djk, l1->ids[k], l2->ids[j], rcut);
        gemv3(T, uj, tmp);
        double f = fc2[j] * exp(-(eta * (sq2[k] + sq2[j] + djk * djk))) * pow(a, xi - 1.0);
        for (int c = 0; c < 3; c++)
          grad[3 * k + c] = grad[3 * k + c] +
                            f * (fc2[k] * fc_jk * tmp[c] +
                                 a * (fc_jk * dfc_ik * uk[c] + fc2[k] * dfc_jk * ujk[c]));
      }
    }
    double sc = pow(2.0, 2.0 - xi);
    for (int q = 0; q < 3 * n1; q++) grad[q] = grad[q] * sc;
  } else {
    for (int k = 0; k < n1; k++) {
      double rk = l1->dist[k];
      double fc_ik = cutoff_wo(rk, atomId, l1->ids[k], rcut);
      double dfc_ik = -2.0 * eta * rk * fc_ik + dfcutoff_wo(rk, atomId, l1->ids[k], rcut);
      double uik[3];
      for (int c = 0; c < 3; c++) uik[c] = (l1->crd[3 * k + c] - ci[c]) / rk;
      t_matr(uik, rk, T);
      for (int q = 0; q < 9; q++) T[q] = T[q] * lam * xi;
      for (int j = 0; j < n2; j++) {
        const double *uj = u2 + 3 * j;
        double dot = uj[0] * uik[0];
        dot = dot + uj[1] * uik[1];
        dot = dot + uj[2] * uik[2];
        double a = 1.0 + lam * dot;
        if (gf->type == 5) {
          gemv3(T, uj, tmp);
          double f = fc2[j] * exp(-(eta * (rk * rk + sq2[j]))) * pow(a, xi - 1.0);
          for (int c = 0; c < 3; c++)
            grad[3 * k + c] = grad[3 * k + c] + f * (fc_ik * tmp[c] + a * dfc_ik * uik[c]);
          continue;
        }
        double ujk[3];
        for (int c = 0; c < 3; c++) ujk[c] = l1->crd[3 * k + c] - l2->crd[3 * j + c];
        double djk = norm2v(ujk);
        if (djk > rcut) continue;
        for (int c = 0; c < 3; c++) ujk[c] = ujk[c] / djk;
        double fc_jk = cutoff_wo(djk, l1->ids[k], l2->ids[j], rcut);
        double dfc_jk = -2.0 * eta * djk * fc_jk + dfcutoff_wo(djk, l1->ids[k], l2->ids[j], rcut);
        gemv3(T, uj, tmp);
        double f = fc2[j] * exp(-(eta * (rk * rk + sq2[j] + djk * djk))) * pow(a, xi - 1.0);
        for (int c = 0; c < 3; c++)
          grad[3 * k + c] = grad[3 * k + c] +
                            f * (fc_ik * fc_jk * tmp[c] +
                                 a * (fc_jk * dfc_ik * uik[c] + fc_ik * dfc_jk * ujk[c]));
      }
    }
    double sc = pow(2.0, 1.0 - xi);
    for (int q = 0; q < 3 * n1; q++) grad[q] = grad[q] * sc;
  }
  free(u2);
  free(sq2);
  free(fc2);
}

/* iGeoAcsfGrad with the reference's vector-subscript semantics (acsf.F90:918-933):
 * array(:,g,i,idx(:)) = grad (later entries overwrite earlier ones for repeated atoms), then
 * array(:,g,i,i) = -sum(array(:,g,i,idx(:)), dim=2), evaluated after the assignment. */
#define PR(c, g, i, j) prime[(c) + 3 * ((int64_t)(g) + ng * ((int64_t)(i) + (int64_t)N * (j)))]

int orc_acsf_prime_ex(const orc_batch *b, int32_t s, const orc_gfunc *g, int32_t ng,
                      int32_t physical, double *prime) {
  geo_t geo;
  if (geo_of(b, s, &geo)) return -1;
  int N = geo.natom;
  int64_t a0 = b->atom_offsets[s];
  const int32_t *atnum = b->atnum + a0;
  const double *ext = b->ext ? b->ext + a0 * b->next : NULL;
  memset(prime, 0, sizeof(double) * 3 * (size_t)ng * N * N);
  gwork w;
  memset(&w, 0, sizeof(w));
  w.sel = (int32_t *)malloc((N + 1) * sizeof(int32_t));
  double *grad = NULL;
  int64_t gcap = 0;
  for (int i = 0; i < N; i++) {
    const double *ci = geo.coords + 3 * i;
    for (int k = 0; k < ng; k++) {
      const orc_gfunc *gf = &g[k];
      gctx c;
      build_glists(&geo, atnum, ext, b->next, i, gf, 0, 0.0, &w, &c);
      int64_t need = 3 * (int64_t)((c.l1.n > c.l2.n ? c.l1.n : c.l2.n) + 1);
      if (need > gcap) {
        gcap = need;
        grad = (double *)realloc(grad, gcap * sizeof(double));
      }
      gfunc_grad(gf, ci, c.atomId, &c.l1, &c.l2, grad);
      if (physical) {
        /* every image contributes: dG/dr_j += grad, dG/dr_i -= grad */
        for (int q = 0; q < c.l1.n; q++)
          for (int cc = 0; cc < 3; cc++) {
            PR(cc, k, i, c.l1.idx[q]) += grad[3 * q + cc];
            PR(cc, k, i, i) -= grad[3 * q + cc];
          }
        if (gf->type >= 4 && gf->z1 != gf->z2) {
          glist s1 = c.l2, s2 = c.l1;
          gfunc_grad(gf, ci, c.atomId, &s1, &s2, grad);
          for (int q = 0; q < s1.n; q++)
            for (int cc = 0; cc < 3; cc++) {
              PR(cc, k, i, s1.idx[q]) += grad[3 * q + cc];
              PR(cc, k, i, i) -= grad[3 * q + cc];
            }
        }
        continue;
      }
      for (int q = 0; q < c.l1.n; q++)
        for (int cc = 0; cc < 3; cc++) PR(cc, k, i, c.l1.idx[q]) = grad[3 * q + cc];
      double sum[3] = {0.0, 0.0, 0.0};
      for (int q = 0; q < c.l1.n; q++)
        for (int cc = 0; cc < 3; cc++) sum[cc] = sum[cc] + PR(cc, k, i, c.l1.idx[q]);
      for (int cc = 0; cc < 3; cc++) PR(cc, k, i, i) = -sum[cc];
      if (gf->type >= 4 && gf->z1 != gf->z2) {
        /* Z1 <-> Z2: the swapped call sees list 2 first */
        glist s1 = c.l2, s2 = c.l1;
        /* the swapped lists are backed by the same buffers; copy before reuse */
        gfunc_grad(gf, ci, c.atomId, &s1, &s2, grad);
        for (int q = 0; q < s1.n; q++)
          for (int cc = 0; cc < 3; cc++) PR(cc, k, i, s1.idx[q]) = grad[3 * q + cc];
        double sm[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < s1.n; q++)
          for (int cc = 0; cc < 3; cc++) sm[cc] = sm[cc] + PR(cc, k, i, s1.idx[q]);
        for (int cc = 0; cc < 3; cc++) PR(cc, k, i, i) = PR(cc, k, i, i) - sm[cc];
      }
    }
  }
  free(grad);
  gwork_free(&w);
  return 0;
}

int orc_acsf_prime(const orc_batch *b, int32_t s, const orc_gfunc *g, int32_t ng, double *prime) {
  return orc_acsf_prime_ex(b, s, g, ng, 0, prime);
}

/* ====================================================================================
 * z-score (acsf.F90:445-536)
 * ==================================================================================== */
void orc_zscore_stats(const double *vals, int64_t ntot, int32_t ng, const int64_t *off,
                      int32_t nstruct, const int32_t *weights, double *zprec) {
  (void)ntot;
  for (int k = 0; k < 2 * ng; k++) zprec[k] = 0.0;
  int64_t ntotw = 0;
  for (int s = 0; s < nstruct; s++)
    for (int64_t a = off[s]; a < off[s + 1]; a++) {
      ntotw += weights[s];
      for (int k = 0; k < ng; k++) zprec[k] = zprec[k] + (double)weights[s] * vals[a * ng + k];
    }
  for (int k = 0; k < ng; k++) zprec[k] = zprec[k] / (double)ntotw;
  for (int s = 0; s < nstruct; s++)
    for (int64_t a = off[s]; a < off[s + 1]; a++)
      for (int k = 0; k < ng; k++) {
        double d = vals[a * ng + k] - zprec[k];
        zprec[ng + k] = zprec[ng + k] + (double)weights[s] * (d * d);
      }
  for (int k = 0; k < ng; k++) zprec[ng + k] = sqrt(zprec[ng + k] / (double)ntotw);
}

void orc_zscore_apply(double *vals, int64_t ntot, int32_t ng, const double *zprec) {
  for (int k = 0; k < ng; k++) {
    if (zprec[ng + k] < 1e-08) continue;
    for (int64_t a = 0; a < ntot; a++) vals[a * ng + k] = (vals[a * ng + k] - zprec[k]) / zprec[ng + k];
  }
}

/* ====================================================================================
 * Transfer functions (lib_nn/transfer.F90:53-342)
 * ==================================================================================== */
static double act_f(int t, double x) {
  switch (t) {
    case ORC_ACT_TANH: return tanh(x);
    case ORC_ACT_SIGMOID: return 1.0 / (1.0 + exp(-x));
    case ORC_ACT_RELU: return x > 0.0 ? x : 0.0;
    case ORC_ACT_LRELU: return (0.01 * x > x) ? 0.01 * x : x;
    case ORC_ACT_SOFTPLUS: return log(1.0 + exp(x));
    case ORC_ACT_BENT: return (sqrt(x * x + 1.0) - 1.0) / 2.0 + x;
    case ORC_ACT_ATAN: return atan(x);
    case ORC_ACT_GAUSSIAN: return exp(-(x * x));
    case ORC_ACT_HEAVISIDE: return x > 0.0 ? 1.0 : 0.0;
    default: return x;
  }
}
static double act_d(int t, double x) {
  switch (t) {
    case ORC_ACT_TANH: { double th = tanh(x); return 1.0 - th * th; }
    case ORC_ACT_SIGMOID: { double sg = 1.0 / (1.0 + exp(-x)); return sg * (1.0 - sg); }
    case ORC_ACT_RELU: return x >= 0.0 ? 1.0 : 0.0;
    case ORC_ACT_LRELU: return x >= 0.0 ? 1.0 : 0.01;
    case ORC_ACT_SOFTPLUS: return 1.0 / (1.0 + exp(-x));
    case ORC_ACT_BENT: return x / (2.0 * sqrt(x * x + 1.0)) + 1.0;
    case ORC_ACT_ATAN: return 1.0 / (x * x + 1.0);
    case ORC_ACT_GAUSSIAN: return -2.0 * x * exp(-(x * x));
    case ORC_ACT_HEAVISIDE: return 0.0;
    default: return 1.0;
  }
}

/* ---- one atom through one sub-network: TNetwork_fprop (network.F90:146-180) ---- */
typedef struct {
  double *aa[64], *aarg[64];
} netstate;

static void fprop(const orc_net *net, const double *p, const int64_t *woff, const int64_t *boff,
                  const double *x, netstate *st) {
  int L = net->nlayer;
  for (int i = 0; i < net->dims[0]; i++) st->aa[0][i] = x[i];
  for (int l = 1; l < L; l++) {
    int din = net->dims[l - 1], dout = net->dims[l];
    const double *W = p + woff[l - 1]; /* ww(din, dout) column-major */
    int act = (l == L - 1) ? ORC_ACT_LINEAR : net->activation;
    for (int o = 0; o < dout; o++) {
      double t = 0.0;
      /* gemv with transpose(ww): y(o) = sum_j ww(j,o) * a(j), accumulated over j */
      for (int j = 0; j < din; j++) t = t + st->aa[l - 1][j] * W[j + (int64_t)din * o];
      st->aarg[l][o] = t + p[boff[l] + o];
      st->aa[l][o] = act_f(act, st->aarg[l][o]);
    }
  }
}

static void netstate_alloc(const orc_net *net, netstate *st) {
  for (int l = 0; l < net->nlayer; l++) {
    st->aa[l] = (double *)calloc(net->dims[l], sizeof(double));
    st->aarg[l] = (double *)calloc(net->dims[l], sizeof(double));
  }
}
static void netstate_free(const orc_net *net, netstate *st) {
  for (int l = 0; l < net->nlayer; l++) { free(st->aa[l]); free(st->aarg[l]); }
}

void orc_predict(const orc_net *net, const double *params, int32_t nf, const double *feats,
                 int64_t ntot, const int32_t *species, double *out) {
  int64_t woff[64], boff[64], np;
  layout(net, woff, boff, &np);
  int L = net->nlayer, nout = net->dims[L - 1];
  netstate st;
  netstate_alloc(net, &st);
  for (int64_t a = 0; a < ntot; a++) {
    fprop(net, params + species[a] * np, woff, boff, feats + a * nf, &st);
    for (int o = 0; o < nout; o++) out[a * nout + o] = st.aa[L - 1][o];
  }
  netstate_free(net, &st);
}

/* TNetwork_fdevi (network.F90:183-244): forward-mode Jacobian with diagonal matrices. */
void orc_jacobian(const orc_net *net, const double *params, int32_t nf, const double *feats,
                  int64_t ntot, const int32_t *species, double *jac) {
  int64_t woff[64], boff[64], np;
  layout(net, woff, boff, &np);
  int L = net->nlayer, nout = net->dims[L - 1];
  int dmax = 0;
  for (int l = 0; l < L; l++) dmax = net->dims[l] > dmax ? net->dims[l] : dmax;
  double *J = (double *)malloc(sizeof(double) * dmax * nf);
  double *T = (double *)malloc(sizeof(double) * dmax * nf);
  double *a = (double *)malloc(sizeof(double) * dmax);
  double *z = (double *)malloc(sizeof(double) * dmax);
  for (int64_t at = 0; at < ntot; at++) {
    const double *p = params + species[at] * np;
    int d = nf;
    for (int i = 0; i < nf; i++) a[i] = feats[at * nf + i];
    for (int q = 0; q < nf * nf; q++) J[q] = 0.0;
    for (int i = 0; i < nf; i++) J[i + nf * i] = 1.0;
    for (int l = 1; l < L; l++) {
      int din = net->dims[l - 1], dout = net->dims[l];
      const double *W = p + woff[l - 1];
      int act = (l == L - 1) ? ORC_ACT_LINEAR : net->activation;
      for (int o = 0; o < dout; o++) {
        double t = 0.0;
        for (int j = 0; j < din; j++) t = t + a[j] * W[j + (int64_t)din * o];
        z[o] = t + p[boff[l] + o];
      }
      /* tmpMat = transpose(ww) * jacobi ; jacobi = diag(f'(z)) * tmpMat */
      for (int o = 0; o < dout; o++)
        for (int f = 0; f < nf; f++) {
          double t = 0.0;
          for (int j = 0; j < din; j++) t = t + W[j + (int64_t)din * o] * J[j + (int64_t)d * f];
          T[o + (int64_t)dout * f] = t;
        }
      for (int o = 0; o < dout; o++) {
        double dv = act_d(act, z[o]);
        for (int f = 0; f < nf; f++) J[o + (int64_t)dout * f] = dv * T[o + (int64_t)dout * f];
        a[o] = act_f(act, z[o]);
      }
      d = dout;
    }
    for (int o = 0; o < nout; o++)
      for (int f = 0; f < nf; f++) jac[at * nout * nf + o + (int64_t)nout * f] = J[o + (int64_t)nout * f];
  }
  free(J); free(T); free(a); free(z);
}

/* ====================================================================================
 * Training gradients: sysTrain (bpnn.F90:610-704) + bprop (network.F90:248-296),
 * accumulated like updateGradients (bpnn.F90:394-481).
 * ==================================================================================== */
static double lossgrad(int loss, double p, double t) {
  switch (loss) {
    case ORC_LOSS_RMS: return (p - t) / sqrt((p - t) * (p - t));
    case ORC_LOSS_MAE: return (p - t) / fabs(p - t);
    case ORC_LOSS_MAPE: return 100.0 * (p - t) / (t * t * fabs(p / t - 1.0));
    default: return 2.0 * (p - t);
  }
}

int orc_train_gradients(const orc_net *net, const double *params, int32_t nspecies, int32_t nf,
                        const double *feats, const int32_t *species, int32_t nstruct,
                        const int64_t *off, int32_t ngt, int32_t nat, const double *gt,
                        const double *at, const double *atomic_w, const int32_t *weights,
                        const int32_t *order, int32_t loss, double *dd, double *predicts) {
  int64_t woff[64], boff[64], np;
  layout(net, woff, boff, &np);
  int L = net->nlayer, nout = net->dims[L - 1];
  if (nout != ngt + nat) return -1;
  memset(dd, 0, sizeof(double) * np * nspecies);
  double *ddsys = (double *)calloc(np * nspecies, sizeof(double));
  double *db = (double *)calloc(np, sizeof(double)); /* per-atom gradient in param layout */
  int nmax = 0;
  for (int s = 0; s < nstruct; s++) {
    int n = (int)(off[s + 1] - off[s]);
    nmax = n > nmax ? n : nmax;
  }
  netstate *st = (netstate *)calloc(nmax > 0 ? nmax : 1, sizeof(netstate));
  for (int a = 0; a < nmax; a++) netstate_alloc(net, &st[a]);
  double *lg = (double *)calloc((size_t)(nmax > 0 ? nmax : 1) * nout, sizeof(double));
  double *gp = (double *)calloc(nout + 1, sizeof(double));
  int dmax = 0;
  for (int l = 0; l < L; l++) dmax = net->dims[l] > dmax ? net->dims[l] : dmax;
  double *delta = (double *)calloc(dmax, sizeof(double));
  double *dnext = (double *)calloc(dmax, sizeof(double));
  for (int ii = 0; ii < nstruct; ii++) {
    int s = order[ii] - 1;
    int64_t a0 = off[s];
    int n = (int)(off[s + 1] - a0);
    memset(ddsys, 0, sizeof(double) * np * nspecies);
    for (int a = 0; a < n; a++) {
      fprop(net, params + species[a0 + a] * np, woff, boff, feats + (a0 + a) * nf, &st[a]);
      for (int o = 0; o < nout; o++) predicts[(a0 + a) * nout + o] = st[a].aa[L - 1][o];
    }
    if (ngt > 0) {
      for (int t = 0; t < ngt; t++) {
        double sum = 0.0;
        for (int a = 0; a < n; a++) sum = sum + predicts[(a0 + a) * nout + t];
        gp[t] = lossgrad(loss, sum, gt[(int64_t)s * ngt + t]);
      }
      for (int a = 0; a < n; a++)
        for (int t = 0; t < ngt; t++) lg[a * nout + t] = gp[t];
    }
    if (nat > 0)
      for (int a = 0; a < n; a++)
        for (int t = 0; t < nat; t++)
          lg[a * nout + ngt + t] =
              lossgrad(loss, predicts[(a0 + a) * nout + ngt + t], at[(a0 + a) * nat + t]);
    for (int a = 0; a < n; a++) {
      int sp = species[a0 + a];
      const double *p = params + sp * np;
      memset(db, 0, sizeof(double) * np);
      /* db(L) = lossgrad * f'_L(aarg_L), output layer linear */
      for (int o = 0; o < nout; o++) delta[o] = lg[a * nout + o] * 1.0;
      for (int o = 0; o < nout; o++) db[boff[L - 1] + o] = delta[o];
      for (int l = L - 1; l >= 1; l--) {
        int din = net->dims[l - 1], dout = net->dims[l];
        /* dw(l-1) = aa(l-1) x db(l)  (rank-1 gemm) */
        for (int o = 0; o < dout; o++)
          for (int j = 0; j < din; j++) db[woff[l - 1] + j + (int64_t)din * o] = st[a].aa[l - 1][j] * delta[o];
        if (l - 1 >= 1) {
          const double *W = p + woff[l - 1];
          for (int j = 0; j < din; j++) dnext[j] = 0.0;
          /* gemv(tmpVec, ww(l-1), db(l)) : column-wise accumulation */
          for (int o = 0; o < dout; o++)
            for (int j = 0; j < din; j++) dnext[j] = dnext[j] + delta[o] * W[j + (int64_t)din * o];
          for (int j = 0; j < din; j++) {
            dnext[j] = dnext[j] * act_d(net->activation, st[a].aarg[l - 1][j]);
            db[boff[l - 1] + j] = dnext[j];
          }
          for (int j = 0; j < din; j++) delta[j] = dnext[j];
        }
      }
      double *dst = ddsys + (int64_t)sp * np;
      for (int64_t q = 0; q < np; q++) dst[q] = dst[q] + db[q] * atomic_w[a0 + a] / (double)n;
    }
    double w = (double)weights[s];
    for (int64_t q = 0; q < np * nspecies; q++) dd[q] = dd[q] + ddsys[q] * w;
  }
  for (int a = 0; a < nmax; a++) netstate_free(net, &st[a]);
  free(st); free(lg); free(gp); free(delta); free(dnext); free(ddsys); free(db);
  return 0;
}

double orc_update_prepare(const orc_net *net, const double *params, int32_t nspecies,
                          double *grad, double lam, double alpha, double sum_weights) {
  int64_t woff[64], boff[64], np;
  layout(net, woff, boff, &np);
  int64_t nweights = boff[0]; /* weights precede biases in the layout */
  for (int s = 0; s < nspecies; s++) {
    const double *p = params + s * np;
    double *g = grad + s * np;
    for (int64_t q = 0; q < nweights; q++) {
      double ww = p[q];
      double sgn = ww == 0.0 ? 0.0 : (ww > 0.0 ? 1.0 : -1.0);
      g[q] = g[q] + lam / (double)nweights * ((1.0 - alpha) * ww + alpha * sgn);
    }
  }
  double ss = 0.0;
  for (int64_t q = 0; q < np * nspecies; q++) {
    grad[q] = grad[q] / sum_weights;
    ss = ss + grad[q] * grad[q];
  }
  return sqrt(ss);
}

/* ====================================================================================
 * Forces: forceAnalysis_analytical (forces.F90:317-425) on the dense dG/dR of
 * iGeoAcsfGrad, z-scored like applyZscorePrime (acsf.F90:515-536).
 * ==================================================================================== */
typedef struct {
  const orc_batch *b;
  const orc_gfunc *g;
  int ng;
  const double *zprec;
  int nout;
  const double *jac;
  int physical;
  double *forces;
} fjob;

static int forces_struct(void *vctx, int s, void *scratch) {
  (void)scratch;
  fjob *J = (fjob *)vctx;
  const orc_batch *b = J->b;
  const int ng = J->ng, nout = J->nout;
  int64_t a0 = b->atom_offsets[s];
  int N = (int)(b->atom_offsets[s + 1] - a0);
  double *prime = (double *)malloc(sizeof(double) * 3 * (size_t)ng * N * N + 8);
  if (orc_acsf_prime_ex(b, s, J->g, ng, J->physical, prime)) {
    free(prime);
    return -1;
  }
  if (J->zprec)
    for (int k = 0; k < ng; k++) {
      if (J->zprec[ng + k] < 1e-08) continue;
      for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
          for (int c = 0; c < 3; c++) PR(c, k, i, j) = PR(c, k, i, j) / J->zprec[ng + k];
    }
  double *forces = J->forces;
  for (int q = 0; q < N * 3 * nout; q++) forces[a0 * 3 * nout + q] = 0.0;
  for (int fa = 0; fa < N; fa++)
    for (int i = 0; i < N; i++)
      for (int k = 0; k < ng; k++)
        for (int c = 0; c < 3; c++)
          for (int o = 0; o < nout; o++) {
            double *F = forces + (a0 + fa) * 3 * nout;
            F[c + 3 * o] = F[c + 3 * o] - J->jac[(a0 + i) * nout * ng + o + (int64_t)nout * k] * PR(c, k, i, fa);
          }
  free(prime);
  return 0;
}

int orc_forces_mt(const orc_batch *b, const orc_gfunc *g, int32_t ng, const double *zprec,
                  int32_t nout, const double *jac, int32_t physical, double *forces,
                  int32_t nthreads) {
  fjob J = {b, g, ng, zprec, nout, jac, physical, forces};
  return run_blocks(b->nstruct, nthreads, &J, forces_struct, 8, NULL);
}

int orc_forces_ex(const orc_batch *b, const orc_gfunc *g, int32_t ng, const double *zprec,
                  int32_t nout, const double *jac, int32_t physical, double *forces) {
  return orc_forces_mt(b, g, ng, zprec, nout, jac, physical, forces, 1);
}
#undef PR

int orc_forces(const orc_batch *b, const orc_gfunc *g, int32_t ng, const double *zprec,
               int32_t nout, const double *jac, double *forces) {
  return orc_forces_ex(b, g, ng, zprec, nout, jac, 0, forces);
}

/* ====================================================================================
 * Optimisers
 * ==================================================================================== */
typedef struct {
  int kind; /* 0 = SD, 1 = L-BFGS */
  int n;
  /* SD */
  double *xold, tol, maxdisp, lr;
  int converged;
  /* L-BFGS */
  double *xx, *gg, *ss, *yy, *rho, *dir;
  int mem, iter, linesearch;
  double qn_maxdisp, alpha;
  /* line minimiser (linemin.F90) */
  int lm_state, lm_miter, lm_iiter, lm_conv;
  double *lm_x0, *lm_d0, lm_xx[2], lm_dx[2], lm_xcur, lm_tol, lm_maxdisp, lm_maxx, lm_first;
} opt_t;

void *orc_sd_new(int32_t n, double tol, double maxdisp, double lr, const double *x0) {
  opt_t *o = (opt_t *)calloc(1, sizeof(opt_t));
  o->kind = 0;
  o->n = n;
  o->tol = tol;
  o->maxdisp = maxdisp;
  o->lr = lr;
  o->xold = (double *)malloc(sizeof(double) * n);
  memcpy(o->xold, x0, sizeof(double) * n);
  return o;
}

/* SteepDesc_next / next_local (steepdesc.F90:126-204) */
int orc_sd_next(void *h, const double *grad, double *xnew) {
  opt_t *o = (opt_t *)h;
  int n = o->n;
  if (o->converged) {
    memcpy(xnew, o->xold, sizeof(double) * n);
    return 1;
  }
  double gmax = 0.0;
  for (int i = 0; i < n; i++) gmax = fabs(grad[i]) > gmax ? fabs(grad[i]) : gmax;
  if (gmax < o->tol) {
    o->converged = 1;
    memcpy(xnew, o->xold, sizeof(double) * n);
    return 1;
  }
  double maxx = 0.0;
  for (int i = 0; i < n; i++) {
    xnew[i] = -1.0 * o->lr * grad[i];
    maxx = fabs(xnew[i]) > maxx ? fabs(xnew[i]) : maxx;
  }
  if (maxx <= o->maxdisp) {
    for (int i = 0; i < n; i++) xnew[i] = o->xold[i] + xnew[i];
  } else {
    for (int i = 0; i < n; i++) xnew[i] = o->xold[i] + (o->maxdisp / maxx) * xnew[i];
  }
  memcpy(o->xold, xnew, sizeof(double) * n);
  return 0;
}

void *orc_lbfgs_new(int32_t n, double tol, double mindisp, double maxdisp, int32_t mem,
                    int32_t linesearch, int32_t qndisp, const double *x0) {
  (void)mindisp;
  opt_t *o = (opt_t *)calloc(1, sizeof(opt_t));
  o->kind = 1;
  o->n = n;
  o->tol = tol;
  o->mem = mem;
  o->xx = (double *)calloc(n, sizeof(double));
  o->xold = (double *)calloc(n, sizeof(double));
  o->gg = (double *)calloc(n, sizeof(double));
  o->ss = (double *)calloc((size_t)n * mem, sizeof(double));
  o->yy = (double *)calloc((size_t)n * mem, sizeof(double));
  o->rho = (double *)calloc(mem, sizeof(double));
  o->dir = (double *)calloc(n, sizeof(double));
  o->linesearch = linesearch;
  o->qn_maxdisp = -1.0;
  if (linesearch) {
    o->lm_x0 = (double *)calloc(n, sizeof(double));
    o->lm_d0 = (double *)calloc(n, sizeof(double));
    o->lm_miter = 10;
    o->lm_tol = tol;
    o->lm_maxdisp = maxdisp;
  } else if (qndisp) {
    o->qn_maxdisp = maxdisp;
  }
  /* TLbfgs_reset (lbfgs.F90:368-383) */
  o->alpha = 1.0;
  memcpy(o->xx, x0, sizeof(double) * n);
  memcpy(o->xold, x0, sizeof(double) * n);
  o->iter = 0;
  return o;
}

static double dotn(const double *a, const double *b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + a[i] * b[i];
  return s;
}

/* TLbfgs_calcDirection (lbfgs.F90:387-488) */
static void lbfgs_direction(opt_t *o, const double *xx, const double *gg) {
  int n = o->n, mem = o->mem;
  if (o->iter == 0) {
    memcpy(o->gg, gg, sizeof(double) * n);
    for (int i = 0; i < n; i++) o->dir[i] = -gg[i];
    o->iter = o->iter + 1;
    return;
  }
  int ne = ((o->iter - 1) % mem); /* 0-based newElem */
  double *s = o->ss + (size_t)n * ne, *y = o->yy + (size_t)n * ne;
  for (int i = 0; i < n; i++) {
    s[i] = xx[i] - o->xold[i];
    y[i] = gg[i] - o->gg[i];
  }
  double beta = dotn(y, s, n);
  o->rho[ne] = 1.0 / (fabs(beta) > DP_EPS ? fabs(beta) : DP_EPS);
  memcpy(o->xold, xx, sizeof(double) * n);
  memcpy(o->gg, gg, sizeof(double) * n);
  double diag;
  if (o->iter == 1) {
    diag = 1.0;
  } else {
    double yy2 = dotn(y, y, n);
    diag = dotn(s, y, n) / (yy2 > DP_EPS ? yy2 : DP_EPS);
  }
  double *qq = (double *)malloc(sizeof(double) * n);
  double *al = (double *)calloc(mem, sizeof(double));
  memcpy(qq, gg, sizeof(double) * n);
  for (int m = 0; m < mem; m++) {
    int ii = (((ne + 1) - m - 1) % mem + mem) % mem;
    al[ii] = o->rho[ii] * dotn(o->ss + (size_t)n * ii, qq, n);
    for (int i = 0; i < n; i++) qq[i] = qq[i] - al[ii] * o->yy[(size_t)n * ii + i];
  }
  for (int i = 0; i < n; i++) o->dir[i] = diag * qq[i];
  int oldest = ((ne + 1) % mem); /* 0-based */
  for (int m = 0; m < mem; m++) {
    int ii = (oldest + m) % mem;
    double b = o->rho[ii] * dotn(o->yy + (size_t)n * ii, o->dir, n);
    for (int i = 0; i < n; i++) o->dir[i] = o->dir[i] + o->ss[(size_t)n * ii + i] * (al[ii] - b);
  }
  o->iter = o->iter + 1;
  for (int i = 0; i < n; i++) o->dir[i] = -o->dir[i];
  free(qq);
  free(al);
}

/* TLineMin reset / next_local (linemin.F90:141-391) */
static void lm_reset(opt_t *o, const double *x0, const double *d0, double first) {
  int n = o->n;
  o->lm_state = 1;
  o->lm_iiter = 0;
  o->lm_xx[0] = o->lm_xx[1] = 0.0;
  o->lm_dx[0] = o->lm_dx[1] = 0.0;
  memcpy(o->lm_x0, x0, sizeof(double) * n);
  double tmp = sqrt(dotn(d0, d0, n));
  double dmax = 0.0;
  for (int i = 0; i < n; i++) {
    o->lm_d0[i] = d0[i] / tmp;
    dmax = fabs(o->lm_d0[i]) > dmax ? fabs(o->lm_d0[i]) : dmax;
  }
  o->lm_xcur = 0.0;
  o->lm_first = first;
  o->lm_maxx = o->lm_maxdisp / dmax;
  o->lm_conv = 0;
}

static int lm_next(opt_t *o, double fu, const double *du, double *uu) {
  int n = o->n;
  if (o->lm_conv) {
    memcpy(uu, o->lm_x0, sizeof(double) * n);
    return 1;
  }
  double *x0 = o->lm_x0, *d0 = o->lm_d0, *xx = o->lm_xx, *dx = o->lm_dx;
  double xnew = 0.0, tmp, qq, aa, bb, cc;
  int next_state = o->lm_state, done;
  o->lm_iiter = o->lm_iiter + 1;
  double dcur = dotn(du, d0, n);
  if ((fabs(dcur) < o->lm_tol && o->lm_state == 3) || o->lm_iiter > o->lm_miter) {
    for (int i = 0; i < n; i++) x0[i] = x0[i] + o->lm_xcur * d0[i];
    memcpy(d0, du, sizeof(double) * n);
    memcpy(uu, x0, sizeof(double) * n);
    xx[0] = fu;
    xx[1] = o->lm_xcur;
    o->lm_conv = 1;
    return 1;
  }
  if (o->lm_state == 1) {
    if (dcur > 0.0) {
      for (int i = 0; i < n; i++) d0[i] = -d0[i];
      dcur = -dcur;
    }
    xx[0] = o->lm_xcur;
    dx[0] = dcur;
    xnew = o->lm_first;
    next_state = 2;
  }
  if (o->lm_state == 2) {
    if (dcur < 0.0) {
      xnew = o->lm_xcur + GOLDEN_MEAN_P1 * (o->lm_xcur - xx[0]);
      xx[0] = o->lm_xcur;
      dx[0] = dcur;
      next_state = 2;
    } else {
      o->lm_state = 3;
    }
  }
  if (o->lm_state == 3) {
    double xcur = o->lm_xcur;
    done = 0;
    next_state = 3;
    if (o->lm_iiter > 2 && fabs(xx[0] - xx[1]) > DP_EPS) {
      qq = (xcur - xx[0]) / (xx[0] - xx[1]);
      tmp = dcur - dx[0];
      cc = qq * qq * (dx[1] - dx[0]);
      aa = qq * tmp + cc;
      bb = 2.0 * qq * tmp + cc + tmp;
      cc = (qq + 1.0) * dcur;
      tmp = bb * bb - 4 * aa * cc;
      if (tmp >= 0.0) {
        tmp = sqrt(tmp);
        if (bb > 0.0) aa = bb + tmp;
        else aa = bb - tmp;
        if (fabs(aa) > DP_EPS) {
          xnew = xcur - (xcur - xx[0]) * 2.0 * cc / aa;
          if (((xx[0] < xnew) == (xnew < xx[1])) && ((dcur < 0.0) == (xnew > xcur))) {
            if (xnew > xcur) {
              xx[0] = xcur;
              dx[0] = dcur;
            } else {
              xx[1] = xcur;
              dx[1] = dcur;
            }
            done = 1;
          }
        }
      }
    }
    if (!done) {
      if (dcur < 0.0) {
        xx[0] = xcur;
        dx[0] = dcur;
      } else {
        xx[1] = xcur;
        dx[1] = dcur;
      }
      tmp = dx[0] - dx[1];
      if (fabs(tmp) > DP_EPS) {
        xnew = (xx[1] * dx[0] - xx[0] * dx[1]) / tmp;
        if ((xx[0] < xnew) == (xnew < xx[1])) done = 1;
      }
    }
    if (!done) xnew = 0.5 * (xx[0] + xx[1]);
  }
  tmp = xnew - o->lm_xcur;
  if (fabs(tmp) <= o->lm_maxx) o->lm_xcur = xnew;
  else o->lm_xcur = o->lm_xcur + copysign(o->lm_maxx, tmp);
  for (int i = 0; i < n; i++) uu[i] = x0[i] + o->lm_xcur * d0[i];
  o->lm_state = next_state;
  return 0;
}

/* TLbfgs_next (lbfgs.F90:283-359) */
int orc_lbfgs_next(void *h, double fx, const double *dx, double *xnew) {
  opt_t *o = (opt_t *)h;
  int n = o->n;
  double gmax = 0.0;
  for (int i = 0; i < n; i++) gmax = fabs(dx[i]) > gmax ? fabs(dx[i]) : gmax;
  if (gmax < o->tol) {
    memcpy(xnew, o->xx, sizeof(double) * n);
    return 1;
  }
  double *dxt = (double *)malloc(sizeof(double) * n);
  memcpy(dxt, dx, sizeof(double) * n);
  if (o->linesearch && o->iter > 0) {
    int lconv = lm_next(o, fx, dx, o->xx);
    if (lconv) {
      memcpy(dxt, o->lm_d0, sizeof(double) * n);
    } else {
      memcpy(xnew, o->xx, sizeof(double) * n);
      free(dxt);
      return 0;
    }
  }
  lbfgs_direction(o, o->xx, dxt);
  if (o->linesearch) {
    o->alpha = 1.0;
    lm_reset(o, o->xx, o->dir, o->alpha);
    lm_next(o, fx, dx, o->xx);
  } else {
    if (o->qn_maxdisp > 0.0) {
      double dmax = 0.0;
      for (int i = 0; i < n; i++) dmax = fabs(o->dir[i]) > dmax ? fabs(o->dir[i]) : dmax;
      if (dmax > o->qn_maxdisp)
        for (int i = 0; i < n; i++) o->dir[i] = o->dir[i] * o->qn_maxdisp / dmax;
    }
    for (int i = 0; i < n; i++) o->xx[i] = o->xx[i] + o->dir[i];
  }
  memcpy(xnew, o->xx, sizeof(double) * n);
  free(dxt);
  return 0;
}

/* ---- conjugate gradients (conjgrad.F90:121-260): Polak-Ribiere directions with the line
 * minimiser of linemin.F90 (10 evaluations per line, tolerance 1e4) ---------------------- */
void *orc_cg_new(int32_t n, double tol, double maxdisp, const double *x0) {
  opt_t *o = (opt_t *)calloc(1, sizeof(opt_t));
  o->kind = 2;
  o->n = n;
  o->tol = tol;
  o->gg = (double *)calloc(n, sizeof(double));  /* gg */
  o->dir = (double *)calloc(n, sizeof(double)); /* hh */
  o->xx = (double *)calloc(n, sizeof(double));  /* uu */
  o->lm_x0 = (double *)calloc(n, sizeof(double));
  o->lm_d0 = (double *)calloc(n, sizeof(double));
  o->lm_miter = 10;
  o->lm_tol = 10000.0;
  o->lm_maxdisp = maxdisp;
  memcpy(o->xx, x0, sizeof(double) * n); /* conjGrad_reset */
  o->iter = 0;                           /* state st_1 */
  o->converged = 0;
  return o;
}

/* conjGrad_next / next_local (conjgrad.F90:142-260) */
int orc_cg_next(void *h, double fu, const double *du, double *xnew) {
  opt_t *o = (opt_t *)h;
  const int n = o->n;
  double *gg = o->gg, *hh = o->dir, *uu = o->xx;
  if (!o->converged) {
    if (o->iter == 0) {
      double gmax = 0.0;
      for (int i = 0; i < n; i++) gmax = fabs(du[i]) > gmax ? fabs(du[i]) : gmax;
      if (gmax < o->tol) {
        o->converged = 1;
        memcpy(gg, du, sizeof(double) * n);
        for (int i = 0; i < n; i++) hh[i] = 0.0;
        hh[0] = fu;
      } else {
        for (int i = 0; i < n; i++) {
          gg[i] = -du[i];
          hh[i] = gg[i];
        }
      }
      lm_reset(o, uu, hh, 5.0 * sqrt(dotn(gg, gg, n)));
      o->iter = 1; /* state st_2 */
    }
    int conv_line = 1;
    while (!o->converged && conv_line) {
      conv_line = lm_next(o, fu, du, uu);
      if (conv_line) {
        const double *xi = o->lm_d0; /* getMinGrad */
        double gmax = 0.0;
        for (int i = 0; i < n; i++) gmax = fabs(xi[i]) > gmax ? fabs(xi[i]) : gmax;
        if (gmax < o->tol) {
          o->converged = 1;
        } else {
          const double gg_abs = dotn(gg, gg, n);
          double dg_abs = 0.0;
          for (int i = 0; i < n; i++) dg_abs = dg_abs + (xi[i] + gg[i]) * xi[i];
          if (gg_abs < DP_EPS) {
            o->converged = 1;
          } else {
            for (int i = 0; i < n; i++) {
              gg[i] = -xi[i];
              hh[i] = gg[i] + (dg_abs / gg_abs) * hh[i];
            }
            memcpy(uu, o->lm_x0, sizeof(double) * n); /* getMinX */
            lm_reset(o, uu, hh, o->lm_xx[1]);          /* getMinLambda */
          }
        }
      }
    }
    if (o->converged) memcpy(uu, o->lm_x0, sizeof(double) * n);
  }
  memcpy(xnew, uu, sizeof(double) * n);
  return o->converged;
}

/* ---- FIRE (fire.F90:90-205) ---------------------------------------------------------- */
void *orc_fire_new(int32_t n, double tol, double maxstep, const double *x0) {
  opt_t *o = (opt_t *)calloc(1, sizeof(opt_t));
  o->kind = 3;
  o->n = n;
  o->tol = tol;
  o->xx = (double *)calloc(n, sizeof(double));   /* x */
  o->dir = (double *)calloc(n, sizeof(double));  /* velocity */
  o->maxdisp = maxstep;                          /* dt_max */
  memcpy(o->xx, x0, sizeof(double) * n);         /* reset */
  o->iter = 0;
  o->mem = 0;                                    /* resetStep */
  o->alpha = 0.1;                                /* a = a_start */
  o->lr = 0.1 * maxstep;                         /* dt = dt_init */
  return o;
}

static double magn(const double *v, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + v[i] * v[i];
  return sqrt(s);
}

int orc_fire_next(void *h, const double *dx, double *xnew) {
  opt_t *o = (opt_t *)h;
  const int n = o->n;
  double *x = o->xx, *v = o->dir;
  int conv;
  double gmax = 0.0;
  for (int i = 0; i < n; i++) gmax = fabs(dx[i]) > gmax ? fabs(dx[i]) : gmax;
  if (gmax < o->tol) {
    conv = 1;
  } else {
    /* fireModifyVelocity */
    const double p = -1.0 * dotn(v, dx, n);
    const double mv = magn(v, n), md = magn(dx, n);
    for (int i = 0; i < n; i++) v[i] = (1.0 - o->alpha) * v[i] - o->alpha * dx[i] * mv / md;
    if (p < 0.0) {
      for (int i = 0; i < n; i++) v[i] = 0.0;
      o->mem = o->iter;
      o->lr = o->lr * 0.5;
      o->alpha = 0.1;
    } else if (o->iter - o->mem > 5) {
      o->lr = o->lr * 1.1 < o->maxdisp ? o->lr * 1.1 : o->maxdisp;
      o->alpha = o->alpha * 0.99;
    }
    for (int i = 0; i < n; i++) v[i] = v[i] - o->lr * dx[i];
    for (int i = 0; i < n; i++) x[i] = x[i] + v[i] * o->lr;
    conv = 0;
  }
  memcpy(xnew, x, sizeof(double) * n);
  o->iter = o->iter + 1;
  return conv;
}

void orc_opt_free(void *h) {
  opt_t *o = (opt_t *)h;
  if (!o) return;
  free(o->xold); free(o->xx); free(o->gg); free(o->ss); free(o->yy); free(o->rho); free(o->dir);
  free(o->lm_x0); free(o->lm_d0);
  free(o);
}
