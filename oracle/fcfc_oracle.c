/*
 * fcfc_oracle.c -- CPU restatement of FCFC's pair-counting hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU engine in
 * fcfc_gb300/: only tests/, the smoke check and the CPU-baseline leg of
 * bench.py load it.  Nothing in the product links or calls it.
 *
 * Parity is pinned: tests/golden/ holds pair-count files written by the
 * upstream FCFC executables (compiled from their own sources by
 * oracle/Makefile.ref) and tests/test_oracle_golden.py checks this file
 * against every one of them, bin for bin.
 *
 * What is restated (file:line in the FCFC v1.0.1 tree):
 *   - rescale factor for linear bins     src/fcfc/2pt_box/setup_cf.c:308-376
 *                                        (least_fac2 / least_fac4)
 *   - integer / hybrid lookup tables     src/util/create_lut.c:58-140
 *   - separation-bin tables              src/fcfc/2pt_box/setup_cf.c:385-430
 *   - (s_perp, pi) tables                src/fcfc/2pt_box/setup_cf.c:439-503,
 *                                        survey squares pi: src/fcfc/2pt/setup_cf.c:455-502
 *   - mu table                           src/fcfc/2pt_box/setup_cf.c:513-531
 *   - coordinate rescale / |x|^2         src/fcfc/2pt_box/build_tree.c:121-131,
 *                                        src/fcfc/2pt/build_tree.c:35-133
 *   - per-pair separation and binning    src/fcfc/2pt_box/metric_common.c:140-235
 *                                        (scalar FP64 build, no FMA contraction),
 *                                        src/fcfc/2pt/metric_common.c:142-260
 *   - hybrid walk-down                   src/fcfc/2pt_box/metric_common.c:56-64
 *   - RA/Dec/z -> comoving coordinates   src/fcfc/2pt/cnvt_coord.c:113-186
 *                                        (redshift samples), :202-250
 *                                        (integrand, Gauss-Legendre sum),
 *                                        :267-307 (order), :321-337
 *                                        (integration), :58-95 (spline
 *                                        lookup), src/math/cspline.c:34-110
 *
 * The dual k-d tree of the reference (src/fcfc/2pt_box/dual_tree.c) only
 * decides which pairs are visited; every visited pair is binned by the
 * per-pair formula above.  Here pairs are visited through a periodic (box) or
 * bounded (survey) cell grid, or by brute force for small inputs.
 *
 * Periodic images.  The reference adds the image shift to the first point of
 * a node pair, (x1 + shift) - x2 (metric_common.c:996-999).  For cross counts
 * the first point is from the first catalogue; for auto counts the node order
 * depends on the tree, so this file fixes it: the point with the smaller
 * input index is the first one.  The two orders can differ only in the last
 * bit of a wrapped separation.
 *
 * Build: gcc -O2 -std=c99 -ffp-contract=off -fopenmp -shared -fPIC
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FCO_BIN_ISO 0
#define FCO_BIN_SMU 1
#define FCO_BIN_SPI 2
#define FCO_TAB_INT 0
#define FCO_TAB_HYBRID 1

#define FCO_LUT_INT_MAX 40960      /* src/fcfc/2pt_box/define.h:79 */
#define FCO_LUT_HYB_MAX 32768      /* define.h:80 */
#define FCO_LUT_HYB_MIN 8192       /* define.h:81 */
#define FCO_MAX_DIGIT 4            /* define.h:84 */
#define FCO_TOL 1e-10              /* DOUBLE_TOL, src/util/define_comm.h:131 */
#define FCO_MAXINT 0x1p+53         /* REAL_MAXINT for double */

typedef struct {
  int survey;          /* 0: periodic box, 1: survey (no wrap) */
  int bintype;
  int ns, np, nmu;
  int tabtype;
  double rescale;
  double *sbin_raw, *pbin_raw;  /* as given (ns+1, np+1) */
  double *sbin, *s2bin;         /* rescaled */
  double *pbin, *p2bin;         /* rescaled; p2bin only for survey */
  uint16_t *stab, *ptab;        /* table entries widened to 16 bits */
  long nstab, nptab;
  long smin_i, pmin_i;          /* (int) of the lower edges, the table offset */
  uint8_t *mutab;
  double bsize[3];              /* rescaled box */
  long ntot;
  int mu_one;                   /* -DWITH_MU_ONE build */
} fco_bins;

/* ------------------------------------------------------------------------ */
/* Rescale factors.                                                          */

static size_t fco_gcd(size_t a, size_t b) {
  while (b) { size_t t = a % b; a = b; b = t; }
  return a;
}

/* The smallest power-of-ten multiple (up to 10^4) that turns every value
 * into an integer, divided by the common divisor of those integers.
 * Returns 0 when no such factor exists.  Follows least_fac2/least_fac4. */
static double fco_least_fac(double *v, int n, int two) {
  for (int k = 0; k < n; k++)
    if (v[k] < 0 || v[k] > FCO_MAXINT) return 0;
  if (two) {
    if (v[0] == 0) return 1 / v[1];
    if (v[1] == 0) return 1 / v[0];
  }
  size_t i = 0, ifac = 1;
  for (;;) {
    int ok = 1;
    for (int k = 0; k < n; k++)
      if (fabs(round(v[k]) - v[k]) >= FCO_TOL) { ok = 0; break; }
    if (ok) break;
    for (int k = 0; k < n; k++) v[k] *= 10;
    ifac *= 10;
    if (++i > FCO_MAX_DIGIT) break;
  }
  if (i == FCO_MAX_DIGIT + 1) return 0;
  for (int k = 0; k < n; k++) if (v[k] > FCO_MAXINT) return 0;
  size_t g = 0;
  if (two) {
    g = fco_gcd((size_t) round(v[0]), (size_t) round(v[1]));
  } else {
    /* least_fac4 rounds the first non-zero value, then takes the gcd with
     * the truncated later ones (setup_cf.c:364-372). */
    for (int k = 0; k < n; k++) {
      if (v[k] == 0) continue;
      if (g == 0) g = (size_t) round(v[k]);
      else g = fco_gcd(g, (size_t) v[k]);
    }
    if (g == 0) g = 1;
  }
  return ifac / (double) g;
}

/* ------------------------------------------------------------------------ */
/* Lookup tables (create_lut.c).  Entry i covers [i + (long) e[0], +1).      */

static uint16_t *fco_lut_int(const double *e, int num, long *ntab) {
  long lo = (long) e[0], hi = (long) e[num];
  long n = hi - lo;
  uint16_t *t = malloc(sizeof *t * (n > 0 ? n : 1));
  if (!t) return NULL;
  int k = 1;
  for (long i = 0; i < n; i++) {
    while (k <= num && !((double) (i + lo) < e[k])) k++;
    if (k > num) { free(t); return NULL; }
    t[i] = (uint16_t) (k - 1);
  }
  *ntab = n;
  return t;
}

static uint16_t *fco_lut_hybrid(const double *e, int num, long *ntab) {
  long lo = (long) e[0], hi = (long) ceil(e[num]);
  long n = hi - lo;
  uint16_t *t = malloc(sizeof *t * (n > 0 ? n : 1));
  if (!t) return NULL;
  int k = 1;
  long edge = (long) e[k];
  for (long i = 0; i < n; i++) {
    if (i + lo < edge) { t[i] = (uint16_t) (k - 1); continue; }
    /* Passed the truncated edge: the next edge whose truncation is above i
     * gives the starting bin of a downward walk. */
    int found = 0;
    while (++k <= num) {
      edge = (long) e[k];
      if (i + lo < edge) { t[i] = (uint16_t) (num + k - 1); found = 1; break; }
    }
    if (!found) {
      for (; i < n; i++) t[i] = (uint16_t) (2 * num);
      break;
    }
  }
  *ntab = n;
  return t;
}

static uint8_t *fco_lut_mu(int nmu) {
  int n2 = nmu * nmu;
  uint8_t *t = malloc(n2);
  if (!t) return NULL;
  for (int k = 0; k < nmu; k++)
    for (int i = k * k; i < (k + 1) * (k + 1); i++) t[i] = (uint8_t) k;
  return t;
}

/* ------------------------------------------------------------------------ */

void fco_bins_free(fco_bins *b) {
  if (!b) return;
  free(b->sbin_raw); free(b->pbin_raw); free(b->sbin); free(b->s2bin);
  free(b->pbin); free(b->p2bin); free(b->stab); free(b->ptab);
  free(b->mutab); free(b);
}

/*
 * Bin set-up, as cf_setup does it (src/fcfc/2pt_box/setup_cf.c:599-680).
 *   lin_s: linear s bins from (smin, ds, ns); otherwise sedge[0..ns] as
 *          read_bins produces them.  Same for pi.
 *   bsize: box sides (box geometry), ignored for surveys.
 * Returns NULL on failure.
 */
fco_bins *fco_bins_new(int survey, int bintype, int lin_s, double smin,
    double ds, int ns, const double *sedge, int nmu, int lin_p, double pmin,
    double dpi, int np, const double *pedge, const double *bsize) {
  fco_bins *b = calloc(1, sizeof *b);
  if (!b) return NULL;
  b->survey = survey;
  b->bintype = bintype;
  b->ns = ns;
  b->np = (bintype == FCO_BIN_SPI) ? np : 0;
  b->nmu = (bintype == FCO_BIN_SMU) ? nmu : 1;
  b->sbin_raw = malloc(sizeof(double) * (ns + 1));
  b->sbin = malloc(sizeof(double) * (ns + 1));
  b->s2bin = malloc(sizeof(double) * (ns + 1));
  if (!b->sbin_raw || !b->sbin || !b->s2bin) goto fail;
  for (int i = 0; i <= ns; i++)
    b->sbin[i] = lin_s ? smin + ds * i : sedge[i];
  memcpy(b->sbin_raw, b->sbin, sizeof(double) * (ns + 1));
  if (bintype == FCO_BIN_SPI) {
    b->pbin_raw = malloc(sizeof(double) * (np + 1));
    b->pbin = malloc(sizeof(double) * (np + 1));
    b->p2bin = malloc(sizeof(double) * (np + 1));
    if (!b->pbin_raw || !b->pbin || !b->p2bin) goto fail;
    for (int i = 0; i <= np; i++)
      b->pbin[i] = lin_p ? pmin + dpi * i : pedge[i];
    memcpy(b->pbin_raw, b->pbin, sizeof(double) * (np + 1));
  }

  if (bintype != FCO_BIN_SPI) {
    /* create_tab_sbin */
    int done = 0;
    if (lin_s) {
      double v[2] = {smin, ds};
      double fac = fco_least_fac(v, 2, 1);
      if (fac != 0) {
        double lo = round((b->sbin[0] * fac) * (b->sbin[0] * fac));
        double hi = round((b->sbin[ns] * fac) * (b->sbin[ns] * fac));
        if (lo <= FCO_MAXINT && hi <= FCO_MAXINT &&
            (size_t) hi - (size_t) lo <= FCO_LUT_INT_MAX) {
          b->rescale = fac;
          for (int i = 0; i <= ns; i++) {
            b->sbin[i] = round(b->sbin[i] * fac);
            b->s2bin[i] = b->sbin[i] * b->sbin[i];
          }
          b->tabtype = FCO_TAB_INT;
          b->stab = fco_lut_int(b->s2bin, ns, &b->nstab);
          done = 1;
        }
      }
    }
    if (!done) {
      double s2max = b->sbin[ns] * b->sbin[ns];
      double fac = FCO_LUT_HYB_MAX / s2max;
      fac = pow(FLT_RADIX, logb(fac));
      while (fac * s2max > FCO_LUT_HYB_MIN * 2) fac *= 0.5;
      b->rescale = fac;
      for (int i = 0; i <= ns; i++) {
        b->sbin[i] *= fac;
        b->s2bin[i] = b->sbin[i] * b->sbin[i];
      }
      b->tabtype = FCO_TAB_HYBRID;
      b->stab = fco_lut_hybrid(b->s2bin, ns, &b->nstab);
    }
    if (!b->stab) goto fail;
    if (bintype == FCO_BIN_SMU) {
      if (!(b->mutab = fco_lut_mu(nmu))) goto fail;
    }
  } else {
    /* create_tab_sp_pi; the survey tables run over squared pi */
    int done = 0;
    if (lin_s && lin_p) {
      double v[4] = {smin, ds, pmin, dpi};
      double fac = fco_least_fac(v, 4, 0);
      if (fac != 0) {
        double s1 = round((b->sbin[0] * fac) * (b->sbin[0] * fac));
        double s2 = round((b->sbin[ns] * fac) * (b->sbin[ns] * fac));
        if (s1 <= FCO_MAXINT && s2 <= FCO_MAXINT) {
          double p1 = b->pbin[0] * fac;
          double p2 = b->pbin[np] * fac;
          size_t nts = (size_t) s2 - (size_t) s1;
          size_t ntp = (size_t) p2 - (size_t) p1;
          if (nts <= FCO_LUT_INT_MAX && ntp <= FCO_LUT_INT_MAX) {
            b->rescale = fac;
            for (int i = 0; i <= ns; i++) {
              b->sbin[i] = round(b->sbin[i] * fac);
              b->s2bin[i] = b->sbin[i] * b->sbin[i];
            }
            for (int i = 0; i <= np; i++) {
              b->pbin[i] = round(b->pbin[i] * fac);
              b->p2bin[i] = b->pbin[i] * b->pbin[i];
            }
            b->tabtype = FCO_TAB_INT;
            b->stab = fco_lut_int(b->s2bin, ns, &b->nstab);
            b->ptab = fco_lut_int(survey ? b->p2bin : b->pbin, np, &b->nptab);
            done = 1;
          }
        }
      }
    }
    if (!done) {
      double s2max = b->sbin[ns] * b->sbin[ns];
      double pm = b->pbin[np];
      if (survey) pm *= pm;
      double larger = (s2max >= pm) ? s2max : pm;
      double smaller = (s2max >= pm) ? pm : s2max;
      double fac = FCO_LUT_HYB_MAX / larger;
      fac = pow(FLT_RADIX, logb(fac));
      while (fac * smaller > FCO_LUT_HYB_MIN * 2) fac *= 0.5;
      b->rescale = fac;
      for (int i = 0; i <= ns; i++) {
        b->sbin[i] *= fac;
        b->s2bin[i] = b->sbin[i] * b->sbin[i];
      }
      for (int i = 0; i <= np; i++) {
        b->pbin[i] *= fac;
        b->p2bin[i] = b->pbin[i] * b->pbin[i];
      }
      b->tabtype = FCO_TAB_HYBRID;
      b->stab = fco_lut_hybrid(b->s2bin, ns, &b->nstab);
      b->ptab = fco_lut_hybrid(survey ? b->p2bin : b->pbin, np, &b->nptab);
    }
    if (!b->stab || !b->ptab) goto fail;
  }
  b->smin_i = (long) b->s2bin[0];
  if (bintype == FCO_BIN_SPI)
    b->pmin_i = survey ? (long) b->p2bin[0] : (long) b->pbin[0];
  if (!survey && bsize)
    for (int k = 0; k < 3; k++) b->bsize[k] = bsize[k] * b->rescale;
  b->ntot = (long) ns * (bintype == FCO_BIN_SPI ? np :
      (bintype == FCO_BIN_SMU ? nmu : 1));
  return b;
fail:
  fco_bins_free(b);
  return NULL;
}

/* Accessors for ctypes. */
double fco_bins_rescale(const fco_bins *b) { return b->rescale; }
void fco_bins_set_mu_one(fco_bins *b, int on) { b->mu_one = on ? 1 : 0; }
int fco_bins_tabtype(const fco_bins *b) { return b->tabtype; }
long fco_bins_ntot(const fco_bins *b) { return b->ntot; }
long fco_bins_nstab(const fco_bins *b) { return b->nstab; }
long fco_bins_nptab(const fco_bins *b) { return b->nptab; }
void fco_bins_tables(const fco_bins *b, uint16_t *st, uint16_t *pt,
    double *s2, double *p) {
  if (st) memcpy(st, b->stab, sizeof(uint16_t) * b->nstab);
  if (pt && b->ptab) memcpy(pt, b->ptab, sizeof(uint16_t) * b->nptab);
  if (s2) memcpy(s2, b->s2bin, sizeof(double) * (b->ns + 1));
  if (p && b->pbin) memcpy(p, b->survey ? b->p2bin : b->pbin,
      sizeof(double) * (b->np + 1));
}
void fco_bins_box(const fco_bins *b, double *out) {
  for (int k = 0; k < 3; k++) out[k] = b->bsize[k];
}

/* ------------------------------------------------------------------------ */
/* Per-pair binning (metric_common.c).  Returns the histogram index or -1.   */

static inline int fco_lookup(const uint16_t *tab, long off, int num,
    const double *edge, double v) {
  int idx = tab[(long) (int) v - off];
  if (idx >= num) {           /* hybrid entry: walk down (metric_common.c:59) */
    idx -= num;
    while (idx != 0 && v < edge[idx]) idx--;
  }
  return idx;
}

/* Box: dx, dy, dz already formed as (x1 + shift) - x2. */
static inline long fco_bin_box(const fco_bins *b, double dx, double dy,
    double dz) {
  const double s2max = b->s2bin[b->ns], s2min = b->s2bin[0];
  const int smin0 = (s2min == 0);
  if (b->bintype == FCO_BIN_SPI) {
    double pi = fabs(dz);
    const double pmax = b->pbin[b->np], pmin = b->pbin[0];
    if (pi >= pmax) return -1;
    if (pmin != 0 && pi < pmin) return -1;
    double d = dx * dx + dy * dy;
    if (d >= s2max) return -1;
    if (!smin0 && d < s2min) return -1;
    int si = fco_lookup(b->stab, b->smin_i, b->ns, b->s2bin, d);
    int pi_ = fco_lookup(b->ptab, b->pmin_i, b->np, b->pbin, pi);
    return si + (long) pi_ * b->ns;
  }
  double d;
  double dz2 = dz * dz;
  d = dx * dx + dy * dy + dz2;
  if (d >= s2max) return -1;
  if (!smin0 && d < s2min) return -1;
  long mi = 0;
  if (b->bintype == FCO_BIN_SMU) {
    const int nmu2 = b->nmu * b->nmu;
    int p = (d < DBL_EPSILON) ? 0 : (int) ((dz2 / d) * nmu2);
    /* mu = 1 excluded, or with WITH_MU_ONE put in the last bin
     * (src/fcfc/2pt_box/metric_common.c:185-189) */
    if (p >= nmu2) {
      if (!b->mu_one) return -1;
      p = nmu2 - 1;
    }
    mi = b->mutab[p];
  }
  int si = fco_lookup(b->stab, b->smin_i, b->ns, b->s2bin, d);
  return si + mi * b->ns;
}

/* Survey: coordinates plus precomputed |x|^2 (src/fcfc/2pt/metric_common.c). */
static inline long fco_bin_survey(const fco_bins *b, double x1, double y1,
    double z1, double s1, double x2, double y2, double z2, double s2) {
  const double s2max = b->s2bin[b->ns], s2min = b->s2bin[0];
  const int smin0 = (s2min == 0);
  if (b->bintype == FCO_BIN_ISO) {
    double dx = x1 - x2, dy = y1 - y2, dz = z1 - z2;
    double d = dx * dx + dy * dy + dz * dz;
    if (d >= s2max) return -1;
    if (!smin0 && d < s2min) return -1;
    return fco_lookup(b->stab, b->smin_i, b->ns, b->s2bin, d);
  }
  double t = (x1 * x2 + y1 * y2 + z1 * z2) * 2;
  double s = s1 + s2;
  if (b->bintype == FCO_BIN_SMU) {
    double d = s - t;
    if (d >= s2max) return -1;
    if (!smin0 && d < s2min) return -1;
    double dd = s1 - s2;
    double pi2 = dd * dd / (s + t);
    const int nmu2 = b->nmu * b->nmu;
    int p = (d < DBL_EPSILON) ? 0 : (int) ((pi2 / d) * nmu2);
    if (p >= nmu2) {           /* src/fcfc/2pt/metric_common.c:209-214 */
      if (!b->mu_one) return -1;
      p = nmu2 - 1;
    }
    long mi = b->mutab[p];
    int si = fco_lookup(b->stab, b->smin_i, b->ns, b->s2bin, d);
    return si + mi * b->ns;
  }
  double dd = s1 - s2;
  double pi2 = dd * dd / (s + t);
  const double p2max = b->p2bin[b->np], p2min = b->p2bin[0];
  if (pi2 >= p2max) return -1;
  if (p2min != 0 && pi2 < p2min) return -1;
  double d = s - t - pi2;
  if (d >= s2max) return -1;
  if (!smin0 && d < s2min) return -1;
  if (d < 0) d = 0;  /* (int) of a value in (-1,0) is 0 in the reference */
  int si = fco_lookup(b->stab, b->smin_i, b->ns, b->s2bin, d);
  int pi_ = fco_lookup(b->ptab, b->pmin_i, b->np, b->p2bin, pi2);
  return si + (long) pi_ * b->ns;
}

/* ------------------------------------------------------------------------ */
/* Catalogues: rescaled FP64 coordinates, survey |x|^2, weights.            */

typedef struct {
  size_t n;
  double *x, *y, *z, *s, *w;
  uint32_t *id;       /* input index, for the auto-count shift order */
} fco_cat;

static void fco_cat_free(fco_cat *c) {
  free(c->x); free(c->y); free(c->z); free(c->s); free(c->w); free(c->id);
}

static int fco_cat_make(fco_cat *c, const fco_bins *b, size_t n,
    const double *x, const double *y, const double *z, const double *w) {
  memset(c, 0, sizeof *c);
  c->n = n;
  size_t m = n ? n : 1;
  c->x = malloc(sizeof(double) * m); c->y = malloc(sizeof(double) * m);
  c->z = malloc(sizeof(double) * m); c->s = malloc(sizeof(double) * m);
  c->w = malloc(sizeof(double) * m); c->id = malloc(sizeof(uint32_t) * m);
  if (!c->x || !c->y || !c->z || !c->s || !c->w || !c->id) {
    fco_cat_free(c); return -1;
  }
  const double f = b->rescale;
  for (size_t i = 0; i < n; i++) {
    double a = x[i], bb = y[i], cc = z[i];
    if (f != 1) { a *= f; bb *= f; cc *= f; }  /* build_tree.c:121-131 */
    c->x[i] = a; c->y[i] = bb; c->z[i] = cc;
    c->s[i] = a * a + bb * bb + cc * cc;         /* src/fcfc/2pt/build_tree.c:53 */
    c->w[i] = w ? w[i] : 1.0;
    c->id[i] = (uint32_t) i;
  }
  return 0;
}

/* Evaluate one ordered pair; (i from a, j from b, image shift applied to the
 * a-side point).  For auto counts the shift goes to the smaller input index. */
static inline long fco_pair(const fco_bins *b, const fco_cat *A, size_t i,
    const fco_cat *B, size_t j, const double sh[3], int isauto) {
  if (b->survey)
    return fco_bin_survey(b, A->x[i], A->y[i], A->z[i], A->s[i],
        B->x[j], B->y[j], B->z[j], B->s[j]);
  double dx, dy, dz;
  if (!isauto || A->id[i] < B->id[j]) {
    dx = (A->x[i] + sh[0]) - B->x[j];
    dy = (A->y[i] + sh[1]) - B->y[j];
    dz = (A->z[i] + sh[2]) - B->z[j];
  } else {
    dx = (B->x[j] - sh[0]) - A->x[i];
    dy = (B->y[j] - sh[1]) - A->y[i];
    dz = (B->z[j] - sh[2]) - A->z[i];
  }
  return fco_bin_box(b, dx, dy, dz);
}

/* Minimal-image shift for point a relative to b (valid for s_max < L/2). */
static inline void fco_min_image(const fco_bins *b, double ax, double ay,
    double az, double bx, double by, double bz, double sh[3]) {
  const double d[3] = {ax - bx, ay - by, az - bz};
  for (int k = 0; k < 3; k++) {
    double h = b->bsize[k] * 0.5;
    sh[k] = (d[k] > h) ? -b->bsize[k] : ((d[k] < -h) ? b->bsize[k] : 0);
  }
}

/* ------------------------------------------------------------------------ */
/* Cell grid.                                                                */

typedef struct {
  int n[3];
  double cw[3], lo[3];
  size_t *start;      /* ncell + 1 */
  size_t *perm;       /* sorted position -> catalogue index */
} fco_grid;

static void fco_grid_free(fco_grid *g) { free(g->start); free(g->perm); }

static int fco_cell_of(const fco_grid *g, double x, int k) {
  long c = (long) floor((x - g->lo[k]) / g->cw[k]);
  if (c < 0) c = 0;
  if (c >= g->n[k]) c = g->n[k] - 1;
  return (int) c;
}

static int fco_grid_build(fco_grid *g, const fco_cat *c) {
  size_t nc = (size_t) g->n[0] * g->n[1] * g->n[2];
  g->start = calloc(nc + 1, sizeof(size_t));
  g->perm = malloc(sizeof(size_t) * (c->n ? c->n : 1));
  size_t *cell = malloc(sizeof(size_t) * (c->n ? c->n : 1));
  if (!g->start || !g->perm || !cell) { free(cell); return -1; }
  for (size_t i = 0; i < c->n; i++) {
    size_t id = ((size_t) fco_cell_of(g, c->z[i], 2) * g->n[1] +
        fco_cell_of(g, c->y[i], 1)) * g->n[0] + fco_cell_of(g, c->x[i], 0);
    cell[i] = id;
    g->start[id + 1]++;
  }
  for (size_t k = 0; k < nc; k++) g->start[k + 1] += g->start[k];
  size_t *fill = malloc(sizeof(size_t) * (nc ? nc : 1));
  if (!fill) { free(cell); return -1; }
  memcpy(fill, g->start, sizeof(size_t) * nc);
  for (size_t i = 0; i < c->n; i++) g->perm[fill[cell[i]]++] = i;
  free(fill); free(cell);
  return 0;
}

/*
 * Count pairs.  mode 0: cell grid with cells of side s_max; mode 1: brute
 * force over all pairs; mode k >= 2: cells of side s_max / k.
 * isauto: unordered pairs of catalogue A with itself (counted once each,
 * as count_pairs does before eval_pairs doubles them).
 * Outputs: icnt (unweighted) or wcnt (weighted), ntot entries, zeroed here.
 * nthread <= 0: OpenMP default.
 * Return 0, or negative on error.
 */
int fco_count(const fco_bins *b, size_t na, const double *ax, const double *ay,
    const double *az, const double *aw, size_t nb, const double *bx,
    const double *by, const double *bz, const double *bw, int isauto,
    int withwt, int mode, int nthread, int64_t *icnt, double *wcnt) {
  fco_cat A, B;
  const long ntot = b->ntot;
  if (fco_cat_make(&A, b, na, ax, ay, az, aw)) return -1;
  if (isauto) B = A;
  else if (fco_cat_make(&B, b, nb, bx, by, bz, bw)) { fco_cat_free(&A); return -1; }
#ifdef _OPENMP
  int nth = nthread > 0 ? nthread : omp_get_max_threads();
#else
  int nth = 1;
  (void) nthread;
#endif
  int64_t *ih = calloc((size_t) ntot * nth, sizeof(int64_t));
  double *wh = calloc((size_t) ntot * nth, sizeof(double));
  if (!ih || !wh) goto oom;

  double smax = b->sbin[b->ns];
  if (b->bintype == FCO_BIN_SPI) {
    double pm = b->pbin[b->np];
    smax = sqrt(smax * smax + pm * pm);
  }

  if (mode == 1) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (size_t i = 0; i < A.n; i++) {
#ifdef _OPENMP
      int t = omp_get_thread_num();
#else
      int t = 0;
#endif
      int64_t *hi = ih + (size_t) t * ntot;
      double *hw = wh + (size_t) t * ntot;
      for (size_t j = isauto ? i + 1 : 0; j < B.n; j++) {
        double sh[3] = {0, 0, 0};
        if (!b->survey)
          fco_min_image(b, A.x[i], A.y[i], A.z[i], B.x[j], B.y[j], B.z[j], sh);
        long k = fco_pair(b, &A, i, &B, j, sh, isauto);
        if (k < 0) continue;
        if (withwt) hw[k] += A.w[i] * B.w[j];
        else hi[k]++;
      }
    }
  } else {
    /* Grid with cells of side >= reach / kc and a stencil of cell offsets
     * pruned by the smallest distance between the two cells; images come
     * from the offsets, so small boxes (few cells per side) stay correct. */
    const int kc = (mode >= 2) ? mode : 1;
    fco_grid g;
    memset(&g, 0, sizeof g);
    double reach[3] = {smax, smax, smax};
    if (!b->survey && b->bintype == FCO_BIN_SPI) {
      reach[0] = reach[1] = b->sbin[b->ns] * (1 + 1e-9);
      reach[2] = b->pbin[b->np] * (1 + 1e-9);
    }
    if (b->survey) {
      double lo[3], hi[3];
      for (int k = 0; k < 3; k++) { lo[k] = INFINITY; hi[k] = -INFINITY; }
      const fco_cat *cs[2] = {&A, &B};
      for (int q = 0; q < 2; q++)
        for (size_t i = 0; i < cs[q]->n; i++) {
          double v[3] = {cs[q]->x[i], cs[q]->y[i], cs[q]->z[i]};
          for (int k = 0; k < 3; k++) {
            if (v[k] < lo[k]) lo[k] = v[k];
            if (v[k] > hi[k]) hi[k] = v[k];
          }
        }
      for (int k = 0; k < 3; k++) {
        if (!(hi[k] >= lo[k])) { lo[k] = 0; hi[k] = 1; }
        double ext = hi[k] - lo[k];
        int n = (int) (ext / (reach[k] / kc * (1 + 1e-6)));
        if (n < 1) n = 1;
        if (n > 512) n = 512;
        g.n[k] = n; g.lo[k] = lo[k];
        g.cw[k] = (ext > 0 ? ext : 1) / n * (1 + 1e-12);
      }
    } else {
      for (int k = 0; k < 3; k++) {
        int n = (int) (b->bsize[k] / (reach[k] / kc * (1 + 1e-6)));
        if (n < 1) n = 1;
        if (n > 512) n = 512;
        g.n[k] = n; g.lo[k] = 0; g.cw[k] = b->bsize[k] / n;
      }
    }
    fco_grid gb = g;
    if (fco_grid_build(&g, &A)) goto oom;
    if (isauto) gb = g;
    else if (fco_grid_build(&gb, &B)) { fco_grid_free(&g); goto oom; }

    /* stencil */
    int r[3];
    for (int k = 0; k < 3; k++) {
      r[k] = (int) ceil(reach[k] * (1 + 1e-9) / g.cw[k]);
      if (b->survey && r[k] > g.n[k] - 1) r[k] = g.n[k] - 1;
    }
    int nst = 0;
    int *st = malloc(sizeof(int) * 3 * (2 * r[0] + 1) * (2 * r[1] + 1) *
                     (2 * r[2] + 1));
    if (!st) { fco_grid_free(&g); if (!isauto) fco_grid_free(&gb); goto oom; }
    for (int oz = -r[2]; oz <= r[2]; oz++)
      for (int oy = -r[1]; oy <= r[1]; oy++)
        for (int ox = -r[0]; ox <= r[0]; ox++) {
          int o[3] = {ox, oy, oz};
          if (isauto) {
            int sgn = oz ? oz : (oy ? oy : ox);
            if (sgn < 0) continue;
          }
          double gap[3];
          for (int k = 0; k < 3; k++) {
            int a = abs(o[k]);
            gap[k] = (a > 0 ? a - 1 : 0) * g.cw[k];
          }
          if (!b->survey && b->bintype == FCO_BIN_SPI) {
            if (gap[2] > reach[2] * (1 + 1e-6)) continue;
            if (gap[0] * gap[0] + gap[1] * gap[1] >
                reach[0] * reach[0] * (1 + 1e-6)) continue;
          } else if (gap[0] * gap[0] + gap[1] * gap[1] + gap[2] * gap[2] >
                     smax * smax * (1 + 1e-6)) {
            continue;
          }
          st[3 * nst] = ox; st[3 * nst + 1] = oy; st[3 * nst + 2] = oz;
          nst++;
        }
    const size_t nc = (size_t) g.n[0] * g.n[1] * g.n[2];
#pragma omp parallel for schedule(dynamic, 4) num_threads(nth)
    for (size_t ca = 0; ca < nc; ca++) {
#ifdef _OPENMP
      int t = omp_get_thread_num();
#else
      int t = 0;
#endif
      int64_t *hi = ih + (size_t) t * ntot;
      double *hw = wh + (size_t) t * ntot;
      if (g.start[ca] == g.start[ca + 1]) continue;
      int c[3] = {(int) (ca % g.n[0]), (int) ((ca / g.n[0]) % g.n[1]),
          (int) (ca / ((size_t) g.n[0] * g.n[1]))};
      for (int q = 0; q < nst; q++) {
        const int *o = st + 3 * q;
        const int zero = (o[0] == 0 && o[1] == 0 && o[2] == 0);
        int cb[3];
        double sh[3] = {0, 0, 0};
        int skip = 0;
        for (int k = 0; k < 3; k++) {
          int v = c[k] + o[k];
          if (b->survey) {
            if (v < 0 || v >= g.n[k]) { skip = 1; break; }
          } else {
            int w = (int) floor((double) v / g.n[k]);
            v -= w * g.n[k];
            sh[k] = -(double) w * b->bsize[k];
          }
          cb[k] = v;
        }
        if (skip) continue;
        size_t cbid = ((size_t) cb[2] * g.n[1] + cb[1]) * g.n[0] + cb[0];
        for (size_t pa = g.start[ca]; pa < g.start[ca + 1]; pa++) {
          size_t i = g.perm[pa];
          size_t pb0 = gb.start[cbid];
          if (isauto && zero) pb0 = pa + 1;
          for (size_t pb = pb0; pb < gb.start[cbid + 1]; pb++) {
            size_t j = gb.perm[pb];
            long k = fco_pair(b, &A, i, &B, j, sh, isauto);
            if (k < 0) continue;
            if (withwt) hw[k] += A.w[i] * B.w[j];
            else hi[k]++;
          }
        }
      }
    }
    free(st);
    fco_grid_free(&g);
    if (!isauto) fco_grid_free(&gb);
  }

  for (long k = 0; k < ntot; k++) {
    int64_t si = 0;
    double sw = 0;
    for (int t = 0; t < nth; t++) {
      si += ih[(size_t) t * ntot + k];
      sw += wh[(size_t) t * ntot + k];
    }
    if (icnt) icnt[k] = si;
    if (wcnt) wcnt[k] = sw;
  }
  free(ih); free(wh);
  fco_cat_free(&A);
  if (!isauto) fco_cat_free(&B);
  return 0;
oom:
  free(ih); free(wh);
  fco_cat_free(&A);
  if (!isauto) fco_cat_free(&B);
  return -1;
}

/* ------------------------------------------------------------------------ */
/* RA/Dec/z -> comoving coordinates (COORD_CONVERT), FP64 with the C        */
/* library's cos/sin/pow/sqrt, in the reference's operation order.  The     */
/* Gauss-Legendre nodes and weights are the engine's generated table, whose  */
/* every entry equals the reference's legauss.c (checked by the generator).  */

#include "../fcfc_gb300/csrc/legauss_tab.h"

static const double fco_glx[FCFCG_GL_LEN] = FCFCG_GL_X_INIT;
static const double fco_glw[FCFCG_GL_LEN] = FCFCG_GL_W_INIT;

typedef struct { double om, ol, ok, widx; } fco_cosmo;

/* cnvt_integrand, cnvt_coord.c:202-212 */
static double fco_integrand(const fco_cosmo *c, double z) {
  double z1 = z + 1;
  double z2 = z1 * z1;
  double d = c->om * z2 * z1;
  if (c->ok) d += c->ok * z2;
  if (c->widx) d += c->ol * pow(z1, c->widx);
  else d += c->ol;
  d = 299792.458 * 0.01 / sqrt(d);
  return d;
}

/* cnvt_legauss, cnvt_coord.c:227-250 */
static double fco_legauss(const fco_cosmo *c, int order, double z) {
  double zp = z * 0.5;
  double sum = 0;
  int i;
  for (i = FCFCG_GL_START(order);
       i < FCFCG_GL_START(order) + (order >> 1); i++) {
    double x = fco_glx[i];
    double w = fco_glw[i];
    double z1 = zp * (1 + x);
    double z2 = zp * (1 - x);
    sum += w * (fco_integrand(c, z1) + fco_integrand(c, z2));
  }
  if (order & 1) sum += fco_glw[i] * fco_integrand(c, zp);
  return sum * zp;
}

/* cnvt_legauss_order (cnvt_coord.c:267-307) over cnvt_z_sample's 128
 * redshifts (:113-186); -1 when no order up to 32 converges. */
int fco_cnvt_order(double om, double ol, double ok, double widx, double err,
    size_t n, const double *z) {
  fco_cosmo c = {om, ol, ok, widx};
  double zmax = -DBL_MAX, zmin = DBL_MAX;
  for (size_t i = 0; i < n; i++) {
    if (zmax < z[i]) zmax = z[i];
    if (zmin > z[i]) zmin = z[i];
  }
  if (zmin > zmax) return -1;
  const int num = 128;
  int order = 0;
  for (int i = 0; i < num; i++) {
    double zt = zmin + i * (zmax - zmin) / (num - 1);
    double oint, nint = 0;
    int k = FCFCG_GL_MIN_ORDER - 1;
    do {
      if (k >= FCFCG_GL_MAX_ORDER) return -1;
      oint = nint;
      nint = fco_legauss(&c, ++k, zt);
    } while (fabs(nint - oint) > nint * err);
    if (order < k) order = k;
  }
  return order;
}

/* cnvt_coord_integr, cnvt_coord.c:321-337 (x, y, zc may alias the input) */
void fco_cnvt_integr(double om, double ol, double ok, double widx, int order,
    size_t n, const double *ra, const double *dec, const double *z,
    double *x, double *y, double *zc) {
  fco_cosmo c = {om, ol, ok, widx};
  const double d2r = 0x1.1df46a2529d39p-6;   /* DEGREE_2_RAD */
#ifdef _OPENMP
#pragma omp parallel for
#endif
  for (size_t i = 0; i < n; i++) {
    double a = ra[i] * d2r;
    double b = dec[i] * d2r;
    double dist = fco_legauss(&c, order, z[i]);
    x[i] = dist * cos(b) * cos(a);
    y[i] = dist * cos(b) * sin(a);
    zc[i] = dist * sin(b);
  }
}

/* Natural cubic spline through (zs, ds), zs sorted ascending
 * (cspline_ypp / cspline_eval, src/math/cspline.c:34-110), evaluated as
 * sample_interp does (cnvt_coord.c:58-72); returns the number of redshifts
 * outside [zs[0], zs[m-1]) (their distance is HUGE_VAL). */
size_t fco_cnvt_spline(size_t m, const double *zs, const double *ds,
    size_t n, const double *ra, const double *dec, const double *z,
    double *x, double *y, double *zc) {
  double *ypp = malloc(m * sizeof(double)), *cp = malloc(m * sizeof(double));
  double newx = zs[1], newy = ds[1];
  double c = zs[1] - zs[0];
  double newd = (ds[1] - ds[0]) / c;
  cp[0] = cp[m - 1] = ypp[0] = ypp[m - 1] = 0;
  size_t j = 1;
  while (j < m - 1) {
    double oldx = newx, oldy = newy, a = c, oldd = newd;
    newx = zs[j + 1];
    newy = ds[j + 1];
    c = newx - oldx;
    newd = (newy - oldy) / c;
    double b = (c + a) * 2;
    double invd = 1 / (b - a * cp[j - 1]);
    double d = (newd - oldd) * 6;
    ypp[j] = (d - a * ypp[j - 1]) * invd;
    cp[j] = c * invd;
    j += 1;
  }
  while (j) {
    j -= 1;
    ypp[j] -= cp[j] * ypp[j + 1];
  }
  const double d2r = 0x1.1df46a2529d39p-6;
  size_t bad = 0;
  for (size_t k = 0; k < n; k++) {
    double v = z[k], dist;
    size_t i = 0, l = 0, u = m - 1;
    if (v < zs[l] || v >= zs[u]) {
      dist = HUGE_VAL;
      bad++;
    } else {
      while (l <= u) {
        i = (l + u) >> 1;
        if (zs[i + 1] <= v) l = i + 1;
        else if (zs[i] > v) u = i - 1;
        else break;
      }
      size_t jj = i + 1;
      double ba = zs[jj] - zs[i];
      double xa = v - zs[i];
      double bx = zs[jj] - v;
      double ba2 = ba * ba;
      double lower = xa * ds[jj] + bx * ds[i];
      double cc = (xa * xa - ba2) * xa * ypp[jj];
      double dd = (bx * bx - ba2) * bx * ypp[i];
      dist = (lower + 0x1.5555555555555p-3 * (cc + dd)) / ba;
    }
    double a = ra[k] * d2r;
    double b = dec[k] * d2r;
    x[k] = dist * cos(b) * cos(a);
    y[k] = dist * cos(b) * sin(a);
    zc[k] = dist * sin(b);
  }
  free(ypp);
  free(cp);
  return bad;
}

/* ------------------------------------------------------------------------ */
/* Per-object gradient of sum_b g_b C_b, C_b the weighted count (the engine's */
/* adjoint has no reference counterpart; this is its CPU reference).        */
/* Brute force over pairs, FP64: dwa[i] = sum_j w_j g[bin(i, j)], dwb[j] =   */
/* sum_i w_i g[bin(i, j)]; for auto counts every unordered pair feeds both   */
/* points of dwa.  Returns 0, or -1 when out of memory.                      */
int fco_adjoint(const fco_bins *b, size_t na, const double *ax,
    const double *ay, const double *az, const double *aw, size_t nb,
    const double *bx, const double *by, const double *bz, const double *bw,
    int isauto, const double *g, double *dwa, double *dwb) {
  fco_cat A, B;
  if (fco_cat_make(&A, b, na, ax, ay, az, aw)) return -1;
  if (isauto) B = A;
  else if (fco_cat_make(&B, b, nb, bx, by, bz, bw)) { fco_cat_free(&A); return -1; }
  for (size_t i = 0; i < A.n; i++) dwa[i] = 0;
  if (!isauto && dwb)
    for (size_t j = 0; j < B.n; j++) dwb[j] = 0;
  for (size_t i = 0; i < A.n; i++) {
    for (size_t j = isauto ? i + 1 : 0; j < B.n; j++) {
      double sh[3] = {0, 0, 0};
      if (!b->survey)
        fco_min_image(b, A.x[i], A.y[i], A.z[i], B.x[j], B.y[j], B.z[j], sh);
      long k = fco_pair(b, &A, i, &B, j, sh, isauto);
      if (k < 0) continue;
      dwa[i] += B.w[j] * g[k];
      if (isauto) dwa[j] += A.w[i] * g[k];
      else if (dwb) dwb[j] += A.w[i] * g[k];
    }
  }
  fco_cat_free(&A);
  if (!isauto) fco_cat_free(&B);
  return 0;
}
