/*
 * bins.c -- bin set-up of the engine: rescale factor, rescaled edges and the
 * lookup tables FCFC bins separations with, plus the FP32 edge-window tables
 * the fast path uses to decide when a pair must be re-binned in FP64.
 *
 * The reference part follows FCFC v1.0.1 step for step, because the bins a
 * pair lands in are defined by it:
 *   rescale factor    src/fcfc/2pt_box/setup_cf.c:308-376 (least_fac2/4)
 *   s bins            src/fcfc/2pt_box/setup_cf.c:385-430 (create_tab_sbin)
 *   (s_perp, pi)      src/fcfc/2pt_box/setup_cf.c:439-503 (create_tab_sp_pi);
 *                     surveys square the pi edges, src/fcfc/2pt/setup_cf.c:455-502
 *   tables            src/util/create_lut.c:58-140
 *   checks            src/fcfc/2pt_box/load_conf.c:985-1003,1040-1060,1120-1126
 * FCFC builds a separate mu table (setup_cf.c:513-531); it maps
 * (int)(mu^2 nmu^2) to floor(sqrt(.)), i.e. to floor(nmu mu), which the
 * kernels compute directly.
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fcfcg_internal.h"

#define LUT_INT_MAX 40960      /* FCFC_LOOKUP_INT_MAX_SIZE */
#define LUT_HYB_MAX 32768      /* FCFC_LOOKUP_HYBRID_MAX_SIZE */
#define LUT_HYB_MIN 8192       /* FCFC_LOOKUP_HYBRID_MIN_SIZE */
#define MAX_DIGIT 4            /* FCFC_BIN_MAX_DIGIT_TO_INT */
#define DBL_TOL_ 1e-10         /* DOUBLE_TOL */
#define MAXINT_ 0x1p+53        /* REAL_MAXINT (double) */
#define MAX_NSBIN 10000        /* FCFC_MAX_NSBIN */
#define MAX_NMU 255            /* FCFC_MAX_NMU */

int fcfcg_linear_nbin(double vmin, double vmax, double step) {
  if (!(step > 0) || !isfinite(step)) return -1;
  double v = vmin;
  int n = 0;
  while (v < vmax - DBL_TOL_) {
    v += step;
    if (++n > MAX_NSBIN) return -1;
  }
  return n;
}

static size_t gcd_sz(size_t a, size_t b) {
  while (b) {
    size_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

static int is_int_tol(double v) { return fabs(round(v) - v) < DBL_TOL_; }

/* Factor turning (a, b) into integers: 10^k / gcd, or 0 (least_fac2). */
static double fac_pair(double a, double b) {
  if (a < 0 || a > MAXINT_ || b < 0 || b > MAXINT_) return 0;
  if (a == 0) return 1 / b;
  if (b == 0) return 1 / a;
  size_t ifac = 1;
  int k = 0;
  while (!(is_int_tol(a) && is_int_tol(b))) {
    if (k == MAX_DIGIT + 1) break;
    a *= 10;
    b *= 10;
    ifac *= 10;
    k++;
  }
  if (!(is_int_tol(a) && is_int_tol(b)) && k == MAX_DIGIT + 1) return 0;
  if (k == MAX_DIGIT + 1) return 0;
  if (a > MAXINT_ || b > MAXINT_) return 0;
  size_t g = gcd_sz((size_t) round(a), (size_t) round(b));
  return ifac / (double) g;
}

/* Same for four numbers (least_fac4): the divisor starts from the first
 * non-zero value rounded, later ones enter truncated. */
static double fac_quad(double v[4]) {
  for (int i = 0; i < 4; i++)
    if (v[i] < 0 || v[i] > MAXINT_) return 0;
  size_t ifac = 1;
  int k = 0;
  for (;;) {
    int all = 1;
    for (int i = 0; i < 4; i++) all &= is_int_tol(v[i]);
    if (all) break;
    if (k == MAX_DIGIT + 1) return 0;
    for (int i = 0; i < 4; i++) v[i] *= 10;
    ifac *= 10;
    k++;
  }
  if (k == MAX_DIGIT + 1) return 0;
  for (int i = 0; i < 4; i++)
    if (v[i] > MAXINT_) return 0;
  size_t g = 0;
  for (int i = 0; i < 4; i++) {
    if (v[i] == 0) continue;
    g = g ? gcd_sz(g, (size_t) v[i]) : (size_t) round(v[i]);
  }
  if (!g) g = 1;
  return ifac / (double) g;
}

/* Integer table: entry i -> bin of values in [i + lo, i + lo + 1). */
static uint16_t *lut_int(const double *e, int n, long *len, long *off) {
  long lo = (long) e[0], hi = (long) e[n];
  long m = hi - lo;
  uint16_t *t = malloc(sizeof *t * (m > 0 ? m : 1));
  if (!t) return NULL;
  int k = 1;
  for (long i = 0; i < m; i++) {
    while (k <= n && (double) (i + lo) >= e[k]) k++;
    if (k > n) {
      free(t);
      return NULL;
    }
    t[i] = (uint16_t) (k - 1);
  }
  *len = m;
  *off = lo;
  return t;
}

/* Hybrid table: a direct bin, or n + k meaning "walk down from bin k while
 * the value is below its lower edge", or 2n past the last edge.  Edges are
 * compared after truncation to integers, as create_lut_hybrid does. */
static uint16_t *lut_hybrid(const double *e, int n, long *len, long *off) {
  long lo = (long) e[0], hi = (long) ceil(e[n]);
  long m = hi - lo;
  uint16_t *t = malloc(sizeof *t * (m > 0 ? m : 1));
  if (!t) return NULL;
  int k = 1;
  long cut = (long) e[1];
  long i = 0;
  for (; i < m; i++) {
    if (i + lo < cut) {
      t[i] = (uint16_t) (k - 1);
      continue;
    }
    int hit = 0;
    while (++k <= n) {
      cut = (long) e[k];
      if (i + lo < cut) {
        t[i] = (uint16_t) (n + k - 1);
        hit = 1;
        break;
      }
    }
    if (!hit) break;
  }
  for (; i < m; i++) t[i] = (uint16_t) (2 * n);
  *len = m;
  *off = lo;
  return t;
}

/* Bin of the exact value v on an axis (FCFC's table semantics), or -1. */
static int axis_bin(const fcfcg_axis *a, double v) {
  if (v >= a->vmax) return -1;
  if (!a->min0 && v < a->vmin) return -1;
  int k = 0;
  while (k + 1 < a->nbin && a->edge[k + 1] <= v) k++;
  return k;
}

/* FP32 bit pattern of a positive double rounded to float, and back. */
static uint32_t fbits(double v) {
  const float f = (float) v;
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

static double bits_value(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return (double) f;
}

/* Flags and start bin of the table cell [x0, x1) (see FCFCG_FTAB_*). */
static unsigned ftab_cell(const fcfcg_axis *a, double x0, double x1) {
  const double w = x1 - x0;
  const int first = a->min0 ? 1 : 0;
  int b = axis_bin(a, x0);
  unsigned v = (b < 0) ? FCFCG_FTAB_BIN_MASK : (unsigned) b;
  int inside = 0;
  for (int k = first; k <= a->nbin; k++) {
    const double e = a->edge[k];
    if (e >= x0 - 0.5 * w && e <= x0) v |= FCFCG_FTAB_LO;
    if (e >= x1 && e <= x1 + 0.5 * w) v |= FCFCG_FTAB_HI;
    if (e > x0 && e < x1) inside++;
  }
  if (inside == 1) v |= FCFCG_FTAB_CX1;
  else if (inside > 1) v |= FCFCG_FTAB_CXM;
  return v;
}

/*
 * Bit-pattern table: cell c holds the positive FP32 values whose bit
 * pattern >> sh is c, i.e. a fixed fraction 2^(sh - 23) of each octave --
 * what bins spaced in ratio (log bins) need.  The coarsest sh from 19 (16
 * cells per octave) down to 8 (2^15) that fits the table and has no cell
 * holding several edges; the axis is left alone when there is none, or when
 * it starts at zero.
 */
static int axis_ftab_log(fcfcg_axis *a) {
  if (a->min0 || !(a->vmin > 0)) return 0;
  for (int sh = 19; sh >= 8; sh--) {
    /* from at least one whole cell below the lowest edge to one above the
     * highest, as the uniform tables */
    const long lo = (long) (fbits(a->vmin) >> sh) - 2;
    const long hi = (long) (fbits(a->vmax) >> sh) + 3;
    const long m = hi - lo;
    if (lo < 1 || m > FCFCG_FTAB_MAXLEN) break;   /* finer: too long */
    uint16_t *t = malloc(sizeof(uint16_t) * m);
    if (!t) return FCFCG_ERR_MEMORY;
    int multi = 0;
    for (long c = 0; c < m && !multi; c++) {
      const double x0 = bits_value((uint32_t) (lo + c) << sh);
      const double x1 = bits_value((uint32_t) (lo + c + 1) << sh);
      t[c] = (uint16_t) ftab_cell(a, x0, x1);
      multi = (t[c] & FCFCG_FTAB_CXM) != 0;
    }
    if (multi) {
      free(t);
      continue;
    }
    free(a->ftab);
    a->ftab = t;
    a->foff = lo;
    a->nftab = m;
    a->fshift = 0;
    a->flog = sh;
    return 0;
  }
  return 0;
}

int fcfcg_axis_ftab(fcfcg_axis *a, int allow_log) {
  /* cell width: the smallest power of two (>= 1 unit) that keeps the table
   * within FCFCG_FTAB_MAXLEN cells */
  int sh = 0;
  for (;;) {
    const double w = ldexp(1.0, sh);
    long lo = a->min0 ? 0 : (long) floor(a->vmin / w) - 1;
    long hi = (long) ceil(a->vmax / w) + 2;
    if (hi - lo <= FCFCG_FTAB_MAXLEN || sh > 40) break;
    sh++;
  }
  const double w = ldexp(1.0, sh);
  long lo = a->min0 ? 0 : (long) floor(a->vmin / w) - 1;
  long hi = (long) ceil(a->vmax / w) + 2;
  long m = hi - lo;
  free(a->ftab);
  free(a->fedge);
  a->ftab = malloc(sizeof(uint16_t) * m);
  a->fedge = malloc(sizeof(float) * (a->nbin + 1));
  if (!a->ftab || !a->fedge) return FCFCG_ERR_MEMORY;
  for (int k = 0; k <= a->nbin; k++) a->fedge[k] = (float) a->edge[k];
  int multi = 0;
  for (long c = 0; c < m; c++) {
    const double x0 = (double) (lo + c) * w, x1 = x0 + w;
    a->ftab[c] = (uint16_t) ftab_cell(a, x0, x1);
    multi |= (a->ftab[c] & FCFCG_FTAB_CXM) != 0;
  }
  a->foff = lo;
  a->nftab = m;
  a->fshift = sh;
  a->flog = 0;
  /* cells holding several edges send every value in them to the FP64
   * recheck: bins that are not linear get a bit-pattern table if that
   * resolves them */
  if (multi && allow_log) return axis_ftab_log(a);
  return FCFCG_OK;
}

/* allow_log: the kernels can use a bit-pattern FP32 table for this axis
 * (the s or s_perp axis in a box) */
static int axis_finish(fcfcg_axis *a, const double *edge, int n, int hybrid,
    int allow_log) {
  a->nbin = n;
  a->tabtype = hybrid ? FCFCG_TAB_HYBRID : FCFCG_TAB_INT;
  a->edge = malloc(sizeof(double) * (n + 1));
  if (!a->edge) return FCFCG_ERR_MEMORY;
  memcpy(a->edge, edge, sizeof(double) * (n + 1));
  a->vmin = edge[0];
  a->vmax = edge[n];
  a->min0 = (edge[0] == 0);
  a->rtab = hybrid ? lut_hybrid(edge, n, &a->nrtab, &a->roff)
                   : lut_int(edge, n, &a->nrtab, &a->roff);
  if (!a->rtab) return FCFCG_ERR_CF;
  if (n <= FCFCG_FTAB_MAXBIN) return fcfcg_axis_ftab(a, allow_log);
  return FCFCG_OK;
}

static void axis_free(fcfcg_axis *a) {
  free(a->edge);
  free(a->rtab);
  free(a->ftab);
  free(a->fedge);
  memset(a, 0, sizeof *a);
}

void fcfcg_bins_release(fcfcg_bins *b) {
  if (!b) return;
  free(b->sbin_raw);
  free(b->pbin_raw);
  axis_free(&b->s);
  axis_free(&b->p);
  memset(b, 0, sizeof *b);
}

#define FAIL(code, ...)                       \
  do {                                        \
    if (err) snprintf(err, errlen, __VA_ARGS__); \
    rc = (code);                              \
    goto fail;                                \
  } while (0)

int fcfcg_bins_setup(const fcfcg_binning *cfg, fcfcg_bins *b, char *err,
    size_t errlen) {
  int rc = FCFCG_OK;
  double *sb = NULL, *s2 = NULL, *pb = NULL, *p2 = NULL;
  memset(b, 0, sizeof *b);
  if (!cfg) FAIL(FCFCG_ERR_ARG, "no binning configuration");
  const int box = (cfg->geometry == FCFCG_GEOM_BOX);
  if (cfg->geometry != FCFCG_GEOM_BOX && cfg->geometry != FCFCG_GEOM_SURVEY)
    FAIL(FCFCG_ERR_ARG, "unknown geometry %d", cfg->geometry);
  if (cfg->bintype < FCFCG_BIN_ISO || cfg->bintype > FCFCG_BIN_SPI)
    FAIL(FCFCG_ERR_CFG, "BINNING_SCHEME must be 0, 1 or 2");
  const int ns = cfg->ns;
  if (ns < 1 || ns > MAX_NSBIN)
    FAIL(FCFCG_ERR_CFG, "number of separation bins must be in [1,%d]",
         MAX_NSBIN);
  const int spi = (cfg->bintype == FCFCG_BIN_SPI);
  const int np = spi ? cfg->np : 0;
  if (spi && (np < 1 || np > MAX_NSBIN))
    FAIL(FCFCG_ERR_CFG, "number of pi bins must be in [1,%d]", MAX_NSBIN);
  const int nmu = (cfg->bintype == FCFCG_BIN_SMU) ? cfg->nmu : 1;
  if (cfg->bintype == FCFCG_BIN_SMU && (nmu < 2 || nmu > MAX_NMU))
    FAIL(FCFCG_ERR_CFG, "MU_BIN_NUM must be in [2,%d]", MAX_NMU);
  if (box) {
    for (int k = 0; k < 3; k++)
      if (!isfinite(cfg->box[k]) || cfg->box[k] <= 0)
        FAIL(FCFCG_ERR_CFG, "BOX_SIZE must be finite and positive");
  }
  b->geometry = cfg->geometry;
  b->bintype = cfg->bintype;
  b->ns = ns;
  b->np = np;
  b->nmu = nmu;
  b->mu_one = cfg->with_mu_one ? 1 : 0;
  b->ntot = (long) ns * (spi ? np : nmu);

  sb = malloc(sizeof(double) * (ns + 1));
  s2 = malloc(sizeof(double) * (ns + 1));
  b->sbin_raw = malloc(sizeof(double) * (ns + 1));
  if (!sb || !s2 || !b->sbin_raw) FAIL(FCFCG_ERR_MEMORY, "out of memory");
  for (int i = 0; i <= ns; i++)
    sb[i] = cfg->sedges ? cfg->sedges[i] : cfg->smin + cfg->ds * i;
  for (int i = 0; i < ns; i++)
    if (!(sb[i + 1] > sb[i]) || !isfinite(sb[i]) || sb[0] < 0)
      FAIL(FCFCG_ERR_CFG, "separation bin edges must be increasing and >= 0");
  memcpy(b->sbin_raw, sb, sizeof(double) * (ns + 1));
  if (spi) {
    pb = malloc(sizeof(double) * (np + 1));
    p2 = malloc(sizeof(double) * (np + 1));
    b->pbin_raw = malloc(sizeof(double) * (np + 1));
    if (!pb || !p2 || !b->pbin_raw) FAIL(FCFCG_ERR_MEMORY, "out of memory");
    for (int i = 0; i <= np; i++)
      pb[i] = cfg->pedges ? cfg->pedges[i] : cfg->pmin + cfg->dpi * i;
    for (int i = 0; i < np; i++)
      if (!(pb[i + 1] > pb[i]) || !isfinite(pb[i]) || pb[0] < 0)
        FAIL(FCFCG_ERR_CFG, "pi bin edges must be increasing and >= 0");
    memcpy(b->pbin_raw, pb, sizeof(double) * (np + 1));
  }
  if (box) {
    for (int k = 0; k < 3; k++) {
      if (sb[ns] >= cfg->box[k] * 0.5)
        FAIL(FCFCG_ERR_CFG,
             "the maximum separation must be smaller than half the box size");
      if (spi && pb[np] >= cfg->box[k] * 0.5)
        FAIL(FCFCG_ERR_CFG,
             "the maximum pi must be smaller than half the box size");
    }
  }

  int hybrid = 1;
  double fac = 0;
  if (!spi) {
    if (!cfg->sedges) {
      fac = fac_pair(cfg->smin, cfg->ds);
      if (fac != 0) {
        double lo = round((sb[0] * fac) * (sb[0] * fac));
        double hi = round((sb[ns] * fac) * (sb[ns] * fac));
        if (lo <= MAXINT_ && hi <= MAXINT_ &&
            (size_t) hi - (size_t) lo <= LUT_INT_MAX) {
          for (int i = 0; i <= ns; i++) {
            sb[i] = round(sb[i] * fac);
            s2[i] = sb[i] * sb[i];
          }
          hybrid = 0;
        }
      }
    }
    if (hybrid) {
      double s2max = sb[ns] * sb[ns];
      fac = pow(FLT_RADIX, logb(LUT_HYB_MAX / s2max));
      while (fac * s2max > LUT_HYB_MIN * 2) fac *= 0.5;
      for (int i = 0; i <= ns; i++) {
        sb[i] *= fac;
        s2[i] = sb[i] * sb[i];
      }
    }
  } else {
    if (!cfg->sedges && !cfg->pedges) {
      double v[4] = {cfg->smin, cfg->ds, cfg->pmin, cfg->dpi};
      fac = fac_quad(v);
      if (fac != 0) {
        double a1 = round((sb[0] * fac) * (sb[0] * fac));
        double a2 = round((sb[ns] * fac) * (sb[ns] * fac));
        if (a1 <= MAXINT_ && a2 <= MAXINT_) {
          double q1 = pb[0] * fac, q2 = pb[np] * fac;
          size_t nts = (size_t) a2 - (size_t) a1;
          size_t ntp = (size_t) q2 - (size_t) q1;
          if (nts <= LUT_INT_MAX && ntp <= LUT_INT_MAX) {
            for (int i = 0; i <= ns; i++) {
              sb[i] = round(sb[i] * fac);
              s2[i] = sb[i] * sb[i];
            }
            for (int i = 0; i <= np; i++) {
              pb[i] = round(pb[i] * fac);
              p2[i] = pb[i] * pb[i];
            }
            hybrid = 0;
          }
        }
      }
    }
    if (hybrid) {
      double s2max = sb[ns] * sb[ns];
      double pm = pb[np];
      if (!box) pm *= pm;
      double larger = (s2max >= pm) ? s2max : pm;
      double smaller = (s2max >= pm) ? pm : s2max;
      fac = pow(FLT_RADIX, logb(LUT_HYB_MAX / larger));
      while (fac * smaller > LUT_HYB_MIN * 2) fac *= 0.5;
      for (int i = 0; i <= ns; i++) {
        sb[i] *= fac;
        s2[i] = sb[i] * sb[i];
      }
      for (int i = 0; i <= np; i++) {
        pb[i] *= fac;
        p2[i] = pb[i] * pb[i];
      }
    }
  }
  b->rescale = fac;
  if (box)
    for (int k = 0; k < 3; k++) {
      b->box_raw[k] = cfg->box[k];
      b->box[k] = cfg->box[k] * fac;
    }
  /* a bit-pattern s table pays in a box (log bins; the kernels have
   * variants for it); a survey's s_perp^2 = s^2 - pi^2 carries the rounding
   * of s^2, so small s_perp stays ambiguous whatever the table */
  if ((rc = axis_finish(&b->s, s2, ns, hybrid, box)))
    FAIL(rc, "failed to create the separation lookup table");
  if (spi && (rc = axis_finish(&b->p, box ? pb : p2, np, hybrid, 0)))
    FAIL(rc, "failed to create the pi lookup table");
  free(sb);
  free(s2);
  free(pb);
  free(p2);
  return FCFCG_OK;
fail:
  free(sb);
  free(s2);
  free(pb);
  free(p2);
  fcfcg_bins_release(b);
  return rc;
}
