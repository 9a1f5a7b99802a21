/*
 * epilogue.c -- what FCFC does with the counts after count_pairs returns:
 * normalisation and analytic RR (src/fcfc/2pt_box/eval_cf.c:117-241),
 * Legendre multipoles and w_p (eval_cf.c:326-388, src/math/legpoly.h:45-61),
 * and the pair-count / correlation-function files (save_res.c:45-373,
 * read_res.c:256-479).  The arithmetic is written in the reference's order so
 * the printed values agree digit for digit; the file layouts are FCFC's
 * because other tools read them.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fcfcg_internal.h"

#ifndef M_PI
#define M_PI 0x1.921fb54442d18p+1
#endif


double fcfcg_norm(int isauto, int withwt, double a, double b) {
  (void) withwt;
  if (isauto) return a * (a - 1);
  return a * b;
}

static double legpoly(int ell, double x) {
  if (ell == 0) return 1;
  const double x2 = x * x;
  switch (ell) {
    case 1: return x;
    case 2: return 1.5 * x2 - 0.5;
    case 3: return 2.5 * x * (x2 - 0.6);
    case 4: return 4.375 * x2 * x2 - 3.75 * x2 + 0.375;
    case 5: return 8.75 * x * (0.9 * x2 * x2 - x2 + 0x1.b6db6db6db6dbp-3);
    case 6: return 14.4375 * x2 * x2 * x2 - 19.6875 * x2 * x2 +
                   6.5625 * x2 - 0.3125;
    default: return 0;
  }
}

int fcfcg_analytic_rr(const fcfcg_ctx *c, double *rr) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !rr) return FCFCG_ERR_ARG;
  if (b->geometry != FCFCG_GEOM_BOX) return FCFCG_ERR_ARG;
  const double *L = fcfcg_ctx_box_raw(c);
  if (b->bintype == FCFCG_BIN_SPI) {
    double fac = 2 * M_PI / ((double) L[0] * L[1] * L[2]);
    for (int i = 0; i < b->np; i++) {
      double dpi = b->pbin_raw[i + 1] - b->pbin_raw[i];
      for (int j = 0; j < b->ns; j++)
        rr[j + i * b->ns] = fac * dpi *
            (b->sbin_raw[j + 1] * b->sbin_raw[j + 1] -
             b->sbin_raw[j] * b->sbin_raw[j]);
    }
  } else {
    double fac = 4 * M_PI / (3 * b->nmu * (double) L[0] * L[1] * L[2]);
    for (int i = 0; i < b->ns; i++) {
      double v = fac * (pow(b->sbin_raw[i + 1], 3) - pow(b->sbin_raw[i], 3));
      for (int j = 0; j < b->nmu; j++) rr[i + j * b->ns] = v;
    }
  }
  return FCFCG_OK;
}

int fcfcg_multipoles(const fcfcg_ctx *c, const double *xi, int npole,
    const int *poles, double *mp) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !xi || !mp || npole < 0 || (npole && !poles)) return FCFCG_ERR_ARG;
  if (b->bintype != FCFCG_BIN_SMU) return FCFCG_ERR_ARG;
  for (int l = 0; l < npole; l++)
    if (poles[l] < 0 || poles[l] > 6) return FCFCG_ERR_ARG;
  memset(mp, 0, sizeof(double) * (size_t) npole * b->ns);
  for (int l = 0; l < npole; l++) {
    const int ell = poles[l];
    const double fac = (2 * ell + 1) / (double) b->nmu;
    for (int j = 0; j < b->nmu; j++) {
      const double mu = (j + 0.5) / (double) b->nmu;
      for (int k = 0; k < b->ns; k++)
        mp[k + l * b->ns] += xi[k + j * b->ns] * fac * legpoly(ell, mu);
    }
  }
  return FCFCG_OK;
}

int fcfcg_wp(const fcfcg_ctx *c, const double *xi, double *wp) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !xi || !wp) return FCFCG_ERR_ARG;
  if (b->bintype != FCFCG_BIN_SPI) return FCFCG_ERR_ARG;
  memset(wp, 0, sizeof(double) * b->ns);
  for (int j = 0; j < b->np; j++) {
    const double dpi = b->pbin_raw[j + 1] - b->pbin_raw[j];
    for (int k = 0; k < b->ns; k++) wp[k] += 2 * xi[k + j * b->ns] * dpi;
  }
  return FCFCG_OK;
}

/* ------------------------------------------------------------------------ */
/* Files.                                                                    */

#define OFMT "%.10lg"

static const char *code_name(const fcfcg_bins *b) {
  return b->geometry == FCFCG_GEOM_BOX ? "FCFC_2PT_BOX" : "FCFC_2PT";
}

static int put_rec(FILE *fp, const void *src, uint64_t size) {
  if (fwrite(&size, sizeof size, 1, fp) != 1) return -1;
  if (size && fwrite(src, 1, size, fp) != size) return -1;
  if (fwrite(&size, sizeof size, 1, fp) != 1) return -1;
  return 0;
}

static int write_bin(const fcfcg_bins *b, FILE *fp, int isauto, int withwt,
    const uint64_t ntr[2], const double wtr[2], double norm,
    const double *ncnt, const int64_t *icnt, const double *wcnt) {
  if (fprintf(fp, "# Created by %s v%s (%d) ; format = %d\n", code_name(b),
              FCFCG_FCFC_VERSION, 2, 0) < 0)
    return -1;
  int32_t spec[8];
  spec[0] = 1;                                  /* double precision */
  spec[1] = b->mu_one;                          /* WITH_MU_ONE build */
  spec[2] = (b->geometry == FCFCG_GEOM_BOX);    /* periodic */
  spec[3] = isauto ? 0 : 1;
  spec[4] = withwt ? 1 : 0;
  spec[5] = b->bintype;
  spec[6] = b->ns;
  spec[7] = (b->bintype == FCFCG_BIN_SMU) ? b->nmu :
            (b->bintype == FCFCG_BIN_SPI ? b->np : 0);
  uint64_t ssz = (b->bintype == FCFCG_BIN_ISO ? 7 : 8) * sizeof(int32_t);
  if (put_rec(fp, spec, ssz)) return -1;
  if (b->geometry == FCFCG_GEOM_BOX && put_rec(fp, b->box, 3 * sizeof(double)))
    return -1;
  if (put_rec(fp, b->sbin_raw, (b->ns + 1) * sizeof(double))) return -1;
  if (b->bintype == FCFCG_BIN_SPI &&
      put_rec(fp, b->pbin_raw, (b->np + 1) * sizeof(double)))
    return -1;
  if (isauto) {
    if (withwt) {
      if (put_rec(fp, wtr, sizeof(double))) return -1;
    } else if (put_rec(fp, ntr, sizeof(uint64_t))) {
      return -1;
    }
  } else {
    if (withwt) {
      if (put_rec(fp, wtr, 2 * sizeof(double))) return -1;
    } else if (put_rec(fp, ntr, 2 * sizeof(uint64_t))) {
      return -1;
    }
  }
  if (put_rec(fp, &norm, sizeof(double))) return -1;
  if (put_rec(fp, ncnt, b->ntot * sizeof(double))) return -1;
  if (withwt) return put_rec(fp, wcnt, b->ntot * sizeof(double));
  return put_rec(fp, icnt, b->ntot * sizeof(int64_t));
}

static int write_ascii_pc(const fcfcg_bins *b, FILE *fp, int isauto,
    int withwt, const uint64_t ntr[2], const double wtr[2], double norm,
    const double *ncnt) {
  fprintf(fp, "# Created by %s v%s (%d) ; format = %d\n", code_name(b),
          FCFCG_FCFC_VERSION, 2, 1);
  if (isauto) {
    fprintf(fp, "# Number of tracers: %llu (auto pair counts",
            (unsigned long long) ntr[0]);
    if (withwt) fprintf(fp, ", weighted number: " OFMT " ", wtr[0]);
    fprintf(fp, ")\n");
  } else {
    fprintf(fp, "# Numbers of tracers: %llu and %llu",
            (unsigned long long) ntr[0], (unsigned long long) ntr[1]);
    if (withwt)
      fprintf(fp, " (weighted numbers: " OFMT " and " OFMT " )", wtr[0],
              wtr[1]);
    fprintf(fp, "\n");
  }
  fprintf(fp, "# Normalization (total number of pairs): " OFMT "\n", norm);
  const double *sb = b->sbin_raw;
  if (b->bintype == FCFCG_BIN_SMU) {
    fprintf(fp, "# Columns: s_min(1) s_max(2) mu_min(3) mu_max(4) "
            "normalized_pair_count(5)\n");
    for (int j = 0; j < b->nmu; j++)
      for (int i = 0; i < b->ns; i++)
        fprintf(fp, OFMT " " OFMT " " OFMT " " OFMT " " OFMT "\n", sb[i],
                sb[i + 1], j / (double) b->nmu, (j + 1) / (double) b->nmu,
                ncnt[i + j * b->ns]);
  } else if (b->bintype == FCFCG_BIN_SPI) {
    fprintf(fp, "# Columns: s_perp_min(1) s_perp_max(2) pi_min(3) pi_max(4)"
            " normalized_pair_count(5)\n");
    for (int j = 0; j < b->np; j++)
      for (int i = 0; i < b->ns; i++)
        fprintf(fp, OFMT " " OFMT " " OFMT " " OFMT " " OFMT "\n", sb[i],
                sb[i + 1], b->pbin_raw[j], b->pbin_raw[j + 1],
                ncnt[i + j * b->ns]);
  } else {
    fprintf(fp, "# Columns: s_min(1) s_max(2) normalized_pair_count(3)\n");
    for (int i = 0; i < b->ns; i++)
      fprintf(fp, OFMT " " OFMT " " OFMT "\n", sb[i], sb[i + 1], ncnt[i]);
  }
  return ferror(fp) ? -1 : 0;
}

int fcfcg_write_paircount(const fcfcg_ctx *c, const char *fname, int ofmt,
    int isauto, int withwt, const uint64_t ntr[2], const double wtr[2],
    double norm, const double *ncnt, const int64_t *icnt, const double *wcnt) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !fname || !ncnt || !ntr || (withwt && (!wcnt || !wtr)) ||
      (!withwt && !icnt) || (ofmt != 0 && ofmt != 1))
    return FCFCG_ERR_ARG;
  FILE *fp = fopen(fname, ofmt ? "w" : "wb");
  if (!fp) return FCFCG_ERR_FILE;
  int e = ofmt ? write_ascii_pc(b, fp, isauto, withwt, ntr, wtr, norm, ncnt)
               : write_bin(b, fp, isauto, withwt, ntr, wtr, norm, ncnt, icnt,
                           wcnt);
  if (fclose(fp)) e = -1;
  return e ? FCFCG_ERR_SAVE : FCFCG_OK;
}

static int get_rec(FILE *fp, void *dst, uint64_t want) {
  uint64_t a, z;
  if (fread(&a, sizeof a, 1, fp) != 1 || a != want) return -1;
  if (want && fread(dst, 1, want, fp) != want) return -1;
  if (fread(&z, sizeof z, 1, fp) != 1 || z != a) return -1;
  return 0;
}

int fcfcg_read_paircount(const fcfcg_ctx *c, const char *fname, int *isauto,
    int *withwt, uint64_t ntr[2], double wtr[2], double *norm, double *ncnt,
    int64_t *icnt, double *wcnt) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !fname) return FCFCG_ERR_ARG;
  FILE *fp = fopen(fname, "rb");
  if (!fp) return FCFCG_ERR_FILE;
  int rc = FCFCG_ERR_FILE;
  double *tmp = NULL;
  int ch;
  while ((ch = fgetc(fp)) != EOF && ch != '\n') continue;
  if (ch == EOF) goto done;
  int32_t spec[8] = {0};
  uint64_t ssz = (b->bintype == FCFCG_BIN_ISO ? 7 : 8) * sizeof(int32_t);
  if (get_rec(fp, spec, ssz)) goto done;
  /* spec[0] = 0: a SINGLE_PREC build wrote the box and the edges as float;
   * spec[1] (WITH_MU_ONE) only draws a warning from FCFC
   * (src/fcfc/2pt_box/read_res.c:270-300) */
  if ((spec[0] != 0 && spec[0] != 1) ||
      spec[2] != (b->geometry == FCFCG_GEOM_BOX) || spec[5] != b->bintype ||
      spec[6] != b->ns)
    goto done;
  if (b->bintype == FCFCG_BIN_SMU && spec[7] != b->nmu) goto done;
  if (b->bintype == FCFCG_BIN_SPI && spec[7] != b->np) goto done;
  const int au = (spec[3] == 0), wt = (spec[4] == 1);
  const int sp = (spec[0] == 0);
  const size_t rsz = sp ? sizeof(float) : sizeof(double);
  const double tol = sp ? 1e-5 : 1e-10;          /* FLOAT_TOL, DOUBLE_TOL */
  tmp = malloc(sizeof(double) * (b->ntot > 16 ? b->ntot : 16) +
               sizeof(double) * (b->ns + b->np + 8));
  if (!tmp) {
    rc = FCFCG_ERR_MEMORY;
    goto done;
  }
  float *tf = (float *) tmp;
  if (b->geometry == FCFCG_GEOM_BOX) {
    if (get_rec(fp, tmp, 3 * rsz)) goto done;
    for (int k = 0; k < 3; k++)
      if (fabs((sp ? (double) tf[k] : tmp[k]) - b->box[k]) > tol) goto done;
  }
  if (get_rec(fp, tmp, (b->ns + 1) * rsz)) goto done;
  for (int i = 0; i <= b->ns; i++)
    if (fabs((sp ? (double) tf[i] : tmp[i]) - b->sbin_raw[i]) > tol) goto done;
  if (b->bintype == FCFCG_BIN_SPI) {
    if (get_rec(fp, tmp, (b->np + 1) * rsz)) goto done;
    for (int i = 0; i <= b->np; i++)
      if (fabs((sp ? (double) tf[i] : tmp[i]) - b->pbin_raw[i]) > tol)
        goto done;
  }
  uint64_t t2[2] = {0, 0};
  double w2[2] = {0, 0};
  if (wt) {
    if (get_rec(fp, w2, (au ? 1 : 2) * sizeof(double))) goto done;
  } else if (get_rec(fp, t2, (au ? 1 : 2) * sizeof(uint64_t))) {
    goto done;
  }
  double nm;
  if (get_rec(fp, &nm, sizeof(double))) goto done;
  if (get_rec(fp, tmp, b->ntot * sizeof(double))) goto done;
  if (ncnt) memcpy(ncnt, tmp, b->ntot * sizeof(double));
  if (wt) {
    if (get_rec(fp, tmp, b->ntot * sizeof(double))) goto done;
    if (wcnt) memcpy(wcnt, tmp, b->ntot * sizeof(double));
  } else {
    if (get_rec(fp, tmp, b->ntot * sizeof(int64_t))) goto done;
    if (icnt) memcpy(icnt, tmp, b->ntot * sizeof(int64_t));
  }
  if (isauto) *isauto = au;
  if (withwt) *withwt = wt;
  if (ntr) {
    ntr[0] = t2[0];
    ntr[1] = t2[1];
  }
  if (wtr) {
    wtr[0] = w2[0];
    wtr[1] = w2[1];
  }
  if (norm) *norm = nm;
  rc = FCFCG_OK;
done:
  free(tmp);
  fclose(fp);
  return rc;
}

int fcfcg_write_cf(const fcfcg_ctx *c, const char *fname, const double *xi) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !fname || !xi) return FCFCG_ERR_ARG;
  FILE *fp = fopen(fname, "w");
  if (!fp) return FCFCG_ERR_FILE;
  const double *sb = b->sbin_raw;
  if (b->bintype == FCFCG_BIN_SMU) {
    fprintf(fp, "# Columns: s_min(1) s_max(2) mu_min(3) mu_max(4) xi(5)\n");
    for (int j = 0; j < b->nmu; j++)
      for (int i = 0; i < b->ns; i++)
        fprintf(fp, OFMT " " OFMT " " OFMT " " OFMT " " OFMT "\n", sb[i],
                sb[i + 1], j / (double) b->nmu, (j + 1) / (double) b->nmu,
                xi[i + j * b->ns]);
  } else if (b->bintype == FCFCG_BIN_SPI) {
    fprintf(fp, "# Columns: s_perp_min(1) s_perp_max(2) pi_min(3) pi_max(4)"
            " xi(5)\n");
    for (int j = 0; j < b->np; j++)
      for (int i = 0; i < b->ns; i++)
        fprintf(fp, OFMT " " OFMT " " OFMT " " OFMT " " OFMT "\n", sb[i],
                sb[i + 1], b->pbin_raw[j], b->pbin_raw[j + 1],
                xi[i + j * b->ns]);
  } else {
    fprintf(fp, "# Columns: s_cen(1) s_min(2) s_max(3) xi_iso(4)\n");
    for (int i = 0; i < b->ns; i++)
      fprintf(fp, OFMT " " OFMT " " OFMT " " OFMT "\n",
              (sb[i] + sb[i + 1]) * 0.5, sb[i], sb[i + 1], xi[i]);
  }
  int e = ferror(fp);
  if (fclose(fp)) e = 1;
  return e ? FCFCG_ERR_SAVE : FCFCG_OK;
}

int fcfcg_write_multipoles(const fcfcg_ctx *c, const char *fname, int npole,
    const int *poles, const double *mp) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !fname || !mp || npole < 1 || !poles) return FCFCG_ERR_ARG;
  FILE *fp = fopen(fname, "w");
  if (!fp) return FCFCG_ERR_FILE;
  const double *sb = b->sbin_raw;
  fprintf(fp, "# Columns: s_cen(1) s_min(2) s_max(3)");
  for (int i = 0; i < npole; i++) fprintf(fp, " xi_%d(%d)", poles[i], 4 + i);
  fprintf(fp, "\n");
  for (int i = 0; i < b->ns; i++) {
    fprintf(fp, OFMT " " OFMT " " OFMT, (sb[i] + sb[i + 1]) * 0.5, sb[i],
            sb[i + 1]);
    for (int j = 0; j < npole; j++) fprintf(fp, " " OFMT, mp[i + j * b->ns]);
    fprintf(fp, "\n");
  }
  int e = ferror(fp);
  if (fclose(fp)) e = 1;
  return e ? FCFCG_ERR_SAVE : FCFCG_OK;
}

int fcfcg_write_wp(const fcfcg_ctx *c, const char *fname, const double *wp) {
  const fcfcg_bins *b = fcfcg_ctx_bins(c);
  if (!b || !fname || !wp) return FCFCG_ERR_ARG;
  FILE *fp = fopen(fname, "w");
  if (!fp) return FCFCG_ERR_FILE;
  const double *sb = b->sbin_raw;
  fprintf(fp, "# Columns: s_perp_cen(1) s_perp_min(2) s_perp_max(3) wp(4)\n");
  for (int i = 0; i < b->ns; i++)
    fprintf(fp, OFMT " " OFMT " " OFMT " " OFMT "\n",
            (sb[i] + sb[i + 1]) * 0.5, sb[i], sb[i + 1], wp[i]);
  int e = ferror(fp);
  if (fclose(fp)) e = 1;
  return e ? FCFCG_ERR_SAVE : FCFCG_OK;
}

/* ------------------------------------------------------------------------ */
/* Correlation-function estimators.                                          */

/*
 * FCFC evaluates CF_ESTIMATOR strings per bin with libast after replacing
 * each pair label by its normalised counts and "@@" by the analytic RR
 * (src/fcfc/2pt_box/setup_cf.c:130-215, eval_cf.c:258-315).  This is a
 * recursive-descent evaluator for the arithmetic part of that language:
 * numbers, pair labels, @@, parentheses, unary minus, ** (power), * / %,
 * + -, and the functions abs, sqrt, ln, log (base 10).  Operators bind as
 * in libast: unary minus before **, ** before * / %, then + -.
 */
typedef struct {
  const char *s;
  int npc;
  const char *labels;
  const double *ncnt;
  const double *rr;
  long ntot, bin;
  int err;
} est_t;

static void est_ws(est_t *e) {
  while (*e->s == ' ' || *e->s == '\t') e->s++;
}

static double est_add(est_t *e);

static double est_primary(est_t *e) {
  est_ws(e);
  const char *c = e->s;
  if (*c == '(') {
    e->s++;
    double v = est_add(e);
    est_ws(e);
    if (*e->s != ')') {
      e->err = 1;
      return 0;
    }
    e->s++;
    return v;
  }
  if (c[0] == '@' && c[1] == '@') {
    e->s += 2;
    if (!e->rr) {
      e->err = 2;
      return 0;
    }
    return e->rr[e->bin];
  }
  if (c[0] >= 'A' && c[0] <= 'Z' && c[1] >= 'A' && c[1] <= 'Z') {
    for (int k = 0; k < e->npc; k++) {
      if (e->labels[2 * k] == c[0] && e->labels[2 * k + 1] == c[1]) {
        e->s += 2;
        return e->ncnt[(size_t) k * e->ntot + e->bin];
      }
    }
    e->err = 3;
    return 0;
  }
  static const char *fn[] = {"abs", "sqrt", "ln", "log"};
  for (int k = 0; k < 4; k++) {
    size_t l = strlen(fn[k]);
    if (!strncmp(c, fn[k], l)) {
      const char *d = c + l;
      while (*d == ' ') d++;
      if (*d != '(') break;
      e->s = d;
      double v = est_primary(e);
      switch (k) {
        case 0: return fabs(v);
        case 1: return sqrt(v);
        case 2: return log(v);
        default: return log10(v);
      }
    }
  }
  if ((*c >= '0' && *c <= '9') || *c == '.') {
    char *end;
    double v = strtod(c, &end);
    if (end == c) {
      e->err = 4;
      return 0;
    }
    e->s = end;
    return v;
  }
  e->err = 5;
  return 0;
}

static double est_unary(est_t *e) {
  est_ws(e);
  if (*e->s == '-') {
    e->s++;
    return -est_unary(e);
  }
  if (*e->s == '+') {
    e->s++;
    return est_unary(e);
  }
  return est_primary(e);
}

static double est_pow(est_t *e) {
  double v = est_unary(e);
  est_ws(e);
  if (e->s[0] == '*' && e->s[1] == '*') {
    e->s += 2;
    double r = est_pow(e);
    return pow(v, r);
  }
  return v;
}

static double est_mul(est_t *e) {
  double v = est_pow(e);
  for (;;) {
    est_ws(e);
    char op = *e->s;
    if ((op == '*' && e->s[1] != '*') || op == '/' || op == '%') {
      e->s++;
      double r = est_pow(e);
      v = (op == '*') ? v * r : (op == '/' ? v / r : fmod(v, r));
    } else {
      return v;
    }
  }
}

static double est_add(est_t *e) {
  double v = est_mul(e);
  for (;;) {
    est_ws(e);
    char op = *e->s;
    if (op == '+' || op == '-') {
      e->s++;
      double r = est_mul(e);
      v = (op == '+') ? v + r : v - r;
    } else {
      return v;
    }
  }
}

int fcfcg_cf_eval(const char *expr, int npc, const char *labels,
    const double *ncnt, const double *rr, long ntot, double *out) {
  if (!expr || npc < 0 || (npc && (!labels || !ncnt)) || ntot < 1 || !out)
    return FCFCG_ERR_ARG;
  for (long b = 0; b < ntot; b++) {
    est_t e = {expr, npc, labels, ncnt, rr, ntot, b, 0};
    double v = est_add(&e);
    est_ws(&e);
    if (e.err || *e.s) return FCFCG_ERR_CFG;
    out[b] = v;
  }
  return FCFCG_OK;
}
