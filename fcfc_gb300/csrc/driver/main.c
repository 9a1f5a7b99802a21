/*
 * main.c -- FCFC_2PT_BOX_GPU / FCFC_2PT_GPU: FCFC's command line run flow
 * over the engine's C ABI.
 *
 * The flow of FCFC's main (src/fcfc/2pt_box/fcfc.c:19-82, survey
 * src/fcfc/2pt/fcfc.c): read the configuration (load_conf.c; conf.c here),
 * set up the
 * bins (cf_setup), and for every entry of PAIR_COUNT read the catalogues
 * (tree_create: ASCII reading, RA/Dec/z conversion for FCFC_2PT, rescaling
 * on the device), count the pairs (count_pairs -> fcfcg_count; when the
 * run's catalogues fit the context's 8 slots, all its counts -- DD, DR,
 * RR, ... -- go through one CUDA graph, fcfcg_graph_*), normalise
 * and save them (eval_pairs, save_res) or read an existing pair-count file
 * back (OVERWRITE = 1, check_output); then evaluate CF_ESTIMATOR and write
 * the correlation function, its multipoles or w_p (eval_cf).
 *
 * Built twice by fcfc_gb300/build.py: as FCFC_2PT_BOX_GPU and, with
 * -DFCFCG_SURVEY, as FCFC_2PT_GPU.
 *
 *   FCFC_2PT_BOX_GPU [-c fcfc_2pt_box.conf] [FCFC's options] [--fp64]
 *                    [--with-mu-one] [--no-graph]
 */
#define _POSIX_C_SOURCE 200809L
#include <ctype.h>
#include <pthread.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "../../../include/fcfcg.h"
#include "catalog.h"
#include "conf.h"

#ifdef FCFCG_SURVEY
#define GEOM FCFCG_GEOM_SURVEY
#else
#define GEOM FCFCG_GEOM_BOX
#endif

#define MAXCAT 26

#ifdef FCFCG_SURVEY
#define CNVT(i) (cnvt[(i)])   /* COORD_CONVERT of catalogue i */
#else
#define CNVT(i) 0
#endif

/* ------------------------------------------------------------------------ */

static void check(fcfcg_ctx *ctx, int rc, const char *what) {
  if (rc)
    die("%s: %s (%s)", what, fcfcg_strerror(rc),
        ctx ? fcfcg_last_error(ctx) : "");
}

/* SEP_BIN_FILE / PI_BIN_FILE: (lower, upper) rows -> ns + 1 edges, a
 * discontinuity of more than 1e-10 rejected (setup_cf.c:74-119) */
static double *read_bins(const char *fname, int *nbin) {
  double *lo, *hi;
  size_t n;
  char err[256];
  if (cat_read_table(fname, &lo, &hi, &n, err, sizeof err) || n < 1)
    die("cannot read the bin file `%s'", fname);
  double *e = malloc(sizeof(double) * (n + 1));
  e[0] = lo[0];
  for (size_t i = 1; i < n; i++) {
    if (fabs(lo[i] - hi[i - 1]) > 1e-10) die("discontinuous bins in `%s'", fname);
    e[i] = (lo[i] == hi[i - 1]) ? lo[i] : 0.5 * (lo[i] + hi[i - 1]);
  }
  e[n] = hi[n - 1];
  free(lo);
  free(hi);
  *nbin = (int) n;
  return e;
}

/* Catalogue i read from its ASCII file into host arrays. */
typedef struct {
  const conf_t *C;
  int i, weighted;
  char label;
  double *xyz[3], *w;
  size_t n;
  double secs;      /* reading time */
  int rc;
  char err[512];
} cat_host_t;

static double elapsed(const struct timespec *a, const struct timespec *b) {
  return (double) (b->tv_sec - a->tv_sec) +
         1e-9 * (double) (b->tv_nsec - a->tv_nsec);
}

static void read_cat(cat_host_t *r) {
  const conf_t *C = r->C;
  const int i = r->i;
  const char *pos[3] = {conf_str(C, "POSITION", 3 * i),
                        conf_str(C, "POSITION", 3 * i + 1),
                        conf_str(C, "POSITION", 3 * i + 2)};
  const char *fmtr = conf_str(C, "ASCII_FORMATTER", i);
  const char *cm = conf_str(C, "ASCII_COMMENT", i);
  const char *sel = conf_str(C, "SELECTION", i);
  struct timespec t0, t1;
  r->w = NULL;
  if (!fmtr || !*fmtr) {
    snprintf(r->err, sizeof r->err,
             "ASCII_FORMATTER is not set for catalogue %c", r->label);
    r->rc = 1;
    return;
  }
  clock_gettime(CLOCK_MONOTONIC, &t0);
  r->rc = cat_read_ascii(conf_str(C, "CATALOG", i), fmtr, pos,
                         r->weighted ? conf_str(C, "WEIGHT", i) : NULL,
                         (sel && *sel) ? sel : NULL,
                         conf_long(C, "ASCII_SKIP", i, 0),
                         (cm && *cm) ? cm[0] : 0, r->xyz, &r->w, &r->n,
                         r->err, sizeof r->err);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  r->secs = elapsed(&t0, &t1);
}

/* Host catalogue -> a slot of the context; the host arrays are freed. */
static void upload_cat(fcfcg_ctx *ctx, cat_host_t *r, int slot, int cnvt,
    const fcfcg_cosmo *cosmo, int verbose) {
  if (r->rc) die("%s", r->err);
  struct timespec t1, t2;
  clock_gettime(CLOCK_MONOTONIC, &t1);
  int rc;
  if (cnvt)
    rc = fcfcg_load_catalog_radecz(ctx, slot, r->n, r->xyz[0], r->xyz[1],
                                   r->xyz[2], r->w, cosmo);
  else
    rc = fcfcg_load_catalog(ctx, slot, r->n, r->xyz[0], r->xyz[1], r->xyz[2],
                            r->w);
  check(ctx, rc, "loading a catalogue");
  for (int k = 0; k < 3; k++) free(r->xyz[k]);
  free(r->w);
  clock_gettime(CLOCK_MONOTONIC, &t2);
  if (verbose)
    printf("catalogue %c: %zu objects (read %.3f s, to the device %.3f s)\n",
           r->label, r->n, r->secs, elapsed(&t1, &t2));
}

static void load_cat(fcfcg_ctx *ctx, const conf_t *C, int i, int slot,
    int weighted, int cnvt, const fcfcg_cosmo *cosmo, char label,
    int verbose) {
  cat_host_t r;
  memset(&r, 0, sizeof r);
  r.C = C;
  r.i = i;
  r.weighted = weighted;
  r.label = label;
  read_cat(&r);
  upload_cat(ctx, &r, slot, cnvt, cosmo, verbose);
}

/* The catalogues of a run, read one after another on a helper thread while
 * the main thread sets up the device (CUDA context, tables). */
typedef struct {
  cat_host_t *r;
  int n;
} prefetch_t;

static void *prefetch_run(void *p) {
  prefetch_t *P = (prefetch_t *) p;
  for (int k = 0; k < P->n; k++) read_cat(P->r + k);
  return NULL;
}

static int cmp_int(const void *a, const void *b) {
  const int x = *(const int *) a, y = *(const int *) b;
  return (x > y) - (x < y);
}

/* eval_pairs after the count: double auto counts, normalise, write the
 * pair-count file (src/fcfc/2pt_box/eval_cf.c:117-167). */
static void finish_pair(fcfcg_ctx *ctx, const char *fn, int ofmt, int isauto,
    int wt, int sa, int sb, long ntot, int64_t *icnt, double *wcnt,
    double *nc) {
  size_t na, nb;
  double wa, wbs;
  fcfcg_catalog_info(ctx, sa, &na, &wa);
  fcfcg_catalog_info(ctx, sb, &nb, &wbs);
  const double norm = wt ? fcfcg_norm(isauto, 1, wa, wbs)
                         : fcfcg_norm(isauto, 0, (double) na, (double) nb);
  for (long j = 0; j < ntot; j++) {
    if (wt) {
      if (isauto) wcnt[j] *= 2;
      nc[j] = wcnt[j] / norm;
    } else {
      if (isauto) icnt[j] *= 2;
      nc[j] = (double) icnt[j] / norm;
    }
  }
  uint64_t ntr[2] = {na, nb};
  double wtr[2] = {wa, wbs};
  check(ctx, fcfcg_write_paircount(ctx, fn, ofmt, isauto, wt, ntr, wtr, norm,
                                   nc, wt ? NULL : icnt, wt ? wcnt : NULL),
        "writing a pair-count file");
}

int main(int argc, char **argv) {
  struct timespec t_start, t_now;
  clock_gettime(CLOCK_MONOTONIC, &t_start);
  int fp64 = 0, mu_one = 0, graph = 1;
  conf_t C = {0};
  conf_parse_args(&C, argc, argv, &fp64, &mu_one, &graph);
  const int prec = fp64 ? FCFCG_PREC_FP64 : FCFCG_PREC_FP32_RECHECK;
  /* the configuration file: CONFIG_FILE, else FCFC's default name; one that
   * cannot be read leaves the command line's values alone, as in FCFC
   * (src/fcfc/2pt_box/load_conf.c:535-540) */
  const char *cfile = conf_str(&C, "CONFIG_FILE", 0);
  if (!cfile || !*cfile) cfile = DEFAULT_CONF;
  FILE *cfp = fopen(cfile, "r");
  if (cfp) {
    fclose(cfp);
    conf_read(&C, cfile);
  } else {
    fprintf(stderr, "Warning: cannot access the configuration file: `%s'\n",
            cfile);
  }
  /* VERBOSE defaults to T, as in FCFC (src/fcfc/2pt_box/define.h:119) */
  const char *vb = conf_str(&C, "VERBOSE", 0);
  const int verbose = (vb && *vb) ? is_true(vb) : 1;

  /* catalogues */
  const int ncat = conf_len(&C, "CATALOG");
  if (ncat < 1 || ncat > MAXCAT) die("CATALOG must list 1 to 26 catalogues");
  char label[MAXCAT];
  for (int i = 0; i < ncat; i++) {
    const char *l = conf_str(&C, "CATALOG_LABEL", i);
    label[i] = (conf_len(&C, "CATALOG_LABEL") && l) ? l[0] : (char) ('A' + i);
    /* capital letters, each once (load_conf.c:675-705) */
    if (label[i] < 'A' || label[i] > 'Z')
      die("invalid CATALOG_LABEL: %c", label[i]);
    for (int j = 0; j < i; j++)
      if (label[j] == label[i]) die("duplicate CATALOG_LABEL: %c", label[i]);
  }
  for (int i = 0; i < ncat; i++) {
    const char *t = conf_str(&C, "CATALOG_TYPE", i);
    if (t && strtol(t, NULL, 10) != 0)
      die("only ASCII catalogues (CATALOG_TYPE = 0) are supported");
    /* load_conf.c:738-773 */
    if (conf_long(&C, "ASCII_SKIP", i, 0) < 0)
      die("ASCII_SKIP cannot be negative");
    const char *cm = conf_str(&C, "ASCII_COMMENT", i);
    if (cm && cm[0] && !isgraph((unsigned char) cm[0]))
      die("invalid ASCII_COMMENT: '%c' (ASCII code: %d)", cm[0], cm[0]);
  }
  if (conf_len(&C, "POSITION") != 3 * ncat)
    die("POSITION needs 3 entries per catalogue");

  /* bins */
  fcfcg_binning b;
  memset(&b, 0, sizeof b);
  b.geometry = GEOM;
  /* DATA_STRUCT: FCFC's k-d tree (0) or ball tree (1); both map to the
   * engine's cell grid, other values are rejected as FCFC does
   * (load_conf.c:825-834) */
  {
    const long ds = conf_long(&C, "DATA_STRUCT", 0, 0);
    if (ds != 0 && ds != 1) die("invalid DATA_STRUCT: %ld", ds);
  }
  b.bintype = (int) conf_long(&C, "BINNING_SCHEME", 0, 0);
  b.with_mu_one = mu_one;
  double *sedges = NULL, *pedges = NULL;
#ifndef FCFCG_SURVEY
  {
    int nb = conf_len(&C, "BOX_SIZE");
    if (nb != 1 && nb != 3) die("BOX_SIZE needs 1 or 3 numbers");
    for (int k = 0; k < 3; k++)
      b.box[k] = strtod(conf_str(&C, "BOX_SIZE", nb == 1 ? 0 : k), NULL);
  }
#endif
  if (conf_str(&C, "SEP_BIN_FILE", 0)) {
    sedges = read_bins(conf_str(&C, "SEP_BIN_FILE", 0), &b.ns);
    b.sedges = sedges;
  } else {
    b.smin = conf_dbl(&C, "SEP_BIN_MIN", 0);
    b.ds = conf_dbl(&C, "SEP_BIN_SIZE", 0);
    b.ns = fcfcg_linear_nbin(b.smin, conf_dbl(&C, "SEP_BIN_MAX", 0), b.ds);
    if (b.ns < 1) die("invalid SEP_BIN_MIN / SEP_BIN_MAX / SEP_BIN_SIZE");
  }
  if (b.bintype == FCFCG_BIN_SMU) b.nmu = (int) conf_long(&C, "MU_BIN_NUM", 0, 0);
  if (b.bintype == FCFCG_BIN_SPI) {
    if (conf_str(&C, "PI_BIN_FILE", 0)) {
      pedges = read_bins(conf_str(&C, "PI_BIN_FILE", 0), &b.np);
      b.pedges = pedges;
    } else {
      b.pmin = conf_dbl(&C, "PI_BIN_MIN", 0);
      b.dpi = conf_dbl(&C, "PI_BIN_SIZE", 0);
      b.np = fcfcg_linear_nbin(b.pmin, conf_dbl(&C, "PI_BIN_MAX", 0), b.dpi);
      if (b.np < 1) die("invalid PI_BIN_MIN / PI_BIN_MAX / PI_BIN_SIZE");
    }
  }
  /* the pairs, and which catalogues the counts need -- decided before the
   * device set-up, so that reading the catalogues can overlap it */
  const int npair = conf_len(&C, "PAIR_COUNT");
  if (npair < 1) die("PAIR_COUNT is not set");
  if (conf_len(&C, "PAIR_COUNT_FILE") < npair)
    die("PAIR_COUNT_FILE needs one file per pair");
  const int ofmt = (int) conf_long(&C, "OUTPUT_FORMAT", 0, 0);
  const int ovw = (int) conf_long(&C, "OVERWRITE", 0, 0);
  char labels[2 * 64 + 1];
  int weighted[MAXCAT];
  for (int i = 0; i < ncat; i++) {
    const char *w = conf_str(&C, "WEIGHT", i);
    /* an empty weight or "1" means no weights (load_conf.c:780-789) */
    weighted[i] = (conf_len(&C, "WEIGHT") && w && *w && strcmp(w, "1"));
  }
  if (npair > 64) die("too many pairs");
  /* pairs with an existing file (OVERWRITE <= 1) are read back */
  int pia[64], pib[64], todo[64], ntodo = 0, existing[64];
  for (int k = 0; k < npair; k++) {
    const char *pr = conf_str(&C, "PAIR_COUNT", k);
    const char *fn = conf_str(&C, "PAIR_COUNT_FILE", k);
    if (!pr || strlen(pr) != 2) die("invalid PAIR_COUNT entry `%s'", pr ? pr : "");
    labels[2 * k] = pr[0];
    labels[2 * k + 1] = pr[1];
    /* a pair read back from its file needs no catalogue
     * (load_conf.c:877-896) */
    existing[k] = check_output(fn, "PAIR_COUNT_FILE", ovw, 2);
    int ia = -1, ib = -1;
    for (int i = 0; i < ncat; i++) {
      if (label[i] == pr[0]) ia = i;
      if (label[i] == pr[1]) ib = i;
    }
    if (!existing[k] && (ia < 0 || ib < 0))
      die("unknown catalogue label in PAIR_COUNT `%s'", pr);
    pia[k] = ia;
    pib[k] = ib;
    if (!existing[k]) todo[ntodo++] = k;
  }
  /* the correlation function outputs (load_conf.c:899-965): one file per
   * estimator, checked like the pair-count files; multipoles sorted, without
   * duplicates, between 0 and 6 */
  const int nest = conf_len(&C, "CF_ESTIMATOR");
  int npole = 0, poles[7];
  const int dowp = (b.bintype == FCFCG_BIN_SPI) &&
                   is_true(conf_str(&C, "PROJECTED_CF", 0));
  if (nest > 0) {
    /* each estimator parses and names only counted pairs (setup_cf.c:
     * 128-200): evaluated once on zero counts before any device work */
    double zero[64] = {0}, dummy;
#ifdef FCFCG_SURVEY
    const double *rr0 = NULL;       /* no analytic RR for surveys */
#else
    const double rr_zero = 0, *rr0 = &rr_zero;
#endif
    for (int e = 0; e < nest; e++) {
      const char *ex = conf_str(&C, "CF_ESTIMATOR", e);
      if (!ex || !*ex) die("unexpected empty CF_ESTIMATOR");
      if (fcfcg_cf_eval(ex, npair, labels, zero, rr0, 1, &dummy))
        die("invalid CF_ESTIMATOR `%s' (a syntax error, or a pair not in "
            "PAIR_COUNT)", ex);
    }
    const char *outk[3] = {"CF_OUTPUT_FILE", NULL, NULL};
    if (b.bintype == FCFCG_BIN_SMU && conf_len(&C, "MULTIPOLE") > 0) {
      const int nin = conf_len(&C, "MULTIPOLE");
      int *pl = malloc(sizeof(int) * (size_t) nin);
      if (!pl) die("out of memory");
      for (int j = 0; j < nin; j++)
        pl[j] = (int) strtol(conf_str(&C, "MULTIPOLE", j), NULL, 10);
      qsort(pl, (size_t) nin, sizeof(int), cmp_int);
      if (pl[0] < 0 || pl[nin - 1] > 6)
        die("MULTIPOLE must be between 0 and 6");
      for (int j = 0; j < nin; j++)
        if (j == 0 || pl[j] != pl[j - 1]) poles[npole++] = pl[j];
      free(pl);
      outk[1] = "MULTIPOLE_FILE";
    }
    if (dowp) outk[2] = "PROJECTED_FILE";
    for (int q = 0; q < 3; q++) {
      if (!outk[q]) continue;
      const int nf = conf_len(&C, outk[q]);
      if (nf == 0) die("%s is not set", outk[q]);
      if (nf < nest) die("too few elements of %s", outk[q]);
      for (int e = 0; e < nest; e++)
        check_output(conf_str(&C, outk[q], e), outk[q], ovw, 1);
    }
  }
  /* the catalogues the counts need, in order of first use */
  int slot_of[MAXCAT], use[MAXCAT], nuse = 0;
  for (int i = 0; i < ncat; i++) slot_of[i] = -1;
  for (int t = 0; t < ntodo; t++) {
    const int need[2] = {pia[todo[t]], pib[todo[t]]};
    for (int q = 0; q < 2; q++)
      if (slot_of[need[q]] < 0) {
        slot_of[need[q]] = nuse;
        use[nuse++] = need[q];
      }
  }
  /* every count at once when the catalogues fit the context's 8 slots:
   * they are read on a helper thread meanwhile */
  const int at_once = (ntodo > 0 && nuse <= 8 && graph);
  cat_host_t pre[8];
  prefetch_t pf = {pre, at_once ? nuse : 0};
  pthread_t pf_tid;
  int pf_started = 0;
  memset(pre, 0, sizeof pre);
  for (int u = 0; u < pf.n; u++) {
    pre[u].C = &C;
    pre[u].i = use[u];
    pre[u].weighted = weighted[use[u]];
    pre[u].label = label[use[u]];
  }
  if (pf.n > 0) pf_started = !pthread_create(&pf_tid, NULL, prefetch_run, &pf);

  fcfcg_ctx *ctx = NULL;
  int rc = fcfcg_create(&b, -1, &ctx);
  check(ctx, rc, "bin set-up");
  if (verbose) {
    clock_gettime(CLOCK_MONOTONIC, &t_now);
    printf("bins and device set up at %.3f s\n", elapsed(&t_start, &t_now));
  }
  fcfcg_bins_info info;
  check(ctx, fcfcg_bins_info_get(ctx, &info), "bin set-up");
  const long ntot = (long) info.ntot;

#ifdef FCFCG_SURVEY
  /* coordinate conversion */
  int cnvt[MAXCAT] = {0};
  fcfcg_cosmo cosmo;
  memset(&cosmo, 0, sizeof cosmo);
  double *zs = NULL, *zd = NULL;
  {
    int nc = conf_len(&C, "COORD_CONVERT"), any = 0;
    if (nc > 1 && nc < ncat) die("too few elements of COORD_CONVERT");
    for (int i = 0; i < ncat && nc; i++)
      any |= (cnvt[i] = is_true(conf_str(&C, "COORD_CONVERT", nc == 1 ? 0 : i)));
    if (any) {
      const char *zf = conf_str(&C, "Z_CMVDST_FILE", 0);
      if (zf && *zf) {
        char err[256];
        size_t ns;
        if (cat_read_table(zf, &zs, &zd, &ns, err, sizeof err)) die("%s", err);
        cosmo.nsample = ns;
        cosmo.z_sample = zs;
        cosmo.d_sample = zd;
      } else {
        if (!conf_str(&C, "OMEGA_M", 0)) die("OMEGA_M is not set");
        cosmo.omega_m = conf_dbl(&C, "OMEGA_M", 0);
        if (conf_str(&C, "OMEGA_LAMBDA", 0)) {
          cosmo.has_omega_l = 1;
          cosmo.omega_l = conf_dbl(&C, "OMEGA_LAMBDA", 0);
        }
        cosmo.dew = conf_dbl(&C, "DE_EOS_W", 0);
        cosmo.cmvdst_err = conf_dbl(&C, "CMVDST_ERR", 0);
      }
    }
  }
#endif

  double *ncnt_all = calloc((size_t) npair * ntot, sizeof(double));
  int64_t *icnt = malloc(sizeof(int64_t) * ntot);
  double *wcnt = malloc(sizeof(double) * ntot);
  double *tmp = malloc(sizeof(double) * ntot);
  if (!ncnt_all || !icnt || !wcnt || !tmp) die("out of memory");
  for (int k = 0; k < npair; k++) {
    if (!existing[k]) continue;
    int au, ww;
    uint64_t nt[2];
    double wtr[2], norm;
    check(ctx, fcfcg_read_paircount(ctx, conf_str(&C, "PAIR_COUNT_FILE", k),
                                    &au, &ww, nt, wtr, &norm,
                                    ncnt_all + (size_t) k * ntot, icnt, wcnt),
          "reading an existing pair-count file");
    if (verbose)
      printf("read %s from `%s'\n", conf_str(&C, "PAIR_COUNT", k),
             conf_str(&C, "PAIR_COUNT_FILE", k));
  }
  const fcfcg_cosmo *cs = NULL;
#ifdef FCFCG_SURVEY
  cs = &cosmo;
#endif
  if (at_once) {
    /* every count at once: the catalogues in slots 0 .. nuse - 1, the
     * counts (DD, DR, RR, ...) captured and run as one CUDA graph */
    if (pf_started) pthread_join(pf_tid, NULL);
    else prefetch_run(&pf);
    if (verbose) {
      clock_gettime(CLOCK_MONOTONIC, &t_now);
      printf("catalogues read at %.3f s\n", elapsed(&t_start, &t_now));
    }
    for (int u = 0; u < nuse; u++)
      upload_cat(ctx, pre + u, u, CNVT(use[u]), cs, verbose);
    fcfcg_count_item items[64];
    int64_t *ic = malloc(sizeof(int64_t) * (size_t) ntodo * ntot);
    double *wc = malloc(sizeof(double) * (size_t) ntodo * ntot);
    if (!ic || !wc) die("out of memory");
    for (int t = 0; t < ntodo; t++) {
      const int k = todo[t];
      memset(items + t, 0, sizeof items[t]);
      items[t].slot_a = slot_of[pia[k]];
      items[t].slot_b = slot_of[pib[k]];
      items[t].isauto = (pia[k] == pib[k]);
      items[t].withwt = weighted[pia[k]] || weighted[pib[k]];
      if (items[t].withwt) items[t].wcnt = wc + (size_t) t * ntot;
      else items[t].icnt = ic + (size_t) t * ntot;
    }
    fcfcg_graph *gr = NULL;
    check(ctx, fcfcg_graph_create(ctx, items, ntodo, prec, &gr),
          "capturing the counts");
    check(ctx, fcfcg_graph_run(gr), "counting pairs");
    if (verbose) {
      fcfcg_stats st;
      fcfcg_stats_get(ctx, &st);
      clock_gettime(CLOCK_MONOTONIC, &t_now);
      printf("%d counts in one CUDA graph: %.3f ms on the device, done at "
             "%.3f s\n", ntodo, st.ms_total, elapsed(&t_start, &t_now));
    }
    fcfcg_graph_destroy(gr);
    for (int t = 0; t < ntodo; t++) {
      const int k = todo[t];
      finish_pair(ctx, conf_str(&C, "PAIR_COUNT_FILE", k), ofmt,
                  items[t].isauto, items[t].withwt, items[t].slot_a,
                  items[t].slot_b, ntot, ic + (size_t) t * ntot,
                  wc + (size_t) t * ntot, ncnt_all + (size_t) k * ntot);
    }
    free(ic);
    free(wc);
  } else {
    /* one count at a time, catalogue i in slot i % 8 */
    int loaded[MAXCAT] = {0};
    for (int t = 0; t < ntodo; t++) {
      const int k = todo[t], ia = pia[k], ib = pib[k];
      const char *pr = conf_str(&C, "PAIR_COUNT", k);
      const int need[2] = {ia, ib};
      for (int q = 0; q < 2; q++) {
        const int i = need[q];
        if (loaded[i]) continue;
        load_cat(ctx, &C, i, i % 8, weighted[i], CNVT(i), cs, label[i],
                 verbose);
        /* slots are per catalogue index modulo 8: drop what this evicts */
        for (int j = 0; j < ncat; j++)
          if (j != i && j % 8 == i % 8) loaded[j] = 0;
        loaded[i] = 1;
      }
      if (!loaded[ia] || !loaded[ib])
        die("catalogues %c and %c share a slot: at most 8 catalogues per pair "
            "set", label[ia], label[ib]);
      const int sa = ia % 8, sb = ib % 8, isauto = (ia == ib);
      const int wt = weighted[ia] || weighted[ib];
      rc = fcfcg_count(ctx, sa, sb, isauto, wt, prec, icnt, wcnt);
      check(ctx, rc, "counting pairs");
      if (verbose) {
        fcfcg_stats st;
        fcfcg_stats_get(ctx, &st);
        printf("%s: %llu pairs in range, %.3f ms on the device\n", pr,
               (unsigned long long) st.in_range, st.ms_total);
      }
      finish_pair(ctx, conf_str(&C, "PAIR_COUNT_FILE", k), ofmt, isauto, wt,
                  sa, sb, ntot, icnt, wcnt, ncnt_all + (size_t) k * ntot);
    }
  }

  /* correlation functions */
  double *rr = NULL;
#ifndef FCFCG_SURVEY
  rr = malloc(sizeof(double) * ntot);
  check(ctx, fcfcg_analytic_rr(ctx, rr), "analytic RR");
#endif
  for (int e = 0; e < nest; e++) {
    const char *ex = conf_str(&C, "CF_ESTIMATOR", e);
    check(ctx, fcfcg_cf_eval(ex, npair, labels, ncnt_all, rr, ntot, tmp),
          "CF_ESTIMATOR");
    check(ctx, fcfcg_write_cf(ctx, conf_str(&C, "CF_OUTPUT_FILE", e), tmp),
          "writing CF_OUTPUT_FILE");
    if (npole > 0) {
      double *mp = malloc(sizeof(double) * npole * b.ns);
      check(ctx, fcfcg_multipoles(ctx, tmp, npole, poles, mp), "multipoles");
      check(ctx, fcfcg_write_multipoles(ctx, conf_str(&C, "MULTIPOLE_FILE", e),
                                        npole, poles, mp),
            "writing MULTIPOLE_FILE");
      free(mp);
    } else if (dowp) {
      double *wp = malloc(sizeof(double) * b.ns);
      check(ctx, fcfcg_wp(ctx, tmp, wp), "w_p");
      check(ctx, fcfcg_write_wp(ctx, conf_str(&C, "PROJECTED_FILE", e), wp),
            "writing PROJECTED_FILE");
      free(wp);
    }
  }
  if (verbose) {
    clock_gettime(CLOCK_MONOTONIC, &t_now);
    printf("done at %.3f s\n", elapsed(&t_start, &t_now));
  }
  fcfcg_destroy(ctx);
  free(rr);
  free(ncnt_all);
  free(icnt);
  free(wcnt);
  free(tmp);
  free(sedges);
  free(pedges);
#ifdef FCFCG_SURVEY
  free(zs);
  free(zd);
#endif
  return 0;
}
