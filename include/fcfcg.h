/*
 * fcfcg.h -- C ABI of the GB300 pair-counting engine for FCFC's hot path.
 *
 * The engine replaces FCFC's pair counter
 *     int count_pairs(const void *tree1, const void *tree2, CF *cf,
 *                     COUNT *cnt, bool isauto, bool withwt)
 * (src/fcfc/2pt_box/count_func.h:54-59, survey twin src/fcfc/2pt/count_func.h)
 * together with the set-up it depends on (binning, src/fcfc/2pt_box/setup_cf.c and src/fcfc/2pt/setup_cf.c;
 * catalogue rescaling, src/fcfc/2pt_box/build_tree.c and src/fcfc/2pt/build_tree.c) and the post-processing that
 * follows it (normalisation, analytic RR, multipoles, w_p and the pair-count
 * files, src/fcfc/2pt_box/eval_cf.c and save_res.c).
 *
 * Conventions
 *   - Every function returns FCFCG_OK (0) or a negative error code; the codes
 *     mirror FCFC's FCFC_ERR_* (src/util/define_comm.h:218-234) and add
 *     FCFCG_ERR_CUDA / FCFCG_ERR_TIMEOUT / FCFCG_ERR_UNSUPPORTED.
 *   - No exceptions or aborts cross the ABI.  fcfcg_strerror() names a code,
 *     fcfcg_last_error() gives the message of the last failure on a context.
 *   - A context owns all its device memory and one CUDA stream.  Contexts are
 *     thread-compatible, not thread-safe: one host thread per context.
 *   - Host arrays are plain pointers and sizes; nothing here needs a CUDA or
 *     PyTorch header.
 *   - There is no CPU fallback: without a usable CUDA device fcfcg_create()
 *     fails with FCFCG_ERR_CUDA.
 */
#ifndef FCFCG_H
#define FCFCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FCFCG_VERSION "0.1.0"
#define FCFCG_FCFC_VERSION "1.0.1"   /* FCFC version whose files are written */

/* Error codes (FCFC_ERR_* values from src/util/define_comm.h:218-234). */
#define FCFCG_OK                 0
#define FCFCG_ERR_MEMORY        (-1)
#define FCFCG_ERR_ARG           (-2)
#define FCFCG_ERR_FILE          (-3)
#define FCFCG_ERR_CFG           (-4)
#define FCFCG_ERR_DATA          (-21)
#define FCFCG_ERR_CNVT          (-22)
#define FCFCG_ERR_CF            (-24)
#define FCFCG_ERR_SAVE          (-25)
#define FCFCG_ERR_UNKNOWN       (-99)
#define FCFCG_ERR_CUDA          (-100)  /* CUDA runtime failure / no device */
#define FCFCG_ERR_TIMEOUT       (-101)  /* a bounded device wait ran out */
#define FCFCG_ERR_UNSUPPORTED   (-102)  /* configuration outside the engine */

/* BINNING_SCHEME (src/fcfc/2pt_box/define.h:46-48). */
#define FCFCG_BIN_ISO 0
#define FCFCG_BIN_SMU 1
#define FCFCG_BIN_SPI 2

/* Geometry: FCFC_2PT_BOX (periodic) or FCFC_2PT (survey). */
#define FCFCG_GEOM_BOX    0
#define FCFCG_GEOM_SURVEY 1

/* Precision of the separation arithmetic. */
#define FCFCG_PREC_FP32_RECHECK 0  /* FP32 separations, FP64 recheck near edges */
#define FCFCG_PREC_FP64         1  /* every pair in FP64 */

/* Lookup-table kinds (FCFC_LOOKUP_TYPE_*). */
#define FCFCG_TAB_INT    0
#define FCFCG_TAB_HYBRID 1

typedef struct fcfcg_ctx fcfcg_ctx;

/*
 * Binning configuration, as FCFC's keys give it.  Separation (or s_perp)
 * bins are linear from SEP_BIN_MIN / SEP_BIN_SIZE with ns bins when
 * sedges == NULL, otherwise the ns+1 edges SEP_BIN_FILE yields after
 * read_bins (src/fcfc/2pt_box/setup_cf.c:74-119).  Likewise for pi.
 * ns / np for linear bins are the counts conf_verify derives
 * (src/fcfc/2pt_box/load_conf.c:985-995); fcfcg_linear_nbin() computes them.
 */
typedef struct {
  int geometry;          /* FCFCG_GEOM_BOX or FCFCG_GEOM_SURVEY */
  int bintype;           /* BINNING_SCHEME */
  double box[3];         /* BOX_SIZE (box geometry only) */
  int ns;                /* number of s (or s_perp) bins */
  double smin, ds;       /* SEP_BIN_MIN, SEP_BIN_SIZE (linear bins) */
  const double *sedges;  /* ns+1 edges, or NULL for linear bins */
  int nmu;               /* MU_BIN_NUM ((s,mu) only) */
  int np;                /* number of pi bins ((s_perp,pi) only) */
  double pmin, dpi;      /* PI_BIN_MIN, PI_BIN_SIZE (linear bins) */
  const double *pedges;  /* np+1 edges, or NULL */
  int with_mu_one;       /* FCFC built with -DWITH_MU_ONE: mu = 1 counted in
                            the last mu bin, not dropped
                            (src/fcfc/2pt_box/metric_common.c:185-189) */
} fcfcg_binning;

/* Summary of the bin set-up cf_setup would produce. */
typedef struct {
  int ns, nmu, np;
  int64_t ntot;          /* ns * (nmu | np | 1) */
  int tabtype;           /* FCFCG_TAB_INT or FCFCG_TAB_HYBRID */
  double rescale;        /* coordinate rescale factor */
  double box_rescaled[3];
  int64_t nstab, nptab;  /* lookup-table lengths */
  int ftab_cells_per_octave;  /* the FP32 s (or s_perp) window table: cells
                                 per octave of a bit-pattern table (log bins
                                 in a box), 0 for a uniform table */
} fcfcg_bins_info;

/* Counters of the last fcfcg_count() call. */
typedef struct {
  uint64_t candidates;   /* pairs whose separation was evaluated */
  uint64_t in_range;     /* unique pairs that landed in a bin */
  uint64_t rechecked;    /* pairs re-binned in FP64 */
  uint64_t recheck_inline; /* rechecks done inline after the queue filled */
  double ms_grid;        /* device time of the cell-grid build (ms) */
  double ms_count;       /* device time of the counting kernel (ms) */
  double ms_recheck;     /* device time of the recheck kernel (ms) */
  double ms_total;       /* device time of the whole call (ms) */
  int cells_per_smax;    /* grid refinement used */
  int ncell[3];
  int nstencil;
  uint64_t nchunks;
  int precision_used;    /* FCFCG_PREC_*: FP32 windows too wide fall to FP64 */
  uint64_t launches;     /* kernels launched by this context since creation */
  int warp_queue;        /* FP32 kernel: entries of a warp's candidate queue */
} fcfcg_stats;

const char *fcfcg_strerror(int err);
const char *fcfcg_last_error(const fcfcg_ctx *ctx);

/* Number of linear bins conf_verify derives from (min, max, step). */
int fcfcg_linear_nbin(double vmin, double vmax, double step);

/*
 * Create a context for one binning set-up on CUDA device `device` (-1: the
 * current device).  Replaces cf_setup's binning part
 * (src/fcfc/2pt_box/setup_cf.c:599-680, survey src/fcfc/2pt/setup_cf.c).
 * Fails with FCFCG_ERR_CFG where cf_setup/conf_verify would reject the
 * bins (e.g. s_max >= half the box, src/fcfc/2pt_box/load_conf.c:1000-1003).
 */
int fcfcg_create(const fcfcg_binning *cfg, int device, fcfcg_ctx **ctx);
void fcfcg_destroy(fcfcg_ctx *ctx);

/* Host-only bin set-up (no device needed): the same tables fcfcg_create
 * builds, for inspection.  The returned handle is freed with
 * fcfcg_destroy(). */
int fcfcg_create_host(const fcfcg_binning *cfg, fcfcg_ctx **ctx);

int fcfcg_bins_info_get(const fcfcg_ctx *ctx, fcfcg_bins_info *out);
/* Raw (unrescaled) edges: sbin[ns+1], pbin[np+1] (either may be NULL). */
int fcfcg_bins_edges(const fcfcg_ctx *ctx, double *sbin, double *pbin);
/* Reference lookup tables widened to 16 bits (stab[nstab], ptab[nptab]) and
 * the rescaled squared-s edges / (squared for surveys) pi edges. */
int fcfcg_bins_tables(const fcfcg_ctx *ctx, uint16_t *stab, uint16_t *ptab,
    double *s2bin, double *pbin);

/*
 * Load a catalogue into slot (0..7): host FP64 coordinates as FCFC reads them
 * (not rescaled; the engine rescales like tree_create,
 * src/fcfc/2pt_box/build_tree.c:121-131) and optional weights (NULL:
 * unweighted).  Box catalogues must lie in [0, BOX_SIZE) up to rounding.
 * The host arrays are copied; they may be freed after the call.
 */
int fcfcg_load_catalog(fcfcg_ctx *ctx, int slot, size_t n, const double *x,
    const double *y, const double *z, const double *w);

/* Same, from device pointers (FP64, n elements each; w may be NULL). */
int fcfcg_load_catalog_device(fcfcg_ctx *ctx, int slot, size_t n,
    const double *x, const double *y, const double *z, const double *w);

/*
 * One catalogue of a batch (fcfcg_count_batch): a periodic box with its own
 * size, counted for DD with the context's bins.  No reference counterpart as
 * one call: FCFC counts one catalogue per run, so a batch replaces a loop of
 * FCFC_2PT_BOX runs (src/fcfc/2pt_box/fcfc.c:19-82) over mock boxes.
 *   n, x, y, z, w   coordinates as read (FP64) and optional weights; host or
 *                   device pointers (the on_device argument).
 *   box             BOX_SIZE of this catalogue.
 *   icnt / wcnt     host outputs, ntot each: undoubled auto counts (icnt,
 *                   unweighted) or weighted sums (wcnt), as fcfcg_count.
 *   sumw            out: the sum of weights (n when unweighted).
 *   status          out: FCFCG_OK, or this catalogue's error
 *                   (FCFCG_ERR_CFG: s_max or pi_max not below half the box,
 *                   as FCFC's conf_verify rejects it; FCFCG_ERR_DATA:
 *                   points outside the box or non-finite values).
 */
typedef struct {
  size_t n;
  const double *x, *y, *z, *w;
  double box[3];
  int64_t *icnt;
  double *wcnt;
  double sumw;
  int status;
} fcfcg_job;

/*
 * Count DD pairs of many periodic-box catalogues (mocks) with one set of bins
 * in a single persistent FP32 launch: all catalogues are cell-sorted into one
 * array with per-catalogue grids, and the CTAs draw (catalogue, cell chunk)
 * items from one device work counter; ambiguous pairs of every catalogue go
 * through one FP64 recheck.  Box contexts only.  precision FCFCG_PREC_FP64
 * counts the catalogues one after the other with the all-FP64 kernel (the
 * comparison path).  Returns FCFCG_OK when the batch ran (per-catalogue
 * errors are in jobs[i].status), or an error of the whole call.
 */
int fcfcg_count_batch(fcfcg_ctx *ctx, fcfcg_job *jobs, int njobs,
    int withwt, int precision, int on_device);

/* Time fcfcg_count_batch at 1..8 cells per maximum separation (stopping
 * two past the fastest) and keep the fastest for batches of this mean
 * density (as fcfcg_autotune). */
int fcfcg_autotune_batch(fcfcg_ctx *ctx, fcfcg_job *jobs, int njobs,
    int withwt, int on_device, int *best_k, double *best_ms);

/*
 * Fiducial cosmology of FCFC_2PT's coordinate conversion (COORD_CONVERT = T):
 * the keys OMEGA_M, OMEGA_LAMBDA, DE_EOS_W, CMVDST_ERR and Z_CMVDST_FILE
 * (src/fcfc/2pt/load_conf.c:532-536), checked as check_cosmo and conf_verify
 * check them (load_conf.c:700-735, 925-933).
 *   omega_m       0 < omega_m <= 1.
 *   omega_l       >= 0, used when has_omega_l; otherwise flat
 *                 (Omega_Lambda = 1 - omega_m, Omega_k = 0).
 *   dew           dark-energy w <= -1/3; 0 selects -1 (a cosmological
 *                 constant, FCFC's default).
 *   cmvdst_err    integration tolerance >= DBL_EPSILON; 0 selects 1e-8.
 *   nsample, z_sample, d_sample   the (z, comoving distance) table of
 *                 Z_CMVDST_FILE, host arrays in any row order (sorted by z
 *                 inside, stably, as FCFC's timsort does); nsample = 0
 *                 selects Gauss-Legendre integration instead.
 */
typedef struct {
  double omega_m;
  double omega_l;
  int has_omega_l;
  double dew;
  double cmvdst_err;
  size_t nsample;
  const double *z_sample;
  const double *d_sample;
} fcfcg_cosmo;

/*
 * RA, Dec (degrees) and redshift to comoving x, y, z (Mpc/h) on the device,
 * FP64: replaces cnvt_coord (src/fcfc/2pt/cnvt_coord.c:383-441).  With
 * integration the Gauss-Legendre order is chosen as cnvt_legauss_order does
 * (:267-307: the smallest order, from 4, at which consecutive orders agree to
 * cmvdst_err on 128 redshifts spanning the catalogue) and returned in *order
 * (may be NULL; 0 for the spline).  All six arrays are device pointers of n
 * FP64 elements; x/y/zc may alias ra/dec/z.  The call synchronises the
 * context's stream.  Errors: FCFCG_ERR_DATA for a negative or non-finite
 * redshift (FCFC exits on a negative one); FCFCG_ERR_CNVT when the
 * integration does not converge by order 32, the table has fewer than two
 * rows, or a redshift lies outside the table (FCFC would carry an infinite
 * distance on); FCFCG_ERR_CFG for a cosmology FCFC rejects.
 */
int fcfcg_cnvt_coord(fcfcg_ctx *ctx, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const fcfcg_cosmo *cosmo, int *order);

/*
 * Load a catalogue given as RA, Dec, redshift: converted on the device
 * (fcfcg_cnvt_coord), then loaded as fcfcg_load_catalog does — FCFC_2PT's
 * tree_create order (src/fcfc/2pt/build_tree.c:237-262).  Survey contexts
 * only.  *_device takes device pointers.
 */
int fcfcg_load_catalog_radecz(fcfcg_ctx *ctx, int slot, size_t n,
    const double *ra, const double *dec, const double *z, const double *w,
    const fcfcg_cosmo *cosmo);
int fcfcg_load_catalog_radecz_device(fcfcg_ctx *ctx, int slot, size_t n,
    const double *ra, const double *dec, const double *z, const double *w,
    const fcfcg_cosmo *cosmo);

/* Number of objects and sum of weights (n when unweighted) of a slot. */
int fcfcg_catalog_info(const fcfcg_ctx *ctx, int slot, size_t *n,
    double *sumw);

/*
 * Count pairs between slots a and b; replaces count_pairs
 * (src/fcfc/2pt_box/count_func.h:54-59).  isauto: a == b, unordered pairs
 * counted once (not doubled; eval_pairs doubles them).  withwt: weighted
 * sums (catalogues without weights count as unit weights).  Outputs are
 * caller-owned arrays of ntot entries, index s + ns * (mu or pi): icnt for
 * unweighted counts, wcnt for weighted sums (the other may be NULL).
 */
int fcfcg_count(fcfcg_ctx *ctx, int slot_a, int slot_b, int isauto,
    int withwt, int precision, int64_t *icnt, double *wcnt);

/*
 * Count graphs (no reference counterpart): a fixed sequence of counts --
 * typically DD, DR and RR of one survey, the eval_pairs loop of
 * src/fcfc/2pt/eval_cf.c -- captured once as a CUDA graph and replayed.
 * A replay queues, for every item, the sort of its catalogues into the
 * item's cell grid, the chunk list, the count and the FP64 recheck kernels
 * and the copy of the histogram to pinned host memory, with no host
 * synchronisation in between; fcfcg_graph_run then writes each item's
 * icnt or wcnt exactly as fcfcg_count would.  The graph reads the context's
 * catalogue slots when it runs, so reloading them (e.g. a new realisation
 * of the same survey) needs no new graph: each run re-plans the items on
 * the host and captures the graph again, transparently, only when a plan
 * changed (catalogue sizes, bounds, weights, the autotuned grid) or the
 * context reallocated a buffer.  Items use user slots
 * (0 .. FCFCG_MAX_SLOT - 1).
 * Destroy a graph before its context.  fcfcg_stats after a run describes
 * the last item, with ms_total the whole replay.
 */
#define FCFCG_MAX_GRAPH_ITEMS 16

typedef struct {
  int slot_a, slot_b, isauto, withwt;
  int64_t *icnt;      /* ntot: unweighted counts (withwt = 0) */
  double *wcnt;       /* ntot: weighted sums (withwt = 1) */
} fcfcg_count_item;

typedef struct fcfcg_graph fcfcg_graph;

int fcfcg_graph_create(fcfcg_ctx *ctx, const fcfcg_count_item *items,
    int nitem, int precision, fcfcg_graph **graph);
int fcfcg_graph_run(fcfcg_graph *graph);
/* How many times the graph was captured, and kernel launches per run. */
int fcfcg_graph_info(const fcfcg_graph *graph, int *captures,
    uint64_t *launches);
void fcfcg_graph_destroy(fcfcg_graph *graph);

/*
 * Adjoint of the weighted count (no reference counterpart: FCFC has no
 * derivatives).  With C_b = sum over counted pairs (i, j) in bin b of
 * w_i w_j, as fcfcg_count(withwt = 1) returns it, and a cotangent g[ntot]
 * (host), this writes the gradient of sum_b g_b C_b with respect to the
 * weights: dw_a[i] = sum_j w_j g[bin(i, j)] over catalogue a (input order,
 * n_a entries) and, for a cross count, dw_b likewise over catalogue b (may
 * be NULL).  For auto counts every unordered pair feeds both of its points.
 * The pair bins are recomputed, exactly as the count bins them (FP32 windows
 * with the FP64 recheck).  Each product w_j g[b] is rounded once (one
 * FP64 fused multiply-add) to an integer multiple of 2^-S, where S makes
 * max|w| max|g| 2^S <= 2^50; those integers are summed exactly (in
 * 32-bit word pairs, with exact spills to FP64), so every gradient is within
 * n 2^-49 max|w| max|g| (plus the rounding of the final FP64 additions) of
 * the exact sum of its n products.  Catalogues
 * without weights count as unit weights.  Where the count falls back to the
 * all-FP64 kernel (FP32 windows too wide), so does the adjoint, which then
 * sums in FP64.  A non-finite g entry fails with FCFCG_ERR_ARG.
 */
int fcfcg_adjoint(fcfcg_ctx *ctx, int slot_a, int slot_b, int isauto,
    const double *g, double *dw_a, double *dw_b);

int fcfcg_stats_get(const fcfcg_ctx *ctx, fcfcg_stats *out);

/* Grid refinement: cells per maximum separation, 1..8 (0 = automatic:
 * about 24 objects of the first catalogue per cell, counted in the volume
 * it occupies -- for a survey estimated at load time, not its bounding
 * box). */
int fcfcg_set_cells_per_smax(fcfcg_ctx *ctx, int k);

/* Entries of a warp's candidate queue in the FP32 counting kernel: 256,
 * 512 or 1024, or 0 (default) for automatic -- the value fcfcg_autotune
 * found for this binning and density, else the largest queue that keeps
 * the most CTAs per SM.  The counts do not depend on it. */
int fcfcg_set_warp_queue(fcfcg_ctx *ctx, int entries);

/* Capacity of the FP64 recheck queue in pairs.  By default the queue holds
 * 2^25 pairs and grows, after a count that overflowed it, to hold that
 * count's ambiguous pairs (at most 2^28).  A capacity set here (clamped to
 * the allocation) stays, and the queue no longer grows.  Ambiguous pairs
 * beyond it are binned by the FP64 formula inside the counting kernel
 * instead of after it: the counts are the same, only slower.  Meant for
 * tests of that overflow path. */
int fcfcg_set_queue_capacity(fcfcg_ctx *ctx, size_t cap);

/* Unweighted counts in the FP32 kernel: a CTA's shared-memory bins are 32
 * bits wide and take their adds unchecked, so the CTA hands them to the
 * global 64-bit counters before the pairs it may have added since the last
 * hand-over (a chunk of m points with t neighbour points adds at most m t)
 * could pass this threshold, and counts a chunk that alone could pass it
 * in global memory.  1..2^32 - 1, or 0 (default) for 2^32 - 1.  The counts
 * do not depend on it; meant for tests of those two paths. */
int fcfcg_set_hist_handover(fcfcg_ctx *ctx, unsigned long long pairs);

/*
 * Autotune the grid refinement and the kernel's tile for this binning and
 * catalogue pair: times the FP32 count at 1..8 cells per maximum
 * separation (stopping two past the fastest), then at the fastest with a
 * warp candidate queue of 1024, 512 and 256 entries (a smaller queue can
 * free shared memory for another CTA per SM or for L1), and keeps both for
 * catalogues of the same number density (key: log2 of the mean number of
 * objects of the first catalogue within the maximum separation box) and
 * weighting.  Later automatic counts of matching density use them;
 * fcfcg_stats.warp_queue reports the queue a count used.
 */
int fcfcg_autotune(fcfcg_ctx *ctx, int slot_a, int slot_b, int isauto,
    int withwt, int *best_k, double *best_ms);

/* ---------------- post-processing (src/fcfc/2pt_box/eval_cf.c) ----------- */

/* Normalisation of eval_pairs (eval_cf.c:125-149): auto n(n-1) or W(W-1),
 * cross n1*n2 or W1*W2. */
double fcfcg_norm(int isauto, int withwt, double n1_or_w1, double n2_or_w2);

/* Analytic RR per bin for the periodic box (eval_cf.c:220-241). */
int fcfcg_analytic_rr(const fcfcg_ctx *ctx, double *rr);

/* Legendre multipoles of xi(s,mu) (eval_cf.c:326-354): mp[l*ns + s]. */
int fcfcg_multipoles(const fcfcg_ctx *ctx, const double *xi, int npole,
    const int *poles, double *mp);

/* Projected correlation function of xi(s_perp,pi) (eval_cf.c:365-388). */
int fcfcg_wp(const fcfcg_ctx *ctx, const double *xi, double *wp);

/*
 * Write a pair-count file exactly as save_res does
 * (src/fcfc/2pt_box/save_res.c:45-310): ofmt 0 binary, 1 ASCII.
 * ntr[2]/wtr[2]: numbers / weighted numbers of the tracers (the second is
 * ignored for auto pairs).  icnt (unweighted) or wcnt (weighted) are the
 * doubled-for-auto counts FCFC stores.
 */
int fcfcg_write_paircount(const fcfcg_ctx *ctx, const char *fname, int ofmt,
    int isauto, int withwt, const uint64_t ntr[2], const double wtr[2],
    double norm, const double *ncnt, const int64_t *icnt, const double *wcnt);

/* Read the counts back from a binary pair-count file (read_res.c:256-479);
 * checks that the file's bins match the context.  Outputs may be NULL. */
int fcfcg_read_paircount(const fcfcg_ctx *ctx, const char *fname,
    int *isauto, int *withwt, uint64_t ntr[2], double wtr[2], double *norm,
    double *ncnt, int64_t *icnt, double *wcnt);

/*
 * Evaluate a CF_ESTIMATOR expression per bin (eval_cf.c:258-315): pair
 * labels (two capitals, e.g. "DD") stand for the normalised counts of pair
 * k (labels[2k], labels[2k+1]; ncnt[k * ntot + bin]), "@@" for the analytic
 * RR (rr, may be NULL when unused).  Arithmetic as libast: numbers, ( ),
 * unary -, ** , * / %, + -, abs sqrt ln log.  FCFCG_ERR_CFG on a syntax
 * error or an unknown label.
 */
int fcfcg_cf_eval(const char *expr, int npc, const char *labels,
    const double *ncnt, const double *rr, long ntot, double *out);

/* Write xi / multipoles / w_p text files as save_res_ascii does. */
int fcfcg_write_cf(const fcfcg_ctx *ctx, const char *fname, const double *xi);
int fcfcg_write_multipoles(const fcfcg_ctx *ctx, const char *fname,
    int npole, const int *poles, const double *mp);
int fcfcg_write_wp(const fcfcg_ctx *ctx, const char *fname, const double *wp);

/* ---------------- measurement ------------------------------------------- */

/*
 * Measured rate of 32-bit shared-memory atomic adds on CUDA device `device`
 * (-1: the current one), all SMs busy, every lane of a warp on its own bank:
 * the peak the histogram updates of the counting kernels (one per in-range
 * pair, two for weighted sums) are measured against.  Takes a few
 * milliseconds; allocates 4 bytes of device memory for the check.  No
 * counterpart in the reference.
 */
int fcfcg_probe_smem_atomics(int device, double *adds_per_s);

/* ---------------- allocation-free counting ------------------------------ */

/* Bytes of the fixed device scratch fcfcg_count_noalloc works in. */
#define FCFCG_NOALLOC_SCRATCH_BYTES (4u << 20)

/*
 * Unweighted pair counts for callers that cannot allocate device memory:
 * code that runs inside another framework's memory pool (whose allocator
 * owns the device and must not be bypassed), or a host program embedded
 * under a policy that forbids cudaMalloc after start-up.  No counterpart in
 * the reference; it is a variant of the FP64 counting kernel.
 *
 * bins_ctx: a host-only context (fcfcg_create_host) describing the bins; it
 * is only read.  xa/ya/za (na objects) and xb/yb/zb (nb, ignored when
 * isauto) are FP64 device pointers with the coordinates as read (the call
 * rescales them as FCFC does); counts is a device array of ntot int64, set
 * to the undoubled counts of count_pairs.  Every pair is binned by the FP64
 * formula by brute force, so this is meant for modest catalogues.  The
 * work runs on `stream` (a cudaStream_t, NULL for the default stream); the
 * call returns without waiting.
 *
 * The call allocates nothing, host or device.  Its scratch is one static
 * device array of FCFCG_NOALLOC_SCRATCH_BYTES (4 MiB) that every GPU loading
 * the library holds until the process exits; bin set-ups needing more (the
 * 64-bit accumulators of ntot bins plus the lookup tables) are rejected with
 * FCFCG_ERR_UNSUPPORTED.  The scratch is shared by all calls and keeps the
 * last call's contents (the accumulators are cleared at the start of each
 * call), so calls whose work overlaps on a GPU race: order them on one
 * stream.  The first call on a device looks up the device address of the
 * scratch (cudaGetSymbolAddress); make that first call before any stream
 * capture.
 */
int fcfcg_count_noalloc(const fcfcg_ctx *bins_ctx, int isauto, size_t na,
    const double *xa, const double *ya, const double *za, size_t nb,
    const double *xb, const double *yb, const double *zb, long long *counts,
    void *stream);

#ifdef __cplusplus
}
#endif
#endif
