/*
 * fcfcg_internal.h -- structures shared by the C host layer and the CUDA
 * kernels of the pair-counting engine.  Plain C, no CUDA types.
 */
#ifndef FCFCG_INTERNAL_H
#define FCFCG_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include "../../include/fcfcg.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FCFCG_MAX_SLOT 8
#define FCFCG_CHUNK 32            /* chunk length of the FP64 kernel */
#define FCFCG_CHUNK32 64          /* chunk length of the FP32 kernel */
#define FCFCG_MAX_STENCIL 4096
#define FCFCG_FIX_F 51            /* fractional bits of a weight product */
/* FP32 edge-window tables: one uint16 per cell of width w = 2^-shift units
 * of the binned quantity; cell i covers [i w, (i + 1) w). */
#define FCFCG_FTAB_BIN_MASK 0x0FFFu /* bin at the cell start, or "out" */
#define FCFCG_FTAB_LO 0x1000u     /* an edge lies in [i w - w/2, i w] */
#define FCFCG_FTAB_HI 0x2000u     /* an edge lies in [(i+1) w, (i+1) w + w/2] */
#define FCFCG_FTAB_CX1 0x4000u    /* exactly one edge strictly inside */
#define FCFCG_FTAB_CXM 0x8000u    /* several edges strictly inside */
#define FCFCG_FTAB_MAXBIN 4094    /* largest bin index an FP32 table holds */
#define FCFCG_FTAB_MAXLEN 4096    /* cells of an FP32 table */

/*
 * One binned quantity (s^2, s_perp^2, pi or pi^2), as FCFC looks it up:
 * reference table rtab over (int) v - roff with FCFC's integer / hybrid
 * semantics, and the FP32 edge-window table ftab over (int) v - foff.
 */
typedef struct {
  int nbin;
  int tabtype;
  double *edge;          /* nbin + 1 rescaled edges (host) */
  uint16_t *rtab;        /* reference table (host) */
  long nrtab, roff;
  uint16_t *ftab;        /* FP32 window table (host) */
  long nftab, foff;      /* cells, index of the first cell */
  int fshift;            /* cell width 2^fshift units */
  int flog;              /* > 0: cells are the FP32 bit pattern >> flog
                            (2^(23 - flog) cells per octave), for bins
                            that are not linear; 0: uniform cells */
  float *fedge;          /* nbin + 1 edges rounded to FP32 (host) */
  double vmin, vmax;     /* edge[0], edge[nbin] */
  int min0;              /* edge[0] == 0: no lower range check (smin0) */
} fcfcg_axis;

typedef struct {
  int geometry, bintype;
  int ns, nmu, np;
  long ntot;
  double rescale;
  double box[3];         /* rescaled */
  double box_raw[3];     /* as configured */
  double *sbin_raw, *pbin_raw;
  fcfcg_axis s;          /* s^2 (or s_perp^2) */
  fcfcg_axis p;          /* pi (box) or pi^2 (survey) */
  int mu_one;            /* mu = 1 in the last mu bin (WITH_MU_ONE) */
} fcfcg_bins;

int fcfcg_bins_setup(const fcfcg_binning *cfg, fcfcg_bins *b, char *err,
    size_t errlen);
void fcfcg_bins_release(fcfcg_bins *b);
/* Build the FP32 window table of an axis (ftab / foff / nftab); allow_log:
 * a bit-pattern table may replace a uniform one with multi-edge cells. */
int fcfcg_axis_ftab(fcfcg_axis *a, int allow_log);
/* Accessors of the opaque context used by the post-processing code. */
const fcfcg_bins *fcfcg_ctx_bins(const fcfcg_ctx *c);
const double *fcfcg_ctx_box_raw(const fcfcg_ctx *c);

/* ------------------------------------------------------------------------ */
/* Launch parameters of the counting kernels (passed by value).             */

typedef struct {
  /* sorted catalogue on the device */
  const float *l4;       /* float4 per point: local x, y, z, scaled weight */
  const int *wq;         /* int2 per point: round(w 2^30) and the float bits
                            of the remainder, w scaled to |w| <= 1 */
  const double *x, *y, *z, *s, *w;   /* rescaled FP64, |x|^2, weight */
  const uint32_t *id;    /* input index */
  const uint32_t *cstart;/* ncell + 1 */
  int wexp;              /* weights scaled by 2^-wexp */
} fcfcg_dcat;

/* One catalogue of a batch (periodic boxes; all share the bins and the
 * cell stencil, each has its own box, grid and histogram). */
typedef struct {
  int ncell[3];
  uint32_t cell_base;    /* global index of the catalogue's first cell */
  double cw[3];          /* cell widths (rescaled units) */
  double box[3];         /* rescaled box */
  unsigned long long *gcnt;    /* ntot counts */
  unsigned long long *gwt;     /* 2 * ntot: lo, hi words of int128 */
} fcfcg_mock;

typedef struct {
  int geometry, bintype, isauto, withwt;
  int ncell[3];
  double cw[3], lo[3], box[3];
  float cwf[3], lof[3];
  /* stencil: nsten entries of int4 (ox, oy, oz, 0) and float4 (-o * cw) */
  int nsten;
  int nin;          /* the first nin entries: cell pairs within range */
  const int *sten;
  const float *stenD;
  /* chunks: uint4 (cell, first sorted index, count, 0); their number is
   * nchunk, or *nchunk_dev when set (written by an earlier launch) */
  uint32_t nchunk;
  const uint32_t *nchunk_dev;
  const uint32_t *chunks;
  uint32_t *chunk_head;
  fcfcg_dcat A, B;
  /* bins */
  int ns, nmu, np;
  long ntot;
  /* FP32 tables (copied to shared memory) */
  const uint16_t *fs, *fp;
  int nfs, nfp, fsoff, fpoff;
  float fsinv, fpinv;          /* 1 / cell width of the FP32 tables, or
                                  2^-flog for bit-pattern tables */
  int fslog, fplog;            /* the axes' flog (0: uniform cells) */
  float fsamb, fpamb;          /* bit-pattern tables: values below are
                                  ambiguous (the window exceeds the cell) */
  const float *fse, *fpe;      /* FP32 edges (nbin + 1 each) */
  int nsb, npb;                /* bins of the s and pi axes */
  float s_lim, p_lim;          /* values at/above: out of range for sure */
  /* survey (s_perp, pi): a pair with |d.u_b| >= los_p + (los_pr + los_h
   * s^2) / |x_b| (u_b = x_b / |x_b|) has pi >= pi_max for sure; the test
   * is skipped for |x_b|^2 <= los_r2min */
  float los_p, los_pr, los_h, los_r2min;
  float K0, K1, K2;            /* E(s^2) = K2 s^2 + K1 s + K0 */
  /* linear s bins (slin): t = s lin_inv + lin_off, bin floor(t), window
   * lin_A s + lin_B in units of t; lin_k0: bins above it have a lower edge
   * that is a boundary */
  int slin, lin_k0;
  float lin_inv, lin_off, lin_A, lin_B;
  float P0, P1, P2;            /* E(pi) (box) or E(pi^2) (survey) */
  float Q0, Q1, Q2;            /* E(q), q = nmu mu: Q1 / s + Q2 q + Q0 */
  float m2min;                 /* survey: |m|^2 below (next to the observer):
                                  mu and pi^2 are rechecked */
  float tiny;                  /* s^2 below: always recheck */
  float Emax;                  /* E at the top of the s axis (iso, spi) */
  int tzero;                   /* stencil index of the zero offset */
  float fnmu;
  /* FP64 reference binning */
  const uint16_t *rs, *rp;
  long rsoff, rpoff, nrs, nrp;
  int tabtype;
  const double *s2edge, *pedge;
  double s2min, s2max, pmin, pmax;
  int smin0, pmin0;
  int mu_one;                  /* WITH_MU_ONE: clamp the mu bin, not drop */
  /* weights: fixed point with F fractional bits */
  int fixF;
  /* outputs */
  unsigned long long *gcnt;    /* ntot counts */
  unsigned long long *gwt;     /* 2 * ntot: lo, hi words of int128 */
  double *gwd;                 /* ntot FP64 sums (FP64 path) */
  /* recheck queue: uint4 (a, b, code, 0) */
  uint32_t *queue;
  unsigned long long *qcount;  /* fill: 64 bits, so it cannot wrap */
  uint32_t qcap;
  uint32_t qwarp;              /* FP32 kernel: entries of a warp's candidate
                                  queue (256..1024; 0: the launcher picks) */
  unsigned long long *stats;   /* [0] candidates [1] in-range [2] recheck
                                  [3] inline rechecks */
  int hist_smem;               /* histogram in shared memory */
  /* unweighted shared histogram: pairs a CTA adds between hand-overs to
   * the global counters, at most 2^32 - 1 (u32 bins) */
  unsigned long long hs_limit;
  /* batch of catalogues (NULL: one catalogue pair): chunk .w is the
   * catalogue, queue entries carry it too */
  const fcfcg_mock *mocks;
  int nmock;
  /* adjoint of the weighted counts: gadj[ntot] in, FP64 gradients per
   * sorted point out (dA, dB; the same array for auto counts) */
  int adjoint;
  const double *gadj;
  double *dA, *dB;
  /* the FP32 kernel's integer accumulation: gfix[k] = gadj[k] 2^S with S
   * chosen so that every |w g 2^S| <= 2^50; a product w gfix rounds to an
   * int64 and integer sums convert back with gunit = 2^-S */
  const double *gfix;
  double gunit;
} fcfcg_launch;

/* Launchers implemented in the .cu files; return 0 or a CUDA error code. */
/* Rescale, |x|^2, max |w|; with w and wsum, also the sum of the weights in
 * a fixed order (partial: fcfcg_prep_partials() doubles of scratch). */
int fcfcg_k_prep(void *stream, size_t n, const double *x, const double *y,
    const double *z, const double *w, double rescale, int survey,
    double *ox, double *oy, double *oz, double *os, double *ow,
    unsigned long long *wmax_bits, double *partial, double *wsum);
size_t fcfcg_prep_partials(void);
/* Sub-cell bits of a grid of ncell cells holding npoint points: 6 (4 x 4
 * x 4 sub-cells in Morton order within a cell), 3 (2 x 2 x 2) or 0; the
 * sort then uses (ncell << sb) fine counters. */
int fcfcg_grid_sub_bits(size_t ncell, size_t npoint);
/* Counting sort into the grid, cells in order and, within a cell, by
 * sub-cell (sb bits); cstart[0..nc] the cells' first sorted points.
 * Scratch: cell_of (n), fstart and cfill ((nc << sb) + 1 each), scan_tmp
 * (fcfcg_scan_tmp_len((nc << sb) + 1)). */
int fcfcg_k_grid(void *stream, size_t n, const double *x, const double *y,
    const double *z, const double *s, const double *w, int has_w, int wexp,
    const int ncell[3], const double cw[3], const double lo[3], int sb,
    uint32_t *cell_of, uint32_t *cstart, uint32_t *fstart, uint32_t *cfill,
    uint32_t *scan_tmp, size_t scan_tmp_len, float *l4, int *wq, double *sx,
    double *sy, double *sz, double *ss, double *sw, uint32_t *sid);
/* cstart[c] = fstart[c << sb] for c = 0..nc. */
int fcfcg_k_cstart(void *stream, size_t nc, int sb, const uint32_t *fstart,
    uint32_t *cstart);
int fcfcg_k_chunks(void *stream, const uint32_t *cstart, uint32_t ncell,
    uint32_t clen, uint32_t *cchunk, uint32_t *scan_tmp, size_t scan_tmp_len,
    uint32_t *chunks, uint32_t *nchunk_out, const uint32_t *mock_cell_base,
    int nmock);
/* One catalogue of a batch for the preparation kernels: its inputs (device
 * or GPU-readable host memory), its place o in the batch slot, its first
 * tile (tiles of fcfcg_batch_tile() points, numbered across the batch) and,
 * once its range checks pass (live), its grid and weight scale. */
typedef struct {
  const double *x, *y, *z, *w;
  size_t o, n;
  uint32_t tile0;
  int live, wexp;
  int ncell[3];
  uint32_t cell_base;
  double cw[3];
} fcfcg_prep_cat;

size_t fcfcg_batch_tile(void);
/* Every catalogue rescaled into the slot arrays o*; per catalogue a,
 * bstat[8a + 0..5] its bounding box (order-preserving keys, min then max;
 * initialised by the caller to ~0 and 0), bstat[8a + 6] max |w| bits and,
 * with weights, bstat[8a + 7] the weight sum (a double, in a fixed order;
 * partial: ntile doubles of scratch). */
int fcfcg_k_prep_batch(void *stream, const fcfcg_prep_cat *d_cat, int ncat,
    uint32_t ntile, double rescale, int withwt, double *ox, double *oy,
    double *oz, double *ow, unsigned long long *bstat, double *partial);
/* Batch grid: every live catalogue's fine indices (cell numbered from its
 * cell_base, shifted by sb, with the sub-cell) counted into a shared array
 * (k_cell_batch), and its points scattered into the shared sorted arrays
 * after the global scan of the fine counts (k_scatter_batch); the id of
 * slot point i is i. */
int fcfcg_k_cell_batch(void *stream, const fcfcg_prep_cat *d_cat, int ncat,
    uint32_t ntile, int sb, const double *x, const double *y,
    const double *z, uint32_t *cell_of, uint32_t *count);
int fcfcg_k_scatter_batch(void *stream, const fcfcg_prep_cat *d_cat,
    int ncat, uint32_t ntile, int sb, const double *x, const double *y,
    const double *z, const double *w, int has_w, const uint32_t *cell_of,
    const uint32_t *fstart, uint32_t *cfill, float *l4, int *wq, double *sx,
    double *sy, double *sz, double *sw, uint32_t *sid);
/* out[sid[p]] = in[p] for p < n (sorted order back to input order). */
int fcfcg_k_unsort(void *stream, size_t n, const uint32_t *sid,
    const double *in, double *out);
int fcfcg_scan(void *stream, const uint32_t *in, size_t n, uint32_t *out,
    uint32_t *tmp);
/* withwt: 0 unweighted, 1 weighted, 2 adjoint */
size_t fcfcg_k_count32_stage(int nsten, int withwt);
size_t fcfcg_k_count32_tab_bytes(int nfs, int nfp, int nsb, int npb);
int fcfcg_k_bbox(void *stream, size_t n, const double *x, const double *y,
    const double *z, unsigned long long *bits6);
/* The count kernel of a launch.  FP32: L->qwarp 0 lets the launcher pick
 * the warp queue (the largest of 1024 / 512 / 256 entries at the most CTAs
 * per SM); the one used goes to *qwarp_used. */
int fcfcg_k_count(void *stream, const fcfcg_launch *L, int precision,
    int nsm, size_t *smem_used, uint32_t *qwarp_used);
/* Bits of the coarse cells (dim, cells of 1 / inv_cell from lo) that hold
 * an object, and their number (count). */
int fcfcg_k_occupancy(void *stream, size_t n, const double *x,
    const double *y, const double *z, const double lo[3], const int dim[3],
    const double inv_cell[3], uint32_t *bits, size_t nw,
    unsigned long long *count);
/* FP64 recheck of the queued pairs; the kernels read the queue length on
 * the device, nq_bound (>= it) only sizes the grid. */
int fcfcg_k_recheck(void *stream, const fcfcg_launch *L, uint32_t nq_bound);
int fcfcg_k_flush_count(void *stream, const fcfcg_launch *L);
size_t fcfcg_scan_tmp_len(size_t n);
const char *fcfcg_cuda_errstr(int code);

/* RA/Dec/z conversion (cnvt.c host set-up, cnvt.cu kernels). */
typedef struct {
  double om, ol, ok;     /* Omega_m, Omega_Lambda, Omega_k */
  double widx;           /* 3 (1 + w), 0 for a cosmological constant */
  double c01;            /* SPEED_OF_LIGHT * 0.01 */
  int order;             /* Gauss-Legendre order */
} fcfcg_cnvt_par;
int fcfcg_k_zrange(void *stream, size_t n, const double *z,
    unsigned long long *bits2);
int fcfcg_k_cnvt_integr(void *stream, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const fcfcg_cnvt_par *p);
int fcfcg_k_cnvt_spline(void *stream, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const double *zs, const double *ds, const double *ypp, size_t nsp,
    unsigned long long *nbad);
/* Converts n objects on `stream` (device pointers, outputs may alias the
 * inputs); *scratch / *scratch_cap is a device buffer the call may grow;
 * *launches counts kernel launches; a message goes to err. */
int fcfcg_cnvt_device(void *stream, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const fcfcg_cosmo *cosmo, void **scratch, size_t *scratch_cap,
    int *order, long *launches, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
