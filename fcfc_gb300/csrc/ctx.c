/*
 * ctx.c -- host side of the engine: contexts, catalogues, the cell grid and
 * its stencil, the FP32 rounding bounds, and the count driver that replaces
 * FCFC's count_pairs (src/fcfc/2pt_box/count_func.c:4847-7725 and the survey
 * twin src/fcfc/2pt/count_func.c:4846).  C99 on the CUDA runtime C API.
 */
#include <cuda_runtime_api.h>
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fcfcg_internal.h"

typedef struct {
  size_t n, cap;
  int has_w;
  double sumw, wmax;
  int wexp;
  double *x, *y, *z, *s, *w;       /* rescaled FP64 (device) */
  double xabs, s2abs;              /* max |coordinate|, max |x|^2 (host) */
  double bmin[3], bmax[3];         /* bounding box (rescaled) */
  double vol;                      /* survey: occupied volume (rescaled) */
  /* sorted copy for the current grid */
  size_t scap;
  float *l4;
  int *wq;
  double *sx, *sy, *sz, *ss, *sw;
  uint32_t *sid, *cell_of;
  uint32_t *cstart;
  size_t ccap;
  int grid_valid;
  int gsig_n[3];
  double gsig_cw[3], gsig_lo[3];
} slot_t;

struct fcfcg_ctx {
  fcfcg_bins bins;
  int host_only;
  int device, nsm;
  int pageable;                  /* kernels may read pageable host memory */
  cudaStream_t stream;
  char err[512];
  int kcell;
  slot_t slot[FCFCG_MAX_SLOT + 1];   /* the last one holds batches */
  /* shared scratch */
  uint32_t *cfill, *scan_tmp, *cchunk, *chunks;
  size_t cfill_cap, scan_cap, cchunk_cap, chunk_cap;
  uint32_t *fstart;               /* fine (sub-cell) starts of a grid sort */
  size_t fstart_cap;
  uint16_t *d_fs, *d_fp, *d_rs, *d_rp;
  float *d_fse, *d_fpe;
  double *d_s2edge, *d_pedge;
  int *d_sten;
  float *d_stenD;
  unsigned long long *d_cnt, *d_wt, *d_stats, *d_bbox;
  double *d_wd;
  double *d_gfix;                /* adjoint: the scaled cotangent */
  uint32_t *d_head, *d_queue;      /* d_head: chunk counter, pad, fill */
  unsigned long long *d_qcount;    /* queue fill (64-bit), in d_head */
  size_t qcap, qcap_alloc;
  int qcap_user;                  /* capacity set by fcfcg_set_queue_capacity */
  void *h_pinned;
  size_t h_pinned_cap;
  fcfcg_stats stats;
  uint64_t launches;
  cudaEvent_t ev[5];
  int sten[4 * FCFCG_MAX_STENCIL];
  float stD[4 * FCFCG_MAX_STENCIL];
  /* autotuned grid refinement, keyed on the expected neighbours per object */
  int tuned_k;
  int tuned_key;
  /* FP32 kernel's warp queue: forced (fcfcg_set_warp_queue), or autotuned
   * for a key and weighting, else the launcher's choice; the last used */
  uint32_t qwarp_force, tuned_q, last_qwarp;
  /* hand-over threshold of the unweighted shared histogram (0: 2^32 - 1) */
  unsigned long long hs_limit;
  int tuned_q_key, tuned_q_wt;
  /* RA/Dec/z conversion scratch */
  void *d_cnvt;
  size_t cnvt_cap;
  int cnvt_order;
  /* batches */
  int internal;                  /* the batch slot may be addressed */
  fcfcg_mock *h_mock;
  size_t h_mock_cap;
  void *d_mock;
  size_t d_mock_cap;
  uint32_t *d_mbase;
  size_t d_mbase_cap;
  fcfcg_prep_cat *h_pcat;        /* the preparation kernels' catalogue table */
  size_t h_pcat_cap;
  void *d_pcat;
  size_t d_pcat_cap;
  double *d_bpart;               /* per-tile weight sums of a batch */
  size_t d_bpart_cap;
  double *d_wpart;               /* weight-sum partials; [0] the sum */
  double *d_grad;                /* adjoint: sorted and input-order gradients */
  size_t d_grad_cap;
  unsigned long long *d_bout, *d_bstat;
  size_t d_bout_cap, d_bstat_cap;
  /* bumped whenever a catalogue is loaded or a device buffer is
   * reallocated: count graphs captured before are stale */
  unsigned long bufgen;
};

static void set_err(fcfcg_ctx *c, const char *fmt, ...) {
  if (!c) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(c->err, sizeof c->err, fmt, ap);
  va_end(ap);
}

#define CK(call)                                                          \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      set_err(c, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
              __LINE__);                                                  \
      return FCFCG_ERR_CUDA;                                              \
    }                                                                     \
  } while (0)

#define CKK(call)                                                         \
  do {                                                                    \
    int e_ = (call);                                                      \
    if (e_) {                                                             \
      set_err(c, "%s: %s", #call, fcfcg_cuda_errstr(e_));                 \
      return FCFCG_ERR_CUDA;                                              \
    }                                                                     \
  } while (0)

const char *fcfcg_strerror(int err) {
  switch (err) {
    case FCFCG_OK: return "success";
    case FCFCG_ERR_MEMORY: return "memory allocation failed";
    case FCFCG_ERR_ARG: return "invalid argument";
    case FCFCG_ERR_FILE: return "file error";
    case FCFCG_ERR_CFG: return "invalid configuration";
    case FCFCG_ERR_DATA: return "invalid catalogue data";
    case FCFCG_ERR_CNVT: return "coordinate conversion failed";
    case FCFCG_ERR_CF: return "correlation function set-up failed";
    case FCFCG_ERR_SAVE: return "failed to save results";
    case FCFCG_ERR_CUDA: return "CUDA error";
    case FCFCG_ERR_TIMEOUT: return "device wait timed out";
    case FCFCG_ERR_UNSUPPORTED: return "configuration not supported";
    default: return "unknown error";
  }
}

const char *fcfcg_last_error(const fcfcg_ctx *ctx) {
  return ctx ? ctx->err : "no context";
}

/* Grow a device buffer to at least `need` bytes. */
static int grow(fcfcg_ctx *c, void **p, size_t *cap, size_t need) {
  if (*cap >= need && *p) return FCFCG_OK;
  c->bufgen++;
  if (*p) cudaFree(*p);
  *p = NULL;
  *cap = 0;
  size_t alloc = need ? need : 16;
  CK(cudaMalloc(p, alloc));
  *cap = alloc;
  return FCFCG_OK;
}

#define GROW(ptr, capv, bytes)                                              \
  do {                                                                      \
    size_t cap_ = (capv);                                                   \
    int r_ = grow(c, (void **) &(ptr), &cap_, (bytes));                     \
    if (r_) return r_;                                                      \
    (capv) = cap_;                                                          \
  } while (0)

static int upload(fcfcg_ctx *c, void **dst, const void *src, size_t bytes) {
  if (*dst) cudaFree(*dst);
  *dst = NULL;
  CK(cudaMalloc(dst, bytes ? bytes : 16));
  if (bytes) CK(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice,
                                c->stream));
  return FCFCG_OK;
}

static void slot_free(slot_t *s) {
  void *p[] = {s->x, s->y, s->z, s->s, s->w, s->l4, s->wq, s->sx, s->sy,
               s->sz, s->ss, s->sw, s->sid, s->cell_of, s->cstart};
  for (size_t i = 0; i < sizeof p / sizeof p[0]; i++)
    if (p[i]) cudaFree(p[i]);
  memset(s, 0, sizeof *s);
}

void fcfcg_destroy(fcfcg_ctx *c) {
  if (!c) return;
  if (!c->host_only) {
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int i = 0; i <= FCFCG_MAX_SLOT; i++) slot_free(c->slot + i);
    void *p[] = {c->cfill, c->fstart, c->scan_tmp, c->cchunk, c->chunks, c->d_fse,
                 c->d_fpe, c->d_fs,
                 c->d_fp, c->d_rs, c->d_rp, c->d_s2edge, c->d_pedge,
                 c->d_sten, c->d_stenD, c->d_cnt, c->d_wt, c->d_stats,
                 c->d_bbox, c->d_wd, c->d_gfix, c->d_head, c->d_queue, c->d_cnvt,
                 c->d_mock, c->d_mbase, c->d_bout, c->d_bstat, c->d_grad,
                 c->d_wpart, c->d_pcat, c->d_bpart};
    for (size_t i = 0; i < sizeof p / sizeof p[0]; i++)
      if (p[i]) cudaFree(p[i]);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    for (int i = 0; i < 5; i++)
      if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->stream) cudaStreamDestroy(c->stream);
  }
  fcfcg_bins_release(&c->bins);
  free(c->h_mock);
  free(c->h_pcat);
  free(c);
}

int fcfcg_create_host(const fcfcg_binning *cfg, fcfcg_ctx **out) {
  if (!out) return FCFCG_ERR_ARG;
  *out = NULL;
  fcfcg_ctx *c = calloc(1, sizeof *c);
  if (!c) return FCFCG_ERR_MEMORY;
  c->host_only = 1;
  int rc = fcfcg_bins_setup(cfg, &c->bins, c->err, sizeof c->err);
  if (rc) {
    /* keep the message: hand the context back so the caller can read it */
    *out = c;
    return rc;
  }
  *out = c;
  return FCFCG_OK;
}

int fcfcg_create(const fcfcg_binning *cfg, int device, fcfcg_ctx **out) {
  int rc = fcfcg_create_host(cfg, out);
  if (rc) return rc;
  fcfcg_ctx *c = *out;
  c->host_only = 0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev < 1) {
    set_err(c, "no CUDA device available (%s)",
            e ? cudaGetErrorString(e) : "0 devices");
    c->host_only = 1;
    return FCFCG_ERR_CUDA;
  }
  if (device < 0) CK(cudaGetDevice(&device));
  c->device = device;
  CK(cudaSetDevice(device));
  CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
  /* Grace: the GPU reads the host's pageable memory coherently (at the
   * NVLink-C2C rate), so host catalogues go straight into the preparation
   * kernels instead of through one copy per array */
  CK(cudaDeviceGetAttribute(&c->pageable, cudaDevAttrPageableMemoryAccess,
                            device));
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (int i = 0; i < 5; i++) CK(cudaEventCreate(&c->ev[i]));
  const fcfcg_bins *b = &c->bins;
  /* reference tables and FP32 window tables */
  rc = upload(c, (void **) &c->d_rs, b->s.rtab, sizeof(uint16_t) * b->s.nrtab);
  if (rc) return rc;
  rc = upload(c, (void **) &c->d_s2edge, b->s.edge,
              sizeof(double) * (b->s.nbin + 1));
  if (rc) return rc;
  if (b->s.ftab) {
    rc = upload(c, (void **) &c->d_fs, b->s.ftab, sizeof(uint16_t) * b->s.nftab);
    if (rc) return rc;
    rc = upload(c, (void **) &c->d_fse, b->s.fedge, sizeof(float) * (b->s.nbin + 1));
    if (rc) return rc;
  }
  if (b->bintype == FCFCG_BIN_SPI) {
    rc = upload(c, (void **) &c->d_rp, b->p.rtab, sizeof(uint16_t) * b->p.nrtab);
    if (rc) return rc;
    rc = upload(c, (void **) &c->d_pedge, b->p.edge,
                sizeof(double) * (b->p.nbin + 1));
    if (rc) return rc;
    if (b->p.ftab) {
      rc = upload(c, (void **) &c->d_fp, b->p.ftab,
                  sizeof(uint16_t) * b->p.nftab);
      if (rc) return rc;
      rc = upload(c, (void **) &c->d_fpe, b->p.fedge,
                  sizeof(float) * (b->p.nbin + 1));
      if (rc) return rc;
    }
  }
  CK(cudaMalloc((void **) &c->d_cnt, sizeof(unsigned long long) * b->ntot));
  CK(cudaMalloc((void **) &c->d_wt, sizeof(unsigned long long) * 2 * b->ntot));
  CK(cudaMalloc((void **) &c->d_wd, sizeof(double) * b->ntot));
  CK(cudaMalloc((void **) &c->d_gfix, sizeof(double) * b->ntot));
  CK(cudaMalloc((void **) &c->d_stats, sizeof(unsigned long long) * 8));
  CK(cudaMalloc((void **) &c->d_wpart,
                sizeof(double) * (fcfcg_prep_partials() + 1)));
  CK(cudaMalloc((void **) &c->d_bbox, sizeof(unsigned long long) * 6));
  CK(cudaMalloc((void **) &c->d_head, sizeof(uint32_t) * 4));
  c->d_qcount = (unsigned long long *) (c->d_head + 2);
  c->qcap = c->qcap_alloc = (size_t) 1 << 25;   /* 32M pairs, 512 MiB */
  CK(cudaMalloc((void **) &c->d_queue, sizeof(uint32_t) * 4 * c->qcap));
  CK(cudaStreamSynchronize(c->stream));
  return FCFCG_OK;
}

int fcfcg_bins_info_get(const fcfcg_ctx *c, fcfcg_bins_info *o) {
  if (!c || !o) return FCFCG_ERR_ARG;
  const fcfcg_bins *b = &c->bins;
  if (!b->sbin_raw) return FCFCG_ERR_CF;
  o->ns = b->ns;
  o->nmu = b->nmu;
  o->np = b->np;
  o->ntot = b->ntot;
  o->tabtype = b->s.tabtype;
  o->rescale = b->rescale;
  for (int k = 0; k < 3; k++) o->box_rescaled[k] = b->box[k];
  o->nstab = b->s.nrtab;
  o->nptab = (b->bintype == FCFCG_BIN_SPI) ? b->p.nrtab : 0;
  o->ftab_cells_per_octave = b->s.flog ? 1 << (23 - b->s.flog) : 0;
  return FCFCG_OK;
}

int fcfcg_bins_edges(const fcfcg_ctx *c, double *sbin, double *pbin) {
  if (!c || !c->bins.sbin_raw) return FCFCG_ERR_ARG;
  if (sbin) memcpy(sbin, c->bins.sbin_raw, sizeof(double) * (c->bins.ns + 1));
  if (pbin && c->bins.pbin_raw)
    memcpy(pbin, c->bins.pbin_raw, sizeof(double) * (c->bins.np + 1));
  return FCFCG_OK;
}

int fcfcg_bins_tables(const fcfcg_ctx *c, uint16_t *stab, uint16_t *ptab,
    double *s2bin, double *pbin) {
  if (!c || !c->bins.sbin_raw) return FCFCG_ERR_ARG;
  const fcfcg_bins *b = &c->bins;
  if (stab) memcpy(stab, b->s.rtab, sizeof(uint16_t) * b->s.nrtab);
  if (s2bin) memcpy(s2bin, b->s.edge, sizeof(double) * (b->s.nbin + 1));
  if (b->bintype == FCFCG_BIN_SPI) {
    if (ptab) memcpy(ptab, b->p.rtab, sizeof(uint16_t) * b->p.nrtab);
    if (pbin) memcpy(pbin, b->p.edge, sizeof(double) * (b->p.nbin + 1));
  }
  return FCFCG_OK;
}

int fcfcg_set_cells_per_smax(fcfcg_ctx *c, int k) {
  if (!c || k < 0 || k > 8) return FCFCG_ERR_ARG;
  c->kcell = k;
  for (int i = 0; i <= FCFCG_MAX_SLOT; i++) c->slot[i].grid_valid = 0;
  return FCFCG_OK;
}

int fcfcg_set_warp_queue(fcfcg_ctx *c, int entries) {
  if (!c || !(entries == 0 || entries == 256 || entries == 512 ||
              entries == 1024))
    return FCFCG_ERR_ARG;
  c->qwarp_force = (uint32_t) entries;
  return FCFCG_OK;
}

int fcfcg_set_hist_handover(fcfcg_ctx *c, unsigned long long pairs) {
  if (!c || pairs > 0xFFFFFFFFull) return FCFCG_ERR_ARG;
  c->hs_limit = pairs;
  return FCFCG_OK;
}

int fcfcg_set_queue_capacity(fcfcg_ctx *c, size_t cap) {
  if (!c || c->host_only) return FCFCG_ERR_ARG;
  c->qcap = cap < c->qcap_alloc ? cap : c->qcap_alloc;
  c->qcap_user = 1;
  return FCFCG_OK;
}

/* After a count whose ambiguous pairs overflowed the recheck queue (the
 * overflow is binned inside the counting kernel, one lane at a time): grow
 * the queue for the next counts to a power of two above `need`, at most
 * 2^28 pairs (4 GiB).  Not once a capacity was set explicitly.  Called with
 * the stream idle. */
static void queue_grow(fcfcg_ctx *c, unsigned long long need) {
  if (c->qcap_user || need <= c->qcap_alloc) return;
  size_t cap = c->qcap_alloc;
  while (cap < need && cap < ((size_t) 1 << 28)) cap <<= 1;
  if (cap == c->qcap_alloc) return;
  uint32_t *q = NULL;
  if (cudaMalloc((void **) &q, sizeof(uint32_t) * 4 * cap) != cudaSuccess) {
    cudaGetLastError();         /* keep the present queue */
    return;
  }
  cudaFree(c->d_queue);
  c->d_queue = q;
  c->qcap = c->qcap_alloc = cap;
  c->bufgen++;
}

/* ------------------------------------------------------------------------ */
/* Catalogues.                                                               */

/*
 * The volume a survey catalogue occupies (its bounding box can be several
 * times larger): the cells of a coarse grid over the box, sized to hold
 * ~2 objects at the box's mean density, that hold an object.  With M cells
 * of the footprint and n objects spread over them, K = M (1 - exp(-n / M))
 * cells are occupied on average; M is solved for from the count K.
 */
static int occupied_volume(fcfcg_ctx *c, slot_t *s) {
  double ext[3], V = 1;
  for (int k = 0; k < 3; k++) {
    ext[k] = fmax(s->bmax[k] - s->bmin[k], 1e-9 * fmax(1.0, s->xabs));
    V *= ext[k];
  }
  double cell = cbrt(2.0 * V / (double) s->n);
  int dim[3];
  size_t tot;
  for (;;) {
    tot = 1;
    for (int k = 0; k < 3; k++) {
      double d = ceil(ext[k] / cell);
      dim[k] = (int) (d < 1 ? 1 : (d > 4096 ? 4096 : d));
      tot *= (size_t) dim[k];
    }
    if (tot <= ((size_t) 1 << 24)) break;
    cell *= 1.26;
  }
  double inv[3];
  for (int k = 0; k < 3; k++) inv[k] = dim[k] / ext[k];
  const size_t nw = (tot + 31) / 32;
  GROW(c->cfill, c->cfill_cap, sizeof(uint32_t) * nw);
  unsigned long long *dcount = c->d_stats + 6;
  CKK(fcfcg_k_occupancy(c->stream, s->n, s->x, s->y, s->z, s->bmin, dim, inv,
                        c->cfill, nw, dcount));
  c->launches += 2;
  unsigned long long K = 0;
  CK(cudaMemcpyAsync(&K, dcount, sizeof K, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const double n = (double) s->n, T = (double) tot;
  double M;
  if (T * -expm1(-n / T) <= (double) K) {
    M = T;
  } else {
    double lo = (double) K, hi = T;
    for (int it = 0; it < 100; it++) {
      const double mid = 0.5 * (lo + hi);
      if (mid * -expm1(-n / mid) < (double) K) lo = mid;
      else hi = mid;
    }
    M = 0.5 * (lo + hi);
  }
  s->vol = M * (V / T);
  return FCFCG_OK;
}

static int load_common(fcfcg_ctx *c, int slot, size_t n, const double *x,
    const double *y, const double *z, const double *w, int on_device,
    const fcfcg_cosmo *cosmo) {
  if (!c || c->host_only) return FCFCG_ERR_ARG;
  if (slot < 0 || slot >= FCFCG_MAX_SLOT + c->internal) {
    set_err(c, "slot %d out of range", slot);
    return FCFCG_ERR_ARG;
  }
  if (n > 0xFFFFFFF0u) {
    set_err(c, "catalogue too large (%zu objects)", n);
    return FCFCG_ERR_ARG;
  }
  if (n && (!x || !y || !z)) return FCFCG_ERR_ARG;
  CK(cudaSetDevice(c->device));
  slot_t *s = c->slot + slot;
  const int survey = (c->bins.geometry == FCFCG_GEOM_SURVEY);
  if (s->cap < n || !s->x) {
    c->bufgen++;
    slot_free(s);
    size_t m = n ? n : 1;
    CK(cudaMalloc((void **) &s->x, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->y, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->z, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->s, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->w, sizeof(double) * m));
    s->cap = m;
  }
  s->n = n;
  s->has_w = (w != NULL);
  s->grid_valid = 0;
  double *tx = NULL, *ty = NULL, *tz = NULL, *tw = NULL;
  const double *ix = x, *iy = y, *iz = z, *iw = w;
  if (!on_device && n && !c->pageable) {
    /* stage raw input in the output arrays, then rescale in place */
    CK(cudaMemcpyAsync(s->x, x, sizeof(double) * n, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync(s->y, y, sizeof(double) * n, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync(s->z, z, sizeof(double) * n, cudaMemcpyHostToDevice,
                       c->stream));
    if (w)
      CK(cudaMemcpyAsync(s->w, w, sizeof(double) * n, cudaMemcpyHostToDevice,
                         c->stream));
    ix = tx = s->x;
    iy = ty = s->y;
    iz = tz = s->z;
    iw = w ? (tw = s->w) : NULL;
  }
  (void) tx; (void) ty; (void) tz; (void) tw;
  if (cosmo) {
    /* RA/Dec/z -> comoving x, y, z into the slot's arrays (in place for
     * host input), before rescaling, as tree_create orders them */
    long nl = 0;
    int rc = fcfcg_cnvt_device(c->stream, n, ix, iy, iz, s->x, s->y, s->z,
                               cosmo, &c->d_cnvt, &c->cnvt_cap,
                               &c->cnvt_order, &nl, c->err, sizeof c->err);
    c->launches += (uint64_t) nl;
    if (rc) {
      s->n = 0;
      return rc;
    }
    ix = s->x;
    iy = s->y;
    iz = s->z;
  }
  unsigned long long *wbits = c->d_stats + 7;
  CK(cudaMemsetAsync(wbits, 0, sizeof(unsigned long long), c->stream));
  CKK(fcfcg_k_prep(c->stream, n, ix, iy, iz, iw, c->bins.rescale, survey,
                   s->x, s->y, s->z, s->s, s->w, wbits, c->d_wpart + 1,
                   c->d_wpart));
  c->launches += n ? (w ? 3 : 2) : 0;
  /* bounding box of the rescaled catalogue and max |w| */
  unsigned long long init[6] = {~0ull, ~0ull, ~0ull, 0, 0, 0};
  CK(cudaMemcpyAsync(c->d_bbox, init, sizeof init, cudaMemcpyHostToDevice,
                     c->stream));
  CKK(fcfcg_k_bbox(c->stream, n, s->x, s->y, s->z, c->d_bbox));
  unsigned long long hb[7];
  CK(cudaMemcpyAsync(hb, c->d_bbox, sizeof(unsigned long long) * 6,
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(hb + 6, wbits, sizeof(unsigned long long),
                     cudaMemcpyDeviceToHost, c->stream));
  double wsum = 0;
  if (w && n)
    CK(cudaMemcpyAsync(&wsum, c->d_wpart, sizeof(double),
                       cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double mn[3], mx[3];
  for (int k = 0; k < 3; k++) {
    unsigned long long a = hb[k], bb = hb[3 + k];
    a = (a >> 63) ? (a & 0x7FFFFFFFFFFFFFFFull) : ~a;
    bb = (bb >> 63) ? (bb & 0x7FFFFFFFFFFFFFFFull) : ~bb;
    memcpy(mn + k, &a, 8);
    memcpy(mx + k, &bb, 8);
  }
  s->xabs = 0;
  s->s2abs = 0;
  if (n) {
    for (int k = 0; k < 3; k++) {
      if (!isfinite(mn[k]) || !isfinite(mx[k])) {
        set_err(c, "catalogue in slot %d holds non-finite coordinates", slot);
        return FCFCG_ERR_DATA;
      }
      double a = fmax(fabs(mn[k]), fabs(mx[k]));
      s->xabs = fmax(s->xabs, a);
      s->s2abs += a * a;
      if (c->bins.geometry == FCFCG_GEOM_BOX) {
        const double L = c->bins.box[k];
        const double tol = L * 1e-9;
        if (mn[k] < -tol || mx[k] > L + tol) {
          set_err(c, "catalogue in slot %d leaves the box along axis %d "
                  "([%g, %g] after rescaling, box %g)", slot, k, mn[k],
                  mx[k], L);
          return FCFCG_ERR_DATA;
        }
      }
      s->bmin[k] = mn[k];
      s->bmax[k] = mx[k];
    }
  }
  memcpy(&s->wmax, hb + 6, 8);
  if (!w) s->wmax = 1;
  if (w && !isfinite(s->wmax)) {
    set_err(c, "catalogue in slot %d holds non-finite weights", slot);
    return FCFCG_ERR_DATA;
  }
  s->wexp = (s->wmax > 0) ? (int) ceil(log2(s->wmax)) : 0;
  if (ldexp(1.0, s->wexp) < s->wmax) s->wexp++;
  /* the sum of the weights, summed on the device in a fixed order (FCFC
   * sums with an OpenMP reduction, whose order varies with the threads) */
  s->sumw = w ? wsum : (double) n;
  s->vol = 0;
  if (survey && n) return occupied_volume(c, s);
  return FCFCG_OK;
}

int fcfcg_load_catalog(fcfcg_ctx *c, int slot, size_t n, const double *x,
    const double *y, const double *z, const double *w) {
  return load_common(c, slot, n, x, y, z, w, 0, NULL);
}

int fcfcg_load_catalog_device(fcfcg_ctx *c, int slot, size_t n,
    const double *x, const double *y, const double *z, const double *w) {
  return load_common(c, slot, n, x, y, z, w, 1, NULL);
}

static int radecz_ok(fcfcg_ctx *c, const fcfcg_cosmo *cosmo) {
  if (!c || c->host_only || !cosmo) return FCFCG_ERR_ARG;
  if (c->bins.geometry != FCFCG_GEOM_SURVEY) {
    set_err(c, "coordinate conversion applies to survey catalogues only");
    return FCFCG_ERR_ARG;
  }
  return FCFCG_OK;
}

int fcfcg_load_catalog_radecz(fcfcg_ctx *c, int slot, size_t n,
    const double *ra, const double *dec, const double *z, const double *w,
    const fcfcg_cosmo *cosmo) {
  int rc = radecz_ok(c, cosmo);
  if (rc) return rc;
  return load_common(c, slot, n, ra, dec, z, w, 0, cosmo);
}

int fcfcg_load_catalog_radecz_device(fcfcg_ctx *c, int slot, size_t n,
    const double *ra, const double *dec, const double *z, const double *w,
    const fcfcg_cosmo *cosmo) {
  int rc = radecz_ok(c, cosmo);
  if (rc) return rc;
  return load_common(c, slot, n, ra, dec, z, w, 1, cosmo);
}

int fcfcg_cnvt_coord(fcfcg_ctx *c, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const fcfcg_cosmo *cosmo, int *order) {
  if (!c || c->host_only || !cosmo) return FCFCG_ERR_ARG;
  CK(cudaSetDevice(c->device));
  long nl = 0;
  int rc = fcfcg_cnvt_device(c->stream, n, ra, dec, z, x, y, zc, cosmo,
                             &c->d_cnvt, &c->cnvt_cap, order, &nl, c->err,
                             sizeof c->err);
  c->launches += (uint64_t) nl;
  return rc;
}

int fcfcg_catalog_info(const fcfcg_ctx *c, int slot, size_t *n,
    double *sumw) {
  if (!c || slot < 0 || slot >= FCFCG_MAX_SLOT) return FCFCG_ERR_ARG;
  if (n) *n = c->slot[slot].n;
  if (sumw) *sumw = c->slot[slot].sumw;
  return FCFCG_OK;
}

/* ------------------------------------------------------------------------ */
/* Grid, stencil and bounds.                                                 */

typedef struct {
  int n[3];
  double cw[3], lo[3];
  double reach[3];     /* largest separation along each axis that counts */
  double reach3;       /* largest 3D separation that counts */
  int k;
  int key;             /* autotuning key */
} grid_t;

/* Autotuning key: log2 of the mean number of objects in a reach box. */
static int tune_key(double density, const double reach[3]) {
  double v = density * reach[0] * reach[1] * reach[2];
  return (int) floor(log2(v > 1e-30 ? v : 1e-30) + 0.5);
}

static double box_volume(const double v[3]) { return v[0] * v[1] * v[2]; }

/* Cells per maximum separation: about 24 objects of the chunk side per
 * cell, 1 to 8.  (Timed over k = 1..8 on boxes and surveys of 1e5 to 1e7
 * objects, the fastest refinement held 15 to 50 objects per cell.) */
/* Default refinement: about `per_cell` objects per cell at the given
 * density (timed over k = 1..8: boxes 24 objects of the chunk catalogue;
 * survey s and (s, mu) counts 130 at the geometric mean of the two
 * catalogues' densities in their occupied volumes -- on 1e6 data and 1e7
 * randoms with the packed direct binning, RR fastest at k = 6 (2046 ms,
 * 2324 at the old 8), DR at k = 4 (427 ms, 495 at the old 5); survey
 * (s_perp, pi) counts, which keep the candidate test, 30 of the chunk
 * catalogue: RR at k = 5 (430 ms), DR and DD at k = 2 (100, 5.6 ms)). */
static int pick_k(double density, double reach, double per_cell) {
  const int k = (int) floor(reach * cbrt(density / per_cell) + 0.5);
  return k < 1 ? 1 : (k > 8 ? 8 : k);
}

/* Largest separation that counts, per axis and in 3D (rescaled). */
static void grid_reach(const fcfcg_ctx *c, grid_t *g) {
  const fcfcg_bins *b = &c->bins;
  const int box = (b->geometry == FCFCG_GEOM_BOX);
  double r3;
  if (b->bintype == FCFCG_BIN_SPI) {
    double smax = sqrt(b->s.vmax);
    double pmax = box ? b->p.vmax : sqrt(b->p.vmax);
    r3 = sqrt(b->s.vmax + pmax * pmax);
    if (box) {
      g->reach[0] = g->reach[1] = smax;
      g->reach[2] = pmax;
    } else {
      g->reach[0] = g->reach[1] = g->reach[2] = r3;
    }
  } else {
    r3 = sqrt(b->s.vmax);
    g->reach[0] = g->reach[1] = g->reach[2] = r3;
  }
  g->reach3 = r3;
}

static int grid_setup(fcfcg_ctx *c, grid_t *g, const slot_t *A,
    const slot_t *B) {
  const fcfcg_bins *b = &c->bins;
  const int box = (b->geometry == FCFCG_GEOM_BOX);
  grid_reach(c, g);
  const double r3 = g->reach3;
  double lo[3], hi[3];
  if (box) {
    for (int k = 0; k < 3; k++) {
      lo[k] = 0;
      hi[k] = b->box[k];
    }
  } else {
    for (int k = 0; k < 3; k++) {
      lo[k] = fmin(A->bmin[k], B->bmin[k]);
      hi[k] = fmax(A->bmax[k], B->bmax[k]);
      if (!(hi[k] > lo[k])) hi[k] = lo[k] + 1;
    }
  }
  double ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  double vol = box_volume(ext);
  /* density of the chunk side, in the volume it occupies; surveys take
   * the geometric mean with the neighbour side's */
  const double vbox = vol;
  if (!box && A->vol > 0 && A->vol < vol) vol = A->vol;
  double density = (double) A->n / (vol > 0 ? vol : 1);
  const int spi = (b->bintype == FCFCG_BIN_SPI);
  if (!box && !spi && B != A) {
    double vb = vbox;
    if (B->vol > 0 && B->vol < vb) vb = B->vol;
    density = sqrt(density * ((double) B->n / (vb > 0 ? vb : 1)));
  }
  g->key = tune_key(density, g->reach);
  int k = c->kcell;
  if (!k) k = (c->tuned_k && c->tuned_key == g->key)
                  ? c->tuned_k
                  : pick_k(density, r3, box ? 24.0 : (spi ? 30.0 : 130.0));
  g->k = k;
  const double maxcells = 16.0 * 1024 * 1024;
  double scale = 1;
  for (;;) {
    double tot = 1;
    for (int d = 0; d < 3; d++) {
      /* cells a little wider than reach / k, so that k layers of neighbours
       * cover every separation below the reach */
      double cwt = g->reach[d] / k * scale * (1 + 1e-6);
      int n = (int) floor(ext[d] / cwt);
      if (n < 1) n = 1;
      if (n > 4096) n = 4096;
      g->n[d] = n;
      tot *= n;
    }
    if (tot <= maxcells) break;
    scale *= 1.25;
  }
  for (int d = 0; d < 3; d++) {
    g->lo[d] = lo[d];
    g->cw[d] = box ? b->box[d] / g->n[d] : ext[d] / g->n[d] * (1 + 1e-12);
  }
  return FCFCG_OK;
}

/* Cell offsets whose cell pairs can hold a counted pair; half of them (with
 * the zero offset) for auto counts.  D = -offset * cell width.  The offsets
 * whose cell pairs lie entirely within the counting range (for cells up to
 * cw_far wide; NULL: the grid's) come first, nin of them: their candidates
 * need no distance test (the binning still checks every pair). */
static int stencil_build(fcfcg_ctx *c, const grid_t *g, int isauto, int *sten,
    float *stD, int *nsten, double *dmax, const double *cw_far, int *nin) {
  const fcfcg_bins *b = &c->bins;
  const int box = (b->geometry == FCFCG_GEOM_BOX);
  if (!cw_far) cw_far = g->cw;
  unsigned char *ins = malloc(FCFCG_MAX_STENCIL);
  if (!ins) return FCFCG_ERR_MEMORY;
  const double margin = 1 + 1e-9;
  int r[3];
  for (int d = 0; d < 3; d++) {
    r[d] = (int) ceil(g->reach[d] * margin / g->cw[d]);
    if (!box && r[d] > g->n[d] - 1) r[d] = g->n[d] - 1;
    if (r[d] < 0) r[d] = 0;
  }
  int cnt = 0;
  *dmax = 0;
  for (int oz = -r[2]; oz <= r[2]; oz++)
    for (int oy = -r[1]; oy <= r[1]; oy++)
      for (int ox = -r[0]; ox <= r[0]; ox++) {
        if (isauto) {
          int sgn = oz ? oz : (oy ? oy : ox);
          if (sgn < 0) continue;
        }
        const int o[3] = {ox, oy, oz};
        double gap[3], far[3];
        for (int d = 0; d < 3; d++) {
          int a = abs(o[d]);
          gap[d] = (a > 0 ? a - 1 : 0) * g->cw[d];
          far[d] = (a + 1) * g->cw[d];
        }
        if (b->bintype == FCFCG_BIN_SPI && box) {
          if (gap[2] > b->p.vmax * margin) continue;
          if (gap[0] * gap[0] + gap[1] * gap[1] > b->s.vmax * margin) continue;
          if (!b->s.min0 &&
              far[0] * far[0] + far[1] * far[1] < b->s.vmin / margin)
            continue;
          if (!b->p.min0 && far[2] < b->p.vmin / margin) continue;
        } else {
          double g2 = gap[0] * gap[0] + gap[1] * gap[1] + gap[2] * gap[2];
          if (g2 > g->reach3 * g->reach3 * margin) continue;
          if (b->bintype != FCFCG_BIN_SPI && !b->s.min0) {
            double f2 = far[0] * far[0] + far[1] * far[1] + far[2] * far[2];
            if (f2 < b->s.vmin / margin) continue;
          }
        }
        if (cnt >= FCFCG_MAX_STENCIL) {
          set_err(c, "cell stencil too large");
          free(ins);
          return FCFCG_ERR_UNSUPPORTED;
        }
        /* every pair of the cell pair within range (outer limits only) */
        double fz[3];
        for (int d = 0; d < 3; d++) fz[d] = (abs(o[d]) + 1) * cw_far[d];
        if (b->bintype == FCFCG_BIN_SPI && box)
          ins[cnt] = (fz[0] * fz[0] + fz[1] * fz[1] < b->s.vmax) &&
                     (fz[2] < b->p.vmax);
        else
          ins[cnt] = (fz[0] * fz[0] + fz[1] * fz[1] + fz[2] * fz[2] <
                      ((b->bintype == FCFCG_BIN_SPI) ? b->s.vmax + b->p.vmax
                                                     : b->s.vmax));
        sten[4 * cnt + 0] = ox;
        sten[4 * cnt + 1] = oy;
        sten[4 * cnt + 2] = oz;
        sten[4 * cnt + 3] = 0;
        for (int d = 0; d < 3; d++) {
          double D = -o[d] * g->cw[d];
          stD[4 * cnt + d] = (float) D;
          if (fabs(D) > *dmax) *dmax = fabs(D);
        }
        stD[4 * cnt + 3] = 0;
        cnt++;
      }
  /* the offsets within range first (stable) */
  int *ts = malloc(sizeof(int) * 4 * (cnt ? cnt : 1));
  float *td = malloc(sizeof(float) * 4 * (cnt ? cnt : 1));
  if (!ts || !td) {
    free(ts);
    free(td);
    free(ins);
    return FCFCG_ERR_MEMORY;
  }
  int k = 0;
  for (int pass = 1; pass >= 0; pass--)
    for (int t = 0; t < cnt; t++)
      if (ins[t] == pass) {
        memcpy(ts + 4 * k, sten + 4 * t, sizeof(int) * 4);
        memcpy(td + 4 * k, stD + 4 * t, sizeof(float) * 4);
        k++;
      }
  int n1 = 0;
  for (int t = 0; t < cnt; t++) n1 += ins[t];
  memcpy(sten, ts, sizeof(int) * 4 * cnt);
  memcpy(stD, td, sizeof(float) * 4 * cnt);
  free(ts);
  free(td);
  free(ins);
  *nsten = cnt;
  *nin = n1;
  return FCFCG_OK;
}

/* Sort a slot into the grid (skipped when already sorted for it). */
/* Is slot s sorted into grid g? */
static int slot_in_grid(const slot_t *s, const grid_t *g) {
  const size_t nc = (size_t) g->n[0] * g->n[1] * g->n[2];
  return s->grid_valid && s->ccap >= nc + 1 &&
         !memcmp(s->gsig_n, g->n, sizeof g->n) &&
         !memcmp(s->gsig_cw, g->cw, sizeof g->cw) &&
         !memcmp(s->gsig_lo, g->lo, sizeof g->lo);
}

/* Record that slot s is (or, once queued work ran, will be) in grid g. */
static void slot_mark(slot_t *s, const grid_t *g) {
  memcpy(s->gsig_n, g->n, sizeof g->n);
  memcpy(s->gsig_cw, g->cw, sizeof g->cw);
  memcpy(s->gsig_lo, g->lo, sizeof g->lo);
  s->grid_valid = 1;
}

/* Buffers for sorting slot s into grid g (host side; may allocate). */
static int slot_reserve(fcfcg_ctx *c, slot_t *s, const grid_t *g) {
  const size_t nc = (size_t) g->n[0] * g->n[1] * g->n[2];
  const size_t n = s->n, m = n ? n : 1;
  if (s->scap < m) {
    c->bufgen++;
    void *p[] = {s->l4, s->wq, s->sx, s->sy, s->sz, s->ss, s->sw, s->sid,
                 s->cell_of};
    for (size_t i = 0; i < sizeof p / sizeof p[0]; i++)
      if (p[i]) cudaFree(p[i]);
    CK(cudaMalloc((void **) &s->l4, sizeof(float) * 4 * m));
    CK(cudaMalloc((void **) &s->wq, sizeof(int) * 2 * m));
    CK(cudaMalloc((void **) &s->sx, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->sy, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->sz, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->ss, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->sw, sizeof(double) * m));
    CK(cudaMalloc((void **) &s->sid, sizeof(uint32_t) * m));
    CK(cudaMalloc((void **) &s->cell_of, sizeof(uint32_t) * m));
    s->scap = m;
  }
  if (s->ccap < nc + 1) {
    c->bufgen++;
    if (s->cstart) cudaFree(s->cstart);
    s->cstart = NULL;
    CK(cudaMalloc((void **) &s->cstart, sizeof(uint32_t) * (nc + 1)));
    s->ccap = nc + 1;
  }
  const size_t nf = nc << fcfcg_grid_sub_bits(nc, n);
  GROW(c->cfill, c->cfill_cap, sizeof(uint32_t) * (nf + 1));
  GROW(c->fstart, c->fstart_cap, sizeof(uint32_t) * (nf + 1));
  size_t st = fcfcg_scan_tmp_len(nf + 1) + 16;
  GROW(c->scan_tmp, c->scan_cap, sizeof(uint32_t) * st);
  return FCFCG_OK;
}

/* Queue the sort of slot s into grid g (stream work only). */
static int slot_sort(fcfcg_ctx *c, slot_t *s, const grid_t *g) {
  const size_t nc = (size_t) g->n[0] * g->n[1] * g->n[2];
  const size_t n = s->n;
  const int sb = fcfcg_grid_sub_bits(nc, n);
  size_t st = fcfcg_scan_tmp_len((nc << sb) + 1) + 16;
  const int survey = (c->bins.geometry == FCFCG_GEOM_SURVEY);
  CKK(fcfcg_k_grid(c->stream, n, s->x, s->y, s->z, survey ? s->s : NULL,
                   s->w, s->has_w, s->wexp, g->n, g->cw, g->lo, sb,
                   s->cell_of, s->cstart, c->fstart, c->cfill, c->scan_tmp,
                   st, s->l4, s->wq, s->sx, s->sy, s->sz,
                   survey ? s->ss : NULL, s->sw, s->sid));
  c->launches += n ? 6 : 4;
  return FCFCG_OK;
}

/* Lower end of cell c of a bit-pattern table (FP32 bits c << sh). */
static double ftab_cell_value(long c, int sh) {
  const uint32_t u = (uint32_t) c << sh;
  float f;
  memcpy(&f, &u, 4);
  return (double) f;
}

/* Rounding bounds of the FP32 path; returns 0 when the FP32 windows stay
 * below half a table unit, i.e. the FP32 path applies. */
/*
 * Error windows of the FP32 kernels (every constant below is derived here;
 * the kernels' arithmetic is in count32.cuh bin_pair / lin_bin / mu_bin /
 * ftab_bin).  u = 2^-24, v = 2^-53; CUDA's documented maximum errors:
 * rsqrtf 2 ulp (relative <= 2^-22), __fdividef 2 ulp for divisors in
 * [2^-126, 2^126]; every other FP32 operation is correctly rounded.
 *
 * 1. One separation component.  The reference forms dx_ref = fl(X_a (+
 *    shift) - X_b) from FP64 rescaled coordinates X.  The kernel forms
 *    dx = fl32(l_a - fl32(l_b - D)): l = fl32(fl64(X - c)) is a point's
 *    offset from its FP64 cell centre c (|X - c| <= hw), D = fl32(-o cw)
 *    the cell displacement (|D| <= dmax).  Roundings: l_a, l_b (u hw each),
 *    D (u dmax), l_b - D (u (hw + dmax)), the difference (u |dx| <= u R);
 *    FP64 terms: the centres (3 v |c| each), the box side against n cw
 *    (v L), the reference's own two roundings (v (xabs + L + R)).  So
 *      |dx - dx_ref| <= dc = 1.25 [u (3 hw + 2 dmax + R) + 10 v (xabs + R)].
 * 2. s^2 (and s_perp^2).  The kernel's fma chain is within 3u (2u) of the
 *    exact sum of its squared components; the reference's within 3v of its
 *    own; the components differ by <= dc each, so the exact sums differ by
 *    <= 2 sqrt(3) dc s + 3 dc^2 (Cauchy-Schwarz).  Survey pairs add the
 *    reference's S - t rounding: s_i (3v |x|^2), S (2v sabs), t (6v sabs),
 *    S - t exact (Sterbenz) or v s^2: <= 14 v sabs, carried as refs2 =
 *    64 v sabs.  Hence |s2 - s2_ref| <= E = K2' s^2 + K1 s + K0' with
 *      K2' = 3.0002 u + 3.0001 v   (taken as 4 u),
 *      K1  = 1.1 * 2 sqrt(3) dc    (2 sqrt(2) for s_perp^2; the 1.1 covers
 *            E's own FP32 evaluation and s = s2 rsqrtf(s2) against the
 *            exact root),
 *      K0' = 4 dc^2 + refs2.
 *    The kernel's table lookup of an FP32 value adds the rounding of its
 *    cell position, fl(v / w) (u v), and of 1 - fr against the window
 *    (u w / 2): the table windows use K2 = K2' + u, K0 = K0' + u w.
 * 3. mu in a box: FCFC's bin is floor(sqrt(Q)), Q = fl(fl(dz^2 / s^2)
 *    nmu^2) (the (int) cut and the mu table reduce to that); sqrt(Q) is
 *    within 1.5 v of nmu |dz_ref| / sqrt(s2_ref).  The kernel's q =
 *    fl(fl(nmu |dz|) rsqrtf(s2)) is within 3 2^-23 q (rsqrtf and two
 *    products) of nmu |dz| / sqrt(s2); |dz - dz_ref| <= dc contributes
 *    nmu dc / s, the root of s2 against s2_ref contributes q E / (2 s^2) =
 *    q (K2'/2 + K1 / (2 s) + K0' / (2 s^2)), q <= nmu.  So
 *      Eq = Q1 / s + Q2 q + Q0, Q1 = 1.25 nmu (dc + K1 / 2),
 *      Q2 = 1.25 (K2' / 2 + 2^-21 + 2 v + 2 u), Q0 = 1e-6 + u,
 *    the 1e-6 covering nmu K0' / (2 s^2) <= 5e-7 (pairs with s^2 < tiny =
 *    1e6 K0' nmu are rechecked whatever their value); the kernel tests
 *    the window's ends fl(q -+ Eq), each within u (q + Eq) of q -+ Eq
 *    (Eq < 1/2): the 2 u of Q2 and the u of Q0.
 * 4. Survey mu and pi^2 use the line of sight m = x_a + x_b.  The kernel
 *    forms m = fl(fl(2 b + c2) + d) with b the neighbour's offset from the
 *    chunk cell's centre c and c2 = fl32(2 c) (the centre in FP64, rounded
 *    once): per component |dm| <= 3 dc + 2u |c| + u (|m| + s) + u |m|,
 *    and with |x_a| <= (|m| + s) / 2, |c| <= |x_a| + hw:
 *      |dm| / |m| <= dmr = sqrt(3) (3 dc + 2 u (hw + R)) / |m| +
 *                         3.0001 sqrt(3) u,
 *    bounded by requiring |m| >= 2 R (pairs with |m|^2 < m2min = (2.01
 *    R)^2, i.e. next to the observer, are rechecked).  The direction m/|m|
 *    moves by <= 2 dmr.  The reference's dd = s1 - s2 = d.m carries
 *    6 v sabs, its S + t = |m|^2 carries 8 v sabs.
 *    mu: q = nmu |d.m| / (|m| s): d contributes nmu sqrt(3) dc / s (the
 *    length of d is E's business), m 2 nmu dmr, the kernel's roundings
 *    (dm 3u absolute, mm, the product, rsqrtf, two products: 8u relative)
 *    and the reference's (6 v nmu sabs / (2 R s), 4 v sabs / |m|^2):
 *      Q1 = 1.25 nmu (sqrt(3) dc + K1 / 2 + 3 v sabs / R),
 *      Q2 = 1.25 (K2' / 2 + 8 u + v sabs / R^2 + 2 v + 2 u),
 *      Q0 = 1.25 nmu (3 u + 2 dmr) + 1e-6 + u (the ends, as in a box).
 *    pi^2 = (d.m)^2 / |m|^2: |d pi| <= sqrt(3) dc + s (2 dmr + 3u), so
 *      Ep = P2 s^2 + P1 s + P0, P1 = 1.25 (2 sqrt(3) dc + 6 v sabs / R),
 *      P2 = 1.25 (4 dmr + 14 u + 2 v sabs / R^2 + 2 v + u) (dm^2, mm and
 *      __fdividef: 8u relative; the table position: u),
 *      P0 = 1.25 (6 dc^2 + u w_pi) + 1e-12.
 *    s_perp^2 = s^2 - pi^2 takes E + Ep.
 * 5. pi in a box is |dz|: P0 = 1.25 (dc + u w_pi).
 * Every constant carries a factor >= 1.1 over its derived value; the
 * near-edge tests place pairs on every bin edge and check that each one is
 * rechecked.
 */
static int fp32_bounds(const fcfcg_ctx *c, const grid_t *g, double dmax,
    const slot_t *A, const slot_t *B, fcfcg_launch *L) {
  const fcfcg_bins *b = &c->bins;
  const int box = (b->geometry == FCFCG_GEOM_BOX);
  const double u = ldexp(1.0, -24), v = ldexp(1.0, -53);
  double hw = 0;
  for (int d = 0; d < 3; d++) hw = fmax(hw, 0.5 * g->cw[d] * (1 + 1e-6));
  const double R = g->reach3 * 1.01;
  double xabs = fmax(A->xabs, B->xabs);
  double sabs = fmax(A->s2abs, B->s2abs);
  if (box) xabs = fmax(xabs, fmax(b->box[0], fmax(b->box[1], b->box[2])));
  const double dc = 1.25 * (u * (3 * hw + 2 * dmax + R) + 10 * v * (xabs + R)) +
                    1e-300;
  const double refs2 = box ? 0 : 64 * v * sabs;
  const double s3 = sqrt(3.0);
  /* cell widths of the FP32 tables (uniform ones; 0 for bit patterns) */
  const double ws = b->s.ftab && !b->s.flog ? ldexp(1.0, b->s.fshift) : 0;
  const double wp = (b->bintype == FCFCG_BIN_SPI && b->p.ftab && !b->p.flog)
                        ? ldexp(1.0, b->p.fshift) : 0;
  const double K2a = 4 * u, K0a = 4 * dc * dc + refs2;   /* arithmetic */
  const double K1 = 1.1 * 2 * ((b->bintype == FCFCG_BIN_SPI && box)
                                   ? sqrt(2.0) : s3) * dc;
  L->K2 = (float) (K2a + u);
  L->K1 = (float) K1;
  L->K0 = (float) (K0a + u * ws + 1e-30);
  double nmu = b->nmu;
  L->fnmu = (float) nmu;
  /* survey: relative error of the line of sight for |m| >= 2 R */
  const double dmr = s3 * (3 * dc + 2 * u * (hw + R)) / (2 * R) +
                     3.0001 * s3 * u;
  L->m2min = box ? 0.f : (float) (2.01 * R * 2.01 * R);
  if (box) {
    L->Q1 = (float) (1.25 * nmu * (dc + 0.5 * K1));
    L->Q2 = (float) (1.25 * (0.5 * K2a + ldexp(1.0, -21) + 2 * v + 2 * u));
    L->Q0 = (float) (1e-6 + u);
  } else {
    L->Q1 = (float) (1.25 * nmu * (s3 * dc + 0.5 * K1 + 3 * v * sabs / R));
    L->Q2 = (float) (1.25 * (0.5 * K2a + 8 * u + v * sabs / (R * R) + 2 * v +
                             2 * u));
    L->Q0 = (float) (1.25 * nmu * (3 * u + 2 * dmr) + 1e-6 + u);
  }
  double tiny = 1e6 * K0a * (nmu > 1 ? nmu : 1);
  if (tiny < 1e-20) tiny = 1e-20;
  L->tiny = (float) tiny;
  /*
   * Linear s bins as FCFC's integer table sees them: rescaled edges
   * e_k = a + k d with integers a >= 0, d >= 1, so that the table's edges
   * e_k^2 are integers and FCFC's bin is the k with e_k <= sqrt(s2_ref) <
   * e_k+1.  The kernel then bins s itself: k = floor(t), t = (s - a) / d.
   * Window of t, for a pair with s^2 >= tiny (smaller ones are rechecked):
   *   |s_32 - sqrt(s2_ref)| <= eta s_32 (1 + 2 eta) + E(s) / sqrt(s2_32),
   *   with eta = 2^-22 + 2^-24 (s_32 = fl(s2 rsqrtf(s2)): rsqrtf within 2
   *   ulp, CUDA's documented bound, then the product's rounding), E(s) =
   *   K2 s^2 + K1 s + K0 the bound on |s2_32 - s2_ref| above, and
   *   sqrt(s2_32) >= s_32 / (1 + eta), K0 / s <= K0 / sqrt(tiny);
   *   t = fl(fma(s, fl(1 / d), fl(-a / d))) adds u (s + a) / d + u |t|,
   *   |t| <= ns + 1 where the window matters; the kernel tests the ends
   *   fl(t -+ W), each within u (|t| + W) <= u (ns + 2) of t -+ W (W <
   *   0.45), plus 3 u of slack.  The factor 1.01 covers W's own FP32
   *   evaluation.
   */
  L->slin = 0;
  if (b->bintype != FCFCG_BIN_SPI && b->s.tabtype == FCFCG_TAB_INT &&
      b->s.nbin >= 1) {
    int ok = 1;
    double a = 0, d = 0;
    for (int k = 0; k <= b->s.nbin && ok; k++) {
      const double e = sqrt(b->s.edge[k]);
      if (!(e == floor(e) && e * e == b->s.edge[k] && e < 1e6)) ok = 0;
      else if (k == 0) a = e;
      else if (k == 1) d = e - a;
      else if (e != a + k * d) ok = 0;
    }
    if (ok && d >= 1) {
      const double eta = ldexp(1.0, -22) + ldexp(1.0, -24);
      const double uu = ldexp(1.0, -24);
      const double A = 1.01 * (eta * (1 + 2 * eta) + (double) L->K2 * (1 + eta)
                               + uu) / d;
      const double Bw = 1.01 * (((double) L->K1 + (double) L->K0 /
                                 sqrt((double) L->tiny)) * (1 + eta) / d +
                                uu * a / d + uu * (b->s.nbin + 1) +
                                uu * (b->s.nbin + 2) + 3 * uu);
      const double smax = a + d * b->s.nbin;
      if (A * (smax + d) + Bw < 0.45) {
        L->slin = 1;
        L->lin_inv = (float) (1.0 / d);
        L->lin_off = (float) (-a / d);
        L->lin_A = (float) A;
        if ((double) L->lin_A < A) L->lin_A = nextafterf(L->lin_A, INFINITY);
        L->lin_B = (float) Bw;
        if ((double) L->lin_B < Bw) L->lin_B = nextafterf(L->lin_B, INFINITY);
        L->lin_k0 = b->s.min0 ? 0 : -1;
      }
    }
  }
  /* worst windows at the top of the ranges */
  double smax2 = b->s.vmax;
  double Es = L->K2 * smax2 + L->K1 * sqrt(smax2) + L->K0;
  double Ep = 0;
  if (b->bintype == FCFCG_BIN_SPI) {
    if (box) {
      L->P0 = (float) (1.25 * (dc + u * wp));
      L->P1 = L->P2 = 0;
      Ep = L->P0;
      L->p_lim = (float) (b->p.vmax + Ep + 1e-6 * (1 + b->p.vmax));
      L->s_lim = (float) (smax2 + Es + 1e-6 * (1 + smax2));
    } else {
      double r2 = b->s.vmax + b->p.vmax;
      L->P0 = (float) (1.25 * (6 * dc * dc + u * wp) + 1e-12);
      L->P1 = (float) (1.25 * (2 * s3 * dc + 6 * v * sabs / R));
      L->P2 = (float) (1.25 * (4 * dmr + 15 * u + 2 * v * sabs / (R * R) +
                               2 * v));
      Ep = L->P2 * r2 + L->P1 * sqrt(r2) + L->P0;
      Es = L->K2 * r2 + L->K1 * sqrt(r2) + L->K0 + Ep;
      L->s_lim = (float) (r2 + Es + 1e-6 * (1 + r2));
      L->p_lim = 0;
      /* line-of-sight prefilter.  With m = x_a + x_b = 2 x_b + d,
       * pi = |d.m| / |m| and |m| <= 2 |x_b| + s, pi < pi_max implies
       *   |d.u_b| < pi_max + (pi_max s + s^2) / (2 |x_b|),
       * and s <= Rs, the outer range.  The constants carry a factor
       * 1 + 2^-8 and an absolute slack far above the FP32 rounding of d,
       * u_b and |x_b| (below 1e-5 relative where the test applies,
       * |x_b| >= Rs) */
      const double pm = sqrt(b->p.vmax), Rs = sqrt((double) L->s_lim);
      const double f = 1 + ldexp(1.0, -8);
      L->los_p = (float) (pm * f + ldexp(Rs, -12) + 1e-6);
      L->los_pr = (float) (0.5 * f * pm * Rs);
      L->los_h = (float) (0.5 * f);
      L->los_r2min = (float) (Rs * Rs);
    }
  } else {
    L->s_lim = (float) (smax2 + Es + 1e-6 * (1 + smax2));
  }
  L->Emax = (float) (Es * 1.01);
  if (b->s.nbin > FCFCG_FTAB_MAXBIN || !b->s.ftab) return -1;
  if (b->bintype == FCFCG_BIN_SPI &&
      (b->p.nbin > FCFCG_FTAB_MAXBIN || !b->p.ftab))
    return -1;
  /* windows below half a table cell: over the whole uniform tables; for a
   * bit-pattern table, whose cells shrink with the value, from a threshold
   * up -- values below it are sent to the recheck */
  L->fsamb = L->fpamb = -1.f;
  if (b->s.flog) {
    /* the window the s-axis lookups use at value v (an upper bound): with
     * a bit-pattern table every kernel variant takes it per pair (only
     * boxes get such tables, so p2, for a survey's s_perp^2 = s^2 - pi^2,
     * is 0 today) */
    const double p2 = (b->bintype == FCFCG_BIN_SPI && !box) ? b->p.vmax : 0;
    double amb = -1;
    for (long c = b->s.nftab - 1; c >= 0; c--) {
      const double x0 = ftab_cell_value(b->s.foff + c, b->s.flog);
      const double x1 = ftab_cell_value(b->s.foff + c + 1, b->s.flog);
      const double v = x1 + p2;
      double W = (double) L->K2 * v + (double) L->K1 * sqrt(v) + (double) L->K0;
      if (p2 > 0)
        W += (double) L->P2 * v + (double) L->P1 * sqrt(v) + (double) L->P0;
      W *= 1.01;
      if (!(W < 0.45 * (x1 - x0))) {
        amb = x1;
        break;
      }
    }
    L->fsamb = (float) amb;
    if (amb > 0 && (double) L->fsamb < amb)   /* round up: still ambiguous */
      L->fsamb = nextafterf(L->fsamb, INFINITY);
  } else if (!(Es < 0.45 * ldexp(1.0, b->s.fshift))) {
    return -1;
  }
  if (b->bintype == FCFCG_BIN_SPI) {
    if (b->p.flog) {
      double amb = -1;
      for (long c = b->p.nftab - 1; c >= 0; c--) {
        const double x0 = ftab_cell_value(b->p.foff + c, b->p.flog);
        const double x1 = ftab_cell_value(b->p.foff + c + 1, b->p.flog);
        if (!(Ep * 1.01 < 0.45 * (x1 - x0))) {
          amb = x1;
          break;
        }
      }
      L->fpamb = (float) amb;
      if (amb > 0 && (double) L->fpamb < amb)
        L->fpamb = nextafterf(L->fpamb, INFINITY);
    } else if (!(Ep < 0.45 * ldexp(1.0, b->p.fshift))) {
      return -1;
    }
  }
  /* Values beyond either end of an FP32 table need no check: a table runs
   * from at least one cell below its lowest edge to at least one cell above
   * its highest (fcfcg_axis_ftab), so an FP32 value outside it is more than
   * a cell, hence more than its window, away from every edge. */
  return 0;
}

/* Launch fields of a sorted catalogue. */
static void launch_cat(fcfcg_dcat *D, const slot_t *S) {
  D->l4 = S->l4;
  D->wq = S->wq;
  D->x = S->sx;
  D->y = S->sy;
  D->z = S->sz;
  D->s = S->ss;
  D->w = S->sw;
  D->id = S->sid;
  D->cstart = S->cstart;
  D->wexp = S->wexp;
}

/* Launch fields of the bins (FP64 reference binning), the outputs and the
 * recheck queue. */
static void launch_bins(const fcfcg_ctx *c, fcfcg_launch *L) {
  const fcfcg_bins *b = &c->bins;
  L->ns = b->ns;
  L->nmu = b->nmu;
  L->np = b->np;
  L->ntot = b->ntot;
  L->rs = c->d_rs;
  L->rp = c->d_rp;
  L->rsoff = b->s.roff;
  L->rpoff = b->p.roff;
  L->nrs = b->s.nrtab;
  L->nrp = b->p.nrtab;
  L->tabtype = b->s.tabtype;
  L->s2edge = c->d_s2edge;
  L->pedge = c->d_pedge;
  L->s2min = b->s.vmin;
  L->s2max = b->s.vmax;
  L->smin0 = b->s.min0;
  L->mu_one = b->mu_one;
  if (b->bintype == FCFCG_BIN_SPI) {
    L->pmin = b->p.vmin;
    L->pmax = b->p.vmax;
    L->pmin0 = b->p.min0;
  }
  L->fixF = FCFCG_FIX_F;
  L->gcnt = c->d_cnt;
  L->gwt = c->d_wt;
  L->gwd = c->d_wd;
  L->queue = c->d_queue;
  L->qcount = c->d_qcount;
  L->qcap = (uint32_t) c->qcap;
  L->stats = c->d_stats;
}

/* Launch fields of the FP32 edge-window tables. */
static void launch_fp32_tables(const fcfcg_ctx *c, fcfcg_launch *L) {
  const fcfcg_bins *b = &c->bins;
  L->fs = c->d_fs;
  L->nfs = (int) b->s.nftab;
  L->fsoff = (int) b->s.foff;
  L->fslog = b->s.flog;
  L->fsinv = (float) ldexp(1.0, b->s.flog ? -b->s.flog : -b->s.fshift);
  L->fse = c->d_fse;
  L->nsb = b->s.nbin;
  if (b->bintype == FCFCG_BIN_SPI) {
    L->fp = c->d_fp;
    L->nfp = (int) b->p.nftab;
    L->fpoff = (int) b->p.foff;
    L->fplog = b->p.flog;
    L->fpinv = (float) ldexp(1.0, b->p.flog ? -b->p.flog : -b->p.fshift);
    L->fpe = c->d_fpe;
    L->npb = b->p.nbin;
  }
}

static int ensure_pinned(fcfcg_ctx *c, size_t bytes) {
  if (c->h_pinned_cap >= bytes) return FCFCG_OK;
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  c->h_pinned = NULL;
  c->h_pinned_cap = 0;
  CK(cudaMallocHost(&c->h_pinned, bytes));
  c->h_pinned_cap = bytes;
  return FCFCG_OK;
}

/* Adjoint request of count_impl: cotangent in, gradients out (host). */
typedef struct {
  const double *g;
  double *dwa, *dwb;
} adj_req;

static int count_impl(fcfcg_ctx *c, int sa, int sb, int isauto, int withwt,
    int precision, int64_t *icnt, double *wcnt, const adj_req *adj);

int fcfcg_count(fcfcg_ctx *c, int sa, int sb, int isauto, int withwt,
    int precision, int64_t *icnt, double *wcnt) {
  return count_impl(c, sa, sb, isauto, withwt, precision, icnt, wcnt, NULL);
}

int fcfcg_adjoint(fcfcg_ctx *c, int sa, int sb, int isauto, const double *g,
    double *dwa, double *dwb) {
  if (!c || !g || !dwa) return FCFCG_ERR_ARG;
  adj_req r = {g, dwa, isauto ? NULL : dwb};
  return count_impl(c, sa, sb, isauto, 1, FCFCG_PREC_FP32_RECHECK, NULL,
                    NULL, &r);
}

/*
 * A count in three parts.  count_plan_make (host side; may allocate): the
 * grid, the stencil, the precision and the launch parameters, with every
 * buffer the launches touch grown to size.  count_launch (stream work only:
 * no allocation and no host synchronisation, so that it can be captured in
 * a CUDA graph): sort the catalogues into the grid, cut its cells into
 * chunks, count, recheck, and copy the histogram and the statistics to
 * pinned host memory.  count_finish (once the stream has finished): the
 * caller's histogram and the statistics.
 */
typedef struct {
  slot_t *A, *B;
  size_t na, nb;                 /* catalogue sizes and weights planned for */
  int hwa, hwb;
  int isauto, withwt, prec;
  grid_t g;
  int nsten, nin;                /* stencil entries, those within range */
  uint32_t ncell;
  size_t st;                     /* scan scratch length of the chunk list */
  fcfcg_launch L;                /* stencil pointers: set by the caller */
} count_plan;

#define STAT_WORDS 5   /* candidates, in range, rechecked, inline, chunks */

static int count_plan_make(fcfcg_ctx *c, slot_t *A, slot_t *B, int isauto,
    int withwt, int precision, int adj, int *sten, float *stD,
    count_plan *P) {
  const fcfcg_bins *b = &c->bins;
  int rc;
  memset(P, 0, sizeof *P);
  P->A = A;
  P->B = B;
  P->na = A->n;
  P->nb = B->n;
  P->hwa = A->has_w;
  P->hwb = B->has_w;
  P->isauto = isauto;
  P->withwt = withwt;
  grid_t *g = &P->g;
  if ((rc = grid_setup(c, g, A, B))) return rc;
  double dmax = 0;
  if ((rc = stencil_build(c, g, isauto, sten, stD, &P->nsten, &dmax, NULL,
                         &P->nin)))
    return rc;
  if ((rc = slot_reserve(c, A, g))) return rc;
  if (B != A && (rc = slot_reserve(c, B, g))) return rc;
  P->ncell = (uint32_t) ((size_t) g->n[0] * g->n[1] * g->n[2]);
  GROW(c->cchunk, c->cchunk_cap,
       sizeof(uint32_t) * 2 * ((size_t) P->ncell + 1));
  P->st = fcfcg_scan_tmp_len(P->ncell + 1) + 16;
  GROW(c->scan_tmp, c->scan_cap, sizeof(uint32_t) * P->st);
  size_t maxchunk = A->n / FCFCG_CHUNK + P->ncell + 1;
  GROW(c->chunks, c->chunk_cap, sizeof(uint32_t) * 4 * maxchunk);
  fcfcg_launch *L = &P->L;
  L->geometry = b->geometry;
  L->bintype = b->bintype;
  L->isauto = isauto;
  L->withwt = withwt;
  for (int d = 0; d < 3; d++) {
    L->ncell[d] = g->n[d];
    L->cw[d] = g->cw[d];
    L->lo[d] = g->lo[d];
    L->box[d] = b->box[d];
    L->cwf[d] = (float) g->cw[d];
    L->lof[d] = (float) g->lo[d];
  }
  L->nsten = P->nsten;
  L->nin = P->nin;
  L->tzero = -1;
  for (int t = 0; t < P->nsten; t++)
    if (!sten[4 * t] && !sten[4 * t + 1] && !sten[4 * t + 2]) L->tzero = t;
  L->chunks = c->chunks;
  L->chunk_head = c->d_head;
  /* k_chunks leaves the number of chunks after the ncell + 1 counts and
   * ncell offsets in cchunk */
  L->nchunk_dev = c->cchunk + ((size_t) P->ncell + 1) + P->ncell;
  launch_cat(&L->A, A);
  launch_cat(&L->B, B);
  launch_bins(c, L);
  int prec = precision;
  if (prec == FCFCG_PREC_FP32_RECHECK && fp32_bounds(c, g, dmax, A, B, L))
    prec = FCFCG_PREC_FP64;
  if (prec == FCFCG_PREC_FP32_RECHECK) launch_fp32_tables(c, L);
  size_t tabbytes = (prec == FCFCG_PREC_FP32_RECHECK)
      ? fcfcg_k_count32_tab_bytes(L->nfs, L->nfp, L->nsb, L->npb) : 0;
  size_t hbytes = (size_t) b->ntot * (withwt ? 8 : 4);
  size_t stage = (prec == FCFCG_PREC_FP32_RECHECK)
      ? fcfcg_k_count32_stage(P->nsten, withwt + (adj ? 1 : 0)) : 0;
  if (tabbytes + stage > 200 * 1024) {
    prec = FCFCG_PREC_FP64;
    tabbytes = 0;
    stage = 0;
  }
  L->hist_smem = (tabbytes + stage + hbytes <= 200 * 1024);
  L->hs_limit = c->hs_limit ? c->hs_limit : 0xFFFFFFFFull;
  L->qwarp = c->qwarp_force ? c->qwarp_force
      : ((c->tuned_q && c->tuned_q_key == g->key && c->tuned_q_wt == withwt)
             ? c->tuned_q : 0);
  P->prec = prec;
  return FCFCG_OK;
}

/* Stream side of a count.  sort_a / sort_b: sort that catalogue into the
 * plan's grid first.  timed: record the context's events (not while
 * capturing).  res (pinned, 2 ntot words) and stats (pinned, STAT_WORDS
 * words): where the histogram and the statistics go; NULL for none. */
static int count_launch(fcfcg_ctx *c, const count_plan *P, int sort_a,
    int sort_b, int timed, void *res, unsigned long long *stats) {
  const fcfcg_bins *b = &c->bins;
  const fcfcg_launch *L = &P->L;
  int rc;
  if (timed) CK(cudaEventRecord(c->ev[0], c->stream));
  if (sort_a && (rc = slot_sort(c, P->A, &P->g))) return rc;
  if (sort_b && P->B != P->A && (rc = slot_sort(c, P->B, &P->g))) return rc;
  /* work chunks: 64 points per CTA in the FP32 kernel, 32 per warp in the
   * FP64 kernel */
  const uint32_t clen = (P->prec == FCFCG_PREC_FP32_RECHECK) ? FCFCG_CHUNK32
                                                             : FCFCG_CHUNK;
  CKK(fcfcg_k_chunks(c->stream, P->A->cstart, P->ncell, clen, c->cchunk,
                     c->scan_tmp, P->st, c->chunks, NULL, NULL, 0));
  c->launches += 5;
  if (timed) CK(cudaEventRecord(c->ev[1], c->stream));
  CK(cudaMemsetAsync(c->d_cnt, 0, sizeof(unsigned long long) * b->ntot,
                     c->stream));
  CK(cudaMemsetAsync(c->d_wt, 0, sizeof(unsigned long long) * 2 * b->ntot,
                     c->stream));
  if (!L->adjoint)
    CK(cudaMemsetAsync(c->d_wd, 0, sizeof(double) * b->ntot, c->stream));
  CK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * 4,
                     c->stream));
  CK(cudaMemsetAsync(c->d_head, 0, sizeof(uint32_t) * 4, c->stream));
  if (timed) CK(cudaEventRecord(c->ev[2], c->stream));
  size_t smem = 0;
  CKK(fcfcg_k_count(c->stream, L, P->prec, c->nsm, &smem, &c->last_qwarp));
  c->launches += 1;
  if (timed) CK(cudaEventRecord(c->ev[3], c->stream));
  if (P->prec == FCFCG_PREC_FP32_RECHECK) {
    /* sized for a full queue; the kernel reads the fill on the device */
    CKK(fcfcg_k_recheck(c->stream, L, (uint32_t) c->qcap));
    c->launches += 1;
  }
  if (timed) CK(cudaEventRecord(c->ev[4], c->stream));
  if (res) {
    if (P->withwt && P->prec == FCFCG_PREC_FP64)
      CK(cudaMemcpyAsync(res, c->d_wd, sizeof(double) * b->ntot,
                         cudaMemcpyDeviceToHost, c->stream));
    else if (P->withwt)
      CK(cudaMemcpyAsync(res, c->d_wt,
                         sizeof(unsigned long long) * 2 * b->ntot,
                         cudaMemcpyDeviceToHost, c->stream));
    else
      CK(cudaMemcpyAsync(res, c->d_cnt, sizeof(unsigned long long) * b->ntot,
                         cudaMemcpyDeviceToHost, c->stream));
  }
  if (stats) {
    CK(cudaMemcpyAsync(stats, c->d_stats, sizeof(unsigned long long) * 4,
                       cudaMemcpyDeviceToHost, c->stream));
    /* the chunk count (32 bits) into the low half of the last word */
    stats[4] = 0;
    CK(cudaMemcpyAsync(stats + 4, L->nchunk_dev, sizeof(uint32_t),
                       cudaMemcpyDeviceToHost, c->stream));
  }
  return FCFCG_OK;
}

/* Host side after the stream finished: the caller's histogram and the
 * statistics (timings are the caller's). */
static void count_finish(fcfcg_ctx *c, const count_plan *P, const void *res,
    const unsigned long long *stats, int64_t *icnt, double *wcnt) {
  const fcfcg_bins *b = &c->bins;
  const unsigned long long *hres = (const unsigned long long *) res;
  if (P->withwt && P->prec == FCFCG_PREC_FP64) {
    memcpy(wcnt, res, sizeof(double) * b->ntot);
  } else if (P->withwt) {
    const int ex = P->A->wexp + P->B->wexp - P->L.fixF;
    for (long i = 0; i < b->ntot; i++) {
      __int128 v = (__int128) (((unsigned __int128) hres[2 * i + 1] << 64) |
                               (unsigned __int128) hres[2 * i]);
      wcnt[i] = ldexp((double) v, ex);
    }
  } else {
    for (long i = 0; i < b->ntot; i++) icnt[i] = (int64_t) hres[i];
  }
  fcfcg_stats *o = &c->stats;
  o->candidates = stats[0];
  o->in_range = stats[1];
  o->rechecked = stats[2];
  o->recheck_inline = stats[3];
  o->cells_per_smax = P->g.k;
  for (int d = 0; d < 3; d++) o->ncell[d] = P->g.n[d];
  o->nstencil = P->nsten;
  o->nchunks = (uint32_t) stats[4];
  o->precision_used = P->prec;
  o->warp_queue = P->prec == FCFCG_PREC_FP32_RECHECK ? (int) c->last_qwarp : 0;
  o->launches = c->launches;
}

/* Check the slots of a count: 0 or an error code. */
static int count_args(fcfcg_ctx *c, int sa, int sb, int isauto,
    int precision, int nslot) {
  if (sa < 0 || sa >= nslot || sb < 0 || sb >= nslot) {
    set_err(c, "slot out of range");
    return FCFCG_ERR_ARG;
  }
  if (isauto && sa != sb) {
    set_err(c, "auto counts need the same slot twice");
    return FCFCG_ERR_ARG;
  }
  if (precision != FCFCG_PREC_FP32_RECHECK && precision != FCFCG_PREC_FP64)
    return FCFCG_ERR_ARG;
  if (!c->slot[sa].x || !c->slot[sb].x) {
    set_err(c, "catalogue slot not loaded");
    return FCFCG_ERR_ARG;
  }
  return FCFCG_OK;
}

static int count_impl(fcfcg_ctx *c, int sa, int sb, int isauto, int withwt,
    int precision, int64_t *icnt, double *wcnt, const adj_req *adj) {
  if (!c || c->host_only) return FCFCG_ERR_ARG;
  int rc = count_args(c, sa, sb, isauto, precision,
                      FCFCG_MAX_SLOT + c->internal);
  if (rc) return rc;
  if (!adj && ((withwt && !wcnt) || (!withwt && !icnt))) return FCFCG_ERR_ARG;
  CK(cudaSetDevice(c->device));
  const fcfcg_bins *b = &c->bins;
  slot_t *A = c->slot + sa, *B = c->slot + sb;
  memset(&c->stats, 0, sizeof c->stats);
  if (A->n == 0 || B->n == 0) {
    if (icnt) memset(icnt, 0, sizeof(int64_t) * b->ntot);
    if (wcnt) memset(wcnt, 0, sizeof(double) * b->ntot);
    if (adj) {
      memset(adj->dwa, 0, sizeof(double) * A->n);
      if (adj->dwb) memset(adj->dwb, 0, sizeof(double) * B->n);
    }
    return FCFCG_OK;
  }
  count_plan P;
  rc = count_plan_make(c, A, B, isauto, withwt, precision, adj != NULL,
                       c->sten, c->stD, &P);
  if (rc) return rc;
  rc = upload(c, (void **) &c->d_sten, c->sten, sizeof(int) * 4 * P.nsten);
  if (rc) return rc;
  rc = upload(c, (void **) &c->d_stenD, c->stD, sizeof(float) * 4 * P.nsten);
  if (rc) return rc;
  P.L.sten = c->d_sten;
  P.L.stenD = c->d_stenD;
  const int sort_a = !slot_in_grid(A, &P.g);
  const int sort_b = (B != A) && !slot_in_grid(B, &P.g);
  fcfcg_launch *L = &P.L;
  if (adj) {
    const size_t ng = A->n + (isauto ? 0 : B->n);
    GROW(c->d_grad, c->d_grad_cap, sizeof(double) * 2 * ng);
    L->adjoint = 1;
    L->gadj = c->d_wd;
    L->dA = c->d_grad;
    L->dB = isauto ? c->d_grad : c->d_grad + A->n;
    CK(cudaMemcpyAsync(c->d_wd, adj->g, sizeof(double) * b->ntot,
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->d_grad, 0, sizeof(double) * ng, c->stream));
    double gmax = 0;
    for (size_t k = 0; k < (size_t) b->ntot; k++) {
      if (!isfinite(adj->g[k])) {
        set_err(c, "non-finite cotangent");
        return FCFCG_ERR_ARG;
      }
      if (fabs(adj->g[k]) > gmax) gmax = fabs(adj->g[k]);
    }
    if (P.prec == FCFCG_PREC_FP32_RECHECK) {
      /* unit of the integer gradient sums: 2^-S with |w| |g| 2^S <= 2^50
       * for every weight and cotangent entry */
      int gexp = 0;
      if (gmax > 0) {
        gexp = (int) ceil(log2(gmax));
        if (ldexp(1.0, gexp) < gmax) gexp++;
      }
      const int wexp = A->wexp > B->wexp ? A->wexp : B->wexp;
      int S = 50 - wexp - gexp;
      if (S < -1000) {
        set_err(c, "weights times cotangent out of range");
        return FCFCG_ERR_ARG;
      }
      if (S > 1000) S = 1000;   /* products stay below 2^50 */
      double *gf = malloc(sizeof(double) * b->ntot);
      if (!gf) return FCFCG_ERR_MEMORY;
      for (size_t k = 0; k < (size_t) b->ntot; k++)
        gf[k] = ldexp(adj->g[k], S);
      cudaError_t ce = cudaMemcpyAsync(c->d_gfix, gf,
          sizeof(double) * b->ntot, cudaMemcpyHostToDevice, c->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
      free(gf);
      CK(ce);
      L->gfix = c->d_gfix;
      L->gunit = ldexp(1.0, -S);
    }
  }
  size_t rbytes = sizeof(unsigned long long) * (2 * b->ntot + STAT_WORDS);
  if ((rc = ensure_pinned(c, rbytes))) return rc;
  unsigned long long *hres = (unsigned long long *) c->h_pinned;
  unsigned long long *hstats = hres + 2 * b->ntot;
  rc = count_launch(c, &P, sort_a, sort_b, 1, adj ? NULL : hres, hstats);
  if (rc) return rc;
  slot_mark(A, &P.g);
  if (B != A) slot_mark(B, &P.g);
  if (adj) {
    /* sorted order back to input order, then to the host */
    const size_t ng = A->n + (isauto ? 0 : B->n);
    double *unsorted = c->d_grad + ng;
    CKK(fcfcg_k_unsort(c->stream, A->n, A->sid, L->dA, unsorted));
    if (!isauto)
      CKK(fcfcg_k_unsort(c->stream, B->n, B->sid, L->dB, unsorted + A->n));
    c->launches += isauto ? 1 : 2;
    CK(cudaMemcpyAsync(adj->dwa, unsorted, sizeof(double) * A->n,
                       cudaMemcpyDeviceToHost, c->stream));
    if (!isauto && adj->dwb)
      CK(cudaMemcpyAsync(adj->dwb, unsorted + A->n, sizeof(double) * B->n,
                         cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  if (adj) {
    fcfcg_stats *o = &c->stats;
    o->candidates = hstats[0];
    o->in_range = hstats[1];
    o->rechecked = hstats[2];
    o->recheck_inline = hstats[3];
    o->cells_per_smax = P.g.k;
    o->nchunks = (uint32_t) hstats[4];
    o->precision_used = P.prec;
    o->warp_queue = P.prec == FCFCG_PREC_FP32_RECHECK ? (int) c->last_qwarp : 0;
    o->launches = c->launches;
  } else {
    count_finish(c, &P, hres, hstats, icnt, wcnt);
  }
  if (hstats[3]) queue_grow(c, hstats[2] + hstats[2] / 4);
  fcfcg_stats *o = &c->stats;
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
  o->ms_grid = ms;
  cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
  o->ms_count = ms;
  cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]);
  o->ms_recheck = ms;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[4]);
  o->ms_total = ms;
  return FCFCG_OK;
}

/* ------------------------------------------------------------------------ */
/* Count graphs.                                                             */

struct fcfcg_graph {
  fcfcg_ctx *c;
  int n, precision;
  fcfcg_count_item item[FCFCG_MAX_GRAPH_ITEMS];
  count_plan plan[FCFCG_MAX_GRAPH_ITEMS];
  int empty[FCFCG_MAX_GRAPH_ITEMS];
  int *d_sten[FCFCG_MAX_GRAPH_ITEMS];
  float *d_stenD[FCFCG_MAX_GRAPH_ITEMS];
  unsigned long long *h_stage;   /* pinned: per item 2 ntot + STAT_WORDS */
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  unsigned long bufgen;          /* the context's, when captured */
  uint64_t launches;             /* kernel launches per run */
  int captures;
  /* the grid each slot is left sorted into by a run */
  grid_t last[FCFCG_MAX_SLOT];
  int has_last[FCFCG_MAX_SLOT];
};

static void graph_release(fcfcg_graph *G) {
  if (G->exec) cudaGraphExecDestroy(G->exec);
  if (G->graph) cudaGraphDestroy(G->graph);
  G->exec = NULL;
  G->graph = NULL;
  for (int i = 0; i < G->n; i++) {
    if (G->d_sten[i]) cudaFree(G->d_sten[i]);
    if (G->d_stenD[i]) cudaFree(G->d_stenD[i]);
    G->d_sten[i] = NULL;
    G->d_stenD[i] = NULL;
  }
}

static unsigned long long *stage_of(const fcfcg_graph *G, int i) {
  return G->h_stage + (size_t) i * (2 * (size_t) G->c->bins.ntot + STAT_WORDS);
}

/* Plan every item and capture their launches as one graph. */
static int graph_build(fcfcg_graph *G) {
  fcfcg_ctx *c = G->c;
  graph_release(G);
  CK(cudaSetDevice(c->device));
  /* the first pass grows the context's buffers, the second takes their
   * final addresses */
  for (int pass = 0; pass < 2; pass++) {
    const unsigned long gen0 = c->bufgen;
    for (int i = 0; i < G->n; i++) {
      const fcfcg_count_item *it = G->item + i;
      slot_t *A = c->slot + it->slot_a, *B = c->slot + it->slot_b;
      G->empty[i] = (A->n == 0 || B->n == 0);
      if (G->empty[i]) continue;
      int rc = count_plan_make(c, A, B, it->isauto, it->withwt,
                               G->precision, 0, c->sten, c->stD,
                               G->plan + i);
      if (rc) return rc;
      if (pass == 1) {
        const size_t ns = (size_t) G->plan[i].nsten;
        CK(cudaMalloc((void **) &G->d_sten[i], sizeof(int) * 4 * (ns ? ns : 1)));
        CK(cudaMalloc((void **) &G->d_stenD[i],
                      sizeof(float) * 4 * (ns ? ns : 1)));
        CK(cudaMemcpy(G->d_sten[i], c->sten, sizeof(int) * 4 * ns,
                      cudaMemcpyHostToDevice));
        CK(cudaMemcpy(G->d_stenD[i], c->stD, sizeof(float) * 4 * ns,
                      cudaMemcpyHostToDevice));
        G->plan[i].L.sten = G->d_sten[i];
        G->plan[i].L.stenD = G->d_stenD[i];
      }
    }
    if (pass == 1 && c->bufgen != gen0) {
      set_err(c, "count graph: buffers moved while planning");
      return FCFCG_ERR_CUDA;
    }
  }
  G->bufgen = c->bufgen;
  CK(cudaStreamSynchronize(c->stream));
  const uint64_t l0 = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  int rc = FCFCG_OK;
  for (int i = 0; i < G->n && !rc; i++) {
    if (G->empty[i]) continue;
    unsigned long long *st = stage_of(G, i);
    rc = count_launch(c, G->plan + i, 1, 1, 0, st,
                      st + 2 * (size_t) c->bins.ntot);
  }
  cudaGraph_t gr = NULL;
  cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
  if (rc || e != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    if (!rc) {
      set_err(c, "CUDA: %s", cudaGetErrorString(e));
      rc = FCFCG_ERR_CUDA;
    }
    return rc;
  }
  G->graph = gr;
  CK(cudaGraphInstantiate(&G->exec, gr, 0));
  G->captures++;
  G->launches = c->launches - l0;
  c->launches = l0;
  /* a run leaves each slot sorted into the grid of its last count; until
   * then their order is unknown to plain counts */
  memset(G->has_last, 0, sizeof G->has_last);
  for (int i = 0; i < G->n; i++) {
    if (G->empty[i]) continue;
    const int s2[2] = {G->item[i].slot_a, G->item[i].slot_b};
    for (int k = 0; k < 2; k++) {
      G->last[s2[k]] = G->plan[i].g;
      G->has_last[s2[k]] = 1;
      c->slot[s2[k]].grid_valid = 0;
    }
  }
  return FCFCG_OK;
}

int fcfcg_graph_create(fcfcg_ctx *c, const fcfcg_count_item *items,
    int nitem, int precision, fcfcg_graph **out) {
  if (!c || c->host_only || !items || !out || nitem < 1 ||
      nitem > FCFCG_MAX_GRAPH_ITEMS)
    return FCFCG_ERR_ARG;
  *out = NULL;
  for (int i = 0; i < nitem; i++) {
    const fcfcg_count_item *it = items + i;
    int rc = count_args(c, it->slot_a, it->slot_b, it->isauto, precision,
                        FCFCG_MAX_SLOT);
    if (rc) return rc;
    if ((it->withwt && !it->wcnt) || (!it->withwt && !it->icnt))
      return FCFCG_ERR_ARG;
  }
  CK(cudaSetDevice(c->device));
  fcfcg_graph *G = calloc(1, sizeof *G);
  if (!G) return FCFCG_ERR_MEMORY;
  G->c = c;
  G->n = nitem;
  G->precision = precision;
  memcpy(G->item, items, sizeof *items * nitem);
  const size_t words = (size_t) nitem * (2 * (size_t) c->bins.ntot + STAT_WORDS);
  cudaError_t e = cudaMallocHost((void **) &G->h_stage,
                                 sizeof(unsigned long long) * words);
  if (e != cudaSuccess) {
    free(G);
    set_err(c, "CUDA: %s", cudaGetErrorString(e));
    return FCFCG_ERR_CUDA;
  }
  memset(G->h_stage, 0, sizeof(unsigned long long) * words);
  int rc = graph_build(G);
  if (rc) {
    fcfcg_graph_destroy(G);
    return rc;
  }
  *out = G;
  return FCFCG_OK;
}

int fcfcg_graph_run(fcfcg_graph *G) {
  if (!G) return FCFCG_ERR_ARG;
  fcfcg_ctx *c = G->c;
  CK(cudaSetDevice(c->device));
  for (int i = 0; i < G->n; i++) {
    /* a slot emptied or unloaded since the capture */
    const fcfcg_count_item *it = G->item + i;
    if (!c->slot[it->slot_a].x || !c->slot[it->slot_b].x) {
      set_err(c, "catalogue slot not loaded");
      return FCFCG_ERR_ARG;
    }
  }
  /* capture again when a buffer moved or the plan of an item changed (new
   * catalogue sizes, bounding boxes, weights or an autotuned grid); a slot
   * reloaded with data that plans the same replays as it is */
  int stale = !G->exec || c->bufgen != G->bufgen;
  for (int i = 0; i < G->n && !stale; i++) {
    const fcfcg_count_item *it = G->item + i;
    slot_t *A = c->slot + it->slot_a, *B = c->slot + it->slot_b;
    const int empty = (A->n == 0 || B->n == 0);
    if (empty != G->empty[i]) stale = 1;
    if (empty || stale) continue;
    count_plan P;
    int rc = count_plan_make(c, A, B, it->isauto, it->withwt, G->precision,
                             0, c->sten, c->stD, &P);
    if (rc) return rc;
    P.L.sten = G->plan[i].L.sten;
    P.L.stenD = G->plan[i].L.stenD;
    stale = (c->bufgen != G->bufgen) || memcmp(&P, G->plan + i, sizeof P);
  }
  if (stale) {
    int rc = graph_build(G);
    if (rc) return rc;
  }
  CK(cudaEventRecord(c->ev[0], c->stream));
  CK(cudaGraphLaunch(G->exec, c->stream));
  CK(cudaEventRecord(c->ev[4], c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->launches += G->launches;
  memset(&c->stats, 0, sizeof c->stats);
  for (int i = 0; i < G->n; i++) {
    const fcfcg_count_item *it = G->item + i;
    const long ntot = c->bins.ntot;
    if (G->empty[i]) {
      if (it->icnt) memset(it->icnt, 0, sizeof(int64_t) * ntot);
      if (it->wcnt) memset(it->wcnt, 0, sizeof(double) * ntot);
      continue;
    }
    const unsigned long long *st = stage_of(G, i);
    count_finish(c, G->plan + i, st, st + 2 * (size_t) ntot,
                 it->withwt ? NULL : it->icnt, it->withwt ? it->wcnt : NULL);
  }
  for (int s = 0; s < FCFCG_MAX_SLOT; s++)
    if (G->has_last[s]) slot_mark(c->slot + s, G->last + s);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[4]);
  c->stats.ms_total = ms;
  return FCFCG_OK;
}

int fcfcg_graph_info(const fcfcg_graph *G, int *captures,
    uint64_t *launches) {
  if (!G) return FCFCG_ERR_ARG;
  if (captures) *captures = G->captures;
  if (launches) *launches = G->launches;
  return FCFCG_OK;
}

void fcfcg_graph_destroy(fcfcg_graph *G) {
  if (!G) return;
  cudaSetDevice(G->c->device);
  graph_release(G);
  if (G->h_stage) cudaFreeHost(G->h_stage);
  free(G);
}

const fcfcg_bins *fcfcg_ctx_bins(const fcfcg_ctx *c) {
  return (c && c->bins.sbin_raw) ? &c->bins : NULL;
}

const double *fcfcg_ctx_box_raw(const fcfcg_ctx *c) {
  return c ? c->bins.box_raw : NULL;
}

int fcfcg_autotune(fcfcg_ctx *c, int sa, int sb, int isauto, int withwt,
    int *best_k, double *best_ms) {
  if (!c || c->host_only) return FCFCG_ERR_ARG;
  const long ntot = c->bins.ntot;
  int64_t *ic = malloc(sizeof(int64_t) * ntot);
  double *wc = malloc(sizeof(double) * ntot);
  if (!ic || !wc) {
    free(ic);
    free(wc);
    return FCFCG_ERR_MEMORY;
  }
  const int saved = c->kcell;
  int bk = 0, key = 0, rc = FCFCG_OK;
  double bms = 1e300;
  /* k = 1..8, until two refinements in a row are slower than the best */
  for (int k = 1; k <= 8 && (!bk || k <= bk + 2); k++) {
    c->kcell = k;
    double ms = 0;
    for (int rep = 0; rep < 2 && rc == FCFCG_OK; rep++) {
      rc = fcfcg_count(c, sa, sb, isauto, withwt, FCFCG_PREC_FP32_RECHECK,
                       ic, wc);
      ms = c->stats.ms_count + c->stats.ms_recheck;
    }
    if (rc == FCFCG_ERR_UNSUPPORTED) {   /* stencil too large: stop here */
      rc = FCFCG_OK;
      break;
    }
    if (rc) break;
    if (ms < bms) {
      bms = ms;
      bk = k;
    }
  }
  /* then the warp queue at that refinement */
  uint32_t bq = 0;
  const uint32_t saved_q = c->qwarp_force;
  if (rc == FCFCG_OK && bk) {
    c->kcell = bk;
    static const uint32_t qs[3] = {1024, 512, 256};
    double qms = 1e300;
    for (int i = 0; i < 3 && rc == FCFCG_OK; i++) {
      c->qwarp_force = qs[i];
      double ms = 0;
      for (int rep = 0; rep < 2 && rc == FCFCG_OK; rep++) {
        rc = fcfcg_count(c, sa, sb, isauto, withwt, FCFCG_PREC_FP32_RECHECK,
                         ic, wc);
        ms = c->stats.ms_count + c->stats.ms_recheck;
      }
      if (rc == FCFCG_OK && ms < qms) {
        qms = ms;
        bq = qs[i];
      }
    }
    if (qms < bms) bms = qms;
  }
  c->qwarp_force = saved_q;
  c->kcell = saved;
  if (rc == FCFCG_OK && bk) {
    /* the key of this catalogue pair, as the grid set-up computes it */
    grid_t g;
    memset(&g, 0, sizeof g);
    grid_setup(c, &g, c->slot + sa, c->slot + sb);
    key = g.key;
    c->tuned_k = bk;
    c->tuned_key = key;
    c->tuned_q = bq;
    c->tuned_q_key = key;
    c->tuned_q_wt = withwt;
  }
  free(ic);
  free(wc);
  if (best_k) *best_k = bk;
  if (best_ms) *best_ms = bms;
  return rc;
}

int fcfcg_stats_get(const fcfcg_ctx *c, fcfcg_stats *out) {
  if (!c || !out) return FCFCG_ERR_ARG;
  *out = c->stats;
  return FCFCG_OK;
}

/* ------------------------------------------------------------------------ */
/* Batches of periodic-box catalogues.                                       */

/* The all-FP64 comparison path: the catalogues one after the other through
 * the internal slot, each with its own box. */
static int batch_fp64(fcfcg_ctx *c, fcfcg_job *jobs, int njobs, int withwt,
    int on_device) {
  fcfcg_bins *b = &c->bins;
  double box0[3], raw0[3];
  memcpy(box0, b->box, sizeof box0);
  memcpy(raw0, b->box_raw, sizeof raw0);
  fcfcg_stats tot;
  memset(&tot, 0, sizeof tot);
  int rc = FCFCG_OK;
  c->internal = 1;
  for (int j = 0; j < njobs && rc == FCFCG_OK; j++) {
    fcfcg_job *J = jobs + j;
    if (J->status) continue;
    for (int k = 0; k < 3; k++) {
      b->box_raw[k] = J->box[k];
      b->box[k] = J->box[k] * b->rescale;
    }
    int e = load_common(c, FCFCG_MAX_SLOT, J->n, J->x, J->y, J->z,
                        withwt ? J->w : NULL, on_device, NULL);
    if (e == FCFCG_ERR_DATA) {
      J->status = e;
      continue;
    }
    if (e) {
      rc = e;
      break;
    }
    J->sumw = c->slot[FCFCG_MAX_SLOT].sumw;
    e = fcfcg_count(c, FCFCG_MAX_SLOT, FCFCG_MAX_SLOT, 1, withwt,
                    FCFCG_PREC_FP64, J->icnt, J->wcnt);
    if (e) {
      rc = e;
      break;
    }
    tot.candidates += c->stats.candidates;
    tot.in_range += c->stats.in_range;
    tot.ms_grid += c->stats.ms_grid;
    tot.ms_count += c->stats.ms_count;
    tot.ms_total += c->stats.ms_total;
  }
  c->internal = 0;
  c->slot[FCFCG_MAX_SLOT].grid_valid = 0;
  memcpy(b->box, box0, sizeof box0);
  memcpy(b->box_raw, raw0, sizeof raw0);
  tot.precision_used = FCFCG_PREC_FP64;
  tot.launches = c->launches;
  c->stats = tot;
  return rc;
}

int fcfcg_count_batch(fcfcg_ctx *c, fcfcg_job *jobs, int njobs, int withwt,
    int precision, int on_device) {
  if (!c || c->host_only || njobs < 0 || (njobs && !jobs))
    return FCFCG_ERR_ARG;
  fcfcg_bins *b = &c->bins;
  if (b->geometry != FCFCG_GEOM_BOX) {
    set_err(c, "batches are periodic boxes: use a box context");
    return FCFCG_ERR_ARG;
  }
  if (precision != FCFCG_PREC_FP32_RECHECK && precision != FCFCG_PREC_FP64)
    return FCFCG_ERR_ARG;
  CK(cudaSetDevice(c->device));
  memset(&c->stats, 0, sizeof c->stats);
  /* per-catalogue checks of conf_verify: s_max (and pi_max) below half the
   * box (src/fcfc/2pt_box/load_conf.c:1000-1003) */
  const double smax_raw = b->sbin_raw[b->ns];
  const double pmax_raw = (b->bintype == FCFCG_BIN_SPI) ? b->pbin_raw[b->np] : 0;
  for (int j = 0; j < njobs; j++) {
    fcfcg_job *J = jobs + j;
    J->status = FCFCG_OK;
    J->sumw = 0;
    if ((withwt && !J->wcnt) || (!withwt && !J->icnt) ||
        (J->n && (!J->x || !J->y || !J->z)) || (withwt && J->n && !J->w)) {
      J->status = FCFCG_ERR_ARG;
      continue;
    }
    for (int k = 0; k < 3; k++) {
      if (!(J->box[k] > 0) || !isfinite(J->box[k]) ||
          smax_raw >= J->box[k] * 0.5 ||
          (b->bintype == FCFCG_BIN_SPI && pmax_raw >= J->box[k] * 0.5))
        J->status = FCFCG_ERR_CFG;
    }
    if (!J->status) {
      if (withwt) memset(J->wcnt, 0, sizeof(double) * b->ntot);
      else memset(J->icnt, 0, sizeof(int64_t) * b->ntot);
    }
  }
  if (precision == FCFCG_PREC_FP64)
    return batch_fp64(c, jobs, njobs, withwt, on_device);

  /* 1. catalogues side by side in the batch slot, rescaled */
  int *acc = malloc(sizeof(int) * (njobs ? njobs : 1));
  size_t *base = malloc(sizeof(size_t) * (njobs ? njobs + 1 : 1));
  if (!acc || !base) {
    free(acc);
    free(base);
    return FCFCG_ERR_MEMORY;
  }
  int rc = FCFCG_OK;
  int na = 0;
  size_t N = 0;
  for (int j = 0; j < njobs; j++) {
    if (jobs[j].status || !jobs[j].n) continue;
    acc[na] = j;
    base[na++] = N;
    N += jobs[j].n;
  }
  base[na] = N;
#define BFAIL(code)                                                       \
  do {                                                                    \
    rc = (code);                                                          \
    goto out;                                                             \
  } while (0)
#define BCK(call)                                                         \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      set_err(c, "%s: %s", #call, cudaGetErrorString(e_));                \
      BFAIL(FCFCG_ERR_CUDA);                                              \
    }                                                                     \
  } while (0)
#define BCKK(call)                                                        \
  do {                                                                    \
    int e_ = (call);                                                      \
    if (e_) {                                                             \
      set_err(c, "%s: %s", #call, fcfcg_cuda_errstr(e_));                 \
      BFAIL(FCFCG_ERR_CUDA);                                              \
    }                                                                     \
  } while (0)
#define BGROW(ptr, capv, bytes)                                           \
  do {                                                                    \
    size_t cap_ = (capv);                                                 \
    int r_ = grow(c, (void **) &(ptr), &cap_, (bytes));                   \
    if (r_) BFAIL(r_);                                                    \
    (capv) = cap_;                                                        \
  } while (0)
  if (N > 0xFFFFFFF0u) {
    set_err(c, "batch too large (%zu objects)", N);
    BFAIL(FCFCG_ERR_ARG);
  }
  if (na == 0) goto out;
  BCK(cudaEventRecord(c->ev[0], c->stream));
  slot_t *S = c->slot + FCFCG_MAX_SLOT;
  S->grid_valid = 0;
  if (S->cap < N || !S->x) {
    slot_free(S);
    BCK(cudaMalloc((void **) &S->x, sizeof(double) * N));
    BCK(cudaMalloc((void **) &S->y, sizeof(double) * N));
    BCK(cudaMalloc((void **) &S->z, sizeof(double) * N));
    BCK(cudaMalloc((void **) &S->s, sizeof(double) * N));
    BCK(cudaMalloc((void **) &S->w, sizeof(double) * N));
    S->cap = N;
  }
  S->n = N;
  S->has_w = withwt;
  /* per catalogue: bounding box (6), max |w| bits, weight sum (double) */
  BGROW(c->d_bstat, c->d_bstat_cap, sizeof(unsigned long long) * 8 * na);
  {
    unsigned long long *init = malloc(sizeof(unsigned long long) * 8 * na);
    if (!init) BFAIL(FCFCG_ERR_MEMORY);
    for (int a = 0; a < na; a++) {
      for (int k = 0; k < 3; k++) {
        init[8 * a + k] = ~0ull;
        init[8 * a + 3 + k] = 0;
      }
      init[8 * a + 6] = 0;
      init[8 * a + 7] = 0;
    }
    cudaError_t e = cudaMemcpy(c->d_bstat, init,
                               sizeof(unsigned long long) * 8 * na,
                               cudaMemcpyHostToDevice);
    free(init);
    BCK(e);
  }
  /* the catalogue table: inputs, slot offsets, first tiles */
  if (c->h_pcat_cap < (size_t) na) {
    free(c->h_pcat);
    c->h_pcat = malloc(sizeof(fcfcg_prep_cat) * na);
    c->h_pcat_cap = c->h_pcat ? (size_t) na : 0;
    if (!c->h_pcat) BFAIL(FCFCG_ERR_MEMORY);
  }
  fcfcg_prep_cat *P = c->h_pcat;
  const size_t tile = fcfcg_batch_tile();
  uint32_t ntile = 0;
  for (int a = 0; a < na; a++) {
    const fcfcg_job *J = jobs + acc[a];
    const size_t o = base[a], n = J->n;
    fcfcg_prep_cat *Q = P + a;
    memset(Q, 0, sizeof *Q);
    Q->x = J->x;
    Q->y = J->y;
    Q->z = J->z;
    Q->w = withwt ? J->w : NULL;
    Q->o = o;
    Q->n = n;
    Q->tile0 = ntile;
    ntile += (uint32_t) ((n + tile - 1) / tile);
    if (!on_device && !c->pageable) {
      BCK(cudaMemcpyAsync(S->x + o, J->x, sizeof(double) * n,
                          cudaMemcpyHostToDevice, c->stream));
      BCK(cudaMemcpyAsync(S->y + o, J->y, sizeof(double) * n,
                          cudaMemcpyHostToDevice, c->stream));
      BCK(cudaMemcpyAsync(S->z + o, J->z, sizeof(double) * n,
                          cudaMemcpyHostToDevice, c->stream));
      if (withwt)
        BCK(cudaMemcpyAsync(S->w + o, J->w, sizeof(double) * n,
                            cudaMemcpyHostToDevice, c->stream));
      Q->x = S->x + o;
      Q->y = S->y + o;
      Q->z = S->z + o;
      Q->w = withwt ? S->w + o : NULL;
    }
  }
  BGROW(c->d_pcat, c->d_pcat_cap, sizeof(fcfcg_prep_cat) * na);
  BGROW(c->d_bpart, c->d_bpart_cap, sizeof(double) * ntile);
  BCK(cudaMemcpyAsync(c->d_pcat, P, sizeof(fcfcg_prep_cat) * na,
                      cudaMemcpyHostToDevice, c->stream));
  BCKK(fcfcg_k_prep_batch(c->stream, (const fcfcg_prep_cat *) c->d_pcat, na,
                          ntile, b->rescale, withwt, S->x, S->y, S->z, S->w,
                          c->d_bstat, c->d_bpart));
  c->launches += withwt ? 2 : 1;
  /* 2. per-catalogue range checks, weight scales and sums */
  unsigned long long *hb = malloc(sizeof(unsigned long long) * 8 * na);
  if (!hb) BFAIL(FCFCG_ERR_MEMORY);
  {
    cudaError_t e = cudaMemcpyAsync(hb, c->d_bstat,
                                    sizeof(unsigned long long) * 8 * na,
                                    cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) {
      free(hb);
      BCK(e);
    }
  }
  int *wexp = malloc(sizeof(int) * na);
  if (!wexp) {
    free(hb);
    BFAIL(FCFCG_ERR_MEMORY);
  }
  for (int a = 0; a < na; a++) {
    fcfcg_job *J = jobs + acc[a];
    for (int k = 0; k < 3; k++) {
      unsigned long long lo = hb[8 * a + k], hi = hb[8 * a + 3 + k];
      lo = (lo >> 63) ? (lo & 0x7FFFFFFFFFFFFFFFull) : ~lo;
      hi = (hi >> 63) ? (hi & 0x7FFFFFFFFFFFFFFFull) : ~hi;
      double mn, mx;
      memcpy(&mn, &lo, 8);
      memcpy(&mx, &hi, 8);
      const double L = J->box[k] * b->rescale, tol = L * 1e-9;
      if (!isfinite(mn) || !isfinite(mx) || mn < -tol || mx > L + tol)
        J->status = FCFCG_ERR_DATA;
    }
    double wmax = 1;
    if (withwt) memcpy(&wmax, hb + 8 * a + 6, 8);
    if (!isfinite(wmax)) J->status = FCFCG_ERR_DATA;
    int we = (wmax > 0) ? (int) ceil(log2(wmax)) : 0;
    if (ldexp(1.0, we) < wmax) we++;
    wexp[a] = we;
    P[a].wexp = we;
    if (J->status) continue;
    if (withwt) memcpy(&J->sumw, hb + 8 * a + 7, 8);
    else J->sumw = (double) J->n;
  }
  free(hb);
  /* 3. grids: one refinement k for the batch, each catalogue's cells tile
   * its own box */
  grid_t gr;
  memset(&gr, 0, sizeof gr);
  grid_reach(c, &gr);
  double vol = 0, nsum = 0;
  for (int a = 0; a < na; a++) {
    const fcfcg_job *J = jobs + acc[a];
    if (J->status) continue;
    vol += J->box[0] * J->box[1] * J->box[2] * b->rescale * b->rescale *
           b->rescale;
    nsum += (double) J->n;
  }
  const double density = nsum / (vol > 0 ? vol : 1);
  const int key = tune_key(density, gr.reach) + 1000;   /* batch keys */
  int k = c->kcell;
  if (!k) k = (c->tuned_k && c->tuned_key == key) ? c->tuned_k
                                                  : pick_k(density, gr.reach3, 24.0);
  BGROW(c->d_mbase, c->d_mbase_cap, sizeof(uint32_t) * (na + 1));
  if (c->h_mock_cap < (size_t) na) {
    free(c->h_mock);
    c->h_mock = malloc(sizeof(fcfcg_mock) * na);
    c->h_mock_cap = c->h_mock ? (size_t) na : 0;
    if (!c->h_mock) {
      free(wexp);
      BFAIL(FCFCG_ERR_MEMORY);
    }
  }
  uint32_t *hbase = malloc(sizeof(uint32_t) * (na + 1));
  if (!hbase) {
    free(wexp);
    BFAIL(FCFCG_ERR_MEMORY);
  }
  grid_t gmin = gr, gmax = gr;
  for (int d = 0; d < 3; d++) {
    gmin.cw[d] = 1e300;
    gmax.cw[d] = 0;
  }
  size_t cells = 0;
  double xabs = 0;
  for (int a = 0; a < na; a++) {
    const fcfcg_job *J = jobs + acc[a];
    fcfcg_mock *M = c->h_mock + a;
    memset(M, 0, sizeof *M);
    hbase[a] = (uint32_t) cells;
    if (J->status) continue;     /* no cells: never visited */
    size_t nc = 1;
    for (int d = 0; d < 3; d++) {
      const double L = J->box[d] * b->rescale;
      const double cwt = gr.reach[d] / k * (1 + 1e-6);
      int n = (int) floor(L / cwt);
      if (n < 1) n = 1;
      if (n > 4096) n = 4096;
      M->ncell[d] = n;
      M->cw[d] = L / n;
      M->box[d] = L;
      nc *= (size_t) n;
      gmin.cw[d] = fmin(gmin.cw[d], M->cw[d]);
      gmax.cw[d] = fmax(gmax.cw[d], M->cw[d]);
      xabs = fmax(xabs, L);
    }
    M->cell_base = (uint32_t) cells;
    P[a].live = 1;
    P[a].cell_base = M->cell_base;
    for (int d = 0; d < 3; d++) {
      P[a].ncell[d] = M->ncell[d];
      P[a].cw[d] = M->cw[d];
    }
    cells += nc;
    if (cells > 0x7FFFFFF0u) {
      free(wexp);
      free(hbase);
      set_err(c, "batch grid too large");
      BFAIL(FCFCG_ERR_UNSUPPORTED);
    }
  }
  hbase[na] = (uint32_t) cells;
  /* 4. one stencil for all: built for the narrowest cells (a superset of
   * every catalogue's own); bounds for the widest */
  int nsten = 0;
  double dmin = 0;
  gmin.k = gmax.k = k;
  if (gmin.cw[0] > 1e299) {        /* every catalogue failed its checks */
    free(wexp);
    free(hbase);
    goto out;
  }
  int nin = 0;
  if ((rc = stencil_build(c, &gmin, 1, c->sten, c->stD, &nsten, &dmin,
                          gmax.cw, &nin))) {
    free(wexp);
    free(hbase);
    goto out;
  }
  double dmax = 0;
  for (int t = 0; t < nsten; t++)
    for (int d = 0; d < 3; d++)
      dmax = fmax(dmax, fabs((double) c->sten[4 * t + d]) * gmax.cw[d]);
  /* 5. cell sort of every catalogue into the shared sorted arrays */
  const size_t m = N;
  if (S->scap < m) {
    void *pp[] = {S->l4, S->wq, S->sx, S->sy, S->sz, S->ss, S->sw, S->sid,
                  S->cell_of};
    for (size_t i = 0; i < sizeof pp / sizeof pp[0]; i++)
      if (pp[i]) cudaFree(pp[i]);
    S->l4 = NULL;
    S->scap = 0;
    cudaError_t e = cudaMalloc((void **) &S->l4, sizeof(float) * 4 * m);
    if (!e) e = cudaMalloc((void **) &S->wq, sizeof(int) * 2 * m);
    if (!e) e = cudaMalloc((void **) &S->sx, sizeof(double) * m);
    if (!e) e = cudaMalloc((void **) &S->sy, sizeof(double) * m);
    if (!e) e = cudaMalloc((void **) &S->sz, sizeof(double) * m);
    if (!e) e = cudaMalloc((void **) &S->ss, sizeof(double) * 1);
    if (!e) e = cudaMalloc((void **) &S->sw, sizeof(double) * m);
    if (!e) e = cudaMalloc((void **) &S->sid, sizeof(uint32_t) * m);
    if (!e) e = cudaMalloc((void **) &S->cell_of, sizeof(uint32_t) * m);
    if (e) {
      free(wexp);
      free(hbase);
      BCK(e);
    }
    S->scap = m;
  }
  if (S->ccap < cells + 1) {
    if (S->cstart) cudaFree(S->cstart);
    S->cstart = NULL;
    S->ccap = 0;
    cudaError_t e = cudaMalloc((void **) &S->cstart,
                               sizeof(uint32_t) * (cells + 1));
    if (e) {
      free(wexp);
      free(hbase);
      BCK(e);
    }
    S->ccap = cells + 1;
  }
  /* fine counters: cells x sub-cells (the points of a cell grouped by
   * sub-cell in the sorted arrays) */
  const int sb = fcfcg_grid_sub_bits(cells, N);
  const size_t nf = cells << sb;
  BGROW(c->cfill, c->cfill_cap, sizeof(uint32_t) * (nf + 1));
  BGROW(c->fstart, c->fstart_cap, sizeof(uint32_t) * (nf + 1));
  const size_t stl = fcfcg_scan_tmp_len(nf + 1) + 16;
  BGROW(c->scan_tmp, c->scan_cap, sizeof(uint32_t) * stl);
  BCK(cudaMemsetAsync(c->cfill, 0, sizeof(uint32_t) * (nf + 1), c->stream));
  /* the table again, with the grids (the stream is idle: the range checks
   * synchronised it) */
  BCK(cudaMemcpyAsync(c->d_pcat, P, sizeof(fcfcg_prep_cat) * na,
                      cudaMemcpyHostToDevice, c->stream));
  BCKK(fcfcg_k_cell_batch(c->stream, (const fcfcg_prep_cat *) c->d_pcat, na,
                          ntile, sb, S->x, S->y, S->z, S->cell_of, c->cfill));
  BCKK(fcfcg_scan(c->stream, c->cfill, nf, c->fstart, c->scan_tmp));
  BCKK(fcfcg_k_cstart(c->stream, cells, sb, c->fstart, S->cstart));
  BCK(cudaMemsetAsync(c->cfill, 0, sizeof(uint32_t) * (nf + 1), c->stream));
  BCKK(fcfcg_k_scatter_batch(c->stream, (const fcfcg_prep_cat *) c->d_pcat,
                             na, ntile, sb, S->x, S->y, S->z,
                             withwt ? S->w : NULL, withwt, S->cell_of,
                             c->fstart, c->cfill, S->l4, S->wq, S->sx, S->sy,
                             S->sz, S->sw, S->sid));
  c->launches += 6;
  /* 6. per-catalogue histograms and the catalogue table */
  const size_t per = (size_t) b->ntot * (withwt ? 2 : 1);
  BGROW(c->d_bout, c->d_bout_cap, sizeof(unsigned long long) * per * na);
  BCK(cudaMemsetAsync(c->d_bout, 0, sizeof(unsigned long long) * per * na,
                      c->stream));
  for (int a = 0; a < na; a++) {
    c->h_mock[a].gcnt = withwt ? NULL : c->d_bout + per * a;
    c->h_mock[a].gwt = withwt ? c->d_bout + per * a : NULL;
  }
  BGROW(c->d_mock, c->d_mock_cap, sizeof(fcfcg_mock) * na);
  BCK(cudaMemcpyAsync(c->d_mock, c->h_mock, sizeof(fcfcg_mock) * na,
                      cudaMemcpyHostToDevice, c->stream));
  BCK(cudaMemcpyAsync(c->d_mbase, hbase, sizeof(uint32_t) * (na + 1),
                      cudaMemcpyHostToDevice, c->stream));
  /* the copies read host memory that is freed below */
  BCK(cudaStreamSynchronize(c->stream));
  free(hbase);
  /* 7. launch parameters */
  fcfcg_launch L;
  memset(&L, 0, sizeof L);
  L.geometry = FCFCG_GEOM_BOX;
  L.bintype = b->bintype;
  L.isauto = 1;
  L.withwt = withwt;
  for (int d = 0; d < 3; d++) {
    L.ncell[d] = 1;
    L.box[d] = b->box[d];
  }
  S->xabs = xabs;
  S->s2abs = 0;
  S->wexp = 0;
  launch_cat(&L.A, S);
  launch_cat(&L.B, S);
  launch_bins(c, &L);
  L.mocks = (const fcfcg_mock *) c->d_mock;
  L.nmock = na;
  int prec = FCFCG_PREC_FP32_RECHECK;
  if (fp32_bounds(c, &gmax, dmax, S, S, &L)) prec = FCFCG_PREC_FP64;
  size_t tabbytes = 0, stage = 0;
  if (prec == FCFCG_PREC_FP32_RECHECK) {
    launch_fp32_tables(c, &L);
    tabbytes = fcfcg_k_count32_tab_bytes(L.nfs, L.nfp, L.nsb, L.npb);
    stage = fcfcg_k_count32_stage(nsten, withwt);
    if (tabbytes + stage > 200 * 1024) prec = FCFCG_PREC_FP64;
  }
  if (prec != FCFCG_PREC_FP32_RECHECK) {
    /* FP32 windows too wide for these boxes: count them in FP64 */
    free(wexp);
    free(acc);
    free(base);
    return batch_fp64(c, jobs, njobs, withwt, on_device);
  }
  const size_t hbytes = (size_t) b->ntot * (withwt ? 8 : 4);
  L.hist_smem = (tabbytes + stage + hbytes <= 200 * 1024);
  L.hs_limit = c->hs_limit ? c->hs_limit : 0xFFFFFFFFull;
  L.nsten = nsten;
  L.nin = nin;
  L.tzero = -1;
  for (int t = 0; t < nsten; t++)
    if (!c->sten[4 * t] && !c->sten[4 * t + 1] && !c->sten[4 * t + 2])
      L.tzero = t;
  if ((rc = upload(c, (void **) &c->d_sten, c->sten,
                   sizeof(int) * 4 * nsten))) {
    free(wexp);
    goto out;
  }
  if ((rc = upload(c, (void **) &c->d_stenD, c->stD,
                   sizeof(float) * 4 * nsten))) {
    free(wexp);
    goto out;
  }
  L.sten = c->d_sten;
  L.stenD = c->d_stenD;
  /* 8. work chunks of every catalogue, in catalogue order */
  BGROW(c->cchunk, c->cchunk_cap, sizeof(uint32_t) * 2 * (cells + 1));
  const size_t maxchunk = N / FCFCG_CHUNK + cells + 1;
  BGROW(c->chunks, c->chunk_cap, sizeof(uint32_t) * 4 * maxchunk);
  uint32_t nchunk = 0;
  BCKK(fcfcg_k_chunks(c->stream, S->cstart, (uint32_t) cells, FCFCG_CHUNK32,
                      c->cchunk, c->scan_tmp, stl, c->chunks, &nchunk,
                      c->d_mbase, na));
  c->launches += 5;
  BCK(cudaEventRecord(c->ev[1], c->stream));
  BCK(cudaStreamSynchronize(c->stream));
  L.nchunk = nchunk;
  L.chunks = c->chunks;
  L.chunk_head = c->d_head;
  BCK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * 4,
                      c->stream));
  BCK(cudaMemsetAsync(c->d_head, 0, sizeof(uint32_t) * 4, c->stream));
  BCK(cudaEventRecord(c->ev[2], c->stream));
  size_t smem = 0;
  L.qwarp = c->qwarp_force ? c->qwarp_force
      : ((c->tuned_q && c->tuned_q_key == key && c->tuned_q_wt == withwt)
             ? c->tuned_q : 0);
  BCKK(fcfcg_k_count(c->stream, &L, prec, c->nsm, &smem, &c->last_qwarp));
  c->launches += 1;
  BCK(cudaEventRecord(c->ev[3], c->stream));
  unsigned long long nq = 0;
  BCK(cudaMemcpyAsync(&nq, c->d_qcount, sizeof nq, cudaMemcpyDeviceToHost,
                      c->stream));
  BCK(cudaStreamSynchronize(c->stream));
  if (nq > c->qcap) nq = c->qcap;
  BCKK(fcfcg_k_recheck(c->stream, &L, (uint32_t) nq));
  c->launches += nq ? 1 : 0;
  BCK(cudaEventRecord(c->ev[4], c->stream));
  /* 9. results */
  {
    unsigned long long *hres = malloc(sizeof(unsigned long long) * per * na);
    unsigned long long hstats[4];
    if (!hres) {
      free(wexp);
      BFAIL(FCFCG_ERR_MEMORY);
    }
    cudaError_t e = cudaMemcpyAsync(hres, c->d_bout,
                                    sizeof(unsigned long long) * per * na,
                                    cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaMemcpyAsync(hstats, c->d_stats, sizeof hstats,
                                cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) {
      free(hres);
      free(wexp);
      BCK(e);
    }
    for (int a = 0; a < na; a++) {
      fcfcg_job *J = jobs + acc[a];
      if (J->status) continue;
      const unsigned long long *r = hres + per * a;
      if (withwt) {
        const int ex = 2 * wexp[a] - L.fixF;
        for (long i = 0; i < b->ntot; i++) {
          __int128 v = (__int128) (((unsigned __int128) r[2 * i + 1] << 64) |
                                   (unsigned __int128) r[2 * i]);
          J->wcnt[i] = ldexp((double) v, ex);
        }
      } else {
        for (long i = 0; i < b->ntot; i++) J->icnt[i] = (int64_t) r[i];
      }
    }
    free(hres);
    fcfcg_stats *o = &c->stats;
    o->candidates = hstats[0];
    o->in_range = hstats[1];
    o->rechecked = hstats[2];
    o->recheck_inline = hstats[3];
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
    o->ms_grid = ms;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    o->ms_count = ms;
    cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]);
    o->ms_recheck = ms;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[4]);
    o->ms_total = ms;
    o->cells_per_smax = k;
    o->nstencil = nsten;
    o->nchunks = nchunk;
    o->precision_used = prec;
    o->warp_queue = prec == FCFCG_PREC_FP32_RECHECK ? (int) c->last_qwarp : 0;
    o->launches = c->launches;
    if (hstats[3]) queue_grow(c, hstats[2] + hstats[2] / 4);
  }
  free(wexp);
out:
  free(acc);
  free(base);
  return rc;
#undef BFAIL
#undef BCK
#undef BCKK
#undef BGROW
}

int fcfcg_autotune_batch(fcfcg_ctx *c, fcfcg_job *jobs, int njobs,
    int withwt, int on_device, int *best_k, double *best_ms) {
  if (!c || c->host_only) return FCFCG_ERR_ARG;
  const int saved = c->kcell;
  int bk = 0, rc = FCFCG_OK;
  double bms = 1e300;
  /* k = 1..8, until two refinements in a row are slower than the best */
  for (int k = 1; k <= 8 && rc == FCFCG_OK && (!bk || k <= bk + 2); k++) {
    c->kcell = k;
    double ms = 0;
    for (int rep = 0; rep < 2 && rc == FCFCG_OK; rep++) {
      rc = fcfcg_count_batch(c, jobs, njobs, withwt, FCFCG_PREC_FP32_RECHECK,
                             on_device);
      ms = c->stats.ms_count + c->stats.ms_recheck;
    }
    if (rc == FCFCG_ERR_UNSUPPORTED) {
      rc = FCFCG_OK;
      break;
    }
    if (rc == FCFCG_OK && ms > 0 && ms < bms) {
      bms = ms;
      bk = k;
    }
  }
  /* then the warp queue at that refinement */
  uint32_t bq = 0;
  const uint32_t saved_q = c->qwarp_force;
  if (rc == FCFCG_OK && bk) {
    c->kcell = bk;
    static const uint32_t qs[3] = {1024, 512, 256};
    double qms = 1e300;
    for (int i = 0; i < 3 && rc == FCFCG_OK; i++) {
      c->qwarp_force = qs[i];
      double ms = 0;
      for (int rep = 0; rep < 2 && rc == FCFCG_OK; rep++) {
        rc = fcfcg_count_batch(c, jobs, njobs, withwt,
                               FCFCG_PREC_FP32_RECHECK, on_device);
        ms = c->stats.ms_count + c->stats.ms_recheck;
      }
      if (rc == FCFCG_OK && ms > 0 && ms < qms) {
        qms = ms;
        bq = qs[i];
      }
    }
    if (qms < bms) bms = qms;
  }
  c->qwarp_force = saved_q;
  c->kcell = saved;
  if (rc == FCFCG_OK && bk) {
    /* the key fcfcg_count_batch computes for this batch */
    grid_t gr;
    memset(&gr, 0, sizeof gr);
    grid_reach(c, &gr);
    const fcfcg_bins *b = &c->bins;
    double vol = 0, nsum = 0;
    for (int j = 0; j < njobs; j++) {
      if (jobs[j].status || !jobs[j].n) continue;
      vol += jobs[j].box[0] * jobs[j].box[1] * jobs[j].box[2] * b->rescale *
             b->rescale * b->rescale;
      nsum += (double) jobs[j].n;
    }
    c->tuned_k = bk;
    c->tuned_key = tune_key(nsum / (vol > 0 ? vol : 1), gr.reach) + 1000;
    c->tuned_q = bq;
    c->tuned_q_key = c->tuned_key;
    c->tuned_q_wt = withwt;
  }
  if (best_k) *best_k = bk;
  if (best_ms) *best_ms = bms;
  return rc;
}
