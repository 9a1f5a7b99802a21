/*
 * count.cu -- host-side launchers of the counting kernels, the all-FP64
 * counting kernel, the FP64 recheck of queued pairs, and the
 * allocation-free FP64 counter.  The FP32 counting kernel is count32.cuh,
 * instantiated by the count32_*.cu files.
 */
#include "count_common.cuh"

/*
 * FP64 counting kernel: the same traversal, every pair binned by the
 * reference's FP64 formula.  Weighted sums are FP64 products accumulated
 * in FP64.
 */
template <int GEOM, int WT, int ADJ>
__global__ void __launch_bounds__(CT_THREADS)
k_count64(const fcfcg_launch L) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t *h32 = (uint32_t *) smem;
  double *hd = (double *) smem;
  if (!ADJ && L.hist_smem) {
    if (WT)
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) hd[i] = 0;
    else
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) h32[i] = 0;
  }
  __syncthreads();
  unsigned long long n_cand = 0, n_in = 0;
  WarpChunk w;
  while (next_chunk(L, w)) {
    double ga = 0;      /* adjoint: this lane's share of dL/dw of its point */
    for (int t = 0; t < L.nsten; t++) {
      const int4 o = __ldg((const int4 *) L.sten + t);
      uint32_t cb, code;
      if (!neighbour(L, w, o, cb, code)) continue;
      const uint32_t bstart = __ldg(L.B.cstart + cb);
      const uint32_t bend = __ldg(L.B.cstart + cb + 1);
      if (bstart == bend || !w.active) continue;
      const bool self = L.isauto && o.x == 0 && o.y == 0 && o.z == 0;
      const int nb = (int) (bend - bstart);
      for (int j = first_j(w, self, bstart); j < nb; j += w.G) {
        const uint32_t bj = bstart + (uint32_t) j;
        n_cand++;
        int bin = ref_bin_pair(L, w.ai, bj, code, L.box);
        if (bin < 0) continue;
        n_in++;
        if (ADJ) {
          const double g = __ldg(L.gadj + bin);
          ga = __dadd_rn(ga, __dmul_rn(L.B.w[bj], g));
          atomicAdd(L.dB + bj, __dmul_rn(L.A.w[w.ai], g));
        } else if (WT) {
          double v = __dmul_rn(L.A.w[w.ai], L.B.w[bj]);
          if (L.hist_smem) atomicAdd(hd + bin, v);
          else atomicAdd(L.gwd + bin, v);
        } else {
          if (L.hist_smem) hist_add_count(h32, L.gcnt, bin);
          else atomicAdd(L.gcnt + bin, 1ull);
        }
      }
    }
    if (ADJ && ga != 0.0) atomicAdd(L.dA + w.ai, ga);
  }
  for (int o = 16; o > 0; o >>= 1) {
    n_cand += __shfl_xor_sync(FULLMASK, n_cand, o);
    n_in += __shfl_xor_sync(FULLMASK, n_in, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(L.stats + 0, n_cand);
    atomicAdd(L.stats + 1, n_in);
  }
  __syncthreads();
  if (!ADJ && L.hist_smem) {
    for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) {
      if (WT) {
        double v = hd[i];
        if (v != 0) atomicAdd(L.gwd + i, v);
      } else {
        uint32_t v = h32[i];
        if (v) atomicAdd(L.gcnt + i, (unsigned long long) v);
      }
    }
  }
}

/* Queued pairs to recheck: the queue's fill, at most its capacity. */
__device__ __forceinline__ uint32_t queue_len(const fcfcg_launch &L) {
  const unsigned long long n = *(volatile const unsigned long long *) L.qcount;
  return n < L.qcap ? (uint32_t) n : L.qcap;
}

/* Adjoint: FP64 recheck of queued pairs. */
__global__ void k_recheck_adj(const fcfcg_launch L) {
  const uint32_t nq = queue_len(L);
  unsigned long long n_in = 0;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq;
       q += gridDim.x * blockDim.x) {
    const uint4 e = ((const uint4 *) L.queue)[q];
    int bin = ref_bin_pair(L, e.x, e.y, e.z, L.box);
    if (bin < 0) continue;
    n_in++;
    adj_pair(L, e.x, e.y, bin);
  }
  for (int o = 16; o > 0; o >>= 1)
    n_in += __shfl_xor_sync(FULLMASK, n_in, o);
  if ((threadIdx.x & 31) == 0 && n_in) atomicAdd(L.stats + 1, n_in);
}

/* FP64 recheck of queued pairs. */
template <int WT>
__global__ void k_recheck(const fcfcg_launch L) {
  const uint32_t nq = queue_len(L);
  unsigned long long n_in = 0;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq;
       q += gridDim.x * blockDim.x) {
    const uint4 e = ((const uint4 *) L.queue)[q];
    const fcfcg_mock *M = L.mocks ? L.mocks + e.w : NULL;
    int bin = ref_bin_pair(L, e.x, e.y, e.z, M ? M->box : L.box);
    if (bin < 0) continue;
    n_in++;
    if (WT) add128((M ? M->gwt : L.gwt) + 2 * bin, fix_prod_pair(L, e.x, e.y));
    else atomicAdd((M ? M->gcnt : L.gcnt) + bin, 1ull);
  }
  for (int o = 16; o > 0; o >>= 1)
    n_in += __shfl_xor_sync(FULLMASK, n_in, o);
  if ((threadIdx.x & 31) == 0 && n_in) atomicAdd(L.stats + 1, n_in);
}

/* ------------------------------------------------------------------------ */

static kfun_t pick32(int geom, int bin, int wt, int batch, int adj) {
  if (adj) return fcfcg_pick32_adj(geom, bin);
  if (batch) return geom == FCFCG_GEOM_BOX ? fcfcg_pick32_batch(bin, wt) : 0;
  return geom == FCFCG_GEOM_BOX ? fcfcg_pick32_box(bin, wt)
                                : fcfcg_pick32_survey(bin, wt);
}

static kfun_t pick64(int geom, int wt, int adj) {
  if (adj)
    return geom == FCFCG_GEOM_BOX ? (kfun_t) k_count64<FCFCG_GEOM_BOX, 1, 1>
                                  : (kfun_t) k_count64<FCFCG_GEOM_SURVEY, 1, 1>;
  if (geom == FCFCG_GEOM_BOX)
    return wt ? (kfun_t) k_count64<FCFCG_GEOM_BOX, 1, 0>
              : (kfun_t) k_count64<FCFCG_GEOM_BOX, 0, 0>;
  return wt ? (kfun_t) k_count64<FCFCG_GEOM_SURVEY, 1, 0>
            : (kfun_t) k_count64<FCFCG_GEOM_SURVEY, 0, 0>;
}

extern "C" int fcfcg_k_count(void *stream, const fcfcg_launch *L,
    int precision, int nsm, size_t *smem_used, uint32_t *qwarp_used) {
  kfun_t f;
  size_t smem;
  int threads;
  fcfcg_launch Lq = *L;
  cudaError_t e;
  int per_sm = 0;
  if (precision == FCFCG_PREC_FP64) {
    f = pick64(L->geometry, L->withwt, L->adjoint);
    smem = (L->hist_smem && !L->adjoint)
               ? (size_t) L->ntot * (L->withwt ? 8 : 4) : 0;
    threads = CT_THREADS;
    if (!f) return (int) cudaErrorInvalidValue;
    if ((e = cudaFuncSetAttribute((const void *) f,
             cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)) ||
        (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
             &per_sm, (const void *) f, threads, smem)))
      return (int) e;
  } else {
    /* a bit-pattern s table selects the kernel's log variant */
    int bin = !L->fslog ? L->bintype
        : (L->bintype == FCFCG_BIN_SPI ? BIN_SPIL
           : (L->bintype == FCFCG_BIN_ISO ? BIN_ISOL : BIN_SMUL));
    /* linear s bins: the s bin from s itself */
    if (L->slin && L->bintype == FCFCG_BIN_ISO) bin = BIN_ISOLIN;
    if (L->slin && L->bintype == FCFCG_BIN_SMU) bin = BIN_SMULIN;
    f = pick32(L->geometry, bin, L->withwt, L->mocks != NULL, L->adjoint);
    if (!f) return (int) cudaErrorInvalidValue;
    size_t tab = fcfcg_k_count32_tab_bytes(L->nfs, L->nfp, L->nsb, L->npb);
    size_t fixed = tab + (L->hist_smem ? (size_t) L->ntot * (L->withwt ? 8 : 4)
                                        : 0);
    fixed = (fixed + 15) & ~(size_t) 15;
    threads = CT32_THREADS;
    /* the warp queue: as given, or the largest of 1024 / 512 / 256 entries
     * that reaches the most CTAs per SM the kernel can hold (a smaller
     * queue can free shared memory for another CTA) */
    const uint32_t cand[3] = {QWARP_MAX, 512u, QWARP_MIN};
    uint32_t q = 0;
    int best = 0, occ[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {
      if (L->qwarp && cand[k] != L->qwarp) continue;
      const size_t sm = fixed + stage_bytes(L->nsten, L->withwt + L->adjoint,
                                            cand[k]);
      if ((e = cudaFuncSetAttribute((const void *) f,
               cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm)))
        return (int) e;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
               &occ[k], (const void *) f, threads, sm)))
        return (int) e;
      if (occ[k] > best) best = occ[k];
    }
    for (int k = 0; k < 3 && !q; k++)
      if ((!L->qwarp || cand[k] == L->qwarp) && occ[k] == best && best > 0)
        q = cand[k];
    if (!q) return (int) cudaErrorInvalidConfiguration;
    smem = fixed + stage_bytes(L->nsten, L->withwt + L->adjoint, q);
    Lq.qwarp = q;
    if ((e = cudaFuncSetAttribute((const void *) f,
             cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)))
      return (int) e;
    per_sm = best;
    if (qwarp_used) *qwarp_used = q;
  }
  if (per_sm < 1) return (int) cudaErrorInvalidConfiguration;
  if (smem_used) *smem_used = smem;
  f<<<nsm * per_sm, threads, smem, (cudaStream_t) stream>>>(Lq);
  return (int) cudaGetLastError();
}

/* Shared memory of the FP32 tables and edges (aligned for the histogram). */
extern "C" size_t fcfcg_k_count32_tab_bytes(int nfs, int nfp, int nsb,
    int npb) {
  size_t n = (((size_t) (nfs + nfp) * 2 + 3) & ~(size_t) 3);
  n += sizeof(float) * ((size_t) nsb + 1 + (npb ? (size_t) npb + 1 : 0));
  return (n + 15) & ~(size_t) 15;
}

/* Shared memory the FP32 kernel needs beyond its histogram, with the
 * smallest warp queue (whether the kernel fits at all). */
extern "C" size_t fcfcg_k_count32_stage(int nsten, int withwt) {
  return stage_bytes(nsten, withwt, QWARP_MIN);
}

extern "C" int fcfcg_k_recheck(void *stream, const fcfcg_launch *L,
    uint32_t nq_bound) {
  if (!nq_bound) return 0;
  unsigned blocks = (nq_bound + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (L->adjoint)
    k_recheck_adj<<<blocks, 256, 0, (cudaStream_t) stream>>>(*L);
  else if (L->withwt)
    k_recheck<1><<<blocks, 256, 0, (cudaStream_t) stream>>>(*L);
  else
    k_recheck<0><<<blocks, 256, 0, (cudaStream_t) stream>>>(*L);
  return (int) cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* Allocation-free variant of the FP64 counting kernel.                     */

/*
 * Scratch of fcfcg_count_noalloc: the 64-bit bin accumulators followed by the
 * FP64 binning tables, in one fixed device array.  Every GPU that loads the
 * library keeps these bytes until the process exits.
 */
static __device__ __align__(256) unsigned char
    g_noalloc_scratch[FCFCG_NOALLOC_SCRATCH_BYTES];

#define NOALLOC_MAX_DEV 64
static void *g_noalloc_addr[NOALLOC_MAX_DEV];

#define NA_TILE 256

/* All pairs of two catalogues (raw FP64 coordinates on the device), each
 * pair binned by the reference's FP64 formula and counted in the scratch
 * accumulators.  Periodic images: the minimal image, with the shift on the
 * first catalogue's point (cross) or the smaller index (auto). */
template <int GEOM>
__global__ void __launch_bounds__(NA_TILE)
k_count64_noalloc(const fcfcg_launch L, double rescale, size_t na,
    const double *__restrict__ xa, const double *__restrict__ ya,
    const double *__restrict__ za, size_t nb, const double *__restrict__ xb,
    const double *__restrict__ yb, const double *__restrict__ zb,
    unsigned long long *acc) {
  __shared__ double tx[NA_TILE], ty[NA_TILE], tz[NA_TILE], ts[NA_TILE];
  const size_t ntile = (nb + NA_TILE - 1) / NA_TILE;
  const size_t nblk = (na + NA_TILE - 1) / NA_TILE;
  for (size_t w = blockIdx.x; w < nblk * ntile; w += gridDim.x) {
    const size_t ib = w / ntile, jt = w % ntile;
    if (L.isauto && jt < ib) continue;           /* j >= i blocks only */
    const size_t i = ib * NA_TILE + threadIdx.x;
    double x1 = 0, y1 = 0, z1 = 0, s1 = 0;
    if (i < na) {
      x1 = xa[i];
      y1 = ya[i];
      z1 = za[i];
      if (rescale != 1) {
        x1 = __dmul_rn(x1, rescale);
        y1 = __dmul_rn(y1, rescale);
        z1 = __dmul_rn(z1, rescale);
      }
      s1 = __dadd_rn(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)),
                     __dmul_rn(z1, z1));
    }
    __syncthreads();
    const size_t j0 = jt * NA_TILE;
    {
      const size_t j = j0 + threadIdx.x;
      double a = 0, b = 0, c = 0;
      if (j < nb) {
        a = xb[j];
        b = yb[j];
        c = zb[j];
        if (rescale != 1) {
          a = __dmul_rn(a, rescale);
          b = __dmul_rn(b, rescale);
          c = __dmul_rn(c, rescale);
        }
      }
      tx[threadIdx.x] = a;
      ty[threadIdx.x] = b;
      tz[threadIdx.x] = c;
      ts[threadIdx.x] = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)),
                                  __dmul_rn(c, c));
    }
    __syncthreads();
    if (i < na) {
      const int jn = (int) ((nb - j0 < NA_TILE) ? nb - j0 : NA_TILE);
      for (int k = 0; k < jn; k++) {
        const size_t j = j0 + (size_t) k;
        if (L.isauto && j <= i) continue;
        int bin;
        if (GEOM == FCFCG_GEOM_SURVEY) {
          bin = ref_bin_survey(L, x1, y1, z1, s1, tx[k], ty[k], tz[k], ts[k]);
        } else {
          const double d[3] = {__dsub_rn(x1, tx[k]), __dsub_rn(y1, ty[k]),
                               __dsub_rn(z1, tz[k])};
          const double p[3] = {x1, y1, z1}, q[3] = {tx[k], ty[k], tz[k]};
          double r[3];
          for (int a = 0; a < 3; a++) {
            const double hL = L.box[a] * 0.5;
            const double sh = (d[a] > hL) ? -L.box[a] : ((d[a] < -hL) ? L.box[a] : 0.0);
            r[a] = __dsub_rn(__dadd_rn(p[a], sh), q[a]);
          }
          bin = ref_bin_box(L, r[0], r[1], r[2]);
        }
        if (bin >= 0) atomicAdd(acc + bin, 1ull);
      }
    }
  }
}

__global__ void k_noalloc_copy(const unsigned long long *acc, long n,
    long long *out) {
  for (long i = blockIdx.x * (long) blockDim.x + threadIdx.x; i < n;
       i += (long) gridDim.x * blockDim.x)
    out[i] = (long long) acc[i];
}

static size_t na_align(size_t n) { return (n + 255) & ~(size_t) 255; }

extern "C" int fcfcg_count_noalloc(const fcfcg_ctx *bins_ctx, int isauto,
    size_t na, const double *xa, const double *ya, const double *za,
    size_t nb, const double *xb, const double *yb, const double *zb,
    long long *counts, void *stream) {
  const fcfcg_bins *b = fcfcg_ctx_bins(bins_ctx);
  if (!b || !counts || (na && (!xa || !ya || !za))) return FCFCG_ERR_ARG;
  if (isauto) {
    nb = na;
    xb = xa;
    yb = ya;
    zb = za;
  } else if (nb && (!xb || !yb || !zb)) {
    return FCFCG_ERR_ARG;
  }
  /* layout of the scratch: accumulators, then the reference tables */
  const size_t o_acc = 0;
  const size_t o_rs = na_align(o_acc + sizeof(unsigned long long) * b->ntot);
  const size_t o_se = na_align(o_rs + sizeof(uint16_t) * b->s.nrtab);
  const int spi = (b->bintype == FCFCG_BIN_SPI);
  const size_t o_rp = na_align(o_se + sizeof(double) * (b->s.nbin + 1));
  const size_t o_pe = na_align(o_rp + (spi ? sizeof(uint16_t) * b->p.nrtab : 0));
  const size_t end = o_pe + (spi ? sizeof(double) * (b->p.nbin + 1) : 0);
  if (end > FCFCG_NOALLOC_SCRATCH_BYTES) return FCFCG_ERR_UNSUPPORTED;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return FCFCG_ERR_CUDA;
  if (dev < 0 || dev >= NOALLOC_MAX_DEV) return FCFCG_ERR_UNSUPPORTED;
  if (!g_noalloc_addr[dev]) {
    /* first call on this device: the device address of the scratch array
     * (the host-side symbol is only a stand-in) */
    void *p = NULL;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e || !p) return FCFCG_ERR_CUDA;
    g_noalloc_addr[dev] = p;
  }
  unsigned char *base = (unsigned char *) g_noalloc_addr[dev];
  cudaStream_t st = (cudaStream_t) stream;
  fcfcg_launch L;
  memset(&L, 0, sizeof L);
  L.geometry = b->geometry;
  L.bintype = b->bintype;
  L.isauto = isauto;
  for (int k = 0; k < 3; k++) L.box[k] = b->box[k];
  L.ns = b->ns;
  L.nmu = b->nmu;
  L.mu_one = b->mu_one;
  L.np = b->np;
  L.ntot = b->ntot;
  L.rs = (const uint16_t *) (base + o_rs);
  L.rsoff = b->s.roff;
  L.nrs = b->s.nrtab;
  L.s2edge = (const double *) (base + o_se);
  L.s2min = b->s.vmin;
  L.s2max = b->s.vmax;
  L.smin0 = b->s.min0;
  if (spi) {
    L.rp = (const uint16_t *) (base + o_rp);
    L.rpoff = b->p.roff;
    L.nrp = b->p.nrtab;
    L.pedge = (const double *) (base + o_pe);
    L.pmin = b->p.vmin;
    L.pmax = b->p.vmax;
    L.pmin0 = b->p.min0;
  }
  unsigned long long *acc = (unsigned long long *) (base + o_acc);
  if ((e = cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * b->ntot, st)))
    return FCFCG_ERR_CUDA;
  if ((e = cudaMemcpyAsync(base + o_rs, b->s.rtab,
                           sizeof(uint16_t) * b->s.nrtab,
                           cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(base + o_se, b->s.edge,
                           sizeof(double) * (b->s.nbin + 1),
                           cudaMemcpyHostToDevice, st)))
    return FCFCG_ERR_CUDA;
  if (spi &&
      ((e = cudaMemcpyAsync(base + o_rp, b->p.rtab,
                            sizeof(uint16_t) * b->p.nrtab,
                            cudaMemcpyHostToDevice, st)) ||
       (e = cudaMemcpyAsync(base + o_pe, b->p.edge,
                            sizeof(double) * (b->p.nbin + 1),
                            cudaMemcpyHostToDevice, st))))
    return FCFCG_ERR_CUDA;
  if (na && nb) {
    const size_t work = ((na + NA_TILE - 1) / NA_TILE) *
                        ((nb + NA_TILE - 1) / NA_TILE);
    const unsigned blocks = (unsigned) (work < 152 * 8 ? work : 152 * 8);
    if (b->geometry == FCFCG_GEOM_SURVEY)
      k_count64_noalloc<FCFCG_GEOM_SURVEY><<<blocks, NA_TILE, 0, st>>>(
          L, b->rescale, na, xa, ya, za, nb, xb, yb, zb, acc);
    else
      k_count64_noalloc<FCFCG_GEOM_BOX><<<blocks, NA_TILE, 0, st>>>(
          L, b->rescale, na, xa, ya, za, nb, xb, yb, zb, acc);
    if ((e = cudaGetLastError())) return FCFCG_ERR_CUDA;
  }
  k_noalloc_copy<<<(unsigned) ((b->ntot + 255) / 256 < 1024 ? (b->ntot + 255) / 256 : 1024),
                   256, 0, st>>>(acc, b->ntot, counts);
  if ((e = cudaGetLastError())) return FCFCG_ERR_CUDA;
  return FCFCG_OK;
}
