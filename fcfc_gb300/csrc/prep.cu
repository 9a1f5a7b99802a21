/*
 * prep.cu -- catalogue preparation on the device: rescaling (as FCFC's
 * tree_create does, src/fcfc/2pt_box/build_tree.c:121-131), |x|^2 for
 * surveys (src/fcfc/2pt/build_tree.c:35-133), weight range, bounding box,
 * and the cell grid: a counting sort of the points into cells, stored as
 * SoA FP64 copies plus one float4 per point (FP32 offsets from the cell
 * centre and the scaled high part of the weight) for the FP32 kernels.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fcfcg_internal.h"

#define PREP_THREADS 256
#define SCAN_THREADS 1024
#define SCAN_ITEMS 4
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

static int grid_for(size_t n, int threads) {
  size_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int) b;
}

/* Order-preserving map of a double to an unsigned key. */
__device__ __forceinline__ unsigned long long dkey(double v) {
  unsigned long long b = (unsigned long long) __double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_prep(size_t n, const double *__restrict__ x,
    const double *__restrict__ y, const double *__restrict__ z,
    const double *__restrict__ w, double rescale, int survey,
    double *__restrict__ ox, double *__restrict__ oy, double *__restrict__ oz,
    double *__restrict__ os, double *__restrict__ ow,
    unsigned long long *wmax_bits, double *__restrict__ partial) {
  __shared__ double sh_sum[PREP_THREADS];
  unsigned long long wm = 0;
  double ws = 0;
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    double a = x[i], b = y[i], c = z[i];
    if (rescale != 1) {
      a = __dmul_rn(a, rescale);
      b = __dmul_rn(b, rescale);
      c = __dmul_rn(c, rescale);
    }
    ox[i] = a;
    oy[i] = b;
    oz[i] = c;
    if (survey)
      os[i] = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)),
                        __dmul_rn(c, c));
    if (w) {
      double v = w[i];
      ow[i] = v;
      ws = __dadd_rn(ws, v);
      unsigned long long bits =
          (unsigned long long) __double_as_longlong(fabs(v));
      wm = bits > wm ? bits : wm;
    }
  }
  if (w && partial) {
    /* this block's weight sum, in a fixed order (deterministic) */
    sh_sum[threadIdx.x] = ws;
    __syncthreads();
    for (int o = PREP_THREADS / 2; o > 0; o >>= 1) {
      if ((int) threadIdx.x < o)
        sh_sum[threadIdx.x] = __dadd_rn(sh_sum[threadIdx.x],
                                        sh_sum[threadIdx.x + o]);
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh_sum[0];
  }
  if (w) {
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long t = __shfl_xor_sync(0xffffffffu, wm, o);
      wm = t > wm ? t : wm;
    }
    if ((threadIdx.x & 31) == 0 && wm) atomicMax(wmax_bits, wm);
  }
}

/* Sum of the per-block partial sums, in a fixed order. */
__global__ void k_sum_partials(int nb, const double *__restrict__ partial,
    double *out) {
  __shared__ double sh[PREP_THREADS];
  double v = 0;
  for (int i = threadIdx.x; i < nb; i += PREP_THREADS)
    v = __dadd_rn(v, partial[i]);
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = PREP_THREADS / 2; o > 0; o >>= 1) {
    if ((int) threadIdx.x < o)
      sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

extern "C" size_t fcfcg_prep_partials(void) { return 152 * 32; }

extern "C" int fcfcg_k_prep(void *stream, size_t n, const double *x,
    const double *y, const double *z, const double *w, double rescale,
    int survey, double *ox, double *oy, double *oz, double *os, double *ow,
    unsigned long long *wmax_bits, double *partial, double *wsum) {
  if (!n) return 0;
  const int nb = grid_for(n, PREP_THREADS);
  k_prep<<<nb, PREP_THREADS, 0, (cudaStream_t) stream>>>(
      n, x, y, z, w, rescale, survey, ox, oy, oz, os, ow, wmax_bits,
      (w && wsum) ? partial : NULL);
  cudaError_t e = cudaGetLastError();
  if (e || !w || !wsum) return (int) e;
  k_sum_partials<<<1, PREP_THREADS, 0, (cudaStream_t) stream>>>(nb, partial,
                                                                 wsum);
  return (int) cudaGetLastError();
}

__global__ void k_bbox(size_t n, const double *__restrict__ x,
    const double *__restrict__ y, const double *__restrict__ z,
    unsigned long long *bits6) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  const double *p[3] = {x, y, z};
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    for (int k = 0; k < 3; k++) {
      unsigned long long v = dkey(p[k][i]);
      lo[k] = v < lo[k] ? v : lo[k];
      hi[k] = v > hi[k] ? v : hi[k];
    }
  }
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long a = __shfl_xor_sync(0xffffffffu, lo[k], o);
      unsigned long long b = __shfl_xor_sync(0xffffffffu, hi[k], o);
      lo[k] = a < lo[k] ? a : lo[k];
      hi[k] = b > hi[k] ? b : hi[k];
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(bits6 + k, lo[k]);
      atomicMax(bits6 + 3 + k, hi[k]);
    }
  }
}

extern "C" int fcfcg_k_bbox(void *stream, size_t n, const double *x,
    const double *y, const double *z, unsigned long long *bits6) {
  if (!n) return 0;
  k_bbox<<<grid_for(n, PREP_THREADS), PREP_THREADS, 0,
           (cudaStream_t) stream>>>(n, x, y, z, bits6);
  return (int) cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* Exclusive scan of uint32 (n + 1 outputs: out[n] = total).               */

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v,
    uint32_t *sh_warp, uint32_t *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) sh_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t s = (lane < (int) (blockDim.x >> 5)) ? sh_warp[lane] : 0;
    uint32_t si = s;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    sh_warp[lane] = si - s;
    if (lane == 31) *total = si;
  }
  __syncthreads();
  uint32_t r = sh_warp[wid] + inc - v;
  __syncthreads();
  return r;
}

__global__ void k_scan_tiles(const uint32_t *__restrict__ in, size_t n,
    uint32_t *__restrict__ tile_sum) {
  __shared__ uint32_t shw[32];
  __shared__ uint32_t tot;
  size_t base = (size_t) blockIdx.x * SCAN_TILE;
  uint32_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + (size_t) k * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  block_excl_scan(s, shw, &tot);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

__global__ void k_scan_sums(uint32_t *__restrict__ tile_sum, size_t ntile) {
  __shared__ uint32_t shw[32];
  __shared__ uint32_t tot;
  uint32_t carry = 0;
  for (size_t b = 0; b < ntile; b += SCAN_THREADS) {
    size_t i = b + threadIdx.x;
    uint32_t v = (i < ntile) ? tile_sum[i] : 0;
    uint32_t e = block_excl_scan(v, shw, &tot);
    if (i < ntile) tile_sum[i] = e + carry;
    carry += tot;
    __syncthreads();
  }
}

__global__ void k_scan_apply(const uint32_t *__restrict__ in, size_t n,
    const uint32_t *__restrict__ tile_sum, uint32_t *__restrict__ out) {
  __shared__ uint32_t shw[32];
  __shared__ uint32_t tot;
  size_t base = (size_t) blockIdx.x * SCAN_TILE;
  /* each thread owns SCAN_ITEMS consecutive items */
  uint32_t v[SCAN_ITEMS];
  uint32_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + (size_t) threadIdx.x * SCAN_ITEMS + k;
    v[k] = (i < n) ? in[i] : 0;
    s += v[k];
  }
  uint32_t e = block_excl_scan(s, shw, &tot) + tile_sum[blockIdx.x];
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + (size_t) threadIdx.x * SCAN_ITEMS + k;
    if (i < n) out[i] = e;
    e += v[k];
    if (i == n - 1) out[n] = e;
  }
}

extern "C" size_t fcfcg_scan_tmp_len(size_t n) {
  return (n + SCAN_TILE - 1) / SCAN_TILE + 1;
}

/* out[0..n] = exclusive scan of in[0..n-1], out[n] = total. */
static int scan_u32(cudaStream_t s, const uint32_t *in, size_t n,
    uint32_t *out, uint32_t *tmp) {
  if (n == 0) {
    return (int) cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
  }
  size_t ntile = (n + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<(unsigned) ntile, SCAN_THREADS, 0, s>>>(in, n, tmp);
  k_scan_sums<<<1, SCAN_THREADS, 0, s>>>(tmp, ntile);
  k_scan_apply<<<(unsigned) ntile, SCAN_THREADS, 0, s>>>(in, n, tmp, out);
  return (int) cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* Cell grid.                                                               */

/*
 * The fine index of a point: its global cell (cells of one grid numbered
 * from cell_base), shifted left by sb, and with sb = 3 or 6 its sub-cell
 * (2 or 4 per axis) in Morton order.  Sorting by the fine index keeps each
 * cell's points contiguous and, within the cell, groups them by sub-cell,
 * so that runs of 32 or 64 consecutive points (the count kernel's
 * neighbour blocks and chunks) are compact.  The cell of an axis is
 * floor((v - lo) / cw) clamped to [0, n).
 */
__device__ __forceinline__ uint32_t fine_of_point(double a, double b,
    double d, int nx, int ny, int nz, double cwx, double cwy, double cwz,
    double lox, double loy, double loz, uint32_t cell_base, int sb) {
  const double v[3] = {a, b, d}, lo[3] = {lox, loy, loz},
               cw[3] = {cwx, cwy, cwz};
  const int n[3] = {nx, ny, nz};
  const int r = sb / 3;                   /* bits per axis */
  int c[3];
  uint32_t m = 0;
  for (int k = 0; k < 3; k++) {
    const double q = (v[k] - lo[k]) / cw[k];
    const double t = floor(q);
    c[k] = (t < 0) ? 0 : (t >= n[k] ? n[k] - 1 : (int) t);
    if (r) {
      const int lim = (1 << r) - 1;
      int s = (int) floor((q - (double) c[k]) * (double) (1 << r));
      s = s < 0 ? 0 : (s > lim ? lim : s);
      for (int bit = 0; bit < r; bit++)
        m |= (uint32_t) ((s >> bit) & 1) << (3 * bit + k);
    }
  }
  const uint32_t cell = cell_base + ((uint32_t) c[2] * ny + c[1]) * nx + c[0];
  return (cell << sb) | m;
}

__global__ void k_cell(size_t n, const double *__restrict__ x,
    const double *__restrict__ y, const double *__restrict__ z, int nx,
    int ny, int nz, double cwx, double cwy, double cwz, double lox,
    double loy, double loz, uint32_t cell_base, int sb,
    uint32_t *__restrict__ cell_of, uint32_t *__restrict__ count) {
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    uint32_t c = fine_of_point(x[i], y[i], z[i], nx, ny, nz, cwx, cwy, cwz,
                               lox, loy, loz, cell_base, sb);
    cell_of[i] = c;
    atomicAdd(count + c, 1u);
  }
}

/* Point i (input order) of a grid to its sorted place pos: the FP32
 * offsets from its cell centre and its weight's scaled high part (l4), the
 * weight's fixed-point split (wq), FP64 copies and its id. */
__device__ __forceinline__ void scatter_point(uint32_t c, uint32_t pos,
    double a, double b, double d, double wv, int wexp, int nx, int ny,
    double cwx, double cwy, double cwz, double lox, double loy, double loz,
    uint32_t cell_base, uint32_t id, float4 *__restrict__ l4,
    int2 *__restrict__ wq, double *__restrict__ sx, double *__restrict__ sy,
    double *__restrict__ sz, double *__restrict__ sw,
    uint32_t *__restrict__ sid) {
  const uint32_t cl = c - cell_base;
  int cx = (int) (cl % (uint32_t) nx);
  int cy = (int) ((cl / (uint32_t) nx) % (uint32_t) ny);
  int cz = (int) (cl / ((uint32_t) nx * (uint32_t) ny));
  double ccx = lox + (cx + 0.5) * cwx;
  double ccy = loy + (cy + 0.5) * cwy;
  double ccz = loz + (cz + 0.5) * cwz;
  double ws = ldexp(wv, -wexp);            /* |ws| <= 1 */
  int wi = (int) __double2ll_rn(ws * 1073741824.0);
  float wr = (float) (ws - (double) wi * (1.0 / 1073741824.0));
  float4 v;
  v.x = (float) (a - ccx);
  v.y = (float) (b - ccy);
  v.z = (float) (d - ccz);
  v.w = (float) ws;
  l4[pos] = v;
  wq[pos] = make_int2(wi, __float_as_int(wr));
  sx[pos] = a;
  sy[pos] = b;
  sz[pos] = d;
  sw[pos] = wv;
  sid[pos] = id;
}

__global__ void k_scatter(size_t n, const double *__restrict__ x,
    const double *__restrict__ y, const double *__restrict__ z,
    const double *__restrict__ s, const double *__restrict__ w, int has_w,
    int wexp, int nx, int ny, double cwx, double cwy, double cwz, double lox,
    double loy, double loz, uint32_t cell_base, uint32_t id_base, int sb,
    const uint32_t *__restrict__ cell_of,
    const uint32_t *__restrict__ fstart, uint32_t *__restrict__ cfill,
    float4 *__restrict__ l4, int2 *__restrict__ wq, double *__restrict__ sx,
    double *__restrict__ sy, double *__restrict__ sz, double *__restrict__ ss,
    double *__restrict__ sw, uint32_t *__restrict__ sid) {
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    const uint32_t f = cell_of[i];
    uint32_t pos = fstart[f] + atomicAdd(cfill + f, 1u);
    scatter_point(f >> sb, pos, x[i], y[i], z[i], has_w ? w[i] : 1.0, wexp, nx, ny,
                  cwx, cwy, cwz, lox, loy, loz, cell_base,
                  id_base + (uint32_t) i, l4, wq, sx, sy, sz, sw, sid);
    if (ss) ss[pos] = s[i];
  }
}

/* cstart[c] = fstart[c << sb], c = 0..nc: the cells' first sorted points
 * from the fine (sub-cell) starts. */
__global__ void k_cstart(size_t nc, int sb, const uint32_t *__restrict__ fstart,
    uint32_t *__restrict__ cstart) {
  for (size_t c = blockIdx.x * (size_t) blockDim.x + threadIdx.x; c <= nc;
       c += (size_t) gridDim.x * blockDim.x)
    cstart[c] = fstart[c << sb];
}

extern "C" int fcfcg_grid_sub_bits(size_t ncell, size_t npoint) {
  /* sub-cells where cells hold many points on average, with the fine
   * counters at most ~4 per point (and 32-bit fine indices) */
  const size_t lim = npoint * 4 > ((size_t) 1 << 22) ? npoint * 4
                                                   : ((size_t) 1 << 22);
  if (ncell << 6 <= lim && (ncell << 6) < 0xFFFFFFF0u) return 6;
  if (ncell << 3 <= lim && (ncell << 3) < 0xFFFFFFF0u) return 3;
  return 0;
}

extern "C" int fcfcg_k_grid(void *stream, size_t n, const double *x,
    const double *y, const double *z, const double *s, const double *w,
    int has_w, int wexp, const int ncell[3], const double cw[3],
    const double lo[3], int sb, uint32_t *cell_of, uint32_t *cstart,
    uint32_t *fstart, uint32_t *cfill, uint32_t *scan_tmp,
    size_t scan_tmp_len, float *l4, int *wq, double *sx, double *sy,
    double *sz, double *ss, double *sw, uint32_t *sid) {
  cudaStream_t st = (cudaStream_t) stream;
  const size_t nc = (size_t) ncell[0] * ncell[1] * ncell[2];
  const size_t nf = nc << sb;
  (void) scan_tmp_len;
  cudaError_t e = cudaMemsetAsync(cfill, 0, sizeof(uint32_t) * nf, st);
  if (e) return (int) e;
  if (n) {
    k_cell<<<grid_for(n, PREP_THREADS), PREP_THREADS, 0, st>>>(
        n, x, y, z, ncell[0], ncell[1], ncell[2], cw[0], cw[1], cw[2], lo[0],
        lo[1], lo[2], 0u, sb, cell_of, cfill);
    if ((e = cudaGetLastError())) return (int) e;
  }
  int r = scan_u32(st, cfill, nf, fstart, scan_tmp);
  if (r) return r;
  k_cstart<<<grid_for(nc + 1, PREP_THREADS), PREP_THREADS, 0, st>>>(
      nc, sb, fstart, cstart);
  if ((e = cudaGetLastError())) return (int) e;
  if ((e = cudaMemsetAsync(cfill, 0, sizeof(uint32_t) * nf, st))) return (int) e;
  if (n) {
    k_scatter<<<grid_for(n, PREP_THREADS), PREP_THREADS, 0, st>>>(
        n, x, y, z, s, w, has_w, wexp, ncell[0], ncell[1], cw[0], cw[1],
        cw[2], lo[0], lo[1], lo[2], 0u, 0u, sb, cell_of, fstart, cfill,
        (float4 *) l4, (int2 *) wq, sx, sy, sz, ss, sw, sid);
    if ((e = cudaGetLastError())) return (int) e;
  }
  return 0;
}

extern "C" int fcfcg_k_cstart(void *stream, size_t nc, int sb,
    const uint32_t *fstart, uint32_t *cstart) {
  k_cstart<<<grid_for(nc + 1, PREP_THREADS), PREP_THREADS, 0,
             (cudaStream_t) stream>>>(nc, sb, fstart, cstart);
  return (int) cudaGetLastError();
}

extern "C" int fcfcg_scan(void *stream, const uint32_t *in, size_t n,
    uint32_t *out, uint32_t *tmp) {
  return scan_u32((cudaStream_t) stream, in, n, out, tmp);
}

/* ------------------------------------------------------------------------ */
/* Batches: one launch per stage over every catalogue.  Block t handles tile
 * t (BATCH_TILE points of one catalogue); the catalogue table lists each
 * catalogue's first tile, so a block finds its catalogue by bisection. */

#define BATCH_ITEMS 8
#define BATCH_TILE (PREP_THREADS * BATCH_ITEMS)

extern "C" size_t fcfcg_batch_tile(void) { return BATCH_TILE; }

__device__ __forceinline__ int batch_cat(const fcfcg_prep_cat *__restrict__ cat,
    int ncat, uint32_t t) {
  int lo = 0, hi = ncat;          /* the last lo with cat[lo].tile0 <= t */
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (cat[mid].tile0 <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

/* Rescale every catalogue into the batch slot (as k_prep), with each
 * catalogue's bounding box (order-preserving keys, bstat[8a + 0..5]), max
 * |w| bits (bstat[8a + 6]) and this tile's weight sum in a fixed order
 * (partial[t]). */
__global__ void __launch_bounds__(PREP_THREADS) k_prep_batch(
    const fcfcg_prep_cat *__restrict__ cat, int ncat, double rescale,
    int withwt, double *ox, double *oy, double *oz, double *ow,
    unsigned long long *bstat, double *__restrict__ partial) {
  __shared__ double sh_sum[PREP_THREADS];
  const uint32_t t = blockIdx.x;
  const int a = batch_cat(cat, ncat, t);
  const fcfcg_prep_cat *C = cat + a;
  const double *x = C->x, *y = C->y, *z = C->z, *w = withwt ? C->w : NULL;
  const size_t o = C->o, n = C->n;
  const size_t i0 = (size_t) (t - C->tile0) * BATCH_TILE;
  const size_t i1 = (i0 + BATCH_TILE < n) ? i0 + BATCH_TILE : n;
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  unsigned long long wm = 0;
  double ws = 0;
  for (size_t i = i0 + threadIdx.x; i < i1; i += PREP_THREADS) {
    double v[3] = {x[i], y[i], z[i]};
    if (rescale != 1)
      for (int k = 0; k < 3; k++) v[k] = __dmul_rn(v[k], rescale);
    ox[o + i] = v[0];
    oy[o + i] = v[1];
    oz[o + i] = v[2];
    for (int k = 0; k < 3; k++) {
      const unsigned long long q = dkey(v[k]);
      lo[k] = q < lo[k] ? q : lo[k];
      hi[k] = q > hi[k] ? q : hi[k];
    }
    if (w) {
      const double u = w[i];
      ow[o + i] = u;
      ws = __dadd_rn(ws, u);
      const unsigned long long bits =
          (unsigned long long) __double_as_longlong(fabs(u));
      wm = bits > wm ? bits : wm;
    }
  }
  unsigned long long *B = bstat + 8 * (size_t) a;
  for (int k = 0; k < 3; k++) {
    for (int s = 16; s > 0; s >>= 1) {
      const unsigned long long p = __shfl_xor_sync(0xffffffffu, lo[k], s);
      const unsigned long long q = __shfl_xor_sync(0xffffffffu, hi[k], s);
      lo[k] = p < lo[k] ? p : lo[k];
      hi[k] = q > hi[k] ? q : hi[k];
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(B + k, lo[k]);
      atomicMax(B + 3 + k, hi[k]);
    }
  }
  if (!withwt) return;
  for (int s = 16; s > 0; s >>= 1) {
    const unsigned long long p = __shfl_xor_sync(0xffffffffu, wm, s);
    wm = p > wm ? p : wm;
  }
  if ((threadIdx.x & 31) == 0 && wm) atomicMax(B + 6, wm);
  sh_sum[threadIdx.x] = ws;
  __syncthreads();
  for (int s = PREP_THREADS / 2; s > 0; s >>= 1) {
    if ((int) threadIdx.x < s)
      sh_sum[threadIdx.x] = __dadd_rn(sh_sum[threadIdx.x],
                                      sh_sum[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[t] = sh_sum[0];
}

/* Block a: catalogue a's weight sum from its tiles' sums, in a fixed order,
 * into bstat[8a + 7] (as a double). */
__global__ void __launch_bounds__(PREP_THREADS) k_sum_batch(
    const fcfcg_prep_cat *__restrict__ cat, int ncat, uint32_t ntile,
    const double *__restrict__ partial, unsigned long long *bstat) {
  __shared__ double sh[PREP_THREADS];
  const int a = blockIdx.x;
  const uint32_t t0 = cat[a].tile0;
  const uint32_t t1 = (a + 1 < ncat) ? cat[a + 1].tile0 : ntile;
  double v = 0;
  for (uint32_t t = t0 + threadIdx.x; t < t1; t += PREP_THREADS)
    v = __dadd_rn(v, partial[t]);
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = PREP_THREADS / 2; s > 0; s >>= 1) {
    if ((int) threadIdx.x < s)
      sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    bstat[8 * (size_t) a + 7] =
        (unsigned long long) __double_as_longlong(sh[0]);
}

extern "C" int fcfcg_k_prep_batch(void *stream, const fcfcg_prep_cat *d_cat,
    int ncat, uint32_t ntile, double rescale, int withwt, double *ox,
    double *oy, double *oz, double *ow, unsigned long long *bstat,
    double *partial) {
  if (!ncat || !ntile) return 0;
  cudaStream_t st = (cudaStream_t) stream;
  k_prep_batch<<<ntile, PREP_THREADS, 0, st>>>(d_cat, ncat, rescale, withwt,
                                               ox, oy, oz, ow, bstat,
                                               partial);
  cudaError_t e = cudaGetLastError();
  if (e || !withwt) return (int) e;
  k_sum_batch<<<ncat, PREP_THREADS, 0, st>>>(d_cat, ncat, ntile, partial,
                                             bstat);
  return (int) cudaGetLastError();
}

/* Cells of every live catalogue's points (slot arrays x, y, z), numbered
 * from the catalogue's cell_base into the shared count array. */
__global__ void __launch_bounds__(PREP_THREADS) k_cell_batch(
    const fcfcg_prep_cat *__restrict__ cat, int ncat, int sb,
    const double *__restrict__ x, const double *__restrict__ y,
    const double *__restrict__ z, uint32_t *__restrict__ cell_of,
    uint32_t *__restrict__ count) {
  const uint32_t t = blockIdx.x;
  const fcfcg_prep_cat *C = cat + batch_cat(cat, ncat, t);
  if (!C->live) return;
  const size_t o = C->o, n = C->n;
  const size_t i0 = (size_t) (t - C->tile0) * BATCH_TILE;
  const size_t i1 = (i0 + BATCH_TILE < n) ? i0 + BATCH_TILE : n;
  const int nx = C->ncell[0], ny = C->ncell[1], nz = C->ncell[2];
  const double cwx = C->cw[0], cwy = C->cw[1], cwz = C->cw[2];
  const uint32_t base = C->cell_base;
  for (size_t i = o + i0 + threadIdx.x; i < o + i1; i += PREP_THREADS) {
    const uint32_t c = fine_of_point(x[i], y[i], z[i], nx, ny, nz, cwx, cwy,
                                     cwz, 0.0, 0.0, 0.0, base, sb);
    cell_of[i] = c;
    atomicAdd(count + c, 1u);
  }
}

/* Every live catalogue's points to their sorted places (as k_scatter); the
 * id of point i of the slot is i. */
__global__ void __launch_bounds__(PREP_THREADS) k_scatter_batch(
    const fcfcg_prep_cat *__restrict__ cat, int ncat, int sb,
    const double *__restrict__ x, const double *__restrict__ y,
    const double *__restrict__ z, const double *__restrict__ w, int has_w,
    const uint32_t *__restrict__ cell_of,
    const uint32_t *__restrict__ fstart, uint32_t *__restrict__ cfill,
    float4 *__restrict__ l4, int2 *__restrict__ wq, double *__restrict__ sx,
    double *__restrict__ sy, double *__restrict__ sz, double *__restrict__ sw,
    uint32_t *__restrict__ sid) {
  const uint32_t t = blockIdx.x;
  const fcfcg_prep_cat *C = cat + batch_cat(cat, ncat, t);
  if (!C->live) return;
  const size_t o = C->o, n = C->n;
  const size_t i0 = (size_t) (t - C->tile0) * BATCH_TILE;
  const size_t i1 = (i0 + BATCH_TILE < n) ? i0 + BATCH_TILE : n;
  const int nx = C->ncell[0], ny = C->ncell[1], wexp = C->wexp;
  const double cwx = C->cw[0], cwy = C->cw[1], cwz = C->cw[2];
  const uint32_t base = C->cell_base;
  for (size_t i = o + i0 + threadIdx.x; i < o + i1; i += PREP_THREADS) {
    const uint32_t f = cell_of[i];
    const uint32_t pos = fstart[f] + atomicAdd(cfill + f, 1u);
    scatter_point(f >> sb, pos, x[i], y[i], z[i], has_w ? w[i] : 1.0, wexp, nx, ny,
                  cwx, cwy, cwz, 0.0, 0.0, 0.0, base, (uint32_t) i, l4, wq,
                  sx, sy, sz, sw, sid);
  }
}

extern "C" int fcfcg_k_cell_batch(void *stream, const fcfcg_prep_cat *d_cat,
    int ncat, uint32_t ntile, int sb, const double *x, const double *y,
    const double *z, uint32_t *cell_of, uint32_t *count) {
  if (!ncat || !ntile) return 0;
  k_cell_batch<<<ntile, PREP_THREADS, 0, (cudaStream_t) stream>>>(
      d_cat, ncat, sb, x, y, z, cell_of, count);
  return (int) cudaGetLastError();
}

extern "C" int fcfcg_k_scatter_batch(void *stream,
    const fcfcg_prep_cat *d_cat, int ncat, uint32_t ntile, int sb,
    const double *x, const double *y, const double *z, const double *w,
    int has_w, const uint32_t *cell_of, const uint32_t *fstart,
    uint32_t *cfill, float *l4, int *wq, double *sx, double *sy, double *sz,
    double *sw, uint32_t *sid) {
  if (!ncat || !ntile) return 0;
  k_scatter_batch<<<ntile, PREP_THREADS, 0, (cudaStream_t) stream>>>(
      d_cat, ncat, sb, x, y, z, w, has_w, cell_of, fstart, cfill, (float4 *) l4,
      (int2 *) wq, sx, sy, sz, sw, sid);
  return (int) cudaGetLastError();
}

/* Work chunks: every cell is cut into pieces of at most clen points, as
 * evenly as possible. */
__global__ void k_chunk_count(const uint32_t *__restrict__ cstart,
    uint32_t ncell, uint32_t clen, uint32_t *__restrict__ cchunk) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
       c += gridDim.x * blockDim.x) {
    uint32_t m = cstart[c + 1] - cstart[c];
    cchunk[c] = (m + clen - 1) / clen;
  }
}

/* mbase (nmock + 1 entries, may be NULL): first cell of each catalogue of a
 * batch; the chunk's .w is the catalogue holding its cell. */
__global__ void k_chunk_emit(const uint32_t *__restrict__ cstart,
    uint32_t ncell, uint32_t clen, const uint32_t *__restrict__ coff,
    uint4 *__restrict__ chunks, const uint32_t *__restrict__ mbase,
    int nmock) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
       c += gridDim.x * blockDim.x) {
    uint32_t a = cstart[c], m = cstart[c + 1] - a;
    uint32_t k = coff[c];
    uint32_t nch = (m + clen - 1) / clen;
    uint32_t mk = 0;
    if (mbase) {
      int lo = 0, hi = nmock;   /* last lo with mbase[lo] <= c */
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (mbase[mid] <= c) lo = mid;
        else hi = mid;
      }
      mk = (uint32_t) lo;
    }
    for (uint32_t q = 0; q < nch; q++) {
      uint32_t b0 = (uint32_t) (((unsigned long long) m * q) / nch);
      uint32_t b1 = (uint32_t) (((unsigned long long) m * (q + 1)) / nch);
      chunks[k++] = make_uint4(c, a + b0, b1 - b0, mk);
    }
  }
}

extern "C" int fcfcg_k_chunks(void *stream, const uint32_t *cstart,
    uint32_t ncell, uint32_t clen, uint32_t *cchunk, uint32_t *scan_tmp,
    size_t scan_tmp_len, uint32_t *chunks, uint32_t *nchunk_out,
    const uint32_t *mock_cell_base, int nmock) {
  cudaStream_t st = (cudaStream_t) stream;
  (void) scan_tmp_len;
  k_chunk_count<<<grid_for(ncell, PREP_THREADS), PREP_THREADS, 0, st>>>(
      cstart, ncell, clen, cchunk);
  cudaError_t e = cudaGetLastError();
  if (e) return (int) e;
  /* cchunk holds ncell + 1 slots: scan in place via the offset array */
  uint32_t *coff = cchunk + ncell + 1;
  int r = scan_u32(st, cchunk, ncell, coff, scan_tmp);
  if (r) return r;
  if (chunks) {
    k_chunk_emit<<<grid_for(ncell, PREP_THREADS), PREP_THREADS, 0, st>>>(
        cstart, ncell, clen, coff, (uint4 *) chunks, mock_cell_base, nmock);
    if ((e = cudaGetLastError())) return (int) e;
  }
  if (nchunk_out)
    if ((e = cudaMemcpyAsync(nchunk_out, coff + ncell, sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, st)))
      return (int) e;
  return 0;
}

/* Occupancy of a coarse grid over a catalogue's bounding box: one bit per
 * cell that holds an object (the occupied-volume estimate of a survey). */
__global__ void k_occupy(size_t n, const double *__restrict__ x,
    const double *__restrict__ y, const double *__restrict__ z, double lox,
    double loy, double loz, double icx, double icy, double icz, int nx,
    int ny, int nz, uint32_t *__restrict__ bits) {
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    int cx = (int) floor((x[i] - lox) * icx);
    int cy = (int) floor((y[i] - loy) * icy);
    int cz = (int) floor((z[i] - loz) * icz);
    cx = cx < 0 ? 0 : (cx >= nx ? nx - 1 : cx);
    cy = cy < 0 ? 0 : (cy >= ny ? ny - 1 : cy);
    cz = cz < 0 ? 0 : (cz >= nz ? nz - 1 : cz);
    const size_t c = ((size_t) cz * ny + cy) * nx + cx;
    atomicOr(bits + (c >> 5), 1u << (c & 31));
  }
}

__global__ void k_popc(size_t nw, const uint32_t *__restrict__ bits,
    unsigned long long *count) {
  unsigned long long t = 0;
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < nw;
       i += (size_t) gridDim.x * blockDim.x)
    t += (unsigned long long) __popc(bits[i]);
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0 && t) atomicAdd(count, t);
}

extern "C" int fcfcg_k_occupancy(void *stream, size_t n, const double *x,
    const double *y, const double *z, const double lo[3], const int dim[3],
    const double inv_cell[3], uint32_t *bits, size_t nw,
    unsigned long long *count) {
  cudaStream_t st = (cudaStream_t) stream;
  cudaError_t e = cudaMemsetAsync(bits, 0, sizeof(uint32_t) * nw, st);
  if (!e) e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
  if (e) return (int) e;
  if (n) {
    k_occupy<<<grid_for(n, PREP_THREADS), PREP_THREADS, 0, st>>>(
        n, x, y, z, lo[0], lo[1], lo[2], inv_cell[0], inv_cell[1],
        inv_cell[2], dim[0], dim[1], dim[2], bits);
    if ((e = cudaGetLastError())) return (int) e;
  }
  k_popc<<<grid_for(nw, PREP_THREADS), PREP_THREADS, 0, st>>>(nw, bits,
                                                               count);
  return (int) cudaGetLastError();
}

__global__ void k_unsort(size_t n, const uint32_t *__restrict__ sid,
    const double *__restrict__ in, double *__restrict__ out) {
  for (size_t p = blockIdx.x * (size_t) blockDim.x + threadIdx.x; p < n;
       p += (size_t) gridDim.x * blockDim.x)
    out[sid[p]] = in[p];
}

extern "C" int fcfcg_k_unsort(void *stream, size_t n, const uint32_t *sid,
    const double *in, double *out) {
  if (!n) return 0;
  k_unsort<<<grid_for(n, PREP_THREADS), PREP_THREADS, 0,
             (cudaStream_t) stream>>>(n, sid, in, out);
  return (int) cudaGetLastError();
}

extern "C" const char *fcfcg_cuda_errstr(int code) {
  return cudaGetErrorString((cudaError_t) code);
}
