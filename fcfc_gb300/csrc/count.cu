/*
 * count.cu -- pair-counting kernels.
 *
 * Work decomposition (replaces FCFC's dual k-d tree, src/fcfc/2pt_box/
 * dual_tree.c:245-373, and its OpenMP/MPI node-pair scheduler,
 * count_func.c:7431-7722):
 *   - points are sorted into a uniform cell grid; a cell is cut into chunks
 *     of at most 32 points;
 *   - a persistent warp takes the next chunk from a global counter, holds one
 *     chunk point per lane (lanes are replicated over the neighbour's points
 *     when the chunk is short) and walks the cell-offset stencil, streaming
 *     the neighbour cell's points from L1/L2;
 *   - auto counts use half of the stencil and i<j inside a cell.
 *
 * Per pair (FP32 path): separations on coordinates relative to the cell
 * centres, bin lookup in shared-memory tables, and a rounding bound: a pair
 * whose s^2, mu, s_perp^2 or pi lies within the bound of a bin edge is queued
 * and re-binned by the FP64 formula of the reference (metric_common.c of
 * src/fcfc/2pt_box and src/fcfc/2pt), so integer counts equal the FP64 build.
 *
 * Histograms live in shared memory (u32 counts, or int64 fixed-point weight
 * products) and are merged into global 64/128-bit integer accumulators, so
 * the results do not depend on the order of the additions.
 */
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "fcfcg_internal.h"

#define CT_THREADS 256
#define FULLMASK 0xffffffffu

/* ------------------------------------------------------------------------ */
/* Accumulators.                                                            */

/* Add a signed 64-bit value to a 128-bit two's complement accumulator. */
__device__ __forceinline__ void add128(unsigned long long *lohi, long long v) {
  unsigned long long u = (unsigned long long) v;
  unsigned long long old = atomicAdd(lohi, u);
  unsigned long long hi = ((old + u) < old ? 1ull : 0ull) +
                          (v < 0 ? ~0ull : 0ull);
  if (hi) atomicAdd(lohi + 1, hi);
}

/* Fixed-point product of two scaled weights (|w| <= 1), each split into
 * float hi + lo parts: round(w_a w_b 2^F) up to the dropped lo*lo term.
 * Shared by every path so that a pair contributes the same integer. */
__device__ __forceinline__ long long fix_prod(float ah, float al, float bh,
    float bl, float twoF) {
  float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  float c = __fmaf_rn(ah, bl, __fmul_rn(al, bh));
  long long hi = __float2ll_rn(__fmul_rn(p, twoF));
  int lo = __float2int_rn(__fmul_rn(__fadd_rn(e, c), twoF));
  return hi + (long long) lo;
}

#define HALF_U32 0x80000000u
#define FIX_LIMIT (1ll << 61)

__device__ __forceinline__ void hist_add_count(uint32_t *h,
    unsigned long long *gcnt, int bin) {
  uint32_t old = atomicAdd(h + bin, 1u);
  if (old == HALF_U32 - 1u) {       /* move 2^31 to the global counter */
    atomicSub(h + bin, HALF_U32);
    atomicAdd(gcnt + bin, (unsigned long long) HALF_U32);
  }
}

__device__ __forceinline__ void hist_add_fix(long long *h,
    unsigned long long *gwt, int bin, long long v) {
  long long old = (long long) atomicAdd((unsigned long long *) (h + bin),
                                        (unsigned long long) v);
  long long nv = old + v;
  if (nv >= FIX_LIMIT && old < FIX_LIMIT) {
    atomicAdd((unsigned long long *) (h + bin),
              (unsigned long long) (-FIX_LIMIT));
    add128(gwt + 2 * bin, FIX_LIMIT);
  } else if (nv <= -FIX_LIMIT && old > -FIX_LIMIT) {
    atomicAdd((unsigned long long *) (h + bin), (unsigned long long) FIX_LIMIT);
    add128(gwt + 2 * bin, -FIX_LIMIT);
  }
}

/* ------------------------------------------------------------------------ */
/* FP64 binning of one pair, exactly as the reference's scalar FP64 code.   */

__device__ __forceinline__ int ref_lookup(const uint16_t *__restrict__ tab,
    long off, long ntab, int num, const double *__restrict__ edge, double v) {
  long t = (long) __double2int_rz(v) - off;
  if (!(v == v) || t < 0 || t >= ntab) return -1;   /* never indexes outside */
  int idx = __ldg(tab + t);
  if (idx >= num) {                 /* hybrid entry: walk down */
    idx -= num;
    while (idx != 0 && v < __ldg(edge + idx)) idx--;
  }
  return idx;
}

/* Periodic box, src/fcfc/2pt_box/metric_common.c:140-235.
 * (dx, dy, dz) = (x1 + shift) - x2 already formed. */
__device__ int ref_bin_box(const fcfcg_launch &L, double dx, double dy,
    double dz) {
  if (L.bintype == FCFCG_BIN_SPI) {
    double pi = fabs(dz);
    if (pi >= L.pmax) return -1;
    if (!L.pmin0 && pi < L.pmin) return -1;
    double d = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (d >= L.s2max) return -1;
    if (!L.smin0 && d < L.s2min) return -1;
    int si = ref_lookup(L.rs, L.rsoff, L.nrs, L.ns, L.s2edge, d);
    int pi_ = ref_lookup(L.rp, L.rpoff, L.nrp, L.np, L.pedge, pi);
    if (si < 0 || pi_ < 0) return -1;
    return si + pi_ * L.ns;
  }
  double dz2 = __dmul_rn(dz, dz);
  double d = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), dz2);
  if (d >= L.s2max) return -1;
  if (!L.smin0 && d < L.s2min) return -1;
  int mi = 0;
  if (L.bintype == FCFCG_BIN_SMU) {
    const int nmu2 = L.nmu * L.nmu;
    int p = (d < DBL_EPSILON) ? 0
            : __double2int_rz(__dmul_rn(__ddiv_rn(dz2, d), (double) nmu2));
    if (p >= nmu2 || p < 0) return -1;
    /* mutab[p] = floor(sqrt(p)) (setup_cf.c:513-531) */
    int k = (int) sqrt((double) p);
    while (k * k > p) k--;
    while ((k + 1) * (k + 1) <= p) k++;
    mi = k;
  }
  int si = ref_lookup(L.rs, L.rsoff, L.nrs, L.ns, L.s2edge, d);
  if (si < 0) return -1;
  return si + mi * L.ns;
}

/* Survey, src/fcfc/2pt/metric_common.c:142-260. */
__device__ int ref_bin_survey(const fcfcg_launch &L, double x1, double y1,
    double z1, double s1, double x2, double y2, double z2, double s2) {
  if (L.bintype == FCFCG_BIN_ISO) {
    double dx = __dsub_rn(x1, x2), dy = __dsub_rn(y1, y2),
           dz = __dsub_rn(z1, z2);
    double d = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                         __dmul_rn(dz, dz));
    if (d >= L.s2max) return -1;
    if (!L.smin0 && d < L.s2min) return -1;
    return ref_lookup(L.rs, L.rsoff, L.nrs, L.ns, L.s2edge, d);
  }
  double t = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(x1, x2),
                                           __dmul_rn(y1, y2)),
                                 __dmul_rn(z1, z2)), 2.0);
  double s = __dadd_rn(s1, s2);
  if (L.bintype == FCFCG_BIN_SMU) {
    double d = __dsub_rn(s, t);
    if (d >= L.s2max) return -1;
    if (!L.smin0 && d < L.s2min) return -1;
    double dd = __dsub_rn(s1, s2);
    double pi2 = __ddiv_rn(__dmul_rn(dd, dd), __dadd_rn(s, t));
    const int nmu2 = L.nmu * L.nmu;
    int p = (d < DBL_EPSILON) ? 0
            : __double2int_rz(__dmul_rn(__ddiv_rn(pi2, d), (double) nmu2));
    if (p >= nmu2 || p < 0) return -1;
    int k = (int) sqrt((double) p);
    while (k * k > p) k--;
    while ((k + 1) * (k + 1) <= p) k++;
    int si = ref_lookup(L.rs, L.rsoff, L.nrs, L.ns, L.s2edge, d);
    if (si < 0) return -1;
    return si + k * L.ns;
  }
  double dd = __dsub_rn(s1, s2);
  double pi2 = __ddiv_rn(__dmul_rn(dd, dd), __dadd_rn(s, t));
  if (pi2 >= L.pmax) return -1;
  if (!L.pmin0 && pi2 < L.pmin) return -1;
  double d = __dsub_rn(__dsub_rn(s, t), pi2);
  if (d >= L.s2max) return -1;
  if (!L.smin0 && d < L.s2min) return -1;
  if (d < 0) d = 0;      /* (int) of a value in (-1, 0) is 0 */
  int si = ref_lookup(L.rs, L.rsoff, L.nrs, L.ns, L.s2edge, d);
  int pi_ = ref_lookup(L.rp, L.rpoff, L.nrp, L.np, L.pedge, pi2);
  if (si < 0 || pi_ < 0) return -1;
  return si + pi_ * L.ns;
}

/* Exact bin of sorted point a (catalogue A) and b (catalogue B) with the
 * image code of the cell pair (box).  The image shift goes to the A point,
 * or for auto counts to the point with the smaller input index. */
__device__ int ref_bin_pair(const fcfcg_launch &L, uint32_t a, uint32_t b,
    uint32_t code) {
  if (L.geometry == FCFCG_GEOM_SURVEY)
    return ref_bin_survey(L, L.A.x[a], L.A.y[a], L.A.z[a], L.A.s[a],
                          L.B.x[b], L.B.y[b], L.B.z[b], L.B.s[b]);
  const int wx = (int) (code & 3u) - 1, wy = (int) ((code >> 2) & 3u) - 1,
            wz = (int) ((code >> 4) & 3u) - 1;
  const double shx = -wx * L.box[0], shy = -wy * L.box[1],
               shz = -wz * L.box[2];
  const double xa = L.A.x[a], ya = L.A.y[a], za = L.A.z[a];
  const double xb = L.B.x[b], yb = L.B.y[b], zb = L.B.z[b];
  double dx, dy, dz;
  if (!L.isauto || L.A.id[a] < L.B.id[b]) {
    dx = __dsub_rn(__dadd_rn(xa, shx), xb);
    dy = __dsub_rn(__dadd_rn(ya, shy), yb);
    dz = __dsub_rn(__dadd_rn(za, shz), zb);
  } else {
    dx = __dsub_rn(__dsub_rn(xb, shx), xa);
    dy = __dsub_rn(__dsub_rn(yb, shy), ya);
    dz = __dsub_rn(__dsub_rn(zb, shz), za);
  }
  return ref_bin_box(L, dx, dy, dz);
}

/* ------------------------------------------------------------------------ */
/* FP32 edge-window lookup.                                                 */

/* Bin of an FP32 value v with error bound E (< 1/2) on an axis table,
 * or FCFCG_FTAB_BIN_MASK when out of range; *amb set when an edge lies
 * within E of v. */
__device__ __forceinline__ unsigned ftab_bin(const uint16_t *tab, int off,
    int ntab, float v, float E, bool &amb) {
  if (!(v == v)) {
    amb = true;
    return FCFCG_FTAB_BIN_MASK;
  }
  int i = __float2int_rz(v);
  int t = i - off;
  if (t < 0 || t >= ntab) return FCFCG_FTAB_BIN_MASK;
  unsigned e = tab[t];
  float fr = v - (float) i;
  amb |= ((e & FCFCG_FTAB_CX) != 0) | (((e & FCFCG_FTAB_LO) != 0) & (fr <= E)) |
         (((e & FCFCG_FTAB_HI) != 0) & (fr >= 1.f - E));
  return e & FCFCG_FTAB_BIN_MASK;
}

/* Integer bin of q = nmu * mu with error Eq; edges at every integer >= 1. */
__device__ __forceinline__ int mu_bin(float q, float Eq, bool &amb) {
  int qi = __float2int_rz(q);
  float fq = q - (float) qi;
  amb |= ((qi > 0) & (fq <= Eq)) | (fq >= 1.f - Eq) | !(fq == fq);
  return qi;
}

/* ------------------------------------------------------------------------ */

struct WarpChunk {
  uint32_t cell, first, m;
  int g, G, ia, grp;
  bool active;
  uint32_t ai;
  int cx, cy, cz;
};

__device__ __forceinline__ bool next_chunk(const fcfcg_launch &L,
    WarpChunk &w) {
  const int lane = threadIdx.x & 31;
  uint32_t c = 0;
  if (lane == 0) c = atomicAdd(L.chunk_head, 1u);
  c = __shfl_sync(FULLMASK, c, 0);
  if (c >= L.nchunk) return false;
  const uint4 ch = __ldg(((const uint4 *) L.chunks) + c);
  w.cell = ch.x;
  w.first = ch.y;
  w.m = ch.z;
  int g = 1;
  while (g < (int) w.m) g <<= 1;
  w.g = g;
  w.G = 32 / g;
  w.ia = lane & (g - 1);
  w.grp = lane / g;
  w.active = (uint32_t) w.ia < w.m;
  w.ai = w.first + (uint32_t) w.ia;
  w.cx = (int) (w.cell % (uint32_t) L.ncell[0]);
  w.cy = (int) ((w.cell / (uint32_t) L.ncell[0]) % (uint32_t) L.ncell[1]);
  w.cz = (int) (w.cell / ((uint32_t) L.ncell[0] * (uint32_t) L.ncell[1]));
  return true;
}

/* Neighbour cell of the chunk's cell for stencil entry o; false if it lies
 * outside a survey grid.  code: image of the cell pair (box). */
__device__ __forceinline__ bool neighbour(const fcfcg_launch &L,
    const WarpChunk &w, int4 o, uint32_t &cb, uint32_t &code) {
  int q[3] = {w.cx + o.x, w.cy + o.y, w.cz + o.z};
  int wr[3] = {0, 0, 0};
  for (int k = 0; k < 3; k++) {
    const int n = L.ncell[k];
    if (L.geometry == FCFCG_GEOM_SURVEY) {
      if (q[k] < 0 || q[k] >= n) return false;
    } else {
      while (q[k] < 0) {
        q[k] += n;
        wr[k]--;
      }
      while (q[k] >= n) {
        q[k] -= n;
        wr[k]++;
      }
    }
  }
  cb = ((uint32_t) q[2] * L.ncell[1] + q[1]) * L.ncell[0] + q[0];
  code = (uint32_t) (wr[0] + 1) | ((uint32_t) (wr[1] + 1) << 2) |
         ((uint32_t) (wr[2] + 1) << 4);
  return true;
}

/* First neighbour index of this lane: its group for ordinary offsets, the
 * first j > i (same residue) for the self offset of an auto count. */
__device__ __forceinline__ int first_j(const WarpChunk &w, bool self,
    uint32_t bstart) {
  if (!self) return w.grp;
  int t = (int) (w.ai - bstart) + 1;
  int r = (w.grp - t) % w.G;
  if (r < 0) r += w.G;
  return t + r;
}

/* Queue a pair for the FP64 recheck; when the queue is full, bin it here. */
template <int WT>
__device__ __forceinline__ void enqueue(const fcfcg_launch &L, uint32_t a,
    uint32_t b, uint32_t code, uint32_t *h32, long long *h64,
    unsigned long long &n_inline) {
  uint32_t slot = atomicAdd(L.qcount, 1u);
  if (slot < L.qcap) {
    *((uint4 *) L.queue + slot) = make_uint4(a, b, code, 0u);
    return;
  }
  n_inline++;
  int bin = ref_bin_pair(L, a, b, code);
  if (bin < 0) return;
  if (WT) {
    const float2 wa = make_float2(((const float4 *) L.A.l4)[a].w, L.A.wlo[a]);
    const float2 wb = make_float2(((const float4 *) L.B.l4)[b].w, L.B.wlo[b]);
    long long v = fix_prod(wa.x, wa.y, wb.x, wb.y, ldexpf(1.f, L.fixF));
    if (L.hist_smem) hist_add_fix(h64, L.gwt, bin, v);
    else add128(L.gwt + 2 * bin, v);
  } else {
    if (L.hist_smem) hist_add_count(h32, L.gcnt, bin);
    else atomicAdd(L.gcnt + bin, 1ull);
  }
}

/*
 * FP32 counting kernel.  GEOM: box / survey; BIN: iso / smu / spi;
 * WT: weighted.  Shared memory: FP32 tables then the histogram.
 */
template <int GEOM, int BIN, int WT>
__global__ void __launch_bounds__(CT_THREADS)
k_count32(const fcfcg_launch L) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint16_t *fs = (uint16_t *) smem;
  uint16_t *fp = fs + L.nfs;
  size_t hoff = ((size_t) (L.nfs + L.nfp) * sizeof(uint16_t) + 15) & ~(size_t) 15;
  uint32_t *h32 = (uint32_t *) (smem + hoff);
  long long *h64 = (long long *) (smem + hoff);
  for (int i = threadIdx.x; i < L.nfs; i += blockDim.x) fs[i] = L.fs[i];
  for (int i = threadIdx.x; i < L.nfp; i += blockDim.x) fp[i] = L.fp[i];
  if (L.hist_smem) {
    if (WT)
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) h64[i] = 0;
    else
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) h32[i] = 0;
  }
  __syncthreads();

  const float4 *__restrict__ Al4 = (const float4 *) L.A.l4;
  const float4 *__restrict__ Bl4 = (const float4 *) L.B.l4;
  const int4 *__restrict__ sten = (const int4 *) L.sten;
  const float4 *__restrict__ stD = (const float4 *) L.stenD;
  const float twoF = ldexpf(1.f, L.fixF);
  unsigned long long n_cand = 0, n_in = 0, n_q = 0, n_inline = 0;

  WarpChunk w;
  while (next_chunk(L, w)) {
    float4 pa = make_float4(0.f, 0.f, 0.f, 0.f);
    float walo = 0.f;
    if (w.active) {
      pa = Al4[w.ai];
      if (WT) walo = L.A.wlo[w.ai];
    }
    for (int t = 0; t < L.nsten; t++) {
      const int4 o = __ldg(sten + t);
      uint32_t cb, code;
      if (!neighbour(L, w, o, cb, code)) continue;
      const uint32_t bstart = __ldg(L.B.cstart + cb);
      const uint32_t bend = __ldg(L.B.cstart + cb + 1);
      if (bstart == bend || !w.active) continue;
      const bool self = L.isauto && o.x == 0 && o.y == 0 && o.z == 0;
      const float4 D = __ldg(stD + t);
      const float xi = pa.x + D.x, yi = pa.y + D.y, zi = pa.z + D.z;
      float cbx = 0.f, cby = 0.f, cbz = 0.f;
      if (GEOM == FCFCG_GEOM_SURVEY) {
        /* twice the centre of cell B: m = x_a + x_b = 2 c_B + 2 l_b + d */
        const int qx = w.cx + o.x, qy = w.cy + o.y, qz = w.cz + o.z;
        cbx = 2.f * fmaf((float) qx + 0.5f, L.cwf[0], L.lof[0]);
        cby = 2.f * fmaf((float) qy + 0.5f, L.cwf[1], L.lof[1]);
        cbz = 2.f * fmaf((float) qz + 0.5f, L.cwf[2], L.lof[2]);
      }
      const int nb = (int) (bend - bstart);
      for (int j = first_j(w, self, bstart); j < nb; j += w.G) {
        const uint32_t bj = bstart + (uint32_t) j;
        const float4 pb = Bl4[bj];
        const float dx = xi - pb.x, dy = yi - pb.y, dz = zi - pb.z;
        n_cand++;
        bool amb = false;
        int bin = -1;
        if (BIN == FCFCG_BIN_SPI && GEOM == FCFCG_GEOM_BOX) {
          const float pi = fabsf(dz);
          if (!(pi < L.p_lim)) continue;
          const float sp2 = fmaf(dy, dy, dx * dx);
          if (!(sp2 < L.s_lim)) continue;
          const float rs = rsqrtf(sp2);
          const float s = sp2 * rs;
          const float E = fmaf(L.K2, sp2, fmaf(L.K1, s, L.K0));
          amb = !(sp2 >= L.tiny);
          unsigned sb = ftab_bin(fs, L.fsoff, L.nfs, sp2, E, amb);
          unsigned pbn = ftab_bin(fp, L.fpoff, L.nfp, pi, L.P0, amb);
          if (!amb) {
            if (sb == FCFCG_FTAB_BIN_MASK || pbn == FCFCG_FTAB_BIN_MASK) continue;
            bin = (int) sb + (int) pbn * L.ns;
          }
        } else {
          const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          if (!(s2 < L.s_lim)) continue;
          const float rs = rsqrtf(s2);
          const float s = s2 * rs;
          const float E = fmaf(L.K2, s2, fmaf(L.K1, s, L.K0));
          amb = !(s2 >= L.tiny);
          if (BIN == FCFCG_BIN_ISO) {
            unsigned sb = ftab_bin(fs, L.fsoff, L.nfs, s2, E, amb);
            if (!amb) {
              if (sb == FCFCG_FTAB_BIN_MASK) continue;
              bin = (int) sb;
            }
          } else if (BIN == FCFCG_BIN_SMU) {
            float q;
            if (GEOM == FCFCG_GEOM_BOX) {
              q = L.fnmu * fabsf(dz) * rs;
            } else {
              const float mx = fmaf(2.f, pb.x, cbx) + dx;
              const float my = fmaf(2.f, pb.y, cby) + dy;
              const float mz = fmaf(2.f, pb.z, cbz) + dz;
              const float dm = fmaf(dz, mz, fmaf(dy, my, dx * mx));
              const float mm = fmaf(mz, mz, fmaf(my, my, mx * mx));
              q = L.fnmu * fabsf(dm) * rsqrtf(mm * s2);
            }
            const float Eq = fmaf(L.Q1, rs, fmaf(L.Q2, q, L.Q0));
            int qi = mu_bin(q, Eq, amb);
            unsigned sb = ftab_bin(fs, L.fsoff, L.nfs, s2, E, amb);
            if (!amb) {
              if (sb == FCFCG_FTAB_BIN_MASK || qi >= L.nmu) continue;
              bin = (int) sb + qi * L.ns;
            }
          } else {
            /* survey (s_perp, pi): pi^2 = (d.m)^2 / |m|^2 */
            const float mx = fmaf(2.f, pb.x, cbx) + dx;
            const float my = fmaf(2.f, pb.y, cby) + dy;
            const float mz = fmaf(2.f, pb.z, cbz) + dz;
            const float dm = fmaf(dz, mz, fmaf(dy, my, dx * mx));
            const float mm = fmaf(mz, mz, fmaf(my, my, mx * mx));
            const float pi2 = __fdividef(dm * dm, mm);
            const float sp2 = s2 - pi2;
            const float Ep = fmaf(L.P2, s2, fmaf(L.P1, s, L.P0));
            unsigned pbn = ftab_bin(fp, L.fpoff, L.nfp, pi2, Ep, amb);
            unsigned sb = ftab_bin(fs, L.fsoff, L.nfs, sp2 < 0.f ? 0.f : sp2,
                                   E + Ep, amb);
            if (!amb) {
              if (sb == FCFCG_FTAB_BIN_MASK || pbn == FCFCG_FTAB_BIN_MASK) continue;
              bin = (int) sb + (int) pbn * L.ns;
            }
          }
        }
        if (amb) {
          n_q++;
          enqueue<WT>(L, w.ai, bj, code, h32, h64, n_inline);
          continue;
        }
        n_in++;
        if (WT) {
          const float wblo = L.B.wlo[bj];
          const long long v = fix_prod(pa.w, walo, pb.w, wblo, twoF);
          if (L.hist_smem) hist_add_fix(h64, L.gwt, bin, v);
          else add128(L.gwt + 2 * bin, v);
        } else {
          if (L.hist_smem) hist_add_count(h32, L.gcnt, bin);
          else atomicAdd(L.gcnt + bin, 1ull);
        }
      }
    }
  }

  /* statistics */
  for (int o = 16; o > 0; o >>= 1) {
    n_cand += __shfl_xor_sync(FULLMASK, n_cand, o);
    n_in += __shfl_xor_sync(FULLMASK, n_in, o);
    n_q += __shfl_xor_sync(FULLMASK, n_q, o);
    n_inline += __shfl_xor_sync(FULLMASK, n_inline, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(L.stats + 0, n_cand);
    atomicAdd(L.stats + 1, n_in);
    atomicAdd(L.stats + 2, n_q);
    atomicAdd(L.stats + 3, n_inline);
  }
  __syncthreads();
  if (L.hist_smem) {
    for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) {
      if (WT) {
        long long v = h64[i];
        if (v) add128(L.gwt + 2 * i, v);
      } else {
        uint32_t v = h32[i];
        if (v) atomicAdd(L.gcnt + i, (unsigned long long) v);
      }
    }
  }
}

/*
 * FP64 counting kernel: the same traversal, every pair binned by the
 * reference's FP64 formula.  Weighted sums are FP64 products accumulated
 * in FP64.
 */
template <int GEOM, int WT>
__global__ void __launch_bounds__(CT_THREADS)
k_count64(const fcfcg_launch L) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t *h32 = (uint32_t *) smem;
  double *hd = (double *) smem;
  if (L.hist_smem) {
    if (WT)
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) hd[i] = 0;
    else
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) h32[i] = 0;
  }
  __syncthreads();
  unsigned long long n_cand = 0, n_in = 0;
  WarpChunk w;
  while (next_chunk(L, w)) {
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
        int bin = ref_bin_pair(L, w.ai, bj, code);
        if (bin < 0) continue;
        n_in++;
        if (WT) {
          double v = __dmul_rn(L.A.w[w.ai], L.B.w[bj]);
          if (L.hist_smem) atomicAdd(hd + bin, v);
          else atomicAdd(L.gwd + bin, v);
        } else {
          if (L.hist_smem) hist_add_count(h32, L.gcnt, bin);
          else atomicAdd(L.gcnt + bin, 1ull);
        }
      }
    }
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
  if (L.hist_smem) {
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

/* FP64 recheck of queued pairs. */
template <int WT>
__global__ void k_recheck(const fcfcg_launch L, uint32_t nq) {
  const float twoF = ldexpf(1.f, L.fixF);
  unsigned long long n_in = 0;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq;
       q += gridDim.x * blockDim.x) {
    const uint4 e = ((const uint4 *) L.queue)[q];
    int bin = ref_bin_pair(L, e.x, e.y, e.z);
    if (bin < 0) continue;
    n_in++;
    if (WT) {
      const float ah = ((const float4 *) L.A.l4)[e.x].w, al = L.A.wlo[e.x];
      const float bh = ((const float4 *) L.B.l4)[e.y].w, bl = L.B.wlo[e.y];
      add128(L.gwt + 2 * bin, fix_prod(ah, al, bh, bl, twoF));
    } else {
      atomicAdd(L.gcnt + bin, 1ull);
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    n_in += __shfl_xor_sync(FULLMASK, n_in, o);
  if ((threadIdx.x & 31) == 0 && n_in) atomicAdd(L.stats + 1, n_in);
}

/* ------------------------------------------------------------------------ */

typedef void (*kfun_t)(const fcfcg_launch);

static kfun_t pick32(int geom, int bin, int wt) {
#define K32(G, B)                                                          \
  if (geom == G && bin == B)                                               \
    return wt ? (kfun_t) k_count32<G, B, 1> : (kfun_t) k_count32<G, B, 0>;
  K32(FCFCG_GEOM_BOX, FCFCG_BIN_ISO)
  K32(FCFCG_GEOM_BOX, FCFCG_BIN_SMU)
  K32(FCFCG_GEOM_BOX, FCFCG_BIN_SPI)
  K32(FCFCG_GEOM_SURVEY, FCFCG_BIN_ISO)
  K32(FCFCG_GEOM_SURVEY, FCFCG_BIN_SMU)
  K32(FCFCG_GEOM_SURVEY, FCFCG_BIN_SPI)
#undef K32
  return 0;
}

static kfun_t pick64(int geom, int wt) {
  if (geom == FCFCG_GEOM_BOX)
    return wt ? (kfun_t) k_count64<FCFCG_GEOM_BOX, 1>
              : (kfun_t) k_count64<FCFCG_GEOM_BOX, 0>;
  return wt ? (kfun_t) k_count64<FCFCG_GEOM_SURVEY, 1>
            : (kfun_t) k_count64<FCFCG_GEOM_SURVEY, 0>;
}

extern "C" int fcfcg_k_count(void *stream, const fcfcg_launch *L,
    int precision, int nsm, size_t *smem_used) {
  kfun_t f;
  size_t smem;
  if (precision == FCFCG_PREC_FP64) {
    f = pick64(L->geometry, L->withwt);
    smem = L->hist_smem ? (size_t) L->ntot * (L->withwt ? 8 : 4) : 0;
  } else {
    f = pick32(L->geometry, L->bintype, L->withwt);
    size_t tab = (((size_t) (L->nfs + L->nfp) * 2) + 15) & ~(size_t) 15;
    smem = tab + (L->hist_smem ? (size_t) L->ntot * (L->withwt ? 8 : 4) : 0);
  }
  if (!f) return (int) cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute((const void *) f,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (e) return (int) e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *) f,
                                                    CT_THREADS, smem);
  if (e) return (int) e;
  if (per_sm < 1) return (int) cudaErrorInvalidConfiguration;
  if (smem_used) *smem_used = smem;
  f<<<nsm * per_sm, CT_THREADS, smem, (cudaStream_t) stream>>>(*L);
  return (int) cudaGetLastError();
}

extern "C" int fcfcg_k_recheck(void *stream, const fcfcg_launch *L,
    uint32_t nq) {
  if (!nq) return 0;
  unsigned blocks = (nq + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (L->withwt)
    k_recheck<1><<<blocks, 256, 0, (cudaStream_t) stream>>>(*L, nq);
  else
    k_recheck<0><<<blocks, 256, 0, (cudaStream_t) stream>>>(*L, nq);
  return (int) cudaGetLastError();
}
