/*
 * count_common.cuh -- device code shared by the counting kernels: the
 * integer accumulators, the reference's FP64 binning of one pair, the FP32
 * edge-window lookups, and the shared-memory layout of the FP32 kernel.
 * Included by count.cu and by the count32_*.cu translation units.
 */
#ifndef FCFCG_COUNT_COMMON_CUH
#define FCFCG_COUNT_COMMON_CUH
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <string.h>

#include "fcfcg_internal.h"

/* Kernel binning codes: the public FCFCG_BIN_* (0 iso, 1 (s,mu), 2
 * (s_perp,pi)), and the same binnings with an FP32 table of s^2 or s_perp^2
 * indexed by bit pattern (bins spaced in ratio, boxes only): 3 (s_perp,pi),
 * 4 iso, 5 (s,mu); and iso (6) and (s,mu) (7) with linear s bins, whose s
 * bin comes from s itself with no table. */
#define BIN_SPIL 3
#define BIN_ISOL 4
#define BIN_SMUL 5
#define BIN_ISOLIN 6
#define BIN_SMULIN 7
#define IS_SPI(B) ((B) == FCFCG_BIN_SPI || (B) == BIN_SPIL)
#define IS_ISO(B) ((B) == FCFCG_BIN_ISO || (B) == BIN_ISOL || (B) == BIN_ISOLIN)
#define IS_SMU(B) ((B) == FCFCG_BIN_SMU || (B) == BIN_SMUL || (B) == BIN_SMULIN)
#define LOGTAB(B) ((B) >= BIN_SPIL && (B) <= BIN_SMUL)
/* linear s bins: the s bin is floor((s - a) / d), no table */
#define LINS(B) ((B) == BIN_ISOLIN || (B) == BIN_SMULIN)
/* survey (s_perp, pi): the scan applies the line-of-sight prefilter */
#define LOSCUT(G, B) ((G) == FCFCG_GEOM_SURVEY && (B) == FCFCG_BIN_SPI)

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

/*
 * Fixed-point product of two weights scaled to |w| <= 1, with F = 51
 * fractional bits (FCFCG_FIX_F).  A weight is held as an integer part
 * wi = round(w 2^30) and a float remainder wr = w - wi 2^-30 (|wr| <= 2^-31):
 *   w_a w_b 2^51 = wi_a wi_b 2^-9 + (w_a wr_b + wr_a w_b) 2^51 (+ wr wr).
 * The first term is an exact 64-bit product rounded by a shift; the cross
 * term (|.| <= 2^21) is rounded with the 1.5 * 2^23 float trick; wr wr
 * (<= 2^-11 of a unit) is dropped.  No 64-bit float conversions.  The
 * function is symmetric in a and b (two rounded products and a commutative
 * sum, no fused multiply-add), and every path uses it, so a pair adds the
 * same integer whichever point is the chunk's: weighted sums do not depend
 * on the order of the points within a cell.
 */
__device__ __forceinline__ long long fix_prod(int ia, float ra, float fa,
    int ib, float rb, float fb) {
  const long long p = (long long) ia * (long long) ib;
  const long long main = (p + (1ll << 8)) >> 9;
  const float c = __fadd_rn(__fmul_rn(fa, rb), __fmul_rn(ra, fb));
  const float t = __fmaf_rn(c, 2251799813685248.0f /* 2^51 */, 12582912.0f);
  return main + (long long) (__float_as_int(t) - 0x4B400000);
}

__device__ __forceinline__ long long fix_prod_pair(const fcfcg_launch &L,
    uint32_t a, uint32_t b) {
  const int2 wa = ((const int2 *) L.A.wq)[a];
  const int2 wb = ((const int2 *) L.B.wq)[b];
  const float fa = ((const float4 *) L.A.l4)[a].w;
  const float fb = ((const float4 *) L.B.l4)[b].w;
  return fix_prod(wa.x, __int_as_float(wa.y), fa, wb.x, __int_as_float(wb.y),
                  fb);
}

#define HALF_U32 0x80000000u
#define FIX_LIMIT (1ll << 61)
#define HI_LIMIT (1 << 30)

/* Weighted bin in shared memory as two 32-bit words, value = hi 2^32 + lo
 * (lo unsigned, hi signed): native 32-bit atomics, the carry out of lo is
 * read from the returned value, and 2^30 of hi (2^62) moves to the global
 * 128-bit accumulator whenever hi crosses +-2^30. */
__device__ __forceinline__ void hist_add_fix32(uint32_t *lo, int *hi,
    unsigned long long *gwt, int bin, long long v) {
  const uint32_t vl = (uint32_t) v;
  const uint32_t old = atomicAdd(lo + bin, vl);
  const int h = (int) (v >> 32) + (((old + vl) < old) ? 1 : 0);
  if (h) {
    const int oh = atomicAdd(hi + bin, h);
    const int nh = oh + h;
    if (nh >= HI_LIMIT && oh < HI_LIMIT) {
      atomicSub(hi + bin, HI_LIMIT);
      add128(gwt + 2 * bin, 1ll << 62);
    } else if (nh <= -HI_LIMIT && oh > -HI_LIMIT) {
      atomicAdd(hi + bin, HI_LIMIT);
      add128(gwt + 2 * bin, -(1ll << 62));
    }
  }
}

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
static __device__ int ref_bin_box(const fcfcg_launch &L, double dx, double dy,
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
    if (p < 0) return -1;
    if (p >= nmu2) {
      if (!L.mu_one) return -1;
      p = nmu2 - 1;
    }
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
static __device__ int ref_bin_survey(const fcfcg_launch &L, double x1, double y1,
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
    if (p < 0) return -1;
    if (p >= nmu2) {
      if (!L.mu_one) return -1;
      p = nmu2 - 1;
    }
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
static __device__ int ref_bin_pair(const fcfcg_launch &L, uint32_t a, uint32_t b,
    uint32_t code, const double *box) {
  if (L.geometry == FCFCG_GEOM_SURVEY)
    return ref_bin_survey(L, L.A.x[a], L.A.y[a], L.A.z[a], L.A.s[a],
                          L.B.x[b], L.B.y[b], L.B.z[b], L.B.s[b]);
  const int wx = (int) (code & 3u) - 1, wy = (int) ((code >> 2) & 3u) - 1,
            wz = (int) ((code >> 4) & 3u) - 1;
  const double shx = -wx * box[0], shy = -wy * box[1],
               shz = -wz * box[2];
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

/* Bin of an FP32 value v with error bound E on an axis table (cells of
 * width 1 / inv, E < half a cell), or FCFCG_FTAB_BIN_MASK when out of
 * range; *amb is set when an edge lies within E of v.  A cell with one edge
 * inside compares v with that edge (fe: the edges rounded to FP32).
 * CHECK_NAN: the value may be NaN (survey geometry). */
template <bool CHECK_NAN, bool LOG>
__device__ __forceinline__ unsigned ftab_bin(const uint16_t *tab, int off,
    int ntab, float inv, const float *fe, int nbin, float v, float E,
    bool &amb, int lg, float vamb) {
  if (CHECK_NAN && !(v == v)) {
    amb = true;
    return FCFCG_FTAB_BIN_MASK;
  }
  int i;
  float fr, Eu;
  if (LOG) {
    /* bit-pattern table: cell = FP32 bits >> lg, a fixed fraction of the
     * octave; below vamb the window is wider than half a cell */
    amb |= v < vamb;
    const uint32_t bits = __float_as_uint(v);
    i = (int) (bits >> lg);
    if ((unsigned) (i - off) >= (unsigned) ntab) return FCFCG_FTAB_BIN_MASK;
    fr = __uint2float_rz(bits & ((1u << lg) - 1u)) * inv;
    /* 1 / cell width: 2^(23 - lg) / 2^exponent(v) */
    Eu = E * __uint_as_float((277u - (uint32_t) lg - (bits >> 23)) << 23);
  } else {
    const float u = v * inv;
    i = __float2int_rz(u);
    if ((unsigned) (i - off) >= (unsigned) ntab) return FCFCG_FTAB_BIN_MASK;
    fr = u - (float) i;
    Eu = E * inv;
  }
  const unsigned e = tab[i - off];
  const unsigned m = FCFCG_FTAB_CXM | (fr <= Eu ? FCFCG_FTAB_LO : 0u) |
                     (fr >= 1.f - Eu ? FCFCG_FTAB_HI : 0u);
  amb |= (e & m) != 0u;
  unsigned b = e & FCFCG_FTAB_BIN_MASK;
  if (e & FCFCG_FTAB_CX1) {
    const int k = (b == FCFCG_FTAB_BIN_MASK) ? 0 : (int) b + 1;
    const float ef = fe[k];
    const float d = v - ef;
    amb |= fabsf(d) <= fmaf(fabsf(ef), 1.2e-7f, E);
    if (d >= 0.f) b = (k == nbin) ? FCFCG_FTAB_BIN_MASK : (unsigned) k;
  }
  return b;
}

/* Bin of s for linear bins (rescaled edges a + k d, integers, so FCFC's bin
 * k is the one with (a + k d)^2 <= s^2 < (a + (k + 1) d)^2): k = floor(t),
 * t = (s - a) / d, and the pair is ambiguous when t is within the window
 * W = lin_A s + lin_B of an integer that is a bin boundary (every integer
 * from the lowest bin's lower edge up -- its lower edge only when s_min > 0
 * -- lin_k0 = -1 then, 0 for s_min = 0).  W bounds |t - t_ref| against the
 * reference's sqrt(s^2) (the bound is derived where lin_A, lin_B are set).
 * Returns k; in range when 0 <= k < ns. */
__device__ __forceinline__ int lin_bin(const fcfcg_launch &L, float s,
    bool &amb) {
  const float t = fmaf(s, L.lin_inv, L.lin_off);
  const float W = fmaf(L.lin_A, s, L.lin_B);
  /* an edge k > lin_k0 in [t - W, t + W]: the two ends fall in different
   * bins (the window carries the rounding of t -+ W) */
  const int lo = max(__float2int_rd(t - W), L.lin_k0);
  const int k = __float2int_rd(t + W);
  amb |= (lo != k);
  return k;
}

/* Integer bin of q = nmu * mu >= 0 with error Eq < 1/2; edges at every
 * integer >= 1: one lies in [q - Eq, q + Eq] when the two ends truncate
 * differently (the window carries the rounding of q -+ Eq; q - Eq > -1
 * truncates to 0, so 0 is no edge).  q is finite: pairs with s^2 < tiny,
 * the only ones whose q could be NaN, are ambiguous already. */
__device__ __forceinline__ int mu_bin(float q, float Eq, bool &amb) {
  const int lo = __float2int_rz(q - Eq);
  const int qi = __float2int_rz(q + Eq);
  amb |= (lo != qi);
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
  if (c >= (L.nchunk_dev ? __ldg(L.nchunk_dev) : L.nchunk)) return false;
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

/* The catalogue a CTA of a batched launch is working on (shared memory):
 * its grid, box and global histogram. */
struct MockSh {
  int nc[3];
  uint32_t base;
  float cwf[3], cwl[3];  /* cell widths: float + float residual */
  double box[3];
  unsigned long long *g;     /* gcnt, or gwt when weighted */
  uint32_t id;
};

/* Histogram of the FP32 kernel in shared memory: ntot u32 counts, or
 * ntot u32 low words followed by ntot s32 high words for weighted sums
 * (their overflow goes to the global histogram of the current catalogue).
 * hs: the shared histogram takes the add.  Unweighted shared bins take it
 * unchecked: the kernel hands them to the global counters before the adds
 * since the last hand-over could pass 2^32 - 1, and a chunk that alone
 * could (m x total pairs) counts in global memory (hs false). */
template <int WT, int BATCH>
__device__ __forceinline__ void hist_add(const fcfcg_launch &L,
    const MockSh *ms, uint32_t *h, int bin, long long w, bool hs) {
  unsigned long long *g = BATCH ? ms->g : (WT ? L.gwt : L.gcnt);
  if (WT) {
    if (L.hist_smem) hist_add_fix32(h, (int *) (h + L.ntot), g, bin, w);
    else add128(g + 2 * bin, w);
  } else {
    if (hs) atomicAdd(h + bin, 1u);
    else atomicAdd(g + bin, 1ull);
  }
}

/* Queue a pair for the FP64 recheck; when the queue is full, bin it here.
 * Every ambiguous pair takes a ticket from the fill counter, queued or not,
 * so one launch can take more than 2^32 of them: the counter is 64-bit, or
 * it would wrap and hand out slots of pairs still waiting in the queue. */
template <int WT, int BATCH>
__device__ __forceinline__ void enqueue(const fcfcg_launch &L,
    const MockSh *ms, uint32_t a, uint32_t b, uint32_t code, uint32_t *h,
    unsigned long long &n_inline, uint32_t &n_in, bool hs) {
  const unsigned long long slot = atomicAdd(L.qcount, 1ull);
  if (slot < L.qcap) {
    *((uint4 *) L.queue + slot) = make_uint4(a, b, code, BATCH ? ms->id : 0u);
    return;
  }
  n_inline++;
  int bin = ref_bin_pair(L, a, b, code, BATCH ? ms->box : L.box);
  if (bin < 0) return;
  n_in++;
  hist_add<WT, BATCH>(L, ms, h, bin, WT ? fix_prod_pair(L, a, b) : 0, hs);
}

/*
 * Adjoint terms of the FP32 kernel as integers.  With g' = g 2^S the scaled
 * cotangent (|w g'| <= 2^50 for every weight), one fused multiply-add onto
 * 1.5 2^52 rounds the exact product w g' to the nearest integer, which is
 * then the low bits of the result (the classic magic-number conversion).
 * Sums of these integers are exact; they convert back with 2^-S.
 */
#define ADJ_MAGIC 6755399441055744.0         /* 1.5 * 2^52 */
#define ADJ_MAGIC_BITS 0x4338000000000000ll

__device__ __forceinline__ long long adj_term(double w, double g) {
  return __double_as_longlong(__fma_rn(w, g, ADJ_MAGIC)) - ADJ_MAGIC_BITS;
}

/* Add a term to a chunk point's accumulator: two 32-bit words, value
 * hi 2^32 + lo (lo unsigned, hi signed), as the weighted histograms keep
 * theirs -- native 32-bit shared atomics, the carry out of lo read from the
 * returned value.  The thread whose add carries hi across +-2^30 moves 2^62
 * to the point's FP64 gradient (an exact transfer), so with terms below
 * 2^51 the words cannot wrap. */
__device__ __forceinline__ void adj_acc(uint32_t *lo, int *hi, long long v,
    double *dst, double unit) {
  const uint32_t vl = (uint32_t) v;
  const uint32_t old = atomicAdd(lo, vl);
  const int h = (int) (v >> 32) + (((old + vl) < old) ? 1 : 0);
  if (h) {
    const int oh = atomicAdd(hi, h);
    const int nh = oh + h;
    if (nh >= HI_LIMIT && oh < HI_LIMIT) {
      atomicSub(hi, HI_LIMIT);
      atomicAdd(dst, ldexp(unit, 62));
    } else if (nh <= -HI_LIMIT && oh > -HI_LIMIT) {
      atomicAdd(hi, HI_LIMIT);
      atomicAdd(dst, -ldexp(unit, 62));
    }
  }
}

/* Adjoint: FP64 gradient contributions of one pair with a known bin. */
__device__ __forceinline__ void adj_pair(const fcfcg_launch &L, uint32_t a,
    uint32_t b, int bin) {
  const double g = __ldg(L.gadj + bin);
  atomicAdd(L.dA + a, __dmul_rn(L.B.w[b], g));
  atomicAdd(L.dB + b, __dmul_rn(L.A.w[a], g));
}

/* Adjoint: queue an ambiguous pair for the FP64 recheck, or bin it here
 * when the queue is full. */
__device__ __forceinline__ void enqueue_adj(const fcfcg_launch &L,
    uint32_t a, uint32_t b, uint32_t code, unsigned long long &n_inline,
    uint32_t &n_in) {
  const unsigned long long slot = atomicAdd(L.qcount, 1ull);
  if (slot < L.qcap) {
    *((uint4 *) L.queue + slot) = make_uint4(a, b, code, 0u);
    return;
  }
  n_inline++;
  int bin = ref_bin_pair(L, a, b, code, L.box);
  if (bin < 0) return;
  n_in++;
  adj_pair(L, a, b, bin);
}

/* Add a CTA's shared histogram to a global one and clear it. */
template <int WT>
__device__ __forceinline__ void hist_flush(const fcfcg_launch &L,
    uint32_t *h, unsigned long long *g) {
  for (long i = threadIdx.x; i < L.ntot; i += blockDim.x) {
    if (WT) {
      const long long v = ((long long) ((int *) h)[L.ntot + i] << 32) +
                          (long long) h[i];
      if (v) add128(g + 2 * i, v);
      h[i] = 0;
      h[L.ntot + i] = 0;
    } else {
      const uint32_t v = h[i];
      if (v) atomicAdd(g + i, (unsigned long long) v);
      h[i] = 0;
    }
  }
}

#define CT32_THREADS 256
#define FCHUNK 64                 /* chunk points a CTA holds (FP32 path) */
/* A warp's queue of candidates holds qwarp entries (a launch parameter:
 * 256, 512 or 1024); a smaller queue frees shared memory for another CTA
 * per SM or for L1. */
#define QWARP_MAX 1024
#define QWARP_MIN 256

/* Shared memory of the FP32 kernel after the tables and the histogram.
 * Per CTA: the chunk points (and weights) and the neighbour list of the
 * chunk; per warp: the 32 neighbour points of its current block and the
 * block's in-range pairs (chunk point | lane << 6). */
struct Stage {
  float4 *a;        /* FCHUNK: chunk point local x y z, scaled weight */
  /* FCHUNK / 2: chunk points 2k and 2k + 1 side by side, for the packed
   * FP32 candidate test: (x, x', y, y') and (z, z') */
  float4 *pxy;
  float2 *pz;
  int2 *aw;         /* FCHUNK: chunk point integer weight, remainder bits */
  uint32_t *pre;    /* nsten + 1: prefix of neighbour sizes */
  uint32_t *bst;    /* nsten: first sorted index of each neighbour */
  float4 *b;        /* per warp, 32: neighbour (l_b - D) x y z, index */
  float4 *bw;       /* per warp, 32: weight, integer weight, remainder */
  uint16_t *bt;     /* per warp, 32: stencil entry */
  uint16_t *q;      /* per warp, qwarp: queued pairs */
  /* adjoint only: gradient sums in units of 2^-S, FP64 weights */
  unsigned long long *ga;   /* FCHUNK x 8 bytes: the 32-bit lo words of
                               the chunk points, then their hi words */
  double *wa;               /* FCHUNK */
  long long *gb;            /* per warp, 32: the neighbour points */
  double *wb;               /* per warp, 32 */
};

/* wt: 0 unweighted, 1 weighted, 2 adjoint (weighted + FP64 gradients) */
__host__ __device__ __forceinline__ size_t stage_cta_bytes(int nsten, int wt) {
  size_t n = (size_t) FCHUNK * 16 + (size_t) FCHUNK * 12 +
             (wt ? (size_t) FCHUNK * 8 : 0);
  n += (((size_t) nsten + 1) * 4 + 15) & ~(size_t) 15;
  n += (((size_t) nsten) * 4 + 15) & ~(size_t) 15;
  if (wt == 2) n += (size_t) FCHUNK * 16;
  return n;
}

__host__ __device__ __forceinline__ size_t stage_warp_bytes(int wt,
    uint32_t qwarp) {
  return 32 * 16 + (wt ? 32 * 16 : 0) + 32 * 2 + (size_t) qwarp * 2 +
         (wt == 2 ? 32 * 16 : 0);
}

__host__ __device__ __forceinline__ size_t stage_bytes(int nsten, int wt,
    uint32_t qwarp) {
  return stage_cta_bytes(nsten, wt) +
         (size_t) (CT32_THREADS / 32) * stage_warp_bytes(wt, qwarp);
}

typedef void (*kfun_t)(const fcfcg_launch);

/* The FP32 counting kernel's instantiations, one family per translation
 * unit (count32_box.cu, count32_survey.cu, count32_batch.cu,
 * count32_adj.cu): the kernel for a binning code and weighting, or NULL. */
kfun_t fcfcg_pick32_box(int bin, int wt);
kfun_t fcfcg_pick32_survey(int bin, int wt);
kfun_t fcfcg_pick32_batch(int bin, int wt);
kfun_t fcfcg_pick32_adj(int geom, int bin);

#endif
