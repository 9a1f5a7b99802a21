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
#include <string.h>

#include "fcfcg_internal.h"

/* Kernel binning codes: the public FCFCG_BIN_* (0 iso, 1 (s,mu), 2
 * (s_perp,pi)), and the same binnings with an FP32 table of s^2 or s_perp^2
 * indexed by bit pattern (bins spaced in ratio, boxes only): 3 (s_perp,pi),
 * 4 iso, 5 (s,mu). */
#define BIN_SPIL 3
#define BIN_ISOL 4
#define BIN_SMUL 5
#define IS_SPI(B) ((B) == FCFCG_BIN_SPI || (B) == BIN_SPIL)
#define IS_ISO(B) ((B) == FCFCG_BIN_ISO || (B) == BIN_ISOL)
#define IS_SMU(B) ((B) == FCFCG_BIN_SMU || (B) == BIN_SMUL)
#define LOGTAB(B) ((B) >= BIN_SPIL)
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
__device__ int ref_bin_pair(const fcfcg_launch &L, uint32_t a, uint32_t b,
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
 * ntot u32 low words followed by ntot s32 high words for weighted sums.
 * Overflow goes to the global histogram of the current catalogue. */
template <int WT, int BATCH>
__device__ __forceinline__ void hist_add(const fcfcg_launch &L,
    const MockSh *ms, uint32_t *h, int bin, long long w) {
  unsigned long long *g = BATCH ? ms->g : (WT ? L.gwt : L.gcnt);
  if (WT) {
    if (L.hist_smem) hist_add_fix32(h, (int *) (h + L.ntot), g, bin, w);
    else add128(g + 2 * bin, w);
  } else {
    if (L.hist_smem) hist_add_count(h, g, bin);
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
    unsigned long long &n_inline) {
  const unsigned long long slot = atomicAdd(L.qcount, 1ull);
  if (slot < L.qcap) {
    *((uint4 *) L.queue + slot) = make_uint4(a, b, code, BATCH ? ms->id : 0u);
    return;
  }
  n_inline++;
  int bin = ref_bin_pair(L, a, b, code, BATCH ? ms->box : L.box);
  if (bin < 0) return;
  hist_add<WT, BATCH>(L, ms, h, bin, WT ? fix_prod_pair(L, a, b) : 0);
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
    uint32_t a, uint32_t b, uint32_t code, unsigned long long &n_inline) {
  const unsigned long long slot = atomicAdd(L.qcount, 1ull);
  if (slot < L.qcap) {
    *((uint4 *) L.queue + slot) = make_uint4(a, b, code, 0u);
    return;
  }
  n_inline++;
  int bin = ref_bin_pair(L, a, b, code, L.box);
  if (bin >= 0) adj_pair(L, a, b, bin);
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
#define QCAP 1024                 /* queued pairs per round */

/* Shared memory of the FP32 kernel after the tables and the histogram.
 * Per CTA: the chunk points (and weights) and the neighbour list of the
 * chunk; per warp: the 32 neighbour points of its current block and the
 * block's in-range pairs (chunk point | lane << 6). */
struct Stage {
  float4 *a;        /* FCHUNK: chunk point local x y z, scaled weight */
  int2 *aw;         /* FCHUNK: chunk point integer weight, remainder bits */
  uint32_t *pre;    /* nsten + 1: prefix of neighbour sizes */
  uint32_t *bst;    /* nsten: first sorted index of each neighbour */
  float4 *b;        /* per warp, 32: neighbour (l_b - D) x y z, index */
  float4 *bw;       /* per warp, 32: weight, integer weight, remainder */
  uint16_t *bt;     /* per warp, 32: stencil entry */
  uint16_t *q;      /* per warp, QCAP: queued pairs */
  /* adjoint only: gradient sums in units of 2^-S, FP64 weights */
  unsigned long long *ga;   /* FCHUNK x 8 bytes: the 32-bit lo words of
                               the chunk points, then their hi words */
  double *wa;               /* FCHUNK */
  long long *gb;            /* per warp, 32: the neighbour points */
  double *wb;               /* per warp, 32 */
};

/* wt: 0 unweighted, 1 weighted, 2 adjoint (weighted + FP64 gradients) */
__host__ __device__ __forceinline__ size_t stage_cta_bytes(int nsten, int wt) {
  size_t n = (size_t) FCHUNK * 16 + (wt ? (size_t) FCHUNK * 8 : 0);
  n += (((size_t) nsten + 1) * 4 + 15) & ~(size_t) 15;
  n += (((size_t) nsten) * 4 + 15) & ~(size_t) 15;
  if (wt == 2) n += (size_t) FCHUNK * 16;
  return n;
}

__host__ __device__ __forceinline__ size_t stage_warp_bytes(int wt) {
  return 32 * 16 + (wt ? 32 * 16 : 0) + 32 * 2 + QCAP * 2 +
         (wt == 2 ? 32 * 16 : 0);
}

__host__ __device__ __forceinline__ size_t stage_bytes(int nsten, int wt) {
  return stage_cta_bytes(nsten, wt) +
         (size_t) (CT32_THREADS / 32) * stage_warp_bytes(wt);
}

/* Image code of the neighbour cell of a stencil offset (box). */
__device__ __forceinline__ uint32_t nb_code(const int *ncell, int cx,
    int cy, int cz, int4 o) {
  int q[3] = {cx + o.x, cy + o.y, cz + o.z};
  uint32_t code = 0;
  for (int k = 0; k < 3; k++) {
    const int n = ncell[k];
    int w = 0;
    while (q[k] < 0) { q[k] += n; w--; }
    while (q[k] >= n) { q[k] -= n; w++; }
    code |= (uint32_t) (w + 1) << (2 * k);
  }
  return code;
}

/*
 * Bin one queued pair per lane.  FP32 windows decide; ambiguous pairs go to
 * the FP64 recheck queue.  c2 = twice the chunk cell's centre (survey).
 */
template <int GEOM, int BIN, int WT, int BATCH, int ADJ>
__device__ __forceinline__ void bin_pair(const fcfcg_launch &L,
    const MockSh *ms, const Stage &S, uint32_t ent, uint32_t first, int cx,
    int cy, int cz,
    float c2x, float c2y, float c2z, const uint16_t *fs, const uint16_t *fp,
    const float *fse, const float *fpe, uint32_t *h, uint32_t &n_in,
    uint32_t &n_q, unsigned long long &n_inline, long long &gbv) {
  const int i = (int) (ent & 63u), src = (int) (ent >> 6);
  const float4 pa = S.a[i];
  const float4 pb = S.b[src];
  const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
  bool amb = false;
  int bin = -1;
  if (IS_SPI(BIN) && GEOM == FCFCG_GEOM_BOX) {
    const float sp2 = fmaf(dy, dy, dx * dx);
    const float pi = fabsf(dz);
    amb = !(sp2 >= L.tiny);
    /* with a bit-pattern table (log bins, narrow near zero) the window of
     * s_perp^2 follows s_perp; otherwise its value at s_perp max (tiny sp2
     * is ambiguous anyway) */
    const float Es = LOGTAB(BIN)
        ? fmaf(L.K2, sp2, fmaf(L.K1, sp2 * rsqrtf(sp2), L.K0)) : L.Emax;
    unsigned sb = ftab_bin<false, LOGTAB(BIN)>(fs, L.fsoff, L.nfs, L.fsinv, fse, L.nsb, sp2, Es, amb, L.fslog, L.fsamb);
    unsigned pbn = ftab_bin<false, false>(fp, L.fpoff, L.nfp, L.fpinv, fpe, L.npb, pi, L.P0, amb, L.fplog, L.fpamb);
    if (!amb) {
      if (sb == FCFCG_FTAB_BIN_MASK || pbn == FCFCG_FTAB_BIN_MASK) return;
      bin = (int) sb + (int) pbn * L.ns;
    }
  } else {
    const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    amb = !(s2 >= L.tiny);
    if (IS_ISO(BIN)) {
      /* with a bit-pattern table the window follows s (log bins near zero
       * are narrower than its value at s max) */
      const float Es = LOGTAB(BIN)
          ? fmaf(L.K2, s2, fmaf(L.K1, s2 * rsqrtf(s2), L.K0)) : L.Emax;
      unsigned sb = ftab_bin<false, LOGTAB(BIN)>(fs, L.fsoff, L.nfs, L.fsinv, fse, L.nsb, s2, Es, amb, L.fslog, L.fsamb);
      if (!amb) {
        if (sb == FCFCG_FTAB_BIN_MASK) return;
        bin = (int) sb;
      }
    } else {
      const float rs = rsqrtf(s2);
      const float s = s2 * rs;
      const float E = fmaf(L.K2, s2, fmaf(L.K1, s, L.K0));
      float mx = 0.f, my = 0.f, mz = 0.f;
      if (GEOM == FCFCG_GEOM_SURVEY) {
        /* line of sight m = x_a + x_b = 2 (l_b - D) + 2 c_A + d */
        mx = fmaf(2.f, pb.x, c2x) + dx;
        my = fmaf(2.f, pb.y, c2y) + dy;
        mz = fmaf(2.f, pb.z, c2z) + dz;
      }
      if (IS_SMU(BIN)) {
        float q;
        if (GEOM == FCFCG_GEOM_BOX) {
          q = L.fnmu * fabsf(dz) * rs;
        } else {
          const float dm = fmaf(dz, mz, fmaf(dy, my, dx * mx));
          const float mm = fmaf(mz, mz, fmaf(my, my, mx * mx));
          q = L.fnmu * fabsf(dm) * rsqrtf(mm * s2);
        }
        const float Eq = fmaf(L.Q1, rs, fmaf(L.Q2, q, L.Q0));
        int qi = mu_bin(q, Eq, amb);
        unsigned sb = ftab_bin<GEOM == FCFCG_GEOM_SURVEY, LOGTAB(BIN)>(fs, L.fsoff, L.nfs, L.fsinv, fse, L.nsb,
                                                            s2, E, amb, L.fslog, L.fsamb);
        if (!amb) {
          if (qi >= L.nmu) {
            if (!L.mu_one) return;
            qi = L.nmu - 1;
          }
          if (sb == FCFCG_FTAB_BIN_MASK) return;
          bin = (int) sb + qi * L.ns;
        }
      } else {
        /* survey (s_perp, pi): pi^2 = (d.m)^2 / |m|^2 */
        const float dm = fmaf(dz, mz, fmaf(dy, my, dx * mx));
        const float mm = fmaf(mz, mz, fmaf(my, my, mx * mx));
        const float pi2 = __fdividef(dm * dm, mm);
        const float sp2 = s2 - pi2;
        const float Ep = fmaf(L.P2, s2, fmaf(L.P1, s, L.P0));
        unsigned pbn = ftab_bin<true, false>(fp, L.fpoff, L.nfp, L.fpinv, fpe, L.npb, pi2, Ep, amb, L.fplog, L.fpamb);
        unsigned sb = ftab_bin<true, LOGTAB(BIN)>(fs, L.fsoff, L.nfs, L.fsinv, fse, L.nsb,
                                     sp2 < 0.f ? 0.f : sp2, E + Ep, amb, L.fslog, L.fsamb);
        if (!amb) {
          if (sb == FCFCG_FTAB_BIN_MASK || pbn == FCFCG_FTAB_BIN_MASK) return;
          bin = (int) sb + (int) pbn * L.ns;
        }
      }
    }
  }
  const uint32_t ai = first + (uint32_t) i;
  const uint32_t bj = __float_as_uint(pb.w);
  if (amb) {
    n_q++;
    uint32_t code = 0;
    if (GEOM == FCFCG_GEOM_BOX)
      code = nb_code(BATCH ? ms->nc : L.ncell, cx, cy, cz,
                     __ldg((const int4 *) L.sten + S.bt[src]));
    if (ADJ) enqueue_adj(L, ai, bj, code, n_inline);
    else enqueue<WT, BATCH>(L, ms, ai, bj, code, h, n_inline);
    return;
  }
  n_in++;
  if (ADJ) {
    /* d/dw_a of w_a w_b g[bin] is w_b g[bin], and the other way round; the
     * neighbour side is summed across the warp by the caller */
    const double g = L.hist_smem ? ((const double *) h)[bin] : __ldg(L.gfix + bin);
    adj_acc((uint32_t *) S.ga + i, (int *) S.ga + FCHUNK + i,
            adj_term(S.wb[src], g), L.dA + ai, L.gunit);
    gbv = adj_term(S.wa[i], g);
    return;
  }
  long long w = 0;
  if (WT) {
    const int2 wa = S.aw[i];
    const float4 bw = S.bw[src];
    w = fix_prod(wa.x, __int_as_float(wa.y), pa.w, __float_as_int(bw.y), bw.z,
                 bw.x);
  }
  hist_add<WT, BATCH>(L, ms, h, bin, w);
}

/* Compare a neighbour point (one per lane) with chunk points [i0, i1):
 * bit i - i0 of the result marks a candidate inside the outer range.  For
 * survey (s_perp, pi) counts (u, lh, lP) is the lane's line-of-sight
 * prefilter: a pair is dropped when |d.u| >= lP + lh s^2, where its pi
 * exceeds pi_max for sure. */
template <int GEOM, int BIN, bool LIMIT>
__device__ __forceinline__ uint32_t scan_chunk_(const fcfcg_launch &L,
    const float4 *a, int i0, int i1, int ilim, float bx, float by,
    float bz, float ux, float uy, float uz, float lh, float lP) {
  uint32_t msk = 0;
  const float s_lim = L.s_lim, p_lim = L.p_lim;
#pragma unroll 4
  for (int i = i0; i < i1; i++) {
    const float4 pa = a[i];
    const float dx = pa.x - bx, dy = pa.y - by, dz = pa.z - bz;
    bool inr;
    if (IS_SPI(BIN) && GEOM == FCFCG_GEOM_BOX) {
      const float v = fmaf(dy, dy, dx * dx);
      inr = (fabsf(dz) < p_lim) & (v < s_lim);
    } else if (LOSCUT(GEOM, BIN)) {
      const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      const float t = fmaf(dz, uz, fmaf(dy, uy, dx * ux));
      inr = (v < s_lim) & (fabsf(t) < fmaf(v, lh, lP));
    } else {
      const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      inr = v < s_lim;
    }
    if (LIMIT) inr &= (i < ilim);
    msk |= (uint32_t) inr << (i - i0);
  }
  return msk;
}

/* The i < ilim test only matters in the chunk's own cell (auto counts). */
template <int GEOM, int BIN>
__device__ __forceinline__ uint32_t scan_chunk(const fcfcg_launch &L,
    const float4 *a, int i0, int i1, int ilim, float bx, float by,
    float bz, float ux, float uy, float uz, float lh, float lP) {
  if (__all_sync(FULLMASK, ilim >= i1))
    return scan_chunk_<GEOM, BIN, false>(L, a, i0, i1, ilim, bx, by, bz, ux,
                                         uy, uz, lh, lP);
  return scan_chunk_<GEOM, BIN, true>(L, a, i0, i1, ilim, bx, by, bz, ux, uy,
                                      uz, lh, lP);
}

/*
 * FP32 counting kernel.  GEOM: box / survey; BIN: iso / smu / spi;
 * WT: weighted.  Shared memory: FP32 tables, the histogram, the CTA's chunk
 * and neighbour list, and per warp a block of neighbour points and a queue.
 *
 * A CTA holds one chunk (<= 64 points of a cell).  The non-empty neighbour
 * cells of the stencil are laid end to end (a prefix sum per chunk); the
 * warps take blocks of 32 consecutive neighbour points from a shared
 * counter, and each lane compares its point with every chunk point
 * (broadcast from shared
 * memory), recording those inside the outer range as mask bits.  A block's
 * in-range pairs are then compacted into the warp queue and binned 32 at a
 * time, every lane busy.
 */
/* (s, mu) binning keeps more values live: 3 CTAs per SM (85 registers)
 * measure faster there, 4 CTAs (64 registers) for the other binnings. */
template <int GEOM, int BIN, int WT, int BATCH, int ADJ>
__global__ void __launch_bounds__(CT32_THREADS, IS_SMU(BIN) ? 3 : 4)
k_count32(const fcfcg_launch L) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t sh_chunk;
  __shared__ uint32_t sh_blk;   /* next neighbour block of the chunk */
  __shared__ MockSh sh_mock;   /* batched launch: the current catalogue */
  int cur = -1;
  uint16_t *fs = (uint16_t *) smem;
  uint16_t *fp = fs + L.nfs;
  float *fse = (float *) (smem + (((size_t) (L.nfs + L.nfp) * 2 + 3) & ~(size_t) 3));
  float *fpe = fse + L.nsb + 1;
  size_t hoff = (size_t) ((unsigned char *) (fpe + (L.npb ? L.npb + 1 : 0)) - smem);
  hoff = (hoff + 15) & ~(size_t) 15;
  uint32_t *h = (uint32_t *) (smem + hoff);
  size_t soff = hoff + (L.hist_smem ? (size_t) L.ntot * (WT ? 8 : 4) : 0);
  soff = (soff + 15) & ~(size_t) 15;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Stage S;
  {
    unsigned char *b = smem + soff;
    S.a = (float4 *) b;
    b += (size_t) FCHUNK * 16;
    S.aw = (int2 *) b;
    b += WT ? (size_t) FCHUNK * 8 : 0;
    S.pre = (uint32_t *) b;
    b += (((size_t) L.nsten + 1) * 4 + 15) & ~(size_t) 15;
    S.bst = (uint32_t *) b;
    b += (((size_t) L.nsten) * 4 + 15) & ~(size_t) 15;
    if (ADJ) {
      S.ga = (unsigned long long *) b;
      b += (size_t) FCHUNK * 8;
      S.wa = (double *) b;
      b += (size_t) FCHUNK * 8;
    }
    b += (size_t) warp * stage_warp_bytes(WT + ADJ);
    S.b = (float4 *) b;
    b += 32 * 16;
    S.bw = (float4 *) b;
    b += WT ? 32 * 16 : 0;
    S.bt = (uint16_t *) b;
    b += 32 * 2;
    S.q = (uint16_t *) b;
    if (ADJ) {
      b += QCAP * 2;
      S.gb = (long long *) b;
      b += 32 * 8;
      S.wb = (double *) b;
    }
  }
  for (int i = threadIdx.x; i < L.nfs; i += blockDim.x) fs[i] = L.fs[i];
  for (int i = threadIdx.x; i < L.nfp; i += blockDim.x) fp[i] = L.fp[i];
  for (int i = threadIdx.x; i <= L.nsb; i += blockDim.x) fse[i] = L.fse[i];
  if (L.npb)
    for (int i = threadIdx.x; i <= L.npb; i += blockDim.x) fpe[i] = L.fpe[i];
  if (ADJ) {
    /* the cotangent of the counts takes the histogram's place */
    if (L.hist_smem)
      for (long i = threadIdx.x; i < L.ntot; i += blockDim.x)
        ((double *) h)[i] = L.gfix[i];
    for (int i = threadIdx.x; i < FCHUNK; i += blockDim.x) S.ga[i] = 0;
    if (lane < 32) S.gb[lane] = 0;
  } else if (L.hist_smem) {
    for (long i = threadIdx.x; i < L.ntot * (WT ? 2 : 1); i += blockDim.x) h[i] = 0;
  }

  const float4 *__restrict__ Bl4 = (const float4 *) L.B.l4;
  const int2 *__restrict__ Bwq = (const int2 *) L.B.wq;
  const int4 *__restrict__ sten = (const int4 *) L.sten;
  const float4 *__restrict__ stD = (const float4 *) L.stenD;
  unsigned long long n_cand = 0, n_in64 = 0, n_q64 = 0, n_inline = 0;
  const uint32_t nchunk = L.nchunk_dev ? __ldg(L.nchunk_dev) : L.nchunk;

  for (;;) {
    __syncthreads();    /* the previous chunk is done with a / pre / bst */
    if (threadIdx.x == 0) {
      sh_chunk = atomicAdd(L.chunk_head, 1u);
      sh_blk = 0;
    }
    __syncthreads();
    const uint32_t c = sh_chunk;
    if (c >= nchunk) break;
    const uint4 ch = __ldg(((const uint4 *) L.chunks) + c);
    int ncl[3] = {L.ncell[0], L.ncell[1], L.ncell[2]};
    uint32_t cbase = 0;
    if (BATCH) {
      /* chunks come in catalogue order: on a change of catalogue, hand the
       * shared histogram to the previous one's global histogram */
      const int mk = (int) ch.w;
      if (mk != cur) {
        if (cur >= 0 && L.hist_smem) hist_flush<WT>(L, h, sh_mock.g);
        __syncthreads();
        if (threadIdx.x == 0) {
          const fcfcg_mock *M = L.mocks + mk;
          for (int k = 0; k < 3; k++) {
            sh_mock.nc[k] = M->ncell[k];
            const float f = (float) M->cw[k];
            sh_mock.cwf[k] = f;
            sh_mock.cwl[k] = (float) (M->cw[k] - (double) f);
            sh_mock.box[k] = M->box[k];
          }
          sh_mock.base = M->cell_base;
          sh_mock.g = WT ? M->gwt : M->gcnt;
          sh_mock.id = (uint32_t) mk;
        }
        __syncthreads();
        cur = mk;
      }
      ncl[0] = sh_mock.nc[0];
      ncl[1] = sh_mock.nc[1];
      ncl[2] = sh_mock.nc[2];
      cbase = sh_mock.base;
    }
    const uint32_t cell = ch.x, first = ch.y;
    const uint32_t lcell = cell - cbase;
    const int m = (int) ch.z;
    const int cx = (int) (lcell % (uint32_t) ncl[0]);
    const int cy = (int) ((lcell / (uint32_t) ncl[0]) % (uint32_t) ncl[1]);
    const int cz = (int) (lcell / ((uint32_t) ncl[0] * (uint32_t) ncl[1]));
    const int aoff = (int) (first - __ldg(L.A.cstart + cell));
    float c2x = 0.f, c2y = 0.f, c2z = 0.f;
    if (GEOM == FCFCG_GEOM_SURVEY) {
      c2x = 2.f * fmaf((float) cx + 0.5f, L.cwf[0], L.lof[0]);
      c2y = 2.f * fmaf((float) cy + 0.5f, L.cwf[1], L.lof[1]);
      c2z = 2.f * fmaf((float) cz + 0.5f, L.cwf[2], L.lof[2]);
    }
    if (warp == 1) {
      for (int k = lane; k < m; k += 32) {
        S.a[k] = ((const float4 *) L.A.l4)[first + k];
        if (WT) S.aw[k] = ((const int2 *) L.A.wq)[first + k];
        if (ADJ) S.wa[k] = L.A.w[first + k];
      }
    } else if (warp == 0) {
      /* neighbour cells of this chunk, laid end to end */
      uint32_t run = 0;
      for (int t0 = 0; t0 < L.nsten; t0 += 32) {
        const int t = t0 + lane;
        uint32_t nb = 0, bs = 0;
        if (t < L.nsten) {
          const int4 o = __ldg(sten + t);
          int q[3] = {cx + o.x, cy + o.y, cz + o.z};
          bool ok = true;
          for (int k = 0; k < 3; k++) {
            const int n = ncl[k];
            if (GEOM == FCFCG_GEOM_SURVEY) {
              ok &= (q[k] >= 0) & (q[k] < n);
            } else {
              while (q[k] < 0) q[k] += n;
              while (q[k] >= n) q[k] -= n;
            }
          }
          if (ok) {
            const uint32_t cb = cbase +
                ((uint32_t) q[2] * ncl[1] + q[1]) * ncl[0] + q[0];
            bs = __ldg(L.B.cstart + cb);
            nb = __ldg(L.B.cstart + cb + 1) - bs;
          }
        }
        uint32_t inc = nb;
        for (int s = 1; s < 32; s <<= 1) {
          uint32_t u = __shfl_up_sync(FULLMASK, inc, s);
          if (lane >= s) inc += u;
        }
        if (t < L.nsten) {
          S.pre[t] = run + inc - nb;
          S.bst[t] = bs;
        }
        run += __shfl_sync(FULLMASK, inc, 31);
      }
      if (lane == 0) S.pre[L.nsten] = run;
    }
    __syncthreads();
    const uint32_t total = S.pre[L.nsten];
    /* neighbour positions [0, pin): cells whose pairs with the chunk's cell
     * all lie within the outer range (their stencil entries come first) */
    const uint32_t pin = S.pre[L.nin];
    if (warp == 0 && lane == 0) n_cand += (unsigned long long) m * total;
    uint32_t n_in = 0, n_q = 0;

    /* the warps take the chunk's blocks of 32 neighbour points as they
     * become free (their work varies), so they reach the next chunk's
     * barrier together */
    for (;;) {
      uint32_t blk = 0;
      if (lane == 0) blk = atomicAdd(&sh_blk, 1u);
      const uint32_t base = __shfl_sync(FULLMASK, blk, 0) * 32u;
      if (base >= total) break;
      const uint32_t p = base + (uint32_t) lane;
      float bx = 0.f, by = 0.f, bz = 0.f;
      float ux = 0.f, uy = 0.f, uz = 0.f, lh = 0.f, lP = 0.f;
      int ilim = 0;
      uint32_t bjl = 0;
      if (p < total) {
        /* neighbour cell of position p: last t with pre[t] <= p */
        int lo = 0, hi = L.nsten;
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (S.pre[mid] <= p) lo = mid;
          else hi = mid;
        }
        const int t = lo;
        const uint32_t jc = p - S.pre[t];
        const uint32_t bj = S.bst[t] + jc;
        const float4 pb = Bl4[bj];
        float4 D;
        if (BATCH) {
          /* -offset * cell width of this catalogue, rounded once: the width
           * is held as a float plus its float residual, and the fused
           * multiply-add rounds (-o) (cwf + cwl) a single time, as the
           * single-catalogue stencil table is rounded (no FP64 needed) */
          const int4 o = __ldg(sten + t);
          const float ox = (float) (-o.x), oy = (float) (-o.y),
                      oz = (float) (-o.z);
          D = make_float4(
              __fmaf_rn(ox, sh_mock.cwf[0], __fmul_rn(ox, sh_mock.cwl[0])),
              __fmaf_rn(oy, sh_mock.cwf[1], __fmul_rn(oy, sh_mock.cwl[1])),
              __fmaf_rn(oz, sh_mock.cwf[2], __fmul_rn(oz, sh_mock.cwl[2])),
              0.f);
        } else {
          D = __ldg(stD + t);
        }
        bx = pb.x - D.x;
        by = pb.y - D.y;
        bz = pb.z - D.z;
        if (LOSCUT(GEOM, BIN)) {
          /* x_b = (bx, by, bz) + c_A: its direction and 1 / |x_b| */
          const float xx = fmaf(0.5f, c2x, bx), xy = fmaf(0.5f, c2y, by),
                      xz = fmaf(0.5f, c2z, bz);
          const float r2 = fmaf(xz, xz, fmaf(xy, xy, xx * xx));
          if (r2 > L.los_r2min) {
            const float ir = rsqrtf(r2);
            ux = xx * ir;
            uy = xy * ir;
            uz = xz * ir;
            lh = L.los_h * ir;
            lP = fmaf(L.los_pr, ir, L.los_p);
          } else {
            lP = FLT_MAX;   /* near the observer: no prefilter */
          }
        }
        ilim = m;
        if (L.isauto && t == L.tzero) ilim = min(m, (int) jc - aoff);
        S.b[lane] = make_float4(bx, by, bz, __uint_as_float(bj));
        S.bt[lane] = (uint16_t) t;
        bjl = bj;
        if (ADJ) S.wb[lane] = L.B.w[bj];
        if (WT) {
          const int2 wq = Bwq[bj];
          S.bw[lane] = make_float4(pb.w, __int_as_float(wq.x),
                                   __int_as_float(wq.y), 0.f);
        }
      }
      /* compare with every chunk point (two 32-point halves); in weighted
       * counts a block wholly in cells within range takes every chunk point
       * (below ilim) without a test -- the binning checks each pair anyway
       * (measured: 1-2 % faster weighted; the unweighted kernel's code runs
       * 6 % slower with the branch, so it keeps the test) */
      uint32_t m0, m1;
      if (WT && !LOSCUT(GEOM, BIN) && base + 32u <= pin) {
        const int lim = min(ilim, m);
        m0 = (lim <= 0) ? 0u : (lim >= 32 ? ~0u : (1u << lim) - 1u);
        m1 = (lim <= 32) ? 0u
                         : (lim >= 64 ? ~0u : (1u << (lim - 32)) - 1u);
      } else {
        m0 = scan_chunk<GEOM, BIN>(L, S.a, 0, min(m, 32), ilim, bx, by, bz,
                                   ux, uy, uz, lh, lP);
        m1 = (m > 32) ? scan_chunk<GEOM, BIN>(L, S.a, 32, m, ilim, bx, by,
                                              bz, ux, uy, uz, lh, lP)
                      : 0u;
      }
      /* compact the block's in-range pairs into the queue, QCAP per round */
      const uint32_t cnt = __popc(m0) + __popc(m1);
      uint32_t inc = cnt;
      for (int s = 1; s < 32; s <<= 1) {
        uint32_t u = __shfl_up_sync(FULLMASK, inc, s);
        if (lane >= s) inc += u;
      }
      const uint32_t tot = __shfl_sync(FULLMASK, inc, 31);
      const uint32_t excl = inc - cnt;
      for (uint32_t r0 = 0; r0 < tot; r0 += QCAP) {
        /* this lane's entries with positions in [r0, r0 + QCAP) */
        uint32_t lo = excl > r0 ? excl : r0;
        uint32_t hi = excl + cnt < r0 + QCAP ? excl + cnt : r0 + QCAP;
        if (lo < hi) {
          uint32_t b0 = m0, b1 = m1;
          for (uint32_t sk = lo - excl; sk > 0; sk--) {
            if (b0) b0 &= b0 - 1;
            else b1 &= b1 - 1;
          }
          for (uint32_t pos = lo; pos < hi; pos++) {
            uint32_t i;
            if (b0) {
              i = (uint32_t) (__ffs(b0) - 1);
              b0 &= b0 - 1;
            } else {
              i = 32u + (uint32_t) (__ffs(b1) - 1);
              b1 &= b1 - 1;
            }
            S.q[pos - r0] = (uint16_t) (i | ((uint32_t) lane << 6));
          }
        }
        __syncwarp();
        const uint32_t nr = (tot - r0 < QCAP) ? tot - r0 : QCAP;
        /* pass k: lane l takes entry 32 k + l */
        const uint32_t np = (nr + 31) >> 5;
        for (uint32_t k = 0; k < np; k++) {
          const uint32_t e = k * 32u + (uint32_t) lane;
          long long gbv = 0;
          int key = -1;
          if (e < nr) {
            const uint32_t ent = S.q[e];
            key = (int) (ent >> 6);
            bin_pair<GEOM, BIN, WT, BATCH, ADJ>(L, &sh_mock, S, ent, first,
                                                cx, cy, cz, c2x, c2y, c2z, fs,
                                                fp, fse, fpe, h, n_in, n_q,
                                                n_inline, gbv);
          }
          if (ADJ) {
            /* the pass's entries run in neighbour order: sum each run of
             * equal neighbours across the lanes (suffix sums within a run)
             * and let the run's first lane add it -- the neighbour block is
             * this warp's own, so no atomic is needed */
            for (int o = 1; o < 32; o <<= 1) {
              const long long t = __shfl_down_sync(FULLMASK, gbv, o);
              const int k2 = __shfl_down_sync(FULLMASK, key, o);
              if (lane + o < 32 && k2 == key) gbv += t;
            }
            const int kp = __shfl_up_sync(FULLMASK, key, 1);
            if (key >= 0 && (lane == 0 || kp != key)) S.gb[key] += gbv;
            __syncwarp();
          }
        }
        __syncwarp();
      }
      if (ADJ) {
        /* the block's neighbour points are done: their gradients out */
        if (p < total) {
          const long long v = S.gb[lane];
          if (v != 0) atomicAdd(L.dB + bjl, (double) v * L.gunit);
          S.gb[lane] = 0;
        }
        __syncwarp();
      }
    }
    if (ADJ) {
      /* the chunk is done: its points' gradients out */
      __syncthreads();
      uint32_t *glo = (uint32_t *) S.ga;
      int *ghi = (int *) S.ga + FCHUNK;
      for (int k = threadIdx.x; k < m; k += blockDim.x) {
        const long long v = (long long) ghi[k] * 4294967296ll + glo[k];
        if (v != 0) atomicAdd(L.dA + first + k, (double) v * L.gunit);
        glo[k] = 0;
        ghi[k] = 0;
      }
    }
    n_in64 += n_in;
    n_q64 += n_q;
  }

  /* statistics */
  for (int o = 16; o > 0; o >>= 1) {
    n_in64 += __shfl_xor_sync(FULLMASK, n_in64, o);
    n_q64 += __shfl_xor_sync(FULLMASK, n_q64, o);
    n_inline += __shfl_xor_sync(FULLMASK, n_inline, o);
  }
  if (lane == 0) {
    if (warp == 0) atomicAdd(L.stats + 0, n_cand);
    atomicAdd(L.stats + 1, n_in64);
    atomicAdd(L.stats + 2, n_q64);
    atomicAdd(L.stats + 3, n_inline);
  }
  __syncthreads();
  if (!ADJ && L.hist_smem && (!BATCH || cur >= 0))
    hist_flush<WT>(L, h, BATCH ? sh_mock.g : (WT ? L.gwt : L.gcnt));
}

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

typedef void (*kfun_t)(const fcfcg_launch);

static kfun_t pick32(int geom, int bin, int wt, int batch, int adj) {
  if (adj) {
#define K32A(G, B)                                                         \
  if (geom == G && bin == B) return (kfun_t) k_count32<G, B, 1, 0, 1>;
    K32A(FCFCG_GEOM_BOX, FCFCG_BIN_ISO)
    K32A(FCFCG_GEOM_BOX, FCFCG_BIN_SMU)
    K32A(FCFCG_GEOM_BOX, FCFCG_BIN_SPI)
    K32A(FCFCG_GEOM_SURVEY, FCFCG_BIN_ISO)
    K32A(FCFCG_GEOM_SURVEY, FCFCG_BIN_SMU)
    K32A(FCFCG_GEOM_SURVEY, FCFCG_BIN_SPI)
    K32A(FCFCG_GEOM_BOX, BIN_SPIL)
    K32A(FCFCG_GEOM_BOX, BIN_ISOL)
    K32A(FCFCG_GEOM_BOX, BIN_SMUL)
#undef K32A
    return 0;
  }
  if (batch) {
    if (geom != FCFCG_GEOM_BOX) return 0;
#define K32B(B)                                                            \
  if (bin == B)                                                            \
    return wt ? (kfun_t) k_count32<FCFCG_GEOM_BOX, B, 1, 1, 0>             \
              : (kfun_t) k_count32<FCFCG_GEOM_BOX, B, 0, 1, 0>;
    K32B(FCFCG_BIN_ISO)
    K32B(FCFCG_BIN_SMU)
    K32B(FCFCG_BIN_SPI)
    K32B(BIN_SPIL)
    K32B(BIN_ISOL)
    K32B(BIN_SMUL)
#undef K32B
    return 0;
  }
#define K32(G, B)                                                          \
  if (geom == G && bin == B)                                               \
    return wt ? (kfun_t) k_count32<G, B, 1, 0, 0>                          \
              : (kfun_t) k_count32<G, B, 0, 0, 0>;
  K32(FCFCG_GEOM_BOX, FCFCG_BIN_ISO)
  K32(FCFCG_GEOM_BOX, FCFCG_BIN_SMU)
  K32(FCFCG_GEOM_BOX, FCFCG_BIN_SPI)
  K32(FCFCG_GEOM_SURVEY, FCFCG_BIN_ISO)
  K32(FCFCG_GEOM_SURVEY, FCFCG_BIN_SMU)
  K32(FCFCG_GEOM_SURVEY, FCFCG_BIN_SPI)
  K32(FCFCG_GEOM_BOX, BIN_SPIL)
  K32(FCFCG_GEOM_BOX, BIN_ISOL)
  K32(FCFCG_GEOM_BOX, BIN_SMUL)
#undef K32
  return 0;
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
    int precision, int nsm, size_t *smem_used) {
  kfun_t f;
  size_t smem;
  int threads;
  if (precision == FCFCG_PREC_FP64) {
    f = pick64(L->geometry, L->withwt, L->adjoint);
    smem = (L->hist_smem && !L->adjoint)
               ? (size_t) L->ntot * (L->withwt ? 8 : 4) : 0;
    threads = CT_THREADS;
  } else {
    /* a bit-pattern s table selects the kernel's log variant */
    const int bin = !L->fslog ? L->bintype
        : (L->bintype == FCFCG_BIN_SPI ? BIN_SPIL
           : (L->bintype == FCFCG_BIN_ISO ? BIN_ISOL : BIN_SMUL));
    f = pick32(L->geometry, bin, L->withwt, L->mocks != NULL, L->adjoint);
    size_t tab = fcfcg_k_count32_tab_bytes(L->nfs, L->nfp, L->nsb, L->npb);
    smem = tab + (L->hist_smem ? (size_t) L->ntot * (L->withwt ? 8 : 4) : 0);
    smem = ((smem + 15) & ~(size_t) 15) +
           stage_bytes(L->nsten, L->withwt + L->adjoint);
    threads = CT32_THREADS;
  }
  if (!f) return (int) cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute((const void *) f,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (e) return (int) e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *) f,
                                                    threads, smem);
  if (e) return (int) e;
  if (per_sm < 1) return (int) cudaErrorInvalidConfiguration;
  if (smem_used) *smem_used = smem;
  f<<<nsm * per_sm, threads, smem, (cudaStream_t) stream>>>(*L);
  return (int) cudaGetLastError();
}

/* Shared memory of the FP32 tables and edges (aligned for the histogram). */
extern "C" size_t fcfcg_k_count32_tab_bytes(int nfs, int nfp, int nsb,
    int npb) {
  size_t n = (((size_t) (nfs + nfp) * 2 + 3) & ~(size_t) 3);
  n += sizeof(float) * ((size_t) nsb + 1 + (npb ? (size_t) npb + 1 : 0));
  return (n + 15) & ~(size_t) 15;
}

/* Shared memory the FP32 kernel needs beyond its histogram. */
extern "C" size_t fcfcg_k_count32_stage(int nsten, int withwt) {
  return stage_bytes(nsten, withwt);
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
