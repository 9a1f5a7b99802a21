/*
 * count32.cuh -- the FP32 pair-counting kernel (instantiated by count32_*.cu).
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
 */#ifndef FCFCG_COUNT32_CUH
#define FCFCG_COUNT32_CUH
#include "count_common.cuh"

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
    uint32_t &n_q, unsigned long long &n_inline, long long &gbv, bool hs) {
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
    if (IS_ISO(BIN) && LINS(BIN)) {
      const int k = lin_bin(L, s2 * rsqrtf(s2), amb);
      if (!amb) {
        if ((unsigned) k >= (unsigned) L.ns) return;
        bin = k;
      }
    } else if (IS_ISO(BIN)) {
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
      const float E = LINS(BIN) ? 0.f : fmaf(L.K2, s2, fmaf(L.K1, s, L.K0));
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
          amb |= !(mm >= L.m2min);
          q = L.fnmu * fabsf(dm) * rsqrtf(mm * s2);
        }
        const float Eq = fmaf(L.Q1, rs, fmaf(L.Q2, q, L.Q0));
        int qi = mu_bin(q, Eq, amb);
        if (LINS(BIN)) {
          const int k = lin_bin(L, s, amb);
          if (!amb) {
            if (qi >= L.nmu) {
              if (!L.mu_one) return;
              qi = L.nmu - 1;
            }
            if ((unsigned) k >= (unsigned) L.ns) return;
            bin = k + qi * L.ns;
          }
        } else {
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
        }
      } else {
        /* survey (s_perp, pi): pi^2 = (d.m)^2 / |m|^2 */
        const float dm = fmaf(dz, mz, fmaf(dy, my, dx * mx));
        const float mm = fmaf(mz, mz, fmaf(my, my, mx * mx));
        amb |= !(mm >= L.m2min);
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
    if (ADJ) enqueue_adj(L, ai, bj, code, n_inline, n_in);
    else enqueue<WT, BATCH>(L, ms, ai, bj, code, h, n_inline, n_in, hs);
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
  hist_add<WT, BATCH>(L, ms, h, bin, w, hs);
}

/* Is chunk point pa a candidate for the lane's neighbour (bx, by, bz):
 * inside the outer range (and, for survey (s_perp, pi) counts, not beyond
 * pi_max for sure by the line-of-sight prefilter (u, lh, lP))? */
template <int GEOM, int BIN>
__device__ __forceinline__ bool candidate(const fcfcg_launch &L, float4 pa,
    float bx, float by, float bz, float ux, float uy, float uz, float lh,
    float lP) {
  const float dx = pa.x - bx, dy = pa.y - by, dz = pa.z - bz;
  if (IS_SPI(BIN) && GEOM == FCFCG_GEOM_BOX) {
    const float v = fmaf(dy, dy, dx * dx);
    return (fabsf(dz) < L.p_lim) & (v < L.s_lim);
  } else if (LOSCUT(GEOM, BIN)) {
    const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float t = fmaf(dz, uz, fmaf(dy, uy, dx * ux));
    return (v < L.s_lim) & (fabsf(t) < fmaf(v, lh, lP));
  }
  const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  return v < L.s_lim;
}

/* candidate() for chunk points 2k and 2k + 1 at once (pxy = (x, x', y, y'),
 * pz = (z, z')): packed FP32 operations round each component as the scalar
 * ones do, so c0 and c1 are candidate()'s answers bit for bit. */
template <int GEOM, int BIN>
__device__ __forceinline__ void candidate2(const fcfcg_launch &L, float4 pxy,
    float2 pz, float bx, float by, float bz, float ux, float uy, float uz,
    float lh, float lP, bool &c0, bool &c1) {
  const float2 dx = __fadd2_rn(make_float2(pxy.x, pxy.y), make_float2(-bx, -bx));
  const float2 dy = __fadd2_rn(make_float2(pxy.z, pxy.w), make_float2(-by, -by));
  const float2 dz = __fadd2_rn(pz, make_float2(-bz, -bz));
  if (IS_SPI(BIN) && GEOM == FCFCG_GEOM_BOX) {
    const float2 v = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
    c0 = (fabsf(dz.x) < L.p_lim) & (v.x < L.s_lim);
    c1 = (fabsf(dz.y) < L.p_lim) & (v.y < L.s_lim);
  } else if (LOSCUT(GEOM, BIN)) {
    const float2 v = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 t = __ffma2_rn(dz, make_float2(uz, uz),
        __ffma2_rn(dy, make_float2(uy, uy), __fmul2_rn(dx, make_float2(ux, ux))));
    const float2 r = __ffma2_rn(v, make_float2(lh, lh), make_float2(lP, lP));
    c0 = (v.x < L.s_lim) & (fabsf(t.x) < r.x);
    c1 = (v.y < L.s_lim) & (fabsf(t.y) < r.y);
  } else {
    const float2 v = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    c0 = v.x < L.s_lim;
    c1 = v.y < L.s_lim;
  }
}

/* Binnings whose direct blocks take the packed path below: linear s bins
 * (s or (s, mu); boxes and surveys) and box (s_perp, pi) (FP32 tables).  Their direct blocks are those with a point within range
 * of the whole chunk (the others: every pair a candidate); the binning
 * drops the pairs beyond s_max (those whose mu window holds an edge go to
 * the recheck, which drops them: dropping them here, when the s window lies
 * beyond s_max, took two registers and measured 1 % slower than the 6 %
 * more rechecks). */
#define PACKED_DIRECT(G, B) \
  (LINS(B) || ((G) == FCFCG_GEOM_BOX && IS_SPI(B)))

/*
 * A direct block with linear s bins: the lane's neighbour (bx, by, bz;
 * sorted index bj) against every chunk point, two chunk points per step
 * (pxy = (x, x', y, y'), pz = (z, z')).  Packed FP32 operations round each
 * component as bin_pair's scalar ones do (q - Eq and t - W are formed as
 * fma(-1, Eq, q) and fma(-1, W, t), fl(q |dz| ...) as |fl(q dz ...)|: the
 * same roundings), so every pair gets bin_pair's bin and ambiguity bit for
 * bit; the neighbour's point, weight and index stay in the lane's
 * registers.  Surveys: the line of sight m = (2 l_b + c2) + d with the
 * lane's part formed once, as bin_pair forms it.
 */
template <int GEOM, int BIN, int WT, int BATCH, int ADJ>
__device__ __forceinline__ void bin_direct2(const fcfcg_launch &L,
    const MockSh *ms, const Stage &S, int m, uint32_t first, int cx, int cy,
    int cz, float c2x, float c2y, float c2z, float bx, float by, float bz,
    uint32_t bj, int lane, const uint16_t *fs, const uint16_t *fp,
    const float *fse, const float *fpe, uint32_t *h, uint32_t &n_in,
    uint32_t &n_q, unsigned long long &n_inline, bool hs, long long &gsum) {
  const float2 nbx = make_float2(-bx, -bx), nby = make_float2(-by, -by),
               nbz = make_float2(-bz, -bz);
  const float2 m1 = make_float2(-1.f, -1.f);
  float2 mbx, mby, mbz;                      /* survey: 2 l_b + c2 */
  if (GEOM == FCFCG_GEOM_SURVEY) {
    const float vx = fmaf(2.f, bx, c2x), vy = fmaf(2.f, by, c2y),
                vz = fmaf(2.f, bz, c2z);
    mbx = make_float2(vx, vx);
    mby = make_float2(vy, vy);
    mbz = make_float2(vz, vz);
  }
  float4 bw = make_float4(0.f, 0.f, 0.f, 0.f);
  if (WT && !ADJ) bw = S.bw[lane];
  double wbl = 0;                 /* adjoint: the neighbour's FP64 weight */
  if (ADJ) wbl = S.wb[lane];
  for (int k = 0; k < m; k += 2) {
    const float4 pxy = S.pxy[k >> 1];
    const float2 dx = __fadd2_rn(make_float2(pxy.x, pxy.y), nbx);
    const float2 dy = __fadd2_rn(make_float2(pxy.z, pxy.w), nby);
    const float2 dz = __fadd2_rn(S.pz[k >> 1], nbz);
    bool a[2], ok[2];
    int bin[2];
    if (IS_SPI(BIN)) {
      /* box (s_perp, pi): bin_pair's table lookups, per pair */
      const float2 sp2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const float v = e ? sp2.y : sp2.x;
        const float pi = fabsf(e ? dz.y : dz.x);
        bool am = !(v >= L.tiny);
        const float Es = LOGTAB(BIN)
            ? fmaf(L.K2, v, fmaf(L.K1, v * rsqrtf(v), L.K0)) : L.Emax;
        const unsigned sb = ftab_bin<false, LOGTAB(BIN)>(fs, L.fsoff, L.nfs,
            L.fsinv, fse, L.nsb, v, Es, am, L.fslog, L.fsamb);
        const unsigned pbn = ftab_bin<false, false>(fp, L.fpoff, L.nfp,
            L.fpinv, fpe, L.npb, pi, L.P0, am, L.fplog, L.fpamb);
        const bool valid = (e == 0) || (k + 1 < m);
        a[e] = valid && am;
        ok[e] = valid && !am && sb != FCFCG_FTAB_BIN_MASK &&
                pbn != FCFCG_FTAB_BIN_MASK;
        bin[e] = (int) sb + (int) pbn * L.ns;
      }
    } else {
      const float2 s2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
      const float2 rs = make_float2(rsqrtf(s2.x), rsqrtf(s2.y));
      const float2 s = __fmul2_rn(s2, rs);
      int qi[2] = {0, 0}, kb[2], klo[2];
      bool amb[2] = {!(s2.x >= L.tiny), !(s2.y >= L.tiny)};
      if (IS_SMU(BIN)) {
        float2 q;
        if (GEOM == FCFCG_GEOM_BOX) {
          q = __fmul2_rn(__fmul2_rn(make_float2(L.fnmu, L.fnmu), dz), rs);
        } else {
          const float2 mx = __fadd2_rn(mbx, dx), my = __fadd2_rn(mby, dy),
                       mz = __fadd2_rn(mbz, dz);
          const float2 dm = __ffma2_rn(dz, mz, __ffma2_rn(dy, my, __fmul2_rn(dx, mx)));
          const float2 mm = __ffma2_rn(mz, mz, __ffma2_rn(my, my, __fmul2_rn(mx, mx)));
          amb[0] |= !(mm.x >= L.m2min);
          amb[1] |= !(mm.y >= L.m2min);
          const float2 p = __fmul2_rn(mm, s2);
          q = __fmul2_rn(__fmul2_rn(make_float2(L.fnmu, L.fnmu), dm),
                         make_float2(rsqrtf(p.x), rsqrtf(p.y)));
        }
        q = make_float2(fabsf(q.x), fabsf(q.y));
        const float2 Eq = __ffma2_rn(make_float2(L.Q1, L.Q1), rs,
            __ffma2_rn(make_float2(L.Q2, L.Q2), q, make_float2(L.Q0, L.Q0)));
        const float2 qlo = __ffma2_rn(m1, Eq, q);
        const float2 qhi = __fadd2_rn(q, Eq);
        qi[0] = __float2int_rz(qhi.x);
        qi[1] = __float2int_rz(qhi.y);
        amb[0] |= (__float2int_rz(qlo.x) != qi[0]);
        amb[1] |= (__float2int_rz(qlo.y) != qi[1]);
      }
      const float2 t = __ffma2_rn(s, make_float2(L.lin_inv, L.lin_inv),
                                  make_float2(L.lin_off, L.lin_off));
      const float2 W = __ffma2_rn(make_float2(L.lin_A, L.lin_A), s,
                                  make_float2(L.lin_B, L.lin_B));
      const float2 tlo = __ffma2_rn(m1, W, t);
      const float2 thi = __fadd2_rn(t, W);
      kb[0] = __float2int_rd(thi.x);
      kb[1] = __float2int_rd(thi.y);
      klo[0] = max(__float2int_rd(tlo.x), L.lin_k0);
      klo[1] = max(__float2int_rd(tlo.y), L.lin_k0);
      /* per pair, without branches: ambiguous (a), binned (ok), its bin;
       * the second pair of an odd chunk's last step is neither */
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const bool valid = (e == 0) || (k + 1 < m);
        a[e] = valid && (amb[e] | (klo[e] != kb[e]));
        int q = qi[e];
        bool in = valid && !a[e] && (unsigned) kb[e] < (unsigned) L.ns;
        if (IS_SMU(BIN)) {
          in = in && (q < L.nmu || L.mu_one);
          q = min(q, L.nmu - 1);
        }
        ok[e] = in;
        bin[e] = kb[e] + (IS_SMU(BIN) ? q * L.ns : 0);
      }
    }
    n_in += (uint32_t) ok[0] + (uint32_t) ok[1];
    if (!WT && !ADJ && hs) {
      if (ok[0]) atomicAdd(h + bin[0], 1u);
      if (ok[1]) atomicAdd(h + bin[1], 1u);
    } else {
#pragma unroll
      for (int e = 0; e < 2; e++) {
        if (!ok[e]) continue;
        if (ADJ) {
          /* as bin_pair: the chunk point's term to its accumulator, the
           * neighbour's summed in the lane (at most 64 terms below 2^50) */
          const double g = L.hist_smem ? ((const double *) h)[bin[e]]
                                       : __ldg(L.gfix + bin[e]);
          adj_acc((uint32_t *) S.ga + (k + e), (int *) S.ga + FCHUNK + (k + e),
                  adj_term(wbl, g), L.dA + first + (uint32_t) (k + e),
                  L.gunit);
          gsum += adj_term(S.wa[k + e], g);
          continue;
        }
        long long w = 0;
        if (WT) {
          const int2 wa = S.aw[k + e];
          w = fix_prod(wa.x, __int_as_float(wa.y), S.a[k + e].w,
                       __float_as_int(bw.y), bw.z, bw.x);
        }
        hist_add<WT, BATCH>(L, ms, h, bin[e], w, hs);
      }
    }
    /* the rare ambiguous pairs: to the FP64 recheck */
    if (__any_sync(FULLMASK, a[0] | a[1])) {
#pragma unroll
      for (int e = 0; e < 2; e++) {
        if (!a[e]) continue;
        n_q++;
        const uint32_t code = (GEOM == FCFCG_GEOM_BOX)
            ? nb_code(BATCH ? ms->nc : L.ncell, cx, cy, cz,
                      __ldg((const int4 *) L.sten + S.bt[lane]))
            : 0u;
        const uint32_t ai = first + (uint32_t) (k + e);
        if (ADJ) enqueue_adj(L, ai, bj, code, n_inline, n_in);
        else enqueue<WT, BATCH>(L, ms, ai, bj, code, h, n_inline, n_in, hs);
      }
    }
  }
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
/* 4 CTAs per SM (64 registers) measure fastest for the counts: the packed
 * direct path would take 66-70 registers and lose the fourth CTA (weighted
 * box (s, mu) 40.6 ms against 35.4 ms with a 4-byte spill at 64, survey
 * (s, mu) RR 93.9 against 84.4 ms).  The survey (s, mu) adjoint keeps 3
 * (78 registers). */
template <int GEOM, int BIN, int WT, int BATCH, int ADJ>
__global__ void __launch_bounds__(CT32_THREADS,
    (IS_SMU(BIN) && GEOM != FCFCG_GEOM_BOX && ADJ) ? 3 : 4)
k_count32(const fcfcg_launch L) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t sh_chunk;
  __shared__ uint32_t sh_blk;   /* next neighbour block of the chunk */
  __shared__ MockSh sh_mock;   /* batched launch: the current catalogue */
  __shared__ float sh_box[6];  /* the chunk points' bounding box (lo, hi) */
  /* unweighted shared histogram: pairs added at most since the CTA last
   * handed its bins to the global counters, and this chunk's mode (0 add,
   * 1 hand over first, 2 count in global memory) */
  __shared__ unsigned long long sh_hs_added;
  __shared__ int sh_hs_mode;
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
    S.pxy = (float4 *) b;
    b += (size_t) FCHUNK * 8;
    S.pz = (float2 *) b;
    b += (size_t) FCHUNK * 4;
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
    b += (size_t) warp * stage_warp_bytes(WT + ADJ, L.qwarp);
    S.b = (float4 *) b;
    b += 32 * 16;
    S.bw = (float4 *) b;
    b += WT ? 32 * 16 : 0;
    S.bt = (uint16_t *) b;
    b += 32 * 2;
    S.q = (uint16_t *) b;
    if (ADJ) {
      b += (size_t) L.qwarp * 2;
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
  if (threadIdx.x == 0) sh_hs_added = 0;
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
          sh_hs_added = 0;
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
      /* twice the chunk cell's centre: the FP64 centre the local
       * coordinates are relative to, rounded once */
      c2x = (float) (2.0 * (L.lo[0] + ((double) cx + 0.5) * L.cw[0]));
      c2y = (float) (2.0 * (L.lo[1] + ((double) cy + 0.5) * L.cw[1]));
      c2z = (float) (2.0 * (L.lo[2] + ((double) cz + 0.5) * L.cw[2]));
    }
    if (warp == 1) {
      float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
      float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
      float *pxy = (float *) S.pxy, *pz = (float *) S.pz;
      for (int k = lane; k < m; k += 32) {
        const float4 v = ((const float4 *) L.A.l4)[first + k];
        S.a[k] = v;
        pxy[(k >> 1) * 4 + (k & 1)] = v.x;
        pxy[(k >> 1) * 4 + 2 + (k & 1)] = v.y;
        pz[k] = v.z;
        lo[0] = fminf(lo[0], v.x);
        lo[1] = fminf(lo[1], v.y);
        lo[2] = fminf(lo[2], v.z);
        hi[0] = fmaxf(hi[0], v.x);
        hi[1] = fmaxf(hi[1], v.y);
        hi[2] = fmaxf(hi[2], v.z);
        if (WT) S.aw[k] = ((const int2 *) L.A.wq)[first + k];
        if (ADJ) S.wa[k] = L.A.w[first + k];
      }
      for (int o = 16; o > 0; o >>= 1)
        for (int d = 0; d < 3; d++) {
          lo[d] = fminf(lo[d], __shfl_xor_sync(FULLMASK, lo[d], o));
          hi[d] = fmaxf(hi[d], __shfl_xor_sync(FULLMASK, hi[d], o));
        }
      if (lane == 0) {
        for (int d = 0; d < 3; d++) {
          sh_box[d] = lo[d];
          sh_box[3 + d] = hi[d];
        }
        if (m & 1) {
          /* the odd chunk's last pair: a partner no test passes (its
           * squared separation overflows, its |dz| exceeds any pi_max) */
          pxy[(m >> 1) * 4 + 1] = 1e30f;
          pxy[(m >> 1) * 4 + 3] = 1e30f;
          pz[m] = 1e30f;
        }
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
      if (lane == 0) {
        S.pre[L.nsten] = run;
        /* the chunk adds at most m x total pairs to the u32 shared bins:
         * hand them over first if the sum since the last hand-over could
         * pass hs_limit (<= 2^32 - 1), or count in global memory if the
         * chunk alone could */
        if (!WT && !ADJ && L.hist_smem) {
          const unsigned long long add = (unsigned long long) m * run;
          int mode = 0;
          if (add > L.hs_limit) {
            mode = 2;
          } else {
            if (sh_hs_added + add > L.hs_limit) {
              mode = 1;
              sh_hs_added = 0;
            }
            sh_hs_added += add;
          }
          sh_hs_mode = mode;
        }
      }
    }
    __syncthreads();
    const uint32_t total = S.pre[L.nsten];
    /* neighbour positions [0, pin): cells whose pairs with the chunk's cell
     * all lie within the outer range (their stencil entries come first) */
    const uint32_t pin = S.pre[L.nin];
    if (warp == 0 && lane == 0) n_cand += (unsigned long long) m * total;
    uint32_t n_in = 0, n_q = 0;
    bool hs = L.hist_smem;
    if (!WT && !ADJ && L.hist_smem) {
      const int mode = sh_hs_mode;
      if (mode == 1) {
        hist_flush<WT>(L, h, BATCH ? sh_mock.g : L.gcnt);
        __syncthreads();
      }
      hs = (mode != 2);
    }

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
      /* a block none of whose points is within the outer range of the
       * chunk points' bounding box holds no candidate: skip it.  The
       * box distance is formed as the candidate test forms a pair's
       * separation (the same roundings, each monotone), so it never
       * exceeds that of any pair of the block */
      /* and a block all of whose points are within the outer range of
       * the whole box (its farthest corner, rounded the same way) is binned
       * without the test, as a block of cells wholly in range (with the
       * packed binning, a block with one such point) */
      bool near_all = base + 32u <= pin;
      if (!near_all) {
        bool far = true, near = false;
        if (p < total) {
          const float lx = sh_box[0] - bx, hx = sh_box[3] - bx;
          const float ly = sh_box[1] - by, hy = sh_box[4] - by;
          const float lz = sh_box[2] - bz, hz = sh_box[5] - bz;
          const float ex = fmaxf(fmaxf(lx, -hx), 0.f);
          const float ey = fmaxf(fmaxf(ly, -hy), 0.f);
          const float ez = fmaxf(fmaxf(lz, -hz), 0.f);
          const float fx = fmaxf(fabsf(lx), fabsf(hx));
          const float fy = fmaxf(fabsf(ly), fabsf(hy));
          const float fz = fmaxf(fabsf(lz), fabsf(hz));
          if (IS_SPI(BIN) && GEOM == FCFCG_GEOM_BOX) {
            far = (ez >= L.p_lim) | (fmaf(ey, ey, ex * ex) >= L.s_lim);
            near = (fz < L.p_lim) & (fmaf(fy, fy, fx * fx) < L.s_lim);
          } else {
            far = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) >= L.s_lim;
            near = fmaf(fz, fz, fmaf(fy, fy, fx * fx)) < L.s_lim;
          }
        }
        if (__all_sync(FULLMASK, far)) continue;
        /* the packed direct binning costs less per pair than the test, the
         * queue and the scalar binning as soon as about a third of a
         * block's pairs are in range: it takes every block with a point
         * within range of the whole chunk (measured: one such point 333
         * ms, eight 340, all 32 374 on 48 large mocks) */
        near_all = PACKED_DIRECT(GEOM, BIN) ? __any_sync(FULLMASK, near)
                                            : __all_sync(FULLMASK, near);
      }
      if (!ADJ) {
        /*
         * The block's candidates go to the warp's queue chunk point by chunk
         * point (entry i | lane << 6), compacted by one ballot per chunk
         * point, and are binned 32 at a time with every lane busy: when the
         * next chunk point could overflow the queue, and at the end of the
         * block.  A block wholly in cells within range of the chunk's cell
         * (every pair a candidate) skips the test and the queue: pass k bins
         * chunk point k against every lane's neighbour.
         */
        const bool all_lim = __all_sync(FULLMASK, ilim >= m);
        const bool direct = !LOSCUT(GEOM, BIN) && all_lim && near_all;
        if (PACKED_DIRECT(GEOM, BIN) && direct) {
          long long gsum = 0;
          bin_direct2<GEOM, BIN, WT, BATCH, 0>(L, &sh_mock, S, m, first, cx,
                                               cy, cz, c2x, c2y, c2z, bx, by,
                                               bz, bjl, lane, fs, fp, fse, fpe,
                                               h, n_in, n_q, n_inline, hs,
                                               gsum);
          continue;
        }
        const uint32_t lt = (1u << lane) - 1u;
        uint32_t nq = direct ? (uint32_t) m * 32u : 0u;
        int i = direct ? m : 0;
        for (;;) {
          /* scan from chunk point i until the next one could overflow the
           * queue (the binning below is the only copy of that code) */
          if (all_lim) {
            /* two chunk points per step (i even), each of their tests
             * rounded as the scalar test is */
            for (; i < m && nq <= L.qwarp - 64u; i += 2) {
              bool c0, c1;
              candidate2<GEOM, BIN>(L, S.pxy[i >> 1], S.pz[i >> 1], bx, by, bz,
                                    ux, uy, uz, lh, lP, c0, c1);
              const uint32_t b0 = __ballot_sync(FULLMASK, c0);
              const uint32_t b1 = __ballot_sync(FULLMASK, c1);
              if (c0) S.q[nq + __popc(b0 & lt)] = (uint16_t) (i | (lane << 6));
              nq += __popc(b0);
              if (c1)
                S.q[nq + __popc(b1 & lt)] = (uint16_t) ((i + 1) | (lane << 6));
              nq += __popc(b1);
            }
          } else {
            /* the chunk's own cell in an auto count (j > i only), or lanes
             * past the end of the neighbour list (ilim 0) */
            for (; i < m && nq <= L.qwarp - 32u; i++) {
              const bool inr = (i < ilim) &&
                  candidate<GEOM, BIN>(L, S.a[i], bx, by, bz, ux, uy, uz, lh,
                                       lP);
              const uint32_t bal = __ballot_sync(FULLMASK, inr);
              if (inr) S.q[nq + __popc(bal & lt)] = (uint16_t) (i | (lane << 6));
              nq += __popc(bal);
            }
          }
          __syncwarp();
          const uint32_t np = (nq + 31) >> 5;
          for (uint32_t k = 0; k < np; k++) {
            const uint32_t e = k * 32u + (uint32_t) lane;
            long long gbv = 0;
            if (e < nq) {
              const uint32_t ent = direct ? (k | ((uint32_t) lane << 6))
                                          : (uint32_t) S.q[e];
              bin_pair<GEOM, BIN, WT, BATCH, ADJ>(L, &sh_mock, S, ent, first,
                                                  cx, cy, cz, c2x, c2y, c2z,
                                                  fs, fp, fse, fpe, h, n_in,
                                                  n_q, n_inline, gbv, hs);
            }
          }
          __syncwarp();
          nq = 0;
          if (i >= m) break;
        }
        continue;
      }
      /* the adjoint's direct blocks (linear s bins): the packed binning,
       * the lane's neighbour terms summed in a register */
      if (PACKED_DIRECT(GEOM, BIN) && near_all &&
          __all_sync(FULLMASK, ilim >= m)) {
        long long gsum = 0;
        bin_direct2<GEOM, BIN, WT, BATCH, ADJ>(L, &sh_mock, S, m, first, cx,
                                               cy, cz, c2x, c2y, c2z, bx, by,
                                               bz, bjl, lane, fs, fp, fse, fpe,
                                               h, n_in, n_q, n_inline, hs,
                                               gsum);
        S.gb[lane] += gsum;
        __syncwarp();
      } else {
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
        /* compact the block's in-range pairs into the queue, qwarp per round */
        const uint32_t cnt = __popc(m0) + __popc(m1);
        uint32_t inc = cnt;
        for (int s = 1; s < 32; s <<= 1) {
          uint32_t u = __shfl_up_sync(FULLMASK, inc, s);
          if (lane >= s) inc += u;
        }
        const uint32_t tot = __shfl_sync(FULLMASK, inc, 31);
        const uint32_t excl = inc - cnt;
        for (uint32_t r0 = 0; r0 < tot; r0 += L.qwarp) {
          /* this lane's entries with positions in [r0, r0 + qwarp) */
          uint32_t lo = excl > r0 ? excl : r0;
          uint32_t hi = excl + cnt < r0 + L.qwarp ? excl + cnt : r0 + L.qwarp;
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
          const uint32_t nr = (tot - r0 < L.qwarp) ? tot - r0 : L.qwarp;
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
                                                  n_inline, gbv, hs);
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

#endif
