/*
 * cnvt.c -- host set-up of the RA/Dec/z conversion (cnvt.cu does the
 * per-object work on the device).
 *
 *   - cosmology checks as FCFC's check_cosmo / conf_verify
 *     (src/fcfc/2pt/load_conf.c:700-735, 925-933);
 *   - the Gauss-Legendre order chosen as cnvt_legauss_order does
 *     (src/fcfc/2pt/cnvt_coord.c:267-307) on 128 redshifts spanning the
 *     catalogue (cnvt_z_sample, :113-186), with the same integrand and sums
 *     as the device kernel, in this file's FMA-free FP64 (built with
 *     -ffp-contract=off) and the C library's pow and sqrt;
 *   - for a (z, d) table: a stable sort by z (read_sample, :40-47, sorts
 *     with timsort) and the natural-spline second derivatives
 *     (cspline_ypp, src/math/cspline.c:34-81).
 */
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "fcfcg_internal.h"
#include "legauss_tab.h"

#define NUM_ZSP 128                 /* FCFC_INT_NUM_ZSP, define.h:99 */
#define SPEED_OF_LIGHT 299792.458   /* km/s, src/util/define_comm.h:124 */

static const double gl_x[FCFCG_GL_LEN] = FCFCG_GL_X_INIT;
static const double gl_w[FCFCG_GL_LEN] = FCFCG_GL_W_INIT;

static void msg(char *err, size_t len, const char *fmt, ...) {
  if (!err || !len) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, len, fmt, ap);
  va_end(ap);
}

static double integrand(const fcfcg_cnvt_par *p, double z) {
  double z1 = z + 1;
  double z2 = z1 * z1;
  double d = p->om * z2 * z1;
  if (p->ok != 0) d += p->ok * z2;
  if (p->widx != 0) d += p->ol * pow(z1, p->widx);
  else d += p->ol;
  return p->c01 / sqrt(d);
}

static double comoving(const fcfcg_cnvt_par *p, int order, double z) {
  double zp = z * 0.5;
  double sum = 0;
  int i = FCFCG_GL_START(order);
  const int i1 = i + (order >> 1);
  for (; i < i1; i++) {
    double x = gl_x[i], w = gl_w[i];
    double za = zp * (1 + x);
    double zb = zp * (1 - x);
    sum += w * (integrand(p, za) + integrand(p, zb));
  }
  if (order & 1) sum += gl_w[i] * integrand(p, zp);
  return sum * zp;
}

/* check_cosmo + CMVDST_ERR; fills the kernel parameters (order unset). */
static int cosmo_params(const fcfcg_cosmo *cs, fcfcg_cnvt_par *p,
    double *tol, char *err, size_t errlen) {
  if (!(cs->omega_m > 0 && cs->omega_m <= 1)) {
    msg(err, errlen, "OMEGA_M must be > 0 and <= 1");
    return FCFCG_ERR_CFG;
  }
  p->om = cs->omega_m;
  if (!cs->has_omega_l) {
    p->ol = 1 - cs->omega_m;
    p->ok = 0;
  } else if (!(cs->omega_l >= 0)) {
    msg(err, errlen, "OMEGA_LAMBDA must be >= 0");
    return FCFCG_ERR_CFG;
  } else {
    p->ol = cs->omega_l;
    p->ok = 1 - cs->omega_m - cs->omega_l;
  }
  const double dew = (cs->dew == 0) ? -1 : cs->dew;
  if (dew > -1 / (double) 3 || dew != dew) {
    msg(err, errlen, "DE_EOS_W must be <= -1/3");
    return FCFCG_ERR_CFG;
  }
  const double w3 = dew * 3;
  const double wi = w3 + 1;
  if (p->ok * pow(p->ol * (-wi), wi / w3) <= p->ol * w3 * pow(p->om, wi / w3)) {
    msg(err, errlen, "negative H^2 given the cosmological parameters");
    return FCFCG_ERR_CFG;
  }
  p->widx = (dew == -1) ? 0 : 3 * (1 + dew);
  p->c01 = SPEED_OF_LIGHT * 0.01;
  *tol = (cs->cmvdst_err == 0) ? 1e-8 : cs->cmvdst_err;
  if (!(*tol >= DBL_EPSILON)) {
    msg(err, errlen, "CMVDST_ERR is smaller than the machine epsilon");
    return FCFCG_ERR_CFG;
  }
  return FCFCG_OK;
}

/* cnvt_legauss_order: the largest, over 128 sampled redshifts, of the first
 * order at which two consecutive orders agree to tol. */
static int pick_order(const fcfcg_cnvt_par *p, double tol, double zmin,
    double zmax, int *order) {
  int best = 0;
  for (int i = 0; i < NUM_ZSP; i++) {
    const double zt = zmin + i * (zmax - zmin) / (NUM_ZSP - 1);
    double oint, nint = 0;
    int n = FCFCG_GL_MIN_ORDER - 1;
    do {
      if (n >= FCFCG_GL_MAX_ORDER) return FCFCG_ERR_CNVT;
      oint = nint;
      nint = comoving(p, ++n, zt);
    } while (fabs(nint - oint) > nint * tol);
    if (best < n) best = n;
  }
  *order = best;
  return FCFCG_OK;
}

/* Stable merge sort of indices by key (timsort is stable too). */
static void msort(size_t *idx, size_t *tmp, size_t n, const double *key) {
  for (size_t w = 1; w < n; w <<= 1) {
    for (size_t lo = 0; lo < n; lo += 2 * w) {
      size_t mid = lo + w < n ? lo + w : n;
      size_t hi = lo + 2 * w < n ? lo + 2 * w : n;
      size_t a = lo, b = mid, k = lo;
      while (a < mid && b < hi)
        tmp[k++] = (key[idx[b]] < key[idx[a]]) ? idx[b++] : idx[a++];
      while (a < mid) tmp[k++] = idx[a++];
      while (b < hi) tmp[k++] = idx[b++];
    }
    memcpy(idx, tmp, n * sizeof *idx);
  }
}

/* Natural cubic spline second derivatives (the tridiagonal solve of
 * cspline_ypp, same operation order). */
static void spline_ypp(const double *x, const double *y, size_t n,
    double *ypp, double *cp) {
  double newx = x[1], newy = y[1];
  double c = x[1] - x[0];
  double newd = (y[1] - y[0]) / c;
  cp[0] = cp[n - 1] = ypp[0] = ypp[n - 1] = 0;
  size_t j = 1;
  while (j < n - 1) {
    double oldx = newx, oldy = newy, a = c, oldd = newd;
    newx = x[j + 1];
    newy = y[j + 1];
    c = newx - oldx;
    newd = (newy - oldy) / c;
    double b = (c + a) * 2;
    double invd = 1 / (b - a * cp[j - 1]);
    double d = (newd - oldd) * 6;
    ypp[j] = (d - a * ypp[j - 1]) * invd;
    cp[j] = c * invd;
    j += 1;
  }
  while (j) {
    j -= 1;
    ypp[j] -= cp[j] * ypp[j + 1];
  }
}

static int grow(void **buf, size_t *cap, size_t need) {
  if (*cap >= need && *buf) return 0;
  if (*buf) cudaFree(*buf);
  *buf = NULL;
  *cap = 0;
  if (cudaMalloc(buf, need) != cudaSuccess) return -1;
  *cap = need;
  return 0;
}

#define CUDA_OK(call)                                                     \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      msg(err, errlen, "%s: %s", #call, cudaGetErrorString(e_));          \
      rc = FCFCG_ERR_CUDA;                                                \
      goto done;                                                          \
    }                                                                     \
  } while (0)

#define KERNEL_OK(call)                                                   \
  do {                                                                    \
    int e_ = (call);                                                      \
    if (e_) {                                                             \
      msg(err, errlen, "%s: %s", #call, fcfcg_cuda_errstr(e_));           \
      rc = FCFCG_ERR_CUDA;                                                \
      goto done;                                                          \
    }                                                                     \
    (*launches)++;                                                        \
  } while (0)

int fcfcg_cnvt_device(void *stream, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const fcfcg_cosmo *cosmo, void **scratch, size_t *scratch_cap,
    int *order, long *launches, char *err, size_t errlen) {
  int rc = FCFCG_OK;
  size_t *idx = NULL, *tmp = NULL;
  double *hs = NULL;
  cudaStream_t st = (cudaStream_t) stream;
  if (order) *order = 0;
  if (!cosmo) return FCFCG_ERR_ARG;
  if (n && (!ra || !dec || !z || !x || !y || !zc)) return FCFCG_ERR_ARG;

  if (cosmo->nsample) {   /* Z_CMVDST_FILE: cubic spline */
    const size_t m = cosmo->nsample;
    if (m < 2 || !cosmo->z_sample || !cosmo->d_sample) {
      msg(err, errlen, "the redshift-distance table needs at least 2 rows");
      return FCFCG_ERR_CNVT;
    }
    idx = malloc(m * sizeof *idx);
    tmp = malloc(m * sizeof *tmp);
    hs = malloc(5 * m * sizeof *hs);
    if (!idx || !tmp || !hs) {
      rc = FCFCG_ERR_MEMORY;
      goto done;
    }
    for (size_t i = 0; i < m; i++) idx[i] = i;
    msort(idx, tmp, m, cosmo->z_sample);
    double *zs = hs, *ds = hs + m, *ypp = hs + 2 * m, *cp = hs + 3 * m;
    for (size_t i = 0; i < m; i++) {
      zs[i] = cosmo->z_sample[idx[i]];
      ds[i] = cosmo->d_sample[idx[i]];
    }
    spline_ypp(zs, ds, m, ypp, cp);
    if (!n) goto done;
    const size_t off = 256;
    if (grow(scratch, scratch_cap, off + 3 * m * sizeof(double))) {
      msg(err, errlen, "cannot allocate %zu bytes of device memory",
          off + 3 * m * sizeof(double));
      rc = FCFCG_ERR_MEMORY;
      goto done;
    }
    unsigned long long *dbad = (unsigned long long *) *scratch;
    double *dz = (double *) ((char *) *scratch + off);
    CUDA_OK(cudaMemsetAsync(dbad, 0, sizeof *dbad, st));
    CUDA_OK(cudaMemcpyAsync(dz, hs, 3 * m * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    KERNEL_OK(fcfcg_k_cnvt_spline(stream, n, ra, dec, z, x, y, zc, dz,
                                  dz + m, dz + 2 * m, m, dbad));
    unsigned long long nbad = 0;
    CUDA_OK(cudaMemcpyAsync(&nbad, dbad, sizeof nbad, cudaMemcpyDeviceToHost,
                            st));
    CUDA_OK(cudaStreamSynchronize(st));
    if (nbad) {
      msg(err, errlen, "%llu redshifts outside the table [%g, %g)", nbad,
          zs[0], zs[m - 1]);
      rc = FCFCG_ERR_CNVT;
    }
    goto done;
  }

  /* Gauss-Legendre integration */
  fcfcg_cnvt_par p;
  double tol;
  memset(&p, 0, sizeof p);
  if ((rc = cosmo_params(cosmo, &p, &tol, err, errlen))) goto done;
  if (!n) goto done;
  if (grow(scratch, scratch_cap, 256)) {
    rc = FCFCG_ERR_MEMORY;
    goto done;
  }
  unsigned long long init[2] = {~0ull, 0}, hb[2];
  unsigned long long *dbits = (unsigned long long *) *scratch;
  CUDA_OK(cudaMemcpyAsync(dbits, init, sizeof init, cudaMemcpyHostToDevice,
                          st));
  KERNEL_OK(fcfcg_k_zrange(stream, n, z, dbits));
  CUDA_OK(cudaMemcpyAsync(hb, dbits, sizeof hb, cudaMemcpyDeviceToHost, st));
  CUDA_OK(cudaStreamSynchronize(st));
  double zr[2];
  for (int k = 0; k < 2; k++) {
    unsigned long long b = hb[k];
    b = (b >> 63) ? (b & 0x7FFFFFFFFFFFFFFFull) : ~b;
    memcpy(zr + k, &b, 8);
  }
  if (!isfinite(zr[0]) || !isfinite(zr[1])) {
    msg(err, errlen, "non-finite redshift in the catalogue");
    rc = FCFCG_ERR_DATA;
    goto done;
  }
  if (zr[0] < 0) {
    msg(err, errlen, "invalid negative redshift in the catalogue (%g)", zr[0]);
    rc = FCFCG_ERR_DATA;
    goto done;
  }
  int ord = 0;
  if (pick_order(&p, tol, zr[0], zr[1], &ord)) {
    msg(err, errlen, "the redshift integration does not converge to %g by "
        "Gauss-Legendre order %d", tol, FCFCG_GL_MAX_ORDER);
    rc = FCFCG_ERR_CNVT;
    goto done;
  }
  p.order = ord;
  if (order) *order = ord;
  KERNEL_OK(fcfcg_k_cnvt_integr(stream, n, ra, dec, z, x, y, zc, &p));
  CUDA_OK(cudaStreamSynchronize(st));

done:
  free(idx);
  free(tmp);
  free(hs);
  return rc;
}
