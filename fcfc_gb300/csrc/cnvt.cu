/*
 * cnvt.cu -- RA/Dec/redshift to comoving Cartesian coordinates on the
 * device, FP64, one thread per object (FCFC_2PT's COORD_CONVERT,
 * src/fcfc/2pt/cnvt_coord.c).
 *
 *   integration:  d(z) = (c/100) * integral_0^z dz' / E(z') by Gauss-Legendre
 *                 quadrature of a fixed order (cnvt_legauss, :227-250), with
 *                 E^2 = Om (1+z)^3 + Ok (1+z)^2 + OL (1+z)^widx
 *                 (cnvt_integrand, :202-212);
 *   spline:       d(z) from a natural cubic spline through a (z, d) table
 *                 (sample_interp, :58-72, and cspline_eval,
 *                 src/math/cspline.c:96-110);
 *   then          x = d cos(dec) cos(ra), y = d cos(dec) sin(ra),
 *                 z = d sin(dec)  (cnvt_coord_integr, :321-337).
 *
 * Every sum and product is an explicit round-to-nearest intrinsic in the
 * reference's operation order, so nothing is contracted into an FMA; the
 * division and square root are IEEE correctly rounded like the host's.  sin,
 * cos and pow are CUDA's, whose results can differ from the host C library's
 * in the last bits; the tests bound that difference.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fcfcg_internal.h"
#include "legauss_tab.h"

#define CNVT_THREADS 256

__constant__ double c_glx[FCFCG_GL_LEN] = FCFCG_GL_X_INIT;
__constant__ double c_glw[FCFCG_GL_LEN] = FCFCG_GL_W_INIT;

static int grid_for(size_t n) {
  size_t b = (n + CNVT_THREADS - 1) / CNVT_THREADS;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int) b;
}

__device__ __forceinline__ unsigned long long zkey(double v) {
  unsigned long long b = (unsigned long long) __double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

/* Smallest and largest redshift (order-preserving keys: a NaN lands at one
 * end and is caught by the host's finiteness check). */
__global__ void k_zrange(size_t n, const double *__restrict__ z,
    unsigned long long *bits2) {
  unsigned long long lo = ~0ull, hi = 0;
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    unsigned long long v = zkey(z[i]);
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o);
    unsigned long long b = __shfl_xor_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(bits2, lo);
    atomicMax(bits2 + 1, hi);
  }
}

__device__ __forceinline__ double integrand(const fcfcg_cnvt_par &p,
    double z) {
  const double z1 = __dadd_rn(z, 1.0);
  const double z2 = __dmul_rn(z1, z1);
  double d = __dmul_rn(__dmul_rn(p.om, z2), z1);
  if (p.ok != 0) d = __dadd_rn(d, __dmul_rn(p.ok, z2));
  if (p.widx != 0) d = __dadd_rn(d, __dmul_rn(p.ol, pow(z1, p.widx)));
  else d = __dadd_rn(d, p.ol);
  return __ddiv_rn(p.c01, __dsqrt_rn(d));
}

__device__ __forceinline__ double comoving(const fcfcg_cnvt_par &p,
    double z) {
  const double zp = __dmul_rn(z, 0.5);
  double sum = 0;
  const int i0 = FCFCG_GL_START(p.order), i1 = i0 + (p.order >> 1);
  int i = i0;
  for (; i < i1; i++) {
    const double x = c_glx[i], w = c_glw[i];
    const double za = __dmul_rn(zp, __dadd_rn(1.0, x));
    const double zb = __dmul_rn(zp, __dsub_rn(1.0, x));
    sum = __dadd_rn(sum, __dmul_rn(w, __dadd_rn(integrand(p, za),
                                                integrand(p, zb))));
  }
  if (p.order & 1) sum = __dadd_rn(sum, __dmul_rn(c_glw[i], integrand(p, zp)));
  return __dmul_rn(sum, zp);
}

__device__ __forceinline__ void to_xyz(double ra, double dec, double dist,
    double *x, double *y, double *z, size_t i) {
  /* degrees to radians with the double nearest pi/180 */
  const double d2r = 0x1.1df46a2529d39p-6;
  const double a = __dmul_rn(ra, d2r), b = __dmul_rn(dec, d2r);
  const double cb = cos(b), sb = sin(b), ca = cos(a), sa = sin(a);
  const double dc = __dmul_rn(dist, cb);
  x[i] = __dmul_rn(dc, ca);
  y[i] = __dmul_rn(dc, sa);
  z[i] = __dmul_rn(dist, sb);
}

/* Outputs may alias the inputs: each thread reads object i before it
 * writes object i. */
__global__ void k_cnvt_integr(size_t n, const double *ra, const double *dec,
    const double *zr, double *x, double *y, double *z, fcfcg_cnvt_par p) {
  for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
       i += (size_t) gridDim.x * blockDim.x) {
    const double a = ra[i], b = dec[i], r = zr[i];
    to_xyz(a, b, comoving(p, r), x, y, z, i);
  }
}

__global__ void k_cnvt_spline(size_t n, const double *ra, const double *dec,
    const double *zr, double *x, double *y, double *z,
    const double *__restrict__ zs, const double *__restrict__ ds,
    const double *__restrict__ ypp, size_t nsp, unsigned long long *nbad) {
  unsigned long long bad = 0;
  for (size_t k = blockIdx.x * (size_t) blockDim.x + threadIdx.x; k < n;
       k += (size_t) gridDim.x * blockDim.x) {
    const double a = ra[k], b = dec[k], v = zr[k];
    double dist;
    if (!(v >= zs[0] && v < zs[nsp - 1])) {
      dist = HUGE_VAL;   /* outside the table, as sample_interp returns */
      bad++;
    } else {
      /* the interval zs[i] <= v < zs[i+1] (unique for a sorted table) */
      size_t lo = 0, hi = nsp - 1;
      while (hi - lo > 1) {
        const size_t mid = (lo + hi) >> 1;
        if (zs[mid] <= v) lo = mid;
        else hi = mid;
      }
      const size_t i = lo, j = lo + 1;
      const double ba = __dsub_rn(zs[j], zs[i]);
      const double xa = __dsub_rn(v, zs[i]);
      const double bx = __dsub_rn(zs[j], v);
      const double ba2 = __dmul_rn(ba, ba);
      const double lower = __dadd_rn(__dmul_rn(xa, ds[j]), __dmul_rn(bx, ds[i]));
      const double c = __dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(xa, xa), ba2),
                                           xa), ypp[j]);
      const double d = __dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(bx, bx), ba2),
                                           bx), ypp[i]);
      dist = __ddiv_rn(__dadd_rn(lower, __dmul_rn(1.0 / 6.0, __dadd_rn(c, d))),
                       ba);
    }
    to_xyz(a, b, dist, x, y, z, k);
  }
  for (int o = 16; o > 0; o >>= 1)
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(nbad, bad);
}

extern "C" int fcfcg_k_zrange(void *stream, size_t n, const double *z,
    unsigned long long *bits2) {
  if (!n) return 0;
  k_zrange<<<grid_for(n), CNVT_THREADS, 0, (cudaStream_t) stream>>>(n, z,
                                                                    bits2);
  return (int) cudaGetLastError();
}

extern "C" int fcfcg_k_cnvt_integr(void *stream, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const fcfcg_cnvt_par *p) {
  if (!n) return 0;
  k_cnvt_integr<<<grid_for(n), CNVT_THREADS, 0, (cudaStream_t) stream>>>(
      n, ra, dec, z, x, y, zc, *p);
  return (int) cudaGetLastError();
}

extern "C" int fcfcg_k_cnvt_spline(void *stream, size_t n, const double *ra,
    const double *dec, const double *z, double *x, double *y, double *zc,
    const double *zs, const double *ds, const double *ypp, size_t nsp,
    unsigned long long *nbad) {
  if (!n) return 0;
  k_cnvt_spline<<<grid_for(n), CNVT_THREADS, 0, (cudaStream_t) stream>>>(
      n, ra, dec, z, x, y, zc, zs, ds, ypp, nsp, nbad);
  return (int) cudaGetLastError();
}
