/* cpu_nufft.c -- TEST INFRASTRUCTURE ONLY.
 *
 * The CPU FINUFFT restatement's spreader and interpolator (OpenMP), used by
 * oracle.py's CpuPlan as the CPU library's arithmetic in tests and as the
 * timed CPU baseline of bench.py. Nothing in the GB300 engine links, loads or
 * calls this file.
 *
 * It follows the CPU library's design:
 *   - fold of a coordinate to the fine grid, x/2pi + 1/2 reduced to [0,1) and
 *     scaled by nf (include/finufft/simd.hpp:318-325), first support cell
 *     ceil(r - ns/2) (include/finufft/spread.hpp:53-451);
 *   - a stable counting sort of the points into 16 x 4 x 4 bins, x fastest
 *     (include/finufft/spread.hpp:459-584);
 *   - type-1 spreading in subproblems of consecutive sorted points: at least
 *     one per thread, at most 1e5 points each in 2D/3D (1e4 in 1D)
 *     (include/finufft/spreadinterp.hpp:370-380 and makeplan.hpp:195), each
 *     summed into a private padded box that is then added into the periodic
 *     grid with atomic adds (spreadinterp.hpp:395-480);
 *   - the kernel from ns piecewise polynomials in Horner form, evaluated for
 *     all ns cells at once (the CPU library's precomputed Horner tables,
 *     src/common/kernel.cpp), and arithmetic in the plan precision.
 * The inner loops are specialised on the kernel width so the compiler
 * vectorises them (the CPU library specialises by templates and xsimd).
 * Complex arrays are interleaved (re, im).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CN_INV_2PI 0.159154943091895335768883763372514362
#define CN_MAXNS 16
#define CN_MAXNC 24

static int cn_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

#define CN_DEFINE(T, SUF)                                                                    \
  /* grid position of x: first support cell i1 and t0 = i1 - r (in (-ns/2-1, -ns/2]) */    \
  static inline void cn_place_##SUF(T x, int nf, int ns, int *i1, T *t0) {                  \
    T r = x * (T)CN_INV_2PI + (T)0.5;                                                        \
    r = (r - floor(r)) * (T)nf;                                                              \
    T s = ceil(r - (T)0.5 * ns);                                                             \
    *i1 = (int)s;                                                                            \
    *t0 = s - r;                                                                             \
  }                                                                                          \
  /* stable counting sort into 16 x 4 x 4 bins (x fastest) */                               \
  void or_cpu_sort_##SUF(int dim, int64_t M, const T *const *xyz, const int *nf,            \
                         int32_t *perm) {                                                    \
    const int bs[3] = {16, 4, 4};                                                            \
    int nb[3] = {1, 1, 1};                                                                   \
    for (int d = 0; d < dim; ++d) nb[d] = nf[d] / bs[d] + 1;                                 \
    const int64_t nbins = (int64_t)nb[0] * nb[1] * nb[2];                                    \
    int64_t *cnt = (int64_t *)calloc((size_t)nbins + 1, sizeof(int64_t));                    \
    uint32_t *key = (uint32_t *)malloc((size_t)(M > 0 ? M : 1) * sizeof(uint32_t));          \
    _Pragma("omp parallel for schedule(static)") for (int64_t i = 0; i < M; ++i) {         \
      int64_t k = 0, st = 1;                                                                 \
      for (int d = 0; d < dim; ++d) {                                                        \
        T r = xyz[d][i] * (T)CN_INV_2PI + (T)0.5;                                            \
        r = (r - floor(r)) * (T)nf[d];                                                       \
        int b = (int)(r / bs[d]);                                                            \
        if (b >= nb[d]) b = nb[d] - 1;                                                       \
        if (b < 0) b = 0;                                                                    \
        k += st * b;                                                                         \
        st *= nb[d];                                                                         \
      }                                                                                      \
      key[i] = (uint32_t)k;                                                                  \
    }                                                                                        \
    for (int64_t i = 0; i < M; ++i) cnt[key[i] + 1]++;                                       \
    for (int64_t b = 0; b < nbins; ++b) cnt[b + 1] += cnt[b];                                \
    for (int64_t i = 0; i < M; ++i) perm[cnt[key[i]]++] = (int32_t)i;                        \
    free(cnt);                                                                               \
    free(key);                                                                               \
  }

CN_DEFINE(float, f)
CN_DEFINE(double, d)

/* Kernel values at the ns cells of a point: coefficient table ct[k][j]
 * (k = 0 the highest degree, NC rows of NS) at u = 2 t0 + ns - 1. */
#define CN_HORNER(T, NS, nc, ct, t0, ker)                                                    \
  do {                                                                                       \
    const T u_ = (T)2 * (t0) + (T)((NS)-1);                                                  \
    for (int j_ = 0; j_ < (NS); ++j_) (ker)[j_] = (ct)[j_];                                  \
    for (int k_ = 1; k_ < (nc); ++k_)                                                        \
      for (int j_ = 0; j_ < (NS); ++j_) (ker)[j_] = (ker)[j_] * u_ + (ct)[k_ * (NS) + j_];  \
  } while (0)

/* One subproblem's points [p0, p1) summed into box (interleaved complex,
 * extent ext[0] x ext[1] x ext[2], origin lo) with width NS. */
#define CN_SPREAD_BOX(T, SUF, NS)                                                            \
  static void cn_box_##SUF##_##NS(int dim, const T *const *xyz, const T *c, const int *nf,  \
                                  int nc, const T *ct, int64_t n, const int *lo,             \
                                  const int64_t *ext, T *box) {                              \
    T kx[NS], ky[NS], kz[NS], kx2[2 * NS];                                                   \
    for (int64_t j = 0; j < n; ++j) {                                                        \
      int ix, iy = 0, iz = 0;                                                                \
      T t0;                                                                                  \
      cn_place_##SUF(xyz[0][j], nf[0], NS, &ix, &t0);                                        \
      CN_HORNER(T, NS, nc, ct, t0, kx);                                                      \
      const T cr = c[2 * j], ci = c[2 * j + 1];                                              \
      for (int q = 0; q < NS; ++q) {                                                         \
        kx2[2 * q] = kx[q] * cr;                                                             \
        kx2[2 * q + 1] = kx[q] * ci;                                                         \
      }                                                                                      \
      if (dim == 1) {                                                                        \
        T *row = box + 2 * (ix - lo[0]);                                                     \
        for (int i = 0; i < 2 * NS; ++i) row[i] += kx2[i];                                   \
        continue;                                                                            \
      }                                                                                      \
      cn_place_##SUF(xyz[1][j], nf[1], NS, &iy, &t0);                                        \
      CN_HORNER(T, NS, nc, ct, t0, ky);                                                      \
      if (dim == 2) {                                                                        \
        for (int b = 0; b < NS; ++b) {                                                       \
          T *row = box + 2 * ((ix - lo[0]) + ext[0] * (iy - lo[1] + b));                     \
          const T w = ky[b];                                                                 \
          for (int i = 0; i < 2 * NS; ++i) row[i] += w * kx2[i];                             \
        }                                                                                    \
        continue;                                                                            \
      }                                                                                      \
      cn_place_##SUF(xyz[2][j], nf[2], NS, &iz, &t0);                                        \
      CN_HORNER(T, NS, nc, ct, t0, kz);                                                      \
      for (int a = 0; a < NS; ++a)                                                           \
        for (int b = 0; b < NS; ++b) {                                                       \
          T *row = box + 2 * ((ix - lo[0]) + ext[0] * ((iy - lo[1] + b) +                    \
                                                        ext[1] * (iz - lo[2] + a)));         \
          const T w = ky[b] * kz[a];                                                         \
          for (int i = 0; i < 2 * NS; ++i) row[i] += w * kx2[i];                             \
        }                                                                                    \
    }                                                                                        \
  }                                                                                          \
  /* sum of grid values at one point, width NS */                                            \
  static void cn_interp_##SUF##_##NS(int dim, const T *const *xyz, const int32_t *perm,     \
                                     const T *grid, const int *nf, int nc, const T *ct,      \
                                     int64_t p0, int64_t p1, T *c) {                         \
    const int64_t n0 = nf[0], n1 = dim > 1 ? nf[1] : 1, n2 = dim > 2 ? nf[2] : 1;           \
    T kx[NS], ky[NS], kz[NS];                                                                \
    int64_t gxs[NS];                                                                         \
    for (int64_t p = p0; p < p1; ++p) {                                                      \
      const int64_t j = perm[p];                                                             \
      int ix, iy = 0, iz = 0;                                                                \
      T t0;                                                                                  \
      cn_place_##SUF(xyz[0][j], nf[0], NS, &ix, &t0);                                        \
      CN_HORNER(T, NS, nc, ct, t0, kx);                                                      \
      ky[0] = kz[0] = (T)1;                                                                  \
      if (dim > 1) {                                                                         \
        cn_place_##SUF(xyz[1][j], nf[1], NS, &iy, &t0);                                      \
        CN_HORNER(T, NS, nc, ct, t0, ky);                                                    \
      }                                                                                      \
      if (dim > 2) {                                                                         \
        cn_place_##SUF(xyz[2][j], nf[2], NS, &iz, &t0);                                      \
        CN_HORNER(T, NS, nc, ct, t0, kz);                                                    \
      }                                                                                      \
      for (int q = 0; q < NS; ++q) gxs[q] = ((ix + q) % n0 + n0) % n0;                       \
      const int ny = dim > 1 ? NS : 1, nz = dim > 2 ? NS : 1;                                \
      T sr = 0, si = 0;                                                                      \
      for (int a = 0; a < nz; ++a) {                                                         \
        const int64_t gz = dim > 2 ? ((iz + a) % n2 + n2) % n2 : 0;                          \
        for (int b = 0; b < ny; ++b) {                                                       \
          const int64_t gy = dim > 1 ? ((iy + b) % n1 + n1) % n1 : 0;                        \
          const T *g = grid + 2 * n0 * (gy + n1 * gz);                                       \
          T rr = 0, ri = 0;                                                                  \
          for (int q = 0; q < NS; ++q) {                                                     \
            rr += kx[q] * g[2 * gxs[q]];                                                     \
            ri += kx[q] * g[2 * gxs[q] + 1];                                                 \
          }                                                                                  \
          const T w = ky[b] * kz[a];                                                         \
          sr += w * rr;                                                                      \
          si += w * ri;                                                                      \
        }                                                                                    \
      }                                                                                      \
      c[2 * j] = sr;                                                                         \
      c[2 * j + 1] = si;                                                                     \
    }                                                                                        \
  }

#define CN_ALL_NS(T, SUF)                                                                    \
  CN_SPREAD_BOX(T, SUF, 2)                                                                   \
  CN_SPREAD_BOX(T, SUF, 3)                                                                   \
  CN_SPREAD_BOX(T, SUF, 4)                                                                   \
  CN_SPREAD_BOX(T, SUF, 5)                                                                   \
  CN_SPREAD_BOX(T, SUF, 6)                                                                   \
  CN_SPREAD_BOX(T, SUF, 7)                                                                   \
  CN_SPREAD_BOX(T, SUF, 8)                                                                   \
  CN_SPREAD_BOX(T, SUF, 9)                                                                   \
  CN_SPREAD_BOX(T, SUF, 10)                                                                  \
  CN_SPREAD_BOX(T, SUF, 11)                                                                  \
  CN_SPREAD_BOX(T, SUF, 12)                                                                  \
  CN_SPREAD_BOX(T, SUF, 13)                                                                  \
  CN_SPREAD_BOX(T, SUF, 14)                                                                  \
  CN_SPREAD_BOX(T, SUF, 15)                                                                  \
  CN_SPREAD_BOX(T, SUF, 16)

CN_ALL_NS(float, f)
CN_ALL_NS(double, d)

#define CN_CASES(F, SUF, ARGS)                                                               \
  switch (ns) {                                                                              \
  case 2: F##_##SUF##_2 ARGS; break;                                                         \
  case 3: F##_##SUF##_3 ARGS; break;                                                         \
  case 4: F##_##SUF##_4 ARGS; break;                                                         \
  case 5: F##_##SUF##_5 ARGS; break;                                                         \
  case 6: F##_##SUF##_6 ARGS; break;                                                         \
  case 7: F##_##SUF##_7 ARGS; break;                                                         \
  case 8: F##_##SUF##_8 ARGS; break;                                                         \
  case 9: F##_##SUF##_9 ARGS; break;                                                         \
  case 10: F##_##SUF##_10 ARGS; break;                                                       \
  case 11: F##_##SUF##_11 ARGS; break;                                                       \
  case 12: F##_##SUF##_12 ARGS; break;                                                       \
  case 13: F##_##SUF##_13 ARGS; break;                                                       \
  case 14: F##_##SUF##_14 ARGS; break;                                                       \
  case 15: F##_##SUF##_15 ARGS; break;                                                       \
  default: F##_##SUF##_16 ARGS; break;                                                       \
  }

#define CN_DRIVERS(T, SUF)                                                                   \
  /* grid (zeroed by the caller) += spread of c over the sorted points; the kernel is      \
   * ns Horner pieces of nc coefficients, coef[k*ns + j] (k = 0 highest degree) */          \
  void or_cpu_spread_##SUF(int dim, int64_t M, const T *const *xyz, const int32_t *perm,    \
                           const T *c, const int *nf, int ns, int nc, const double *coef,   \
                           int maxsub, T *grid) {                                            \
    if (M <= 0) return;                                                                      \
    T ct[CN_MAXNC * CN_MAXNS];                                                               \
    for (int i = 0; i < nc * ns; ++i) ct[i] = (T)coef[i];                                    \
    if (maxsub <= 0) maxsub = dim == 1 ? 10000 : 100000;                                     \
    int64_t nb = cn_threads();                                                               \
    if (nb > M) nb = M;                                                                      \
    if (nb * (int64_t)maxsub < M) nb = 1 + (M - 1) / maxsub;                                 \
    const int64_t n0 = nf[0], n1 = dim > 1 ? nf[1] : 1, n2 = dim > 2 ? nf[2] : 1;           \
    _Pragma("omp parallel for schedule(dynamic, 1)") for (int64_t sp = 0; sp < nb; ++sp) {  \
      const int64_t p0 = (M * sp + nb - 1) / nb, p1 = (M * (sp + 1) + nb - 1) / nb;          \
      if (p1 <= p0) continue;                                                                \
      /* local copies of the subproblem's points and strengths (the gathers through   \
       * perm are independent loads, overlapped by the core), and its bounding box */   \
      const int64_t n = p1 - p0;                                                             \
      T *loc = (T *)malloc((size_t)(dim + 2) * n * sizeof(T));                               \
      const T *lxyz[3] = {loc, loc + n, loc + 2 * n};                                        \
      T *lc = loc + dim * n;                                                                 \
      for (int64_t q = 0; q < n; ++q) {                                                      \
        const int64_t j = perm[p0 + q];                                                      \
        for (int d = 0; d < dim; ++d) loc[d * n + q] = xyz[d][j];                            \
        lc[2 * q] = c[2 * j];                                                                \
        lc[2 * q + 1] = c[2 * j + 1];                                                        \
      }                                                                                      \
      int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};                                              \
      for (int d = 0; d < dim; ++d) {                                                        \
        lo[d] = 1 << 30;                                                                     \
        hi[d] = -(1 << 30);                                                                  \
        for (int64_t q = 0; q < n; ++q) {                                                    \
          int i1;                                                                            \
          T t0;                                                                              \
          cn_place_##SUF(loc[d * n + q], nf[d], ns, &i1, &t0);                               \
          if (i1 < lo[d]) lo[d] = i1;                                                        \
          if (i1 > hi[d]) hi[d] = i1;                                                        \
        }                                                                                    \
      }                                                                                      \
      int64_t ext[3] = {1, 1, 1};                                                            \
      for (int d = 0; d < dim; ++d) ext[d] = hi[d] - lo[d] + ns;                             \
      T *box = (T *)calloc((size_t)(2 * ext[0] * ext[1] * ext[2]), sizeof(T));               \
      CN_CASES(cn_box, SUF, (dim, lxyz, lc, nf, nc, ct, n, lo, ext, box))                    \
      free(loc);                                                                             \
      for (int64_t bz = 0; bz < ext[2]; ++bz) {                                              \
        const int64_t gz = dim > 2 ? ((lo[2] + bz) % n2 + n2) % n2 : 0;                      \
        for (int64_t by = 0; by < ext[1]; ++by) {                                            \
          const int64_t gy = dim > 1 ? ((lo[1] + by) % n1 + n1) % n1 : 0;                    \
          const T *row = box + 2 * ext[0] * (by + ext[1] * bz);                              \
          T *grow = grid + 2 * n0 * (gy + n1 * gz);                                          \
          int64_t gx = ((lo[0]) % n0 + n0) % n0;                                             \
          for (int64_t bx = 0; bx < ext[0]; ++bx) {                                          \
            const T vr = row[2 * bx], vi = row[2 * bx + 1];                                  \
            if (vr != (T)0 || vi != (T)0) {                                                  \
              _Pragma("omp atomic") grow[2 * gx] += vr;                                      \
              _Pragma("omp atomic") grow[2 * gx + 1] += vi;                                  \
            }                                                                                \
            if (++gx == n0) gx = 0;                                                          \
          }                                                                                  \
        }                                                                                    \
      }                                                                                      \
      free(box);                                                                             \
    }                                                                                        \
  }                                                                                          \
  /* c[j] = interpolation of the periodic grid at the points (sorted traversal) */          \
  void or_cpu_interp_##SUF(int dim, int64_t M, const T *const *xyz, const int32_t *perm,    \
                           const T *grid, const int *nf, int ns, int nc, const double *coef, \
                           T *c) {                                                           \
    if (M <= 0) return;                                                                      \
    T ct[CN_MAXNC * CN_MAXNS];                                                               \
    for (int i = 0; i < nc * ns; ++i) ct[i] = (T)coef[i];                                    \
    const int64_t chunk = 4096, nchunk = (M + chunk - 1) / chunk;                            \
    _Pragma("omp parallel for schedule(dynamic, 4)") for (int64_t k = 0; k < nchunk; ++k) { \
      const int64_t p0 = k * chunk, p1 = p0 + chunk < M ? p0 + chunk : M;                    \
      CN_CASES(cn_interp, SUF, (dim, xyz, perm, grid, nf, nc, ct, p0, p1, c))                \
    }                                                                                        \
  }

CN_DRIVERS(float, f)
CN_DRIVERS(double, d)
