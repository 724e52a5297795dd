/* oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of flatironinstitute/finufft arithmetic, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * Nothing in the GB300 engine links, loads or calls this file.
 *
 * Contents (each function cites the reference code it follows):
 *   - FP64 direct NUDFTs of types 1, 2, 3 in 1D/2D/3D (test/utils/dirft1d.hpp,
 *     dirft2d.hpp, dirft3d.hpp), on all or a sampled subset of outputs;
 *   - planning math: next235, Gauss-Legendre nodes, GPU kernel width/beta,
 *     type-3 grid (src/common/utils.cpp, src/cuda/makeplan.cu:43-119,
 *     include/finufft_common/kernel.h:165-181);
 *   - the engine's FP64 fold-rescale and a stable counting sort by bin,
 *     the host replica the device permutation must match bit for bit;
 *   - spreading / interpolation with the ES kernel in FP64 (the GPU library's
 *     kernel, include/cufinufft/spreadinterp.hpp:29-39);
 *   - an OpenMP subproblem spreader/interpolator with a tabulated
 *     piecewise-polynomial kernel (the CPU library's design,
 *     include/finufft/spreadinterp.hpp:310-485, spread.hpp:53-451) used for
 *     the CPU FINUFFT restatement with its PSWF kernel.
 * Complex arrays are interleaved (re, im) doubles or floats.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.141592653589793238462643383279502884
#define OR_INV_2PI 0.159154943091895335768883763372514362

/* ------------------------------------------------------------ planning ---- */

static int smooth235(int64_t n) {
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  return n == 1;
}

/* next235(n, 2) of src/common/utils.cpp:117-121: 2*(smallest smooth m, 2m >= n) */
int64_t or_next235_even(int64_t n) {
  if (n < 1) n = 1;
  int64_t m = (n + 1) / 2;
  while (!smooth235(m)) ++m;
  return 2 * m;
}

/* n-node Gauss-Legendre nodes (ascending) and weights via Newton on the
 * three-term Legendre recurrence (src/common/utils.cpp:17-57). */
void or_gauss_legendre(int n, double *x, double *w) {
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = cos(OR_PI * (i + 0.75) / (n + 0.5)), p0 = 1, p1 = z, dp = 1;
    for (int it = 0; it < 100; ++it) {
      p0 = 1.0;
      p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    p0 = 1.0;
    p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = (n == 1) ? 1.0 : n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

/* GPU kernel width and beta (src/cuda/makeplan.cu:43-119), arithmetic in the
 * plan precision (is_float). Returns ns; beta in *beta. Error codes as the
 * reference: -8 Horner with nonstandard sigma, -7 sigma <= 1. */
int or_gpu_kernel(double tol, double sigma, int kerevalmeth, int is_float, double *beta) {
  if (sigma != 2.0 && sigma != 1.25) {
    if (kerevalmeth == 1) return -8;
    if (sigma <= 1.0) return -7;
  }
  int ns;
  if (is_float) {
    float eps = (float)tol, s = (float)sigma;
    if (eps < 1.1920929e-7f) eps = 1.1920929e-7f;
    ns = (int)ceilf(-log10f(eps / 10.0f));
    if (s != 2.0f) ns = (int)ceilf(-logf(eps) / ((float)OR_PI * sqrtf(1.0f - 1.0f / s)));
    if (ns < 2) ns = 2;
    if (ns > 12) ns = 12;
    float bon = 2.30f;
    if (ns == 2) bon = 2.20f;
    if (ns == 3) bon = 2.26f;
    if (ns == 4) bon = 2.38f;
    if (s != 2.0f) bon = 0.97f * (float)OR_PI * (1.0f - 1.0f / (2.0f * s));
    *beta = (double)(bon * (float)ns);
  } else {
    double eps = tol;
    if (eps < 2.220446049250313e-16) eps = 2.220446049250313e-16;
    ns = (int)ceil(-log10(eps / 10.0));
    if (sigma != 2.0) ns = (int)ceil(-log(eps) / (OR_PI * sqrt(1.0 - 1.0 / sigma)));
    if (ns < 2) ns = 2;
    if (ns > 16) ns = 16;
    double bon = 2.30;
    if (ns == 2) bon = 2.20;
    if (ns == 3) bon = 2.26;
    if (ns == 4) bon = 2.38;
    if (sigma != 2.0) bon = 0.97 * OR_PI * (1.0 - 1.0 / (2.0 * sigma));
    *beta = bon * ns;
  }
  return ns;
}

/* type 1/2 fine grid (src/cuda/fft.cu:166-179) */
int64_t or_fine_grid(int64_t ms, double sigma, int ns) {
  int64_t nf = (int64_t)ceil(sigma * (double)ms);
  if (nf < 2 * ns) nf = 2 * ns;
  if (nf < 2147483647LL) nf = or_next235_even(nf);
  return nf;
}

/* type-3 grid (include/finufft_common/kernel.h:165-181): out = {nf, h, gam} */
void or_type3_grid(double sigma, double X, double S, int ns, double *out) {
  double Xs = X, Ss = S;
  if (Xs == 0.0) {
    if (Ss == 0.0) Xs = Ss = 1.0;
    else Xs = 1.0 / Ss;
  } else if (Ss < 1.0 / Xs)
    Ss = 1.0 / Xs;
  double nfd = 2.0 * sigma * Ss * Xs / OR_PI + (ns + 1);
  if (!isfinite(nfd)) nfd = 0.0;
  int64_t nf = (int64_t)nfd;
  if (nf < 2 * ns) nf = 2 * ns;
  if (nf < 2147483647LL) nf = or_next235_even(nf);
  out[0] = (double)nf;
  out[1] = 2.0 * OR_PI / (double)nf;
  out[2] = (double)nf / (2.0 * sigma * Ss);
}

double or_es_kernel(double x, int ns, double beta) {
  double z = 2.0 * x / ns;
  if (fabs(z) >= 1.0) return 0.0;
  return exp(beta * (sqrt(1.0 - z * z) - 1.0));
}

/* --------------------------------------------------- fold and bin sort ---- */

/* The engine's fold: y = (x - shift)*scale, r = frac(y/2pi + 1/2)*nf in FP64
 * with round-to-nearest steps (compile with -ffp-contract=off), NaN -> 0,
 * cell = floor(r) wrapped, frac = r - floor(r). */
void or_fold_cell(double x, double shift, double scale, int nf, int *cell, double *frac) {
  double y = (x - shift) * scale;
  double r = fma(y, OR_INV_2PI, 0.5);
  r = r - floor(r);
  r = r * (double)nf;
  if (!(r >= 0.0 && r <= (double)nf)) r = 0.0;
  double fl = floor(r);
  int c = (int)fl;
  if (c >= nf) c -= nf;
  *cell = c;
  *frac = r - fl;
}

/* The engine's single-precision fold for float coordinates on the identity
 * map (shift 0, scale 1, nf < 2^20): x/2pi + 1/2 as an unevaluated float sum
 * (error-free product by fmaf, two-sum), its fraction times nf as another,
 * then the integer part of the fraction moved into the cell; NaN/Inf -> cell 0. Every
 * step is a float operation rounded to nearest (-ffp-contract=off). */
void or_fold_cell_f32(float x, int nf, int *cell, float *frac) {
  const float c_hi = (float)OR_INV_2PI;
  const float c_lo = (float)(OR_INV_2PI - (double)c_hi);
  const float nff = (float)nf;
  if (!(x - x == 0.f)) { /* NaN or Inf */
    *cell = 0;
    *frac = 0.f;
    return;
  }
  const float ph = x * c_hi;
  const float pl = fmaf(x, c_lo, fmaf(x, c_hi, -ph));
  const float s = ph + 0.5f;
  const float bb = s - ph;
  const float lo = ((ph - (s - bb)) + (0.5f - bb)) + pl;
  /* fraction of s as an exact two-sum, then times nf */
  const float fls = -floorf(s);
  const float fh = s + fls;
  const float fb = fh - s;
  const float fl = (s - (fh - fb)) + (fls - fb);
  const float gh = fh * nff;
  const float gl = fmaf(fl + lo, nff, fmaf(fh, nff, -gh));
  float c = floorf(gh);
  float fr = (gh - c) + gl;
  const float k = floorf(fr); /* fr in (-2, 3) */
  c = c + k;
  fr = fr - k;
  if (fr >= 1.f) { /* a tiny negative fraction plus one rounded to 1 */
    c = c + 1.f;
    fr = 0.f;
  }
  int ci = (int)c;
  if (ci < 0) ci += nf;
  else if (ci >= nf) ci -= nf;
  *cell = ci;
  *frac = fr;
}

/* both folds over an array of float coordinates (accuracy checks):
 * grid position cell + frac of each */
void or_fold_many(int64_t n, const float *x, int nf, int f32, int *cell, double *frac) {
  for (int64_t i = 0; i < n; ++i) {
    if (f32) {
      float f;
      or_fold_cell_f32(x[i], nf, &cell[i], &f);
      frac[i] = f;
    } else {
      or_fold_cell((double)x[i], 0.0, 1.0, nf, &cell[i], &frac[i]);
    }
  }
}

/* one axis of a point: cell, and the bin-local coordinate in double (FP64
 * fold) or as the float the single-precision path stores */
static void or_axis(double x, double shift, double scale, int nf, int bin, int f32, int *cell,
                    double *local, double *frac) {
  if (f32) {
    float f;
    or_fold_cell_f32((float)x, nf, cell, &f);
    *local = (double)((float)(*cell % bin) + f);
    *frac = f;
  } else {
    double f;
    or_fold_cell(x, shift, scale, nf, cell, &f);
    *local = (double)(*cell - (*cell / bin) * bin) + f;
    *frac = f;
  }
}

/* Stable counting sort of the points, as the CPU library's bin sort
 * (include/finufft/spread.hpp:459-584: bins x fastest, input order kept inside
 * a key) with the engine's fold and integer bins. The key is the bin, times the
 * bin volume plus the cell inside the bin (x fastest) whenever
 * bins * bin volume fits 32 bits -- the engine's device key.
 * coords: dim arrays of doubles (float inputs converted exactly). Outputs
 * perm[M] and loc[dim*M] (bin-local coordinates, rounded to float when
 * loc_is_float; with float_inputs (coordinates given as floats) and the
 * identity map they take the single-precision fold, as the engine's device
 * sort does for float plans). Returns 0. */
int or_bin_sort(int dim, int64_t M, const double *const *coords, const double *shift,
                const double *scale, const int *nf, const int *bin, int32_t *perm,
                void *loc, int loc_is_float, int float_inputs, int ns, int bin_only) {
  int nb[3] = {1, 1, 1};
  int bn[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) {
    nb[d] = (nf[d] + bin[d] - 1) / bin[d];
    bn[d] = bin[d];
  }
  const uint64_t nbins = (uint64_t)nb[0] * nb[1] * nb[2];
  uint64_t binvol = (uint64_t)bn[0] * bn[1] * bn[2];
  /* bin_only: the reference's ordering, bin index (x fastest) and input order
   * within a bin (include/cufinufft/spreadinterp.hpp:139-150,
   * include/finufft/spread.hpp:459-584) */
  const int cell_keys = !bin_only && nbins * binvol <= 0xffffffffull;
  /* odd kernel widths: start-cell keys (cell + 1 when the fraction is at
   * least one half, so bin + 1 values per dimension) when they still fit 32
   * bits, as the engine's sort */
  uint64_t sbinvol = 1;
  for (int d = 0; d < dim; ++d) sbinvol *= (uint64_t)bin[d] + 1;
  const int half = cell_keys && ns % 2 == 1 && nbins * sbinvol <= 0xffffffffull;
  const uint32_t ex = half ? 1u : 0u;
  if (half) binvol = sbinvol;
  const uint64_t nkeys = cell_keys ? nbins * binvol : nbins;
  int f32 = loc_is_float && float_inputs;
  for (int d = 0; d < dim; ++d)
    f32 = f32 && shift[d] == 0.0 && scale[d] == 1.0 && nf[d] < (1 << 20);
  int64_t *cnt = (int64_t *)calloc((size_t)nkeys + 1, sizeof(int64_t));
  uint32_t *key = (uint32_t *)malloc((size_t)(M > 0 ? M : 1) * sizeof(uint32_t));
  for (int64_t i = 0; i < M; ++i) {
    uint32_t k = 0, stride = 1, lc = 0, lstride = 1;
    for (int d = 0; d < dim; ++d) {
      int c;
      double l, fr;
      or_axis(coords[d][i], shift[d], scale[d], nf[d], bin[d], f32, &c, &l, &fr);
      k += stride * (uint32_t)(c / bin[d]);
      const uint32_t cm = (uint32_t)(c - (c / bin[d]) * bin[d]);
      lc += lstride * (cm + (half && fr >= 0.5 ? 1u : 0u));
      stride *= (uint32_t)nb[d];
      lstride *= (uint32_t)bin[d] + ex;
    }
    key[i] = cell_keys ? k * (uint32_t)binvol + lc : k;
    cnt[key[i] + 1]++;
  }
  for (uint64_t b = 0; b < nkeys; ++b) cnt[b + 1] += cnt[b];
  for (int64_t i = 0; i < M; ++i) perm[cnt[key[i]]++] = (int32_t)i;
  for (int64_t p = 0; p < M; ++p) {
    int64_t i = perm[p];
    for (int d = 0; d < dim; ++d) {
      int c;
      double l, fr;
      or_axis(coords[d][i], shift[d], scale[d], nf[d], bin[d], f32, &c, &l, &fr);
      if (loc_is_float) ((float *)loc)[(size_t)d * M + p] = (float)l;
      else ((double *)loc)[(size_t)d * M + p] = l;
    }
  }
  free(cnt);
  free(key);
  return 0;
}

/* ------------------------------------------------------- direct sums ---- */

/* mode index of CMCL-ordered position i along an axis of length n */
static inline int64_t or_mode(int64_t i, int64_t n) { return i - n / 2; }

/* Type 1 (test/utils/dirft*d.hpp): f[k] = sum_j c[j] exp(i isign k.x_j) at the
 * modes with flat CMCL positions kidx[0..nk) (x fastest); kidx NULL = all modes. */
void or_dirft1(int dim, int64_t M, const double *const *xyz, const double *c, int isign,
               const int64_t *nm, int64_t nk, const int64_t *kidx, double *out) {
  const double sg = isign >= 0 ? 1.0 : -1.0;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < nk; ++q) {
    int64_t flat = kidx ? kidx[q] : q;
    double k[3] = {0, 0, 0};
    k[0] = (double)or_mode(flat % nm[0], nm[0]);
    if (dim > 1) k[1] = (double)or_mode((flat / nm[0]) % nm[1], nm[1]);
    if (dim > 2) k[2] = (double)or_mode(flat / (nm[0] * nm[1]), nm[2]);
    double sr = 0, si = 0;
    for (int64_t j = 0; j < M; ++j) {
      double ph = k[0] * xyz[0][j];
      if (dim > 1) ph += k[1] * xyz[1][j];
      if (dim > 2) ph += k[2] * xyz[2][j];
      double cs = cos(ph), sn = sg * sin(ph);
      sr += c[2 * j] * cs - c[2 * j + 1] * sn;
      si += c[2 * j] * sn + c[2 * j + 1] * cs;
    }
    out[2 * q] = sr;
    out[2 * q + 1] = si;
  }
}

/* Type 2: c[j] = sum_k f[k] exp(i isign k.x_j) for the points jidx[0..nj)
 * (NULL = all M); f has all modes in CMCL order. */
void or_dirft2(int dim, int64_t M, const double *const *xyz, int isign, const int64_t *nm,
               const double *f, int64_t nj, const int64_t *jidx, double *out) {
  const double sg = isign >= 0 ? 1.0 : -1.0;
  const int64_t ntot = nm[0] * (dim > 1 ? nm[1] : 1) * (dim > 2 ? nm[2] : 1);
  (void)M;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t q = 0; q < nj; ++q) {
    int64_t j = jidx ? jidx[q] : q;
    double sr = 0, si = 0;
    for (int64_t flat = 0; flat < ntot; ++flat) {
      double ph = (double)or_mode(flat % nm[0], nm[0]) * xyz[0][j];
      if (dim > 1) ph += (double)or_mode((flat / nm[0]) % nm[1], nm[1]) * xyz[1][j];
      if (dim > 2) ph += (double)or_mode(flat / (nm[0] * nm[1]), nm[2]) * xyz[2][j];
      double cs = cos(ph), sn = sg * sin(ph);
      sr += f[2 * flat] * cs - f[2 * flat + 1] * sn;
      si += f[2 * flat] * sn + f[2 * flat + 1] * cs;
    }
    out[2 * q] = sr;
    out[2 * q + 1] = si;
  }
}

/* Type 3: f[k] = sum_j c[j] exp(i isign s_k.x_j) for targets kidx[0..nk) (NULL = all). */
void or_dirft3(int dim, int64_t M, const double *const *xyz, const double *c, int isign,
               const double *const *stu, int64_t nk, const int64_t *kidx, double *out) {
  const double sg = isign >= 0 ? 1.0 : -1.0;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < nk; ++q) {
    int64_t k = kidx ? kidx[q] : q;
    double sr = 0, si = 0;
    for (int64_t j = 0; j < M; ++j) {
      double ph = stu[0][k] * xyz[0][j];
      if (dim > 1) ph += stu[1][k] * xyz[1][j];
      if (dim > 2) ph += stu[2][k] * xyz[2][j];
      double cs = cos(ph), sn = sg * sin(ph);
      sr += c[2 * j] * cs - c[2 * j + 1] * sn;
      si += c[2 * j] * sn + c[2 * j + 1] * cs;
    }
    out[2 * q] = sr;
    out[2 * q + 1] = si;
  }
}

/* ------------------------------------- GPU-rule spread / interp (FP64) ---- */

/* Grid weights of one point along one axis with the ES kernel (or a tabulated
 * kernel, coef != NULL): first cell
 * (wrapped into [0,nf)) and ns kernel values, as the GPU library places a point
 * (include/cufinufft/spreadinterp.hpp:166-196) but from the engine's FP64 fold. */
static void or_axis_es(double x, double shift, double scale, int nf, int ns, double beta,
                       int ncoef, const double *coef, int *start, double *ker) {
  int c;
  double f;
  or_fold_cell(x, shift, scale, nf, &c, &f);
  double r = (double)c + f;
  double s = ceil(r - 0.5 * ns);
  if (coef) {
    /* tabulated kernel (the PSWF): piece j of the support holds cell j, all at
     * the same local variable u = 2 (s - r + ns/2) - 1; coef[k*ns + j] is the
     * coefficient of u^(ncoef-1-k) of piece j */
    const double u = 2.0 * (s - r + 0.5 * ns) - 1.0;
    for (int j = 0; j < ns; ++j) {
      double v = 0.0;
      for (int k = 0; k < ncoef; ++k) v = v * u + coef[k * ns + j];
      ker[j] = v;
    }
  } else
    for (int j = 0; j < ns; ++j) ker[j] = or_es_kernel(s - r + j, ns, beta);
  int st = (int)s % nf;
  if (st < 0) st += nf;
  *start = st;
}

/* grid[g] += sum_j c_j phi(g - r_j) over the periodic grid nf[0..dim) (x fastest). */
void or_spread_es(int dim, int64_t M, const double *const *xyz, const double *shift,
                  const double *scale, const double *c, const int *nf, int ns, double beta,
                  int ncoef, const double *coef, double *grid) {
  double ker[3][32];
  int st[3] = {0, 0, 0};
  const int n1 = dim > 1 ? ns : 1, n2 = dim > 2 ? ns : 1;
  for (int64_t j = 0; j < M; ++j) {
    for (int d = 0; d < dim; ++d)
      or_axis_es(xyz[d][j], shift[d], scale[d], nf[d], ns, beta, ncoef, coef, &st[d], ker[d]);
    for (int cz = 0; cz < n2; ++cz) {
      int64_t gz = dim > 2 ? (st[2] + cz) % nf[2] : 0;
      double wz = dim > 2 ? ker[2][cz] : 1.0;
      for (int cy = 0; cy < n1; ++cy) {
        int64_t gy = dim > 1 ? (st[1] + cy) % nf[1] : 0;
        double wy = wz * (dim > 1 ? ker[1][cy] : 1.0);
        for (int cx = 0; cx < ns; ++cx) {
          int64_t gx = (st[0] + cx) % nf[0];
          int64_t g = gx + (int64_t)nf[0] * (gy + (int64_t)(dim > 1 ? nf[1] : 1) * gz);
          double w = wy * ker[0][cx];
          grid[2 * g] += w * c[2 * j];
          grid[2 * g + 1] += w * c[2 * j + 1];
        }
      }
    }
  }
}

/* c[j] = sum_g grid[g] phi(g - r_j) */
void or_interp_es(int dim, int64_t M, const double *const *xyz, const double *shift,
                  const double *scale, const double *grid, const int *nf, int ns, double beta,
                  int ncoef, const double *coef, double *c) {
  const int n1 = dim > 1 ? ns : 1, n2 = dim > 2 ? ns : 1;
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < M; ++j) {
    double ker[3][32];
    int st[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d)
      or_axis_es(xyz[d][j], shift[d], scale[d], nf[d], ns, beta, ncoef, coef, &st[d], ker[d]);
    double sr = 0, si = 0;
    for (int cz = 0; cz < n2; ++cz) {
      int64_t gz = dim > 2 ? (st[2] + cz) % nf[2] : 0;
      double wz = dim > 2 ? ker[2][cz] : 1.0;
      for (int cy = 0; cy < n1; ++cy) {
        int64_t gy = dim > 1 ? (st[1] + cy) % nf[1] : 0;
        double wy = wz * (dim > 1 ? ker[1][cy] : 1.0);
        for (int cx = 0; cx < ns; ++cx) {
          int64_t gx = (st[0] + cx) % nf[0];
          int64_t g = gx + (int64_t)nf[0] * (gy + (int64_t)(dim > 1 ? nf[1] : 1) * gz);
          double w = wy * ker[0][cx];
          sr += w * grid[2 * g];
          si += w * grid[2 * g + 1];
        }
      }
    }
    c[2 * j] = sr;
    c[2 * j + 1] = si;
  }
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
