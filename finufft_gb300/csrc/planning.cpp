// Host-side planning math for the GB300 NUFFT engine.
//
// Each function states the reference behaviour it reproduces (file:line in
// flatironinstitute/finufft). The code is written from the mathematics: the
// rules (kernel width per tolerance, grid sizes) must agree with the reference
// so that plans built here have the same accuracy contract.
#include "planning.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>

#include "common.h"

namespace gbn {

namespace {
// true when n has no prime factor other than 2, 3, 5
bool smooth235(int64_t n) {
  for (int p : {2, 3, 5})
    while (n % p == 0) n /= p;
  return n == 1;
}
} // namespace

int64_t next235_even(int64_t n)
// Same value as FINUFFT next235(n, 2) (src/common/utils.cpp:117-121):
// 2 * (smallest 2,3,5-smooth m with 2m >= n), n clamped to >= 1.
{
  if (n < 1) n = 1;
  int64_t m = (n + 1) / 2;
  while (!smooth235(m)) ++m;
  return 2 * m;
}

void gauss_legendre(int n, double *x, double *w)
// Gauss-Legendre nodes by Newton's method on P_n from Chebyshev-point guesses,
// weights w_i = 2 / ((1-x_i^2) P_n'(x_i)^2). Nodes ascending, as in
// src/common/utils.cpp:17-57 (gaussquad).
{
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) {
        p1 = z;
        p0 = 1.0;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    // recompute derivative at the converged node
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = (n == 1) ? 1.0 : n * (z * p1 - p0) / (z * z - 1.0);
    double wi = 2.0 / ((1.0 - z * z) * dp * dp);
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = wi;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

double es_kernel(double x, int ns, double beta) {
  double z = 2.0 * x / ns;
  if (std::fabs(z) >= 1.0) return 0.0;
  return std::exp(beta * (std::sqrt(1.0 - z * z) - 1.0));
}

namespace {
// Legendre coefficients of the prolate spheroidal wave function psi_0^c on
// [-1, 1] (Bouwkamp's expansion; Xiao, Rokhlin & Yarvin, Inverse Problems 17
// (2001) 805-838): in the basis of normalised even Legendre polynomials
// sqrt(n + 1/2) P_n, n = 2k, the prolate operator
// -d/dz (1 - z^2) d/dz + c^2 z^2 is symmetric tridiagonal, and psi_0 is the
// eigenvector of its smallest eigenvalue. That eigenvalue is bracketed by
// bisection on the Sturm sequence count; the eigenvector comes from inverse
// iteration with the shift just below it, where the shifted matrix is
// positive definite and the LDL^T recurrence needs no pivoting. Returns a[k],
// the coefficient of P_{2k} (unnormalised: psi(z) = sum_k a[k] P_{2k}(z)).
std::vector<double> pswf0_legendre(double c) {
  const int K = (int)c + 40; // the coefficients decay super-exponentially past k ~ c/2
  std::vector<double> d(K), e(K > 1 ? K - 1 : 1, 0.0);
  for (int k = 0; k < K; ++k) {
    const double n = 2.0 * k;
    d[k] = n * (n + 1) + c * c * (2 * n * n + 2 * n - 1) / ((2 * n - 1) * (2 * n + 3));
  }
  for (int k = 0; k + 1 < K; ++k) {
    const double n = 2.0 * k;
    e[k] = c * c * (n + 1) * (n + 2) / ((2 * n + 3) * std::sqrt((2 * n + 1) * (2 * n + 5)));
  }
  // Gershgorin bounds of the smallest eigenvalue
  double lo = d[0] - std::fabs(e[0]), hi = d[0] + std::fabs(e[0]);
  for (int k = 1; k < K; ++k) {
    const double r = std::fabs(e[k - 1]) + (k + 1 < K ? std::fabs(e[k]) : 0.0);
    lo = std::min(lo, d[k] - r);
  }
  // number of eigenvalues below x (Sturm count of the LDL^T pivots of T - x)
  auto below = [&](double x) {
    int cnt = 0;
    double q = d[0] - x;
    if (q < 0) ++cnt;
    for (int k = 1; k < K; ++k) {
      if (q == 0.0) q = 1e-300;
      q = d[k] - x - e[k - 1] * e[k - 1] / q;
      if (q < 0) ++cnt;
    }
    return cnt;
  };
  for (int it = 0; it < 200 && hi - lo > 4e-16 * std::max(1.0, std::fabs(hi)); ++it) {
    const double mid = 0.5 * (lo + hi);
    if (below(mid) >= 1) hi = mid;
    else lo = mid;
  }
  // inverse iteration on T - sh, the shift a hair below the bracket (so below
  // the eigenvalue whatever the rounding of the Sturm counts: T - sh is
  // positive definite and its LDL^T pivots are positive)
  const double sh = lo - 1e-9 * std::max(1.0, std::fabs(lo));
  auto safe = [](double p) { return std::fabs(p) < 1e-300 ? (p < 0 ? -1e-300 : 1e-300) : p; };
  std::vector<double> v(K, 1.0), piv(K), w(K);
  for (int it = 0; it < 4; ++it) {
    piv[0] = safe(d[0] - sh);
    w[0] = v[0];
    for (int k = 1; k < K; ++k) {
      const double l = e[k - 1] / piv[k - 1];
      piv[k] = safe(d[k] - sh - l * e[k - 1]);
      w[k] = v[k] - l * w[k - 1];
    }
    v[K - 1] = w[K - 1] / piv[K - 1];
    for (int k = K - 2; k >= 0; --k) v[k] = (w[k] - e[k] * v[k + 1]) / piv[k];
    double nrm = 0;
    for (double t : v) nrm += t * t;
    nrm = std::sqrt(nrm);
    for (double &t : v) t /= nrm;
  }
  for (int k = 0; k < K; ++k) v[k] *= std::sqrt(2.0 * k + 0.5);
  return v;
}

// sum_k a[k] P_{2k}(z) by the three-term Legendre recurrence
double legendre_even_sum(const std::vector<double> &a, double z) {
  double p0 = 1.0, p1 = z, s = a[0];
  const int nmax = 2 * ((int)a.size() - 1);
  for (int n = 1; n < nmax; ++n) {
    const double p2 = ((2.0 * n + 1.0) * z * p1 - n * p0) / (n + 1.0);
    p0 = p1;
    p1 = p2;
    if ((n + 1) % 2 == 0) s += a[(n + 1) / 2] * p1;
  }
  return s;
}
} // namespace

KernelFn make_kernel_fn(int form, int ns, double beta) {
  KernelFn f;
  f.form = form;
  f.ns = ns;
  f.beta = beta;
  if (form == KERNEL_PSWF) {
    f.leg = pswf0_legendre(beta);
    f.scale = 1.0 / legendre_even_sum(f.leg, 0.0);
  }
  return f;
}

double KernelFn::operator()(double x) const {
  if (form != KERNEL_PSWF) return es_kernel(x, ns, beta);
  const double z = 2.0 * x / ns;
  if (std::fabs(z) > 1.0) return 0.0;
  return scale * legendre_even_sum(leg, z);
}

KernelChoice choose_kernel(double tol, double sigma, int kerevalmeth, int is_float,
                           int spreadinterponly, int debug)
// GPU kernel-shape rule of src/cuda/makeplan.cu:43-119 (setup_spreadinterp):
// ns = ceil(-log10(tol/10)) at sigma=2, else ceil(-ln(tol)/(pi sqrt(1-1/sigma)));
// clipped to [2, 12 (float) | 16 (double)]; beta = (2.30, or small-ns tweaks, or
// 0.97 pi (1-1/(2 sigma)) off sigma=2) * ns. The arithmetic runs in the plan's
// precision so the chosen width agrees with the reference's.
{
  if (sigma != 2.0 && sigma != 1.25) {
    if (kerevalmeth == 1) {
      fprintf(stderr,
              "[gbnufft] error: upsampfac=%.3g needs gpu_kerevalmeth=0 (Horner tables only "
              "for 2.0 and 1.25)\n",
              sigma);
      GBN_THROW(FINUFFT_ERR_HORNER_WRONG_BETA, "kerevalmeth=1 needs sigma 2 or 1.25");
    }
    if (sigma <= 1.0) {
      fprintf(stderr, "[gbnufft] error: upsampfac=%.3g <= 1\n", sigma);
      GBN_THROW(FINUFFT_ERR_UPSAMPFAC_TOO_SMALL, "upsampfac too small");
    }
    if (!spreadinterponly && sigma > 4.0)
      fprintf(stderr, "[gbnufft] warning: upsampfac=%.3g is too large to be beneficial\n",
              sigma);
  }
  const int maxns = is_float ? MAX_NS_FLOAT : MAX_NS;
  int ns;
  double beta;
  if (is_float) {
    float eps = (float)tol;
    if (eps < FLT_EPSILON) {
      fprintf(stderr, "[gbnufft] warning: increasing tol=%.3g to eps_mach=%.3g\n", tol,
              (double)FLT_EPSILON);
      eps = FLT_EPSILON;
    }
    const float s = (float)sigma;
    ns = (int)std::ceil(-std::log10(eps / 10.0f));
    if (s != 2.0f) ns = (int)std::ceil(-std::log(eps) / ((float)PI * std::sqrt(1.0f - 1.0f / s)));
    ns = std::max(2, ns);
    if (ns > maxns) {
      fprintf(stderr, "[gbnufft] warning: tol=%.3g needs ns=%d at sigma=%.3g; clipping to %d\n",
              tol, ns, sigma, maxns);
      ns = maxns;
    }
    float bon = 2.30f;
    if (ns == 2) bon = 2.20f;
    if (ns == 3) bon = 2.26f;
    if (ns == 4) bon = 2.38f;
    if (s != 2.0f) bon = 0.97f * (float)PI * (1.0f - 1.0f / (2.0f * s));
    beta = (double)(bon * (float)ns);
  } else {
    double eps = tol;
    if (eps < DBL_EPSILON) {
      fprintf(stderr, "[gbnufft] warning: increasing tol=%.3g to eps_mach=%.3g\n", tol,
              DBL_EPSILON);
      eps = DBL_EPSILON;
    }
    ns = (int)std::ceil(-std::log10(eps / 10.0));
    if (sigma != 2.0) ns = (int)std::ceil(-std::log(eps) / (PI * std::sqrt(1.0 - 1.0 / sigma)));
    ns = std::max(2, ns);
    if (ns > maxns) {
      fprintf(stderr, "[gbnufft] warning: tol=%.3g needs ns=%d at sigma=%.3g; clipping to %d\n",
              tol, ns, sigma, maxns);
      ns = maxns;
    }
    double bon = 2.30;
    if (ns == 2) bon = 2.20;
    if (ns == 3) bon = 2.26;
    if (ns == 4) bon = 2.38;
    if (sigma != 2.0) bon = 0.97 * PI * (1.0 - 1.0 / (2.0 * sigma));
    beta = bon * ns;
  }
  if (debug)
    printf("[gbnufft] tol=%.3g sigma=%.3g: ns=%d beta=%.4g\n", tol, sigma, ns, beta);
  return {ns, beta};
}

KernelChoice choose_kernel_pswf(double tol, double sigma, int dim, int type, int is_float,
                                int kerformula, int kerevalmeth, int spreadinterponly,
                                int debug)
// The CPU library's kernel (src/common/kernel.cpp:79-146): the PSWF psi_0^beta
// with the width law ns = ceil(ln(tolfac/tol) / (pi sqrt(1 - 1/sigma)) + 1),
// tolfac = 0.18 * 1.4^(dim-1) * (1.4 for type 3), and the shape parameter of
// kerformula 8 (the default; beta = pi ns (1 - 1/(2 sigma)) - 0.05), 7 (Beatty)
// or 9 (least-squares fit in t = beta_cutoff / pi). The width is the larger of
// that law and the GPU library's rule above, so the kernel is never narrower
// than the reference GPU's at the same tolerance; clipped as above.
{
  if (kerformula != 0 && (kerformula < 7 || kerformula > 9)) {
    fprintf(stderr, "[gbnufft] error: kerformula=%d is not a PSWF shape choice (0, 7, 8, 9)\n",
            kerformula);
    GBN_THROW(FINUFFT_ERR_KERFORMULA_NOTVALID, "kerformula");
  }
  // argument checks (with kerevalmeth 1 the GPU interface's: Horner evaluation
  // at sigma 2 and 1.25 only) and the GPU width rule
  const KernelChoice g = choose_kernel(tol, sigma, kerevalmeth, is_float, spreadinterponly, 0);
  const double eps_mach = is_float ? (double)FLT_EPSILON : DBL_EPSILON;
  const double t = std::max(tol, eps_mach);
  const double tolfac = 0.18 * std::pow(1.4, dim - 1) * (type == 3 ? 1.4 : 1.0);
  int ns = (int)std::ceil(std::log(tolfac / t) / (PI * std::sqrt(1.0 - 1.0 / sigma)) + 1.0);
  ns = std::max(ns, g.ns);
  ns = std::max(2, std::min(ns, is_float ? MAX_NS_FLOAT : MAX_NS));
  const double cut = PI * ns * (1.0 - 1.0 / (2.0 * sigma));
  double beta = cut - 0.05;
  if (kerformula == 7) {
    const double cb = ns == 2 ? 0.5 : 0.8;
    beta = std::sqrt(cut * cut - cb / (PI * PI));
  } else if (kerformula == 9) {
    const double tt = cut / PI;
    beta = ((-0.00149087 * tt + 0.0218459) * tt + 3.06269) * tt - 0.0365245;
  }
  if (debug)
    printf("[gbnufft] PSWF kernel: tol=%.3g sigma=%.3g: ns=%d beta=%.4g\n", tol, sigma, ns,
           beta);
  return {ns, beta};
}

int64_t ladder_grid_len(int64_t n) {
  int64_t best = 0;
  for (int64_t p2 = 8; best == 0 || p2 <= best; p2 *= 2) {
    for (const int64_t v : {p2, p2 * 5 / 4, p2 * 3 / 2, p2 * 15 / 8})
      if (v % 2 == 0 && v >= n && (best == 0 || v < best)) best = v;
    if (p2 > (int64_t)1 << 40) break;
  }
  return best;
}

int64_t fine_grid_len(int64_t ms, double sigma, int ns)
// src/cuda/fft.cu:166-179 (set_nf_type12): ceil(sigma*ms), at least 2*ns, then
// rounded up to an even 2,3,5-smooth length.
{
  int64_t nf = (int64_t)std::ceil(sigma * (double)ms);
  if (nf < 2 * ns) nf = 2 * ns;
  if (nf < (int64_t)std::numeric_limits<int32_t>::max()) nf = next235_even(nf);
  return nf;
}

void type3_grid(double sigma, double X, double S, int ns, int64_t *nf, double *h,
                double *gam)
// Type-3 fine grid of include/finufft_common/kernel.h:165-181 (nhg_type3):
// make X*S >= 1, nf = 2 sigma S X / pi + ns + 1 (at least 2 ns, then 2,3,5-smooth),
// h = 2 pi / nf, gamma = nf / (2 sigma S).
{
  double Xs = X, Ss = S;
  if (Xs == 0.0) {
    if (Ss == 0.0)
      Xs = Ss = 1.0;
    else
      Xs = 1.0 / Ss;
  } else
    Ss = std::max(Ss, 1.0 / Xs);
  double nfd = 2.0 * sigma * Ss * Xs / PI + (ns + 1);
  if (!std::isfinite(nfd)) nfd = 0.0;
  int64_t n = std::max((int64_t)nfd, (int64_t)(2 * ns));
  if (n < (int64_t)std::numeric_limits<int32_t>::max()) n = next235_even(n);
  *nf = n;
  *h = 2.0 * PI / (double)n;
  *gam = (double)n / (2.0 * sigma * Ss);
}

void width_center(double lo, double hi, double *w, double *c)
// include/cufinufft/utils.hpp:119-130 (arraywidcen): centre only if that shrinks
// the half-width by more than 10% of it.
{
  double ww = (hi - lo) / 2, cc = (hi + lo) / 2;
  if (std::fabs(cc) < 0.1 * ww) {
    ww += std::fabs(cc);
    cc = 0.0;
  }
  *w = ww;
  *c = cc;
}

int horner_fit(const KernelFn &phi, double target_err, int maxcoef, std::vector<double> &coef,
               double *maxerr_out)
// Piecewise polynomial of the kernel phi: piece j of ns covers
// x in [-ns/2 + j, -ns/2 + j + 1]; it is the Chebyshev interpolant of degree
// d-1 at d first-kind points in u = 2(x - start) - 1, rewritten in monomials of u.
// The degree grows until the sampled max error is below target_err.
{
  const int nsample = 64;
  const int ns = phi.ns;
  maxcoef = std::min(maxcoef, MAX_HCOEF);
  int d = std::min(maxcoef, ns + 2);
  for (;; ++d) {
    coef.assign((size_t)MAX_HCOEF * MAX_NS, 0.0);
    double maxerr = 0.0;
    for (int j = 0; j < ns; ++j) {
      auto xof = [&](double u) { return -ns / 2.0 + j + (u + 1.0) / 2.0; };
      // Chebyshev coefficients a_m of the interpolant at d points
      std::vector<long double> a(d, 0.0L), fv(d);
      for (int i = 0; i < d; ++i) {
        long double th = (long double)PI * (i + 0.5L) / d;
        fv[i] = phi(xof((double)cosl(th)));
      }
      for (int m = 0; m < d; ++m) {
        long double s = 0;
        for (int i = 0; i < d; ++i) s += fv[i] * cosl((long double)PI * m * (i + 0.5L) / d);
        a[m] = s * (m == 0 ? 1.0L : 2.0L) / d;
      }
      // monomial coefficients: sum_m a_m T_m(u), T_m via T_{m+1} = 2u T_m - T_{m-1}
      std::vector<long double> mono(d, 0.0L), tprev(d, 0.0L), tcur(d, 0.0L), tnext(d, 0.0L);
      tprev[0] = 1.0L;           // T_0
      if (d > 1) tcur[1] = 1.0L; // T_1
      mono[0] += a[0];
      for (int m = 1; m < d; ++m) {
        for (int k = 0; k < d; ++k) mono[k] += a[m] * tcur[k];
        std::fill(tnext.begin(), tnext.end(), 0.0L);
        for (int k = 0; k + 1 < d; ++k) tnext[k + 1] += 2.0L * tcur[k];
        for (int k = 0; k < d; ++k) tnext[k] -= tprev[k];
        tprev = tcur;
        tcur = tnext;
      }
      for (int k = 0; k < d; ++k) coef[(size_t)k * MAX_NS + j] = (double)mono[d - 1 - k];
      for (int t = 0; t <= nsample; ++t) {
        double u = -1.0 + 2.0 * t / nsample;
        double p = 0.0;
        for (int k = 0; k < d; ++k) p = p * u + coef[(size_t)k * MAX_NS + j];
        maxerr = std::max(maxerr, std::fabs(p - phi(xof(u))));
      }
    }
    if (maxerr <= target_err || d >= maxcoef) {
      *maxerr_out = maxerr;
      return d;
    }
  }
}

int kernel_ft_nodes(const KernelFn &phi, double nodes_per_halfwidth, double *z, double *f)
// Quadrature for the kernel's Fourier transform, as in src/cuda/fft.cu:185-202
// (type 1/2: q = 2 + 1.5 ns) and :144-157 (type 3: q = 2 + ns): Gauss-Legendre
// with 2q nodes on [-1,1]; by symmetry of the kernel only q nodes are kept and
// the integral is 2 sum_n f_n cos(k z_n) with z_n in grid units.
{
  const double J2 = phi.ns / 2.0;
  const int q = (int)(2 + nodes_per_halfwidth * J2);
  std::vector<double> x(2 * q), w(2 * q);
  gauss_legendre(2 * q, x.data(), w.data());
  for (int n = 0; n < q; ++n) {
    z[n] = J2 * x[n];
    f[n] = J2 * w[n] * phi(z[n]);
  }
  return q;
}

template <typename T>
double build_kernel_shape(const KernelFn &phi, int use_horner, double tol, KernelShape<T> *K) {
  std::memset(K, 0, sizeof(*K));
  const int ns = phi.ns;
  K->ns = ns;
  K->form = phi.form;
  K->beta = (T)phi.beta;
  K->es_c = (T)(4.0 / (double(ns) * ns));
  // direct evaluation exists for the ES form only; the PSWF is always fitted
  K->use_horner = (use_horner || phi.form == KERNEL_PSWF) ? 1 : 0;
  // pieces are fitted for any sigma; the reference only carries tables for
  // sigma 2 and 1.25, which the option check already enforces
  std::vector<double> coef;
  double err = 0;
  const bool is_float = std::is_same_v<T, float>;
  const double target = std::max(1e-2 * tol, is_float ? 2e-7 : 4e-15);
  const int H = horner_len(ns);
  const int ncoef = horner_fit(phi, target, H, coef, &err);
  K->ncoef = H;
  for (int k = 0; k < H; ++k)
    for (int j = 0; j < ns; ++j) {
      const int src = k - (H - ncoef); // zero-pad the high-degree end
      K->coef[k][j] = src >= 0 ? (T)coef[(size_t)src * MAX_NS + j] : T(0);
    }
  return err;
}
template double build_kernel_shape<float>(const KernelFn &, int, double, KernelShape<float> *);
template double build_kernel_shape<double>(const KernelFn &, int, double, KernelShape<double> *);

} // namespace gbn
