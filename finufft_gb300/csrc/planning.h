// Host-side planning math: kernel width and shape, fine-grid sizes, quadrature
// nodes, Horner fits and bin sizes. Pure C++, no CUDA calls.
#pragma once
#include <cstdint>
#include <vector>

#include "common.h"

namespace gbn {

// Smallest even 2,3,5-smooth integer >= n (FINUFFT's next235(n, 2)).
int64_t next235_even(int64_t n);

// n-node Gauss-Legendre rule on [-1,1]: nodes ascending, weights.
void gauss_legendre(int n, double *x, double *w);

// ES kernel width and beta for a requested tolerance (GPU library rule).
struct KernelChoice {
  int ns;
  double beta;
};
// Throws Error(FINUFFT_ERR_HORNER_WRONG_BETA / UPSAMPFAC_TOO_SMALL) as the reference does.
KernelChoice choose_kernel(double tol, double sigma, int kerevalmeth, int is_float,
                           int spreadinterponly, int debug);

// The CPU library's kernel choice: PSWF of width max(its width law, the GPU
// rule) and shape parameter by kerformula (0 or 8: default, 7, 9; any other
// value throws FINUFFT_ERR_KERFORMULA_NOTVALID).
// kerevalmeth 1 applies the GPU interface's sigma check (FINUFFT_ERR_HORNER_WRONG_BETA
// off sigma 2 and 1.25) to a user-given sigma.
KernelChoice choose_kernel_pswf(double tol, double sigma, int dim, int type, int is_float,
                                int kerformula, int kerevalmeth, int spreadinterponly,
                                int debug);

// ES kernel value at x (grid units), support |x| < ns/2.
double es_kernel(double x, int ns, double beta);

// A spreading kernel as a host function of x in grid units (support |x| <= ns/2):
// the ES kernel exp(beta (sqrt(1 - (2x/ns)^2) - 1)) of the GPU library, or the
// PSWF psi_0^beta(2x/ns) / psi_0^beta(0) of the CPU library. Used to fit the
// Horner pieces and the quadrature of the kernel's Fourier transform.
struct KernelFn {
  int form = KERNEL_ES;
  int ns = 2;
  double beta = 0;
  std::vector<double> leg; // PSWF: Legendre coefficients of psi_0 (even degrees)
  double scale = 1;        // PSWF: 1 / psi_0(0)
  double operator()(double x) const;
};
KernelFn make_kernel_fn(int form, int ns, double beta);

// Fine grid length for a type 1/2 dimension with ms modes.
int64_t fine_grid_len(int64_t ms, double sigma, int ns);
// The smallest even size of the ladder 2^k * {1, 5/4, 3/2, 15/8} (5-smooth)
// that is >= n: batches of many problem sizes then share few FFT shapes (at
// most 25% more cells per dimension than n, four sizes per octave).
int64_t ladder_grid_len(int64_t n);

// Type-3 grid: given source half-width X and frequency half-width S.
void type3_grid(double sigma, double X, double S, int ns, int64_t *nf, double *h,
                double *gam);

// Half-width and centre of an interval [lo,hi], re-centring only when it pays.
void width_center(double lo, double hi, double *w, double *c);

// Horner fit of the kernel: fills coef[k*16 + j] (k = 0 highest degree),
// returns the number of coefficients per piece (<= maxcoef) and the max abs error seen.
int horner_fit(const KernelFn &phi, double target_err, int maxcoef, std::vector<double> &coef,
               double *maxerr);

// Quadrature nodes/weights for the kernel Fourier transform:
//   phihat(k) = sum_n f[n] * 2 cos(k z[n]),  z in grid units.
// q = number of nodes used.
int kernel_ft_nodes(const KernelFn &phi, double nodes_per_halfwidth, double *z, double *f);

// Fill the kernel description passed to spread/interp kernels: the shape, and
// Horner pieces fitted to max(tol/100, a few ulps). Returns the fit's max error.
template <typename T>
double build_kernel_shape(const KernelFn &phi, int use_horner, double tol, KernelShape<T> *K);

} // namespace gbn
