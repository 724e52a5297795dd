// TEST INFRASTRUCTURE: a C shim over the reference's own host planning code
// (src/common/{utils,kernel,pswf}.cpp of flatironinstitute/finufft, compiled
// from the reference tree by oracle/Makefile into _ref/). Used only to pin the
// oracle's restatement and to generate tests/golden fixtures.
#include <finufft_common/common.h>
#include <finufft_common/kernel.h>
#include <finufft_common/pswf.h>
#include <finufft_common/spread_opts.h>
#include <finufft_common/utils.h>

extern "C" {
long long ref_next235(long long n, long long f) { return finufft::common::next235(n, f); }
void ref_gaussquad(int n, double *x, double *w) { finufft::common::gaussquad(n, x, w); }
void ref_nhg_type3(double sigma, double X, double S, int ns, double *out) {
  auto [nf, h, gam] = finufft::common::nhg_type3(sigma, X, S, ns, 2147483647LL);
  out[0] = (double)nf;
  out[1] = h;
  out[2] = gam;
}
// CPU library kernel width and PSWF shape (kerformula 8, the default)
int ref_cpu_kernel(double tol, int dim, int type, double sigma, double *beta) {
  finufft_spread_opts o;
  o.upsampfac = sigma;
  o.kerformula = 8;
  int ns = finufft::kernel::theoretical_kernel_ns(tol, dim, type, o);
  o.nspread = ns;
  finufft::kernel::set_kernel_shape_given_ns(o, 0);
  *beta = o.beta;
  return ns;
}
// PSWF psi_0^c(z) normalized to 1 at z = 0, at n points
void ref_pswf(double c, int n, const double *z, double *out) {
  finufft::common::PSWF0 p(c);
  for (int i = 0; i < n; ++i) out[i] = p(z[i]);
}
}
