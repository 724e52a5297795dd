// Elementwise and small reduction kernels around the spread/FFT/interp core.
#pragma once
#include "common.h"

namespace gbn {

struct QuadNodes {
  int q;
  double z[MAX_NQUAD]; // nodes in grid units
  double f[MAX_NQUAD]; // weights times kernel values
};

// inv[k] = 1 / phihat(k), k = 0..nf/2, phihat(k) = (-1)^k sum_n f_n 2cos(2 pi k z_n / nf)
template <typename T> void launch_inv_fseries(int nf, const QuadNodes &Q, T *inv, cudaStream_t s);

// Type 1 deconvolution: fk[t][k] = fw[t][g(k)] * prod_d inv_d[|k_d|].
template <typename T>
void launch_deconv(int dim, const int ms[3], const int nf[3], int modeord, const T *const inv[3],
                   const cplx<T> *fw, int64_t nf_total, cplx<T> *fk, int ntr, cudaStream_t s);

// Type 2 amplification: fw[t][g] = fk[t][k(g)] * prod_d inv_d[|k_d|] for the
// cells that carry a mode, 0 elsewhere (writes the whole fine grid).
template <typename T>
void launch_amplify(int dim, const int ms[3], const int nf[3], int modeord,
                    const T *const inv[3], const cplx<T> *fk, cplx<T> *fw, int64_t nf_total,
                    int ntr, cudaStream_t s);

// min and max of a[0..n) (host result; synchronizes the stream).
template <typename T> void array_range(const T *a, int n, double *lo, double *hi, cudaStream_t s);

// Type 3 pre-phase: pre[j] = exp(i isign sum_d D_d x_d[j]), phase in FP64.
template <typename T>
void launch_t3_prephase(int dim, const T *const xyz[3], int M, const double D[3], int isign,
                        cplx<T> *pre, cudaStream_t s);

// Type 3 post factor: post[k] = exp(i isign sum_d C_d (s_d[k] - D_d)) / prod_d phihat(s'_d),
// s'_d = scale_d (s_d[k] - D_d), phihat(w) = sum_n f_n 2 cos(w z_n); all FP64.
template <typename T>
void launch_t3_postfactor(int dim, const T *const stu[3], int N, const double C[3],
                          const double D[3], const double scale[3], int isign,
                          const QuadNodes &Q, cplx<T> *post, cudaStream_t s);

// Measured conflict-free shared-memory f32 atomicAdd rate of a device
// (lane operations per second): the denominator of the spreading roofline.
double smem_atomic_rate(int device, bool i32 = false);

} // namespace gbn
