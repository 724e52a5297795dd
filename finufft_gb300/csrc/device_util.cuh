// Device helpers shared by the GB300 NUFFT kernels.
#pragma once
#include <cmath>

#include "common.h"

namespace gbn {

// Affine map of one coordinate axis onto the periodic fine grid.
// y = (x - shift) * scale is folded into [0, nf) (period 2 pi) and split into
// an integer cell and a fraction. Types 1/2 use shift 0, scale 1 (y == x
// exactly); type 3 uses it for its rescaled sources and targets.
struct AxisMap {
  double shift, scale;
  int nf, bin;
};

// Fold-rescale of a coordinate, in double precision with round-to-nearest
// on every step (IEEE fma, floor, sub, mul), so a host replica reproduces it
// bit for bit. Follows the fold of include/cufinufft/spreadinterp.hpp:61-89
// (r = x/2pi + 1/2 mod 1, times nf) but in FP64, which keeps float inputs at
// full accuracy on large grids. NaN/Inf coordinates land on cell 0.
__host__ __device__ inline void fold_cell(double x, const AxisMap &a, int &cell,
                                          double &frac) {
#ifdef __CUDA_ARCH__
  double y = __dmul_rn(__dsub_rn(x, a.shift), a.scale);
  double r = __fma_rn(y, INV_2PI, 0.5);
  r = __dsub_rn(r, floor(r));
  r = __dmul_rn(r, (double)a.nf);
#else
  double y = (x - a.shift) * a.scale;
  double r = fma(y, INV_2PI, 0.5);
  r = r - floor(r);
  r = r * (double)a.nf;
#endif
  if (!(r >= 0.0 && r <= (double)a.nf)) r = 0.0;
  double fl = floor(r);
  int c = (int)fl;
  if (c >= a.nf) c -= a.nf;
  cell = c;
  frac = r - fl;
}

#ifdef __CUDACC__
template <typename T> __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  cplx<T> r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// a * b, or a * conj(b) when conj_b is set
template <typename T>
__device__ __forceinline__ cplx<T> cmul_opt(cplx<T> a, cplx<T> b, int conj_b) {
  if (conj_b) b.y = -b.y;
  return cmul<T>(a, b);
}

// ker[j] = phi(t + j), j = 0..NS-1, t in [-NS/2, -NS/2+1]: the kernel weights
// of the NS grid points starting at the point's first support cell.
template <typename T, int NS>
__device__ __forceinline__ void eval_kernel(T *ker, T t, const KernelShape<T> &K) {
  if (K.use_horner) {
    const T u = T(2) * t + T(NS - 1); // in [-1, 1]
#pragma unroll
    for (int j = 0; j < NS; ++j) ker[j] = K.coef[0][j];
#pragma unroll
    for (int k = 1; k < horner_len(NS); ++k) {
#pragma unroll
      for (int j = 0; j < NS; ++j) ker[j] = fma(ker[j], u, K.coef[k][j]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const T x = t + T(j);
      const T z2 = K.es_c * x * x;
      ker[j] = z2 < T(1) ? exp(K.beta * (sqrt(T(1) - z2) - T(1))) : T(0);
    }
  }
}

__device__ __forceinline__ void atomic_add_cplx_global(float2 *p, float2 v) {
  atomicAdd(p, v); // vector f32x2 reduction (sm_90 and newer)
}
__device__ __forceinline__ void atomic_add_cplx_global(double2 *p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

#endif // __CUDACC__

} // namespace gbn
