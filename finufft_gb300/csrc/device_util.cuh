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

// Single-precision fold for float coordinates on the identity map (types 1
// and 2) with nf < 2^24: x/(2 pi) + 1/2 is formed as an unevaluated float sum
// hi + lo (error-free product and sum: fma gives the exact rounding error of a
// product, Knuth's two-sum that of a sum), so the fold keeps ~48 bits like the
// FP64 fold while running on the FP32 pipe. Every operation is rounded to
// nearest with no contraction, so a host replica (fmaf) reproduces it bit for
// bit. NaN/Inf coordinates land on cell 0.
__host__ __device__ inline void fold_cell_f32(float x, int nf, int &cell, float &frac) {
  constexpr float C_HI = (float)INV_2PI;
  constexpr float C_LO = (float)(INV_2PI - (double)(float)INV_2PI);
  const float nff = (float)nf;
  if (!(x - x == 0.f)) { // NaN or Inf
    cell = 0;
    frac = 0.f;
    return;
  }
#ifdef __CUDA_ARCH__
#define GBN_MUL(a, b) __fmul_rn(a, b)
#define GBN_ADD(a, b) __fadd_rn(a, b)
#define GBN_SUB(a, b) __fsub_rn(a, b)
#define GBN_FMA(a, b, c) __fmaf_rn(a, b, c)
#else
#define GBN_MUL(a, b) ((a) * (b))
#define GBN_ADD(a, b) ((a) + (b))
#define GBN_SUB(a, b) ((a) - (b))
#define GBN_FMA(a, b, c) fmaf(a, b, c)
#endif
  // x/2pi + 1/2 = s + lo exactly enough: error-free product, then two-sum
  const float ph = GBN_MUL(x, C_HI);
  const float pl = GBN_FMA(x, C_LO, GBN_FMA(x, C_HI, -ph));
  const float s = GBN_ADD(ph, 0.5f);
  const float bb = GBN_SUB(s, ph);
  const float lo = GBN_ADD(GBN_ADD(GBN_SUB(ph, GBN_SUB(s, bb)), GBN_SUB(0.5f, bb)), pl);
  // fraction of s as an exact two-sum (s - floor(s) rounds to 1 for a tiny
  // negative s): fh + fl, then scaled by nf: gh + gl
  const float fls = -floorf(s);
  const float fh = GBN_ADD(s, fls);
  const float fb = GBN_SUB(fh, s);
  const float fl = GBN_ADD(GBN_SUB(s, GBN_SUB(fh, fb)), GBN_SUB(fls, fb));
  const float gh = GBN_MUL(fh, nff);
  const float gl = GBN_FMA(GBN_ADD(fl, lo), nff, GBN_FMA(fh, nff, -gh));
  float c = floorf(gh);
  float fr = GBN_ADD(GBN_SUB(gh, c), gl);
  // |gl| < 2, so fr is in (-2, 3): move its integer part into the cell; a tiny
  // negative fraction plus one rounds to 1, which goes to the next cell
  const float k = floorf(fr);
  c = GBN_ADD(c, k);
  fr = GBN_SUB(fr, k);
  if (fr >= 1.f) {
    c = GBN_ADD(c, 1.f);
    fr = 0.f;
  }
#undef GBN_MUL
#undef GBN_ADD
#undef GBN_SUB
#undef GBN_FMA
  int ci = (int)c;
  if (ci < 0) ci += nf;
  else if (ci >= nf) ci -= nf;
  cell = ci;
  frac = fr;
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

// As eval_kernel, using the kernel's evenness for Horner pieces: piece
// NS-1-j at u is piece j at -u (phi(x) = phi(-x) maps the two intervals onto
// each other), so with p_j(u) = E_j(u^2) + u O_j(u^2) one pass over piece j's
// coefficients gives ker[j] = E + u O and ker[NS-1-j] = E - u O: about half
// the fused multiply-adds of evaluating every piece. The mirrored weights
// carry piece j's fit error instead of their own piece's (both within the
// fit target).
template <typename T, int NS>
__device__ __forceinline__ void eval_kernel_sym(T *ker, T t, const KernelShape<T> &K) {
  if (!K.use_horner) {
    eval_kernel<T, NS>(ker, t, K);
    return;
  }
  constexpr int H = horner_len(NS);
  const T u = T(2) * t + T(NS - 1);
  const T w = u * u;
#pragma unroll
  for (int j = 0; j < (NS + 1) / 2; ++j) {
    T e = T(0), o = T(0);
#pragma unroll
    for (int k = 0; k < H; ++k) { // coefficient k multiplies u^(H-1-k)
      if ((H - 1 - k) % 2 == 0) e = fma(e, w, K.coef[k][j]);
      else o = fma(o, w, K.coef[k][j]);
    }
    ker[j] = fma(u, o, e);
    if (j != NS - 1 - j) ker[NS - 1 - j] = fma(-u, o, e);
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
