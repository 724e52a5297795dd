#include <algorithm>
#include <limits>
#include <map>
#include <mutex>
// Deconvolution / amplification, kernel Fourier series and type-3 phase
// kernels, plus the host dispatch of the spread/interp translation units.
#include <vector>

#include "device_util.cuh"
#include "elementwise.h"
#include "spreadinterp.h"
#include "tile_layout.h"

namespace gbn {

template <typename T, int DIM>
void spread_dim(const PointLayout<T> &, const KernelShape<T> &, const cplx<T> *,
                const cplx<T> *, int, cplx<T> *, int64_t, int, const SpreadConfig &,
                cudaStream_t);
template <typename T, int DIM>
void interp_dim(const PointLayout<T> &, const KernelShape<T> &, const cplx<T> *, int64_t,
                const cplx<T> *, int, cplx<T> *, int, cudaStream_t);

template <typename T> size_t spread_tile_smem(int dim, int ns, const int bin[3], int threads) {
  if (dim == 3) // tile (padded pitches) + per-warp staging of 32 points
    return tile3_bytes<T>(ns, bin[0], bin[1], bin[2]) +
           (size_t)(threads / 32) * stage_bytes_per_warp<T>(ns);
  size_t cells = (size_t)(bin[0] + ns);
  if (dim > 1) cells *= (size_t)(bin[1] + ns);
  return 2 * sizeof(T) * cells;
}
template <typename T> size_t spread_tile3w_bytes(int ns, const int bin[3]) {
  return tile3_bytes<T>(ns, bin[0], bin[1], bin[2]) + t3w_stage_bytes(ns, (int)sizeof(T));
}
template <typename T> size_t spread_tile3m_bytes(int ns, const int bin[3], int warps) {
  return tile3_bytes<T>(ns, bin[0], bin[1], bin[2]) +
         (size_t)warps * t3m_stage_bytes(ns, (int)sizeof(T));
}
template <typename T> size_t spread_tile3v_bytes(int ns, const int bin[3], int warps) {
  return tile3v_bytes<T>(ns, bin[0], bin[1], bin[2]) +
         (size_t)warps * t3v_stage_bytes(ns, (int)sizeof(T));
}
template size_t spread_tile3v_bytes<float>(int, const int[3], int);
template size_t spread_tile3v_bytes<double>(int, const int[3], int);
template <typename T> size_t spread_tile2m_bytes(int ns, const int bin[3], int warps) {
  const size_t tile = (2 * sizeof(T) * (size_t)tile_pitch_x(3, bin[0] + ns) * (bin[1] + ns) + 15) /
                      16 * 16;
  const size_t stage = (33 * (ns + 4 * ((ns + 3) / 4) + 2) * sizeof(T) + 33 * 4 + 15) / 16 * 16;
  return tile + (size_t)warps * stage;
}
template <typename T> size_t spread_output_driven_bytes(int dim, int ns, const int bin[3]) {
  size_t cells = 1;
  for (int d = 0; d < dim; ++d) cells *= (size_t)(bin[d] + ns);
  return 2 * sizeof(T) * cells + 64 * ((size_t)dim * ns * sizeof(T) + 2 * sizeof(T) + dim * 4);
}
template size_t spread_output_driven_bytes<float>(int, int, const int[3]);
template size_t spread_output_driven_bytes<double>(int, int, const int[3]);

size_t spread_tile3x_bytes(int ns, const int bin[3]) {
  return t3x_bytes(ns, bin[0], bin[1], bin[2]);
}
template size_t spread_tile2m_bytes<float>(int, const int[3], int);
template size_t spread_tile2m_bytes<double>(int, const int[3], int);
template size_t spread_tile3m_bytes<float>(int, const int[3], int);
template size_t spread_tile3m_bytes<double>(int, const int[3], int);
template size_t spread_tile3w_bytes<float>(int, const int[3]);
template size_t spread_tile3w_bytes<double>(int, const int[3]);
template size_t spread_tile_smem<float>(int, int, const int[3], int);
template size_t spread_tile_smem<double>(int, int, const int[3], int);

namespace {
std::mutex err_mu;
std::map<int, int *> err_words;
} // namespace

int *device_error_word() {
  int dev = 0;
  GBN_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(err_mu);
  int *&w = err_words[dev];
  if (!w) {
    GBN_CUDA(cudaMalloc((void **)&w, sizeof(int)));
    GBN_CUDA(cudaMemset(w, 0, sizeof(int)));
  }
  return w;
}

int device_error_take() {
  int *w = device_error_word();
  int v = 0;
  GBN_CUDA(cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) GBN_CUDA(cudaMemset(w, 0, sizeof(int)));
  return v;
}

template <typename T>
void launch_spread(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *c,
                   const cplx<T> *pre, int conj_pre, cplx<T> *fw, int64_t nf_total, int ntr,
                   const SpreadConfig &cfg, cudaStream_t s) {
  if (L.nsub <= 0 || ntr <= 0) return;
  if (L.dim == 1) spread_dim<T, 1>(L, K, c, pre, conj_pre, fw, nf_total, ntr, cfg, s);
  else if (L.dim == 2) spread_dim<T, 2>(L, K, c, pre, conj_pre, fw, nf_total, ntr, cfg, s);
  else spread_dim<T, 3>(L, K, c, pre, conj_pre, fw, nf_total, ntr, cfg, s);
}
template <typename T>
void launch_interp(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *fw,
                   int64_t nf_total, const cplx<T> *post, int conj_post, cplx<T> *out, int ntr,
                   cudaStream_t s) {
  if (L.nsub <= 0 || ntr <= 0) return;
  // sorted-order results reach user order only through the inverse permutation
  if (L.sorted_out && !L.iperm) GBN_THROW(FINUFFT_ERR_UNKNOWN_EXCEPTION, "sorted output without iperm");
  if (L.dim == 1) interp_dim<T, 1>(L, K, fw, nf_total, post, conj_post, out, ntr, s);
  else if (L.dim == 2) interp_dim<T, 2>(L, K, fw, nf_total, post, conj_post, out, ntr, s);
  else interp_dim<T, 3>(L, K, fw, nf_total, post, conj_post, out, ntr, s);
}
template void launch_spread<float>(const PointLayout<float> &, const KernelShape<float> &,
                                   const float2 *, const float2 *, int, float2 *, int64_t, int,
                                   const SpreadConfig &, cudaStream_t);
template void launch_spread<double>(const PointLayout<double> &, const KernelShape<double> &,
                                    const double2 *, const double2 *, int, double2 *, int64_t,
                                    int, const SpreadConfig &, cudaStream_t);
template void launch_interp<float>(const PointLayout<float> &, const KernelShape<float> &,
                                   const float2 *, int64_t, const float2 *, int, float2 *, int,
                                   cudaStream_t);
template void launch_interp<double>(const PointLayout<double> &, const KernelShape<double> &,
                                    const double2 *, int64_t, const double2 *, int, double2 *,
                                    int, cudaStream_t);

namespace {
inline unsigned blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

// mode index of fk position i along one axis of length m
__device__ __forceinline__ int mode_of(int i, int m, int modeord) {
  return modeord == 0 ? i - m / 2 : (i < m - m / 2 ? i : i - m);
}
// fk position of mode k along one axis of length m
__device__ __forceinline__ int pos_of(int k, int m, int modeord) {
  return modeord == 0 ? k + m / 2 : (k >= 0 ? k : k + m);
}

template <typename T>
__global__ void inv_fseries_kernel(int nf, QuadNodes Q, T *inv) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nf / 2; k += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int n = 0; n < Q.q; ++n) acc += Q.f[n] * 2.0 * cos((double)k * (2.0 * PI * Q.z[n] / nf));
    if (k & 1) acc = -acc; // grid origin sits at x = -pi
    inv[k] = (T)(1.0 / acc);
  }
}

// Deconvolution and amplification walk rows along x in warp items: a warp
// takes DC_W consecutive x positions of one row (a row = fixed y, z and
// transform), finds the row's indices, its y/z factor and its grid row once
// with 32-bit arithmetic, and its lanes read and write contiguous x runs
// (eight positions each); warps stride over the items.
constexpr int DC_THREADS = 256;
constexpr int DC_W = 256; // x positions per warp item

__device__ __forceinline__ int dc_items(int len) { return (len + DC_W - 1) / DC_W; }

// fk[t][k] = fw[t][wrap(k)] / (phihat_x(kx) phihat_y(ky) phihat_z(kz)) (type 1)
template <typename T, int DIM>
__global__ void __launch_bounds__(DC_THREADS)
    deconv_kernel(int ms0, int ms1, int ms2, int nf0, int nf1, int nf2, int modeord,
                  const T *__restrict__ i0, const T *__restrict__ i1, const T *__restrict__ i2,
                  const cplx<T> *__restrict__ fw, int64_t nf_total, cplx<T> *__restrict__ fk,
                  int64_t nmodes, int64_t nitems) {
  const int lane = threadIdx.x & 31;
  const int xchunks = dc_items(ms0);
  const int64_t wstride = (int64_t)gridDim.x * (DC_THREADS / 32);
  for (int64_t it = (int64_t)blockIdx.x * (DC_THREADS / 32) + (threadIdx.x >> 5); it < nitems;
       it += wstride) {
    const int row = (int)(it / xchunks);
    const int x0 = (int)(it - (int64_t)row * xchunks) * DC_W;
    int iy = 0, iz = 0, tr = row;
    if (DIM > 1) {
      iy = tr % ms1;
      tr /= ms1;
    }
    if (DIM > 2) {
      iz = tr % ms2;
      tr /= ms2;
    }
    T fyz = T(1);
    int64_t grow = (int64_t)tr * nf_total;
    if (DIM > 1) {
      const int ky = mode_of(iy, ms1, modeord);
      grow += (int64_t)nf0 * (ky >= 0 ? ky : nf1 + ky);
      fyz = i1[ky >= 0 ? ky : -ky];
    }
    if (DIM > 2) {
      const int kz = mode_of(iz, ms2, modeord);
      grow += (int64_t)nf0 * nf1 * (kz >= 0 ? kz : nf2 + kz);
      fyz *= i2[kz >= 0 ? kz : -kz];
    }
    const int64_t orow = (int64_t)tr * nmodes + (int64_t)ms0 * (iy + (int64_t)ms1 * iz);
    const int x1 = min(ms0, x0 + DC_W);
    for (int ix = x0 + lane; ix < x1; ix += 32) {
      const int kx = mode_of(ix, ms0, modeord);
      const cplx<T> v = fw[grow + (kx >= 0 ? kx : nf0 + kx)];
      const T f = fyz * i0[kx >= 0 ? kx : -kx];
      cplx<T> r;
      r.x = v.x * f;
      r.y = v.y * f;
      fk[orow + ix] = r;
    }
  }
}

// fw[t][g] = fk[t][mode(g)] / prod phihat for retained modes, 0 elsewhere (type 2)
template <typename T, int DIM>
__global__ void __launch_bounds__(DC_THREADS)
    amplify_kernel(int ms0, int ms1, int ms2, int nf0, int nf1, int nf2, int modeord,
                   const T *__restrict__ i0, const T *__restrict__ i1, const T *__restrict__ i2,
                   const cplx<T> *__restrict__ fk, int64_t nmodes, cplx<T> *__restrict__ fw,
                   int64_t nf_total, int64_t nitems) {
  const int lane = threadIdx.x & 31;
  const int xchunks = dc_items(nf0);
  const int64_t wstride = (int64_t)gridDim.x * (DC_THREADS / 32);
  for (int64_t it = (int64_t)blockIdx.x * (DC_THREADS / 32) + (threadIdx.x >> 5); it < nitems;
       it += wstride) {
    const int row = (int)(it / xchunks);
    const int x0 = (int)(it - (int64_t)row * xchunks) * DC_W;
    int gy = 0, gz = 0, tr = row;
    if (DIM > 1) {
      gy = tr % nf1;
      tr /= nf1;
    }
    if (DIM > 2) {
      gz = tr % nf2;
      tr /= nf2;
    }
    bool in = true;
    T fyz = T(1);
    int64_t irow = (int64_t)tr * nmodes;
    if (DIM > 1) {
      const int ky = gy <= (ms1 - 1) / 2 ? gy : (gy >= nf1 - ms1 / 2 ? gy - nf1 : INT32_MIN);
      in = ky != INT32_MIN;
      if (in) {
        irow += (int64_t)ms0 * pos_of(ky, ms1, modeord);
        fyz = i1[ky >= 0 ? ky : -ky];
      }
    }
    if (DIM > 2 && in) {
      const int kz = gz <= (ms2 - 1) / 2 ? gz : (gz >= nf2 - ms2 / 2 ? gz - nf2 : INT32_MIN);
      in = kz != INT32_MIN;
      if (in) {
        irow += (int64_t)ms0 * ms1 * pos_of(kz, ms2, modeord);
        fyz *= i2[kz >= 0 ? kz : -kz];
      }
    }
    const int64_t grow = (int64_t)tr * nf_total + (int64_t)nf0 * (gy + (int64_t)nf1 * gz);
    const int x1 = min(nf0, x0 + DC_W);
    for (int gx = x0 + lane; gx < x1; gx += 32) {
      cplx<T> r;
      r.x = T(0);
      r.y = T(0);
      if (in) {
        const int kx = gx <= (ms0 - 1) / 2 ? gx : (gx >= nf0 - ms0 / 2 ? gx - nf0 : INT32_MIN);
        if (kx != INT32_MIN) {
          const cplx<T> v = fk[irow + pos_of(kx, ms0, modeord)];
          const T f = fyz * i0[kx >= 0 ? kx : -kx];
          r.x = v.x * f;
          r.y = v.y * f;
        }
      }
      fw[grow + gx] = r;
    }
  }
}

template <typename T>
__global__ void range_kernel(const T *__restrict__ a, int n, double *__restrict__ out) {
  double lo = INFINITY, hi = -INFINITY;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = (double)a[i];
    lo = fmin(lo, v);
    hi = fmax(hi, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
  }
  __shared__ double slo[32], shi[32];
  if ((threadIdx.x & 31) == 0) {
    slo[threadIdx.x >> 5] = lo;
    shi[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      lo = fmin(lo, slo[w]);
      hi = fmax(hi, shi[w]);
    }
    out[2 * blockIdx.x] = lo;
    out[2 * blockIdx.x + 1] = hi;
  }
}

template <typename T>
__global__ void t3_prephase_kernel(int dim, const T *__restrict__ x, const T *__restrict__ y,
                                   const T *__restrict__ z, int M, double D0, double D1, double D2,
                                   int isign, cplx<T> *__restrict__ pre) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x) {
    double ph = D0 * (double)x[j];
    if (dim > 1) ph += D1 * (double)y[j];
    if (dim > 2) ph += D2 * (double)z[j];
    double sn, cs;
    sincos(ph, &sn, &cs);
    cplx<T> r;
    r.x = (T)cs;
    r.y = (T)(isign * sn);
    pre[j] = r;
  }
}

template <typename T>
__global__ void t3_post_kernel(int dim, const T *__restrict__ s, const T *__restrict__ t,
                               const T *__restrict__ u, int N, double C0, double C1, double C2,
                               double D0, double D1, double D2, double sc0, double sc1,
                               double sc2, int isign, QuadNodes Q, cplx<T> *__restrict__ post) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    const double a[3] = {(double)s[k] - D0, dim > 1 ? (double)t[k] - D1 : 0.0,
                         dim > 2 ? (double)u[k] - D2 : 0.0};
    const double sc[3] = {sc0, sc1, sc2};
    double phihat = 1.0;
    for (int d = 0; d < dim; ++d) {
      const double w = sc[d] * a[d];
      double acc = 0.0;
      for (int n = 0; n < Q.q; ++n) acc += Q.f[n] * 2.0 * cos(w * Q.z[n]);
      phihat *= acc;
    }
    const double ph = C0 * a[0] + C1 * a[1] + C2 * a[2];
    double sn, cs;
    sincos(ph, &sn, &cs);
    cplx<T> r;
    r.x = (T)(cs / phihat);
    r.y = (T)(isign * sn / phihat);
    post[k] = r;
  }
}
} // namespace

template <typename T> void launch_inv_fseries(int nf, const QuadNodes &Q, T *inv, cudaStream_t s) {
  inv_fseries_kernel<T><<<blocks_for(nf / 2 + 1, 256), 256, 0, s>>>(nf, Q, inv);
  GBN_LAUNCH_CHECK();
}

// warp items of a row walk: rows x ceil(len / DC_W); blocks of 8 warps, at
// most 16 per SM (they stride over the items)
inline unsigned dc_blocks(int64_t nitems) {
  const int64_t want = (nitems + DC_THREADS / 32 - 1) / (DC_THREADS / 32);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, 152 * 16));
}

template <typename T>
void launch_deconv(int dim, const int ms[3], const int nf[3], int modeord, const T *const inv[3],
                   const cplx<T> *fw, int64_t nf_total, cplx<T> *fk, int ntr, cudaStream_t s) {
  const int64_t nmodes = (int64_t)ms[0] * ms[1] * ms[2];
  const int64_t nitems = (int64_t)((ms[0] + DC_W - 1) / DC_W) * ms[1] * ms[2] * ntr;
  if (nitems <= 0) return;
  if ((int64_t)ms[1] * ms[2] * ntr > std::numeric_limits<int32_t>::max())
    GBN_THROW(FINUFFT_ERR_MAXNALLOC, "deconvolution rows");
  const unsigned g = dc_blocks(nitems);
  if (dim == 1)
    deconv_kernel<T, 1><<<g, DC_THREADS, 0, s>>>(ms[0], 1, 1, nf[0], 1, 1, modeord, inv[0],
                                                 inv[0], inv[0], fw, nf_total, fk, nmodes,
                                                 nitems);
  else if (dim == 2)
    deconv_kernel<T, 2><<<g, DC_THREADS, 0, s>>>(ms[0], ms[1], 1, nf[0], nf[1], 1, modeord,
                                                 inv[0], inv[1], inv[1], fw, nf_total, fk,
                                                 nmodes, nitems);
  else
    deconv_kernel<T, 3><<<g, DC_THREADS, 0, s>>>(ms[0], ms[1], ms[2], nf[0], nf[1], nf[2],
                                                 modeord, inv[0], inv[1], inv[2], fw, nf_total,
                                                 fk, nmodes, nitems);
  GBN_LAUNCH_CHECK();
}

template <typename T>
void launch_amplify(int dim, const int ms[3], const int nf[3], int modeord,
                    const T *const inv[3], const cplx<T> *fk, cplx<T> *fw, int64_t nf_total,
                    int ntr, cudaStream_t s) {
  const int64_t nmodes = (int64_t)ms[0] * ms[1] * ms[2];
  const int64_t nitems = (int64_t)((nf[0] + DC_W - 1) / DC_W) * nf[1] * nf[2] * ntr;
  if (nitems <= 0) return;
  if ((int64_t)nf[1] * nf[2] * ntr > std::numeric_limits<int32_t>::max())
    GBN_THROW(FINUFFT_ERR_MAXNALLOC, "amplification rows");
  const unsigned g = dc_blocks(nitems);
  if (dim == 1)
    amplify_kernel<T, 1><<<g, DC_THREADS, 0, s>>>(ms[0], 1, 1, nf[0], 1, 1, modeord, inv[0],
                                                  inv[0], inv[0], fk, nmodes, fw, nf_total,
                                                  nitems);
  else if (dim == 2)
    amplify_kernel<T, 2><<<g, DC_THREADS, 0, s>>>(ms[0], ms[1], 1, nf[0], nf[1], 1, modeord,
                                                  inv[0], inv[1], inv[1], fk, nmodes, fw,
                                                  nf_total, nitems);
  else
    amplify_kernel<T, 3><<<g, DC_THREADS, 0, s>>>(ms[0], ms[1], ms[2], nf[0], nf[1], nf[2],
                                                  modeord, inv[0], inv[1], inv[2], fk, nmodes,
                                                  fw, nf_total, nitems);
  GBN_LAUNCH_CHECK();
}

template <typename T> void array_range(const T *a, int n, double *lo, double *hi, cudaStream_t s) {
  const int blocks = 256;
  double *d = nullptr;
  GBN_CUDA(cudaMallocAsync((void **)&d, 2 * blocks * sizeof(double), s));
  range_kernel<T><<<blocks, 256, 0, s>>>(a, n, d);
  GBN_LAUNCH_CHECK();
  std::vector<double> h(2 * blocks);
  GBN_CUDA(cudaMemcpyAsync(h.data(), d, 2 * blocks * sizeof(double), cudaMemcpyDeviceToHost, s));
  GBN_CUDA(cudaFreeAsync(d, s));
  GBN_CUDA(cudaStreamSynchronize(s));
  double l = INFINITY, u = -INFINITY;
  for (int b = 0; b < blocks; ++b) {
    l = std::fmin(l, h[2 * b]);
    u = std::fmax(u, h[2 * b + 1]);
  }
  *lo = l;
  *hi = u;
}

template <typename T>
void launch_t3_prephase(int dim, const T *const xyz[3], int M, const double D[3], int isign,
                        cplx<T> *pre, cudaStream_t s) {
  if (M <= 0) return;
  t3_prephase_kernel<T><<<blocks_for(M, 256), 256, 0, s>>>(
      dim, xyz[0], dim > 1 ? xyz[1] : xyz[0], dim > 2 ? xyz[2] : xyz[0], M, D[0], D[1], D[2],
      isign, pre);
  GBN_LAUNCH_CHECK();
}

template <typename T>
void launch_t3_postfactor(int dim, const T *const stu[3], int N, const double C[3],
                          const double D[3], const double scale[3], int isign,
                          const QuadNodes &Q, cplx<T> *post, cudaStream_t s) {
  if (N <= 0) return;
  t3_post_kernel<T><<<blocks_for(N, 256), 256, 0, s>>>(
      dim, stu[0], dim > 1 ? stu[1] : stu[0], dim > 2 ? stu[2] : stu[0], N, C[0], C[1], C[2],
      D[0], D[1], D[2], scale[0], scale[1], scale[2], isign, Q, post);
  GBN_LAUNCH_CHECK();
}

namespace {
// Conflict-free shared-memory atomicAdd loop (f32, or int32 for the
// fixed-point tile): each warp adds into 32 consecutive words, so one
// instruction touches 32 distinct banks.
template <typename U> __global__ void smem_atomic_probe(float *out, int iters) {
  __shared__ U s[8192];
  for (int i = threadIdx.x; i < 8192; i += blockDim.x) s[i] = U(0);
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const U v = (U)(1.0f + threadIdx.x * 1e-3f);
#pragma unroll 4
  for (int it = 0; it < iters; ++it) atomicAdd(&s[(((it * 8 + w) * 32) & 8191) + lane], v);
  __syncthreads();
  if (threadIdx.x == 0) out[blockIdx.x] = (float)s[blockIdx.x & 8191];
}
} // namespace

double smem_atomic_rate(int device, bool i32) {
  auto probe = i32 ? smem_atomic_probe<int> : smem_atomic_probe<float>;
  int sms = 0;
  GBN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int grid = sms * 8, iters = 1 << 14;
  float *d = nullptr;
  GBN_CUDA(cudaMalloc(&d, (size_t)grid * sizeof(float)));
  cudaEvent_t a, b;
  GBN_CUDA(cudaEventCreate(&a));
  GBN_CUDA(cudaEventCreate(&b));
  probe<<<grid, 256>>>(d, iters); // warm-up
  GBN_CUDA(cudaEventRecord(a));
  probe<<<grid, 256>>>(d, iters);
  GBN_CUDA(cudaEventRecord(b));
  GBN_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  return (double)grid * 256.0 * iters / (ms * 1e-3);
}

#define GBN_INST(T)                                                                            \
  template void launch_inv_fseries<T>(int, const QuadNodes &, T *, cudaStream_t);            \
  template void launch_deconv<T>(int, const int[3], const int[3], int, const T *const[3],   \
                                 const cplx<T> *, int64_t, cplx<T> *, int, cudaStream_t);    \
  template void launch_amplify<T>(int, const int[3], const int[3], int, const T *const[3],  \
                                  const cplx<T> *, cplx<T> *, int64_t, int, cudaStream_t);   \
  template void array_range<T>(const T *, int, double *, double *, cudaStream_t);           \
  template void launch_t3_prephase<T>(int, const T *const[3], int, const double[3], int,    \
                                      cplx<T> *, cudaStream_t);                              \
  template void launch_t3_postfactor<T>(int, const T *const[3], int, const double[3],       \
                                        const double[3], const double[3], int,              \
                                        const QuadNodes &, cplx<T> *, cudaStream_t);
GBN_INST(float)
GBN_INST(double)

// iperm[perm[p]] = p: the inverse of the sort permutation, for the type-2
// gather from sorted-order results to user order
__global__ void invert_perm_kernel(const int *__restrict__ perm, int M, int *__restrict__ iperm) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < M; p += gridDim.x * blockDim.x)
    iperm[perm[p]] = p;
}
void launch_invert_perm(const int *perm, int M, int *iperm, cudaStream_t s) {
  if (M <= 0) return;
  const unsigned g = (unsigned)std::min<int64_t>((M + 255) / 256, 152 * 8);
  invert_perm_kernel<<<g, 256, 0, s>>>(perm, M, iperm);
  GBN_LAUNCH_CHECK();
}

} // namespace gbn
