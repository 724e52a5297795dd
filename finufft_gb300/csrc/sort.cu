// setpts on the device: fold-rescale, bin keys, a stable LSD radix sort of the
// points by bin, per-bin ranges and the subproblem table.
//
// The reference (include/cufinufft/spreadinterp.hpp:299-350,
// src/cuda/spread_subprob_inst.cu:136-181) ranks points inside a bin with
// global atomics, so its in-bin order changes from run to run. Here the sort is
// stable: points of one bin keep their input order, which is exactly the
// permutation a host counting sort produces (include/finufft/spread.hpp:459-584
// for the CPU library's bin ordering: x fastest, then y, then z).
#include "sort.h"

#include <map>
#include <mutex>

namespace gbn {

// ---------------------------------------------------------------- scan ----
namespace {
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

__global__ void scan_block_sums(const int *__restrict__ in, int64_t n, int *__restrict__ sums) {
  __shared__ int red[32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  int s = 0;
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int64_t i = base + (int64_t)j * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = red[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
  }
}

__global__ void scan_chunks(const int *__restrict__ in, int64_t n,
                            const int *__restrict__ chunk_off, int *__restrict__ out) {
  __shared__ int wexcl[32];
  __shared__ int wtot[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int sum = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int64_t i = base + j;
    v[j] = (i < n) ? in[i] : 0;
    sum += v[j];
  }
  // inclusive warp scan of thread sums
  int x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wtot[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = wtot[lane];
    int t = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    wexcl[lane] = t - s;
  }
  __syncthreads();
  int run = (chunk_off ? chunk_off[blockIdx.x] : 0) + wexcl[w] + (x - sum);
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int64_t i = base + j;
    if (i < n) out[i] = run;
    run += v[j];
  }
}
} // namespace

void exclusive_scan_i32(const int *in, int *out, int64_t n, cudaStream_t s, Arena *arena) {
  if (n <= 0) return;
  const int64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb == 1) {
    scan_chunks<<<1, SCAN_THREADS, 0, s>>>(in, n, nullptr, out);
    GBN_LAUNCH_CHECK();
    return;
  }
  AsyncBuf sums(nb * sizeof(int), s, arena), offs(nb * sizeof(int), s, arena);
  scan_block_sums<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums.as<int>());
  GBN_LAUNCH_CHECK();
  exclusive_scan_i32(sums.as<int>(), offs.as<int>(), nb, s, arena);
  scan_chunks<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, offs.as<int>(), out);
  GBN_LAUNCH_CHECK();
}

// ------------------------------------------------------------ bin keys ----
namespace {
// Sort key of a point: its bin (x fastest), times the bin volume, plus its
// cell inside the bin (x fastest) when cell_keys is set. Sorting by this key
// groups points by bin and, inside a bin, points that share a grid cell, so
// the spreader can sum such runs in registers.
template <typename T, int DIM>
__global__ void bin_key_kernel(const T *__restrict__ x, const T *__restrict__ y,
                               const T *__restrict__ z, int M, AxisMap a0, AxisMap a1,
                               AxisMap a2, int nb0, int nb1, int cell_keys,
                               uint32_t *__restrict__ keys, T *__restrict__ rec) {
  // cell_keys: 0 bin only, 1 bin and cell, 2 bin and start cell (the cell, or
  // the next one when the fraction is at least one half: where an odd-width
  // kernel's support starts), bin + 1 values per dimension
  const uint32_t ex = cell_keys == 2 ? 1u : 0u;
  const uint32_t binvol = ((uint32_t)a0.bin + ex) * (DIM > 1 ? (uint32_t)a1.bin + ex : 1u) *
                          (DIM > 2 ? (uint32_t)a2.bin + ex : 1u);
  // float coordinates on the identity map: single-precision fold and a
  // reciprocal division (exact below 2^20 cells after one correction step)
  const AxisMap am[3] = {a0, a1, a2};
  bool f32 = sizeof(T) == 4;
  for (int d = 0; d < DIM; ++d)
    f32 = f32 && am[d].shift == 0.0 && am[d].scale == 1.0 && am[d].nf < (1 << 20);
  if constexpr (sizeof(T) == 4) if (f32) {
    const T *const xs[3] = {x, y, z};
    float inv[3];
    for (int d = 0; d < DIM; ++d) inv[d] = 1.0f / (float)am[d].bin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
      T lc[4] = {T(0), T(0), T(0), T(0)};
      uint32_t key = 0, loc = 0, ks = 1, ls = 1;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        int c;
        float f;
        fold_cell_f32((float)xs[d][i], am[d].nf, c, f);
        const int b = am[d].bin;
        int q = __float2int_rz(__fmul_rn((float)c, inv[d]));
        int r = c - q * b;
        if (r < 0) {
          --q;
          r += b;
        } else if (r >= b) {
          ++q;
          r -= b;
        }
        key += ks * (uint32_t)q;
        loc += ls * ((uint32_t)r + (ex && f >= 0.5f ? 1u : 0u));
        ks *= (uint32_t)(d == 0 ? nb0 : nb1);
        ls *= (uint32_t)b + ex;
        lc[d] = (T)__fadd_rn((float)r, f);
      }
      keys[i] = cell_keys ? key * binvol + loc : key;
      if (rec) reinterpret_cast<float4 *>(rec)[i] = make_float4(lc[0], lc[1], lc[2], 0.f);
    }
    return;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    int c;
    double f;
    T lc[4] = {T(0), T(0), T(0), T(0)};
    auto cellkey = [&](int cm, double fr) {
      return (uint32_t)cm + (ex && fr >= 0.5 ? 1u : 0u);
    };
    fold_cell((double)x[i], a0, c, f);
    uint32_t key = (uint32_t)(c / a0.bin);
    uint32_t loc = cellkey(c - (c / a0.bin) * a0.bin, f);
    lc[0] = (T)((double)(c - (c / a0.bin) * a0.bin) + f);
    if (DIM > 1) {
      fold_cell((double)y[i], a1, c, f);
      key += (uint32_t)nb0 * (uint32_t)(c / a1.bin);
      loc += ((uint32_t)a0.bin + ex) * cellkey(c - (c / a1.bin) * a1.bin, f);
      lc[1] = (T)((double)(c - (c / a1.bin) * a1.bin) + f);
    }
    if (DIM > 2) {
      fold_cell((double)z[i], a2, c, f);
      key += (uint32_t)nb0 * (uint32_t)nb1 * (uint32_t)(c / a2.bin);
      loc += ((uint32_t)a0.bin + ex) * ((uint32_t)a1.bin + ex) *
             cellkey(c - (c / a2.bin) * a2.bin, f);
      lc[2] = (T)((double)(c - (c / a2.bin) * a2.bin) + f);
    }
    keys[i] = cell_keys ? key * binvol + loc : key;
    if (rec) { // bin-local coordinates of point i as one aligned 4-element record
      if constexpr (sizeof(T) == 4) {
        reinterpret_cast<float4 *>(rec)[i] = make_float4(lc[0], lc[1], lc[2], 0.f);
      } else {
        double2 *r2 = reinterpret_cast<double2 *>(rec) + 2 * (size_t)i;
        r2[0] = make_double2(lc[0], lc[1]);
        r2[1] = make_double2(lc[2], 0.0);
      }
    }
  }
}

// sorted bin-local coordinates gathered from the records the key pass wrote
// (one 16- or 32-byte record per point instead of a refold of x, y, z)
template <typename T, int DIM>
__global__ void gather_local_kernel(const T *__restrict__ rec, const int *__restrict__ perm,
                                    int M, T *__restrict__ l0, T *__restrict__ l1,
                                    T *__restrict__ l2) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < M; p += gridDim.x * blockDim.x) {
    const int i = perm[p];
    T a, b = T(0), c = T(0);
    if constexpr (sizeof(T) == 4) {
      const float4 v = reinterpret_cast<const float4 *>(rec)[i];
      a = v.x;
      b = v.y;
      c = v.z;
    } else {
      const double2 *r2 = reinterpret_cast<const double2 *>(rec) + 2 * (size_t)i;
      const double2 u = r2[0];
      a = u.x;
      b = u.y;
      if (DIM > 2) c = r2[1].x;
    }
    l0[p] = a;
    if (DIM > 1) l1[p] = b;
    if (DIM > 2) l2[p] = c;
  }
}

template <typename T, int DIM>
__global__ void sorted_local_kernel(const T *__restrict__ x, const T *__restrict__ y,
                                    const T *__restrict__ z, const int *__restrict__ perm,
                                    int M, AxisMap a0, AxisMap a1, AxisMap a2,
                                    T *__restrict__ l0, T *__restrict__ l1,
                                    T *__restrict__ l2) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < M; p += gridDim.x * blockDim.x) {
    const int i = perm[p];
    int c;
    double f;
    fold_cell((double)x[i], a0, c, f);
    l0[p] = (T)((double)(c - (c / a0.bin) * a0.bin) + f);
    if (DIM > 1) {
      fold_cell((double)y[i], a1, c, f);
      l1[p] = (T)((double)(c - (c / a1.bin) * a1.bin) + f);
    }
    if (DIM > 2) {
      fold_cell((double)z[i], a2, c, f);
      l2[p] = (T)((double)(c - (c / a2.bin) * a2.bin) + f);
    }
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 64) b = 152 * 64;
  return (unsigned)(b < 1 ? 1 : b);
}
} // namespace

template <typename T>
void launch_bin_keys(int dim, const T *const xyz[3], int M, const AxisMap ax[3],
                     const int nbin[3], int cell_keys, uint32_t *keys, cudaStream_t s,
                     T *rec) {
  if (M <= 0) return;
  const unsigned g = grid_for(M, 256);
  if (dim == 1)
    bin_key_kernel<T, 1><<<g, 256, 0, s>>>(xyz[0], xyz[0], xyz[0], M, ax[0], ax[0], ax[0],
                                           nbin[0], 1, cell_keys, keys, rec);
  else if (dim == 2)
    bin_key_kernel<T, 2><<<g, 256, 0, s>>>(xyz[0], xyz[1], xyz[1], M, ax[0], ax[1], ax[1],
                                           nbin[0], nbin[1], cell_keys, keys, rec);
  else
    bin_key_kernel<T, 3><<<g, 256, 0, s>>>(xyz[0], xyz[1], xyz[2], M, ax[0], ax[1], ax[2],
                                           nbin[0], nbin[1], cell_keys, keys, rec);
  GBN_LAUNCH_CHECK();
}

template <typename T>
void launch_gather_local(int dim, const T *rec, const int *perm, int M, T *const loc[3],
                         cudaStream_t s) {
  if (M <= 0) return;
  const unsigned g = grid_for(M, 256);
  if (dim == 1)
    gather_local_kernel<T, 1><<<g, 256, 0, s>>>(rec, perm, M, loc[0], loc[0], loc[0]);
  else if (dim == 2)
    gather_local_kernel<T, 2><<<g, 256, 0, s>>>(rec, perm, M, loc[0], loc[1], loc[1]);
  else
    gather_local_kernel<T, 3><<<g, 256, 0, s>>>(rec, perm, M, loc[0], loc[1], loc[2]);
  GBN_LAUNCH_CHECK();
}
template void launch_gather_local<float>(int, const float *, const int *, int,
                                         float *const[3], cudaStream_t);
template void launch_gather_local<double>(int, const double *, const int *, int,
                                          double *const[3], cudaStream_t);

template <typename T>
void launch_sorted_local(int dim, const T *const xyz[3], const int *perm, int M,
                         const AxisMap ax[3], T *const loc[3], cudaStream_t s) {
  if (M <= 0) return;
  const unsigned g = grid_for(M, 256);
  if (dim == 1)
    sorted_local_kernel<T, 1><<<g, 256, 0, s>>>(xyz[0], xyz[0], xyz[0], perm, M, ax[0], ax[0],
                                                ax[0], loc[0], loc[0], loc[0]);
  else if (dim == 2)
    sorted_local_kernel<T, 2><<<g, 256, 0, s>>>(xyz[0], xyz[1], xyz[1], perm, M, ax[0], ax[1],
                                                ax[1], loc[0], loc[1], loc[1]);
  else
    sorted_local_kernel<T, 3><<<g, 256, 0, s>>>(xyz[0], xyz[1], xyz[2], perm, M, ax[0], ax[1],
                                                ax[2], loc[0], loc[1], loc[2]);
  GBN_LAUNCH_CHECK();
}

template void launch_bin_keys<float>(int, const float *const[3], int, const AxisMap[3],
                                     const int[3], int, uint32_t *, cudaStream_t, float *);
template void launch_bin_keys<double>(int, const double *const[3], int, const AxisMap[3],
                                      const int[3], int, uint32_t *, cudaStream_t, double *);
template void launch_sorted_local<float>(int, const float *const[3], const int *, int,
                                         const AxisMap[3], float *const[3], cudaStream_t);
template void launch_sorted_local<double>(int, const double *const[3], const int *, int,
                                          const AxisMap[3], double *const[3], cudaStream_t);

// --------------------------------------------------------- radix sort ----
namespace {
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS; // 4096 keys per block
constexpr int RS_WARP_SPAN = RS_TILE / RS_WARPS; // 512 consecutive keys per warp

__global__ void radix_hist_kernel(const uint32_t *__restrict__ keys, int M, int shift,
                                  int ntiles, int *__restrict__ hist) {
  __shared__ int cnt[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int j = 0; j < RS_ITEMS; ++j) {
    const int64_t i = base + (int64_t)j * RS_THREADS + threadIdx.x;
    if (i < M) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x)
    hist[(int64_t)d * ntiles + blockIdx.x] = cnt[d];
}

// Stable scatter: rank of a key among equal digits of its tile follows index
// order (warp 0's 512 keys, then warp 1's, ...; inside a warp 32 keys per step).
__global__ void radix_scatter_kernel(const uint32_t *__restrict__ kin,
                                     const int *__restrict__ vin, uint32_t *__restrict__ kout,
                                     int *__restrict__ vout, int M, int shift, int ntiles,
                                     const int *__restrict__ offs) {
  __shared__ int wcnt[RS_WARPS][256];
  __shared__ int dstart[257];               // first tile position of each digit
  __shared__ uint32_t tk[RS_TILE];          // the tile's keys in (digit, input) order
  __shared__ int tv[RS_TILE];               // and their values
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += blockDim.x) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * RS_WARP_SPAN;
  const unsigned lt = (1u << lane) - 1u;
  uint32_t key[RS_ITEMS];
  int rank[RS_ITEMS];
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    const int64_t i = base + j * 32 + lane;
    const bool ok = i < M;
    const uint32_t k = ok ? kin[i] : 0u;
    const int d = ok ? (int)((k >> shift) & 255u) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    int r = 0;
    if (ok) r = wcnt[w][d] + __popc(peers & lt);
    __syncwarp();
    if (ok && (peers & lt) == 0u) wcnt[w][d] += __popc(peers);
    __syncwarp();
    key[j] = k;
    rank[j] = r;
  }
  __syncthreads();
  // per digit: warp offsets inside the digit, and the digit's tile total
  int total = 0;
  if (threadIdx.x < 256) {
    const int d = threadIdx.x;
#pragma unroll
    for (int ww = 0; ww < RS_WARPS; ++ww) {
      const int t = wcnt[ww][d];
      wcnt[ww][d] = total;
      total += t;
    }
  }
  // exclusive scan of the 256 digit totals (thread d holds digit d; 256 threads)
  {
    int v = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    __shared__ int wsum[RS_WARPS];
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    int add = 0;
    for (int ww = 0; ww < w; ++ww) add += wsum[ww];
    if (threadIdx.x < 256) dstart[threadIdx.x] = v - total + add;
  }
  __syncthreads();
  // reorder the tile by digit in shared memory (stable: ranks follow input order)
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    const int64_t i = base + j * 32 + lane;
    if (i < M) {
      const int d = (int)((key[j] >> shift) & 255u);
      const int t = dstart[d] + wcnt[w][d] + rank[j];
      tk[t] = key[j];
      tv[t] = vin ? vin[i] : (int)i;
    }
  }
  __syncthreads();
  // write out in tile order: consecutive threads store consecutive positions of
  // each digit's run
  const int64_t tile0 = (int64_t)blockIdx.x * RS_TILE;
  const int n = (int)min((int64_t)RS_TILE, (int64_t)M - tile0);
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const uint32_t k = tk[t];
    const int d = (int)((k >> shift) & 255u);
    const int pos = offs[(int64_t)d * ntiles + blockIdx.x] + (t - dstart[d]);
    kout[pos] = k;
    vout[pos] = tv[t];
  }
}

__global__ void iota_kernel(int *v, int M) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x)
    v[i] = i;
}
} // namespace

void stable_sort_by_bin(uint32_t *keys_in, int M, int keybits, uint32_t *keys_out,
                        int *perm_out, cudaStream_t s, Arena *arena) {
  if (M <= 0) return;
  const int passes = (keybits + 7) / 8;
  if (passes == 0) { // single bin: identity permutation
    iota_kernel<<<grid_for(M, 256), 256, 0, s>>>(perm_out, M);
    GBN_LAUNCH_CHECK();
    GBN_CUDA(cudaMemcpyAsync(keys_out, keys_in, (size_t)M * 4, cudaMemcpyDeviceToDevice, s));
    return;
  }
  const int ntiles = (int)(((int64_t)M + RS_TILE - 1) / RS_TILE);
  AsyncBuf hist((size_t)256 * ntiles * sizeof(int), s, arena);
  AsyncBuf offs((size_t)256 * ntiles * sizeof(int), s, arena);
  AsyncBuf ktmp((size_t)M * 4, s, arena), vtmp((size_t)M * 4, s, arena);
  // ping-pong so the last pass lands in (keys_out, perm_out)
  const uint32_t *ks = keys_in;
  const int *vs = nullptr; // pass 0 uses the identity as values
  for (int p = 0; p < passes; ++p) {
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t *kd = to_out ? keys_out : ktmp.as<uint32_t>();
    int *vd = to_out ? perm_out : vtmp.as<int>();
    const int shift = 8 * p;
    radix_hist_kernel<<<ntiles, RS_THREADS, 0, s>>>(ks, M, shift, ntiles, hist.as<int>());
    GBN_LAUNCH_CHECK();
    exclusive_scan_i32(hist.as<int>(), offs.as<int>(), (int64_t)256 * ntiles, s, arena);
    radix_scatter_kernel<<<ntiles, RS_THREADS, 0, s>>>(ks, vs, kd, vd, M, shift, ntiles,
                                                       offs.as<int>());
    GBN_LAUNCH_CHECK();
    ks = kd;
    vs = vd;
  }
}

// ----------------------------------------------------------- subproblems ----
namespace {
__global__ void bin_bounds_kernel(const uint32_t *__restrict__ sk, int M, uint32_t binvol,
                                  int *__restrict__ bstart, int *__restrict__ bend) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    const uint32_t b = sk[i] / binvol;
    if (i == 0 || sk[i - 1] / binvol != b) bstart[b] = i;
    if (i == M - 1 || sk[i + 1] / binvol != b) bend[b] = i + 1;
  }
}
__global__ void bin_nsub_kernel(const int *__restrict__ bstart, int *__restrict__ bend_to_cnt,
                                int *__restrict__ nsub, int nbins, int maxsub) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
    const int cnt = bend_to_cnt[b] - bstart[b];
    bend_to_cnt[b] = cnt;
    nsub[b] = (cnt + maxsub - 1) / maxsub;
  }
}
__global__ void fill_subproblems_kernel(const int *__restrict__ bstart, const int *__restrict__ bcnt,
                                        const int *__restrict__ nsub,
                                        const int *__restrict__ substart, int nbins, int maxsub,
                                        int *__restrict__ sbin, int *__restrict__ sstart,
                                        int *__restrict__ scount) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
    const int n = nsub[b], o = substart[b], st = bstart[b], c = bcnt[b];
    for (int k = 0; k < n; ++k) {
      sbin[o + k] = b;
      sstart[o + k] = st + k * maxsub;
      scount[o + k] = min(maxsub, c - k * maxsub);
    }
  }
}
} // namespace

cudaMemPool_t scratch_pool() {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  int dev = 0;
  GBN_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool;
  GBN_CUDA(cudaMemPoolCreate(&pool, &props));
  uint64_t keep = UINT64_MAX;
  GBN_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  pools[dev] = pool;
  return pool;
}

void trim_scratch_pool() {
  cudaMemPoolTrimTo(scratch_pool(), 0);
}

int build_subproblems(const uint32_t *sorted_keys, int M, int nbins, uint32_t binvol,
                      int maxsub, SubproblemArrays *out, cudaStream_t s, Arena *arena) {
  AsyncBuf bstart((size_t)nbins * 4, s, arena), bcnt((size_t)nbins * 4, s, arena),
      nsub((size_t)nbins * 4, s, arena), substart((size_t)nbins * 4, s, arena);
  GBN_CUDA(cudaMemsetAsync(bstart.p, 0, (size_t)nbins * 4, s));
  GBN_CUDA(cudaMemsetAsync(bcnt.p, 0, (size_t)nbins * 4, s));
  if (M > 0) {
    bin_bounds_kernel<<<grid_for(M, 256), 256, 0, s>>>(sorted_keys, M, binvol, bstart.as<int>(),
                                                       bcnt.as<int>());
    GBN_LAUNCH_CHECK();
  }
  bin_nsub_kernel<<<grid_for(nbins, 256), 256, 0, s>>>(bstart.as<int>(), bcnt.as<int>(),
                                                       nsub.as<int>(), nbins, maxsub);
  GBN_LAUNCH_CHECK();
  exclusive_scan_i32(nsub.as<int>(), substart.as<int>(), nbins, s, arena);
  int last[2] = {0, 0};
  GBN_CUDA(cudaMemcpyAsync(&last[0], substart.as<int>() + nbins - 1, 4, cudaMemcpyDeviceToHost, s));
  GBN_CUDA(cudaMemcpyAsync(&last[1], nsub.as<int>() + nbins - 1, 4, cudaMemcpyDeviceToHost, s));
  GBN_CUDA(cudaStreamSynchronize(s));
  const int total = last[0] + last[1];
  const size_t nalloc = (size_t)(total > 0 ? total : 1) * 4;
  if (arena) {
    out->bin = (int *)arena->take(nalloc);
    out->start = (int *)arena->take(nalloc);
    out->count = (int *)arena->take(nalloc);
  } else if (!out->bin || out->cap * 4 < nalloc) {
    if (out->bin) cudaFree(out->bin);
    if (out->start) cudaFree(out->start);
    if (out->count) cudaFree(out->count);
    out->bin = out->start = out->count = nullptr;
    out->cap = 0;
    GBN_CUDA(cudaMalloc(&out->bin, nalloc));
    GBN_CUDA(cudaMalloc(&out->start, nalloc));
    GBN_CUDA(cudaMalloc(&out->count, nalloc));
    out->cap = nalloc / 4;
  }
  fill_subproblems_kernel<<<grid_for(nbins, 256), 256, 0, s>>>(
      bstart.as<int>(), bcnt.as<int>(), nsub.as<int>(), substart.as<int>(), nbins, maxsub,
      out->bin, out->start, out->count);
  GBN_LAUNCH_CHECK();
  return total;
}

} // namespace gbn
