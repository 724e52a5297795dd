// Spreading and interpolation kernels, templated on precision, dimension and
// kernel width. Included by one translation unit per dimension.
//
// Both work on subproblems: a run of at most maxsubprobsize bin-sorted points
// that all fall in one bin, so their kernel supports lie in a tile of
// (bin + ns) cells per dimension whose origin is the bin origin minus
// floor(ns/2). A point's bin-local coordinate l is in [0, bin]; its first
// support cell in tile coordinates is s = ceil(l - ns/2) + floor(ns/2) in
// [0, bin] and its kernel weights are phi(ceil(l - ns/2) - l + j), j < ns.
#pragma once
#include <cuda.h>

#include <algorithm>
#include <cstdlib>
#include "device_util.cuh"
#include "spreadinterp.h"
#include "tile_layout.h"

namespace gbn {

template <int DIM> struct TileGeom {
  int t[3];    // tile extent per dimension (bin + ns, 1 beyond DIM)
  int org[3];  // global index of tile cell 0 per dimension (may be negative)
  int cells;
};

template <typename T, int DIM, int NS>
__device__ __forceinline__ TileGeom<DIM> tile_of(const PointLayout<T> &L, int b) {
  TileGeom<DIM> g;
  int bc[3] = {0, 0, 0};
  bc[0] = b % L.nbin[0];
  if (DIM > 1) bc[1] = (b / L.nbin[0]) % L.nbin[1];
  if (DIM > 2) bc[2] = b / (L.nbin[0] * L.nbin[1]);
  g.cells = 1;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (d < DIM) {
      g.t[d] = L.bin[d] + NS;
      g.org[d] = bc[d] * L.bin[d] - NS / 2;
    } else {
      g.t[d] = 1;
      g.org[d] = 0;
    }
    g.cells *= g.t[d];
  }
  return g;
}

// periodic wrap of a global index that may be slightly outside [0, n)
__device__ __forceinline__ int wrap_idx(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// periodic index for i in [-n, 2n); used when the tile is not longer than the grid
__device__ __forceinline__ int wrap_once(int i, int n) {
  return i < 0 ? i + n : (i >= n ? i - n : i);
}

// Geometry of the problem a subproblem belongs to: for a batch, replaces the
// layout's grid and bin counts by the problem's and returns its grid offset;
// b becomes the bin index inside the problem.
template <typename T>
__device__ __forceinline__ int64_t resolve_problem(const PointLayout<T> &L, PointLayout<T> &Lb,
                                                   int &b) {
  Lb = L;
  if (!L.probs) return 0;
  const BatchProb P = L.probs[L.binprob[b]];
  b -= P.binoff;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    Lb.nf[d] = P.nf[d];
    Lb.nbin[d] = P.nbin[d];
  }
  return P.gridoff;
}

// first support cell (tile coordinates) and kernel weights of one point (the
// even/odd evaluation of mirrored Horner pieces: 3D single-precision spread
// 14.82 -> 13.89 ms per 1e8 clustered points against one Horner per piece)
template <typename T, int NS>
__device__ __forceinline__ int point_weights(T l, int binsz, const KernelShape<T> &K, T *ker) {
  const T sd = ceil(l - T(NS) * T(0.5));
  int s = (int)sd + NS / 2;
  s = s < 0 ? 0 : (s > binsz ? binsz : s);
  eval_kernel_sym<T, NS>(ker, sd - l, K);
  return s;
}

// ---------------------------------------------------------------------------
// Method 2: tiled spreading in shared memory. The tile is planar (all real
// parts, then all imaginary parts) so that consecutive cells sit in
// consecutive banks. 3D uses one warp per point: lanes cover an 8 x 4 (x, y)
// patch of the point's support, so the 32 atomics of one instruction hit 32
// distinct banks (row pitch = 8 mod 32). 1D and 2D use one thread per point.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(256)
    spread_tile_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ c,
                       const cplx<T> *__restrict__ pre, int conj_pre,
                       cplx<T> *__restrict__ fw, int64_t nf_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sub = blockIdx.x;
  const int tr = blockIdx.y;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<DIM> G = tile_of<T, DIM, NS>(L, b);
  // padded pitches (3D: x pitch = 8 mod 32 words so 4 rows hit disjoint bank octets)
  const int px = tile_pitch_x(DIM, G.t[0]);
  const int py = G.t[1];
  const int ncell_pad = px * py * G.t[2];
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + ncell_pad;
  for (int i = threadIdx.x; i < ncell_pad; i += blockDim.x) {
    re[i] = T(0);
    im[i] = T(0);
  }
  __syncthreads();
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  if constexpr (DIM < 3) {
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const int p = p0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      T kx[NS], ky[NS];
      const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, kx);
      if constexpr (DIM == 1) {
#pragma unroll
        for (int a = 0; a < NS; ++a) {
          atomicAdd(re + sx + a, v.x * kx[a]);
          atomicAdd(im + sx + a, v.y * kx[a]);
        }
      } else {
        const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, ky);
#pragma unroll
        for (int bb = 0; bb < NS; ++bb) {
          const T wr = v.x * ky[bb], wi = v.y * ky[bb];
          const int row = (sy + bb) * px + sx;
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            atomicAdd(re + row + a, wr * kx[a]);
            atomicAdd(im + row + a, wi * kx[a]);
          }
        }
      }
    }
  } else {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarp = blockDim.x >> 5;
    const int lx = lane & 7;  // x offset in the support
    const int ly = lane >> 3; // y offset within a group of 4 rows
    for (int i = warp; i < np; i += nwarp) {
      const int p = p0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      T kx[NS], ky[NS], kz[NS];
      const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, kx);
      const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, ky);
      const int sz = point_weights<T, NS>(L.loc[2][p], L.bin[2], K, kz);
      // this lane's x weight (lanes with lx >= NS idle)
      T wx = T(0);
#pragma unroll
      for (int a = 0; a < NS; ++a)
        if (a == lx) wx = kx[a];
#pragma unroll
      for (int yb = 0; yb < (NS + 3) / 4; ++yb) {
        const int yy = yb * 4 + ly;
        T wy = T(0);
#pragma unroll
        for (int a = 0; a < NS; ++a)
          if (a == yy) wy = ky[a];
        const bool on = (lx < NS) && (yy < NS);
        const T wxy = wx * wy;
        const int base = (sy + yy) * px + sx + lx;
#pragma unroll
        for (int zz = 0; zz < NS; ++zz) {
          if (on) {
            const T w = wxy * kz[zz];
            const int q = base + (sz + zz) * (px * py);
            atomicAdd(re + q, v.x * w);
            atomicAdd(im + q, v.y * w);
          }
        }
      }
    }
  }
  __syncthreads();
  // write the tile back: every tile cell adds into its periodic image
  cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
  for (int q = threadIdx.x; q < G.cells; q += blockDim.x) {
    const int x = q % G.t[0];
    const int y = (q / G.t[0]) % G.t[1];
    const int z = q / (G.t[0] * G.t[1]);
    const int sidx = (z * py + y) * px + x;
    cplx<T> v;
    v.x = re[sidx];
    v.y = im[sidx];
    int64_t g = wrap_idx(G.org[0] + x, L.nf[0]);
    if (DIM > 1) g += (int64_t)L.nf[0] * wrap_idx(G.org[1] + y, L.nf[1]);
    if (DIM > 2) g += (int64_t)L.nf[0] * L.nf[1] * wrap_idx(G.org[2] + z, L.nf[2]);
    atomic_add_cplx_global(fwt + g, v);
  }
}

// ---------------------------------------------------------------------------
// Method 3, output-driven spreading (the reference's gpu_method 3,
// src/cuda/spread_output_driven_inst.cu:17-158): the subproblem's points are
// staged in batches of OD_BATCH with their kernel weights, then taken one at a
// time, the block's threads splitting that point's ns^d support cells among
// themselves, so every cell has one writer and the tile takes plain adds (a
// block barrier between points); the tile is then added into the grid.
constexpr int OD_BATCH = 64;
constexpr int OD_THREADS = 256;

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(OD_THREADS)
    spread_output_driven_kernel(PointLayout<T> L0, KernelShape<T> K,
                                const cplx<T> *__restrict__ c, const cplx<T> *__restrict__ pre,
                                int conj_pre, cplx<T> *__restrict__ fw, int64_t nf_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sub = blockIdx.x;
  const int tr = blockIdx.y;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<DIM> G = tile_of<T, DIM, NS>(L, b);
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + G.cells;
  T *kw = im + G.cells;                        // [OD_BATCH][DIM][NS]
  T *vr = kw + OD_BATCH * DIM * NS;            // [OD_BATCH]
  T *vi = vr + OD_BATCH;                       // [OD_BATCH]
  int *st = reinterpret_cast<int *>(vi + OD_BATCH); // [OD_BATCH][DIM] start cells
  for (int i = threadIdx.x; i < G.cells; i += blockDim.x) {
    re[i] = T(0);
    im[i] = T(0);
  }
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  constexpr int TOTAL = DIM == 1 ? NS : (DIM == 2 ? NS * NS : NS * NS * NS);
  for (int b0 = 0; b0 < np; b0 += OD_BATCH) {
    const int nb = min(OD_BATCH, np - b0);
    __syncthreads(); // the previous batch's readers are done (and the tile is zeroed)
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      const int p = p0 + b0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      vr[i] = v.x;
      vi[i] = v.y;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        T kk[NS];
        st[i * DIM + d] = point_weights<T, NS>(L.loc[d][p], L.bin[d], K, kk);
#pragma unroll
        for (int a = 0; a < NS; ++a) kw[(i * DIM + d) * NS + a] = kk[a];
      }
    }
    __syncthreads();
    for (int i = 0; i < nb; ++i) {
      const T *k = kw + i * DIM * NS;
      for (int idx = threadIdx.x; idx < TOTAL; idx += blockDim.x) {
        const int dx = idx % NS;
        int t = dx + st[i * DIM];
        T w = k[dx];
        if (DIM > 1) {
          const int dy = (idx / NS) % NS;
          w *= k[NS + dy];
          t += G.t[0] * (dy + st[i * DIM + 1]);
        }
        if (DIM > 2) {
          const int dz = idx / (NS * NS);
          w *= k[2 * NS + dz];
          t += G.t[0] * G.t[1] * (dz + st[i * DIM + 2]);
        }
        re[t] += vr[i] * w;
        im[t] += vi[i] * w;
      }
      __syncthreads(); // the next point's support may overlap this one's
    }
  }
  __syncthreads();
  cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
  for (int q = threadIdx.x; q < G.cells; q += blockDim.x) {
    cplx<T> v;
    v.x = re[q];
    v.y = im[q];
    if (v.x == T(0) && v.y == T(0)) continue;
    const int x = q % G.t[0];
    int64_t g = wrap_idx(G.org[0] + x, L.nf[0]);
    if (DIM > 1) g += (int64_t)L.nf[0] * wrap_idx(G.org[1] + (q / G.t[0]) % G.t[1], L.nf[1]);
    if (DIM > 2) g += (int64_t)L.nf[0] * L.nf[1] * wrap_idx(G.org[2] + q / (G.t[0] * G.t[1]), L.nf[2]);
    atomic_add_cplx_global(fwt + g, v);
  }
}

// ---------------------------------------------------------------------------
// Method 2 in 3D: tiled spreading with warp-cooperative, bank-conflict-free
// shared-memory atomics.
//  * Each warp takes 32 points at a time: lane l loads point l (coalesced),
//    evaluates its 3*NS kernel weights once and stages them, the start cell
//    and the strength in a per-warp shared-memory area.
//  * The warp then adds the 32 points one after another. Lane (lx, lp) =
//    (lane & 7, lane >> 3) covers x offset dx = 8*xb + lx and the (y, z)
//    offset pair number 4*r + lp of the NS*NS pairs, i.e. an 8-cell x run
//    for 4 consecutive (y, z) pairs per instruction (75% of lanes busy at
//    NS = 6, against 56% for a fixed 8 x 4 (x, y) patch).
//  * Pitches are chosen so those 32 cells sit in 32 distinct banks: the x
//    pitch px is 8 mod 16 and the y extent is padded to py = NS mod 4, which
//    makes the word offset of pair p congruent to px*p mod 32.
// Returns of the kernel are identical to the other spreaders up to the
// order of floating-point additions.
template <typename T, int NS>
__global__ void __launch_bounds__(256)
    spread_tile3_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ c,
                        const cplx<T> *__restrict__ pre, int conj_pre,
                        cplx<T> *__restrict__ fw, int64_t nf_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SK = STAGE_STRIDE;
  constexpr int NXB = (NS + 7) / 8;
  constexpr int NPAIR = NS * NS;
  constexpr int NROUND = (NPAIR + 3) / 4;
  const int sub = blockIdx.x;
  const int tr = blockIdx.y;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<3> G = tile_of<T, 3, NS>(L, b);
  const int px = tile_pitch_x(3, G.t[0]);
  const int py = tile3_py(G.t[1], NS);
  const int Q = px * py;
  const int ncell = Q * G.t[2];
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + ncell;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  unsigned char *stage = smem_raw + tile3_bytes<T>(NS, L.bin[0], L.bin[1], L.bin[2]) +
                         (size_t)warp * stage_bytes_per_warp<T>(NS);
  T *kx = reinterpret_cast<T *>(stage);
  T *ky = kx + NS * SK;
  T *kz = ky + NS * SK;
  T *vre = kz + NS * SK;
  T *vim = vre + SK;
  int *spk = reinterpret_cast<int *>(vim + SK);
  for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
    re[i] = T(0);
    im[i] = T(0);
  }
  __syncthreads();
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  const int lx = lane & 7, lp = lane >> 3;
  for (int base = warp * 32; base < np; base += nwarp * 32) {
    const int i = base + lane;
    if (i < np) {
      const int p = p0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      T kk[NS];
      const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, kk);
#pragma unroll
      for (int a = 0; a < NS; ++a) kx[a * SK + lane] = kk[a];
      const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, kk);
#pragma unroll
      for (int a = 0; a < NS; ++a) ky[a * SK + lane] = kk[a];
      const int sz = point_weights<T, NS>(L.loc[2][p], L.bin[2], K, kk);
#pragma unroll
      for (int a = 0; a < NS; ++a) kz[a * SK + lane] = kk[a];
      vre[lane] = v.x;
      vim[lane] = v.y;
      spk[lane] = sx | (sy << 10) | (sz << 20);
    }
    __syncwarp();
    const int cnt = min(32, np - base);
    for (int q = 0; q < cnt; ++q) {
      const int sp = spk[q];
      const int rowbase = (sp >> 20) * Q + ((sp >> 10) & 1023) * px + (sp & 1023);
      const T vr = vre[q], vi = vim[q];
#pragma unroll
      for (int xb = 0; xb < NXB; ++xb) {
        const int dx = xb * 8 + lx;
        const bool xin = dx < NS;
        const T wx = kx[dx * SK + q]; // dx >= NS reads (unused) staged y weights
        const T ar = vr * wx, ai = vi * wx;
#pragma unroll
        for (int r = 0; r < NROUND; ++r) {
          const int pp = 4 * r + lp;
          if (xin && pp < NPAIR) {
            const int dy = pp % NS, dz = pp / NS;
            const T w = ky[dy * SK + q] * kz[dz * SK + q];
            const int a = rowbase + dz * Q + dy * px + dx;
            atomicAdd(re + a, ar * w);
            atomicAdd(im + a, ai * w);
          }
        }
      }
    }
    __syncwarp();
  }
  __syncthreads();
  cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
  for (int q = threadIdx.x; q < G.cells; q += blockDim.x) {
    const int x = q % G.t[0];
    const int y = (q / G.t[0]) % G.t[1];
    const int z = q / (G.t[0] * G.t[1]);
    const int sidx = z * Q + y * px + x;
    cplx<T> v;
    v.x = re[sidx];
    v.y = im[sidx];
    const int64_t g = wrap_idx(G.org[0] + x, L.nf[0]) +
                      (int64_t)L.nf[0] * (wrap_idx(G.org[1] + y, L.nf[1]) +
                                          (int64_t)L.nf[1] * wrap_idx(G.org[2] + z, L.nf[2]));
    atomic_add_cplx_global(fwt + g, v);
  }
}

// ---------------------------------------------------------------------------
// Method 2 in 3D, double precision: variant 4, an int64 fixed-point tile with
// integer products. GB300 issues FP64 at a small fraction of its integer and
// FP32 rates, and shared-memory double atomics are compare-and-swap loops
// around an FP64 add, so a double spread that forms and adds its 2 ns^3
// per-point updates (4394 at ns = 13) in FP64 is bound by the FP64 pipe.
// Here the per-cell work is integer only:
//  - each block sums S = sum_j (|Re c_j| + |Im c_j|) over its subproblem; a
//    tile cell's sum is at most S (kernel values are at most 1; margin 1.01),
//    so the tile holds round(value * 2^e) in int64 with 2^e <= 2^62 / (1.01 S),
//    summed by native 64-bit integer shared-memory adds;
//  - per point (FP64, ~3 ns Horner evaluations): U_z = round(c 2^e phi_z) as
//    int64 and the y and x weights as 62-bit fractions W = round(phi 2^62);
//  - per (y, z) row of the support a lane forms U_zy = U_z W_y / 2^64 and per
//    cell U_zy W_x / 2^64, each from three 32 x 32-bit integer multiplies
//    (mulfix below); the tile then holds sums of c phi 2^(e-4).
// Each contribution carries the double products' relative error (2^-53) plus
// a few units of S 2^-58 from the truncated products: double-precision
// accuracy. Subproblems whose S is not finite or needs 2^e beyond 2^1000 sum
// doubles (strengths scaled by a power of two) in the same tile instead.
// The block's threads each own one (y, z) row of the support for a range of
// the subproblem's points and sum it in registers over runs of points that
// share their start cells; staged points come in two alternating buffers, so
// the next points' FP64 weights are computed while the current ones are added.

// u W / 2^64 for |u| <= 2^62 and W = wh 2^32 + wl (0 <= wh <= 2^30 + 1, wl
// unsigned): uh wh + hi(uh wl) + hi(ul wh) + 1 from one wide and two high
// 32-bit multiplies (hi: the high word of a 32 x 32-bit product; uh signed, so
// hi(uh wl) = hi of the unsigned product minus wl when uh < 0). The high words
// floor and the dropped ul wl / 2^64 lies in [0, 1); the constant 1 centres
// the error (exact-integer emulation: |error| < 2 units, mean -0.06 units)
__device__ __forceinline__ long long mulfix(long long u, int wh, unsigned wl) {
  const int uh = (int)(u >> 32);
  const unsigned ul = (unsigned)u;
  const unsigned neg = (unsigned)(uh >> 31);
  const long long t1 = (long long)uh * wh;
  const int t2 = (int)(__umulhi((unsigned)uh, wl) - (wl & neg));
  const unsigned t3 = __umulhi(ul, (unsigned)wh);
  return t1 + (long long)t2 + (long long)t3 + 1;
}
// acc += u W / 2^64 - 1 (mulfix without its centring constant, which a run
// adds once per point at its flush), with u given as its words (uh, ul) and
// neg = uh >> 31; one wide and two high multiplies and a carry chain
__device__ __forceinline__ void mulfix_acc(long long &acc, int uh, unsigned ul, unsigned neg,
                                           int wh, unsigned wl) {
  asm("{\n\t"
      ".reg .u32 t2, t3, m, s2, alo, ahi, plo, phi;\n\t"
      ".reg .s64 t1;\n\t"
      "mul.wide.s32 t1, %1, %4;\n\t"
      "mul.hi.u32 t2, %1, %5;\n\t"
      "and.b32 m, %5, %3;\n\t"
      "sub.u32 t2, t2, m;\n\t"
      "mul.hi.u32 t3, %2, %4;\n\t"
      "shr.s32 s2, t2, 31;\n\t"
      "mov.b64 {alo, ahi}, %0;\n\t"
      "mov.b64 {plo, phi}, t1;\n\t"
      "add.cc.u32 alo, alo, plo;\n\t"
      "addc.u32 ahi, ahi, phi;\n\t"
      "add.cc.u32 alo, alo, t2;\n\t"
      "addc.u32 ahi, ahi, s2;\n\t"
      "add.cc.u32 alo, alo, t3;\n\t"
      "addc.u32 ahi, ahi, 0;\n\t"
      "mov.b64 %0, {alo, ahi};\n\t"
      "}"
      : "+l"(acc)
      : "r"(uh), "r"(ul), "r"(neg), "r"(wh), "r"(wl));
}
// a weight as the (wh, wl) words of round(w 2^62); fitted kernel values can
// dip a few ulps below zero at the support's edge, and are clamped to 0
__device__ __forceinline__ int2 wfix(double w) {
  const long long v = __double2ll_rn(fmax(w, 0.0) * 0x1p62);
  return make_int2((int)(v >> 32), (int)(unsigned)v);
}

template <int NS>
__global__ void __launch_bounds__(T3X_THREADS, 1)
    spread_tile3x_kernel(PointLayout<double> L0, KernelShape<double> K,
                         const double2 *__restrict__ c, const double2 *__restrict__ pre,
                         int conj_pre, double2 *__restrict__ fw, int64_t nf_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[16];
  __shared__ int mode; // 0: fixed point, 1: double atomics, 2: all strengths zero
  __shared__ double scale_d, inv_scale;
  constexpr int SB = t3x_sb(NS);
  constexpr int PS = t3x_point_bytes(NS);
  constexpr int NPAIR = NS * NS;
  const int sub = blockIdx.x;
  const int tr = blockIdx.y;
  int b = L0.sub_bin[sub];
  PointLayout<double> Lg;
  const int64_t goff = resolve_problem<double>(L0, Lg, b);
  const PointLayout<double> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  if (np <= 0) return;
  const TileGeom<3> G = tile_of<double, 3, NS>(L, b);
  const int px = G.t[0], py = G.t[1];
  const int Q = px * py;
  const int ncell = Q * G.t[2];
  long long *ire = reinterpret_cast<long long *>(smem_raw);
  long long *iim = ire + ncell;
  double *dre = reinterpret_cast<double *>(ire), *dim_ = reinterpret_cast<double *>(iim);
  unsigned char *stg0 = smem_raw + t3x_tile_bytes(ncell);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const double2 *ct = c + (int64_t)tr * L.M;
  // the subproblem's strength sum S, and the tile's scale
  double part = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int j = L.perm[p0 + i];
    double2 v = ct[j];
    if (pre) v = cmul_opt<double>(v, pre[j], conj_pre);
    part += fabs(v.x) + fabs(v.y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) red[warp] = part;
  {
    uint4 *z4 = reinterpret_cast<uint4 *>(smem_raw);
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < ncell; i += blockDim.x) { // 2 ncell int64 = ncell uint4
      z4[i] = zero;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0;
    for (int w = 0; w < nwarp; ++w) S += red[w];
    int m = 2, e = 0;
    if (!(S < 1e300)) {
      m = 1; // inf or NaN strengths: IEEE propagation (scale 1)
    } else if (S > 0.0) {
      m = 0;
      e = 62 - (int)ceil(log2(1.01 * S));
      if (e > 1000) { // S below about 2^-938: doubles, strengths scaled to at most 1
        m = 1;
        e = -(int)ceil(log2(S));
      }
    }
    mode = m;
    scale_d = ldexp(1.0, e);
    // the two products divide by 2^64 against weights scaled by 2^62
    inv_scale = ldexp(1.0, m == 0 ? 4 - e : -e);
  }
  __syncthreads();
  if (mode == 2) return; // nothing to add (mulfix's offset would not be zero)
  const bool fx = mode == 0;
  const double sc = scale_d;
  // Work split: thread t owns support row r = t % NPAIR (y = r % NS, z =
  // r / NS) for group g = t / NPAIR. The subproblem's points are cut into NG
  // contiguous ranges, one per group, staged SBG per group and batch. A
  // thread sums its row's NS cells over consecutive points that share their
  // start cells in registers and adds the sums to the tile when the start
  // cells change (points are sorted by bin and cell, and clustered points
  // often share cells), instead of one 64-bit shared add per cell and point.
  constexpr int NG = T3X_THREADS / NPAIR; // groups of the block (launched with T3X_THREADS)
  constexpr int SBG = SB / NG;    // points per group and batch
  constexpr int NSLOT = NG * SBG;
  static_assert(NG >= 1 && SBG >= 1, "staging holds a point per group");
  const int chunk = (np + NG - 1) / NG;
  const int nbatch = (chunk + SBG - 1) / SBG;
  // stage batch bt into buffer k: item t < 3 NSLOT computes dimension
  // t / NSLOT of slot t % NSLOT (the z weights also give U_z). The items go
  // to a multiple of four warps (IPW lanes each), so that the FP64 work is
  // spread over the SM's four schedulers and their FP64 units
  constexpr int NSTW = 4 * ((3 * NSLOT + 127) / 128), IPW = (3 * NSLOT + NSTW - 1) / NSTW;
  static_assert(NSTW <= 16 && IPW <= 32, "staging items exceed the block");
  auto stage = [&](int bt, int k) {
    unsigned char *stg = stg0 + (size_t)k * SB * PS;
    const int t = warp * IPW + lane;
    if (warp < NSTW && lane < IPW && t < 3 * NSLOT) {
      const int sl = t % NSLOT, d = t / NSLOT;
      const int g = sl / SBG, i = g * chunk + bt * SBG + (sl - g * SBG);
      if (i < min(np, (g + 1) * chunk)) {
        const int p = p0 + i;
        double kk[NS];
        // (selects, not a runtime index into the layout, which would copy it
        // to local memory)
        const double *ld = d == 0 ? L.loc[0] : (d == 1 ? L.loc[1] : L.loc[2]);
        const int bd = d == 0 ? L.bin[0] : (d == 1 ? L.bin[1] : L.bin[2]);
        const double l = ld[p];
        const double sd = ceil(l - double(NS) * 0.5);
        const int s = min(max((int)sd + NS / 2, 0), bd); // as point_weights
        eval_kernel_sym<double, NS>(kk, sd - l, K);
        unsigned char *P = stg + (size_t)sl * PS;
        if (d == 2) {
          const int j = L.perm[p];
          double2 v = ct[j];
          if (pre) v = cmul_opt<double>(v, pre[j], conj_pre);
          const double vr = v.x * sc, vi = v.y * sc;
          longlong2 *U = reinterpret_cast<longlong2 *>(P);
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            if (fx)
              U[a] = make_longlong2(__double2ll_rn(vr * kk[a]), __double2ll_rn(vi * kk[a]));
            else
              U[a] = make_longlong2(__double_as_longlong(vr * kk[a]),
                                    __double_as_longlong(vi * kk[a]));
          }
        } else {
          int2 *W = reinterpret_cast<int2 *>(P + 16 * NS + 8 * NS * d); // x: 16 NS, y: 24 NS
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            if (fx) {
              W[a] = wfix(kk[a]);
            } else {
              const long long bits = __double_as_longlong(kk[a]);
              W[a] = make_int2((int)(bits >> 32), (int)bits);
            }
          }
        }
        // start cell of dimension d (one word each: no read-modify-write
        // between the three threads of a point)
        reinterpret_cast<int *>(P + 32 * NS)[d] = s;
      }
    }
  };
  const int r = threadIdx.x % NPAIR, grp = threadIdx.x / NPAIR;
  const int dy = r % NS, dz = r / NS;
  const int gbeg = grp * chunk, gend = min(np, gbeg + chunk);
  long long accr[NS], acci[NS]; // the run's row sums (mode 1: double bits)
  int cur = -1;                 // the run's start cells, x | y << 10 | z << 20
  int nrun = 0;                 // points in the run (mulfix_acc's offsets)
  auto flush = [&]() {
    const int row = ((cur >> 20) + dz) * Q + (((cur >> 10) & 1023) + dy) * px + (cur & 1023);
#pragma unroll
    for (int a = 0; a < NS; ++a) {
      if (fx) {
        atomicAdd(reinterpret_cast<unsigned long long *>(ire + row + a),
                  (unsigned long long)(accr[a] + nrun));
        atomicAdd(reinterpret_cast<unsigned long long *>(iim + row + a),
                  (unsigned long long)(acci[a] + nrun));
      } else {
        atomicAdd(dre + row + a, __longlong_as_double(accr[a]));
        atomicAdd(dim_ + row + a, __longlong_as_double(acci[a]));
      }
    }
  };
  stage(0, 0);
  __syncthreads();
  int k = 0;
  for (int bt = 0; bt < nbatch; ++bt, k ^= 1) {
    if (bt + 1 < nbatch) stage(bt + 1, k ^ 1);
    const unsigned char *stg = stg0 + (size_t)k * SB * PS;
    if (grp < NG) {
      const int cnt = min(SBG, gend - (gbeg + bt * SBG)); // may be <= 0
      for (int i = 0; i < cnt; ++i) {
        const unsigned char *P = stg + (size_t)(grp * SBG + i) * PS;
        const int4 s4 = *reinterpret_cast<const int4 *>(P + 32 * NS);
        const int sp = s4.x | (s4.y << 10) | (s4.z << 20);
        if (sp != cur) {
          if (cur >= 0) flush();
#pragma unroll
          for (int a = 0; a < NS; ++a) accr[a] = acci[a] = 0;
          cur = sp;
          nrun = 0;
        }
        ++nrun;
        const longlong2 U = reinterpret_cast<const longlong2 *>(P)[dz];
        const int2 wy = reinterpret_cast<const int2 *>(P + 24 * NS)[dy];
        const int2 *wx = reinterpret_cast<const int2 *>(P + 16 * NS);
        if (fx) {
          const long long ur = mulfix(U.x, wy.x, (unsigned)wy.y);
          const long long ui = mulfix(U.y, wy.x, (unsigned)wy.y);
          const int urh = (int)(ur >> 32), uih = (int)(ui >> 32);
          const unsigned url = (unsigned)ur, uil = (unsigned)ui;
          const unsigned urn = (unsigned)(urh >> 31), uin = (unsigned)(uih >> 31);
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            const int2 w = wx[a];
            mulfix_acc(accr[a], urh, url, urn, w.x, (unsigned)w.y);
            mulfix_acc(acci[a], uih, uil, uin, w.x, (unsigned)w.y);
          }
        } else {
          const double fy = __longlong_as_double(((long long)wy.x << 32) | (unsigned)wy.y);
          const double ur = __longlong_as_double(U.x) * fy, ui = __longlong_as_double(U.y) * fy;
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            const int2 w = wx[a];
            const double f = __longlong_as_double(((long long)w.x << 32) | (unsigned)w.y);
            accr[a] = __double_as_longlong(__longlong_as_double(accr[a]) + ur * f);
            acci[a] = __double_as_longlong(__longlong_as_double(acci[a]) + ui * f);
          }
        }
      }
    }
    __syncthreads();
  }
  if (grp < NG && cur >= 0) flush();
  __syncthreads();
  double2 *fwt = fw + (int64_t)tr * nf_total + goff;
  const double is = inv_scale;
  for (int q = threadIdx.x; q < G.cells; q += blockDim.x) {
    const int x = q % G.t[0];
    const int y = (q / G.t[0]) % G.t[1];
    const int z = q / (G.t[0] * G.t[1]);
    const int sidx = z * Q + y * px + x;
    double2 v;
    if (fx) {
      const long long a = ire[sidx], bb = iim[sidx];
      if ((a | bb) == 0) continue;
      v.x = (double)a * is;
      v.y = (double)bb * is;
    } else {
      v.x = dre[sidx] * is;
      v.y = dim_[sidx] * is;
      if (v.x == 0.0 && v.y == 0.0) continue;
    }
    const int64_t g = wrap_idx(G.org[0] + x, L.nf[0]) +
                      (int64_t)L.nf[0] * (wrap_idx(G.org[1] + y, L.nf[1]) +
                                          (int64_t)L.nf[1] * wrap_idx(G.org[2] + z, L.nf[2]));
    atomic_add_cplx_global(fwt + g, v);
  }
}

// threads of the warp-aggregated 3D spread: 12 warps share a tile in single
// precision, 8 in double (twice the accumulator registers); 2 blocks per SM
template <typename T> __host__ __device__ constexpr int t3m_threads() {
  return sizeof(T) == 8 ? 256 : 384;
}

// ---------------------------------------------------------------------------
// Method 2 in 3D, warp-aggregated variant: the tile is shared by the block's
// warps (atomics, as in spread_tile3_kernel), but each warp takes a contiguous
// range of the (bin, cell)-sorted points and sums the contributions of a run
// of points with the same first support cell in registers, issuing the tile
// atomics once per run instead of once per point. Staging and lane mapping
// are those of spread_tile3_kernel.
template <typename T, int NS>
__global__ void __launch_bounds__(t3m_threads<T>(), 2)
    spread_tile3m_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ c,
                         const cplx<T> *__restrict__ pre, int conj_pre,
                         cplx<T> *__restrict__ fw, int64_t nf_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SK = STAGE_STRIDE;
  constexpr int NXB = (NS + 7) / 8;
  constexpr int NR = (NS * NS + 3) / 4;
  constexpr int NSLOT = NXB * NR;
  const int sub = blockIdx.x;
  const int tr = blockIdx.y;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<3> G = tile_of<T, 3, NS>(L, b);
  const int px = tile_pitch_x(3, G.t[0]);
  const int py = tile3_py(G.t[1], NS);
  const int Q = px * py;
  const size_t tile_bytes = tile3_bytes<T>(NS, L.bin[0], L.bin[1], L.bin[2]);
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + Q * G.t[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  // per-warp staging: x weights, (y,z) weight products (NS*NS rows padded to
  // 4*NR), strengths and packed start cells of 32 points
  T *kx = reinterpret_cast<T *>(smem_raw + tile_bytes +
                                (size_t)warp * t3m_stage_bytes(NS, (int)sizeof(T)));
  T *yz = kx + NS * SK;
  T *vre = yz + 4 * NR * SK;
  T *vim = vre + SK;
  int *spk = reinterpret_cast<int *>(vim + SK);
  {
    uint4 *z4 = reinterpret_cast<uint4 *>(smem_raw);
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < (int)(tile_bytes / 16); i += blockDim.x) z4[i] = zero;
  }
  __syncthreads();
  const int lx = lane & 7, lp = lane >> 3;
  int off[NSLOT];
  bool ok[NSLOT];
#pragma unroll
  for (int xb = 0; xb < NXB; ++xb)
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const int pp = 4 * r + lp, dx = 8 * xb + lx, k = xb * NR + r;
      ok[k] = dx < NS && pp < NS * NS;
      off[k] = (pp / NS) * Q + (pp % NS) * px + dx;
    }
  T ar[NSLOT], ai[NSLOT];
  int cur = -1;
  // contiguous share of the subproblem's points for this warp (keeps runs whole)
  const int per = (np + nwarp - 1) / nwarp;
  const int w0 = min(np, warp * per), w1 = min(np, w0 + per);
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  const T *kxl = kx + lx * SK;       // this lane's x weight row (x chunk 0)
  const T *yzl = yz + lp * SK;       // this lane's first (y,z) pair row
  for (int base = w0; base < w1; base += 32) {
    const int i = base + lane;
    if (i < w1) {
      const int p = p0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      T ka[NS], kb[NS], kc[NS];
      const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, ka);
      const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, kb);
      const int sz = point_weights<T, NS>(L.loc[2][p], L.bin[2], K, kc);
#pragma unroll
      for (int a = 0; a < NS; ++a) kx[a * SK + lane] = ka[a];
#pragma unroll
      for (int zz = 0; zz < NS; ++zz)
#pragma unroll
        for (int yy = 0; yy < NS; ++yy) yz[(zz * NS + yy) * SK + lane] = kb[yy] * kc[zz];
      vre[lane] = v.x;
      vim[lane] = v.y;
      spk[lane] = sx | (sy << 10) | (sz << 20);
    }
    __syncwarp();
    const int cnt = min(32, w1 - base);
    for (int q = 0; q < cnt; ++q) {
      const int sp = spk[q];
      if (sp != cur) {
        if (cur >= 0) {
          const int rb = (cur >> 20) * Q + ((cur >> 10) & 1023) * px + (cur & 1023);
#pragma unroll
          for (int k = 0; k < NSLOT; ++k)
            if (ok[k]) {
              atomicAdd(re + rb + off[k], ar[k]);
              atomicAdd(im + rb + off[k], ai[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < NSLOT; ++k) ar[k] = ai[k] = T(0);
        cur = sp;
      }
      const T vr = vre[q], vi = vim[q];
#pragma unroll
      for (int xb = 0; xb < NXB; ++xb) {
        const T wx = kxl[8 * xb * SK + q]; // x offsets >= NS read staged products (unused)
        const T xr = vr * wx, xi = vi * wx;
#pragma unroll
        for (int r = 0; r < NR; ++r) {
          const T w = yzl[4 * r * SK + q];
          ar[xb * NR + r] = fma(xr, w, ar[xb * NR + r]);
          ai[xb * NR + r] = fma(xi, w, ai[xb * NR + r]);
        }
      }
    }
    __syncwarp();
  }
  if (cur >= 0) {
    const int rb = (cur >> 20) * Q + ((cur >> 10) & 1023) * px + (cur & 1023);
#pragma unroll
    for (int k = 0; k < NSLOT; ++k)
      if (ok[k]) {
        atomicAdd(re + rb + off[k], ar[k]);
        atomicAdd(im + rb + off[k], ai[k]);
      }
  }
  __syncthreads();
  // write back: lanes cover (x, row) pairs; rows advance by a fixed stride
  cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
  const int tx = G.t[0], ty = G.t[1], tz = G.t[2];
  const bool fits = tx <= L.nf[0] && ty <= L.nf[1] && tz <= L.nf[2] && NS <= 2 * L.nf[0] &&
                    NS <= 2 * L.nf[1] && NS <= 2 * L.nf[2];
  int txp = 1;
  while (txp < tx && txp < 32) txp <<= 1;
  const int rows_per = blockDim.x / txp;
  const int rows = ty * tz;
  const int64_t plane = (int64_t)L.nf[0] * L.nf[1];
  for (int x0 = 0; x0 < tx; x0 += txp) {
    const int x = x0 + (threadIdx.x & (txp - 1));
    const int gx = fits ? wrap_once(G.org[0] + x, L.nf[0]) : wrap_idx(G.org[0] + x, L.nf[0]);
    int r0 = threadIdx.x / txp;
    int y = r0 % ty, z = r0 / ty; // advanced incrementally below
    const int dy = rows_per % ty, dz = rows_per / ty;
    for (; r0 < rows; r0 += rows_per) {
      if (x < tx) {
        const int sidx = z * Q + y * px + x;
        cplx<T> v;
        v.x = re[sidx];
        v.y = im[sidx];
        if (v.x != T(0) || v.y != T(0)) {
          const int gy = fits ? wrap_once(G.org[1] + y, L.nf[1]) : wrap_idx(G.org[1] + y, L.nf[1]);
          const int gz = fits ? wrap_once(G.org[2] + z, L.nf[2]) : wrap_idx(G.org[2] + z, L.nf[2]);
          atomic_add_cplx_global(fwt + gx + (int64_t)L.nf[0] * gy + plane * gz, v);
        }
      }
      y += dy;
      z += dz;
      if (y >= ty) {
        y -= ty;
        ++z;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Method 2 in 3D, warp-aggregated with x slack and vector staging (variant 3,
// ns <= 8). As spread_tile3m_kernel, but a register run also absorbs points
// whose x start lies up to 8 - ns cells right of the run's first point (the
// 8 x lanes then cover the shifted footprint; x weights are read from
// zero-padded rows), each point's (y, z) products are staged so a lane reads
// its share as 16-byte vectors, the next batch's points are fetched while the
// current batch is summed, and with (bin, cell)-sorted points only the z planes
// the subproblem can touch are cleared and written back.
// 32-bit shared-memory loads for the interpolation tile: a row's address is
// formed once and its cells are read at constant offsets. volatile keeps them
// ordered against the block barriers around each tile reload (the tile does
// not change between barriers, so no memory clobber is needed).
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void lds_cplx(uint32_t a, float &x, float &y) {
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(x), "=f"(y) : "r"(a));
}
__device__ __forceinline__ void lds_cplx(uint32_t a, double &x, double &y) {
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "r"(a));
}
__device__ __forceinline__ float lds_real(uint32_t a, float) {
  float x;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(x) : "r"(a));
  return x;
}
__device__ __forceinline__ double lds_real(uint32_t a, double) {
  double x;
  asm volatile("ld.shared.f64 %0, [%1];" : "=d"(x) : "r"(a));
  return x;
}

template <typename T> struct Vec16;
template <> struct Vec16<float> {
  using type = float4;
};
template <> struct Vec16<double> {
  using type = double2;
};
// component u of a 16-byte vector and a vector from components (u is a
// constant after unrolling, so these select registers without moves)
__device__ __forceinline__ float vget(const float4 &v, int u) {
  return u == 0 ? v.x : (u == 1 ? v.y : (u == 2 ? v.z : v.w));
}
__device__ __forceinline__ double vget(const double2 &v, int u) { return u == 0 ? v.x : v.y; }
__device__ __forceinline__ float4 vmake(const float *e) { return make_float4(e[0], e[1], e[2], e[3]); }
__device__ __forceinline__ double2 vmake(const double *e) { return make_double2(e[0], e[1]); }

// FX (single precision): the tile holds int32 fixed point. The block first sums
// |c_j| over its subproblem (S); every tile cell and every register run sum is
// at most S (kernel values are at most 1), so values scaled by the power of two
// at most 2^30 / (1.01 S) stay within int32, and the run flushes become native
// integer shared-memory adds instead of compare-and-swap loops. The scale rides
// on the staged x weights (exact: a power of two). The sums are exact; each
// flushed value is rounded once to at most S * 2^-29 (about 21 significant bits
// for a dense 4096-point subproblem, against 24 for a float tile rounded at
// every add).
// A subproblem whose S is outside (2^-96, 2^100), inf or NaN keeps float atomics.
//
// Grid: the ntr transforms of a batch are interleaved fastest, ntrx of them
// per subproblem along x (block x = sub * ntrx + t), the remaining groups of
// ntrx along y. The blocks of one subproblem then run close together and all
// but the first find the subproblem's sorted coordinates and permutation in
// L2 rather than streaming them from HBM once per transform.
template <typename T, int NS, bool FX = false>
__global__ void __launch_bounds__(t3v_max_threads<T>(), 2)
    spread_tile3v_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ c,
                         const cplx<T> *__restrict__ pre, int conj_pre,
                         cplx<T> *__restrict__ fw, int64_t nf_total, int ntrx, int ntr) {
  using V = typename Vec16<T>::type;
  constexpr int TS = (int)sizeof(T);
  constexpr int VW = t3v_vw(TS), NR = t3v_nr(NS), NRV = t3v_nrv(NS, TS);
  constexpr int LPS = t3v_lps(NS, TS), QS = t3v_qs(NS, TS);
  constexpr int XS = t3v_xs(NS), KXR = t3v_kxr(NS), SK = STAGE_STRIDE;
  constexpr int HDR = 4 * LPS; // header vector(s) of a point block
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sub = (int)(blockIdx.x / (unsigned)ntrx);
  const int tr = (int)(blockIdx.y * (unsigned)ntrx + blockIdx.x % (unsigned)ntrx);
  if (tr >= ntr) return;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  if (np <= 0) return;
  const TileGeom<3> G = tile_of<T, 3, NS>(L, b);
  const int px = tile_pitch_x(3, L.bin[0] + 8);
  const int py = tile3_py(G.t[1], NS);
  const int Q = px * py;
  const size_t tile_bytes = tile3v_bytes<T>(NS, L.bin[0], L.bin[1], L.bin[2]);
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + Q * G.t[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  unsigned char *stg = smem_raw + tile_bytes + (size_t)warp * t3v_stage_bytes(NS, TS);
  T *kx = reinterpret_cast<T *>(stg); // x weights [KXR][SK], rows XS..XS+NS-1 live
  V *pts = reinterpret_cast<V *>(stg + (KXR * SK * TS + 15) / 16 * 16); // [32][QS]
  // z planes the subproblem can touch: start cells lie in [cell, cell + 1] and
  // cell-sorted points are z-major inside a bin (loc may round up to cell + 1)
  int zlo = 0, zhi = G.t[2] - 1;
  if (L.cell_sorted) {
    zlo = max(0, (int)floor(L.loc[2][p0]) - 1);
    zhi = min(G.t[2] - 1, (int)floor(L.loc[2][p0 + np - 1]) + NS);
  }
  // contiguous share of the subproblem's points for this warp
  const int per = (np + nwarp - 1) / nwarp;
  const int w0 = min(np, warp * per), w1 = min(np, w0 + per);
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  cplx<T> pv;
  T pl0 = T(0), pl1 = T(0), pl2 = T(0);
  pv.x = pv.y = T(0);
  auto fetch = [&](int i) {
    if (i < w1) {
      const int p = p0 + i;
      const int j = L.perm[p];
      pv = ct[j];
      if (pre) pv = cmul_opt<T>(pv, pre[j], conj_pre);
      pl0 = L.loc[0][p];
      pl1 = L.loc[1][p];
      pl2 = L.loc[2][p];
    }
  };
  fetch(w0 + lane);
  float fsc = 1.f, finv = 1.f; // fixed point: tile cell = round(value * fsc)
  bool fxb = false;
  if constexpr (FX) {
    __shared__ float s_sum[32];
    float acc = 0.f;
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const int j = L.perm[p0 + i];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      acc += sqrtf((float)v.x * (float)v.x + (float)v.y * (float)v.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_sum[warp] = acc;
    __syncthreads();
    float S = 0.f;
    for (int w = 0; w < nwarp; ++w) S += s_sum[w];
    const float bound = S * 1.01f;
    // scale in (2^-70, 2^126): bounds outside (2^-96, 2^100), inf and NaN keep
    // float atomics (an all-zero subproblem needs no scale)
    fxb = bound == 0.f || (bound > 0x1p-96f && bound < 0x1p100f);
    if (fxb && bound > 0.f) {
      // a power of two (exact scaling), at most 2^30 / bound; the staged x
      // weights carry it, so a run's sums are already in tile units
      fsc = __int_as_float(__float_as_int(0x1p30f / bound) & 0x7f800000);
      finv = 1.f / fsc;
    }
  }
  {
    uint4 *z4 = reinterpret_cast<uint4 *>(re + (size_t)zlo * Q);
    uint4 *z4i = reinterpret_cast<uint4 *>(im + (size_t)zlo * Q);
    const int n16 = (zhi - zlo + 1) * Q * TS / 16;
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < n16; i += blockDim.x) {
      z4[i] = zero;
      z4i[i] = zero;
    }
#pragma unroll
    for (int t = 0; t < KXR; ++t)
      if (t < XS || t >= XS + NS) kx[t * SK + lane] = T(0);
  }
  __syncthreads();
  const int lx = lane & 7, lp = lane >> 3;
  int off[NR];
  bool ok[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const int pp = 4 * r + lp;
    ok[r] = pp < NS * NS;
    off[r] = (pp / NS) * Q + (pp % NS) * px + lx;
  }
  T ar[NR], ai[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) ar[r] = ai[r] = T(0);
  int cur = -1; // run base (packed start cells)
  const T *kxl = kx + (lx + XS) * SK; // row lx - dx + XS is kxl - dx * SK
  auto flush = [&]() {
    const int rb = (cur >> 20) * Q + ((cur >> 10) & 1023) * px + (cur & 1023);
    if constexpr (FX) {
      if (fxb) {
#pragma unroll
        for (int r = 0; r < NR; ++r)
          if (ok[r]) {
            atomicAdd(reinterpret_cast<int *>(re + rb + off[r]), __float2int_rn(ar[r]));
            atomicAdd(reinterpret_cast<int *>(im + rb + off[r]), __float2int_rn(ai[r]));
          }
        return;
      }
    }
#pragma unroll
    for (int r = 0; r < NR; ++r)
      if (ok[r]) {
        atomicAdd(re + rb + off[r], ar[r]);
        atomicAdd(im + rb + off[r], ai[r]);
      }
  };
  for (int base = w0; base < w1; base += 32) {
    if (base + lane < w1) {
      T ka[NS], kb[NS], kc[NS];
      const int sx = point_weights<T, NS>(pl0, L.bin[0], K, ka);
      const int sy = point_weights<T, NS>(pl1, L.bin[1], K, kb);
      const int sz = point_weights<T, NS>(pl2, L.bin[2], K, kc);
#pragma unroll
      for (int a = 0; a < NS; ++a) kx[(XS + a) * SK + lane] = ka[a] * (T)fsc;
      V *pb = pts + lane * QS;
#pragma unroll
      for (int l4 = 0; l4 < 4; ++l4)
#pragma unroll
        for (int v = 0; v < NRV; ++v) {
          T e[VW];
#pragma unroll
          for (int u = 0; u < VW; ++u) {
            const int r = v * VW + u, pp = 4 * r + l4;
            e[u] = (r < NR && pp < NS * NS) ? kb[pp % NS] * kc[pp / NS] : T(0);
          }
          pb[l4 * LPS + v] = vmake(e);
        }
      const int spk = sx | (sy << 10) | (sz << 20);
      if constexpr (VW == 4) {
        const float he[4] = {(float)pv.x, (float)pv.y, __int_as_float(spk), 0.f};
        pb[HDR] = vmake(he);
      } else {
        const double he[2] = {(double)pv.x, (double)pv.y};
        const double h2[2] = {__longlong_as_double((long long)spk), 0.0};
        pb[HDR] = vmake(he);
        pb[HDR + 1] = vmake(h2);
      }
    }
    fetch(base + 32 + lane); // next batch, in flight while this one is summed
    __syncwarp();
    const int cnt = min(32, w1 - base);
#pragma unroll 4 // (measured: 4 -1 %, 2 +3.6 % against no unrolling)
    for (int q = 0; q < cnt; ++q) {
      const V *pq = pts + q * QS;
      const V h = pq[HDR];
      const T vr = vget(h, 0), vi = vget(h, 1);
      int sp;
      if constexpr (VW == 4) sp = __float_as_int(vget(h, 2));
      else sp = (int)__double_as_longlong(pq[HDR + 1].x);
      int dx = (sp & 1023) - (cur & 1023);
      if (((sp ^ cur) >> 10) != 0 || (unsigned)dx > (unsigned)XS) {
        if (cur >= 0) flush();
#pragma unroll
        for (int r = 0; r < NR; ++r) ar[r] = ai[r] = T(0);
        cur = sp;
        dx = 0;
      }
      const T wx = kxl[q - dx * SK];
      const T xr = vr * wx, xi = vi * wx;
      const V *wl = pq + lp * LPS;
      if constexpr (VW == 4) {
        // single precision: rows r and r + 1 as one packed two-lane FMA
        // (fma.rn.f32x2, sm_100 and newer; each lane an IEEE FMA as before):
        // the staged weights of the pair sit in adjacent registers of the
        // 16-byte load, and the run's strength product is broadcast to both
        // lanes once per point (spread -4.0 % against scalar FMAs)
        unsigned long long xr2, xi2;
        asm("mov.b64 %0, {%1, %1};" : "=l"(xr2) : "f"((float)xr));
        asm("mov.b64 %0, {%1, %1};" : "=l"(xi2) : "f"((float)xi));
#pragma unroll
        for (int v = 0; v < NRV; ++v) {
          const V w = wl[v];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int r = v * 4 + 2 * h;
            if (r < NR) {
              const float w0 = h ? (float)vget(w, 2) : (float)vget(w, 0);
              const float w1 = h ? (float)vget(w, 3) : (float)vget(w, 1);
              float a1 = r + 1 < NR ? (float)ar[r + 1 < NR ? r + 1 : r] : 0.f;
              float b1 = r + 1 < NR ? (float)ai[r + 1 < NR ? r + 1 : r] : 0.f;
              float a0 = (float)ar[r], b0 = (float)ai[r];
              asm("{\n\t.reg .b64 acc, ww;\n\tmov.b64 acc, {%0, %1};\n\tmov.b64 ww, {%3, %4};\n\t"
                  "fma.rn.f32x2 acc, %2, ww, acc;\n\tmov.b64 {%0, %1}, acc;\n\t}"
                  : "+f"(a0), "+f"(a1) : "l"(xr2), "f"(w0), "f"(w1));
              asm("{\n\t.reg .b64 acc, ww;\n\tmov.b64 acc, {%0, %1};\n\tmov.b64 ww, {%3, %4};\n\t"
                  "fma.rn.f32x2 acc, %2, ww, acc;\n\tmov.b64 {%0, %1}, acc;\n\t}"
                  : "+f"(b0), "+f"(b1) : "l"(xi2), "f"(w0), "f"(w1));
              ar[r] = a0;
              ai[r] = b0;
              if (r + 1 < NR) {
                ar[r + 1 < NR ? r + 1 : r] = a1;
                ai[r + 1 < NR ? r + 1 : r] = b1;
              }
            }
          }
        }
      } else {
#pragma unroll
        for (int v = 0; v < NRV; ++v) {
          const V w = wl[v];
#pragma unroll
          for (int u = 0; u < VW; ++u) {
            const int r = v * VW + u;
            if (r < NR) {
              const T wu = vget(w, u);
              ar[r] = fma(xr, wu, ar[r]);
              ai[r] = fma(xi, wu, ai[r]);
            }
          }
        }
      }
    }
    __syncwarp();
  }
  if (cur >= 0) flush();
  __syncthreads();
  // write back planes zlo..zhi. Lanes take x units of two cells whose first
  // global index is even, added with one 16-byte reduction (float: (re, im)
  // of both cells) when that address is 16-byte aligned; edge cells, tiles
  // wider than the grid and unaligned pairs go one by one
  cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
  const int tx = G.t[0], ty = G.t[1], tz = G.t[2];
  const bool fits = tx <= L.nf[0] && ty <= L.nf[1] && tz <= L.nf[2] && NS <= 2 * L.nf[0] &&
                    NS <= 2 * L.nf[1] && NS <= 2 * L.nf[2];
  const int par = G.org[0] & 1;         // unit u starts at tile x = 2u - par
  const int nun = (tx + par + 1) >> 1;  // units covering x = 0 .. tx-1
  // groups of exactly nun lanes (at most 32) take one row each; the threads
  // past the last whole group idle (a power-of-two group left a quarter of the
  // lanes idle at 12 units per row: 2.7 % of the spread's time)
  const int txp = nun < 32 ? nun : 32;
  const int rows_per = blockDim.x / txp;
  const int rows = ty * (zhi - zlo + 1);
  const int64_t plane = (int64_t)L.nf[0] * L.nf[1];
  for (int u0 = 0; u0 < nun; u0 += txp) {
    if ((int)threadIdx.x >= rows_per * txp) break;
    const int u = u0 + (int)threadIdx.x % txp;
    const int xa = 2 * u - par, xb = xa + 1; // the unit's cells (valid if in [0, tx))
    const bool va = u < nun && xa >= 0, vb = u < nun && xb < tx;
    const int gxa = va ? (fits ? wrap_once(G.org[0] + xa, L.nf[0]) : wrap_idx(G.org[0] + xa, L.nf[0])) : 0;
    const int gxb = vb ? (fits ? wrap_once(G.org[0] + xb, L.nf[0]) : wrap_idx(G.org[0] + xb, L.nf[0])) : 0;
    const bool pair = va && vb && gxb == gxa + 1 && sizeof(T) == 4;
    int r0 = threadIdx.x / txp;
    int y = r0 % ty, z = zlo + r0 / ty;
    const int dy = rows_per % ty, dz = rows_per / ty;
    for (; r0 < rows; r0 += rows_per) {
      if (va || vb) {
        const int sidx = z * Q + y * px;
        cplx<T> a, b;
        a.x = va ? re[sidx + xa] : T(0);
        a.y = va ? im[sidx + xa] : T(0);
        b.x = vb ? re[sidx + xb] : T(0);
        b.y = vb ? im[sidx + xb] : T(0);
        if constexpr (FX) {
          if (fxb) {
            a.x = (T)__float_as_int((float)a.x) * finv;
            a.y = (T)__float_as_int((float)a.y) * finv;
            b.x = (T)__float_as_int((float)b.x) * finv;
            b.y = (T)__float_as_int((float)b.y) * finv;
          }
        }
        const bool nza = a.x != T(0) || a.y != T(0), nzb = b.x != T(0) || b.y != T(0);
        if (nza || nzb) {
          const int gy = fits ? wrap_once(G.org[1] + y, L.nf[1]) : wrap_idx(G.org[1] + y, L.nf[1]);
          const int gz = fits ? wrap_once(G.org[2] + z, L.nf[2]) : wrap_idx(G.org[2] + z, L.nf[2]);
          cplx<T> *row = fwt + (int64_t)L.nf[0] * gy + plane * gz;
          if constexpr (sizeof(T) == 4) {
            // (16-byte alignment is checked: spread-only grids may have odd sizes)
            if (pair && (reinterpret_cast<uintptr_t>(row + gxa) & 15u) == 0) {
              atomicAdd(reinterpret_cast<float4 *>(row + gxa),
                        make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y));
              goto next_row;
            }
          }
          if (va && nza) atomic_add_cplx_global(row + gxa, a);
          if (vb && nzb) atomic_add_cplx_global(row + gxb, b);
        }
      }
    next_row:
      y += dy;
      z += dz;
      if (y >= ty) {
        y -= ty;
        ++z;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Method 2 in 3D, exclusive-warp variant: one warp per block owns its tile, so
// the tile is updated with plain shared-memory read-modify-writes instead of
// atomics. Points arrive sorted by (bin, cell inside the bin); the contributions
// of a run of points that share their first support cell (frequent in
// clustered data) are summed in registers and written to the tile once per run.
// Lane mapping and bank-conflict-free pitches are those of spread_tile3_kernel;
// the per-point weight products phi_y*phi_z of all NS*NS (y, z) pairs are
// staged once per point by the lane that loaded it.
template <typename T, int NS> struct Tile3W {
  static constexpr int CH = t3w_chunk(NS, (int)sizeof(T)); // points staged at once
  static constexpr int SK = CH + 1;                               // staging stride
  static constexpr int NXB = (NS + 7) / 8;
  static constexpr int NR = (NS * NS + 3) / 4;
  static constexpr int NSLOT = NXB * NR;
  static constexpr bool MERGE = NS <= 8; // register accumulators for same-cell runs
};

template <typename T, int NS>
__global__ void __launch_bounds__(32)
    spread_tile3w_kernel(PointLayout<T> L, KernelShape<T> K, const cplx<T> *__restrict__ c,
                         const cplx<T> *__restrict__ pre, int conj_pre,
                         cplx<T> *__restrict__ fw, int64_t nf_total) {
  using W = Tile3W<T, NS>;
  constexpr int SK = W::SK, NR = W::NR, NXB = W::NXB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sub = blockIdx.x, tr = blockIdx.y, lane = threadIdx.x;
  const int b = L.sub_bin[sub];
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<3> G = tile_of<T, 3, NS>(L, b);
  const int px = tile_pitch_x(3, G.t[0]);
  const int py = tile3_py(G.t[1], NS);
  const int Q = px * py;
  const int ncell = Q * G.t[2];
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + ncell;
  const size_t tile_bytes = tile3_bytes<T>(NS, L.bin[0], L.bin[1], L.bin[2]);
  T *kx = reinterpret_cast<T *>(smem_raw + tile_bytes);
  T *yz = kx + NS * SK;
  T *vre = yz + 4 * NR * SK;
  T *vim = vre + SK;
  int *spk = reinterpret_cast<int *>(vim + SK);
  {
    uint4 *z4 = reinterpret_cast<uint4 *>(smem_raw);
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int i = lane; i < (int)(tile_bytes / 16); i += 32) z4[i] = zero;
  }
  __syncwarp();
  const int lx = lane & 7, lp = lane >> 3;
  // tile offset of each of this lane's (x run, pair) slots
  int off[W::MERGE ? W::NSLOT : 1];
  bool ok[W::MERGE ? W::NSLOT : 1];
  if constexpr (W::MERGE) {
#pragma unroll
    for (int xb = 0; xb < NXB; ++xb)
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int pp = 4 * r + lp, dx = 8 * xb + lx;
        off[xb * NR + r] = (pp / NS) * Q + (pp % NS) * px + dx;
        ok[xb * NR + r] = dx < NS && pp < NS * NS;
      }
  }
  T ar_[W::MERGE ? W::NSLOT : 1], ai_[W::MERGE ? W::NSLOT : 1];
  int cur = -1;
  auto flush = [&](int sp) {
    if constexpr (W::MERGE) {
      const int rowbase = (sp >> 20) * Q + ((sp >> 10) & 1023) * px + (sp & 1023);
#pragma unroll
      for (int k = 0; k < W::NSLOT; ++k)
        if (ok[k]) {
          re[rowbase + off[k]] += ar_[k];
          im[rowbase + off[k]] += ai_[k];
        }
      __syncwarp();
    }
  };
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  for (int base = 0; base < np; base += W::CH) {
    const int i = base + lane;
    if (lane < W::CH && i < np) {
      const int p = p0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      T ka[NS], kb[NS], kc[NS];
      const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, ka);
      const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, kb);
      const int sz = point_weights<T, NS>(L.loc[2][p], L.bin[2], K, kc);
#pragma unroll
      for (int a = 0; a < NS; ++a) kx[a * SK + lane] = ka[a];
#pragma unroll
      for (int zz = 0; zz < NS; ++zz)
#pragma unroll
        for (int yy = 0; yy < NS; ++yy) yz[(zz * NS + yy) * SK + lane] = kb[yy] * kc[zz];
      vre[lane] = v.x;
      vim[lane] = v.y;
      spk[lane] = sx | (sy << 10) | (sz << 20);
    }
    __syncwarp();
    const int cnt = min(W::CH, np - base);
    if constexpr (W::MERGE) {
      // software pipeline: the staged data of point q+1 is loaded while point q
      // is accumulated
      int sp_n = spk[0];
      T vr_n = vre[0], vi_n = vim[0];
      T wx_n[NXB], w_n[NR];
#pragma unroll
      for (int xb = 0; xb < NXB; ++xb) wx_n[xb] = kx[(8 * xb + lx) * SK];
#pragma unroll
      for (int r = 0; r < NR; ++r) w_n[r] = yz[(4 * r + lp) * SK];
      for (int q = 0; q < cnt; ++q) {
        const int sp = sp_n;
        const T vr = vr_n, vi = vi_n;
        T wx[NXB], w[NR];
#pragma unroll
        for (int xb = 0; xb < NXB; ++xb) wx[xb] = wx_n[xb];
#pragma unroll
        for (int r = 0; r < NR; ++r) w[r] = w_n[r];
        const int qn = q + 1 < cnt ? q + 1 : q;
        sp_n = spk[qn];
        vr_n = vre[qn];
        vi_n = vim[qn];
#pragma unroll
        for (int xb = 0; xb < NXB; ++xb) wx_n[xb] = kx[(8 * xb + lx) * SK + qn];
#pragma unroll
        for (int r = 0; r < NR; ++r) w_n[r] = yz[(4 * r + lp) * SK + qn];
        if (sp != cur) {
          if (cur >= 0) flush(cur);
#pragma unroll
          for (int k = 0; k < W::NSLOT; ++k) ar_[k] = ai_[k] = T(0);
          cur = sp;
        }
#pragma unroll
        for (int xb = 0; xb < NXB; ++xb) {
          const T xr = vr * wx[xb], xi = vi * wx[xb];
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            ar_[xb * NR + r] = fma(xr, w[r], ar_[xb * NR + r]);
            ai_[xb * NR + r] = fma(xi, w[r], ai_[xb * NR + r]);
          }
        }
      }
    } else {
      for (int q = 0; q < cnt; ++q) {
        const int sp = spk[q];
        const T vr = vre[q], vi = vim[q];
        const int rowbase = (sp >> 20) * Q + ((sp >> 10) & 1023) * px + (sp & 1023);
#pragma unroll
        for (int xb = 0; xb < NXB; ++xb) {
          const int dx = 8 * xb + lx;
          const T wx = kx[dx * SK + q]; // x offsets >= NS read staged yz (unused)
          const T xr = vr * wx, xi = vi * wx;
#pragma unroll 4
          for (int r = 0; r < NR; ++r) {
            const int pp = 4 * r + lp;
            if (dx < NS && pp < NS * NS) {
              const T wv = yz[pp * SK + q];
              const int a = rowbase + (pp / NS) * Q + (pp % NS) * px + dx;
              re[a] += xr * wv;
              im[a] += xi * wv;
            }
          }
        }
        __syncwarp();
      }
    }
    __syncwarp();
  }
  if constexpr (W::MERGE)
    if (cur >= 0) flush(cur);
  __syncwarp();
  // write back: lanes cover (x, row) with rows of tx cells, 32/txp rows per step
  cplx<T> *fwt = fw + (int64_t)tr * nf_total;
  const int tx = G.t[0], ty = G.t[1], tz = G.t[2];
  const bool fits = tx <= L.nf[0] && ty <= L.nf[1] && tz <= L.nf[2] && NS <= 2 * L.nf[0] &&
                    NS <= 2 * L.nf[1] && NS <= 2 * L.nf[2];
  int txp = 1;
  while (txp < tx && txp < 32) txp <<= 1;
  const int rows_per = 32 / txp;
  const int rows = ty * tz;
  for (int x0 = 0; x0 < tx; x0 += txp) {
    const int x = x0 + (lane & (txp - 1));
    const int gx = fits ? wrap_once(G.org[0] + x, L.nf[0]) : wrap_idx(G.org[0] + x, L.nf[0]);
    for (int r0 = lane / txp; r0 < rows; r0 += rows_per) {
      const int y = r0 % ty, z = r0 / ty;
      if (x < tx) {
        const int sidx = z * Q + y * px + x;
        cplx<T> v;
        v.x = re[sidx];
        v.y = im[sidx];
        if (v.x != T(0) || v.y != T(0)) {
          const int gy = fits ? wrap_once(G.org[1] + y, L.nf[1]) : wrap_idx(G.org[1] + y, L.nf[1]);
          const int gz = fits ? wrap_once(G.org[2] + z, L.nf[2]) : wrap_idx(G.org[2] + z, L.nf[2]);
          atomic_add_cplx_global(fwt + gx + (int64_t)L.nf[0] * (gy + (int64_t)L.nf[1] * gz), v);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Method 2 in 2D, warp-aggregated: the 2D analogue of spread_tile3m_kernel.
// Lanes (lx, ly) = (lane & 7, lane >> 3) cover an 8-cell x run of 4 rows; the
// row pitch is 8 mod 16 words so the 4 rows fall in disjoint bank octets.
// Points are (bin, cell)-sorted; each warp sums runs of points sharing their
// first support cell in registers and adds them to the tile once per run.
// staging: x weights (ns rows), y weights padded to 4*ceil(ns/4) rows (lanes
// read rows 4r + ly up to that bound), strengths, packed start cells
template <typename T> __host__ __device__ constexpr int t2m_stage_bytes(int ns) {
  return (33 * (ns + 4 * ((ns + 3) / 4) + 2) * (int)sizeof(T) + 33 * 4 + 15) / 16 * 16;
}
template <typename T> __host__ __device__ constexpr size_t tile2m_bytes(int ns, int bx, int by) {
  return (2 * sizeof(T) * (size_t)tile_pitch_x(3, bx + ns) * (by + ns) + 15) / 16 * 16;
}

// EXCL: one warp per block owns the tile, so a run is added with plain
// read-modify-writes (shared f32 atomics are compare-and-swap loops); the 2D
// tile is small enough (~12 KB at 32x32 bins) for many such blocks per SM.
template <typename T, int NS, bool EXCL = false>
__global__ void __launch_bounds__(256)
    spread_tile2m_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ c,
                         const cplx<T> *__restrict__ pre, int conj_pre,
                         cplx<T> *__restrict__ fw, int64_t nf_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SK = STAGE_STRIDE;
  constexpr int NXB = (NS + 7) / 8;
  constexpr int NRY = (NS + 3) / 4;
  constexpr int NSLOT = NXB * NRY;
  const int sub = blockIdx.x, tr = blockIdx.y;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<2> G = tile_of<T, 2, NS>(L, b);
  const int px = tile_pitch_x(3, G.t[0]);
  const size_t tile_bytes = tile2m_bytes<T>(NS, L.bin[0], L.bin[1]);
  T *re = reinterpret_cast<T *>(smem_raw);
  T *im = re + px * G.t[1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  T *kx = reinterpret_cast<T *>(smem_raw + tile_bytes + (size_t)warp * t2m_stage_bytes<T>(NS));
  T *ky = kx + NS * SK;
  T *vre = ky + 4 * NRY * SK;
  T *vim = vre + SK;
  int *spk = reinterpret_cast<int *>(vim + SK);
  {
    uint4 *z4 = reinterpret_cast<uint4 *>(smem_raw);
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < (int)(tile_bytes / 16); i += blockDim.x) z4[i] = zero;
  }
  __syncthreads();
  const int lx = lane & 7, ly = lane >> 3;
  int off[NSLOT];
  bool ok[NSLOT];
#pragma unroll
  for (int xb = 0; xb < NXB; ++xb)
#pragma unroll
    for (int r = 0; r < NRY; ++r) {
      const int dx = 8 * xb + lx, dy = 4 * r + ly, k = xb * NRY + r;
      ok[k] = dx < NS && dy < NS;
      off[k] = dy * px + dx;
    }
  T ar[NSLOT], ai[NSLOT];
  int cur = -1;
  const int per = (np + nwarp - 1) / nwarp;
  const int w0 = min(np, warp * per), w1 = min(np, w0 + per);
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  const T *kxl = kx + lx * SK;
  const T *kyl = ky + ly * SK;
  for (int base = w0; base < w1; base += 32) {
    const int i = base + lane;
    if (i < w1) {
      const int p = p0 + i;
      const int j = L.perm[p];
      cplx<T> v = ct[j];
      if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
      T kk[NS];
      const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, kk);
#pragma unroll
      for (int a = 0; a < NS; ++a) kx[a * SK + lane] = kk[a];
      const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, kk);
#pragma unroll
      for (int a = 0; a < NS; ++a) ky[a * SK + lane] = kk[a];
      vre[lane] = v.x;
      vim[lane] = v.y;
      spk[lane] = sx | (sy << 16);
    }
    __syncwarp();
    const int cnt = min(32, w1 - base);
    for (int q = 0; q < cnt; ++q) {
      const int sp = spk[q];
      if (sp != cur) {
        if (cur >= 0) {
          const int rb = (cur >> 16) * px + (cur & 0xffff);
#pragma unroll
          for (int k = 0; k < NSLOT; ++k)
            if (ok[k]) {
              if constexpr (EXCL) {
                re[rb + off[k]] += ar[k];
                im[rb + off[k]] += ai[k];
              } else {
                atomicAdd(re + rb + off[k], ar[k]);
                atomicAdd(im + rb + off[k], ai[k]);
              }
            }
        }
#pragma unroll
        for (int k = 0; k < NSLOT; ++k) ar[k] = ai[k] = T(0);
        cur = sp;
      }
      const T vr = vre[q], vi = vim[q];
#pragma unroll
      for (int xb = 0; xb < NXB; ++xb) {
        const T wx = kxl[8 * xb * SK + q]; // x offsets >= NS read staged y weights (unused)
        const T xr = vr * wx, xi = vi * wx;
#pragma unroll
        for (int r = 0; r < NRY; ++r) {
          const T w = kyl[4 * r * SK + q];
          ar[xb * NRY + r] = fma(xr, w, ar[xb * NRY + r]);
          ai[xb * NRY + r] = fma(xi, w, ai[xb * NRY + r]);
        }
      }
    }
    __syncwarp();
  }
  if (cur >= 0) {
    const int rb = (cur >> 16) * px + (cur & 0xffff);
#pragma unroll
    for (int k = 0; k < NSLOT; ++k)
      if (ok[k]) {
        if constexpr (EXCL) {
          re[rb + off[k]] += ar[k];
          im[rb + off[k]] += ai[k];
        } else {
          atomicAdd(re + rb + off[k], ar[k]);
          atomicAdd(im + rb + off[k], ai[k]);
        }
      }
  }
  __syncthreads();
  cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
  const int tx = G.t[0], ty = G.t[1];
  const bool fits = tx <= L.nf[0] && ty <= L.nf[1] && NS <= 2 * L.nf[0] && NS <= 2 * L.nf[1];
  int txp = 1;
  while (txp < tx && txp < 32) txp <<= 1;
  const int rows_per = blockDim.x / txp;
  for (int x0 = 0; x0 < tx; x0 += txp) {
    const int x = x0 + (threadIdx.x & (txp - 1));
    const int gx = fits ? wrap_once(G.org[0] + x, L.nf[0]) : wrap_idx(G.org[0] + x, L.nf[0]);
    for (int y = threadIdx.x / txp; y < ty; y += rows_per) {
      if (x < tx) {
        cplx<T> v;
        v.x = re[y * px + x];
        v.y = im[y * px + x];
        if (v.x != T(0) || v.y != T(0)) {
          const int gy = fits ? wrap_once(G.org[1] + y, L.nf[1]) : wrap_idx(G.org[1] + y, L.nf[1]);
          atomic_add_cplx_global(fwt + gx + (int64_t)L.nf[0] * gy, v);
        }
      }
    }
  }
}

// Method 1: point-driven spreading straight into global memory with vector
// atomics (no tile). Points are still processed in bin order for locality.
constexpr int GLOBAL_SPREAD_THREADS = 128;

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(GLOBAL_SPREAD_THREADS)
    spread_global_kernel(PointLayout<T> L, KernelShape<T> K, const cplx<T> *__restrict__ c,
                         const cplx<T> *__restrict__ pre, int conj_pre,
                         cplx<T> *__restrict__ fw, int64_t nf_total) {
  const int sub = blockIdx.x;
  const int tr = blockIdx.y;
  const int b = L.sub_bin[sub];
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<DIM> G = tile_of<T, DIM, NS>(L, b);
  const cplx<T> *ct = c + (int64_t)tr * L.M;
  cplx<T> *fwt = fw + (int64_t)tr * nf_total;
  __shared__ T zst[DIM == 3 ? GLOBAL_SPREAD_THREADS * (NS + 1) : 1];
  __shared__ int zsti[DIM == 3 ? GLOBAL_SPREAD_THREADS * (NS + 1) : 1];
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int p = p0 + i;
    const int j = L.perm[p];
    cplx<T> v = ct[j];
    if (pre) v = cmul_opt<T>(v, pre[j], conj_pre);
    T ker[DIM][NS];
    int gi[DIM][NS];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int s = point_weights<T, NS>(L.loc[d][p], L.bin[d], K, ker[d]);
#pragma unroll
      for (int a = 0; a < NS; ++a) gi[d][a] = wrap_idx(G.org[d] + s + a, L.nf[d]);
    }
    if constexpr (DIM == 1) {
#pragma unroll
      for (int a = 0; a < NS; ++a) {
        cplx<T> u;
        u.x = v.x * ker[0][a];
        u.y = v.y * ker[0][a];
        atomic_add_cplx_global(fwt + gi[0][a], u);
      }
    } else if constexpr (DIM == 2) {
#pragma unroll
      for (int bb = 0; bb < NS; ++bb) {
        const int64_t row = (int64_t)gi[DIM > 1 ? 1 : 0][bb] * L.nf[0];
        const T wr = v.x * ker[DIM > 1 ? 1 : 0][bb], wi = v.y * ker[DIM > 1 ? 1 : 0][bb];
#pragma unroll
        for (int a = 0; a < NS; ++a) {
          cplx<T> u;
          u.x = wr * ker[0][a];
          u.y = wi * ker[0][a];
          atomic_add_cplx_global(fwt + row + gi[0][a], u);
        }
      }
    } else {
      T *kzs = zst + threadIdx.x * (NS + 1);
      int *gzs = zsti + threadIdx.x * (NS + 1);
#pragma unroll
      for (int cc = 0; cc < NS; ++cc) {
        kzs[cc] = ker[DIM > 2 ? 2 : 0][cc];
        gzs[cc] = gi[DIM > 2 ? 2 : 0][cc];
      }
#pragma unroll 1
      for (int cc = 0; cc < NS; ++cc) {
        const int64_t plane = (int64_t)gzs[cc] * L.nf[0] * L.nf[1];
        const T zr = v.x * kzs[cc], zi = v.y * kzs[cc];
#pragma unroll
        for (int bb = 0; bb < NS; ++bb) {
          const int64_t row = plane + (int64_t)gi[DIM > 1 ? 1 : 0][bb] * L.nf[0];
          const T wr = zr * ker[DIM > 1 ? 1 : 0][bb], wi = zi * ker[DIM > 1 ? 1 : 0][bb];
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            cplx<T> u;
            u.x = wr * ker[0][a];
            u.y = wi * ker[0][a];
            atomic_add_cplx_global(fwt + row + gi[0][a], u);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Interpolation: one thread per point, gathering the NS^DIM support values of
// the fine grid (read through L1/L2: the points of a subproblem share a tile).
constexpr int INTERP_THREADS = 128;
constexpr int INTERP_TILE_THREADS = 256;

// Interpolation: one thread per point; the point's kernel weights and grid
// indices are computed once and reused for every transform of the batch.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(INTERP_THREADS)
    interp_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ fw,
                  int64_t nf_total, const cplx<T> *__restrict__ post, int conj_post,
                  cplx<T> *__restrict__ out, int ntr) {
  const int sub = blockIdx.x;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  const TileGeom<DIM> G = tile_of<T, DIM, NS>(L, b);
  __shared__ T zst[DIM == 3 ? INTERP_THREADS * (NS + 1) : 1];
  __shared__ int zsti[DIM == 3 ? INTERP_THREADS * (NS + 1) : 1];
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int p = p0 + i;
    const int j = L.perm[p];
    T ker[DIM][NS];
    int gi[DIM][NS];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int s = point_weights<T, NS>(L.loc[d][p], L.bin[d], K, ker[d]);
#pragma unroll
      for (int a = 0; a < NS; ++a) gi[d][a] = wrap_idx(G.org[d] + s + a, L.nf[d]);
    }
    T *kzs = zst + threadIdx.x * (NS + 1);
    int *gzs = zsti + threadIdx.x * (NS + 1);
    if constexpr (DIM == 3) {
      // z weights and planes go through shared memory: a dynamic index into a
      // register array would put it in local memory
#pragma unroll
      for (int cc = 0; cc < NS; ++cc) {
        kzs[cc] = ker[DIM > 2 ? 2 : 0][cc];
        gzs[cc] = gi[DIM > 2 ? 2 : 0][cc];
      }
    }
    cplx<T> pf;
    pf.x = T(1);
    pf.y = T(0);
    if (post) {
      pf = post[j];
      if (conj_post) pf.y = -pf.y;
    }
#pragma unroll 1
    for (int tr = 0; tr < ntr; ++tr) {
      const cplx<T> *fwt = fw + (int64_t)tr * nf_total + goff;
      T accr = T(0), acci = T(0);
      if constexpr (DIM == 1) {
#pragma unroll
        for (int a = 0; a < NS; ++a) {
          const cplx<T> g = __ldg(fwt + gi[0][a]);
          accr = fma(g.x, ker[0][a], accr);
          acci = fma(g.y, ker[0][a], acci);
        }
      } else if constexpr (DIM == 2) {
        constexpr int UB = NS > 8 ? 2 : NS; // bound the number of loads kept in flight
#pragma unroll UB
        for (int bb = 0; bb < NS; ++bb) {
          const int64_t row = (int64_t)gi[DIM > 1 ? 1 : 0][bb] * L.nf[0];
          T rr = T(0), ri = T(0);
#pragma unroll
          for (int a = 0; a < NS; ++a) {
            const cplx<T> g = __ldg(fwt + row + gi[0][a]);
            rr = fma(g.x, ker[0][a], rr);
            ri = fma(g.y, ker[0][a], ri);
          }
          accr = fma(rr, ker[DIM > 1 ? 1 : 0][bb], accr);
          acci = fma(ri, ker[DIM > 1 ? 1 : 0][bb], acci);
        }
      } else {
#pragma unroll 1
        for (int cc = 0; cc < NS; ++cc) {
          const int64_t plane = (int64_t)gzs[cc] * L.nf[0] * L.nf[1];
          T pr = T(0), pi = T(0);
#pragma unroll
          for (int bb = 0; bb < NS; ++bb) {
            const int64_t row = plane + (int64_t)gi[DIM > 1 ? 1 : 0][bb] * L.nf[0];
            T rr = T(0), ri = T(0);
#pragma unroll
            for (int a = 0; a < NS; ++a) {
              const cplx<T> g = __ldg(fwt + row + gi[0][a]);
              rr = fma(g.x, ker[0][a], rr);
              ri = fma(g.y, ker[0][a], ri);
            }
            pr = fma(rr, ker[DIM > 1 ? 1 : 0][bb], pr);
            pi = fma(ri, ker[DIM > 1 ? 1 : 0][bb], pi);
          }
          accr = fma(pr, kzs[cc], accr);
          acci = fma(pi, kzs[cc], acci);
        }
      }
      cplx<T> r;
      r.x = accr * pf.x - acci * pf.y;
      r.y = accr * pf.y + acci * pf.x;
      out[(int64_t)tr * L.M + j] = r;
    }
  }
}

// Interpolation from a shared-memory tile (types 2 and 3, 2D and 3D): the
// block stages its subproblem's (bin + ns)^d cells of the fine grid once per
// transform with coalesced loads (periodic wrap applied while loading), for
// up to tb transforms per round, then each thread evaluates its points'
// weights once per round and reads the ns^d cells from shared memory.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(INTERP_TILE_THREADS)
    interp_tile_kernel(PointLayout<T> L0, KernelShape<T> K, const cplx<T> *__restrict__ fw,
                       int64_t nf_total, const cplx<T> *__restrict__ post, int conj_post,
                       cplx<T> *__restrict__ out, int ntr, int tb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sub = blockIdx.x;
  int b = L0.sub_bin[sub];
  PointLayout<T> Lg;
  const int64_t goff = resolve_problem<T>(L0, Lg, b);
  const PointLayout<T> &L = Lg;
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  if (np <= 0) return;
  const TileGeom<DIM> G = tile_of<T, DIM, NS>(L, b);
  const int tx = G.t[0], ty = G.t[1];
  const int cells = G.cells, txy = tx * ty;
  cplx<T> *tile = reinterpret_cast<cplx<T> *>(smem_raw); // [tb][cells]
  T *kzs = reinterpret_cast<T *>(tile + (size_t)tb * cells) + threadIdx.x * (NS + 1);
  const int64_t plane = (int64_t)L.nf[0] * L.nf[1];
  for (int t0 = 0; t0 < ntr; t0 += tb) {
    const int nt = min(tb, ntr - t0);
    __syncthreads(); // the previous round's readers are done
    // rows of the tile (one per warp at a time, lanes along x): no per-cell division
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int rows = cells / tx;
    for (int k = 0; k < nt; ++k) {
      const cplx<T> *src = fw + (int64_t)(t0 + k) * nf_total + goff;
      cplx<T> *dst = tile + (size_t)k * cells;
      for (int r = threadIdx.x >> 5; r < rows; r += nw) {
        int64_t rb = (int64_t)L.nf[0] * wrap_idx(G.org[1] + (DIM == 3 ? r % ty : r), L.nf[1]);
        if constexpr (DIM == 3) rb += plane * wrap_idx(G.org[2] + r / ty, L.nf[2]);
        for (int x = lane; x < tx; x += 32)
          dst[r * tx + x] = src[rb + wrap_idx(G.org[0] + x, L.nf[0])];
      }
    }
    __syncthreads();
    // per point: weights once per round, then the tile rows at constant offsets
    // from a 32-bit shared address (3D)
    constexpr uint32_t CS = sizeof(cplx<T>);
    const uint32_t tile_s = smem_addr(tile), kz_s = smem_addr(kzs);
    const uint32_t rs = (uint32_t)tx * CS, ps = (uint32_t)txy * CS;
    // (3D: the next point's index and coordinates are prefetched; in 2D that
    // measured slower with many transforms per round)
    int i = threadIdx.x;
    int jn = 0;
    T ln0 = T(0), ln1 = T(0), ln2 = T(0);
    if (DIM == 3 && i < np) {
      jn = L.perm[p0 + i];
      ln0 = L.loc[0][p0 + i];
      ln1 = L.loc[1][p0 + i];
      ln2 = L.loc[DIM - 1][p0 + i];
    }
    for (; i < np; i += blockDim.x) {
      int j;
      T l0, l1, l2;
      if constexpr (DIM == 3) {
        j = jn;
        l0 = ln0;
        l1 = ln1;
        l2 = ln2;
        const int inext = i + blockDim.x;
        if (inext < np) {
          jn = L.perm[p0 + inext];
          ln0 = L.loc[0][p0 + inext];
          ln1 = L.loc[1][p0 + inext];
          ln2 = L.loc[2][p0 + inext];
        }
      } else {
        j = L.perm[p0 + i];
        l0 = L.loc[0][p0 + i];
        l1 = L.loc[1][p0 + i];
        l2 = T(0);
      }
      T kx[NS], ky[NS];
      const int sx = point_weights<T, NS>(l0, L.bin[0], K, kx);
      const int sy = point_weights<T, NS>(l1, L.bin[1], K, ky);
      int sz = 0;
      if constexpr (DIM == 3) {
        T kz[NS];
        sz = point_weights<T, NS>(l2, L.bin[2], K, kz);
#pragma unroll
        for (int cc = 0; cc < NS; ++cc) kzs[cc] = kz[cc]; // read back with a dynamic index
      }
      cplx<T> pf;
      pf.x = T(1);
      pf.y = T(0);
      if (post) {
        pf = post[j];
        if (conj_post) pf.y = -pf.y;
      }
      const uint32_t base_s = tile_s + (uint32_t)(sz * txy + sy * tx + sx) * CS;
#pragma unroll 1
      for (int k = 0; k < nt; ++k) {
        const uint32_t tk = base_s + (uint32_t)(k * cells) * CS;
        T accr = T(0), acci = T(0);
        if constexpr (DIM == 2) {
          // 2D: plain loads (the compiler interleaves them across the rows
          // better than volatile ones when many transforms share a round)
          const cplx<T> *tl = tile + (size_t)k * cells + (sy * tx + sx);
#pragma unroll
          for (int bb = 0; bb < NS; ++bb) {
            T rr = T(0), ri = T(0);
#pragma unroll
            for (int a = 0; a < NS; ++a) {
              const cplx<T> g = tl[bb * tx + a];
              rr = fma(g.x, kx[a], rr);
              ri = fma(g.y, kx[a], ri);
            }
            accr = fma(rr, ky[bb], accr);
            acci = fma(ri, ky[bb], acci);
          }
        } else {
#pragma unroll 1
          for (int cc = 0; cc < NS; ++cc) {
            const uint32_t plane = tk + (uint32_t)cc * ps;
            T pr = T(0), pi = T(0);
#pragma unroll
            for (int bb = 0; bb < NS; ++bb) {
              const uint32_t row = plane + (uint32_t)bb * rs;
              T rr = T(0), ri = T(0);
#pragma unroll
              for (int a = 0; a < NS; ++a) {
                T gx, gy;
                lds_cplx(row + a * CS, gx, gy);
                rr = fma(gx, kx[a], rr);
                ri = fma(gy, kx[a], ri);
              }
              pr = fma(rr, ky[bb], pr);
              pi = fma(ri, ky[bb], pi);
            }
            const T wz = lds_real(kz_s + (uint32_t)cc * (uint32_t)sizeof(T), T(0));
            accr = fma(pr, wz, accr);
            acci = fma(pi, wz, acci);
          }
        }
        cplx<T> r;
        r.x = accr * pf.x - acci * pf.y;
        r.y = accr * pf.y + acci * pf.x;
        if (L.sorted_out)
          static_cast<cplx<T> *>(L.sorted_out)[(int64_t)(t0 + k) * L.M + p0 + i] = r;
        else
          out[(int64_t)(t0 + k) * L.M + j] = r;
      }
    }
  }
}

#include "interp_tma.cuh"

// out[t*M + j] = src[t*M + iperm[j]]: sorted-order interpolation results to
// user order, transform by transform (blockIdx.y). The writes are coalesced
// and evict-first, as are the loads of the inverse permutation; the random
// 8-byte reads fall in one transform's sorted results, which stay in L2. (16
// vectors of 1e7 2D points: 3.70 ms per execute, against 5.09 ms for the
// scatter out[t*M + perm[p]] = src[t*M + p], whose partial-sector writes had to
// merge in L2.)
template <typename T>
__global__ void __launch_bounds__(256)
    gather_sorted_kernel(const cplx<T> *__restrict__ src, const int *__restrict__ iperm, int M,
                         cplx<T> *__restrict__ out) {
  const int64_t o = (int64_t)blockIdx.y * M;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x)
    __stcs(&out[o + j], src[o + __ldcs(&iperm[j])]);
}

// ------------------------------------------------------------- dispatch ----
// Tensor map of the fine grids for the TMA interpolation: rank dim + 1
// (x, y, [z], transform), 8-byte elements (x counted in doubles for double
// precision), box (BX, BY, BZ, 1). False when the CUDA driver rejects it.
template <typename T>
bool encode_grid_map(CUtensorMap *map, const void *base, int dim, const int nf[3], int ntr,
                     int BX, int BY, int BZ) {
  using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                              const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                              const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &f, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    cudaGetLastError();
    return reinterpret_cast<Encode>(f);
  }();
  if (!fn || (reinterpret_cast<uintptr_t>(base) & 15)) return false;
  const int xm = sizeof(T) == 8 ? 2 : 1;
  const int rank = dim + 1;
  const cuuint64_t esz = 8;
  cuuint64_t gdim[4], gstr[3];
  cuuint32_t box[4], estr[4] = {1, 1, 1, 1};
  gdim[0] = (cuuint64_t)nf[0] * xm;
  gdim[1] = (cuuint64_t)nf[1];
  box[0] = (cuuint32_t)(BX * xm);
  box[1] = (cuuint32_t)BY;
  gstr[0] = (cuuint64_t)nf[0] * xm * esz;
  if (dim == 2) {
    gdim[2] = (cuuint64_t)ntr;
    box[2] = 1;
    gstr[1] = gstr[0] * nf[1];
  } else {
    gdim[2] = (cuuint64_t)nf[2];
    gdim[3] = (cuuint64_t)ntr;
    box[2] = (cuuint32_t)BZ;
    box[3] = 1;
    gstr[1] = gstr[0] * nf[1];
    gstr[2] = gstr[1] * nf[2];
  }
  const CUtensorMapDataType ty =
      sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_INT64;
  const CUresult r = fn(map, ty, (cuuint32_t)rank, const_cast<void *>(base), gdim, gstr, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <typename T, int DIM> struct Dispatch {
  template <int NS>
  static void spread(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *c,
                     const cplx<T> *pre, int conj_pre, cplx<T> *fw, int64_t nf_total, int ntr,
                     const SpreadConfig &cfg, cudaStream_t s) {
    dim3 grid((unsigned)L.nsub, (unsigned)ntr);
    if (cfg.method == 3) {
      auto ko = spread_output_driven_kernel<T, DIM, NS>;
      GBN_CUDA(cudaFuncSetAttribute(ko, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)cfg.smem));
      ko<<<grid, OD_THREADS, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
      GBN_LAUNCH_CHECK();
      return;
    }
    if (cfg.method == 1) {
      spread_global_kernel<T, DIM, NS><<<grid, GLOBAL_SPREAD_THREADS, 0, s>>>(L, K, c, pre, conj_pre, fw,
                                                                    nf_total);
    } else if constexpr (DIM == 3) {
      if (NS <= 8 && cfg.variant == 3) {
        auto kv = spread_tile3v_kernel<T, (NS <= 8 ? NS : 8)>;
        if constexpr (sizeof(T) == 4 && NS <= 8) // ns 7-8 only when asked (option 2)
          if (cfg.fixed) kv = spread_tile3v_kernel<T, NS, true>;
        GBN_CUDA(cudaFuncSetAttribute(kv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)cfg.smem));
        // transforms interleaved fastest; gridDim.x stays within 2^31 - 1
        const int ntrx = (int)std::max<int64_t>(
            1, std::min<int64_t>(ntr, INT32_MAX / std::max(L.nsub, 1)));
        const dim3 gv((unsigned)L.nsub * (unsigned)ntrx, (unsigned)((ntr + ntrx - 1) / ntrx));
        kv<<<gv, cfg.threads, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total, ntrx, ntr);
        GBN_LAUNCH_CHECK();
        return;
      }
      if (NS <= 8 && cfg.variant == 2) {
        auto km = spread_tile3m_kernel<T, (NS <= 8 ? NS : 8)>;
        GBN_CUDA(cudaFuncSetAttribute(km, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)cfg.smem));
        km<<<grid, t3m_threads<T>(), cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
        GBN_LAUNCH_CHECK();
        return;
      }
      if constexpr (sizeof(T) == 8) {
        if (cfg.variant == 4) {
          auto kx = spread_tile3x_kernel<NS>;
          GBN_CUDA(cudaFuncSetAttribute(kx, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)cfg.smem));
          // the kernel's row mapping is built for T3X_THREADS threads
          kx<<<grid, T3X_THREADS, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
          GBN_LAUNCH_CHECK();
          return;
        }
      }
      if (cfg.variant == 1) {
        auto kw = spread_tile3w_kernel<T, NS>;
        GBN_CUDA(cudaFuncSetAttribute(kw, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)cfg.smem));
        kw<<<grid, 32, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
        GBN_LAUNCH_CHECK();
        return;
      }
      auto kern = spread_tile3_kernel<T, NS>;
      GBN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)cfg.smem));
      kern<<<grid, cfg.threads, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
    } else if (DIM == 2 && cfg.variant == 1) {
      auto k1 = spread_tile2m_kernel<T, NS, true>;
      GBN_CUDA(cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)cfg.smem));
      k1<<<grid, 32, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
    } else if (DIM == 2 && cfg.variant == 2) {
      auto k2 = spread_tile2m_kernel<T, NS>;
      GBN_CUDA(cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)cfg.smem));
      k2<<<grid, 256, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
    } else {
      auto kern = spread_tile_kernel<T, DIM, NS>;
      GBN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)cfg.smem));
      kern<<<grid, cfg.threads, cfg.smem, s>>>(L, K, c, pre, conj_pre, fw, nf_total);
    }
    GBN_LAUNCH_CHECK();
  }
  template <int NS>
  static void interp(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *fw,
                     int64_t nf_total, const cplx<T> *post, int conj_post, cplx<T> *out,
                     int ntr, cudaStream_t s) {
    if constexpr (DIM >= 2) {
      // TMA-staged tiles (interp_mode 0 or 3) for single problems whose boxes fit
      // the copy engine's limits and two buffers fit beside another block
      if (!L.probs && (L.interp_mode == 0 || L.interp_mode == 3) && L.M > 0) {
        const int t0 = L.bin[0] + NS, t1 = L.bin[1] + NS, t2 = DIM == 3 ? L.bin[2] + NS : 1;
        const int BX = (t0 + 2) & ~1; // even, at least t0 + 1
        const int xm = sizeof(T) == 8 ? 2 : 1;
        const size_t box = (size_t)BX * t1 * t2 * sizeof(cplx<T>);
        // one buffer for a single transform (no copy to overlap: more blocks per
        // SM), two otherwise; + alignment slack
        const size_t smem = (ntr > 1 ? 2 : 1) * ((box + 127) / 128 * 128) + 128;
        CUtensorMap map;
        if (BX * xm <= 256 && t1 <= 256 && t2 <= 256 && BX <= L.nf[0] && smem <= 112 * 1024 &&
            encode_grid_map<T>(&map, fw, DIM, L.nf, ntr, BX, t1, t2)) {
          auto kt = interp_tma_kernel<T, DIM, NS>;
          GBN_CUDA(cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
          kt<<<(unsigned)L.nsub, INTERP_TMA_THREADS, smem, s>>>(
              map, L, K, fw, nf_total, post, conj_post, out, ntr, BX, t1, t2,
              device_error_word());
          GBN_LAUNCH_CHECK();
          if (L.sorted_out) {
            const unsigned gx = (unsigned)std::min<int64_t>((L.M + 255) / 256, 152 * 8);
            gather_sorted_kernel<T><<<dim3(gx, (unsigned)ntr), 256, 0, s>>>(
                static_cast<const cplx<T> *>(L.sorted_out), L.iperm, L.M, out);
            GBN_LAUNCH_CHECK();
          }
          return;
        }
      }
      // tile-staged interpolation when one transform's tile fits the per-block
      // budget (three blocks per SM); interp_mode 1 keeps the gather
      const int imethod = L.interp_mode == 1 ? 0 : 1;
      size_t cells = 1;
      for (int d = 0; d < DIM; ++d) cells *= (size_t)(L.bin[d] + NS);
      const size_t tbytes = cells * sizeof(cplx<T>);
      const size_t kzb = DIM == 3 ? (size_t)INTERP_TILE_THREADS * (NS + 1) * sizeof(T) : 0;
      const size_t budget = 72 * 1024;
      // transforms per round at most (2D: four transforms' tiles per block keep four
      // blocks per SM, measured best on 16 vectors of 1e7 points)
      const int tbmax = DIM == 2 ? 4 : 8;
      if (imethod != 0 && tbytes + kzb <= budget) {
        int tb = (int)((budget - kzb) / tbytes);
        tb = std::max(1, std::min(tb, std::min(ntr, tbmax)));
        const size_t smem = (size_t)tb * tbytes + kzb;
        auto kt = interp_tile_kernel<T, DIM, NS>;
        GBN_CUDA(cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        kt<<<(unsigned)L.nsub, INTERP_TILE_THREADS, smem, s>>>(L, K, fw, nf_total, post, conj_post,
                                                         out, ntr, tb);
        GBN_LAUNCH_CHECK();
        if (L.sorted_out && L.M > 0) {
          const unsigned gx = (unsigned)std::min<int64_t>((L.M + 255) / 256, 152 * 8);
          gather_sorted_kernel<T><<<dim3(gx, (unsigned)ntr), 256, 0, s>>>(
              static_cast<const cplx<T> *>(L.sorted_out), L.iperm, L.M, out);
          GBN_LAUNCH_CHECK();
        }
        return;
      }
    }
    interp_kernel<T, DIM, NS><<<(unsigned)L.nsub, INTERP_THREADS, 0, s>>>(L, K, fw, nf_total, post,
                                                                         conj_post, out, ntr);
    GBN_LAUNCH_CHECK();
  }
};

template <typename T, int DIM, typename F> void ns_switch(int ns, F &&f) {
  switch (ns) {
  case 2: f.template operator()<2>(); break;
  case 3: f.template operator()<3>(); break;
  case 4: f.template operator()<4>(); break;
  case 5: f.template operator()<5>(); break;
  case 6: f.template operator()<6>(); break;
  case 7: f.template operator()<7>(); break;
  case 8: f.template operator()<8>(); break;
  case 9: f.template operator()<9>(); break;
  case 10: f.template operator()<10>(); break;
  case 11: f.template operator()<11>(); break;
  case 12: f.template operator()<12>(); break;
  default:
    if constexpr (std::is_same_v<T, double>) {
      switch (ns) {
      case 13: f.template operator()<13>(); break;
      case 14: f.template operator()<14>(); break;
      case 15: f.template operator()<15>(); break;
      case 16: f.template operator()<16>(); break;
      default: GBN_THROW(FINUFFT_ERR_SPREAD_BOX_SMALL, "unsupported kernel width");
      }
    } else {
      GBN_THROW(FINUFFT_ERR_SPREAD_BOX_SMALL, "unsupported kernel width");
    }
  }
}

template <typename T, int DIM>
void spread_dim(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *c,
                const cplx<T> *pre, int conj_pre, cplx<T> *fw, int64_t nf_total, int ntr,
                const SpreadConfig &cfg, cudaStream_t s) {
  ns_switch<T, DIM>(K.ns, [&]<int NS>() {
    Dispatch<T, DIM>::template spread<NS>(L, K, c, pre, conj_pre, fw, nf_total, ntr, cfg, s);
  });
}

template <typename T, int DIM>
void interp_dim(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *fw,
                int64_t nf_total, const cplx<T> *post, int conj_post, cplx<T> *out, int ntr,
                cudaStream_t s) {
  ns_switch<T, DIM>(K.ns, [&]<int NS>() {
    Dispatch<T, DIM>::template interp<NS>(L, K, fw, nf_total, post, conj_post, out, ntr, s);
  });
}

} // namespace gbn
