// Type-2 interpolation from fine-grid tiles staged by the Tensor Memory
// Accelerator (cp.async.bulk.tensor): the reference's subproblem interpolation
// (src/cuda/interp_subprob_inst.cu:16-113) loads each tile with per-thread
// loads; here one elected thread of the block issues one bulk tensor copy per
// transform into a shared-memory buffer, completion counted on an mbarrier,
// and the copy of transform k+1 runs while the block interpolates transform k
// (two buffers). Each thread owns up to PPT points of the subproblem, whose
// kernel weights it evaluates once (registers) and reuses for every transform.
//
// The tensor map views this GPU's fine grids as a (dim + 1)-rank array
// (x, y, [z], transform) of 8-byte elements (double precision: x counted in
// doubles). A box starts at an even x (the 16-byte rule of tiled copies: the
// tile origin is rounded down and the box is one cell wider), and is used
// only for tiles that do not wrap around the periodic grid; tiles on the
// boundary are loaded with per-thread loads (wrap applied) into the same
// buffer layout. No cluster multicast is used.
// Included inside namespace gbn by spreadinterp_impl.cuh (after its shared-
// memory load helpers).
#pragma once

constexpr int INTERP_TMA_THREADS = 256;
constexpr long long TMA_WAIT_LIMIT = 1ll << 26; // polls of an mbarrier before giving up

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\t"
               "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}
// bounded wait: false after TMA_WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < TMA_WAIT_LIMIT; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void *map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const void *map, int c0, int c1, int c2,
                                            int c3, uint32_t bar) {
  asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
               "r"(bar)
               : "memory");
}

// points per thread: the weights of PPT points stay in registers
template <typename T, int DIM, int NS> __host__ __device__ constexpr int tma_ppt() {
  return DIM * NS * (int)sizeof(T) / 4 <= 12 ? 4 : (DIM * NS * (int)sizeof(T) / 4 <= 24 ? 2 : 1);
}

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(INTERP_TMA_THREADS)
    interp_tma_kernel(const __grid_constant__ CUtensorMap tmap, PointLayout<T> L,
                      KernelShape<T> K, const cplx<T> *__restrict__ fw, int64_t nf_total,
                      const cplx<T> *__restrict__ post, int conj_post, cplx<T> *__restrict__ out,
                      int ntr, int BX, int BY, int BZ, int *err) {
  constexpr int PPT = tma_ppt<T, DIM, NS>();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bars[2];
  const int sub = blockIdx.x;
  const int b = L.sub_bin[sub];
  const int p0 = L.sub_start[sub];
  const int np = L.sub_count[sub];
  if (np <= 0) return;
  const TileGeom<DIM> G = tile_of<T, DIM, NS>(L, b);
  const int xs = G.org[0] - (G.org[0] & 1); // even first x of the box
  const int xoff = G.org[0] - xs;
  bool interior = xs >= 0 && xs + BX <= L.nf[0] && G.org[1] >= 0 && G.org[1] + G.t[1] <= L.nf[1];
  if (DIM == 3) interior = interior && G.org[2] >= 0 && G.org[2] + G.t[2] <= L.nf[2];
  const int bz = DIM == 3 ? BZ : 1;
  const uint32_t box_bytes = (uint32_t)(BX * BY * bz) * (uint32_t)sizeof(cplx<T>);
  const uint32_t buf_stride = (box_bytes + 127u) / 128u * 128u;
  // the copies' destinations must be 128-byte aligned: the dynamic buffer is
  // aligned here (the launch reserves 128 bytes of slack), whatever alignment
  // the shared-memory layout gave it; a misaligned result leaves the block on
  // per-thread loads and records the error
  const uint32_t sraw = smem_addr(smem_raw);
  const uint32_t pad = (128u - (sraw & 127u)) & 127u;
  unsigned char *sm = smem_raw + pad;
  const uint32_t sbuf0 = sraw + pad;
  if ((sbuf0 & 127u) != 0u) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    interior = false;
  }
  const uint32_t bar[2] = {smem_addr(&bars[0]), smem_addr(&bars[1])};
  if (interior && threadIdx.x == 0) {
    mbar_init(bar[0], 1);
    mbar_init(bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t uses[2] = {0u, 0u}; // completed phases awaited per buffer
  const int64_t plane = (int64_t)L.nf[0] * L.nf[1];
  const int xmul = sizeof(T) == 8 ? 2 : 1; // x in tensor-map elements
  auto issue = [&](int k) {
    const int s = k & 1;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar[s], box_bytes);
    if constexpr (DIM == 2)
      tma_load_3d(sbuf0 + s * buf_stride, &tmap, xs * xmul, G.org[1], k, bar[s]);
    else
      tma_load_4d(sbuf0 + s * buf_stride, &tmap, xs * xmul, G.org[1], G.org[2], k, bar[s]);
  };
  // weights of the thread's points of one chunk (PPT * blockDim points): kept
  // across transforms when one chunk holds the subproblem, else recomputed per
  // transform while the tile of that transform serves every chunk
  const int per_chunk = PPT * (int)blockDim.x;
  const bool one_chunk = np <= per_chunk;
  T kx[PPT][NS], ky[PPT][NS], kz[PPT][DIM == 3 ? NS : 1];
  int off[PPT], jj[PPT];
  cplx<T> pf[PPT];
  auto load_weights = [&](int c0) {
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
      const int i = c0 + threadIdx.x + q * (int)blockDim.x;
      off[q] = -1;
      jj[q] = 0;
      pf[q].x = T(1);
      pf[q].y = T(0);
      if (i < np) {
        const int p = p0 + i;
        jj[q] = L.perm[p];
        const int sx = point_weights<T, NS>(L.loc[0][p], L.bin[0], K, kx[q]);
        const int sy = point_weights<T, NS>(L.loc[1][p], L.bin[1], K, ky[q]);
        int sz = 0;
        if constexpr (DIM == 3) sz = point_weights<T, NS>(L.loc[2][p], L.bin[2], K, kz[q]);
        off[q] = (sz * BY + sy) * BX + sx + xoff;
        if (post) {
          pf[q] = post[jj[q]];
          if (conj_post) pf[q].y = -pf[q].y;
        }
      }
    }
  };
  if (one_chunk) load_weights(0);
  for (int k = 0; k < ntr; ++k) {
    const int s = k & 1;
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(sm + s * buf_stride);
    if (interior) {
      if (threadIdx.x == 0) {
        if (k == 0) issue(0);
        if (k + 1 < ntr) issue(k + 1); // its buffer was released at the end of k - 1
      }
      if (!mbar_wait(bar[s], uses[s] & 1u)) {
        // give up: flag it, wait (bounded) for this block's other copy, leave
        if (threadIdx.x == 0) atomicExch(err, 1);
        if (k + 1 < ntr) mbar_wait(bar[s ^ 1], uses[s ^ 1] & 1u);
        return;
      }
      ++uses[s];
    } else {
      // boundary tile: per-thread loads with the periodic wrap, same layout
      const cplx<T> *src = fw + (int64_t)k * nf_total;
      const int rows = G.t[1] * (DIM == 3 ? G.t[2] : 1);
      for (int r = threadIdx.x >> 5; r < rows; r += blockDim.x >> 5) {
        const int y = r % G.t[1], z = r / G.t[1];
        int64_t rb = (int64_t)L.nf[0] * wrap_idx(G.org[1] + y, L.nf[1]);
        if constexpr (DIM == 3) rb += plane * wrap_idx(G.org[2] + z, L.nf[2]);
        cplx<T> *dst = buf + (z * BY + y) * BX + xoff;
        for (int x = threadIdx.x & 31; x < G.t[0]; x += 32)
          dst[x] = src[rb + wrap_idx(G.org[0] + x, L.nf[0])];
      }
      __syncthreads();
    }
    const uint32_t sb = sbuf0 + s * buf_stride;
    constexpr uint32_t CS = sizeof(cplx<T>);
    const uint32_t rs = (uint32_t)BX * CS, ps = (uint32_t)(BX * BY) * CS;
    for (int c0 = 0; c0 < np; c0 += per_chunk) {
      if (!one_chunk) load_weights(c0);
#pragma unroll
      for (int q = 0; q < PPT; ++q) {
        if (off[q] < 0) continue;
        const uint32_t base = sb + (uint32_t)off[q] * CS;
        T accr = T(0), acci = T(0);
#pragma unroll 1
        for (int cc = 0; cc < (DIM == 3 ? NS : 1); ++cc) {
          const uint32_t pl = base + (uint32_t)cc * ps;
          T pr = T(0), pi = T(0);
#pragma unroll
          for (int bb = 0; bb < NS; ++bb) {
            const uint32_t row = pl + (uint32_t)bb * rs;
            T rr = T(0), ri = T(0);
#pragma unroll
            for (int a = 0; a < NS; ++a) {
              T gx, gy;
              lds_cplx(row + a * CS, gx, gy);
              rr = fma(gx, kx[q][a], rr);
              ri = fma(gy, kx[q][a], ri);
            }
            pr = fma(rr, ky[q][bb], pr);
            pi = fma(ri, ky[q][bb], pi);
          }
          if constexpr (DIM == 3) {
            T wz = T(0);
#pragma unroll
            for (int a = 0; a < NS; ++a)
              if (a == cc) wz = kz[q][a];
            accr = fma(pr, wz, accr);
            acci = fma(pi, wz, acci);
          } else {
            accr = pr;
            acci = pi;
          }
        }
        cplx<T> r;
        r.x = accr * pf[q].x - acci * pf[q].y;
        r.y = accr * pf[q].y + acci * pf[q].x;
        const int i = c0 + threadIdx.x + q * (int)blockDim.x;
        if (L.sorted_out)
          static_cast<cplx<T> *>(L.sorted_out)[(int64_t)k * L.M + p0 + i] = r;
        else
          out[(int64_t)k * L.M + jj[q]] = r;
      }
    }
    __syncthreads(); // buffer s is free for the copy of transform k + 2
  }
}
