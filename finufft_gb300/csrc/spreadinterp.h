// Spread (type 1) and interpolation (type 2) kernel launchers.
#pragma once
#include "common.h"

namespace gbn {

struct SpreadConfig {
  int method;       // 1: point-driven global atomics, 2: tiled shared memory,
                    // 3: output-driven tiles (one writer per cell)
  int threads;      // CTA size
  size_t smem;      // dynamic shared memory bytes for method 2
  int variant = 0;  // 3D method 2: 0 shared tile + atomics, 1 exclusive warp tiles
  int fixed = 0;    // 3D variant 3, single precision, ns <= 6: int32 fixed-point tile
};

// Shared-memory bytes of the tiled spread for a given tile and kernel width.
template <typename T> size_t spread_tile_smem(int dim, int ns, const int bin[3], int threads);
// Shared-memory bytes of the exclusive-warp 3D spread (variant 1).
template <typename T> size_t spread_tile3w_bytes(int ns, const int bin[3]);
// Shared-memory bytes of the warp-aggregated 2D spread (variant 2, 8 warps).
template <typename T> size_t spread_tile2m_bytes(int ns, const int bin[3], int warps = 8);
template <typename T> size_t spread_tile3v_bytes(int ns, const int bin[3], int warps);
// Shared-memory bytes of the warp-aggregated 3D spread (variant 2).
template <typename T> size_t spread_tile3m_bytes(int ns, const int bin[3], int warps);
// Shared-memory bytes of the output-driven spread (method 3).
template <typename T> size_t spread_output_driven_bytes(int dim, int ns, const int bin[3]);
// Shared-memory bytes of the double-precision int64 fixed-point 3D spread (variant 4).
size_t spread_tile3x_bytes(int ns, const int bin[3]);

// A device word (one per device, allocated at first use) where kernels whose
// bounded waits give up record it; device_error_take reads and clears it.
int *device_error_word();
int device_error_take();

// iperm[perm[p]] = p for p < M (perm a permutation of 0 .. M-1).
void launch_invert_perm(const int *perm, int M, int *iperm, cudaStream_t s);

// fw[t*nf + g] += sum_j c[t*M + j] (* pre[j] or conj(pre[j])) phi(g - x_j), t < ntr.
// fw must be zeroed by the caller.
template <typename T>
void launch_spread(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *c,
                   const cplx<T> *pre, int conj_pre, cplx<T> *fw, int64_t nf_total, int ntr,
                   const SpreadConfig &cfg, cudaStream_t s);

// out[t*M + j] = (post ? post[j] : 1) * sum_g fw[t*nf + g] phi(g - x_j), t < ntr.
template <typename T>
void launch_interp(const PointLayout<T> &L, const KernelShape<T> &K, const cplx<T> *fw,
                   int64_t nf_total, const cplx<T> *post, int conj_post, cplx<T> *out, int ntr,
                   cudaStream_t s);

} // namespace gbn
