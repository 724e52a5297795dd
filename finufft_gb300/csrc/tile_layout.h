// Shared-memory tile geometry of the spreading kernels (host and device).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace gbn {

// x pitch of the shared tile: in 3D a multiple of 16 plus 8 words, so the four
// rows an 8 x 4 lane patch touches start in disjoint bank octets.
__host__ __device__ constexpr int tile_pitch_x(int dim, int tx) {
  return dim == 3 ? (tx <= 8 ? 8 : 16 * ((tx - 8 + 15) / 16) + 8) : tx;
}

__host__ __device__ constexpr int tile3_py(int ty, int ns) {
  return ty + (((ns - ty) % 4) + 4) % 4;
}
constexpr int STAGE_STRIDE = 33; // padded so 32 lanes write/read distinct banks
template <typename T> __host__ __device__ constexpr int stage_bytes_per_warp(int ns) {
  return ((STAGE_STRIDE * (3 * ns + 2) * (int)sizeof(T) + STAGE_STRIDE * 4) + 15) / 16 * 16;
}
template <typename T>
__host__ __device__ constexpr size_t tile3_bytes(int ns, int bx, int by, int bz) {
  return (2 * sizeof(T) * (size_t)tile_pitch_x(3, bx + ns) * tile3_py(by + ns, ns) * (bz + ns) +
          15) / 16 * 16;
}

// Exclusive-warp 3D spread: points staged per step and staging bytes.
__host__ __device__ constexpr int t3w_chunk(int ns, int tsize) {
  return (tsize == 8 && ns > 8) ? 16 : 32;
}
__host__ __device__ constexpr int t3w_stage_bytes(int ns, int tsize) {
  return ((t3w_chunk(ns, tsize) + 1) * (ns + 4 * ((ns * ns + 3) / 4) + 2) * tsize +
          (t3w_chunk(ns, tsize) + 1) * 4 + 15) / 16 * 16;
}

// Warp-aggregated 3D spread: staging of one warp (x weights, (y,z) weight
// products padded to 4*ceil(ns^2/4) rows, strengths, packed start cells).
__host__ __device__ constexpr int t3m_stage_bytes(int ns, int tsize) {
  return (33 * (ns + 4 * ((ns * ns + 3) / 4) + 2) * tsize + 33 * 4 + 15) / 16 * 16;
}

} // namespace gbn
