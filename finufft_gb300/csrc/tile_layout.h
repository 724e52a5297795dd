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

// Warp-aggregated 3D spread with x slack and vector staging (ns <= 8). A run of
// points sharing their (y, z) start cells whose x starts lie within 8 - ns
// cells of the run's first point is summed in registers over an 8-cell x
// window. Per point, the (y, z) weight products a lane needs (pairs 4r + lane
// row) are stored contiguously so a lane reads them as 16-byte vectors; the
// last vectors of a point block hold its strength and packed start cells.
//   vw: elements per 16-byte vector; nrv: vectors per lane row; lps: lane-row
//   stride in vectors (the four rows read at once fall in distinct bank groups);
//   qs: point stride in vectors (odd, so 8 points' stores hit distinct groups)
__host__ __device__ constexpr int t3v_vw(int tsize) { return 16 / tsize; }
__host__ __device__ constexpr int t3v_nr(int ns) { return (ns * ns + 3) / 4; }
__host__ __device__ constexpr int t3v_nrv(int ns, int tsize) {
  return (t3v_nr(ns) + t3v_vw(tsize) - 1) / t3v_vw(tsize);
}
__host__ __device__ constexpr int t3v_lps(int ns, int tsize) {
  return t3v_nrv(ns, tsize) % 4 == 0 ? t3v_nrv(ns, tsize) + 1 : t3v_nrv(ns, tsize);
}
__host__ __device__ constexpr int t3v_hdr(int tsize) { return tsize == 4 ? 1 : 2; }
__host__ __device__ constexpr int t3v_qs(int ns, int tsize) {
  return (4 * t3v_lps(ns, tsize) + t3v_hdr(tsize)) | 1;
}
__host__ __device__ constexpr int t3v_xs(int ns) { return 8 - ns; }    // x slack of a run
__host__ __device__ constexpr int t3v_kxr(int ns) { return 8 + t3v_xs(ns); } // x rows
__host__ __device__ constexpr int t3v_stage_bytes(int ns, int tsize) {
  return (t3v_kxr(ns) * 33 * tsize + 15) / 16 * 16 + 32 * t3v_qs(ns, tsize) * 16;
}
// threads per block of that kernel at most (its register budget assumes two
// blocks per SM)
template <typename T> __host__ __device__ constexpr int t3v_max_threads() {
  return sizeof(T) == 4 ? 320 : 256;
}
template <typename T>
__host__ __device__ constexpr size_t tile3v_bytes(int ns, int bx, int by, int bz) {
  return (2 * sizeof(T) * (size_t)tile_pitch_x(3, bx + 8) * tile3_py(by + ns, ns) * (bz + ns) +
          15) / 16 * 16;
}

// Double-precision 3D spread into an int64 fixed-point tile (variant 4). The
// tile is (bin + ns) cells per dimension, unpadded, re and im as int64 planes.
// Staging: sb points per buffer, two buffers; a point holds U_z (ns x two
// int64), the y and x weights (ns x two int32 each) and its three start cells.
constexpr int T3X_THREADS = 512; // block size the kernel's row mapping assumes
__host__ __device__ constexpr int t3x_sb(int ns) { return ns <= 8 ? 128 : (ns <= 13 ? 64 : 32); }
__host__ __device__ constexpr int t3x_point_bytes(int ns) { return 32 * ns + 16; }
__host__ __device__ constexpr size_t t3x_tile_bytes(int ncell) { return (size_t)16 * ncell; }
__host__ __device__ constexpr size_t t3x_bytes(int ns, int bx, int by, int bz) {
  return t3x_tile_bytes((bx + ns) * (by + ns) * (bz + ns)) +
         (size_t)2 * t3x_sb(ns) * t3x_point_bytes(ns);
}

} // namespace gbn
