// Device bin sort of nonuniform points (setpts stage).
#pragma once
#include <cstdint>
#include "common.h"
#include "device_util.cuh"

namespace gbn {

// A caller-provided block of device memory handed out front to back
// (256-byte aligned pieces, never freed individually).
struct Arena {
  unsigned char *base = nullptr;
  size_t cap = 0, used = 0;
  void *take(size_t bytes) {
    const size_t at = (used + 255) / 256 * 256;
    if (at + bytes > cap) GBN_THROW(FINUFFT_ERR_ALLOC, "scratch arena exhausted");
    used = at + bytes;
    return base + at;
  }
};

// Device scratch: from an Arena when one is given, else stream-ordered
// cudaMallocAsync / cudaFreeAsync.
// Stream-ordered pool of the current device for setpts scratch (keys,
// records, sort buffers). It keeps freed memory for the next setpts instead of
// returning it to the CUDA driver at every synchronisation (the default pool's
// behaviour), which would re-map gigabytes per call; gbnufft_trim_scratch
// releases it.
cudaMemPool_t scratch_pool();
void trim_scratch_pool(); // release the current device's cached scratch

struct AsyncBuf {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  bool owned = false;
  AsyncBuf() = default;
  AsyncBuf(size_t bytes, cudaStream_t st, Arena *arena = nullptr) : s(st) {
    if (!bytes) return;
    if (arena) {
      p = arena->take(bytes);
    } else {
      GBN_CUDA(cudaMallocFromPoolAsync(&p, bytes, scratch_pool(), st));
      owned = true;
    }
  }
  ~AsyncBuf() {
    if (p && owned) cudaFreeAsync(p, s);
  }
  AsyncBuf(const AsyncBuf &) = delete;
  AsyncBuf &operator=(const AsyncBuf &) = delete;
  template <typename U> U *as() const { return (U *)p; }
};

// Exclusive prefix sum of n int32 values (out may alias nothing of in).
void exclusive_scan_i32(const int *in, int *out, int64_t n, cudaStream_t s,
                        Arena *arena = nullptr);

// Sort key of every point: bin = bx + nb0*(by + nb1*bz) (x fastest); with
// cell_keys, bin * binvol + the cell inside the bin (x fastest).
template <typename T>
// With rec non-null it also writes each point's bin-local coordinates, in
// input order, as one record of 4 T (x, y, z, 0) at rec + 4 * i.
void launch_bin_keys(int dim, const T *const xyz[3], int M, const AxisMap ax[3],
                     const int nbin[3], int cell_keys, uint32_t *keys, cudaStream_t s,
                     T *rec = nullptr);

// Stable LSD radix sort of (key, index) pairs by the low `keybits` bits of key.
// On return perm_out[p] is the user index of the p-th point in bin order and
// keys_out[p] its bin. keys_in is clobbered.
void stable_sort_by_bin(uint32_t *keys_in, int M, int keybits, uint32_t *keys_out,
                        int *perm_out, cudaStream_t s, Arena *arena = nullptr);

// Per-bin [start, count) of the sorted keys and subproblem decomposition.
// Returns the number of subproblems (one device->host copy, stream sync).
struct SubproblemArrays {
  int *bin = nullptr, *start = nullptr, *count = nullptr;
  size_t cap = 0; // entries the three arrays hold
};
// binvol: keys per bin (1 for plain bin keys). With an arena the three output
// arrays are carved from it (nothing to free); otherwise the arrays in *out
// are kept when they hold enough entries, else cudaFree'd and cudaMalloc'd.
int build_subproblems(const uint32_t *sorted_keys, int M, int nbins, uint32_t binvol,
                      int maxsub, SubproblemArrays *out, cudaStream_t s,
                      Arena *arena = nullptr);

// Sorted bin-local coordinates loc[d][p] in [0, bin_d], grid units.
template <typename T>
void launch_sorted_local(int dim, const T *const xyz[3], const int *perm, int M,
                         const AxisMap ax[3], T *const loc[3], cudaStream_t s);
// The same from the records of launch_bin_keys (a gather, no refold).
template <typename T>
void launch_gather_local(int dim, const T *rec, const int *perm, int M, T *const loc[3],
                         cudaStream_t s);

} // namespace gbn
