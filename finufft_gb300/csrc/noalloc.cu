// Spreading without device allocation: cufinufftf_spread_noalloc.
//
// Who needs this: a caller whose device memory is not its own to allocate --
// for instance a plugin running inside a host framework that owns the GPU's
// memory through its own pool and forbids foreign cudaMalloc calls, or a
// real-time pipeline that reserves all device memory at start-up and must not
// grow its footprint (or pay cudaMalloc's synchronization) once running.
// Such a caller passes its inputs and output grid and this entry point works
// entirely inside a fixed scratch area compiled into the library.
//
// The scratch is one file-scope __device__ array of NOALLOC_SCRATCH_BYTES.
// Every GPU that loads the library holds it until the process exits. All calls
// share it: two calls that overlap on the GPU (different streams, or
// different host threads without ordering) race on it and corrupt each
// other's results; order them on one stream or serialize them.
#include <cstdio>
#include <mutex>

#include "common.h"
#include "cufinufft.h"
#include "gbnufft_ext.h"
#include "plan.h"
#include "planning.h"
#include "sort.h"

namespace gbn {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20; // 32 MiB per GPU
constexpr int64_t NOALLOC_MAX_POINTS = int64_t(1) << 19;    // 524288 points
constexpr int64_t NOALLOC_MAX_CELLS = int64_t(1) << 24;     // grid cells

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
void *g_scratch_addr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device. In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached. The cached address
// is checked at every call: after a reset of the device's context the module
// is loaded again and the array may move, so an address the runtime no longer
// knows as device memory of this device is looked up again.
void *scratch_address() {
  int dev = 0;
  GBN_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "device index");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_addr[dev]) {
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, g_scratch_addr[dev]);
    if (e != cudaSuccess || a.type != cudaMemoryTypeDevice || a.device != dev) {
      cudaGetLastError();
      g_scratch_addr[dev] = nullptr;
    }
  }
  if (!g_scratch_addr[dev]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      fprintf(stderr, "[gbnufft] cudaGetSymbolAddress of the no-alloc scratch failed: %s\n",
              cudaGetErrorString(e));
      GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "scratch symbol");
    }
    g_scratch_addr[dev] = ptr;
  }
  return g_scratch_addr[dev];
}

int spread_noalloc_f(int dim, const int64_t *n_grid, int64_t M, const float *x, const float *y,
                     const float *z, const float2 *c, float2 *grid, float eps,
                     cudaStream_t stream) {
  if (dim < 1 || dim > 3) return FINUFFT_ERR_DIM_NOTVALID;
  if (!n_grid || M < 0) return FINUFFT_ERR_NDATA_NOTVALID;
  int nf[3] = {1, 1, 1};
  int64_t cells = 1;
  for (int d = 0; d < dim; ++d) {
    if (n_grid[d] < 1 || n_grid[d] > NOALLOC_MAX_CELLS) return FINUFFT_ERR_NDATA_NOTVALID;
    nf[d] = (int)n_grid[d];
    cells *= n_grid[d];
  }
  if (cells > NOALLOC_MAX_CELLS || M > NOALLOC_MAX_POINTS) {
    fprintf(stderr,
            "[gbnufft] cufinufftf_spread_noalloc: %lld points / %lld cells exceed the fixed "
            "scratch limits (%lld points, %lld cells)\n",
            (long long)M, (long long)cells, (long long)NOALLOC_MAX_POINTS,
            (long long)NOALLOC_MAX_CELLS);
    return FINUFFT_ERR_MAXNALLOC;
  }
  if (M > 0 && (!x || (dim > 1 && !y) || (dim > 2 && !z) || !c))
    return FINUFFT_ERR_INVALID_ARGUMENT;
  if (!grid) return FINUFFT_ERR_INVALID_ARGUMENT;
  try {
    cufinufft_opts opts;
    cufinufft_default_opts(&opts);
    opts.gpu_spreadinterponly = 1;
    GBN_CUDA(cudaGetDevice(&opts.gpu_device_id));
    gbnufft_opts ext;
    gbnufft_default_opts(&ext);
    // kernel and tiling exactly as a spread-only type-1 plan with default options
    // (a spread-only plan keeps the GPU library's ES kernel: its output is the
    // raw spread, whose values depend on the kernel shape)
    const KernelChoice kc = choose_kernel(eps, 2.0, 1, 1, 1, 0);
    KernelShape<float> K;
    build_kernel_shape<float>(make_kernel_fn(KERNEL_ES, kc.ns, kc.beta), 1, eps, &K);
    const SpreadSetup S = spread_setup<float>(dim, kc.ns, nf, opts, ext, false);

    Arena arena;
    arena.base = static_cast<unsigned char *>(scratch_address());
    arena.cap = NOALLOC_SCRATCH_BYTES;
    const size_t mb = (size_t)(M > 0 ? M : 1);
    uint32_t *keys = (uint32_t *)arena.take(mb * 4);
    uint32_t *skeys = (uint32_t *)arena.take(mb * 4);
    int *perm = (int *)arena.take(mb * 4);
    float *loc[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < dim; ++d) loc[d] = (float *)arena.take(mb * 4);
    for (int d = dim; d < 3; ++d) loc[d] = loc[0];

    // sort keys as a plan's (Plan::sort_points): bin and cell, for odd widths
    // bin and start cell of the support (bin + 1 values per dimension)
    const int nb = S.nbins[0] * S.nbins[1] * S.nbins[2];
    const uint64_t binvol0 = (uint64_t)S.bins[0] * S.bins[1] * S.bins[2];
    uint64_t sbinvol = 1;
    for (int d = 0; d < dim; ++d) sbinvol *= (uint64_t)S.bins[d] + 1;
    int cell_keys = (uint64_t)nb * binvol0 <= 0xffffffffull ? 1 : 0;
    if (cell_keys && kc.ns % 2 == 1 && (uint64_t)nb * sbinvol <= 0xffffffffull) cell_keys = 2;
    const uint64_t binvol = cell_keys == 2 ? sbinvol : binvol0;
    const uint64_t nkeys = cell_keys ? (uint64_t)nb * binvol : (uint64_t)nb;
    int keybits = 0;
    while ((1ull << keybits) < nkeys) ++keybits;
    AxisMap ax[3];
    for (int d = 0; d < 3; ++d) ax[d] = AxisMap{0.0, 1.0, nf[d], S.bins[d]};
    const float *xyz[3] = {x, dim > 1 ? y : x, dim > 2 ? z : x};
    if (M > 0) {
      launch_bin_keys<float>(dim, xyz, (int)M, ax, S.nbins, cell_keys, keys, stream);
      stable_sort_by_bin(keys, (int)M, keybits, skeys, perm, stream, &arena);
      launch_sorted_local<float>(dim, xyz, perm, (int)M, ax, loc, stream);
    }
    SubproblemArrays sa;
    const int nsub = build_subproblems(skeys, (int)M, nb, cell_keys ? (uint32_t)binvol : 1u,
                                       S.maxsub, &sa, stream, &arena);
    // the output starts at zero; nothing else in the scratch needs clearing
    // (bin counters are cleared inside build_subproblems)
    GBN_CUDA(cudaMemsetAsync(grid, 0, (size_t)cells * sizeof(float2), stream));
    PointLayout<float> L;
    L.dim = dim;
    for (int d = 0; d < 3; ++d) {
      L.nf[d] = nf[d];
      L.bin[d] = S.bins[d];
      L.nbin[d] = S.nbins[d];
      L.loc[d] = loc[d];
    }
    L.M = (int)M;
    L.nsub = nsub;
    L.sub_bin = sa.bin;
    L.sub_start = sa.start;
    L.sub_count = sa.count;
    L.perm = perm;
    L.cell_sorted = cell_keys ? 1 : 0;
    launch_spread<float>(L, K, c, nullptr, 0, grid, cells, 1, S.cfg, stream);
    GBN_CUDA(cudaGetLastError());
    return 0;
  } catch (const Error &e) {
    return e.code;
  } catch (...) {
    return FINUFFT_ERR_UNKNOWN_EXCEPTION;
  }
}

} // namespace
} // namespace gbn

extern "C" int cufinufftf_spread_noalloc(int dim, const int64_t *n_grid, int64_t M,
                                         const float *d_x, const float *d_y, const float *d_z,
                                         const cuFloatComplex *d_c, cuFloatComplex *d_grid,
                                         float eps, void *stream) {
  return gbn::spread_noalloc_f(dim, n_grid, M, d_x, d_y, d_z, (const float2 *)d_c,
                               (float2 *)d_grid, eps, (cudaStream_t)stream);
}
