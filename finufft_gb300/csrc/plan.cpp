// NUFFT plan orchestration: makeplan, setpts, execute (types 1, 2, 3), adjoint.
//
// Stage order follows the reference GPU library (src/cuda/makeplan.cu:223-398,
// src/cuda/setpts.cu:25-314, src/cuda/execute.cu:105-258); buffers are sized at
// plan/setpts time so execute allocates nothing and can be captured in a CUDA graph.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <cfloat>

#include "planning.h"
#include "sort.h"
#include "tile_layout.h"

extern "C" void gbnufft_default_opts(gbnufft_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->planner = 0;
  o->spread_variant = -1;
}

namespace gbn {

int plan_kernel_form(const gbnufft_opts &ext, const cufinufft_opts &opts)
// gbnufft_opts.kernel_form 0 (auto): the CPU library's PSWF, except under the
// reference-heuristic planner, with direct kernel evaluation (gpu_kerevalmeth
// 0; ES is the only form with a closed-form value) and for spread- or
// interpolation-only plans, which keep the GPU library's ES kernel.
// 1: ES, 2: PSWF.
{
  if (ext.kernel_form == KERNEL_ES || ext.kernel_form == KERNEL_PSWF) return ext.kernel_form;
  if (ext.kernel_form != 0) {
    fprintf(stderr, "[gbnufft] invalid kernel_form %d (0 auto, 1 ES, 2 PSWF)\n", ext.kernel_form);
    GBN_THROW(FINUFFT_ERR_KERFORMULA_NOTVALID, "kernel_form");
  }
  if (ext.planner == 1 || opts.gpu_kerevalmeth == 0) return KERNEL_ES;
  // a spread/interpolation-only plan returns the raw spread (or reads a raw
  // grid), whose values depend on the kernel shape: keep the GPU library's
  if (opts.gpu_spreadinterponly) return KERNEL_ES;
  return KERNEL_PSWF;
}

DeviceScope::DeviceScope(int dev) {
  GBN_CUDA(cudaGetDevice(&prev));
  if (dev != prev) {
    GBN_CUDA(cudaSetDevice(dev));
    switched = true;
  }
}
DeviceScope::~DeviceScope() {
  if (switched) cudaSetDevice(prev);
}

namespace {
int max_smem_optin(int dev) {
  int v = 0;
  GBN_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  return v;
}
int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
} // namespace

template <typename T>
Plan<T>::Plan(int type_, int dim_, const int64_t *modes_in, int iflag_, int ntransf_,
              double tol_, const cufinufft_opts &opts_, const gbnufft_opts *ext_)
    : type(type_), dim(dim_), ntransf(ntransf_), iflag(iflag_ >= 0 ? 1 : -1), batchsize(1),
      tol(tol_), opts(opts_) {
  if (ext_) ext = *ext_;
  else gbnufft_default_opts(&ext);
  // planners 0 and 1 are fixed rules; 2 and 3 set this at setpts (1 on fallback)
  planner_used = (ext.planner == 1) ? 1 : 0;
  if (dim < 1 || dim > 3) GBN_THROW(FINUFFT_ERR_DIM_NOTVALID, "dim");
  DeviceScope ds(opts.gpu_device_id);
  if (type < 1 || type > 3) {
    fprintf(stderr, "[gbnufft] invalid type (%d): should be 1, 2, or 3\n", type);
    GBN_THROW(FINUFFT_ERR_TYPE_NOTVALID, "type");
  }
  if (ntransf < 1) {
    fprintf(stderr, "[gbnufft] invalid ntransf (%d): should be at least 1\n", ntransf);
    GBN_THROW(FINUFFT_ERR_NTRANS_NOTVALID, "ntransf");
  }
  if (opts.gpu_method < 0 || opts.gpu_method > 4) GBN_THROW(FINUFFT_ERR_METHOD_NOTVALID, "method");
  if (opts.gpu_method == 4 && dim != 3) GBN_THROW(FINUFFT_ERR_METHOD_NOTVALID, "method 4 is 3D only");
  stream = (cudaStream_t)opts.gpu_stream;
  if (ext.planner < 0 || ext.planner > 3) {
    fprintf(stderr, "[gbnufft] invalid planner %d (0 engine, 1 reference heuristic, 2 learned, "
                    "3 autotuned)\n", ext.planner);
    GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "planner");
  }
  form = plan_kernel_form(ext, opts);
  if (type == 3) opts.gpu_spreadinterponly = 1; // the outer type 1 only spreads
  else
    for (int d = 0; d < dim; ++d) ms[d] = (int)modes_in[d];
  nmodes = (int64_t)ms[0] * ms[1] * ms[2];
  batchsize = opts.gpu_maxbatchsize > 0 ? opts.gpu_maxbatchsize : std::min(ntransf, 8);
  if (type == 3) batchsize = std::min(batchsize, ntransf);
  user_sigma = opts.upsampfac != 0.0;
  if (opts.upsampfac == 0.0) {
    // reference rule (src/cuda/makeplan.cu:289-297): 2, or 1.25 for type 3 at
    // tol >= 1e-9. In single precision sigma 1.25 loses digits to the wide range
    // of 1/phihat (4e-4 error at tol 1e-6), so this engine keeps 2 there below 1e-4.
    opts.upsampfac = 2.0;
    const bool f32 = std::is_same_v<T, float>;
    if (type == 3 && tol >= 1e-9 && (ext.planner == 1 || !f32 || (float)tol >= 1e-4f))
      opts.upsampfac = 1.25;
  }
  make_kernel();
  if (type != 3) make_grid();
  if (opts.debug)
    printf("[gbnufft] type %d dim %d ntr %d: ns=%d beta=%.4g sigma=%.3g nf=(%d,%d,%d) "
           "method=%d bins=(%d,%d,%d) batch=%d horner_err=%.2e\n",
           type, dim, ntransf, K.ns, (double)K.beta, opts.upsampfac, nf[0], nf[1], nf[2],
           method, bins[0], bins[1], bins[2], batchsize, horner_err);
}

// Kernel width and shape at the plan's tolerance and upsampling factor.
template <typename T> void Plan<T>::make_kernel() {
  const bool is_float = std::is_same_v<T, float>;
  const KernelChoice kc =
      form == KERNEL_PSWF
          ? choose_kernel_pswf(tol, opts.upsampfac, dim, type, is_float, ext.kerformula,
                               user_sigma ? opts.gpu_kerevalmeth : 0, opts.gpu_spreadinterponly,
                               opts.debug)
          : choose_kernel(tol, opts.upsampfac, opts.gpu_kerevalmeth, is_float,
                          opts.gpu_spreadinterponly, opts.debug);
  horner_err = build_kernel_shape<T>(make_kernel_fn(form, kc.ns, kc.beta),
                                     opts.gpu_kerevalmeth == 1, tol, &K);
}

// Types 1/2: fine grid, spread configuration, grid buffers, FFT plan and
// 1/phihat (again when a planner changes the upsampling factor at setpts).
template <typename T> void Plan<T>::make_grid() {
  for (int d = 0; d < dim; ++d)
    nf[d] = opts.gpu_spreadinterponly ? ms[d] : (int)fine_grid_len(ms[d], opts.upsampfac, K.ns);
  nf_total = (int64_t)nf[0] * nf[1] * nf[2];
  choose_spread_config(opts.gpu_method != 0);
  if (!opts.gpu_spreadinterponly) {
    // 3D type 2: transforms per batch at most as many as keep their fine grids
    // within half of L2. Each interpolation tile re-reads its halo (3.6x the
    // bin's cells at 16x12x8 bins and ns 6), cheap while the grid is in L2
    // (5e6 points, 192^3 grids, 8 vectors: batches of 1 4.70 ms per execute, of
    // 8 5.29 ms). 2D and type 1 batch freely: the interpolation reuses each
    // point's weights over the batch's transforms and the batched FFT is more
    // efficient (2D type 2, 16 vectors of 1e7 points, 2048^2 grids: batches of
    // 2 6.27 ms, of 16 5.70 ms; 3D type 1 as above: 7.23 against 6.95 ms).
    // gpu_maxbatchsize is an upper bound; gbnufft_opts.batch_cap = 1 lifts the cap.
    int dev = 0, l2 = 0;
    GBN_CUDA(cudaGetDevice(&dev));
    GBN_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
    const double gbytes = (double)nf_total * sizeof(cplx<T>);
    if (ext.batch_cap == 0 && dim == 3 && type == 2 && 2.0 * gbytes <= (double)l2)
      batchsize = std::min(batchsize, std::max(1, (int)((double)l2 / (2.0 * gbytes))));
    destroy_fft();
    fw.resize((size_t)nf_total * batchsize);
    make_fft();
    make_fseries();
  }
}

template <typename T> void Plan<T>::destroy_fft() {
  if (have_fft) cufftDestroy(fftplan);
  if (fft_x) cufftDestroy(fft_x);
  if (fft_rest0) cufftDestroy(fft_rest0);
  if (fft_rest1) cufftDestroy(fft_rest1);
  have_fft = pruned = false;
  fftplan = fft_x = fft_rest0 = fft_rest1 = 0;
}

template <typename T> Plan<T>::~Plan() {
  try {
    DeviceScope ds(opts.gpu_device_id);
    destroy_fft();
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  } catch (...) {
  }
}

template <typename T>
SpreadSetup spread_setup(int dim, int ns, const int nf[3], const cufinufft_opts &opts,
                         const gbnufft_opts &ext, bool user_method) {
  SpreadSetup S;
  // bins: the user's values, else this engine's defaults per dimension
  const int limit = max_smem_optin(opts.gpu_device_id);
  const int threads = (dim == 3 && !std::is_same_v<T, float>) ? 128 : 256;
  int def = dim == 1 ? 1024 : (dim == 2 ? 32 : 8);
  if (ext.planner == 1) {
    // the reference library's bin sizes (src/cuda/heuristics.cu:50-57,373-392):
    // method 1 (its default for type 2) 1D 1024, 2D 40, 3D 8; method 2 1D 1024,
    // 2D 40, 3D from a shared-memory budget of 50/90/100% by width
    def = dim == 1 ? 1024 : (dim == 2 ? 40 : (opts.gpu_method == 1 ? 8 : 0));
    if (dim == 3 && def == 0) {
      const double load = ns <= 6 ? 0.5 : (ns <= 10 ? 0.9 : 1.0);
      auto fit = [&](double bytes) {
        const double elems = std::floor(bytes / (2.0 * sizeof(T)));
        return (int)std::floor(std::pow(elems, 1.0 / 3.0)) - (ns + 1);
      };
      def = fit(limit * load);
      if (def < 1) def = fit(limit);
      if (def < 1) def = 1;
    }
  } else if (dim == 3) { // largest even bin (<= 8) whose tile and staging fit
    while (def > 2) {
      const int b3[3] = {def, def, def};
      if (spread_tile_smem<T>(3, ns, b3, threads) <= (size_t)limit) break;
      def -= 2;
    }
  }
  int defb[3] = {def, def, def};
  // single-precision 3D spread with register runs (variant 3): wider bins and
  // larger subproblems amortise the tile clear and write-back (measured on the
  // 1e8-point clustered 512^3 case: 16x12x8 bins, 4096-point subproblems)
  const bool v3_default = dim == 3 && ext.planner == 0 && std::is_same_v<T, float> && ns <= 8 &&
                          (ext.spread_variant < 0 || ext.spread_variant == 3);
  if (v3_default) {
    defb[0] = 16;
    defb[1] = ns <= 6 ? 12 : 8;
    defb[2] = 8;
  }
  int *bins = S.bins, *nbins = S.nbins;
  bins[0] = opts.gpu_binsizex > 0 ? opts.gpu_binsizex : defb[0];
  bins[1] = dim > 1 ? (opts.gpu_binsizey > 0 ? opts.gpu_binsizey : defb[1]) : 1;
  bins[2] = dim > 2 ? (opts.gpu_binsizez > 0 ? opts.gpu_binsizez : defb[2]) : 1;
  // the reference default (1024) stands for "not set" under this engine's planner
  S.maxsub = opts.gpu_maxsubprobsize;
  if (v3_default && opts.gpu_maxsubprobsize == 1024) S.maxsub = 4096;
  for (int d = 0; d < 3; ++d) {
    if (d >= dim) bins[d] = 1;
    nbins[d] = d < dim ? ceil_div(nf[d], bins[d]) : 1;
  }
  if (dim == 3 && (bins[0] > 1000 || bins[1] > 1000 || bins[2] > 1000))
    GBN_THROW(FINUFFT_ERR_BINSIZE_NOTVALID, "3D bins must be < 1000");
  if (opts.gpu_maxsubprobsize < 1) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "maxsubprobsize");
  // methods: 1 global atomics, 2 shared-memory tiles (also for 4, the reference's
  // block-gather, accepted for compatibility), 3 output-driven tiles
  S.method = opts.gpu_method == 0 ? 2 : (opts.gpu_method == 1 ? 1 : (opts.gpu_method == 3 ? 3 : 2));
  if (S.method == 3) {
    S.smem = spread_output_driven_bytes<T>(dim, ns, bins);
    if (S.smem > (size_t)limit) {
      fprintf(stderr, "[gbnufft] output-driven tile needs %zu bytes of shared memory, %d "
                      "available\n", S.smem, limit);
      GBN_THROW(FINUFFT_ERR_INSUFFICIENT_SHMEM, "tile too large");
    }
    S.cfg.method = 3;
    S.cfg.threads = 256;
    S.cfg.smem = S.smem;
    S.cfg.variant = 0;
    return S;
  }
  S.smem = spread_tile_smem<T>(dim, ns, bins, threads);
  if (S.method == 2 && S.smem > (size_t)limit) {
    if (user_method) {
      fprintf(stderr, "[gbnufft] tile needs %zu bytes of shared memory, %d available\n", S.smem,
              limit);
      GBN_THROW(FINUFFT_ERR_INSUFFICIENT_SHMEM, "tile too large");
    }
    S.method = 1;
  }
  S.cfg.method = S.method;
  S.cfg.threads = threads;
  S.cfg.smem = S.method == 2 ? S.smem : 0;
  S.cfg.variant = 0;
  if (dim == 2 && S.method == 2) {
    // 2D: 0 shared tile + per-point atomics (thread per point), 1 one warp per
    // tile with same-cell runs added by plain read-modify-writes, 2 eight warps
    // per tile with runs added by atomics
    int variant = ext.planner == 1 ? 0 : 2;
    if (ext.spread_variant >= 0) variant = ext.spread_variant;
    if (variant < 0 || variant > 2) variant = 0;
    const int warps2 = variant == 1 ? 1 : 8;
    const size_t sm2 = spread_tile2m_bytes<T>(ns, bins, warps2);
    if (variant >= 1 && (sm2 > (size_t)limit || bins[0] + ns >= 65536 || bins[1] + ns >= 32768))
      variant = 0;
    if (variant >= 1) {
      S.cfg.variant = variant;
      S.cfg.threads = 32 * warps2;
      S.cfg.smem = sm2;
      S.smem = sm2;
    }
  }
  if (dim == 3 && S.method == 2) {
    // 3D tiled variants: 0 shared tile + per-point atomics, 1 exclusive-warp tiles,
    // 2 shared tile + per-run (warp-aggregated) atomics, 3 as 2 with x-slack runs
    // and vector staging
    const size_t wsm = spread_tile3w_bytes<T>(ns, bins);
    // per-run register accumulators cost 2*ceil(ns/8)*ceil(ns^2/4) registers, so
    // the warp-aggregated variant is used for ns <= 8 only
    // default: 3 where its accumulators fit the register budget without spills
    // (single precision ns <= 8, double ns <= 5), else 2 for ns <= 8, else 0
    // double precision above that: 4, the int64 fixed-point tile summed with
    // integer products (no FP64 in the per-cell work)
    const bool dbl = std::is_same_v<T, double>;
    const bool v3ok = !dbl ? ns <= 8 : ns <= 5;
    int variant = ext.planner == 1 ? 0 : (v3ok ? 3 : (dbl ? 4 : (ns <= 8 ? 2 : 0)));
    if (ext.spread_variant >= 0) variant = ext.spread_variant;
    if (variant == 1 && wsm > (size_t)limit) variant = 2;
    if (variant == 4 && dbl) {
      // one block of 16 warps per SM sharing the tile and the staging buffers
      const size_t xsm = spread_tile3x_bytes(ns, bins);
      if (xsm <= (size_t)limit) {
        S.cfg.variant = 4;
        S.cfg.threads = T3X_THREADS;
        S.cfg.smem = xsm;
        S.smem = xsm;
        return S;
      }
      variant = 0;
    }
    if (variant < 0 || variant > 3 || (variant >= 2 && ns > 8)) variant = 0;
    if (variant == 3) {
      // 3: variant 2 with x-slack runs and vector staging; the most warps (within
      // the kernel's launch bound) that keep two blocks per SM, else that fit one
      const int half = 113 * 1024;
      const int wmax = t3v_max_threads<T>() / 32;
      int w = wmax;
      while (w > 4 && spread_tile3v_bytes<T>(ns, bins, w) > (size_t)half) --w;
      if (spread_tile3v_bytes<T>(ns, bins, w) > (size_t)half) {
        w = wmax;
        while (w > 1 && spread_tile3v_bytes<T>(ns, bins, w) > (size_t)limit) --w;
      }
      const size_t vsm = spread_tile3v_bytes<T>(ns, bins, w);
      if (vsm > (size_t)limit) {
        variant = 2;
      } else {
        S.cfg.variant = 3;
        S.cfg.fixed = std::is_same_v<T, float> && ext.spread_float_tile != 1 &&
                      (ns <= 6 || ext.spread_float_tile == 2);
        S.cfg.threads = 32 * w;
        S.cfg.smem = vsm;
        S.smem = vsm;
        return S;
      }
    }
    const int mwarps = std::is_same_v<T, float> ? 12 : 8;
    const size_t msm = spread_tile3m_bytes<T>(ns, bins, mwarps);
    if (variant == 2 && msm > (size_t)limit) variant = 0;
    S.cfg.variant = variant;
    if (variant == 2) {
      S.cfg.threads = 32 * mwarps;
      S.cfg.smem = msm;
      S.smem = msm;
    }
    if (variant == 1) {
      S.cfg.threads = 32;
      S.cfg.smem = wsm;
      S.smem = wsm;
    }
  }
  return S;
}
template SpreadSetup spread_setup<float>(int, int, const int[3], const cufinufft_opts &,
                                         const gbnufft_opts &, bool);
template SpreadSetup spread_setup<double>(int, int, const int[3], const cufinufft_opts &,
                                          const gbnufft_opts &, bool);

template <typename T> void Plan<T>::choose_spread_config(bool user_method) {
  // the reference heuristic's automatic method (src/cuda/makeplan.cu:310-314):
  // method 2 for types 1 and 3, method 1 (per-point interpolation) for type 2
  cufinufft_opts o = opts;
  if (ext.planner == 1 && o.gpu_method == 0 && type == 2) o.gpu_method = 1;
  const SpreadSetup S = spread_setup<T>(dim, K.ns, nf, o, ext, user_method);
  for (int d = 0; d < 3; ++d) {
    bins[d] = S.bins[d];
    nbins[d] = S.nbins[d];
  }
  method = S.method;
  spread_smem = S.smem;
  scfg = S.cfg;
  maxsub = S.maxsub;
}

template <typename T> void Plan<T>::make_fft() {
  long long n[3];
  for (int d = 0; d < dim; ++d) n[d] = nf[dim - 1 - d]; // slowest dimension first
  size_t work = 0;
  if (cufftCreate(&fftplan) != CUFFT_SUCCESS) GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "cufftCreate");
  have_fft = true;
  const cufftType ty = std::is_same_v<T, float> ? CUFFT_C2C : CUFFT_Z2Z;
  cufftResult r = cufftMakePlanMany64(fftplan, dim, n, nullptr, 1, nf_total, nullptr, 1,
                                      nf_total, ty, batchsize, &work);
  if (r != CUFFT_SUCCESS) {
    fprintf(stderr, "[gbnufft] cufftMakePlanMany64 failed (%d)\n", (int)r);
    GBN_THROW(r == CUFFT_ALLOC_FAILED ? FINUFFT_ERR_ALLOC : FINUFFT_ERR_CUDA_FAILURE, "cufft");
  }
  cufftSetStream(fftplan, stream);
  if (dim >= 2 && ext.fft_prune == 1) make_pruned_fft();
}

// Pruned FFT: the retained modes use only the x columns [0, keep0) and
// [nf0 - keep1, nf0), so after (type 1) or before (type 2) a full 1D pass
// along x, the passes over y (and z) run on those columns alone.
template <typename T> void Plan<T>::make_pruned_fft() {
  const cufftType ty = std::is_same_v<T, float> ? CUFFT_C2C : CUFFT_Z2Z;
  keep0 = ms[0] - ms[0] / 2;
  keep1 = ms[0] / 2;
  auto check = [](cufftResult r) {
    if (r != CUFFT_SUCCESS)
      GBN_THROW(r == CUFFT_ALLOC_FAILED ? FINUFFT_ERR_ALLOC : FINUFFT_ERR_CUDA_FAILURE, "cufft");
  };
  size_t work = 0;
  long long nx[1] = {nf[0]};
  check(cufftCreate(&fft_x));
  check(cufftMakePlanMany64(fft_x, 1, nx, nx, 1, nf[0], nx, 1, nf[0], ty,
                            (long long)nf[1] * nf[2] * batchsize, &work));
  cufftSetStream(fft_x, stream);
  long long nr[2];
  for (int d = 1; d < dim; ++d) nr[d - 1] = nf[dim - d]; // slowest dimension first
  auto rest = [&](cufftHandle *h, int cols) {
    check(cufftCreate(h));
    check(cufftMakePlanMany64(*h, dim - 1, nr, nr, nf[0], 1, nr, nf[0], 1, ty, cols, &work));
    cufftSetStream(*h, stream);
  };
  rest(&fft_rest0, keep0);
  if (keep1 > 0) rest(&fft_rest1, keep1);
  pruned = true;
}

template <typename T> void Plan<T>::make_fseries() {
  QuadNodes Q;
  Q.q = kernel_ft_nodes(make_kernel_fn(K.form, K.ns, (double)K.beta), 3.0, Q.z, Q.f);
  for (int d = 0; d < dim; ++d) {
    invphihat[d].resize((size_t)nf[d] / 2 + 1);
    launch_inv_fseries<T>(nf[d], Q, invphihat[d].p, stream);
  }
}

// ---------------------------------------------------------- planners 2, 3 ----
template <typename T> bool Plan<T>::candidate_valid(const Candidate &c) const {
  return planner_candidate_valid(c, type, dim, std::is_same_v<T, double>, tol);
}

template <typename T> void Plan<T>::apply_sigma(double sigma) {
  if (sigma == opts.upsampfac) return;
  opts.upsampfac = sigma;
  user_sigma = false; // the planner's choice: fitted pieces for any sigma
  make_kernel();
  if (type != 3) make_grid();
}

template <typename T> void Plan<T>::apply_shape(const Candidate &c) {
  cufinufft_opts o = opts;
  gbnufft_opts e = ext;
  if (c.reference) {
    e.planner = 1;
    o.gpu_binsizex = o.gpu_binsizey = o.gpu_binsizez = 0;
    o.gpu_maxsubprobsize = 1024;
    e.spread_variant = -1;
  } else {
    e.planner = 0;
    o.gpu_binsizex = c.bins[0];
    o.gpu_binsizey = c.bins[1];
    o.gpu_binsizez = c.bins[2];
    o.gpu_maxsubprobsize = c.maxsub;
    e.spread_variant = c.variant;
  }
  // the reference heuristic's slot takes its automatic method too: 1 (per-point
  // interpolation) for type 2, else 2
  o.gpu_method = (c.reference && type == 2) ? 1 : 0;
  const SpreadSetup S = spread_setup<T>(dim, K.ns, nf, o, e, false);
  for (int d = 0; d < 3; ++d) {
    bins[d] = S.bins[d];
    nbins[d] = S.nbins[d];
  }
  method = S.method;
  spread_smem = S.smem;
  scfg = S.cfg;
  maxsub = S.maxsub;
}

namespace {
// autotuner cache: problem class -> chosen slot (process-wide)
std::mutex tune_mu;
std::map<std::vector<int>, int> tune_cache;
} // namespace

template <typename T>
double Plan<T>::time_candidate(const Candidate &c, int64_t Ms, const T *const xs[3]) {
  apply_sigma(c.sigma);
  apply_shape(c);
  AxisMap ax[3];
  for (int d = 0; d < 3; ++d) ax[d] = AxisMap{0.0, 1.0, nf[d], bins[d]};
  sort_points(Ms, xs, ax);
  const PointLayout<T> L = layout();
  // the batch's transforms together, as execute runs them (the FFT plan is the
  // batch's; batched interpolation reuses each point's weights)
  const int nt = std::max(1, batchsize);
  const size_t cbytes = (size_t)std::max<int64_t>(Ms, 1) * nt * sizeof(cplx<T>);
  AsyncBuf cv(cbytes, stream);
  GBN_CUDA(cudaMemsetAsync(cv.p, 0x3c, cbytes, stream)); // any finite nonzero strengths
  cudaEvent_t e0, e1, e2;
  GBN_CUDA(cudaEventCreate(&e0));
  GBN_CUDA(cudaEventCreate(&e1));
  GBN_CUDA(cudaEventCreate(&e2));
  float best = 1e30f, fft_ms = 0;
  for (int rep = 0; rep < 3; ++rep) {
    GBN_CUDA(cudaEventRecord(e0, stream));
    if (type == 1)
      launch_spread<T>(L, K, cv.as<cplx<T>>(), nullptr, 0, fw.p, nf_total, nt, scfg, stream);
    else
      launch_interp<T>(L, K, fw.p, nf_total, nullptr, 0, cv.as<cplx<T>>(), nt, stream);
    GBN_CUDA(cudaEventRecord(e1, stream));
    fft(fw.p, 1, type == 1);
    GBN_CUDA(cudaEventRecord(e2, stream));
    GBN_CUDA(cudaEventSynchronize(e2));
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b, e1, e2);
    if (rep > 0) { // the first run warms up
      best = std::min(best, a);
      fft_ms = b;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  // the sample's spread (or interpolation) scaled to all points, plus the FFT
  return (double)best * ((double)Mtune / (double)std::max<int64_t>(Ms, 1)) + fft_ms;
}

template <typename T>
Candidate Plan<T>::plan_shape(int64_t Mp, const T *const xyz[3], int64_t Np) {
  const bool dbl = std::is_same_v<T, double>;
  double shift[3] = {-PI, -PI, -PI}, scale[3] = {0.5 / PI, 0.5 / PI, 0.5 / PI};
  double xs_product = 0;
  if (type == 3)
    for (int d = 0; d < dim; ++d) {
      const double X = t3X[d] > 0 ? t3X[d] : 1.0;
      shift[d] = t3C[d] - X;
      scale[d] = 0.5 / X;
      xs_product += std::log10(t3X[d] * t3S[d] + 1.0) / dim;
    }
  float feat[PLANNER_NF];
  point_features<T>(dim, type, dbl, Mp, xyz, shift, scale,
                    type == 3 ? (double)Np : (double)nmodes, tol, batchsize,
                    std::pow(10.0, xs_product) - 1.0, feat, stream);
  std::copy(feat, feat + PLANNER_NF, features);
  int best = -1;
  if (ext.planner == 2) {
    double pred[PLANNER_K];
    if (planner_predict(feat, pred, stream)) {
      double best_ms = 1e300;
      for (int k = 0; k < PLANNER_K; ++k) {
        Candidate c;
        if (!planner_candidate(dim, dbl, k, &c) || !candidate_valid(c)) continue;
        if (pred[k] < best_ms) {
          best_ms = pred[k];
          best = k;
        }
      }
      Candidate c0;
      if (best > 0 && planner_candidate(dim, dbl, 0, &c0) && candidate_valid(c0) &&
          pred[0] <= best_ms * PLANNER_KEEP_DEFAULT)
        best = 0;
    }
  } else if (type != 3 && Mp > 0) {
    // autotuner: time every valid candidate on a strided sample of the points,
    // once per problem class
    std::vector<int> key = {type, dim, (int)dbl, (int)std::lround(-4 * std::log10(tol)),
                            (int)std::lround(2 * std::log2((double)nmodes)),
                            (int)std::lround(4 * std::log10((double)Mp)),
                            (int)std::lround(8 * feat[7]), (int)std::lround(10 * feat[8]),
                            batchsize};
    {
      std::lock_guard<std::mutex> g(tune_mu);
      auto it = tune_cache.find(key);
      if (it != tune_cache.end()) best = it->second;
    }
    if (best < 0) {
      const int64_t Ms = std::min<int64_t>(Mp, (int64_t)1 << 21);
      const int64_t stride = Mp / Ms;
      AsyncBuf sb((size_t)Ms * dim * sizeof(T), stream);
      const T *xs[3];
      for (int d = 0; d < dim; ++d) {
        T *dst = sb.as<T>() + (size_t)d * Ms;
        GBN_CUDA(cudaMemcpy2DAsync(dst, sizeof(T), xyz[d], stride * sizeof(T), sizeof(T),
                                   (size_t)Ms, cudaMemcpyDeviceToDevice, stream));
        xs[d] = dst;
      }
      for (int d = dim; d < 3; ++d) xs[d] = xs[0];
      Mtune = Mp;
      double best_ms = 1e300;
      for (int k = 0; k < PLANNER_K; ++k) {
        Candidate c;
        if (!planner_candidate(dim, dbl, k, &c) || !candidate_valid(c)) continue;
        const double ms_k = time_candidate(c, Ms, xs);
        tune_ms[k] = ms_k;
        if (ms_k < best_ms) {
          best_ms = ms_k;
          best = k;
        }
      }
      if (best >= 0) {
        std::lock_guard<std::mutex> g(tune_mu);
        tune_cache[key] = best;
      }
    }
  }
  Candidate c;
  if (best >= 0 && planner_candidate(dim, dbl, best, &c)) {
    planned_slot = best;
    planner_used = ext.planner;
    return c;
  }
  // fallback: the reference heuristic's shape at the current sigma
  planned_slot = -1;
  planner_used = 1;
  c = Candidate{opts.upsampfac, {0, 0, 0}, 1024, -1, 1};
  return c;
}

template <typename T> PointLayout<T> Plan<T>::layout() const {
  PointLayout<T> L;
  L.dim = dim;
  for (int d = 0; d < 3; ++d) {
    L.nf[d] = nf[d];
    L.bin[d] = bins[d];
    L.nbin[d] = nbins[d];
    L.loc[d] = loc[d].p ? loc[d].p : loc[0].p;
  }
  L.M = M;
  L.nsub = nsub;
  L.sub_bin = sub_bin_.p;
  L.sub_start = sub_start_.p;
  L.sub_count = sub_count_.p;
  L.perm = perm.p;
  L.cell_sorted = cell_sorted;
  L.sorted_out = isort.p;
  L.iperm = isort.p ? iperm.p : nullptr;
  // method 1 (asked for, or the reference heuristic's choice for type 2)
  // interpolates one point per thread from the grid, as the reference's
  // method 1 does; method 2 uses the tiled schedules
  L.interp_mode = (method == 1 && ext.interp_mode == 0) ? 1 : ext.interp_mode;
  return L;
}

template <typename T>
void Plan<T>::sort_points(int64_t Mp, const T *const xyz[3], const AxisMap ax[3]) {
  M = (int)Mp;
  perm.resize(std::max<int64_t>(Mp, 1));
  for (int d = 0; d < dim; ++d) loc[d].resize(std::max<int64_t>(Mp, 1));
  const int nb = nbins[0] * nbins[1] * nbins[2];
  // keys carry the cell inside the bin when bins * bin volume fits 32 bits;
  // for odd kernel widths the start cell of the support instead (the cell, or
  // the next one when the fraction is at least one half: bin + 1 values per
  // dimension), so points sharing their first support cell are adjacent
  const uint64_t binvol0 = (uint64_t)bins[0] * bins[1] * bins[2];
  uint64_t sbinvol = 1;
  for (int d = 0; d < dim; ++d) sbinvol *= (uint64_t)bins[d] + 1;
  int cell_keys = (uint64_t)nb * binvol0 <= 0xffffffffull ? 1 : 0;
  // gbnufft_opts.sort_keys = 2: bin keys only, the reference's ordering (bin
  // index x fastest, include/cufinufft/spreadinterp.hpp:139-150; points of a
  // bin in input order, as the CPU library's stable counting sort,
  // include/finufft/spread.hpp:459-584)
  if (ext.sort_keys == 2) cell_keys = 0;
  // gbnufft_opts.sort_keys = 1 keeps whole-cell keys for odd widths too
  if (cell_keys && K.ns % 2 == 1 && (uint64_t)nb * sbinvol <= 0xffffffffull &&
      ext.sort_keys != 1)
    cell_keys = 2;
  const uint64_t binvol = cell_keys == 2 ? sbinvol : binvol0;
  cell_sorted = cell_keys ? 1 : 0;
  const uint64_t nkeys = cell_keys ? (uint64_t)nb * binvol : (uint64_t)nb;
  int keybits = 0;
  while ((1ull << keybits) < nkeys) ++keybits;
  AsyncBuf keys((size_t)std::max<int64_t>(Mp, 1) * 4, stream);
  AsyncBuf skeys((size_t)std::max<int64_t>(Mp, 1) * 4, stream);
  if (M > 0) {
    // one fold per point: the key pass also writes the bin-local coordinates,
    // which are gathered into sorted order after the sort
    AsyncBuf rec((size_t)Mp * 4 * sizeof(T), stream);
    launch_bin_keys<T>(dim, xyz, M, ax, nbins, cell_keys, keys.as<uint32_t>(), stream,
                       rec.as<T>());
    stable_sort_by_bin(keys.as<uint32_t>(), M, keybits, skeys.as<uint32_t>(), perm.p, stream);
    T *const lp[3] = {loc[0].p, dim > 1 ? loc[1].p : loc[0].p, dim > 2 ? loc[2].p : loc[0].p};
    launch_gather_local<T>(dim, rec.as<T>(), perm.p, M, lp, stream);
  }
  // the subproblem arrays are reused while they hold enough entries
  SubproblemArrays sa;
  sa.bin = sub_bin_.p;
  sa.start = sub_start_.p;
  sa.count = sub_count_.p;
  sa.cap = sub_bin_.n;
  nsub = build_subproblems(skeys.as<uint32_t>(), M, nb, cell_keys ? (uint32_t)binvol : 1u,
                           maxsub, &sa, stream);
  sub_bin_.p = sa.bin;
  sub_start_.p = sa.start;
  sub_count_.p = sa.count;
  sub_bin_.n = sub_start_.n = sub_count_.n = sa.cap;
  // 2D type-2 batches whose per-transform output fits in L2: interpolate into
  // sorted order, then gather transform by transform into user order through
  // the inverse permutation (coalesced writes; the random reads of one
  // transform's sorted results hit L2). 16 vectors of 1e7 2D points, batches
  // of 16: 3.70 ms per execute, against 5.09 ms scattering through perm and
  // 6.84 ms writing user order from the interpolation. Not for one transform
  // (1e7 2D points: 0.437 ms per execute through the sorted copy, 0.389 ms
  // writing user order directly: no weights are shared across transforms to
  // pay for the extra pass). Not in 3D, where the
  // interpolation's own scattered writes cost less than the extra pass in
  // the scatter form (1.25e7 clustered points, 4 vectors at 128^3: 4.98 ms
  // direct, 5.85 ms through the sorted copy). The sorted copy of a batch's
  // outputs is only taken when it costs at most an eighth of the device
  // memory free at setpts. gbnufft_opts.interp_mode 1 or 2 writes user order
  // directly.
  isort.release();
  iperm.release();
  if (type == 2 && batchsize > 1 && batchsize <= 65535 && dim == 2 && M > 0 &&
      ext.interp_mode == 0 && method != 1) { // (the gather's grid has one row per transform)
    int dev = 0, l2 = 0;
    GBN_CUDA(cudaGetDevice(&dev));
    GBN_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
    size_t freeb = 0, totb = 0;
    GBN_CUDA(cudaMemGetInfo(&freeb, &totb));
    const double bytes = (double)batchsize * M * sizeof(cplx<T>) + (double)M * sizeof(int);
    if ((double)M * sizeof(cplx<T>) <= 0.75 * (double)l2 && bytes <= 0.125 * (double)freeb) {
      isort.resize((size_t)batchsize * M);
      iperm.resize((size_t)M);
      launch_invert_perm(perm.p, (int)M, iperm.p, stream);
    }
  }
}

template <typename T>
void Plan<T>::setpts(int64_t Mp, const T *x, const T *y, const T *z, int64_t Np, const T *s,
                     const T *t, const T *u) {
  DeviceScope ds(opts.gpu_device_id);
  if (Mp < 0 || Mp > std::numeric_limits<int32_t>::max())
    GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "M");
  const T *xyz[3] = {x, dim > 1 ? y : x, dim > 2 ? z : x};
  if (Mp > 0 && (!x || (dim > 1 && !y) || (dim > 2 && !z)))
    GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null coordinate array");
  if (type != 3) {
    if ((ext.planner == 2 || ext.planner == 3) && (dim == 2 || dim == 3) &&
        !opts.gpu_spreadinterponly) {
      const Candidate c = plan_shape(Mp, xyz, 0);
      apply_sigma(c.sigma);
      apply_shape(c);
    }
    AxisMap ax[3];
    for (int d = 0; d < 3; ++d) ax[d] = AxisMap{0.0, 1.0, nf[d], bins[d]};
    sort_points(Mp, xyz, ax);
    pts_set = true;
    return;
  }
  // ---- type 3: choose the grid from the extents of sources and targets
  if (Np < 0 || Np > std::numeric_limits<int32_t>::max()) {
    fprintf(stderr, "[gbnufft] invalid number of targets N=%lld\n", (long long)Np);
    GBN_THROW(FINUFFT_ERR_NUM_NU_PTS_INVALID, "N");
  }
  if (!s || (dim > 1 && !t) || (dim > 2 && !u)) {
    fprintf(stderr, "[gbnufft] type 3 needs target arrays for every dimension\n");
    GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null target array");
  }
  N = (int)Np;
  const T *stu[3] = {s, dim > 1 ? t : s, dim > 2 ? u : s};
  for (int d = 0; d < 3; ++d) {
    t3X[d] = t3C[d] = t3S[d] = t3D[d] = 0.0;
    if (d >= dim) continue;
    double lo, hi;
    if (Mp > 0) {
      array_range<T>(xyz[d], (int)Mp, &lo, &hi, stream);
      width_center(lo, hi, &t3X[d], &t3C[d]);
    }
    if (Np > 0) {
      array_range<T>(stu[d], (int)Np, &lo, &hi, stream);
      width_center(lo, hi, &t3S[d], &t3D[d]);
    }
  }
  // planners 2/3: the upsampling factor and the outer spread's shape
  Candidate t3c{};
  const bool t3planned = (ext.planner == 2 || ext.planner == 3) && (dim == 2 || dim == 3);
  if (t3planned) {
    t3c = plan_shape(Mp, xyz, Np);
    apply_sigma(t3c.sigma);
  }
  int64_t nft[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) {
    type3_grid(opts.upsampfac, t3X[d], t3S[d], K.ns, &nft[d], &t3h[d], &t3gam[d]);
    if (nft[d] > std::numeric_limits<int32_t>::max()) GBN_THROW(FINUFFT_ERR_MAXNALLOC, "nf");
    nf[d] = (int)nft[d];
  }
  nf_total = (int64_t)nf[0] * nf[1] * nf[2];
  if (nf_total * batchsize > std::numeric_limits<int32_t>::max()) {
    fprintf(stderr, "[gbnufft] type-3 fine grid batch would exceed %d cells\n",
            std::numeric_limits<int32_t>::max());
    GBN_THROW(FINUFFT_ERR_MAXNALLOC, "nf*batch");
  }
  if (opts.debug)
    for (int d = 0; d < dim; ++d)
      printf("[gbnufft] t3 dim %d: X=%.3g C=%.3g S=%.3g D=%.3g gam=%.4g nf=%d h=%.3g\n", d,
             t3X[d], t3C[d], t3S[d], t3D[d], t3gam[d], nf[d], t3h[d]);
  choose_spread_config(opts.gpu_method != 0);
  if (t3planned) apply_shape(t3c);
  // pre-phase exp(i isign D.x) (skipped when D = 0) and the post factor
  const bool needpre = t3D[0] != 0.0 || t3D[1] != 0.0 || t3D[2] != 0.0;
  if (needpre && Mp > 0) {
    t3pre.resize((size_t)Mp);
    launch_t3_prephase<T>(dim, xyz, (int)Mp, t3D, iflag, t3pre.p, stream);
  } else
    t3pre.release();
  double scale[3];
  for (int d = 0; d < 3; ++d) scale[d] = t3h[d] * t3gam[d];
  QuadNodes Q;
  Q.q = kernel_ft_nodes(make_kernel_fn(K.form, K.ns, (double)K.beta), 2.0, Q.z, Q.f);
  double Cphase[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d)
    if (std::isfinite(t3C[d])) Cphase[d] = t3C[d];
  t3post.resize((size_t)std::max<int64_t>(Np, 1));
  launch_t3_postfactor<T>(dim, stu, (int)Np, Cphase, t3D, scale, iflag, Q, t3post.p, stream);
  // sort the rescaled sources x' = (x - C)/gamma on the outer grid
  AxisMap ax[3];
  for (int d = 0; d < 3; ++d)
    ax[d] = AxisMap{d < dim ? t3C[d] : 0.0, d < dim ? 1.0 / t3gam[d] : 1.0, nf[d], bins[d]};
  sort_points(Mp, xyz, ax);
  fw.resize((size_t)nf_total * batchsize);
  // inner type 2 on the outer grid, evaluated at s' = h gamma (s - D)
  cufinufft_opts io = opts;
  io.gpu_spreadinterponly = 0;
  io.gpu_method = 0;
  io.modeord = 0;
  io.gpu_maxbatchsize = batchsize;
  io.gpu_binsizex = io.gpu_binsizey = io.gpu_binsizez = 0;
  int64_t inner_modes[3] = {nf[0], nf[1], nf[2]};
  inner.reset();
  gbnufft_opts iext = ext;
  if (iext.planner >= 2) iext.planner = 0; // the inner type 2 takes the engine's shape
  inner.reset(new Plan<T>(2, dim, inner_modes, iflag, batchsize, tol, io, &iext));
  AxisMap iax[3];
  for (int d = 0; d < 3; ++d)
    iax[d] = AxisMap{d < dim ? t3D[d] : 0.0, d < dim ? scale[d] : 1.0, inner->nf[d],
                     inner->bins[d]};
  inner->sort_points(Np, stu, iax);
  inner->pts_set = true;
  pts_set = true;
}

template <typename T> void Plan<T>::check_ready() const {
  if (!pts_set) {
    fprintf(stderr, "[gbnufft] execute called before setpts\n");
    GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "setpts first");
  }
}

template <typename T> void Plan<T>::fft(cplx<T> *data, int sign, bool spread_first) {
  const int dir = sign > 0 ? CUFFT_INVERSE : CUFFT_FORWARD;
  auto exec = [&](cufftHandle h, cplx<T> *d) {
    cufftResult r;
    if constexpr (std::is_same_v<T, float>)
      r = cufftExecC2C(h, (cufftComplex *)d, (cufftComplex *)d, dir);
    else
      r = cufftExecZ2Z(h, (cufftDoubleComplex *)d, (cufftDoubleComplex *)d, dir);
    if (r != CUFFT_SUCCESS) GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "cufftExec");
  };
  if (!pruned) {
    exec(fftplan, data);
    return;
  }
  auto rest = [&]() {
    for (int b = 0; b < batchsize; ++b) {
      cplx<T> *g = data + (int64_t)b * nf_total;
      exec(fft_rest0, g);
      if (keep1 > 0) exec(fft_rest1, g + (nf[0] - keep1));
    }
  };
  if (spread_first) {
    exec(fft_x, data);
    rest();
  } else {
    rest();
    exec(fft_x, data);
  }
}

// Type-1 pipeline on ntr transforms: spread -> FFT(sign) -> deconvolve.
template <typename T>
void Plan<T>::run_type1(const cplx<T> *c, cplx<T> *fk, int ntr, int sign, const cplx<T> *pre,
                        int conj_pre) {
  const PointLayout<T> L = layout();
  const T *inv[3] = {invphihat[0].p, dim > 1 ? invphihat[1].p : invphihat[0].p,
                     dim > 2 ? invphihat[2].p : invphihat[0].p};
  for (int i = 0; i * batchsize < ntr; ++i) {
    const int blk = std::min(ntr - i * batchsize, batchsize);
    const cplx<T> *cb = c + (int64_t)i * batchsize * M;
    cplx<T> *fkb = fk + (int64_t)i * batchsize * nmodes;
    cplx<T> *grid = opts.gpu_spreadinterponly ? fkb : fw.p;
    if (time_stages) GBN_CUDA(cudaEventRecord(ev[0], stream));
    GBN_CUDA(cudaMemsetAsync(grid, 0, (size_t)blk * nf_total * sizeof(cplx<T>), stream));
    launch_spread<T>(L, K, cb, pre, conj_pre, grid, nf_total, blk, scfg, stream);
    if (time_stages) GBN_CUDA(cudaEventRecord(ev[1], stream));
    if (!opts.gpu_spreadinterponly) {
      fft(fw.p, sign, true);
      if (time_stages) GBN_CUDA(cudaEventRecord(ev[2], stream));
      launch_deconv<T>(dim, ms, nf, opts.modeord, inv, fw.p, nf_total, fkb, blk, stream);
    } else if (time_stages) {
      GBN_CUDA(cudaEventRecord(ev[2], stream));
    }
    if (time_stages) {
      GBN_CUDA(cudaEventRecord(ev[3], stream));
      stage_tick();
    }
  }
}

// Stage timing (a diagnostic mode, outside graph capture): waits for the
// batch's last event and adds its stage intervals to the execute's sums, so
// that plans running their transforms in several batches report every batch.
template <typename T> void Plan<T>::stage_tick() {
  GBN_CUDA(cudaEventSynchronize(ev[3]));
  float t[4] = {0, 0, 0, 0};
  cudaEventElapsedTime(&t[0], ev[0], ev[1]);
  cudaEventElapsedTime(&t[1], ev[1], ev[2]);
  cudaEventElapsedTime(&t[2], ev[2], ev[3]);
  cudaEventElapsedTime(&t[3], ev[0], ev[3]);
  for (int k = 0; k < 4; ++k) stage_acc[k] += t[k];
}

// Type-2 pipeline on ntr transforms: amplify -> FFT(sign) -> interpolate.
template <typename T>
void Plan<T>::run_type2(const cplx<T> *fk, cplx<T> *c, int ntr, int sign,
                        const cplx<T> *post, int conj_post) {
  const PointLayout<T> L = layout();
  const T *inv[3] = {invphihat[0].p, dim > 1 ? invphihat[1].p : invphihat[0].p,
                     dim > 2 ? invphihat[2].p : invphihat[0].p};
  for (int i = 0; i * batchsize < ntr; ++i) {
    const int blk = std::min(ntr - i * batchsize, batchsize);
    const cplx<T> *fkb = fk + (int64_t)i * batchsize * nmodes;
    cplx<T> *cb = c + (int64_t)i * batchsize * M;
    const cplx<T> *grid = fkb;
    if (time_stages) GBN_CUDA(cudaEventRecord(ev[0], stream));
    if (!opts.gpu_spreadinterponly) {
      launch_amplify<T>(dim, ms, nf, opts.modeord, inv, fkb, fw.p, nf_total, blk, stream);
      if (time_stages) GBN_CUDA(cudaEventRecord(ev[1], stream));
      fft(fw.p, sign, false);
      grid = fw.p;
    } else if (time_stages)
      GBN_CUDA(cudaEventRecord(ev[1], stream));
    if (time_stages) GBN_CUDA(cudaEventRecord(ev[2], stream));
    launch_interp<T>(L, K, grid, nf_total, post, conj_post, cb, blk, stream);
    if (time_stages) {
      GBN_CUDA(cudaEventRecord(ev[3], stream));
      stage_tick();
    }
  }
}

template <typename T> void Plan<T>::execute(cplx<T> *c, cplx<T> *fk) {
  execute_range(c, fk, 0, ntransf, false);
}

// Adjoint of the planned transform (reference CPU semantics,
// include/finufft/execute.hpp:318-357): type 1 -> type 2 with the opposite
// sign (fk in, c out), type 2 -> type 1 with the opposite sign (c in, fk out),
// type 3 -> the planned factors applied backwards and conjugated.
template <typename T> void Plan<T>::execute_adjoint(cplx<T> *c, cplx<T> *fk) {
  execute_range(c, fk, 0, ntransf, true);
}

// Transforms [t0, t0 + nt) of the planned ntransf; c and fk point at the full
// arrays (transform t at c + t*M, fk + t*(modes or targets)).
template <typename T>
void Plan<T>::execute_range(cplx<T> *c, cplx<T> *fk, int t0, int nt, bool adjoint) {
  DeviceScope ds(opts.gpu_device_id);
  check_ready();
  if (t0 < 0 || nt < 0 || t0 + nt > ntransf)
    GBN_THROW(FINUFFT_ERR_NTRANS_NOTVALID, "transform range");
  if (nt == 0) return;
  c += (int64_t)t0 * M;
  fk += (int64_t)t0 * (type == 3 ? (int64_t)N : nmodes);
  const bool timed = time_stages && !adjoint;
  const bool tmp_ts = time_stages;
  time_stages = timed;
  if (timed) {
    for (auto &e : ev)
      if (!e) GBN_CUDA(cudaEventCreate(&e));
    for (float &a : stage_acc) a = 0.f;
  }
  if (!adjoint) {
    if (type == 1) run_type1(c, fk, nt, iflag, nullptr, 0);
    else if (type == 2) run_type2(fk, c, nt, iflag, nullptr, 0);
  } else {
    if (type == 1) run_type2(fk, c, nt, -iflag, nullptr, 0);
    else if (type == 2) run_type1(c, fk, nt, -iflag, nullptr, 0);
  }
  if (type == 3) {
    const PointLayout<T> L = layout();
    if (timed) GBN_CUDA(cudaEventRecord(ev[0], stream));
    for (int i = 0; i * batchsize < nt; ++i) {
      const int blk = std::min(nt - i * batchsize, batchsize);
      cplx<T> *cb = c + (int64_t)i * batchsize * M;
      cplx<T> *fb = fk + (int64_t)i * batchsize * N;
      if (!adjoint) {
        // pre-phase+spread onto the outer grid, inner type 2, post factor
        GBN_CUDA(cudaMemsetAsync(fw.p, 0, (size_t)blk * nf_total * sizeof(cplx<T>), stream));
        launch_spread<T>(L, K, cb, t3pre.p ? t3pre.p : nullptr, 0, fw.p, nf_total, blk, scfg,
                         stream);
        inner->run_type2(fw.p, fb, blk, iflag, t3post.p, 0);
      } else {
        // adjoint of (post * inner type 2): inner type 1 with conj(post) pre-factor,
        // then the adjoint of (spread * pre): interpolate, times conj(pre)
        inner->run_type1(fb, fw.p, blk, -iflag, t3post.p, 1);
        launch_interp<T>(L, K, fw.p, nf_total, t3pre.p ? t3pre.p : nullptr, 1, cb, blk,
                         stream);
      }
    }
    if (timed) { // stage timing of type 3: total only
      for (int k = 3; k >= 1; --k) GBN_CUDA(cudaEventRecord(ev[k], stream));
      stage_tick();
    }
  }
  time_stages = tmp_ts;
  GBN_LAUNCH_CHECK();
  if (timed) {
    // per batch, events: ev0 | spread or amplify | ev1 | FFT | ev2 | deconvolve
    // or interp | ev3, summed over the batches by stage_tick
    const float a = stage_acc[0], b = stage_acc[2];
    times.fft_ms = stage_acc[1];
    times.total_ms = stage_acc[3];
    times.spread_or_interp_ms = type == 2 ? b : a;
    times.deconv_ms = type == 2 ? a : b;
    if (type == 3) times.spread_or_interp_ms = times.fft_ms = times.deconv_ms = 0;
  }
}

template class Plan<float>;
template class Plan<double>;

} // namespace gbn
