// The NUFFT plan: owns every device buffer of one transform set and runs the
// makeplan -> setpts -> execute pipeline on one CUDA stream.
#pragma once
#include <cufft.h>

#include <memory>
#include <vector>

#include "common.h"
#include "cufinufft_opts.h"
#include "gbnufft_ext.h"
#include "device_util.cuh"
#include "elementwise.h"
#include "planner.h"
#include "spreadinterp.h"

namespace gbn {

// Owning device buffer (cudaMalloc).
template <typename U> struct DevArray {
  U *p = nullptr;
  size_t n = 0;
  DevArray() = default;
  DevArray(const DevArray &) = delete;
  DevArray &operator=(const DevArray &) = delete;
  ~DevArray() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void resize(size_t count) {
    if (count == n && p) return;
    release();
    if (count) GBN_CUDA(cudaMalloc((void **)&p, count * sizeof(U)));
    n = count;
  }
};

// Makes opts.gpu_device_id current for a scope and restores the caller's device.
struct DeviceScope {
  int prev = 0;
  bool switched = false;
  explicit DeviceScope(int dev);
  ~DeviceScope();
};

// Per-stage device timings of the last execute (milliseconds).
struct StageTimes {
  float spread_or_interp_ms = 0, fft_ms = 0, deconv_ms = 0, total_ms = 0;
};

// Bins, method and launch configuration of the spreader for a grid.
struct SpreadSetup {
  int bins[3] = {1, 1, 1};
  int nbins[3] = {1, 1, 1};
  int method = 2;
  size_t smem = 0;
  SpreadConfig cfg{2, 256, 0};
  int maxsub = 1024; // points per subproblem at most
};
// Kernel form of a plan (KERNEL_ES or KERNEL_PSWF) from the options.
int plan_kernel_form(const gbnufft_opts &ext, const cufinufft_opts &opts);

template <typename T>
SpreadSetup spread_setup(int dim, int ns, const int nf[3], const cufinufft_opts &opts,
                         const gbnufft_opts &ext, bool user_method);

template <typename T> class Plan {
public:
  Plan(int type, int dim, const int64_t *nmodes, int iflag, int ntransf, double tol,
       const cufinufft_opts &opts, const gbnufft_opts *ext = nullptr);
  ~Plan();
  void setpts(int64_t M, const T *x, const T *y, const T *z, int64_t N, const T *s,
              const T *t, const T *u);
  void execute(cplx<T> *c, cplx<T> *fk);
  void execute_adjoint(cplx<T> *c, cplx<T> *fk);
  // transforms [t0, t0 + nt) only (c, fk: the full arrays)
  void execute_range(cplx<T> *c, cplx<T> *fk, int t0, int nt, bool adjoint);

  // introspection (tests, planner, benchmarks)
  int type, dim, ntransf, iflag, batchsize;
  double tol;
  cufinufft_opts opts;
  gbnufft_opts ext;
  int ms[3] = {1, 1, 1};
  int nf[3] = {1, 1, 1};
  int64_t nf_total = 1, nmodes = 1;
  int M = 0, N = 0;
  KernelShape<T> K;
  double horner_err = 0;
  int method = 2;
  int bins[3] = {1, 1, 1};
  int nbins[3] = {1, 1, 1};
  int nsub = 0;
  int cell_sorted = 0; // points sorted by (bin, cell in bin)
  int maxsub = 1024;   // points per subproblem at most
  size_t spread_smem = 0;
  cudaStream_t stream = nullptr;
  StageTimes times;
  bool time_stages = false;
  float stage_acc[4] = {0, 0, 0, 0}; // stage sums over an execute's batches
  // sorted point layout (device)
  DevArray<int> perm;
  DevArray<T> loc[3];
  DevArray<int> sub_bin_, sub_start_, sub_count_;
  PointLayout<T> layout() const;
  int spread_variant_in_use() const { return scfg.variant; }
  int spread_fixed_in_use() const { return scfg.variant == 3 ? scfg.fixed : 0; }

  // type 3 parameters (per dimension)
  double t3X[3] = {0, 0, 0}, t3C[3] = {0, 0, 0}, t3S[3] = {0, 0, 0}, t3D[3] = {0, 0, 0};
  double t3h[3] = {1, 1, 1}, t3gam[3] = {1, 1, 1};
  std::unique_ptr<Plan<T>> inner; // type 3: the type-2 plan on the outer grid

  int form = KERNEL_PSWF; // kernel form (KERNEL_ES / KERNEL_PSWF)
  bool user_sigma = false; // the upsampling factor was given by the caller
  int planned_slot = -1;  // planners 2/3: the candidate slot chosen at setpts
  int planner_used = 0;   // planner whose choice is in use (2/3 fall back to 1)
  float features[PLANNER_NF] = {}; // planners 2/3: the features of the last setpts
  double tune_ms[PLANNER_K] = {};  // planner 3: estimated execute ms per slot (0: not timed)
  int64_t Mtune = 0;               // points the autotuner's estimates are scaled to

private:
  void choose_spread_config(bool user_method);
  void make_kernel();
  void make_grid();
  void destroy_fft();
  // planners 2 (learned) and 3 (autotuned) at setpts: pick a candidate shape;
  // returns it (the reference heuristic's shape when the planner falls back)
  Candidate plan_shape(int64_t M, const T *const xyz[3], int64_t N);
  bool candidate_valid(const Candidate &c) const;
  void apply_sigma(double sigma);      // kernel (and types 1/2: grid) at sigma
  void apply_shape(const Candidate &c); // bins, subproblem size, variant
  double time_candidate(const Candidate &c, int64_t Ms, const T *const xs[3]);
  void make_fft();
  void make_pruned_fft();
  void make_fseries();
  void sort_points(int64_t M, const T *const xyz[3], const AxisMap ax[3]);
  void stage_tick();
  void run_type1(const cplx<T> *c, cplx<T> *fk, int ntr, int sign, const cplx<T> *pre,
                 int conj_pre);
  void run_type2(const cplx<T> *fk, cplx<T> *c, int ntr, int sign, const cplx<T> *post,
                 int conj_post);
  // FFT of the batch in place; spread_first: the type-1 order (the grid came
  // from a spread, only the retained modes are read afterwards), else the
  // type-2 order (only the retained modes are nonzero before it)
  void fft(cplx<T> *data, int sign, bool spread_first);
  void check_ready() const;

  cufftHandle fftplan = 0;
  bool have_fft = false;
  // pruned FFT (2D/3D): a batched 1D pass along x over all lines, and passes
  // over the other dimensions on the x columns of the retained modes only
  // (the two ranges [0, keep0) and [nf0 - keep1, nf0))
  bool pruned = false;
  cufftHandle fft_x = 0, fft_rest0 = 0, fft_rest1 = 0;
  int keep0 = 0, keep1 = 0;
  DevArray<cplx<T>> fw;        // batchsize fine grids
  DevArray<T> invphihat[3];    // 1/phihat per dimension, nf/2+1 each
  DevArray<cplx<T>> t3pre;     // type 3 pre-phase, M
  DevArray<cplx<T>> t3post;    // type 3 post factor, N
  DevArray<cplx<T>> isort;     // type 2: sorted-order interpolation output, batchsize * M
  DevArray<int> iperm;         // with isort: iperm[perm[p]] = p, M
  bool pts_set = false;
  SpreadConfig scfg{2, 256, 0};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

} // namespace gbn
