// C-ABI entry points: cufinufft_* (device pointers), finufft_* (host pointers)
// and the gbnufft extensions. Every entry point maps C++ exceptions to the
// FINUFFT integer error codes, as src/cuda/c_interface.cpp and
// include/finufft_common/safe_call.h:57-80 do upstream.
#include <complex>
#include <cstring>
#include <limits>
#include <memory>
#include <new>

#include "cufinufft.h"
#include "finufft.h"
#include "gbnufft_ext.h"
#include "plan.h"
#include "planning.h"
#include "sort.h"

using gbn::Plan;

namespace {

template <class F> int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (const gbn::Error &e) {
    return e.code;
  } catch (const std::bad_alloc &) {
    return FINUFFT_ERR_ALLOC;
  } catch (...) {
    return FINUFFT_ERR_UNKNOWN_EXCEPTION;
  }
}

// src/cuda/c_interface.cpp:14-31: modes must be in [1, INT32_MAX] with an int32 product;
// type 3 ignores them.
bool invalid_modes(int type, int dim, const int64_t *m) {
  if (type == 3) return false;
  if (!m) return true;
  int64_t tot = 1;
  for (int d = 0; d < dim; ++d) {
    if (m[d] <= 0 || m[d] > std::numeric_limits<int32_t>::max()) return true;
    tot *= m[d];
    if (tot > std::numeric_limits<int32_t>::max()) return true;
  }
  return false;
}

template <typename T> struct GraphState {
  cudaGraphExec_t exec = nullptr;
  ~GraphState() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// what a cufinufft plan handle points to
template <typename T> struct DevHandle {
  std::unique_ptr<Plan<T>> plan;
  GraphState<T> graph;
};

template <typename T>
int makeplan_dev(int type, int dim, const int64_t *nmodes, int iflag, int ntr, double tol,
                 void **out, const cufinufft_opts *opts, const gbnufft_opts *ext = nullptr) {
  return guarded([&] {
    if (!out) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null plan pointer");
    if (dim < 1 || dim > 3) {
      fprintf(stderr, "[gbnufft] invalid dim (%d), should be 1, 2 or 3\n", dim);
      GBN_THROW(FINUFFT_ERR_DIM_NOTVALID, "dim");
    }
    if (invalid_modes(type, dim, nmodes)) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "modes");
    cufinufft_opts o;
    if (opts) o = *opts;
    else cufinufft_default_opts(&o);
    auto h = std::make_unique<DevHandle<T>>();
    int64_t m3[3] = {1, 1, 1};
    if (type != 3)
      for (int d = 0; d < dim; ++d) m3[d] = nmodes[d];
    h->plan.reset(new Plan<T>(type, dim, m3, iflag, ntr, tol, o, ext));
    *out = h.release();
  });
}

template <typename T> DevHandle<T> *dev(void *p) {
  if (!p) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "null plan");
  return static_cast<DevHandle<T> *>(p);
}

template <typename T>
int setpts_dev(void *p, int64_t M, const T *x, const T *y, const T *z, int N, const T *s,
               const T *t, const T *u) {
  return guarded([&] {
    if (M < 0 || M > std::numeric_limits<int32_t>::max())
      GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "M");
    auto *h = dev<T>(p);
    if (h->graph.exec) {
      cudaGraphExecDestroy(h->graph.exec);
      h->graph.exec = nullptr;
    }
    h->plan->setpts(M, x, y, z, N, s, t, u);
  });
}

template <typename T> int execute_dev(void *p, void *c, void *fk, bool adjoint) {
  return guarded([&] {
    auto *h = dev<T>(p);
    if (adjoint) h->plan->execute_adjoint((gbn::cplx<T> *)c, (gbn::cplx<T> *)fk);
    else h->plan->execute((gbn::cplx<T> *)c, (gbn::cplx<T> *)fk);
  });
}

template <typename T> int destroy_dev(void *p) {
  return guarded([&] {
    if (!p) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "null plan");
    delete static_cast<DevHandle<T> *>(p);
  });
}

template <typename T> int info_dev(void *p, gbnufft_plan_info *info) {
  return guarded([&] {
    if (!info) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "info");
    const Plan<T> &P = *dev<T>(p)->plan;
    std::memset(info, 0, sizeof(*info));
    info->type = P.type;
    info->dim = P.dim;
    info->ntransf = P.ntransf;
    info->batchsize = P.batchsize;
    info->ns = P.K.ns;
    info->beta = (double)P.K.beta;
    info->upsampfac = P.opts.upsampfac;
    for (int d = 0; d < 3; ++d) {
      info->nf[d] = P.nf[d];
      info->bins[d] = P.bins[d];
      info->inner_nf[d] = P.inner ? P.inner->nf[d] : 0;
    }
    info->method = P.method;
    info->nsub = P.nsub;
    info->M = P.M;
    info->N = P.N;
    info->spread_smem = P.spread_smem;
    info->horner_err = P.horner_err;
    info->spread_variant = P.spread_variant_in_use();
    info->maxsubprobsize = P.maxsub;
    info->spread_fixed = P.spread_fixed_in_use();
    info->kernel_form = P.K.form;
    info->planner_used = P.planner_used;
    info->planned_slot = P.planned_slot;
    for (int f = 0; f < gbn::PLANNER_NF; ++f) info->features[f] = P.features[f];
    for (int k = 0; k < gbn::PLANNER_K; ++k) info->tune_ms[k] = P.tune_ms[k];
  });
}

template <typename T> int times_dev(void *p, int enable, float *ms) {
  return guarded([&] {
    Plan<T> &P = *dev<T>(p)->plan;
    P.time_stages = enable != 0;
    if (ms) {
      ms[0] = P.times.spread_or_interp_ms;
      ms[1] = P.times.fft_ms;
      ms[2] = P.times.deconv_ms;
      ms[3] = P.times.total_ms;
    }
  });
}

template <typename T> int get_sort_dev(void *p, int *perm, T *loc) {
  return guarded([&] {
    Plan<T> &P = *dev<T>(p)->plan;
    gbn::DeviceScope ds(P.opts.gpu_device_id);
    GBN_CUDA(cudaStreamSynchronize(P.stream));
    if (perm && P.M > 0)
      GBN_CUDA(cudaMemcpy(perm, P.perm.p, (size_t)P.M * sizeof(int), cudaMemcpyDeviceToHost));
    if (loc && P.M > 0)
      for (int d = 0; d < P.dim; ++d)
        GBN_CUDA(cudaMemcpy(loc + (size_t)d * P.M, P.loc[d].p, (size_t)P.M * sizeof(T),
                            cudaMemcpyDeviceToHost));
  });
}

template <typename T> int graph_capture_dev(void *p, void *c, void *fk) {
  return guarded([&] {
    auto *h = dev<T>(p);
    Plan<T> &P = *h->plan;
    if (!P.stream) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "graph capture needs gpu_stream");
    gbn::DeviceScope ds(P.opts.gpu_device_id);
    if (h->graph.exec) {
      cudaGraphExecDestroy(h->graph.exec);
      h->graph.exec = nullptr;
    }
    const bool ts = P.time_stages;
    P.time_stages = false;
    cudaGraph_t g = nullptr;
    GBN_CUDA(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
    try {
      P.execute((gbn::cplx<T> *)c, (gbn::cplx<T> *)fk);
    } catch (...) {
      cudaStreamEndCapture(P.stream, &g);
      if (g) cudaGraphDestroy(g);
      P.time_stages = ts;
      throw;
    }
    GBN_CUDA(cudaStreamEndCapture(P.stream, &g));
    P.time_stages = ts;
    cudaError_t e = cudaGraphInstantiate(&h->graph.exec, g, 0);
    cudaGraphDestroy(g);
    GBN_CUDA(e);
  });
}

template <typename T> int graph_launch_dev(void *p) {
  return guarded([&] {
    auto *h = dev<T>(p);
    if (!h->graph.exec) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "no captured graph");
    gbn::DeviceScope ds(h->plan->opts.gpu_device_id);
    GBN_CUDA(cudaGraphLaunch(h->graph.exec, h->plan->stream));
  });
}

// -------------------------------------------------------------- simple ----
template <typename T>
int simple_dev(int dim, int type, int ntr, int64_t nj, const T *x, const T *y, const T *z,
               void *c, int iflag, T eps, const int64_t *modes, int64_t nk, const T *s,
               const T *t, const T *u, void *fk, const cufinufft_opts *opts) {
  if (nj > std::numeric_limits<int32_t>::max()) return FINUFFT_ERR_NDATA_NOTVALID;
  if (nk > std::numeric_limits<int32_t>::max()) return FINUFFT_ERR_NDATA_NOTVALID;
  void *plan = nullptr;
  int ier = makeplan_dev<T>(type, dim, modes, iflag, ntr, (double)eps, &plan, opts);
  if (ier) return ier;
  ier = setpts_dev<T>(plan, nj, x, y, z, (int)nk, s, t, u);
  if (!ier) ier = execute_dev<T>(plan, c, fk, false);
  const int ier2 = destroy_dev<T>(plan);
  return ier ? ier : ier2;
}

} // namespace

// =================================================== cufinufft (device) ====
extern "C" {

void cufinufft_default_opts(cufinufft_opts *opts)
// defaults of src/cuda/c_interface.cpp:134-174
{
  if (!opts) return;
  opts->upsampfac = 0.0;
  opts->gpu_method = 0;
  opts->gpu_sort = 1;
  opts->gpu_binsizex = opts->gpu_binsizey = opts->gpu_binsizez = 0;
  opts->gpu_obinsizex = opts->gpu_obinsizey = opts->gpu_obinsizez = 0;
  opts->gpu_maxsubprobsize = 1024;
  opts->gpu_kerevalmeth = 1;
  opts->gpu_spreadinterponly = 0;
  opts->gpu_maxbatchsize = 0;
  opts->gpu_device_id = 0;
  opts->gpu_stream = nullptr;
  opts->modeord = 0;
  opts->gpu_np = 0;
  opts->debug = 0;
}

int cufinufft_makeplan(int type, int dim, const int64_t *n_modes, int iflag, int ntr,
                       double eps, cufinufft_plan *p, const cufinufft_opts *o) {
  return makeplan_dev<double>(type, dim, n_modes, iflag, ntr, eps, (void **)p, o);
}
int cufinufftf_makeplan(int type, int dim, const int64_t *n_modes, int iflag, int ntr,
                        float eps, cufinufftf_plan *p, const cufinufft_opts *o) {
  return makeplan_dev<float>(type, dim, n_modes, iflag, ntr, (double)eps, (void **)p, o);
}
int cufinufft_setpts(cufinufft_plan p, int64_t M, const double *x, const double *y,
                     const double *z, int N, const double *s, const double *t, const double *u) {
  return setpts_dev<double>(p, M, x, y, z, N, s, t, u);
}
int cufinufftf_setpts(cufinufftf_plan p, int64_t M, const float *x, const float *y,
                      const float *z, int N, const float *s, const float *t, const float *u) {
  return setpts_dev<float>(p, M, x, y, z, N, s, t, u);
}
int cufinufft_execute(cufinufft_plan p, cuDoubleComplex *c, cuDoubleComplex *fk) {
  return execute_dev<double>(p, c, fk, false);
}
int cufinufftf_execute(cufinufftf_plan p, cuFloatComplex *c, cuFloatComplex *fk) {
  return execute_dev<float>(p, c, fk, false);
}
int cufinufft_destroy(cufinufft_plan p) { return destroy_dev<double>(p); }
int cufinufftf_destroy(cufinufftf_plan p) { return destroy_dev<float>(p); }

#define GBN_EXT_DEFS(P, PLAN, T, C)                                                       \
  int P##_makeplan_ext(int ty, int dim, const int64_t *n, int fl, int ntr, T eps, PLAN *p, \
                       const cufinufft_opts *o, const gbnufft_opts *e) {                  \
    return makeplan_dev<T>(ty, dim, n, fl, ntr, (double)eps, (void **)p, o, e);           \
  }                                                                                       \
  int P##_execute_adjoint(PLAN p, C *c, C *fk) { return execute_dev<T>(p, c, fk, true); } \
  int P##_plan_info(PLAN p, gbnufft_plan_info *i) { return info_dev<T>(p, i); }           \
  int P##_stage_times(PLAN p, int en, float ms[4]) { return times_dev<T>(p, en, ms); }    \
  int P##_get_sort(PLAN p, int *perm, T *loc) { return get_sort_dev<T>(p, perm, loc); }   \
  int P##_graph_capture(PLAN p, C *c, C *fk) { return graph_capture_dev<T>(p, c, fk); }   \
  int P##_graph_launch(PLAN p) { return graph_launch_dev<T>(p); }
GBN_EXT_DEFS(cufinufft, cufinufft_plan, double, cuDoubleComplex)
GBN_EXT_DEFS(cufinufftf, cufinufftf_plan, float, cuFloatComplex)

const char *gbnufft_version(void) { return "gb300-nufft 0.1 (sm_103a)"; }

int gbnufft_trim_scratch(int device) {
  return guarded([&] {
    gbn::DeviceScope ds(device);
    gbn::trim_scratch_pool();
  });
}

int gbnufft_kernel_choice(double tol, double sigma, int dim, int type, int is_float, int form,
                          int kerformula, int *ns, double *beta) {
  return guarded([&] {
    if (!ns || !beta) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "ns/beta");
    const gbn::KernelChoice kc =
        form == gbn::KERNEL_PSWF
            ? gbn::choose_kernel_pswf(tol, sigma, dim, type, is_float, kerformula, 0, 0, 0)
            : gbn::choose_kernel(tol, sigma, 0, is_float, 0, 0);
    *ns = kc.ns;
    *beta = kc.beta;
  });
}

int gbnufft_kernel_eval(int form, int ns, double beta, int64_t n, const double *x,
                        double *out) {
  return guarded([&] {
    if (form != gbn::KERNEL_ES && form != gbn::KERNEL_PSWF)
      GBN_THROW(FINUFFT_ERR_KERFORMULA_NOTVALID, "form");
    if (ns < 2 || ns > gbn::MAX_NS || n < 0 || (n > 0 && (!x || !out)))
      GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "ns/n");
    const gbn::KernelFn phi = gbn::make_kernel_fn(form, ns, beta);
    for (int64_t i = 0; i < n; ++i) out[i] = phi(x[i]);
  });
}

int gbnufft_planner_dims(int *nfeat, int *hidden, int *nslots, int *nweights) {
  return guarded([&] {
    if (!nfeat || !hidden || !nslots || !nweights) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null");
    *nfeat = gbn::PLANNER_NF;
    *hidden = gbn::PLANNER_H;
    *nslots = gbn::PLANNER_K;
    *nweights = gbn::PLANNER_NW;
  });
}

int gbnufft_planner_candidate(int dim, int is_double, int slot, double *sigma, int *bins,
                              int *maxsub, int *variant, int *reference) {
  return guarded([&] {
    gbn::Candidate c;
    if (!gbn::planner_candidate(dim, is_double != 0, slot, &c))
      GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "slot");
    if (sigma) *sigma = c.sigma;
    if (bins)
      for (int d = 0; d < 3; ++d) bins[d] = c.bins[d];
    if (maxsub) *maxsub = c.maxsub;
    if (variant) *variant = c.variant;
    if (reference) *reference = c.reference;
  });
}

int gbnufft_planner_valid(int type, int dim, int is_double, double tol, int slot, int *valid) {
  return guarded([&] {
    if (!valid) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "valid");
    gbn::Candidate c;
    if (!gbn::planner_candidate(dim, is_double != 0, slot, &c))
      GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "slot");
    *valid = gbn::planner_candidate_valid(c, type, dim, is_double != 0, tol) ? 1 : 0;
  });
}

int gbnufft_planner_model(int *trained, float *weights, float *mean, float *stdev, float *lo,
                          float *hi, float *ymean, float *ystd) {
  return guarded([&] {
    const gbn::PlannerModel &m = gbn::planner_model();
    if (trained) *trained = m.trained ? 1 : 0;
    if (mean) std::memcpy(mean, m.mean, sizeof(float) * gbn::PLANNER_NF);
    if (stdev) std::memcpy(stdev, m.stdev, sizeof(float) * gbn::PLANNER_NF);
    if (lo) std::memcpy(lo, m.lo, sizeof(float) * gbn::PLANNER_NF);
    if (hi) std::memcpy(hi, m.hi, sizeof(float) * gbn::PLANNER_NF);
    if (ymean) *ymean = m.ymean;
    if (ystd) *ystd = m.ystd;
    if (weights) gbn::planner_weights_host(weights);
  });
}

int gbnufft_planner_forward(const float *d_weights, int n, const float *d_x, float *d_y,
                            void *stream) {
  return guarded([&] {
    if (n < 0 || (n > 0 && (!d_weights || !d_x || !d_y)))
      GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "forward");
    gbn::mlp_forward(d_weights, n, d_x, d_y, (cudaStream_t)stream);
  });
}

int gbnufft_planner_train(int n, const float *x, const float *t, const float *mask, int epochs,
                          int batch, float lr, float weight_decay, unsigned seed, float *w,
                          float *loss) {
  return guarded([&] {
    if (n < 1 || epochs < 1 || batch < 1 || !x || !t || !mask || !w)
      GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "train");
    gbn::mlp_train(n, x, t, mask, epochs, batch, lr, weight_decay, seed, w, loss);
  });
}

int gbnufft_point_features(int dim, int type, int is_double, int64_t M, const void *d_x,
                           const void *d_y, const void *d_z, const double *shift,
                           const double *scale, double nmodes, double tol, int ntr,
                           double xs_product, float *feat, void *stream) {
  return guarded([&] {
    if (dim < 1 || dim > 3 || M < 0 || !shift || !scale || !feat)
      GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "features");
    const cudaStream_t s = (cudaStream_t)stream;
    if (is_double) {
      const double *xyz[3] = {(const double *)d_x, (const double *)(dim > 1 ? d_y : d_x),
                              (const double *)(dim > 2 ? d_z : d_x)};
      gbn::point_features<double>(dim, type, true, M, xyz, shift, scale, nmodes, tol, ntr,
                                  xs_product, feat, s);
    } else {
      const float *xyz[3] = {(const float *)d_x, (const float *)(dim > 1 ? d_y : d_x),
                             (const float *)(dim > 2 ? d_z : d_x)};
      gbn::point_features<float>(dim, type, false, M, xyz, shift, scale, nmodes, tol, ntr,
                                 xs_product, feat, s);
    }
  });
}

int gbnufft_device_error(int device, int *code) {
  return guarded([&] {
    if (!code) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "code");
    gbn::DeviceScope ds(device);
    *code = gbn::device_error_take();
  });
}

int gbnufft_smem_atomic_rate(int device, double *rate) {
  return guarded([&] {
    if (!rate) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "rate");
    gbn::DeviceScope ds(device);
    *rate = gbn::smem_atomic_rate(device);
  });
}

int gbnufft_smem_atomic_rate_i32(int device, double *rate) {
  return guarded([&] {
    if (!rate) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "rate");
    gbn::DeviceScope ds(device);
    *rate = gbn::smem_atomic_rate(device, true);
  });
}

// 36 simple interfaces (include/cufinufft.h:39-186)
#define GBN_SIMPLE_DEFS(P, T, C)                                                                \
  int P##1d1many(int nt, int64_t nj, const T *x, const C *c, int fl, T e, int64_t ms, C *fk,   \
                 const cufinufft_opts *o) {                                                     \
    const int64_t m[3] = {ms, 1, 1};                                                            \
    return simple_dev<T>(1, 1, nt, nj, x, nullptr, nullptr, (void *)c, fl, e, m, 0, nullptr,    \
                         nullptr, nullptr, fk, o);                                              \
  }                                                                                             \
  int P##1d1(int64_t nj, const T *x, const C *c, int fl, T e, int64_t ms, C *fk,               \
             const cufinufft_opts *o) {                                                         \
    return P##1d1many(1, nj, x, c, fl, e, ms, fk, o);                                           \
  }                                                                                             \
  int P##1d2many(int nt, int64_t nj, const T *x, C *c, int fl, T e, int64_t ms, const C *fk,   \
                 const cufinufft_opts *o) {                                                     \
    const int64_t m[3] = {ms, 1, 1};                                                            \
    return simple_dev<T>(1, 2, nt, nj, x, nullptr, nullptr, c, fl, e, m, 0, nullptr, nullptr,   \
                         nullptr, (void *)fk, o);                                               \
  }                                                                                             \
  int P##1d2(int64_t nj, const T *x, C *c, int fl, T e, int64_t ms, const C *fk,               \
             const cufinufft_opts *o) {                                                         \
    return P##1d2many(1, nj, x, c, fl, e, ms, fk, o);                                           \
  }                                                                                             \
  int P##1d3many(int nt, int64_t nj, const T *x, const C *c, int fl, T e, int64_t nk,          \
                 const T *s, C *fk, const cufinufft_opts *o) {                                  \
    return simple_dev<T>(1, 3, nt, nj, x, nullptr, nullptr, (void *)c, fl, e, nullptr, nk, s,   \
                         nullptr, nullptr, fk, o);                                              \
  }                                                                                             \
  int P##1d3(int64_t nj, const T *x, const C *c, int fl, T e, int64_t nk, const T *s, C *fk,   \
             const cufinufft_opts *o) {                                                         \
    return P##1d3many(1, nj, x, c, fl, e, nk, s, fk, o);                                        \
  }                                                                                             \
  int P##2d1many(int nt, int64_t nj, const T *x, const T *y, const C *c, int fl, T e,          \
                 int64_t ms, int64_t mt, C *fk, const cufinufft_opts *o) {                      \
    const int64_t m[3] = {ms, mt, 1};                                                           \
    return simple_dev<T>(2, 1, nt, nj, x, y, nullptr, (void *)c, fl, e, m, 0, nullptr, nullptr, \
                         nullptr, fk, o);                                                       \
  }                                                                                             \
  int P##2d1(int64_t nj, const T *x, const T *y, const C *c, int fl, T e, int64_t ms,          \
             int64_t mt, C *fk, const cufinufft_opts *o) {                                      \
    return P##2d1many(1, nj, x, y, c, fl, e, ms, mt, fk, o);                                    \
  }                                                                                             \
  int P##2d2many(int nt, int64_t nj, const T *x, const T *y, C *c, int fl, T e, int64_t ms,    \
                 int64_t mt, const C *fk, const cufinufft_opts *o) {                            \
    const int64_t m[3] = {ms, mt, 1};                                                           \
    return simple_dev<T>(2, 2, nt, nj, x, y, nullptr, c, fl, e, m, 0, nullptr, nullptr,         \
                         nullptr, (void *)fk, o);                                               \
  }                                                                                             \
  int P##2d2(int64_t nj, const T *x, const T *y, C *c, int fl, T e, int64_t ms, int64_t mt,    \
             const C *fk, const cufinufft_opts *o) {                                            \
    return P##2d2many(1, nj, x, y, c, fl, e, ms, mt, fk, o);                                    \
  }                                                                                             \
  int P##2d3many(int nt, int64_t nj, const T *x, const T *y, const C *c, int fl, T e,          \
                 int64_t nk, const T *s, const T *t, C *fk, const cufinufft_opts *o) {          \
    return simple_dev<T>(2, 3, nt, nj, x, y, nullptr, (void *)c, fl, e, nullptr, nk, s, t,      \
                         nullptr, fk, o);                                                       \
  }                                                                                             \
  int P##2d3(int64_t nj, const T *x, const T *y, const C *c, int fl, T e, int64_t nk,          \
             const T *s, const T *t, C *fk, const cufinufft_opts *o) {                          \
    return P##2d3many(1, nj, x, y, c, fl, e, nk, s, t, fk, o);                                  \
  }                                                                                             \
  int P##3d1many(int nt, int64_t nj, const T *x, const T *y, const T *z, const C *c, int fl,   \
                 T e, int64_t ms, int64_t mt, int64_t mu, C *fk, const cufinufft_opts *o) {     \
    const int64_t m[3] = {ms, mt, mu};                                                          \
    return simple_dev<T>(3, 1, nt, nj, x, y, z, (void *)c, fl, e, m, 0, nullptr, nullptr,       \
                         nullptr, fk, o);                                                       \
  }                                                                                             \
  int P##3d1(int64_t nj, const T *x, const T *y, const T *z, const C *c, int fl, T e,          \
             int64_t ms, int64_t mt, int64_t mu, C *fk, const cufinufft_opts *o) {              \
    return P##3d1many(1, nj, x, y, z, c, fl, e, ms, mt, mu, fk, o);                             \
  }                                                                                             \
  int P##3d2many(int nt, int64_t nj, const T *x, const T *y, const T *z, C *c, int fl, T e,    \
                 int64_t ms, int64_t mt, int64_t mu, const C *fk, const cufinufft_opts *o) {    \
    const int64_t m[3] = {ms, mt, mu};                                                          \
    return simple_dev<T>(3, 2, nt, nj, x, y, z, c, fl, e, m, 0, nullptr, nullptr, nullptr,      \
                         (void *)fk, o);                                                        \
  }                                                                                             \
  int P##3d2(int64_t nj, const T *x, const T *y, const T *z, C *c, int fl, T e, int64_t ms,    \
             int64_t mt, int64_t mu, const C *fk, const cufinufft_opts *o) {                    \
    return P##3d2many(1, nj, x, y, z, c, fl, e, ms, mt, mu, fk, o);                             \
  }                                                                                             \
  int P##3d3many(int nt, int64_t nj, const T *x, const T *y, const T *z, const C *c, int fl,   \
                 T e, int64_t nk, const T *s, const T *t, const T *u, C *fk,                    \
                 const cufinufft_opts *o) {                                                     \
    return simple_dev<T>(3, 3, nt, nj, x, y, z, (void *)c, fl, e, nullptr, nk, s, t, u, fk, o); \
  }                                                                                             \
  int P##3d3(int64_t nj, const T *x, const T *y, const T *z, const C *c, int fl, T e,          \
             int64_t nk, const T *s, const T *t, const T *u, C *fk, const cufinufft_opts *o) {  \
    return P##3d3many(1, nj, x, y, z, c, fl, e, nk, s, t, u, fk, o);                            \
  }
GBN_SIMPLE_DEFS(cufinufft, double, cuDoubleComplex)
GBN_SIMPLE_DEFS(cufinufftf, float, cuFloatComplex)

} // extern "C"
