// Host-pointer interface finufft[f]_* (include/finufft/finufft_eitherprec.h:55-140
// upstream). Arguments are host arrays, as for the CPU library; a plan stages
// them through its own CUDA stream and computes with the device engine.
#include <cfloat>
#include <complex>
#include <cstring>
#include <limits>
#include <memory>
#include <new>

#include "cufinufft.h"
#include "finufft.h"
#include "plan.h"

const int FINUFFT_FFT_DEFAULT = 64;

using gbn::DevArray;
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

template <typename T> struct HostPlan {
  std::unique_ptr<Plan<T>> plan;
  cudaStream_t stream = nullptr;
  int type = 0, dim = 0, ntr = 0;
  int64_t M = 0, N = 0, nmodes = 1;
  DevArray<T> xyz[3], stu[3];
  DevArray<gbn::cplx<T>> dc, dfk;
  // copy streams and events of the pipelined execute (input copy of batch k+1
  // and output copy of batch k-1 overlap the transform of batch k)
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_in = nullptr, ev_done = nullptr;
  ~HostPlan() {
    plan.reset();
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_done) cudaEventDestroy(ev_done);
    if (copy_in) cudaStreamDestroy(copy_in);
    if (copy_out) cudaStreamDestroy(copy_out);
    for (auto &a : xyz) a.release();
    for (auto &a : stu) a.release();
    dc.release();
    dfk.release();
    if (stream) cudaStreamDestroy(stream);
  }
};

template <typename T>
int makeplan_host(int type, int dim, const int64_t *n_modes, int iflag, int ntr, T tol,
                  void **out, const finufft_opts *o) {
  return guarded([&] {
    if (!out) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null plan pointer");
    finufft_opts fo;
    if (o) fo = *o;
    else finufft_default_opts(&fo);
    if (type < 1 || type > 3) GBN_THROW(FINUFFT_ERR_TYPE_NOTVALID, "type");
    if (dim < 1 || dim > 3) GBN_THROW(FINUFFT_ERR_DIM_NOTVALID, "dim");
    if (ntr < 1) GBN_THROW(FINUFFT_ERR_NTRANS_NOTVALID, "ntrans");
    const double eps_mach = std::is_same_v<T, float> ? FLT_EPSILON : DBL_EPSILON;
    if ((double)tol < eps_mach && !fo.allow_eps_too_small)
      GBN_THROW(FINUFFT_ERR_EPS_TOO_SMALL, "tol below machine epsilon");
    int64_t m3[3] = {1, 1, 1};
    if (type != 3) {
      if (!n_modes) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "modes");
      int64_t tot = 1;
      for (int d = 0; d < dim; ++d) {
        if (n_modes[d] < 1) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "modes");
        m3[d] = n_modes[d];
        tot *= n_modes[d];
        if (tot > std::numeric_limits<int32_t>::max()) GBN_THROW(FINUFFT_ERR_MAXNALLOC, "modes");
      }
    }
    cufinufft_opts co;
    cufinufft_default_opts(&co);
    co.modeord = fo.modeord;
    co.gpu_spreadinterponly = fo.spreadinterponly;
    co.debug = fo.debug;
    co.upsampfac = fo.upsampfac;
    // batches of the pipelined execute: at least four when ntr allows, at most 8
    // transforms each, so that copies of one batch overlap the next
    co.gpu_maxbatchsize = fo.maxbatchsize > 0 ? fo.maxbatchsize
                                              : std::min(8, std::max(1, (ntr + 3) / 4));
    if (fo.spread_max_sp_size > 0) co.gpu_maxsubprobsize = fo.spread_max_sp_size;
    // the CPU library's kernel: the PSWF with its shape choice (any sigma > 1;
    // the pieces are fitted for the sigma given), spread/interp-only included.
    // kerevalmeth 0 only lifts the GPU interface's restriction of Horner
    // evaluation to sigma 2 and 1.25 (the PSWF is always evaluated by Horner)
    if (fo.upsampfac != 0.0 && fo.upsampfac != 2.0 && fo.upsampfac != 1.25)
      co.gpu_kerevalmeth = 0;
    gbnufft_opts ext;
    gbnufft_default_opts(&ext);
    ext.kernel_form = gbn::KERNEL_PSWF;
    ext.kerformula = fo.spread_kerformula;
    int dev = 0;
    GBN_CUDA(cudaGetDevice(&dev));
    co.gpu_device_id = dev;
    auto h = std::make_unique<HostPlan<T>>();
    GBN_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    GBN_CUDA(cudaStreamCreateWithFlags(&h->copy_in, cudaStreamNonBlocking));
    GBN_CUDA(cudaStreamCreateWithFlags(&h->copy_out, cudaStreamNonBlocking));
    GBN_CUDA(cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming));
    GBN_CUDA(cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming));
    co.gpu_stream = h->stream;
    h->type = type;
    h->dim = dim;
    h->ntr = ntr;
    h->nmodes = m3[0] * m3[1] * m3[2];
    h->plan.reset(new Plan<T>(type, dim, m3, iflag, ntr, (double)tol, co, &ext));
    *out = h.release();
  });
}

template <typename T> HostPlan<T> *hp(void *p) {
  if (!p) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "null plan");
  return static_cast<HostPlan<T> *>(p);
}

template <typename T>
int setpts_host(void *p, int64_t M, const T *x, const T *y, const T *z, int64_t N, const T *s,
                const T *t, const T *u) {
  return guarded([&] {
    HostPlan<T> *h = hp<T>(p);
    if (M < 0 || M > std::numeric_limits<int32_t>::max())
      GBN_THROW(FINUFFT_ERR_NUM_NU_PTS_INVALID, "M");
    const T *in[3] = {x, y, z};
    const T *tin[3] = {s, t, u};
    for (int d = 0; d < h->dim; ++d) {
      if (M > 0 && !in[d]) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null coordinates");
      h->xyz[d].resize((size_t)std::max<int64_t>(M, 1));
      if (M > 0)
        GBN_CUDA(cudaMemcpyAsync(h->xyz[d].p, in[d], (size_t)M * sizeof(T),
                                 cudaMemcpyHostToDevice, h->stream));
    }
    if (h->type == 3) {
      if (N < 0 || N > std::numeric_limits<int32_t>::max())
        GBN_THROW(FINUFFT_ERR_NUM_NU_PTS_INVALID, "N");
      for (int d = 0; d < h->dim; ++d) {
        if (!tin[d]) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null targets");
        h->stu[d].resize((size_t)std::max<int64_t>(N, 1));
        if (N > 0)
          GBN_CUDA(cudaMemcpyAsync(h->stu[d].p, tin[d], (size_t)N * sizeof(T),
                                   cudaMemcpyHostToDevice, h->stream));
      }
    }
    h->M = M;
    h->N = h->type == 3 ? N : 0;
    h->plan->setpts(M, h->xyz[0].p, h->xyz[1].p, h->xyz[2].p, (int)h->N, h->stu[0].p,
                    h->stu[1].p, h->stu[2].p);
    const int64_t nout = h->type == 3 ? h->N : h->nmodes;
    h->dc.resize((size_t)std::max<int64_t>(M * h->ntr, 1));
    h->dfk.resize((size_t)std::max<int64_t>(nout * h->ntr, 1));
  });
}

// c: weights at the sources (M per transform); f: modes (type 1, 2) or target values (type 3).
// The transforms run in the plan's batches, pipelined over three streams: the
// input copy of batch k+1 and the output copy of batch k-1 overlap batch k (with
// pinned host arrays the copies are asynchronous DMA; with pageable arrays the
// driver stages them and the overlap is partial).
template <typename T>
int execute_host(void *p, std::complex<T> *c, std::complex<T> *f, bool adjoint) {
  return guarded([&] {
    HostPlan<T> *h = hp<T>(p);
    const int64_t per_c = h->M;
    const int64_t per_f = h->type == 3 ? h->N : h->nmodes;
    // which side is input: type 1/3 forward and type 2 adjoint read c
    const bool c_in = (h->type != 2) != adjoint;
    const int64_t per_in = c_in ? per_c : per_f, per_out = c_in ? per_f : per_c;
    gbn::cplx<T> *din = c_in ? h->dc.p : h->dfk.p, *dout = c_in ? h->dfk.p : h->dc.p;
    std::complex<T> *hin = c_in ? c : f, *hout = c_in ? f : c;
    const size_t esz = sizeof(std::complex<T>);
    const int bs = std::max(1, h->plan->batchsize);
    const int nb = (h->ntr + bs - 1) / bs;
    auto copy_in = [&](int b) {
      const int t0 = b * bs, nt = std::min(bs, h->ntr - t0);
      const size_t bytes = (size_t)nt * per_in * esz;
      if (bytes)
        GBN_CUDA(cudaMemcpyAsync(din + (int64_t)t0 * per_in, hin + (int64_t)t0 * per_in, bytes,
                                 cudaMemcpyHostToDevice, h->copy_in));
      GBN_CUDA(cudaEventRecord(h->ev_in, h->copy_in));
    };
    copy_in(0);
    for (int b = 0; b < nb; ++b) {
      const int t0 = b * bs, nt = std::min(bs, h->ntr - t0);
      GBN_CUDA(cudaStreamWaitEvent(h->stream, h->ev_in, 0));
      h->plan->execute_range(h->dc.p, h->dfk.p, t0, nt, adjoint);
      GBN_CUDA(cudaEventRecord(h->ev_done, h->stream));
      if (b + 1 < nb) copy_in(b + 1);
      GBN_CUDA(cudaStreamWaitEvent(h->copy_out, h->ev_done, 0));
      const size_t bytes = (size_t)nt * per_out * esz;
      if (bytes)
        GBN_CUDA(cudaMemcpyAsync(hout + (int64_t)t0 * per_out, dout + (int64_t)t0 * per_out,
                                 bytes, cudaMemcpyDeviceToHost, h->copy_out));
    }
    GBN_CUDA(cudaStreamSynchronize(h->copy_out));
    GBN_CUDA(cudaStreamSynchronize(h->stream));
  });
}

template <typename T> int destroy_host(void *p) {
  return guarded([&] {
    if (!p) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "null plan");
    delete static_cast<HostPlan<T> *>(p);
  });
}

template <typename T>
int simple_host(int dim, int type, int ntr, int64_t nj, const T *x, const T *y, const T *z,
                std::complex<T> *c, int iflag, T eps, const int64_t *modes, int64_t nk,
                const T *s, const T *t, const T *u, std::complex<T> *f, const finufft_opts *o) {
  void *plan = nullptr;
  int ier = makeplan_host<T>(type, dim, modes, iflag, ntr, eps, &plan, o);
  if (ier) return ier;
  ier = setpts_host<T>(plan, nj, x, y, z, nk, s, t, u);
  if (!ier) ier = execute_host<T>(plan, c, f, false);
  const int ier2 = destroy_host<T>(plan);
  return ier ? ier : ier2;
}

} // namespace

extern "C" {

void finufft_default_opts(finufft_opts *o)
// defaults of include/finufft/plan.hpp:294-335
{
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->modeord = 0;
  o->spreadinterponly = 0;
  o->debug = 0;
  o->spread_debug = 0;
  o->showwarn = 1;
  o->nthreads = 0;
  o->fftw = FINUFFT_FFT_DEFAULT;
  o->spread_sort = 2;
  o->spread_kerevalmeth = 1;
  o->spread_kerpad = 1;
  o->upsampfac = 0.0;
  o->spread_thread = 0;
  o->maxbatchsize = 0;
  o->spread_nthr_atomic = -1;
  o->spread_max_sp_size = 0;
  o->spread_kerformula = 0;
  o->allow_eps_too_small = 0;
  o->fftw_lock_fun = nullptr;
  o->fftw_unlock_fun = nullptr;
  o->fftw_lock_data = nullptr;
}
void finufftf_default_opts(finufft_opts *o) { finufft_default_opts(o); }

#define GBN_HOST_GURU(P, T, PLAN)                                                             \
  int P##_makeplan(int type, int dim, const int64_t *n, int iflag, int ntr, T tol, PLAN *pp,  \
                   const finufft_opts *o) {                                                   \
    return makeplan_host<T>(type, dim, n, iflag, ntr, tol, (void **)pp, o);                   \
  }                                                                                           \
  int P##_setpts(PLAN p, int64_t M, const T *x, const T *y, const T *z, int64_t N,           \
                 const T *s, const T *t, const T *u) {                                        \
    return setpts_host<T>(p, M, x, y, z, N, s, t, u);                                         \
  }                                                                                           \
  int P##_execute(PLAN p, std::complex<T> *c, std::complex<T> *f) {                           \
    return execute_host<T>(p, c, f, false);                                                   \
  }                                                                                           \
  int P##_execute_adjoint(PLAN p, std::complex<T> *c, std::complex<T> *f) {                   \
    return execute_host<T>(p, c, f, true);                                                    \
  }                                                                                           \
  int P##_destroy(PLAN p) { return destroy_host<T>(p); }
GBN_HOST_GURU(finufft, double, finufft_plan)
GBN_HOST_GURU(finufftf, float, finufftf_plan)

#define GBN_HOST_SIMPLE(P, T)                                                                  \
  int P##1d1(int64_t nj, const T *x, const std::complex<T> *c, int fl, T e, int64_t ms,       \
             std::complex<T> *fk, const finufft_opts *o) {                                     \
    return P##1d1many(1, nj, x, c, fl, e, ms, fk, o);                                          \
  }                                                                                            \
  int P##1d1many(int nt, int64_t nj, const T *x, const std::complex<T> *c, int fl, T e,       \
                 int64_t ms, std::complex<T> *fk, const finufft_opts *o) {                     \
    const int64_t m[3] = {ms, 1, 1};                                                           \
    return simple_host<T>(1, 1, nt, nj, x, nullptr, nullptr, (std::complex<T> *)c, fl, e, m,   \
                          0, nullptr, nullptr, nullptr, fk, o);                                \
  }                                                                                            \
  int P##1d2(int64_t nj, const T *x, std::complex<T> *c, int fl, T e, int64_t ms,             \
             const std::complex<T> *fk, const finufft_opts *o) {                               \
    return P##1d2many(1, nj, x, c, fl, e, ms, fk, o);                                          \
  }                                                                                            \
  int P##1d2many(int nt, int64_t nj, const T *x, std::complex<T> *c, int fl, T e, int64_t ms, \
                 const std::complex<T> *fk, const finufft_opts *o) {                           \
    const int64_t m[3] = {ms, 1, 1};                                                           \
    return simple_host<T>(1, 2, nt, nj, x, nullptr, nullptr, c, fl, e, m, 0, nullptr, nullptr, \
                          nullptr, (std::complex<T> *)fk, o);                                  \
  }                                                                                            \
  int P##1d3(int64_t nj, const T *x, const std::complex<T> *c, int fl, T e, int64_t nk,       \
             const T *s, std::complex<T> *f, const finufft_opts *o) {                          \
    return P##1d3many(1, nj, x, c, fl, e, nk, s, f, o);                                        \
  }                                                                                            \
  int P##1d3many(int nt, int64_t nj, const T *x, const std::complex<T> *c, int fl, T e,       \
                 int64_t nk, const T *s, std::complex<T> *f, const finufft_opts *o) {          \
    return simple_host<T>(1, 3, nt, nj, x, nullptr, nullptr, (std::complex<T> *)c, fl, e,      \
                          nullptr, nk, s, nullptr, nullptr, f, o);                             \
  }                                                                                            \
  int P##2d1(int64_t nj, const T *x, const T *y, const std::complex<T> *c, int fl, T e,       \
             int64_t ms, int64_t mt, std::complex<T> *fk, const finufft_opts *o) {             \
    return P##2d1many(1, nj, x, y, c, fl, e, ms, mt, fk, o);                                   \
  }                                                                                            \
  int P##2d1many(int nt, int64_t nj, const T *x, const T *y, const std::complex<T> *c,        \
                 int fl, T e, int64_t ms, int64_t mt, std::complex<T> *fk,                     \
                 const finufft_opts *o) {                                                      \
    const int64_t m[3] = {ms, mt, 1};                                                          \
    return simple_host<T>(2, 1, nt, nj, x, y, nullptr, (std::complex<T> *)c, fl, e, m, 0,      \
                          nullptr, nullptr, nullptr, fk, o);                                   \
  }                                                                                            \
  int P##2d2(int64_t nj, const T *x, const T *y, std::complex<T> *c, int fl, T e, int64_t ms, \
             int64_t mt, const std::complex<T> *fk, const finufft_opts *o) {                   \
    return P##2d2many(1, nj, x, y, c, fl, e, ms, mt, fk, o);                                   \
  }                                                                                            \
  int P##2d2many(int nt, int64_t nj, const T *x, const T *y, std::complex<T> *c, int fl, T e, \
                 int64_t ms, int64_t mt, const std::complex<T> *fk, const finufft_opts *o) {   \
    const int64_t m[3] = {ms, mt, 1};                                                          \
    return simple_host<T>(2, 2, nt, nj, x, y, nullptr, c, fl, e, m, 0, nullptr, nullptr,       \
                          nullptr, (std::complex<T> *)fk, o);                                  \
  }                                                                                            \
  int P##2d3(int64_t nj, const T *x, const T *y, const std::complex<T> *c, int fl, T e,       \
             int64_t nk, const T *s, const T *t, std::complex<T> *f, const finufft_opts *o) {  \
    return P##2d3many(1, nj, x, y, c, fl, e, nk, s, t, f, o);                                  \
  }                                                                                            \
  int P##2d3many(int nt, int64_t nj, const T *x, const T *y, const std::complex<T> *c,        \
                 int fl, T e, int64_t nk, const T *s, const T *t, std::complex<T> *f,          \
                 const finufft_opts *o) {                                                      \
    return simple_host<T>(2, 3, nt, nj, x, y, nullptr, (std::complex<T> *)c, fl, e, nullptr,   \
                          nk, s, t, nullptr, f, o);                                            \
  }                                                                                            \
  int P##3d1(int64_t nj, const T *x, const T *y, const T *z, const std::complex<T> *c, int fl, \
             T e, int64_t ms, int64_t mt, int64_t mu, std::complex<T> *fk,                     \
             const finufft_opts *o) {                                                          \
    return P##3d1many(1, nj, x, y, z, c, fl, e, ms, mt, mu, fk, o);                            \
  }                                                                                            \
  int P##3d1many(int nt, int64_t nj, const T *x, const T *y, const T *z,                      \
                 const std::complex<T> *c, int fl, T e, int64_t ms, int64_t mt, int64_t mu,    \
                 std::complex<T> *fk, const finufft_opts *o) {                                 \
    const int64_t m[3] = {ms, mt, mu};                                                         \
    return simple_host<T>(3, 1, nt, nj, x, y, z, (std::complex<T> *)c, fl, e, m, 0, nullptr,   \
                          nullptr, nullptr, fk, o);                                            \
  }                                                                                            \
  int P##3d2(int64_t nj, const T *x, const T *y, const T *z, std::complex<T> *c, int fl, T e, \
             int64_t ms, int64_t mt, int64_t mu, const std::complex<T> *fk,                    \
             const finufft_opts *o) {                                                          \
    return P##3d2many(1, nj, x, y, z, c, fl, e, ms, mt, mu, fk, o);                            \
  }                                                                                            \
  int P##3d2many(int nt, int64_t nj, const T *x, const T *y, const T *z, std::complex<T> *c,  \
                 int fl, T e, int64_t ms, int64_t mt, int64_t mu, const std::complex<T> *fk,   \
                 const finufft_opts *o) {                                                      \
    const int64_t m[3] = {ms, mt, mu};                                                         \
    return simple_host<T>(3, 2, nt, nj, x, y, z, c, fl, e, m, 0, nullptr, nullptr, nullptr,    \
                          (std::complex<T> *)fk, o);                                           \
  }                                                                                            \
  int P##3d3(int64_t nj, const T *x, const T *y, const T *z, const std::complex<T> *c, int fl, \
             T e, int64_t nk, const T *s, const T *t, const T *u, std::complex<T> *f,          \
             const finufft_opts *o) {                                                          \
    return P##3d3many(1, nj, x, y, z, c, fl, e, nk, s, t, u, f, o);                            \
  }                                                                                            \
  int P##3d3many(int nt, int64_t nj, const T *x, const T *y, const T *z,                      \
                 const std::complex<T> *c, int fl, T e, int64_t nk, const T *s, const T *t,    \
                 const T *u, std::complex<T> *f, const finufft_opts *o) {                      \
    return simple_host<T>(3, 3, nt, nj, x, y, z, (std::complex<T> *)c, fl, e, nullptr, nk, s,  \
                          t, u, f, o);                                                         \
  }
GBN_HOST_SIMPLE(finufft, double)
GBN_HOST_SIMPLE(finufftf, float)

} // extern "C"
