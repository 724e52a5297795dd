// Learned planner: candidate table, device point features, and the 2x64 MLP's
// CUDA kernels (inference, training by minibatch Adam).
//
// Features (raw, before standardisation), per problem:
//   0 dim, 1 type, 2 double precision (0/1), 3 log10(M + 1),
//   4 log10(modes + 1) (type 3: targets), 5 -log10(tol), 6 log2(transforms per batch),
//   7 coefficient of variation of the point counts on a coarse grid (32^3 cells in
//     3D, 128^2 in 2D, 4096 in 1D), 8 fraction of empty coarse cells,
//   9 log10(max count / mean count), 10 log10((M + 1) / (modes + 1)),
//   11 type 3: mean over dimensions of log10(X_d S_d + 1) (space-bandwidth), else 0.
// Outputs: standardised log10 of the execute time (ms) of each candidate slot.
#include "planner.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <random>
#include <vector>

#include "planning.h"
#include "sort.h"

namespace gbn {

#include "planner_weights.inc"

bool planner_candidate(int dim, bool dbl, int k, Candidate *c) {
  if (k < 0 || k >= PLANNER_K || (dim != 2 && dim != 3)) return false;
  static const double sig[3] = {2.0, 1.5, 1.25};
  const int si = k / 4, shape = k % 4;
  // 1.25 in single precision loses digits to the range of 1/phihat (the CPU
  // library caps single-precision widths below sigma 1.4 for the same reason)
  if (si == 2 && !dbl) return false;
  Candidate r{};
  r.sigma = sig[si];
  r.maxsub = 1024;
  r.variant = -1;
  r.reference = 0;
  if (dim == 3) {
    static const int b3[3][3] = {{16, 12, 8}, {16, 8, 8}, {8, 8, 8}};
    static const int ms3[3] = {4096, 4096, 2048};
    if (shape < 3) {
      std::copy(b3[shape], b3[shape] + 3, r.bins);
      r.maxsub = ms3[shape];
    } else {
      r.reference = 1;
    }
  } else {
    static const int b2[3][3] = {{32, 32, 1}, {64, 32, 1}, {64, 64, 1}};
    if (shape < 3) {
      std::copy(b2[shape], b2[shape] + 3, r.bins);
      r.maxsub = 1024;
    } else {
      r.reference = 1;
    }
  }
  if (r.reference) r.bins[0] = r.bins[1] = r.bins[2] = 0; // the heuristic's
  *c = r;
  return true;
}

bool planner_candidate_valid(const Candidate &c, int type, int dim, bool dbl, double tol) {
  // analytic rejection: the kernel width for tol at this sigma -- the larger of
  // the PSWF width law and the GPU rule, as the plan would pick it -- must fit
  // the precision's widest kernel (unclipped, the law's aliasing bound reaches
  // tol). In single precision a sigma below 2 also needs tol >= 1e-5: the
  // larger range of 1/phihat lifts the float rounding above the tolerance
  // below that (the engine's own timing and error sweeps: 16% of the sigma-1.5
  // float plans at tol < 1e-5 had errors above 2 tol, none at sigma 2).
  const double t = std::max(tol, dbl ? DBL_EPSILON : (double)FLT_EPSILON);
  const double tolfac = 0.18 * std::pow(1.4, dim - 1) * (type == 3 ? 1.4 : 1.0);
  const double u = PI * std::sqrt(1.0 - 1.0 / c.sigma);
  const int ns_law = (int)std::ceil(std::log(tolfac / t) / u + 1.0);
  const int ns_gpu = c.sigma == 2.0 ? (int)std::ceil(-std::log10(t / 10.0))
                                    : (int)std::ceil(-std::log(t) / u);
  const int ns = std::max(2, std::max(ns_law, ns_gpu));
  const int maxns = dbl ? MAX_NS : MAX_NS_FLOAT;
  if (!dbl && c.sigma < 2.0 && tol < 1e-5) return false;
  return ns <= maxns && kernel_tol_bound(ns, c.sigma, dim, type) <= t * (1 + 1e-9);
}

double kernel_tol_bound(int ns, double sigma, int dim, int type) {
  const double tolfac = 0.18 * std::pow(1.4, dim - 1) * (type == 3 ? 1.4 : 1.0);
  return tolfac * std::exp(-PI * (ns - 1) * std::sqrt(1.0 - 1.0 / sigma));
}

// ------------------------------------------------------------- features ----
namespace {
constexpr int HIST_THREADS = 512;

int coarse_side(int dim) { return dim == 3 ? 32 : (dim == 2 ? 128 : 4096); }

template <typename T>
__global__ void coarse_hist_kernel(int dim, const T *x, const T *y, const T *z, int64_t nsamp,
                                   int64_t stride, double3 shift, double3 scale, int G,
                                   unsigned *hist) {
  extern __shared__ unsigned h[];
  const int cells = dim == 3 ? G * G * G : (dim == 2 ? G * G : G);
  for (int i = threadIdx.x; i < cells; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nsamp;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = s * stride;
    const T *xs[3] = {x, y, z};
    const double sh[3] = {shift.x, shift.y, shift.z}, sc[3] = {scale.x, scale.y, scale.z};
    int idx = 0, st = 1;
    for (int d = 0; d < dim; ++d) {
      double u = ((double)xs[d][j] - sh[d]) * sc[d];
      u -= floor(u);
      int c = (int)(u * G);
      c = c < 0 ? 0 : (c >= G ? G - 1 : c);
      idx += st * c;
      st *= G;
    }
    atomicAdd(&h[idx], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cells; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

// one block: sum, sum of squares, nonzero cells and maximum of the histogram
__global__ void hist_stats_kernel(const unsigned *hist, int cells, double *out) {
  __shared__ double s1[HIST_THREADS], s2[HIST_THREADS], nz[HIST_THREADS], mx[HIST_THREADS];
  double a = 0, b = 0, c = 0, m = 0;
  for (int i = threadIdx.x; i < cells; i += blockDim.x) {
    const double v = hist[i];
    a += v;
    b += v * v;
    c += v > 0 ? 1.0 : 0.0;
    m = v > m ? v : m;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  nz[threadIdx.x] = c;
  mx[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
      nz[threadIdx.x] += nz[threadIdx.x + w];
      mx[threadIdx.x] = fmax(mx[threadIdx.x], mx[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s1[0];
    out[1] = s2[0];
    out[2] = nz[0];
    out[3] = mx[0];
  }
}
} // namespace

template <typename T>
void point_features(int dim, int type, bool dbl, int64_t M, const T *const xyz[3],
                    const double shift[3], const double scale[3], double nmodes, double tol,
                    int ntr, double xs_product, float feat[PLANNER_NF], cudaStream_t s) {
  const int G = coarse_side(dim);
  const int cells = dim == 3 ? G * G * G : (dim == 2 ? G * G : G);
  double st[4] = {0, 0, 0, 0};
  if (M > 0) {
    const int64_t maxsamp = (int64_t)1 << 22;
    const int64_t stride = std::max<int64_t>(1, (M + maxsamp - 1) / maxsamp);
    const int64_t nsamp = (M + stride - 1) / stride;
    AsyncBuf hist((size_t)cells * sizeof(unsigned), s);
    AsyncBuf stats(4 * sizeof(double), s);
    GBN_CUDA(cudaMemsetAsync(hist.p, 0, (size_t)cells * sizeof(unsigned), s));
    const size_t smem = (size_t)cells * sizeof(unsigned);
    auto k = coarse_hist_kernel<T>;
    GBN_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0;
    GBN_CUDA(cudaGetDevice(&dev));
    GBN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t want = (nsamp + HIST_THREADS - 1) / HIST_THREADS;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, sms));
    k<<<blocks, HIST_THREADS, smem, s>>>(dim, xyz[0], xyz[1], xyz[2], nsamp, stride,
                                         make_double3(shift[0], shift[1], shift[2]),
                                         make_double3(scale[0], scale[1], scale[2]), G,
                                         hist.as<unsigned>());
    GBN_LAUNCH_CHECK();
    hist_stats_kernel<<<1, HIST_THREADS, 0, s>>>(hist.as<unsigned>(), cells, stats.as<double>());
    GBN_LAUNCH_CHECK();
    GBN_CUDA(cudaMemcpyAsync(st, stats.p, sizeof(st), cudaMemcpyDeviceToHost, s));
    GBN_CUDA(cudaStreamSynchronize(s));
  }
  const double n = st[0] > 0 ? st[0] : 1.0;
  const double mean = n / cells;
  const double var = std::max(0.0, st[1] / cells - mean * mean);
  feat[0] = (float)dim;
  feat[1] = (float)type;
  feat[2] = dbl ? 1.0f : 0.0f;
  feat[3] = (float)std::log10((double)M + 1.0);
  feat[4] = (float)std::log10(nmodes + 1.0);
  feat[5] = (float)(-std::log10(tol));
  feat[PLANNER_F_BATCH] = (float)std::log2((double)std::max(ntr, 1));
  feat[7] = (float)(std::sqrt(var) / mean);
  feat[8] = (float)(1.0 - st[2] / cells);
  feat[9] = (float)std::log10(std::max(st[3], 1.0) / mean);
  feat[10] = (float)std::log10(((double)M + 1.0) / (nmodes + 1.0));
  feat[11] = (float)std::log10(xs_product + 1.0);
}
template void point_features<float>(int, int, bool, int64_t, const float *const[3],
                                    const double[3], const double[3], double, double, int,
                                    double, float[PLANNER_NF], cudaStream_t);
template void point_features<double>(int, int, bool, int64_t, const double *const[3],
                                     const double[3], const double[3], double, double, int,
                                     double, float[PLANNER_NF], cudaStream_t);

// ------------------------------------------------------------------ MLP ----
namespace {
// one sample through the network, one thread per hidden unit (blockDim.x ==
// PLANNER_H): a0 input, a1/a2 hidden activations, y outputs (all shared)
__device__ void mlp_sample_forward(const float *w, const float *a0, float *a1, float *a2,
                                   float *y) {
  const int h = threadIdx.x;
  float z = w[PLANNER_OFF_B1 + h];
  for (int f = 0; f < PLANNER_NF; ++f) z += w[PLANNER_OFF_W1 + h * PLANNER_NF + f] * a0[f];
  a1[h] = tanhf(z);
  __syncthreads();
  z = w[PLANNER_OFF_B2 + h];
  for (int i = 0; i < PLANNER_H; ++i) z += w[PLANNER_OFF_W2 + h * PLANNER_H + i] * a1[i];
  a2[h] = tanhf(z);
  __syncthreads();
  if (h < PLANNER_K) {
    float o = w[PLANNER_OFF_B3 + h];
    for (int i = 0; i < PLANNER_H; ++i) o += w[PLANNER_OFF_W3 + h * PLANNER_H + i] * a2[i];
    y[h] = o;
  }
  __syncthreads();
}

__global__ void mlp_forward_kernel(const float *w, int n, const float *x, float *y) {
  __shared__ float a0[PLANNER_NF], a1[PLANNER_H], a2[PLANNER_H], o[PLANNER_K];
  for (int s = blockIdx.x; s < n; s += gridDim.x) {
    if (threadIdx.x < PLANNER_NF) a0[threadIdx.x] = x[(int64_t)s * PLANNER_NF + threadIdx.x];
    __syncthreads();
    mlp_sample_forward(w, a0, a1, a2, o);
    if (threadIdx.x < PLANNER_K) y[(int64_t)s * PLANNER_K + threadIdx.x] = o[threadIdx.x];
    __syncthreads();
  }
}

// Gradient of sum_k mask (y_k - t_k)^2 / norm over the samples idx[b*per ..
// (b+1)*per) of a minibatch. Each block keeps its gradient in shared memory
// (thread h owns row h of W1 and W2, column h of W3) and adds it to g once.
__global__ void mlp_grad_kernel(const float *w, const float *x, const float *t,
                                const float *mask, const int *idx, int nb, int per,
                                float inv_norm, float *g, float *loss) {
  __shared__ float a0[PLANNER_NF], a1[PLANNER_H], a2[PLANNER_H], y[PLANNER_K];
  __shared__ float dy[PLANNER_K], dz2[PLANNER_H], dz1[PLANNER_H];
  __shared__ float gw2[PLANNER_H * PLANNER_H];
  const int h = threadIdx.x;
  float gw1[PLANNER_NF], gb1 = 0, gb2 = 0, gw3[PLANNER_K], gb3 = 0, lsum = 0;
  for (int f = 0; f < PLANNER_NF; ++f) gw1[f] = 0;
  for (int k = 0; k < PLANNER_K; ++k) gw3[k] = 0;
  for (int i = 0; i < PLANNER_H; ++i) gw2[h * PLANNER_H + i] = 0;
  const int b0 = blockIdx.x * per, b1 = min(nb, b0 + per);
  for (int q = b0; q < b1; ++q) {
    const int s = idx[q];
    if (h < PLANNER_NF) a0[h] = x[(int64_t)s * PLANNER_NF + h];
    __syncthreads();
    mlp_sample_forward(w, a0, a1, a2, y);
    if (h < PLANNER_K) {
      const float m = mask[(int64_t)s * PLANNER_K + h];
      const float e = m > 0 ? y[h] - t[(int64_t)s * PLANNER_K + h] : 0.0f;
      dy[h] = 2.0f * e * inv_norm;
      lsum += e * e * inv_norm;
    }
    __syncthreads();
    // output layer: column h of W3
    float da2 = 0;
    for (int k = 0; k < PLANNER_K; ++k) {
      gw3[k] += dy[k] * a2[h];
      da2 += w[PLANNER_OFF_W3 + k * PLANNER_H + h] * dy[k];
    }
    if (h < PLANNER_K) gb3 += dy[h];
    dz2[h] = da2 * (1.0f - a2[h] * a2[h]);
    __syncthreads();
    // second hidden layer: row h of W2; back-propagate to the first
    for (int i = 0; i < PLANNER_H; ++i) gw2[h * PLANNER_H + i] += dz2[h] * a1[i];
    gb2 += dz2[h];
    float da1 = 0;
    for (int j = 0; j < PLANNER_H; ++j) da1 += w[PLANNER_OFF_W2 + j * PLANNER_H + h] * dz2[j];
    dz1[h] = da1 * (1.0f - a1[h] * a1[h]);
    __syncthreads();
    for (int f = 0; f < PLANNER_NF; ++f) gw1[f] += dz1[h] * a0[f];
    gb1 += dz1[h];
    __syncthreads();
  }
  for (int f = 0; f < PLANNER_NF; ++f) atomicAdd(&g[PLANNER_OFF_W1 + h * PLANNER_NF + f], gw1[f]);
  atomicAdd(&g[PLANNER_OFF_B1 + h], gb1);
  for (int i = 0; i < PLANNER_H; ++i)
    atomicAdd(&g[PLANNER_OFF_W2 + h * PLANNER_H + i], gw2[h * PLANNER_H + i]);
  atomicAdd(&g[PLANNER_OFF_B2 + h], gb2);
  for (int k = 0; k < PLANNER_K; ++k) atomicAdd(&g[PLANNER_OFF_W3 + k * PLANNER_H + h], gw3[k]);
  if (h < PLANNER_K) {
    atomicAdd(&g[PLANNER_OFF_B3 + h], gb3);
    atomicAdd(loss, lsum);
  }
}

__global__ void adam_kernel(float *w, const float *g, float *m, float *v, int nw, float lr,
                            float beta1, float beta2, float eps, float wd, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nw) return;
  const float gi = g[i] + wd * w[i];
  m[i] = beta1 * m[i] + (1.0f - beta1) * gi;
  v[i] = beta2 * v[i] + (1.0f - beta2) * gi * gi;
  w[i] -= lr * (m[i] / bc1) / (sqrtf(v[i] / bc2) + eps);
}
} // namespace

void mlp_forward(const float *w, int n, const float *x, float *y, cudaStream_t s) {
  if (n <= 0) return;
  mlp_forward_kernel<<<std::min(n, 4096), PLANNER_H, 0, s>>>(w, n, x, y);
  GBN_LAUNCH_CHECK();
}

namespace {
template <typename U> struct DevBuf {
  U *p = nullptr;
  explicit DevBuf(size_t n) { GBN_CUDA(cudaMalloc((void **)&p, std::max<size_t>(n, 1) * sizeof(U))); }
  ~DevBuf() { cudaFree(p); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
};
} // namespace

void mlp_train(int n, const float *x, const float *t, const float *mask, int epochs,
               int batch, float lr, float wd, unsigned seed, float *w, float *loss) {
  if (n <= 0 || epochs <= 0) return;
  batch = std::max(1, std::min(batch, n));
  DevBuf<float> dx((size_t)n * PLANNER_NF), dt((size_t)n * PLANNER_K), dm((size_t)n * PLANNER_K);
  DevBuf<float> dw(PLANNER_NW), dg(PLANNER_NW), am(PLANNER_NW), av(PLANNER_NW), dl(1);
  DevBuf<int> didx(n);
  GBN_CUDA(cudaMemcpy(dx.p, x, sizeof(float) * n * PLANNER_NF, cudaMemcpyHostToDevice));
  GBN_CUDA(cudaMemcpy(dt.p, t, sizeof(float) * n * PLANNER_K, cudaMemcpyHostToDevice));
  GBN_CUDA(cudaMemcpy(dm.p, mask, sizeof(float) * n * PLANNER_K, cudaMemcpyHostToDevice));
  GBN_CUDA(cudaMemcpy(dw.p, w, sizeof(float) * PLANNER_NW, cudaMemcpyHostToDevice));
  GBN_CUDA(cudaMemset(am.p, 0, sizeof(float) * PLANNER_NW));
  GBN_CUDA(cudaMemset(av.p, 0, sizeof(float) * PLANNER_NW));
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::mt19937 rng(seed);
  int step = 0;
  const int per = 8; // samples per block of the gradient kernel
  for (int e = 0; e < epochs; ++e) {
    std::shuffle(order.begin(), order.end(), rng);
    GBN_CUDA(cudaMemcpy(didx.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GBN_CUDA(cudaMemset(dl.p, 0, sizeof(float)));
    for (int b0 = 0; b0 < n; b0 += batch) {
      const int nb = std::min(batch, n - b0);
      double msum = 0;
      for (int q = b0; q < b0 + nb; ++q)
        for (int k = 0; k < PLANNER_K; ++k) msum += mask[(size_t)order[q] * PLANNER_K + k] > 0;
      const float inv = msum > 0 ? (float)(1.0 / msum) : 0.0f;
      GBN_CUDA(cudaMemset(dg.p, 0, sizeof(float) * PLANNER_NW));
      mlp_grad_kernel<<<(nb + per - 1) / per, PLANNER_H>>>(dw.p, dx.p, dt.p, dm.p, didx.p + b0,
                                                           nb, per, inv, dg.p, dl.p);
      GBN_LAUNCH_CHECK();
      ++step;
      const float b1 = 0.9f, b2 = 0.999f;
      adam_kernel<<<(PLANNER_NW + 255) / 256, 256>>>(
          dw.p, dg.p, am.p, av.p, PLANNER_NW, lr, b1, b2, 1e-8f, wd,
          1.0f - std::pow(b1, (float)step), 1.0f - std::pow(b2, (float)step));
      GBN_LAUNCH_CHECK();
    }
    float l = 0;
    GBN_CUDA(cudaMemcpy(&l, dl.p, sizeof(float), cudaMemcpyDeviceToHost));
    // the per-minibatch losses are means; average them over the minibatches
    if (loss) loss[e] = l / (float)((n + batch - 1) / batch);
  }
  GBN_CUDA(cudaMemcpy(w, dw.p, sizeof(float) * PLANNER_NW, cudaMemcpyDeviceToHost));
}

const PlannerModel &planner_model() {
  static const PlannerModel m{GBN_PLANNER_TRAINED != 0, kPlannerMean, kPlannerStd, kPlannerLo,
                              kPlannerHi, kPlannerYMean, kPlannerYStd};
  return m;
}

void planner_weights_host(float *w) {
  GBN_CUDA(cudaMemcpyFromSymbol(w, g_planner_w, sizeof(float) * PLANNER_NW));
}

bool planner_predict(const float feat[PLANNER_NF], double ms_out[PLANNER_K], cudaStream_t s) {
  const PlannerModel &m = planner_model();
  if (!m.trained) return false;
  float z[PLANNER_NF];
  for (int f = 0; f < PLANNER_NF; ++f) {
    float v = feat[f];
    // log2 of the transforms per batch saturates at the top of the model's
    // range: more transforms scale every slot's time alike (the sweeps batch
    // at most 4), so the ranking the model gives there holds
    if (f == PLANNER_F_BATCH && v > m.hi[f]) v = m.hi[f];
    if (v < m.lo[f] || v > m.hi[f]) return false; // outside the training range
    z[f] = m.stdev[f] > 0 ? (v - m.mean[f]) / m.stdev[f] : 0.0f;
  }
  float *w = nullptr;
  GBN_CUDA(cudaGetSymbolAddress((void **)&w, g_planner_w));
  AsyncBuf io((PLANNER_NF + PLANNER_K) * sizeof(float), s);
  float *dx = io.as<float>(), *dy = dx + PLANNER_NF;
  GBN_CUDA(cudaMemcpyAsync(dx, z, sizeof(z), cudaMemcpyHostToDevice, s));
  mlp_forward(w, 1, dx, dy, s);
  float y[PLANNER_K];
  GBN_CUDA(cudaMemcpyAsync(y, dy, sizeof(y), cudaMemcpyDeviceToHost, s));
  GBN_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < PLANNER_K; ++k)
    ms_out[k] = std::pow(10.0, (double)(y[k] * m.ystd + m.ymean));
  return true;
}

} // namespace gbn
