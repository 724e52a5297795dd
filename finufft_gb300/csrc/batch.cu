// Batched execution of many independent transforms of one type and dimension
// with different mode counts and point sets ("uneven batches"): one sort over
// all points, one spread (or interpolation) launch over all subproblems of all
// problems, cuFFT batched over problems of equal grid shape, and one
// deconvolution (or amplification) launch over all problems.
//
// Problem p has modes ms_p (x fastest), M_p points; its points, strengths and
// modes are contiguous slices of concatenated arrays, in problem order.
#include <algorithm>
#include <map>
#include <numeric>
#include <vector>

#include "batch.h"
#include "planning.h"
#include "sort.h"

namespace gbn {
namespace {

inline unsigned blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

// index k with off[k] <= i < off[k+1] (off ascending, n+1 entries)
template <typename I> __device__ __forceinline__ int find_slot(const I *off, int n, int64_t i) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((int64_t)off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct DevProb {
  int nf[3], nbin[3], bin[3], ms[3];
  int binoff;
  int invoff[3];
  int64_t gridoff, modeoff;
  int pointoff, npts;
};

template <typename T, int DIM>
__global__ void batch_keys_kernel(const T *__restrict__ x, const T *__restrict__ y,
                                  const T *__restrict__ z, int Mtot, const int *__restrict__ poff,
                                  int nprob, const DevProb *__restrict__ P, uint32_t binvol,
                                  uint32_t ex, uint32_t *__restrict__ keys) {
  // ex = 1: start-cell keys for odd kernel widths (the cell, or the next one
  // when the fraction is at least one half; bin + 1 values per dimension)
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < Mtot; j += gridDim.x * blockDim.x) {
    const DevProb &pr = P[find_slot(poff, nprob, j)];
    const T *xyz[3] = {x, y, z};
    uint32_t bin = 0, loc = 0, sb = 1, sl = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      int c;
      double f;
      fold_cell((double)xyz[d][j], AxisMap{0.0, 1.0, pr.nf[d], pr.bin[d]}, c, f);
      const int bc = c / pr.bin[d];
      bin += sb * (uint32_t)bc;
      loc += sl * ((uint32_t)(c - bc * pr.bin[d]) + (ex && f >= 0.5 ? 1u : 0u));
      sb *= (uint32_t)pr.nbin[d];
      sl *= (uint32_t)pr.bin[d] + ex;
    }
    keys[j] = ((uint32_t)pr.binoff + bin) * binvol + loc;
  }
}

template <typename T, int DIM>
__global__ void batch_local_kernel(const T *__restrict__ x, const T *__restrict__ y,
                                   const T *__restrict__ z, const int *__restrict__ perm, int Mtot,
                                   const int *__restrict__ poff, int nprob,
                                   const DevProb *__restrict__ P, T *__restrict__ l0,
                                   T *__restrict__ l1, T *__restrict__ l2) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Mtot; q += gridDim.x * blockDim.x) {
    const int j = perm[q];
    const DevProb &pr = P[find_slot(poff, nprob, j)];
    const T *xyz[3] = {x, y, z};
    T *out[3] = {l0, l1, l2};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      int c;
      double f;
      fold_cell((double)xyz[d][j], AxisMap{0.0, 1.0, pr.nf[d], pr.bin[d]}, c, f);
      out[d][q] = (T)((double)(c - (c / pr.bin[d]) * pr.bin[d]) + f);
    }
  }
}

__global__ void batch_binprob_kernel(const int *__restrict__ binoff, int nprob, int nbins,
                                     int *__restrict__ binprob) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x)
    binprob[b] = find_slot(binoff, nprob, b);
}

__device__ __forceinline__ int mode_of_pos(int i, int m, int modeord) {
  return modeord == 0 ? i - m / 2 : (i < m - m / 2 ? i : i - m);
}
__device__ __forceinline__ int pos_of_mode(int k, int m, int modeord) {
  return modeord == 0 ? k + m / 2 : (k >= 0 ? k : k + m);
}

template <typename T, int DIM>
__global__ void batch_deconv_kernel(const cplx<T> *__restrict__ fw, cplx<T> *__restrict__ fk,
                                    int64_t nmodes_tot, const int64_t *__restrict__ moff,
                                    int nprob, const DevProb *__restrict__ P,
                                    const T *__restrict__ inv, int modeord) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nmodes_tot;
       q += (int64_t)gridDim.x * blockDim.x) {
    const DevProb &pr = P[find_slot(moff, nprob, q)];
    int64_t i = q - pr.modeoff;
    int64_t g = 0, stride = 1;
    T f = T(1);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int id = (int)(i % pr.ms[d]);
      i /= pr.ms[d];
      const int k = mode_of_pos(id, pr.ms[d], modeord);
      g += stride * (k >= 0 ? k : pr.nf[d] + k);
      stride *= pr.nf[d];
      f *= inv[pr.invoff[d] + (k >= 0 ? k : -k)];
    }
    const cplx<T> v = fw[pr.gridoff + g];
    cplx<T> r;
    r.x = v.x * f;
    r.y = v.y * f;
    fk[q] = r;
  }
}

// grid position -> problem through the grid-order table (grids are stored in
// cuFFT shape groups, not in problem order)
template <typename T, int DIM>
__global__ void batch_amplify_kernel(const cplx<T> *__restrict__ fk, cplx<T> *__restrict__ fw,
                                     int64_t ncell_tot, const int64_t *__restrict__ gstart,
                                     const int *__restrict__ gprob, int nprob,
                                     const DevProb *__restrict__ P, const T *__restrict__ inv,
                                     int modeord) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncell_tot;
       q += (int64_t)gridDim.x * blockDim.x) {
    const DevProb &pr = P[gprob[find_slot(gstart, nprob, q)]];
    int64_t g = q - pr.gridoff;
    int64_t i = 0, stride = 1;
    T f = T(1);
    bool in = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int gd = (int)(g % pr.nf[d]);
      g /= pr.nf[d];
      const int m = pr.ms[d];
      const int k = gd <= (m - 1) / 2 ? gd : (gd >= pr.nf[d] - m / 2 ? gd - pr.nf[d] : INT32_MIN);
      if (k == INT32_MIN) {
        in = false;
        break;
      }
      i += stride * pos_of_mode(k, m, modeord);
      stride *= m;
      f *= inv[pr.invoff[d] + (k >= 0 ? k : -k)];
    }
    cplx<T> r;
    r.x = T(0);
    r.y = T(0);
    if (in) {
      const cplx<T> v = fk[pr.modeoff + i];
      r.x = v.x * f;
      r.y = v.y * f;
    }
    fw[q] = r;
  }
}

} // namespace

template <typename T>
BatchPlan<T>::BatchPlan(int type_, int dim_, int nprob_, const int64_t *modes, int iflag_,
                        double tol_, const cufinufft_opts &opts_, const gbnufft_opts *ext_)
    : type(type_), dim(dim_), nprob(nprob_), iflag(iflag_ >= 0 ? 1 : -1), tol(tol_),
      opts(opts_) {
  if (ext_) ext = *ext_;
  else gbnufft_default_opts(&ext);
  if (dim < 1 || dim > 3) GBN_THROW(FINUFFT_ERR_DIM_NOTVALID, "dim");
  if (type != 1 && type != 2) GBN_THROW(FINUFFT_ERR_TYPE_NOTVALID, "batched types are 1 and 2");
  if (nprob < 1) GBN_THROW(FINUFFT_ERR_NTRANS_NOTVALID, "nprob");
  if (!modes) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "modes");
  DeviceScope ds(opts.gpu_device_id);
  stream = (cudaStream_t)opts.gpu_stream;
  if (opts.upsampfac == 0.0) opts.upsampfac = 2.0;
  const int form = plan_kernel_form(ext, opts);
  const KernelChoice kc =
      form == KERNEL_PSWF
          ? choose_kernel_pswf(tol, opts.upsampfac, dim, type, std::is_same_v<T, float>,
                               ext.kerformula, 0, 0, opts.debug)
          : choose_kernel(tol, opts.upsampfac, opts.gpu_kerevalmeth, std::is_same_v<T, float>,
                          0, opts.debug);
  build_kernel_shape<T>(make_kernel_fn(form, kc.ns, kc.beta), opts.gpu_kerevalmeth == 1, tol,
                        &K);
  probs.resize(nprob);
  int nfmax[3] = {1, 1, 1};
  for (int p = 0; p < nprob; ++p) {
    HostProb &h = probs[p];
    for (int d = 0; d < 3; ++d) {
      const int64_t m = d < dim ? modes[3 * p + d] : 1;
      if (m < 1 || m > (1 << 30)) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "modes");
      h.ms[d] = (int)m;
      // grids on the size ladder: the FFTs of problems with equal grid shapes
      // run as one batched cuFFT call, and thousands of distinct shapes would
      // be launch-bound (a finer grid at the same kernel width only lowers
      // the error)
      h.nf[d] = d < dim ? (int)ladder_grid_len(fine_grid_len(m, opts.upsampfac, K.ns)) : 1;
      nfmax[d] = std::max(nfmax[d], h.nf[d]);
    }
  }
  S = spread_setup<T>(dim, K.ns, nfmax, opts, ext, false);
  if (dim == 2 && S.cfg.variant != 1 && S.cfg.variant != 2 && S.method == 2)
    GBN_THROW(FINUFFT_ERR_INSUFFICIENT_SHMEM, "batched spreading needs the tiled kernel");
  if (S.method != 2) GBN_THROW(FINUFFT_ERR_INSUFFICIENT_SHMEM, "batched spreading needs tiles");
  if (dim == 3 && S.cfg.variant == 1) // the exclusive-warp tiles serve single problems only
    GBN_THROW(FINUFFT_ERR_INSUFFICIENT_SHMEM, "batched 3D spreading needs variant 0, 2 or 3");
  // group problems by fine-grid shape (one batched cuFFT plan per shape); grids
  // are laid out group by group
  std::map<std::array<int, 3>, std::vector<int>> shapes;
  for (int p = 0; p < nprob; ++p) shapes[{probs[p].nf[0], probs[p].nf[1], probs[p].nf[2]}].push_back(p);
  int64_t goff = 0;
  for (auto &kv : shapes) {
    Group g;
    g.nf = kv.first;
    g.count = (int)kv.second.size();
    g.offset = goff;
    const int64_t cells = (int64_t)g.nf[0] * g.nf[1] * g.nf[2];
    for (int p : kv.second) {
      probs[p].gridoff = goff;
      grid_order.push_back(p);
      grid_start.push_back(goff);
      goff += cells;
    }
    groups.push_back(g);
  }
  grid_total = goff;
  int64_t moff = 0;
  int binoff = 0;
  for (int p = 0; p < nprob; ++p) {
    HostProb &h = probs[p];
    h.modeoff = moff;
    moff += (int64_t)h.ms[0] * h.ms[1] * h.ms[2];
    for (int d = 0; d < 3; ++d)
      h.nbin[d] = d < dim ? (h.nf[d] + S.bins[d] - 1) / S.bins[d] : 1;
    h.binoff = binoff;
    binoff += h.nbin[0] * h.nbin[1] * h.nbin[2];
  }
  modes_total = moff;
  nbins_total = binoff;
  fw.resize((size_t)std::max<int64_t>(grid_total, 1));
  // 1/phihat per distinct grid length, shared by the problems that use it
  QuadNodes Qn;
  Qn.q = kernel_ft_nodes(make_kernel_fn(K.form, K.ns, (double)K.beta), 3.0, Qn.z, Qn.f);
  std::map<int, int> invat;
  int invlen = 0;
  for (int p = 0; p < nprob; ++p)
    for (int d = 0; d < dim; ++d)
      if (!invat.count(probs[p].nf[d])) {
        invat[probs[p].nf[d]] = invlen;
        invlen += probs[p].nf[d] / 2 + 1;
      }
  inv.resize((size_t)std::max(invlen, 1));
  for (auto &kv : invat) launch_inv_fseries<T>(kv.first, Qn, inv.p + kv.second, stream);
  for (int p = 0; p < nprob; ++p)
    for (int d = 0; d < 3; ++d) probs[p].invoff[d] = d < dim ? invat[probs[p].nf[d]] : 0;
  // cuFFT plans per shape group
  const cufftType ty = std::is_same_v<T, float> ? CUFFT_C2C : CUFFT_Z2Z;
  for (Group &g : groups) {
    long long n[3];
    for (int d = 0; d < dim; ++d) n[d] = g.nf[dim - 1 - d];
    const long long dist = (long long)g.nf[0] * g.nf[1] * g.nf[2];
    size_t work = 0;
    if (cufftCreate(&g.plan) != CUFFT_SUCCESS) GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "cufftCreate");
    g.have = true;
    if (cufftMakePlanMany64(g.plan, dim, n, nullptr, 1, dist, nullptr, 1, dist, ty, g.count,
                            &work) != CUFFT_SUCCESS)
      GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "cufftMakePlanMany64");
    cufftSetStream(g.plan, stream);
  }
  upload_tables(nullptr);
}

template <typename T> BatchPlan<T>::~BatchPlan() {
  try {
    DeviceScope ds(opts.gpu_device_id);
    for (Group &g : groups)
      if (g.have) cufftDestroy(g.plan);
  } catch (...) {
  }
}

template <typename T> void BatchPlan<T>::upload_tables(const int64_t *npts) {
  std::vector<DevProb> dp(nprob);
  std::vector<int> binoffs(nprob + 1), poff(nprob + 1, 0);
  std::vector<int64_t> moffs(nprob + 1);
  int64_t acc = 0;
  for (int p = 0; p < nprob; ++p) {
    const HostProb &h = probs[p];
    DevProb &d = dp[p];
    for (int k = 0; k < 3; ++k) {
      d.nf[k] = h.nf[k];
      d.nbin[k] = h.nbin[k];
      d.bin[k] = S.bins[k];
      d.ms[k] = h.ms[k];
      d.invoff[k] = h.invoff[k];
    }
    d.binoff = h.binoff;
    d.gridoff = h.gridoff;
    d.modeoff = h.modeoff;
    poff[p] = (int)acc;
    d.pointoff = (int)acc;
    d.npts = npts ? (int)npts[p] : 0;
    acc += npts ? npts[p] : 0;
    binoffs[p] = h.binoff;
    moffs[p] = h.modeoff;
  }
  poff[nprob] = (int)acc;
  binoffs[nprob] = nbins_total;
  moffs[nprob] = modes_total;
  std::vector<BatchProb> bp(nprob);
  for (int p = 0; p < nprob; ++p) {
    for (int k = 0; k < 3; ++k) {
      bp[p].nf[k] = probs[p].nf[k];
      bp[p].nbin[k] = probs[p].nbin[k];
    }
    bp[p].binoff = probs[p].binoff;
    bp[p].pad_ = 0;
    bp[p].gridoff = probs[p].gridoff;
  }
  d_prob.resize(nprob * sizeof(DevProb));
  d_bprob.resize(nprob);
  d_binoff.resize(nprob + 1);
  d_poff.resize(nprob + 1);
  d_moff.resize(nprob + 1);
  d_gstart.resize(nprob + 1);
  d_gprob.resize(nprob);
  std::vector<int64_t> gs(grid_start);
  gs.push_back(grid_total);
  GBN_CUDA(cudaMemcpyAsync(d_prob.p, dp.data(), nprob * sizeof(DevProb), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaMemcpyAsync(d_bprob.p, bp.data(), nprob * sizeof(BatchProb), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaMemcpyAsync(d_binoff.p, binoffs.data(), (nprob + 1) * sizeof(int), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaMemcpyAsync(d_poff.p, poff.data(), (nprob + 1) * sizeof(int), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaMemcpyAsync(d_moff.p, moffs.data(), (nprob + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaMemcpyAsync(d_gstart.p, gs.data(), (nprob + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaMemcpyAsync(d_gprob.p, grid_order.data(), nprob * sizeof(int), cudaMemcpyHostToDevice, stream));
  GBN_CUDA(cudaStreamSynchronize(stream)); // host vectors go out of scope
}

template <typename T>
void BatchPlan<T>::setpts(const int64_t *npts, const T *x, const T *y, const T *z) {
  DeviceScope ds(opts.gpu_device_id);
  if (!npts) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "point counts");
  int64_t tot = 0;
  for (int p = 0; p < nprob; ++p) {
    if (npts[p] < 0) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "M");
    tot += npts[p];
  }
  if (tot > std::numeric_limits<int32_t>::max()) GBN_THROW(FINUFFT_ERR_NDATA_NOTVALID, "M total");
  if (tot > 0 && (!x || (dim > 1 && !y) || (dim > 2 && !z)))
    GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "null coordinates");
  Mtot = (int)tot;
  upload_tables(npts);
  // odd kernel widths sort by the support's start cell when the keys fit
  uint64_t binvol = (uint64_t)S.bins[0] * S.bins[1] * S.bins[2], sbinvol = 1;
  for (int d = 0; d < dim; ++d) sbinvol *= (uint64_t)S.bins[d] + 1;
  const uint32_t ex = K.ns % 2 == 1 && (uint64_t)nbins_total * sbinvol <= 0xffffffffull ? 1u : 0u;
  if (ex) binvol = sbinvol;
  const uint64_t nkeys = (uint64_t)nbins_total * binvol;
  if (nkeys > 0xffffffffull) GBN_THROW(FINUFFT_ERR_MAXNALLOC, "batch too large for 32-bit keys");
  int keybits = 0;
  while ((1ull << keybits) < nkeys) ++keybits;
  perm.resize((size_t)std::max(Mtot, 1));
  for (int d = 0; d < dim; ++d) loc[d].resize((size_t)std::max(Mtot, 1));
  AsyncBuf keys((size_t)std::max(Mtot, 1) * 4, stream), skeys((size_t)std::max(Mtot, 1) * 4, stream);
  const DevProb *P = reinterpret_cast<const DevProb *>(d_prob.p);
  const T *ys = dim > 1 ? y : x, *zs = dim > 2 ? z : x;
  if (Mtot > 0) {
    const unsigned g = blocks_for(Mtot, 256);
    if (dim == 1) batch_keys_kernel<T, 1><<<g, 256, 0, stream>>>(x, ys, zs, Mtot, d_poff.p, nprob, P, (uint32_t)binvol, ex, keys.as<uint32_t>());
    else if (dim == 2) batch_keys_kernel<T, 2><<<g, 256, 0, stream>>>(x, ys, zs, Mtot, d_poff.p, nprob, P, (uint32_t)binvol, ex, keys.as<uint32_t>());
    else batch_keys_kernel<T, 3><<<g, 256, 0, stream>>>(x, ys, zs, Mtot, d_poff.p, nprob, P, (uint32_t)binvol, ex, keys.as<uint32_t>());
    GBN_LAUNCH_CHECK();
    stable_sort_by_bin(keys.as<uint32_t>(), Mtot, keybits, skeys.as<uint32_t>(), perm.p, stream);
    T *l0 = loc[0].p, *l1 = dim > 1 ? loc[1].p : l0, *l2 = dim > 2 ? loc[2].p : l0;
    if (dim == 1) batch_local_kernel<T, 1><<<g, 256, 0, stream>>>(x, ys, zs, perm.p, Mtot, d_poff.p, nprob, P, l0, l1, l2);
    else if (dim == 2) batch_local_kernel<T, 2><<<g, 256, 0, stream>>>(x, ys, zs, perm.p, Mtot, d_poff.p, nprob, P, l0, l1, l2);
    else batch_local_kernel<T, 3><<<g, 256, 0, stream>>>(x, ys, zs, perm.p, Mtot, d_poff.p, nprob, P, l0, l1, l2);
    GBN_LAUNCH_CHECK();
  }
  binprob.resize((size_t)std::max(nbins_total, 1));
  batch_binprob_kernel<<<blocks_for(nbins_total, 256), 256, 0, stream>>>(d_binoff.p, nprob, nbins_total, binprob.p);
  GBN_LAUNCH_CHECK();
  SubproblemArrays sa;
  nsub = build_subproblems(skeys.as<uint32_t>(), Mtot, nbins_total, (uint32_t)binvol,
                           S.maxsub, &sa, stream);
  sub_bin.release();
  sub_start.release();
  sub_count.release();
  sub_bin.p = sa.bin;
  sub_start.p = sa.start;
  sub_count.p = sa.count;
  sub_bin.n = sub_start.n = sub_count.n = (size_t)std::max(nsub, 1);
  pts_set = true;
}

template <typename T> PointLayout<T> BatchPlan<T>::layout() const {
  PointLayout<T> L;
  L.dim = dim;
  for (int d = 0; d < 3; ++d) {
    L.nf[d] = 1;
    L.bin[d] = S.bins[d];
    L.nbin[d] = 1;
    L.loc[d] = loc[d].p ? loc[d].p : loc[0].p;
  }
  L.M = Mtot;
  L.nsub = nsub;
  L.sub_bin = sub_bin.p;
  L.sub_start = sub_start.p;
  L.sub_count = sub_count.p;
  L.perm = perm.p;
  L.probs = d_bprob.p;
  L.binprob = binprob.p;
  L.cell_sorted = 1;
  return L;
}

template <typename T> void BatchPlan<T>::execute(cplx<T> *c, cplx<T> *fk) {
  DeviceScope ds(opts.gpu_device_id);
  if (!pts_set) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "setpts first");
  const PointLayout<T> L = layout();
  const DevProb *P = reinterpret_cast<const DevProb *>(d_prob.p);
  const int dir = iflag > 0 ? CUFFT_INVERSE : CUFFT_FORWARD;
  auto fft_all = [&]() {
    for (const Group &g : groups) {
      cufftResult r;
      if constexpr (std::is_same_v<T, float>)
        r = cufftExecC2C(g.plan, (cufftComplex *)(fw.p + g.offset),
                         (cufftComplex *)(fw.p + g.offset), dir);
      else
        r = cufftExecZ2Z(g.plan, (cufftDoubleComplex *)(fw.p + g.offset),
                         (cufftDoubleComplex *)(fw.p + g.offset), dir);
      if (r != CUFFT_SUCCESS) GBN_THROW(FINUFFT_ERR_CUDA_FAILURE, "cufftExec");
    }
  };
  if (type == 1) {
    GBN_CUDA(cudaMemsetAsync(fw.p, 0, (size_t)grid_total * sizeof(cplx<T>), stream));
    launch_spread<T>(L, K, c, nullptr, 0, fw.p, grid_total, 1, S.cfg, stream);
    fft_all();
    const unsigned g = blocks_for(modes_total, 256);
    if (dim == 1) batch_deconv_kernel<T, 1><<<g, 256, 0, stream>>>(fw.p, fk, modes_total, d_moff.p, nprob, P, inv.p, opts.modeord);
    else if (dim == 2) batch_deconv_kernel<T, 2><<<g, 256, 0, stream>>>(fw.p, fk, modes_total, d_moff.p, nprob, P, inv.p, opts.modeord);
    else batch_deconv_kernel<T, 3><<<g, 256, 0, stream>>>(fw.p, fk, modes_total, d_moff.p, nprob, P, inv.p, opts.modeord);
    GBN_LAUNCH_CHECK();
  } else {
    const unsigned g = blocks_for(grid_total, 256);
    if (dim == 1) batch_amplify_kernel<T, 1><<<g, 256, 0, stream>>>(fk, fw.p, grid_total, d_gstart.p, d_gprob.p, nprob, P, inv.p, opts.modeord);
    else if (dim == 2) batch_amplify_kernel<T, 2><<<g, 256, 0, stream>>>(fk, fw.p, grid_total, d_gstart.p, d_gprob.p, nprob, P, inv.p, opts.modeord);
    else batch_amplify_kernel<T, 3><<<g, 256, 0, stream>>>(fk, fw.p, grid_total, d_gstart.p, d_gprob.p, nprob, P, inv.p, opts.modeord);
    GBN_LAUNCH_CHECK();
    fft_all();
    launch_interp<T>(L, K, fw.p, grid_total, nullptr, 0, c, 1, stream);
  }
  GBN_LAUNCH_CHECK();
}

template class BatchPlan<float>;
template class BatchPlan<double>;

} // namespace gbn

// ------------------------------------------------------------------ C ABI ----
namespace {
template <class F> int guarded_b(F &&f) {
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
} // namespace

#define GBN_BATCH_DEFS(P, PLAN, T, C)                                                         \
  int P##_batch_makeplan(int type, int dim, int nprob, const int64_t *n_modes, int iflag,    \
                         T eps, PLAN *plan, const cufinufft_opts *opts,                      \
                         const gbnufft_opts *ext) {                                           \
    return guarded_b([&] {                                                                    \
      if (!plan) GBN_THROW(FINUFFT_ERR_INVALID_ARGUMENT, "plan");                             \
      cufinufft_opts o;                                                                       \
      if (opts) o = *opts;                                                                    \
      else cufinufft_default_opts(&o);                                                        \
      *plan = (PLAN) new gbn::BatchPlan<T>(type, dim, nprob, n_modes, iflag, (double)eps, o,  \
                                           ext);                                              \
    });                                                                                       \
  }                                                                                           \
  int P##_batch_setpts(PLAN plan, const int64_t *M, const T *x, const T *y, const T *z) {     \
    return guarded_b([&] {                                                                    \
      if (!plan) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "plan");                                \
      ((gbn::BatchPlan<T> *)plan)->setpts(M, x, y, z);                                        \
    });                                                                                       \
  }                                                                                           \
  int P##_batch_execute(PLAN plan, C *c, C *fk) {                                             \
    return guarded_b([&] {                                                                    \
      if (!plan) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "plan");                                \
      ((gbn::BatchPlan<T> *)plan)->execute((gbn::cplx<T> *)c, (gbn::cplx<T> *)fk);            \
    });                                                                                       \
  }                                                                                           \
  int P##_batch_destroy(PLAN plan) {                                                          \
    return guarded_b([&] {                                                                    \
      if (!plan) GBN_THROW(FINUFFT_ERR_PLAN_NOTVALID, "plan");                                \
      delete (gbn::BatchPlan<T> *)plan;                                                       \
    });                                                                                       \
  }

extern "C" {
GBN_BATCH_DEFS(cufinufft, cufinufft_batch_plan, double, cuDoubleComplex)
GBN_BATCH_DEFS(cufinufftf, cufinufftf_batch_plan, float, cuFloatComplex)
}
