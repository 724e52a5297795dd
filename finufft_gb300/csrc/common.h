// Shared definitions for the GB300 NUFFT engine: complex types, error
// propagation and the plain-old-data structs that kernels receive by value.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <type_traits>

#include "finufft_errors.h"

namespace gbn {

constexpr int MAX_NS = 16;       // widest kernel (double precision)
constexpr int MAX_NS_FLOAT = 12; // widest kernel in single precision
constexpr int MAX_HCOEF = 24;    // max coefficients of one Horner piece
constexpr int MAX_NQUAD = 100;   // max Gauss-Legendre nodes for kernel transforms
constexpr double PI = 3.141592653589793238462643383279502884;
constexpr double INV_2PI = 0.159154943091895335768883763372514362;

template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };
template <typename T> using cplx = typename cplx_t<T>::type;

// Number of Horner coefficients used for kernel width ns: pieces are fitted
// with at most this many and zero-padded at the high-degree end, so the
// evaluation loop has a compile-time trip count.
__host__ __device__ constexpr int horner_len(int ns) {
  return ns + 6 < MAX_HCOEF ? ns + 6 : MAX_HCOEF;
}

// Exception carrying a FINUFFT error code; caught at the C-ABI boundary.
struct Error {
  int code;
  const char *msg;
};

#define GBN_THROW(code_, msg_) throw ::gbn::Error{(code_), (msg_)}
#define GBN_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      cudaGetLastError(); /* clear a non-sticky error so it does not leak to the caller */ \
      fprintf(stderr, "[gbnufft] CUDA error %s at %s:%d\n", cudaGetErrorString(e_),      \
              __FILE__, __LINE__);                                                       \
      throw ::gbn::Error{FINUFFT_ERR_CUDA_FAILURE, cudaGetErrorString(e_)};              \
    }                                                                                    \
  } while (0)
#define GBN_LAUNCH_CHECK() GBN_CUDA(cudaGetLastError())

// Kernel forms: the GPU library's ES ("exponential of semicircle") kernel
// phi(x) = exp(beta*(sqrt(1-(2x/ns)^2)-1)) and the CPU library's prolate
// spheroidal wave function phi(x) = psi_0^beta(2x/ns), both on |x| < ns/2.
enum { KERNEL_ES = 1, KERNEL_PSWF = 2 };

// The spreading kernel and its piecewise-polynomial (Horner) form: piece j covers
// x in [-ns/2+j, -ns/2+j+1], written as a polynomial in u = 2*(x - piece start) - 1.
// coef[k][j] is the coefficient of u^(ndeg-1-k) of piece j (highest degree first).
template <typename T> struct KernelShape {
  int ns;
  int use_horner; // 1: Horner pieces, 0: direct exp(sqrt())
  int ncoef;      // number of Horner coefficients per piece
  int form;       // KERNEL_ES or KERNEL_PSWF (PSWF: always Horner)
  T beta;
  T es_c; // (2/ns)^2
  T coef[MAX_HCOEF][MAX_NS];
};

// Where the nonuniform points sit after the device bin sort, and how the
// fine grid is tiled. Passed by value to spread/interp kernels.
// One problem of a batch of independent transforms (batched execution): its
// fine grid, bin counts, first global bin and grid offset.
struct BatchProb {
  int nf[3];
  int nbin[3];
  int binoff;   // first global bin of this problem
  int pad_;
  int64_t gridoff; // offset of its fine grid in the batch's grid array
};

template <typename T> struct PointLayout {
  int dim;
  int nf[3];       // fine grid size per dimension
  int bin[3];      // bin (tile interior) size per dimension
  int nbin[3];     // number of bins per dimension
  int M;           // number of points
  int nsub;        // number of subproblems
  const int *sub_bin;   // subproblem -> bin index (x fastest)
  const int *sub_start; // subproblem -> first sorted point
  const int *sub_count; // subproblem -> number of points
  const int *perm;      // sorted position -> user index
  const T *loc[3];      // sorted bin-local coordinates in grid units, [0, bin]
  // batched execution: subproblem bins are global; binprob maps them to
  // problems, whose grids and bin counts replace nf/nbin above (null otherwise)
  const BatchProb *probs = nullptr;
  const int *binprob = nullptr;
  // 1 when points inside a bin are also sorted by cell (x fastest, z slowest)
  int cell_sorted = 0;
  // interpolation: when set (cplx<T>[ntr * M]), the tiled interpolation writes
  // its results in sorted order here and a gather pass per transform moves
  // them to user order through iperm (the inverse of perm): coalesced writes,
  // and the random reads of one transform's results hit L2
  void *sorted_out = nullptr;
  const int *iperm = nullptr;
  // interpolation schedule: 0 auto, 1 gather per point, 2 shared-memory tiles
  int interp_mode = 0;
};

} // namespace gbn
