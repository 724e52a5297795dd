// Spread/interp kernels for dimension 1 (one translation unit per dimension
// keeps the per-width template instantiations compiling in parallel).
#include "spreadinterp_impl.cuh"

namespace gbn {
template void spread_dim<float, 1>(const PointLayout<float> &, const KernelShape<float> &,
                                      const float2 *, const float2 *, int, float2 *, int64_t,
                                      int, const SpreadConfig &, cudaStream_t);
template void spread_dim<double, 1>(const PointLayout<double> &, const KernelShape<double> &,
                                       const double2 *, const double2 *, int, double2 *,
                                       int64_t, int, const SpreadConfig &, cudaStream_t);
template void interp_dim<float, 1>(const PointLayout<float> &, const KernelShape<float> &,
                                      const float2 *, int64_t, const float2 *, int, float2 *,
                                      int, cudaStream_t);
template void interp_dim<double, 1>(const PointLayout<double> &, const KernelShape<double> &,
                                       const double2 *, int64_t, const double2 *, int,
                                       double2 *, int, cudaStream_t);
} // namespace gbn
