// Batched execution of many independent transforms with different sizes.
#pragma once
#include <cufft.h>

#include <array>
#include <limits>
#include <vector>

#include "cufinufft.h"
#include "gbnufft_ext.h"
#include "plan.h"

namespace gbn {

template <typename T> class BatchPlan {
public:
  BatchPlan(int type, int dim, int nprob, const int64_t *modes, int iflag, double tol,
            const cufinufft_opts &opts, const gbnufft_opts *ext);
  ~BatchPlan();
  void setpts(const int64_t *npts, const T *x, const T *y, const T *z);
  void execute(cplx<T> *c, cplx<T> *fk);

  struct HostProb {
    int ms[3], nf[3], nbin[3], invoff[3];
    int binoff;
    int64_t gridoff, modeoff;
  };
  struct Group {
    std::array<int, 3> nf;
    int count = 0;
    int64_t offset = 0;
    cufftHandle plan = 0;
    bool have = false;
  };
  int type, dim, nprob, iflag;
  double tol;
  cufinufft_opts opts;
  gbnufft_opts ext;
  cudaStream_t stream = nullptr;
  KernelShape<T> K;
  SpreadSetup S;
  std::vector<HostProb> probs;
  std::vector<Group> groups;
  std::vector<int> grid_order;
  std::vector<int64_t> grid_start;
  int64_t grid_total = 0, modes_total = 0;
  int nbins_total = 0, Mtot = 0, nsub = 0;
  bool pts_set = false;

private:
  PointLayout<T> layout() const;
  void upload_tables(const int64_t *npts);
  DevArray<cplx<T>> fw;
  DevArray<T> inv;
  DevArray<unsigned char> d_prob;
  DevArray<BatchProb> d_bprob;
  DevArray<int> d_binoff, d_poff, d_gprob, binprob, perm, sub_bin, sub_start, sub_count;
  DevArray<int64_t> d_moff, d_gstart;
  DevArray<T> loc[3];
};

} // namespace gbn
