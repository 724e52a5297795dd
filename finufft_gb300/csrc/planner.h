// Learned planner and autotuner: the candidate plan shapes a plan may take at
// setpts (upsampling factor, bins, subproblem size, spread variant), point
// features computed on the device, and a 2x64 multilayer perceptron that
// predicts each candidate's execute time from those features (inference and
// training in hand-written CUDA kernels).
//
// The reference decides these by fixed rules: sigma at makeplan
// (src/cuda/makeplan.cu:289-329) and bins from the shared-memory budget
// (src/cuda/heuristics.cu:325-445); that heuristic is the fallback here.
#pragma once
#include <cstdint>

#include "common.h"
#include "device_util.cuh"

namespace gbn {

constexpr int PLANNER_NF = 12; // input features
constexpr int PLANNER_F_BATCH = 6; // feature: log2 of the transforms per batch
constexpr int PLANNER_H = 64;  // width of each of the two hidden layers
constexpr int PLANNER_K = 12;  // candidate slots (outputs)
// parameters: W1[H][NF] b1[H] W2[H][H] b2[H] W3[K][H] b3[K]
constexpr int PLANNER_OFF_W1 = 0;
constexpr int PLANNER_OFF_B1 = PLANNER_OFF_W1 + PLANNER_H * PLANNER_NF;
constexpr int PLANNER_OFF_W2 = PLANNER_OFF_B1 + PLANNER_H;
constexpr int PLANNER_OFF_B2 = PLANNER_OFF_W2 + PLANNER_H * PLANNER_H;
constexpr int PLANNER_OFF_W3 = PLANNER_OFF_B2 + PLANNER_H;
constexpr int PLANNER_OFF_B3 = PLANNER_OFF_W3 + PLANNER_K * PLANNER_H;
constexpr int PLANNER_NW = PLANNER_OFF_B3 + PLANNER_K;

// One candidate plan shape. reference = 1: the reference library's heuristic
// (its bins, per-point atomics, 1024-point subproblems) at this sigma.
struct Candidate {
  double sigma;
  int bins[3];
  int maxsub;
  int variant; // -1: the engine's choice for the width
  int reference;
};

// Candidate slot k (0..PLANNER_K-1) for a dimension (2 or 3) and precision.
// Returns false for an unused slot. Slots are (sigma index) * 4 + shape.
bool planner_candidate(int dim, bool dbl, int k, Candidate *c);

// Tolerance the kernel of width ns reaches at upsampling factor sigma (the
// CPU library's aliasing law tolfac * exp(-pi (ns-1) sqrt(1 - 1/sigma)),
// src/common/kernel.cpp:60-95): a candidate whose width had to be clipped
// below the law's width for tol is rejected.
double kernel_tol_bound(int ns, double sigma, int dim, int type);
// Whether a plan of this type/dimension/precision at tol may take candidate c
// (the analytic rejection of the learned planner and the autotuner).
bool planner_candidate_valid(const Candidate &c, int type, int dim, bool dbl, double tol);

// Raw features of a problem (see planner.cu for the list); the occupancy
// statistics come from a coarse histogram of (a strided sample of) the points,
// built on the device. u_d = (x_d - shift_d) * scale_d is wrapped into [0,1).
template <typename T>
void point_features(int dim, int type, bool dbl, int64_t M, const T *const xyz[3],
                    const double shift[3], const double scale[3], double nmodes_or_targets,
                    double tol, int ntr, double xs_product, float feat[PLANNER_NF],
                    cudaStream_t s);

// MLP on device buffers: y[n][K] = f(x[n][NF]) for weights w[PLANNER_NW]
// (x already standardised; y in standardised log-time units).
void mlp_forward(const float *w, int n, const float *x, float *y, cudaStream_t s);

// Trains w (in place, host arrays) on n samples with the masked squared error
// of the K outputs, minibatch Adam; loss[e] = mean masked loss after epoch e.
void mlp_train(int n, const float *x, const float *t, const float *mask, int epochs,
               int batch, float lr, float weight_decay, unsigned seed, float *w, float *loss);

// The trained planner compiled into the library: standardisation of the
// features, the training range, and the weights (false when none is compiled).
struct PlannerModel {
  bool trained;
  const float *mean, *stdev, *lo, *hi; // PLANNER_NF each
  float ymean, ystd;
};
const PlannerModel &planner_model();
// The compiled weights copied to a host array of PLANNER_NW floats.
void planner_weights_host(float *w);

// Standardised features -> predicted execute time (ms) of each slot, on the
// device with the compiled weights. Returns false when no model is compiled
// or a feature lies outside the training range (the caller then falls back
// to the reference heuristic).
bool planner_predict(const float feat[PLANNER_NF], double ms_out[PLANNER_K], cudaStream_t s);
// The learned planner leaves the engine's default slot (0) only for a slot
// predicted this much faster: on the held-out sweeps this keeps the mean
// picked time (1.053x the fastest slot) and cuts the picks measured more than
// 2% slower than slot 0 from 99 to 60 of 703.
constexpr double PLANNER_KEEP_DEFAULT = 1.037;

} // namespace gbn
