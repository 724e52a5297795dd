/* Extensions of the GB300 NUFFT engine. None of these has a counterpart in
 * the reference C API; existing cufinufft/finufft callers never need them.
 * They expose the adjoint on device pointers, plan introspection, per-stage
 * timing and CUDA-graph replay of execute.
 */
#ifndef GBNUFFT_EXT_H
#define GBNUFFT_EXT_H

#include <stddef.h>
#include <stdint.h>
#include "cufinufft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Planning options beyond cufinufft_opts (which must keep the reference's
 * layout). Pass to cufinufft[f]_makeplan_ext; NULL means the defaults of
 * gbnufft_default_opts. */
typedef struct gbnufft_opts {
  int planner;        /* 0: this engine's defaults; 1: the reference library's heuristic
                         (cuFINUFFT 2.6 bin sizes, method and subproblem size,
                         src/cuda/heuristics.cu:325-445); 2: learned: at setpts a 2x64
                         MLP predicts the execute time of each candidate shape
                         (upsampling factor, bins, subproblem size, spread variant)
                         from features of the points and the plan keeps the fastest
                         candidate whose kernel reaches tol (no trained model, or
                         features outside its training range: planner 1's shape);
                         3: autotuned: at setpts every candidate is timed on a sample
                         of the points (cached per problem class). 2D and 3D types
                         1, 2, 3; 1D takes planner 0 */
  int spread_variant; /* -1 auto; tiled spread: 0 shared tile with per-point
                         atomics, 1 one warp per tile (no atomics, same-cell runs in
                         registers), 2 shared tile with same-cell register runs,
                         3 (3D) as 2 with x-slack runs and vector staging (ns <= 8),
                         4 (3D double precision, the default for ns >= 6) an int64
                         fixed-point tile with integer products, one thread per
                         support row summing runs of points in registers */
  int fft_prune;      /* 1: 2D/3D FFTs as a 1D pass along x plus passes over the other
                         dimensions on the x columns of the retained modes only
                         (measured slower than one cuFFT plan on GB300; default 0) */
  int spread_float_tile; /* 1: the 3D single-precision spread (variant 3) sums into a
                         float tile with float atomics; 0 (default): for ns <= 6 it sums
                         into an int32 fixed-point tile scaled per subproblem by the sum
                         of its |c_j| (native integer adds; each flushed value rounded
                         once to that sum times 2^-30); 2: the fixed-point tile for ns 7
                         and 8 too, faster but less accurate there (1e8 clustered points:
                         tol 1e-6 error 1.5e-6 -> 2.2e-6, tol 1.2e-7 4.2e-7 -> 2.1e-6) */
  int kernel_form;    /* 0 auto: the CPU library's PSWF kernel (psi_0, width and shape of
                         src/common/kernel.cpp:79-146, never narrower than the GPU rule)
                         fitted by Horner pieces, except under planner 1 or
                         gpu_kerevalmeth 0, which keep the GPU library's ES kernel;
                         1: ES (src/cuda/makeplan.cu:43-119); 2: PSWF */
  int kerformula;     /* PSWF shape parameter choice as finufft_opts.spread_kerformula:
                         0 or 8 (default), 7, 9; other values are rejected */
  int sort_keys;      /* 0 (default): points sorted by bin and, inside the bin, by the
                         first cell of their kernel support; 1: by bin and cell;
                         2: by bin only, points of a bin in input order (the
                         reference's bin ordering; fewer same-cell runs) */
  int interp_mode;    /* type 2 interpolation: 0 auto (3 where its boxes fit, else 2, and
                         batches may write sorted order and scatter it per transform);
                         1 one thread per point gathering from the grid; 2 tiles loaded
                         into shared memory by the block's threads, user order written
                         directly; 3 tiles copied by the tensor memory accelerator
                         (bulk tensor copies, two buffers: the next transform's tile
                         loads while the current one is interpolated) */
  int batch_cap;      /* 0 (default): 3D type-2 plans run at most as many transforms
                         per batch as keep their fine grids within half of L2 (the
                         interpolation tiles re-read their halos); other plans
                         batch gpu_maxbatchsize transforms; 1: gpu_maxbatchsize as
                         given everywhere */
  int reserved[7];
} gbnufft_opts;

typedef struct gbnufft_plan_info {
  int type, dim, ntransf, batchsize;
  int ns;              /* kernel width */
  double beta;         /* kernel shape parameter (ES beta or PSWF c) */
  double upsampfac;    /* sigma actually used */
  int nf[3];           /* fine grid (type 3: outer grid) */
  int bins[3];         /* bin size per dimension */
  int method;          /* 1 global atomics, 2 shared-memory tiles */
  int nsub;            /* subproblems after setpts */
  int64_t M, N;        /* points / targets after setpts */
  size_t spread_smem;  /* shared memory per spread block (method 2) */
  double horner_err;   /* max abs error of the fitted kernel pieces */
  int inner_nf[3];     /* type 3: fine grid of the inner type-2 plan */
  int spread_variant;  /* 3D tiled spread variant in use */
  int maxsubprobsize;  /* points per subproblem in use */
  int spread_fixed;    /* 1: the 3D spread sums into the int32 fixed-point tile */
  int kernel_form;     /* 1 ES, 2 PSWF */
  int planner_used;    /* planner whose shape is in use (2 and 3 fall back to 1) */
  int planned_slot;    /* planners 2/3: candidate slot chosen at setpts (-1: none) */
  float features[12];  /* planners 2/3: the problem's features at the last setpts */
  double tune_ms[12];  /* planner 3: estimated execute ms per slot (0: not timed) */
} gbnufft_plan_info;

GBNUFFT_EXPORT void gbnufft_default_opts(gbnufft_opts *o);

#define GBNUFFT_EXT_DECLS(P, PLAN, T, C)                                                   \
  /* makeplan with engine options (ext may be NULL)                                 */  \
  GBNUFFT_EXPORT int P##_makeplan_ext(int type, int dim, const int64_t *n_modes, int iflag, \
                                      int ntr, T eps, PLAN *plan,                        \
                                      const cufinufft_opts *opts,                        \
                                      const gbnufft_opts *ext);                          \
  /* Adjoint of the planned transform on device pointers (type 1 and 3: fk in,      */  \
  /* c out; type 2: c in, fk out), same semantics as finufft_execute_adjoint.       */  \
  GBNUFFT_EXPORT int P##_execute_adjoint(PLAN plan, C *d_c, C *d_fk);                    \
  GBNUFFT_EXPORT int P##_plan_info(PLAN plan, gbnufft_plan_info *info);                  \
  /* enable != 0 turns on CUDA-event timing of the stages of later executes;        */  \
  /* ms[0..3] = spread-or-interp, FFT, deconvolve-or-amplify, total of the last one */  \
  /* (type 3: total only, the other three are 0)                                    */  \
  GBNUFFT_EXPORT int P##_stage_times(PLAN plan, int enable, float ms[4]);                \
  /* Copies the device bin sort to host arrays: perm[M] (sorted position -> input   */  \
  /* index) and loc[dim*M] (bin-local coordinates, dimension-major).                */  \
  GBNUFFT_EXPORT int P##_get_sort(PLAN plan, int *perm, T *loc);                         \
  /* Captures execute(d_c, d_fk) into a CUDA graph on the plan's stream (which must */  \
  /* not be the legacy default stream); graph_launch replays it on that stream.     */  \
  GBNUFFT_EXPORT int P##_graph_capture(PLAN plan, C *d_c, C *d_fk);                      \
  GBNUFFT_EXPORT int P##_graph_launch(PLAN plan);

GBNUFFT_EXT_DECLS(cufinufft, cufinufft_plan, double, cuDoubleComplex)
GBNUFFT_EXT_DECLS(cufinufftf, cufinufftf_plan, float, cuFloatComplex)

/* Uneven batches: nprob independent transforms of one type (1 or 2) and
 * dimension with different mode counts and point sets, executed by one sort,
 * one spread/interpolation launch over all problems, cuFFT batched over
 * problems of equal grid shape and one deconvolution launch. n_modes holds
 * 3 int64 per problem (x fastest; unused dimensions ignored). M holds the
 * point count of each problem (host array); x/y/z, c and fk are concatenated
 * device arrays in problem order (c: sum M strengths; fk: sum prod(n_modes)).
 * ext may be NULL. */
typedef struct cufinufft_batch_s *cufinufft_batch_plan;
typedef struct cufinufftf_batch_s *cufinufftf_batch_plan;
#define GBNUFFT_BATCH_DECLS(P, PLAN, T, C)                                                 \
  GBNUFFT_EXPORT int P##_batch_makeplan(int type, int dim, int nprob,                    \
                                        const int64_t *n_modes, int iflag, T eps,        \
                                        PLAN *plan, const cufinufft_opts *opts,          \
                                        const gbnufft_opts *ext);                        \
  GBNUFFT_EXPORT int P##_batch_setpts(PLAN plan, const int64_t *M, const T *d_x,         \
                                      const T *d_y, const T *d_z);                       \
  GBNUFFT_EXPORT int P##_batch_execute(PLAN plan, C *d_c, C *d_fk);                      \
  GBNUFFT_EXPORT int P##_batch_destroy(PLAN plan);
GBNUFFT_BATCH_DECLS(cufinufft, cufinufft_batch_plan, double, cuDoubleComplex)
GBNUFFT_BATCH_DECLS(cufinufftf, cufinufftf_batch_plan, float, cuFloatComplex)

/* Host-only planning queries (no device work). kernel_choice: the kernel
 * width ns and shape parameter beta a plan of this type and dimension picks at
 * tol and upsampling factor sigma, for form 1 (the GPU library's ES rule,
 * src/cuda/makeplan.cu:43-119) or 2 (the CPU library's PSWF,
 * src/common/kernel.cpp:79-146, never narrower than the GPU rule).
 * kernel_eval: the kernel's values at n offsets x (grid units; support
 * |x| <= ns/2), ES exp(beta (sqrt(1 - (2x/ns)^2) - 1)) or PSWF
 * psi_0^beta(2x/ns) / psi_0^beta(0), as the Horner pieces are fitted to. */
GBNUFFT_EXPORT int gbnufft_kernel_choice(double tol, double sigma, int dim, int type,
                                         int is_float, int form, int kerformula, int *ns,
                                         double *beta);
GBNUFFT_EXPORT int gbnufft_kernel_eval(int form, int ns, double beta, int64_t n,
                                       const double *x, double *out);

/* The learned planner (no counterpart in the reference, whose heuristic is
 * src/cuda/heuristics.cu:325-445). Sizes: features, hidden width (two hidden
 * layers), candidate slots, weights (W1[H][NF] b1 W2[H][H] b2 W3[K][H] b3).
 * planner_candidate: the shape of slot k for a dimension and precision
 * (reference = 1: the reference heuristic's shape at that sigma);
 * FINUFFT_ERR_INVALID_ARGUMENT for an unused slot. planner_model: the model
 * compiled into the library (trained = 0: none; weights of nweights floats;
 * feature standardisation mean/stdev and training range lo/hi of nfeat floats;
 * output standardisation of log10 ms). planner_forward: the MLP's CUDA forward
 * pass on device arrays x[n][nfeat] -> y[n][nslots]. planner_train: minibatch
 * Adam on the masked squared error with the CUDA training kernels, host arrays,
 * w updated in place, loss[epochs]. point_features: the features of a point set
 * (device coordinates; u = (x - shift) * scale wrapped into [0,1) for the
 * occupancy histogram). */
GBNUFFT_EXPORT int gbnufft_planner_dims(int *nfeat, int *hidden, int *nslots, int *nweights);
GBNUFFT_EXPORT int gbnufft_planner_candidate(int dim, int is_double, int slot, double *sigma,
                                             int *bins, int *maxsub, int *variant,
                                             int *reference);
/* planner_valid: whether a plan of this type, dimension, precision and tol may
 * take slot k (its kernel width at the slot's sigma fits unclipped; single
 * precision takes sigma < 2 only at tol >= 1e-5). */
GBNUFFT_EXPORT int gbnufft_planner_valid(int type, int dim, int is_double, double tol, int slot,
                                         int *valid);
GBNUFFT_EXPORT int gbnufft_planner_model(int *trained, float *weights, float *mean,
                                         float *stdev, float *lo, float *hi, float *ymean,
                                         float *ystd);
GBNUFFT_EXPORT int gbnufft_planner_forward(const float *d_weights, int n, const float *d_x,
                                           float *d_y, void *stream);
GBNUFFT_EXPORT int gbnufft_planner_train(int n, const float *x, const float *t,
                                         const float *mask, int epochs, int batch, float lr,
                                         float weight_decay, unsigned seed, float *w,
                                         float *loss);
GBNUFFT_EXPORT int gbnufft_point_features(int dim, int type, int is_double, int64_t M,
                                          const void *d_x, const void *d_y, const void *d_z,
                                          const double *shift, const double *scale,
                                          double nmodes, double tol, int ntr,
                                          double xs_product, float *feat, void *stream);

/* Reads and clears the device's error word: nonzero when a kernel's bounded
 * wait gave up (a bulk tensor copy of the interpolation tiles that did not
 * complete); that launch's outputs are then incomplete. 0 or a FINUFFT_ERR_*. */
GBNUFFT_EXPORT int gbnufft_device_error(int device, int *code);

/* Measures the device's conflict-free shared-memory f32 atomicAdd rate
 * (lane operations per second), the peak the spreading kernels are held to. */
GBNUFFT_EXPORT int gbnufft_smem_atomic_rate(int device, double *rate);
/* The same for native int32 shared-memory atomicAdd (the fixed-point tile's
 * operation). */
GBNUFFT_EXPORT int gbnufft_smem_atomic_rate_i32(int device, double *rate);

/* Spread-only type 1 without device allocation (no counterpart in the
 * reference): grid[g] = sum_j c[j] phi(g - x_j) on the periodic grid of
 * n_grid[0..dim) cells (x fastest), the same result as a cufinufftf plan of
 * type 1 with gpu_spreadinterponly = 1 and default options. For callers that
 * may not allocate device memory (a foreign allocator owns the GPU, or all
 * memory is reserved at start-up): every intermediate lives in a fixed 32 MiB
 * scratch array compiled into the library, which each GPU that loads the
 * library holds until exit. Limits: M <= 2^19 points, at most 2^24 grid cells;
 * larger inputs return FINUFFT_ERR_MAXNALLOC. The first call on a device looks
 * up the scratch address on that device; make that first call before any
 * stream capture. Calls share the scratch, so calls that overlap on the GPU
 * race: order them on one stream. Blocks the host until the bin sort is done,
 * as setpts does. All pointers are device pointers; stream may be NULL. */
GBNUFFT_EXPORT int cufinufftf_spread_noalloc(int dim, const int64_t *n_grid, int64_t M,
                                             const float *d_x, const float *d_y,
                                             const float *d_z, const cuFloatComplex *d_c,
                                             cuFloatComplex *d_grid, float eps, void *stream);

/* setpts takes its temporary buffers (sort keys, coordinate records, radix  */
/* sort storage) from a stream-ordered pool per device that keeps freed      */
/* memory for the next setpts. This returns that memory to the CUDA driver  */
/* for `device` (plans stay valid). 0 or a FINUFFT_ERR_* code.                */
GBNUFFT_EXPORT int gbnufft_trim_scratch(int device);

/* Library build identification string. */
GBNUFFT_EXPORT const char *gbnufft_version(void);

#ifdef __cplusplus
}
#endif
#endif
