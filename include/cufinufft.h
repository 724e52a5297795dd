/* Device-pointer NUFFT interface: a drop-in for libcufinufft.
 *
 * Every declaration here replaces the entry point of the same name in
 * flatironinstitute/finufft include/cufinufft.h (guru interface :15-37,
 * 36 simple interfaces :39-186; implemented upstream in
 * src/cuda/c_interface.cpp:33-470). Signatures, argument meaning, ownership
 * and return codes are the same, so code written against cufinufft links
 * against this library unchanged:
 *   - every data pointer is a caller-owned DEVICE pointer;
 *   - the plan keeps the x/y/z (and s/t/u) pointers given to setpts and reads
 *     them again in execute, so they must stay valid until destroy;
 *   - execute runs asynchronously on opts.gpu_stream;
 *   - returns 0 on success, else a FINUFFT_ERR_* code (finufft_errors.h).
 * Batched arrays are contiguous per transform: c + t*M, fk + t*prod(N).
 */
#ifndef GBNUFFT_CUFINUFFT_H
#define GBNUFFT_CUFINUFFT_H

#include <stdint.h>
#include <cuComplex.h>
#include "cufinufft_opts.h"
#include "finufft_errors.h"

#ifndef GBNUFFT_EXPORT
#define GBNUFFT_EXPORT __attribute__((visibility("default")))
#endif

typedef struct cufinufft_plan_s *cufinufft_plan;   /* double precision plan */
typedef struct cufinufft_fplan_s *cufinufftf_plan; /* single precision plan */

#ifdef __cplusplus
extern "C" {
#endif

/* reference: include/cufinufft.h:16 */
GBNUFFT_EXPORT void cufinufft_default_opts(cufinufft_opts *opts);

/* reference: include/cufinufft.h:18-23 */
GBNUFFT_EXPORT int cufinufft_makeplan(int type, int dim, const int64_t *n_modes, int iflag,
                                      int ntr, double eps, cufinufft_plan *d_plan_ptr,
                                      const cufinufft_opts *opts);
GBNUFFT_EXPORT int cufinufftf_makeplan(int type, int dim, const int64_t *n_modes, int iflag,
                                       int ntr, float eps, cufinufftf_plan *d_plan_ptr,
                                       const cufinufft_opts *opts);

/* reference: include/cufinufft.h:25-30 */
GBNUFFT_EXPORT int cufinufft_setpts(cufinufft_plan d_plan, int64_t M, const double *d_x,
                                    const double *d_y, const double *d_z, int N,
                                    const double *d_s, const double *d_t, const double *d_u);
GBNUFFT_EXPORT int cufinufftf_setpts(cufinufftf_plan d_plan, int64_t M, const float *d_x,
                                     const float *d_y, const float *d_z, int N,
                                     const float *d_s, const float *d_t, const float *d_u);

/* reference: include/cufinufft.h:32-35 */
GBNUFFT_EXPORT int cufinufft_execute(cufinufft_plan d_plan, cuDoubleComplex *d_c,
                                     cuDoubleComplex *d_fk);
GBNUFFT_EXPORT int cufinufftf_execute(cufinufftf_plan d_plan, cuFloatComplex *d_c,
                                      cuFloatComplex *d_fk);

/* reference: include/cufinufft.h:37-38 */
GBNUFFT_EXPORT int cufinufft_destroy(cufinufft_plan d_plan);
GBNUFFT_EXPORT int cufinufftf_destroy(cufinufftf_plan d_plan);

/* The 36 simple (one-shot) interfaces: 3 dims x 3 types x {single, many} x
 * {double, float}. Each makes a plan, sets points, executes and destroys.
 * reference: include/cufinufft.h:39-186. */
#define GBNUFFT_SIMPLE_DECLS(P, T, C)                                                        \
  GBNUFFT_EXPORT int P##1d1many(int n_transf, int64_t nj, const T *xj, const C *cj,          \
                                int iflag, T eps, int64_t ms, C *fk,                         \
                                const cufinufft_opts *opts);                                 \
  GBNUFFT_EXPORT int P##1d1(int64_t nj, const T *xj, const C *cj, int iflag, T eps,          \
                            int64_t ms, C *fk, const cufinufft_opts *opts);                  \
  GBNUFFT_EXPORT int P##1d2many(int n_transf, int64_t nj, const T *xj, C *cj, int iflag,     \
                                T eps, int64_t ms, const C *fk, const cufinufft_opts *opts); \
  GBNUFFT_EXPORT int P##1d2(int64_t nj, const T *xj, C *cj, int iflag, T eps, int64_t ms,    \
                            const C *fk, const cufinufft_opts *opts);                        \
  GBNUFFT_EXPORT int P##1d3many(int n_transf, int64_t nj, const T *xj, const C *cj,          \
                                int iflag, T eps, int64_t nk, const T *s, C *fk,             \
                                const cufinufft_opts *opts);                                 \
  GBNUFFT_EXPORT int P##1d3(int64_t nj, const T *xj, const C *cj, int iflag, T eps,          \
                            int64_t nk, const T *s, C *fk, const cufinufft_opts *opts);      \
  GBNUFFT_EXPORT int P##2d1many(int n_transf, int64_t nj, const T *xj, const T *yj,          \
                                const C *cj, int iflag, T eps, int64_t ms, int64_t mt,       \
                                C *fk, const cufinufft_opts *opts);                          \
  GBNUFFT_EXPORT int P##2d1(int64_t nj, const T *xj, const T *yj, const C *cj, int iflag,    \
                            T eps, int64_t ms, int64_t mt, C *fk,                            \
                            const cufinufft_opts *opts);                                     \
  GBNUFFT_EXPORT int P##2d2many(int n_transf, int64_t nj, const T *xj, const T *yj, C *cj,   \
                                int iflag, T eps, int64_t ms, int64_t mt, const C *fk,       \
                                const cufinufft_opts *opts);                                 \
  GBNUFFT_EXPORT int P##2d2(int64_t nj, const T *xj, const T *yj, C *cj, int iflag, T eps,   \
                            int64_t ms, int64_t mt, const C *fk,                             \
                            const cufinufft_opts *opts);                                     \
  GBNUFFT_EXPORT int P##2d3many(int n_transf, int64_t nj, const T *xj, const T *yj,          \
                                const C *cj, int iflag, T eps, int64_t nk, const T *s,       \
                                const T *t, C *fk, const cufinufft_opts *opts);              \
  GBNUFFT_EXPORT int P##2d3(int64_t nj, const T *xj, const T *yj, const C *cj, int iflag,    \
                            T eps, int64_t nk, const T *s, const T *t, C *fk,                \
                            const cufinufft_opts *opts);                                     \
  GBNUFFT_EXPORT int P##3d1many(int n_transf, int64_t nj, const T *xj, const T *yj,          \
                                const T *zj, const C *cj, int iflag, T eps, int64_t ms,      \
                                int64_t mt, int64_t mu, C *fk, const cufinufft_opts *opts);  \
  GBNUFFT_EXPORT int P##3d1(int64_t nj, const T *xj, const T *yj, const T *zj, const C *cj,  \
                            int iflag, T eps, int64_t ms, int64_t mt, int64_t mu, C *fk,     \
                            const cufinufft_opts *opts);                                     \
  GBNUFFT_EXPORT int P##3d2many(int n_transf, int64_t nj, const T *xj, const T *yj,          \
                                const T *zj, C *cj, int iflag, T eps, int64_t ms,            \
                                int64_t mt, int64_t mu, const C *fk,                         \
                                const cufinufft_opts *opts);                                 \
  GBNUFFT_EXPORT int P##3d2(int64_t nj, const T *xj, const T *yj, const T *zj, C *cj,        \
                            int iflag, T eps, int64_t ms, int64_t mt, int64_t mu,            \
                            const C *fk, const cufinufft_opts *opts);                        \
  GBNUFFT_EXPORT int P##3d3many(int n_transf, int64_t nj, const T *xj, const T *yj,          \
                                const T *zj, const C *cj, int iflag, T eps, int64_t nk,      \
                                const T *s, const T *t, const T *u, C *fk,                   \
                                const cufinufft_opts *opts);                                 \
  GBNUFFT_EXPORT int P##3d3(int64_t nj, const T *xj, const T *yj, const T *zj, const C *cj,  \
                            int iflag, T eps, int64_t nk, const T *s, const T *t,            \
                            const T *u, C *fk, const cufinufft_opts *opts);

GBNUFFT_SIMPLE_DECLS(cufinufft, double, cuDoubleComplex)
GBNUFFT_SIMPLE_DECLS(cufinufftf, float, cuFloatComplex)

#ifdef __cplusplus
}
#endif
#endif
