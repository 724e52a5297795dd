/* Host-pointer NUFFT interface: a drop-in for the FINUFFT C API.
 *
 * These entry points replace the ones of the same name in
 * flatironinstitute/finufft include/finufft/finufft_eitherprec.h
 * (guru interface :55-67, 18 simple interfaces per precision :69-140),
 * implemented upstream in src/c_interface.cpp. Arguments are HOST pointers,
 * exactly as in FINUFFT; this library stages them to the GPU (pinned
 * staging buffers, one plan-owned CUDA stream) and computes there, so a
 * program linked against FINUFFT can switch to the GB300 engine by relinking.
 * finufft_opts has the same field layout as FINUFFT's; fields that only make
 * sense for a CPU library (nthreads, fftw, FFTW lock functions...) are
 * accepted and ignored.
 */
#ifndef GBNUFFT_FINUFFT_H
#define GBNUFFT_FINUFFT_H

#include <stdint.h>
#include "finufft_errors.h"

#ifndef GBNUFFT_EXPORT
#define GBNUFFT_EXPORT __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
#include <complex>
#define GBNUFFT_CPX(T) std::complex<T>
extern "C" {
#else
#include <complex.h>
#define GBNUFFT_CPX(T) T _Complex
#endif

/* Same layout as FINUFFT's finufft_opts (include/finufft_opts.h:32-71). */
typedef struct finufft_opts {
  int modeord;            /* 0 CMCL order, 1 FFT order (types 1, 2) */
  int spreadinterponly;   /* 1: spread (type 1) or interpolate (type 2) only */
  int debug;
  int spread_debug;
  int showwarn;
  int nthreads;           /* ignored (GPU engine) */
  int fftw;               /* ignored */
  int spread_sort;        /* ignored: points are always bin-sorted on the device */
  int spread_kerevalmeth; /* deprecated upstream; ignored */
  int spread_kerpad;      /* deprecated upstream; ignored */
  double upsampfac;       /* sigma; 0.0 = auto */
  int spread_thread;      /* deprecated upstream; ignored */
  int maxbatchsize;       /* transforms per batch, 0 = auto */
  int spread_nthr_atomic; /* ignored */
  int spread_max_sp_size; /* if >0, max points per subproblem */
  int spread_kerformula;  /* ignored (this engine uses the ES kernel) */
  int allow_eps_too_small;
  void (*fftw_lock_fun)(void *);
  void (*fftw_unlock_fun)(void *);
  void *fftw_lock_data;
} finufft_opts;

GBNUFFT_EXPORT extern const int FINUFFT_FFT_DEFAULT;

typedef struct finufft_plan_s *finufft_plan;
typedef struct finufftf_plan_s *finufftf_plan;

#define GBNUFFT_GURU_DECLS(P, T, PLAN)                                                        \
  GBNUFFT_EXPORT void P##_default_opts(finufft_opts *o);                                      \
  GBNUFFT_EXPORT int P##_makeplan(int type, int dim, const int64_t *n_modes, int iflag,       \
                                  int n_transf, T tol, PLAN *plan, const finufft_opts *o);    \
  GBNUFFT_EXPORT int P##_setpts(PLAN plan, int64_t M, const T *xj, const T *yj,              \
                                const T *zj, int64_t N, const T *s, const T *t, const T *u); \
  GBNUFFT_EXPORT int P##_execute(PLAN plan, GBNUFFT_CPX(T) * weights,                         \
                                 GBNUFFT_CPX(T) * result);                                    \
  GBNUFFT_EXPORT int P##_execute_adjoint(PLAN plan, GBNUFFT_CPX(T) * weights,                 \
                                         GBNUFFT_CPX(T) * result);                            \
  GBNUFFT_EXPORT int P##_destroy(PLAN plan);

/* reference: include/finufft/finufft_eitherprec.h:55-67 */
GBNUFFT_GURU_DECLS(finufft, double, finufft_plan)
GBNUFFT_GURU_DECLS(finufftf, float, finufftf_plan)

/* The 18 simple interfaces per precision.
 * reference: include/finufft/finufft_eitherprec.h:69-140 */
#define GBNUFFT_HOST_SIMPLE_DECLS(P, T)                                                       \
  GBNUFFT_EXPORT int P##1d1(int64_t nj, const T *xj, const GBNUFFT_CPX(T) * cj, int iflag,    \
                            T eps, int64_t ms, GBNUFFT_CPX(T) * fk, const finufft_opts *o);   \
  GBNUFFT_EXPORT int P##1d1many(int nt, int64_t nj, const T *xj, const GBNUFFT_CPX(T) * cj,   \
                                int iflag, T eps, int64_t ms, GBNUFFT_CPX(T) * fk,            \
                                const finufft_opts *o);                                       \
  GBNUFFT_EXPORT int P##1d2(int64_t nj, const T *xj, GBNUFFT_CPX(T) * cj, int iflag, T eps,   \
                            int64_t ms, const GBNUFFT_CPX(T) * fk, const finufft_opts *o);    \
  GBNUFFT_EXPORT int P##1d2many(int nt, int64_t nj, const T *xj, GBNUFFT_CPX(T) * cj,         \
                                int iflag, T eps, int64_t ms, const GBNUFFT_CPX(T) * fk,      \
                                const finufft_opts *o);                                       \
  GBNUFFT_EXPORT int P##1d3(int64_t nj, const T *x, const GBNUFFT_CPX(T) * c, int iflag,      \
                            T eps, int64_t nk, const T *s, GBNUFFT_CPX(T) * f,                \
                            const finufft_opts *o);                                           \
  GBNUFFT_EXPORT int P##1d3many(int nt, int64_t nj, const T *x, const GBNUFFT_CPX(T) * c,     \
                                int iflag, T eps, int64_t nk, const T *s,                     \
                                GBNUFFT_CPX(T) * f, const finufft_opts *o);                   \
  GBNUFFT_EXPORT int P##2d1(int64_t nj, const T *xj, const T *yj, const GBNUFFT_CPX(T) * cj,  \
                            int iflag, T eps, int64_t ms, int64_t mt, GBNUFFT_CPX(T) * fk,    \
                            const finufft_opts *o);                                           \
  GBNUFFT_EXPORT int P##2d1many(int nt, int64_t nj, const T *xj, const T *yj,                 \
                                const GBNUFFT_CPX(T) * c, int iflag, T eps, int64_t ms,       \
                                int64_t mt, GBNUFFT_CPX(T) * fk, const finufft_opts *o);      \
  GBNUFFT_EXPORT int P##2d2(int64_t nj, const T *xj, const T *yj, GBNUFFT_CPX(T) * cj,        \
                            int iflag, T eps, int64_t ms, int64_t mt,                         \
                            const GBNUFFT_CPX(T) * fk, const finufft_opts *o);                \
  GBNUFFT_EXPORT int P##2d2many(int nt, int64_t nj, const T *xj, const T *yj,                 \
                                GBNUFFT_CPX(T) * c, int iflag, T eps, int64_t ms, int64_t mt, \
                                const GBNUFFT_CPX(T) * fk, const finufft_opts *o);            \
  GBNUFFT_EXPORT int P##2d3(int64_t nj, const T *x, const T *y, const GBNUFFT_CPX(T) * cj,    \
                            int iflag, T eps, int64_t nk, const T *s, const T *t,             \
                            GBNUFFT_CPX(T) * fk, const finufft_opts *o);                      \
  GBNUFFT_EXPORT int P##2d3many(int nt, int64_t nj, const T *x, const T *y,                   \
                                const GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t nk,      \
                                const T *s, const T *t, GBNUFFT_CPX(T) * fk,                  \
                                const finufft_opts *o);                                       \
  GBNUFFT_EXPORT int P##3d1(int64_t nj, const T *xj, const T *yj, const T *zj,                \
                            const GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t ms,          \
                            int64_t mt, int64_t mu, GBNUFFT_CPX(T) * fk,                      \
                            const finufft_opts *o);                                           \
  GBNUFFT_EXPORT int P##3d1many(int nt, int64_t nj, const T *xj, const T *yj, const T *zj,    \
                                const GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t ms,      \
                                int64_t mt, int64_t mu, GBNUFFT_CPX(T) * fk,                  \
                                const finufft_opts *o);                                       \
  GBNUFFT_EXPORT int P##3d2(int64_t nj, const T *xj, const T *yj, const T *zj,                \
                            GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t ms, int64_t mt,    \
                            int64_t mu, const GBNUFFT_CPX(T) * fk, const finufft_opts *o);    \
  GBNUFFT_EXPORT int P##3d2many(int nt, int64_t nj, const T *xj, const T *yj, const T *zj,    \
                                GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t ms,            \
                                int64_t mt, int64_t mu, const GBNUFFT_CPX(T) * fk,            \
                                const finufft_opts *o);                                       \
  GBNUFFT_EXPORT int P##3d3(int64_t nj, const T *x, const T *y, const T *z,                   \
                            const GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t nk,          \
                            const T *s, const T *t, const T *u, GBNUFFT_CPX(T) * fk,          \
                            const finufft_opts *o);                                           \
  GBNUFFT_EXPORT int P##3d3many(int nt, int64_t nj, const T *x, const T *y, const T *z,       \
                                const GBNUFFT_CPX(T) * cj, int iflag, T eps, int64_t nk,      \
                                const T *s, const T *t, const T *u, GBNUFFT_CPX(T) * fk,      \
                                const finufft_opts *o);

GBNUFFT_HOST_SIMPLE_DECLS(finufft, double)
GBNUFFT_HOST_SIMPLE_DECLS(finufftf, float)

#ifdef __cplusplus
}
#endif
#endif
