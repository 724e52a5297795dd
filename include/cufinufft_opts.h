/* Options for the device-pointer (cufinufft_*) interface.
 *
 * Field order, types and meaning are identical to cufinufft_opts in
 * flatironinstitute/finufft (include/cufinufft_opts.h:7-40): the Python
 * ctypes binding and other language bindings lay this struct out by hand, so
 * it must stay byte-for-byte compatible. Options this engine adds live in
 * gbnufft_ext.h, never here.
 * Defaults are set by cufinufft_default_opts().
 */
#ifndef GBNUFFT_CUFINUFFT_OPTS_H
#define GBNUFFT_CUFINUFFT_OPTS_H

typedef struct cufinufft_opts {
  double upsampfac;         /* sigma; 0.0 = choose automatically */
  int gpu_method;           /* 0 auto, 1 point-driven (GM), 2 tiled subproblems (SM), 3 output-driven */
  int gpu_sort;             /* point-driven only: 0 keep user order, 1 bin-sort */
  int gpu_binsizex;         /* bin (tile interior) size per dimension, 0 = auto */
  int gpu_binsizey;
  int gpu_binsizez;
  int gpu_obinsizex;        /* accepted for ABI compatibility (block-gather method) */
  int gpu_obinsizey;
  int gpu_obinsizez;
  int gpu_maxsubprobsize;   /* max points per subproblem (tile work unit) */
  int gpu_kerevalmeth;      /* 0 direct exp(sqrt()), 1 piecewise polynomial (Horner) */
  int gpu_spreadinterponly; /* 1: spread (type 1) or interpolate (type 2) only */
  int gpu_maxbatchsize;     /* transforms per batch, 0 = auto */
  int gpu_device_id;        /* device the plan lives on */
  void *gpu_stream;         /* cudaStream_t the plan runs on (NULL = legacy default) */
  int modeord;              /* 0 CMCL order (-N/2..N/2-1), 1 FFT order */
  int gpu_np;               /* output-driven method: points staged per block */
  int debug;                /* 0 silent, 1 plan summary, 2 stage timings */
} cufinufft_opts;

#endif
