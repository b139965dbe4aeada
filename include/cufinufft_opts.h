/* cufinufft_opts -- algorithm options for a type-1/type-2 NUFFT plan.
 *
 * Byte-identical to the reference struct (include/cufinufft_opts.h:4-26 of
 * cuFINUFFT v1.3) and to its ctypes mirror (python/cufinufft/_cufinufft.py:
 * 77-93): one double followed by thirteen ints, in this order.  Fill it with
 * cufinufft_default_opts() and change fields before cufinufft_makeplan().
 * A value <= 0 in a bin-size field (the default -1) lets the library choose.
 */
#ifndef CUFINUFFT_OPTS_H
#define CUFINUFFT_OPTS_H

typedef struct cufinufft_opts {
  double upsampfac;          /* upsampling ratio sigma (2.0 default)        */
  int gpu_method;            /* 1: NU-point driven, 2: shared-memory bins,
                                3: (2D type 1) accepted, runs as 2,
                                4: (3D type 1) accepted, runs as 2 on
                                   8x8x8 output bins                       */
  int gpu_sort;              /* method 1 only: 1 sort points by bin first  */
  int gpu_binsizex;          /* bin (tile interior) size, fine-grid cells  */
  int gpu_binsizey;
  int gpu_binsizez;
  int gpu_obinsizex;         /* method 4 output-bin size                   */
  int gpu_obinsizey;
  int gpu_obinsizez;
  int gpu_maxsubprobsize;    /* max points per shared-memory subproblem    */
  int gpu_nstreams;          /* accepted for ABI parity, unused            */
  int gpu_kerevalmeth;       /* 0: exp(beta*sqrt(1-c x^2)), 1: piecewise
                                polynomial (Horner) fitted at plan time    */
  int gpu_spreadinterponly;  /* 1: spread/interpolate only -- nmodes is the
                                fine grid itself (each >= 2 ns), execute()
                                spreads c into fk (type 1) or interpolates
                                fk to c (type 2), no FFT or deconvolution;
                                the reference sets this flag in its
                                spread/interp tests (test/spread2d_test.cu:80) */
  int gpu_device_id;         /* CUDA device the plan lives on              */
} cufinufft_opts;

#endif
