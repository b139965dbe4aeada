/* cufinufft.h -- C ABI of the GB300-native type-1/type-2 NUFFT library.
 *
 * Drop-in for the public interface of cuFINUFFT v1.3: the ten entry points
 * below have the reference's names, argument lists and meanings
 * (include/cufinufft_eitherprec.h:311-324 of the reference, documented in its
 * docs/cppdoc.md), and cufinufft_opts is byte-identical (cufinufft_opts.h).
 * "cufinufft_*" is the FP64 library, "cufinufftf_*" the FP32 one.
 *
 * Semantics kept from the reference:
 *   - plans are opaque pointers; one plan is not re-entrant, distinct plans
 *     may be used from distinct host threads;
 *   - x, y, z, c, fk are DEVICE pointers owned by the caller; nmodes[0] is
 *     the fastest (x) dimension; fk is in CMCL order, k = -N/2..(N-1)/2 with
 *     k1 fastest, then the transform index; c is transform-major;
 *   - iflag >= 0 selects exp(+i k.x), otherwise exp(-i k.x); sums are not
 *     normalised; points lie in [-pi, pi) (one period either side,
 *     [-3pi, 3pi), is folded in);
 *   - the stages may be repeated: 1234, 123334 and 1232334 are valid;
 *   - return value 0 = success; makeplan swallows the tolerance warning (1).
 * Differences, by design:
 *   - setpts copies the bin-sorted, rescaled points into plan memory, so the
 *     coordinate arrays may be freed or reused after setpts returns;
 *   - CUDA and cuFFT failures are returned as error codes (the reference
 *     calls exit() inside the library);
 *   - work is queued on a plan-owned blocking stream (ordered after the
 *     legacy default stream), or on the stream given to *_set_stream.
 */
#ifndef CUFINUFFT_GB300_H
#define CUFINUFFT_GB300_H

#include <cuComplex.h>
#include <cuda_runtime_api.h>

#include "cufinufft_opts.h"

/* Return codes.  1..9 are the reference's (contrib/utils.h:28-36 and the
 * method checks in src/2d/spread2d_wrapper.cu:155); 10.. are this library's. */
#define CUFINUFFT_WARN_EPS_TOO_SMALL 1
#define CUFINUFFT_ERR_GENERIC 1        /* also: bad type, bad binsize, NULL plan */
#define CUFINUFFT_ERR_METHOD 2         /* gpu_method not valid for this dim/type */
#define CUFINUFFT_ERR_UPSAMPFAC_TOO_SMALL 7
#define CUFINUFFT_ERR_HORNER_WRONG_BETA 8
#define CUFINUFFT_ERR_NDATA_NOTVALID 9
#define CUFINUFFT_ERR_CUDA 10          /* a CUDA runtime call failed        */
#define CUFINUFFT_ERR_CUFFT 11         /* a cuFFT call failed               */
#define CUFINUFFT_ERR_ALLOC 12         /* device allocation failed          */
#define CUFINUFFT_ERR_ARG 13           /* invalid argument (sizes, pointers) */
#define CUFINUFFT_ERR_SHMEM 14         /* bin tile exceeds shared memory    */

typedef struct cufinufft_plan_s* cufinufft_plan;
typedef struct cufinufftf_plan_s* cufinufftf_plan;

#ifdef __cplusplus
extern "C" {
#endif

/* Fill *opts with the defaults for (type, dim).  Replaces
 * cufinufft[f]_default_opts, src/cufinufft.cu:639-730. */
int cufinufft_default_opts(int type, int dim, cufinufft_opts* opts);
int cufinufftf_default_opts(int type, int dim, cufinufft_opts* opts);

/* Make a plan.  Replaces CUFINUFFT_MAKEPLAN, src/cufinufft.cu:78-273
 * (include/cufinufft_eitherprec.h:313-315).  opts may be NULL (defaults on
 * device 0).  maxbatchsize 0 picks min(ntransf, 8). */
int cufinufft_makeplan(int type, int dim, int* nmodes, int iflag, int ntransf,
                       double tol, int maxbatchsize, cufinufft_plan* plan,
                       cufinufft_opts* opts);
int cufinufftf_makeplan(int type, int dim, int* nmodes, int iflag, int ntransf,
                        float tol, int maxbatchsize, cufinufftf_plan* plan,
                        cufinufft_opts* opts);

/* Set the M nonuniform points (device arrays; y unused in 1D, z unused in
 * 1D/2D; N, s, t, u are the type-3 arguments and are ignored).  Replaces
 * CUFINUFFT_SETPTS, src/cufinufft.cu:275-493. */
int cufinufft_setpts(int M, double* x, double* y, double* z, int N, double* s,
                     double* t, double* u, cufinufft_plan plan);
int cufinufftf_setpts(int M, float* x, float* y, float* z, int N, float* s,
                      float* t, float* u, cufinufftf_plan plan);

/* Run ntransf transforms: type 1 reads c (ntransf*M) and writes fk
 * (ntransf*N1*N2*N3); type 2 reads fk and writes c.  Replaces
 * CUFINUFFT_EXECUTE, src/cufinufft.cu:495-569.  With stage timing off the
 * launch sequence is captured as a CUDA graph the first time a pair (c, fk)
 * is seen and replayed after that; setpts / set_layout, or other arrays,
 * capture it again (CUFINUFFT_GRAPH=0: direct launches every time). */
int cufinufft_execute(cuDoubleComplex* c, cuDoubleComplex* fk,
                      cufinufft_plan plan);
int cufinufftf_execute(cuFloatComplex* c, cuFloatComplex* fk,
                       cufinufftf_plan plan);

/* Free a plan and its device memory.  Replaces CUFINUFFT_DESTROY,
 * src/cufinufft.cu:571-637.  Returns 1 for a NULL plan, as the reference. */
int cufinufft_destroy(cufinufft_plan plan);
int cufinufftf_destroy(cufinufftf_plan plan);

/* ---- extensions (no counterpart in the reference) ----------------------- */

/* Queue all later work of this plan on `stream` (NULL restores the plan's
 * own stream).  The reference has no stream argument; this lets a caller
 * order a plan with its own work and capture execute() in a CUDA graph. */
int cufinufft_set_stream(cufinufft_plan plan, cudaStream_t stream);
int cufinufftf_set_stream(cufinufftf_plan plan, cudaStream_t stream);

/* Plan facts for callers and tools: fine-grid sizes, kernel width, the
 * method actually run, total bins and subproblems of the last setpts. */
typedef struct cufinufft_plan_info {
  int type, dim, ms, mt, mu, nf1, nf2, nf3, ns, M, ntransf, maxbatchsize;
  int method, sort, binsizex, binsizey, binsizez, nbins, nsubprob, kerevalmeth;
  double beta, es_c;
  int line_fft;   /* 1: pruned line FFTs (fftpass.cu), 0: cuFFT over the whole grid */
  int cell_order; /* 1: method 2 spreading over cell-ordered points (cell-run kernel) */
  int width_rule; /* kernel-width rule the plan was made under (cufinufft_set_width_rule) */
  int chain_fp32; /* 1: an FP64 plan running its spread/interp, FFT and deconvolution in FP32 */
  int half_fft;   /* 1: pruned power-of-two FFT passes (halffft.cu) instead of cuFFT */
  int fp64_df;    /* 1: an FP64 type-2 method-2 plan interpolating in double-float (FP32 pairs) */
  int df_fft;     /* 1: an FP64 2D plan transforming its grid in double-float (fft_df.cu) */
} cufinufft_plan_info;
int cufinufft_get_info(cufinufft_plan plan, cufinufft_plan_info* info);
int cufinufftf_get_info(cufinufftf_plan plan, cufinufft_plan_info* info);

/* Kernel-width rule (no counterpart in the reference; it sets no field of
 * cufinufft_opts, whose layout is the reference's).  The reference picks
 * ns = ceil(-log10(tol/10)) at upsampfac 2 (contrib/spreadinterp.cpp:42),
 * which leaves relative l2 errors of one to four times tol.  Rule 1 picks
 * the narrowest width whose error, as measured with an FP64 restatement of
 * the algorithm against direct sums (uniform random points and data, the
 * plan's dimension, with a 25% margin), is at most tol -- usually one more
 * than the reference's width -- and never wider than the reference's width
 * at the precision's machine epsilon.  Rule 0 is the reference's (the
 * default).  The rule applies to the makeplan calls that follow on the
 * calling thread; -1 returns to the process default, which the environment
 * variable CUFINUFFT_WIDTH_RULE ("tol" or "1": rule 1) sets.  *previous
 * (when not NULL) receives the thread's earlier setting. */
int cufinufft_set_width_rule(int rule, int* previous);

/* Stage timing.  With timing on, execute() records CUDA events around its
 * three stages on the plan stream; stage_times() waits for them and returns
 * the accumulated milliseconds ms[0] = spread (type 1) or interp (type 2)
 * kernel, ms[1] = cuFFT, ms[2] = deconvolve (type 1, with the grid clear)
 * or amplify (type 2), plus the number of batches timed; reset != 0 clears
 * the totals. */
int cufinufft_set_timing(cufinufft_plan plan, int on);
int cufinufftf_set_timing(cufinufftf_plan plan, int on);
int cufinufft_stage_times(cufinufft_plan plan, double* ms, long long* batches, int reset);
int cufinufftf_stage_times(cufinufftf_plan plan, double* ms, long long* batches, int reset);

/* Layout and autotuning (no counterpart in the reference).  set_layout
 * switches a plan whose points are set to another method, bin size and
 * subproblem cap by re-sorting the stored points -- results do not change,
 * only the schedule.  Methods: 1 (NU-point driven), 2 (subproblems), 5
 * (type 1 only: method 2 over points sorted by cell inside their bin, with
 * runs of points on one cell accumulated in registers -- the cell-run
 * spread; at most 512 taps per point and 2^24 (bin, cell) keys).
 * autotune times the plan's spread (type 1) or interp (type 2) stage under
 * the twelve layout classes (0-2: method 1 with small, medium, large bins;
 * 3-8: method 2 with those bins x subproblem cap 256 or 1024; 9-11: method 5
 * with those bins, cap 1024; bins 1D 256/1024/4096, 2D 16^2/32^2/64^2, 3D
 * 8x8x8/16x16x2/16x16x4) on the plan's own points, keeps the fastest, and
 * reports the chosen entry first followed by the twelve classes in order
 * (ms = -2: not runnable). */
typedef struct cufinufft_tune_entry {
  int method, binsizex, binsizey, binsizez, maxsubprobsize;
  float ms;
} cufinufft_tune_entry;
int cufinufft_set_layout(cufinufft_plan plan, int method, int binsizex, int binsizey, int binsizez,
                         int maxsubprobsize);
int cufinufftf_set_layout(cufinufftf_plan plan, int method, int binsizex, int binsizey,
                          int binsizez, int maxsubprobsize);
int cufinufft_autotune(cufinufft_plan plan, cufinufft_tune_entry* entries, int max_entries,
                       int* n_entries);
int cufinufftf_autotune(cufinufftf_plan plan, cufinufft_tune_entry* entries, int max_entries,
                        int* n_entries);

/* Learned layout selector (no counterpart in the reference).
 * features() writes CUFINUFFT_MLP_FEATURES numbers describing a plan whose
 * points are set: 0 dim, 1 type, 2 FP32 (1) or FP64 (0), 3 kernel width,
 * 4 log2(M+1), 5 log2(modes), 6 log2(fine-grid cells), 7 log2((M+1)/cells),
 * 8 log2(ntransf), and occupancy statistics of the points over fixed
 * feature bins (1D 64, 2D 16x16, 3D 8x8x8 cells): 9 fraction of bins that
 * hold points, 10 coefficient of variation of the counts of those bins,
 * 11 log2(max / mean count), 12 log2(mean count of occupied bins),
 * 13 log2(participation ratio nbins * sum c^2 / (sum c)^2).
 * The network maps standardised features to the predicted log2 time ratio
 * of each of the twelve layout classes (see autotune); its parameters are one
 * flat FP32 array of CUFINUFFT_MLP_PARAMS floats,
 *   W1[H][F], b1[H], W2[H][H], b2[H], W3[K][H], b3[K].
 * mlp_forward: X [B][F] -> Y [B][K]; work holds 2*B*H floats.
 * mlp_grad: masked mean squared error against T with mask (mask_sum = its
 *   sum) and the gradient of every parameter; work holds B*(4H+2K) floats.
 * mlp_adam: one Adam step (beta 0.9 / 0.999, eps 1e-8) at step >= 1.
 * All pointers are device pointers; work is queued on `stream`. */
#define CUFINUFFT_MLP_FEATURES 14
#define CUFINUFFT_MLP_HIDDEN 32
#define CUFINUFFT_MLP_CLASSES 12
#define CUFINUFFT_MLP_PARAMS                                                             \
  (CUFINUFFT_MLP_HIDDEN * CUFINUFFT_MLP_FEATURES + CUFINUFFT_MLP_HIDDEN +                 \
   CUFINUFFT_MLP_HIDDEN * CUFINUFFT_MLP_HIDDEN + CUFINUFFT_MLP_HIDDEN +                   \
   CUFINUFFT_MLP_CLASSES * CUFINUFFT_MLP_HIDDEN + CUFINUFFT_MLP_CLASSES)
int cufinufft_features(cufinufft_plan plan, float* features);
int cufinufftf_features(cufinufftf_plan plan, float* features);
/* Switch a plan with points set to layout class cls (0-11, see autotune). */
int cufinufft_set_layout_class(cufinufft_plan plan, int cls);
int cufinufftf_set_layout_class(cufinufftf_plan plan, int cls);
int cufinufft_mlp_forward(const float* params, const float* X, int B, float* Y, float* work,
                          cudaStream_t stream);
int cufinufft_mlp_grad(const float* params, const float* X, const float* T, const float* mask,
                       int B, float mask_sum, float* grad, float* loss, float* work,
                       cudaStream_t stream);
int cufinufft_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr,
                       cudaStream_t stream);

/* Batches (no counterpart in the reference): many plans of one type,
 * dimension, precision and kernel width -- different N, M and ntransf --
 * executed together.  batch_make takes plans whose points are set (they must
 * outlive the batch and keep their points); batch_execute takes host arrays
 * of nplans device pointers (c[i], fk[i] as for plan i's execute) and runs
 * every plan's whole ntransf at once: one CUDA-graph replay of every plan's
 * own execute on parallel branches (captured again when the arrays change;
 * with CUFINUFFT_BATCH=tables, multi-plan spread/interp and
 * deconvolve/amplify kernels over a descriptor table plus one cuFFT call per
 * plan).  A plan must not run on its own while its batch runs.  Results are
 * ordered before later work on the legacy default stream. */
typedef struct cufinufft_batch_s* cufinufft_batch;
typedef struct cufinufftf_batch_s* cufinufftf_batch;
int cufinufft_batch_make(int nplans, cufinufft_plan* plans, cufinufft_batch* batch);
int cufinufftf_batch_make(int nplans, cufinufftf_plan* plans, cufinufftf_batch* batch);
int cufinufft_batch_execute(cufinufft_batch batch, cuDoubleComplex** c, cuDoubleComplex** fk);
int cufinufftf_batch_execute(cufinufftf_batch batch, cuFloatComplex** c, cuFloatComplex** fk);
int cufinufft_batch_destroy(cufinufft_batch batch);
int cufinufftf_batch_destroy(cufinufftf_batch batch);

/* Allocation-free spreading; it has no counterpart in the reference.  For
 * callers that cannot allocate device memory at the point of use (code inside
 * a framework that owns all device memory, real-time loops, memory-budgeted
 * services): spreads M points (x, y in [-3pi, 3pi), strengths c, all device
 * arrays) onto the caller's nf1 x nf2 fine grid fw (x fastest), which this
 * call zeroes first, with the ES kernel of FP32 tolerance tol, on `stream`,
 * without allocating.  It runs the type-1 spreading stage of a plan with
 * that fine grid (bin sort, 32x32 bins, shared-memory subproblems) in plain
 * bin order and always evaluates the ES kernel directly (exp form, not the
 * fitted polynomials), so its grid matches that plan's spreading within
 * FP32 rounding, not bit for bit.  Its sort scratch is a fixed device array
 * of about 3.2 MB that every GPU loading the library holds.  Limits:
 * M <= 131072 and at most 4096 bins (fine grids up to 2048 x 2048); larger
 * requests return CUFINUFFT_ERR_ARG.  All calls on a device share that
 * scratch: calls whose GPU work overlaps race and must be serialised by the
 * caller.  The first call on each device looks up the scratch address, so
 * make it before any stream capture; the address is kept for the life of
 * the process, so a device reset (cudaDeviceReset) after that first call is
 * not supported. */
int cufinufftf_spread2d_noalloc(int M, const float* x, const float* y, const cuFloatComplex* c,
                                int nf1, int nf2, float tol, cuFloatComplex* fw,
                                cudaStream_t stream);

/* Measured accumulation ceilings of the current device (no counterpart in
 * the reference): lane operations per second of kind 0 = shared-memory FP32
 * atomicAdd, 1 = shared-memory int32 atomicAdd, 2 = global 8-byte
 * red.global.add.v2.f32 into L2-resident addresses, 3 = shared-memory 64-bit
 * integer atomicAdd, every lane of a warp on its own address.  The spread kernels are bound by these rather than by
 * HBM; the benchmark's type-1 roofline divides by them.  Allocates, runs
 * two short launches on a private stream and synchronises it. */
int cufinufft_atomic_rate(int kind, double* lane_ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* CUFINUFFT_GB300_H */
