/*
 * fftw3_gb300.h -- extensions of libfftw3_gb300 beyond the reference API.
 *
 * None of these has a counterpart in the reference (api/fftw3.h); they
 * expose what a GPU execution adds: the CUDA stream a plan runs on, an
 * asynchronous execute, the error status that execute (a void function in
 * the reference) cannot return, and introspection of the compiled passes.
 */
#ifndef FFTW3_GB300_H
#define FFTW3_GB300_H

#include <stddef.h>
#include "fftw3.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Planner flag (a bit the reference leaves unused): run the radix-16 stages
 * of f32 c2c passes of 256 to 4096 points (a power of two) on the tensor cores,
 * as split-FP16 (hi + lo) DFT-matrix GEMMs with FP32 accumulation. */
#define FFTW_GB300_TENSOR_CORE (1U << 28)

/* Message of the last planner or execute failure in this thread. */
extern const char *fftw_gb300_last_error(void);
/* Number of execute calls that failed since the library was loaded. */
extern int fftw_gb300_failures(void);
/* Dry run: plans are compiled without touching a GPU (no allocation, no
 * launch) so the planner can be inspected on a machine without one. */
extern void fftw_gb300_set_dry_run(int on);
/* Test hook: the device table allocation after the next k (k >= 0) fails
 * once, as a refused cudaMalloc would, so the planner's failure path (a NULL
 * plan, the message in fftw_gb300_last_error) can be exercised on the host;
 * -1 cancels.  Works in dry runs. */
extern void fftw_gb300_fail_alloc_after(int k);
/* Number of kernels this library has launched since it was loaded. */
extern long long fftw_gb300_launch_count(void);
/* Read and clear the device status word: 0 when no kernel reported a
 * problem, else a code (2: a work-queue dependency wait gave up, 3: a bulk
 * copy never completed); kernels bound every wait instead of hanging. */
extern int fftw_gb300_device_status(void);
/* Tensor-core path self-test: D = A . B^T with A 128 x 16ks and B 32 x 16ks
 * (IEEE half, row-major, device memory) and D 128 x 32 (float, device);
 * ks in 1..6.  Returns 0 on success. */
extern int fftw_gb300_tc_selftest(const void *A, const void *B, float *D, int ks);
/* FP64 fused multiply-add rate of the current GPU in GFLOP/s (two flops per
 * FMA), measured with CUDA events: the roofline of double-precision passes,
 * which this part's few FP64 units bound before HBM does.  0 on error. */
extern double fftw_gb300_fp64_fma_gflops(void);

/* No counterpart in the reference: a batched f32 1D c2c DFT that allocates
 * no device memory, for callers that cannot call cudaMalloc (device memory
 * owned by their own arena or budget; loops that cannot take cudaMalloc's
 * implicit synchronisation).  It runs the two-pass (four-step) kernels of
 * a long 1D plan with their scratch and twiddle tables in one fixed device
 * array of the library, which every GPU it runs on holds until exit
 * (16 MiB + 30.75 KiB).  howmany contiguous transforms of length n at distance
 * n; in and out are device arrays (they may be the same); n is a power of
 * two from 2^12 to 2^21 and n * howmany <= FFTWF_GB300_NOALLOC_MAX_POINTS,
 * else it returns -1 without launching.  Enqueues on cuda_stream and
 * returns 0, or -1 with fftw_gb300_last_error() set.  The first call on a
 * device looks up the array's address (set-up); make it before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race. */
#define FFTWF_GB300_NOALLOC_MAX_POINTS (1 << 21)
extern int fftwf_gb300_dft_1d_noalloc(int n, int howmany, const fftwf_complex *in, fftwf_complex *out,
                                      int sign, void *cuda_stream);

#define GB_FFTW_EXT_DECLARE(PFX)                                                       \
extern int PFX##gb300_set_stream(PFX##plan p, void *cuda_stream);                     \
extern int PFX##gb300_set_async(PFX##plan p, int async);                              \
extern int PFX##gb300_npasses(PFX##plan p);                                           \
extern int PFX##gb300_pass_info(PFX##plan p, int i, int *kind, int *nfft, int *variant,\
                                int *tb, int *threads, int *smem, long long *blocks); \
extern size_t PFX##gb300_scratch_bytes(PFX##plan p);                                  \
/* Plan sets: many rank-1 c2c plans (uneven lengths, device arrays) run by  \
 * one persistent work-queue kernel, captured once as a CUDA graph; each     \
 * execute is one graph launch equivalent to executing every plan.          */\
typedef struct PFX##gb300_set_s *PFX##gb300_set;                                      \
extern PFX##gb300_set PFX##gb300_plan_set(int nplans, const PFX##plan *plans,         \
                                          unsigned flags);                            \
extern int PFX##gb300_execute_set(PFX##gb300_set s);                                  \
extern int PFX##gb300_set_stream_set(PFX##gb300_set s, void *cuda_stream, int async); \
extern int PFX##gb300_set_info(PFX##gb300_set s, int *nitems, int *ntransforms,       \
                               int *nlong, int *grid, int *smem);                     \
/* Item i in queue order: kind (gb_kind), FFT length, transforms, body      \
 * (variant), queue (0 small tiles, 1 large tiles), role (1 a column tile   \
 * row tiles wait for, 2 a row tile that waits, 0 a single).  Sets planned  \
 * under fftw_gb300_set_dry_run(1) keep their items on the host (grid 0,    \
 * no execute).                                                             */\
extern int PFX##gb300_set_item_info(PFX##gb300_set s, int i, int *kind, int *nfft,    \
                                    int *tb, int *variant, int *queue, int *role);    \
/* Bound (seconds, default 2) on a row tile's device-side wait for the      \
 * column tiles of its transform; a wait that runs out skips the tile and   \
 * sets device status 2.  Test hook: set_test_stall(s, 1) makes the first   \
 * row tile wait for one column tile more than exist (its wait runs out on  \
 * every execute), set_test_stall(s, 0) undoes it.                          */\
extern int PFX##gb300_set_wait_limit(PFX##gb300_set s, double seconds);               \
extern int PFX##gb300_set_test_stall(PFX##gb300_set s, int on);                       \
extern void PFX##gb300_destroy_set(PFX##gb300_set s);

GB_FFTW_EXT_DECLARE(fftw_)
GB_FFTW_EXT_DECLARE(fftwf_)

#ifdef __cplusplus
}
#endif
#endif
