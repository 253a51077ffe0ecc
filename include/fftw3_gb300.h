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

/* Message of the last planner or execute failure in this thread. */
extern const char *fftw_gb300_last_error(void);
/* Number of execute calls that failed since the library was loaded. */
extern int fftw_gb300_failures(void);
/* Dry run: plans are compiled without touching a GPU (no allocation, no
 * launch) so the planner can be inspected on a machine without one. */
extern void fftw_gb300_set_dry_run(int on);
/* Number of kernels this library has launched since it was loaded. */
extern long long fftw_gb300_launch_count(void);

#define GB_FFTW_EXT_DECLARE(PFX)                                                       \
extern int PFX##gb300_set_stream(PFX##plan p, void *cuda_stream);                     \
extern int PFX##gb300_set_async(PFX##plan p, int async);                              \
extern int PFX##gb300_npasses(PFX##plan p);                                           \
extern int PFX##gb300_pass_info(PFX##plan p, int i, int *kind, int *nfft, int *variant,\
                                int *tb, int *threads, int *smem, long long *blocks); \
extern size_t PFX##gb300_scratch_bytes(PFX##plan p);

GB_FFTW_EXT_DECLARE(fftw_)
GB_FFTW_EXT_DECLARE(fftwf_)

#ifdef __cplusplus
}
#endif
#endif
