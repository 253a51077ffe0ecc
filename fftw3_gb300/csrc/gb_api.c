/*
 * libfftw3_gb300 public entry points: the reference's fftw3.h API for the
 * double (fftw_) and float (fftwf_) prefixes, plus the extensions declared
 * in include/fftw3_gb300.h.  The per-precision bodies are in gb_api_impl.h.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "fftw3_gb300.h"
#include "gb_host.h"

/* ---------------------------------------------------------------- state */
static double gb_timelimit = -1.0;
static int gb_nthreads = 1;
static int gb_fail_count = 0;

void gb_set_timelimit(double t) { gb_timelimit = t; }
double gb_get_timelimit(void) { return gb_timelimit; }
void gb_set_nthreads(int n) { gb_nthreads = n < 1 ? 1 : n; }
int gb_get_nthreads(void) { return gb_nthreads; }
void gb_note_failure(void) { __atomic_add_fetch(&gb_fail_count, 1, __ATOMIC_RELAXED); }
void gb_cleanup_tables(void) { if (!gb_dry_run()) gb_tables_free(); }

/* fftw_malloc: page-locked host memory when a GPU is present (host arrays
 * are staged to the device at DMA speed), 64-byte aligned host memory
 * otherwise (api/malloc.c:24-50 only promises SIMD alignment).  Arrays of
 * 1 MiB or more start on a 4 KiB page boundary: copy engines and the
 * kernels' direct reads of host memory lose a quarter of their bandwidth
 * on arrays that start part-way into a page. */
typedef struct { void *base; int pinned; } gb_alloc_hdr;

void *gb_malloc(size_t n)
{
     void *base = 0;
     int pinned = 0;
     const size_t off = n >= ((size_t)1 << 20) ? 4096 : 64;
     size_t tot = n + off;
     char *p;
     if (!gb_dry_run() && gb_cuda_ready() && !getenv("FFTW_GB300_PAGEABLE")) {
          if (cudaMallocHost(&base, tot) == cudaSuccess) pinned = 1;
          else { cudaGetLastError(); base = 0; }
     }
     if (!base && posix_memalign(&base, off, tot) != 0) return 0;
     p = (char *)base + off;
     ((gb_alloc_hdr *)(p - sizeof(gb_alloc_hdr)))->base = base;
     ((gb_alloc_hdr *)(p - sizeof(gb_alloc_hdr)))->pinned = pinned;
     return p;
}

void gb_free(void *p)
{
     gb_alloc_hdr h;
     if (!p) return;
     h = *(gb_alloc_hdr *)((char *)p - sizeof(gb_alloc_hdr));
     if (h.pinned) cudaFreeHost(h.base);
     else free(h.base);
}

/* version strings (api/version.c:21-40) */
const char fftw_version[] = "fftw-3.3.10-gb300";
const char fftwf_version[] = "fftw-3.3.10-gb300";
const char fftw_cc[] = "nvcc -gencode arch=compute_103a,code=sm_103a; gcc";
const char fftwf_cc[] = "nvcc -gencode arch=compute_103a,code=sm_103a; gcc";
const char fftw_codelet_optim[] = "sm_103a register/shared-memory stages";
const char fftwf_codelet_optim[] = "sm_103a register/shared-memory stages";

/* ---------------------------------------------------------------- API */
#define C fftw_complex
#define R double
#define PFX(name) fftw_##name
#include "gb_api_impl.h"
#undef C
#undef R
#undef PFX

#define C fftwf_complex
#define R float
#define PFX(name) fftwf_##name
#include "gb_api_impl.h"
#undef C
#undef R
#undef PFX

/* ---------------------------------------------------------------- extensions */
const char *fftw_gb300_last_error(void) { return gb_last_error(); }
int fftw_gb300_failures(void) { return __atomic_load_n(&gb_fail_count, __ATOMIC_RELAXED); }
void fftw_gb300_set_dry_run(int on) { gb_set_dry_run(on); }
void fftw_gb300_fail_alloc_after(int k) { gb_fail_alloc_after(k); }
long long fftw_gb300_launch_count(void) { return gb_launch_count(); }

#define GB_EXT(PFX_, PLAN)                                                              \
     int PFX_##gb300_set_stream(PLAN p, void *stream)                                  \
     {                                                                                 \
          if (!p) return -1;                                                           \
          p->g->stream = stream;                                                       \
          return 0;                                                                    \
     }                                                                                 \
     int PFX_##gb300_set_async(PLAN p, int async)                                      \
     {                                                                                 \
          if (!p) return -1;                                                           \
          p->g->async = async;                                                         \
          return 0;                                                                    \
     }                                                                                 \
     int PFX_##gb300_npasses(PLAN p) { return p ? p->g->nstep : -1; }                  \
     int PFX_##gb300_pass_info(PLAN p, int i, int *kind, int *nfft, int *variant,      \
                               int *tb, int *threads, int *smem, long long *blocks)    \
     {                                                                                 \
          const gb_pass *P;                                                            \
          if (!p || i < 0 || i >= p->g->nstep) return -1;                              \
          P = &p->g->step[i].pass;                                                     \
          *kind = P->kind; *nfft = P->nfft; *variant = P->variant; *tb = P->tb;        \
          *threads = P->threads; *smem = P->smem; *blocks = P->nblocks;                \
          return 0;                                                                    \
     }                                                                                 \
     size_t PFX_##gb300_scratch_bytes(PLAN p) { return p ? p->g->scratch_bytes : 0; }

GB_EXT(fftw_, fftw_plan)
GB_EXT(fftwf_, fftwf_plan)

/* plan sets: one work-queue kernel (one CUDA graph launch) for many plans */
#define GB_SET_EXT(PFX_, PLAN, SET, PREC)                                               \
     SET PFX_##gb300_plan_set(int nplans, const PLAN *plans, unsigned flags)           \
     {                                                                                 \
          gb_plan **g;                                                                 \
          gb_set *s;                                                                   \
          int i;                                                                       \
          if (nplans < 0 || (nplans > 0 && !plans)) return 0;                          \
          g = (gb_plan **)malloc(sizeof(gb_plan *) * (size_t)(nplans ? nplans : 1));   \
          for (i = 0; i < nplans; ++i) g[i] = plans[i] ? plans[i]->g : 0;              \
          gb_lock();                                                                   \
          s = gb_mkset(PREC, nplans, g, flags);                                        \
          gb_unlock();                                                                 \
          free(g);                                                                     \
          return (SET)s;                                                               \
     }                                                                                 \
     int PFX_##gb300_execute_set(SET s)                                                \
     {                                                                                 \
          if (!s) return -1;                                                           \
          if (gb_execute_set((gb_set *)s)) {                                           \
               gb_note_failure();                                                      \
               return -1;                                                              \
          }                                                                            \
          return 0;                                                                    \
     }                                                                                 \
     int PFX_##gb300_set_stream_set(SET s, void *stream, int async)                    \
     {                                                                                 \
          if (!s) return -1;                                                           \
          gb_set_stream_of_set((gb_set *)s, stream, async);                            \
          return 0;                                                                    \
     }                                                                                 \
     int PFX_##gb300_set_info(SET s, int *nitems, int *ntransforms, int *nlong,        \
                              int *grid, int *smem)                                    \
     {                                                                                 \
          if (!s) return -1;                                                           \
          gb_set_info((const gb_set *)s, nitems, ntransforms, nlong, grid, smem);      \
          return 0;                                                                    \
     }                                                                                 \
     int PFX_##gb300_set_item_info(SET s, int i, int *kind, int *nfft, int *tb,        \
                                   int *variant, int *queue, int *role)               \
     {                                                                                 \
          return s ? gb_set_item_info((const gb_set *)s, i, kind, nfft, tb, variant,   \
                                      queue, role)                                     \
                   : -1;                                                               \
     }                                                                                 \
     int PFX_##gb300_set_wait_limit(SET s, double seconds)                             \
     {                                                                                 \
          return s ? gb_set_wait_limit((gb_set *)s, seconds) : -1;                     \
     }                                                                                 \
     int PFX_##gb300_set_test_stall(SET s, int on)                                     \
     {                                                                                 \
          return s ? gb_set_test_stall((gb_set *)s, on) : -1;                          \
     }                                                                                 \
     void PFX_##gb300_destroy_set(SET s)                                               \
     {                                                                                 \
          gb_lock();                                                                   \
          gb_destroy_set((gb_set *)s);                                                 \
          gb_unlock();                                                                 \
     }

GB_SET_EXT(fftw_, fftw_plan, fftw_gb300_set, 8)
GB_SET_EXT(fftwf_, fftwf_plan, fftwf_gb300_set, 4)

int fftw_gb300_device_status(void) { return gb_device_status(); }
int fftw_gb300_tc_selftest(const void *A, const void *B, float *D, int ks) { return gb_tc_selftest(A, B, D, ks); }
