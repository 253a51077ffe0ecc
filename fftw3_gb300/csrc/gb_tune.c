/*
 * Tuner: replaces the reference's measuring planner (kernel/planner.c:
 * 518-615 search, kernel/timer.c:142-181 measurement) for the choices this
 * library has for one batched 1D c2c transform of length n:
 *   - the kernel variant of a power-of-two length (bulk-copy fed persistent
 *     CTAs vs plain register kernel), and the bulk-copy pass's threads per
 *     CTA (one or two compute groups),
 *   - the radix order of a smooth, not power-of-two length (runtime-radix
 *     stages: radix 16 first, radix 8 at most, or the odd primes first),
 *   - the transforms per CTA (tile) of a single-pass kernel,
 *   - the split n = n1 * n2 of a two-pass length,
 *   - Bluestein vs Rader for a prime length.
 * Each candidate is recorded as a temporary wisdom entry, the plan is rebuilt
 * under it and timed with CUDA events on scratch device arrays (never the
 * caller's arrays, which the reference overwrites under FFTW_MEASURE,
 * kernel/timer.c:148-149); the fastest is kept in wisdom (exported with
 * fftw_export_wisdom) and the plan is rebuilt with it.  FFTW_ESTIMATE skips
 * tuning; FFTW_PATIENT / FFTW_EXHAUSTIVE try more tiles; fftw_set_timelimit
 * bounds the search.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

static double now_s(void)
{
     struct timespec ts;
     clock_gettime(CLOCK_MONOTONIC, &ts);
     return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* time one plan (ms per execute, best of reps) on scratch arrays */
static double time_plan(gb_plan *q, void *din, void *dout, int reps)
{
     cudaEvent_t a, b;
     float ms, best = 1e30f;
     int i;
     void *st = q->stream;
     int async = q->async;
     q->async = 1;
     if (gb_execute(q, din, dout)) { q->async = async; return 1e30; }
     cudaEventCreate(&a);
     cudaEventCreate(&b);
     for (i = 0; i < reps; ++i) {
          cudaEventRecord(a, (cudaStream_t)st);
          if (gb_execute(q, din, dout)) { best = 1e30f; break; }
          cudaEventRecord(b, (cudaStream_t)st);
          cudaEventSynchronize(b);
          cudaEventElapsedTime(&ms, a, b);
          if (ms < best) best = ms;
     }
     cudaEventDestroy(a);
     cudaEventDestroy(b);
     q->async = async;
     return best;
}

static size_t extent_bytes(const gb_problem *prb, int which)
{
     long long hi = 0, lo = 0;
     int i, es = 2 * prb->prec;
     for (i = 0; i < prb->rank; ++i) {
          long long n = prb->sz[i].n, s = which ? prb->sz[i].os : prb->sz[i].is;
          if (s >= 0) hi += (n - 1) * s; else lo += (n - 1) * s;
     }
     for (i = 0; i < prb->vrank; ++i) {
          long long n = prb->vec[i].n, s = which ? prb->vec[i].os : prb->vec[i].is;
          if (n > 0) { if (s >= 0) hi += (n - 1) * s; else lo += (n - 1) * s; }
     }
     return (size_t)(hi - lo + 1) * es;
}

static int is_prime_ll(long long n)
{
     long long d;
     if (n < 2) return 0;
     for (d = 2; d * d <= n; ++d) if (n % d == 0) return 0;
     return 1;
}

int gb_tune(gb_plan *p, unsigned flags)
{
     const gb_problem *prb = &p->prb;
     char key[128];
     gb_wisdom_entry cand[64], best_e;
     int nc = 0, i;
     const gb_wisdom_entry *w;
     double best = 1e30, t0 = now_s(), limit = gb_get_timelimit();
     void *din = 0, *dout = 0;
     size_t bi, bo;
     long long n;
     int reps = (flags & (FFTW_PATIENT | FFTW_EXHAUSTIVE)) ? 7 : 3;
     if (prb->kind != GB_PROB_DFT || prb->rank != 1) return 0;
     n = prb->sz[0].n;
     snprintf(key, sizeof key, "c2c p%d n%lld", prb->prec, n);
     w = gb_wisdom_lookup(key);
     if (w) return 0;   /* already tuned (or imported) */

     /* candidates */
     memset(cand, 0, sizeof cand);
     {
          int tbs[] = {1, 2, 4, 8, 16, 32, 64};
          int ntb = (flags & (FFTW_PATIENT | FFTW_EXHAUSTIVE)) ? 7 : 4;
          cand[nc].variant = -1; cand[nc].tb = 0; cand[nc].n1 = 0; ++nc;    /* the heuristic choice */
          if ((n & (n - 1)) == 0 && n >= 64 && n <= 8192) {
               cand[nc].variant = GB_VAR_REG; cand[nc].tb = 0; ++nc;       /* no bulk-copy pipeline */
               if (prb->prec == 4) {
                    /* threads per CTA of the bulk-copy pass: one or two
                     * compute groups (over two or three tile buffers) */
                    cand[nc].variant = -1; cand[nc].groups = 1; ++nc;
                    cand[nc].variant = -1; cand[nc].groups = 2; ++nc;
               }
          } else if ((n & (n - 1)) != 0) {
               /* radix order of the runtime-radix stages */
               int rad[GB_MAXRAD], o;
               for (o = 1; o < GB_RADIX_ORDERS; ++o)
                    if (gb_factor_order(n, rad, o) > 0) { cand[nc].variant = -1; cand[nc].order = o; ++nc; }
          }
          for (i = 0; i < ntb && nc < 40; ++i) {
               cand[nc].variant = -1; cand[nc].tb = tbs[i]; ++nc;
          }
          if (is_prime_ll(n)) {
               cand[nc].variant = GB_KIND_RADER; ++nc;
               cand[nc].variant = GB_KIND_BLUESTEIN; ++nc;
          } else {
               long long d;
               for (d = 2; d * d <= n && nc < 60; ++d)
                    if (n % d == 0 && n / d >= 16 && d >= 16 && n > 16384) {
                         cand[nc].variant = -1; cand[nc].n1 = (int)d; ++nc;
                    }
          }
     }
     bi = extent_bytes(prb, 0);
     bo = extent_bytes(prb, 1);
     if (cudaMalloc(&din, bi) != cudaSuccess || cudaMalloc(&dout, bo) != cudaSuccess) {
          cudaGetLastError();
          if (din) cudaFree(din);
          return 0;
     }
     cudaMemset(din, 0, bi);
     best_e = cand[0];
     for (i = 0; i < nc; ++i) {
          gb_plan *q;
          double t;
          if (limit > 0 && now_s() - t0 > limit) break;
          strcpy(cand[i].key, key);
          gb_wisdom_store(&cand[i]);
          q = gb_mkplan(prb, flags);
          if (!q) continue;
          q->stream = p->stream;
          t = time_plan(q, (char *)din + 0, (char *)dout + 0, reps);
          gb_destroy(q);
          if (t < best) { best = t; best_e = cand[i]; }
     }
     cudaFree(din);
     cudaFree(dout);
     strcpy(best_e.key, key);
     gb_wisdom_store(&best_e);
     {
          /* rebuild the plan under the chosen configuration */
          gb_plan *q = gb_mkplan(prb, flags);
          if (q) {
               gb_plan keep = *p;
               *p = *q;
               /* the plan keeps its own (unlocked: tuning runs before the
                * plan is returned) execute lock */
               p->exec_mtx = keep.exec_mtx;
               pthread_mutex_destroy(&q->exec_mtx);
               p->refcnt = keep.refcnt;
               p->stream = keep.stream;
               p->async = keep.async;
               p->measured_ms = best;
               free(q);
               if (keep.scratch) cudaFree(keep.scratch);
               if (keep.scratch2) cudaFree(keep.scratch2);
               if (keep.stage_in) cudaFree(keep.stage_in);
               if (keep.stage_out) cudaFree(keep.stage_out);
          }
     }
     return 0;
}
