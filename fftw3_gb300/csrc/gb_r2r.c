/*
 * 1D real-to-real transforms (fftw_plan_r2r_1d, plan_many_r2r and the guru
 * r2r planners of rank 1; kinds as api/fftw3.h:96-100), each run as one
 * real DFT of the same length n between a pre- and a post-processing
 * kernel (fft_r2r.cu), with the definitions of doc/reference.texi:
 *   R2HC    r2c, then the halfcomplex packing: y_k = Re Y_k (k <= n/2),
 *           y_{n-k} = Im Y_k                        (reference.texi:1923-2020)
 *   HC2R    unpack the halfcomplex array into the half spectrum, then c2r
 *   DHT     r2c, then y_k = Re Y_k - Im Y_k over the full (Hermitian) spectrum
 *   REDFT10 (DCT-II)  v = even-indexed x then odd-indexed x reversed, r2c,
 *           y_k = 2 Re(exp(-i pi k / 2n) V_k)         (reference.texi:2022-2175)
 *   REDFT01 (DCT-III) V_k = (x_k - i x_{n-k}) exp(i pi k / 2n), c2r,
 *           y_{2m} = v_m, y_{2m+1} = v_{n-1-m}
 *   RODFT10 (DST-II)  DCT-II of (-1)^j x_j, output reversed  (reference.texi:2176-2300)
 *   RODFT01 (DST-III) (-1)^k DCT-III of x reversed
 * (the reduction of DCT-II/III to one real DFT of length n is Makhoul's).
 * The other kinds (REDFT00/11, RODFT00/11) and multi-dimensional r2r return
 * NULL.  Arrays in device or page-locked host memory are used in place;
 * pageable host arrays are staged through device copies of their extents.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

static int r2r_supported(int kind)
{
     return kind == FFTW_R2HC || kind == FFTW_HC2R || kind == FFTW_DHT || kind == FFTW_REDFT10 ||
            kind == FFTW_REDFT01 || kind == FFTW_RODFT10 || kind == FFTW_RODFT01;
}

static int r2r_backward_core(int kind) { return kind == FFTW_HC2R || kind == FFTW_REDFT01 || kind == FFTW_RODFT01; }

gb_plan *gb_mkr2r(int prec, int kind, long long n, long long hm, long long is, long long idist, long long os,
                  long long odist, void *in, void *out, unsigned flags)
{
     gb_problem q;
     gb_plan *p;
     const long long nc = n / 2 + 1;
     if (!r2r_supported(kind)) {
          gb_set_error("r2r kind %d is not provided by this library (REDFT00/11, RODFT00/11)", kind);
          return 0;
     }
     if (n <= 0 || hm < 0) return 0;
     p = (gb_plan *)calloc(1, sizeof *p);
     if (!p) return 0;
     p->refcnt = 1;
     p->flags = flags;
     p->prb.kind = GB_PROB_R2R;
     p->prb.prec = prec;
     p->prb.rank = 1;
     p->prb.sz[0].n = n; p->prb.sz[0].is = is; p->prb.sz[0].os = os;
     p->prb.vrank = 1;
     p->prb.vec[0].n = hm; p->prb.vec[0].is = idist; p->prb.vec[0].os = odist;
     p->prb.in = in; p->prb.out = out;
     p->r2r_kind = kind;
     if (hm > 0 && !gb_dry_run()) {
          const size_t b0 = (size_t)(hm * n) * (size_t)prec, b1 = (size_t)(hm * nc) * 2 * (size_t)prec;
          const size_t bytes = b0 > b1 ? b0 : b1;
          if (cudaMalloc(&p->r2r_buf[0], bytes) != cudaSuccess || cudaMalloc(&p->r2r_buf[1], bytes) != cudaSuccess) {
               cudaGetLastError();
               gb_set_error("cudaMalloc(%zu) for r2r buffers failed", bytes);
               gb_destroy(p);
               return 0;
          }
     }
     /* the real DFT of length n on the dense buffers: r2c [hm][n] -> [hm][nc],
      * or c2r [hm][nc] -> [hm][n] */
     memset(&q, 0, sizeof q);
     q.prec = prec;
     q.rank = 1;
     q.sz[0].n = n; q.sz[0].is = 1; q.sz[0].os = 1;
     q.vrank = 1;
     q.vec[0].n = hm > 0 ? hm : 1;
     if (r2r_backward_core(kind)) {
          q.kind = GB_PROB_C2R; q.sign = FFTW_BACKWARD;
          q.vec[0].is = nc; q.vec[0].os = n;
     } else {
          q.kind = GB_PROB_R2C; q.sign = FFTW_FORWARD;
          q.vec[0].is = n; q.vec[0].os = nc;
     }
     q.in = p->r2r_buf[0];
     q.out = p->r2r_buf[1];
     if (gb_dry_run()) { q.in = (void *)(uintptr_t)(1 << 20); q.out = (void *)(uintptr_t)(1 << 30); }
     p->r2r_inner = gb_mkplan(&q, flags);
     if (!p->r2r_inner) {
          gb_destroy(p);
          return 0;
     }
     p->nstep = p->r2r_inner->nstep;
     memcpy(p->step, p->r2r_inner->step, sizeof p->step);
     p->add = p->r2r_inner->add; p->mul = p->r2r_inner->mul; p->fma = p->r2r_inner->fma;
     snprintf(p->desc, sizeof p->desc, "(gb300-r2r-%s kind %d n %lld pre %s post)", prec == 4 ? "f32" : "f64", kind, n,
              p->r2r_inner->desc);
     return p;
}

static int r2r_device(const void *ptr, void **dev)
{
     struct cudaPointerAttributes a;
     if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
          cudaGetLastError();
          return 0;
     }
     if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) { *dev = (void *)ptr; return 1; }
     if (a.type == cudaMemoryTypeHost && a.devicePointer) { *dev = a.devicePointer; return 1; }
     return 0;
}

/* element span [lo, hi] (in reals) of n elements at stride s for hm transforms at distance d */
static void r2r_span(long long n, long long s, long long hm, long long d, long long *lo, long long *hi)
{
     *lo = 0; *hi = 0;
     if (s >= 0) *hi += (n - 1) * s; else *lo += (n - 1) * s;
     if (hm > 0) { if (d >= 0) *hi += (hm - 1) * d; else *lo += (hm - 1) * d; }
}

int gb_execute_r2r(gb_plan *p, void *in, void *out)
{
     const int prec = p->prb.prec, kind = p->r2r_kind;
     const long long n = p->prb.sz[0].n, is = p->prb.sz[0].is, os = p->prb.sz[0].os;
     const long long hm = p->prb.vec[0].n, idist = p->prb.vec[0].is, odist = p->prb.vec[0].os;
     cudaStream_t st = (cudaStream_t)p->stream;
     void *din = 0, *dout = 0, *sin_ = 0, *sout = 0;
     long long ilo, ihi, olo, ohi;
     size_t ib, ob;
     int rc = -1;
     if (gb_dry_run() || hm == 0) return 0;
     if (!p->r2r_inner) { gb_set_error("not an r2r plan"); return -1; }
     r2r_span(n, is, hm, idist, &ilo, &ihi);
     r2r_span(n, os, hm, odist, &olo, &ohi);
     ib = (size_t)(ihi - ilo + 1) * prec;
     ob = (size_t)(ohi - olo + 1) * prec;
     if (!r2r_device(in, &din)) {
          if (cudaMalloc(&sin_, ib) != cudaSuccess ||
              cudaMemcpyAsync(sin_, (char *)in + ilo * prec, ib, cudaMemcpyDefault, st) != cudaSuccess)
               goto done;
          din = (char *)sin_ - ilo * prec;
     }
     if (!r2r_device(out, &dout)) {
          /* copy-in first: gaps in the output keep the caller's values */
          if (cudaMalloc(&sout, ob) != cudaSuccess ||
              cudaMemcpyAsync(sout, (char *)out + olo * prec, ob, cudaMemcpyDefault, st) != cudaSuccess)
               goto done;
          dout = (char *)sout - olo * prec;
     }
     if (gb_r2r_pre(prec, kind, n, hm, din, is, idist, p->r2r_buf[0], st)) goto done;
     p->r2r_inner->stream = p->stream;
     p->r2r_inner->async = 1;
     if (gb_execute(p->r2r_inner, p->r2r_buf[0], p->r2r_buf[1])) goto done;
     if (gb_r2r_post(prec, kind, n, hm, p->r2r_buf[1], dout, os, odist, st)) goto done;
     if (sout && cudaMemcpyAsync((char *)out + olo * prec, sout, ob, cudaMemcpyDefault, st) != cudaSuccess) goto done;
     if ((sin_ || sout || !p->async) && cudaStreamSynchronize(st) != cudaSuccess) goto done;
     rc = 0;
done:
     if (rc) {
          cudaError_t e = cudaGetLastError();
          if (e != cudaSuccess) gb_set_error("CUDA error in r2r execute: %s", cudaGetErrorString(e));
     }
     if (sin_ || sout) cudaStreamSynchronize(st);
     if (sin_) cudaFree(sin_);
     if (sout) cudaFree(sout);
     return rc;
}
