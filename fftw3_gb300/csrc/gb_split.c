/*
 * Split-array plans: the real and imaginary parts of the complex side live
 * in separate real arrays and every stride counts reals.
 *   c2c (fftw_plan_guru_split_dft, fftw_execute_split_dft): always the
 *       forward DFT of x = ri + i ii into ro + i io
 *       (api/plan-guru-split-dft.h:23-38, api/execute-split-dft.c:23-27; a
 *       backward transform swaps the roles of the real and imaginary arrays)
 *   r2c (plan_guru_split_dft_r2c, execute_split_dft_r2c): real in -> ro, io
 *   c2r (plan_guru_split_dft_c2r, execute_split_dft_c2r): ri, ii -> real out
 *       (api/plan-guru-split-dft-r2c.h, api/plan-guru-split-dft-c2r.h,
 *       api/execute-split-dft-r2c.c, api/execute-split-dft-c2r.c); the
 *       complex side's last dim has n/2+1 entries.
 *
 * When c2c arrays interleave (ii = ri + 1, io = ro + 1, even strides) the
 * API layer plans them as an ordinary complex transform.  Otherwise the
 * plan here copies the input into a dense device buffer (complex pairs, or
 * reals for r2c), runs the c2c / r2c / c2r plan from it into a second dense
 * buffer, and copies that out to the caller's arrays; every copy is one
 * strided-copy kernel.  Arrays in device memory or page-locked host memory
 * are accessed in place; pageable host arrays are staged through device
 * copies of their extents.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

/* elements of the real (cplx = 0) or complex (cplx = 1) side of a split
 * problem: the complex side of r2c/c2r has n/2+1 in the last dim */
static long long split_count(const gb_plan *p, int cplx)
{
     long long t = 1;
     int d;
     for (d = 0; d < p->split_nd; ++d) {
          long long n = p->split_n[d];
          if (cplx && p->split_kind != GB_PROB_DFT && d == p->split_nd - 1) n = n / 2 + 1;
          t *= n;
     }
     return t;
}

gb_plan *gb_mksplit(int kind, int prec, int rank, const gb_dim *dims, int vrank, const gb_dim *vdims, void *ri,
                    void *ii, void *ro, void *io, unsigned flags)
{
     gb_problem q;
     gb_plan *p, *inner;
     long long din = 1, dout = 1;
     size_t b0, b1;
     int d, nd = vrank + rank;
     if (rank < 0 || vrank < 0 || rank > GB_MAXRANK || vrank > GB_MAXRANK || nd > GB_SPLIT_MAXD) return 0;
     if (kind != GB_PROB_DFT && rank < 1) return 0;
     for (d = 0; d < rank; ++d) if (dims[d].n <= 0) return 0;
     for (d = 0; d < vrank; ++d) if (vdims[d].n < 0) return 0;
     /* the inner problem: same sizes, dense row-major, vector dims outermost
      * (r2c / c2r: the complex side's last dim holds n/2+1) */
     memset(&q, 0, sizeof q);
     q.kind = kind;
     q.prec = prec;
     q.sign = kind == GB_PROB_C2R ? FFTW_BACKWARD : FFTW_FORWARD;
     q.rank = rank;
     for (d = rank - 1; d >= 0; --d) {
          const long long nr = dims[d].n, nc = (kind != GB_PROB_DFT && d == rank - 1) ? nr / 2 + 1 : nr;
          q.sz[d].n = nr;
          q.sz[d].is = din;
          q.sz[d].os = dout;
          din *= kind == GB_PROB_C2R ? nc : nr;
          dout *= kind == GB_PROB_R2C ? nc : nr;
     }
     q.vrank = vrank;
     for (d = vrank - 1; d >= 0; --d) {
          q.vec[d].n = vdims[d].n;
          q.vec[d].is = din;
          q.vec[d].os = dout;
          din *= vdims[d].n;
          dout *= vdims[d].n;
     }
     p = gb_plan_alloc();
     if (!p) return 0;
     p->flags = flags;
     p->split_kind = kind;
     p->prb.kind = kind;
     p->prb.prec = prec;
     p->prb.sign = q.sign;
     p->prb.rank = rank;
     p->prb.vrank = vrank;
     for (d = 0; d < rank; ++d) p->prb.sz[d] = dims[d];
     for (d = 0; d < vrank; ++d) p->prb.vec[d] = vdims[d];
     p->split_nd = nd;
     for (d = 0; d < vrank; ++d) {
          p->split_n[d] = vdims[d].n; p->split_is[d] = vdims[d].is; p->split_os[d] = vdims[d].os;
     }
     for (d = 0; d < rank; ++d) {
          p->split_n[vrank + d] = dims[d].n; p->split_is[vrank + d] = dims[d].is; p->split_os[vrank + d] = dims[d].os;
     }
     p->split_arr[0] = ri; p->split_arr[1] = ii; p->split_arr[2] = ro; p->split_arr[3] = io;
     /* dense buffers: complex pairs, or reals on the real side */
     b0 = (size_t)din * (size_t)prec * (kind == GB_PROB_R2C ? 1 : 2);
     b1 = (size_t)dout * (size_t)prec * (kind == GB_PROB_C2R ? 1 : 2);
     if (din > 0 && dout > 0 && !gb_dry_run()) {
          if (cudaMalloc(&p->split_buf[0], b0) != cudaSuccess || cudaMalloc(&p->split_buf[1], b1) != cudaSuccess) {
               cudaGetLastError();
               gb_set_error("cudaMalloc(%zu) for split-array buffers failed", b0 > b1 ? b0 : b1);
               gb_destroy(p);
               return 0;
          }
     }
     q.in = p->split_buf[0];
     q.out = p->split_buf[1];
     if (gb_dry_run()) { q.in = (void *)(uintptr_t)(1 << 20); q.out = (void *)(uintptr_t)(1 << 30); }
     inner = gb_mkplan(&q, flags);
     if (!inner) {
          gb_destroy(p);
          return 0;
     }
     p->split_inner = inner;
     p->nstep = inner->nstep;
     memcpy(p->step, inner->step, sizeof p->step);
     p->add = inner->add; p->mul = inner->mul; p->fma = inner->fma;
     snprintf(p->desc, sizeof p->desc, "(gb300-split-%s-%s pack %s unpack)",
              kind == GB_PROB_DFT ? "dft" : kind == GB_PROB_R2C ? "dft-r2c" : "dft-c2r", prec == 4 ? "f32" : "f64",
              inner->desc);
     return p;
}

typedef struct { long long lo, hi; } split_extent;

/* element offsets (in reals) an array of the problem touches; cplx: the
 * complex side of r2c / c2r (n/2+1 in the last dim) */
static split_extent split_span(const gb_plan *p, int out, int cplx)
{
     split_extent e = {0, 0};
     int d;
     for (d = 0; d < p->split_nd; ++d) {
          long long n = p->split_n[d], s = out ? p->split_os[d] : p->split_is[d];
          if (cplx && p->split_kind != GB_PROB_DFT && d == p->split_nd - 1) n = n / 2 + 1;
          if (n <= 0) continue;
          if (s >= 0) e.hi += (n - 1) * s; else e.lo += (n - 1) * s;
     }
     return e;
}

static int split_device(const void *ptr, void **dev)
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

/* A pair of arrays (re, im) seen from the device: in place when both are
 * device-accessible, else through staged device copies of their spans (a
 * copy-in first for outputs keeps the values in the gaps).  One staged copy
 * covers both arrays only when their spans overlap (then the union lies
 * within the caller's arrays); otherwise each array has its own, so no byte
 * outside the caller's arrays is ever copied back. */
typedef struct {
     void *re, *im;         /* device addresses used by the kernels */
     int nstage;
     void *stage[2];        /* staged spans (device) */
     char *host[2];         /* caller's address of each span's first byte */
     size_t bytes[2];
} split_pair;

static int stage_span(split_pair *sp, char *lo, char *hi, int load, cudaStream_t st)
{
     const int k = sp->nstage;
     sp->bytes[k] = (size_t)(hi - lo);
     sp->host[k] = lo;
     if (cudaMalloc(&sp->stage[k], sp->bytes[k]) != cudaSuccess) {
          cudaGetLastError();
          sp->stage[k] = 0;
          gb_set_error("cudaMalloc(%zu) for split-array staging failed", sp->bytes[k]);
          return -1;
     }
     sp->nstage = k + 1;
     if (load && cudaMemcpyAsync(sp->stage[k], lo, sp->bytes[k], cudaMemcpyDefault, st) != cudaSuccess) return -1;
     return 0;
}

static int split_pair_open(split_pair *sp, void *re, void *im, split_extent e, int es, int load, cudaStream_t st)
{
     char *r = (char *)re, *i = (char *)im;
     char *rlo = r + e.lo * es, *rhi = r + (e.hi + 1) * es, *ilo = i + e.lo * es, *ihi = i + (e.hi + 1) * es;
     memset(sp, 0, sizeof *sp);
     if (split_device(re, &sp->re) && split_device(im, &sp->im)) return 0;
     if (rlo < ihi && ilo < rhi) {
          char *lo = rlo < ilo ? rlo : ilo, *hi = rhi > ihi ? rhi : ihi;
          if (stage_span(sp, lo, hi, load, st)) return -1;
          sp->re = (char *)sp->stage[0] + (r - lo);
          sp->im = (char *)sp->stage[0] + (i - lo);
          return 0;
     }
     if (stage_span(sp, rlo, rhi, load, st) || stage_span(sp, ilo, ihi, load, st)) return -1;
     sp->re = (char *)sp->stage[0] + (r - rlo);
     sp->im = (char *)sp->stage[1] + (i - ilo);
     return 0;
}

static void split_pair_close(split_pair *sp)
{
     int k;
     for (k = 0; k < sp->nstage; ++k)
          if (sp->stage[k]) cudaFree(sp->stage[k]);
}

/* c2c: (ri, ii) -> (ro, io); r2c: a0 = real input -> (a2, a3) = (ro, io);
 * c2r: (a0, a1) = (ri, ii) -> a2 = real output */
static int execute_split_locked(gb_plan *p, void *a0, void *a1, void *a2, void *a3);

/* One call at a time per plan (its dense buffers are plan-owned); calls from
 * several host threads on one plan queue up on the plan's lock. */
int gb_execute_split(gb_plan *p, void *a0, void *a1, void *a2, void *a3)
{
     int r;
     pthread_mutex_lock(&p->exec_mtx);
     r = execute_split_locked(p, a0, a1, a2, a3);
     pthread_mutex_unlock(&p->exec_mtx);
     return r;
}

static int execute_split_locked(gb_plan *p, void *a0, void *a1, void *a2, void *a3)
{
     const int es = p->prb.prec, kind = p->split_kind;
     cudaStream_t st = (cudaStream_t)p->stream;
     split_pair in, out;
     long long nd_in[GB_SPLIT_MAXD], nd_out[GB_SPLIT_MAXD];
     long long cin, cout_;
     int d, k, rc = -1;
     const int real_in = kind == GB_PROB_R2C, real_out = kind == GB_PROB_C2R;
     if (gb_dry_run()) return 0;
     if (!p->split_inner) { gb_set_error("not a split-array plan"); return -1; }
     cin = split_count(p, !real_in);
     cout_ = split_count(p, !real_out);
     if (cin == 0 || cout_ == 0) return 0;
     for (d = 0; d < p->split_nd; ++d) {
          const int last = d == p->split_nd - 1 && kind != GB_PROB_DFT;
          nd_in[d] = (last && !real_in) ? p->split_n[d] / 2 + 1 : p->split_n[d];
          nd_out[d] = (last && !real_out) ? p->split_n[d] / 2 + 1 : p->split_n[d];
     }
     memset(&in, 0, sizeof in);
     memset(&out, 0, sizeof out);
     if (split_pair_open(&in, a0, real_in ? a0 : a1, split_span(p, 0, !real_in), es, 1, st)) goto done;
     if (split_pair_open(&out, a2, real_out ? a2 : a3, split_span(p, 1, !real_out), es, 1, st)) goto done;
     if (gb_split_copy(1, es, p->split_nd, nd_in, p->split_is, cin, in.re, real_in ? 0 : in.im, p->split_buf[0],
                       st)) {
          gb_set_error("split pack failed: %s", gb_last_cuda_error());
          goto done;
     }
     p->split_inner->stream = p->stream;
     p->split_inner->async = 1;
     if (gb_execute(p->split_inner, p->split_buf[0], p->split_buf[1])) goto done;
     if (gb_split_copy(0, es, p->split_nd, nd_out, p->split_os, cout_, out.re, real_out ? 0 : out.im,
                       p->split_buf[1], st)) {
          gb_set_error("split unpack failed: %s", gb_last_cuda_error());
          goto done;
     }
     for (k = 0; k < out.nstage; ++k)
          if (cudaMemcpyAsync(out.host[k], out.stage[k], out.bytes[k], cudaMemcpyDefault, st) != cudaSuccess)
               goto done;
     if ((in.nstage || out.nstage || !p->async) && cudaStreamSynchronize(st) != cudaSuccess) goto done;
     rc = 0;
done:
     if (rc) {
          cudaError_t e = cudaGetLastError();
          if (e != cudaSuccess) gb_set_error("CUDA error in split execute: %s", cudaGetErrorString(e));
     }
     if (in.nstage || out.nstage) cudaStreamSynchronize(st);
     split_pair_close(&in);
     split_pair_close(&out);
     return rc;
}
