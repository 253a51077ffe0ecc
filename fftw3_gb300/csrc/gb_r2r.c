/*
 * Real-to-real transforms (fftw_plan_r2r_1d/2d/3d, plan_r2r, plan_many_r2r
 * and the guru r2r planners; kinds as api/fftw3.h:96-100).  A transform of
 * rank r is the separable product of 1D r2r transforms along its dims
 * (doc/reference.texi, "Real-to-Real Transforms"), run as one stage per dim,
 * last dim first; every stage is a pre kernel, one core transform of length
 * L on dense buffers and a post kernel (fft_r2r.cu), with the definitions of
 * doc/reference.texi:
 *   R2HC    r2c, then the halfcomplex packing: y_k = Re Y_k (k <= n/2),
 *           y_{n-k} = Im Y_k                        (reference.texi:1923-2020)
 *   HC2R    unpack the halfcomplex array into the half spectrum, then c2r
 *   DHT     r2c, then y_k = Re Y_k - Im Y_k over the full (Hermitian) spectrum
 *   REDFT00 (DCT-I)   r2c of the even extension of length 2(n-1), y_k = Re E_k
 *                                                    (reference.texi:2072-2085)
 *   REDFT10 (DCT-II)  v = even-indexed x then odd-indexed x reversed, r2c,
 *           y_k = 2 Re(exp(-i pi k / 2n) V_k)         (reference.texi:2022-2175)
 *   REDFT01 (DCT-III) V_k = (x_k - i x_{n-k}) exp(i pi k / 2n), c2r,
 *           y_{2m} = v_m, y_{2m+1} = v_{n-1-m}
 *   REDFT11 (DCT-IV)  even n: z_m = (x_{2m} + i x_{n-1-2m}) exp(-i pi (4m+1)/4n),
 *           complex DFT of n/2, u_p = Z_p exp(-i pi p / n), y_{2p} = 2 Re u_p,
 *           y_{n-1-2p} = -2 Im u_p;  odd n: complex DFT of length 2n of
 *           x_m exp(-i pi m / 2n) zero-padded, y_k = 2 Re(Z_k exp(-i pi (2k+1)/4n))
 *   RODFT00 (DST-I)   r2c of the odd extension of length 2(n+1),
 *           y_k = -Im O_{k+1}                        (reference.texi:2225-2240)
 *   RODFT10 (DST-II)  DCT-II of (-1)^j x_j, output reversed  (reference.texi:2176-2300)
 *   RODFT01 (DST-III) (-1)^k DCT-III of x reversed
 *   RODFT11 (DST-IV)  (-1)^k DCT-IV of x reversed
 * (the reductions of DCT-II/III to one real DFT of length n are Makhoul's;
 * DCT-IV through a complex DFT of n/2 is the standard half-length form).
 * A size-1 REDFT00 is not defined and returns NULL, as in the reference
 * (reference.texi:820-821).  Rank 0 is a copy of the howmany elements
 * (through a dense buffer, so in-place and overlapping layouts are safe).
 * Arrays in device or page-locked host memory are used in place; pageable
 * host arrays are staged through device copies of their extents.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

static int r2r_supported(int kind) { return kind >= FFTW_R2HC && kind <= FFTW_RODFT11; }

/* reals per transform the pre kernel writes (in) / the post kernel reads (out) */
static long long r2r_core_reals(int core, long long L, int out)
{
     if (core == GB_R2R_CORE_C2C) return 2 * L;
     if ((core == GB_R2R_CORE_R2C) == (out != 0)) return 2 * (L / 2 + 1);
     return L;
}

/* the vector loop of a stage: drop length-1 dims, merge neighbours that
 * are contiguous on both sides */
static void r2r_vec_compress(gb_r2r_vec *v)
{
     int i, k = 0;
     for (i = 0; i < v->nv; ++i) {
          if (v->n[i] == 1) continue;
          if (k > 0 && v->n[i] > 0 && v->is[k - 1] == v->n[i] * v->is[i] && v->os[k - 1] == v->n[i] * v->os[i]) {
               v->n[k - 1] *= v->n[i];
               v->is[k - 1] = v->is[i];
               v->os[k - 1] = v->os[i];
               continue;
          }
          v->n[k] = v->n[i]; v->is[k] = v->is[i]; v->os[k] = v->os[i];
          ++k;
     }
     v->nv = k;
}

gb_plan *gb_mkr2r(int prec, int rank, const gb_dim *dims, const int *kinds, int vrank, const gb_dim *vdims, void *in,
                  void *out, unsigned flags)
{
     gb_plan *p;
     long long dsz[GB_MAXRANK], dvec[GB_MAXRANK], total = 1, tr = 1;
     size_t bytes = 0;
     int d, e, i, len;
     if (rank < 0 || rank > GB_MAXRANK || vrank < 0 || vrank > GB_MAXRANK) {
          gb_set_error("r2r rank %d / howmany rank %d is not provided by this library", rank, vrank);
          return 0;
     }
     for (d = 0; d < rank; ++d) {
          if (dims[d].n <= 0) return 0;
          if (!r2r_supported(kinds[d])) {
               gb_set_error("r2r kind %d is not an fftw_r2r_kind", kinds[d]);
               return 0;
          }
          if (kinds[d] == FFTW_REDFT00 && dims[d].n == 1) {
               gb_set_error("a size-1 REDFT00 is not defined");
               return 0;
          }
     }
     for (d = 0; d < vrank; ++d) if (vdims[d].n < 0) return 0;
     p = gb_plan_alloc();
     if (!p) return 0;
     p->flags = flags;
     p->prb.kind = GB_PROB_R2R;
     p->prb.prec = prec;
     p->prb.rank = rank;
     for (d = 0; d < rank; ++d) p->prb.sz[d] = dims[d];
     p->prb.vrank = vrank;
     for (d = 0; d < vrank; ++d) p->prb.vec[d] = vdims[d];
     p->prb.in = in; p->prb.out = out;
     /* dense row-major strides of the intermediate: vector dims outermost */
     for (d = rank - 1; d >= 0; --d) { dsz[d] = tr; tr *= dims[d].n; }
     total = tr;
     for (d = vrank - 1; d >= 0; --d) { dvec[d] = total; total *= vdims[d].n; }
     p->r2r_naxis = rank;
     p->r2r_ax = (gb_r2r_axis *)calloc((size_t)(rank > 0 ? rank : 1), sizeof *p->r2r_ax);
     if (!p->r2r_ax) { gb_destroy(p); return 0; }
     if (rank == 0) bytes = (size_t)total * (size_t)prec;   /* the copy's dense buffer */
     for (i = 0; i < rank; ++i) {
          gb_r2r_axis *a = &p->r2r_ax[i];
          gb_r2r_vec *v = &a->vec;
          d = rank - 1 - i;
          a->kind = kinds[d];
          a->n = dims[d].n;
          a->core = gb_r2r_core(a->kind, a->n, &a->L);
          a->src_mid = i > 0;
          a->dst_mid = i < rank - 1;
          a->is = a->src_mid ? dsz[d] : dims[d].is;
          a->os = a->dst_mid ? dsz[d] : dims[d].os;
          v->nv = 0;
          for (e = 0; e < vrank; ++e) {
               v->n[v->nv] = vdims[e].n;
               v->is[v->nv] = a->src_mid ? dvec[e] : vdims[e].is;
               v->os[v->nv] = a->dst_mid ? dvec[e] : vdims[e].os;
               v->nv++;
          }
          for (e = 0; e < rank; ++e) {
               if (e == d) continue;
               v->n[v->nv] = dims[e].n;
               v->is[v->nv] = a->src_mid ? dsz[e] : dims[e].is;
               v->os[v->nv] = a->dst_mid ? dsz[e] : dims[e].os;
               v->nv++;
          }
          r2r_vec_compress(v);
          a->V = 1;
          for (e = 0; e < v->nv; ++e) a->V *= v->n[e];
          if (a->V > 0) {
               const size_t b0 = (size_t)(a->V * r2r_core_reals(a->core, a->L, 0)) * (size_t)prec;
               const size_t b1 = (size_t)(a->V * r2r_core_reals(a->core, a->L, 1)) * (size_t)prec;
               if (b0 > bytes) bytes = b0;
               if (b1 > bytes) bytes = b1;
          }
     }
     if (total > 0 && !gb_dry_run()) {
          if (cudaMalloc(&p->r2r_buf[0], bytes) != cudaSuccess ||
              (rank > 0 && cudaMalloc(&p->r2r_buf[1], bytes) != cudaSuccess) ||
              (rank > 1 && cudaMalloc(&p->r2r_mid, (size_t)total * (size_t)prec) != cudaSuccess)) {
               cudaGetLastError();
               gb_set_error("cudaMalloc(%zu) for r2r buffers failed", bytes);
               gb_destroy(p);
               return 0;
          }
     }
     len = snprintf(p->desc, sizeof p->desc, "(gb300-r2r-%s%s", prec == 4 ? "f32" : "f64", rank ? "" : " copy");
     for (i = 0; i < rank && total > 0; ++i) {
          gb_r2r_axis *a = &p->r2r_ax[i];
          gb_problem q;
          int s;
          memset(&q, 0, sizeof q);
          q.prec = prec;
          q.rank = 1;
          q.sz[0].n = a->L; q.sz[0].is = 1; q.sz[0].os = 1;
          q.vrank = 1;
          q.vec[0].n = a->V;
          if (a->core == GB_R2R_CORE_C2C) {
               q.kind = GB_PROB_DFT; q.sign = FFTW_FORWARD;
               q.vec[0].is = a->L; q.vec[0].os = a->L;
          } else if (a->core == GB_R2R_CORE_C2R) {
               q.kind = GB_PROB_C2R; q.sign = FFTW_BACKWARD;
               q.vec[0].is = a->L / 2 + 1; q.vec[0].os = a->L;
          } else {
               q.kind = GB_PROB_R2C; q.sign = FFTW_FORWARD;
               q.vec[0].is = a->L; q.vec[0].os = a->L / 2 + 1;
          }
          q.in = p->r2r_buf[0];
          q.out = p->r2r_buf[1];
          if (gb_dry_run()) { q.in = (void *)(uintptr_t)(1 << 20); q.out = (void *)(uintptr_t)(1 << 30); }
          a->inner = gb_mkplan(&q, flags);
          if (!a->inner) {
               gb_destroy(p);
               return 0;
          }
          if (gb_r2r_table_len(a->kind, a->n) > 0 && !gb_dry_run()) {
               /* the stage's twiddles, once, on the legacy stream before any execute */
               const size_t tb = (size_t)gb_r2r_table_len(a->kind, a->n) * 2 * (size_t)prec;
               if (cudaMalloc(&a->tw, tb) != cudaSuccess || gb_r2r_table(prec, a->kind, a->n, a->tw, 0) ||
                   cudaStreamSynchronize(0) != cudaSuccess) {
                    cudaGetLastError();
                    gb_set_error("r2r twiddle table (%zu bytes) failed", tb);
                    gb_destroy(p);
                    return 0;
               }
          }
          /* REDFT10 of unit-stride rows whose starts are 16-byte aligned, of a
           * power-of-two length the bulk-copy kernel takes: the permuted load,
           * the r2c and the cosine post-twiddle in one pass (one read and one
           * write of the array instead of three of each) */
          if (a->kind == FFTW_REDFT10 && a->is == 1 && a->os == 1 && a->n >= 128 && a->n <= 16384 &&
              (a->n & (a->n - 1)) == 0 && a->vec.nv >= 1 && a->vec.nv <= GB_MAXV && (a->tw || gb_dry_run())) {
               gb_dim vd[GB_MAXV];
               int ok = 1;
               for (e = 0; e < a->vec.nv; ++e) {
                    vd[e].n = a->vec.n[e]; vd[e].is = a->vec.is[e]; vd[e].os = a->vec.os[e];
                    if ((a->vec.is[e] * prec) % 16) ok = 0;
               }
               if (ok && gb_config_pass(&a->fpass, prec, GB_KIND_R2C, a->n, -1, 1, 1, a->vec.nv, vd) == 0 &&
                   a->fpass.variant == GB_VAR_TMA && gb_pass_tables(&a->fpass) == 0) {
                    a->fpass.kind = GB_KIND_DCT2;
                    a->fpass.chirp = a->tw;
                    a->fused = 1;
               }
          }
          for (s = 0; s < a->inner->nstep && p->nstep < GB_MAXPASS; ++s) p->step[p->nstep++] = a->inner->step[s];
          p->add += a->inner->add; p->mul += a->inner->mul; p->fma += a->inner->fma;
          if (len < (int)sizeof p->desc)
               len += snprintf(p->desc + len, sizeof p->desc - (size_t)len, " (dim %d kind %d n %lld %s%s post)",
                               rank - 1 - i, a->kind, a->n, a->fused ? "fused-dct2 or pre " : "pre ",
                               a->inner->desc);
     }
     if (len < (int)sizeof p->desc) snprintf(p->desc + len, sizeof p->desc - (size_t)len, ")");
     return p;
}

/* the core plans, for the tuner */
int gb_r2r_tune(gb_plan *p, unsigned flags)
{
     int i, rc = 0;
     for (i = 0; i < p->r2r_naxis; ++i)
          if (p->r2r_ax[i].inner && gb_tune(p->r2r_ax[i].inner, flags)) rc = -1;
     return rc;
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

/* device (or managed) memory, which the bulk-copy kernels may read */
static int r2r_in_hbm(const void *ptr)
{
     struct cudaPointerAttributes a;
     if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
          cudaGetLastError();
          return 0;
     }
     return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

/* element span [lo, hi] (in reals) the problem touches on the input (out = 0)
 * or output side */
static void r2r_span(const gb_problem *q, int out, long long *lo, long long *hi)
{
     int d;
     *lo = 0; *hi = 0;
     for (d = 0; d < q->rank + q->vrank; ++d) {
          const gb_dim *g = d < q->rank ? &q->sz[d] : &q->vec[d - q->rank];
          const long long s = out ? g->os : g->is;
          if (g->n <= 0) continue;
          if (s >= 0) *hi += (g->n - 1) * s; else *lo += (g->n - 1) * s;
     }
}

static int execute_r2r_locked(gb_plan *p, void *in, void *out);

/* One call at a time per plan (its core buffers and intermediate are
 * plan-owned); calls from several host threads queue up on the plan's lock. */
int gb_execute_r2r(gb_plan *p, void *in, void *out)
{
     int r;
     pthread_mutex_lock(&p->exec_mtx);
     r = execute_r2r_locked(p, in, out);
     pthread_mutex_unlock(&p->exec_mtx);
     return r;
}

static int execute_r2r_locked(gb_plan *p, void *in, void *out)
{
     const int prec = p->prb.prec;
     cudaStream_t st = (cudaStream_t)p->stream;
     void *din = 0, *dout = 0, *sin_ = 0, *sout = 0;
     long long ilo, ihi, olo, ohi, total = 1;
     size_t ib, ob;
     int d, i, rc = -1;
     for (d = 0; d < p->prb.rank; ++d) total *= p->prb.sz[d].n;
     for (d = 0; d < p->prb.vrank; ++d) total *= p->prb.vec[d].n;
     if (gb_dry_run() || total == 0) return 0;
     if (!p->r2r_ax) { gb_set_error("not an r2r plan"); return -1; }
     r2r_span(&p->prb, 0, &ilo, &ihi);
     r2r_span(&p->prb, 1, &olo, &ohi);
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
     if (p->r2r_naxis == 0) {
          /* rank 0: copy the howmany elements through the dense buffer */
          long long vn[GB_SPLIT_MAXD], vis[GB_SPLIT_MAXD], vos[GB_SPLIT_MAXD];
          const int nv = p->prb.vrank;
          for (d = 0; d < nv; ++d) { vn[d] = p->prb.vec[d].n; vis[d] = p->prb.vec[d].is; vos[d] = p->prb.vec[d].os; }
          if (gb_split_copy(1, prec, nv, vn, vis, total, din, 0, p->r2r_buf[0], st) ||
              gb_split_copy(0, prec, nv, vn, vos, total, dout, 0, p->r2r_buf[0], st)) {
               gb_set_error("r2r copy failed: %s", gb_last_cuda_error());
               goto done;
          }
     }
     for (i = 0; i < p->r2r_naxis; ++i) {
          gb_r2r_axis *a = &p->r2r_ax[i];
          const void *src = a->src_mid ? p->r2r_mid : din;
          void *dst = a->dst_mid ? p->r2r_mid : dout;
          if (a->fused && ((uintptr_t)src % 16) == 0 && r2r_in_hbm(src) && r2r_in_hbm(dst)) {
               /* the bulk copies read device memory at 16-byte aligned rows */
               if (gb_launch_pass(&a->fpass, src, dst, st)) {
                    gb_set_error("r2r pass launch failed: %s", gb_last_cuda_error());
                    goto done;
               }
               continue;
          }
          if (gb_r2r_pre(prec, a->kind, a->n, a->V, src, a->is, &a->vec, p->r2r_buf[0], a->tw, st)) goto done;
          a->inner->stream = p->stream;
          a->inner->async = 1;
          if (gb_execute(a->inner, p->r2r_buf[0], p->r2r_buf[1])) goto done;
          if (gb_r2r_post(prec, a->kind, a->n, a->V, p->r2r_buf[1], dst, a->os, &a->vec, a->tw, st)) goto done;
     }
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
