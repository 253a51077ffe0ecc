/*
 * Execution of a compiled plan: pointer classification, host staging, and
 * the pass launches.  Counterpart of the reference's execute path
 * (api/execute.c:23-27 -> plan->adt->solve -> plan_dft.apply), which here
 * becomes a sequence of kernel launches on one CUDA stream.
 *
 * Arrays may live in device memory (used in place) or in host memory
 * (copied to device staging buffers before the passes and back after).  A
 * device array whose address is not aligned to one complex element is
 * staged the same way, so every kernel sees naturally aligned data.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

typedef struct { long long lo, hi; } extent;   /* element offsets, [lo, hi] */

static extent tensor_extent(const gb_problem *prb, int which, long long *count)
{
     /* which: 0 = input tensor, 1 = output tensor */
     extent e = {0, 0};
     long long cnt = 1;
     int i;
     for (i = 0; i < prb->rank; ++i) {
          long long n = prb->sz[i].n, s = which ? prb->sz[i].os : prb->sz[i].is;
          if (i == prb->rank - 1) {
               if (prb->kind == GB_PROB_R2C && which == 1) n = n / 2 + 1;
               if (prb->kind == GB_PROB_C2R && which == 0) n = n / 2 + 1;
          }
          cnt *= n;
          if (s >= 0) e.hi += (n - 1) * s; else e.lo += (n - 1) * s;
     }
     for (i = 0; i < prb->vrank; ++i) {
          long long n = prb->vec[i].n, s = which ? prb->vec[i].os : prb->vec[i].is;
          cnt *= n;
          if (n == 0) { cnt = 0; continue; }
          if (s >= 0) e.hi += (n - 1) * s; else e.lo += (n - 1) * s;
     }
     *count = cnt;
     return e;
}

static int elsize(const gb_problem *prb, int which)
{
     int c = 2 * prb->prec;
     if (prb->kind == GB_PROB_R2C && which == 0) return prb->prec;
     if (prb->kind == GB_PROB_C2R && which == 1) return prb->prec;
     return c;
}

static int device_accessible(const void *ptr)
{
     struct cudaPointerAttributes a;
     if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
          cudaGetLastError();
          return 0;
     }
     return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

/* Page-locked host memory mapped into the device address space (what
 * fftw_malloc returns): its device address, else NULL. */
static void *mapped_host(const void *ptr)
{
     struct cudaPointerAttributes a;
     if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
          cudaGetLastError();
          return 0;
     }
     return (a.type == cudaMemoryTypeHost) ? a.devicePointer : 0;
}

static int ensure(void **buf, size_t *have, size_t need)
{
     if (*have >= need) return 0;
     /* an earlier call's copies may still be queued on the old buffer */
     if (*buf && cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("staging: %s", cudaGetErrorString(cudaGetLastError()));
          return -1;
     }
     if (*buf) cudaFree(*buf);
     *buf = 0;
     *have = 0;
     if (cudaMalloc(buf, need) != cudaSuccess) {
          cudaGetLastError();
          gb_set_error("cudaMalloc(%zu) for staging failed", need);
          return -1;
     }
     *have = need;
     return 0;
}

static int run_step(const gb_plan *p, const gb_step *s, char *bufs[4], int esz[4], int real_pairs_ok[4],
                    int direct_host)
{
     gb_pass P = s->pass;
     long long idx[GB_MAXLOOP];
     int i, done = 0;
     const int si = s->src, di = s->dst;
     if (P.kind == GB_KIND_R2C && !real_pairs_ok[si]) P.real_pairs = 0;
     else if (P.kind == GB_KIND_R2C) {
          int ok = (P.is == 1);
          for (i = 0; i < P.nv; ++i) if (P.vis[i] % 2) ok = 0;
          if (s->src_off % 2) ok = 0;
          P.real_pairs = ok;
     }
     if (P.kind == GB_KIND_C2R) {
          int ok = (P.os == 1) && real_pairs_ok[di];
          for (i = 0; i < P.nv; ++i) if (P.vos[i] % 2) ok = 0;
          if (s->dst_off % 2) ok = 0;
          P.real_pairs = ok;
     }
     if (P.variant == GB_VAR_TMA_COLS && (direct_host || ((uintptr_t)(bufs[si] + s->src_off * esz[si]) % 16) || s->nloop)) {
          /* host memory or an input not 16-byte aligned: same tile, plain loads */
          P.variant = GB_VAR_REG;
          P.smem = P.tb * gb_reg_sms(P.nfft) * 2 * P.prec;
     }
     if (P.variant == GB_VAR_TMA && (direct_host || ((uintptr_t)(bufs[si] + s->src_off * esz[si]) % 16))) {
          /* host memory or an input not 16-byte aligned: same tile, plain loads
           * (register kernel) instead of bulk copies */
          P.variant = GB_VAR_REG;
          P.smem = P.tb * gb_reg_sms(P.nfft) * 2 * P.prec;
     }
     for (i = 0; i < s->nloop; ++i) idx[i] = 0;
     while (!done) {
          long long oi = s->src_off, oo = s->dst_off;
          for (i = 0; i < s->nloop; ++i) { oi += idx[i] * s->loop[i].is; oo += idx[i] * s->loop[i].os; }
          if (P.variant == GB_VAR_TMA && ((uintptr_t)(bufs[si] + oi * esz[si]) % 16)) {
               P.variant = GB_VAR_REG;
               P.smem = P.tb * gb_reg_sms(P.nfft) * 2 * P.prec;
          }
          if (gb_launch_pass(&P, bufs[si] + oi * esz[si], bufs[di] + oo * esz[di], p->stream)) {
               gb_set_error("pass launch failed: %s", gb_last_cuda_error());
               return -1;
          }
          for (i = s->nloop - 1; i >= 0; --i) {
               if (++idx[i] < s->loop[i].n) break;
               idx[i] = 0;
          }
          if (i < 0) done = 1;
     }
     return 0;
}

/* ------------------------------------------------ pipelined host staging */

/* Input bytes per chunk: large enough that each copy runs at full link
 * speed, small enough that a long batch gives several chunks to overlap. */
#define GB_CHUNK_BYTES (96LL << 20)

/* Decide whether the batch can be cut into chunks along one vector
 * dimension d (the one with the largest input stride): every transform's
 * input and output must lie inside one stride of d (chunks are disjoint
 * byte ranges), the output of a chunk must be dense (no gaps whose host
 * values a copy-out would overwrite), and an in-place transform must use
 * the same byte range for input and output.  On success allocates three
 * device slots per side, two streams and the events, and compiles the
 * chunk plans.  Returns 1 when ready, 0 when not applicable, -1 on error. */
static int chunk_prepare(gb_plan *p, int inplace)
{
     gb_problem q = p->prb;
     const gb_problem *prb = &p->prb;
     extent ei, eo;
     long long ci, co, nd, m, bi, bo;
     int d = -1, i, j, esin = elsize(prb, 0), esout = elsize(prb, 1);
     if (p->chunk_state) return p->chunk_state > 0 ? 1 : 0;
     p->chunk_state = -1;   /* not applicable, unless set up below */
     for (i = 0; i < prb->vrank; ++i)
          if (prb->vec[i].n >= 2 && prb->vec[i].is > 0 && prb->vec[i].os > 0 &&
              (d < 0 || prb->vec[i].is * esin > prb->vec[d].is * esin))
               d = i;
     if (d < 0) return 0;
     nd = prb->vec[d].n;
     q.vec[d].n = 1;
     ei = tensor_extent(&q, 0, &ci);
     eo = tensor_extent(&q, 1, &co);
     if (ei.lo != 0 || eo.lo != 0) return 0;
     if ((ei.hi + 1) > prb->vec[d].is || (eo.hi + 1) != prb->vec[d].os || co != eo.hi + 1) return 0;
     if (inplace && prb->vec[d].is * esin != prb->vec[d].os * esout) return 0;
     if (nd * prb->vec[d].is * esin < 2 * GB_CHUNK_BYTES || prb->vec[d].is * esin > GB_CHUNK_BYTES) return 0;
     m = GB_CHUNK_BYTES / (prb->vec[d].is * esin);
     if (m < 1) m = 1;
     if (m > nd / 2) m = nd / 2;
     bi = ((m - 1) * prb->vec[d].is + ei.hi + 1) * esin;
     bo = m * prb->vec[d].os * esout;
     if (inplace && bo > bi) bi = bo;
     for (j = 0; j < GB_CHUNK_SLOTS; ++j) {
          if (cudaMalloc(&p->chunk_buf[0][j], (size_t)bi + 256) != cudaSuccess) goto fail;
          if (!inplace && cudaMalloc(&p->chunk_buf[1][j], (size_t)bo + 256) != cudaSuccess) goto fail;
     }
     p->chunk_bytes[0] = (size_t)bi;
     p->chunk_bytes[1] = (size_t)bo;
     for (i = 0; i < 2; ++i)
          if (cudaStreamCreateWithFlags((cudaStream_t *)&p->chunk_stream[i], cudaStreamNonBlocking) != cudaSuccess) goto fail;
     for (i = 0; i < 3; ++i)
          for (j = 0; j < GB_CHUNK_SLOTS; ++j)
               if (cudaEventCreateWithFlags((cudaEvent_t *)&p->chunk_ev[i][j], cudaEventDisableTiming) != cudaSuccess)
                    goto fail;
     q = p->prb;
     q.in = p->chunk_buf[0][0];
     q.out = inplace ? q.in : p->chunk_buf[1][0];
     q.vec[d].n = m;
     p->chunk_plan[0] = gb_mkplan(&q, FFTW_ESTIMATE);
     if (!p->chunk_plan[0]) return -1;
     if (nd % m) {
          q.vec[d].n = nd % m;
          p->chunk_plan[1] = gb_mkplan(&q, FFTW_ESTIMATE);
          if (!p->chunk_plan[1]) return -1;
     }
     p->chunk_dim = d;
     p->chunk_m = m;
     p->chunk_state = 1;
     return 1;
fail:
     cudaGetLastError();
     gb_set_error("device slots for pipelined staging: %s", cudaGetErrorString(cudaGetLastError()));
     return -1;
}

/* Host arrays, chunk by chunk on three streams: copy-in (H2D), the plan's
 * stream (the chunk plan's passes) and copy-out (D2H).  Slot s = c mod 3 is
 * reused by chunk c only after chunk c-3 has been transformed (input slot)
 * and copied out (output slot), which the events order on the device. */
static int chunk_execute(gb_plan *p, const char *in, char *out, int inplace)
{
     const gb_problem *prb = &p->prb;
     const int d = p->chunk_dim, esin = elsize(prb, 0), esout = elsize(prb, 1);
     const long long nd = prb->vec[d].n, m = p->chunk_m, nc = (nd + m - 1) / m;
     cudaStream_t st = (cudaStream_t)p->stream, sin_ = (cudaStream_t)p->chunk_stream[0],
                  sout = (cudaStream_t)p->chunk_stream[1];
     gb_problem q = p->prb;
     extent ei;
     long long ci, c;
     q.vec[d].n = 1;
     ei = tensor_extent(&q, 0, &ci);
     /* the caller's stream may still be writing the host input (or reading
      * an earlier output): start the copies after what is queued there */
     if (cudaEventRecord((cudaEvent_t)p->chunk_ev[2][0], st) != cudaSuccess ||
         cudaStreamWaitEvent(sin_, (cudaEvent_t)p->chunk_ev[2][0], 0) != cudaSuccess ||
         cudaStreamWaitEvent(sout, (cudaEvent_t)p->chunk_ev[2][0], 0) != cudaSuccess)
          goto cuerr;
     for (c = 0; c < nc; ++c) {
          const int s = (int)(c % GB_CHUNK_SLOTS);
          const long long mm = (c == nc - 1) ? nd - c * m : m;
          gb_plan *cp = (mm == m) ? p->chunk_plan[0] : p->chunk_plan[1];
          const size_t bin = (size_t)(((mm - 1) * prb->vec[d].is + ei.hi + 1) * esin);
          const size_t bout = (size_t)(mm * prb->vec[d].os * esout);
          const size_t oin = (size_t)(c * m * prb->vec[d].is * esin), oout = (size_t)(c * m * prb->vec[d].os * esout);
          char *slot_in = (char *)p->chunk_buf[0][s], *slot_out = inplace ? slot_in : (char *)p->chunk_buf[1][s];
          cudaEvent_t ev_in = (cudaEvent_t)p->chunk_ev[0][s], ev_tr = (cudaEvent_t)p->chunk_ev[1][s],
                      ev_out = (cudaEvent_t)p->chunk_ev[2][s];
          if (c >= GB_CHUNK_SLOTS && cudaStreamWaitEvent(sin_, inplace ? ev_out : ev_tr, 0) != cudaSuccess) goto cuerr;
          if (cudaMemcpyAsync(slot_in, in + oin, bin, cudaMemcpyHostToDevice, sin_) != cudaSuccess) goto cuerr;
          if (cudaEventRecord(ev_in, sin_) != cudaSuccess) goto cuerr;
          if (cudaStreamWaitEvent(st, ev_in, 0) != cudaSuccess) goto cuerr;
          if (c >= GB_CHUNK_SLOTS && !inplace && cudaStreamWaitEvent(st, ev_out, 0) != cudaSuccess) goto cuerr;
          cp->stream = p->stream;
          cp->async = 1;
          if (gb_execute(cp, slot_in, slot_out)) return -1;
          if (cudaEventRecord(ev_tr, st) != cudaSuccess) goto cuerr;
          if (cudaStreamWaitEvent(sout, ev_tr, 0) != cudaSuccess) goto cuerr;
          if (cudaMemcpyAsync(out + oout, slot_out, bout, cudaMemcpyDeviceToHost, sout) != cudaSuccess) goto cuerr;
          if (cudaEventRecord(ev_out, sout) != cudaSuccess) goto cuerr;
     }
     if (cudaStreamSynchronize(sout) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess ||
         cudaStreamSynchronize(sin_) != cudaSuccess)
          goto cuerr;
     return 0;
cuerr:
     gb_set_error("CUDA error during pipelined staging: %s", cudaGetErrorString(cudaGetLastError()));
     return -1;
}

/* One execute with the plan's lock held.  *sync_after = 1 asks the caller
 * to wait for the plan's stream once the lock is released (a synchronous
 * execute on device arrays): the next call may enqueue meanwhile, since the
 * stream orders it after this one. */
static int execute_locked(gb_plan *p, void *in, void *out, int *sync_after)
{
     const gb_problem *prb = &p->prb;
     long long cin, cout;
     extent ein = tensor_extent(prb, 0, &cin), eout = tensor_extent(prb, 1, &cout);
     int esin = elsize(prb, 0), esout = elsize(prb, 1);
     int cs = 2 * prb->prec;
     int inplace = (in == out);
     int stage_i, stage_o, direct_host = 0;
     char *din, *dout;
     char *bufs[4];
     int esz[4], rp[4];
     int k;
     cudaStream_t st = (cudaStream_t)p->stream;

     if (cin == 0 || cout == 0 || p->nstep == 0) {
          if (prb->rank == 0 && in != out && cin > 0) { /* rank-0 in-place is a no-op */ }
          if (p->nstep == 0) return 0;
     }
     if (gb_dry_run()) return 0;

     /* stage host arrays and device arrays not aligned to one complex element
      * (complex arrays) or to one real (real arrays) */
     stage_i = !device_accessible(in) || ((uintptr_t)in % (esin == cs ? cs : prb->prec));
     stage_o = !device_accessible(out) || ((uintptr_t)out % (esout == cs ? cs : prb->prec));
     if (inplace) stage_i = stage_o = (stage_i || stage_o);

     din = (char *)in;
     dout = (char *)out;
     /* single-pass plans on page-locked host arrays: the kernel reads and
      * writes host memory directly over the CPU-GPU link (both directions at
      * once, no staging copies) */
     if ((stage_i || stage_o) && p->nstep == 1 && !getenv("FFTW_GB300_STAGE_HOST")) {
          void *mi = stage_i ? mapped_host(in) : (void *)in, *mo = stage_o ? mapped_host(out) : out;
          if (mi && mo && ((uintptr_t)mi % (esin == cs ? cs : prb->prec)) == 0 &&
              ((uintptr_t)mo % (esout == cs ? cs : prb->prec)) == 0) {
               din = (char *)mi;
               dout = (char *)mo;
               stage_i = stage_o = 0;
               direct_host = 1;
          }
     }
     /* other host input and output (multi-pass plans, pageable memory):
      * pipelined chunks when the batch can be cut, so copies in, passes and
      * copies out overlap */
     if (!direct_host && !device_accessible(in) && !device_accessible(out) && !getenv("FFTW_GB300_STAGE_HOST")) {
          /* (a preparation that fails leaves the plan on the whole-extent
           * staging below) */
          int r = chunk_prepare(p, inplace);
          /* the slots were laid out for the in-place-ness of the first call */
          if (r > 0 && (p->chunk_buf[1][0] == 0) == inplace)
               return chunk_execute(p, (const char *)in, (char *)out, inplace);
     }
     if (inplace && stage_i) {
          long long lo = ein.lo * esin < eout.lo * esout ? ein.lo * esin : eout.lo * esout;
          long long hi = (ein.hi + 1) * esin > (eout.hi + 1) * esout ? (ein.hi + 1) * esin : (eout.hi + 1) * esout;
          size_t bytes = (size_t)(hi - lo);
          if (ensure(&p->stage_in, &p->stage_in_bytes, bytes + 256)) return -1;
          /* keep the host pointer's offset modulo 16 so alignment-dependent
           * choices see the same alignment as the planning arrays */
          if (cudaMemcpyAsync(p->stage_in, (char *)in + lo, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) goto cuerr;
          din = dout = (char *)p->stage_in - lo;
     } else {
          if (stage_i) {
               size_t bytes = (size_t)((ein.hi - ein.lo + 1) * esin);
               if (ensure(&p->stage_in, &p->stage_in_bytes, bytes + 256)) return -1;
               if (cudaMemcpyAsync(p->stage_in, (char *)in + ein.lo * esin, bytes,
                                   device_accessible(in) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st) != cudaSuccess)
                    goto cuerr;
               din = (char *)p->stage_in - ein.lo * esin;
          }
          if (stage_o) {
               size_t bytes = (size_t)((eout.hi - eout.lo + 1) * esout);
               if (ensure(&p->stage_out, &p->stage_out_bytes, bytes + 256)) return -1;
               if (cout != eout.hi - eout.lo + 1) {   /* gaps in the output: keep the caller's values */
                    if (cudaMemcpyAsync(p->stage_out, (char *)out + eout.lo * esout, bytes,
                                        device_accessible(out) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st) != cudaSuccess)
                         goto cuerr;
               }
               dout = (char *)p->stage_out - eout.lo * esout;
          }
     }

     bufs[GB_BUF_IN] = din; bufs[GB_BUF_OUT] = dout;
     bufs[GB_BUF_SCRATCH] = (char *)p->scratch; bufs[GB_BUF_SCRATCH2] = (char *)p->scratch2;
     esz[GB_BUF_IN] = esin; esz[GB_BUF_OUT] = esout; esz[GB_BUF_SCRATCH] = cs; esz[GB_BUF_SCRATCH2] = cs;
     rp[GB_BUF_IN] = ((uintptr_t)din % cs) == 0;
     rp[GB_BUF_OUT] = ((uintptr_t)dout % cs) == 0;
     rp[GB_BUF_SCRATCH] = rp[GB_BUF_SCRATCH2] = 1;
     /* element size of each buffer: r2c reads reals and writes complex;
      * c2r reads complex (its c2c passes work in place there) and writes
      * reals; scratch is complex */
     for (k = 0; k < p->nstep; ++k)
          if (run_step(p, &p->step[k], bufs, esz, rp, direct_host)) return -1;

     if (inplace && stage_i) {
          long long lo = ein.lo * esin < eout.lo * esout ? ein.lo * esin : eout.lo * esout;
          long long hi = (ein.hi + 1) * esin > (eout.hi + 1) * esout ? (ein.hi + 1) * esin : (eout.hi + 1) * esout;
          if (cudaMemcpyAsync((char *)out + lo, p->stage_in, (size_t)(hi - lo), cudaMemcpyDeviceToHost, st) != cudaSuccess) goto cuerr;
     } else if (stage_o) {
          size_t bytes = (size_t)((eout.hi - eout.lo + 1) * esout);
          if (cudaMemcpyAsync((char *)out + eout.lo * esout, p->stage_out, bytes,
                              device_accessible(out) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st) != cudaSuccess)
               goto cuerr;
     }
     if (stage_i || stage_o || direct_host) {
          if (cudaStreamSynchronize(st) != cudaSuccess) goto cuerr;
     } else if (!p->async) {
          *sync_after = 1;
     }
     return 0;
cuerr:
     gb_set_error("CUDA error during execute: %s", cudaGetErrorString(cudaGetLastError()));
     return -1;
}

/* Executes from several host threads on one plan are safe: each takes the
 * plan's lock while it enqueues (and, for host arrays, until its copies
 * are back), so the device sees the calls one after another on the plan's
 * stream and no two share the plan's scratch or staging buffers. */
int gb_execute(gb_plan *p, void *in, void *out)
{
     int sync_after = 0, r;
     pthread_mutex_lock(&p->exec_mtx);
     r = execute_locked(p, in, out, &sync_after);
     pthread_mutex_unlock(&p->exec_mtx);
     if (r == 0 && sync_after && cudaStreamSynchronize((cudaStream_t)p->stream) != cudaSuccess) {
          gb_set_error("CUDA error during execute: %s", cudaGetErrorString(cudaGetLastError()));
          return -1;
     }
     return r;
}
