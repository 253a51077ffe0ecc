/*
 * The FFT pass kernels.  One launch runs one gb_pass: a batch of 1D
 * transforms of one length, each read from HBM once and written once.
 *
 *   k_reg  -- power-of-two nfft <= 16384: each thread owns E = min(16, nfft)
 *             elements in registers; stages of radix <= 16 exchange through
 *             padded shared memory.  Kinds: c2c (with the optional four-step
 *             output twiddle), r2c (hc2c post-pass fused after the last
 *             stage), c2r (hc2c pre-pass fused before the first stage),
 *             Bluestein (any n with a power-of-two convolution length: chirp
 *             multiply, FFT, spectrum multiply, inverse FFT, chirp multiply,
 *             all inside one CTA).
 *   k_gen  -- any length whose factors are in {2,3,4,5,7,8,11,13,16}: stages
 *             ping-pong between two shared-memory buffers with a runtime
 *             radix list.  Kinds: c2c, r2c, c2r (even n through the half-length
 *             complex FFT, odd n through the full-length one), Rader
 *             (prime n with a smooth n-1: permute by generator powers,
 *             convolve with omega through FFT(n-1), unpermute) and
 *             Bluestein; the tile body (gen_tile) is shared with the
 *             work-queue kernel.
 *
 * These replace, on the reference side: dft/ct.c + dft/dftw-direct.c +
 * dft/direct.c with their codelets (the stages), dft/vrank-geq1.c (the batch
 * is the grid), dft/buffered.c and dft/indirect*.c (strided tiles are staged
 * through shared memory), rdft/ct-hc2c.c + rdft/ct-hc2c-direct.c (fused
 * pre/post-passes), dft/generic.c (small prime radices as register
 * butterflies), dft/bluestein.c and dft/rader.c (fused convolutions).
 */
#pragma once
#include "fft_device.cuh"
#include "gb_types.h"

namespace gb {

/* Shared-memory swizzle of k_reg: one (or two) padding elements after every
 * 16.  Two when the first stage is radix 16, so its 16 consecutive outputs
 * stay 16-byte aligned and go out as 128-bit stores; both choices keep the
 * strided stage accesses free of bank conflicts (checked by enumerating the
 * addresses of every warp). */
__host__ __device__ constexpr int pad_mult(int nfft)
{
     int r = nfft;
     while (r > 16) r /= 16;
     return (r == 16 && nfft >= 256) ? 2 : 1;
}
__host__ __device__ constexpr int pad_for(int nfft, int p) { return p + pad_mult(nfft) * (p >> 4); }

/* Shared-memory stride (in complex elements) of one transform in k_reg
 * (the host planner's gb_reg_sms computes the same value). */
__host__ __device__ constexpr int reg_sms(int nfft) { return (nfft + pad_mult(nfft) * (nfft >> 4) + 3) & ~1; }

__host__ __device__ constexpr int reg_e(int nfft) { return nfft < 16 ? nfft : 16; }

__host__ __device__ constexpr int reg_r0(int nfft)
{
     int r = nfft;
     while (r > 16) r /= 16;
     return r;
}

/* Offsets of the tile: the outer vector dimensions (1..nv-1) decoded from the
 * tile index; dimension 0 is tiled by tb. */
struct tile_t {
     long long bi, bo;   /* offsets contributed by dims 1.. */
     long long v0;       /* first index along dim 0 */
     long long vpost;    /* index along dim post_vdim (>= 1) of a four-step pass */
};

__device__ __forceinline__ tile_t tile_of(const gb_pass &P, long long blk)
{
     tile_t t;
     t.bi = 0; t.bo = 0; t.vpost = 0;
     if (P.nblocks <= 0x7fffffffLL) {
          /* every index fits 32 bits: 32-bit divisions, a few times cheaper
           * than the 64-bit ones every thread would otherwise run per tile */
          unsigned rest = (unsigned)blk / (unsigned)P.ntiles0;
          t.v0 = (long long)((unsigned)blk - rest * (unsigned)P.ntiles0) * P.tb;
#pragma unroll
          for (int d = 1; d < GB_MAXV; ++d) {
               if (d < P.nv) {
                    const unsigned q = rest / (unsigned)P.vn[d];
                    const long long i = rest - q * (unsigned)P.vn[d];
                    rest = q;
                    t.bi += i * P.vis[d];
                    t.bo += i * P.vos[d];
                    if (d == P.post_vdim) t.vpost = i;
               }
          }
          return t;
     }
     long long rest = blk / P.ntiles0;
     t.v0 = (blk - rest * P.ntiles0) * P.tb;
#pragma unroll
     for (int d = 1; d < GB_MAXV; ++d) {
          if (d < P.nv) {
               long long q = rest / P.vn[d];
               long long i = rest - q * P.vn[d];
               rest = q;
               t.bi += i * P.vis[d];
               t.bo += i * P.vos[d];
               if (d == P.post_vdim) t.vpost = i;
          }
     }
     return t;
}

/* ---- element access: complex data, or pairs of real data ---------------- */

template <typename C> struct io {
     typedef typename real_of<C>::T R;
     /* complex element j of a transform that starts at 'base' (complex units) */
     static __device__ __forceinline__ C ldc(const void *p, long long base, long long j, long long s)
     {
          return ((const C *)p)[base + j * s];
     }
     static __device__ __forceinline__ void stc(void *p, long long base, long long j, long long s, C v)
     {
          ((C *)p)[base + j * s] = v;
     }
     /* pair j of a real transform: (x[2j*s], x[(2j+1)*s]), base in real units */
     static __device__ __forceinline__ C ldpair(const void *p, long long base, long long j, long long s, int pairs)
     {
          if (pairs) return ((const C *)((const R *)p + base))[j];
          const R *r = (const R *)p + base;
          return mk<C>(r[2 * j * s], r[(2 * j + 1) * s]);
     }
     static __device__ __forceinline__ void stpair(void *p, long long base, long long j, long long s, int pairs, C v)
     {
          if (pairs) { ((C *)((R *)p + base))[j] = v; return; }
          R *r = (R *)p + base;
          r[2 * j * s] = v.x;
          r[(2 * j + 1) * s] = v.y;
     }
};

/* exp(sign 2 pi i m / N) from the two-level table (four-step twiddle);
 * callers pass m = v * k with v < n2 and k < n1, so m < N. */
template <typename C> __device__ __forceinline__ C post_twiddle(const gb_pass &P, long long m)
{
     const long long hi = m >> P.post_lS, lo = m & (P.post_S - 1);
     C a = __ldg((const C *)P.post_lo + lo), b = __ldg((const C *)P.post_hi + hi);
     C w = cmul(a, b);
     if (P.sign > 0) w.y = -w.y;
     return w;
}

/* Four-step twiddles of one thread's elements k = tid + T*e (e < E) for
 * vector index v: W(v k) = W(v tid) * W(v T e), W(m) = exp(sign 2 pi i m/N).
 * For E = 16, W(v tid) and W(v T e) for e = 1, 2, 4, 8 come from the
 * two-level table (10 reads instead of 32) and the element factors are
 * b_r * W(v T 4q) for e = 4q + r, with b_r = W(v tid) W(v T r) and
 * W(v T 4q) products of the read powers: every factor is a product of at
 * most four correctly rounded table entries, as the stage twiddles are.
 * Indices stay below N (v < N / (T E), so 8 v T < N). */
template <typename C, int E, int T>
__device__ __forceinline__ void apply_post_twiddles(const gb_pass &P, long long v, int tid, C (&x)[E])
{
     if constexpr (E != 16) {
#pragma unroll
          for (int e = 0; e < E; ++e) x[e] = cmul(x[e], post_twiddle<C>(P, v * (long long)(tid + T * e)));
     } else {
          const long long s = v * T;
          C a;
          if (P.post_rows && v < P.post_rows_v) {
               /* one correctly rounded entry, read coalesced across the lanes */
               a = __ldg((const C *)P.post_rows + v * T + tid);
               if (P.sign > 0) a.y = -a.y;
          } else {
               a = post_twiddle<C>(P, v * tid);
          }
          const C w1 = post_twiddle<C>(P, s), w2 = post_twiddle<C>(P, 2 * s), w4 = post_twiddle<C>(P, 4 * s),
                  w8 = post_twiddle<C>(P, 8 * s);
          const C b[4] = {a, cmul(a, w1), cmul(a, w2), cmul(a, cmul(w1, w2))};
          const C q[4] = {mk<C>(1, 0), w4, w8, cmul(w8, w4)};
#pragma unroll
          for (int e = 0; e < 16; ++e) x[e] = cmul(x[e], (e < 4) ? b[e & 3] : cmul(b[e & 3], q[e >> 2]));
     }
}

/* Column tiles with a power-of-two tb that divides the CTA: each thread
 * keeps one column t = threadIdx mod tb for the whole tile and walks its
 * rows j = threadIdx / tb, j + J, j + 2J, ... (J = threads / tb) with one
 * pointer that advances by J rows, so a load costs a pointer add and a
 * compare instead of a division-free but 64-bit index computation.
 * Eight loads are in flight per thread before their shared-memory stores. */
template <typename C, bool PADDED>
__device__ __forceinline__ void cols_load(const gb_pass &P, const void *in, C *sm, int sms, const tile_t &tl, int L,
                                          int nfft)
{
     constexpr int U = 4;
     const int t = threadIdx.x & (P.tb - 1);
     const int j0 = threadIdx.x >> P.ltb;
     const int J = blockDim.x >> P.ltb;
     const long long v = tl.v0 + t;
     if (v >= P.vn[0]) return;
     const C *src = (const C *)in + tl.bi + v * P.vis[0] + (long long)j0 * P.is;
     const long long sj = (long long)J * P.is;
     C *dst = sm + t * sms;
     for (int j = j0; j < L; j += U * J) {
          C x[U];
          const C *q = src;
#pragma unroll
          for (int u = 0; u < U; ++u) {
               if (j + u * J < L) x[u] = *q;
               q += sj;
          }
#pragma unroll
          for (int u = 0; u < U; ++u) {
               const int jj = j + u * J;
               if (jj < L) dst[PADDED ? pad_for(nfft, jj) : jj] = x[u];
          }
          src += U * sj;
     }
}

template <typename C, bool PADDED>
__device__ __forceinline__ void cols_store(const gb_pass &P, void *out, const C *sm, int sms, const tile_t &tl, int L,
                                           int nfft)
{
     const int t = threadIdx.x & (P.tb - 1);
     const int j0 = threadIdx.x >> P.ltb;
     const int J = blockDim.x >> P.ltb;
     const long long v = tl.v0 + t;
     if (v >= P.vn[0]) return;
     C *dst = (C *)out + tl.bo + v * P.vos[0] + (long long)j0 * P.os;
     const long long sj = (long long)J * P.os;
     const C *src = sm + t * sms;
     for (int j = j0; j < L; j += J) {
          *dst = src[PADDED ? pad_for(nfft, j) : j];
          dst += sj;
     }
}

/* Cooperative copy of L complex elements per transform between HBM and
 * shared memory, for the tb transforms of one tile.  ROWS walks the element
 * index fastest (unit-stride transforms); COLS walks the transform index
 * fastest (transforms adjacent in memory, e.g. columns of a row-major
 * array).  PADDED applies the k_reg shared-memory swizzle. */
template <typename C, bool PADDED, bool PAIRS_REAL, bool COLS_FAST = true>
__device__ __forceinline__ void coop_load(const gb_pass &P, const void *in, C *sm, int sms, const tile_t &tl,
                                          int L, int mode, int nfft = 0)
{
     if (COLS_FAST && !PAIRS_REAL && mode == GB_MOVE_COLS && P.ltb >= 0 && (blockDim.x & (P.tb - 1)) == 0) {
          cols_load<C, PADDED>(P, in, sm, sms, tl, L, nfft);
          return;
     }
     /* eight loads in flight per thread before their shared-memory stores, so
      * the memory latency is paid once per batch instead of once per element */
     constexpr int U = 8;
     const int tb = P.tb;
     const int total = tb * L;
     for (int base0 = threadIdx.x; base0 < total; base0 += U * blockDim.x) {
          C x[U];
          int slot[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
               const int idx = base0 + u * blockDim.x;
               slot[u] = -1;
               if (idx < total) {
                    int t, j;
                    if (mode == GB_MOVE_COLS) {
                         if (P.ltb >= 0) { t = idx & (tb - 1); j = idx >> P.ltb; }
                         else { t = idx % tb; j = idx / tb; }
                    } else { t = idx / L; j = idx - t * L; }
                    const long long v = tl.v0 + t;
                    if (v < P.vn[0]) {
                         const long long base = tl.bi + v * P.vis[0];
                         x[u] = PAIRS_REAL ? io<C>::ldpair(in, base, j, P.is, P.real_pairs) : io<C>::ldc(in, base, j, P.is);
                         slot[u] = t * sms + (PADDED ? pad_for(nfft, j) : j);
                    }
               }
          }
#pragma unroll
          for (int u = 0; u < U; ++u)
               if (slot[u] >= 0) sm[slot[u]] = x[u];
     }
}

template <typename C, bool PADDED, bool PAIRS_REAL, bool COLS_FAST = true>
__device__ __forceinline__ void coop_store(const gb_pass &P, void *out, const C *sm, int sms, const tile_t &tl,
                                           int L, int mode, int nfft = 0)
{
     if (COLS_FAST && !PAIRS_REAL && mode == GB_MOVE_COLS && P.ltb >= 0 && (blockDim.x & (P.tb - 1)) == 0) {
          cols_store<C, PADDED>(P, out, sm, sms, tl, L, nfft);
          return;
     }
     const int tb = P.tb;
     const int total = tb * L;
     for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
          int t, j;
          if (mode == GB_MOVE_COLS) {
               if (P.ltb >= 0) { t = idx & (tb - 1); j = idx >> P.ltb; }
               else { t = idx % tb; j = idx / tb; }
          } else { t = idx / L; j = idx - t * L; }
          long long v = tl.v0 + t;
          if (v < P.vn[0]) {
               long long base = tl.bo + v * P.vos[0];
               C x = sm[t * sms + (PADDED ? pad_for(nfft, j) : j)];
               if (PAIRS_REAL) io<C>::stpair(out, base, j, P.os, P.real_pairs, x);
               else io<C>::stc(out, base, j, P.os, x);
          }
     }
}

/* ======================================================================
 * k_reg: power-of-two, register-resident
 * ==================================================================== */

/* Twiddles of one radix-RAD butterfly: v[r] *= W_N^(r*m), r = 1..RAD-1,
 * from the table tw (exp(-2 pi i j/N), conjugated for DIR > 0).  Only the
 * powers 1, 2, 4, 8 are read; the others are products of at most two read
 * or derived factors (each factor then carries at most three roundings). */
template <int DIR, int RAD, typename C>
__device__ __forceinline__ void apply_twiddles(C *v, const C *__restrict__ tw, int m)
{
     if constexpr (RAD == 2) {
          v[1] = cmul(v[1], twid<DIR>(tw, m));
     } else if constexpr (RAD == 4) {
          const C w1 = twid<DIR>(tw, m), w2 = twid<DIR>(tw, 2 * m);
          v[1] = cmul(v[1], w1);
          v[2] = cmul(v[2], w2);
          v[3] = cmul(v[3], cmul(w1, w2));
     } else if constexpr (RAD == 8) {
          const C w1 = twid<DIR>(tw, m), w2 = twid<DIR>(tw, 2 * m), w4 = twid<DIR>(tw, 4 * m);
          const C w3 = cmul(w1, w2);
          v[1] = cmul(v[1], w1); v[2] = cmul(v[2], w2); v[3] = cmul(v[3], w3); v[4] = cmul(v[4], w4);
          v[5] = cmul(v[5], cmul(w4, w1)); v[6] = cmul(v[6], cmul(w4, w2)); v[7] = cmul(v[7], cmul(w4, w3));
     } else if constexpr (RAD == 16) {
          const C w1 = twid<DIR>(tw, m), w2 = twid<DIR>(tw, 2 * m), w4 = twid<DIR>(tw, 4 * m),
                  w8 = twid<DIR>(tw, 8 * m);
          const C w3 = cmul(w1, w2), w12 = cmul(w8, w4);
          v[1] = cmul(v[1], w1); v[2] = cmul(v[2], w2); v[3] = cmul(v[3], w3); v[4] = cmul(v[4], w4);
          v[5] = cmul(v[5], cmul(w4, w1)); v[6] = cmul(v[6], cmul(w4, w2)); v[7] = cmul(v[7], cmul(w4, w3));
          v[8] = cmul(v[8], w8);
          v[9] = cmul(v[9], cmul(w8, w1)); v[10] = cmul(v[10], cmul(w8, w2)); v[11] = cmul(v[11], cmul(w8, w3));
          v[12] = cmul(v[12], w12);
          v[13] = cmul(v[13], cmul(w12, w1)); v[14] = cmul(v[14], cmul(w12, w2)); v[15] = cmul(v[15], cmul(w12, w3));
     } else {
#pragma unroll
          for (int r = 1; r < RAD; ++r) v[r] = cmul(v[r], twid<DIR>(tw, r * m));
     }
}

/* Rows per stage of the stage twiddle table (gb_pass.tw_stage) for complex
 * elements of csize bytes: four for float (powers 1, 2, 4, 8), fifteen for
 * double (powers 1..15). */
__host__ __device__ constexpr int stage_tw_rows(int csize) { return csize == 16 ? 15 : 4; }

/* Offset of stage NS's rows in the stage twiddle table of N: rows of NS
 * entries for every earlier twiddled stage. */
__host__ __device__ constexpr int stage_tw_off(int N, int NS, int rows = 4)
{
     int off = 0;
     for (int s = reg_r0(N); s < NS; s *= 16) off += rows * s;
     return off;
}
__host__ __device__ constexpr int stage_tw_len(int N, int rows = 4)
{
     int len = 0;
     if (N >= 32)
          for (int s = reg_r0(N); s * 16 <= N; s *= 16) len += rows * s;
     return len;
}

/* Twiddles of one radix-16 butterfly at position k of a stage of span NS,
 * from that stage's rows of the stage table (tws points at them), read with
 * consecutive k on consecutive lanes (coalesced): W^(k m p), m = N / (16 NS).
 * Double reads all fifteen powers (one rounding each, no FP64 products);
 * float reads the powers 1, 2, 4, 8 and forms the others as products of at
 * most two read or derived factors, as in apply_twiddles. */
template <int DIR, typename C>
__device__ __forceinline__ void apply_stage_twiddles16(C *v, const C *__restrict__ tws, int k, int NS)
{
     if constexpr (sizeof(C) == 16) {
#pragma unroll
          for (int q = 1; q < 16; ++q) v[q] = cmul(v[q], twid<DIR>(tws, (q - 1) * NS + k));
          return;
     }
     const C w1 = twid<DIR>(tws, k), w2 = twid<DIR>(tws, NS + k), w4 = twid<DIR>(tws, 2 * NS + k),
             w8 = twid<DIR>(tws, 3 * NS + k);
     const C w3 = cmul(w1, w2), w12 = cmul(w8, w4);
     v[1] = cmul(v[1], w1); v[2] = cmul(v[2], w2); v[3] = cmul(v[3], w3); v[4] = cmul(v[4], w4);
     v[5] = cmul(v[5], cmul(w4, w1)); v[6] = cmul(v[6], cmul(w4, w2)); v[7] = cmul(v[7], cmul(w4, w3));
     v[8] = cmul(v[8], w8);
     v[9] = cmul(v[9], cmul(w8, w1)); v[10] = cmul(v[10], cmul(w8, w2)); v[11] = cmul(v[11], cmul(w8, w3));
     v[12] = cmul(v[12], w12);
     v[13] = cmul(v[13], cmul(w12, w1)); v[14] = cmul(v[14], cmul(w12, w2)); v[15] = cmul(v[15], cmul(w12, w3));
}

/* x[e] = element tid + T*e of the swizzled transform in shared memory */
template <typename C, int N>
__device__ __forceinline__ void reg_gather(C (&x)[reg_e(N)], int tid, const C *smt)
{
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     if constexpr (T % 16 == 0) {
          const C *s = smt + pad_for(N, tid);
#pragma unroll
          for (int e = 0; e < E; ++e) x[e] = s[e * (T + pad_mult(N) * (T >> 4))];
     } else {
#pragma unroll
          for (int e = 0; e < E; ++e) x[e] = smt[pad_for(N, tid + T * e)];
     }
}

/* Barriers of the stage exchanges: the whole CTA, or one of two groups of
 * threads of a CTA that runs independent groups (named barriers 1 and 2,
 * immediate ids so the kernel reserves three barriers, not sixteen). */
struct cta_sync {
     __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct group_sync {
     unsigned id, n;   /* id 1 or 2; n threads, a multiple of 32 */
     __device__ __forceinline__ void operator()() const
     {
          if (id == 1) asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory");
          else asm volatile("bar.sync 2, %0;" ::"r"(n) : "memory");
     }
};

/* AND of v over the n threads of named barrier id (1 or 2; a barrier as well) */
__device__ __forceinline__ bool group_and(unsigned id, unsigned n, bool v)
{
     unsigned r;
     if (id == 1)
          asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}"
                       : "=r"(r) : "r"((unsigned)v), "r"(n) : "memory");
     else
          asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 2, %2, p;\n selp.u32 %0, 1, 0, q;\n}"
                       : "=r"(r) : "r"((unsigned)v), "r"(n) : "memory");
     return r != 0;
}

/* The stages of one transform of N points held E per thread; tws is the
 * stage twiddle table of N (gb_pass.tw_stage). */
/* barrier + AND of v over the threads a sync object stands for */
__device__ __forceinline__ bool sync_and(const cta_sync &, bool v) { return __syncthreads_and(v); }
__device__ __forceinline__ bool sync_and(const group_sync &s, bool v) { return group_and(s.id, s.n, v); }

/* The barrier of compute group g (of gt threads) in a CTA of G groups: the
 * CTA-wide barrier when there is one group (any thread count), else named
 * barrier 1 + g (gt a multiple of 32: a named barrier counts whole warps). */
template <int G> __device__ __forceinline__ auto group_barrier(int g, int gt)
{
     if constexpr (G == 1) return cta_sync();
     else return group_sync{(unsigned)(1 + g), (unsigned)gt};
}

template <typename C, int N, int DIR, int NS, typename S = cta_sync>
__device__ __forceinline__ void reg_stages(C (&x)[reg_e(N)], int tid, C *smt, const C *__restrict__ tws,
                                           const S &sync = S())
{
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int RAD = (NS == 1) ? reg_r0(N) : E;
     constexpr int B = E / RAD;
     constexpr bool LAST = (NS * RAD == N);
     /* first radix-16 stage of a float transform: 16 consecutive outputs,
      * written as eight 128-bit stores (the swizzle keeps them aligned) */
     constexpr bool VEC = (NS == 1) && (RAD == 16) && !LAST && (sizeof(C) == 8) && (pad_mult(N) == 2);
#pragma unroll
     for (int b = 0; b < B; ++b) {
          const int j = tid + b * T;
          const int k = j & (NS - 1);
          C v[RAD];
#pragma unroll
          for (int r = 0; r < RAD; ++r) v[r] = x[b + r * B];
          if constexpr (NS > 1) {
               static_assert(RAD == 16, "twiddled stages are radix 16");
               apply_stage_twiddles16<DIR>(v, tws + stage_tw_off(N, NS, stage_tw_rows(sizeof(C))), k, NS);
          }
          bfly<RAD, DIR>::run(v);
          if (LAST) {
#pragma unroll
               for (int q = 0; q < RAD; ++q) x[b + q * B] = v[q];
          } else if constexpr (VEC) {
               float4 *d = (float4 *)(smt + pad_for(N, j * 16));
#pragma unroll
               for (int q = 0; q < 8; ++q)
                    d[q] = make_float4(v[2 * q].x, v[2 * q].y, v[2 * q + 1].x, v[2 * q + 1].y);
          } else if constexpr (NS % 16 == 0) {
               /* the swizzle is linear across multiples of 16: one base, constant steps */
               C *d = smt + pad_for(N, (j / NS) * NS * RAD + k);
#pragma unroll
               for (int q = 0; q < RAD; ++q) d[q * (NS + pad_mult(N) * (NS >> 4))] = v[q];
          } else {
               const int base = (j / NS) * NS * RAD + k;
#pragma unroll
               for (int q = 0; q < RAD; ++q) smt[pad_for(N, base + q * NS)] = v[q];
          }
     }
     if constexpr (!LAST) {
          sync();
          reg_gather<C, N>(x, tid, smt);
          sync();
          reg_stages<C, N, DIR, NS * RAD, S>(x, tid, smt, tws, sync);
     }
}

/* Threads per CTA for k_reg: T = nfft/E threads per transform, at most 256
 * per CTA unless one transform needs more (several transforms per CTA for
 * short lengths). */
__host__ __device__ constexpr int reg_maxthreads(int nfft)
{
     return (nfft / reg_e(nfft)) > 256 ? (nfft / reg_e(nfft)) : 256;
}

/* CTAs of k_reg resident per SM that the register budget is sized for:
 * three 256-thread CTAs (80 registers a thread) for f32 c2c, whose strided
 * column passes need the extra warps in flight to cover HBM latency; two
 * (128 registers) where three would spill: f64, and the kinds with pre- or
 * post-processing. */
__host__ __device__ constexpr int reg_minblocks(int nfft, int csize, int kind)
{
     return reg_maxthreads(nfft) > 256 ? 1 : ((csize == 8 && kind == 0) ? 3 : 2);
}

template <typename C, int LOGN, int DIR, int KIND>
__global__ void __launch_bounds__(reg_maxthreads(1 << LOGN), reg_minblocks(1 << LOGN, sizeof(C), KIND)) k_reg(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     typedef typename real_of<C>::T R;
     constexpr int N = 1 << LOGN;
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int SMS = reg_sms(N);
     extern __shared__ __align__(16) unsigned char gb_smem[];
     C *sm = (C *)gb_smem;
     const int tl = threadIdx.x / T;
     const int tid = threadIdx.x - tl * T;
     C *smt = sm + tl * SMS;
     const C *__restrict__ tw = (const C *)P.tw_stage;

     for (long long blk = blockIdx.x; blk < P.nblocks; blk += gridDim.x) {
          const tile_t tile = tile_of(P, blk);
          const long long v = tile.v0 + tl;
          const bool valid = v < P.vn[0];
          const long long bi = tile.bi + v * P.vis[0];
          const long long bo = tile.bo + v * P.vos[0];
          C x[E];

          if constexpr (KIND == GB_KIND_BLUESTEIN) {
               /* dft/bluestein.c:82-128 in one CTA: b = x conj(w) zero-padded to
                * N, FFT, times the chirp spectrum, inverse FFT, times conj(w) */
               const C *__restrict__ w = (const C *)P.chirp;
               const int nn = P.n;
               if (P.load_mode == GB_MOVE_DIRECT) {
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                         const int k = tid + T * e;
                         C a = mk<C>(0, 0);
                         if (valid && k < nn) a = cmul(io<C>::ldc(in, bi, k, P.is), cconj(__ldg(w + k)));
                         x[e] = a;
                    }
               } else {
                    coop_load<C, true, false, (N <= 8192 && sizeof(C) == 8 && KIND == GB_KIND_C2C)>(P, in, sm, SMS, tile, nn, P.load_mode, N);
                    __syncthreads();
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                         const int k = tid + T * e;
                         x[e] = (k < nn) ? cmul(smt[pad_for(N, k)], cconj(__ldg(w + k))) : mk<C>(0, 0);
                    }
                    __syncthreads();
               }
               reg_stages<C, N, -1, 1>(x, tid, smt, tw);
               const C *__restrict__ spec = (const C *)P.chirp_spec;
#pragma unroll
               for (int e = 0; e < E; ++e) x[e] = cmul(x[e], __ldg(spec + tid + T * e));
               reg_stages<C, N, 1, 1>(x, tid, smt, tw);
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int k = tid + T * e;
                    if (k < nn) x[e] = cmul(x[e], cconj(__ldg(w + k)));
               }
               if (P.store_mode == GB_MOVE_DIRECT) {
                    if (valid) {
#pragma unroll
                         for (int e = 0; e < E; ++e) {
                              const int k = tid + T * e;
                              if (k < nn) io<C>::stc(out, bo, k, P.os, x[e]);
                         }
                    }
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
                    __syncthreads();
                    coop_store<C, true, false, (N <= 8192 && sizeof(C) == 8 && KIND == GB_KIND_C2C)>(P, out, sm, SMS, tile, nn, P.store_mode, N);
                    __syncthreads();
               }
               continue;
          }

          /* ---------------- load (and c2r pre-pass) ---------------- */
          if constexpr (KIND == GB_KIND_C2R) {
               /* X[0..N] -> shared, then Z'[k] = (X[k] + conj X[N-k])
                *                 + i conj(W_2N^k) (X[k] - conj X[N-k])  */
               coop_load<C, true, false, (N <= 8192 && sizeof(C) == 8 && KIND == GB_KIND_C2C)>(P, in, sm, SMS, tile, N + 1, P.load_mode, N);
               __syncthreads();
               const C *__restrict__ th = (const C *)P.tw_half;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int k = tid + T * e;
                    C a = smt[pad_for(N, k)], b = smt[pad_for(N, N - k)];
                    if (k == 0) { a.y = 0; b.y = 0; }
                    b.y = -b.y;
                    C s = cadd(a, b), d = csub(a, b);
                    C w = __ldg(th + k);
                    /* conj(w) * d */
                    C cd = mk<C>(w.x * d.x + w.y * d.y, w.x * d.y - w.y * d.x);
                    x[e] = mk<C>(s.x - cd.y, s.y + cd.x);
               }
               __syncthreads();
          } else if (P.load_mode == GB_MOVE_DIRECT) {
               if (valid) {
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                         const long long j = tid + T * e;
                         x[e] = (KIND == GB_KIND_R2C) ? io<C>::ldpair(in, bi, j, P.is, P.real_pairs)
                                                      : io<C>::ldc(in, bi, j, P.is);
                    }
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = mk<C>(0, 0);
               }
          } else {
               coop_load<C, true, KIND == GB_KIND_R2C, (N <= 8192 && sizeof(C) == 8 && KIND == GB_KIND_C2C)>(P, in, sm, SMS, tile, N, P.load_mode, N);
               __syncthreads();
#pragma unroll
               for (int e = 0; e < E; ++e) x[e] = smt[pad_for(N, tid + T * e)];
               __syncthreads();
          }

          /* ---------------- stages ---------------- */
          reg_stages<C, N, DIR, 1>(x, tid, smt, tw);

          /* ---------------- store (and r2c post-pass) ---------------- */
          if constexpr (KIND == GB_KIND_R2C) {
               /* X[k] = (Z[k] + conj Z[N-k])/2 + W_2N^k (Z[k] - conj Z[N-k])/(2i), k = 0..N */
#pragma unroll
               for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
               __syncthreads();
               const C *__restrict__ th = (const C *)P.tw_half;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int k = tid + T * e;
                    C a = smt[pad_for(N, k)], b = smt[pad_for(N, (N - k) & (N - 1))];
                    b.y = -b.y;
                    C ev = cscale(cadd(a, b), (R)0.5);
                    C dd = csub(a, b);
                    C od = mk<C>(dd.y * (R)0.5, -dd.x * (R)0.5);
                    C w = __ldg(th + k);
                    x[e] = cadd(ev, cmul(w, od));
               }
               C last = smt[pad_for(N, 0)];
               __syncthreads();
               if (P.store_mode == GB_MOVE_DIRECT) {
                    if (valid) {
#pragma unroll
                         for (int e = 0; e < E; ++e) io<C>::stc(out, bo, tid + T * e, P.os, x[e]);
                         if (tid == 0) io<C>::stc(out, bo, N, P.os, mk<C>(last.x - last.y, 0));
                    }
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
                    if (tid == 0) smt[pad_for(N, N)] = mk<C>(last.x - last.y, 0);
                    __syncthreads();
                    coop_store<C, true, false, (N <= 8192 && sizeof(C) == 8 && KIND == GB_KIND_C2C)>(P, out, sm, SMS, tile, N + 1, P.store_mode, N);
                    __syncthreads();
               }
          } else {
               if constexpr (KIND == GB_KIND_C2C) {
                    if (P.post_N) {
                         apply_post_twiddles<C, E, T>(P, P.post_vdim ? tile.vpost : v, tid, x);
                    }
               }
               constexpr bool RP = (KIND == GB_KIND_C2R);
               if (P.store_mode == GB_MOVE_DIRECT) {
                    if (valid) {
#pragma unroll
                         for (int e = 0; e < E; ++e) {
                              if (RP) io<C>::stpair(out, bo, tid + T * e, P.os, P.real_pairs, x[e]);
                              else io<C>::stc(out, bo, tid + T * e, P.os, x[e]);
                         }
                    }
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
                    __syncthreads();
                    coop_store<C, true, RP, (N <= 8192 && sizeof(C) == 8 && KIND == GB_KIND_C2C)>(P, out, sm, SMS, tile, N, P.store_mode, N);
                    __syncthreads();
               }
          }
     }
}

/* ======================================================================
 * k_reg_tma: persistent variant of k_reg for unit-stride c2c and r2c
 * batches whose transforms start on 16-byte boundaries.
 *
 * A CTA runs G independent compute groups (tma_threads(nfft) threads each,
 * synchronised by their own named barrier) over G + 1 shared-memory
 * buffers of one tile each.  The CTA's tiles are i = 0, 1, 2, ... (global
 * tile blockIdx.x + i * gridDim.x); tile i is transformed by group i mod G
 * in buffer i mod (G + 1).  The TMA engine copies each tile into its buffer
 * (cp.async.bulk, completion on the buffer's mbarrier): the first G + 1
 * tiles at start, and tile i + G + 1 as soon as the group that transformed
 * tile i has last read that buffer.  A count of the loads issued per buffer
 * lets a group that is ahead wait until its tile's load exists before it
 * waits on the barrier's phase.  So while every group transforms a
 * tile, one more tile is on its way, and a group finds its next tile
 * already resident.  Results are stored straight from registers.
 * One group per CTA (two buffers) leaves each thread 85 registers and puts
 * three CTAs of 256 threads on an SM; two groups (float only: 64 registers a
 * thread) put two CTAs of 2 x 256 threads on an SM, four transforms of 4096
 * in flight against three.  The planner picks the count per length.
 * ==================================================================== */

__host__ __device__ constexpr int tma_sms(int nfft) { return reg_sms(nfft); }

/* Element offsets of r2c inputs count reals; the slot receives the real
 * pairs, i.e. the same N * sizeof(C) bytes as a complex transform. */
template <typename C, int N, int KIND>
__device__ __forceinline__ void tma_issue(const gb_pass &P, const void *in, long long blk, C *dst,
                                          unsigned long long *bar)
{
     typedef typename real_of<C>::T R;
     const tile_t tl = tile_of(P, blk);
     const long long rem = P.vn[0] - tl.v0;
     const int ntr = rem < P.tb ? (int)rem : P.tb;
     const unsigned bytes = (unsigned)(N * sizeof(C));
     mbar_expect_tx(bar, bytes * (unsigned)ntr);
     for (int t = 0; t < ntr; ++t) {
          const long long off = tl.bi + (tl.v0 + t) * P.vis[0];
          const void *src = (KIND == GB_KIND_R2C || KIND == GB_KIND_DCT2) ? (const void *)((const R *)in + off)
                                                                            : (const void *)((const C *)in + off);
          bulk_g2s(dst + t * tma_sms(N), src, bytes, bar);
     }
}

/* threads of one compute group of k_reg_tma: 256, or one transform's T when larger */
__host__ __device__ constexpr int tma_threads(int nfft) { return (nfft / reg_e(nfft)) > 256 ? (nfft / reg_e(nfft)) : 256; }

/* most compute groups per CTA of k_reg_tma (complex element size csize) */
__host__ __device__ constexpr int tma_max_groups(int csize) { return csize == 8 ? 2 : 1; }

/* CTAs per SM the register budget is sized for: 64 registers a thread for
 * two groups, 85 for one group of 256 threads (float), 128 for double, whose
 * elements take two registers each (its CTAs hold half as many transforms:
 * shared memory, not registers, limits how many share an SM) */
__host__ __device__ constexpr int tma_minblocks(int nfft, int G, int csize)
{
     return G * tma_threads(nfft) >= 1024 ? 1 : G == 2 ? 2 : (tma_threads(nfft) > 256 ? 1 : csize == 16 ? 2 : 3);
}

#define GB_WAIT_NS 2000000000ull   /* bound on any wait for a copy: 2 s */

template <typename C, int LOGN, int DIR, int KIND, int G>
__global__ void __launch_bounds__(G * tma_threads(1 << LOGN), tma_minblocks(1 << LOGN, G, sizeof(C)))
k_reg_tma(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     typedef typename real_of<C>::T R;
     constexpr int N = 1 << LOGN;
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int SMS = tma_sms(N);
     constexpr int NB = G + 1;
     extern __shared__ __align__(128) unsigned char gb_smem[];
     __shared__ __align__(8) unsigned long long full[NB];
     __shared__ int issued[NB], consumed[NB];
     const int GT = P.threads;                /* threads of one group */
     const int g = (int)threadIdx.x / GT;
     const int gtid = (int)threadIdx.x - g * GT;
     const int tl = gtid / T;
     const int tid = gtid - tl * T;
     const int tile_elems = P.tb * SMS;
     C *const base = (C *)gb_smem;
     const C *__restrict__ tw = (const C *)P.tw_stage;
     const auto gs = group_barrier<G>(g, GT);
     const long long stride = gridDim.x;

     if (threadIdx.x == 0) {
#pragma unroll
          for (int b = 0; b < NB; ++b) {
               mbar_init(&full[b], 1);
               issued[b] = 0;
               consumed[b] = 0;
          }
          mbar_fence_init();
     }
     __syncthreads();
     if (threadIdx.x == 0) {
#pragma unroll
          for (int b = 0; b < NB; ++b) {
               const long long blk = blockIdx.x + b * stride;
               if (blk < P.nblocks) {
                    tma_issue<C, N, KIND>(P, in, blk, base + b * tile_elems, &full[b]);
                    issued[b] = 1;
               }
          }
     }

     for (int i = g;; i += G) {
          const long long blk = blockIdx.x + (long long)i * stride;
          if (blk >= P.nblocks) break;
          const int b = i % NB;
          C *const cur = base + b * tile_elems;
          /* The load of tile i is buffer b's load number i / NB; another group
           * issues it once it is done with tile i - NB.  A parity wait tells
           * apart only two consecutive phases, so the group's leader first makes
           * sure that load was issued (buffer b's earlier load then has
           * completed, and the barrier's current phase is this tile's); then
           * every thread of the group waits for its bytes. */
          bool ok = true;
          if (gtid == 0) {
               const volatile int *iss = &issued[b];
               const int need = i / NB + 1;
               unsigned long long t0 = 0;
               for (unsigned it = 0; *iss < need; ++it) {
                    if (it == 0) t0 = globaltimer_ns();
                    else if ((it & 63) == 0 && globaltimer_ns() - t0 > GB_WAIT_NS) {
                         ok = false;
                         break;
                    }
               }
          }
          if (!sync_and(gs, ok) || !sync_and(gs, mbar_wait(&full[b], (unsigned)((i / NB) & 1), GB_WAIT_NS))) {
               /* the copy never completed: report and leave (the copies still
                * in flight are drained below) */
               if (gtid == 0 && P.status) atomicExch(P.status, GB_STATUS_COPY_TIMEOUT);
               break;
          }
          if (gtid == 0) atomicAdd(&consumed[b], 1);
          C x[E];
          if constexpr (KIND == GB_KIND_DCT2) {
               /* Makhoul's permutation v_j = x_{2j} (j < N), v_{2N-1-j} = x_{2j+1}
                * read from the slot: complex element m = (v_{2m}, v_{2m+1}) is
                * (x_{4m}, x_{4m+2}) for m < N/2 and, with mm = N-1-m,
                * (x_{4mm+3}, x_{4mm+1}) above: the same four reals serve both */
               const C *s0 = cur + tl * SMS;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int m = tid + T * e;
                    const bool lo = 2 * m < N;
                    const int q = lo ? m : N - 1 - m;
                    const C a = s0[2 * q], c = s0[2 * q + 1];
                    x[e] = lo ? mk<C>(a.x, c.x) : mk<C>(c.y, a.y);
               }
          } else {
               const C *s0 = cur + tl * SMS + tid;
#pragma unroll
               for (int e = 0; e < E; ++e) x[e] = s0[T * e];
          }
          gs();
          reg_stages<C, N, DIR, 1>(x, tid, cur + tl * SMS, tw, gs);
          /* (the tile's indices are formed after the stages, which need every
           * register they can get) */
          C *smt = cur + tl * SMS;
          /* the tile of buffer b after this one: issued by this group once it
           * has last read the buffer */
          const long long nxt = blk + NB * stride;
          const tile_t tile = tile_of(P, blk);
          const long long v = tile.v0 + tl;
          const bool valid = v < P.vn[0];
          const long long bo = tile.bo + v * P.vos[0];
          if constexpr (KIND == GB_KIND_R2C || KIND == GB_KIND_DCT2) {
               /* hc2c post-pass (rdft/ct-hc2c.c:197-210):
                * X[k] = (Z[k] + conj Z[N-k])/2 + W_2N^k (Z[k] - conj Z[N-k])/(2i) */
#pragma unroll
               for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
               gs();
               /* each output straight to HBM as it is formed (no array of
                * results held across the loop) */
               const C *__restrict__ th = (const C *)P.tw_half;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int k = tid + T * e;
                    C a = smt[pad_for(N, k)], bq = smt[pad_for(N, (N - k) & (N - 1))];
                    bq.y = -bq.y;
                    const C ev = cscale(cadd(a, bq), (R)0.5), dd = csub(a, bq);
                    const C od = mk<C>(dd.y * (R)0.5, -dd.x * (R)0.5);
                    const C X = cadd(ev, cmul(__ldg(th + k), od));
                    if constexpr (KIND == GB_KIND_R2C) {
                         if (valid) ((C *)out)[bo + tid + T * e] = X;
                    } else {
                         /* DCT-II (reodft/reodft010e-r2hc.c): p = exp(-i pi k / 2n) V_k,
                          * y_k = 2 Re p and, as exp(-i pi (n-k) / 2n) = -i conj of
                          * the former, y_{n-k} = -2 Im p */
                         const C p = cmul(__ldg((const C *)P.chirp + k), X);
                         if (valid) {
                              R *y = (R *)out + bo;
                              y[k] = (R)2 * p.x;
                              if (k) y[2 * N - k] = (R)-2 * p.y;
                         }
                    }
               }
               if (valid && tid == 0) {
                    const C z0 = smt[pad_for(N, 0)];
                    if constexpr (KIND == GB_KIND_R2C) {
                         ((C *)out)[bo + N] = mk<C>(z0.x - z0.y, 0);
                    } else {
                         /* y_N = 2 Re(exp(-i pi / 4) V_N), V_N real */
                         ((R *)out)[bo + N] = (R)2 * __ldg((const C *)P.chirp + N).x * (z0.x - z0.y);
                    }
               }
               gs();   /* the buffer is the next bulk copy's target */
               if (gtid == 0 && nxt < P.nblocks) {
                    fence_proxy_async_smem();
                    tma_issue<C, N, KIND>(P, in, nxt, cur, &full[b]);
                    atomicAdd(&issued[b], 1);
               }
          } else {
               /* every thread of the group is past the barrier that follows
                * the last read of the buffer (inside the stages) */
               if (gtid == 0 && nxt < P.nblocks) {
                    fence_proxy_async_smem();
                    tma_issue<C, N, KIND>(P, in, nxt, cur, &full[b]);
                    atomicAdd(&issued[b], 1);
               }
               if (P.post_N) {
                    apply_post_twiddles<C, E, T>(P, P.post_vdim ? tile.vpost : v, tid, x);
               }
               if (valid) {
                    /* unit output stride (checked at launch): constant offsets */
                    C *o = (C *)out + bo + tid;
#pragma unroll
                    for (int e = 0; e < E; ++e) o[T * e] = x[e];
               }
          }
     }
     /* a group that gave up may leave copies in flight: wait (bounded) for
      * each before the CTA's shared memory is released */
     __syncthreads();
     if (threadIdx.x == 0) {
#pragma unroll
          for (int b = 0; b < NB; ++b)
               if (issued[b] > consumed[b]) mbar_wait(&full[b], (unsigned)((issued[b] - 1) & 1), GB_WAIT_NS);
     }
}

/* ======================================================================
 * k_gen: runtime radix list, shared-memory ping-pong
 * ==================================================================== */

/* Shared-memory layout of the runtime-radix body: element i of a transform
 * at gpad(i) = i + i/16, transforms gen_sms(N) = N + N/16 + 1 apart.  The
 * gap after every 16 elements spreads the Stockham stores of the first
 * stages (16 j + q, 8 j + q, 4 j + q, ... for consecutive j) over the banks,
 * and the odd stride keeps adjacent transforms (column tiles) apart. */
__device__ __forceinline__ int gpad(int i) { return i + (i >> 4); }

/* One element copied global -> shared without passing through registers
 * (cp.async: 8 bytes through L1 for complex float, 16 bytes around it for
 * complex double), so a thread keeps all its tile loads in flight at once;
 * cp_async_wait_all completes the thread's copies. */
template <typename C> __device__ __forceinline__ void cp_async_elem(C *dst, const C *src)
{
     const unsigned d = smem_u32(dst);
     if constexpr (sizeof(C) == 16)
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
     else
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all_groups()
{
     asm volatile("cp.async.commit_group;" ::: "memory");
     asm volatile("cp.async.wait_all;" ::: "memory");
}
__host__ __device__ constexpr int gen_sms(int nfft) { return nfft + (nfft >> 4) + 1; }

template <typename C, int DIR, int RAD>
__device__ __forceinline__ void gen_stage(const C *src, C *dst, int N, int Ns, int tb, int sms,
                                          const C *__restrict__ tw, const C *__restrict__ tws)
{
     const int nb = N / RAD;
     const int twstep = N / (Ns * RAD);
     /* butterfly idx = t nb + j of transform t, j = jq Ns + k: the divisions
      * are done once, and each step of blockDim.x advances (t, j, jq, k) by
      * precomputed quotients and remainders (nb is a multiple of Ns) */
     const int B = blockDim.x, nq = nb / Ns;
     int t = threadIdx.x / nb, j = threadIdx.x - t * nb;
     int jq = j / Ns, k = j - jq * Ns;
     const int dt = B / nb, dj = B - dt * nb;
     const int djq = dj / Ns, dk = dj - djq * Ns;
     for (int idx = threadIdx.x; idx < tb * nb; idx += B) {
          const C *s = src + t * sms;
          C *d = dst + t * sms;
          C v[RAD];
#pragma unroll
          for (int r = 0; r < RAD; ++r) v[r] = s[gpad(j + r * nb)];
          if (Ns > 1) {
               if (tws) {
                    /* the stage's rows: consecutive k on consecutive lanes */
                    const C *w = tws + (Ns - 1) + k;
#pragma unroll
                    for (int r = 1; r < RAD; ++r) v[r] = cmul(v[r], twid<DIR>(w, (r - 1) * Ns));
               } else {
#pragma unroll
                    for (int r = 1; r < RAD; ++r) v[r] = cmul(v[r], twid<DIR>(tw, r * k * twstep));
               }
          }
          bfly<RAD, DIR>::run(v);
          const int base = jq * Ns * RAD + k;
#pragma unroll
          for (int q = 0; q < RAD; ++q) d[gpad(base + q * Ns)] = v[q];
          t += dt; j += dj; jq += djq; k += dk;
          if (k >= Ns) { k -= Ns; ++jq; }
          if (j >= nb) { j -= nb; jq -= nq; ++t; }
     }
}

/* Runs all stages; returns the buffer holding the result (natural order). */
template <typename C, int DIR>
__device__ C *gen_fft(C *b0, C *b1, const gb_pass &P, int N, int sms, const C *__restrict__ tw)
{
     int Ns = 1;
     C *src = b0, *dst = b1;
     const C *__restrict__ tws = (const C *)P.tw_gen;
     for (int s = 0; s < P.nrad; ++s) {
          const int r = P.rad[s];
          switch (r) {
          case 2: gen_stage<C, DIR, 2>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 3: gen_stage<C, DIR, 3>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 4: gen_stage<C, DIR, 4>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 5: gen_stage<C, DIR, 5>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 7: gen_stage<C, DIR, 7>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 8: gen_stage<C, DIR, 8>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 11: gen_stage<C, DIR, 11>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 13: gen_stage<C, DIR, 13>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          case 16: gen_stage<C, DIR, 16>(src, dst, N, Ns, P.tb, sms, tw, tws); break;
          default: break;
          }
          __syncthreads();
          Ns *= r;
          C *t = src; src = dst; dst = t;
     }
     return src;
}

/* Transform base addresses of one tile: strided (tile.bi + v * vis[0]) or,
 * for work-queue items that group transforms of different arrays, one
 * pointer per transform (pin/pout, element 0 of each transform). */
struct gen_addr {
     const void *in;
     void *out;
     const void *const *pin;
     void *const *pout;
     /* 1: the input was written earlier in this launch by other CTAs (a
      * work-queue item that waited on a counter): load it from L2, never
      * from this SM's L1, which is not kept coherent with other SMs' writes */
     int l2only;
};

template <typename C> __device__ __forceinline__ const C *src_of(const gb_pass &P, const tile_t &tl, const gen_addr &A, int t)
{
     const long long v = tl.v0 + t;
     if (A.pin) return (const C *)A.pin[v];
     return (const C *)A.in + tl.bi + v * P.vis[0];
}
template <typename C> __device__ __forceinline__ C *dst_of(const gb_pass &P, const tile_t &tl, const gen_addr &A, int t)
{
     const long long v = tl.v0 + t;
     if (A.pout) return (C *)A.pout[v];
     return (C *)A.out + tl.bo + v * P.vos[0];
}
__device__ __forceinline__ void tile_index(int idx, int tb, int L, int mode, int &t, int &j, int ltb = -1)
{
     if (mode == GB_MOVE_COLS) {
          if (ltb >= 0) { t = idx & (tb - 1); j = idx >> ltb; }
          else { t = idx % tb; j = idx / tb; }
     } else { t = idx / L; j = idx - t * L; }
}

/* idx = q D + r, walked in steps of B (the block) with one division at the
 * start: each step adds B's quotient and remainder and carries once. */
struct idx_walk {
     int q, r, dq, dr, D;
     __device__ __forceinline__ idx_walk(int idx, int D_, int B) : D(D_)
     {
          q = idx / D;
          r = idx - q * D;
          dq = B / D;
          dr = B - dq * D;
     }
     __device__ __forceinline__ void step()
     {
          q += dq;
          r += dr;
          if (r >= D) { r -= D; ++q; }
     }
};

/* tile_index as a walk: rows of L (t = q, j = r) or columns of tb (j = q,
 * t = r) */
struct tile_walk {
     idx_walk w;
     bool cols;
     __device__ __forceinline__ tile_walk(int idx, int tb, int L, int mode, int B)
         : w(idx, mode == GB_MOVE_COLS ? tb : L, B), cols(mode == GB_MOVE_COLS) {}
     __device__ __forceinline__ int t() const { return cols ? w.r : w.q; }
     __device__ __forceinline__ int j() const { return cols ? w.q : w.r; }
     __device__ __forceinline__ void step() { w.step(); }
};

/* One tile of k_gen: load, stages (direction from P.sign), store.  Also the
 * body of the work-queue kernel.  b0/b1: two shared buffers of
 * tb * gen_sms(nfft). */
template <typename C>
__device__ void gen_tile(const gb_pass &P, const tile_t &tile, const gen_addr &A, C *b0, C *b1)
{
     typedef typename real_of<C>::T R;
     const int N = P.nfft;
     const int sms = gen_sms(N);
     const int tb = P.tb;
     const C *__restrict__ tw = (const C *)P.tw;
     const int n = P.n;
     const int kind = P.kind;
     const bool half = (kind == GB_KIND_R2C || kind == GB_KIND_C2R) && (n % 2 == 0);
     const long long vn0 = P.vn[0];

     /* Pointer-stride walks of a c2c tile: a column tile whose tb (a power of
      * two) divides the block keeps one column t = threadIdx mod tb per thread
      * and walks its rows j0, j0 + J, ... (J = block / tb); a row tile of
      * transforms at least a block long goes transform after transform with
      * the block on consecutive elements.  No index arithmetic per element
      * but the pad; other shapes walk the general way below. */
     const bool ld_fast = kind == GB_KIND_C2C &&
                          ((P.load_mode == GB_MOVE_COLS && P.ltb >= 0 && (blockDim.x & (tb - 1)) == 0) ||
                           (P.load_mode != GB_MOVE_COLS && N >= (int)blockDim.x));
     const bool st_fast = kind == GB_KIND_C2C &&
                          ((P.store_mode == GB_MOVE_COLS && P.ltb >= 0 && (blockDim.x & (tb - 1)) == 0) ||
                           (P.store_mode != GB_MOVE_COLS && N >= (int)blockDim.x));

     /* ---------------- load ---------------- */
     if (ld_fast) {
          const bool cols = P.load_mode == GB_MOVE_COLS;
          const int J = cols ? (int)(blockDim.x >> P.ltb) : (int)blockDim.x;
          const int t0 = cols ? (int)(threadIdx.x & (tb - 1)) : 0, t1 = cols ? t0 + 1 : tb;
          const int j0 = cols ? (int)(threadIdx.x >> P.ltb) : (int)threadIdx.x;
          for (int t = t0; t < t1 && tile.v0 + t < vn0; ++t) {
               const C *sp = src_of<C>(P, tile, A, t) + (long long)j0 * P.is;
               const long long ss = (long long)J * P.is;
               C *dp = b0 + t * sms;
               if (!A.l2only) {
                    /* every copy of the thread in flight at once */
                    for (int j = j0; j < N; j += J, sp += ss) cp_async_elem<C>(dp + gpad(j), sp);
               } else {
                    /* written earlier in this launch: through L2 only */
                    constexpr int U = 4;
                    for (int j = j0; j < N; j += U * J, sp += U * ss) {
                         C x[U];
#pragma unroll
                         for (int u = 0; u < U; ++u)
                              if (j + u * J < N) x[u] = __ldcg(sp + u * ss);
#pragma unroll
                         for (int u = 0; u < U; ++u)
                              if (j + u * J < N) dp[gpad(j + u * J)] = x[u];
                    }
               }
          }
          cp_async_wait_all_groups();
     } else if (kind == GB_KIND_C2C && !A.l2only) {
          /* complex elements straight into b0, every copy of the thread in
           * flight at once (an input written earlier in the same launch,
           * l2only, takes the register path below: it must not be read
           * through L1) */
          tile_walk wk(threadIdx.x, tb, N, P.load_mode, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x, wk.step()) {
               const int t = wk.t(), j = wk.j();
               if (tile.v0 + t < vn0) cp_async_elem<C>(b0 + t * sms + gpad(j), src_of<C>(P, tile, A, t) + (long long)j * P.is);
          }
          cp_async_wait_all_groups();
     } else if (kind == GB_KIND_C2C || kind == GB_KIND_RADER || (kind == GB_KIND_C2R) || (kind == GB_KIND_R2C && half)) {
          /* complex elements (real pairs for even r2c) into b0, or into b1
           * for the kinds that rearrange them afterwards */
          C *dst = (kind == GB_KIND_C2C || kind == GB_KIND_R2C) ? b0 : b1;
          const int L = (kind == GB_KIND_RADER) ? n : (kind == GB_KIND_C2R) ? n / 2 + 1 : N;
          constexpr int U = 4;   /* loads in flight per thread */
          tile_walk wk(threadIdx.x, tb, L, P.load_mode, blockDim.x);
          for (int idx0 = threadIdx.x; idx0 < tb * L; idx0 += U * blockDim.x) {
               C x[U];
               int slot[U];
#pragma unroll
               for (int u = 0; u < U; ++u) {
                    const int idx = idx0 + u * blockDim.x;
                    const int t = wk.t(), j = wk.j();
                    wk.step();
                    slot[u] = -1;
                    if (idx < tb * L) {
                         if (tile.v0 + t < vn0) {
                              if (kind == GB_KIND_R2C) {
                                   const R *r = (const R *)src_of<R>(P, tile, A, t);
                                   x[u] = P.real_pairs ? ((const C *)r)[j] : mk<C>(r[2 * j * P.is], r[(2 * j + 1) * P.is]);
                              } else {
                                   const C *sp = src_of<C>(P, tile, A, t) + (long long)j * P.is;
                                   x[u] = A.l2only ? __ldcg(sp) : *sp;
                              }
                              slot[u] = t * sms + gpad(j);
                         }
                    }
               }
#pragma unroll
               for (int u = 0; u < U; ++u)
                    if (slot[u] >= 0) dst[slot[u]] = x[u];
          }
     } else if (kind == GB_KIND_R2C) {
          /* odd n: real sequence as complex with zero imaginary part */
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x) {
               int t, j;
               tile_index(idx, tb, N, P.load_mode, t, j, P.ltb);
               if (tile.v0 + t < vn0) b0[t * sms + gpad(j)] = mk<C>(src_of<R>(P, tile, A, t)[j * P.is], 0);
          }
     } else if (kind == GB_KIND_BLUESTEIN) {
          /* b = x conj(w), zero-padded to nfft (dft/bluestein.c:82-95) */
          const C *__restrict__ w = (const C *)P.chirp;
          tile_walk wk(threadIdx.x, tb, N, P.load_mode, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x, wk.step()) {
               const int t = wk.t(), j = wk.j();
               C x = mk<C>(0, 0);
               if (j < n && tile.v0 + t < vn0) x = cmul(src_of<C>(P, tile, A, t)[j * P.is], cconj(__ldg(w + j)));
               b0[t * sms + gpad(j)] = x;
          }
     }
     __syncthreads();
     if (kind == GB_KIND_RADER) {
          /* dft/rader.c:95-165: b[k] = x[g^k], k < n-1; x[0] kept in the unused
           * slot N of buffer 0 */
          idx_walk wk(threadIdx.x, N, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x, wk.step()) {
               const int t = wk.q, k = wk.r;
               b0[t * sms + gpad(k)] = b1[t * sms + gpad(__ldg(P.perm + k))];
               if (k == 0) b0[t * sms + gpad(N)] = b1[t * sms];
          }
          __syncthreads();
     } else if (kind == GB_KIND_C2R) {
          const int nc = n / 2 + 1;
          if (half) {
               /* hc2c pre-pass (rdft/ct-hc2c.c:72-83) */
               const C *__restrict__ th = (const C *)P.tw_half;
               for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x) {
                    const int t = idx / N, k = idx - t * N;
                    C a = b1[t * sms + gpad(k)], b = b1[t * sms + gpad(N - k)];
                    if (k == 0) { a.y = 0; b.y = 0; }
                    b.y = -b.y;
                    C s = cadd(a, b), d = csub(a, b);
                    C w = __ldg(th + k);
                    C cd = mk<C>(w.x * d.x + w.y * d.y, w.x * d.y - w.y * d.x);
                    b0[t * sms + gpad(k)] = mk<C>(s.x - cd.y, s.y + cd.x);
               }
          } else {
               /* odd n: Hermitian extension of X[0..(n-1)/2] */
               for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x) {
                    const int t = idx / N, k = idx - t * N;
                    C a = (k < nc) ? b1[t * sms + gpad(k)] : cconj(b1[t * sms + gpad((N - k))]);
                    if (k == 0) a.y = 0;
                    b0[t * sms + gpad(k)] = a;
               }
          }
          __syncthreads();
     }

     /* ---------------- stages ---------------- */
     C *res;
     if (kind == GB_KIND_RADER || kind == GB_KIND_BLUESTEIN) {
          /* convolution: forward FFT, spectrum multiply, inverse FFT.  Rader
           * also records X[0] = x[0] + B[0] in slot N of buffer 1. */
          res = gen_fft<C, -1>(b0, b1, P, N, sms, tw);
          const C *__restrict__ W = (const C *)P.chirp_spec;
          idx_walk wk(threadIdx.x, N, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x, wk.step()) {
               const int t = wk.q, k = wk.r;
               const C bk = res[t * sms + gpad(k)];
               if (kind == GB_KIND_RADER && k == 0) b1[t * sms + gpad(N)] = cadd(b0[t * sms + gpad(N)], bk);
               res[t * sms + gpad(k)] = cmul(bk, __ldg(W + k));
          }
          __syncthreads();
          res = gen_fft<C, 1>(res, res == b0 ? b1 : b0, P, N, sms, tw);
     } else if (P.sign < 0) {
          res = gen_fft<C, -1>(b0, b1, P, N, sms, tw);
     } else {
          res = gen_fft<C, 1>(b0, b1, P, N, sms, tw);
     }

     /* ---------------- store ---------------- */
     if (st_fast) {
          const bool cols = P.store_mode == GB_MOVE_COLS;
          const int J = cols ? (int)(blockDim.x >> P.ltb) : (int)blockDim.x;
          const int t0 = cols ? (int)(threadIdx.x & (tb - 1)) : 0, t1 = cols ? t0 + 1 : tb;
          const int j0 = cols ? (int)(threadIdx.x >> P.ltb) : (int)threadIdx.x;
          for (int t = t0; t < t1 && tile.v0 + t < vn0; ++t) {
               const long long v = tile.v0 + t;
               C *op = dst_of<C>(P, tile, A, t) + (long long)j0 * P.os;
               const long long os = (long long)J * P.os;
               const C *rp = res + t * sms;
               /* four-step twiddle exponent (P.post_vdim ? vpost : v) * k, advanced by J */
               const long long pv = P.post_vdim ? tile.vpost : v;
               long long m = pv * j0;
               const long long ms = pv * J;
               for (int k = j0; k < N; k += J, op += os, m += ms) {
                    C y = rp[gpad(k)];
                    if (P.post_N) y = cmul(y, post_twiddle<C>(P, m));
                    *op = y;
               }
          }
     } else if (kind == GB_KIND_C2C) {
          tile_walk wk(threadIdx.x, tb, N, P.store_mode, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x, wk.step()) {
               const int t = wk.t(), k = wk.j();
               const long long v = tile.v0 + t;
               if (v < vn0) {
                    C y = res[t * sms + gpad(k)];
                    if (P.post_N) y = cmul(y, post_twiddle<C>(P, (P.post_vdim ? tile.vpost : v) * (long long)k));
                    dst_of<C>(P, tile, A, t)[k * P.os] = y;
               }
          }
     } else if (kind == GB_KIND_BLUESTEIN) {
          /* X[k] = conv[k] conj(w[k]), k < n */
          const C *__restrict__ w = (const C *)P.chirp;
          tile_walk wk(threadIdx.x, tb, n, P.store_mode, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * n; idx += blockDim.x, wk.step()) {
               const int t = wk.t(), k = wk.j();
               if (tile.v0 + t < vn0)
                    dst_of<C>(P, tile, A, t)[k * P.os] = cmul(res[t * sms + gpad(k)], cconj(__ldg(w + k)));
          }
     } else if (kind == GB_KIND_RADER) {
          /* X[0] from slot N of buffer 1; X[g^-k] = x[0] + conv[k] */
          const int *__restrict__ lg = P.perm + N;
          tile_walk wk(threadIdx.x, tb, n, P.store_mode, blockDim.x);
          for (int idx = threadIdx.x; idx < tb * n; idx += blockDim.x, wk.step()) {
               const int t = wk.t(), j = wk.j();
               if (tile.v0 + t < vn0) {
                    const C y = (j == 0) ? b1[t * sms + gpad(N)] : cadd(b0[t * sms + gpad(N)], res[t * sms + gpad(__ldg(lg + j - 1))]);
                    dst_of<C>(P, tile, A, t)[j * P.os] = y;
               }
          }
     } else if (kind == GB_KIND_R2C) {
          const int nc = n / 2 + 1;
          C *src = res;
          if (half) {
               /* hc2c post-pass (rdft/ct-hc2c.c:197-210) into the free buffer */
               C *dst = (res == b0) ? b1 : b0;
               const C *__restrict__ th = (const C *)P.tw_half;
               for (int idx = threadIdx.x; idx < tb * nc; idx += blockDim.x) {
                    const int t = idx / nc, k = idx - t * nc;
                    C a = res[t * sms + gpad((k % N))], b = res[t * sms + gpad(((N - k) % N))];
                    b.y = -b.y;
                    C ev = cscale(cadd(a, b), (R)0.5);
                    C dd = csub(a, b);
                    C od = mk<C>(dd.y * (R)0.5, -dd.x * (R)0.5);
                    dst[t * sms + gpad(k)] = cadd(ev, cmul(__ldg(th + k), od));
               }
               __syncthreads();
               src = dst;
          }
          for (int idx = threadIdx.x; idx < tb * nc; idx += blockDim.x) {
               int t, k;
               tile_index(idx, tb, nc, P.store_mode, t, k, P.ltb);
               if (tile.v0 + t < vn0) dst_of<C>(P, tile, A, t)[k * P.os] = src[t * sms + gpad(k)];
          }
     } else if (kind == GB_KIND_C2R) {
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x) {
               int t, j;
               tile_index(idx, tb, N, P.store_mode, t, j, P.ltb);
               if (tile.v0 + t < vn0) {
                    R *r = dst_of<R>(P, tile, A, t);
                    const C y = res[t * sms + gpad(j)];
                    if (!half) r[j * P.os] = y.x;
                    else if (P.real_pairs) ((C *)r)[j] = y;
                    else { r[2 * j * P.os] = y.x; r[(2 * j + 1) * P.os] = y.y; }
               }
          }
     }
     __syncthreads();
}

template <typename C>
__global__ void __launch_bounds__(512) k_gen(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     extern __shared__ __align__(16) unsigned char gb_smem[];
     C *b0 = (C *)gb_smem;
     C *b1 = b0 + P.tb * gen_sms(P.nfft);
     gen_addr A;
     A.in = in; A.out = out; A.pin = 0; A.pout = 0; A.l2only = 0;
     for (long long blk = blockIdx.x; blk < P.nblocks; blk += gridDim.x) {
          const tile_t tile = tile_of(P, blk);
          gen_tile<C>(P, tile, A, b0, b1);
     }
}

/* rank-0 problems: copy (dft/rank0 and rdft/rank0.c semantics) */
template <typename C>
__global__ void k_copy(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     for (long long blk = blockIdx.x; blk < P.nblocks; blk += gridDim.x) {
          const tile_t tile = tile_of(P, blk);
          for (int t = threadIdx.x; t < P.tb; t += blockDim.x) {
               const long long v = tile.v0 + t;
               if (v < P.vn[0])
                    ((C *)out)[tile.bo + v * P.vos[0]] = ((const C *)in)[tile.bi + v * P.vis[0]];
          }
     }
}

} /* namespace gb */
