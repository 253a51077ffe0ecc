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
 *             complex FFT, odd n through the full-length one).
 *
 * These replace, on the reference side: dft/ct.c + dft/dftw-direct.c +
 * dft/direct.c with their codelets (the stages), dft/vrank-geq1.c (the batch
 * is the grid), dft/buffered.c and dft/indirect*.c (strided tiles are staged
 * through shared memory), rdft/ct-hc2c.c + rdft/ct-hc2c-direct.c (fused
 * pre/post-passes), dft/generic.c (small prime radices as register
 * butterflies) and dft/bluestein.c (fused convolution).
 */
#pragma once
#include "fft_device.cuh"
#include "gb_types.h"

namespace gb {

__host__ __device__ constexpr int pad_idx(int p) { return p + (p >> 4); }

/* Shared-memory stride (in complex elements) of one transform in k_reg. */
__host__ __device__ constexpr int reg_sms(int nfft) { return pad_idx(nfft) + 2; }

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
};

__device__ __forceinline__ tile_t tile_of(const gb_pass &P, long long blk)
{
     tile_t t;
     long long rest = blk / P.ntiles0;
     t.v0 = (blk - rest * P.ntiles0) * P.tb;
     t.bi = 0; t.bo = 0;
#pragma unroll
     for (int d = 1; d < GB_MAXV; ++d) {
          if (d < P.nv) {
               long long q = rest / P.vn[d];
               long long i = rest - q * P.vn[d];
               rest = q;
               t.bi += i * P.vis[d];
               t.bo += i * P.vos[d];
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

/* exp(sign 2 pi i m / N) from the two-level table (four-step twiddle) */
template <typename C> __device__ __forceinline__ C post_twiddle(const gb_pass &P, long long m)
{
     m %= P.post_N;
     long long hi = m / P.post_S, lo = m - hi * P.post_S;
     C a = __ldg((const C *)P.post_lo + lo), b = __ldg((const C *)P.post_hi + hi);
     C w = cmul(a, b);
     if (P.sign > 0) w.y = -w.y;
     return w;
}

/* Cooperative copy of L complex elements per transform between HBM and
 * shared memory, for the tb transforms of one tile.  ROWS walks the element
 * index fastest (unit-stride transforms); COLS walks the transform index
 * fastest (transforms adjacent in memory, e.g. columns of a row-major
 * array).  PADDED applies the k_reg shared-memory swizzle. */
template <typename C, bool PADDED, bool PAIRS_REAL>
__device__ __forceinline__ void coop_load(const gb_pass &P, const void *in, C *sm, int sms, const tile_t &tl,
                                          int L, int mode)
{
     const int tb = P.tb;
     const int total = tb * L;
     for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
          int t, j;
          if (mode == GB_MOVE_COLS) { t = idx % tb; j = idx / tb; }
          else { t = idx / L; j = idx - t * L; }
          long long v = tl.v0 + t;
          if (v < P.vn[0]) {
               long long base = tl.bi + v * P.vis[0];
               C x = PAIRS_REAL ? io<C>::ldpair(in, base, j, P.is, P.real_pairs) : io<C>::ldc(in, base, j, P.is);
               sm[t * sms + (PADDED ? pad_idx(j) : j)] = x;
          }
     }
}

template <typename C, bool PADDED, bool PAIRS_REAL>
__device__ __forceinline__ void coop_store(const gb_pass &P, void *out, const C *sm, int sms, const tile_t &tl,
                                           int L, int mode)
{
     const int tb = P.tb;
     const int total = tb * L;
     for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
          int t, j;
          if (mode == GB_MOVE_COLS) { t = idx % tb; j = idx / tb; }
          else { t = idx / L; j = idx - t * L; }
          long long v = tl.v0 + t;
          if (v < P.vn[0]) {
               long long base = tl.bo + v * P.vos[0];
               C x = sm[t * sms + (PADDED ? pad_idx(j) : j)];
               if (PAIRS_REAL) io<C>::stpair(out, base, j, P.os, P.real_pairs, x);
               else io<C>::stc(out, base, j, P.os, x);
          }
     }
}

/* ======================================================================
 * k_reg: power-of-two, register-resident
 * ==================================================================== */

template <typename C, int N, int DIR, int NS>
__device__ __forceinline__ void reg_stages(C (&x)[reg_e(N)], int tid, C *smt, const C *__restrict__ tw)
{
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int RAD = (NS == 1) ? reg_r0(N) : E;
     constexpr int B = E / RAD;
     constexpr bool LAST = (NS * RAD == N);
#pragma unroll
     for (int b = 0; b < B; ++b) {
          const int j = tid + b * T;
          const int k = j & (NS - 1);
          C v[RAD];
#pragma unroll
          for (int r = 0; r < RAD; ++r) v[r] = x[b + r * B];
          if (NS > 1) {
#pragma unroll
               for (int r = 1; r < RAD; ++r) v[r] = cmul(v[r], twid<DIR>(tw, r * k * (N / (NS * RAD))));
          }
          bfly<RAD, DIR>::run(v);
          if (LAST) {
#pragma unroll
               for (int q = 0; q < RAD; ++q) x[b + q * B] = v[q];
          } else {
               const int base = (j / NS) * NS * RAD + k;
#pragma unroll
               for (int q = 0; q < RAD; ++q) smt[pad_idx(base + q * NS)] = v[q];
          }
     }
     if constexpr (!LAST) {
          __syncthreads();
#pragma unroll
          for (int e = 0; e < E; ++e) x[e] = smt[pad_idx(tid + T * e)];
          __syncthreads();
          reg_stages<C, N, DIR, NS * RAD>(x, tid, smt, tw);
     }
}

/* Threads per CTA for k_reg: T = nfft/E threads per transform, at most 512
 * per CTA unless one transform needs more (several transforms per CTA for
 * short lengths). */
__host__ __device__ constexpr int reg_maxthreads(int nfft)
{
     return (nfft / reg_e(nfft)) > 512 ? (nfft / reg_e(nfft)) : 512;
}

template <typename C, int LOGN, int DIR, int KIND>
__global__ void __launch_bounds__(reg_maxthreads(1 << LOGN)) k_reg(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
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
     const C *__restrict__ tw = (const C *)P.tw;

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
                    coop_load<C, true, false>(P, in, sm, SMS, tile, nn, P.load_mode);
                    __syncthreads();
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                         const int k = tid + T * e;
                         x[e] = (k < nn) ? cmul(smt[pad_idx(k)], cconj(__ldg(w + k))) : mk<C>(0, 0);
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
                    for (int e = 0; e < E; ++e) smt[pad_idx(tid + T * e)] = x[e];
                    __syncthreads();
                    coop_store<C, true, false>(P, out, sm, SMS, tile, nn, P.store_mode);
                    __syncthreads();
               }
               continue;
          }

          /* ---------------- load (and c2r pre-pass) ---------------- */
          if constexpr (KIND == GB_KIND_C2R) {
               /* X[0..N] -> shared, then Z'[k] = (X[k] + conj X[N-k])
                *                 + i conj(W_2N^k) (X[k] - conj X[N-k])  */
               coop_load<C, true, false>(P, in, sm, SMS, tile, N + 1, P.load_mode);
               __syncthreads();
               const C *__restrict__ th = (const C *)P.tw_half;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int k = tid + T * e;
                    C a = smt[pad_idx(k)], b = smt[pad_idx(N - k)];
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
               coop_load<C, true, KIND == GB_KIND_R2C>(P, in, sm, SMS, tile, N, P.load_mode);
               __syncthreads();
#pragma unroll
               for (int e = 0; e < E; ++e) x[e] = smt[pad_idx(tid + T * e)];
               __syncthreads();
          }

          /* ---------------- stages ---------------- */
          reg_stages<C, N, DIR, 1>(x, tid, smt, tw);

          /* ---------------- store (and r2c post-pass) ---------------- */
          if constexpr (KIND == GB_KIND_R2C) {
               /* X[k] = (Z[k] + conj Z[N-k])/2 + W_2N^k (Z[k] - conj Z[N-k])/(2i), k = 0..N */
#pragma unroll
               for (int e = 0; e < E; ++e) smt[pad_idx(tid + T * e)] = x[e];
               __syncthreads();
               const C *__restrict__ th = (const C *)P.tw_half;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int k = tid + T * e;
                    C a = smt[pad_idx(k)], b = smt[pad_idx((N - k) & (N - 1))];
                    b.y = -b.y;
                    C ev = cscale(cadd(a, b), (R)0.5);
                    C dd = csub(a, b);
                    C od = mk<C>(dd.y * (R)0.5, -dd.x * (R)0.5);
                    C w = __ldg(th + k);
                    x[e] = cadd(ev, cmul(w, od));
               }
               C last = smt[pad_idx(0)];
               __syncthreads();
               if (P.store_mode == GB_MOVE_DIRECT) {
                    if (valid) {
#pragma unroll
                         for (int e = 0; e < E; ++e) io<C>::stc(out, bo, tid + T * e, P.os, x[e]);
                         if (tid == 0) io<C>::stc(out, bo, N, P.os, mk<C>(last.x - last.y, 0));
                    }
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) smt[pad_idx(tid + T * e)] = x[e];
                    if (tid == 0) smt[pad_idx(N)] = mk<C>(last.x - last.y, 0);
                    __syncthreads();
                    coop_store<C, true, false>(P, out, sm, SMS, tile, N + 1, P.store_mode);
                    __syncthreads();
               }
          } else {
               if constexpr (KIND == GB_KIND_C2C) {
                    if (P.post_N) {
#pragma unroll
                         for (int e = 0; e < E; ++e)
                              x[e] = cmul(x[e], post_twiddle<C>(P, v * (long long)(tid + T * e)));
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
                    for (int e = 0; e < E; ++e) smt[pad_idx(tid + T * e)] = x[e];
                    __syncthreads();
                    coop_store<C, true, RP>(P, out, sm, SMS, tile, N, P.store_mode);
                    __syncthreads();
               }
          }
     }
}

/* ======================================================================
 * k_gen: runtime radix list, shared-memory ping-pong
 * ==================================================================== */

template <typename C, int DIR, int RAD>
__device__ __forceinline__ void gen_stage(const C *src, C *dst, int N, int Ns, int tb, int sms,
                                          const C *__restrict__ tw)
{
     const int nb = N / RAD;
     const int twstep = N / (Ns * RAD);
     for (int idx = threadIdx.x; idx < tb * nb; idx += blockDim.x) {
          const int t = idx / nb;
          const int j = idx - t * nb;
          const C *s = src + t * sms;
          C *d = dst + t * sms;
          C v[RAD];
#pragma unroll
          for (int r = 0; r < RAD; ++r) v[r] = s[j + r * nb];
          const int k = j % Ns;
          if (Ns > 1) {
#pragma unroll
               for (int r = 1; r < RAD; ++r) v[r] = cmul(v[r], twid<DIR>(tw, r * k * twstep));
          }
          bfly<RAD, DIR>::run(v);
          const int base = (j / Ns) * Ns * RAD + k;
#pragma unroll
          for (int q = 0; q < RAD; ++q) d[base + q * Ns] = v[q];
     }
}

/* Runs all stages; returns the buffer holding the result (natural order). */
template <typename C, int DIR>
__device__ C *gen_fft(C *b0, C *b1, const gb_pass &P, int N, int sms, const C *__restrict__ tw)
{
     int Ns = 1;
     C *src = b0, *dst = b1;
     for (int s = 0; s < P.nrad; ++s) {
          const int r = P.rad[s];
          switch (r) {
          case 2: gen_stage<C, DIR, 2>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 3: gen_stage<C, DIR, 3>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 4: gen_stage<C, DIR, 4>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 5: gen_stage<C, DIR, 5>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 7: gen_stage<C, DIR, 7>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 8: gen_stage<C, DIR, 8>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 11: gen_stage<C, DIR, 11>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 13: gen_stage<C, DIR, 13>(src, dst, N, Ns, P.tb, sms, tw); break;
          case 16: gen_stage<C, DIR, 16>(src, dst, N, Ns, P.tb, sms, tw); break;
          default: break;
          }
          __syncthreads();
          Ns *= r;
          C *t = src; src = dst; dst = t;
     }
     return src;
}

template <typename C, int DIR>
__global__ void __launch_bounds__(1024) k_gen(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     typedef typename real_of<C>::T R;
     extern __shared__ __align__(16) unsigned char gb_smem[];
     const int N = P.nfft;
     const int sms = N + 1;
     C *b0 = (C *)gb_smem;
     C *b1 = b0 + P.tb * sms;
     const C *__restrict__ tw = (const C *)P.tw;
     const int n = P.n;
     const int kind = P.kind;
     const bool half = (kind == GB_KIND_R2C || kind == GB_KIND_C2R) && (n % 2 == 0);

     for (long long blk = blockIdx.x; blk < P.nblocks; blk += gridDim.x) {
          const tile_t tile = tile_of(P, blk);
          /* ---------------- load ---------------- */
          if (kind == GB_KIND_C2C) {
               coop_load<C, false, false>(P, in, b0, sms, tile, N, P.load_mode);
          } else if (kind == GB_KIND_R2C) {
               if (half) coop_load<C, false, true>(P, in, b0, sms, tile, N, P.load_mode);
               else {
                    /* odd n: real sequence as complex with zero imaginary part */
                    for (int idx = threadIdx.x; idx < P.tb * N; idx += blockDim.x) {
                         int t, j;
                         if (P.load_mode == GB_MOVE_COLS) { t = idx % P.tb; j = idx / P.tb; }
                         else { t = idx / N; j = idx - t * N; }
                         const long long v = tile.v0 + t;
                         if (v < P.vn[0]) {
                              const R *r = (const R *)in + tile.bi + v * P.vis[0];
                              b0[t * sms + j] = mk<C>(r[j * P.is], 0);
                         }
                    }
               }
          } else if (kind == GB_KIND_C2R) {
               const int nc = n / 2 + 1;
               coop_load<C, false, false>(P, in, b1, sms, tile, nc, P.load_mode);
               __syncthreads();
               if (half) {
                    const C *__restrict__ th = (const C *)P.tw_half;
                    for (int idx = threadIdx.x; idx < P.tb * N; idx += blockDim.x) {
                         const int t = idx / N, k = idx - t * N;
                         C a = b1[t * sms + k], b = b1[t * sms + N - k];
                         if (k == 0) { a.y = 0; b.y = 0; }
                         b.y = -b.y;
                         C s = cadd(a, b), d = csub(a, b);
                         C w = __ldg(th + k);
                         C cd = mk<C>(w.x * d.x + w.y * d.y, w.x * d.y - w.y * d.x);
                         b0[t * sms + k] = mk<C>(s.x - cd.y, s.y + cd.x);
                    }
               } else {
                    /* odd n: Hermitian extension of X[0..(n-1)/2] */
                    for (int idx = threadIdx.x; idx < P.tb * N; idx += blockDim.x) {
                         const int t = idx / N, k = idx - t * N;
                         C a = (k < nc) ? b1[t * sms + k] : cconj(b1[t * sms + (N - k)]);
                         if (k == 0) a.y = 0;
                         b0[t * sms + k] = a;
                    }
               }
          }
          __syncthreads();

          /* ---------------- stages ---------------- */
          C *res;
          if (DIR < 0) {
               res = gen_fft<C, -1>(b0, b1, P, N, sms, tw);
          } else {
               res = gen_fft<C, 1>(b0, b1, P, N, sms, tw);
          }

          /* ---------------- store ---------------- */
          if (kind == GB_KIND_C2C) {
               if (P.post_N) {
                    for (int idx = threadIdx.x; idx < P.tb * N; idx += blockDim.x) {
                         const int t = idx / N, k = idx - t * N;
                         const long long v = tile.v0 + t;
                         res[t * sms + k] = cmul(res[t * sms + k], post_twiddle<C>(P, v * (long long)k));
                    }
                    __syncthreads();
               }
               coop_store<C, false, false>(P, out, res, sms, tile, N, P.store_mode);
          } else if (kind == GB_KIND_R2C) {
               const int nc = n / 2 + 1;
               C *dst = (res == b0) ? b1 : b0;
               if (half) {
                    const C *__restrict__ th = (const C *)P.tw_half;
                    for (int idx = threadIdx.x; idx < P.tb * nc; idx += blockDim.x) {
                         const int t = idx / nc, k = idx - t * nc;
                         C a = res[t * sms + (k % N)], b = res[t * sms + ((N - k) % N)];
                         b.y = -b.y;
                         C ev = cscale(cadd(a, b), (R)0.5);
                         C dd = csub(a, b);
                         C od = mk<C>(dd.y * (R)0.5, -dd.x * (R)0.5);
                         dst[t * sms + k] = cadd(ev, cmul(__ldg(th + k), od));
                    }
                    __syncthreads();
                    coop_store<C, false, false>(P, out, dst, sms, tile, nc, P.store_mode);
               } else {
                    coop_store<C, false, false>(P, out, res, sms, tile, nc, P.store_mode);
               }
          } else if (kind == GB_KIND_C2R) {
               if (half) coop_store<C, false, true>(P, out, res, sms, tile, N, P.store_mode);
               else {
                    for (int idx = threadIdx.x; idx < P.tb * N; idx += blockDim.x) {
                         int t, j;
                         if (P.store_mode == GB_MOVE_COLS) { t = idx % P.tb; j = idx / P.tb; }
                         else { t = idx / N; j = idx - t * N; }
                         const long long v = tile.v0 + t;
                         if (v < P.vn[0]) ((R *)out)[tile.bo + v * P.vos[0] + j * P.os] = res[t * sms + j].x;
                    }
               }
          }
          __syncthreads();
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
