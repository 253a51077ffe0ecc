/*
 * Tensor-core form of the radix-16 stages (tcgen05, split FP16, FP32
 * accumulation), for batched c2c of N = 256 .. 4096 in any layout (rows,
 * adjacent columns, or the two passes of a 65536 = 256 x 256 four-step with
 * its W_N^(n2 k1) twiddle).  N = 512, 1024, 2048 begin with one FP32 stage
 * of radix 2, 4 or 8, as the register kernels do; every radix-16 stage is a
 * GEMM.  Two builds: CTAS = 2, two CTAs per SM, row tiles of aligned
 * transforms copied in by the TMA engine (cp.async.bulk) while the previous
 * tile is transformed; CTAS = 3, three CTAs per SM (80 registers a thread,
 * no copy-in buffer), tiles gathered with plain loads while the SM's other
 * CTAs compute.
 *
 * Per stage, each of the CTA's 256 threads owns one radix-16 butterfly: it
 * gathers its 16 inputs from the shared-memory copy of the transform(s),
 * applies the stage twiddles in FP32, scales the row by a power of two so
 * its largest component sits near 2^12 (exact, undone on the outputs; keeps
 * the FP16 parts in range for inputs spanning many decades), splits every
 * value into FP16 hi + lo and writes its 96-element A row.  One thread then
 * issues, per 128-row group, six K=16 MMAs (128 x 32 x 96) into TMEM and
 * commits them to an mbarrier; every thread reads its row back with
 * tcgen05.ld (32 FP32 columns: 16 real then 16 imaginary outputs), undoes the
 * scale and writes the Stockham outputs for the next stage.  This is the
 * reference's radix-16 codelet (n1_16/t1_16, generated, absent from the
 * checkout) computed as a small complex DFT-matrix GEMM.
 *
 * Waits are bounded (mbarrier try_wait with a 2 s wall-clock limit); on a
 * timeout the CTA records GB_STATUS_COPY_TIMEOUT, frees its TMEM and exits.
 */
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdio.h>
#include "fft_kernels.cuh"
#include "fft_tc.cuh"

namespace gb {

/* layout constants: A tile of one 128-row group (K = 96), B (N = 32, K = 96) */
#define TC_LBO_A 2048u   /* 16 core matrices of 8 rows along M, 128 B each */
#define TC_LBO_B 512u    /* 4 core matrices of 8 rows along N */
#define TC_A_BYTES (12u * TC_LBO_A)
#define TC_B_BYTES (12u * TC_LBO_B)

/* ---------------------------------------------------------------- self test
 * D (128 x 32, f32) = A (128 x 16*ks, f16, row-major) . B (32 x 16*ks)^T,
 * through the same descriptors and TMEM path the FFT kernel uses. */
__global__ void __launch_bounds__(128) k_tc_selftest(const __half *A, const __half *B, float *D, int ks, int *status)
{
     extern __shared__ __align__(1024) unsigned char sm[];
     __shared__ uint32_t tbase;
     __shared__ __align__(8) unsigned long long bar;
     const int K = 16 * ks;
     unsigned char *As = sm, *Bs = sm + TC_A_BYTES;
     for (int i = threadIdx.x; i < 128 * K; i += blockDim.x)
          *(__half *)(As + tc::kmajor_off(i / K, i % K, TC_LBO_A)) = A[i];
     for (int i = threadIdx.x; i < 32 * K; i += blockDim.x)
          *(__half *)(Bs + tc::kmajor_off(i / K, i % K, TC_LBO_B)) = B[i];
     fence_proxy_async_smem();
     if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 32);
     if (threadIdx.x == 0) { mbar_init(&bar, 1); mbar_fence_init(); }
     tc::fence_before_sync();
     __syncthreads();
     tc::fence_after_sync();
     const uint32_t d = tbase;
     if (threadIdx.x == 0) {
          const uint32_t a0 = tc::smem_addr(As), b0 = tc::smem_addr(Bs);
          for (int s = 0; s < ks; ++s)
               tc::mma_f16(d, tc::smem_desc(a0 + 2u * s * TC_LBO_A, TC_LBO_A, 128u),
                           tc::smem_desc(b0 + 2u * s * TC_LBO_B, TC_LBO_B, 128u), tc::idesc_f16(128, 32), s > 0);
          tc::mma_commit(&bar);
     }
     const bool ok = __syncthreads_and(mbar_wait(&bar, 0, 2000000000ull));
     tc::fence_after_sync();
     if (ok) {
          const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
          float v[32];
          tc::tmem_ld32(d + ((uint32_t)(32 * w) << 16), v);
          for (int c = 0; c < 32; ++c) D[(32 * w + lane) * 32 + c] = v[c];
     } else if (threadIdx.x == 0 && status) {
          atomicExch(status, GB_STATUS_COPY_TIMEOUT);
     }
     tc::fence_before_sync();
     __syncthreads();
     if (threadIdx.x < 32) tc::tmem_dealloc(d, 32);
}

/* ---------------------------------------------------------------- FFT */

/* power of two 2^e with e chosen so that max|v| * 2^e lies in [2^12, 2^13) */
__device__ __forceinline__ float row_scale(float m)
{
     if (!(m > 0.f) || !isfinite(m)) return 1.f;
     int e;
     frexpf(m, &e);   /* m = f * 2^e, f in [0.5, 1) */
     return ldexpf(1.f, 13 - e);
}

/* Bulk copy of one row tile (TB transforms of N points, unit stride, each
 * transform 16-byte aligned) into pre, completion on bar (one thread). */
template <int N>
__device__ __forceinline__ void tc_prefetch(const gb_pass &P, const void *in, long long blk, float2 *pre,
                                            unsigned long long *bar)
{
     const tile_t tl = tile_of(P, blk);
     const long long rem = P.vn[0] - tl.v0;
     const int ntr = rem < P.tb ? (int)rem : P.tb;
     mbar_expect_tx(bar, (unsigned)(N * 8) * (unsigned)ntr);
     for (int t = 0; t < ntr; ++t)
          bulk_g2s(pre + t * N, (const float2 *)in + tl.bi + (tl.v0 + t) * P.vis[0], (unsigned)(N * 8), bar);
}

template <int LOGN, int DIR, int CTAS>
__global__ void __launch_bounds__(256, CTAS) k_tc_fft(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     constexpr int N = 1 << LOGN;
     constexpr int T = N / 16;           /* butterflies per transform per stage */
     constexpr int TB = 256 / T;         /* transforms per CTA */
     constexpr int R0 = reg_r0(N);       /* 16, or the radix of an FP32 first stage */
     constexpr int NS0 = R0 == 16 ? 1 : R0;
     constexpr int S = R0 == 16 ? LOGN / 4 : (LOGN - (R0 == 2 ? 1 : R0 == 4 ? 2 : 3)) / 4;   /* GEMM stages */
     /* the tile in dat takes the register kernels' swizzled layout (element p
      * of transform t at t * SMS + pad_for(N, p)): the strided stage stores
      * stay free of bank conflicts */
     constexpr int SMS = reg_sms(N);
     static_assert(256 / T * SMS * 8 <= 2 * (int)TC_A_BYTES, "the swizzled tile fits the A operand's memory");
     extern __shared__ __align__(1024) unsigned char sm[];
     __shared__ uint32_t tbase;
     __shared__ __align__(8) unsigned long long bar, pbar;
     unsigned char *As = sm;                           /* 2 groups x 24 KB */
     unsigned char *Bs = sm + 2 * TC_A_BYTES;          /* 6 KB */
     /* the next row tile, copied in by the TMA engine while this one is
      * transformed (32 KB; two-CTA build only) */
     float2 *pre = (float2 *)(sm + 2 * TC_A_BYTES + TC_B_BYTES);
     /* the tile (TB x N complex, 32 KB) shares the A operand's 48 KB: a
      * stage reads it into registers before A is written, and the MMA has
      * completed before the stage's results are written back */
     float2 *dat = (float2 *)As;
     const float2 *__restrict__ tw = (const float2 *)P.tw;
     const float2 *__restrict__ tws = (const float2 *)P.tw_stage;
     const int m = threadIdx.x;          /* butterfly row */
     const int tl = m / T, j = m - tl * T;
     const int g = m >> 7;               /* 128-row MMA group */

     /* row tiles of 16-byte aligned transforms arrive by bulk copy */
     bool pref = CTAS == 2 && P.load_mode == GB_MOVE_ROWS && P.is == 1 && ((unsigned long long)in & 15) == 0;
     for (int d = 0; d < P.nv; ++d) pref = pref && (P.vis[d] & 1) == 0;

     /* B: real form of the 16-point DFT matrix for this direction, split
      * hi/lo: rows n < 16 give Re(Y[n]), rows 16.. give Im(Y[n-16]) */
     for (int i = threadIdx.x; i < 32 * 96; i += blockDim.x) {
          const int n = i / 96, k = i - n * 96;
          const int q = n & 15, blk = k >> 4, r = k & 15;
          float2 w = __ldg(tw + ((q * r) & 15) * (N / 16));   /* exp(-2 pi i q r / 16) */
          if (DIR > 0) w.y = -w.y;
          /* Re(Y) = Fr Xr - Fi Xi ; Im(Y) = Fi Xr + Fr Xi */
          float c;
          const bool xr = (blk == 0 || blk == 2 || blk == 4);
          if (n < 16) c = xr ? w.x : -w.y;
          else c = xr ? w.y : w.x;
          const __half ch = __float2half_rn(c);
          const __half cl = __float2half_rn(c - __half2float(ch));
          *(__half *)(Bs + tc::kmajor_off(n, k, TC_LBO_B)) = (blk >= 4) ? cl : ch;
     }
     if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 64);
     if (threadIdx.x == 0) {
          mbar_init(&bar, 1);
          mbar_init(&pbar, 1);
          mbar_fence_init();
     }
     tc::fence_before_sync();
     __syncthreads();
     tc::fence_after_sync();
     const uint32_t tmem = tbase;
     unsigned phase = 0, pphase = 0;
     bool ok = true, pending = false;
     if (pref && threadIdx.x == 0 && blockIdx.x < P.nblocks) tc_prefetch<N>(P, in, blockIdx.x, pre, &pbar);
     pending = pref && blockIdx.x < P.nblocks;

     for (long long blk = blockIdx.x; blk < P.nblocks && ok; blk += gridDim.x) {
          const tile_t tile = tile_of(P, blk);
          /* src: where the first stage reads the tile (the bulk-copied buffer,
           * or the tile gathered into dat with plain loads) */
          const float2 *src = dat;
          if (pref) {
               ok = __syncthreads_and(mbar_wait(&pbar, pphase, 2000000000ull));
               if (!ok) break;   /* (the copy stays pending: waited for below) */
               pphase ^= 1u;
               pending = false;
               src = pre;
          } else {
               /* element-fast for unit-stride rows, transform-fast for
                * adjacent columns (four-step tiles, strided axes) */
               for (int i = threadIdx.x; i < TB * N; i += blockDim.x) {
                    int t, e;
                    if (P.load_mode == GB_MOVE_COLS) { t = i & (TB - 1); e = i / TB; }
                    else { t = i / N; e = i - t * N; }
                    const long long v = tile.v0 + t;
                    dat[t * SMS + pad_for(N, e)] = (v < P.vn[0]) ? ((const float2 *)in)[tile.bi + v * P.vis[0] + e * P.is]
                                                                 : make_float2(0.f, 0.f);
               }
               __syncthreads();
          }
          if constexpr (R0 != 16) {
               /* first stage of radix R0 in FP32 (as the register kernels'),
                * from src into dat */
               constexpr int B = 16 / R0;
               float2 x[16];
               if (src == pre) {
#pragma unroll
                    for (int e = 0; e < 16; ++e) x[e] = pre[tl * N + j + e * T];
               } else {
#pragma unroll
                    for (int e = 0; e < 16; ++e) x[e] = dat[tl * SMS + pad_for(N, j + e * T)];
               }
               __syncthreads();
#pragma unroll
               for (int b = 0; b < B; ++b) {
                    float2 v[R0];
#pragma unroll
                    for (int r = 0; r < R0; ++r) v[r] = x[b + r * B];
                    bfly<R0, DIR>::run(v);
                    const int jj = j + b * T;
#pragma unroll
                    for (int q = 0; q < R0; ++q) dat[tl * SMS + pad_for(N, jj * R0 + q)] = v[q];
               }
               if (src == pre && threadIdx.x == 0 && blk + gridDim.x < P.nblocks) {
                    /* every thread has read the buffer (the barrier above) */
                    fence_proxy_async_smem();
                    tc_prefetch<N>(P, in, blk + gridDim.x, pre, &pbar);
               }
               pending = src == pre && blk + gridDim.x < P.nblocks;
               src = dat;
               __syncthreads();
          }
          int NS = NS0;
#pragma unroll 1
          for (int s = 0; s < S; ++s) {
               float2 x[16];
               float2 *dt = dat + tl * SMS;
               if (src == pre) {
#pragma unroll
                    for (int r = 0; r < 16; ++r) x[r] = pre[tl * N + j + r * T];
               } else {
#pragma unroll
                    for (int r = 0; r < 16; ++r) x[r] = dt[pad_for(N, j + r * T)];
               }
               const int k = j & (NS - 1);
               if (NS > 1) apply_stage_twiddles16<DIR>(x, tws + stage_tw_off(N, NS), k, NS);
               float mx = 0.f;
#pragma unroll
               for (int r = 0; r < 16; ++r) mx = fmaxf(mx, fmaxf(fabsf(x[r].x), fabsf(x[r].y)));
               const float sc = row_scale(mx), inv = 1.f / sc;
               /* every thread has its x: the tile's memory becomes A (and a
                * bulk-copied tile's buffer is free for the next one) */
               __syncthreads();
               if (src == pre) {
                    if (threadIdx.x == 0 && blk + gridDim.x < P.nblocks) {
                         fence_proxy_async_smem();
                         tc_prefetch<N>(P, in, blk + gridDim.x, pre, &pbar);
                    }
                    pending = blk + gridDim.x < P.nblocks;
                    src = dat;
               }
               /* A row: [hi.re | hi.im | lo.re | lo.im | hi.re | hi.im] */
               {
                    __half hr[16], hi[16], lr[16], li[16];
#pragma unroll
                    for (int r = 0; r < 16; ++r) {
                         const float a = x[r].x * sc, b = x[r].y * sc;
                         hr[r] = __float2half_rn(a);
                         hi[r] = __float2half_rn(b);
                         lr[r] = __float2half_rn(a - __half2float(hr[r]));
                         li[r] = __float2half_rn(b - __half2float(hi[r]));
                    }
                    unsigned char *arow = As + g * TC_A_BYTES;
                    const int row = m & 127;
#pragma unroll
                    for (int c = 0; c < 12; ++c) {   /* 12 chunks of 8 K-elements */
                         const __half *hsrc = (c < 2) ? hr + 8 * c : (c < 4) ? hi + 8 * (c - 2) : (c < 6) ? lr + 8 * (c - 4)
                                            : (c < 8) ? li + 8 * (c - 6) : (c < 10) ? hr + 8 * (c - 8) : hi + 8 * (c - 10);
                         uint4 pk;
                         pk.x = (uint32_t)__half_as_ushort(hsrc[0]) | ((uint32_t)__half_as_ushort(hsrc[1]) << 16);
                         pk.y = (uint32_t)__half_as_ushort(hsrc[2]) | ((uint32_t)__half_as_ushort(hsrc[3]) << 16);
                         pk.z = (uint32_t)__half_as_ushort(hsrc[4]) | ((uint32_t)__half_as_ushort(hsrc[5]) << 16);
                         pk.w = (uint32_t)__half_as_ushort(hsrc[6]) | ((uint32_t)__half_as_ushort(hsrc[7]) << 16);
                         *(uint4 *)(arow + tc::kmajor_off(row, 8 * c, TC_LBO_A)) = pk;
                    }
               }
               fence_proxy_async_smem();
               tc::fence_before_sync();
               __syncthreads();
               tc::fence_after_sync();
               if (threadIdx.x == 0) {
                    const uint32_t b0 = tc::smem_addr(Bs);
                    for (int gg = 0; gg < 2; ++gg) {
                         const uint32_t a0 = tc::smem_addr(As + gg * TC_A_BYTES);
#pragma unroll 1
                         for (int q = 0; q < 6; ++q)
                              tc::mma_f16(tmem + 32u * gg, tc::smem_desc(a0 + 2u * q * TC_LBO_A, TC_LBO_A, 128u),
                                          tc::smem_desc(b0 + 2u * q * TC_LBO_B, TC_LBO_B, 128u), tc::idesc_f16(128, 32),
                                          q > 0);
                    }
                    tc::mma_commit(&bar);
               }
               ok = __syncthreads_and(mbar_wait(&bar, phase, 2000000000ull));
               phase ^= 1u;
               if (!ok) break;
               tc::fence_after_sync();
               float v[32];
               {
                    const int w = threadIdx.x >> 5;
                    tc::tmem_ld32(tmem + ((uint32_t)(32 * (w & 3)) << 16) + 32u * (uint32_t)(w >> 2), v);
               }
               const bool last = (s == S - 1);
               if (!last) {
                    const int base = (j / NS) * NS * 16 + k;
                    if (NS == 1 && pad_mult(N) == 2) {
                         /* 16 consecutive outputs, 16-byte aligned in the swizzle:
                          * eight 128-bit stores, a quarter warp's conflict-free */
                         float4 *d4 = (float4 *)(dt + pad_for(N, base));
#pragma unroll
                         for (int q = 0; q < 8; ++q)
                              d4[q] = make_float4(v[2 * q] * inv, v[16 + 2 * q] * inv, v[2 * q + 1] * inv,
                                                  v[17 + 2 * q] * inv);
                    } else {
#pragma unroll
                         for (int q = 0; q < 16; ++q) dt[pad_for(N, base + q * NS)] = make_float2(v[q] * inv, v[16 + q] * inv);
                    }
               } else {
                    /* outputs j + q*T in natural order; four-step passes also
                     * apply W_postN^(v*k) */
                    const long long vv = tile.v0 + tl;
                    float2 y[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) y[q] = make_float2(v[q] * inv, v[16 + q] * inv);
                    if (P.post_N) apply_post_twiddles<float2, 16, T>(P, P.post_vdim ? tile.vpost : vv, j, y);
                    if (P.store_mode == GB_MOVE_DIRECT) {
                         if (vv < P.vn[0]) {
                              float2 *o = (float2 *)out + tile.bo + vv * P.vos[0] + j;
#pragma unroll
                              for (int q = 0; q < 16; ++q) o[q * T] = y[q];
                         }
                    } else {
#pragma unroll
                         for (int q = 0; q < 16; ++q) dt[pad_for(N, j + q * T)] = y[q];
                    }
               }
               tc::fence_before_sync();
               __syncthreads();
               tc::fence_after_sync();
               NS *= 16;
          }
          if (ok && P.store_mode != GB_MOVE_DIRECT) {
               for (int i = threadIdx.x; i < TB * N; i += blockDim.x) {
                    int t, e;
                    if (P.store_mode == GB_MOVE_COLS) { t = i & (TB - 1); e = i / TB; }
                    else { t = i / N; e = i - t * N; }
                    const long long v = tile.v0 + t;
                    if (v < P.vn[0]) ((float2 *)out)[tile.bo + v * P.vos[0] + e * P.os] = dat[t * SMS + pad_for(N, e)];
               }
               __syncthreads();
          }
     }
     if (!ok && threadIdx.x == 0 && P.status) atomicExch(P.status, GB_STATUS_COPY_TIMEOUT);
     /* a copy still in flight lands before the CTA's shared memory goes */
     if (pending && threadIdx.x == 0) mbar_wait(&pbar, pphase, 2000000000ull);
     tc::fence_before_sync();
     __syncthreads();
     if (threadIdx.x < 32) tc::tmem_dealloc(tmem, 64);
}

} /* namespace gb */

using namespace gb;

extern "C" int *gb_device_status_ptr(void);

/* bytes of dynamic shared memory the tensor-core FFT needs: A (shared with
 * the tile), B, and (two-CTA build) the buffer the next row tile is copied
 * into */
extern "C" int gb_tc_smem(int nfft, int ctas)
{
     return (int)(2 * TC_A_BYTES + TC_B_BYTES) + (ctas == 2 ? 256 * 16 * 8 : 0) + 0 * nfft;
}

template <int CTAS> static const void *tc_kernel(int nfft, int dir)
{
     switch (nfft) {
     case 256: return dir < 0 ? (const void *)k_tc_fft<8, -1, CTAS> : (const void *)k_tc_fft<8, 1, CTAS>;
     case 512: return dir < 0 ? (const void *)k_tc_fft<9, -1, CTAS> : (const void *)k_tc_fft<9, 1, CTAS>;
     case 1024: return dir < 0 ? (const void *)k_tc_fft<10, -1, CTAS> : (const void *)k_tc_fft<10, 1, CTAS>;
     case 2048: return dir < 0 ? (const void *)k_tc_fft<11, -1, CTAS> : (const void *)k_tc_fft<11, 1, CTAS>;
     case 4096: return dir < 0 ? (const void *)k_tc_fft<12, -1, CTAS> : (const void *)k_tc_fft<12, 1, CTAS>;
     default: return 0;
     }
}

/* the build for ctas CTAs per SM (2 or 3) */
extern "C" const void *gb_tc_kernel(int nfft, int dir, int ctas)
{
     return ctas == 3 ? tc_kernel<3>(nfft, dir) : ctas == 2 ? tc_kernel<2>(nfft, dir) : 0;
}

/* One-CTA GEMM through the tcgen05 path (device pointers): D = A . B^T,
 * A 128 x 16ks, B 32 x 16ks (f16, row-major), D 128 x 32 (f32). */
extern "C" int gb_tc_selftest(const void *A, const void *B, float *D, int ks)
{
     int smem = 64 * 1024;
     if (ks < 1 || ks > 6) return -1;
     if (cudaFuncSetAttribute((const void *)k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
          return -1;
     k_tc_selftest<<<1, 128, smem>>>((const __half *)A, (const __half *)B, D, ks, gb_device_status_ptr());
     if (cudaGetLastError() != cudaSuccess) return -1;
     return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}
