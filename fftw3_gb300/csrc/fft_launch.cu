/*
 * C-ABI launch layer: the host planner (C) reaches every device kernel
 * through the functions in this file.  No torch types, no C++ in the
 * signatures.  Also holds the FP64 twiddle / chirp generators, which replace
 * the reference's plan-time trig tables (kernel/twiddle.c:124-222,
 * kernel/trig.c:169-227, dft/bluestein.c:37-50) with device generation:
 * each factor is computed in FP64 with an exact integer argument reduction
 * and rounded once to the working precision.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <pthread.h>
#include "fft_kernels.cuh"

extern "C" const void *gb_reg_kernel_f(int logn, int kind, int dir);
extern "C" const void *gb_reg_kernel_d(int logn, int kind, int dir);
extern "C" const void *gb_tma_kernel_f(int logn, int kind, int dir, int groups);
extern "C" const void *gb_tma_kernel_d(int logn, int kind, int dir, int groups);
extern "C" const void *gb_tc_kernel(int nfft, int dir, int ctas);
extern "C" const void *gb_cols_tma_kernel(int logn, int dir, int groups);
extern "C" int gb_tc_smem(int nfft, int ctas);

namespace gb {

template <typename C>
__global__ void k_twiddles(C *dst, long long n, long long count, long long mul)
{
     typedef typename real_of<C>::T R;
     for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < count;
          j += (long long)gridDim.x * blockDim.x) {
          double c, s;
          long long m = (long long)(((unsigned long long)j * (unsigned long long)mul) % (unsigned long long)n);
          cexp_fp64(m, n, -1, &c, &s);
          dst[j] = mk<C>((R)c, (R)s);
     }
}

/* Stage twiddle table of a power-of-two length N (layout of gb_pass.tw_stage):
 * entry (stage NS, row q, k) = exp(-2 pi i k (N / (16 NS)) p / N) with
 * p = 2^q (four rows, float) or p = q + 1 (fifteen rows, double), FP64 with
 * the exact octant reduction, rounded once. */
template <typename C>
__global__ void k_stage_twiddles(C *dst, int N, int len)
{
     typedef typename real_of<C>::T R;
     constexpr int rows = stage_tw_rows(sizeof(C));
     for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < len; j += gridDim.x * blockDim.x) {
          int ns = reg_r0(N), idx = j;
          while (idx >= rows * ns) {
               idx -= rows * ns;
               ns *= 16;
          }
          const int q = idx / ns, k = idx - q * ns;
          const long long p = rows == 4 ? (1LL << q) : (long long)(q + 1);
          const long long m = ((long long)k * (N / (16 * ns)) * p) % N;
          double c, s;
          cexp_fp64(m, N, -1, &c, &s);
          dst[j] = mk<C>((R)c, (R)s);
     }
}

/* Stage twiddles of a runtime-radix pass (layout of gb_pass.tw_gen): the
 * stage of span Ns and radix R holds entries Ns - 1 + (r - 1) Ns + k =
 * exp(-2 pi i r k / (Ns R)), r = 1..R-1, k < Ns; the same values as the
 * full table's entries r k N / (Ns R) (FP64, exact octant reduction, rounded
 * once). */
struct gen_radices { int n; int r[GB_MAXRAD]; };
template <typename C>
__global__ void k_gen_stage_twiddles(C *dst, int N, gen_radices R)
{
     typedef typename real_of<C>::T RT;
     for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N - 1; j += gridDim.x * blockDim.x) {
          int ns = 1;
          for (int s = 0; s < R.n; ++s) {
               const int span = ns * R.r[s];
               if (j < span - 1) {
                    const int loc = j - (ns - 1), r = loc / ns + 1, k = loc - (r - 1) * ns;
                    double c, sn;
                    cexp_fp64((long long)r * k * (N / span), N, -1, &c, &sn);
                    dst[j] = mk<C>((RT)c, (RT)sn);
                    break;
               }
               ns = span;
          }
     }
}

/* Rows of the four-step twiddle: entry v T + t = exp(-2 pi i v t / N). */
template <typename C>
__global__ void k_post_rows(C *dst, long long N, int T, long long count)
{
     typedef typename real_of<C>::T R;
     for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < count;
          j += (long long)gridDim.x * blockDim.x) {
          const long long v = j / T, t = j - v * T;
          double c, s;
          cexp_fp64((v * t) % N, N, -1, &c, &s);
          dst[j] = mk<C>((R)c, (R)s);
     }
}

/* Bluestein chirp w[k] = exp(-sign * i * pi * k^2 / n): the index k^2 is
 * reduced modulo 2n exactly in 64-bit integers (dft/bluestein.c:37-50). */
template <typename C>
__global__ void k_chirp(C *dst, long long n, int sign)
{
     typedef typename real_of<C>::T R;
     for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
          k += (long long)gridDim.x * blockDim.x) {
          unsigned long long n2 = 2ull * (unsigned long long)n;
          unsigned long long ksq = ((unsigned long long)k * (unsigned long long)k) % n2;
          double c, s;
          cexp_fp64((long long)ksq, (long long)n2, -sign, &c, &s);
          dst[k] = mk<C>((R)c, (R)s);
     }
}

/* Padded chirp / nb, the convolution kernel whose spectrum Bluestein
 * multiplies by (dft/bluestein.c:52-80). */
template <typename C>
__global__ void k_chirp_pad(C *dst, const C *w, long long n, long long nb)
{
     typedef typename real_of<C>::T R;
     for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nb;
          k += (long long)gridDim.x * blockDim.x) {
          C v = mk<C>(0, 0);
          if (k < n) v = w[k];
          else if (nb - k < n) v = w[nb - k];
          dst[k] = mk<C>(v.x / (R)nb, v.y / (R)nb);
     }
}

/* Rader's omega[k] = exp(sign 2 pi i g^-k / p) / (p-1), with g^-k read from
 * the generator-power table as g^((p-1-k) mod (p-1)) (dft/rader.c:45-74). */
template <typename C>
__global__ void k_rader_omega(C *dst, const int *gpow, long long p, int sign)
{
     typedef typename real_of<C>::T R;
     const long long m = p - 1;
     for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m;
          k += (long long)gridDim.x * blockDim.x) {
          double c, s;
          cexp_fp64(gpow[(m - k) % m], p, sign, &c, &s);
          dst[k] = mk<C>((R)(c / (double)m), (R)(s / (double)m));
     }
}

/* Element-wise passes between the FFT passes of multi-pass plans: each CTA
 * takes a chunk of 4096 elements of one transform.  Tables: tw_half
 * (exp(-2 pi i k/n), k <= n/2) for the hc2c passes (rdft/ct-hc2c.c), chirp
 * and chirp_spec for Bluestein (dft/bluestein.c:82-128). */
template <typename C>
__global__ void __launch_bounds__(256) k_pointwise(const gb_pass P, const void *__restrict__ in, void *__restrict__ out)
{
     typedef typename real_of<C>::T R;
     const int M = P.nfft;
     const int L = (P.pw == GB_PW_HC2C_POST) ? M + 1
                 : (P.pw == GB_PW_CHIRP_OUT || P.pw == GB_PW_CHIRP_OUT_REAL) ? P.n
                 : (P.pw == GB_PW_HALF_COPY || P.pw == GB_PW_CHIRP_OUT_HALF) ? P.n / 2 + 1 : M;
     for (long long blk = blockIdx.x; blk < P.nblocks; blk += gridDim.x) {
          const long long tr = blk / P.pw_chunks;
          const int k0 = (int)(blk - tr * P.pw_chunks) * 4096;
          const tile_t tile = tile_of(P, tr);
          const long long ioff = tile.bi + tile.v0 * P.vis[0], ooff = tile.bo + tile.v0 * P.vos[0];
          const C *src = (const C *)in + ioff;
          C *dst = (C *)out + ooff;
          /* real transforms around a c2c or a convolution: offsets and strides
           * of the real side count reals */
          const R *rs = (const R *)in + ioff;
          R *rd = (R *)out + ooff;
          if (P.pw == GB_PW_PROMOTE || P.pw == GB_PW_REAL_PART || P.pw == GB_PW_HERM_EXT || P.pw == GB_PW_HALF_COPY) {
               for (int k = k0 + threadIdx.x; k < L && k < k0 + 4096; k += blockDim.x) {
                    if (P.pw == GB_PW_PROMOTE) dst[(long long)k * P.os] = mk<C>(rs[(long long)k * P.is], (R)0);
                    else if (P.pw == GB_PW_REAL_PART) rd[(long long)k * P.os] = src[(long long)k * P.is].x;
                    else if (P.pw == GB_PW_HALF_COPY) dst[(long long)k * P.os] = src[(long long)k * P.is];
                    else {
                         const int h = (2 * k <= P.n) ? k : P.n - k;
                         C z = src[(long long)h * P.is];
                         if (k == 0) z.y = 0;
                         else if (h != k) z.y = -z.y;
                         dst[(long long)k * P.os] = z;
                    }
               }
               continue;
          }
          for (int k = k0 + threadIdx.x; k < L && k < k0 + 4096; k += blockDim.x) {
               C y;
               if (P.pw == GB_PW_HC2C_POST) {
                    C a = src[(long long)(k % M) * P.is], b = src[(long long)((M - k) % M) * P.is];
                    b.y = -b.y;
                    C ev = cscale(cadd(a, b), (R)0.5), dd = csub(a, b);
                    C od = mk<C>(dd.y * (R)0.5, -dd.x * (R)0.5);
                    y = cadd(ev, cmul(__ldg((const C *)P.tw_half + k), od));
               } else if (P.pw == GB_PW_HC2C_PRE) {
                    C a = src[(long long)k * P.is], b = src[(long long)(M - k) * P.is];
                    if (k == 0) { a.y = 0; b.y = 0; }
                    b.y = -b.y;
                    C sm = cadd(a, b), d = csub(a, b), w = __ldg((const C *)P.tw_half + k);
                    C cd = mk<C>(w.x * d.x + w.y * d.y, w.x * d.y - w.y * d.x);
                    y = mk<C>(sm.x - cd.y, sm.y + cd.x);
               } else if (P.pw == GB_PW_CHIRP_IN) {
                    y = (k < P.n) ? cmul(src[(long long)k * P.is], cconj(__ldg((const C *)P.chirp + k))) : mk<C>(0, 0);
               } else if (P.pw == GB_PW_CHIRP_IN_REAL) {
                    y = (k < P.n) ? cscale(cconj(__ldg((const C *)P.chirp + k)), rs[(long long)k * P.is]) : mk<C>(0, 0);
               } else if (P.pw == GB_PW_CHIRP_IN_HERM) {
                    y = mk<C>(0, 0);
                    if (k < P.n) {
                         /* X_k = X_h (k <= n/2) or conj X_{n-k}; the imaginary
                          * parts of X_0 and X_{n/2} are ignored */
                         const int h = (2 * k <= P.n) ? k : P.n - k;
                         C z = src[(long long)h * P.is];
                         if (k == 0 || 2 * k == P.n) z.y = 0;
                         else if (h != k) z.y = -z.y;
                         y = cmul(z, cconj(__ldg((const C *)P.chirp + k)));
                    }
               } else if (P.pw == GB_PW_SPEC_MUL) {
                    y = cmul(src[(long long)k * P.is], __ldg((const C *)P.chirp_spec + k));
               } else {
                    y = cmul(src[(long long)k * P.is], cconj(__ldg((const C *)P.chirp + k)));
                    if (P.pw == GB_PW_CHIRP_OUT_REAL) {
                         rd[(long long)k * P.os] = y.x;
                         continue;
                    }
               }
               dst[(long long)k * P.os] = y;
          }
     }
}

} /* namespace gb */

using namespace gb;

static __thread char gb_errbuf[256];
/* FFTW_GB300_TRACE set: every launch is logged with its grid */
static const int gb_trace = getenv("FFTW_GB300_TRACE") != 0;
static unsigned long long gb_launches = 0;

extern "C" long long gb_launch_count(void) { return (long long)__atomic_load_n(&gb_launches, __ATOMIC_RELAXED); }

extern "C" void gb_count_launch(void) { __atomic_add_fetch(&gb_launches, 1ull, __ATOMIC_RELAXED); }

extern "C" const char *gb_last_cuda_error(void) { return gb_errbuf; }

static int gb_check(cudaError_t e, const char *what)
{
     if (e != cudaSuccess) {
          snprintf(gb_errbuf, sizeof gb_errbuf, "%s: %s", what, cudaGetErrorString(e));
          return -1;
     }
     return 0;
}

extern "C" int gb_device_smem_per_sm(void)
{
     int dev = 0, v = 0;
     if (cudaGetDevice(&dev) != cudaSuccess) return 0;
     if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess) return 0;
     return v;
}

extern "C" int gb_device_max_smem(void)
{
     int dev = 0, v = 0;
     if (cudaGetDevice(&dev) != cudaSuccess) return 0;
     if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
     return v;
}

/* Split arrays <-> dense interleaved buffer: element L of the dense buffer
 * (row-major over the nd dims) is (re[o], im[o]) with o = sum idx_d * s_d. */
struct gb_split_dims {
     int nd;
     long long n[GB_SPLIT_MAXD], s[GB_SPLIT_MAXD];
};

template <typename R, bool PACK>
__global__ void k_split_copy(const gb_split_dims D, long long total, R *re, R *im, void *buf)
{
     typedef typename cplx_of<R>::T C;
     C *b = (C *)buf;
     for (long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x; L < total;
          L += (long long)gridDim.x * blockDim.x) {
          long long rest = L, o = 0;
          for (int d = D.nd - 1; d >= 0; --d) {
               const long long q = rest / D.n[d];
               o += (rest - q * D.n[d]) * D.s[d];
               rest = q;
          }
          if (!im) {
               /* one real array: dense reals in buf */
               if (PACK) ((R *)buf)[L] = re[o];
               else re[o] = ((const R *)buf)[L];
          } else if (PACK) {
               b[L] = mk<C>(re[o], im[o]);
          } else {
               const C v = b[L];
               re[o] = v.x;
               im[o] = v.y;
          }
     }
}

extern "C" int gb_split_copy(int pack, int prec, int nd, const long long *n, const long long *s, long long total,
                             void *re, void *im, void *buf, void *stream)
{
     gb_split_dims D;
     long long blocks = (total + 255) / 256;
     if (nd < 0 || nd > GB_SPLIT_MAXD) return -1;
     if (total <= 0) return 0;
     D.nd = nd;
     for (int d = 0; d < nd; ++d) { D.n[d] = n[d]; D.s[d] = s[d]; }
     if (blocks > 65536) blocks = 65536;
     cudaStream_t st = (cudaStream_t)stream;
     if (prec == 4) {
          if (pack) k_split_copy<float, true><<<(unsigned)blocks, 256, 0, st>>>(D, total, (float *)re, (float *)im, buf);
          else k_split_copy<float, false><<<(unsigned)blocks, 256, 0, st>>>(D, total, (float *)re, (float *)im, buf);
     } else {
          if (pack) k_split_copy<double, true><<<(unsigned)blocks, 256, 0, st>>>(D, total, (double *)re, (double *)im, buf);
          else k_split_copy<double, false><<<(unsigned)blocks, 256, 0, st>>>(D, total, (double *)re, (double *)im, buf);
     }
     __atomic_add_fetch(&gb_launches, 1ull, __ATOMIC_RELAXED);
     return gb_check(cudaGetLastError(), pack ? "split pack" : "split unpack");
}

extern "C" int gb_twiddles(void *dst, int prec, long long n, long long count, long long mul, void *stream)
{
     int blocks = (int)((count + 255) / 256);
     if (blocks > 4096) blocks = 4096;
     if (blocks < 1) blocks = 1;
     if (prec == 4) k_twiddles<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, n, count, mul);
     else k_twiddles<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, n, count, mul);
     return gb_check(cudaGetLastError(), "twiddle generation");
}

extern "C" int gb_stage_twiddles(void *dst, int prec, int nfft, void *stream)
{
     const int len = stage_tw_len(nfft, stage_tw_rows(2 * prec));
     int blocks = (len + 255) / 256;
     if (len != gb_stage_tw_len(nfft, prec)) {
          snprintf(gb_errbuf, sizeof gb_errbuf, "stage twiddle layouts of host and device disagree");
          return -1;
     }
     if (len == 0) return 0;
     if (prec == 4) k_stage_twiddles<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, nfft, len);
     else k_stage_twiddles<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, nfft, len);
     return gb_check(cudaGetLastError(), "stage twiddle generation");
}

extern "C" int gb_gen_stage_twiddles(void *dst, int prec, int nfft, const int *rad, int nrad, void *stream)
{
     gen_radices R;
     long long prod = 1;
     int i;
     if (nrad < 0 || nrad > GB_MAXRAD) return -1;
     R.n = nrad;
     for (i = 0; i < nrad; ++i) {
          R.r[i] = rad[i];
          prod *= rad[i];
     }
     if (prod != nfft || nfft < 2) {
          snprintf(gb_errbuf, sizeof gb_errbuf, "runtime-radix stage twiddles: radices do not multiply to %d", nfft);
          return -1;
     }
     const int blocks = (nfft - 1 + 255) / 256;
     if (prec == 4) k_gen_stage_twiddles<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, nfft, R);
     else k_gen_stage_twiddles<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, nfft, R);
     return gb_check(cudaGetLastError(), "runtime-radix stage twiddle generation");
}

extern "C" int gb_post_rows(void *dst, int prec, long long N, int T, long long rows, void *stream)
{
     const long long count = rows * T;
     long long blocks = (count + 255) / 256;
     if (blocks > 4096) blocks = 4096;
     if (count <= 0) return 0;
     if (prec == 4) k_post_rows<float2><<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, N, T, count);
     else k_post_rows<double2><<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, N, T, count);
     return gb_check(cudaGetLastError(), "four-step twiddle rows");
}

extern "C" int gb_chirp(void *dst, int prec, long long n, int sign, void *stream)
{
     int blocks = (int)((n + 255) / 256);
     if (blocks > 4096) blocks = 4096;
     if (prec == 4) k_chirp<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, n, sign);
     else k_chirp<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, n, sign);
     return gb_check(cudaGetLastError(), "chirp generation");
}

extern "C" int gb_chirp_pad(void *dst, const void *w, int prec, long long n, long long nb, void *stream)
{
     int blocks = (int)((nb + 255) / 256);
     if (blocks > 4096) blocks = 4096;
     if (prec == 4) k_chirp_pad<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, (const float2 *)w, n, nb);
     else k_chirp_pad<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, (const double2 *)w, n, nb);
     return gb_check(cudaGetLastError(), "chirp padding");
}

extern "C" int gb_rader_omega(void *dst, const int *gpow, int prec, long long p, int sign, void *stream)
{
     int blocks = (int)((p + 255) / 256);
     if (blocks > 4096) blocks = 4096;
     if (prec == 4) k_rader_omega<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)dst, gpow, p, sign);
     else k_rader_omega<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>((double2 *)dst, gpow, p, sign);
     return gb_check(cudaGetLastError(), "Rader omega");
}

static const void *pick_kernel(const gb_pass *p)
{
     if (p->kind == GB_KIND_POINTWISE)
          return p->prec == 4 ? (const void *)k_pointwise<float2> : (const void *)k_pointwise<double2>;
     if (p->kind == GB_KIND_COPY)
          return p->prec == 4 ? (const void *)k_copy<float2> : (const void *)k_copy<double2>;
     if (p->variant == GB_VAR_TC)
          return (p->kind == GB_KIND_C2C && p->prec == 4) ? gb_tc_kernel(p->nfft, p->sign, p->groups) : 0;
     if (p->variant == GB_VAR_TMA_COLS) {
          int logn = 0;
          while ((1 << logn) < p->nfft) ++logn;
          return (p->kind == GB_KIND_C2C && p->prec == 4) ? gb_cols_tma_kernel(logn, p->sign, p->groups) : 0;
     }
     if (p->variant == GB_VAR_REG || p->variant == GB_VAR_TMA) {
          int logn = 0;
          while ((1 << logn) < p->nfft) ++logn;
          if (p->variant == GB_VAR_TMA)
               return (p->kind == GB_KIND_C2C || p->kind == GB_KIND_R2C || p->kind == GB_KIND_DCT2)
                           ? (p->prec == 4 ? gb_tma_kernel_f(logn, p->kind, p->sign, p->groups)
                                           : gb_tma_kernel_d(logn, p->kind, p->sign, p->groups))
                           : 0;
          return p->prec == 4 ? gb_reg_kernel_f(logn, p->kind, p->sign) : gb_reg_kernel_d(logn, p->kind, p->sign);
     }
     return p->prec == 4 ? (const void *)k_gen<float2> : (const void *)k_gen<double2>;
}

/* Threads of one CTA: a k_reg_tma or k_cols_tma CTA runs p->groups groups
 * of p->threads threads. */
static int cta_threads(const gb_pass *p)
{
     return (p->variant == GB_VAR_TMA || p->variant == GB_VAR_TMA_COLS) ? p->groups * p->threads : p->threads;
}

/* Number of CTAs launched for a pass: all tiles, capped; kernels stride over
 * the rest.  Persistent (TMA-fed) passes launch exactly as many CTAs as fit
 * on the device at once. */
static unsigned grid_of(const gb_pass *p, const void *fn)
{
     long long g = p->nblocks;
     if (p->variant == GB_VAR_TMA || p->variant == GB_VAR_TC || p->variant == GB_VAR_TMA_COLS) {
          int dev = 0, sms = 0, per = 0;
          cudaGetDevice(&dev);
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
          const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, cta_threads(p), (size_t)p->smem);
          if (gb_trace)
               fprintf(stderr, "[fftw_gb300] occupancy of variant %d: %d CTAs/SM (%s)\n", p->variant, per, cudaGetErrorString(e));
          if (e != cudaSuccess) {
               cudaGetLastError();
               per = 1;
          }
          /* the calculator may report fewer CTAs per SM for the tensor-core
           * kernel than its registers, shared memory and TMEM (64 columns)
           * leave room for (its build's 2 or 3); its CTAs never wait on one
           * another, so a second wave is harmless if they cannot all be
           * resident */
          if (p->variant == GB_VAR_TC && per < p->groups) per = p->groups;
          if (per < 1) per = 1;
          if (g > (long long)per * sms) g = (long long)per * sms;
     }
     if (g > (1LL << 30)) g = 1LL << 30;
     if (g < 1) g = 1;
     return (unsigned)g;
}

/* One word per device where that device's kernels report a bounded wait
 * that gave up (a kernel may only write its own device's word: another
 * device's memory is not reachable without peer access). */
#define GB_MAX_DEVICES 64
static int *gb_status_word[GB_MAX_DEVICES];
static pthread_mutex_t gb_status_mtx = PTHREAD_MUTEX_INITIALIZER;

static int current_device(void)
{
     int dev = -1;
     if (cudaGetDevice(&dev) != cudaSuccess) {
          cudaGetLastError();
          return -1;
     }
     return (dev >= 0 && dev < GB_MAX_DEVICES) ? dev : -1;
}

/* The current device's status word, allocated (and cleared) on first use. */
extern "C" int *gb_device_status_ptr(void)
{
     const int dev = current_device();
     int *w;
     if (dev < 0) return 0;
     w = __atomic_load_n(&gb_status_word[dev], __ATOMIC_ACQUIRE);
     if (w) return w;
     pthread_mutex_lock(&gb_status_mtx);
     w = gb_status_word[dev];
     if (!w) {
          if (cudaMalloc((void **)&w, sizeof(int)) != cudaSuccess || cudaMemset(w, 0, sizeof(int)) != cudaSuccess) {
               cudaGetLastError();
               w = 0;
          } else {
               __atomic_store_n(&gb_status_word[dev], w, __ATOMIC_RELEASE);
          }
     }
     pthread_mutex_unlock(&gb_status_mtx);
     return w;
}

/* Read and clear the current device's status word (0 = no kernel on this
 * device reported a problem since the last read). */
extern "C" int gb_device_status(void)
{
     const int dev = current_device();
     int v = 0, z = 0;
     int *w = dev >= 0 ? __atomic_load_n(&gb_status_word[dev], __ATOMIC_ACQUIRE) : 0;
     if (!w) return 0;
     if (cudaMemcpy(&v, w, sizeof v, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
     cudaMemcpy(w, &z, sizeof z, cudaMemcpyHostToDevice);
     return v;
}

/* ---- tensor maps for column tiles (k_cols_tma) ---- */

static PFN_cuTensorMapEncodeTiled_v12000 gb_encode_tiled = 0;

/* Plan-time and launch-time conditions of a tensor-map column pass: the
 * tensor map views the input as [outer dims][N rows at stride is][columns]
 * with 8-byte elements, so every stride must be a positive multiple of 16
 * bytes and the base 16-byte aligned; boxes are at most 16 columns x 256
 * rows. */
static int cols_tma_ok(const gb_pass *p, const void *in)
{
     int d;
     const int T = p->nfft / reg_e(p->nfft);
     if (p->kind != GB_KIND_C2C || p->prec != 4 || p->load_mode != GB_MOVE_COLS) return 0;
     if (p->nfft < 16 || p->nfft > 2048 || p->tb < 2 || p->tb > 128 || (p->tb & (p->tb - 1)) || p->ltb < 0) return 0;
     if (p->threads != p->tb * T || p->threads > 256 || p->nv > 4) return 0;
     if (p->groups < 1 || p->groups > 2 || (p->groups == 2 && p->threads % 32) ||
         p->smem < gb_cols_tma_smem(p->nfft, p->tb, p->groups))
          return 0;
     if ((uintptr_t)in % 16 || p->vis[0] != 1 || p->is <= 0 || (p->is * 8) % 16 || p->is * 8 >= (1LL << 40)) return 0;
     if (p->vn[0] >= (1LL << 31)) return 0;
     for (d = 1; d < p->nv; ++d)
          if (p->vis[d] <= 0 || (p->vis[d] * 8) % 16 || p->vis[d] * 8 >= (1LL << 40) || p->vn[d] >= (1LL << 31)) return 0;
     return 1;
}

extern "C" int gb_cols_tma_plan_ok(const gb_pass *p) { return cols_tma_ok(p, (const void *)0); }

/* The output of a column pass as a tensor map for TMA stores: the same
 * view and boxes as the input's, over (out, os, vos). */
static int cols_out_ok(const gb_pass *p, const void *out)
{
     int d;
     if (p->store_mode != GB_MOVE_COLS || p->vos[0] != 1 || (uintptr_t)out % 16 || p->os <= 0 || (p->os * 8) % 16 ||
         p->os * 8 >= (1LL << 40))
          return 0;
     for (d = 1; d < p->nv; ++d)
          if (p->vos[d] <= 0 || (p->vos[d] * 8) % 16 || p->vos[d] * 8 >= (1LL << 40)) return 0;
     return 1;
}

static int encode_cols_map(CUtensorMap *tm, const gb_pass *p, const void *in, int output);

static int encode_cols_map(CUtensorMap *tm, const gb_pass *p, const void *in, int output)
{
     cuuint64_t gdim[5], gstr[4];
     cuuint32_t box[5] = {1, 1, 1, 1, 1}, es[5] = {1, 1, 1, 1, 1};
     const int cb = p->tb < 16 ? p->tb : 16, rank = 1 + p->nv;
     CUtensorMapSwizzle sw = cb == 16 ? CU_TENSOR_MAP_SWIZZLE_128B : cb == 8 ? CU_TENSOR_MAP_SWIZZLE_64B
                           : cb == 4 ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_NONE;
     int d;
     if (!gb_encode_tiled) {
          void *fp = 0;
          cudaDriverEntryPointQueryResult q;
          if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fp, 12000, cudaEnableDefault, &q) != cudaSuccess ||
              q != cudaDriverEntryPointSuccess || !fp) {
               cudaGetLastError();
               return -1;
          }
          gb_encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fp;
     }
     gdim[0] = (cuuint64_t)p->vn[0];
     gdim[1] = (cuuint64_t)p->nfft;
     gstr[0] = (cuuint64_t)(output ? p->os : p->is) * 8;
     for (d = 1; d < p->nv; ++d) {
          gdim[1 + d] = (cuuint64_t)p->vn[d];
          gstr[d] = (cuuint64_t)(output ? p->vos[d] : p->vis[d]) * 8;
     }
     box[0] = (cuuint32_t)cb;
     box[1] = (cuuint32_t)(p->nfft < 256 ? p->nfft : 256);
     return gb_encode_tiled(tm, CU_TENSOR_MAP_DATA_TYPE_INT64, (cuuint32_t)rank, (void *)in, gdim, gstr, box, es,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS ? 0 : -1;
}

extern "C" int gb_launch_pass(const gb_pass *p, const void *in, void *out, void *stream)
{
     const void *fn = pick_kernel(p);
     if (!fn) {
          snprintf(gb_errbuf, sizeof gb_errbuf, "no kernel for kind %d variant %d nfft %d prec %d",
                   p->kind, p->variant, p->nfft, p->prec);
          return -1;
     }
     if (p->nblocks <= 0) return 0;
     /* descriptor checks: a pass that would read a missing table or exceed
      * the launch limits is refused on the host instead of run */
     {
          const char *bad = 0;
          if (p->kind == GB_KIND_POINTWISE) {
               if ((p->pw == GB_PW_HC2C_POST || p->pw == GB_PW_HC2C_PRE) && !p->tw_half) bad = "hc2c table missing";
               else if ((p->pw == GB_PW_CHIRP_IN || p->pw == GB_PW_CHIRP_OUT || p->pw == GB_PW_CHIRP_IN_REAL ||
                         p->pw == GB_PW_CHIRP_IN_HERM || p->pw == GB_PW_CHIRP_OUT_HALF ||
                         p->pw == GB_PW_CHIRP_OUT_REAL) && !p->chirp)
                    bad = "chirp missing";
               else if (p->pw == GB_PW_SPEC_MUL && !p->chirp_spec) bad = "chirp spectrum missing";
               else if (p->pw_chunks < 1 || p->threads != 256 || p->tb != 1) bad = "bad pointwise launch shape";
          } else if (p->kind != GB_KIND_COPY && (p->variant == GB_VAR_GEN || p->variant == GB_VAR_TC) && !p->tw)
               bad = "twiddle table missing";
          else if ((p->variant == GB_VAR_REG || p->variant == GB_VAR_TMA || p->variant == GB_VAR_TMA_COLS ||
                    p->variant == GB_VAR_TC) && p->kind != GB_KIND_COPY && stage_tw_len(p->nfft) > 0 && !p->tw_stage)
               bad = "stage twiddle table missing";
          else if ((p->kind == GB_KIND_R2C || p->kind == GB_KIND_C2R || p->kind == GB_KIND_DCT2) && p->n % 2 == 0 &&
                   !p->tw_half)
               bad = "half-length twiddle table missing";
          else if (p->kind == GB_KIND_DCT2 && (p->variant != GB_VAR_TMA || !p->chirp || p->n != 2 * p->nfft))
               bad = "fused DCT-II pass needs the bulk-copy kernel and its cosine table";
          else if (p->kind == GB_KIND_BLUESTEIN && (!p->chirp || !p->chirp_spec)) bad = "chirp tables missing";
          else if (p->kind == GB_KIND_RADER && (p->variant != GB_VAR_GEN || !p->perm || !p->chirp_spec || p->nfft != p->n - 1))
               bad = "Rader pass needs its permutation and omega tables";
          else if (p->post_N && (!p->post_lo || !p->post_hi || p->post_S <= 0)) bad = "four-step twiddle tables missing";
          else if (p->post_vdim < 0 || p->post_vdim >= p->nv || (p->post_vdim && !p->post_N))
               bad = "four-step twiddle dimension is not a vector dimension of the pass";
          else if (p->threads < 1 || p->threads > 1024 || p->tb < 1 || p->nv < 1 || p->nv > GB_MAXV) bad = "bad launch shape";
          else if ((p->variant == GB_VAR_REG || p->variant == GB_VAR_TMA || p->variant == GB_VAR_TMA_COLS) &&
                   p->kind != GB_KIND_COPY &&
                   p->threads != p->tb * (p->nfft / reg_e(p->nfft))) bad = "thread count does not match the tile";
          else if (p->variant == GB_VAR_REG && p->threads > reg_maxthreads(p->nfft)) bad = "tile exceeds the kernel's launch bounds";
          else if (reg_sms(p->nfft) != gb_reg_sms(p->nfft)) bad = "host and device shared-memory layouts disagree";
          else if (p->ltb >= 0 && (p->ltb > 10 || (1 << p->ltb) != p->tb)) bad = "tile shift does not match the tile";
          else if (p->post_N && (p->post_lS < 0 || (1LL << p->post_lS) != p->post_S || p->post_S * p->post_S < p->post_N))
               bad = "four-step twiddle table split is inconsistent";
          else if (p->variant == GB_VAR_REG && p->smem < p->tb * reg_sms(p->nfft) * 2 * p->prec) bad = "shared memory too small for the tile";
          else if (p->variant == GB_VAR_TMA && (p->threads > tma_threads(p->nfft) || (p->groups > 1 && p->threads % 32) ||
                                                p->is != 1 || p->os != 1 ||
                                                (p->kind != GB_KIND_C2C && p->kind != GB_KIND_R2C && p->kind != GB_KIND_DCT2) ||
                                                ((p->kind == GB_KIND_R2C || p->kind == GB_KIND_DCT2) && p->n != 2 * p->nfft) ||
                                                p->groups < 1 || p->groups > gb_tma_max_groups(p->prec) ||
                                                p->groups * p->threads > 1024 ||
                                                p->smem < (p->groups + 1) * p->tb * tma_sms(p->nfft) * 2 * p->prec))
               bad = "persistent bulk-copy pass needs unit-stride c2c/r2c in and out and one smem buffer per group and one more";
          else if (p->variant == GB_VAR_TMA && ((uintptr_t)in % 16 != 0)) bad = "bulk copies need a 16-byte aligned input";
          else if (p->variant == GB_VAR_TMA_COLS && !cols_tma_ok(p, in))
               bad = "tensor-map column pass needs f32 c2c column tiles of 2..128 columns, 16..2048 points, even positive "
                     "strides, a 16-byte aligned input and two shared slots";
          else if (p->variant == GB_VAR_TC && (p->prec != 4 || p->nfft < 256 || p->nfft > 4096 || (p->nfft & (p->nfft - 1)) ||
                                               p->threads != 256 || p->tb != 256 / (p->nfft / 16) ||
                                               (p->groups != 2 && p->groups != 3) ||
                                               p->smem < gb_tc_smem(p->nfft, p->groups) || (p->store_mode == GB_MOVE_DIRECT && p->os != 1)))
               bad = "tensor-core pass needs f32 c2c of 256 to 4096 points (a power of two), 256 threads, a 2- or 3-CTA build";
          if (bad) {
               snprintf(gb_errbuf, sizeof gb_errbuf, "refused pass (kind %d nfft %d): %s", p->kind, p->nfft, bad);
               return -1;
          }
     }
     if (p->smem > 48 * 1024) {
          if (gb_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, p->smem),
                       "cudaFuncSetAttribute(max dynamic smem)"))
               return -1;
          /* largest shared-memory carveout, so the occupancy the grid is sized
           * for (persistent kernels) is the one the SMs are configured for */
          if (gb_check(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                            cudaSharedmemCarveoutMaxShared),
                       "cudaFuncSetAttribute(shared memory carveout)"))
               return -1;
     }
     gb_pass pv = *p;
     if (!pv.status) pv.status = gb_device_status_ptr();
     CUtensorMap tmap, omap;
     int tstore = 0;
     void *args[6] = {(void *)&pv, (void *)&in, (void *)&out, (void *)&tmap, (void *)&omap, (void *)&tstore};
     memset(&omap, 0, sizeof omap);
     if (p->variant == GB_VAR_TMA_COLS && cols_out_ok(p, out) && !getenv("FFTW_GB300_NO_TMA_STORE"))
          tstore = encode_cols_map(&omap, p, out, 1) == 0;
     if (p->variant == GB_VAR_TMA_COLS && encode_cols_map(&tmap, p, in, 0)) {
          /* the driver refused this view of the array: same tile through
           * the register kernel's plain loads */
          pv.variant = GB_VAR_REG;
          pv.smem = p->tb * reg_sms(p->nfft) * 2 * p->prec;
          fn = pick_kernel(&pv);
          if (!fn) return -1;
          if (pv.smem > 48 * 1024 &&
              gb_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pv.smem),
                       "cudaFuncSetAttribute(max dynamic smem)"))
               return -1;
          p = &pv;
     } else if (p->variant == GB_VAR_TMA_COLS && p->groups == 2 && p->store_mode != GB_MOVE_DIRECT && !tstore) {
          /* plain column stores (no output tensor map) go through the slot
           * with the CTA-wide tile walk: one group per CTA */
          pv.groups = 1;
          fn = pick_kernel(&pv);
          if (!fn) return -1;
          if (pv.smem > 48 * 1024 &&
              (gb_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pv.smem),
                        "cudaFuncSetAttribute(max dynamic smem)") ||
               gb_check(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared),
                        "cudaFuncSetAttribute(shared memory carveout)")))
               return -1;
          p = &pv;
     }
     const unsigned grid = grid_of(p, fn);
     if (gb_trace)
          fprintf(stderr, "[fftw_gb300] launch kind %d variant %d nfft %d tb %d: grid %u x %d threads, %d B smem\n",
                  p->kind, p->variant, p->nfft, p->tb, grid, cta_threads(p), p->smem);
     cudaError_t e = cudaLaunchKernel(fn, dim3(grid), dim3(cta_threads(p)), args, (size_t)pv.smem, (cudaStream_t)stream);
     __atomic_add_fetch(&gb_launches, 1ull, __ATOMIC_RELAXED);
     return gb_check(e, "kernel launch");
}

/* Resource usage of the kernel a pass would launch (registers per thread,
 * static smem, max threads), for the planner's occupancy choices. */
extern "C" int gb_pass_kernel_attrs(const gb_pass *p, int *regs, int *max_threads)
{
     const void *fn = pick_kernel(p);
     cudaFuncAttributes a;
     if (!fn) return -1;
     if (gb_check(cudaFuncGetAttributes(&a, fn), "cudaFuncGetAttributes")) return -1;
     *regs = a.numRegs;
     *max_threads = a.maxThreadsPerBlock;
     return 0;
}
