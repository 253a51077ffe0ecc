/*
 * Pre- and post-processing kernels of the 1D r2r transforms that run as a
 * real DFT of the same length n (see gb_r2r.c for the algorithms and the
 * reference definitions).  Each thread handles one output element of one
 * transform of the batch; twiddles exp(+-i pi k / 2n) come from the FP64
 * octant-reduced cexp rounded once.
 *
 * Buffers: v (pre output / r2c input) dense real [hm][n]; V (r2c output /
 * c2r input) dense complex [hm][n/2+1].
 */
#include <cuda_runtime.h>
#include "fft_kernels.cuh"

namespace gb {

enum { R2R_R2HC = 0, R2R_HC2R = 1, R2R_DHT = 2, R2R_REDFT01 = 4, R2R_REDFT10 = 5, R2R_RODFT01 = 8, R2R_RODFT10 = 9 };

/* exp(i pi k / 2n) for dir > 0, exp(-i pi k / 2n) for dir < 0 */
template <typename C>
__device__ __forceinline__ C quarter_twiddle(long long k, long long n, int dir)
{
     typedef typename real_of<C>::T R;
     double c, s;
     cexp_fp64(k, 4 * n, dir, &c, &s);
     return mk<C>((R)c, (R)s);
}

/* V_k, 0 <= k < n, from the stored half spectrum (Hermitian symmetry) */
template <typename C>
__device__ __forceinline__ C half_spec(const C *V, long long n, long long k)
{
     if (2 * k <= n) return V[k];
     const C z = V[n - k];
     return mk<C>(z.x, -z.y);
}

template <typename R>
__global__ void k_r2r_pre(int kind, long long n, long long hm, const R *__restrict__ in, long long is, long long idist,
                          void *__restrict__ buf)
{
     typedef typename cplx_of<R>::T C;
     const long long nc = n / 2 + 1;
     const long long per = (kind == R2R_HC2R || kind == R2R_REDFT01 || kind == R2R_RODFT01) ? nc : n;
     for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < per * hm;
          g += (long long)gridDim.x * blockDim.x) {
          const long long t = g / per, m = g - t * per;
          const R *x = in + t * idist;
          switch (kind) {
          case R2R_R2HC:
          case R2R_DHT:
               ((R *)buf)[g] = x[m * is];
               break;
          case R2R_REDFT10:
          case R2R_RODFT10: {
               /* v_m = x_{2m} (m < ceil(n/2)), v_{n-1-m} = x_{2m+1}; DST-II
                * alternates the signs of x */
               const long long j = (2 * m < n) ? 2 * m : 2 * (n - 1 - m) + 1;
               R v = x[j * is];
               if (kind == R2R_RODFT10 && (j & 1)) v = -v;
               ((R *)buf)[g] = v;
               break;
          }
          case R2R_HC2R: {
               /* X_0 = h_0, X_k = h_k + i h_{n-k}, X_{n/2} = h_{n/2} (even n) */
               const R re = x[m * is];
               const R im = (m == 0 || 2 * m == n) ? (R)0 : x[(n - m) * is];
               ((C *)buf)[g] = mk<C>(re, im);
               break;
          }
          default: {
               /* REDFT01: V_k = (x_k - i x_{n-k}) exp(i pi k / 2n), x_n = 0;
                * RODFT01 on x reversed */
               const bool rev = (kind == R2R_RODFT01);
               const R a = x[(rev ? n - 1 - m : m) * is];
               const R b = (m == 0) ? (R)0 : x[(rev ? m - 1 : n - m) * is];
               const C w = quarter_twiddle<C>(m, n, 1);
               /* (a - i b) * w */
               ((C *)buf)[g] = mk<C>(a * w.x + b * w.y, a * w.y - b * w.x);
               break;
          }
          }
     }
}

template <typename R>
__global__ void k_r2r_post(int kind, long long n, long long hm, const void *__restrict__ buf, R *__restrict__ out,
                           long long os, long long odist)
{
     typedef typename cplx_of<R>::T C;
     const long long nc = n / 2 + 1;
     for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n * hm;
          g += (long long)gridDim.x * blockDim.x) {
          const long long t = g / n, k = g - t * n;
          R *y = out + t * odist;
          const C *V = (const C *)buf + t * nc;
          const R *v = (const R *)buf + t * n;
          R r;
          switch (kind) {
          case R2R_R2HC:
               r = (2 * k <= n) ? V[k].x : V[n - k].y;
               break;
          case R2R_DHT: {
               const C z = half_spec(V, n, k);
               r = z.x - z.y;
               break;
          }
          case R2R_REDFT10:
          case R2R_RODFT10: {
               /* DCT-II_q = 2 Re(exp(-i pi q / 2n) V_q); DST-II_k = DCT-II_{n-1-k}
                * of the sign-alternated input */
               const long long q = (kind == R2R_RODFT10) ? n - 1 - k : k;
               const C z = half_spec(V, n, q), w = quarter_twiddle<C>(q, n, -1);
               r = 2 * (w.x * z.x - w.y * z.y);
               break;
          }
          case R2R_HC2R:
               r = v[k];
               break;
          default: {
               /* REDFT01: y_{2m} = v_m, y_{2m+1} = v_{n-1-m}; RODFT01 also
                * multiplies y_k by (-1)^k */
               const long long src = (k & 1) ? n - 1 - (k >> 1) : (k >> 1);
               r = v[src];
               if (kind == R2R_RODFT01 && (k & 1)) r = -r;
               break;
          }
          }
          y[k * os] = r;
     }
}

} /* namespace gb */

using namespace gb;

static unsigned r2r_blocks(long long work)
{
     long long b = (work + 255) / 256;
     if (b > 65536) b = 65536;
     if (b < 1) b = 1;
     return (unsigned)b;
}

extern "C" int gb_r2r_pre(int prec, int kind, long long n, long long hm, const void *in, long long is, long long idist,
                          void *buf, void *stream)
{
     cudaStream_t st = (cudaStream_t)stream;
     const long long per = (kind == R2R_HC2R || kind == R2R_REDFT01 || kind == R2R_RODFT01) ? n / 2 + 1 : n;
     if (prec == 4) k_r2r_pre<float><<<r2r_blocks(per * hm), 256, 0, st>>>(kind, n, hm, (const float *)in, is, idist, buf);
     else k_r2r_pre<double><<<r2r_blocks(per * hm), 256, 0, st>>>(kind, n, hm, (const double *)in, is, idist, buf);
     return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" int gb_r2r_post(int prec, int kind, long long n, long long hm, const void *buf, void *out, long long os,
                           long long odist, void *stream)
{
     cudaStream_t st = (cudaStream_t)stream;
     if (prec == 4) k_r2r_post<float><<<r2r_blocks(n * hm), 256, 0, st>>>(kind, n, hm, buf, (float *)out, os, odist);
     else k_r2r_post<double><<<r2r_blocks(n * hm), 256, 0, st>>>(kind, n, hm, buf, (double *)out, os, odist);
     return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
