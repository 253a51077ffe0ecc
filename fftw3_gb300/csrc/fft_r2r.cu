/*
 * Pre- and post-processing kernels of the r2r transforms.  Each kind of
 * length n runs as one core transform of length L (gb_r2r_core) on dense
 * buffers between these two kernels; gb_r2r.c holds the algorithms with the
 * reference definitions.  Each thread handles one element of one transform
 * of the batch; the batch is a vector loop of up to GB_R2R_MAXV dims with
 * strides in reals.  The twiddles come from a per-stage table built once at
 * plan time (k_r2r_table: the FP64 octant-reduced cexp rounded once), so the
 * pre and post kernels do no FP64 work:
 *   REDFT01/10, RODFT01/10:   w[q] = exp(-i pi q / 2n), q < n
 *   REDFT11/RODFT11, even n:  w[m] = exp(-i pi (4m+1) / 4n), m < n/2;
 *                             w[n/2 + p] = exp(-i pi p / n), p < n/2
 *   REDFT11/RODFT11, odd n:   w[m] = exp(-i pi m / 2n), m < n;
 *                             w[n + k] = exp(-i pi (2k+1) / 4n), k < n
 *
 * Core buffers per transform (row t of the batch):
 *   r2c core: pre writes L reals, post reads L/2+1 complex
 *   c2r core: pre writes L/2+1 complex, post reads L reals
 *   c2c core: pre writes L complex, post reads L complex
 */
#include <cuda_runtime.h>
#include "fft_kernels.cuh"

namespace gb {

enum {
     R2R_R2HC = 0, R2R_HC2R = 1, R2R_DHT = 2, R2R_REDFT00 = 3, R2R_REDFT01 = 4, R2R_REDFT10 = 5, R2R_REDFT11 = 6,
     R2R_RODFT00 = 7, R2R_RODFT01 = 8, R2R_RODFT10 = 9, R2R_RODFT11 = 10
};

/* exp(dir * 2 pi i m / M), rounded once from FP64 */
template <typename C>
__device__ __forceinline__ C r2r_twiddle(long long m, long long M, int dir)
{
     typedef typename real_of<C>::T R;
     double c, s;
     cexp_fp64(m, M, dir, &c, &s);
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

/* twiddle table entry i of a stage (layout in the file comment) */
template <typename C>
__device__ __forceinline__ C r2r_table_entry(int kind, long long n, long long i)
{
     if (kind == R2R_REDFT11 || kind == R2R_RODFT11) {
          if (!(n & 1)) return i < n / 2 ? r2r_twiddle<C>(4 * i + 1, 8 * n, -1) : r2r_twiddle<C>(i - n / 2, 2 * n, -1);
          return i < n ? r2r_twiddle<C>(i, 4 * n, -1) : r2r_twiddle<C>(2 * (i - n) + 1, 8 * n, -1);
     }
     return r2r_twiddle<C>(i, 4 * n, -1);
}

template <typename C>
__global__ void k_r2r_table(int kind, long long n, long long len, C *tab)
{
     for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len;
          i += (long long)gridDim.x * blockDim.x)
          tab[i] = r2r_table_entry<C>(kind, n, i);
}

/* element offset (reals) of vector index t on the input (out = 0) or output side */
__device__ __forceinline__ long long vec_offset(const gb_r2r_vec &v, long long t, int out)
{
     if (v.nv == 1) return t * (out ? v.os[0] : v.is[0]);
     long long off = 0;
     for (int d = v.nv - 1; d >= 0; --d) {
          const long long i = t % v.n[d];
          t /= v.n[d];
          off += i * (out ? v.os[d] : v.is[d]);
     }
     return off;
}

/* row and column of element g of a batch of rows of length per (32-bit
 * division when the batch fits) */
__device__ __forceinline__ void r2r_split(long long g, long long per, bool small, long long *t, long long *m)
{
     if (small) {
          const unsigned q = (unsigned)g / (unsigned)per;
          *t = q;
          *m = (long long)((unsigned)g - q * (unsigned)per);
     } else {
          *t = g / per;
          *m = g - *t * per;
     }
}

template <typename R>
__global__ void k_r2r_pre(int kind, long long n, long long L, long long V, const R *__restrict__ in, long long is,
                          const gb_r2r_vec vec, void *__restrict__ buf, const void *__restrict__ twv)
{
     typedef typename cplx_of<R>::T C;
     const C *tw = (const C *)twv;
     long long Lc;
     const int core = gb_r2r_core(kind, n, &Lc);
     const long long per = core == GB_R2R_CORE_C2R ? L / 2 + 1 : L;
     const bool small = per * V < (1LL << 32);
     for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < per * V;
          g += (long long)gridDim.x * blockDim.x) {
          long long t, m;
          r2r_split(g, per, small, &t, &m);
          const R *x = in + vec_offset(vec, t, 0);
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
          case R2R_REDFT00:
               /* even extension of length 2(n-1): e_m = x_m, e_{L-m} = x_m */
               ((R *)buf)[g] = x[(m < n ? m : L - m) * is];
               break;
          case R2R_RODFT00: {
               /* odd extension of length 2(n+1): o_0 = o_{n+1} = 0,
                * o_{m} = x_{m-1}, o_{L-1-j} = -x_j */
               R v = (R)0;
               if (m >= 1 && m <= n) v = x[(m - 1) * is];
               else if (m > n + 1) v = -x[(L - 1 - m) * is];
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
          case R2R_REDFT01:
          case R2R_RODFT01: {
               /* REDFT01: V_k = (x_k - i x_{n-k}) exp(i pi k / 2n), x_n = 0;
                * RODFT01 on x reversed */
               const bool rev = (kind == R2R_RODFT01);
               const R a = x[(rev ? n - 1 - m : m) * is];
               const R b = (m == 0) ? (R)0 : x[(rev ? m - 1 : n - m) * is];
               const C w0 = __ldg(tw + m), w = mk<C>(w0.x, -w0.y);   /* exp(i pi m / 2n) */
               /* (a - i b) * w */
               ((C *)buf)[g] = mk<C>(a * w.x + b * w.y, a * w.y - b * w.x);
               break;
          }
          default: {
               /* REDFT11 (RODFT11 on x reversed).  Even n: z_m = (x_{2m} +
                * i x_{n-1-2m}) exp(-i pi (4m+1) / 4n), m < n/2.  Odd n: z_m =
                * x_m exp(-i pi m / 2n) for m < n, zero up to 2n. */
               const bool rev = (kind == R2R_RODFT11);
               C z;
               if (!(n & 1)) {
                    const long long ja = 2 * m, jb = n - 1 - 2 * m;
                    const R a = x[(rev ? jb : ja) * is], b = x[(rev ? ja : jb) * is];
                    const C w = __ldg(tw + m);
                    z = mk<C>(a * w.x - b * w.y, a * w.y + b * w.x);
               } else if (m < n) {
                    const R a = x[(rev ? n - 1 - m : m) * is];
                    const C w = __ldg(tw + m);
                    z = mk<C>(a * w.x, a * w.y);
               } else {
                    z = mk<C>((R)0, (R)0);
               }
               ((C *)buf)[g] = z;
               break;
          }
          }
     }
}

template <typename R>
__global__ void k_r2r_post(int kind, long long n, long long L, long long V, const void *__restrict__ buf,
                           R *__restrict__ out, long long os, const gb_r2r_vec vec, const void *__restrict__ twv)
{
     typedef typename cplx_of<R>::T C;
     const C *tw = (const C *)twv;
     long long Lc;
     const int core = gb_r2r_core(kind, n, &Lc);
     const long long rowc = core == GB_R2R_CORE_R2C ? L / 2 + 1 : L;   /* complex row length */
     const bool small = n * V < (1LL << 32);
     for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n * V;
          g += (long long)gridDim.x * blockDim.x) {
          long long t, k;
          r2r_split(g, n, small, &t, &k);
          R *y = out + vec_offset(vec, t, 1);
          const C *Z = (const C *)buf + t * rowc;
          const R *v = (const R *)buf + t * L;
          R r;
          switch (kind) {
          case R2R_R2HC:
               r = (2 * k <= n) ? Z[k].x : Z[n - k].y;
               break;
          case R2R_DHT: {
               const C z = half_spec(Z, n, k);
               r = z.x - z.y;
               break;
          }
          case R2R_REDFT10:
          case R2R_RODFT10: {
               /* DCT-II_q = 2 Re(exp(-i pi q / 2n) V_q); DST-II_k = DCT-II_{n-1-k}
                * of the sign-alternated input */
               const long long q = (kind == R2R_RODFT10) ? n - 1 - k : k;
               const C z = half_spec(Z, n, q), w = __ldg(tw + q);
               r = 2 * (w.x * z.x - w.y * z.y);
               break;
          }
          case R2R_REDFT00:
               /* the DFT of the even extension is real: y_k = Re E_k */
               r = Z[k].x;
               break;
          case R2R_RODFT00:
               /* the DFT of the odd extension is imaginary: y_k = -Im O_{k+1} */
               r = -Z[k + 1].y;
               break;
          case R2R_HC2R:
               r = v[k];
               break;
          case R2R_REDFT01:
          case R2R_RODFT01: {
               /* REDFT01: y_{2m} = v_m, y_{2m+1} = v_{n-1-m}; RODFT01 also
                * multiplies y_k by (-1)^k */
               const long long src = (k & 1) ? n - 1 - (k >> 1) : (k >> 1);
               r = v[src];
               if (kind == R2R_RODFT01 && (k & 1)) r = -r;
               break;
          }
          default: {
               /* REDFT11.  Even n: u_p = Z_p exp(-i pi p / n), y_{2p} = 2 Re u_p,
                * y_{n-1-2p} = -2 Im u_p.  Odd n: y_k = 2 Re(Z_k exp(-i pi (2k+1) / 4n)).
                * RODFT11_k = (-1)^k REDFT11_k of x reversed. */
               if (!(n & 1)) {
                    const long long p = (k & 1) ? (n - 1 - k) >> 1 : k >> 1;
                    const C z = Z[p], w = __ldg(tw + n / 2 + p);
                    r = (k & 1) ? -2 * (z.x * w.y + z.y * w.x) : 2 * (z.x * w.x - z.y * w.y);
               } else {
                    const C z = Z[k], w = __ldg(tw + n + k);
                    r = 2 * (z.x * w.x - z.y * w.y);
               }
               if (kind == R2R_RODFT11 && (k & 1)) r = -r;
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

/* twiddle-table length of a stage (0: the kind uses none) */
extern "C" long long gb_r2r_table_len(int kind, long long n)
{
     switch (kind) {
     case R2R_REDFT01: case R2R_REDFT10: case R2R_RODFT01: case R2R_RODFT10: return n;
     case R2R_REDFT11: case R2R_RODFT11: return (n & 1) ? 2 * n : n;
     default: return 0;
     }
}

extern "C" int gb_r2r_table(int prec, int kind, long long n, void *tab, void *stream)
{
     cudaStream_t st = (cudaStream_t)stream;
     const long long len = gb_r2r_table_len(kind, n);
     if (len <= 0) return 0;
     if (prec == 4) k_r2r_table<float2><<<r2r_blocks(len), 256, 0, st>>>(kind, n, len, (float2 *)tab);
     else k_r2r_table<double2><<<r2r_blocks(len), 256, 0, st>>>(kind, n, len, (double2 *)tab);
     return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" int gb_r2r_pre(int prec, int kind, long long n, long long V, const void *in, long long is,
                          const gb_r2r_vec *vec, void *buf, const void *tw, void *stream)
{
     cudaStream_t st = (cudaStream_t)stream;
     long long L;
     const int core = gb_r2r_core(kind, n, &L);
     const long long per = core == GB_R2R_CORE_C2R ? L / 2 + 1 : L;
     if (vec->nv < 0 || vec->nv > GB_R2R_MAXV) return -1;
     if (prec == 4)
          k_r2r_pre<float><<<r2r_blocks(per * V), 256, 0, st>>>(kind, n, L, V, (const float *)in, is, *vec, buf, tw);
     else
          k_r2r_pre<double><<<r2r_blocks(per * V), 256, 0, st>>>(kind, n, L, V, (const double *)in, is, *vec, buf,
                                                                  tw);
     gb_count_launch();
     return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" int gb_r2r_post(int prec, int kind, long long n, long long V, const void *buf, void *out, long long os,
                           const gb_r2r_vec *vec, const void *tw, void *stream)
{
     cudaStream_t st = (cudaStream_t)stream;
     long long L;
     gb_r2r_core(kind, n, &L);
     if (vec->nv < 0 || vec->nv > GB_R2R_MAXV) return -1;
     if (prec == 4)
          k_r2r_post<float><<<r2r_blocks(n * V), 256, 0, st>>>(kind, n, L, V, buf, (float *)out, os, *vec, tw);
     else
          k_r2r_post<double><<<r2r_blocks(n * V), 256, 0, st>>>(kind, n, L, V, buf, (double *)out, os, *vec, tw);
     gb_count_launch();
     return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
