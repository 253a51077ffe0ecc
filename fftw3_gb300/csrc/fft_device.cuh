/*
 * Device building blocks of the GB300 FFT kernels: complex arithmetic,
 * register butterflies of radix 2, 3, 4, 5, 7, 8, 11, 13 and 16, twiddle
 * access, and the Stockham stage of one radix.
 *
 * The butterflies replace the reference's generated n1_* codelets
 * (dft/scalar/codelets/Makefile.am:18-53, not present in the checkout) and
 * the stage replaces one level of dft/ct.c's Cooley-Tukey recursion with its
 * t1_* twiddle codelets (dft/ct.c:34-58, dft/dftw-direct.c:46-56): instead of
 * one HBM pass per level, every level runs on data resident in registers and
 * shared memory.  Stockham autosort order is used, so no bit-reversal pass
 * exists: stage s with radix R and running product Ns of earlier radices maps
 * butterfly j (0 <= j < N/R) from inputs j + r*N/R to outputs
 * (j/Ns)*Ns*R + j%Ns + q*Ns, applying W_{Ns*R}^{r*(j%Ns)} before the DFT_R.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb {

template <typename R> struct cplx_of;
template <> struct cplx_of<float> { typedef float2 T; };
template <> struct cplx_of<double> { typedef double2 T; };
template <typename C> struct real_of;
template <> struct real_of<float2> { typedef float T; };
template <> struct real_of<double2> { typedef double T; };

template <typename C> __device__ __forceinline__ C mk(typename real_of<C>::T a, typename real_of<C>::T b) { C r; r.x = a; r.y = b; return r; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) { return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C> __device__ __forceinline__ C cconj(C a) { return mk<C>(a.x, -a.y); }
template <typename C> __device__ __forceinline__ C cscale(C a, typename real_of<C>::T s) { return mk<C>(a.x * s, a.y * s); }
/* multiply by DIR * i */
template <int DIR, typename C> __device__ __forceinline__ C rot(C a) { return DIR < 0 ? mk<C>(a.y, -a.x) : mk<C>(-a.y, a.x); }
/* multiply by the constant exp(DIR * i * theta) given (cos theta, sin theta) */
template <int DIR, typename C> __device__ __forceinline__ C cmulk(C a, double c, double s)
{
     typedef typename real_of<C>::T R;
     const R cr = (R)c, si = (R)(DIR * s);
     return mk<C>(a.x * cr - a.y * si, a.x * si + a.y * cr);
}

/* table holds exp(-2 pi i j / N); DIR = +1 conjugates */
template <int DIR, typename C> __device__ __forceinline__ C twid(const C *__restrict__ tw, int idx)
{
     C w = __ldg(tw + idx);
     if (DIR > 0) w.y = -w.y;
     return w;
}

/* cos / sin of 2 pi m / p for the odd-prime butterflies */
template <int P, int M> struct kpr;
#include "kpr_table.inc"

#define GB_C8 0.9238795325112867561282
#define GB_S8 0.3826834323650897717285
#define GB_R2 0.7071067811865475244008

template <int R, int DIR> struct bfly;

template <int DIR> struct bfly<1, DIR> { template <typename C> __device__ static __forceinline__ void run(C *) {} };

template <int DIR> struct bfly<2, DIR> {
     template <typename C> __device__ static __forceinline__ void run(C *a)
     {
          C t = a[1];
          a[1] = csub(a[0], t);
          a[0] = cadd(a[0], t);
     }
};

template <int DIR> struct bfly<4, DIR> {
     template <typename C> __device__ static __forceinline__ void run(C *a)
     {
          C s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
          C s13 = cadd(a[1], a[3]), d13 = rot<DIR>(csub(a[1], a[3]));
          a[0] = cadd(s02, s13);
          a[2] = csub(s02, s13);
          a[1] = cadd(d02, d13);
          a[3] = csub(d02, d13);
     }
};

/* 8 = 2 x 4, decimation in time */
template <int DIR> struct bfly<8, DIR> {
     template <typename C> __device__ static __forceinline__ void run(C *a)
     {
          typedef typename real_of<C>::T Rr;
          C b0[4] = {a[0], a[2], a[4], a[6]};
          C b1[4] = {a[1], a[3], a[5], a[7]};
          bfly<4, DIR>::run(b0);
          bfly<4, DIR>::run(b1);
          b1[1] = cscale(mk<C>(b1[1].x - DIR * b1[1].y, b1[1].y + DIR * b1[1].x), (Rr)GB_R2);
          b1[2] = rot<DIR>(b1[2]);
          b1[3] = cscale(mk<C>(-b1[3].x - DIR * b1[3].y, -b1[3].y + DIR * b1[3].x), (Rr)GB_R2);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
               a[q] = cadd(b0[q], b1[q]);
               a[q + 4] = csub(b0[q], b1[q]);
          }
     }
};

/* 16 = 4 x 4, decimation in time */
template <int DIR> struct bfly<16, DIR> {
     template <typename C> __device__ static __forceinline__ void run(C *a)
     {
          C b[4][4];
#pragma unroll
          for (int r1 = 0; r1 < 4; ++r1) {
               b[r1][0] = a[r1]; b[r1][1] = a[r1 + 4]; b[r1][2] = a[r1 + 8]; b[r1][3] = a[r1 + 12];
               bfly<4, DIR>::run(b[r1]);
          }
          b[1][1] = cmulk<DIR>(b[1][1], GB_C8, GB_S8);
          b[1][2] = cmulk<DIR>(b[1][2], GB_R2, GB_R2);
          b[1][3] = cmulk<DIR>(b[1][3], GB_S8, GB_C8);
          b[2][1] = cmulk<DIR>(b[2][1], GB_R2, GB_R2);
          b[2][2] = rot<DIR>(b[2][2]);
          b[2][3] = cmulk<DIR>(b[2][3], -GB_R2, GB_R2);
          b[3][1] = cmulk<DIR>(b[3][1], GB_S8, GB_C8);
          b[3][2] = cmulk<DIR>(b[3][2], -GB_R2, GB_R2);
          b[3][3] = cmulk<DIR>(b[3][3], -GB_C8, -GB_S8);
#pragma unroll
          for (int q1 = 0; q1 < 4; ++q1) {
               C c[4] = {b[0][q1], b[1][q1], b[2][q1], b[3][q1]};
               bfly<4, DIR>::run(c);
               a[q1] = c[0]; a[q1 + 4] = c[1]; a[q1 + 8] = c[2]; a[q1 + 12] = c[3];
          }
     }
};

/* odd prime P: pair inputs j and P-j (sum t_j, difference d_j); output k and
 * P-k share the cosine part and differ in the sign of the sine part. */
template <int P, int DIR, int K, int J> struct oddp_acc {
     template <typename C> __device__ static __forceinline__ void run(const C *t, const C *d, C &u, C &v)
     {
          typedef typename real_of<C>::T Rr;
          constexpr int m = (J * K) % P;
          const Rr c = (Rr)kpr<P, m>::c, s = (Rr)kpr<P, m>::s;
          u.x += c * t[J - 1].x; u.y += c * t[J - 1].y;
          v.x += s * d[J - 1].x; v.y += s * d[J - 1].y;
          oddp_acc<P, DIR, K, J - 1>::run(t, d, u, v);
     }
};
template <int P, int DIR, int K> struct oddp_acc<P, DIR, K, 0> {
     template <typename C> __device__ static __forceinline__ void run(const C *, const C *, C &, C &) {}
};
template <int P, int DIR, int K> struct oddp_out {
     template <typename C> __device__ static __forceinline__ void run(const C *a, const C *t, const C *d, C *o)
     {
          C u = a[0], v = mk<C>(0, 0);
          oddp_acc<P, DIR, K, (P - 1) / 2>::run(t, d, u, v);
          C iv = rot<DIR>(v);
          o[K] = cadd(u, iv);
          o[P - K] = csub(u, iv);
          oddp_out<P, DIR, K - 1>::run(a, t, d, o);
     }
};
template <int P, int DIR> struct oddp_out<P, DIR, 0> {
     template <typename C> __device__ static __forceinline__ void run(const C *, const C *, const C *, C *) {}
};
template <int P, int DIR> struct bfly_oddp {
     template <typename C> __device__ static __forceinline__ void run(C *a)
     {
          constexpr int H = (P - 1) / 2;
          C t[H], d[H], o[P];
          C s = a[0];
#pragma unroll
          for (int j = 1; j <= H; ++j) {
               t[j - 1] = cadd(a[j], a[P - j]);
               d[j - 1] = csub(a[j], a[P - j]);
               s = cadd(s, t[j - 1]);
          }
          oddp_out<P, DIR, H>::run(a, t, d, o);
          o[0] = s;
#pragma unroll
          for (int j = 0; j < P; ++j) a[j] = o[j];
     }
};
template <int DIR> struct bfly<3, DIR> { template <typename C> __device__ static __forceinline__ void run(C *a) { bfly_oddp<3, DIR>::run(a); } };
template <int DIR> struct bfly<5, DIR> { template <typename C> __device__ static __forceinline__ void run(C *a) { bfly_oddp<5, DIR>::run(a); } };
template <int DIR> struct bfly<7, DIR> { template <typename C> __device__ static __forceinline__ void run(C *a) { bfly_oddp<7, DIR>::run(a); } };
template <int DIR> struct bfly<11, DIR> { template <typename C> __device__ static __forceinline__ void run(C *a) { bfly_oddp<11, DIR>::run(a); } };
template <int DIR> struct bfly<13, DIR> { template <typename C> __device__ static __forceinline__ void run(C *a) { bfly_oddp<13, DIR>::run(a); } };

/* Exact twiddle exp(sign * 2 pi i m / n) in FP64, argument reduced to the
 * first octant in integer arithmetic before the sine/cosine (the reduction
 * of kernel/trig.c:57-80), then returned for rounding once by the caller. */
__device__ __forceinline__ void cexp_fp64(long long m, long long n, int sign, double *c_out, double *s_out)
{
     unsigned octant = 0;
     long long q = n;               /* quarter of the scaled period */
     long long nn = 4 * n;
     m = m % n;
     if (m < 0) m += n;
     m *= 4;
     if (m > nn - m) { m = nn - m; octant |= 4; }
     if (m - q > 0) { m = m - q; octant |= 2; }
     if (m > q - m) { m = q - m; octant |= 1; }
     double s, c, t;
     sincospi((2.0 * (double)m) / (double)nn, &s, &c);
     if (octant & 1) { t = c; c = s; s = t; }
     if (octant & 2) { t = c; c = -s; s = t; }
     if (octant & 4) { s = -s; }
     *c_out = c;
     *s_out = sign < 0 ? -s : s;
}

/* ---- asynchronous bulk copies (TMA engine) and mbarriers, inline PTX ---- */

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
     asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

/* make the initialised barriers visible to the async proxy */
__device__ __forceinline__ void mbar_fence_init()
{
     asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
     asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

/* global -> shared bulk copy; bytes multiple of 16, both addresses 16-byte aligned */
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src_gmem, unsigned bytes, unsigned long long *bar)
{
     asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                  ::"r"(smem_u32(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

/* order this thread's earlier generic-proxy shared accesses before later async-proxy ones */
__device__ __forceinline__ void fence_proxy_async_smem()
{
     asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
     unsigned long long t;
     asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
     return t;
}

/* Wait until the barrier's phase with the given parity completes.  Bounded:
 * gives up after limit_ns of wall time and returns false. */
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, unsigned long long limit_ns)
{
     unsigned done = 0;
     unsigned long long t0 = 0;
     for (unsigned it = 0;; ++it) {
          asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                       : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
          if (done) return true;
          if (it == 0) t0 = globaltimer_ns();
          else if ((it & 63) == 0 && globaltimer_ns() - t0 > limit_ns) return false;
     }
}

} /* namespace gb */
