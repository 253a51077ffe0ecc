/* CPU restatement of the reference FFTW algorithms on the execute hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the product library
 * never includes, links or calls it.  Tests, the smoke check and bench.py's
 * CPU-baseline leg are its only users.
 *
 * It is compiled three times by fft_oracle.c with ORC_PREC = 1 (float data,
 * double trig), 2 (double data, double trig) and 3 (long double data and
 * trig), mirroring the reference's R / trigreal pairs (kernel/ifftw.h:65-79,
 * kernel/ifftw.h:896-902).
 *
 * Algorithms restated (each function below cites the reference file:line):
 *   - twiddles by octant-reduced sin/cos              kernel/trig.c:57-80
 *   - Cooley-Tukey DIT, n = r*m, child m-point DFTs over r vectors then
 *     radix-r twiddle butterflies over m columns       dft/ct.c:34-58
 *   - radix choice: smallest prime divisor             kernel/primes.c:183-195
 *   - O(n^2) DFT for small primes (Hartley pairing)    dft/generic.c:34-91
 *   - Rader for primes, generator + inverse perm       dft/rader.c:95-165,
 *                                                      kernel/primes.c:105-122
 *   - Bluestein, exact k^2 mod 2n chirp index          dft/bluestein.c:37-128
 *   - r2c = half-length complex DFT + hc2c post-pass   rdft/ct-hc2c.c:197-210
 *   - c2r = hc2c pre-pass + half-length inverse        rdft/ct-hc2c.c:72-83
 *   - multi-d: trailing axis first, then leading axes
 *     in place on the output (c2r: reversed)           dft/rank-geq2.c:42-52,
 *                                                      rdft/rank-geq2-rdft2.c:40-69
 *   - threads split the vector (howmany) loop          threads/dft-vrank-geq1.c
 *
 * Parity of this restatement is pinned against the reference itself
 * (oracle/_ref, compiled from the reference sources) by committed golden
 * vectors under tests/golden/.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#if ORC_PREC == 1
typedef float R;
typedef double T;
#define P(name) orc_f_##name
#define TSIN sin
#define TCOS cos
#define K2PI_T 6.2831853071795864769252867665590057683943388
#elif ORC_PREC == 2
typedef double R;
typedef double T;
#define P(name) orc_d_##name
#define TSIN sin
#define TCOS cos
#define K2PI_T 6.2831853071795864769252867665590057683943388
#else
typedef long double R;
typedef long double T;
#define P(name) orc_l_##name
#define TSIN sinl
#define TCOS cosl
#define K2PI_T 6.2831853071795864769252867665590057683943388L
#endif

typedef long long I;
typedef struct { R re, im; } C;

/* exp(2*pi*i*m/n) with the argument reduced to [0, pi/4] by octant, as
 * kernel/trig.c:57-80 (real_cexp) does; result in trig precision T. */
static void cexp_t(I m, I n, T *c_out, T *s_out)
{
     T theta, c, s, t;
     unsigned octant = 0;
     I quarter_n = n;
     n += n; n += n;
     m += m; m += m;
     m %= n;
     if (m < 0) m += n;
     if (m > n - m) { m = n - m; octant |= 4; }
     if (m - quarter_n > 0) { m = m - quarter_n; octant |= 2; }
     if (m > quarter_n - m) { m = quarter_n - m; octant |= 1; }
     theta = (K2PI_T * (T)m) / (T)n;
     c = TCOS(theta); s = TSIN(theta);
     if (octant & 1) { t = c; c = s; s = t; }
     if (octant & 2) { t = c; c = -s; s = t; }
     if (octant & 4) { s = -s; }
     *c_out = c; *s_out = s;
}

/* Table of exp(sign*2*pi*i*j/n), j = 0..n-1, rounded once to R. */
static C *mktwiddles(I n, int sign)
{
     C *w = (C *)malloc(sizeof(C) * (size_t)(n > 0 ? n : 1));
     I j;
     for (j = 0; j < n; ++j) {
          T c, s;
          cexp_t(j, n, &c, &s);
          w[j].re = (R)c;
          w[j].im = (R)(sign < 0 ? -s : s);
     }
     return w;
}

static I smallest_divisor(I n)  /* kernel/primes.c first_divisor */
{
     I i;
     if (n <= 1) return n;
     if (n % 2 == 0) return 2;
     for (i = 3; i * i <= n; i += 2)
          if (n % i == 0) return i;
     return n;
}

static int is_prime(I n) { return n > 1 && smallest_divisor(n) == n; }

static I mulmod(I a, I b, I p) { return (I)(((__int128)a * b) % p); }

static I powmod(I b, I e, I p)
{
     I r = 1;
     b %= p;
     while (e > 0) {
          if (e & 1) r = mulmod(r, b, p);
          b = mulmod(b, b, p);
          e >>= 1;
     }
     return r;
}

/* kernel/primes.c:105-122: smallest generator of (Z/p)^* */
static I find_generator(I p)
{
     I f[64], nf = 0, q = p - 1, d, g, i;
     if (p == 2) return 1;
     for (d = 2; d * d <= q; ++d)
          if (q % d == 0) { f[nf++] = d; while (q % d == 0) q /= d; }
     if (q > 1) f[nf++] = q;
     for (g = 2;; ++g) {
          for (i = 0; i < nf; ++i)
               if (powmod(g, (p - 1) / f[i], p) == 1) break;
          if (i == nf) return g;
     }
}

/* Solver selection for one 1D complex DFT of size n. */
enum { M_AUTO = 0, M_CT = 1, M_GENERIC = 2, M_RADER = 3, M_BLUESTEIN = 4 };
#define GENERIC_MAX 173   /* dft/generic.c:112-126, GENERIC_MIN_BAD */

static void dft_rec(I n, const C *in, I is, C *out, I os, int sign,
                    const C *w, I wstride, int method);

/* O(n^2) prime DFT using the Hartley-style pairing of dft/generic.c:54-91:
 * sums over the pairs (j, n-j) share the cos part and differ in sin sign. */
static void dft_generic(I n, const C *in, I is, C *out, I os, int sign,
                        const C *w, I wstride)
{
     I k, j;
     C *xs = (C *)malloc(sizeof(C) * (size_t)n), *xd = (C *)malloc(sizeof(C) * (size_t)n);
     R sr = in[0].re, si = in[0].im;
     for (j = 1; 2 * j < n; ++j) {  /* sums and differences of x[j], x[n-j] */
          C a = in[j * is], b = in[(n - j) * is];
          xs[j].re = a.re + b.re; xs[j].im = a.im + b.im;
          xd[j].re = a.re - b.re; xd[j].im = a.im - b.im;
          sr += xs[j].re; si += xs[j].im;
     }
     out[0].re = sr; out[0].im = si;
     for (k = 1; 2 * k < n; ++k) {
          R rr = in[0].re, ir = in[0].im, ri = 0, ii = 0;
          for (j = 1; 2 * j < n; ++j) {
               const C wj = w[((j * k) % n) * wstride];  /* exp(sign 2pi i jk/n) */
               rr += xs[j].re * wj.re; ir += xs[j].im * wj.re;
               ri += xd[j].re * wj.im; ii += xd[j].im * wj.im;
          }
          /* X[k] = sum_j xs cos + i*sign sin * xd;  X[n-k] = ... - ... */
          out[k * os].re = rr - ii;       out[k * os].im = ir + ri;
          out[(n - k) * os].re = rr + ii; out[(n - k) * os].im = ir - ri;
     }
     if (n % 2 == 0) {  /* not reached for odd primes; kept general */
          R r0 = 0, i0 = 0;
          for (j = 0; j < n; ++j) {
               R sgn = (j & 1) ? -1 : 1;
               r0 += sgn * in[j * is].re; i0 += sgn * in[j * is].im;
          }
          out[(n / 2) * os].re = r0; out[(n / 2) * os].im = i0;
     }
     free(xs); free(xd);
}

/* Rader (dft/rader.c:95-165): for prime p, permute the inputs by powers of
 * a generator g, convolve cyclically (length p-1) with omega, whose DFT is
 * precomputed (dft/rader.c:45-74), and unpermute by powers of g^-1. */
static void dft_rader(I p, const C *in, I is, C *out, I os, int sign)
{
     I g = find_generator(p), ginv = powmod(g, p - 2, p), k, gp;
     I m = p - 1;
     C *buf = (C *)malloc(sizeof(C) * (size_t)m), *tmp = (C *)malloc(sizeof(C) * (size_t)m);
     C *om = (C *)malloc(sizeof(C) * (size_t)m), *omf = (C *)malloc(sizeof(C) * (size_t)m);
     C *wm = mktwiddles(m, -1), *wmi = mktwiddles(m, +1);
     C x0 = in[0];
     /* omega[k] = exp(sign 2 pi i ginv^k / p) / (p-1), then DFT_m (forward) */
     for (k = 0, gp = 1; k < m; ++k, gp = mulmod(gp, ginv, p)) {
          T c, s;
          cexp_t(gp, p, &c, &s);
          om[k].re = (R)(c / (T)m);
          om[k].im = (R)((sign < 0 ? -s : s) / (T)m);
     }
     dft_rec(m, om, 1, omf, 1, -1, wm, 1, M_AUTO);
     for (k = 0, gp = 1; k < m; ++k, gp = mulmod(gp, g, p)) buf[k] = in[gp * is];
     dft_rec(m, buf, 1, tmp, 1, -1, wm, 1, M_AUTO);
     out[0].re = x0.re + tmp[0].re; out[0].im = x0.im + tmp[0].im;
     for (k = 0; k < m; ++k) {  /* pointwise product of spectra */
          C a = tmp[k], b = omf[k];
          buf[k].re = a.re * b.re - a.im * b.im;
          buf[k].im = a.re * b.im + a.im * b.re;
     }
     dft_rec(m, buf, 1, tmp, 1, +1, wmi, 1, M_AUTO);  /* inverse (unnormalized; omega carries 1/m) */
     for (k = 0, gp = 1; k < m; ++k, gp = mulmod(gp, ginv, p)) {
          out[gp * os].re = x0.re + tmp[k].re;
          out[gp * os].im = x0.im + tmp[k].im;
     }
     free(buf); free(tmp); free(om); free(omf); free(wm); free(wmi);
}

static int smooth235(I n)
{
     while (n % 2 == 0) n /= 2;
     while (n % 3 == 0) n /= 3;
     while (n % 5 == 0) n /= 5;
     return n == 1;
}

/* Bluestein (dft/bluestein.c:37-128): chirp w[k] = exp(i*pi*k^2/n) with the
 * index k^2 kept exactly modulo 2n, convolution of length nb = smallest
 * 2,3,5-smooth >= 2n-1 (dft/bluestein.c:180-185). */
static void dft_bluestein(I n, const C *in, I is, C *out, I os, int sign)
{
     I nb = 2 * n - 1, k, ksq = 0, n2 = 2 * n;
     C *w, *W, *b, *wb, *wbi, *tmp;
     while (!smooth235(nb)) ++nb;
     w = (C *)malloc(sizeof(C) * (size_t)n);
     W = (C *)calloc((size_t)nb, sizeof(C));
     b = (C *)calloc((size_t)nb, sizeof(C));
     tmp = (C *)malloc(sizeof(C) * (size_t)nb);
     wb = mktwiddles(nb, -1); wbi = mktwiddles(nb, +1);
     for (k = 0; k < n; ++k) {   /* w[k] = exp(-sign*i*pi*k^2/n) */
          T c, s;
          cexp_t(ksq, n2, &c, &s);
          w[k].re = (R)c; w[k].im = (R)(sign < 0 ? s : -s);
          ksq += 2 * k + 1; while (ksq >= n2) ksq -= n2;
     }
     W[0].re = w[0].re / (R)nb; W[0].im = w[0].im / (R)nb;
     for (k = 1; k < n; ++k) {
          W[k].re = W[nb - k].re = w[k].re / (R)nb;
          W[k].im = W[nb - k].im = w[k].im / (R)nb;
     }
     dft_rec(nb, W, 1, tmp, 1, -1, wb, 1, M_AUTO);
     memcpy(W, tmp, sizeof(C) * (size_t)nb);
     for (k = 0; k < n; ++k) {   /* b = x * conj(w) */
          C x = in[k * is];
          b[k].re = x.re * w[k].re + x.im * w[k].im;
          b[k].im = x.im * w[k].re - x.re * w[k].im;
     }
     dft_rec(nb, b, 1, tmp, 1, -1, wb, 1, M_AUTO);
     for (k = 0; k < nb; ++k) {
          C a = tmp[k], c = W[k];
          b[k].re = a.re * c.re - a.im * c.im;
          b[k].im = a.re * c.im + a.im * c.re;
     }
     dft_rec(nb, b, 1, tmp, 1, +1, wbi, 1, M_AUTO);
     for (k = 0; k < n; ++k) {   /* X = conj(w) * conv */
          C a = tmp[k];
          out[k * os].re = a.re * w[k].re + a.im * w[k].im;
          out[k * os].im = a.im * w[k].re - a.re * w[k].im;
     }
     free(w); free(W); free(b); free(tmp); free(wb); free(wbi);
}

/* Cooley-Tukey DIT step of dft/ct.c:34-58.  n = r*m.  The child computes
 * the r DFTs of length m on inputs x[n1 + r*n2] (input stride r*is) into
 * out[n1*m + k1]; then for each column k1 the radix-r butterfly applies the
 * twiddles W_n^(n1*k1) and a DFT of length r.  The table w holds
 * exp(sign*2*pi*i*j/N) for the top-level N; w[j*wstride] = W_n^j here. */
static void dft_rec(I n, const C *in, I is, C *out, I os, int sign,
                    const C *w, I wstride, int method)
{
     I r, m, n1, k1, k2;
     if (n == 1) { out[0] = in[0]; return; }
     if (method == M_AUTO) {
          if (is_prime(n)) {
               if (n <= 2) method = M_CT;
               else if (n < GENERIC_MAX) method = M_GENERIC;
               else method = M_BLUESTEIN;
          } else method = M_CT;
     }
     if (method == M_GENERIC) { dft_generic(n, in, is, out, os, sign, w, wstride); return; }
     if (method == M_RADER) { dft_rader(n, in, is, out, os, sign); return; }
     if (method == M_BLUESTEIN) { dft_bluestein(n, in, is, out, os, sign); return; }

     r = (n % 4 == 0 && n > 4) ? 4 : smallest_divisor(n);
     if (r == n) {   /* prime radix or n in {2,3,4}: direct O(n^2) */
          if (n == 2) {
               C a = in[0], b = in[is];
               out[0].re = a.re + b.re; out[0].im = a.im + b.im;
               out[os].re = a.re - b.re; out[os].im = a.im - b.im;
               return;
          }
          if (n > 4 && n >= GENERIC_MAX) { dft_bluestein(n, in, is, out, os, sign); return; }
          dft_generic(n, in, is, out, os, sign, w, wstride);
          return;
     }
     m = n / r;
     for (n1 = 0; n1 < r; ++n1)   /* child: r DFTs of length m */
          dft_rec(m, in + n1 * is, r * is, out + n1 * m * os, os, sign, w, wstride * r, M_AUTO);
     {
          C t[64];
          C *tt = r <= 64 ? t : (C *)malloc(sizeof(C) * (size_t)r);
          for (k1 = 0; k1 < m; ++k1) {
               for (n1 = 0; n1 < r; ++n1) {   /* twiddle: W_n^(n1*k1) */
                    C a = out[(n1 * m + k1) * os], tw = w[(n1 * k1) * wstride];
                    tt[n1].re = a.re * tw.re - a.im * tw.im;
                    tt[n1].im = a.re * tw.im + a.im * tw.re;
               }
               if (r == 4) {
                    C a0 = tt[0], a1 = tt[1], a2 = tt[2], a3 = tt[3];
                    R s02r = a0.re + a2.re, s02i = a0.im + a2.im;
                    R d02r = a0.re - a2.re, d02i = a0.im - a2.im;
                    R s13r = a1.re + a3.re, s13i = a1.im + a3.im;
                    R d13r = a1.re - a3.re, d13i = a1.im - a3.im;
                    /* multiply d13 by sign*i */
                    R jr = sign < 0 ? d13i : -d13i, ji = sign < 0 ? -d13r : d13r;
                    out[k1 * os].re = s02r + s13r;           out[k1 * os].im = s02i + s13i;
                    out[(k1 + m) * os].re = d02r + jr;       out[(k1 + m) * os].im = d02i + ji;
                    out[(k1 + 2 * m) * os].re = s02r - s13r; out[(k1 + 2 * m) * os].im = s02i - s13i;
                    out[(k1 + 3 * m) * os].re = d02r - jr;   out[(k1 + 3 * m) * os].im = d02i - ji;
               } else if (r == 2) {
                    C a0 = tt[0], a1 = tt[1];
                    out[k1 * os].re = a0.re + a1.re;       out[k1 * os].im = a0.im + a1.im;
                    out[(k1 + m) * os].re = a0.re - a1.re; out[(k1 + m) * os].im = a0.im - a1.im;
               } else {
                    I wr = (n / r) * wstride;   /* W_r^j = w[j*wr] */
                    for (k2 = 0; k2 < r; ++k2) {
                         R sr = 0, si = 0;
                         for (n1 = 0; n1 < r; ++n1) {
                              C tw = w[((n1 * k2) % r) * wr];
                              sr += tt[n1].re * tw.re - tt[n1].im * tw.im;
                              si += tt[n1].re * tw.im + tt[n1].im * tw.re;
                         }
                         out[(k1 + k2 * m) * os].re = sr; out[(k1 + k2 * m) * os].im = si;
                    }
               }
          }
          if (tt != t) free(tt);
     }
}

/* One 1D complex DFT, any layout, out-of-place-safe. */
static void dft1(I n, const C *in, I is, C *out, I os, int sign, const C *w, int method)
{
     if (in == out) {
          C *tmp = (C *)malloc(sizeof(C) * (size_t)n);
          I j;
          for (j = 0; j < n; ++j) tmp[j] = in[j * is];
          dft_rec(n, tmp, 1, out, os, sign, w, 1, method);
          free(tmp);
     } else dft_rec(n, in, is, out, os, sign, w, 1, method);
}

/* ------------------------------------------------------------ threading */
typedef struct {
     void (*fn)(void *ctx, I lo, I hi);
     void *ctx; I lo, hi;
} job;

static void *job_run(void *a) { job *j = (job *)a; j->fn(j->ctx, j->lo, j->hi); return 0; }

/* Split [0, count) into nthreads contiguous chunks, as
 * threads/dft-vrank-geq1.c splits the vector loop. */
static void parallel_for(int nthreads, I count, void (*fn)(void *, I, I), void *ctx)
{
     if (nthreads <= 1 || count <= 1) { fn(ctx, 0, count); return; }
     if (nthreads > count) nthreads = (int)count;
     {
          pthread_t th[256];
          job jobs[256];
          int t;
          I chunk = (count + nthreads - 1) / nthreads;
          if (nthreads > 256) nthreads = 256;
          for (t = 0; t < nthreads; ++t) {
               jobs[t].fn = fn; jobs[t].ctx = ctx;
               jobs[t].lo = t * chunk;
               jobs[t].hi = (t + 1) * chunk < count ? (t + 1) * chunk : count;
               pthread_create(&th[t], 0, job_run, &jobs[t]);
          }
          for (t = 0; t < nthreads; ++t) pthread_join(th[t], 0);
     }
}

/* Batched 1D pass along one axis of a row-major array: for every index of
 * the other axes, a DFT of length n with element stride s.  Used per axis
 * by the multi-d driver (dft/rank-geq2.c:42-52). */
typedef struct {
     I n, s, outer, inner;   /* array = outer x n x inner, s = inner */
     const C *in; C *out; int sign; const C *w; int method;
} axis_ctx;

static void axis_work(void *c_, I lo, I hi)
{
     axis_ctx *c = (axis_ctx *)c_;
     C *bi = (C *)malloc(sizeof(C) * (size_t)c->n), *bo = (C *)malloc(sizeof(C) * (size_t)c->n);
     I v, j;
     for (v = lo; v < hi; ++v) {
          I o = v / c->inner, i = v % c->inner;
          I base = o * c->n * c->inner + i;
          for (j = 0; j < c->n; ++j) bi[j] = c->in[base + j * c->s];
          dft_rec(c->n, bi, 1, bo, 1, c->sign, c->w, 1, c->method);
          for (j = 0; j < c->n; ++j) c->out[base + j * c->s] = bo[j];
     }
     free(bi); free(bo);
}

static void axis_pass(I outer, I n, I inner, const C *in, C *out, int sign, int nthreads, int method)
{
     axis_ctx c;
     C *w = mktwiddles(n, sign);
     c.n = n; c.s = inner; c.outer = outer; c.inner = inner;
     c.in = in; c.out = out; c.sign = sign; c.w = w; c.method = method;
     parallel_for(nthreads, outer * inner, axis_work, &c);
     free(w);
}

/* ------------------------------------------------------------ public */

/* Batched row-major c2c: howmany arrays of shape n[0..rank-1], contiguous,
 * dist = prod(n).  sign = -1 forward, +1 backward, unnormalized. */
int P(c2c)(int rank, const int *n, I howmany, const C *in, C *out, int sign, int nthreads)
{
     I tot = 1, d, a;
     for (d = 0; d < rank; ++d) tot *= n[d];
     if (rank < 1 || howmany < 0) return -1;
     for (a = rank - 1; a >= 0; --a) {
          I inner = 1, outer;
          for (d = a + 1; d < rank; ++d) inner *= n[d];
          outer = howmany * (tot / (inner * n[a]));
          axis_pass(outer, n[a], inner, a == rank - 1 ? in : out, out, sign, nthreads, M_AUTO);
     }
     return 0;
}

/* Single 1D transform with an explicit solver: method 1 = Cooley-Tukey,
 * 2 = generic O(n^2), 3 = Rader (n prime), 4 = Bluestein. */
int P(dft_method)(I n, const C *in, C *out, int sign, int method)
{
     C *w;
     if (method == M_RADER && !is_prime(n)) return -1;
     w = mktwiddles(n, sign);
     dft1(n, in, 1, out, 1, sign, w, method);
     free(w);
     return 0;
}

/* hc2c post-pass of a real DFT of even length n from the half-length
 * complex DFT Z of z[j] = x[2j] + i x[2j+1] (rdft/ct-hc2c.c:197-210):
 *   X[k] = (Z[k] + conj Z[M-k])/2 - i/2 * W_n^k (Z[k] - conj Z[M-k]). */
typedef struct { I n, rows; const R *in; C *out; } r2c_ctx;

static void r2c_work(void *c_, I lo, I hi)
{
     r2c_ctx *c = (r2c_ctx *)c_;
     I n = c->n, M = n / 2, nc = n / 2 + 1, v, k, j;
     C *z = (C *)malloc(sizeof(C) * (size_t)n), *Z = (C *)malloc(sizeof(C) * (size_t)n);
     C *w = mktwiddles(n, -1), *wm = (n % 2 == 0) ? mktwiddles(M, -1) : mktwiddles(n, -1);
     for (v = lo; v < hi; ++v) {
          const R *x = c->in + v * n;
          C *X = c->out + v * nc;
          if (n % 2 == 1) {   /* odd n: complex DFT of the real sequence */
               for (j = 0; j < n; ++j) { z[j].re = x[j]; z[j].im = 0; }
               dft_rec(n, z, 1, Z, 1, -1, wm, 1, M_AUTO);
               for (k = 0; k < nc; ++k) X[k] = Z[k];
               continue;
          }
          for (j = 0; j < M; ++j) { z[j].re = x[2 * j]; z[j].im = x[2 * j + 1]; }
          dft_rec(M, z, 1, Z, 1, -1, wm, 1, M_AUTO);
          for (k = 0; k <= M; ++k) {
               C a = Z[k % M], b = Z[(M - k) % M], e, o, tw = w[k % n];
               b.im = -b.im;   /* conj Z[M-k] */
               e.re = (a.re + b.re) / 2; e.im = (a.im + b.im) / 2;
               o.re = (a.im - b.im) / 2; o.im = -(a.re - b.re) / 2;   /* (a-b)/(2i) */
               X[k].re = e.re + tw.re * o.re - tw.im * o.im;
               X[k].im = e.im + tw.re * o.im + tw.im * o.re;
          }
     }
     free(z); free(Z); free(w); free(wm);
}

/* hc2c pre-pass of the inverse (rdft/ct-hc2c.c:72-83), even n:
 *   Z'[k] = (X[k] + conj X[M-k]) + i conj(W_n^k) (X[k] - conj X[M-k]),
 * then y[2j] + i y[2j+1] = IDFT_M(Z')[j], unnormalized.  The imaginary
 * parts of X[0] (and X[n/2] for even n) are ignored, as in a halfcomplex
 * array they are not stored. */
typedef struct { I n, rows; const C *in; R *out; } c2r_ctx;

static void c2r_work(void *c_, I lo, I hi)
{
     c2r_ctx *c = (c2r_ctx *)c_;
     I n = c->n, M = n / 2, nc = n / 2 + 1, v, k, j;
     C *Z = (C *)malloc(sizeof(C) * (size_t)n), *z = (C *)malloc(sizeof(C) * (size_t)n);
     C *w = mktwiddles(n, -1), *wm = (n % 2 == 0) ? mktwiddles(M, +1) : mktwiddles(n, +1);
     for (v = lo; v < hi; ++v) {
          const C *X = c->in + v * nc;
          R *y = c->out + v * n;
          if (n % 2 == 1) {   /* odd n: Hermitian extension + inverse DFT */
               Z[0].re = X[0].re; Z[0].im = 0;
               for (k = 1; k < nc; ++k) { Z[k] = X[k]; Z[n - k].re = X[k].re; Z[n - k].im = -X[k].im; }
               dft_rec(n, Z, 1, z, 1, +1, wm, 1, M_AUTO);
               for (j = 0; j < n; ++j) y[j] = z[j].re;
               continue;
          }
          for (k = 0; k < M; ++k) {
               C a = X[k], b = X[M - k], s, d, tw = w[k];
               if (k == 0) { a.im = 0; b.im = 0; }
               b.im = -b.im;
               s.re = a.re + b.re; s.im = a.im + b.im;
               d.re = a.re - b.re; d.im = a.im - b.im;
               /* i * conj(tw) * d */
               {
                    R tr = tw.re * d.re + tw.im * d.im, ti = tw.re * d.im - tw.im * d.re;
                    Z[k].re = s.re - ti; Z[k].im = s.im + tr;
               }
          }
          dft_rec(M, Z, 1, z, 1, +1, wm, 1, M_AUTO);
          for (j = 0; j < M; ++j) { y[2 * j] = z[j].re; y[2 * j + 1] = z[j].im; }
     }
     free(Z); free(z); free(w); free(wm);
}

/* Batched row-major r2c: real arrays n[0..rank-1] (dist prod n) to complex
 * arrays n[0..rank-2] x (n[rank-1]/2+1).  Last axis r2c first, then c2c
 * forward over the leading axes in place on the output
 * (rdft/rank-geq2-rdft2.c:40-51). */
int P(r2c)(int rank, const int *n, I howmany, const R *in, C *out, int nthreads)
{
     I rows = howmany, d, a, nl = n[rank - 1], nc = nl / 2 + 1;
     r2c_ctx c;
     for (d = 0; d < rank - 1; ++d) rows *= n[d];
     c.n = nl; c.rows = rows; c.in = in; c.out = out;
     parallel_for(nthreads, rows, r2c_work, &c);
     for (a = rank - 2; a >= 0; --a) {
          I inner = nc, outer, tot = nc;
          for (d = a + 1; d < rank - 1; ++d) inner *= n[d];
          for (d = 0; d < rank - 1; ++d) tot *= n[d];
          outer = howmany * (tot / (inner * n[a]));
          axis_pass(outer, n[a], inner, out, out, -1, nthreads, M_AUTO);
     }
     return 0;
}

/* Batched row-major c2r (input preserved: works on a copy).  c2c backward
 * over the leading axes first, then c2r on the last axis
 * (rdft/rank-geq2-rdft2.c:56-69). */
int P(c2r)(int rank, const int *n, I howmany, const C *in, R *out, int nthreads)
{
     I rows = howmany, d, a, nl = n[rank - 1], nc = nl / 2 + 1, tot = nc;
     C *tmp;
     c2r_ctx c;
     for (d = 0; d < rank - 1; ++d) { rows *= n[d]; tot *= n[d]; }
     tmp = (C *)malloc(sizeof(C) * (size_t)(rows * nc));
     memcpy(tmp, in, sizeof(C) * (size_t)(rows * nc));
     for (a = rank - 2; a >= 0; --a) {
          I inner = nc, outer;
          for (d = a + 1; d < rank - 1; ++d) inner *= n[d];
          outer = howmany * (tot / (inner * n[a]));
          axis_pass(outer, n[a], inner, tmp, tmp, +1, nthreads, M_AUTO);
     }
     c.n = nl; c.rows = rows; c.in = tmp; c.out = out;
     parallel_for(nthreads, rows, c2r_work, &c);
     free(tmp);
     return 0;
}

/* Twiddle W = exp(sign*2*pi*i*m/n) in trig precision, rounded to R. */
void P(twiddle)(I m, I n, int sign, R *out2)
{
     T c, s;
     cexp_t(m, n, &c, &s);
     out2[0] = (R)c;
     out2[1] = (R)(sign < 0 ? -s : s);
}

/* r2r kinds by their defining sums, O(n^2) per transform with the trig
 * argument reduced exactly (cos/sin of 2 pi m / M with integer m, M), as the
 * reference's manual states them (doc/reference.texi:1923-2020 R2HC/HC2R,
 * 2022-2175 REDFT, 2176-2300 RODFT, and the DHT); kinds use the
 * fftw_r2r_kind values (api/fftw3.h:96-100).  Returns -1 for a kind out of
 * range and for a size-1 REDFT00 (not defined). */
static T r2r_cos(I m, I M) { T c, s; m %= M; if (m < 0) m += M; cexp_t(m, M, &c, &s); return c; }
static T r2r_sin(I m, I M) { T c, s; m %= M; if (m < 0) m += M; cexp_t(m, M, &c, &s); return s; }

int P(r2r)(int kind, I n, I howmany, const R *in, R *out)
{
     I t, j, k;
     for (t = 0; t < howmany; ++t) {
          const R *x = in + t * n;
          R *y = out + t * n;
          for (k = 0; k < n; ++k) {
               T acc = 0;
               switch (kind) {
               case 0: /* R2HC: Re Y_k (k <= n/2), Im Y_{n-k} at n-k */
                    if (2 * k <= n) for (j = 0; j < n; ++j) acc += (T)x[j] * r2r_cos(j * k, n);
                    else for (j = 0; j < n; ++j) acc -= (T)x[j] * r2r_sin(j * (n - k), n);
                    break;
               case 1: /* HC2R: backward DFT of the Hermitian array held in halfcomplex order */
                    for (j = 0; j < n; ++j) {
                         T re, im;
                         if (2 * j <= n) { re = x[j]; im = (j == 0 || 2 * j == n) ? 0 : x[n - j]; }
                         else { re = x[n - j]; im = -(T)x[j]; }
                         acc += re * r2r_cos(j * k, n) - im * r2r_sin(j * k, n);
                    }
                    break;
               case 2: /* DHT: sum x_j (cos + sin)(2 pi j k / n) */
                    for (j = 0; j < n; ++j) acc += (T)x[j] * (r2r_cos(j * k, n) + r2r_sin(j * k, n));
                    break;
               case 3: /* REDFT00: x_0 + (-1)^k x_{n-1} + 2 sum_{0<j<n-1} x_j cos(pi j k / (n-1)); n > 1 */
                    if (n < 2) return -1;
                    acc = (T)x[0] + ((k & 1) ? -(T)x[n - 1] : (T)x[n - 1]);
                    for (j = 1; j + 1 < n; ++j) acc += 2 * (T)x[j] * r2r_cos(j * k, 2 * (n - 1));
                    break;
               case 4: /* REDFT01: x_0 + 2 sum_{j>=1} x_j cos(pi j (2k+1) / 2n) */
                    acc = x[0];
                    for (j = 1; j < n; ++j) acc += 2 * (T)x[j] * r2r_cos(j * (2 * k + 1), 4 * n);
                    break;
               case 5: /* REDFT10: 2 sum x_j cos(pi (2j+1) k / 2n) */
                    for (j = 0; j < n; ++j) acc += 2 * (T)x[j] * r2r_cos((2 * j + 1) * k, 4 * n);
                    break;
               case 6: /* REDFT11: 2 sum x_j cos(pi (2j+1)(2k+1) / 4n) */
                    for (j = 0; j < n; ++j) acc += 2 * (T)x[j] * r2r_cos((2 * j + 1) * (2 * k + 1), 8 * n);
                    break;
               case 7: /* RODFT00: 2 sum x_j sin(pi (j+1)(k+1) / (n+1)) */
                    for (j = 0; j < n; ++j) acc += 2 * (T)x[j] * r2r_sin((j + 1) * (k + 1), 2 * (n + 1));
                    break;
               case 8: /* RODFT01: (-1)^k x_{n-1} + 2 sum_{j<n-1} x_j sin(pi (j+1)(2k+1) / 2n) */
                    acc = (k & 1) ? -(T)x[n - 1] : (T)x[n - 1];
                    for (j = 0; j + 1 < n; ++j) acc += 2 * (T)x[j] * r2r_sin((j + 1) * (2 * k + 1), 4 * n);
                    break;
               case 9: /* RODFT10: 2 sum x_j sin(pi (2j+1)(k+1) / 2n) */
                    for (j = 0; j < n; ++j) acc += 2 * (T)x[j] * r2r_sin((2 * j + 1) * (k + 1), 4 * n);
                    break;
               case 10: /* RODFT11: 2 sum x_j sin(pi (2j+1)(2k+1) / 4n) */
                    for (j = 0; j < n; ++j) acc += 2 * (T)x[j] * r2r_sin((2 * j + 1) * (2 * k + 1), 8 * n);
                    break;
               default:
                    return -1;
               }
               y[k] = (R)acc;
          }
     }
     return 0;
}

/* The same r2r kinds in O(n log n).  DCT/DST-II and -III run as one real
 * DFT of n (r2r_makhoul), DCT/DST-IV of even n as one complex DFT of n/2
 * (r2r_dct4_half); every other kind is the real DFT (this file's r2c / c2r
 * restatement) of a symmetric extension of its input, as the reference's
 * manual defines the REDFT / RODFT kinds: DFTs of real data with even / odd
 * symmetry (doc/reference.texi:1923-2300; DCT-I / DST-I as in the
 * reference's redft00e-r2hc-pad.c and rodft00e-r2hc-pad.c).  Extensions and
 * the bins read back:
 *   R2HC / DHT   r2c of n;  HC2R  c2r of the half spectrum
 *   REDFT00      x even about 0 and n-1: length 2(n-1), Re of bins 0..n-1
 *   RODFT00      x odd about 0 and n+1:  length 2(n+1), -Im of bins 1..n
 *   REDFT10      x_j at odd sample 2j+1 of length 4n, even: Re of bins 0..n-1
 *   RODFT10      the same, odd:                            -Im of bins 1..n
 *   REDFT01      x_j at sample j of length 4n, even:       Re of odd bins 2k+1
 *   RODFT01      x_j at sample j+1, odd (x_{n-1} halved at n): -Im of odd bins
 *   REDFT11      x_j at odd sample 2j+1 of length 8n, even: Re of odd bins 2k+1
 *   RODFT11      the same, odd:                             -Im of odd bins
 * Used by the tests at sizes the defining sums cannot reach and as the
 * host-side timing of r2r.  Returns -1 for a kind out of range or a size-1
 * REDFT00. */
/* DCT-II / DST-II (REDFT10 / RODFT10) and DCT-III / DST-III (REDFT01 /
 * RODFT01) through one real DFT of length n, Makhoul's reduction, the
 * reduction the reference's reodft010e-r2hc.c:42-83 states (it cites the
 * same paper): DCT-II of x is 2 Re(exp(-i pi k / 2n) V_k) with V the DFT of
 * (x_0, x_2, ..., x_3, x_1); DCT-III is its inverse; the DST forms are the
 * DCT forms of the sign-alternated (II) or reversed (III) data. */
static void r2r_makhoul(int kind, I n, I howmany, const R *in, R *out, int nthreads)
{
     const I nc = n / 2 + 1;
     R *v = (R *)malloc(sizeof(R) * (size_t)(howmany * n));
     C *V = (C *)malloc(sizeof(C) * (size_t)(howmany * nc));
     T *wc = (T *)malloc(sizeof(T) * (size_t)n), *ws = (T *)malloc(sizeof(T) * (size_t)n);
     I t, j, k;
     int Ni = (int)n;
     for (k = 0; k < n; ++k) cexp_t(k, 4 * n, &wc[k], &ws[k]);   /* cos, sin of pi k / 2n */
     if (kind == 5 || kind == 9) {
          for (t = 0; t < howmany; ++t)
               for (j = 0; j < n; ++j) {
                    R a = in[t * n + j];
                    if (kind == 9 && (j & 1)) a = -a;
                    v[t * n + ((j & 1) ? n - 1 - (j >> 1) : (j >> 1))] = a;
               }
          P(r2c)(1, &Ni, howmany, v, V, nthreads);
          for (t = 0; t < howmany; ++t)
               for (k = 0; k < n; ++k) {
                    const I q = kind == 9 ? n - 1 - k : k;
                    const I h = (2 * q <= n) ? q : n - q;
                    const T zr = V[t * nc + h].re, zi = (2 * q <= n) ? (T)V[t * nc + h].im : -(T)V[t * nc + h].im;
                    /* exp(-i pi q / 2n) = wc - i ws */
                    out[t * n + k] = (R)(2 * (wc[q] * zr + ws[q] * zi));
               }
     } else {
          for (t = 0; t < howmany; ++t)
               for (k = 0; k < nc; ++k) {
                    const R *x = in + t * n;
                    const T a = kind == 8 ? (T)x[n - 1 - k] : (T)x[k];
                    const T b = k == 0 ? 0 : (kind == 8 ? (T)x[k - 1] : (T)x[n - k]);
                    /* exp(i pi k / 2n) = wc + i ws */
                    V[t * nc + k].re = (R)(a * wc[k] + b * ws[k]);
                    V[t * nc + k].im = (R)(a * ws[k] - b * wc[k]);
               }
          P(c2r)(1, &Ni, howmany, V, v, nthreads);
          for (t = 0; t < howmany; ++t)
               for (k = 0; k < n; ++k) {
                    R r = v[t * n + ((k & 1) ? n - 1 - (k >> 1) : (k >> 1))];
                    if (kind == 8 && (k & 1)) r = -r;
                    out[t * n + k] = r;
               }
     }
     free(v);
     free(V);
     free(wc);
     free(ws);
}

/* DCT-IV / DST-IV (REDFT11 / RODFT11) of even n through one complex DFT of
 * n/2, the half-length reduction (the reference's reodft11e-radix2.c
 * splits the same transform into two halves of n/2): z_m = (x_{2m} +
 * i x_{n-1-2m}) exp(-i pi (4m+1) / 4n), u_p = Z_p exp(-i pi p / n),
 * y_{2p} = 2 Re u_p, y_{n-1-2p} = -2 Im u_p; DST-IV is (-1)^k DCT-IV of x
 * reversed. */
static void r2r_dct4_half(int kind, I n, I howmany, const R *in, R *out, int nthreads)
{
     const I M = n / 2;
     C *z = (C *)malloc(sizeof(C) * (size_t)(howmany * M));
     C *Z = (C *)malloc(sizeof(C) * (size_t)(howmany * M));
     T *w = (T *)malloc(sizeof(T) * (size_t)(4 * M));   /* pre (c, s), post (c, s) per index */
     I t, m, p;
     int Mi = (int)M;
     for (m = 0; m < M; ++m) {
          cexp_t(4 * m + 1, 8 * n, &w[4 * m], &w[4 * m + 1]);   /* pi (4m+1) / 4n */
          cexp_t(m, 2 * n, &w[4 * m + 2], &w[4 * m + 3]);       /* pi m / n */
     }
     for (t = 0; t < howmany; ++t)
          for (m = 0; m < M; ++m) {
               const R *x = in + t * n;
               const I ja = 2 * m, jb = n - 1 - 2 * m;
               const T a = kind == 10 ? (T)x[jb] : (T)x[ja], b = kind == 10 ? (T)x[ja] : (T)x[jb];
               const T c = w[4 * m], s_ = w[4 * m + 1];   /* exp(-i pi (4m+1) / 4n) = c - i s_ */
               z[t * M + m].re = (R)(a * c + b * s_);
               z[t * M + m].im = (R)(b * c - a * s_);
          }
     P(c2c)(1, &Mi, howmany, z, Z, -1, nthreads);
     for (t = 0; t < howmany; ++t)
          for (p = 0; p < M; ++p) {
               const T zr = Z[t * M + p].re, zi = Z[t * M + p].im;
               const T c = w[4 * p + 2], s_ = w[4 * p + 3];   /* exp(-i pi p / n) = c - i s_ */
               T ur, ui;
               R ye, yo;
               ur = zr * c + zi * s_;
               ui = zi * c - zr * s_;
               ye = (R)(2 * ur);
               yo = (R)(-2 * ui);
               /* y_{2p} (even index) and y_{n-1-2p} (odd index: DST-IV flips its sign) */
               out[t * n + 2 * p] = ye;
               out[t * n + n - 1 - 2 * p] = kind == 10 ? -yo : yo;
          }
     free(z);
     free(Z);
     free(w);
}

int P(r2r_fast)(int kind, I n, I howmany, const R *in, R *out, int nthreads)
{
     I N, nc, t, j, k;
     int Ni;
     R *ext;
     C *spec;
     if (kind < 0 || kind > 10 || (kind == 3 && n < 2)) return -1;
     if (kind == 4 || kind == 5 || kind == 8 || kind == 9) {
          r2r_makhoul(kind, n, howmany, in, out, nthreads);
          return 0;
     }
     if ((kind == 6 || kind == 10) && n % 2 == 0) {
          r2r_dct4_half(kind, n, howmany, in, out, nthreads);
          return 0;
     }
     if (kind == 1) {
          /* HC2R: the halfcomplex array as the half spectrum, then c2r */
          nc = n / 2 + 1;
          spec = (C *)malloc(sizeof(C) * (size_t)(howmany * nc));
          for (t = 0; t < howmany; ++t)
               for (k = 0; k < nc; ++k) {
                    spec[t * nc + k].re = in[t * n + k];
                    spec[t * nc + k].im = (k == 0 || 2 * k == n) ? 0 : in[t * n + n - k];
               }
          Ni = (int)n;
          P(c2r)(1, &Ni, howmany, spec, out, nthreads);
          free(spec);
          return 0;
     }
     N = (kind == 0 || kind == 2) ? n : kind == 3 ? 2 * (n - 1) : kind == 7 ? 2 * (n + 1)
         : (kind == 6 || kind == 10) ? 8 * n : 4 * n;
     nc = N / 2 + 1;
     ext = (R *)calloc((size_t)(howmany * N), sizeof(R));
     spec = (C *)malloc(sizeof(C) * (size_t)(howmany * nc));
     for (t = 0; t < howmany; ++t) {
          const R *x = in + t * n;
          R *e = ext + t * N;
          for (j = 0; j < n; ++j) {
               switch (kind) {
               case 0: case 2: e[j] = x[j]; break;
               case 3: e[j] = x[j]; if (j > 0 && j < n - 1) e[N - j] = x[j]; break;
               case 7: e[j + 1] = x[j]; e[N - 1 - j] = -x[j]; break;
               case 5: e[2 * j + 1] = x[j]; e[N - 2 * j - 1] = x[j]; break;
               case 9: e[2 * j + 1] = x[j]; e[N - 2 * j - 1] = -x[j]; break;
               case 4: e[j] = x[j]; if (j > 0) e[N - j] = x[j]; break;
               case 8:
                    if (j + 1 < n) { e[j + 1] = x[j]; e[N - j - 1] = -x[j]; }
                    else { e[n] = x[j] / 2; e[3 * n] = -x[j] / 2; }
                    break;
               case 6: e[2 * j + 1] = x[j]; e[N - 2 * j - 1] = x[j]; break;
               default: e[2 * j + 1] = x[j]; e[N - 2 * j - 1] = -x[j]; break;   /* 10 */
               }
          }
     }
     Ni = (int)N;
     P(r2c)(1, &Ni, howmany, ext, spec, nthreads);
     for (t = 0; t < howmany; ++t) {
          const C *Y = spec + t * nc;
          R *y = out + t * n;
          for (k = 0; k < n; ++k) {
               switch (kind) {
               case 0: y[k] = (2 * k <= n) ? Y[k].re : Y[n - k].im; break;
               case 2: {
                    const I h = (2 * k <= n) ? k : n - k;
                    const T im = (2 * k <= n) ? (T)Y[h].im : -(T)Y[h].im;
                    y[k] = (R)((T)Y[h].re - im);
                    break;
               }
               case 3: case 5: y[k] = Y[k].re; break;
               case 7: case 9: y[k] = -Y[k + 1].im; break;
               case 4: case 6: y[k] = Y[2 * k + 1].re; break;
               default: y[k] = -Y[2 * k + 1].im; break;                         /* 8, 10 */
               }
          }
     }
     free(ext);
     free(spec);
     return 0;
}
