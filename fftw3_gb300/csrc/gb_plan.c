/*
 * The planner: turns a problem (transform tensor + vector tensor + arrays)
 * into a list of GPU passes.
 *
 * Reference counterparts and what replaced them:
 *   kernel/tensor7.c:99-167 (canonicalization: drop n=1 dims, merge
 *     contiguous vector dims)                    -> gb_canon_vec()
 *   dft/rank-geq2.c:42-52, :121-172 (multi-d = trailing axes, then the
 *     leading axes in place on the output)         -> gb_mkplan() axis loop
 *   rdft/rank-geq2-rdft2.c:40-69 (r2c: last axis then c2c; c2r reversed,
 *     the c2c part in place on the input)          -> gb_mkplan() r2c/c2r
 *   dft/vrank-geq1.c:54-65 (loop over the batch) -> the CUDA grid
 *   dft/ct.c + kernel/primes.c:183-195 (radix choice) -> gb_factor()
 *   dft/buffered.c, dft/indirect-transpose.c (strided axes) -> COLS tiles
 *   large n: the reference recurses Cooley-Tukey one memory pass per level;
 *     here n = n1*n2 runs as two passes with the n1-point outputs twiddled
 *     by W_n^(n2*k1) in the first pass (four-step)   -> add_fourstep()
 *   dft/bluestein.c (prime n > 16, conv size 2,3,5-smooth >= 2n-1) ->
 *     GB_KIND_BLUESTEIN with a power-of-two convolution inside one CTA
 *   kernel/planner.c search + api/apiplan.c:86-178 patience loop -> the
 *     configuration heuristics here, refined by measurement (gb_tune) under
 *     FFTW_MEASURE/PATIENT/EXHAUSTIVE and recorded as wisdom.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

/* ------------------------------------------------------------ errors */
static __thread char gb_err[512];
const char *gb_last_error(void) { return gb_err; }
void gb_set_error(const char *fmt, ...)
{
     va_list ap;
     va_start(ap, fmt);
     vsnprintf(gb_err, sizeof gb_err, fmt, ap);
     va_end(ap);
     if (getenv("FFTW_GB300_TRACE")) fprintf(stderr, "[fftw_gb300] %s\n", gb_err);
}

static pthread_mutex_t gb_mtx = PTHREAD_MUTEX_INITIALIZER;
void gb_lock(void) { pthread_mutex_lock(&gb_mtx); }
void gb_unlock(void) { pthread_mutex_unlock(&gb_mtx); }

static int gb_dry = 0;
int gb_dry_run(void) { return gb_dry; }
void gb_set_dry_run(int on) { gb_dry = on; }

int gb_cuda_ready(void)
{
     static int state = -1;
     if (state < 0) {
          int n = 0;
          state = (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) ? 1 : 0;
     }
     return state;
}

/* planner-wide choice set by add_1d from wisdom (the planner runs under the
 * library lock): 1 = do not use the bulk-copy fed persistent variant */
static int cfg_no_tma = 0;
/* and, from the same wisdom entry: compute groups of a bulk-copy pass (0 =
 * the planner's choice) and the radix order of a runtime-radix pass */
static int cfg_groups = 0, cfg_order = 0;

/* shared memory of one SM (two CTAs of a persistent kernel must fit, each
 * with the 1 KB the system reserves) */
static int smem_sm(void)
{
     static int v = 0;
     if (!v) v = (!gb_dry && gb_cuda_ready()) ? gb_device_smem_per_sm() : 233472;
     if (!v) v = 233472;
     return v;
}

static int smem_max(void)
{
     static int v = 0;
     if (!v) v = (!gb_dry && gb_cuda_ready()) ? gb_device_max_smem() : 232448;
     if (!v) v = 232448;
     return v;
}

/* ------------------------------------------------------------ tables */
typedef struct tab { int prec, type; long long a, b, c; void *p; struct tab *next; } tab;
static tab *tabs = 0;

static void *tab_find(int prec, int type, long long a, long long b, long long c)
{
     tab *t;
     for (t = tabs; t; t = t->next)
          if (t->prec == prec && t->type == type && t->a == a && t->b == b && t->c == c) return t->p;
     return 0;
}

/* Test hook for the planner's handling of a failed device allocation: the
 * table allocation after the next k fails once, as a refused cudaMalloc
 * would (-1: none).  Applies in dry runs too, where tables are not cached. */
static int fail_alloc_in = -1;
void gb_fail_alloc_after(int k) { fail_alloc_in = k < 0 ? -1 : k; }

static void *tab_add(int prec, int type, long long a, long long b, long long c, size_t bytes)
{
     tab *t;
     void *p = 0;
     if (fail_alloc_in >= 0 && fail_alloc_in-- == 0) {
          gb_set_error("cudaMalloc(%zu) for a twiddle table failed (injected)", bytes);
          return 0;
     }
     if (gb_dry) {
          static char dummy[64];
          return dummy;
     }
     if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
          gb_set_error("cudaMalloc(%zu) for a twiddle table failed", bytes);
          return 0;
     }
     t = (tab *)malloc(sizeof *t);
     t->prec = prec; t->type = type; t->a = a; t->b = b; t->c = c; t->p = p;
     t->next = tabs; tabs = t;
     return p;
}

/* exp(-2 pi i (j*mul) / n), j < count */
const void *gb_table_twiddle(int prec, long long n, long long count, long long mul)
{
     void *p = tab_find(prec, 0, n, count, mul);
     if (p) return p;
     p = tab_add(prec, 0, n, count, mul, (size_t)count * 2 * prec);
     if (!p || gb_dry) return p;
     if (gb_twiddles(p, prec, n, count, mul, 0) || cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("twiddle generation failed: %s", gb_last_cuda_error());
          return 0;
     }
     return p;
}

/* the radix-16 stage twiddles of a power-of-two nfft in the coalesced layout
 * of gb_pass.tw_stage */
const void *gb_table_stage_twiddle(int prec, int nfft)
{
     const int len = gb_stage_tw_len(nfft, prec);
     void *p = tab_find(prec, 5, nfft, 0, 0);
     if (p) return p;
     p = tab_add(prec, 5, nfft, 0, 0, (size_t)(len ? len : 1) * 2 * prec);
     if (!p || gb_dry) return p;
     if (gb_stage_twiddles(p, prec, nfft, 0) || cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("stage twiddle generation failed: %s", gb_last_cuda_error());
          return 0;
     }
     return p;
}

/* the stage twiddles of a runtime-radix pass with radix list rad (layout of
 * gb_pass.tw_gen); keyed on nfft and the list, four bits a radix - 1 */
static const void *table_gen_stage(int prec, int nfft, const int *rad, int nrad)
{
     long long k0 = 0, k1 = nrad;
     void *p;
     int i;
     for (i = 0; i < nrad; ++i) {
          if (rad[i] < 2 || rad[i] > 16) return 0;
          if (i < 15) k0 |= (long long)(rad[i] - 1) << (4 * i);
          else k1 |= (long long)(rad[i] - 1) << (4 * (i - 15) + 8);
     }
     p = tab_find(prec, 7, nfft, k0, k1);
     if (p) return p;
     p = tab_add(prec, 7, nfft, k0, k1, (size_t)(nfft > 1 ? nfft - 1 : 1) * 2 * prec);
     if (!p || gb_dry) return p;
     if (gb_gen_stage_twiddles(p, prec, nfft, rad, nrad, 0) || cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("runtime-radix stage twiddle generation failed: %s", gb_last_cuda_error());
          return 0;
     }
     return p;
}

/* rows of the four-step twiddle W_N^(v t), v < rows, t < T (gb_pass.post_rows) */
static const void *table_post_rows(int prec, long long N, int T, long long rows)
{
     void *p = tab_find(prec, 6, N, T, rows);
     if (p) return p;
     p = tab_add(prec, 6, N, T, rows, (size_t)(rows * T) * 2 * prec);
     if (!p || gb_dry) return p;
     if (gb_post_rows(p, prec, N, T, rows, 0) || cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("four-step twiddle rows failed: %s", gb_last_cuda_error());
          return 0;
     }
     return p;
}

const void *gb_table_chirp(int prec, long long n, int sign)
{
     void *p = tab_find(prec, 1, n, sign, 0);
     if (p) return p;
     p = tab_add(prec, 1, n, sign, 0, (size_t)n * 2 * prec);
     if (!p || gb_dry) return p;
     if (gb_chirp(p, prec, n, sign, 0) || cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("chirp generation failed: %s", gb_last_cuda_error());
          return 0;
     }
     return p;
}

static int config_pass(gb_pass *P, int prec, int kind, long long n, int sign, long long is, long long os,
                       int nv, const gb_dim *v, int tb_hint, int keep_order);
static int pass_tables(gb_pass *P);

/* Spectrum of the padded chirp / nb (dft/bluestein.c:52-80), computed on the
 * device with this library's own forward FFT. */
const void *gb_table_chirp_spec(int prec, long long n, long long nb, int sign)
{
     void *p = tab_find(prec, 2, n, nb, sign);
     const void *w;
     gb_pass P;
     gb_dim d;
     if (p) return p;
     w = gb_table_chirp(prec, n, sign);
     if (!w) return 0;
     p = tab_add(prec, 2, n, nb, sign, (size_t)nb * 2 * prec);
     if (!p || gb_dry) return p;
     if (gb_chirp_pad(p, w, prec, n, nb, 0)) {
          gb_set_error("chirp padding failed: %s", gb_last_cuda_error());
          return 0;
     }
     d.n = 1; d.is = 0; d.os = 0;
     if (config_pass(&P, prec, GB_KIND_C2C, nb, -1, 1, 1, 1, &d, 0, 0) == 0 && pass_tables(&P) == 0) {
          if (gb_launch_pass(&P, p, p, 0) || cudaDeviceSynchronize() != cudaSuccess) {
               gb_set_error("chirp spectrum failed: %s", gb_last_cuda_error());
               return 0;
          }
          return p;
     }
     {
          /* convolution longer than one CTA: a forward plan of length nb,
           * in place on the table */
          gb_problem prb;
          gb_plan *q;
          int rc;
          memset(&prb, 0, sizeof prb);
          prb.kind = GB_PROB_DFT; prb.prec = prec; prb.sign = -1; prb.rank = 1;
          prb.sz[0].n = nb; prb.sz[0].is = 1; prb.sz[0].os = 1;
          prb.vrank = 1; prb.vec[0].n = 1; prb.vec[0].is = nb; prb.vec[0].os = nb;
          prb.in = p; prb.out = p;
          q = gb_mkplan(&prb, FFTW_ESTIMATE);
          if (!q) return 0;
          rc = gb_execute(q, p, p);
          gb_destroy(q);
          if (rc) return 0;
     }
     return p;
}

/* Rader tables (dft/rader.c:45-74, kernel/primes.c:105-122): generator
 * powers and discrete logs as int32, and the spectrum of omega/(p-1)
 * computed on the device with this library's own forward FFT. */
static long long powmod_ll(long long b, long long e, long long m)
{
     long long r = 1;
     b %= m;
     while (e > 0) {
          if (e & 1) r = (long long)((__int128)r * b % m);
          b = (long long)((__int128)b * b % m);
          e >>= 1;
     }
     return r;
}

static long long find_generator(long long p)
{
     long long f[64], nf = 0, q = p - 1, d, g;
     int i;
     if (p == 2) return 1;
     for (d = 2; d * d <= q; ++d)
          if (q % d == 0) { f[nf++] = d; while (q % d == 0) q /= d; }
     if (q > 1) f[nf++] = q;
     for (g = 2;; ++g) {
          for (i = 0; i < nf; ++i)
               if (powmod_ll(g, (p - 1) / f[i], p) == 1) break;
          if (i == nf) return g;
     }
}

const int *gb_table_rader_perm(long long p)
{
     void *dp = tab_find(4, 3, p, 0, 0);
     int *h;
     long long g, ginv, k, v;
     if (dp) return (const int *)dp;
     dp = tab_add(4, 3, p, 0, 0, (size_t)(2 * (p - 1)) * sizeof(int));
     if (!dp || gb_dry) return (const int *)dp;
     h = (int *)malloc((size_t)(2 * (p - 1)) * sizeof(int));
     g = find_generator(p);
     ginv = powmod_ll(g, p - 2, p);
     for (k = 0, v = 1; k < p - 1; ++k, v = v * g % p) h[k] = (int)v;
     for (k = 0, v = 1; k < p - 1; ++k, v = v * ginv % p) h[(p - 1) + (v - 1)] = (int)k;
     if (cudaMemcpy(dp, h, (size_t)(2 * (p - 1)) * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
          free(h);
          gb_set_error("Rader table upload failed");
          return 0;
     }
     free(h);
     return (const int *)dp;
}

const void *gb_table_rader_spec(int prec, long long p, int sign)
{
     void *dp = tab_find(prec, 4, p, sign, 0);
     const int *perm;
     gb_pass P;
     gb_dim d;
     if (dp) return dp;
     perm = gb_table_rader_perm(p);
     if (!perm) return 0;
     dp = tab_add(prec, 4, p, sign, 0, (size_t)(p - 1) * 2 * prec);
     if (!dp || gb_dry) return dp;
     if (gb_rader_omega(dp, perm, prec, p, sign, 0)) {
          gb_set_error("Rader omega failed: %s", gb_last_cuda_error());
          return 0;
     }
     d.n = 1; d.is = 0; d.os = 0;
     if (config_pass(&P, prec, GB_KIND_C2C, p - 1, -1, 1, 1, 1, &d, 0, 0) != 0 || pass_tables(&P) != 0) {
          gb_set_error("Rader: no forward FFT of length %lld", p - 1);
          return 0;
     }
     if (gb_launch_pass(&P, dp, dp, 0) || cudaDeviceSynchronize() != cudaSuccess) {
          gb_set_error("Rader omega spectrum failed: %s", gb_last_cuda_error());
          return 0;
     }
     return dp;
}

void gb_tables_free(void)
{
     while (tabs) {
          tab *t = tabs;
          tabs = t->next;
          cudaFree(t->p);
          free(t);
     }
}

/* ------------------------------------------------------------ helpers */
static int is_pow2(long long n) { return n > 0 && (n & (n - 1)) == 0; }
static int ilog2(long long n) { int l = 0; while ((1LL << l) < n) ++l; return l; }
static long long llabs_(long long a) { return a < 0 ? -a : a; }

/* radix list for k_gen: 16s first, then 8/4/2, then odd primes <= 13 */
static int gb_factor(long long n, int *rad)
{
     int k = 0;
     static const int odd[] = {3, 5, 7, 11, 13};
     int i;
     while (n % 16 == 0 && k < GB_MAXRAD) { rad[k++] = 16; n /= 16; }
     if (n % 8 == 0) { rad[k++] = 8; n /= 8; }
     if (n % 4 == 0) { rad[k++] = 4; n /= 4; }
     if (n % 2 == 0) { rad[k++] = 2; n /= 2; }
     for (i = 0; i < 5; ++i)
          while (n % odd[i] == 0 && k < GB_MAXRAD) { rad[k++] = odd[i]; n /= odd[i]; }
     return n == 1 ? k : -1;
}

static int csize(int prec) { return 2 * prec; }

int gb_factor_radices(long long n, int *rad) { return gb_factor(n, rad); }

/* The radix list of a runtime-radix pass in one of GB_RADIX_ORDERS orders
 * (the tuner's choice, recorded in wisdom): 0 = radix 16 first, then 8, 4,
 * 2 and the odd primes ascending (gb_factor); 1 = no radix 16: radix 8
 * first, then 4, 2 and the odd primes descending; 2 = the odd primes
 * descending first, then 16, 8, 4, 2.  Returns the number of stages, or -1
 * when n has a prime factor above 13. */
int gb_factor_order(long long n, int *rad, int order)
{
     static const int odd[] = {13, 11, 7, 5, 3};
     int k = 0, i, p2[GB_MAXRAD], np2 = 0, po[GB_MAXRAD], npo = 0;
     if (order <= 0 || order >= GB_RADIX_ORDERS) return gb_factor(n, rad);
     for (i = 0; i < 5; ++i)
          while (n % odd[i] == 0 && npo < GB_MAXRAD) { po[npo++] = odd[i]; n /= odd[i]; }
     if (order == 1) {
          while (n % 8 == 0 && np2 < GB_MAXRAD) { p2[np2++] = 8; n /= 8; }
     } else {
          while (n % 16 == 0 && np2 < GB_MAXRAD) { p2[np2++] = 16; n /= 16; }
          if (n % 8 == 0) { p2[np2++] = 8; n /= 8; }
     }
     if (n % 4 == 0) { p2[np2++] = 4; n /= 4; }
     if (n % 2 == 0) { p2[np2++] = 2; n /= 2; }
     if (n != 1 || np2 + npo > GB_MAXRAD) return -1;
     if (order == 1) {
          for (i = 0; i < np2; ++i) rad[k++] = p2[i];
          for (i = 0; i < npo; ++i) rad[k++] = po[i];
     } else {
          for (i = 0; i < npo; ++i) rad[k++] = po[i];
          for (i = 0; i < np2; ++i) rad[k++] = p2[i];
     }
     return k;
}
static int reg_max_log(int prec) { return prec == 4 ? 14 : 13; }
static int reg_e(int nfft) { return nfft < 16 ? nfft : 16; }
static int reg_sms(int nfft) { return gb_reg_sms(nfft); }
static int reg_maxthreads(int nfft) { int t = nfft / reg_e(nfft); return t > 256 ? t : 256; }
static int tma_sms(int nfft) { return gb_reg_sms(nfft); }

/* FFTW's canonical vector tensor: drop n = 1, merge dims that are
 * contiguous in both input and output (kernel/tensor7.c:99-167). */
static int gb_canon_vec(gb_dim *v, int nv)
{
     int i, j, k = 0;
     for (i = 0; i < nv; ++i)
          if (v[i].n != 1) v[k++] = v[i];
     nv = k;
     for (i = 0; i < nv; ++i)     /* sort by |is| descending, then |os| */
          for (j = i + 1; j < nv; ++j)
               if (llabs_(v[j].is) > llabs_(v[i].is) ||
                   (llabs_(v[j].is) == llabs_(v[i].is) && llabs_(v[j].os) > llabs_(v[i].os))) {
                    gb_dim t = v[i]; v[i] = v[j]; v[j] = t;
               }
     for (i = nv - 1; i > 0; --i) {   /* v[i-1] outer, v[i] inner */
          if (v[i - 1].is == v[i].n * v[i].is && v[i - 1].os == v[i].n * v[i].os) {
               v[i].n *= v[i - 1].n;
               for (j = i - 1; j < nv - 1; ++j) v[j] = v[j + 1];
               --nv;
               i = nv;
          }
     }
     return nv;
}

/* Configure one pass: kernel variant, tile, moves, launch shape.
 * Returns 0 on success, 1 if the length needs more than one CTA
 * (four-step or multi-pass Bluestein), -1 if unsupported. */
static int config_pass(gb_pass *P, int prec, int kind, long long n, int sign, long long is, long long os,
                       int nv, const gb_dim *v_in, int tb_hint, int keep_order)
{
     gb_dim v[GB_MAXV + GB_MAXLOOP];
     int i, best, smax = smem_max();
     long long nfft;
     int half = (kind == GB_KIND_R2C || kind == GB_KIND_C2R) && (n % 2 == 0);
     memset(P, 0, sizeof *P);
     P->ltb = -1;
     if (nv > GB_MAXV) nv = GB_MAXV;
     for (i = 0; i < nv; ++i) v[i] = v_in[i];
     if (nv == 0) { v[0].n = 1; v[0].is = 0; v[0].os = 0; nv = 1; }
     P->kind = kind; P->prec = prec; P->sign = sign; P->n = (int)n;
     nfft = half ? n / 2 : n;
     P->nfft = (int)nfft;
     P->is = is; P->os = os;

     /* tile dimension: the vector dim with the smallest stride */
     best = 0;
     for (i = 1; i < nv && !keep_order; ++i) {
          long long si = llabs_(v[i].is) + llabs_(v[i].os), sb = llabs_(v[best].is) + llabs_(v[best].os);
          if (si < sb) best = i;
     }
     if (best) { gb_dim t = v[0]; v[0] = v[best]; v[best] = t; }
     P->nv = nv;
     for (i = 0; i < nv; ++i) { P->vn[i] = v[i].n; P->vis[i] = v[i].is; P->vos[i] = v[i].os; }

     if (kind == GB_KIND_COPY) {
          P->variant = GB_VAR_GEN;
          P->tb = 256; P->threads = 256; P->smem = 0;
          P->ntiles0 = (v[0].n + P->tb - 1) / P->tb;
          P->nblocks = P->ntiles0;
          for (i = 1; i < nv; ++i) P->nblocks *= v[i].n;
          return 0;
     }

     if (kind == GB_KIND_RADER) { nfft = n - 1; P->nfft = (int)nfft; }
     if (kind == GB_KIND_BLUESTEIN) {   /* convolution length: power of two >= 2n-1 */
          long long nb = 1;
          while (nb < 2 * n - 1) nb <<= 1;
          nfft = nb;
          P->nfft = (int)nb;
     }
     if (is_pow2(nfft) && ilog2(nfft) <= reg_max_log(prec) &&
         (kind == GB_KIND_C2C || kind == GB_KIND_BLUESTEIN || half) && !(kind == GB_KIND_BLUESTEIN && nfft < 32) &&
         kind != GB_KIND_RADER) {
          int E = reg_e((int)nfft), T = (int)nfft / E, tb, maxt = reg_maxthreads((int)nfft);
          int cols_in, cols_out;
          long long sm1 = (long long)reg_sms((int)nfft) * csize(prec);
          P->variant = GB_VAR_REG;
          cols_in = llabs_(is) != 1 && llabs_(P->vis[0]) == 1;
          cols_out = llabs_(os) != 1 && llabs_(P->vos[0]) == 1;
          if (kind == GB_KIND_R2C) cols_in = llabs_(is) != 1 && llabs_(P->vis[0]) <= 2;
          if (kind == GB_KIND_C2R) cols_out = llabs_(os) != 1 && llabs_(P->vos[0]) <= 2;
          tb = 256 / T; if (tb < 1) tb = 1;
          if (cols_in || cols_out) { int want = prec == 4 ? 16 : 8; if (tb < want) tb = want; }
          if (tb_hint > 0) tb = tb_hint;
          while (tb > 1 && (tb * T > maxt || tb * sm1 > smax)) tb >>= 1;
          /* column tiles: at most 256 threads, so two or more CTAs share an SM
           * and one's loads overlap another's stages */
          if ((cols_in || cols_out) && tb_hint == 0)
               while (tb > 1 && tb * T > 256) tb >>= 1;
          while (tb > 1 && (tb >> 1) >= v[0].n) tb >>= 1;
          if (sm1 > smax) return 1;
          P->tb = tb;
          P->threads = tb * T;
          P->smem = (int)(tb * sm1);
          if (llabs_(is) == 1 && !(kind == GB_KIND_R2C && is != 1))
               P->load_mode = (T >= 32 && kind != GB_KIND_C2R) ? GB_MOVE_DIRECT : GB_MOVE_ROWS;
          else if (cols_in) P->load_mode = GB_MOVE_COLS;
          else P->load_mode = (kind == GB_KIND_C2R) ? GB_MOVE_ROWS : GB_MOVE_DIRECT;
          if (llabs_(os) == 1)
               P->store_mode = (T >= 32 && kind != GB_KIND_R2C) ? GB_MOVE_DIRECT : GB_MOVE_ROWS;
          else if (cols_out) P->store_mode = GB_MOVE_COLS;
          else P->store_mode = GB_MOVE_DIRECT;
          if (kind == GB_KIND_R2C && P->store_mode == GB_MOVE_DIRECT && llabs_(os) == 1 && T < 32)
               P->store_mode = GB_MOVE_ROWS;
          /* f32 c2c column tiles whose strides the TMA engine can walk:
           * persistent CTAs fed by tensor-map boxes (k_cols_tma) */
          if (kind == GB_KIND_C2C && prec == 4 && P->load_mode == GB_MOVE_COLS && !cfg_no_tma &&
              !getenv("FFTW_GB300_NO_TMA")) {
               gb_pass t = *P;
               int l = 0;
               while ((1 << l) < tb) ++l;
               t.ltb = ((1 << l) == tb) ? l : -1;
               t.variant = GB_VAR_TMA_COLS;
               /* one compute group over two slots, three CTAs per SM (measured
                * faster than two groups over three slots on every column pass);
                * FFTW_GB300_TMA_GROUPS=2 asks for two where they fit */
               {
                    const char *genv = getenv("FFTW_GB300_TMA_GROUPS");
                    t.groups = (genv && atoi(genv) == 2) ? 2 : 1;
               }
               /* a group of two is whole warps (its named barrier counts warps) */
               if (t.threads % 32) t.groups = 1;
               t.smem = gb_cols_tma_smem((int)nfft, tb, t.groups);
               if (t.smem > smax || 2LL * (t.smem + 1024) > smem_sm()) {
                    t.groups = 1;
                    t.smem = gb_cols_tma_smem((int)nfft, tb, 1);
               }
               if (t.smem <= smax && gb_cols_tma_plan_ok(&t)) {
                    P->variant = GB_VAR_TMA_COLS;
                    P->groups = t.groups;
                    P->smem = t.smem;
               }
          }
          /* unit-stride c2c with 16-byte aligned transform starts: persistent
           * CTAs fed by bulk async copies (k_reg_tma) */
          if ((kind == GB_KIND_C2C || kind == GB_KIND_R2C) && is == 1 && os == 1 && nfft >= 64 && nfft <= 8192 &&
              tb_hint == 0 && !cfg_no_tma && !getenv("FFTW_GB300_NO_TMA")) {
               int ok = 1, tbt = 256 / T;
               long long sm2;
               const int ein = kind == GB_KIND_R2C ? prec : csize(prec);   /* bytes per input element */
               for (i = 0; i < nv; ++i)
                    if ((P->vis[i] * ein) % 16) ok = 0;
               /* compute groups per CTA: two for the float 8192-point core (one
                * CTA of 2 x 512 threads and three buffers an SM: two tiles in
                * flight where one group has one), one elsewhere, where three
                * one-group CTAs an SM measured faster (CTA-wide barriers, 85
                * registers a thread); FFTW_GB300_TMA_GROUPS overrides.  One
                * buffer per group and one more; keep two CTAs of two groups or
                * three of one group per SM */
               const char *genv = getenv("FFTW_GB300_TMA_GROUPS");
               int groups = (prec == 4 && nfft == 8192) ? 2 : 1;
               if (cfg_groups == 1 || cfg_groups == 2) groups = cfg_groups;   /* the tuner's choice */
               if (genv && (atoi(genv) == 1 || atoi(genv) == 2)) groups = atoi(genv);
               if (groups > gb_tma_max_groups(prec)) groups = gb_tma_max_groups(prec);
               const int nbuf = groups + 1;
               const long long cap = groups == 2 ? 113 * 1024 : 76 * 1024;
               if (tbt < 1) tbt = 1;
               /* a group is whole warps (its named barrier counts threads in warps) */
               while (tbt > 1 && (tbt >> 1) >= v[0].n && (tbt >> 1) * T >= 32) tbt >>= 1;
               sm2 = (long long)nbuf * tbt * tma_sms((int)nfft) * csize(prec);
               while (tbt > 1 && sm2 > cap && (tbt >> 1) * T >= 32) {
                    tbt >>= 1;
                    sm2 = (long long)nbuf * tbt * tma_sms((int)nfft) * csize(prec);
               }
               if (ok && sm2 <= smax) {
                    P->variant = GB_VAR_TMA;
                    P->groups = groups;
                    P->tb = tbt;
                    P->threads = tbt * T;
                    P->smem = (int)sm2;
                    P->load_mode = GB_MOVE_DIRECT;
                    P->store_mode = GB_MOVE_DIRECT;
               }
          }
     } else {
          int k, tb;
          long long sm1, L = nfft;
          k = gb_factor_order(nfft, P->rad, cfg_order);
          if (k < 0) return -1;
          P->nrad = k;
          P->variant = GB_VAR_GEN;
          sm1 = 2LL * gb_gen_sms((int)L) * csize(prec);
          if (sm1 > smax) return 1;
          tb = (int)(1024 / nfft); if (tb < 1) tb = 1;
          if (llabs_(is) != 1 || llabs_(os) != 1) { int want = prec == 4 ? 16 : 8; if (tb < want) tb = want; }
          if (tb_hint > 0) tb = tb_hint;
          while (tb > 1 && tb * sm1 > smax) tb >>= 1;
          while (tb > 1 && (tb >> 1) >= v[0].n) tb >>= 1;
          P->tb = tb;
          {
               long long th = ((long long)tb * nfft / 4 + 31) / 32 * 32;
               if (th < 64) th = 64;
               if (th > 512) th = 512;
               P->threads = (int)th;
          }
          P->smem = (int)(tb * sm1);
          P->load_mode = (llabs_(is) != 1 && llabs_(P->vis[0]) <= 2) ? GB_MOVE_COLS : GB_MOVE_ROWS;
          P->store_mode = (llabs_(os) != 1 && llabs_(P->vos[0]) <= 2) ? GB_MOVE_COLS : GB_MOVE_ROWS;
     }
     P->ntiles0 = (v[0].n + P->tb - 1) / P->tb;
     P->nblocks = P->ntiles0;
     for (i = 1; i < nv; ++i) P->nblocks *= v[i].n;
     return 0;
}

/* Fill the device tables a configured pass needs (and the derived shift
 * fields the kernels use instead of divisions). */
static int pass_tables(gb_pass *P)
{
     int prec = P->prec;
     {
          int l = 0;
          while ((1 << l) < P->tb) ++l;
          P->ltb = ((1 << l) == P->tb) ? l : -1;
     }
     if (P->kind == GB_KIND_COPY) return 0;
     P->tw = gb_table_twiddle(prec, P->nfft, P->nfft, 1);
     if (!P->tw) return -1;
     if (P->nfft >= 32 && (P->nfft & (P->nfft - 1)) == 0) {
          P->tw_stage = gb_table_stage_twiddle(prec, P->nfft);
          if (!P->tw_stage) return -1;
     }
     if (P->variant == GB_VAR_GEN && P->nrad > 0 && P->nfft > 1) {
          P->tw_gen = table_gen_stage(prec, P->nfft, P->rad, P->nrad);
          if (!P->tw_gen) return -1;
     }
     if ((P->kind == GB_KIND_R2C || P->kind == GB_KIND_C2R) && P->n % 2 == 0) {
          P->tw_half = gb_table_twiddle(prec, P->n, P->n / 2 + 1, 1);
          if (!P->tw_half) return -1;
     }
     if (P->kind == GB_KIND_RADER) {
          P->perm = gb_table_rader_perm(P->n);
          P->chirp_spec = gb_table_rader_spec(prec, P->n, P->sign);
          if (!P->perm || !P->chirp_spec) return -1;
     }
     if (P->kind == GB_KIND_BLUESTEIN) {
          P->chirp = gb_table_chirp(prec, P->n, P->sign);
          P->chirp_spec = gb_table_chirp_spec(prec, P->n, P->nfft, P->sign);
          if (!P->chirp || !P->chirp_spec) return -1;
     }
     if (P->post_N) {
          long long S = 1;
          int l = 0;
          while (S * S < P->post_N) { S <<= 1; ++l; }
          P->post_S = S;
          P->post_lS = l;
          P->post_lo = gb_table_twiddle(prec, P->post_N, S, 1);
          P->post_hi = gb_table_twiddle(prec, P->post_N, (P->post_N + S - 1) / S, S);
          if (!P->post_lo || !P->post_hi) return -1;
          /* the factor of each thread's first element as one table read per
           * thread, coalesced (register kernels of 16 elements a thread) */
          if (P->nfft >= 256 && (P->nfft & (P->nfft - 1)) == 0 && P->post_N % P->nfft == 0 &&
              P->post_N / 16 <= (1LL << 24)) {
               P->post_rows_v = P->post_N / P->nfft;
               P->post_rows = table_post_rows(prec, P->post_N, P->nfft / 16, P->post_rows_v);
               if (!P->post_rows) return -1;
          }
     }
     return 0;
}

int gb_pass_tables(gb_pass *P) { return pass_tables(P); }

int gb_config_pass(gb_pass *P, int prec, int kind, long long n, int sign, long long is, long long os, int nv,
                   const gb_dim *v)
{
     if (nv > GB_MAXV) return -1;
     return config_pass(P, prec, kind, n, sign, is, os, nv, v, 0, 0);
}

/* ------------------------------------------------------------ plan building */
typedef struct {
     gb_plan *p;
     int err;
} builder;

static gb_step *new_step(builder *b)
{
     gb_step *s;
     if (b->p->nstep >= GB_MAXPASS) { gb_set_error("too many passes"); b->err = 1; return 0; }
     s = &b->p->step[b->p->nstep++];
     memset(s, 0, sizeof *s);
     return s;
}

static void count_ops(gb_plan *p, const gb_pass *P, long long howmany)
{
     double n = P->nfft, lg = n > 1 ? __builtin_log2(n) : 0;
     double per = 5.0 * n * lg;   /* the 5 N log2 N convention (libbench2/mflops.c:21-27) */
     if (P->kind == GB_KIND_BLUESTEIN) per = 2 * per + 12.0 * n;
     p->add += 0.6 * per * howmany;
     p->mul += 0.4 * per * howmany;
}

/* The split-FP16 tensor-core form (FFTW_GB300_TENSOR_CORE): f32 c2c passes of
 * 256 to 4096 points (a power of two), 256 threads (one radix-16 butterfly
 * each).  Each GEMM stage carries the hi + lo split's error (about four
 * times a FP32 radix-16 stage's), so a plan takes the form for at most
 * GB_TC_MAX_STAGES GEMM stages in all (measured: 4096 with 3 stages 6.5e-7,
 * 65536 and 2^20 with 4 stages 8.7e-7 and 9.1e-7, 512^3 with 6 stages
 * 1.3e-6 rel L2, beyond the float bound of 1e-6); later passes of a plan
 * over that budget stay in the FP32 form. */
#define GB_TC_MAX_STAGES 4
static void use_tensor_cores(gb_plan *p, gb_pass *P)
{
     int i, stages, lm, ctas;
     if (P->kind != GB_KIND_C2C || P->prec != 4 || P->nfft < 256 || P->nfft > 4096 || (P->nfft & (P->nfft - 1)))
          return;
     stages = P->nfft == 4096 ? 3 : 2;
     if (p->tc_stages + stages > GB_TC_MAX_STAGES) return;
     p->tc_stages += stages;
     lm = (P->is == 1 || llabs_(P->vis[0]) != 1) ? GB_MOVE_ROWS : GB_MOVE_COLS;
     /* CTAs per SM of the build: 2 for unit-stride rows (their next tile is
      * bulk-copied into a second buffer), 3 for the rest (plain loads, no
      * second buffer; measured: c2c 65536 four-step 4.49 -> 3.54 ms, rows of
      * 4096 1.89 with two against 2.05 ms with three); FFTW_GB300_TC_CTAS=2|3
      * sets it */
     {
          const char *e = getenv("FFTW_GB300_TC_CTAS");
          ctas = (e && (atoi(e) == 2 || atoi(e) == 3)) ? atoi(e) : (lm == GB_MOVE_ROWS && P->is == 1) ? 2 : 3;
     }
     if (gb_tc_smem(P->nfft, ctas) > smem_max()) return;
     P->load_mode = lm;
     P->groups = ctas;
     P->variant = GB_VAR_TC;
     P->tb = 256 / (P->nfft / 16);
     P->threads = 256;
     P->smem = gb_tc_smem(P->nfft, P->groups);
     P->store_mode = (P->os == 1) ? GB_MOVE_DIRECT : (llabs_(P->vos[0]) == 1) ? GB_MOVE_COLS : GB_MOVE_ROWS;
     P->ntiles0 = (P->vn[0] + P->tb - 1) / P->tb;
     P->nblocks = P->ntiles0;
     for (i = 1; i < P->nv; ++i) P->nblocks *= P->vn[i];
}

/* Prime lengths: Rader (dft/rader.c) when n-1 factors into radices <= 13
 * and the wisdom or FFTW_GB300_PRIME=rader asks for it; Bluestein
 * otherwise (one CTA, power-of-two convolution, register stages). */
static int use_rader(int prec, long long n, const gb_wisdom_entry *w)
{
     int rad[GB_MAXRAD];
     const char *e = getenv("FFTW_GB300_PRIME");
     if (n < 3 || gb_factor(n - 1, rad) < 0) return 0;
     {
          long long d;
          for (d = 2; d * d <= n; ++d) if (n % d == 0) return 0;
     }
     if (2LL * n * csize(prec) > smem_max()) return 0;
     if (w) return w->variant == GB_KIND_RADER;
     return e && !strcmp(e, "rader");
}

/* 1 when a c2c of length n runs only as the multi-pass convolution, which
 * needs scratch of its own: a prime factor > 13 and too long for Rader or
 * Bluestein in one CTA */
static int c2c_needs_conv(int prec, long long n)
{
     gb_pass t;
     gb_dim one = {1, 0, 0};
     if (config_pass(&t, prec, GB_KIND_C2C, n, -1, 1, 1, 1, &one, 0, 0) >= 0) return 0;
     if (use_rader(prec, n, 0) && config_pass(&t, prec, GB_KIND_RADER, n, -1, 1, 1, 1, &one, 0, 0) == 0) return 0;
     return config_pass(&t, prec, GB_KIND_BLUESTEIN, n, -1, 1, 1, 1, &one, 0, 0) != 0;
}

/* Adds the steps of one batched 1D transform: length n along (is, os), batch
 * dims v (count nv), from buffer src to dst.  Chooses single-CTA kernels,
 * the in-CTA Bluestein, or the two-pass four-step decomposition. */
static void need_scratch(gb_plan *p, int buf, size_t bytes)
{
     if (buf == GB_BUF_SCRATCH && bytes > p->scratch_bytes) p->scratch_bytes = bytes;
     if (buf == GB_BUF_SCRATCH2 && bytes > p->scratch2_bytes) p->scratch2_bytes = bytes;
}

/* An element-wise pass over nv vector dims (in/out strides), length L per
 * transform as the mode defines it. */
static gb_step *add_pointwise(builder *b, int pw, long long n, long long nfft, int sign, long long is, long long os,
                              int nv, const gb_dim *v, int src, int dst)
{
     gb_plan *p = b->p;
     int prec = p->prb.prec, i;
     long long L = (pw == GB_PW_HC2C_POST) ? nfft + 1 : (pw == GB_PW_CHIRP_OUT || pw == GB_PW_CHIRP_OUT_REAL) ? n
                 : (pw == GB_PW_HALF_COPY || pw == GB_PW_CHIRP_OUT_HALF) ? n / 2 + 1 : nfft;
     gb_step *s = new_step(b);
     gb_pass *P;
     if (!s) return 0;
     if (nv > GB_MAXV) { gb_set_error("element-wise pass with too many vector dims"); b->err = 1; return 0; }
     s->src = src; s->dst = dst;
     P = &s->pass;
     memset(P, 0, sizeof *P);
     P->ltb = -1;
     P->kind = GB_KIND_POINTWISE; P->pw = pw; P->prec = prec; P->sign = sign;
     P->n = (int)n; P->nfft = (int)nfft; P->variant = GB_VAR_GEN;
     P->tb = 1; P->threads = 256; P->smem = 0;
     P->is = is; P->os = os;
     P->nv = nv > 0 ? nv : 1;
     if (nv == 0) { P->vn[0] = 1; P->vis[0] = 0; P->vos[0] = 0; }
     for (i = 0; i < nv; ++i) { P->vn[i] = v[i].n; P->vis[i] = v[i].is; P->vos[i] = v[i].os; }
     P->ntiles0 = P->vn[0];
     P->pw_chunks = (L + 4095) / 4096;
     P->nblocks = P->pw_chunks;
     for (i = 0; i < P->nv; ++i) P->nblocks *= P->vn[i];
     if (pw == GB_PW_PROMOTE || pw == GB_PW_HALF_COPY || pw == GB_PW_HERM_EXT || pw == GB_PW_REAL_PART) {
          /* no tables */
     } else if (pw == GB_PW_HC2C_POST || pw == GB_PW_HC2C_PRE) {
          P->tw_half = gb_table_twiddle(prec, 2 * nfft, nfft + 1, 1);
          if (!P->tw_half) { b->err = 1; return 0; }
     } else {
          P->chirp = gb_table_chirp(prec, n, sign);
          if (pw == GB_PW_SPEC_MUL) P->chirp_spec = gb_table_chirp_spec(prec, n, nfft, sign);
          if (!P->chirp || (pw == GB_PW_SPEC_MUL && !P->chirp_spec)) { b->err = 1; return 0; }
     }
     return s;
}

static void add_1d_mid(builder *b, int kind, long long n, int sign, long long is, long long os,
                       int nv, const gb_dim *v_in, int src, int dst, int mid);

/* An f32 r2c / c2r of even n whose half length M is a power of two of
 * 256..4096 that the multi-pass route can take (unit real stride, even
 * vector strides, caller arrays on both sides) and whose GEMM stages fit the
 * plan's tensor-core budget: run it as the half-length c2c in the
 * tensor-core form plus the hc2c pass (rdft/ct-hc2c.c:31-83). */
static int tc_split_real(const gb_plan *p, int kind, long long n, long long is, long long os, int nvk,
                         const gb_dim *v, int src, int dst)
{
     const long long M = n / 2;
     int i;
     if ((kind != GB_KIND_R2C && kind != GB_KIND_C2R) || p->prb.prec != 4 || n % 2) return 0;
     if (M < 256 || M > 4096 || (M & (M - 1))) return 0;
     if (p->tc_stages + (M == 4096 ? 3 : 2) > GB_TC_MAX_STAGES) return 0;
     /* the route's own intermediate is the first scratch; an r2c may write
      * the second (the padded rows of a 2D r2c's first pass), the c2c of M
      * being one pass that needs no intermediate of its own */
     if (src == GB_BUF_SCRATCH || dst == GB_BUF_SCRATCH || src == GB_BUF_SCRATCH2) return 0;
     if (dst == GB_BUF_SCRATCH2 && kind != GB_KIND_R2C) return 0;
     if (kind == GB_KIND_R2C ? is != 1 : os != 1) return 0;
     for (i = 0; i < nvk; ++i)
          if ((kind == GB_KIND_R2C ? v[i].is : v[i].os) % 2) return 0;
     return 1;
}

static void add_1d(builder *b, int kind, long long n, int sign, long long is, long long os,
                   int nv, const gb_dim *v_in, int src, int dst)
{
     add_1d_mid(b, kind, n, sign, is, os, nv, v_in, src, dst, GB_BUF_SCRATCH);
}

/* dense layout of a batch: transform length L, vector dims v (outermost
 * first) re-strided contiguously, keeping the caller's strides on one side */
static void dense_dims(const gb_dim *v, int nv, long long L, gb_dim *out, int keep_in)
{
     long long d = L;
     int i;
     for (i = nv - 1; i >= 0; --i) {
          out[i].n = v[i].n;
          out[i].is = keep_in ? v[i].is : d;
          out[i].os = keep_in ? d : v[i].os;
          d *= v[i].n;
     }
}

/* Four-step for an axis whose batch has a unit-stride dimension u (columns
 * of a multi-dimensional array): both passes tile along u, so every tile
 * row is a contiguous run of columns.  Scratch holds [outer][n2][k1][u].
 * Pass A: n1-point transforms at element stride n2*is, twiddle
 * W_n^(n2*k1) indexed by vector dimension 1 (n2); pass B: n2-point
 * transforms at scratch stride n1*nup (nup = nu rounded up to 8), written to
 * k1 + n1*k2.
 * Returns 0 when added, -1 when the layout or lengths do not allow it. */
static int add_fourstep_cols(builder *b, long long n, int sign, long long is, long long os,
                             int nvk, const gb_dim *v, int src, int dst, int mid)
{
     gb_plan *p = b->p;
     int prec = p->prb.prec, i, u = -1, no = 0;
     long long n1 = 0, d, nu, nup, dense, outer = 1;
     gb_dim va[GB_MAXV], vb[GB_MAXV], vo[GB_MAXRANK];
     gb_step *sa, *sb;
     for (i = 0; i < nvk; ++i)
          if (llabs_(v[i].is) == 1 && llabs_(v[i].os) == 1 && v[i].n >= 8) { u = i; break; }
     if (u < 0 || nvk - 1 > GB_MAXV - 2) return -1;
     for (d = 2; d * d <= n; ++d) {
          gb_pass t1, t2;
          gb_dim one = {1, 0, 0};
          if (n % d) continue;
          if (config_pass(&t1, prec, GB_KIND_C2C, d, sign, 1, 1, 1, &one, 0, 0) == 0 &&
              config_pass(&t2, prec, GB_KIND_C2C, n / d, sign, 1, 1, 1, &one, 0, 0) == 0 &&
              t1.variant != GB_VAR_GEN && t2.variant != GB_VAR_GEN)
               n1 = d;
     }
     if (!n1) return -1;
     nu = v[u].n;
     /* the scratch rows hold nup >= nu columns: a multiple of 8 complex
      * values, so the second pass's strides suit tensor-map copies */
     nup = (nu + 7) & ~7LL;
     for (i = 0; i < nvk; ++i) if (i != u) { vo[no++] = v[i]; outer *= v[i].n; }
     need_scratch(p, mid, (size_t)(n * nup * outer) * csize(prec));
     /* pass A */
     va[0].n = nu; va[0].is = v[u].is; va[0].os = 1;
     va[1].n = n / n1; va[1].is = is; va[1].os = n1 * nup;
     dense = n * nup;
     for (i = 0; i < no; ++i) { va[2 + i].n = vo[i].n; va[2 + i].is = vo[i].is; va[2 + i].os = dense; dense *= vo[i].n; }
     sa = new_step(b);
     if (!sa) return -1;
     sa->src = src; sa->dst = mid;
     if (config_pass(&sa->pass, prec, GB_KIND_C2C, n1, sign, (n / n1) * is, nup, 2 + no, va, 0, 1)) { --p->nstep; return -1; }
     sa->pass.post_N = n;
     sa->pass.post_vdim = 1;
     if (p->flags & GB_FLAG_TENSOR_CORE) use_tensor_cores(p, &sa->pass);
     if (pass_tables(&sa->pass)) { b->err = 1; return 0; }
     /* pass B */
     vb[0].n = nu; vb[0].is = 1; vb[0].os = v[u].os;
     vb[1].n = n1; vb[1].is = nup; vb[1].os = os;
     dense = n * nup;
     for (i = 0; i < no; ++i) { vb[2 + i].n = vo[i].n; vb[2 + i].is = dense; vb[2 + i].os = vo[i].os; dense *= vo[i].n; }
     sb = new_step(b);
     if (!sb) return -1;
     sb->src = mid; sb->dst = dst;
     if (config_pass(&sb->pass, prec, GB_KIND_C2C, n / n1, sign, n1 * nup, n1 * os, 2 + no, vb, 0, 1)) {
          p->nstep -= 2;
          return -1;
     }
     if (p->flags & GB_FLAG_TENSOR_CORE) use_tensor_cores(p, &sb->pass);
     if (pass_tables(&sb->pass)) { b->err = 1; return 0; }
     count_ops(p, &sa->pass, outer * nu * (n / n1));
     count_ops(p, &sb->pass, outer * nu * n1);
     return 0;
}

static void add_1d_mid(builder *b, int kind, long long n, int sign, long long is, long long os,
                       int nv, const gb_dim *v_in, int src, int dst, int mid)
{
     gb_plan *p = b->p;
     int prec = p->prb.prec, rc, i;
     gb_step *s;
     gb_dim v[GB_MAXRANK + 2];
     long long howmany = 1;
     const gb_wisdom_entry *w = 0;
     int nvk;
     if (b->err) return;
     for (i = 0; i < nv; ++i) v[i] = v_in[i];
     nvk = gb_canon_vec(v, nv);
     for (i = 0; i < nvk; ++i) howmany *= v[i].n;

     if (n == 1 && kind == GB_KIND_C2C) {
          /* size-1 DFT: identity copy (nothing to do in place) */
          if (src == dst) return;
          s = new_step(b);
          if (!s) return;
          {
               gb_dim vv[GB_MAXRANK + 2];
               int k = nvk;
               for (i = 0; i < nvk; ++i) vv[i] = v[i];
               if (k > GB_MAXV) {
                    s->nloop = k - GB_MAXV;
                    for (i = 0; i < s->nloop; ++i) s->loop[i] = vv[i];
                    config_pass(&s->pass, prec, GB_KIND_COPY, 1, sign, is, os, GB_MAXV, vv + s->nloop, 0, 0);
               } else config_pass(&s->pass, prec, GB_KIND_COPY, 1, sign, is, os, k, vv, 0, 0);
          }
          s->src = src; s->dst = dst;
          return;
     }

     if (kind == GB_KIND_C2C) {
          char key[128];
          snprintf(key, sizeof key, "c2c p%d n%lld", prec, n);
          w = gb_wisdom_lookup(key);
     }

     s = new_step(b);
     if (!s) return;
     s->src = src; s->dst = dst;
     if (nvk > GB_MAXV) {
          s->nloop = nvk - GB_MAXV;
          for (i = 0; i < s->nloop; ++i) s->loop[i] = v[i];
     }
     cfg_no_tma = (w && w->variant == GB_VAR_REG);
     cfg_groups = w ? w->groups : 0;
     cfg_order = w ? w->order : 0;
     rc = config_pass(&s->pass, prec, kind, n, sign, is, os, nvk - s->nloop, v + s->nloop,
                      (w && w->tb > 0) ? w->tb : 0, 0);
     cfg_no_tma = 0;
     cfg_groups = 0;
     cfg_order = 0;
     if (rc == 0 && kind == GB_KIND_C2C && !(w && w->tb > 0) && src != mid && dst != mid &&
         (s->pass.load_mode == GB_MOVE_COLS || s->pass.store_mode == GB_MOVE_COLS) &&
         s->pass.tb * csize(prec) < 32 && s->nloop == 0) {
          /* a column pass whose tile rows would be narrower than one 32-byte
           * sector: two passes with wide column tiles move fewer wasted bytes */
          gb_step keep = *s;
          --p->nstep;
          if (add_fourstep_cols(b, n, sign, is, os, nvk, v, src, dst, mid) == 0) return;
          if (b->err) return;
          p->step[p->nstep++] = keep;
          s = &p->step[p->nstep - 1];
     }
     if (rc == 0 && (p->flags & GB_FLAG_TENSOR_CORE)) use_tensor_cores(p, &s->pass);
     /* the tensor-core form of an even r2c / c2r whose half length is a
      * power of two the tensor-core kernel takes: the half-length complex
      * FFT as its own pass (in the tensor-core form) and the hc2c post- or
      * pre-pass beside it, through the multi-pass route below */
     if (rc == 0 && (p->flags & GB_FLAG_TENSOR_CORE) && tc_split_real(p, kind, n, is, os, nvk, v, src, dst)) rc = 1;
     if (rc == 0) {
          if (pass_tables(&s->pass)) { b->err = 1; return; }
          count_ops(p, &s->pass, howmany);
          return;
     }
     --p->nstep;   /* the single-pass attempt is replaced below */

     if (rc < 0 && kind == GB_KIND_C2C && use_rader(prec, n, w)) {
          /* prime with a smooth n-1: Rader in one CTA */
          s = new_step(b);
          s->src = src; s->dst = dst;
          if (nvk > GB_MAXV) { s->nloop = nvk - GB_MAXV; for (i = 0; i < s->nloop; ++i) s->loop[i] = v[i]; }
          rc = config_pass(&s->pass, prec, GB_KIND_RADER, n, sign, is, os, nvk - s->nloop, v + s->nloop, 0, 0);
          if (rc == 0) {
               if (pass_tables(&s->pass)) { b->err = 1; return; }
               count_ops(p, &s->pass, howmany);
               return;
          }
          --p->nstep;
     }
     if (rc < 0 && kind == GB_KIND_C2C) {
          /* length with a prime factor > 13: Bluestein in one CTA */
          s = new_step(b);
          s->src = src; s->dst = dst;
          if (nvk > GB_MAXV) { s->nloop = nvk - GB_MAXV; for (i = 0; i < s->nloop; ++i) s->loop[i] = v[i]; }
          rc = config_pass(&s->pass, prec, GB_KIND_BLUESTEIN, n, sign, is, os, nvk - s->nloop, v + s->nloop, 0, 0);
          if (rc == 0) {
               if (pass_tables(&s->pass)) { b->err = 1; return; }
               count_ops(p, &s->pass, howmany);
               return;
          }
          --p->nstep;
          {
               /* multi-pass Bluestein: chirp multiply into scratch (zero-
                * padded to nb), FFT(nb), spectrum multiply, inverse FFT(nb),
                * chirp multiply into dst (dft/bluestein.c:82-128) */
               long long nb = 1, hm = howmany;
               gb_dim vin[GB_MAXRANK + 2], vmid[GB_MAXRANK + 2], vout[GB_MAXRANK + 2];
               while (nb < 2 * n - 1) nb <<= 1;
               if (src == GB_BUF_SCRATCH || dst == GB_BUF_SCRATCH) {
                    gb_set_error("length %lld: nested multi-pass convolution", n);
                    b->err = 1;
                    return;
               }
               dense_dims(v, nvk, nb, vin, 1);     /* caller's input strides -> dense nb */
               dense_dims(v, nvk, nb, vmid, 0);
               for (i = 0; i < nvk; ++i) vmid[i].is = vmid[i].os = vin[i].os;
               dense_dims(v, nvk, nb, vout, 0);    /* dense nb -> caller's output strides */
               need_scratch(p, GB_BUF_SCRATCH, (size_t)(nb * hm) * csize(prec));
               add_pointwise(b, GB_PW_CHIRP_IN, n, nb, sign, is, 1, nvk, vin, src, GB_BUF_SCRATCH);
               add_1d_mid(b, GB_KIND_C2C, nb, -1, 1, 1, nvk, vmid, GB_BUF_SCRATCH, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
               add_pointwise(b, GB_PW_SPEC_MUL, n, nb, sign, 1, 1, nvk, vmid, GB_BUF_SCRATCH, GB_BUF_SCRATCH);
               add_1d_mid(b, GB_KIND_C2C, nb, 1, 1, 1, nvk, vmid, GB_BUF_SCRATCH, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
               add_pointwise(b, GB_PW_CHIRP_OUT, n, nb, sign, 1, os, nvk, vout, GB_BUF_SCRATCH, dst);
               return;
          }
     }

     if (kind == GB_KIND_C2C && rc == 1) {
          /* four-step: n = n1 * n2, pass A over n1 (stride n2) into scratch
           * laid out [v][n2][k1] with the W_n^(n2 k1) twiddle, pass B over n2
           * from scratch into dst at k1 + n1*k2. */
          long long n1 = 0, n2, d, best = 0, sz;
          gb_dim va[GB_MAXRANK + 3], vb[GB_MAXRANK + 3];
          int na = 0, nb = 0, r1, r2;
          for (d = 2; d * d <= n; ++d) {   /* the most balanced split whose factors fit */
               if (n % d) continue;
               {
                    gb_pass t1, t2;
                    gb_dim one = {1, 0, 0};
                    if (config_pass(&t1, prec, GB_KIND_C2C, d, sign, 1, 1, 1, &one, 0, 0) == 0 &&
                        config_pass(&t2, prec, GB_KIND_C2C, n / d, sign, 1, 1, 1, &one, 0, 0) == 0)
                         best = d;
               }
          }
          if (!best) {
               gb_set_error("length %lld is not supported (no two-pass split)", n);
               b->err = 1;
               return;
          }
          n1 = best; n2 = n / n1;
          if (w && w->n1 > 0 && n % w->n1 == 0) { n1 = w->n1; n2 = n / n1; }
          sz = n * howmany;
          need_scratch(p, mid, (size_t)sz * csize(prec));
          /* pass A: transform over n1 with element stride n2*is; dim0 = n2 */
          va[na].n = n2; va[na].is = is; va[na].os = n1; ++na;
          {
               long long dense = n;
               for (i = nvk - 1; i >= 0; --i) {
                    va[na].n = v[i].n; va[na].is = v[i].is; va[na].os = dense; ++na;
                    dense *= v[i].n;
               }
          }
          s = new_step(b);
          if (!s) return;
          s->src = src; s->dst = mid;
          if (na > GB_MAXV) { gb_set_error("four-step with too many vector dims"); b->err = 1; return; }
          /* dim 0 stays n2: the twiddle W_n^(n2 k1) indexes it */
          r1 = config_pass(&s->pass, prec, GB_KIND_C2C, n1, sign, n2 * is, 1, na, va, 0, 1);
          if (r1 == 0 && (p->flags & GB_FLAG_TENSOR_CORE)) use_tensor_cores(p, &s->pass);
          s->pass.post_N = n;
          if (r1) { if (!b->err) gb_set_error("four-step pass A config failed"); b->err = 1; return; }
          if (pass_tables(&s->pass)) { b->err = 1; return; }   /* the table's own message stands */
          count_ops(p, &s->pass, howmany * n2);
          /* pass B: transform over n2 (scratch stride n1), dim0 = k1 */
          vb[nb].n = n1; vb[nb].is = 1; vb[nb].os = os; ++nb;
          {
               long long dense = n;
               for (i = nvk - 1; i >= 0; --i) {
                    vb[nb].n = v[i].n; vb[nb].is = dense; vb[nb].os = v[i].os; ++nb;
                    dense *= v[i].n;
               }
          }
          s = new_step(b);
          if (!s) return;
          s->src = mid; s->dst = dst;
          if (nb > GB_MAXV) { gb_set_error("four-step with too many vector dims"); b->err = 1; return; }
          r2 = config_pass(&s->pass, prec, GB_KIND_C2C, n2, sign, n1, n1 * os, nb, vb, 0, 1);
          if (r2 == 0 && (p->flags & GB_FLAG_TENSOR_CORE)) use_tensor_cores(p, &s->pass);
          if (r2) { if (!b->err) gb_set_error("four-step pass B config failed"); b->err = 1; return; }
          if (pass_tables(&s->pass)) { b->err = 1; return; }
          count_ops(p, &s->pass, howmany * n1);
          return;
     }
     if ((kind == GB_KIND_R2C || kind == GB_KIND_C2R) && rc != 0 && n % 2 == 0) {
          /* even length beyond one CTA (or with a prime factor beyond the
           * stage kernels): the half-length complex FFT runs as
           * its own (multi-pass) c2c on the real array viewed as pairs, and
           * the hc2c post-pass (r2c) or pre-pass (c2r) as an element-wise
           * pass through scratch (rdft/ct-hc2c.c:31-83) */
          long long M = n / 2;
          gb_dim vp[GB_MAXRANK + 2], vd[GB_MAXRANK + 2];
          int ok = 1;
          if (kind == GB_KIND_R2C) {
               if (is != 1) ok = 0;
               for (i = 0; i < nvk; ++i) if (v[i].is % 2) ok = 0;
          } else {
               if (os != 1) ok = 0;
               for (i = 0; i < nvk; ++i) if (v[i].os % 2) ok = 0;
          }
          if (!ok || src == GB_BUF_SCRATCH || dst == GB_BUF_SCRATCH || c2c_needs_conv(prec, M)) goto conv;
          need_scratch(p, GB_BUF_SCRATCH, (size_t)(M * howmany) * csize(prec));
          if (kind == GB_KIND_R2C) {
               for (i = 0; i < nvk; ++i) { vp[i].n = v[i].n; vp[i].is = v[i].is / 2; }
               dense_dims(v, nvk, M, vd, 0);
               for (i = 0; i < nvk; ++i) vp[i].os = vd[i].is;      /* dense M in scratch */
               add_1d_mid(b, GB_KIND_C2C, M, -1, 1, 1, nvk, vp, src, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
               for (i = 0; i < nvk; ++i) { vd[i].is = vp[i].os; vd[i].os = v[i].os; }
               add_pointwise(b, GB_PW_HC2C_POST, n, M, -1, 1, os, nvk, vd, GB_BUF_SCRATCH, dst);
          } else {
               dense_dims(v, nvk, M, vd, 1);                      /* caller's input -> dense M */
               add_pointwise(b, GB_PW_HC2C_PRE, n, M, 1, is, 1, nvk, vd, src, GB_BUF_SCRATCH);
               for (i = 0; i < nvk; ++i) { vp[i].n = v[i].n; vp[i].is = vd[i].os; vp[i].os = v[i].os / 2; }
               add_1d_mid(b, GB_KIND_C2C, M, 1, 1, 1, nvk, vp, GB_BUF_SCRATCH, dst, GB_BUF_SCRATCH2);
          }
          return;
     }
     if ((kind == GB_KIND_R2C || kind == GB_KIND_C2R) && n % 2 == 1 && n <= (prec == 4 ? 4096 : 2048) &&
         src != GB_BUF_SCRATCH && dst != GB_BUF_SCRATCH && src != GB_BUF_SCRATCH2 && dst != GB_BUF_SCRATCH2) {
          /* odd length with a prime factor beyond the stage kernels: the real
           * array as n complex values with zero imaginary parts, one c2c of
           * length n (Bluestein or Rader in one CTA) in scratch, then the half
           * spectrum (r2c); c2r extends the half spectrum by Hermitian
           * symmetry, runs the backward c2c and keeps the real parts */
          gb_dim vi[GB_MAXRANK + 2], vd[GB_MAXRANK + 2], vo[GB_MAXRANK + 2];
          long long dense = n;
          for (i = nvk - 1; i >= 0; --i) {
               vd[i].n = v[i].n; vd[i].is = dense; vd[i].os = dense;
               vi[i].n = v[i].n; vi[i].is = v[i].is; vi[i].os = dense;
               vo[i].n = v[i].n; vo[i].is = dense; vo[i].os = v[i].os;
               dense *= v[i].n;
          }
          need_scratch(p, GB_BUF_SCRATCH, (size_t)dense * csize(prec));
          if (kind == GB_KIND_R2C) {
               if (!add_pointwise(b, GB_PW_PROMOTE, n, n, -1, is, 1, nvk, vi, src, GB_BUF_SCRATCH)) return;
               add_1d_mid(b, GB_KIND_C2C, n, -1, 1, 1, nvk, vd, GB_BUF_SCRATCH, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
               if (!b->err) add_pointwise(b, GB_PW_HALF_COPY, n, n, -1, 1, os, nvk, vo, GB_BUF_SCRATCH, dst);
          } else {
               if (!add_pointwise(b, GB_PW_HERM_EXT, n, n, 1, is, 1, nvk, vi, src, GB_BUF_SCRATCH)) return;
               add_1d_mid(b, GB_KIND_C2C, n, 1, 1, 1, nvk, vd, GB_BUF_SCRATCH, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
               if (!b->err) add_pointwise(b, GB_PW_REAL_PART, n, n, 1, 1, os, nvk, vo, GB_BUF_SCRATCH, dst);
          }
          return;
     }
conv:
     if ((kind == GB_KIND_R2C || kind == GB_KIND_C2R) && src != GB_BUF_SCRATCH && dst != GB_BUF_SCRATCH &&
         src != GB_BUF_SCRATCH2 && dst != GB_BUF_SCRATCH2) {
          /* a real length none of the paths above takes (odd beyond one CTA
           * with a prime factor > 13, even with a half length that needs its
           * own convolution, or non-unit real strides beyond one CTA):
           * Bluestein's convolution read straight from the real array (r2c)
           * or from the half spectrum extended by Hermitian symmetry (c2r),
           * written back as the half spectrum or the real parts
           * (dft/bluestein.c:82-128) */
          long long nb = 1;
          gb_dim vin[GB_MAXRANK + 2], vmid[GB_MAXRANK + 2], vout[GB_MAXRANK + 2];
          while (nb < 2 * n - 1) nb <<= 1;
          dense_dims(v, nvk, nb, vin, 1);
          dense_dims(v, nvk, nb, vmid, 0);
          for (i = 0; i < nvk; ++i) vmid[i].is = vmid[i].os = vin[i].os;
          dense_dims(v, nvk, nb, vout, 0);
          need_scratch(p, GB_BUF_SCRATCH, (size_t)(nb * howmany) * csize(prec));
          if (!add_pointwise(b, kind == GB_KIND_R2C ? GB_PW_CHIRP_IN_REAL : GB_PW_CHIRP_IN_HERM, n, nb, sign, is, 1,
                             nvk, vin, src, GB_BUF_SCRATCH))
               return;
          add_1d_mid(b, GB_KIND_C2C, nb, -1, 1, 1, nvk, vmid, GB_BUF_SCRATCH, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
          if (!b->err) add_pointwise(b, GB_PW_SPEC_MUL, n, nb, sign, 1, 1, nvk, vmid, GB_BUF_SCRATCH, GB_BUF_SCRATCH);
          add_1d_mid(b, GB_KIND_C2C, nb, 1, 1, 1, nvk, vmid, GB_BUF_SCRATCH, GB_BUF_SCRATCH, GB_BUF_SCRATCH2);
          if (!b->err)
               add_pointwise(b, kind == GB_KIND_R2C ? GB_PW_CHIRP_OUT_HALF : GB_PW_CHIRP_OUT_REAL, n, nb, sign, 1, os,
                             nvk, vout, GB_BUF_SCRATCH, dst);
          return;
     }
     gb_set_error("length %lld is not supported for this transform kind", n);
     b->err = 1;
}

static void describe(gb_plan *p)
{
     int i, off = 0;
     const char *kn[] = {"dft", "rdft2-r2c", "rdft2-c2r"};
     off += snprintf(p->desc + off, sizeof p->desc - off, "(gb300-%s-%s",
                     kn[p->prb.kind], p->prb.prec == 4 ? "f32" : "f64");
     for (i = 0; i < p->nstep && off < (int)sizeof p->desc - 64; ++i) {
          const gb_pass *P = &p->step[i].pass;
          static const char *kk[] = {"c2c", "r2c", "c2r", "bluestein", "copy", "rader", "pointwise", "dct2"};
          static const char *mv[] = {"direct", "rows", "cols"};
          static const char *pw[] = {"hc2c-post", "hc2c-pre", "chirp-in", "spec-mul", "chirp-out", "promote",
                                     "half-copy", "herm-ext", "real-part", "chirp-in-real", "chirp-in-herm",
                                     "chirp-out-half", "chirp-out-real"};
          off += snprintf(p->desc + off, sizeof p->desc - off,
                          "\n  (pass %s%s%s n=%d nfft=%d %s%s tb=%d thr=%d smem=%d ld=%s st=%s is=%lld os=%lld v=%lld%s)",
                          kk[P->kind], P->kind == GB_KIND_POINTWISE ? ":" : "",
                          P->kind == GB_KIND_POINTWISE && P->pw >= 0 && P->pw <= GB_PW_CHIRP_OUT_REAL ? pw[P->pw] : "",
                          P->n, P->nfft, P->variant == GB_VAR_REG ? "reg" : P->variant == GB_VAR_TMA ? "reg-tma" :
                          P->variant == GB_VAR_TMA_COLS ? "cols-tma" :
                          P->variant == GB_VAR_TC ? "tc-split-fp16" : "gen",
                          (P->variant == GB_VAR_TMA || P->variant == GB_VAR_TMA_COLS) && P->groups == 2 ? " groups=2"
                          : P->variant == GB_VAR_TC && P->groups == 3                                     ? " ctas=3"
                                                                                                          : "",
                          P->tb,
                          P->threads, P->smem, mv[P->load_mode], mv[P->store_mode], P->is, P->os,
                          P->vn[0], P->post_N ? " +twiddle" : "");
          if (P->variant == GB_VAR_GEN && P->nrad > 0 && off < (int)sizeof p->desc - 64) {
               /* the runtime radix list, before the closing parenthesis */
               int r;
               --off;
               off += snprintf(p->desc + off, sizeof p->desc - off, " rad=");
               for (r = 0; r < P->nrad && off < (int)sizeof p->desc - 8; ++r)
                    off += snprintf(p->desc + off, sizeof p->desc - off, r ? ".%d" : "%d", P->rad[r]);
               off += snprintf(p->desc + off, sizeof p->desc - off, ")");
          }
          if (off >= (int)sizeof p->desc) off = (int)sizeof p->desc - 1;   /* truncated */
     }
     if (off < (int)sizeof p->desc - 1) snprintf(p->desc + off, sizeof p->desc - off, ")");
}

/* Wisdom key of a whole problem (the reference keys wisdom by the md5 of
 * the problem, kernel/planner.c:651-703): kind, precision, direction, every
 * transform and vector dimension with its strides, in-place-ness and the
 * arrays' alignment, folded into a 64-bit FNV-1a hash. */
void gb_problem_key(const gb_problem *prb, char *key, size_t cap)
{
     unsigned long long h = 1469598103934665603ULL;
     long long f[8 + 6 * GB_MAXRANK];
     int k = 0, i, j;
     f[k++] = prb->kind; f[k++] = prb->prec; f[k++] = prb->sign; f[k++] = prb->rank; f[k++] = prb->vrank;
     for (i = 0; i < prb->rank; ++i) { f[k++] = prb->sz[i].n; f[k++] = prb->sz[i].is; f[k++] = prb->sz[i].os; }
     for (i = 0; i < prb->vrank; ++i) { f[k++] = prb->vec[i].n; f[k++] = prb->vec[i].is; f[k++] = prb->vec[i].os; }
     f[k++] = prb->in == prb->out;
     f[k++] = (long long)((size_t)prb->in % 16);
     f[k++] = (long long)((size_t)prb->out % 16);
     for (i = 0; i < k; ++i)
          for (j = 0; j < 8; ++j) {
               h ^= (unsigned long long)(f[i] >> (8 * j)) & 0xffULL;
               h *= 1099511628211ULL;
          }
     snprintf(key, cap, "prob p%d k%d r%d %016llx", prb->prec, prb->kind, prb->rank, h);
}

gb_plan *gb_plan_alloc(void)
{
     gb_plan *p = (gb_plan *)calloc(1, sizeof *p);
     if (!p) return 0;
     p->refcnt = 1;
     pthread_mutex_init(&p->exec_mtx, 0);
     return p;
}

/* Build the steps of a problem.  Returns NULL (with gb_last_error set) when
 * the problem is invalid or not supported. */
gb_plan *gb_mkplan(const gb_problem *prb, unsigned flags)
{
     gb_plan *p;
     builder b;
     int r = prb->rank, a, i;
     if (!gb_dry && !gb_cuda_ready()) {
          gb_set_error("no CUDA device: libfftw3_gb300 runs transforms on the GPU only");
          return 0;
     }
     p = gb_plan_alloc();
     if (!p) {
          gb_set_error("out of host memory");
          return 0;
     }
     p->prb = *prb;
     p->flags = flags;
     b.p = p; b.err = 0;

     if (prb->kind == GB_PROB_DFT) {
          if (r == 0) {
               gb_dim v[GB_MAXRANK];
               int nv = prb->vrank;
               for (i = 0; i < nv; ++i) v[i] = prb->vec[i];
               if (prb->in != prb->out || gb_dry)
                    add_1d(&b, GB_KIND_C2C, 1, prb->sign, 0, 0, nv, v, GB_BUF_IN, GB_BUF_OUT);
          }
          for (a = r - 1; a >= 0 && !b.err; --a) {
               /* axis a; first pass reads the input, later ones work in place on the output */
               int first = (a == r - 1);
               gb_dim v[2 * GB_MAXRANK];
               int nv = 0;
               for (i = 0; i < r; ++i)
                    if (i != a) { v[nv].n = prb->sz[i].n; v[nv].is = first ? prb->sz[i].is : prb->sz[i].os; v[nv].os = prb->sz[i].os; ++nv; }
               for (i = 0; i < prb->vrank; ++i) {
                    v[nv].n = prb->vec[i].n; v[nv].is = first ? prb->vec[i].is : prb->vec[i].os; v[nv].os = prb->vec[i].os; ++nv;
               }
               add_1d(&b, GB_KIND_C2C, prb->sz[a].n, prb->sign, first ? prb->sz[a].is : prb->sz[a].os,
                      prb->sz[a].os, nv, v, first ? GB_BUF_IN : GB_BUF_OUT, GB_BUF_OUT);
          }
     } else if (prb->kind == GB_PROB_R2C) {
          /* last axis r2c (in -> out), then c2c forward over the leading axes in place on out */
          long long nl = prb->sz[r - 1].n;
          gb_dim v[2 * GB_MAXRANK];
          int nv = 0;
          const long long nc = nl / 2 + 1, n0 = prb->sz[0].n;
          if (r == 2 && prb->prec == 4 && prb->vrank <= 1 && prb->sz[1].os == 1 && (prb->sz[0].os & 1) &&
              n0 >= 16 && (n0 & (n0 - 1)) == 0 && nl >= 32 && nl <= 16384 && (nl & (nl - 1)) == 0 &&
              !getenv("FFTW_GB300_NO_TMA")) {
               /* (both lengths powers of two: one r2c pass that needs no scratch of
                * its own, and column passes that use only the first scratch) */
               /* rows of an odd number of complex values (FFTW's n/2+1 layout)
                * cannot be walked by tensor-map copies: the r2c pass writes rows
                * padded to a multiple of 8 complex values into scratch, and the
                * column pass reads them from there with TMA-fed column tiles */
               const long long P = (nc + 7) & ~7LL;
               const long long hm = prb->vrank ? prb->vec[0].n : 1;
               gb_dim vc[2];
               v[0].n = n0; v[0].is = prb->sz[0].is; v[0].os = P;
               nv = 1;
               if (prb->vrank) { v[1].n = hm; v[1].is = prb->vec[0].is; v[1].os = n0 * P; nv = 2; }
               need_scratch(p, GB_BUF_SCRATCH2, (size_t)(n0 * P * hm) * csize(prb->prec));
               add_1d(&b, GB_KIND_R2C, nl, -1, prb->sz[1].is, 1, nv, v, GB_BUF_IN, GB_BUF_SCRATCH2);
               vc[0].n = nc; vc[0].is = 1; vc[0].os = 1;
               if (prb->vrank) { vc[1].n = hm; vc[1].is = n0 * P; vc[1].os = prb->vec[0].os; }
               if (!b.err)
                    add_1d_mid(&b, GB_KIND_C2C, n0, -1, P, prb->sz[0].os, nv, vc, GB_BUF_SCRATCH2, GB_BUF_OUT,
                               GB_BUF_SCRATCH);
               goto built;
          }
          for (i = 0; i < r - 1; ++i) { v[nv] = prb->sz[i]; ++nv; }
          for (i = 0; i < prb->vrank; ++i) v[nv++] = prb->vec[i];
          add_1d(&b, GB_KIND_R2C, nl, -1, prb->sz[r - 1].is, prb->sz[r - 1].os, nv, v, GB_BUF_IN, GB_BUF_OUT);
          for (a = r - 2; a >= 0 && !b.err; --a) {
               nv = 0;
               for (i = 0; i < r; ++i) {
                    if (i == a) continue;
                    v[nv].n = (i == r - 1) ? nl / 2 + 1 : prb->sz[i].n;
                    v[nv].is = prb->sz[i].os; v[nv].os = prb->sz[i].os; ++nv;
               }
               for (i = 0; i < prb->vrank; ++i) { v[nv].n = prb->vec[i].n; v[nv].is = prb->vec[i].os; v[nv].os = prb->vec[i].os; ++nv; }
               add_1d(&b, GB_KIND_C2C, prb->sz[a].n, -1, prb->sz[a].os, prb->sz[a].os, nv, v, GB_BUF_OUT, GB_BUF_OUT);
          }
     } else {
          /* multi-dimensional c2r works in place on its input; like the
           * reference, no input-preserving algorithm exists for it out of
           * place, while an in-place problem overwrites its input anyway
           * (rdft/rank-geq2-rdft2.c:118-124) */
          if (r > 1 && (flags & FFTW_PRESERVE_INPUT) && prb->in != prb->out) {
               gb_set_error("multi-dimensional c2r cannot preserve its input");
               pthread_mutex_destroy(&p->exec_mtx);
               free(p);
               return 0;
          }
          /* c2r: c2c backward over the leading axes in place on the input
           * (the reference destroys the input here, api/plan-many-dft-c2r.c:41-42),
           * then the last axis c2r from in to out */
          long long nl = prb->sz[r - 1].n;
          gb_dim v[2 * GB_MAXRANK];
          int nv;
          for (a = r - 2; a >= 0 && !b.err; --a) {
               nv = 0;
               for (i = 0; i < r; ++i) {
                    if (i == a) continue;
                    v[nv].n = (i == r - 1) ? nl / 2 + 1 : prb->sz[i].n;
                    v[nv].is = prb->sz[i].is; v[nv].os = prb->sz[i].is; ++nv;
               }
               for (i = 0; i < prb->vrank; ++i) { v[nv].n = prb->vec[i].n; v[nv].is = prb->vec[i].is; v[nv].os = prb->vec[i].is; ++nv; }
               add_1d(&b, GB_KIND_C2C, prb->sz[a].n, 1, prb->sz[a].is, prb->sz[a].is, nv, v, GB_BUF_IN, GB_BUF_IN);
          }
          nv = 0;
          for (i = 0; i < r - 1; ++i) v[nv++] = prb->sz[i];
          for (i = 0; i < prb->vrank; ++i) v[nv++] = prb->vec[i];
          add_1d(&b, GB_KIND_C2R, nl, 1, prb->sz[r - 1].is, prb->sz[r - 1].os, nv, v, GB_BUF_IN, GB_BUF_OUT);
     }
built:
     if (b.err) {
          pthread_mutex_destroy(&p->exec_mtx);
          free(p);
          return 0;
     }
     if (p->scratch2_bytes && !gb_dry) {
          if (cudaMalloc(&p->scratch2, p->scratch2_bytes) != cudaSuccess) {
               cudaGetLastError();
               gb_set_error("cudaMalloc(%zu) for plan scratch failed", p->scratch2_bytes);
               pthread_mutex_destroy(&p->exec_mtx);
               free(p);
               return 0;
          }
     }
     if (p->scratch_bytes && !gb_dry) {
          if (cudaMalloc(&p->scratch, p->scratch_bytes) != cudaSuccess) {
               cudaGetLastError();
               gb_set_error("cudaMalloc(%zu) for plan scratch failed", p->scratch_bytes);
               pthread_mutex_destroy(&p->exec_mtx);
               free(p);
               return 0;
          }
     }
     describe(p);
     if (getenv("FFTW_GB300_TRACE")) fprintf(stderr, "[fftw_gb300] plan %s\n", p->desc);
     return p;
}

void gb_destroy(gb_plan *p)
{
     int i, j;
     if (!p) return;
     if (!gb_dry) {
          if (p->scratch) cudaFree(p->scratch);
          if (p->scratch2) cudaFree(p->scratch2);
          if (p->stage_in) cudaFree(p->stage_in);
          if (p->stage_out) cudaFree(p->stage_out);
          for (i = 0; i < 2; ++i) {
               for (j = 0; j < GB_CHUNK_SLOTS; ++j)
                    if (p->chunk_buf[i][j]) cudaFree(p->chunk_buf[i][j]);
               if (p->chunk_stream[i]) cudaStreamDestroy((cudaStream_t)p->chunk_stream[i]);
          }
          for (i = 0; i < 3; ++i)
               for (j = 0; j < GB_CHUNK_SLOTS; ++j)
                    if (p->chunk_ev[i][j]) cudaEventDestroy((cudaEvent_t)p->chunk_ev[i][j]);
     }
     for (i = 0; i < 2; ++i) {
          if (p->chunk_plan[i]) gb_destroy(p->chunk_plan[i]);
          if (p->split_buf[i] && !gb_dry) cudaFree(p->split_buf[i]);
     }
     if (p->split_inner) gb_destroy(p->split_inner);
     if (p->r2r_ax) {
          for (i = 0; i < p->r2r_naxis; ++i) {
               if (p->r2r_ax[i].inner) gb_destroy(p->r2r_ax[i].inner);
               if (p->r2r_ax[i].tw && !gb_dry) cudaFree(p->r2r_ax[i].tw);
          }
          free(p->r2r_ax);
     }
     for (i = 0; i < 2; ++i)
          if (p->r2r_buf[i] && !gb_dry) cudaFree(p->r2r_buf[i]);
     if (p->r2r_mid && !gb_dry) cudaFree(p->r2r_mid);
     pthread_mutex_destroy(&p->exec_mtx);
     free(p);
}
