/*
 * fftwf_gb300_dft_1d_noalloc: a batched single-precision 1D c2c DFT that
 * allocates no device memory.
 *
 * Some callers of this library cannot call cudaMalloc: applications whose
 * device memory is handed out by their own arena or caching allocator under
 * a fixed budget (a library that allocates behind the arena's back breaks
 * the budget, or fails once the device is full), and latency-critical loops
 * in which cudaMalloc / cudaFree would stall on an implicit device-wide
 * synchronisation.  A plan cannot serve them: planning allocates twiddle
 * tables, and a transform too long for one pass allocates scratch.
 *
 * This entry point runs the same two-pass (four-step) transform as a plan
 * for a long 1D length, n = n1 * n2: pass A does n1-point DFTs down the
 * columns of the n1 x n2 view and multiplies by exp(sign 2 pi i j2 k1 / n);
 * pass B does n2-point DFTs of the result and writes k1 + n1 k2.  Its scratch
 * (the n1 x n2 intermediate of every transform) and its twiddle tables live
 * in one file-scope device array of fixed size, compiled into the library,
 * so nothing is allocated when it runs.  The array's size is the limit:
 * n * howmany <= FFTWF_GB300_NOALLOC_MAX_POINTS (2^21 complex floats,
 * 16 MiB), and every GPU the entry point runs on holds the array (16 MiB +
 * 30.75 KiB of status word and twiddle tables) until the process exits.
 *
 * Set-up: the first call on each device, with that device current, looks up
 * the array's device address (cudaGetSymbolAddress), which can load this
 * file's device code on that device.  Make that first call before any
 * stream capture.  Later calls reuse the address.
 *
 * Sharing: every call uses the same array, and the array keeps whatever the
 * last call left in it.  Each call rewrites the twiddle tables for its own
 * n, clears the status word the kernels report to, and pass A writes every
 * scratch element before pass B reads it, so no call depends on what an
 * earlier one left.  Two calls whose work overlaps on the GPU (calls on
 * different streams, or from different host threads, without ordering
 * between them) race on the array and give wrong results.
 */
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdio.h>
#include "fft_kernels.cuh"
#include "gb_types.h"
#include "fftw3_gb300.h"

extern "C" void gb_set_error(const char *fmt, ...);

namespace {

constexpr long long kMaxPoints = FFTWF_GB300_NOALLOC_MAX_POINTS;
constexpr int kStatusWords = 32;     /* 256 bytes: the status word, padded so the tables start aligned */
constexpr int kMinLog = 12, kMaxLog = 21;
constexpr int kMaxDevices = 64;

/* Table entries one call of length 2^L needs: the stage twiddles of n1 and
 * of n2 (the layout the register kernels read), S + ceil(n / S) for the
 * four-step twiddle, with n1 = 2^(L/2), n2 = n / n1 and S the least power
 * of two whose square reaches n (the same split the entry point uses). */
constexpr long long table_words(int L)
{
     return gb::stage_tw_len(1 << (L / 2)) + gb::stage_tw_len(1 << (L - L / 2)) + (1LL << ((L + 1) / 2)) +
            ((1LL << L) + (1LL << ((L + 1) / 2)) - 1) / (1LL << ((L + 1) / 2));
}
constexpr long long max_table_words(int L)
{
     return L > kMaxLog ? 0 : (table_words(L) > max_table_words(L + 1) ? table_words(L) : max_table_words(L + 1));
}
/* 3888 entries (at n = 2^21: 272 + 544 + 2048 + 1024), rounded up to a
 * multiple of 32 so the scratch that follows stays 256-byte aligned */
constexpr int kTableWords = (int)((max_table_words(kMinLog) + 31) / 32 * 32);
static_assert(table_words(21) == 3888 && table_words(20) == 2592,
              "table layout of the four-step split");
static_assert(kTableWords >= max_table_words(kMinLog), "tables must not reach into the scratch region");

}  // namespace

/* [status (256 B)] [stage twiddles of n1] [stage twiddles of n2]
 * [exp(-2 pi i j / n), j < S] [exp(-2 pi i j S / n), j < ceil(n / S)] ...
 * [scratch: n * howmany] */
static __device__ __align__(256) float2 gb_noalloc_scratch[kStatusWords + kTableWords + kMaxPoints];

static_assert(((kStatusWords + kTableWords) * sizeof(float2)) % 256 == 0, "scratch region must stay 256-byte aligned");

/* Stage-table entry j of a power-of-two length N (the layout of
 * gb_pass.tw_stage): its exponent of exp(-2 pi i m / N). */
__device__ long long stage_exponent(int N, int j)
{
     int ns = gb::reg_r0(N);
     while (j >= 4 * ns) {
          j -= 4 * ns;
          ns *= 16;
     }
     const int q = j / ns, k = j - q * ns;
     return ((long long)k * (N / (16 * ns)) << q) % N;
}

/* The four tables of one call, in one launch, each entry exp(-2 pi i m / N)
 * rounded once from FP64 (the same values the planner's tables hold): the
 * stage tables of n1 and n2, then exp(-2 pi i j / n), j < S, and
 * exp(-2 pi i j S / n), j < ceil(n / S). */
__global__ void k_noalloc_tables(float2 *t, int n1, int n2, long long n, long long S)
{
     const long long l1 = gb::stage_tw_len(n1), l2 = gb::stage_tw_len(n2);
     const long long H = (n + S - 1) / S, total = l1 + l2 + S + H;
     for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total;
          j += (long long)gridDim.x * blockDim.x) {
          long long m, N;
          if (j < l1) { m = stage_exponent(n1, (int)j); N = n1; }
          else if (j < l1 + l2) { m = stage_exponent(n2, (int)(j - l1)); N = n2; }
          else if (j < l1 + l2 + S) { m = j - l1 - l2; N = n; }
          else { m = ((j - l1 - l2 - S) * S) % n; N = n; }
          double c, s;
          gb::cexp_fp64(m, N, -1, &c, &s);
          t[j] = make_float2((float)c, (float)s);
     }
}

static float2 *noalloc_ptr[kMaxDevices];
static pthread_mutex_t noalloc_mtx = PTHREAD_MUTEX_INITIALIZER;

/* The device address of the array on the current device, looked up once per
 * device (the first call on a device does this set-up). */
static float2 *noalloc_area(void)
{
     int dev = -1;
     cudaError_t e = cudaGetDevice(&dev);
     if (e != cudaSuccess) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
          return 0;
     }
     if (dev < 0 || dev >= kMaxDevices) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
          return 0;
     }
     float2 *p = __atomic_load_n(&noalloc_ptr[dev], __ATOMIC_ACQUIRE);
     if (p) return p;
     pthread_mutex_lock(&noalloc_mtx);
     p = noalloc_ptr[dev];
     if (!p) {
          void *q = 0;
          e = cudaGetSymbolAddress(&q, gb_noalloc_scratch);
          if (e != cudaSuccess || !q) {
               cudaGetLastError();
               gb_set_error("fftwf_gb300_dft_1d_noalloc: cudaGetSymbolAddress of the scratch array: %s",
                            cudaGetErrorString(e));
          } else {
               p = (float2 *)q;
               __atomic_store_n(&noalloc_ptr[dev], p, __ATOMIC_RELEASE);
          }
     }
     pthread_mutex_unlock(&noalloc_mtx);
     return p;
}

/* One register-kernel pass over column tiles: tb adjacent transforms per CTA
 * (at most 256 threads), the tile dimension being vector dimension 0. */
static void noalloc_pass(gb_pass *P, int nfft, int sign, long long is, long long os, long long vn0, long long vis0,
                         long long vos0, long long howmany, long long dist, const float2 *tw)
{
     const int E = nfft < 16 ? nfft : 16, T = nfft / E;
     int tb = 256 / T, l = 0;
     if (tb < 1) tb = 1;
     while (tb > 1 && (tb >> 1) >= vn0) tb >>= 1;
     while ((1 << l) < tb) ++l;
     memset(P, 0, sizeof *P);
     P->kind = GB_KIND_C2C;
     P->prec = 4;
     P->sign = sign;
     P->n = nfft;
     P->nfft = nfft;
     P->variant = GB_VAR_REG;
     P->tb = tb;
     P->ltb = l;
     P->threads = tb * T;
     P->smem = tb * gb_reg_sms(nfft) * (int)sizeof(float2);
     P->load_mode = GB_MOVE_COLS;
     P->store_mode = os == 1 ? (T >= 32 ? GB_MOVE_DIRECT : GB_MOVE_ROWS) : GB_MOVE_COLS;
     P->is = is;
     P->os = os;
     P->nv = 2;
     P->vn[0] = vn0; P->vis[0] = vis0; P->vos[0] = vos0;
     P->vn[1] = howmany; P->vis[1] = dist; P->vos[1] = dist;
     P->ntiles0 = (vn0 + tb - 1) / tb;
     P->nblocks = P->ntiles0 * howmany;
     P->tw = tw;        /* (the register kernel reads only the stage table) */
     P->tw_stage = tw;
}

extern "C" int fftwf_gb300_dft_1d_noalloc(int n, int howmany, const fftwf_complex *in, fftwf_complex *out, int sign,
                                          void *cuda_stream)
{
     int L = 0;
     while (L < 31 && (1 << L) < n) ++L;
     if (n <= 0 || (1 << L) != n || L < kMinLog || L > kMaxLog) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: n = %d must be a power of two from 2^%d to 2^%d", n, kMinLog,
                       kMaxLog);
          return -1;
     }
     if (howmany < 1 || (long long)n * howmany > kMaxPoints) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: n * howmany = %lld exceeds the fixed scratch of %lld complex "
                       "points (FFTWF_GB300_NOALLOC_MAX_POINTS)",
                       (long long)n * howmany, kMaxPoints);
          return -1;
     }
     if (sign != -1 && sign != 1) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: sign must be FFTW_FORWARD (-1) or FFTW_BACKWARD (+1)");
          return -1;
     }
     if (!in || !out) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: null array");
          return -1;
     }
     float2 *area = noalloc_area();
     if (!area) return -1;

     cudaStream_t st = (cudaStream_t)cuda_stream;
     const long long n1 = 1LL << (L / 2), n2 = (long long)n / n1;
     long long S = 1;
     int lS = 0;
     while (S * S < n) { S <<= 1; ++lS; }
     const long long l1 = gb::stage_tw_len((int)n1), l2 = gb::stage_tw_len((int)n2);
     if (l1 + l2 + S + (n + S - 1) / S > kTableWords) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: internal: tables of n = %d exceed the fixed table region", n);
          return -1;
     }
     float2 *status = area, *tw1 = area + kStatusWords, *tw2 = tw1 + l1, *lo = tw2 + l2, *hi = lo + S;
     float2 *mid = area + kStatusWords + kTableWords;

     cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), st);
     if (e == cudaSuccess) {
          const long long total = l1 + l2 + S + (n + S - 1) / S;
          k_noalloc_tables<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(tw1, (int)n1, (int)n2, n, S);
          e = cudaGetLastError();
     }
     if (e != cudaSuccess) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: table set-up: %s", cudaGetErrorString(e));
          return -1;
     }

     gb_pass A, B;
     /* pass A: n1 points at stride n2; tiles run along j2 (unit stride);
      * writes k1 contiguous, j2 at stride n1; twiddle index j2 * k1 */
     noalloc_pass(&A, (int)n1, sign, n2, 1, n2, 1, n1, howmany, n, tw1);
     A.post_N = n;
     A.post_S = S;
     A.post_lS = lS;
     A.post_lo = lo;
     A.post_hi = hi;
     A.status = (int *)status;
     /* pass B: n2 points at stride n1 over the scratch, written to k1 + n1 k2 */
     noalloc_pass(&B, (int)n2, sign, n1, n1, n1, 1, 1, howmany, n, tw2);
     B.status = (int *)status;
     if (gb_launch_pass(&A, in, mid, cuda_stream) || gb_launch_pass(&B, mid, out, cuda_stream)) {
          gb_set_error("fftwf_gb300_dft_1d_noalloc: %s", gb_last_cuda_error());
          return -1;
     }
     return 0;
}
