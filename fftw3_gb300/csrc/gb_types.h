/*
 * Descriptors shared by the host planner (C) and the device kernels (CUDA).
 *
 * A plan compiles to a list of passes.  One pass is one kernel launch that
 * runs a batch of 1D transforms of one length, each read once from HBM and
 * written once, with the whole transform resident in shared memory/registers.
 * The batch is described the way the reference describes vector loops: a
 * list of (n, is, os) dimensions (the reference's vecsz tensor,
 * dft/dft.h:34-38), strides in elements.
 */
#ifndef GB_TYPES_H
#define GB_TYPES_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_MAXV 4      /* vector dimensions per pass */
#define GB_MAXRAD 24   /* radix stages per transform */

/* What a pass computes. */
enum gb_kind {
     GB_KIND_C2C = 0,       /* complex n -> complex n */
     GB_KIND_R2C = 1,       /* real n -> complex n/2+1 */
     GB_KIND_C2R = 2,       /* complex n/2+1 -> real n */
     GB_KIND_BLUESTEIN = 3, /* complex n -> complex n through a chirp convolution of length nfft */
     GB_KIND_COPY = 4,      /* rank-0 problem: element copy */
     GB_KIND_RADER = 5,     /* prime n: cyclic convolution of length n-1 through the generator permutation */
     GB_KIND_POINTWISE = 6, /* element-wise pass between multi-pass stages (field pw) */
     GB_KIND_DCT2 = 7       /* REDFT10 of n reals in one pass: permuted load, r2c of n, cosine
                             * post-twiddle (chirp: exp(-i pi q / 2n), q < n), n reals out */
};

/* Element-wise passes of multi-pass plans (lengths beyond one CTA). */
enum gb_pw {
     GB_PW_HC2C_POST = 0,   /* r2c: Z (n/2 complex) -> X (n/2+1): hc2c post-pass */
     GB_PW_HC2C_PRE = 1,    /* c2r: X (n/2+1) -> Z' (n/2): hc2c pre-pass */
     GB_PW_CHIRP_IN = 2,    /* Bluestein: x conj(w), zero-padded to nfft */
     GB_PW_SPEC_MUL = 3,    /* Bluestein: multiply by the chirp spectrum, in place */
     GB_PW_CHIRP_OUT = 4,   /* Bluestein: conv conj(w), first n */
     GB_PW_PROMOTE = 5,     /* odd r2c: n reals -> n complex with zero imaginary parts */
     GB_PW_HALF_COPY = 6,   /* odd r2c: first n/2+1 of n complex */
     GB_PW_HERM_EXT = 7,    /* odd c2r: n/2+1 complex -> n complex, X[n-k] = conj X[k] */
     GB_PW_REAL_PART = 8,   /* odd c2r: n complex -> n reals (real parts) */
     GB_PW_CHIRP_IN_REAL = 9,    /* Bluestein r2c: n reals x conj(w), zero-padded to nfft */
     GB_PW_CHIRP_IN_HERM = 10,   /* Bluestein c2r: n/2+1 complex extended by Hermitian symmetry, x conj(w) */
     GB_PW_CHIRP_OUT_HALF = 11,  /* Bluestein r2c: conv conj(w), first n/2+1 */
     GB_PW_CHIRP_OUT_REAL = 12   /* Bluestein c2r: real part of conv conj(w), first n */
};

/* How the transform is computed inside one CTA. */
enum gb_variant {
     GB_VAR_REG = 0,   /* power-of-two length, register-resident Stockham stages of radix <= 16 */
     GB_VAR_GEN = 1,   /* any smooth length, shared-memory Stockham stages, runtime radix list */
     GB_VAR_TMA = 2,   /* as GB_VAR_REG, persistent CTAs fed by bulk async copies (unit-stride c2c) */
     GB_VAR_TC = 3,    /* radix-16 stages as split-FP16 tcgen05 GEMMs (f32 c2c, nfft a power of two 256..4096) */
     GB_VAR_TMA_COLS = 4   /* as GB_VAR_REG for f32 c2c column tiles, persistent CTAs fed by tensor-map TMA boxes */
};

/* How a tile of transforms moves between HBM and the CTA. */
enum gb_move {
     GB_MOVE_DIRECT = 0,  /* each thread loads/stores its own elements (coalesced when stride is 1) */
     GB_MOVE_ROWS = 1,    /* cooperative copy through shared memory, element index fastest */
     GB_MOVE_COLS = 2     /* cooperative copy through shared memory, transform index fastest */
};

typedef struct gb_pass {
     int kind;          /* enum gb_kind */
     int prec;          /* sizeof(real): 4 or 8 */
     int sign;          /* -1 forward, +1 backward */
     int n;             /* logical length (real length for r2c/c2r) */
     int nfft;          /* length of the complex FFT run by the kernel */
     int variant;       /* enum gb_variant */
     int tb;            /* transforms per CTA (along vector dimension 0) */
     int threads;       /* threads per CTA (per compute group for GB_VAR_TMA) */
     int groups;        /* GB_VAR_TMA: compute groups per CTA (1 or 2), each over its own tile buffer */
     int smem;          /* dynamic shared memory bytes */
     int load_mode;     /* enum gb_move */
     int store_mode;    /* enum gb_move */
     int real_pairs;    /* r2c input / c2r output: stride 1 and 8-/16-byte aligned pairs */
     int pw;            /* GB_KIND_POINTWISE: enum gb_pw */
     long long pw_chunks; /* GB_KIND_POINTWISE: CTAs per transform */
     long long is, os;  /* element stride along the transform (complex or real elements) */
     int nv;            /* number of vector dimensions */
     long long vn[GB_MAXV], vis[GB_MAXV], vos[GB_MAXV];
     long long ntiles0;  /* ceil(vn[0] / tb) */
     long long nblocks;  /* total CTAs */
     int nrad;
     int rad[GB_MAXRAD];
     /* device tables (owned by the plan) */
     const void *tw;      /* exp(-2 pi i j / nfft), j < nfft */
     /* power-of-two nfft: the twiddles of the radix-16 stages, laid out so a
      * warp's reads are coalesced.  For each stage with span NS (NS = r0,
      * 16 r0, 256 r0, ... below nfft, r0 the first stage's radix), rows of NS
      * entries exp(-2 pi i k (nfft / (16 NS)) p / nfft), k < NS: float has four
      * rows, p = 1, 2, 4, 8 (the other powers derived, FP32 multiplies being
      * cheap); double has fifteen, p = 1..15 (FP64 multiplies are the
      * bottleneck of double passes).  Stages follow one another
      * (gb_stage_tw_len entries in all). */
     const void *tw_stage;
     /* runtime-radix passes: the twiddles of each stage (span Ns, radix R) in
      * rows r = 1..R-1 of Ns entries exp(-2 pi i r k / (Ns R)), k < Ns, the
      * stage's rows starting at entry Ns - 1 (nfft - 1 entries in all), so a
      * warp's reads are coalesced; 0 when absent (then read from tw) */
     const void *tw_gen;
     const void *tw_half; /* r2c/c2r: exp(-2 pi i k / n), k <= n/2 */
     /* four-step: multiply output k of the transform whose index along
      * vector dimension 0 is v by exp(sign 2 pi i v k / post_N).  The
      * factor is read from two tables: post_lo[m % post_S] * post_hi[m / post_S]. */
     long long post_N;
     long long post_S;    /* power of two; post_lS = log2(post_S) */
     int post_lS;
     int post_vdim;       /* vector dimension whose index v multiplies k in the twiddle (0 = the tile dim) */
     int ltb;             /* log2(tb) when tb is a power of two, else -1 */
     const void *post_lo;
     const void *post_hi;
     /* power-of-two nfft >= 256 (16 elements a thread, T = nfft / 16 threads a
      * transform): the factor of thread t of transform v, W(v t), read with
      * consecutive t on consecutive lanes: row v of post_rows (post_rows_v
      * rows of T entries exp(sign-free -2 pi i v t / post_N)); 0 when absent */
     const void *post_rows;
     long long post_rows_v;
     /* Bluestein: chirp w[k] (k < n) and the spectrum of the padded chirp / nfft */
     const void *chirp;
     const void *chirp_spec;   /* Bluestein: chirp spectrum; Rader: spectrum of omega / (n-1) */
     const int *perm;          /* Rader: g^k mod n (k < n-1), then log_{g^-1} j (j = 1..n-1) */
     /* status word for bounded-wait and bounds reporting (device, owned by the library) */
     int *status;
} gb_pass;

/* One entry of a plan set's device work queue: a tile of transforms of one
 * length, described by a pass, where the tile starts (v0 along vector
 * dimension 0, bi/bo from the outer dimensions), its arrays, and optional
 * dependencies.  Grouped transforms of different arrays use one pointer per
 * transform (pin/pout, vn[0] of them); otherwise in/out + strides apply.
 * An item with wait_ctr >= 0 starts only after counter wait_ctr reached
 * wait_target; one with signal_ctr >= 0 increments it when done (the two
 * passes of a long transform: column tiles signal, row tiles wait). */
typedef struct gb_qitem {
     gb_pass P;
     long long bi, bo, v0;
     const void *in;
     void *out;
     const void *const *pin;
     void *const *pout;
     int wait_ctr, wait_target, signal_ctr, pad_;
     long long pad2_;   /* the size a multiple of 16 bytes (copied in 16-byte pieces) */
} gb_qitem;

/* Device status codes written to gb_pass.status. */
#define GB_STATUS_OK 0
#define GB_STATUS_BAD_DESCRIPTOR 1
#define GB_STATUS_QUEUE_TIMEOUT 2
#define GB_STATUS_COPY_TIMEOUT 3

/* k_reg shared-memory layout, shared by the host planner and the kernels:
 * transform element p lives at p + m*(p/16), m = 2 when the first radix-16
 * stage writes 16 consecutive elements (nfft = 16^k >= 256), else 1; the
 * per-transform stride is rounded up to an even count (16-byte alignment). */
static inline int gb_pad_mult(int nfft)
{
     int r = nfft;
     while (r > 16) r /= 16;
     return (r == 16 && nfft >= 256) ? 2 : 1;
}
static inline int gb_reg_sms(int nfft) { return (nfft + gb_pad_mult(nfft) * (nfft >> 4) + 3) & ~1; }
/* runtime-radix body layout: element i at i + i/16, transforms nfft + nfft/16 + 1
 * complex elements apart (two buffers of tb transforms) */
static inline int gb_gen_sms(int nfft) { return nfft + (nfft >> 4) + 1; }
/* first-stage radix of a power-of-two length in the register kernels */
static inline int gb_reg_r0(int nfft)
{
     int r = nfft;
     while (r > 16) r /= 16;
     return r;
}
/* rows per stage of the stage twiddle table (prec: bytes per real) */
static inline int gb_stage_tw_rows(int prec) { return prec == 8 ? 15 : 4; }
/* entries of the stage twiddle table of a power-of-two nfft (0 below 32) */
static inline int gb_stage_tw_len(int nfft, int prec)
{
     int len = 0, ns;
     if (nfft < 32) return 0;
     for (ns = gb_reg_r0(nfft); ns * 16 <= nfft; ns *= 16) len += gb_stage_tw_rows(prec) * ns;
     return len;
}

/* Most compute groups a k_reg_tma CTA can run (prec: bytes per real): two
 * for float (64 registers a thread), one for double, whose 16 elements a
 * thread already fill 64 registers.  A CTA of g groups of gb_pass.threads
 * threads has g + 1 shared-memory tile buffers. */
static inline int gb_tma_max_groups(int prec) { return prec == 4 ? 2 : 1; }

/* Launchers implemented in the .cu files (plain C ABI). */
int gb_launch_pass(const gb_pass *p, const void *in, void *out, void *stream);
int gb_launch_queue(const gb_qitem *items, int nitems, int *head, int *ctrs, int prec, int threads, int smem,
                    int grid, unsigned long long wait_ns, void *stream);
int gb_queue_grid(int prec, int threads, int smem);
int gb_pass_configure(gb_pass *p, int max_smem_optin);
int gb_twiddles(void *dst, int prec, long long n, long long count, long long mul, void *stream);
int gb_stage_twiddles(void *dst, int prec, int nfft, void *stream);
int gb_post_rows(void *dst, int prec, long long N, int T, long long rows, void *stream);
int gb_gen_stage_twiddles(void *dst, int prec, int nfft, const int *rad, int nrad, void *stream);
int gb_cols_tma_smem(int nfft, int tb, int groups);
#define GB_SPLIT_MAXD 32   /* dims of a split-array problem: vector + transform dims */
/* split-array pack (pack != 0: re/im strided -> dense complex buf) and
 * unpack (dense complex buf -> re/im strided); n/s: nd dims, strides in
 * reals; im == NULL copies one real array to or from dense reals */
int gb_split_copy(int pack, int prec, int nd, const long long *n, const long long *s, long long total, void *re,
                  void *im, void *buf, void *stream);
int gb_cols_tma_plan_ok(const gb_pass *p);
int gb_chirp(void *dst, int prec, long long n, int sign, void *stream);
int gb_device_max_smem(void);
int gb_device_smem_per_sm(void);
const char *gb_last_cuda_error(void);
long long gb_launch_count(void);
void gb_count_launch(void);   /* one more kernel launched outside gb_launch_pass */
int gb_device_status(void);
int *gb_device_status_ptr(void);
/* r2r transforms (fft_r2r.cu): every kind of length n runs as one core
 * transform of length L between a pre and a post kernel.  The core is a
 * real DFT (r2c or c2r) or, for REDFT11/RODFT11, a complex DFT. */
enum { GB_R2R_CORE_R2C = 0, GB_R2R_CORE_C2R = 1, GB_R2R_CORE_C2C = 2 };
#ifdef __CUDACC__
#define GB_HD __host__ __device__
#else
#define GB_HD
#endif
/* kind: fftw_r2r_kind value; returns the core and sets *len = L */
static inline GB_HD int gb_r2r_core(int kind, long long n, long long *len)
{
     switch (kind) {
     case 1: case 4: case 8:            /* HC2R, REDFT01, RODFT01 */
          *len = n;
          return GB_R2R_CORE_C2R;
     case 3:                            /* REDFT00: even extension, logical 2(n-1) */
          *len = 2 * (n - 1);
          return GB_R2R_CORE_R2C;
     case 7:                            /* RODFT00: odd extension, logical 2(n+1) */
          *len = 2 * (n + 1);
          return GB_R2R_CORE_R2C;
     case 6: case 10:                   /* REDFT11, RODFT11: n/2 complex (even n), 2n zero-padded (odd n) */
          *len = (n & 1) ? 2 * n : n / 2;
          return GB_R2R_CORE_C2C;
     default:                           /* R2HC, DHT, REDFT10, RODFT10 */
          *len = n;
          return GB_R2R_CORE_R2C;
     }
}
/* The vector loop of one r2r axis: nv dims (outermost first) with input and
 * output strides in reals; row t of the dense core buffers is the vector
 * index t in row-major order over these dims. */
#define GB_R2R_MAXV 32
typedef struct {
     int nv;
     long long n[GB_R2R_MAXV], is[GB_R2R_MAXV], os[GB_R2R_MAXV];
} gb_r2r_vec;
long long gb_r2r_table_len(int kind, long long n);
int gb_r2r_table(int prec, int kind, long long n, void *tab, void *stream);
int gb_r2r_pre(int prec, int kind, long long n, long long V, const void *in, long long is, const gb_r2r_vec *vec,
               void *buf, const void *tw, void *stream);
int gb_r2r_post(int prec, int kind, long long n, long long V, const void *buf, void *out, long long os,
                const gb_r2r_vec *vec, const void *tw, void *stream);

#ifdef __cplusplus
}
#endif
#endif
