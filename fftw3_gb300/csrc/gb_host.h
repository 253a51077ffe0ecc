/*
 * Host-side internals of libfftw3_gb300 (C).
 *
 * A problem is stored the way the reference stores one (dft/dft.h:34-38,
 * rdft/rdft.h:117-124): a transform tensor sz of (n, is, os) dims and a
 * vector tensor vecsz, plus the array pointers.  Strides here are in
 * elements of the array they index: complex elements for complex arrays,
 * real elements for real arrays (the reference counts reals throughout,
 * api/plan-many-dft.c:44-47; the factor 2 is applied at the boundary).
 */
#ifndef GB_HOST_H
#define GB_HOST_H

#include <stddef.h>
#include <pthread.h>
#include "gb_types.h"

#define GB_MAXRANK 16
#define GB_FLAG_TENSOR_CORE (1U << 28)   /* FFTW_GB300_TENSOR_CORE */
#define GB_MAXPASS 16
#define GB_MAXLOOP 8

enum gb_prob_kind { GB_PROB_DFT = 0, GB_PROB_R2C = 1, GB_PROB_C2R = 2, GB_PROB_R2R = 3 };

typedef struct { long long n, is, os; } gb_dim;

typedef struct gb_problem {
     int kind;              /* enum gb_prob_kind */
     int prec;              /* 4 or 8 */
     int sign;              /* -1 / +1 (c2c); r2c -1; c2r +1 */
     int rank;
     gb_dim sz[GB_MAXRANK];
     int vrank;
     gb_dim vec[GB_MAXRANK];
     void *in, *out;        /* arrays given at planning time */
} gb_problem;

/* buffer ids a pass reads or writes */
enum { GB_BUF_IN = 0, GB_BUF_OUT = 1, GB_BUF_SCRATCH = 2, GB_BUF_SCRATCH2 = 3 };

typedef struct gb_step {
     gb_pass pass;
     int src, dst;                 /* buffer ids */
     long long src_off, dst_off;   /* element offsets added to the buffer pointer */
     int nloop;                    /* vector dims beyond GB_MAXV, looped on the host */
     gb_dim loop[GB_MAXLOOP];
} gb_step;

#define GB_CHUNK_SLOTS 3

/* one stage of an r2r plan: the r2r of one transform dim over all the
 * other dims (vector loop vec) */
typedef struct gb_r2r_axis {
     int kind, core;            /* fftw_r2r_kind; GB_R2R_CORE_* */
     long long n, L, V;         /* length, core length, transforms in the stage */
     long long is, os;          /* strides along the dim (reals) */
     int src_mid, dst_mid;      /* read from / write to r2r_mid instead of the caller's arrays */
     gb_r2r_vec vec;
     void *tw;                  /* device twiddle table of the stage (NULL: none) */
     struct gb_plan *inner;     /* the core transform on r2r_buf[0] -> r2r_buf[1] */
     int fused;                 /* 1: the stage also runs as the single pass fpass */
     gb_pass fpass;             /* REDFT10 of unit-stride rows: load, r2c and post-twiddle in one kernel */
} gb_r2r_axis;

struct gb_plan {
     int refcnt;
     /* held while one execute enqueues its work: calls on the same plan from
      * several host threads reach the device one whole call after another,
      * so the plan-owned scratch, staging buffers and chunk slots are never
      * shared by two calls in flight (api/execute.c may run concurrently on
      * one plan, doc/threads.texi:243-247) */
     pthread_mutex_t exec_mtx;
     gb_problem prb;
     unsigned flags;
     int nstep;
     gb_step step[GB_MAXPASS];
     size_t scratch_bytes, scratch2_bytes;
     void *scratch, *scratch2;  /* device scratch (intermediates of multi-pass lengths) */
     /* staging buffers for host arrays */
     void *stage_in, *stage_out;
     size_t stage_in_bytes, stage_out_bytes;
     /* pipelined staging of host arrays: the batch is cut along one vector
      * dimension into chunks; a chunk plan transforms chunk c on the plan's
      * stream while chunk c+1 is copied in and chunk c-1 copied out */
     int chunk_state;           /* 0 = not tried yet, 1 = ready, -1 = not applicable */
     int chunk_dim;             /* the vector dimension cut into chunks */
     long long chunk_m;         /* transforms per chunk (vec[chunk_dim] entries) */
     struct gb_plan *chunk_plan[2];   /* chunk of chunk_m; the shorter last chunk */
     void *chunk_buf[2][GB_CHUNK_SLOTS];   /* device slots: [input/output][slot] */
     size_t chunk_bytes[2];
     void *chunk_stream[2];     /* copy-in and copy-out streams */
     void *chunk_ev[3][GB_CHUNK_SLOTS];    /* copied in / transformed / copied out, per slot */
     /* split-array problems (separate real and imaginary arrays): dims
      * [vector dims..., transform dims...] with strides in reals; the
      * transform runs as the forward c2c plan split_inner on dense
      * interleaved buffers, between a pack and an unpack kernel */
     int split_kind;            /* GB_PROB_DFT, GB_PROB_R2C or GB_PROB_C2R */
     int split_nd;
     long long split_n[2 * GB_MAXRANK], split_is[2 * GB_MAXRANK], split_os[2 * GB_MAXRANK];
     void *split_arr[4];        /* ri, ii, ro, io at planning time */
     struct gb_plan *split_inner;
     void *split_buf[2];        /* dense complex input and output of split_inner */
     /* r2r problems: one stage per transform dim (a pre kernel, the core
      * transform on dense buffers, a post kernel), last dim first */
     int r2r_naxis;
     struct gb_r2r_axis *r2r_ax;
     void *r2r_buf[2];          /* dense core input and output */
     void *r2r_mid;             /* dense real intermediate between stages (rank > 1) */
     void *stream;              /* cudaStream_t; 0 = legacy default stream */
     int async;                 /* 1: execute does not wait for completion */
     int tc_stages;             /* tensor-core GEMM stages the plan's passes hold (planning only) */
     int in_align, out_align;   /* alignment of the planning arrays (bytes, capped at 16) */
     double add, mul, fma;      /* operation counts */
     double measured_ms;        /* time of one execute measured by the tuner (0 if not measured) */
     char desc[1024];           /* what print_plan prints */
     char key[256];             /* wisdom key */
};
typedef struct gb_plan gb_plan;

/* planner / problem (gb_plan.c) */
gb_plan *gb_mkplan(const gb_problem *prb, unsigned flags);
gb_plan *gb_plan_alloc(void);   /* zeroed plan with refcnt 1 and its execute lock */
void gb_problem_key(const gb_problem *prb, char *key, size_t cap);   /* wisdom key of a whole problem */
void gb_destroy(gb_plan *p);
int gb_dry_run(void);
void gb_set_dry_run(int on);
void gb_fail_alloc_after(int k);   /* test hook: the table allocation after the next k fails once */
const char *gb_last_error(void);
void gb_set_error(const char *fmt, ...);
void gb_lock(void);
void gb_unlock(void);
int gb_cuda_ready(void);

/* library state (gb_api.c) */
void *gb_malloc(size_t n);
void gb_free(void *p);
void gb_set_timelimit(double t);
double gb_get_timelimit(void);
void gb_set_nthreads(int n);
int gb_get_nthreads(void);
void gb_note_failure(void);
void gb_cleanup_tables(void);

/* tuner (gb_tune.c) */
int gb_tune(gb_plan *p, unsigned flags);

/* execution (gb_exec.c) */
int gb_execute(gb_plan *p, void *in, void *out);
gb_plan *gb_mksplit(int kind, int prec, int rank, const gb_dim *dims, int vrank, const gb_dim *vdims, void *ri,
                    void *ii, void *ro, void *io, unsigned flags);
int gb_execute_split(gb_plan *p, void *a0, void *a1, void *a2, void *a3);
gb_plan *gb_mkr2r(int prec, int rank, const gb_dim *dims, const int *kinds, int vrank, const gb_dim *vdims, void *in,
                  void *out, unsigned flags);
int gb_execute_r2r(gb_plan *p, void *in, void *out);
int gb_r2r_tune(gb_plan *p, unsigned flags);

/* wisdom (gb_wisdom.c) */
typedef struct gb_wisdom_entry {
     char key[256];
     int variant, tb, load_mode, store_mode, n1;
     int groups;    /* compute groups per CTA of a bulk-copy pass (0: the planner's choice) */
     int order;     /* radix order of a runtime-radix pass (0: the planner's; see gb_factor_order) */
} gb_wisdom_entry;
const gb_wisdom_entry *gb_wisdom_lookup(const char *key);
void gb_wisdom_store(const gb_wisdom_entry *e);
void gb_wisdom_forget(void);
int gb_wisdom_export(int prec, void (*emit)(char c, void *), void *data);
int gb_wisdom_import(int prec, int (*getc_fn)(void *), void *data);

/* table cache (gb_plan.c) */
const void *gb_table_twiddle(int prec, long long n, long long count, long long mul);
const void *gb_table_chirp(int prec, long long n, int sign);
const void *gb_table_chirp_spec(int prec, long long n, long long nb, int sign);
void gb_tables_free(void);

/* helpers shared with the plan-set compiler */
int gb_factor_radices(long long n, int *rad);
#define GB_RADIX_ORDERS 3
int gb_factor_order(long long n, int *rad, int order);
int gb_pass_tables(gb_pass *P);
/* one pass of kind over a batch (nv <= GB_MAXV vector dims), as the planner
 * configures its passes; 0 on success */
int gb_config_pass(gb_pass *P, int prec, int kind, long long n, int sign, long long is, long long os, int nv,
                   const gb_dim *v);

/* plan sets (gb_set.c) */
typedef struct gb_set gb_set;
gb_set *gb_mkset(int prec, int nplans, gb_plan *const *plans, unsigned flags);
int gb_execute_set(gb_set *S);
void gb_set_stream_of_set(gb_set *S, void *stream, int async);
void gb_set_info(const gb_set *S, int *nitems, int *ntransforms, int *nlong, int *grid, int *smem);
int gb_set_item_info(const gb_set *S, int i, int *kind, int *nfft, int *tb, int *variant, int *queue, int *role);
int gb_set_wait_limit(gb_set *S, double seconds);
int gb_set_test_stall(gb_set *S, int on);
void gb_destroy_set(gb_set *S);

/* launch layer (fft_launch.cu) */
int gb_chirp_pad(void *dst, const void *w, int prec, long long n, long long nb, void *stream);
int gb_rader_omega(void *dst, const int *gpow, int prec, long long p, int sign, void *stream);
const int *gb_table_rader_perm(long long p);
const void *gb_table_rader_spec(int prec, long long p, int sign);
int gb_pass_kernel_attrs(const gb_pass *p, int *regs, int *max_threads);
int gb_tc_smem(int nfft, int ctas);
int gb_tc_selftest(const void *A, const void *B, float *D, int ks);

#endif
