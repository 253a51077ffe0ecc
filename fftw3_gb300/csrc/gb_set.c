/*
 * Plan sets: many independent c2c plans of uneven lengths executed by one
 * persistent kernel with a device work queue, captured once as a CUDA graph.
 *
 * The reference executes a set of transforms as a loop of fftw_execute calls,
 * one plan after another (each a tree of solver applies, api/execute.c:23-27).
 * Here the set compiles to queue items (gb_qitem):
 *   - a transform that fits one CTA's shared memory (2 buffers of
 *     nfft + nfft/16 + 1 complex, the padded layout; nfft <= 4096 single /
 *     2048 double) is a "single"; singles of
 *     the same length, sign and strides are grouped into items of up to 32
 *     transforms, each transform with its own array pointers;
 *   - a prime length is a Bluestein single (power-of-two convolution) or, if
 *     the tuner or FFTW_GB300_PRIME=rader asks and n-1 is smooth, a Rader single;
 *   - a longer smooth transform is split n = n1*n2 into column tiles (pass A,
 *     with the W_n^(n2 k1) twiddle, into set-owned scratch) and row tiles
 *     (pass B, into the output); row tiles wait for their transform's column
 *     tiles on a device counter.
 * Items are queued column tiles first, then singles by decreasing cost, then
 * row tiles, so no wait can block a claimed item.  Prime singles whose
 * convolution needs twice the tile (nb up to 8192 single / 4096 double) go to
 * a second queue with larger tiles, launched first in the same graph.
 *
 * Per length, the items' configuration is the tuner's when wisdom holds an
 * entry "set p<prec> n<n>" (the item body, register stages or runtime-radix
 * stages; the radix order; Rader or Bluestein for a prime; the split of a long
 * length; transforms per item), else the planner's defaults.  A set planned
 * without FFTW_ESTIMATE tunes every length wisdom does not cover: each
 * candidate runs as a set of that length alone on scratch device arrays,
 * timed with CUDA events, and the fastest is stored in wisdom (exported with
 * fftw_export_wisdom), as the reference's measuring planner times candidate
 * plans (kernel/planner.c:518-615, kernel/timer.c:142-181).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stddef.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "fftw3.h"
#include "gb_host.h"

#define GB_Q_GROUP 32

typedef struct { long long n; int sign; long long is, os; const void *in; void *out; } xform;

struct gb_set {
     int prec;
     int nitems, nctr;
     int nsmall, nlarge;            /* items of the small-tile and large-tile queues */
     int grid, threads, smem;       /* small-tile queue launch */
     int grid_l, threads_l, smem_l; /* large-tile queue launch */
     gb_qitem *d_items;
     int *d_head, *d_ctrs;          /* two queue heads */
     void **d_ptrs;
     void *d_scratch;
     size_t scratch_bytes;
     void *stream;
     int async;
     /* the large-tile queue runs beside the small-tile one: a second stream
      * forked from and joined back into the set's stream inside the capture */
     cudaStream_t side;
     cudaEvent_t ev_fork, ev_join;
     cudaGraph_t graph;
     cudaGraphExec_t gexec;
     gb_qitem *h_items;             /* dry run (no GPU): the items, kept on the host for inspection */
     int nsingle_items, nlong, ntransforms;
     unsigned long long wait_ns;    /* bound on a row tile's wait for its column tiles */
     int stall_item;                /* item whose wait target the test hook raised (-1: none) */
     int stall_target;              /* its true target */
};
typedef struct gb_set gb_set;

static void drop_graph(gb_set *S);

static int is_prime_ll(long long n)
{
     long long d;
     if (n < 2) return 0;
     for (d = 2; d * d <= n; ++d)
          if (n % d == 0) return 0;
     return 1;
}

static long long pow2_at_least(long long v)
{
     long long p = 1;
     while (p < v) p <<= 1;
     return p;
}

/* Fill the pass fields a queue item needs (the shared-memory tile body). */
static int item_pass(gb_pass *P, int prec, int kind, long long n, int sign, long long is, long long os,
                     long long vn0, long long vis0, long long vos0, int tb, int cols_in, int cols_out, int threads,
                     int body, int order)
{
     memset(P, 0, sizeof *P);
     P->ltb = -1;
     P->kind = kind; P->prec = prec; P->sign = sign; P->n = (int)n;
     P->nfft = (int)(kind == GB_KIND_BLUESTEIN ? pow2_at_least(2 * n - 1) : kind == GB_KIND_RADER ? n - 1 : n);
     P->variant = GB_VAR_GEN;
     P->tb = tb;
     P->threads = threads;
     P->smem = 2 * tb * gb_gen_sms(P->nfft) * 2 * prec;
     P->load_mode = cols_in ? GB_MOVE_COLS : GB_MOVE_ROWS;
     P->store_mode = cols_out ? GB_MOVE_COLS : GB_MOVE_ROWS;
     P->is = is; P->os = os;
     P->nv = 1;
     P->vn[0] = vn0; P->vis[0] = vis0; P->vos[0] = vos0;
     P->ntiles0 = 1; P->nblocks = 1;
     P->nrad = (kind == GB_KIND_C2C && order > 0) ? gb_factor_order(P->nfft, P->rad, order)
                                                   : gb_factor_radices(P->nfft, P->rad);
     if (P->nrad < 0) return -1;
     if (gb_pass_tables(P)) return -1;
     if (P->ltb >= 0 && (1 << P->ltb) != P->tb) return -1;
     /* the register body (when asked for) of a power-of-two float c2c of
      * 64..4096 points in the small-tile queue: 256 / (nfft/16) transforms a
      * round; the shared memory holds a round of the register layout (rows
      * beyond the item's transforms included) */
     if (body == GB_VAR_REG && kind == GB_KIND_C2C && prec == 4 && threads == 256 && P->nfft >= 64 &&
         P->nfft <= 4096 && (P->nfft & (P->nfft - 1)) == 0 && (long long)tb * (P->nfft / 16) <= 256) {
          const int round = 256 / (P->nfft / 16), lay = round * gb_reg_sms(P->nfft) * 2 * prec;
          P->variant = GB_VAR_REG;
          if (lay > P->smem) P->smem = lay;
     }
     return 0;
}

/* growable item array */
typedef struct { gb_qitem *v; int n, cap; } qvec;

static gb_qitem *qpush(qvec *q)
{
     if (q->n == q->cap) {
          int nc = q->cap ? 2 * q->cap : 256;
          gb_qitem *nv = (gb_qitem *)realloc(q->v, sizeof(gb_qitem) * (size_t)nc);
          if (!nv) return 0;
          q->v = nv;
          q->cap = nc;
     }
     memset(&q->v[q->n], 0, sizeof(gb_qitem));
     return &q->v[q->n++];
}

static double item_cost(const gb_qitem *q)
{
     double n = q->P.nfft;
     return q->P.tb * n * (n > 1 ? log2(n) : 1) * (q->P.kind == GB_KIND_BLUESTEIN || q->P.kind == GB_KIND_RADER ? 2 : 1);
}

static int cmp_cost_desc(const void *a, const void *b)
{
     double ca = item_cost((const gb_qitem *)a), cb = item_cost((const gb_qitem *)b);
     return ca < cb ? 1 : ca > cb ? -1 : 0;
}

static int cmp_key(const void *a, const void *b)
{
     const xform *x = (const xform *)a, *y = (const xform *)b;
     if (x->n != y->n) return x->n < y->n ? -1 : 1;
     if (x->sign != y->sign) return x->sign - y->sign;
     if (x->is != y->is) return x->is < y->is ? -1 : 1;
     if (x->os != y->os) return x->os < y->os ? -1 : 1;
     return 0;
}

/* The configuration of one length's items in a set. */
typedef struct {
     int body;       /* GB_VAR_REG or GB_VAR_GEN: the body of power-of-two float items */
     int order;      /* radix order of runtime-radix items (gb_factor_order) */
     int prime;      /* GB_KIND_RADER / GB_KIND_BLUESTEIN for a prime, 0: the planner's */
     int tbmax;      /* transforms per single item, 0: as many as the tile holds (up to 32) */
     long long n1;   /* split n = n1 * n2 of a long length, 0: the planner's */
} set_cfg;

static void set_key(char *key, size_t cap, int prec, long long n) { snprintf(key, cap, "set p%d n%lld", prec, n); }

/* A length's configuration: the wisdom entry "set p<prec> n<n>" (variant =
 * the body of a smooth length's items or the kind of a prime's, tb = the
 * transforms per item, n1 = the split, order = the radix order), else the
 * defaults (runtime-radix body, order 0).  FFTW_GB300_QUEUE_BODY=reg|gen
 * overrides the body. */
static set_cfg length_cfg(int prec, long long n)
{
     set_cfg c = {GB_VAR_GEN, 0, 0, 0, 0};
     char key[64];
     const gb_wisdom_entry *w;
     const char *e = getenv("FFTW_GB300_QUEUE_BODY");
     set_key(key, sizeof key, prec, n);
     w = gb_wisdom_lookup(key);
     if (w) {
          if (w->variant == GB_VAR_REG || w->variant == GB_VAR_GEN) c.body = w->variant;
          if (w->variant == GB_KIND_RADER || w->variant == GB_KIND_BLUESTEIN) c.prime = w->variant;
          c.order = w->order;
          c.tbmax = w->tb;
          c.n1 = w->n1;
     }
     if (e && !strcmp(e, "reg")) c.body = GB_VAR_REG;
     else if (e && !strcmp(e, "gen")) c.body = GB_VAR_GEN;
     return c;
}

/* How a prime (or non-smooth) length runs as a single: Rader (n-1 smooth)
 * or Bluestein (power-of-two convolution), in the small-tile queue when its
 * FFT fits cap_s, else in the large-tile queue (cap_l).  want is the set
 * tuner's choice (0: none; then the plan tuner's wisdom or
 * FFTW_GB300_PRIME=rader asks for Rader).  *large is set for the latter; -1
 * when neither fits. */
static int prime_kind(int prec, long long n, int cap_s, int cap_l, int want, int *large)
{
     int rad[GB_MAXRAD];
     const char *e = getenv("FFTW_GB300_PRIME");
     char key[128];
     const gb_wisdom_entry *w;
     int rader = is_prime_ll(n) && gb_factor_radices(n - 1, rad) >= 0;
     long long nb = pow2_at_least(2 * n - 1);
     int want_rader;
     snprintf(key, sizeof key, "c2c p%d n%lld", prec, n);
     w = gb_wisdom_lookup(key);
     if (want) want_rader = rader && want == GB_KIND_RADER;
     else want_rader = rader && ((w && w->variant == GB_KIND_RADER) || (!w && e && !strcmp(e, "rader")));
     if (want == GB_KIND_BLUESTEIN && nb <= cap_l) {
          *large = nb > cap_s;
          return GB_KIND_BLUESTEIN;
     }
     *large = 0;
     if (want_rader && n - 1 <= cap_s) return GB_KIND_RADER;
     if (nb <= cap_s) return GB_KIND_BLUESTEIN;
     if (rader && n - 1 <= cap_s) return GB_KIND_RADER;
     *large = 1;
     if (want_rader && n - 1 <= cap_l) return GB_KIND_RADER;
     if (nb <= cap_l) return GB_KIND_BLUESTEIN;
     if (rader && n - 1 <= cap_l) return GB_KIND_RADER;
     return -1;
}

/* small-tile queue: transforms up to 4096 complex64 (2048 complex128) points,
 * two buffers of 16 (8) x 273 elements (a 256-point transform in the padded
 * layout, gb_gen_sms) = 69.9 KB, three 256-thread CTAs per SM; large-tile
 * queue: twice that, one 512-thread CTA per SM, only for what the small tiles
 * cannot hold */
static int cap_small(int prec) { return prec == 4 ? 4096 : 2048; }
static int qbuf(int prec) { return (prec == 4 ? 16 : 8) * gb_gen_sms(256); }

/* Splits n = d * (n / d) of a long length with both factors within a tile
 * and 13-smooth, d ascending (at most maxd of them). */
static int long_splits(long long n, int cap, long long *d, int maxd)
{
     int rad[GB_MAXRAD], k = 0;
     long long q;
     for (q = 2; q <= cap && k < maxd; ++q)
          if (n % q == 0 && n / q <= cap && gb_factor_radices(q, rad) >= 0 && gb_factor_radices(n / q, rad) >= 0)
               d[k++] = q;
     return k;
}

/* The split of a long length: the configured n1 when it is one of the
 * splits, else the largest n1 <= sqrt(n) (0: none). */
static long long long_n1(long long n, int cap, long long want)
{
     long long d[64], best = 0;
     int k = long_splits(n, cap, d, 64), i;
     for (i = 0; i < k; ++i) {
          if (d[i] == want) return want;
          if (d[i] * d[i] <= n) best = d[i];
     }
     return best;
}

static gb_set *build_set(int prec, xform *xs, int nx);
static void tune_set(int prec, const xform *xs, int nx, unsigned flags);

gb_set *gb_mkset(int prec, int nplans, gb_plan *const *plans, unsigned flags)
{
     gb_set *S;
     xform *xs;
     int nx = 0, i;
     const int cs = 2 * prec;
     if (!gb_dry_run() && !gb_cuda_ready()) {
          gb_set_error("plan sets need a GPU");
          return 0;
     }
     for (i = 0; i < nplans; ++i) {
          const gb_problem *pr;
          if (!plans[i]) { gb_set_error("plan set: plan %d is NULL", i); return 0; }
          pr = &plans[i]->prb;
          if (pr->kind != GB_PROB_DFT || pr->rank != 1 || pr->vrank > 1 || pr->prec != prec || plans[i]->split_inner) {
               gb_set_error("plan set: plan %d is not a rank-1 c2c plan of this precision", i);
               return 0;
          }
          nx += pr->vrank ? (int)pr->vec[0].n : 1;
     }
     xs = (xform *)malloc(sizeof(xform) * (size_t)(nx ? nx : 1));
     nx = 0;
     for (i = 0; i < nplans; ++i) {
          const gb_problem *pr = &plans[i]->prb;
          long long h = pr->vrank ? pr->vec[0].n : 1, t;
          for (t = 0; t < h; ++t) {
               xform *x = &xs[nx++];
               x->n = pr->sz[0].n; x->sign = pr->sign; x->is = pr->sz[0].is; x->os = pr->sz[0].os;
               x->in = (const char *)pr->in + (pr->vrank ? t * pr->vec[0].is : 0) * cs;
               x->out = (char *)pr->out + (pr->vrank ? t * pr->vec[0].os : 0) * cs;
          }
     }
     if (flags & FFTW_WISDOM_ONLY) {
          /* every length needs the tuner's entry */
          for (i = 0; i < nx; ++i) {
               char key[64];
               set_key(key, sizeof key, prec, xs[i].n);
               if (!gb_wisdom_lookup(key)) {
                    gb_set_error("plan set: FFTW_WISDOM_ONLY and no wisdom for length %lld", xs[i].n);
                    free(xs);
                    return 0;
               }
          }
     } else if (!(flags & FFTW_ESTIMATE) && !gb_dry_run()) {
          tune_set(prec, xs, nx, flags);
     }
     S = build_set(prec, xs, nx);
     free(xs);
     return S;
}

/* The queue items of transforms xs (sorted here), their device copies and
 * the set that runs them. */
static gb_set *build_set(int prec, xform *xs, int nx)
{
     gb_set *S;
     int i, j;
     const int cap_s = cap_small(prec), cap_l = 2 * cap_s, cap = cap_s;
     int cs = 2 * prec;
     qvec QA = {0, 0, 0}, QM = {0, 0, 0}, QB = {0, 0, 0}, QL = {0, 0, 0};
     gb_qitem *A, *M, *B, *Lg;
     int na, nm, nb, nl;
     int smem_l = 0;
     void **hptr = 0;
     int nptr = 0, cap_ptr;
     long long scratch_elems = 0;
     int nctr = 0, smem = 0;
     qsort(xs, (size_t)nx, sizeof(xform), cmp_key);
     cap_ptr = 2 * nx + 2;
     hptr = (void **)calloc((size_t)cap_ptr, sizeof(void *));

     for (i = 0; i < nx;) {
          xform *x = &xs[i];
          long long n = x->n;
          int rad[GB_MAXRAD], kind = GB_KIND_C2C, g, large = 0;
          int smooth = gb_factor_radices(n, rad) >= 0;
          const set_cfg cf = length_cfg(prec, n);
          if (n <= cap_s && smooth) kind = GB_KIND_C2C;
          else if (!smooth && (kind = prime_kind(prec, n, cap_s, cap_l, cf.prime, &large)) > 0) { /* single */ }
          else kind = -1;
          if (kind >= 0) {
               /* group transforms with the same key */
               gb_pass tmp;
               int qb = large ? 2 * qbuf(prec) : qbuf(prec), thr = large ? 512 : 256;
               long long nfft = kind == GB_KIND_BLUESTEIN ? pow2_at_least(2 * n - 1) : kind == GB_KIND_RADER ? n - 1 : n;
               int tbmax = qb / gb_gen_sms((int)nfft);
               if (tbmax > GB_Q_GROUP) tbmax = GB_Q_GROUP;
               if (cf.tbmax > 0 && cf.tbmax < tbmax) tbmax = cf.tbmax;
               if (tbmax < 1) tbmax = 1;
               for (g = 0; i + g < nx && g < tbmax && cmp_key(&xs[i], &xs[i + g]) == 0; ++g) {}
               if (item_pass(&tmp, prec, kind, n, x->sign, x->is, x->os, g, 0, 0, g, 0, 0, thr, cf.body, cf.order))
                    goto fail;
               {
                    gb_qitem *q = qpush(large ? &QL : &QM);
                    if (!q) goto fail;
                    q->P = tmp;
                    q->pin = (const void *const *)(size_t)nptr;     /* index now, device address later */
                    q->pout = (void *const *)(size_t)(nptr + g);
                    for (j = 0; j < g; ++j) { hptr[nptr + j] = (void *)xs[i + j].in; hptr[nptr + g + j] = xs[i + j].out; }
                    nptr += 2 * g;
                    q->wait_ctr = -1; q->signal_ctr = -1;
                    if (large) { if (tmp.smem > smem_l) smem_l = tmp.smem; }
                    else if (tmp.smem > smem) smem = tmp.smem;
               }
               i += g;
               continue;
          }
          if (!smooth) {
               gb_set_error("plan set: length %lld is not supported in a set", n);
               goto fail;
          }
          {
               /* long transform: n = n1 * n2 with both factors in one CTA */
               long long n1 = long_n1(n, cap, cf.n1), n2, k0;
               int tbc = prec == 4 ? 16 : 8, ctr = nctr++;
               gb_pass pa, pb;
               int nta = 0;
               if (!n1) { gb_set_error("plan set: length %lld has no two-pass split", n); goto fail; }
               n2 = n / n1;
               /* columns per tile: the tuner's (a power of two) or 16 (8 double) */
               if (cf.tbmax > 0 && cf.tbmax < tbc && (cf.tbmax & (cf.tbmax - 1)) == 0) tbc = cf.tbmax;
               while (tbc > 1 && (long long)tbc * gb_gen_sms((int)(n1 > n2 ? n1 : n2)) > qbuf(prec)) tbc >>= 1;
               /* pass A: columns n2 (stride is), n1-point transforms with
                * element stride n2*is into scratch [n2][k1] */
               if (item_pass(&pa, prec, GB_KIND_C2C, n1, x->sign, n2 * x->is, 1, n2, x->is, n1, tbc, 1, 0, 256, cf.body,
                             cf.order))
                    goto fail;
               pa.post_N = n;
               if (gb_pass_tables(&pa)) goto fail;
               for (k0 = 0; k0 < n2; k0 += tbc) {
                    gb_qitem *q = qpush(&QA);
                    if (!q) goto fail;
                    q->P = pa;
                    q->v0 = k0;
                    q->in = x->in;
                    q->out = (void *)(size_t)scratch_elems;      /* offset now, address later */
                    q->wait_ctr = -1; q->signal_ctr = ctr;
                    ++nta;
               }
               if (pa.smem > smem) smem = pa.smem;
               /* pass B: k1 columns of scratch (stride 1), n2-point transforms
                * with element stride n1, into out[k1 + n1*k2] */
               if (item_pass(&pb, prec, GB_KIND_C2C, n2, x->sign, n1, n1 * x->os, n1, 1, x->os, tbc, 1, 1, 256, cf.body,
                             cf.order))
                    goto fail;
               for (k0 = 0; k0 < n1; k0 += tbc) {
                    gb_qitem *q = qpush(&QB);
                    if (!q) goto fail;
                    q->P = pb;
                    q->v0 = k0;
                    q->in = (const void *)(size_t)scratch_elems;
                    q->out = x->out;
                    q->wait_ctr = ctr; q->wait_target = nta; q->signal_ctr = -1;
               }
               if (pb.smem > smem) smem = pb.smem;
               /* next transform's scratch on a fresh 256-byte boundary, so no
                * cache line holds two transforms' intermediates */
               scratch_elems += (n + 31) & ~31LL;
          }
          ++i;
     }
     A = QA.v; M = QM.v; B = QB.v; Lg = QL.v;
     na = QA.n; nm = QM.n; nb = QB.n; nl = QL.n;
     if (nm) qsort(M, (size_t)nm, sizeof(gb_qitem), cmp_cost_desc);
     if (nl) qsort(Lg, (size_t)nl, sizeof(gb_qitem), cmp_cost_desc);

     S = (gb_set *)calloc(1, sizeof *S);
     S->prec = prec;
     S->nitems = na + nm + nb + nl;
     S->nsmall = na + nm + nb;
     S->nlarge = nl;
     S->nctr = nctr;
     S->threads = 256;
     S->smem = smem;
     S->threads_l = 512;
     S->smem_l = smem_l;
     S->nsingle_items = nm;
     S->nlong = nctr;
     S->ntransforms = nx;
     S->wait_ns = 2000000000ull;
     S->stall_item = -1;
     S->scratch_bytes = (size_t)scratch_elems * cs;
     if (gb_dry_run()) {
          /* no device: the items stay on the host (gb_set_item_info), the
           * launch shape is unknown (grid 0) and the set cannot execute */
          S->h_items = (gb_qitem *)malloc(sizeof(gb_qitem) * (size_t)(S->nitems ? S->nitems : 1));
          if (!S->h_items) { free(S); goto fail; }
          memcpy(S->h_items, A, sizeof(gb_qitem) * (size_t)na);
          memcpy(S->h_items + na, M, sizeof(gb_qitem) * (size_t)nm);
          memcpy(S->h_items + na + nm, B, sizeof(gb_qitem) * (size_t)nb);
          memcpy(S->h_items + na + nm + nb, Lg, sizeof(gb_qitem) * (size_t)nl);
          free(QA.v); free(QM.v); free(QB.v); free(QL.v); free(hptr);
          return S;
     }
     S->grid = S->nsmall ? gb_queue_grid(prec, S->threads, S->smem) : 1;
     S->grid_l = S->nlarge ? gb_queue_grid(prec, S->threads_l, S->smem_l) : 1;
     if (S->grid <= 0 || S->grid_l <= 0) { gb_set_error("plan set: queue kernel does not fit (smem %d/%d)", smem, smem_l); free(S); goto fail; }
     if (cudaMalloc((void **)&S->d_items, sizeof(gb_qitem) * (size_t)(S->nitems ? S->nitems : 1)) != cudaSuccess ||
         cudaMalloc((void **)&S->d_head, 2 * sizeof(int)) != cudaSuccess ||
         cudaMalloc((void **)&S->d_ctrs, sizeof(int) * (size_t)(nctr ? nctr : 1)) != cudaSuccess ||
         cudaMalloc((void **)&S->d_ptrs, sizeof(void *) * (size_t)(nptr ? nptr : 1)) != cudaSuccess ||
         (S->scratch_bytes && cudaMalloc(&S->d_scratch, S->scratch_bytes) != cudaSuccess)) {
          cudaGetLastError();
          gb_set_error("plan set: device allocation failed");
          gb_destroy_set(S);
          goto fail;
     }
     {
          /* resolve indices/offsets into device addresses, then upload */
          gb_qitem *all = (gb_qitem *)malloc(sizeof(gb_qitem) * (size_t)(S->nitems ? S->nitems : 1));
          int k = 0;
          for (i = 0; i < na; ++i) {
               all[k] = A[i];
               all[k].out = (char *)S->d_scratch + (size_t)A[i].out * cs;
               ++k;
          }
          for (i = 0; i < nm; ++i) {
               all[k] = M[i];
               all[k].pin = (const void *const *)(S->d_ptrs + (size_t)M[i].pin);
               all[k].pout = (void *const *)(S->d_ptrs + (size_t)M[i].pout);
               ++k;
          }
          for (i = 0; i < nb; ++i) {
               all[k] = B[i];
               all[k].in = (const char *)S->d_scratch + (size_t)B[i].in * cs;
               ++k;
          }
          for (i = 0; i < nl; ++i) {
               all[k] = Lg[i];
               all[k].pin = (const void *const *)(S->d_ptrs + (size_t)Lg[i].pin);
               all[k].pout = (void *const *)(S->d_ptrs + (size_t)Lg[i].pout);
               ++k;
          }
          if (cudaMemcpy(S->d_items, all, sizeof(gb_qitem) * (size_t)S->nitems, cudaMemcpyHostToDevice) != cudaSuccess ||
              (nptr && cudaMemcpy(S->d_ptrs, hptr, sizeof(void *) * (size_t)nptr, cudaMemcpyHostToDevice) != cudaSuccess)) {
               free(all);
               gb_set_error("plan set: upload failed");
               gb_destroy_set(S);
               goto fail;
          }
          free(all);
     }
     free(QA.v); free(QM.v); free(QB.v); free(QL.v); free(hptr);
     return S;
fail:
     free(QA.v); free(QM.v); free(QB.v); free(QL.v); free(hptr);
     return 0;
}

/* Capture reset + queue launch into a CUDA graph on the set's stream. */
static int build_graph(gb_set *S)
{
     cudaStream_t st = 0;
     int own = 0, rc = 0;
     if (S->gexec) return 0;
     if (!S->stream) {
          if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return -1;
          own = 1;
     } else st = (cudaStream_t)S->stream;
     /* the status word the queue kernels report to is allocated on first
      * use, which must not happen inside the capture; so are the side stream
      * and its events */
     if (!gb_device_status_ptr()) rc = -1;
     if (!rc && S->nlarge && !S->side &&
         (cudaStreamCreateWithFlags(&S->side, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&S->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&S->ev_join, cudaEventDisableTiming) != cudaSuccess))
          rc = -1;
     if (!rc && cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = -1;
     if (!rc) {
          cudaMemsetAsync(S->d_head, 0, 2 * sizeof(int), st);
          if (S->nctr) cudaMemsetAsync(S->d_ctrs, 0, sizeof(int) * (size_t)S->nctr, st);
          if (S->nlarge) {
               /* the large-tile queue (no item of either queue waits on the
                * other's) on the side stream, captured first so its CTAs are
                * placed first; the small-tile queue's persistent CTAs fill
                * what is left and take the SMs the large tiles free */
               if (cudaEventRecord(S->ev_fork, st) != cudaSuccess ||
                   cudaStreamWaitEvent(S->side, S->ev_fork, 0) != cudaSuccess ||
                   gb_launch_queue(S->d_items + S->nsmall, S->nlarge, S->d_head + 1, S->d_ctrs, S->prec, S->threads_l,
                                   S->smem_l, S->grid_l, S->wait_ns, S->side) ||
                   cudaEventRecord(S->ev_join, S->side) != cudaSuccess)
                    rc = -1;
          }
          if (S->nsmall && gb_launch_queue(S->d_items, S->nsmall, S->d_head, S->d_ctrs, S->prec, S->threads,
                                           S->smem, S->grid, S->wait_ns, st))
               rc = -1;
          if (S->nlarge && cudaStreamWaitEvent(st, S->ev_join, 0) != cudaSuccess) rc = -1;
          if (cudaStreamEndCapture(st, &S->graph) != cudaSuccess) rc = -1;
     }
     if (!rc && cudaGraphInstantiate(&S->gexec, S->graph, 0) != cudaSuccess) rc = -1;
     if (own) cudaStreamDestroy(st);
     if (rc) {
          cudaGetLastError();
          gb_set_error("plan set: graph capture failed");
     }
     return rc;
}

int gb_execute_set(gb_set *S)
{
     cudaStream_t st = (cudaStream_t)S->stream;
     if (S->h_items) {
          gb_set_error("plan set: planned in dry run, cannot execute");
          return -1;
     }
     if (build_graph(S)) return -1;
     if (cudaGraphLaunch(S->gexec, st) != cudaSuccess) {
          gb_set_error("plan set: graph launch failed: %s", cudaGetErrorString(cudaGetLastError()));
          return -1;
     }
     if (!S->async && cudaStreamSynchronize(st) != cudaSuccess) {
          gb_set_error("plan set: %s", cudaGetErrorString(cudaGetLastError()));
          return -1;
     }
     return 0;
}

void gb_set_stream_of_set(gb_set *S, void *stream, int async)
{
     if (S->stream != stream) drop_graph(S);
     S->stream = stream;
     S->async = async;
}

static void drop_graph(gb_set *S)
{
     if (S->gexec) {
          cudaGraphExecDestroy(S->gexec);
          cudaGraphDestroy(S->graph);
          S->gexec = 0;
          S->graph = 0;
     }
}

/* Bound on the device-side wait of a row tile (the graph is re-captured
 * with the new limit on the next execute). */
int gb_set_wait_limit(gb_set *S, double seconds)
{
     if (!(seconds > 0) || seconds > 60) {
          gb_set_error("plan set: wait limit must be in (0, 60] seconds");
          return -1;
     }
     S->wait_ns = (unsigned long long)(seconds * 1e9);
     drop_graph(S);
     return 0;
}

/* Test hook for the bounded waits: on != 0 raises the wait target of the
 * set's first row tile one above what its column tiles will reach, so its
 * wait runs out on the next execute (GB_STATUS_QUEUE_TIMEOUT, the tile is
 * skipped); on == 0 puts the true target back.  Returns -1 when the set has
 * no row tile.  Only the device copy of the item changes. */
int gb_set_test_stall(gb_set *S, int on)
{
     const size_t off = offsetof(gb_qitem, wait_target);
     int i, v;
     if (S->h_items) {
          gb_set_error("plan set: planned in dry run");
          return -1;
     }
     if (on && S->stall_item < 0) {
          for (i = 0; i < S->nsmall && S->stall_item < 0; ++i) {
               gb_qitem it;
               if (cudaMemcpy(&it, S->d_items + i, sizeof it, cudaMemcpyDeviceToHost) != cudaSuccess) goto cuerr;
               if (it.wait_ctr >= 0) {
                    S->stall_item = i;
                    S->stall_target = it.wait_target;
               }
          }
          if (S->stall_item < 0) {
               gb_set_error("plan set: no row tile waits on a counter");
               return -1;
          }
          v = S->stall_target + 1;
          if (cudaMemcpy((char *)(S->d_items + S->stall_item) + off, &v, sizeof v, cudaMemcpyHostToDevice) != cudaSuccess)
               goto cuerr;
     } else if (!on && S->stall_item >= 0) {
          v = S->stall_target;
          if (cudaMemcpy((char *)(S->d_items + S->stall_item) + off, &v, sizeof v, cudaMemcpyHostToDevice) != cudaSuccess)
               goto cuerr;
          S->stall_item = -1;
     }
     return 0;
cuerr:
     gb_set_error("plan set: %s", cudaGetErrorString(cudaGetLastError()));
     return -1;
}

void gb_set_info(const gb_set *S, int *nitems, int *ntransforms, int *nlong, int *grid, int *smem)
{
     *nitems = S->nitems; *ntransforms = S->ntransforms; *nlong = S->nlong; *grid = S->grid; *smem = S->smem;
}

int gb_set_large_items(const gb_set *S) { return S->nlarge; }

/* Item i of the set in queue order (the small-tile queue's items, then the
 * large-tile queue's): its kind, FFT length, transforms, body (variant),
 * queue (0 small, 1 large) and role (1 a column tile others wait for, 2 a
 * row tile that waits, 0 a single).  Returns 0, or -1 for a bad index or a
 * failed read. */
int gb_set_item_info(const gb_set *S, int i, int *kind, int *nfft, int *tb, int *variant, int *queue, int *role)
{
     gb_qitem it;
     if (i < 0 || i >= S->nitems) {
          gb_set_error("plan set: no item %d", i);
          return -1;
     }
     if (S->h_items) it = S->h_items[i];
     else if (cudaMemcpy(&it, S->d_items + i, sizeof it, cudaMemcpyDeviceToHost) != cudaSuccess) {
          gb_set_error("plan set: %s", cudaGetErrorString(cudaGetLastError()));
          return -1;
     }
     *kind = it.P.kind;
     *nfft = it.P.nfft;
     *tb = it.P.tb;
     *variant = it.P.variant;
     *queue = i >= S->nsmall;
     *role = it.wait_ctr >= 0 ? 2 : it.signal_ctr >= 0 ? 1 : 0;
     return 0;
}

void gb_destroy_set(gb_set *S)
{
     if (!S) return;
     if (S->h_items) {
          /* a dry-run set holds no device resources */
          free(S->h_items);
          free(S);
          return;
     }
     if (S->gexec) cudaGraphExecDestroy(S->gexec);
     if (S->graph) cudaGraphDestroy(S->graph);
     if (S->side) cudaStreamDestroy(S->side);
     if (S->ev_fork) cudaEventDestroy(S->ev_fork);
     if (S->ev_join) cudaEventDestroy(S->ev_join);
     cudaFree(S->d_items);
     cudaFree(S->d_head);
     cudaFree(S->d_ctrs);
     cudaFree(S->d_ptrs);
     if (S->d_scratch) cudaFree(S->d_scratch);
     free(S);
}

/* ---- set tuner ---- */

static double set_now_s(void)
{
     struct timespec ts;
     clock_gettime(CLOCK_MONOTONIC, &ts);
     return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ms per execute (best of reps) of the set of transforms xs (on scratch
 * arrays) under the configurations wisdom now holds; 1e30 when it does not
 * build or run */
static double time_xforms(int prec, xform *xs, int cnt, cudaStream_t st, int reps)
{
     gb_set *S = build_set(prec, xs, cnt);
     double best = 1e30;
     int i;
     if (!S) return best;
     gb_set_stream_of_set(S, st, 1);
     if (!gb_execute_set(S)) {
          cudaEvent_t a, b;
          cudaEventCreate(&a);
          cudaEventCreate(&b);
          for (i = 0; i < reps; ++i) {
               float ms;
               cudaEventRecord(a, st);
               if (gb_execute_set(S)) { best = 1e30; break; }
               cudaEventRecord(b, st);
               if (cudaEventSynchronize(b) != cudaSuccess) { best = 1e30; break; }
               cudaEventElapsedTime(&ms, a, b);
               if (ms < best) best = ms;
          }
          cudaEventDestroy(a);
          cudaEventDestroy(b);
     }
     cudaStreamSynchronize(st);
     gb_destroy_set(S);
     return best;
}

/* a set of cnt transforms of length n alone, packed on the scratch arrays */
static double time_candidate(int prec, long long n, int sign, int cnt, char *din, char *dout, cudaStream_t st,
                             int reps)
{
     const int cs = 2 * prec;
     xform *xs = (xform *)malloc(sizeof(xform) * (size_t)cnt);
     double t;
     int i;
     if (!xs) return 1e30;
     for (i = 0; i < cnt; ++i) {
          xs[i].n = n; xs[i].sign = sign; xs[i].is = 1; xs[i].os = 1;
          xs[i].in = din + (size_t)i * (size_t)n * cs;
          xs[i].out = dout + (size_t)i * (size_t)n * cs;
     }
     t = time_xforms(prec, xs, cnt, st, reps);
     free(xs);
     return t;
}

/* Kinds of per-length choice, each of which the whole-set check keeps or
 * takes back as one. */
enum { CH_BODY, CH_PRIME, CH_SPLIT, CH_ORDER, CH_TILE, CH_KINDS };

static int entry_has(const gb_wisdom_entry *e, int kind)
{
     switch (kind) {
     case CH_BODY: return e->variant == GB_VAR_REG;
     case CH_PRIME: return e->variant == GB_KIND_RADER || e->variant == GB_KIND_BLUESTEIN;
     case CH_SPLIT: return e->n1 != 0;
     case CH_ORDER: return e->order != 0;
     default: return e->tb != 0;
     }
}

static void entry_reset(gb_wisdom_entry *e, int kind)
{
     switch (kind) {
     case CH_BODY:
     case CH_PRIME: e->variant = -1; break;
     case CH_SPLIT: e->n1 = 0; break;
     case CH_ORDER: e->order = 0; break;
     default: e->tb = 0; break;
     }
}

/* The per-length choices were timed on sets of one length; in the whole
 * set every item runs from one kernel, whose code for all item bodies
 * competes for the instruction cache, and items of all lengths share the
 * SMs.  So each kind of choice (register bodies, prime algorithms, splits,
 * radix orders, tiles) is timed once more on a scratch copy of the whole
 * set against the same set without it, and taken back when the whole set
 * runs more than 1% faster without it. */
typedef struct { long long n, pts; int sign; } lclass;

static void whole_set_check(int prec, const xform *xs, int nx, const lclass *cl, int ncl, cudaStream_t st, int reps)
{
     const int cs = 2 * prec;
     long long tot = 0, off = 0;
     char *din = 0, *dout = 0;
     xform *xw = 0;
     gb_wisdom_entry *ent = 0;
     int *has = 0, i, k, kind;
     double best;
     for (i = 0; i < nx; ++i) tot += xs[i].n;
     xw = (xform *)malloc(sizeof(xform) * (size_t)nx);
     ent = (gb_wisdom_entry *)malloc(sizeof(gb_wisdom_entry) * (size_t)ncl);
     has = (int *)malloc(sizeof(int) * (size_t)ncl);
     if (!xw || !ent || !has || cudaMalloc((void **)&din, (size_t)tot * cs) != cudaSuccess ||
         cudaMalloc((void **)&dout, (size_t)tot * cs) != cudaSuccess) {
          cudaGetLastError();
          goto done;
     }
     cudaMemset(din, 0, (size_t)tot * cs);
     for (i = 0; i < nx; ++i) {
          xw[i] = xs[i];
          xw[i].is = xw[i].os = 1;
          xw[i].in = din + (size_t)off * cs;
          xw[i].out = dout + (size_t)off * cs;
          off += xs[i].n;
     }
     /* each length's entry */
     for (k = 0; k < ncl; ++k) {
          char key[64];
          const gb_wisdom_entry *w;
          set_key(key, sizeof key, prec, cl[k].n);
          w = gb_wisdom_lookup(key);
          has[k] = w != 0;
          if (w) ent[k] = *w;
     }
     best = time_xforms(prec, xw, nx, st, reps);
     for (kind = 0; kind < CH_KINDS; ++kind) {
          int any = 0;
          double t;
          for (k = 0; k < ncl; ++k)
               if (has[k] && entry_has(&ent[k], kind)) {
                    gb_wisdom_entry e = ent[k];
                    entry_reset(&e, kind);
                    gb_wisdom_store(&e);
                    any = 1;
               }
          if (!any) continue;
          t = time_xforms(prec, xw, nx, st, reps);
          for (k = 0; k < ncl; ++k)
               if (has[k] && entry_has(&ent[k], kind)) {
                    if (t * 1.01 < best) entry_reset(&ent[k], kind);   /* the set is faster without them */
                    gb_wisdom_store(&ent[k]);
               }
          if (t * 1.01 < best) best = t;
     }
done:
     if (din) cudaFree(din);
     if (dout) cudaFree(dout);
     free(xw);
     free(ent);
     free(has);
}

/* a radix order whose stage list differs from the default's */
static int order_differs(long long n, int order)
{
     int r0[GB_MAXRAD], r1[GB_MAXRAD], k0 = gb_factor_radices(n, r0), k1 = gb_factor_order(n, r1, order), i;
     if (k1 < 0) return 0;
     if (k0 != k1) return 1;
     for (i = 0; i < k0; ++i)
          if (r0[i] != r1[i]) return 1;
     return 0;
}

static int cmp_class_pts(const void *a, const void *b)
{
     const lclass *x = (const lclass *)a, *y = (const lclass *)b;
     return x->pts < y->pts ? 1 : x->pts > y->pts ? -1 : 0;
}

/* Tune every length of the set that wisdom does not cover, lengths with
 * the most points first, within fftw_set_timelimit. */
static void tune_set(int prec, const xform *xs, int nx, unsigned flags)
{
     const int cap_s = cap_small(prec), cap_l = 2 * cap_s, cs = 2 * prec;
     const long long target = 1LL << 21;   /* points of a candidate's timing set */
     const int patient = (flags & (FFTW_PATIENT | FFTW_EXHAUSTIVE)) != 0, reps = patient ? 7 : 3;
     double t0 = set_now_s(), limit = gb_get_timelimit();
     xform *srt;
     lclass *cl;
     int ncl = 0, i, k, ntuned = 0;
     long long maxn = 0;
     char *din = 0, *dout = 0;
     cudaStream_t st = 0;
     if (nx <= 0) return;
     srt = (xform *)malloc(sizeof(xform) * (size_t)nx);
     cl = (lclass *)malloc(sizeof(lclass) * (size_t)nx);
     if (!srt || !cl) { free(srt); free(cl); return; }
     memcpy(srt, xs, sizeof(xform) * (size_t)nx);
     qsort(srt, (size_t)nx, sizeof(xform), cmp_key);
     for (i = 0; i < nx;) {
          int j = i;
          long long pts = 0;
          while (j < nx && srt[j].n == srt[i].n) pts += srt[j++].n;
          cl[ncl].n = srt[i].n; cl[ncl].sign = srt[i].sign; cl[ncl].pts = pts;
          if (srt[i].n > maxn) maxn = srt[i].n;
          ++ncl;
          i = j;
     }
     free(srt);
     qsort(cl, (size_t)ncl, sizeof(lclass), cmp_class_pts);
     {
          size_t bytes = (size_t)(maxn > target ? maxn : target) * cs;
          if (cudaMalloc((void **)&din, bytes) != cudaSuccess || cudaMalloc((void **)&dout, bytes) != cudaSuccess ||
              cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
               cudaGetLastError();
               goto done;
          }
          cudaMemset(din, 0, bytes);
     }
     for (k = 0; k < ncl; ++k) {
          const long long n = cl[k].n;
          char key[64];
          gb_wisdom_entry cand[8], best_e;
          int nc = 1, c, rad[GB_MAXRAD], cnt;
          const int smooth = gb_factor_radices(n, rad) >= 0, pow2 = (n & (n - 1)) == 0;
          double best = 1e30;
          if (limit > 0 && set_now_s() - t0 > limit) break;
          set_key(key, sizeof key, prec, n);
          if (gb_wisdom_lookup(key)) continue;
          memset(cand, 0, sizeof cand);
          for (c = 0; c < 8; ++c) cand[c].variant = -1;
          /* cand[0]: the defaults */
          if (smooth && n <= cap_s) {
               if (prec == 4 && pow2 && n >= 64 && n <= 4096) cand[nc++].variant = GB_VAR_REG;
               else if (!pow2)
                    for (c = 1; c < GB_RADIX_ORDERS; ++c)
                         if (order_differs(n, c)) cand[nc++].order = c;
               if (patient && n <= 1024) { cand[nc].tb = 8; ++nc; }
          } else if (smooth) {
               long long d[64], def = long_n1(n, cap_s, 0);
               int nd = long_splits(n, cap_s, d, 64), at = -1;
               for (c = 0; c < nd; ++c)
                    if (d[c] == def) at = c;
               if (at > 0) cand[nc++].n1 = (int)d[at - 1];
               if (at >= 0 && at + 1 < nd) cand[nc++].n1 = (int)d[at + 1];
               if (prec == 4 && pow2) cand[nc++].variant = GB_VAR_REG;
               if (patient) { cand[nc].tb = 8; ++nc; }
          } else if (is_prime_ll(n) && n - 1 <= cap_l && gb_factor_radices(n - 1, rad) >= 0 &&
                     pow2_at_least(2 * n - 1) <= cap_l) {
               /* the other algorithm than the planner's choice */
               int large;
               const int def = prime_kind(prec, n, cap_s, cap_l, 0, &large);
               cand[nc++].variant = def == GB_KIND_RADER ? GB_KIND_BLUESTEIN : GB_KIND_RADER;
          }
          best_e = cand[0];
          if (nc > 1) {
               cnt = (int)(target / n);
               if (cnt < 1) cnt = 1;
               for (c = 0; c < nc; ++c) {
                    double t;
                    if (c > 0 && limit > 0 && set_now_s() - t0 > limit) break;
                    strcpy(cand[c].key, key);
                    gb_wisdom_store(&cand[c]);
                    t = time_candidate(prec, n, cl[k].sign, cnt, din, dout, st, reps);
                    /* a set of one length alone only approximates the mix:
                     * another configuration replaces the defaults (cand[0])
                     * when it is faster by more than 5% */
                    if (c > 0) t *= 1.05;
                    if (t < best) { best = t; best_e = cand[c]; }
               }
          }
          strcpy(best_e.key, key);
          gb_wisdom_store(&best_e);
          ++ntuned;
     }
     if (ntuned && st) whole_set_check(prec, xs, nx, cl, ncl, st, reps);
done:
     if (st) cudaStreamDestroy(st);
     if (din) cudaFree(din);
     if (dout) cudaFree(dout);
     free(cl);
}
