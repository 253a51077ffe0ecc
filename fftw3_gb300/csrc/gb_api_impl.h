/*
 * Public API, written once and expanded for the fftw_ (double) and fftwf_
 * (float) prefixes by gb_api.c.  Each function keeps the reference's
 * signature, argument meaning and error behaviour:
 *   - invalid arguments (rank < 0, n[i] <= 0, howmany < 0) return NULL
 *     (api/mktensor-rowmajor.c:58-61);
 *   - strides: plan_many_* take istride/idist in elements of the input
 *     array and ostride/odist in elements of the output array
 *     (api/plan-many-dft.c:44-47, api/plan-many-dft-r2c.c:38-53);
 *   - r2c/c2r default embeddings pad the last dimension to n/2+1 complex
 *     or 2*(n/2+1) reals when in place (api/rdft2-pad.c:24-39);
 *   - an out-of-place c2r may destroy its input (api/plan-many-dft-c2r.c:41-42);
 *   - execute_dft & co. run the plan on new arrays of the same layout
 *     (api/execute-dft.c:25-32).
 * PFX(name) is the prefixed name, R the real type.
 */

typedef R PFX(cpx)[2];
/* view: how the plan was made — 0 complex interface; split interface as
 * 1 interleaved (ii = ri + 1, io = ro + 1: the complex plan on ri -> ro),
 * 2 swapped interleaved (ri = ii + 1: the backward complex plan on ii -> io),
 * 3 general split arrays (pack, c2c, unpack) */
struct PFX(plan_s) { gb_plan *g; int view; };

static PFX(plan) PFX(wrap)(gb_plan *g)
{
     PFX(plan) p;
     if (!g) return 0;
     p = (PFX(plan))malloc(sizeof *p);
     p->g = g;
     p->view = 0;
     return p;
}

static PFX(plan) PFX(mk)(gb_problem *prb, unsigned flags)
{
     gb_plan *g;
     char key[256];
     gb_problem_key(prb, key, sizeof key);
     gb_lock();
     if ((flags & FFTW_WISDOM_ONLY) && !gb_wisdom_lookup(key)) {
          /* the reference returns NULL when wisdom has no entry for the
           * problem (api/apiplan.c:102-107); the entry is the whole problem's
           * key, recorded when a problem of this exact shape was tuned */
          gb_unlock();
          gb_set_error("FFTW_WISDOM_ONLY: no wisdom for this problem");
          return 0;
     }
     g = gb_mkplan(prb, flags);
     if (g && !(flags & (FFTW_ESTIMATE | FFTW_WISDOM_ONLY)) && !gb_dry_run() && gb_tune(g, flags) == 0) {
          gb_wisdom_entry e;
          memset(&e, 0, sizeof e);
          snprintf(e.key, sizeof e.key, "%s", key);
          e.variant = -2;   /* a tuned problem, no pass choice of its own */
          gb_wisdom_store(&e);
     }
     gb_unlock();
     return PFX(wrap)(g);
}

static int PFX(kosher)(int rank, const int *n, int howmany)
{
     int i;
     if (rank < 0 || rank > GB_MAXRANK || howmany < 0) return 0;
     for (i = 0; i < rank; ++i)
          if (!n || n[i] <= 0) return 0;
     return 1;
}

/* row-major tensor with physical (embedding) sizes, strides in elements
 * (api/mktensor-rowmajor.c:23-41) */
static void PFX(rowmajor)(gb_problem *prb, int rank, const int *n, const int *niphys, const int *nophys,
                          long long is, long long os)
{
     int i;
     prb->rank = rank;
     if (rank <= 0) return;
     prb->sz[rank - 1].n = n[rank - 1];
     prb->sz[rank - 1].is = is;
     prb->sz[rank - 1].os = os;
     for (i = rank - 1; i > 0; --i) {
          prb->sz[i - 1].n = n[i - 1];
          prb->sz[i - 1].is = prb->sz[i].is * niphys[i];
          prb->sz[i - 1].os = prb->sz[i].os * nophys[i];
     }
}

PFX(plan) PFX(plan_many_dft)(int rank, const int *n, int howmany, C *in, const int *inembed, int istride,
                             int idist, C *out, const int *onembed, int ostride, int odist, int sign,
                             unsigned flags)
{
     gb_problem prb;
     if (!PFX(kosher)(rank, n, howmany)) return 0;
     if (sign != FFTW_FORWARD && sign != FFTW_BACKWARD) return 0;
     memset(&prb, 0, sizeof prb);
     prb.kind = GB_PROB_DFT; prb.prec = (int)sizeof(R); prb.sign = sign;
     PFX(rowmajor)(&prb, rank, n, inembed ? inembed : n, onembed ? onembed : n, istride, ostride);
     prb.vrank = 1;
     prb.vec[0].n = howmany; prb.vec[0].is = idist; prb.vec[0].os = odist;
     prb.in = in; prb.out = out;
     return PFX(mk)(&prb, flags);
}

PFX(plan) PFX(plan_dft)(int rank, const int *n, C *in, C *out, int sign, unsigned flags)
{
     return PFX(plan_many_dft)(rank, n, 1, in, 0, 1, 1, out, 0, 1, 1, sign, flags);
}
PFX(plan) PFX(plan_dft_1d)(int n, C *in, C *out, int sign, unsigned flags)
{
     return PFX(plan_dft)(1, &n, in, out, sign, flags);
}
PFX(plan) PFX(plan_dft_2d)(int n0, int n1, C *in, C *out, int sign, unsigned flags)
{
     int n[2] = {n0, n1};
     return PFX(plan_dft)(2, n, in, out, sign, flags);
}
PFX(plan) PFX(plan_dft_3d)(int n0, int n1, int n2, C *in, C *out, int sign, unsigned flags)
{
     int n[3] = {n0, n1, n2};
     return PFX(plan_dft)(3, n, in, out, sign, flags);
}

static PFX(plan) PFX(guru_common)(int kind, int rank, const long long *dn, const long long *dis,
                                  const long long *dos, int hrank, const long long *hn,
                                  const long long *his, const long long *hos, void *in, void *out,
                                  int sign, unsigned flags)
{
     gb_problem prb;
     int i;
     if (rank < 0 || rank > GB_MAXRANK || hrank < 0 || hrank > GB_MAXRANK) return 0;
     if ((kind == GB_PROB_R2C || kind == GB_PROB_C2R) && rank < 1) return 0;
     memset(&prb, 0, sizeof prb);
     prb.kind = kind; prb.prec = (int)sizeof(R); prb.sign = sign;
     prb.rank = rank;
     for (i = 0; i < rank; ++i) {
          if (dn[i] <= 0) return 0;
          prb.sz[i].n = dn[i]; prb.sz[i].is = dis[i]; prb.sz[i].os = dos[i];
     }
     prb.vrank = hrank;
     for (i = 0; i < hrank; ++i) {
          if (hn[i] < 0) return 0;
          prb.vec[i].n = hn[i]; prb.vec[i].is = his[i]; prb.vec[i].os = hos[i];
     }
     prb.in = in; prb.out = out;
     return PFX(mk)(&prb, flags);
}

#define GB_UNPACK(dims, k, N_, I_, O_)                                      \
     long long N_[GB_MAXRANK + 1], I_[GB_MAXRANK + 1], O_[GB_MAXRANK + 1]; \
     do {                                                                   \
          int q_;                                                           \
          if ((k) > GB_MAXRANK) return 0;                                   \
          for (q_ = 0; q_ < (k); ++q_) {                                    \
               N_[q_] = (dims)[q_].n; I_[q_] = (dims)[q_].is; O_[q_] = (dims)[q_].os; \
          }                                                                 \
     } while (0)

PFX(plan) PFX(plan_guru_dft)(int rank, const PFX(iodim) *dims, int howmany_rank, const PFX(iodim) *howmany_dims,
                             C *in, C *out, int sign, unsigned flags)
{
     if (sign != FFTW_FORWARD && sign != FFTW_BACKWARD) return 0;
     if (rank < 0 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(guru_common)(GB_PROB_DFT, rank, dn, dis, dos, howmany_rank, hn, his, hos, in, out, sign, flags);
          }
     }
}

PFX(plan) PFX(plan_guru64_dft)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                               const PFX(iodim64) *howmany_dims, C *in, C *out, int sign, unsigned flags)
{
     if (sign != FFTW_FORWARD && sign != FFTW_BACKWARD) return 0;
     if (rank < 0 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(guru_common)(GB_PROB_DFT, rank, dn, dis, dos, howmany_rank, hn, his, hos, in, out, sign, flags);
          }
     }
}

/* api/plan-guru-split-dft.h:23-38: the forward DFT of ri + i ii into
 * ro + i io, strides in reals (kind GB_PROB_DFT); r2c of ri into (ro, io)
 * and c2r of (ri, ii) into ro (api/plan-guru-split-dft-r2c.h,
 * api/plan-guru-split-dft-c2r.h). */
static PFX(plan) PFX(split_common)(int kind, int rank, const long long *dn, const long long *dis,
                                   const long long *dos, int hrank, const long long *hn, const long long *his,
                                   const long long *hos, R *ri, R *ii, R *ro, R *io_, unsigned flags)
{
     gb_dim d[GB_MAXRANK], v[GB_MAXRANK];
     int i, even = 1, ein = 1, eout = 1;
     if (rank < 0 || rank > GB_MAXRANK || hrank < 0 || hrank > GB_MAXRANK) return 0;
     if (kind != GB_PROB_DFT) {
          /* one complex side: interleaved (second array = first + 1, even
           * strides) makes it an ordinary r2c / c2r plan */
          if (rank < 1) return 0;
          for (i = 0; i < rank; ++i) {
               if (dn[i] <= 0) return 0;
               if (dis[i] % 2) ein = 0;
               if (dos[i] % 2) eout = 0;
          }
          for (i = 0; i < hrank; ++i) {
               if (hn[i] < 0) return 0;
               if (his[i] % 2) ein = 0;
               if (hos[i] % 2) eout = 0;
          }
          if ((kind == GB_PROB_R2C && eout && io_ - ro == 1) || (kind == GB_PROB_C2R && ein && ii - ri == 1)) {
               long long a[GB_MAXRANK], b[GB_MAXRANK], c[GB_MAXRANK], e[GB_MAXRANK];
               PFX(plan) p;
               for (i = 0; i < rank; ++i) {
                    a[i] = kind == GB_PROB_C2R ? dis[i] / 2 : dis[i];
                    b[i] = kind == GB_PROB_R2C ? dos[i] / 2 : dos[i];
               }
               for (i = 0; i < hrank; ++i) {
                    c[i] = kind == GB_PROB_C2R ? his[i] / 2 : his[i];
                    e[i] = kind == GB_PROB_R2C ? hos[i] / 2 : hos[i];
               }
               p = PFX(guru_common)(kind, rank, dn, a, b, hrank, hn, c, e, ri, ro,
                                    kind == GB_PROB_R2C ? FFTW_FORWARD : FFTW_BACKWARD, flags);
               if (p) p->view = 1;
               return p;
          }
          goto general;
     }
     for (i = 0; i < rank; ++i) {
          if (dn[i] <= 0) return 0;
          if (dis[i] % 2 || dos[i] % 2) even = 0;
     }
     for (i = 0; i < hrank; ++i) {
          if (hn[i] < 0) return 0;
          if (his[i] % 2 || hos[i] % 2) even = 0;
     }
     if (even && ((ii - ri == 1 && io_ - ro == 1) || (ri - ii == 1 && ro - io_ == 1))) {
          /* interleaved complex arrays: an ordinary plan on half the strides */
          const int swapped = (ri - ii == 1);
          long long a[GB_MAXRANK], b[GB_MAXRANK], c[GB_MAXRANK], e[GB_MAXRANK];
          PFX(plan) p;
          for (i = 0; i < rank; ++i) { a[i] = dis[i] / 2; b[i] = dos[i] / 2; }
          for (i = 0; i < hrank; ++i) { c[i] = his[i] / 2; e[i] = hos[i] / 2; }
          p = PFX(guru_common)(GB_PROB_DFT, rank, dn, a, b, hrank, hn, c, e, swapped ? (void *)ii : (void *)ri,
                               swapped ? (void *)io_ : (void *)ro, swapped ? FFTW_BACKWARD : FFTW_FORWARD, flags);
          if (p) p->view = swapped ? 2 : 1;
          return p;
     }
general:
     for (i = 0; i < rank; ++i) { d[i].n = dn[i]; d[i].is = dis[i]; d[i].os = dos[i]; }
     for (i = 0; i < hrank; ++i) { v[i].n = hn[i]; v[i].is = his[i]; v[i].os = hos[i]; }
     {
          gb_plan *g;
          PFX(plan) p;
          if (!gb_dry_run() && !gb_cuda_ready()) {
               gb_set_error("no CUDA device: libfftw3_gb300 runs transforms on the GPU only");
               return 0;
          }
          gb_lock();
          g = gb_mksplit(kind, (int)sizeof(R), rank, d, hrank, v, ri, ii, ro, io_, flags);
          if (g && !(flags & FFTW_ESTIMATE) && !gb_dry_run()) gb_tune(g->split_inner, flags);
          gb_unlock();
          p = PFX(wrap)(g);
          if (p) p->view = 3;
          return p;
     }
}

PFX(plan) PFX(plan_guru_split_dft)(int rank, const PFX(iodim) *dims, int howmany_rank,
                                   const PFX(iodim) *howmany_dims, R *ri, R *ii, R *ro, R *io_, unsigned flags)
{
     if (rank < 0 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(split_common)(GB_PROB_DFT, rank, dn, dis, dos, howmany_rank, hn, his, hos, ri, ii, ro, io_,
                                        flags);
          }
     }
}
PFX(plan) PFX(plan_guru64_split_dft)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                                     const PFX(iodim64) *howmany_dims, R *ri, R *ii, R *ro, R *io_, unsigned flags)
{
     if (rank < 0 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(split_common)(GB_PROB_DFT, rank, dn, dis, dos, howmany_rank, hn, his, hos, ri, ii, ro, io_,
                                        flags);
          }
     }
}

/* ---------------------------------------------------------------- r2c / c2r */

/* api/rdft2-pad.c:24-39 */
static const int *PFX(pad)(int rank, const int *n, const int *nembed, int inplace, int cmplx, int *buf)
{
     if (!nembed && rank > 0) {
          if (inplace || cmplx) {
               memcpy(buf, n, sizeof(int) * (size_t)rank);
               buf[rank - 1] = (n[rank - 1] / 2 + 1) * (1 + !cmplx);
               return buf;
          }
          return n;
     }
     return nembed;
}

PFX(plan) PFX(plan_many_dft_r2c)(int rank, const int *n, int howmany, R *in, const int *inembed, int istride,
                                 int idist, C *out, const int *onembed, int ostride, int odist, unsigned flags)
{
     gb_problem prb;
     int bi[GB_MAXRANK], bo[GB_MAXRANK];
     int inplace = (void *)in == (void *)out;
     if (!PFX(kosher)(rank, n, howmany) || rank < 1) return 0;
     memset(&prb, 0, sizeof prb);
     prb.kind = GB_PROB_R2C; prb.prec = (int)sizeof(R); prb.sign = FFTW_FORWARD;
     PFX(rowmajor)(&prb, rank, n, PFX(pad)(rank, n, inembed, inplace, 0, bi),
                   PFX(pad)(rank, n, onembed, inplace, 1, bo), istride, ostride);
     prb.vrank = 1;
     prb.vec[0].n = howmany; prb.vec[0].is = idist; prb.vec[0].os = odist;
     prb.in = in; prb.out = out;
     return PFX(mk)(&prb, flags);
}

PFX(plan) PFX(plan_many_dft_c2r)(int rank, const int *n, int howmany, C *in, const int *inembed, int istride,
                                 int idist, R *out, const int *onembed, int ostride, int odist, unsigned flags)
{
     gb_problem prb;
     int bi[GB_MAXRANK], bo[GB_MAXRANK];
     int inplace = (void *)in == (void *)out;
     if (!PFX(kosher)(rank, n, howmany) || rank < 1) return 0;
     if (!inplace) flags |= FFTW_DESTROY_INPUT;
     memset(&prb, 0, sizeof prb);
     prb.kind = GB_PROB_C2R; prb.prec = (int)sizeof(R); prb.sign = FFTW_BACKWARD;
     PFX(rowmajor)(&prb, rank, n, PFX(pad)(rank, n, inembed, inplace, 1, bi),
                   PFX(pad)(rank, n, onembed, inplace, 0, bo), istride, ostride);
     prb.vrank = 1;
     prb.vec[0].n = howmany; prb.vec[0].is = idist; prb.vec[0].os = odist;
     prb.in = in; prb.out = out;
     return PFX(mk)(&prb, flags);
}

PFX(plan) PFX(plan_dft_r2c)(int rank, const int *n, R *in, C *out, unsigned flags)
{
     return PFX(plan_many_dft_r2c)(rank, n, 1, in, 0, 1, 1, out, 0, 1, 1, flags);
}
PFX(plan) PFX(plan_dft_r2c_1d)(int n, R *in, C *out, unsigned flags) { return PFX(plan_dft_r2c)(1, &n, in, out, flags); }
PFX(plan) PFX(plan_dft_r2c_2d)(int n0, int n1, R *in, C *out, unsigned flags)
{
     int n[2] = {n0, n1};
     return PFX(plan_dft_r2c)(2, n, in, out, flags);
}
PFX(plan) PFX(plan_dft_r2c_3d)(int n0, int n1, int n2, R *in, C *out, unsigned flags)
{
     int n[3] = {n0, n1, n2};
     return PFX(plan_dft_r2c)(3, n, in, out, flags);
}
PFX(plan) PFX(plan_dft_c2r)(int rank, const int *n, C *in, R *out, unsigned flags)
{
     return PFX(plan_many_dft_c2r)(rank, n, 1, in, 0, 1, 1, out, 0, 1, 1, flags);
}
PFX(plan) PFX(plan_dft_c2r_1d)(int n, C *in, R *out, unsigned flags) { return PFX(plan_dft_c2r)(1, &n, in, out, flags); }
PFX(plan) PFX(plan_dft_c2r_2d)(int n0, int n1, C *in, R *out, unsigned flags)
{
     int n[2] = {n0, n1};
     return PFX(plan_dft_c2r)(2, n, in, out, flags);
}
PFX(plan) PFX(plan_dft_c2r_3d)(int n0, int n1, int n2, C *in, R *out, unsigned flags)
{
     int n[3] = {n0, n1, n2};
     return PFX(plan_dft_c2r)(3, n, in, out, flags);
}

PFX(plan) PFX(plan_guru_dft_r2c)(int rank, const PFX(iodim) *dims, int howmany_rank, const PFX(iodim) *howmany_dims,
                                 R *in, C *out, unsigned flags)
{
     if (rank < 1 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(guru_common)(GB_PROB_R2C, rank, dn, dis, dos, howmany_rank, hn, his, hos, in, out,
                                       FFTW_FORWARD, flags);
          }
     }
}
PFX(plan) PFX(plan_guru_dft_c2r)(int rank, const PFX(iodim) *dims, int howmany_rank, const PFX(iodim) *howmany_dims,
                                 C *in, R *out, unsigned flags)
{
     if (rank < 1 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(guru_common)(GB_PROB_C2R, rank, dn, dis, dos, howmany_rank, hn, his, hos, in, out,
                                       FFTW_BACKWARD, flags);
          }
     }
}
PFX(plan) PFX(plan_guru64_dft_r2c)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                                   const PFX(iodim64) *howmany_dims, R *in, C *out, unsigned flags)
{
     if (rank < 1 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(guru_common)(GB_PROB_R2C, rank, dn, dis, dos, howmany_rank, hn, his, hos, in, out,
                                       FFTW_FORWARD, flags);
          }
     }
}
PFX(plan) PFX(plan_guru64_dft_c2r)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                                   const PFX(iodim64) *howmany_dims, C *in, R *out, unsigned flags)
{
     if (rank < 1 || howmany_rank < 0) return 0;
     {
          GB_UNPACK(dims, rank, dn, dis, dos);
          {
               GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);
               return PFX(guru_common)(GB_PROB_C2R, rank, dn, dis, dos, howmany_rank, hn, his, hos, in, out,
                                       FFTW_BACKWARD, flags);
          }
     }
}

/* split-array r2c / c2r (api/plan-guru-split-dft-r2c.h,
 * api/plan-guru-split-dft-c2r.h; 64-bit variants api/plan-guru64-*) */
#define GB_SPLIT_REAL(kind, a0, a1, a2, a3)                                                   \
     do {                                                                                 \
          if (rank < 0 || howmany_rank < 0) return 0;                                     \
          {                                                                               \
               GB_UNPACK(dims, rank, dn, dis, dos);                                       \
               {                                                                          \
                    GB_UNPACK(howmany_dims, howmany_rank, hn, his, hos);                  \
                    return PFX(split_common)(kind, rank, dn, dis, dos, howmany_rank, hn, his, hos, a0, \
                                             a1, a2, a3, flags);                          \
               }                                                                          \
          }                                                                               \
     } while (0)
PFX(plan) PFX(plan_guru_split_dft_r2c)(int rank, const PFX(iodim) *dims, int howmany_rank,
                                       const PFX(iodim) *howmany_dims, R *in, R *ro, R *io_, unsigned flags)
{
     GB_SPLIT_REAL(GB_PROB_R2C, in, 0, ro, io_);
}
PFX(plan) PFX(plan_guru_split_dft_c2r)(int rank, const PFX(iodim) *dims, int howmany_rank,
                                       const PFX(iodim) *howmany_dims, R *ri, R *ii, R *out, unsigned flags)
{
     GB_SPLIT_REAL(GB_PROB_C2R, ri, ii, out, 0);
}
PFX(plan) PFX(plan_guru64_split_dft_r2c)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                                         const PFX(iodim64) *howmany_dims, R *in, R *ro, R *io_, unsigned flags)
{
     GB_SPLIT_REAL(GB_PROB_R2C, in, 0, ro, io_);
}
PFX(plan) PFX(plan_guru64_split_dft_c2r)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                                         const PFX(iodim64) *howmany_dims, R *ri, R *ii, R *out, unsigned flags)
{
     GB_SPLIT_REAL(GB_PROB_C2R, ri, ii, out, 0);
}
/* r2r of any rank (rank 0: a copy) with any howmany rank (api/plan-many-r2r.c,
 * api/plan-r2r.c, api/plan-r2r-1d/2d/3d.c, api/plan-guru-r2r.h); strides and
 * distances count reals; one kind per transform dim. */
static PFX(plan) PFX(r2r_common)(int rank, const gb_dim *dims, const int *kinds, int vrank, const gb_dim *vdims,
                                 R *in, R *out, unsigned flags)
{
     gb_plan *g;
     PFX(plan) p;
     if (!gb_dry_run() && !gb_cuda_ready()) {
          gb_set_error("no CUDA device: libfftw3_gb300 runs transforms on the GPU only");
          return 0;
     }
     gb_lock();
     g = gb_mkr2r((int)sizeof(R), rank, dims, kinds, vrank, vdims, in, out, flags);
     if (g && !(flags & FFTW_ESTIMATE) && !gb_dry_run()) gb_r2r_tune(g, flags);
     gb_unlock();
     p = PFX(wrap)(g);
     if (p) p->view = 4;
     return p;
}

PFX(plan) PFX(plan_many_r2r)(int rank, const int *n, int howmany, R *in, const int *inembed, int istride, int idist,
                             R *out, const int *onembed, int ostride, int odist, const PFX(r2r_kind) *kind,
                             unsigned flags)
{
     gb_problem prb;
     gb_dim v;
     int k[GB_MAXRANK], d;
     if (!PFX(kosher)(rank, n, howmany) || !kind) return 0;
     if (rank > GB_MAXRANK) {
          gb_set_error("r2r of rank %d is not provided by this library (rank 0..%d)", rank, GB_MAXRANK);
          return 0;
     }
     memset(&prb, 0, sizeof prb);
     PFX(rowmajor)(&prb, rank, n, inembed ? inembed : n, onembed ? onembed : n, istride, ostride);
     for (d = 0; d < rank; ++d) k[d] = (int)kind[d];
     v.n = howmany; v.is = idist; v.os = odist;
     return PFX(r2r_common)(rank, prb.sz, k, 1, &v, in, out, flags);
}
PFX(plan) PFX(plan_r2r)(int rank, const int *n, R *in, R *out, const PFX(r2r_kind) *kind, unsigned flags)
{
     return PFX(plan_many_r2r)(rank, n, 1, in, 0, 1, 0, out, 0, 1, 0, kind, flags);
}
PFX(plan) PFX(plan_r2r_1d)(int n, R *in, R *out, PFX(r2r_kind) kind, unsigned flags)
{
     return PFX(plan_r2r)(1, &n, in, out, &kind, flags);
}
PFX(plan) PFX(plan_r2r_2d)(int n0, int n1, R *in, R *out, PFX(r2r_kind) kind0, PFX(r2r_kind) kind1, unsigned flags)
{
     const int n[2] = {n0, n1};
     const PFX(r2r_kind) k[2] = {kind0, kind1};
     return PFX(plan_r2r)(2, n, in, out, k, flags);
}
PFX(plan) PFX(plan_r2r_3d)(int n0, int n1, int n2, R *in, R *out, PFX(r2r_kind) kind0, PFX(r2r_kind) kind1,
                           PFX(r2r_kind) kind2, unsigned flags)
{
     const int n[3] = {n0, n1, n2};
     const PFX(r2r_kind) k[3] = {kind0, kind1, kind2};
     return PFX(plan_r2r)(3, n, in, out, k, flags);
}
#define GB_R2R_GURU(dims, rank, howmany_dims, howmany_rank)                                 \
     do {                                                                                    \
          gb_dim dd_[GB_MAXRANK], vv_[GB_MAXRANK];                                           \
          int kk_[GB_MAXRANK], q_;                                                           \
          if (rank < 0 || rank > GB_MAXRANK || howmany_rank < 0 || howmany_rank > GB_MAXRANK) { \
               gb_set_error("r2r of rank %d / howmany rank %d is not provided by this library", \
                            rank, howmany_rank);                                             \
               return 0;                                                                     \
          }                                                                                  \
          if ((rank > 0 && (!dims || !kind)) || (howmany_rank > 0 && !howmany_dims)) return 0; \
          for (q_ = 0; q_ < rank; ++q_) {                                                    \
               dd_[q_].n = (dims)[q_].n; dd_[q_].is = (dims)[q_].is; dd_[q_].os = (dims)[q_].os; \
               kk_[q_] = (int)kind[q_];                                                      \
          }                                                                                  \
          for (q_ = 0; q_ < howmany_rank; ++q_) {                                            \
               vv_[q_].n = (howmany_dims)[q_].n; vv_[q_].is = (howmany_dims)[q_].is;         \
               vv_[q_].os = (howmany_dims)[q_].os;                                           \
          }                                                                                  \
          return PFX(r2r_common)(rank, dd_, kk_, howmany_rank, vv_, in, out, flags);         \
     } while (0)
PFX(plan) PFX(plan_guru_r2r)(int rank, const PFX(iodim) *dims, int howmany_rank, const PFX(iodim) *howmany_dims,
                             R *in, R *out, const PFX(r2r_kind) *kind, unsigned flags)
{
     GB_R2R_GURU(dims, rank, howmany_dims, howmany_rank);
}
PFX(plan) PFX(plan_guru64_r2r)(int rank, const PFX(iodim64) *dims, int howmany_rank,
                               const PFX(iodim64) *howmany_dims, R *in, R *out, const PFX(r2r_kind) *kind,
                               unsigned flags)
{
     GB_R2R_GURU(dims, rank, howmany_dims, howmany_rank);
}

/* ---------------------------------------------------------------- execute */

static void PFX(run)(const PFX(plan) p, void *in, void *out, int kind)
{
     if (!p) return;
     if (p->view >= 3) {
          gb_set_error("execute: a split-array or r2r plan runs through execute, execute_split_dft or execute_r2r");
          fprintf(stderr, "[fftw_gb300] %s\n", gb_last_error());
          return;
     }
     if (kind >= 0 && p->g->prb.kind != kind) {
          gb_set_error("execute: plan kind does not match the new-array execute function");
          fprintf(stderr, "[fftw_gb300] %s\n", gb_last_error());
          return;
     }
     if (gb_execute(p->g, in, out)) {
          gb_note_failure();
          fprintf(stderr, "[fftw_gb300] execute failed: %s\n", gb_last_error());
     }
}

static void PFX(run_split)(const PFX(plan) p, R *ri, R *ii, R *ro, R *io_)
{
     if (gb_execute_split(p->g, ri, ii, ro, io_)) {
          gb_note_failure();
          fprintf(stderr, "[fftw_gb300] execute failed: %s\n", gb_last_error());
     }
}

void PFX(execute)(const PFX(plan) p)
{
     if (!p) return;
     if (p->view == 3)
          PFX(run_split)(p, (R *)p->g->split_arr[0], (R *)p->g->split_arr[1], (R *)p->g->split_arr[2],
                         (R *)p->g->split_arr[3]);
     else if (p->view == 4) PFX(execute_r2r)(p, (R *)p->g->prb.in, (R *)p->g->prb.out);
     else PFX(run)(p, p->g->prb.in, p->g->prb.out, -1);
}
void PFX(execute_dft)(const PFX(plan) p, C *in, C *out) { PFX(run)(p, in, out, GB_PROB_DFT); }
void PFX(execute_dft_r2c)(const PFX(plan) p, R *in, C *out) { PFX(run)(p, in, out, GB_PROB_R2C); }
void PFX(execute_dft_c2r)(const PFX(plan) p, C *in, R *out) { PFX(run)(p, in, out, GB_PROB_C2R); }
/* api/execute-split-dft.c:23-27: the plan's transform on new split arrays
 * of the same layout */
void PFX(execute_split_dft)(const PFX(plan) p, R *ri, R *ii, R *ro, R *io_)
{
     if (!p) return;
     if (p->view == 3 && p->g->split_kind == GB_PROB_DFT) PFX(run_split)(p, ri, ii, ro, io_);
     else if (p->view == 1) PFX(run)(p, ri, ro, GB_PROB_DFT);
     else if (p->view == 2) PFX(run)(p, ii, io_, GB_PROB_DFT);
     else {
          gb_set_error("execute_split_dft: the plan was not made by the split-array interface");
          fprintf(stderr, "[fftw_gb300] %s\n", gb_last_error());
     }
}
/* api/execute-split-dft-r2c.c, api/execute-split-dft-c2r.c */
void PFX(execute_split_dft_r2c)(const PFX(plan) p, R *in, R *ro, R *io_)
{
     if (!p) return;
     if (p->view == 3 && p->g->split_kind == GB_PROB_R2C) PFX(run_split)(p, in, 0, ro, io_);
     else if (p->view == 1 && p->g->prb.kind == GB_PROB_R2C) PFX(run)(p, in, ro, GB_PROB_R2C);
     else {
          gb_set_error("execute_split_dft_r2c: the plan was not made by plan_guru_split_dft_r2c");
          fprintf(stderr, "[fftw_gb300] %s\n", gb_last_error());
     }
}
void PFX(execute_split_dft_c2r)(const PFX(plan) p, R *ri, R *ii, R *out)
{
     if (!p) return;
     if (p->view == 3 && p->g->split_kind == GB_PROB_C2R) PFX(run_split)(p, ri, ii, out, 0);
     else if (p->view == 1 && p->g->prb.kind == GB_PROB_C2R) PFX(run)(p, ri, out, GB_PROB_C2R);
     else {
          gb_set_error("execute_split_dft_c2r: the plan was not made by plan_guru_split_dft_c2r");
          fprintf(stderr, "[fftw_gb300] %s\n", gb_last_error());
     }
}
/* api/execute-r2r.c: the plan's transform on new arrays of the same layout */
void PFX(execute_r2r)(const PFX(plan) p, R *in, R *out)
{
     if (!p) return;
     if (p->view != 4) {
          gb_set_error("execute_r2r: the plan is not an r2r plan");
          fprintf(stderr, "[fftw_gb300] %s\n", gb_last_error());
          return;
     }
     if (gb_execute_r2r(p->g, in, out)) {
          gb_note_failure();
          fprintf(stderr, "[fftw_gb300] execute failed: %s\n", gb_last_error());
     }
}

PFX(plan) PFX(copy_plan)(PFX(plan) p)
{
     if (p) {
          gb_lock();
          p->g->refcnt++;
          gb_unlock();
          {
               PFX(plan) q = (PFX(plan))malloc(sizeof *q);
               q->g = p->g;
               q->view = p->view;
               return q;
          }
     }
     return p;
}

void PFX(destroy_plan)(PFX(plan) p)
{
     if (!p) return;
     gb_lock();
     if (--p->g->refcnt == 0) gb_destroy(p->g);
     gb_unlock();
     free(p);
}

/* ---------------------------------------------------------------- misc */
void PFX(forget_wisdom)(void) { gb_lock(); gb_wisdom_forget(); gb_unlock(); }
void PFX(cleanup)(void) { gb_lock(); gb_wisdom_forget(); gb_cleanup_tables(); gb_unlock(); }
void PFX(set_timelimit)(double t) { gb_set_timelimit(t); }
void PFX(plan_with_nthreads)(int nthreads) { gb_set_nthreads(nthreads); }
int PFX(planner_nthreads)(void) { return gb_get_nthreads(); }
int PFX(init_threads)(void) { return 1; }
void PFX(cleanup_threads)(void) {}
void PFX(threads_set_callback)(void (*parallel_loop)(void *(*work)(char *), char *jobdata, size_t elsize,
                                                     int njobs, void *data), void *data)
{
     (void)parallel_loop; (void)data;
}
void PFX(make_planner_thread_safe)(void) {}

static void PFX(emit_file)(char c, void *d) { putc(c, (FILE *)d); }
typedef struct { char *s; size_t n, cap; } PFX(sbuf);
static void PFX(emit_str)(char c, void *d)
{
     PFX(sbuf) *b = (PFX(sbuf) *)d;
     if (b->n + 2 > b->cap) { b->cap = b->cap ? 2 * b->cap : 256; b->s = (char *)realloc(b->s, b->cap); }
     b->s[b->n++] = c;
     b->s[b->n] = 0;
}
void PFX(export_wisdom)(PFX(write_char_func) write_char, void *data)
{
     gb_lock();
     gb_wisdom_export((int)sizeof(R), (void (*)(char, void *))write_char, data);
     gb_unlock();
}
void PFX(export_wisdom_to_file)(FILE *f) { PFX(export_wisdom)(PFX(emit_file), f); }
char *PFX(export_wisdom_to_string)(void)
{
     PFX(sbuf) b = {0, 0, 0};
     PFX(export_wisdom)(PFX(emit_str), &b);
     if (!b.s) { b.s = (char *)malloc(1); b.s[0] = 0; }
     return b.s;
}
int PFX(export_wisdom_to_filename)(const char *filename)
{
     FILE *f = fopen(filename, "w");
     if (!f) return 0;
     PFX(export_wisdom_to_file)(f);
     return fclose(f) == 0;
}
int PFX(import_wisdom)(PFX(read_char_func) read_char, void *data)
{
     int r;
     gb_lock();
     r = gb_wisdom_import((int)sizeof(R), (int (*)(void *))read_char, data);
     gb_unlock();
     return r;
}
static int PFX(get_file)(void *d) { return getc((FILE *)d); }
typedef struct { const char *s; } PFX(scur);
static int PFX(get_str)(void *d)
{
     PFX(scur) *c = (PFX(scur) *)d;
     return *c->s ? (unsigned char)*c->s++ : EOF;
}
int PFX(import_wisdom_from_file)(FILE *f) { return f ? PFX(import_wisdom)(PFX(get_file), f) : 0; }
int PFX(import_wisdom_from_string)(const char *s)
{
     PFX(scur) c;
     if (!s) return 0;
     c.s = s;
     return PFX(import_wisdom)(PFX(get_str), &c);
}
int PFX(import_wisdom_from_filename)(const char *filename)
{
     FILE *f = fopen(filename, "r");
     int r;
     if (!f) return 0;
     r = PFX(import_wisdom_from_file)(f);
     fclose(f);
     return r;
}
int PFX(import_system_wisdom)(void)
{
     return PFX(import_wisdom_from_filename)(sizeof(R) == 4 ? "/etc/fftw/wisdomf" : "/etc/fftw/wisdom");
}

void PFX(fprint_plan)(const PFX(plan) p, FILE *f)
{
     if (p) fputs(p->g->desc, f);
}
void PFX(print_plan)(const PFX(plan) p) { PFX(fprint_plan)(p, stdout); }
char *PFX(sprint_plan)(const PFX(plan) p)
{
     char *s;
     if (!p) return 0;
     s = (char *)malloc(strlen(p->g->desc) + 1);
     strcpy(s, p->g->desc);
     return s;
}

void *PFX(malloc)(size_t n) { return gb_malloc(n); }
R *PFX(alloc_real)(size_t n) { return (R *)gb_malloc(sizeof(R) * n); }
C *PFX(alloc_complex)(size_t n) { return (C *)gb_malloc(sizeof(C) * n); }
void PFX(free)(void *p) { gb_free(p); }

void PFX(flops)(const PFX(plan) p, double *add, double *mul, double *fmas)
{
     if (!p) { *add = *mul = *fmas = 0; return; }
     *add = p->g->add; *mul = p->g->mul; *fmas = p->g->fma;
}
double PFX(estimate_cost)(const PFX(plan) p) { return p ? p->g->add + p->g->mul + 2 * p->g->fma : 0; }
double PFX(cost)(const PFX(plan) p) { return p ? p->g->measured_ms : 0; }
int PFX(alignment_of)(R *p) { return (int)((uintptr_t)p % 16); }
