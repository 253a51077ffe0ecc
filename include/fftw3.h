/*
 * fftw3.h -- public C ABI of libfftw3_gb300, a GB300-native implementation of
 * FFTW's execute hot path (c2c / r2c / c2r plans and their execution).
 *
 * Every function, type and flag value here is the one the reference FFTW
 * 3.3.x declares in api/fftw3.h (the FFTW_DEFINE_API prototype list,
 * api/fftw3.h:127-466, instantiated for the fftw_ and fftwf_ prefixes at
 * api/fftw3.h:468-470; flag bits api/fftw3.h:489-519).  A program written
 * against the reference header compiles unchanged against this one and links
 * with -lfftw3_gb300 instead of -lfftw3 -lfftw3f (-lfftw3_threads).
 *
 * What runs on the GPU (hand-written sm_103a kernels, no cuFFT):
 *   plan_dft{,_1d,_2d,_3d}, plan_many_dft, plan_guru_dft, plan_guru64_dft,
 *   plan_dft_r2c{,_1d,_2d,_3d}, plan_many_dft_r2c, plan_guru{,64}_dft_r2c,
 *   plan_dft_c2r{,_1d,_2d,_3d}, plan_many_dft_c2r, plan_guru{,64}_dft_c2r,
 *   execute, execute_dft, execute_dft_r2c, execute_dft_c2r;
 *   plan_guru{,64}_split_dft{,_r2c,_c2r}, execute_split_dft{,_r2c,_c2r}
 *   (split real / imaginary arrays);
 *   plan_r2r{,_1d,_2d,_3d}, plan_many_r2r, plan_guru{,64}_r2r, execute_r2r
 *   (all eleven r2r kinds, any rank).
 * Every execute_* entry point does nothing on a NULL plan.
 *
 * Pointer model: arrays may be device memory (cudaMalloc, managed) or host
 * memory (malloc, fftw_malloc).  Host arrays are staged through device
 * buffers inside execute; device arrays are transformed in place in HBM.
 * execute returns when the result is visible to the caller.
 *
 * Extensions beyond the reference API are in fftw3_gb300.h.
 */
#ifndef FFTW3_H
#define FFTW3_H

#include <stdio.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* api/fftw3.h:95-99 */
enum fftw_r2r_kind_do_not_use_me {
     FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2,
     FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6,
     FFTW_RODFT00 = 7, FFTW_RODFT01 = 8, FFTW_RODFT10 = 9, FFTW_RODFT11 = 10
};

/* api/fftw3.h:101-112 */
struct fftw_iodim_do_not_use_me { int n; int is; int os; };
struct fftw_iodim64_do_not_use_me { ptrdiff_t n; ptrdiff_t is; ptrdiff_t os; };

typedef void (*fftw_write_char_func_do_not_use_me)(char c, void *);
typedef int (*fftw_read_char_func_do_not_use_me)(void *);

/* One prototype list, expanded per precision (the reference does the same
 * with FFTW_DEFINE_API, api/fftw3.h:127-466). */
#define GB_FFTW_DECLARE(PFX, R, C)                                                          \
typedef R C[2];                                                                             \
typedef struct PFX##plan_s *PFX##plan;                                                      \
typedef struct fftw_iodim_do_not_use_me PFX##iodim;                                         \
typedef struct fftw_iodim64_do_not_use_me PFX##iodim64;                                     \
typedef enum fftw_r2r_kind_do_not_use_me PFX##r2r_kind;                                     \
typedef fftw_write_char_func_do_not_use_me PFX##write_char_func;                            \
typedef fftw_read_char_func_do_not_use_me PFX##read_char_func;                              \
extern void PFX##execute(const PFX##plan p);                                                \
extern PFX##plan PFX##plan_dft(int rank, const int *n, C *in, C *out, int sign,             \
                               unsigned flags);                                             \
extern PFX##plan PFX##plan_dft_1d(int n, C *in, C *out, int sign, unsigned flags);          \
extern PFX##plan PFX##plan_dft_2d(int n0, int n1, C *in, C *out, int sign, unsigned flags); \
extern PFX##plan PFX##plan_dft_3d(int n0, int n1, int n2, C *in, C *out, int sign,          \
                                  unsigned flags);                                          \
extern PFX##plan PFX##plan_many_dft(int rank, const int *n, int howmany,                    \
                                    C *in, const int *inembed, int istride, int idist,      \
                                    C *out, const int *onembed, int ostride, int odist,     \
                                    int sign, unsigned flags);                              \
extern PFX##plan PFX##plan_guru_dft(int rank, const PFX##iodim *dims, int howmany_rank,     \
                                    const PFX##iodim *howmany_dims, C *in, C *out,          \
                                    int sign, unsigned flags);                              \
extern PFX##plan PFX##plan_guru_split_dft(int rank, const PFX##iodim *dims,                 \
                                          int howmany_rank, const PFX##iodim *howmany_dims, \
                                          R *ri, R *ii, R *ro, R *io, unsigned flags);      \
extern PFX##plan PFX##plan_guru64_dft(int rank, const PFX##iodim64 *dims,                   \
                                      int howmany_rank, const PFX##iodim64 *howmany_dims,   \
                                      C *in, C *out, int sign, unsigned flags);             \
extern PFX##plan PFX##plan_guru64_split_dft(int rank, const PFX##iodim64 *dims,             \
                                            int howmany_rank,                               \
                                            const PFX##iodim64 *howmany_dims,               \
                                            R *ri, R *ii, R *ro, R *io, unsigned flags);    \
extern void PFX##execute_dft(const PFX##plan p, C *in, C *out);                             \
extern void PFX##execute_split_dft(const PFX##plan p, R *ri, R *ii, R *ro, R *io);          \
extern PFX##plan PFX##plan_many_dft_r2c(int rank, const int *n, int howmany,                \
                                        R *in, const int *inembed, int istride, int idist,  \
                                        C *out, const int *onembed, int ostride, int odist, \
                                        unsigned flags);                                    \
extern PFX##plan PFX##plan_dft_r2c(int rank, const int *n, R *in, C *out, unsigned flags);  \
extern PFX##plan PFX##plan_dft_r2c_1d(int n, R *in, C *out, unsigned flags);                \
extern PFX##plan PFX##plan_dft_r2c_2d(int n0, int n1, R *in, C *out, unsigned flags);       \
extern PFX##plan PFX##plan_dft_r2c_3d(int n0, int n1, int n2, R *in, C *out,                \
                                      unsigned flags);                                      \
extern PFX##plan PFX##plan_many_dft_c2r(int rank, const int *n, int howmany,                \
                                        C *in, const int *inembed, int istride, int idist,  \
                                        R *out, const int *onembed, int ostride, int odist, \
                                        unsigned flags);                                    \
extern PFX##plan PFX##plan_dft_c2r(int rank, const int *n, C *in, R *out, unsigned flags);  \
extern PFX##plan PFX##plan_dft_c2r_1d(int n, C *in, R *out, unsigned flags);                \
extern PFX##plan PFX##plan_dft_c2r_2d(int n0, int n1, C *in, R *out, unsigned flags);       \
extern PFX##plan PFX##plan_dft_c2r_3d(int n0, int n1, int n2, C *in, R *out,                \
                                      unsigned flags);                                      \
extern PFX##plan PFX##plan_guru_dft_r2c(int rank, const PFX##iodim *dims, int howmany_rank, \
                                        const PFX##iodim *howmany_dims, R *in, C *out,      \
                                        unsigned flags);                                    \
extern PFX##plan PFX##plan_guru_dft_c2r(int rank, const PFX##iodim *dims, int howmany_rank, \
                                        const PFX##iodim *howmany_dims, C *in, R *out,      \
                                        unsigned flags);                                    \
extern PFX##plan PFX##plan_guru_split_dft_r2c(int rank, const PFX##iodim *dims,             \
                                              int howmany_rank,                             \
                                              const PFX##iodim *howmany_dims,               \
                                              R *in, R *ro, R *io, unsigned flags);         \
extern PFX##plan PFX##plan_guru_split_dft_c2r(int rank, const PFX##iodim *dims,             \
                                              int howmany_rank,                             \
                                              const PFX##iodim *howmany_dims,               \
                                              R *ri, R *ii, R *out, unsigned flags);        \
extern PFX##plan PFX##plan_guru64_dft_r2c(int rank, const PFX##iodim64 *dims,               \
                                          int howmany_rank,                                 \
                                          const PFX##iodim64 *howmany_dims,                 \
                                          R *in, C *out, unsigned flags);                   \
extern PFX##plan PFX##plan_guru64_dft_c2r(int rank, const PFX##iodim64 *dims,               \
                                          int howmany_rank,                                 \
                                          const PFX##iodim64 *howmany_dims,                 \
                                          C *in, R *out, unsigned flags);                   \
extern PFX##plan PFX##plan_guru64_split_dft_r2c(int rank, const PFX##iodim64 *dims,         \
                                                int howmany_rank,                           \
                                                const PFX##iodim64 *howmany_dims,           \
                                                R *in, R *ro, R *io, unsigned flags);       \
extern PFX##plan PFX##plan_guru64_split_dft_c2r(int rank, const PFX##iodim64 *dims,         \
                                                int howmany_rank,                           \
                                                const PFX##iodim64 *howmany_dims,           \
                                                R *ri, R *ii, R *out, unsigned flags);      \
extern void PFX##execute_dft_r2c(const PFX##plan p, R *in, C *out);                         \
extern void PFX##execute_dft_c2r(const PFX##plan p, C *in, R *out);                         \
extern void PFX##execute_split_dft_r2c(const PFX##plan p, R *in, R *ro, R *io);             \
extern void PFX##execute_split_dft_c2r(const PFX##plan p, R *ri, R *ii, R *out);            \
extern PFX##plan PFX##plan_many_r2r(int rank, const int *n, int howmany,                    \
                                    R *in, const int *inembed, int istride, int idist,      \
                                    R *out, const int *onembed, int ostride, int odist,     \
                                    const PFX##r2r_kind *kind, unsigned flags);             \
extern PFX##plan PFX##plan_r2r(int rank, const int *n, R *in, R *out,                       \
                               const PFX##r2r_kind *kind, unsigned flags);                  \
extern PFX##plan PFX##plan_r2r_1d(int n, R *in, R *out, PFX##r2r_kind kind,                 \
                                  unsigned flags);                                          \
extern PFX##plan PFX##plan_r2r_2d(int n0, int n1, R *in, R *out, PFX##r2r_kind kind0,       \
                                  PFX##r2r_kind kind1, unsigned flags);                     \
extern PFX##plan PFX##plan_r2r_3d(int n0, int n1, int n2, R *in, R *out,                    \
                                  PFX##r2r_kind kind0, PFX##r2r_kind kind1,                 \
                                  PFX##r2r_kind kind2, unsigned flags);                     \
extern PFX##plan PFX##plan_guru_r2r(int rank, const PFX##iodim *dims, int howmany_rank,     \
                                    const PFX##iodim *howmany_dims, R *in, R *out,          \
                                    const PFX##r2r_kind *kind, unsigned flags);             \
extern PFX##plan PFX##plan_guru64_r2r(int rank, const PFX##iodim64 *dims,                   \
                                      int howmany_rank, const PFX##iodim64 *howmany_dims,   \
                                      R *in, R *out, const PFX##r2r_kind *kind,             \
                                      unsigned flags);                                      \
extern void PFX##execute_r2r(const PFX##plan p, R *in, R *out);                             \
extern PFX##plan PFX##copy_plan(PFX##plan p);                                               \
extern void PFX##destroy_plan(PFX##plan p);                                                 \
extern void PFX##forget_wisdom(void);                                                       \
extern void PFX##cleanup(void);                                                             \
extern void PFX##set_timelimit(double t);                                                   \
extern void PFX##plan_with_nthreads(int nthreads);                                          \
extern int PFX##planner_nthreads(void);                                                     \
extern int PFX##init_threads(void);                                                         \
extern void PFX##cleanup_threads(void);                                                     \
extern void PFX##threads_set_callback(void (*parallel_loop)(void *(*work)(char *),          \
                                      char *jobdata, size_t elsize, int njobs, void *data), \
                                      void *data);                                          \
extern void PFX##make_planner_thread_safe(void);                                            \
extern int PFX##export_wisdom_to_filename(const char *filename);                            \
extern void PFX##export_wisdom_to_file(FILE *output_file);                                  \
extern char *PFX##export_wisdom_to_string(void);                                            \
extern void PFX##export_wisdom(PFX##write_char_func write_char, void *data);                \
extern int PFX##import_system_wisdom(void);                                                 \
extern int PFX##import_wisdom_from_filename(const char *filename);                          \
extern int PFX##import_wisdom_from_file(FILE *input_file);                                  \
extern int PFX##import_wisdom_from_string(const char *input_string);                        \
extern int PFX##import_wisdom(PFX##read_char_func read_char, void *data);                   \
extern void PFX##fprint_plan(const PFX##plan p, FILE *output_file);                         \
extern void PFX##print_plan(const PFX##plan p);                                             \
extern char *PFX##sprint_plan(const PFX##plan p);                                           \
extern void *PFX##malloc(size_t n);                                                         \
extern R *PFX##alloc_real(size_t n);                                                        \
extern C *PFX##alloc_complex(size_t n);                                                     \
extern void PFX##free(void *p);                                                             \
extern void PFX##flops(const PFX##plan p, double *add, double *mul, double *fmas);          \
extern double PFX##estimate_cost(const PFX##plan p);                                        \
extern double PFX##cost(const PFX##plan p);                                                 \
extern int PFX##alignment_of(R *p);                                                         \
extern const char PFX##version[];                                                           \
extern const char PFX##cc[];                                                                \
extern const char PFX##codelet_optim[];

GB_FFTW_DECLARE(fftw_, double, fftw_complex)
GB_FFTW_DECLARE(fftwf_, float, fftwf_complex)

/* api/fftw3.h:489-519: values must match the reference bit for bit. */
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_NO_TIMELIMIT (-1.0)

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_CONSERVE_MEMORY (1U << 2)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)

#define FFTW_ESTIMATE_PATIENT (1U << 7)
#define FFTW_BELIEVE_PCOST (1U << 8)
#define FFTW_NO_DFT_R2HC (1U << 9)
#define FFTW_NO_NONTHREADED (1U << 10)
#define FFTW_NO_BUFFERING (1U << 11)
#define FFTW_NO_INDIRECT_OP (1U << 12)
#define FFTW_ALLOW_LARGE_GENERIC (1U << 13)
#define FFTW_NO_RANK_SPLITS (1U << 14)
#define FFTW_NO_VRANK_SPLITS (1U << 15)
#define FFTW_NO_VRECURSE (1U << 16)
#define FFTW_NO_SIMD (1U << 17)
#define FFTW_NO_SLOW (1U << 18)
#define FFTW_NO_FIXED_RADIX_LARGE_N (1U << 19)
#define FFTW_ALLOW_PRUNING (1U << 20)

#ifdef __cplusplus
}
#endif
#endif /* FFTW3_H */
