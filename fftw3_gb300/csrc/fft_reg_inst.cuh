/* Instantiation table of k_reg for one precision (included by
 * fft_reg_f.cu / fft_reg_d.cu with GB_REAL and GB_MAXLOG defined). */
#include "fft_kernels.cuh"

namespace gb {
typedef cplx_of<GB_REAL>::T GB_CT;

template <int L>
static const void *reg_pick(int kind, int dir)
{
     if (kind == GB_KIND_C2C) return dir < 0 ? (const void *)k_reg<GB_CT, L, -1, GB_KIND_C2C>
                                             : (const void *)k_reg<GB_CT, L, 1, GB_KIND_C2C>;
     if (kind == GB_KIND_R2C) return (const void *)k_reg<GB_CT, L, -1, GB_KIND_R2C>;
     if (kind == GB_KIND_C2R) return (const void *)k_reg<GB_CT, L, 1, GB_KIND_C2R>;
     if (kind == GB_KIND_BLUESTEIN && L >= 5) return (const void *)k_reg<GB_CT, L, -1, GB_KIND_BLUESTEIN>;
     return 0;
}

template <int L, int G>
static const void *tma_pick(int kind, int dir)
{
     if constexpr (L < 6 || L > 13 || G > tma_max_groups(sizeof(GB_CT))) return 0;
     else {
          if (kind == GB_KIND_R2C) return (const void *)k_reg_tma<GB_CT, L, -1, GB_KIND_R2C, G>;
          if (kind == GB_KIND_DCT2) return (const void *)k_reg_tma<GB_CT, L, -1, GB_KIND_DCT2, G>;
          return dir < 0 ? (const void *)k_reg_tma<GB_CT, L, -1, GB_KIND_C2C, G>
                         : (const void *)k_reg_tma<GB_CT, L, 1, GB_KIND_C2C, G>;
     }
}

template <int L>
static const void *tma_lookup(int logn, int kind, int dir, int groups)
{
     if constexpr (L > 13) return 0;
     else {
          if (logn == L) return groups == 2 ? tma_pick<L, 2>(kind, dir) : groups == 1 ? tma_pick<L, 1>(kind, dir) : 0;
          return tma_lookup<L + 1>(logn, kind, dir, groups);
     }
}

template <int L>
static const void *reg_lookup(int logn, int kind, int dir)
{
     if constexpr (L > GB_MAXLOG) return 0;
     else {
          if (logn == L) return reg_pick<L>(kind, dir);
          return reg_lookup<L + 1>(logn, kind, dir);
     }
}
} /* namespace gb */
