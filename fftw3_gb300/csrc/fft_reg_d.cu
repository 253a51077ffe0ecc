/* k_reg instantiations, double precision (nfft = 2^0 .. 2^13). */
#define GB_REAL double
#define GB_MAXLOG 13
#include "fft_reg_inst.cuh"
extern "C" const void *gb_reg_kernel_d(int logn, int kind, int dir) { return gb::reg_lookup<0>(logn, kind, dir); }
extern "C" const void *gb_tma_kernel_d(int logn, int kind, int dir, int groups)
{
     return gb::tma_lookup<6>(logn, kind, dir, groups);
}
