/*
 * k_cols_tma: persistent kernel for f32 c2c column tiles (tb transforms
 * adjacent in memory, elements at stride is) fed by the TMA engine through
 * a tensor map: the passes along the strided axes of multi-dimensional
 * plans and the passes of the four-step split of long 1D lengths.
 *
 * The tensor map views the pass input as [outer dims][row j < N][column];
 * one tile is tb columns x N rows, fetched as boxes of at most 16 columns
 * (128 bytes) x 256 rows with cp.async.bulk.tensor into one of two shared
 * slots while the tile in the other slot is transformed.  The boxes land
 * row-major with the 16-byte-chunk swizzle that matches their row width
 * (32/64/128 bytes), so the transform-major gather that follows touches
 * eight different 16-byte chunks per eight consecutive rows.  From there the
 * tile runs through the same register stages as k_reg (radix 16, shared
 * exchanges in the slot), the four-step twiddle if any, and is stored
 * directly (unit output stride), or as column tiles: through a second tensor
 * map (cp.async.bulk.tensor stores of the same swizzled boxes) when the
 * output's strides allow, else with plain stores.
 *
 * Every wait on a slot is bounded (2 s of wall time); a copy that never
 * completes sets GB_STATUS_COPY_TIMEOUT and the CTA returns.
 */
#include <cuda.h>
#include "fft_kernels.cuh"

namespace gb {

/* columns per box: 16 (128-byte rows) or the whole tile when narrower */
__host__ __device__ constexpr int ct_cb(int tb) { return tb < 16 ? tb : 16; }

/* bytes of one slot: the tile as boxes, or the k_reg exchange layout */
__host__ __device__ inline int ct_slot_bytes(int nfft, int tb)
{
     const int a = nfft * tb * 8, b = tb * reg_sms(nfft) * 8;
     return a > b ? a : b;
}

/* 16-byte chunk swizzle of a box with rows of cb * 8 bytes (the tensor
 * map's 32B / 64B / 128B mode): chunk bits [4, 4+k) ^= offset bits [7, 7+k) */
__device__ __forceinline__ int ct_swz(int o, int mask) { return o ^ (((o >> 7) & mask) << 4); }

__device__ __forceinline__ void tma_tile_load(void *dst, const CUtensorMap *tm, int rank, const int *c,
                                              unsigned long long *bar)
{
     const unsigned d = smem_u32(dst), b = smem_u32(bar);
     const unsigned long long t = (unsigned long long)tm;
     switch (rank) {
     case 2:
          asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                       ::"r"(d), "l"(t), "r"(c[0]), "r"(c[1]), "r"(b) : "memory");
          break;
     case 3:
          asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                       ::"r"(d), "l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(b) : "memory");
          break;
     case 4:
          asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
                       ::"r"(d), "l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(b) : "memory");
          break;
     default:
          asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
                       ::"r"(d), "l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(b) : "memory");
          break;
     }
}

__device__ __forceinline__ void tma_tile_store(const CUtensorMap *tm, int rank, const int *c, const void *src)
{
     const unsigned sa = smem_u32(src);
     const unsigned long long t = (unsigned long long)tm;
     switch (rank) {
     case 2:
          asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
                       ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(sa) : "memory");
          break;
     case 3:
          asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];"
                       ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(sa) : "memory");
          break;
     case 4:
          asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];"
                       ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(sa) : "memory");
          break;
     default:
          asm volatile("cp.async.bulk.tensor.5d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4, %5}], [%6];"
                       ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(sa) : "memory");
          break;
     }
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
/* the committed stores have finished reading shared memory */
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
/* the committed stores have completed */
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

/* Tensor coordinates of tile blk: c[0] first column, c[2..] the outer
 * vector indices (c[1], the row, is set per box). */
__device__ __forceinline__ void ct_coords(const gb_pass &P, long long blk, int *c)
{
     long long rest = blk / P.ntiles0;
     c[0] = (int)((blk - rest * P.ntiles0) * P.tb);
     c[1] = 0;
     for (int d = 1; d < P.nv; ++d) {
          const long long q = rest / P.vn[d];
          c[1 + d] = (int)(rest - q * P.vn[d]);
          rest = q;
     }
}

/* Issue the boxes of tile blk into slot dst (thread 0 only). */
template <int N>
__device__ __forceinline__ void ct_issue(const gb_pass &P, const CUtensorMap *tm, long long blk, unsigned char *dst,
                                         unsigned long long *bar)
{
     constexpr int ROWS = N < 256 ? N : 256;
     const int tb = P.tb, cb = ct_cb(tb);
     int c[5] = {0, 0, 0, 0, 0};
     ct_coords(P, blk, c);
     mbar_expect_tx(bar, (unsigned)(tb * N * 8));
     const int c0 = c[0];
     for (int k = 0; k < tb / cb; ++k)
          for (int r = 0; r < N / ROWS; ++r) {
               c[0] = c0 + k * cb;
               c[1] = r * ROWS;
               tma_tile_load(dst + (k * N + r * ROWS) * cb * 8, tm, 1 + P.nv, c, bar);
          }
}

template <int LOGN, int DIR>
__global__ void __launch_bounds__(256, 3)
k_cols_tma(const gb_pass P, const void *__restrict__ in, void *__restrict__ out, const __grid_constant__ CUtensorMap tmap,
           const __grid_constant__ CUtensorMap omap, const int tstore)
{
     typedef float2 C;
     constexpr int N = 1 << LOGN;
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int SMS = reg_sms(N);
     /* no static shared memory (it would be padded to 1 KB and cost the third
      * CTA per SM): slots and barriers all live in the dynamic allocation */
     extern __shared__ __align__(1024) unsigned char gb_smem[];
     const int tb = P.tb, cb = ct_cb(tb);
     const int mask = cb >= 16 ? 7 : cb == 8 ? 3 : cb == 4 ? 1 : 0;
     /* slots on 1024-byte boundaries (the swizzle pattern's period) */
     unsigned char *base = (unsigned char *)(((unsigned long long)gb_smem + 1023) & ~1023ull);
     const int sb = (ct_slot_bytes(N, tb) + 1023) & ~1023;
     unsigned char *const s0 = base, *const s1 = base + sb;
     unsigned long long *const bar = (unsigned long long *)(s1 + ((ct_slot_bytes(N, tb) + 15) & ~15));
     const int tl = threadIdx.x / T;
     const int tid = threadIdx.x - tl * T;
     const C *__restrict__ tw = (const C *)P.tw;

     if (threadIdx.x == 0) {
          mbar_init(&bar[0], 1);
          mbar_init(&bar[1], 1);
          mbar_fence_init();
     }
     __syncthreads();
     const long long stride = gridDim.x;
     long long blk = blockIdx.x;
     if (threadIdx.x == 0 && blk < P.nblocks) ct_issue<N>(P, &tmap, blk, s0, &bar[0]);
     unsigned parity = 0;

     for (int it = 0; blk < P.nblocks; blk += stride, ++it) {
          const int b = it & 1;
          unsigned char *const cur = b ? s1 : s0;
          const long long nxt = blk + stride;
          const bool issued = nxt < P.nblocks;
          if (threadIdx.x == 0 && issued) {
               /* that slot's boxes may still be going out to global memory */
               if (tstore) bulk_wait_read();
               fence_proxy_async_smem();
               ct_issue<N>(P, &tmap, nxt, b ? s0 : s1, &bar[b ^ 1]);
          }
          const bool ok = mbar_wait(&bar[b], (parity >> b) & 1u, GB_WAIT_NS);
          if (!__syncthreads_and(ok)) {
               if (threadIdx.x == 0) {
                    if (issued) mbar_wait(&bar[b ^ 1], (parity >> (b ^ 1)) & 1u, GB_WAIT_NS);
                    if (P.status) atomicExch(P.status, GB_STATUS_COPY_TIMEOUT);
               }
               return;
          }
          parity ^= 1u << b;

          const tile_t tile = tile_of(P, blk);
          const long long v = tile.v0 + tl;
          const bool valid = v < P.vn[0];
          /* element j of column tl: box tl / cb, row j, chunk-swizzled */
          const int colbase = (tl / cb) * N * cb * 8 + (tl % cb) * 8;
          C x[E];
#pragma unroll
          for (int e = 0; e < E; ++e) {
               const int o = colbase + (tid + T * e) * cb * 8;
               x[e] = *(const C *)(cur + ct_swz(o, mask));
          }
          __syncthreads();
          C *const sm = (C *)cur;
          C *const smt = sm + tl * SMS;
          reg_stages<C, N, DIR, 1>(x, tid, smt, tw);
          if (P.post_N) {
               apply_post_twiddles<C, E, T>(P, P.post_vdim ? tile.vpost : v, tid, x);
          }
          if (P.store_mode == GB_MOVE_DIRECT) {
               if (valid) {
                    const long long bo = tile.bo + v * P.vos[0];
#pragma unroll
                    for (int e = 0; e < E; ++e) io<C>::stc(out, bo, tid + T * e, P.os, x[e]);
               }
          } else if (tstore) {
               /* column tiles out through the output tensor map: the results
                * take the boxes' swizzled layout in the slot, and one thread
                * hands the boxes to the TMA engine */
               /* layout constants recomputed from the launch parameters
                * rather than kept live across the stages */
               const int cbs = ct_cb(P.tb);
               const int ms = cbs >= 16 ? 7 : cbs == 8 ? 3 : cbs == 4 ? 1 : 0;
               const int cbase = (tl / cbs) * N * cbs * 8 + (tl % cbs) * 8;
#pragma unroll
               for (int e = 0; e < E; ++e) {
                    const int o = cbase + (tid + T * e) * cbs * 8;
                    *(C *)(cur + ct_swz(o, ms)) = x[e];
               }
               fence_proxy_async_smem();
               __syncthreads();
               if (threadIdx.x == 0) {
                    constexpr int ROWS = N < 256 ? N : 256;
                    int c[5] = {0, 0, 0, 0, 0};
                    ct_coords(P, blk, c);
                    const int c0 = c[0];
                    for (int k = 0; k < P.tb / cbs; ++k)
                         for (int r = 0; r < N / ROWS; ++r) {
                              c[0] = c0 + k * cbs;
                              c[1] = r * ROWS;
                              tma_tile_store(&omap, 1 + P.nv, c, cur + (k * N + r * ROWS) * cbs * 8);
                         }
                    bulk_commit();
               }
          } else {
#pragma unroll
               for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
               __syncthreads();
               coop_store<C, true, false>(P, out, sm, SMS, tile, N, P.store_mode, N);
          }
          __syncthreads();   /* the slot is the target of a later tile's boxes */
     }
     if (tstore && threadIdx.x == 0) bulk_wait_all();
}

template <int L>
static const void *ct_lookup(int logn, int dir)
{
     if constexpr (L > 11) return 0;
     else {
          if (logn == L) return dir < 0 ? (const void *)k_cols_tma<L, -1> : (const void *)k_cols_tma<L, 1>;
          return ct_lookup<L + 1>(logn, dir);
     }
}

} /* namespace gb */

extern "C" const void *gb_cols_tma_kernel(int logn, int dir) { return gb::ct_lookup<4>(logn, dir); }

/* Shared memory of a k_cols_tma CTA: two slots on 1024-byte boundaries, the
 * two mbarriers, and the slack to align the first slot. */
extern "C" int gb_cols_tma_smem(int nfft, int tb)
{
     const int sb = (gb::ct_slot_bytes(nfft, tb) + 1023) & ~1023;
     return sb + ((gb::ct_slot_bytes(nfft, tb) + 15) & ~15) + 16 + 1024;
}
