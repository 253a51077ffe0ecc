/*
 * k_cols_tma: persistent kernel for f32 c2c column tiles (tb transforms
 * adjacent in memory, elements at stride is) fed by the TMA engine through
 * a tensor map: the passes along the strided axes of multi-dimensional
 * plans and the passes of the four-step split of long 1D lengths.
 *
 * The tensor map views the pass input as [outer dims][row j < N][column];
 * one tile is tb columns x N rows, fetched as boxes of at most 16 columns
 * (128 bytes) x 256 rows with cp.async.bulk.tensor into a shared slot: a
 * CTA runs one or two compute groups over one slot more than groups, so a
 * tile is on its way while every group transforms one.  The boxes land
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
 * completes sets GB_STATUS_COPY_TIMEOUT and the group leaves its loop.
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

/* CTAs per SM the registers are sized for: three of one group (85
 * registers a thread), two of two groups (64) */
__host__ __device__ constexpr int ct_minblocks(int G) { return G == 2 ? 2 : 3; }

/* Byte offset of slot b: slots on 1024-byte boundaries (the period of the
 * 128-byte swizzle the boxes land in) */
__host__ __device__ inline int ct_slot_off(int nfft, int tb, int b) { return b * ((ct_slot_bytes(nfft, tb) + 1023) & ~1023); }

/* G compute groups (P.threads threads each, own named barrier) over G + 1
 * slots, as k_reg_tma: tile i (global tile blockIdx.x + i gridDim.x) is
 * transformed by group i mod G in slot i mod (G + 1), and the group that
 * finishes with a slot issues the boxes of the slot's next tile. */
template <int LOGN, int DIR, int G>
__global__ void __launch_bounds__(256 * G, ct_minblocks(G))
k_cols_tma(const gb_pass P, const void *__restrict__ in, void *__restrict__ out, const __grid_constant__ CUtensorMap tmap,
           const __grid_constant__ CUtensorMap omap, const int tstore)
{
     typedef float2 C;
     constexpr int N = 1 << LOGN;
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int SMS = reg_sms(N);
     constexpr int NB = G + 1;
     /* no static shared memory (it would be padded to 1 KB and cost a CTA per
      * SM): slots, barriers and counters all live in the dynamic allocation */
     extern __shared__ __align__(1024) unsigned char gb_smem[];
     const int tb = P.tb, cb = ct_cb(tb);
     const int mask = cb >= 16 ? 7 : cb == 8 ? 3 : cb == 4 ? 1 : 0;
     unsigned char *base = (unsigned char *)(((unsigned long long)gb_smem + 1023) & ~1023ull);
     unsigned long long *const full = (unsigned long long *)(base + ct_slot_off(N, tb, NB - 1) +
                                                             ((ct_slot_bytes(N, tb) + 15) & ~15));
     int *const issued = (int *)(full + NB), *const consumed = issued + NB;
     /* a refill each group's leader owes (tile, slot; the slot of its previous
      * tile), read and written by that leader only */
     long long *const pend_tile = (long long *)(consumed + NB);
     int *const pend_slot = (int *)(pend_tile + G);
     const int GT = P.threads;
     const int g = (int)threadIdx.x / GT;
     const int gtid = (int)threadIdx.x - g * GT;
     const int tl = gtid / T;
     const int tid = gtid - tl * T;
     const C *__restrict__ tw = (const C *)P.tw_stage;
     const auto gs = group_barrier<G>(g, GT);
     const long long stride = gridDim.x;

     if (threadIdx.x == 0) {
#pragma unroll
          for (int b = 0; b < NB; ++b) {
               mbar_init(&full[b], 1);
               issued[b] = 0;
               consumed[b] = 0;
          }
          mbar_fence_init();
     }
     __syncthreads();
     if (threadIdx.x == 0) {
#pragma unroll
          for (int b = 0; b < NB; ++b) {
               const long long blk = blockIdx.x + b * stride;
               if (blk < P.nblocks) {
                    ct_issue<N>(P, &tmap, blk, base + ct_slot_off(N, tb, b), &full[b]);
                    issued[b] = 1;
               }
          }
     }

     if (gtid == 0) pend_tile[g] = -1;
     for (int i = g;; i += G) {
          const long long blk = blockIdx.x + (long long)i * stride;
          if (blk >= P.nblocks) break;
          const int b = i % NB;
          unsigned char *const cur = base + ct_slot_off(N, tb, b);
          /* the slot's load for this tile exists (issued by the group done
           * with the slot's previous tile) before its phase is waited on */
          bool ok = true;
          if (gtid == 0) {
               const volatile int *iss = &issued[b];
               const int need = i / NB + 1;
               unsigned long long t0 = 0;
               for (unsigned it = 0; *iss < need; ++it) {
                    if (it == 0) t0 = globaltimer_ns();
                    else if ((it & 63) == 0 && globaltimer_ns() - t0 > GB_WAIT_NS) {
                         ok = false;
                         break;
                    }
               }
          }
          if (!sync_and(gs, ok) || !sync_and(gs, mbar_wait(&full[b], (unsigned)((i / NB) & 1), GB_WAIT_NS))) {
               if (gtid == 0 && P.status) atomicExch(P.status, GB_STATUS_COPY_TIMEOUT);
               break;
          }
          if (gtid == 0) atomicAdd(&consumed[b], 1);

          /* element j of column tl: box tl / cb, row j, chunk-swizzled */
          C x[E];
          {
               const int colbase = (tl / cb) * N * cb * 8 + (tl % cb) * 8;
               if constexpr (T % 8 == 0) {
                    /* rows tid + T e share tid's swizzle (T e moves whole periods
                     * of eight rows): one swizzled base, a constant stride */
                    const unsigned char *p0 = cur + ct_swz(colbase + tid * cb * 8, mask);
                    const int st = T * cb * 8;
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = *(const C *)(p0 + e * st);
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                         const int o = colbase + (tid + T * e) * cb * 8;
                         x[e] = *(const C *)(cur + ct_swz(o, mask));
                    }
               }
          }
          gs();
          /* the previous tile's slot, refilled now that its boxes had the
           * stages' time to be read out by the TMA engine */
          if (gtid == 0 && pend_tile[g] >= 0) {
               const int pb = pend_slot[g];
               bulk_wait_read();
               fence_proxy_async_smem();
               ct_issue<N>(P, &tmap, pend_tile[g], base + ct_slot_off(N, tb, pb), &full[pb]);
               atomicAdd(&issued[pb], 1);
               pend_tile[g] = -1;
          }
          C *const sm = (C *)cur;
          C *const smt = sm + tl * SMS;
          reg_stages<C, N, DIR, 1>(x, tid, smt, tw, gs);
          const tile_t tile = tile_of(P, blk);
          const long long v = tile.v0 + tl;
          const long long nxt = blk + NB * stride;
          if (P.post_N) {
               apply_post_twiddles<C, E, T>(P, P.post_vdim ? tile.vpost : v, tid, x);
          }
          if (P.store_mode == GB_MOVE_DIRECT) {
               /* the slot is free once every thread of the group is past the
                * barrier after its last read (inside the stages) */
               if (gtid == 0 && nxt < P.nblocks) {
                    fence_proxy_async_smem();
                    ct_issue<N>(P, &tmap, nxt, cur, &full[b]);
                    atomicAdd(&issued[b], 1);
               }
               if (v < P.vn[0]) {
                    C *o = (C *)out + tile.bo + v * P.vos[0] + (long long)tid * P.os;
                    const long long st = (long long)T * P.os;
#pragma unroll
                    for (int e = 0; e < E; ++e) o[e * st] = x[e];
               }
          } else if (tstore) {
               /* column tiles out through the output tensor map: the results
                * take the boxes' swizzled layout in the slot, and the group's
                * leader hands the boxes to the TMA engine, waits until they
                * have been read out of the slot, and refills it */
               const int cbs = ct_cb(P.tb);
               const int ms = cbs >= 16 ? 7 : cbs == 8 ? 3 : cbs == 4 ? 1 : 0;
               const int cbase = (tl / cbs) * N * cbs * 8 + (tl % cbs) * 8;
               if constexpr (T % 8 == 0) {
                    unsigned char *p0 = cur + ct_swz(cbase + tid * cbs * 8, ms);
                    const int st = T * cbs * 8;
#pragma unroll
                    for (int e = 0; e < E; ++e) *(C *)(p0 + e * st) = x[e];
               } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                         const int o = cbase + (tid + T * e) * cbs * 8;
                         *(C *)(cur + ct_swz(o, ms)) = x[e];
                    }
               }
               fence_proxy_async_smem();
               gs();
               if (gtid == 0) {
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
                    /* the slot's next tile is issued once the group has gathered
                     * its next tile (above), not here: waiting now for the boxes
                     * to be read out would hold the whole group */
                    if (nxt < P.nblocks) {
                         pend_tile[g] = nxt;
                         pend_slot[g] = b;
                    }
               }
          } else {
               /* plain column stores through the slot (one group per CTA: the
                * launch runs this case with G = 1) */
#pragma unroll
               for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
               gs();
               coop_store<C, true, false>(P, out, sm, SMS, tile, N, P.store_mode, N);
               gs();
               if (gtid == 0 && nxt < P.nblocks) {
                    fence_proxy_async_smem();
                    ct_issue<N>(P, &tmap, nxt, cur, &full[b]);
                    atomicAdd(&issued[b], 1);
               }
          }
     }
     /* a refill still owed is issued (its tile belongs to another group);
      * each leader's stores complete before the CTA ends; a group that gave
      * up may leave loads in flight: wait (bounded) for them */
     if (gtid == 0 && pend_tile[g] >= 0) {
          const int pb = pend_slot[g];
          bulk_wait_read();
          fence_proxy_async_smem();
          ct_issue<N>(P, &tmap, pend_tile[g], base + ct_slot_off(N, tb, pb), &full[pb]);
          atomicAdd(&issued[pb], 1);
     }
     if (tstore && gtid == 0) bulk_wait_all();
     __syncthreads();
     if (threadIdx.x == 0) {
#pragma unroll
          for (int b = 0; b < NB; ++b)
               if (issued[b] > consumed[b]) mbar_wait(&full[b], (unsigned)((issued[b] - 1) & 1), GB_WAIT_NS);
     }
}

template <int L>
static const void *ct_lookup(int logn, int dir, int groups)
{
     if constexpr (L > 11) return 0;
     else {
          if (logn == L) {
               if (groups == 2) return dir < 0 ? (const void *)k_cols_tma<L, -1, 2> : (const void *)k_cols_tma<L, 1, 2>;
               if (groups == 1) return dir < 0 ? (const void *)k_cols_tma<L, -1, 1> : (const void *)k_cols_tma<L, 1, 1>;
               return 0;
          }
          return ct_lookup<L + 1>(logn, dir, groups);
     }
}

} /* namespace gb */

extern "C" const void *gb_cols_tma_kernel(int logn, int dir, int groups) { return gb::ct_lookup<4>(logn, dir, groups); }

/* Shared memory of a k_cols_tma CTA of g groups: g + 1 slots on 1024-byte
 * boundaries, the mbarriers and load counters, each group's owed refill, and
 * the slack to align the first slot. */
extern "C" int gb_cols_tma_smem(int nfft, int tb, int groups)
{
     return gb::ct_slot_off(nfft, tb, groups) + ((gb::ct_slot_bytes(nfft, tb) + 15) & ~15) + (groups + 1) * 16 +
            groups * 16 + 1024;
}
