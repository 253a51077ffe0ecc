/*
 * Work-queue kernel of a plan set: persistent CTAs (as many as fit on the
 * device) claim items from a device queue with one atomic each (one item
 * ahead) and run them with the shared-memory tile body of k_gen, or, for
 * power-of-two float items of 64..4096 points whose set asks for it (the set
 * tuner's wisdom or FFTW_GB300_QUEUE_BODY=reg), with the register stages of
 * k_reg.  Items of one long transform are ordered column tiles first, row
 * tiles last; a row tile waits for its transform's column tiles on a device
 * counter.  Every wait is bounded
 * (wait_ns of wall time, 2 s unless the set says otherwise); a wait that
 * gives up writes GB_STATUS_QUEUE_TIMEOUT to the status word and the item is
 * skipped, so the kernel always finishes.
 *
 * This is the GB300 replacement for running many independent plans one
 * after another (the reference's only way to execute a set of transforms):
 * one launch, captured once in a CUDA graph, runs the whole set.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include "fft_kernels.cuh"

namespace gb {

__device__ __forceinline__ int ld_acquire(const int *p)
{
     int v;
     asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
     return v;
}

__device__ __forceinline__ void red_release_add(int *p, int v)
{
     asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

/* A power-of-two item (64..4096 points, float) with the register kernels'
 * stages: each thread holds 16 elements of one transform, T = N/16 threads a
 * transform, 256 / T transforms a round (threads beyond the item's tb run
 * the stages on scratch rows and store nothing).  Column tiles (adjacent
 * transforms, strided elements) move through shared memory transform-fast,
 * rows are loaded and stored by each thread directly. */
template <typename C, int LOGN, int DIR>
__device__ __noinline__ void reg_item(const gb_pass &P, const tile_t &tile, const gen_addr &A, C *sm)
{
     constexpr int N = 1 << LOGN;
     constexpr int E = reg_e(N);
     constexpr int T = N / E;
     constexpr int SMS = reg_sms(N);
     const int tl = threadIdx.x / T, tid = threadIdx.x - tl * T;
     const int tb = P.tb;
     C *smt = sm + tl * SMS;
     const long long v = tile.v0 + tl;
     const bool valid = tl < tb && v < P.vn[0];
     C x[E];
     if (P.load_mode == GB_MOVE_COLS) {
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x) {
               int t, j;
               tile_index(idx, tb, N, GB_MOVE_COLS, t, j, P.ltb);
               if (tile.v0 + t < P.vn[0]) {
                    const C *sp = src_of<C>(P, tile, A, t) + (long long)j * P.is;
                    sm[t * SMS + pad_for(N, j)] = A.l2only ? __ldcg(sp) : *sp;
               }
          }
          __syncthreads();
#pragma unroll
          for (int e = 0; e < E; ++e) x[e] = smt[pad_for(N, tid + T * e)];
          __syncthreads();
     } else if (valid) {
          const C *sp = src_of<C>(P, tile, A, tl);
#pragma unroll
          for (int e = 0; e < E; ++e) {
               const C *q = sp + (long long)(tid + T * e) * P.is;
               x[e] = A.l2only ? __ldcg(q) : *q;
          }
     } else {
#pragma unroll
          for (int e = 0; e < E; ++e) x[e] = mk<C>(0, 0);
     }
     reg_stages<C, N, DIR, 1>(x, tid, smt, (const C *)P.tw_stage);
     if (P.post_N) apply_post_twiddles<C, E, T>(P, v, tid, x);
     if (P.store_mode == GB_MOVE_COLS) {
#pragma unroll
          for (int e = 0; e < E; ++e) smt[pad_for(N, tid + T * e)] = x[e];
          __syncthreads();
          for (int idx = threadIdx.x; idx < tb * N; idx += blockDim.x) {
               int t, j;
               tile_index(idx, tb, N, GB_MOVE_COLS, t, j, P.ltb);
               if (tile.v0 + t < P.vn[0]) dst_of<C>(P, tile, A, t)[(long long)j * P.os] = sm[t * SMS + pad_for(N, j)];
          }
     } else if (valid) {
          C *dp = dst_of<C>(P, tile, A, tl);
#pragma unroll
          for (int e = 0; e < E; ++e) dp[(long long)(tid + T * e) * P.os] = x[e];
     }
     __syncthreads();
}

/* the register body of a power-of-two item, by length and direction */
template <typename C, int LOGN>
__device__ __forceinline__ bool reg_item_at(const gb_pass &P, const tile_t &tile, const gen_addr &A, C *sm)
{
     if constexpr (LOGN > 12) {
          return false;
     } else {
          if (P.nfft != (1 << LOGN)) return reg_item_at<C, LOGN + 1>(P, tile, A, sm);
          if (P.sign < 0) reg_item<C, LOGN, -1>(P, tile, A, sm);
          else reg_item<C, LOGN, 1>(P, tile, A, sm);
          return true;
     }
}

/* Copy one item descriptor (512 bytes) into shared memory with 16-byte
 * asynchronous copies (threads 0..31), completed by cp_async_wait_all. */
static_assert(sizeof(gb_qitem) % 16 == 0, "queue items are copied in 16-byte pieces");
__device__ __forceinline__ void item_copy_async(gb_qitem *dst, const gb_qitem *src)
{
     constexpr int P16 = (int)(sizeof(gb_qitem) / 16);
     if (threadIdx.x < P16) {
          const unsigned d = (unsigned)__cvta_generic_to_shared((char *)dst + 16 * threadIdx.x);
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"((const char *)src + 16 * threadIdx.x)
                       : "memory");
     }
     asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

/* Each CTA claims its next item and starts copying that item's descriptor
 * before it runs the current one, so the claim's atomic and the descriptor
 * load overlap the current item's work.  A claimed item with a higher index
 * never holds up one with a lower index: row tiles (the only items that
 * wait) come after every column tile they wait for, and a CTA finishes its
 * current item before it starts the one it claimed. */
template <typename C, int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS <= 256 ? 3 : 1) k_queue(const gb_qitem *__restrict__ items, int nitems, int *head,
                                                int *ctrs, int *status, unsigned long long wait_ns)
{
     extern __shared__ __align__(16) unsigned char gb_smem[];
     __shared__ __align__(16) gb_qitem its[2];
     __shared__ int claim, go;
     if (threadIdx.x == 0) claim = atomicAdd(head, 1);
     __syncthreads();
     int i = claim, b = 0;
     if (i < nitems) item_copy_async(&its[0], items + i);
     __syncthreads();
     while (i < nitems) {
          if (threadIdx.x == 0) claim = atomicAdd(head, 1);
          cp_async_wait_all();
          __syncthreads();
          const int inext = claim;
          if (inext < nitems) item_copy_async(&its[b ^ 1], items + inext);
          const gb_qitem &it = its[b];
          if (threadIdx.x == 0) {
               go = 1;
               if (it.wait_ctr >= 0) {
                    const int *c = ctrs + it.wait_ctr;
                    unsigned long long t0 = globaltimer_ns();
                    while (ld_acquire(c) < it.wait_target) {
                         if (globaltimer_ns() - t0 > wait_ns) {
                              go = 0;
                              if (status) atomicExch(status, GB_STATUS_QUEUE_TIMEOUT);
                              break;
                         }
                         __nanosleep(256);
                    }
               }
          }
          __syncthreads();
          if (go) {
               /* an item that waited reads what other CTAs wrote in this
                * launch: thread 0's acquire and the barrier order the reads
                * after the wait, the fence keeps this thread's own earlier
                * accesses from passing it; items that do not wait need none */
               if (it.wait_ctr >= 0) __threadfence();
               C *b0 = (C *)gb_smem;
               C *b1 = b0 + it.P.tb * gen_sms(it.P.nfft);
               tile_t tile;
               tile.bi = it.bi; tile.bo = it.bo; tile.v0 = it.v0; tile.vpost = 0;
               gen_addr A;
               A.in = it.in; A.out = it.out; A.pin = it.pin; A.pout = it.pout;
               A.l2only = it.wait_ctr >= 0;
               bool done = false;
               if constexpr (THREADS == 256 && sizeof(C) == 8) {
                    if (it.P.variant == GB_VAR_REG) done = reg_item_at<C, 6>(it.P, tile, A, b0);
               }
               if (!done) gen_tile<C>(it.P, tile, A, b0, b1);
               if (it.signal_ctr >= 0) {
                    __threadfence();
                    __syncthreads();
                    if (threadIdx.x == 0) red_release_add(ctrs + it.signal_ctr, 1);
               }
          }
          __syncthreads();
          b ^= 1;
          i = inext;
     }
     cp_async_wait_all();
}

} /* namespace gb */

using namespace gb;

extern "C" int *gb_device_status_ptr(void);

/* two instantiations: 256 threads for the small-tile queue (three CTAs per
 * SM), 512 threads for the queue of items that need the largest tiles */
static const void *queue_kernel(int prec, int threads)
{
     if (threads <= 256) return prec == 4 ? (const void *)k_queue<float2, 256> : (const void *)k_queue<double2, 256>;
     return prec == 4 ? (const void *)k_queue<float2, 512> : (const void *)k_queue<double2, 512>;
}

/* CTAs of the queue kernel that fit on the device at once. */
extern "C" int gb_queue_grid(int prec, int threads, int smem)
{
     const void *fn = queue_kernel(prec, threads);
     int dev = 0, sms = 0, per = 0;
     if (smem > 48 * 1024 && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
          return -1;
     cudaGetDevice(&dev);
     cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
     if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, (size_t)smem) != cudaSuccess || per < 1)
          return -1;
     return per * sms;
}

extern "C" int gb_launch_queue(const gb_qitem *items, int nitems, int *head, int *ctrs, int prec, int threads,
                               int smem, int grid, unsigned long long wait_ns, void *stream)
{
     const void *fn = queue_kernel(prec, threads);
     int *status = gb_device_status_ptr();
     void *args[6] = {(void *)&items, (void *)&nitems, (void *)&head, (void *)&ctrs, (void *)&status, (void *)&wait_ns};
     if (smem > 48 * 1024 && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
          return -1;
     return cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, (size_t)smem, (cudaStream_t)stream) == cudaSuccess ? 0 : -1;
}
