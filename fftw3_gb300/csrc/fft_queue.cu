/*
 * Work-queue kernel of a plan set: persistent CTAs (as many as fit on the
 * device) claim items from a device queue with one atomic each and run them
 * with the shared-memory tile body of k_gen.  Items of one long transform
 * are ordered column tiles first, row tiles last; a row tile waits for its
 * transform's column tiles on a device counter.  Every wait is bounded
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

template <typename C, int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS <= 256 ? 3 : 1) k_queue(const gb_qitem *__restrict__ items, int nitems, int *head,
                                                int *ctrs, int *status, unsigned long long wait_ns)
{
     extern __shared__ __align__(16) unsigned char gb_smem[];
     __shared__ __align__(16) gb_qitem it;
     __shared__ int cur, go;
     for (;;) {
          if (threadIdx.x == 0) cur = atomicAdd(head, 1);
          __syncthreads();
          const int i = cur;
          if (i >= nitems) break;
          for (int w = threadIdx.x; w < (int)(sizeof(gb_qitem) / 4); w += blockDim.x)
               ((int *)&it)[w] = ((const int *)(items + i))[w];
          __syncthreads();
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
               __threadfence();
               C *b0 = (C *)gb_smem;
               C *b1 = b0 + it.P.tb * (it.P.nfft + 1);
               tile_t tile;
               tile.bi = it.bi; tile.bo = it.bo; tile.v0 = it.v0; tile.vpost = 0;
               gen_addr A;
               A.in = it.in; A.out = it.out; A.pin = it.pin; A.pout = it.pout;
               A.l2only = it.wait_ctr >= 0;
               gen_tile<C>(it.P, tile, A, b0, b1);
               if (it.signal_ctr >= 0) {
                    __threadfence();
                    __syncthreads();
                    if (threadIdx.x == 0) red_release_add(ctrs + it.signal_ctr, 1);
               }
          }
          __syncthreads();
     }
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
