/*
 * Peak probe for the roofline of double-precision passes: the FP64 FMA rate
 * of the current GPU, measured with CUDA events over a kernel that does
 * nothing but independent FP64 fused multiply-adds.  Double-precision FFT
 * passes on this part are bounded by this rate, not by HBM (its FP64 units
 * are few); the benchmark reports such passes as a fraction of it.
 */
#include <cuda_runtime.h>

namespace gb {

/* eight independent FMA chains per thread, iters steps each; the result is
 * written only under a condition the data never meets, so nothing is
 * folded away and nothing reaches memory */
__global__ void __launch_bounds__(256) k_fp64_fma(double *sink, int iters, double m, double c)
{
     double a[8];
#pragma unroll
     for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
     for (int i = 0; i < iters; ++i) {
#pragma unroll
          for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
     }
     double s = 0;
#pragma unroll
     for (int k = 0; k < 8; ++k) s += a[k];
     if (s == -1.0) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} /* namespace gb */

/* FP64 GFLOP/s (two flops per FMA) of the current device, best of three
 * timed launches after a warm-up; 0 on error. */
extern "C" double fftw_gb300_fp64_fma_gflops(void)
{
     int dev = 0, sms = 0;
     double *sink = 0;
     cudaEvent_t e0 = 0, e1 = 0;
     float best = -1.f;
     const int iters = 4096, threads = 256;
     if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
          goto fail;
     {
          const int grid = sms * 16;
          if (cudaMalloc((void **)&sink, sizeof(double) * grid * threads) != cudaSuccess) goto fail;
          if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto fail;
          gb::k_fp64_fma<<<grid, threads>>>(sink, iters, 0.9999999, 1e-7);
          for (int r = 0; r < 3; ++r) {
               float ms = 0.f;
               cudaEventRecord(e0);
               gb::k_fp64_fma<<<grid, threads>>>(sink, iters, 0.9999999, 1e-7);
               cudaEventRecord(e1);
               if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) goto fail;
               if (best < 0 || ms < best) best = ms;
          }
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          cudaFree(sink);
          return best > 0 ? 2.0 * 8.0 * iters * (double)grid * threads / (best * 1e-3) / 1e9 : 0.0;
     }
fail:
     cudaGetLastError();
     if (e0) cudaEventDestroy(e0);
     if (e1) cudaEventDestroy(e1);
     if (sink) cudaFree(sink);
     return 0.0;
}
