// Arithmetic-pipe throughput probe: independent FMA chains over every SM, timed
// with CUDA events.  The elastic step in FP64 is bound by the FP64 pipe, whose peak
// is not among the measured copy / GEMM figures, so the benchmark measures
// it on the same device with this kernel and reports the operator's FP64 rate as a
// fraction of it.
#include "common.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

constexpr int kChains = 8;

template <typename R>
__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, R a, R b, R* __restrict__ sink)
{
   R acc[kChains];
#pragma unroll
   for (int c = 0; c < kChains; c++) acc[c] = R(threadIdx.x + c) * R(1e-3);
   for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int c = 0; c < kChains; c++) acc[c] = acc[c] * a + b;
   }
   R s = 0;
#pragma unroll
   for (int c = 0; c < kChains; c++) s += acc[c];
   if (s == R(12345.678)) sink[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

int fma_peak(int precision, double* tflops, cudaStream_t s)
{
   int dev = 0, sms = 0;
   if (cudaGetDevice(&dev) != cudaSuccess) return kCudaError;
   if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return kCudaError;
   const int blocks = sms * 8, threads = 256;
   const int iters = precision == 64 ? 2048 : 65536;
   void* sink = nullptr;
   if (cudaMalloc(&sink, blocks * sizeof(double)) != cudaSuccess) return kCudaError;
   cudaEvent_t e0, e1;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   float best = 1e30f;
   for (int rep = 0; rep < 4; rep++) {
      cudaEventRecord(e0, s);
      if (precision == 64)
         fma_probe_kernel<double><<<blocks, threads, 0, s>>>(iters, 0.999999, 1e-7, (double*)sink);
      else
         fma_probe_kernel<float><<<blocks, threads, 0, s>>>(iters, 0.999999f, 1e-7f, (float*)sink);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < best) best = ms;
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   cudaFree(sink);
   const double flops = 2.0 * kChains * (double)iters * blocks * threads;
   *tflops = flops / (best * 1e-3) / 1e12;
   return launch_status();
}

}  // namespace sw4g
