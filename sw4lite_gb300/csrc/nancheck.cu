// Non-finite scan of a solution level: the counterpart of the reference's
// check_nan_dev (src/device-routines.C:8279), launched by EW::check_for_nan_GPU
// (src/EW_cuda.C:652) after the phases of its time loop (src/EW.C:2544-2759).
//
// One grid-stride pass over the level's values (FP64, or the mixed form's hi and lo
// FP32 halves) counts NaN and infinite entries and keeps the smallest offending
// storage offset, tagged with the grid: per warp one atomic add and one atomic
// minimum on a status block in device memory, read by the host after the scan.
// Unlike the reference, infinities are counted too: an overflowing field is as
// unusable as a NaN one.
#include "common.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

__device__ __forceinline__ bool bad(double v)
{
   // exponent bits all set: infinity or NaN (integer test, no FP64 instruction)
   const unsigned long long b = __double_as_longlong(v);
   return ((b >> 52) & 0x7ff) == 0x7ff;
}

__device__ __forceinline__ bool bad(float v) { return ((__float_as_uint(v) >> 23) & 0xff) == 0xff; }

template <typename T>
__global__ void nonfinite_scan_kernel(const T* __restrict__ x, long long n, unsigned long long tag,
                                      unsigned long long* __restrict__ block)
{
   unsigned long long cnt = 0, first = ~0ull;
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x) {
      if (bad(x[q])) {
         if (cnt == 0) first = (unsigned long long)q;
         cnt++;
      }
   }
   const unsigned any = __ballot_sync(0xffffffffu, cnt != 0);
   if (!any) return;
   for (int o = 16; o > 0; o >>= 1) {
      cnt += __shfl_down_sync(0xffffffffu, cnt, o);
      const unsigned long long f = __shfl_down_sync(0xffffffffu, first, o);
      first = f < first ? f : first;
   }
   if ((threadIdx.x & 31) == 0) {
      atomicAdd(block + 1, cnt);
      atomicMin(block + 2, tag | first);
   }
}

}  // namespace

int launch_nonfinite_scan(const void* x, long long n, bool is_float, int grid,
                          unsigned long long* block, cudaStream_t s)
{
   if (n <= 0) return kOk;
   const unsigned long long tag = (unsigned long long)grid << kScanGridShift;
   const int threads = 256;
   const long long want = (n + threads - 1) / threads;
   const int blocks = (int)(want < 152LL * 8 ? want : 152LL * 8);
   if (is_float)
      nonfinite_scan_kernel<float><<<blocks, threads, 0, s>>>(static_cast<const float*>(x), n, tag, block);
   else
      nonfinite_scan_kernel<double><<<blocks, threads, 0, s>>>(static_cast<const double*>(x), n, tag, block);
   return launch_status();
}

}  // namespace sw4g
