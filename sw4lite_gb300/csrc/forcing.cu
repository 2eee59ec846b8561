// Point-source forcing on the device, sm_103a.
//
// The reference expands every source into grid-point sources at setup
// (src/Source.C:1074-1700) and each stage zeroes a dense F and accumulates
// F(i,j,k) += amp * g(t - t0) over the grid-point sources that share a point
// (src/EW.C:3085-3124, unique points from src/EW.C:6370-6433; GPU twin
// forcing_dev, src/device-routines.C:8306).  Here the grid-point sources are a
// device-resident list grouped by point, one thread per point:
//   * force_dense_kernel writes F at the source points of a zeroed dense F (the
//     phase-level ForceCU replacement);
//   * force_update_kernel adds coef/rho * F directly into the new time level,
//     which is what the fused stage kernels use instead of a dense F.
#include <math.h>

#include "common.cuh"
#include "kernels.h"

namespace sw4g {

// Source time functions (src/time_functions.C).  kind: 0 Gaussian (:284, :311),
// 1 C6SmoothBump (:1637, :1676), 2 Ricker wavelet (:175, :202),
// 3 VerySmoothBump (:36, :72).  The Gaussian cut-off exponent -700 is the value
// the reference's Source sets (src/Source.C:2183-2187).
__host__ __device__ inline double timefunc(int kind, double freq, double t, bool tt)
{
   const double pi = 3.14159265358979323846;
   if (kind == 0) {
      const double f = (t * freq) * (t * freq) / 2;
      if (!(-f > -700.0)) return 0.0;
      const double g = freq / sqrt(2 * pi) * exp(-f);
      return tt ? g * freq * freq * (2 * f - 1) : g;
   }
   if (kind == 1) {
      const double x = t * freq;
      if (x < 0 || x > 1) return 0.0;
      const double y = x * (1 - x);
      if (!tt) return 51480 * pow(y, 7);
      return 51480 * freq * freq * 7 * (6 * (1 - 2 * x) * (1 - 2 * x) * pow(y, 5) - 2 * pow(y, 6));
   }
   if (kind == 2) {
      // Ricker: R = (2a - 1) exp(-a) with a = (pi f t)^2; d2R/dt2 = (pi f)^2 (6 - 24a + 8a^2) exp(-a)
      const double a = (pi * freq * t) * (pi * freq * t);
      if (!(-a > -700.0)) return 0.0;
      if (!tt) return (2 * a - 1) * exp(-a);
      return pi * pi * freq * freq * (6 - 24 * a + 8 * a * a) * exp(-a);
   }
   // VerySmoothBump: 1024 x^5 - 5120 x^6 + 10240 x^7 - 10240 x^8 + 5120 x^9 - 1024 x^10 on [0,1]
   const double x = t * freq;
   if (x < 0 || x > 1) return 0.0;
   if (!tt)
      return (((((-1024 * x + 5120) * x - 10240) * x + 10240) * x - 5120) * x + 1024) * x * x * x * x * x;
   return freq * freq *
          ((((((-90 * 1024.0 * x + 72 * 5120.0) * x - 56 * 10240.0) * x + 42 * 10240.0) * x -
            30 * 5120.0) * x + 20 * 1024.0) * x * x * x);
}

namespace {

__global__ void force_dense_kernel(Box b, double* __restrict__ f, SourceSet src, double t, int tt)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= src.npoints) return;
   double acc[3] = {0, 0, 0};
   for (int s = src.start[r]; s < src.start[r + 1]; s++) {
      const double g = timefunc(src.kind[s], src.freq[s], t - src.t0[s], tt != 0);
      acc[0] += src.amp[3 * s] * g;
      acc[1] += src.amp[3 * s + 1] * g;
      acc[2] += src.amp[3 * s + 2] * g;
   }
   const int s0 = src.start[r];
   const int i = src.ijk[3 * s0], j = src.ijk[3 * s0 + 1], k = src.ijk[3 * s0 + 2];
   for (int c = 0; c < 3; c++) f[cidx(b, c, i, j, k)] += acc[c];
}

template <typename S>
__global__ void force_update_kernel(Box b, S* __restrict__ up, const double* __restrict__ rho,
                                    SourceSet src, double t, int tt, double coef,
                                    const double* __restrict__ clk)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= src.npoints) return;
   if (clk) t = clk[0];  // the device clock of a captured time loop
   double acc[3] = {0, 0, 0};
   for (int s = src.start[r]; s < src.start[r + 1]; s++) {
      const double g = timefunc(src.kind[s], src.freq[s], t - src.t0[s], tt != 0);
      acc[0] += src.amp[3 * s] * g;
      acc[1] += src.amp[3 * s + 1] * g;
      acc[2] += src.amp[3 * s + 2] * g;
   }
   const int s0 = src.start[r];
   const int i = src.ijk[3 * s0], j = src.ijk[3 * s0 + 1], k = src.ijk[3 * s0 + 2];
   const double c0 = coef / rho[pidx(b, i, j, k)];
   for (int c = 0; c < 3; c++) {
      const long long q = cidx(b, c, i, j, k);
      up[q] = (S)((double)up[q] + c0 * acc[c]);
   }
}

// Same as force_update_kernel for a double-float level: the add runs in FP64.
__global__ void force_update_df_kernel(Box b, DFField up, const double* __restrict__ rho,
                                       SourceSet src, double t, int tt, double coef,
                                       const double* __restrict__ clk)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= src.npoints) return;
   if (clk) t = clk[0];
   double acc[3] = {0, 0, 0};
   for (int s = src.start[r]; s < src.start[r + 1]; s++) {
      const double g = timefunc(src.kind[s], src.freq[s], t - src.t0[s], tt != 0);
      acc[0] += src.amp[3 * s] * g;
      acc[1] += src.amp[3 * s + 1] * g;
      acc[2] += src.amp[3 * s + 2] * g;
   }
   const int s0 = src.start[r];
   const int i = src.ijk[3 * s0], j = src.ijk[3 * s0 + 1], k = src.ijk[3 * s0 + 2];
   const double c0 = coef / rho[pidx(b, i, j, k)];
   for (int c = 0; c < 3; c++) {
      const long long q = cidx(b, c, i, j, k);
      up.set(q, up.get(q) + c0 * acc[c]);
   }
}

// The device clock of a captured time loop: [0] time of the next stage's forcing,
// [1] next record row, [2] residual row of the next adjoint step.
__global__ void clock_advance_kernel(double* clk, double dt, double drow, double dres)
{
   if (threadIdx.x == 0 && blockIdx.x == 0) {
      clk[0] += dt;
      clk[1] += drow;
      clk[2] += dres;
   }
}

}  // namespace

int launch_clock_advance(double* clk, double dt, double drow, double dres, cudaStream_t s)
{
   clock_advance_kernel<<<1, 32, 0, s>>>(clk, dt, drow, dres);
   return launch_status();
}

int launch_force_update_df(int ib, int ie, int jb, int je, int kb, int ke, float* uph,
                           const double* rho, const SourceSet& src, double t, int tt, double coef,
                           cudaStream_t s, const double* clk)
{
   if (src.npoints == 0) return kOk;
   Box b = make_box(1, ib, ie, jb, je, kb, ke);
   force_update_df_kernel<<<blocks_for(src.npoints, 128), 128, 0, s>>>(b, DFField{uph, 3 * b.npts},
                                                                      rho, src, t, tt, coef, clk);
   return launch_status();
}

int launch_force_dense(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* f,
                       const SourceSet& src, double t, int tt, cudaStream_t s)
{
   Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   if (cudaMemsetAsync(f, 0, 3 * b.npts * sizeof(double), s) != cudaSuccess) return kCudaError;
   if (src.npoints > 0)
      force_dense_kernel<<<blocks_for(src.npoints, 128), 128, 0, s>>>(b, f, src, t, tt);
   return launch_status();
}

int launch_force_update(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                        const double* rho, const SourceSet& src, double t, int tt, double coef,
                        cudaStream_t s, const double* clk)
{
   if (src.npoints == 0) return kOk;
   Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   force_update_kernel<double><<<blocks_for(src.npoints, 128), 128, 0, s>>>(b, up, rho, src, t, tt,
                                                                            coef, clk);
   return launch_status();
}

int launch_force_update_f32(int soa, int ib, int ie, int jb, int je, int kb, int ke, float* up,
                            const double* rho, const SourceSet& src, double t, int tt,
                            double coef, cudaStream_t s)
{
   if (src.npoints == 0) return kOk;
   Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   force_update_kernel<float><<<blocks_for(src.npoints, 128), 128, 0, s>>>(b, up, rho, src, t, tt,
                                                                           coef, nullptr);
   return launch_status();
}

}  // namespace sw4g
