// Receiver recording on the device, sm_103a.
//
// The reference samples every receiver (TimeSeries) once per time step after the
// corrector and the boundary conditions, before the levels rotate
// (src/EW.C:2797-2835), with the Cartesian formulas of EW::extractRecordData
// (src/EW.C:5854-6072; GPU twin extractRecordData_dev, src/device-routines.C:13818)
// and copies the values to the host every step.  Here one launch per step writes
// one row of a device-resident record array (receivers x values), so a step
// sequence never reads back to the host; the caller fetches the whole record
// array when it wants it.
#include "common.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

template <class Field>
__global__ void record_kernel(Box b, Field up, Field um, ReceiverSet r, double* __restrict__ row,
                              double dt, double inv2h, int initial, const double* __restrict__ clk,
                              int nvals)
{
   const int n = blockIdx.x * blockDim.x + threadIdx.x;
   if (n >= r.n) return;
   if (clk) row += (long long)clk[1] * nvals;  // the row from the device clock
   const int i = r.ijk[3 * n], j = r.ijk[3 * n + 1], k = r.ijk[3 * n + 2];
   double* out = row + r.off[n];
   auto U = [&](int c, int ii, int jj, int kk) { return up.get(cidx(b, c, ii, jj, kk)); };
   const int mode = r.mode[n];
   if (mode == kRecDisplacement) {
      for (int c = 0; c < 3; c++) out[c] = U(c, i, j, k);
      return;
   }
   if (mode == kRecVelocity) {
      // second-order centred difference in time; undefined for the initial data,
      // which the reference does not record (src/EW.C:2489-2491)
      for (int c = 0; c < 3; c++)
         out[c] = initial ? 0.0 : (U(c, i, j, k) - um.get(cidx(b, c, i, j, k))) / (2 * dt);
      return;
   }
   // centred first differences du_c/dx_a, scaled by 1/(2h)
   double g[3][3];
   for (int c = 0; c < 3; c++) {
      g[c][0] = (U(c, i + 1, j, k) - U(c, i - 1, j, k)) * inv2h;
      g[c][1] = (U(c, i, j + 1, k) - U(c, i, j - 1, k)) * inv2h;
      g[c][2] = (U(c, i, j, k + 1) - U(c, i, j, k - 1)) * inv2h;
   }
   if (mode == kRecDiv) {
      // the reference sums the three differences before scaling
      out[0] = ((U(0, i + 1, j, k) - U(0, i - 1, j, k) + U(1, i, j + 1, k) - U(1, i, j - 1, k) +
                 U(2, i, j, k + 1) - U(2, i, j, k - 1)) *
                inv2h);
   } else if (mode == kRecCurl) {
      out[0] = g[2][1] - g[1][2];
      out[1] = g[0][2] - g[2][0];
      out[2] = g[1][0] - g[0][1];
   } else if (mode == kRecStrains) {
      out[0] = g[0][0];
      out[1] = g[1][1];
      out[2] = g[2][2];
      out[3] = 0.5 * (g[1][0] + g[0][1]);
      out[4] = 0.5 * (g[2][0] + g[0][2]);
      out[5] = 0.5 * (g[1][2] + g[2][1]);
   } else {  // displacement gradient, row-major du_c/dx_a
      for (int c = 0; c < 3; c++)
         for (int a = 0; a < 3; a++) out[3 * c + a] = g[c][a];
   }
}

}  // namespace

int receiver_values(int mode)
{
   switch (mode) {
      case kRecDisplacement: return 3;
      case kRecDiv: return 1;
      case kRecCurl: return 3;
      case kRecStrains: return 6;
      case kRecVelocity: return 3;
      case kRecGradient: return 9;
      default: return 0;
   }
}

int launch_record(const Box& b, const double* up, const double* um, const ReceiverSet& r,
                  double* row, double dt, double h, int initial, cudaStream_t s, const double* clk,
                  int nvals)
{
   if (r.n == 0) return kOk;
   record_kernel<<<blocks_for(r.n, 64), 64, 0, s>>>(b, F64Field{const_cast<double*>(up)},
                                                    F64Field{const_cast<double*>(um)}, r, row,
                                                    dt, 1 / (2 * h), initial, clk, nvals);
   return launch_status();
}

int launch_record_df(const Box& b, const float* up, const float* um, const ReceiverSet& r,
                     double* row, double dt, double h, int initial, cudaStream_t s,
                     const double* clk, int nvals)
{
   if (r.n == 0) return kOk;
   const long long lo = 3 * b.npts;
   record_kernel<<<blocks_for(r.n, 64), 64, 0, s>>>(b, DFField{const_cast<float*>(up), lo},
                                                    DFField{const_cast<float*>(um), lo}, r, row,
                                                    dt, 1 / (2 * h), initial, clk, nvals);
   return launch_status();
}

}  // namespace sw4g
