// Receiver recording on the device, sm_103a.
//
// The reference samples every receiver (TimeSeries) once per time step after the
// corrector and the boundary conditions, before the levels rotate
// (src/EW.C:2797-2835), with the formulas of EW::extractRecordData
// (src/EW.C:5854-6072; GPU twin extractRecordData_dev, src/device-routines.C:13818)
// and copies the values to the host every step.  A receiver on the curvilinear grid
// (topography) takes its derivatives from centred differences along q, r, s and the
// metric at its point: d/dx = (m1 d/dq + m2 d/ds) / (2 sqrt J), d/dy = (m1 d/dr + m3
// d/ds) / (2 sqrt J), d/dz = m4 d/ds / (2 sqrt J), each mode grouping its sums and
// scalings as the reference's curvilinear branches do.  Here one launch per step writes
// one row of a device-resident record array (receivers x values), so a step
// sequence never reads back to the host; the caller fetches the whole record
// array when it wants it.
#include "common.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

template <class Field>
__global__ void record_kernel(Box b, Field up, Field um, Box cb, Field cup, Field cum,
                              const double* __restrict__ met, const double* __restrict__ jac,
                              ReceiverSet r, double* __restrict__ row, double dt, double inv2h,
                              int initial, const double* __restrict__ clk, int nvals)
{
   const int n = blockIdx.x * blockDim.x + threadIdx.x;
   if (n >= r.n) return;
   if (clk) row += (long long)clk[1] * nvals;  // the row from the device clock
   const int i = r.ijk[3 * n], j = r.ijk[3 * n + 1], k = r.ijk[3 * n + 2];
   double* out = row + r.off[n];
   const bool curv = r.grid && r.grid[n] == 1;
   const Box& bb = curv ? cb : b;
   const Field f = curv ? cup : up, fm = curv ? cum : um;
   auto U = [&](int c, int ii, int jj, int kk) { return f.get(cidx(bb, c, ii, jj, kk)); };
   const int mode = r.mode[n];
   if (mode == kRecDisplacement) {
      for (int c = 0; c < 3; c++) out[c] = U(c, i, j, k);
      return;
   }
   if (mode == kRecVelocity) {
      // second-order centred difference in time; undefined for the initial data,
      // which the reference does not record (src/EW.C:2489-2491)
      for (int c = 0; c < 3; c++)
         out[c] = initial ? 0.0 : (U(c, i, j, k) - fm.get(cidx(bb, c, i, j, k))) / (2 * dt);
      return;
   }
   // undivided centred differences along the three index directions
   double dq[3], dr[3], ds[3];
   for (int c = 0; c < 3; c++) {
      dq[c] = U(c, i + 1, j, k) - U(c, i - 1, j, k);
      dr[c] = U(c, i, j + 1, k) - U(c, i, j - 1, k);
      ds[c] = U(c, i, j, k + 1) - U(c, i, j, k - 1);
   }
   double g[3][3];  // du_c/dx_a
   if (!curv) {
      for (int c = 0; c < 3; c++) {
         g[c][0] = dq[c] * inv2h;
         g[c][1] = dr[c] * inv2h;
         g[c][2] = ds[c] * inv2h;
      }
      if (mode == kRecDiv) {
         // the reference sums the six values left to right before scaling
         out[0] = (U(0, i + 1, j, k) - U(0, i - 1, j, k) + U(1, i, j + 1, k) - U(1, i, j - 1, k) +
                   U(2, i, j, k + 1) - U(2, i, j, k - 1)) *
                  inv2h;
         return;
      }
      if (mode == kRecCurl) {
         out[0] = g[2][1] - g[1][2];
         out[1] = g[0][2] - g[2][0];
         out[2] = g[1][0] - g[0][1];
         return;
      }
   } else {
      const long long p = pidx(cb, i, j, k);
      const double m1 = met[p], m2 = met[cb.npts + p], m3 = met[2 * cb.npts + p],
                   m4 = met[3 * cb.npts + p];
      const double fac = 0.5 / sqrt(jac[p]);
      if (mode == kRecDiv) {  // src/EW.C:5882-5891
         out[0] = (m1 * dq[0] + m1 * dr[1] + m2 * ds[0] + m3 * ds[1] + m4 * ds[2]) * fac;
         return;
      }
      // x: m1 d/dq + m2 d/ds, y: m1 d/dr + m3 d/ds, z: m4 d/ds, unscaled
      double d[3][3];
      for (int c = 0; c < 3; c++) {
         d[c][0] = m1 * dq[c] + m2 * ds[c];
         d[c][1] = m1 * dr[c] + m3 * ds[c];
         d[c][2] = m4 * ds[c];
      }
      if (mode == kRecCurl) {  // scaled after the difference (src/EW.C:5922-5944)
         out[0] = (d[2][1] - d[1][2]) * fac;
         out[1] = (d[0][2] - d[2][0]) * fac;
         out[2] = (d[1][0] - d[0][1]) * fac;
         return;
      }
      for (int c = 0; c < 3; c++)
         for (int a = 0; a < 3; a++) g[c][a] = d[c][a] * fac;
   }
   if (mode == kRecStrains) {
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
                  int nvals, const RecCurv* cv)
{
   if (r.n == 0) return kOk;
   const RecCurv c = cv ? *cv : RecCurv{};
   auto fld = [](const void* p) { return F64Field{static_cast<double*>(const_cast<void*>(p))}; };
   record_kernel<<<blocks_for(r.n, 64), 64, 0, s>>>(b, fld(up), fld(um), c.b, fld(c.up), fld(c.um), c.met,
                                                    c.jac, r, row, dt, 1 / (2 * h), initial, clk, nvals);
   return launch_status();
}

int launch_record_df(const Box& b, const float* up, const float* um, const ReceiverSet& r,
                     double* row, double dt, double h, int initial, cudaStream_t s,
                     const double* clk, int nvals, const RecCurv* cv)
{
   if (r.n == 0) return kOk;
   const RecCurv c = cv ? *cv : RecCurv{};
   const long long lo = 3 * b.npts, clo = 3 * c.b.npts;
   auto fld = [](const void* p, long long l) {
      return DFField{static_cast<float*>(const_cast<void*>(p)), l};
   };
   record_kernel<<<blocks_for(r.n, 64), 64, 0, s>>>(b, fld(up, lo), fld(um, lo), c.b, fld(c.up, clo),
                                                    fld(c.um, clo), c.met, c.jac, r, row, dt, 1 / (2 * h),
                                                    initial, clk, nvals);
   return launch_status();
}

}  // namespace sw4g
