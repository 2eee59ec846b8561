// Curvilinear-grid kernels for the elastic time step over topography, sm_103a.
//
// The grid is Cartesian in x, y (x = (i-1)h, y = (j-1)h) and follows the
// topography in z, z = z(i,j,k).  With index-space derivatives z_p, z_q, z_r the
// metric is m1 = sqrt(z_r), m2 = -z_p/m1, m3 = -z_q/m1, m4 = h/m1 and the
// Jacobian J = h^2 z_r (EW::metric_rev, src/curvilinear-c.C:175).  The operator
// (rhs4sgcurv / rhs4sgcurv_rev, src/rhs4sgcurv*.C:34) is
//   Lu_c = (sx sy / J) * sum over axis pairs (a, b) of D_a( C^{ab}_{cd} D_b u_d )
// with 4th-order variable-coefficient second differences for a == b (SBP rows
// acof/ghcof in r at a free-surface top) and outer/inner 4th-order centred first
// differences for a != b (SBP rows bope in r at the top).  Which coefficient
// multiplies which component, and the 1/sx, 1/sy factors, are the reference's;
// they are tabulated in kCross / kSame below.
//
// These are the kernel-level entry points (one thread per point) and the
// set-up kernels of a curvilinear grid: metric, grid over a Gaussian hill, the
// curvilinear free-surface ghost plane (freesurfcurvisg, src/curvilinear-c.C:621),
// supergrid damping in x, y (addsgd4cfort, src/ew-cfromfort.C:1160/1323) and the
// curvilinear time-step limit (EW::computeDT, src/EW.C:5066-5125).
#include <math.h>

#include "common.cuh"
#include "kernels.h"
#include "sbp.h"

namespace sw4g {
namespace {

__constant__ double c_acof[384];
__constant__ double c_bope[48];
__constant__ double c_ghcof[6];
bool g_curv_tables[64] = {};

int upload_curv_tables()
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess) return kCudaError;
   if (dev < 0 || dev >= 64) return kBadArgument;
   if (g_curv_tables[dev]) return kOk;
   double acof[384], ghcof[6], bope[48], sbop[5];
   sbp_coefficients(acof, ghcof, bope, sbop);
   if (cudaMemcpyToSymbol(c_acof, acof, sizeof(acof)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(c_bope, bope, sizeof(bope)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(c_ghcof, ghcof, sizeof(ghcof)) != cudaSuccess) return kCudaError;
   g_curv_tables[dev] = true;
   return kOk;
}

constexpr double kC1 = 2.0 / 3, kC2 = -1.0 / 12;

// Coefficient kinds at a point; sx, sy taken at that point's i, j.
enum Kind : int {
   K_2ML_11_SX, K_MU_11_SX, K_MU_11_SY, K_2ML_11_SY, K_MU_11, K_LA_11, K_2ML_21_SX, K_MU_31,
   K_MU_41, K_LA_31_SY, K_LA_41, K_MU_31_SY, K_LA_21, K_MU_21, K_LA_31, K_MU_21_SX, K_2ML_31_SY,
};

struct XEnt {
   int kind, comp, scale;  // scale: 0 -> 1, 1 -> 1/sx, 2 -> 1/sy (of the centre point)
};
struct XTerm {
   int n;
   XEnt e[3];
};

// axis pairs (outer, inner): PQ, QP, PR, RP, QR, RQ
__device__ constexpr int kOuter[6] = {1, 0, 2, 0, 2, 1};
__device__ constexpr int kInner[6] = {0, 1, 0, 2, 1, 2};

__device__ constexpr XTerm kCross[3][6] = {
   {{1, {{K_MU_11, 1, 0}}},
    {1, {{K_LA_11, 1, 0}}},
    {3, {{K_2ML_21_SX, 0, 2}, {K_MU_31, 1, 0}, {K_MU_41, 2, 2}}},
    {3, {{K_2ML_21_SX, 0, 2}, {K_LA_31_SY, 1, 2}, {K_LA_41, 2, 2}}},
    {2, {{K_MU_31_SY, 0, 1}, {K_LA_21, 1, 0}}},
    {2, {{K_MU_31_SY, 0, 1}, {K_MU_21, 1, 0}}}},
   {{1, {{K_LA_11, 0, 0}}},
    {1, {{K_MU_11, 0, 0}}},
    {2, {{K_LA_31, 0, 0}, {K_MU_21_SX, 1, 2}}},
    {2, {{K_MU_31, 0, 0}, {K_MU_21_SX, 1, 2}}},
    {3, {{K_MU_21, 0, 0}, {K_2ML_31_SY, 1, 1}, {K_MU_41, 2, 1}}},
    {3, {{K_LA_21, 0, 0}, {K_2ML_31_SY, 1, 1}, {K_LA_41, 2, 1}}}},
   {{0, {}},
    {0, {}},
    {2, {{K_LA_41, 0, 2}, {K_MU_21_SX, 2, 2}}},
    {2, {{K_MU_41, 0, 2}, {K_MU_21_SX, 2, 2}}},
    {2, {{K_MU_31_SY, 2, 1}, {K_LA_41, 1, 1}}},
    {2, {{K_MU_31_SY, 2, 1}, {K_MU_41, 1, 1}}}},
};

// same-axis coefficient kinds [equation][p, q]
__device__ constexpr int kSame[3][2] = {
   {K_2ML_11_SX, K_MU_11_SY}, {K_MU_11_SX, K_2ML_11_SY}, {K_MU_11_SX, K_MU_11_SY}};

struct CurvView {
   Box b;
   long long mcs, mps;  // metric component / point stride
   const double* u;
   const double* mu;
   const double* la;
   const double* met;
   const double* jac;
   const double* sx;
   const double* sy;

   __device__ __forceinline__ long long p(int i, int j, int k) const { return pidx(b, i, j, k); }
   __device__ __forceinline__ double U(int c, int i, int j, int k) const
   {
      return __ldg(u + c * b.cs + b.ps * p(i, j, k));
   }
   __device__ __forceinline__ double M(int c, long long q) const { return __ldg(met + c * mcs + mps * q); }
   __device__ __forceinline__ double SX(int i) const { return __ldg(sx + (i - b.ib)); }
   __device__ __forceinline__ double SY(int j) const { return __ldg(sy + (j - b.jb)); }

   __device__ __forceinline__ double coef(int kind, int i, int j, int k) const
   {
      const long long q = p(i, j, k);
      const double m = __ldg(mu + q), l = __ldg(la + q), m1 = M(0, q);
      switch (kind) {
         case K_2ML_11_SX: return (2 * m + l) * m1 * m1 * SX(i);
         case K_MU_11_SX: return m * m1 * m1 * SX(i);
         case K_MU_11_SY: return m * m1 * m1 * SY(j);
         case K_2ML_11_SY: return (2 * m + l) * m1 * m1 * SY(j);
         case K_MU_11: return m * m1 * m1;
         case K_LA_11: return l * m1 * m1;
         case K_2ML_21_SX: return (2 * m + l) * M(1, q) * m1 * SX(i);
         case K_MU_31: return m * M(2, q) * m1;
         case K_MU_41: return m * M(3, q) * m1;
         case K_LA_31_SY: return l * M(2, q) * m1 * SY(j);
         case K_LA_41: return l * M(3, q) * m1;
         case K_MU_31_SY: return m * M(2, q) * m1 * SY(j);
         case K_LA_21: return l * M(1, q) * m1;
         case K_MU_21: return m * M(1, q) * m1;
         case K_LA_31: return l * M(2, q) * m1;
         case K_MU_21_SX: return m * M(1, q) * m1 * SX(i);
         default: return (2 * m + l) * M(2, q) * m1 * SY(j);  // K_2ML_31_SY
      }
   }

   // r-r coefficient matrix entry A_cd at (i,j,k) with the column's stretching
   __device__ __forceinline__ double rr(int c, int d, int i, int j, int k, double sxc,
                                        double syc) const
   {
      const long long q = p(i, j, k);
      const double m = __ldg(mu + q), l = __ldg(la + q);
      const double g[3] = {M(1, q), M(2, q), M(3, q)};
      if (c == d) {
         const double s[3] = {g[0] * sxc, g[1] * syc, g[2]};
         double o = 0;
#pragma unroll
         for (int e = 0; e < 3; e++)
            if (e != c) o += s[e] * s[e];
         return (2 * m + l) * s[c] * s[c] + m * o;
      }
      return (m + l) * g[c] * g[d];
   }
};

__device__ __forceinline__ void step_axis(int ax, int m, int& i, int& j, int& k)
{
   if (ax == 0) i += m;
   else if (ax == 1) j += m;
   else k += m;
}

__device__ __forceinline__ double d2v(const double c[5], const double f[5])
{
   const double w1 = c[1] - 0.75 * (c[2] + c[0]);
   const double w2 = c[0] + c[3] + 3 * (c[2] + c[1]);
   const double w3 = c[1] + c[4] + 3 * (c[3] + c[2]);
   const double w4 = c[3] - 0.75 * (c[2] + c[4]);
   return (w1 * (f[0] - f[2]) + w2 * (f[1] - f[2]) + w3 * (f[3] - f[2]) + w4 * (f[4] - f[2])) *
          (1.0 / 6);
}

template <bool BND>
__device__ void curv_point(const CurvView& a, int i, int j, int k, double r[3])
{
   const double sxc = a.SX(i), syc = a.SY(j);
   const double istrx = 1 / sxc, istry = 1 / syc, istrxy = istry * istrx;
   const double scl[3] = {1, istrx, istry};
   r[0] = r[1] = r[2] = 0;
#pragma unroll
   for (int c = 0; c < 3; c++)
#pragma unroll
      for (int ax = 0; ax < 2; ax++) {
         double cf[5], f[5];
#pragma unroll
         for (int m = -2; m <= 2; m++) {
            int ii = i, jj = j, kk = k;
            step_axis(ax, m, ii, jj, kk);
            cf[m + 2] = a.coef(kSame[c][ax], ii, jj, kk);
            f[m + 2] = a.U(c, ii, jj, kk);
         }
         r[c] += d2v(cf, f) * (ax == 0 ? istry : istrx);
      }
   const double rs[3][3] = {{istrxy, 1, istry}, {1, istrxy, istrx}, {istry, istrx, istrxy}};
#pragma unroll
   for (int c = 0; c < 3; c++)
#pragma unroll
      for (int d = 0; d < 3; d++) {
         double s = 0;
         if (!BND) {
            double cf[5], f[5];
#pragma unroll
            for (int m = -2; m <= 2; m++) {
               cf[m + 2] = a.rr(c, d, i, j, k + m, sxc, syc);
               f[m + 2] = a.U(d, i, j, k + m);
            }
            s = d2v(cf, f);
         } else {
            double cm[8];
#pragma unroll
            for (int m = 1; m <= 8; m++) cm[m - 1] = a.rr(c, d, i, j, m, sxc, syc);
#pragma unroll
            for (int q = 1; q <= 8; q++) {
               double cq = 0;
#pragma unroll
               for (int m = 1; m <= 8; m++) cq += c_acof[(k - 1) + 6 * (q - 1) + 48 * (m - 1)] * cm[m - 1];
               s += cq * a.U(d, i, j, q);
            }
            s += c_ghcof[k - 1] * cm[0] * a.U(d, i, j, 0);
         }
         r[c] += rs[c][d] * s;
      }
#pragma unroll
   for (int c = 0; c < 3; c++)
#pragma unroll
      for (int pr = 0; pr < 6; pr++) {
         const XTerm& t = kCross[c][pr];
         if (t.n == 0) continue;
         const int ao = kOuter[pr], ai = kInner[pr];
         const bool bo = BND && ao == 2, bi = BND && ai == 2;
         constexpr int NQ = BND ? 8 : 5;
         double G[NQ];
#pragma unroll
         for (int s = 0; s < (bo ? 8 : 5); s++) {
            int ii = i, jj = j, kk = k;
            if (bo) kk = s + 1;
            else step_axis(ao, s - 2, ii, jj, kk);
            double g = 0;
#pragma unroll
            for (int e = 0; e < 3; e++) {
               if (e >= t.n) break;
               const XEnt& x = t.e[e];
               double du;
               if (bi) {
                  du = 0;
#pragma unroll
                  for (int q = 1; q <= 8; q++) du += c_bope[(k - 1) + 6 * (q - 1)] * a.U(x.comp, ii, jj, q);
               } else {
                  double f[5];
#pragma unroll
                  for (int m = -2; m <= 2; m++) {
                     int i2 = ii, j2 = jj, k2 = kk;
                     step_axis(ai, m, i2, j2, k2);
                     f[m + 2] = a.U(x.comp, i2, j2, k2);
                  }
                  du = kC2 * (f[4] - f[0]) + kC1 * (f[3] - f[1]);
               }
               g += a.coef(x.kind, ii, jj, kk) * scl[x.scale] * du;
            }
            G[s] = g;
         }
         double d;
         if (bo) {
            d = 0;
#pragma unroll
            for (int q = 1; q <= 8; q++) d += c_bope[(k - 1) + 6 * (q - 1)] * G[q - 1];
         } else {
            d = kC2 * (G[4] - G[0]) + kC1 * (G[3] - G[1]);
         }
         r[c] += d;
      }
   const double ijac = sxc * syc / __ldg(a.jac + a.p(i, j, k));
   r[0] *= ijac;
   r[1] *= ijac;
   r[2] *= ijac;
}

template <bool BND>
__global__ void __launch_bounds__(128) rhs4sgcurv_kernel(CurvView a, double* __restrict__ lu,
                                                         int k1, int k2)
{
   const int i = a.b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = a.b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = k1 + blockIdx.z;
   if (i > a.b.ie - 2 || j > a.b.je - 2 || k > k2) return;
   double r[3];
   curv_point<BND>(a, i, j, k, r);
   const long long q = a.p(i, j, k);
#pragma unroll
   for (int c = 0; c < 3; c++) lu[c * a.b.cs + a.b.ps * q] = r[c];
}

// index-space first derivative along a line of n values at position q: centred
// 4th order inside, 6-point one-sided 4th-order differences on the two outermost
// points at each end (src/curvilinear-c.C:197-276)
__device__ double line_diff(const double* f, long long st, int q, int n)
{
   auto F = [&](int m) { return f[(long long)(q + m) * st]; };
   if (q >= 2 && q <= n - 3) return kC2 * (F(2) - F(-2)) + kC1 * (F(1) - F(-1));
   if (q == 0)
      return -2.25 * F(0) + (4 + 5.0 / 6) * F(1) - 14.0 / 3 * F(2) + 3 * F(3) - (1 + 1.0 / 12) * F(4) +
             F(5) / 6;
   if (q == 1)
      return -F(-1) / 6 - 1.25 * F(0) + (1 + 4.0 / 3) * F(1) - 4.0 / 3 * F(2) + 0.5 * F(3) - F(4) / 12;
   if (q == n - 2)
      return F(1) / 6 + 1.25 * F(0) - (1 + 4.0 / 3) * F(-1) + 4.0 / 3 * F(-2) - 0.5 * F(-3) + F(-4) / 12;
   return 2.25 * F(0) - (4 + 5.0 / 6) * F(-1) + 14.0 / 3 * F(-2) - 3 * F(-3) + (1 + 1.0 / 12) * F(-4) -
          F(-5) / 6;
}

__global__ void metric_kernel(Box b, long long mcs, long long mps, double h,
                              const double* __restrict__ z, double* __restrict__ met,
                              double* __restrict__ jac, int* __restrict__ bad)
{
   const int ni = b.ie - b.ib + 1, nj = b.je - b.jb + 1, nk = b.ke - b.kb + 1;
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const int ii = (int)(p % ni), jj = (int)((p / ni) % nj), kk = (int)(p / b.nij);
      const double zr = line_diff(z + (p - (long long)kk * b.nij), b.nij, kk, nk);
      const double zq = line_diff(z + (p - (long long)jj * b.ni), b.ni, jj, nj);
      const double zp = line_diff(z + (p - ii), 1, ii, ni);
      if (!(zr > 0)) {
         atomicOr(bad, 1);
         continue;
      }
      const double s = sqrt(zr);
      jac[p] = h * h * zr;
      met[0 * mcs + mps * p] = s;
      met[1 * mcs + mps * p] = -zp / s;
      met[2 * mcs + mps * p] = -zq / s;
      met[3 * mcs + mps * p] = h / s;
   }
}

__global__ void hill_kernel(Box b, int nz, double h, double zmax, double izb, int order, double amp,
                            double xc, double yc, double ilx2, double ily2, double* __restrict__ z)
{
   const int ni = b.ie - b.ib + 1, nj = b.je - b.jb + 1;
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(p % ni), j = b.jb + (int)((p / ni) % nj), k = b.kb + (int)(p / b.nij);
      const double x = (i - 1.0) * h, y = (j - 1.0) * h;
      const double zs = -amp * exp(-(x - xc) * (x - xc) * ilx2 - (y - yc) * (y - yc) * ily2);
      const double sa = (k - 1) * izb;
      double om = 1 - sa;
      for (int l = 2; l <= order; l++) om *= (1 - sa);
      double zz = zmax - (nz - k) * h;
      if (sa < 1) zz -= om * (zmax - (nz - 1) * h - zs);
      z[p] = zz;
   }
}

// Free-surface ghost plane; one thread per (i,j)
template <class Field>
__global__ void freesurf_curv_kernel(CurvView a, int k, int kl, double s0, double s1, double s2,
                                     double s3, double s4, const double* __restrict__ forcing,
                                     Field u)
{
   auto U = [&](int c, int ii, int jj, int kk) { return u.get(c * a.b.cs + a.b.ps * a.p(ii, jj, kk)); };
   const int i = a.b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = a.b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   if (i > a.b.ie - 2 || j > a.b.je - 2) return;
   const double sxv = a.SX(i), syv = a.SY(j);
   const double istrx = 1 / sxv, istry = 1 / syv;
   const double scl[3] = {1, istrx, istry};
   double rhs[3];
#pragma unroll
   for (int c = 0; c < 3; c++) {
      double g = 0;
#pragma unroll
      for (int pr = 2; pr <= 4; pr += 2) {  // PR and QR: the traction's tangential part
         const XTerm& t = kCross[c][pr];
         const int ai = kInner[pr];
#pragma unroll
         for (int e = 0; e < 3; e++) {
            if (e >= t.n) break;
            const XEnt& x = t.e[e];
            double f[5];
#pragma unroll
            for (int m = -2; m <= 2; m++) {
               int i2 = i, j2 = j, k2 = k;
               step_axis(ai, m, i2, j2, k2);
               f[m + 2] = U(x.comp, i2, j2, k2);
            }
            g += a.coef(x.kind, i, j, k) * scl[x.scale] * (kC2 * (f[4] - f[0]) + kC1 * (f[3] - f[1]));
         }
      }
      const double fo = forcing ? forcing[3 * ((i - a.b.ib) + a.b.ni * (j - a.b.jb)) + c] : 0.0;
      rhs[c] = g - fo;
   }
   const long long q = a.p(i, j, k);
   const double m2 = a.M(1, q), m3 = a.M(2, q), m4 = a.M(3, q);
   const double mu0 = __ldg(a.mu + q), la0 = __ldg(a.la + q);
   const double ac = sxv * istry * m2 * m2 + syv * istrx * m3 * m3 + m4 * m4 * istry * istrx;
   const double bc = 1 / (mu0 * ac);
   const double cc = (mu0 + la0) / (2 * mu0 + la0) * bc / ac;
   const double xoy = sqrt(sxv * istry), yox = 1 / xoy, ixy = istrx * xoy;
   const double dc = cc * (xoy * m2 * rhs[0] + yox * m3 * rhs[1] + ixy * m4 * rhs[2]);
   const double nrm[3] = {m2 * xoy, m3 * yox, m4 * ixy};
   const double sb[4] = {s1, s2, s3, s4};
#pragma unroll
   for (int c = 0; c < 3; c++) {
      double s = 0;
#pragma unroll
      for (int w = 0; w < 4; w++) s += sb[w] * U(c, i, j, k + w * kl);
      u.set(c * a.b.cs + a.b.ps * a.p(i, j, k - kl), -(1 / s0) * (s + bc * rhs[c] - dc * nrm[c]));
   }
}

__global__ void addsgd4c_kernel(Box b, double* __restrict__ up, const double* __restrict__ u,
                                const double* __restrict__ um, const double* __restrict__ rho,
                                const double* __restrict__ dcx, const double* __restrict__ dcy,
                                const double* __restrict__ strx, const double* __restrict__ stry,
                                const double* __restrict__ jac, const double* __restrict__ cox,
                                const double* __restrict__ coy, double beta)
{
   const int i = b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = b.kb + 2 + blockIdx.z;
   if (i > b.ie - 2 || j > b.je - 2 || k > b.ke - 2) return;
   const long long p = pidx(b, i, j, k);
   const double irhoj = beta / (rho[p] * jac[p]);
#pragma unroll
   for (int c = 0; c < 3; c++) {
      const long long o = c * b.cs;
      double acc = 0;
#pragma unroll
      for (int ax = 0; ax < 2; ax++) {
         const long long st = ax == 0 ? 1 : b.ni;
         const double* dc = ax == 0 ? dcx : dcy;
         const int q = ax == 0 ? i - b.ib : j - b.jb;
         const double w = ax == 0 ? strx[i - b.ib] * coy[j - b.jb] : stry[j - b.jb] * cox[i - b.ib];
         double s = 0;
#pragma unroll
         for (int m = -1; m <= 1; m++) {
            const long long pm = p + m * st;
            const double e = rho[pm] * dc[q + m] * jac[pm];
            const double du = u[o + b.ps * (pm + st)] - 2 * u[o + b.ps * pm] + u[o + b.ps * (pm - st)];
            const double dm = um[o + b.ps * (pm + st)] - 2 * um[o + b.ps * pm] + um[o + b.ps * (pm - st)];
            s += (m == 0 ? -2 : 1) * e * (du - dm);
         }
         acc += w * s;
      }
      up[o + b.ps * p] -= irhoj * acc;
   }
}

// Smallest eigenvalue of a symmetric 3x3 matrix by the trigonometric method
// (O. K. Smith, "Eigenvalues of a symmetric 3x3 matrix", Commun. ACM 4(4), 1961).
__device__ double sym3_min_eig(double a00, double a01, double a02, double a11, double a12, double a22)
{
   const double p1 = a01 * a01 + a02 * a02 + a12 * a12;
   const double q = (a00 + a11 + a22) / 3;
   if (p1 == 0) return fmin(a00, fmin(a11, a22));
   const double p2 = (a00 - q) * (a00 - q) + (a11 - q) * (a11 - q) + (a22 - q) * (a22 - q) + 2 * p1;
   const double p = sqrt(p2 / 6);
   const double b00 = (a00 - q) / p, b11 = (a11 - q) / p, b22 = (a22 - q) / p;
   const double b01 = a01 / p, b02 = a02 / p, b12 = a12 / p;
   double r = 0.5 * (b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) +
                     b02 * (b01 * b12 - b11 * b02));
   r = fmin(1.0, fmax(-1.0, r));
   const double phi = acos(r) / 3;
   return q + 2 * p * cos(phi + 2 * 3.14159265358979323846 / 3);
}

// per-block maximum of -lambda_min(A)/(4 rho); A from EW::computeDT (src/EW.C:5085-5097)
__global__ void curv_eig_kernel(long long n, long long mcs, long long mps,
                                const double* __restrict__ rho, const double* __restrict__ mu,
                                const double* __restrict__ la, const double* __restrict__ met,
                                const double* __restrict__ jac, double* __restrict__ blockmax)
{
   __shared__ double red[256];
   double best = -1;
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
        p += (long long)gridDim.x * blockDim.x) {
      const double l = la[p], m = mu[p], l2m = l + 2 * m, ji = 1 / jac[p];
      const double m1 = met[mps * p], m2 = met[mcs + mps * p], m3 = met[2 * mcs + mps * p],
                   m4 = met[3 * mcs + mps * p];
      const double e = -sym3_min_eig(
                           -4 * (m1 * m1 * l2m + m1 * m1 * m + m2 * m2 * l2m + m3 * m3 * m + m4 * m4 * m) * ji,
                           -4 * m2 * m3 * (m + l) * ji, -4 * m2 * m4 * (m + l) * ji,
                           -4 * (m1 * m1 * m + m1 * m1 * l2m + m2 * m2 * m + m3 * m3 * l2m + m4 * m4 * m) * ji,
                           -4 * m3 * m4 * (m + l) * ji,
                           -4 * (m1 * m1 * m + m1 * m1 * m + m2 * m2 * m + m3 * m3 * m + m4 * m4 * l2m) * ji) /
                       (4 * rho[p]);
      best = fmax(best, e);
   }
   red[threadIdx.x] = best;
   __syncthreads();
   for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
      __syncthreads();
   }
   if (threadIdx.x == 0) blockmax[blockIdx.x] = red[0];
}

// enforceCartTopo (src/EW.C:3504-3530) with 2 ghost points: Cartesian k = -1, 0
// from curvilinear k = nzc-2, nzc-1, and curvilinear k = nzc..nzc+2 from Cartesian
// k = 1..3, over the shared i, j range; one thread per (i, j).
// The double-float form copies hi and lo (Field::copy).
template <class Field>
__global__ void cart_topo_kernel(Box bc, Box bv, int nzc, Field uc, Field uv)
{
   const int i = bc.ib + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = bc.jb + blockIdx.y * blockDim.y + threadIdx.y;
   if (i > bc.ie || j > bc.je) return;
#pragma unroll
   for (int c = 0; c < 3; c++) {
#pragma unroll
      for (int q = 0; q < 2; q++)
         Field::copy(uc, c * bc.cs + pidx(bc, i, j, bc.kb + q), uv, c * bv.cs + pidx(bv, i, j, nzc - 2 + q));
#pragma unroll
      for (int q = 0; q <= 2; q++)
         Field::copy(uv, c * bv.cs + pidx(bv, i, j, bv.ke - q), uc, c * bc.cs + pidx(bc, i, j, bc.kb + 4 - q));
   }
}

int grid_stride(long long n)
{
   long long b = (n + 255) / 256;
   if (b > 152 * 16) b = 152 * 16;
   return (int)(b > 0 ? b : 1);
}

CurvView make_view(const CurvSpec& s)
{
   CurvView v;
   v.b = make_box(s.soa, s.ib, s.ie, s.jb, s.je, s.kb, s.ke);
   v.mcs = s.soa ? v.b.npts : 1;
   v.mps = s.soa ? 1 : 4;
   v.u = s.u;
   v.mu = s.mu;
   v.la = s.la;
   v.met = s.met;
   v.jac = s.jac;
   v.sx = s.strx;
   v.sy = s.stry;
   return v;
}

}  // namespace

int launch_rhs4sgcurv(const CurvSpec& s, const int onesided[6], double* lu, cudaStream_t st)
{
   SW4G_TRY(upload_curv_tables());
   const CurvView v = make_view(s);
   const dim3 blk(32, 4);
   const int ni = s.ie - s.ib - 3, nj = s.je - s.jb - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const bool top = onesided && onesided[4] == 1;
   int k1 = s.kb + 2;
   if (top) {
      if (s.kb > 0 || s.ke < 8) return kBadArgument;  // the closure reads planes 0..8
      const dim3 g((ni + 31) / 32, (nj + 3) / 4, 6);
      rhs4sgcurv_kernel<true><<<g, blk, 0, st>>>(v, lu, 1, 6);
      SW4G_TRY(launch_status());
      k1 = 7;
   }
   const int k2 = s.ke - 2;
   if (k2 >= k1) {
      const dim3 g((ni + 31) / 32, (nj + 3) / 4, k2 - k1 + 1);
      rhs4sgcurv_kernel<false><<<g, blk, 0, st>>>(v, lu, k1, k2);
   }
   return launch_status();
}

int launch_rhs4sgcurv_top(const CurvSpec& s, double* lu, cudaStream_t st)
{
   SW4G_TRY(upload_curv_tables());
   if (s.kb > 0 || s.ke < 8) return kBadArgument;
   const CurvView v = make_view(s);
   const int ni = s.ie - s.ib - 3, nj = s.je - s.jb - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const dim3 blk(32, 4), g((ni + 31) / 32, (nj + 3) / 4, 6);
   rhs4sgcurv_kernel<true><<<g, blk, 0, st>>>(v, lu, 1, 6);
   return launch_status();
}

int launch_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double h, const double* z,
                  double* met, double* jac, int* bad_flag, cudaStream_t st)
{
   const Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   if (ie - ib + 1 < 6 || je - jb + 1 < 6 || ke - kb + 1 < 6) return kBadArgument;
   metric_kernel<<<grid_stride(b.npts), 256, 0, st>>>(b, soa ? b.npts : 1, soa ? 1 : 4, h, z, met,
                                                       jac, bad_flag);
   return launch_status();
}

int launch_gaussian_hill_z(int ib, int ie, int jb, int je, int kb, int ke, int nz, double h,
                           double zmax, double zeta_break, int order, double amp, double xc,
                           double yc, double lx, double ly, double* z, cudaStream_t st)
{
   const Box b = make_box(1, ib, ie, jb, je, kb, ke);
   hill_kernel<<<grid_stride(b.npts), 256, 0, st>>>(b, nz, h, zmax, 1.0 / (zeta_break * (nz - 1)),
                                                     order, amp, xc, yc, 1 / (lx * lx),
                                                     1 / (ly * ly), z);
   return launch_status();
}

int launch_freesurfcurvisg(const CurvSpec& s, int nz, int side, const double* sbop,
                           const double* forcing, double* u, cudaStream_t st)
{
   if (side != 5 && side != 6) return kBadArgument;
   CurvView v = make_view(s);
   v.u = u;
   const int k = side == 5 ? 1 : nz, kl = side == 5 ? 1 : -1;
   const int ni = s.ie - s.ib - 3, nj = s.je - s.jb - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const dim3 blk(32, 4), g((ni + 31) / 32, (nj + 3) / 4);
   freesurf_curv_kernel<<<g, blk, 0, st>>>(v, k, kl, sbop[0], sbop[1], sbop[2], sbop[3], sbop[4],
                                           forcing, F64Field{u});
   return launch_status();
}

int launch_freesurfcurvisg_df(const CurvSpec& s, int nz, int side, const double* sbop, float* uh,
                              cudaStream_t st)
{
   if (side != 5 && side != 6) return kBadArgument;
   if (!s.soa) return kNotSupported;
   CurvView v = make_view(s);
   const int k = side == 5 ? 1 : nz, kl = side == 5 ? 1 : -1;
   const int ni = s.ie - s.ib - 3, nj = s.je - s.jb - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const dim3 blk(32, 4), g((ni + 31) / 32, (nj + 3) / 4);
   freesurf_curv_kernel<<<g, blk, 0, st>>>(v, k, kl, sbop[0], sbop[1], sbop[2], sbop[3], sbop[4],
                                           nullptr, DFField{uh, 3 * v.b.npts});
   return launch_status();
}

int launch_addsgd4c(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                    const double* u, const double* um, const double* rho, const double* dcx,
                    const double* dcy, const double* strx, const double* stry, const double* jac,
                    const double* cox, const double* coy, double beta, cudaStream_t st)
{
   if (beta == 0) return kOk;
   const Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   const int ni = ie - ib - 3, nj = je - jb - 3, nk = ke - kb - 3;
   if (ni <= 0 || nj <= 0 || nk <= 0) return kOk;
   const dim3 blk(32, 4), g((ni + 31) / 32, (nj + 3) / 4, nk);
   addsgd4c_kernel<<<g, blk, 0, st>>>(b, up, u, um, rho, dcx, dcy, strx, stry, jac, cox, coy, beta);
   return launch_status();
}

int launch_cart_topo(const Box& cart, const Box& curv, int nzc, double* ucart, double* ucurv,
                     cudaStream_t st)
{
   const dim3 blk(32, 4), g((cart.ie - cart.ib + 32) / 32, (cart.je - cart.jb + 4) / 4);
   cart_topo_kernel<<<g, blk, 0, st>>>(cart, curv, nzc, F64Field{ucart}, F64Field{ucurv});
   return launch_status();
}

int launch_cart_topo_df(const Box& cart, const Box& curv, int nzc, float* ucart, float* ucurv,
                        cudaStream_t st)
{
   const dim3 blk(32, 4), g((cart.ie - cart.ib + 32) / 32, (cart.je - cart.jb + 4) / 4);
   cart_topo_kernel<<<g, blk, 0, st>>>(cart, curv, nzc, DFField{ucart, 3 * cart.npts},
                                       DFField{ucurv, 3 * curv.npts});
   return launch_status();
}

int launch_curv_eig(int soa, long long n, const double* rho, const double* mu, const double* la,
                    const double* met, const double* jac, double* blockmax, int nblocks,
                    cudaStream_t st)
{
   curv_eig_kernel<<<nblocks, 256, 0, st>>>(n, soa ? n : 1, soa ? 1 : 4, rho, mu, la, met, jac,
                                            blockmax);
   return launch_status();
}

}  // namespace sw4g
