// Sixth-order supergrid damping on the curvilinear grid, and on the double-float
// levels of the FP32-mixed form, sm_103a.
//
//   up += beta / (2 e) sum_axes w_a sum_{m=-2..1} s_m (e(m) + e(m+1)) D3_m(u - um)
//
// with D3_m the third difference across the half point m + 1/2, s = (-1, 3, -3, 1),
// e = rho (Cartesian) or rho J (curvilinear), and w_a = str_a times the corner
// tapers of the other axes.  The Cartesian grid damps along x, y and z (addsgd6fort,
// src/ew-cfromfort.C:1059-1158; the FP64 kernel is in pointwise.cu), the curvilinear
// grid along x and y only (addsgd6cfort(_indrev), src/ew-cfromfort.C:1241-1322,
// :1405).  Both apply to every point three away from each array edge.
//
// The double-float kernel keeps the mixed form's precision rules (stage_mixed.cu):
// u - um is formed exactly from the (hi, lo) pairs and rounded once to FP32, the
// damping sum runs in FP32 on FP32 coefficients, and the result is added to the
// level with TwoSum / FastTwoSum.
#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

struct Sg6Prof {
   const double* dc[3];
   const double* st[3];
   const double* co[3];
};

__global__ void __launch_bounds__(256)
    addsgd6c_kernel(Box b, double* __restrict__ up, const double* __restrict__ u,
                    const double* __restrict__ um, const double* __restrict__ rho,
                    const double* __restrict__ dcx, const double* __restrict__ dcy,
                    const double* __restrict__ strx, const double* __restrict__ stry,
                    const double* __restrict__ jac, const double* __restrict__ cox,
                    const double* __restrict__ coy, double beta)
{
   const int i = b.ib + 3 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + 3 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = b.kb + 3 + blockIdx.z;
   if (i > b.ie - 3 || j > b.je - 3) return;
   const double kS6[4] = {-1, 3, -3, 1};  // signs and weights of the four half points
   const long long p = pidx(b, i, j, k);
   const double birhoj = 0.5 * beta / (rho[p] * jac[p]);
   const double w[2] = {strx[i - b.ib] * coy[j - b.jb], stry[j - b.jb] * cox[i - b.ib]};
   double e[2][5];
#pragma unroll
   for (int ax = 0; ax < 2; ax++) {
      const long long st = ax == 0 ? 1 : b.ni;
      const double* dc = ax == 0 ? dcx : dcy;
      const int q = ax == 0 ? i - b.ib : j - b.jb;
#pragma unroll
      for (int m = -2; m <= 2; m++) e[ax][m + 2] = rho[p + m * st] * dc[q + m] * jac[p + m * st];
   }
#pragma unroll
   for (int c = 0; c < 3; c++) {
      double acc = 0;
#pragma unroll
      for (int ax = 0; ax < 2; ax++) {
         const long long st = ax == 0 ? 1 : b.ni;
         double d[7];
#pragma unroll
         for (int m = -3; m <= 3; m++) {
            const long long x = c * b.cs + b.ps * (p + m * st);
            d[m + 3] = u[x] - um[x];
         }
         double s = 0;
#pragma unroll
         for (int m = -2; m <= 1; m++) {
            const double d3 = d[m + 5] - 3 * d[m + 4] + 3 * d[m + 3] - d[m + 2];
            s += kS6[m + 2] * (e[ax][m + 3] + e[ax][m + 2]) * d3;
         }
         acc += w[ax] * s;
      }
      up[c * b.cs + b.ps * p] += birhoj * acc;
   }
}

// The transpose of the Cartesian sixth-order damping on the interior points, as the
// adjoint's scaled recursion applies it (adjoint.cu): the reference's damping acts at
// the points three away from every array edge (the set Q) and reads u - um anywhere,
// so its transpose acts at every interior point (two away) on u - um taken as zero
// outside Q.  FP64.
__device__ __forceinline__ bool in_q(const Box& b, int i, int j, int k)
{
   return i >= b.ib + 3 && i <= b.ie - 3 && j >= b.jb + 3 && j <= b.je - 3 && k >= b.kb + 3 && k <= b.ke - 3;
}

__global__ void __launch_bounds__(256)
    addsgd6_adj_kernel(Box b, double* __restrict__ up, const double* __restrict__ u,
                       const double* __restrict__ um, const double* __restrict__ rho, Sg6Prof f, double beta)
{
   const int i = b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = b.kb + 2 + blockIdx.z;
   if (i > b.ie - 2 || j > b.je - 2) return;
   const double kS6[4] = {-1, 3, -3, 1};
   const long long p = pidx(b, i, j, k);
   const double birho = 0.5 * beta / rho[p];
   const int qv[3] = {i - b.ib, j - b.jb, k - b.kb};
   const double w[3] = {f.st[0][qv[0]] * f.co[1][qv[1]] * f.co[2][qv[2]],
                        f.st[1][qv[1]] * f.co[0][qv[0]] * f.co[2][qv[2]],
                        f.st[2][qv[2]] * f.co[0][qv[0]] * f.co[1][qv[1]]};
   const long long stv[3] = {1, b.ni, b.nij};
#pragma unroll
   for (int c = 0; c < 3; c++) {
      double tot = 0;
#pragma unroll
      for (int ax = 0; ax < 3; ax++) {
         double e[5], d[7];
#pragma unroll
         for (int m = -2; m <= 2; m++) e[m + 2] = rho[p + m * stv[ax]] * f.dc[ax][qv[ax] + m];
#pragma unroll
         for (int m = -3; m <= 3; m++) {
            const int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m, kk = k + (ax == 2) * m;
            const long long x = c * b.cs + b.ps * (p + m * stv[ax]);
            d[m + 3] = in_q(b, ii, jj, kk) ? u[x] - um[x] : 0.0;
         }
         double s = 0;
#pragma unroll
         for (int m = -2; m <= 1; m++) {
            const double d3 = d[m + 5] - 3 * d[m + 4] + 3 * d[m + 3] - d[m + 2];
            s += kS6[m + 2] * (e[m + 3] + e[m + 2]) * d3;
         }
         tot += w[ax] * s;
      }
      up[c * b.cs + b.ps * p] += birho * tot;
   }
}

struct Sg6DF {
   Box b;
   float* out;  // double-float level: hi at [c npts + p], lo 3 npts further
   const float* u;
   const float* um;
   const float* e;  // rho (Cartesian) or rho J (curvilinear), FP32
   const float* dc[3];
   const float* st[3];
   const float* co[3];
   int naxes;  // 3 Cartesian, 2 curvilinear
   float beta;
   int adj;  // 1: the transpose on the interior (every point two from the edges, the
             // input taken as zero outside the points three from every edge)
};

__global__ void __launch_bounds__(256) addsgd6_df_kernel(Sg6DF a)
{
   const Box& b = a.b;
   const int lo0 = a.adj ? 2 : 3;
   const int i = b.ib + lo0 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + lo0 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = b.kb + lo0 + blockIdx.z;
   if (i > b.ie - lo0 || j > b.je - lo0) return;
   const float kS6[4] = {-1.f, 3.f, -3.f, 1.f};
   const long long p = pidx(b, i, j, k), lo = 3 * b.npts;
   const int qv[3] = {i - b.ib, j - b.jb, k - b.kb};
   const long long stv[3] = {1, b.ni, b.nij};
   const float birho = 0.5f * a.beta / a.e[p];
   float w[3], e[3][5];
   for (int ax = 0; ax < a.naxes; ax++) {
      const int o1 = (ax + 1) % 3, o2 = (ax + 2) % 3;
      float wa = a.st[ax][qv[ax]];
      if (o1 < a.naxes) wa *= a.co[o1][qv[o1]];
      if (o2 < a.naxes) wa *= a.co[o2][qv[o2]];
      w[ax] = wa;
#pragma unroll
      for (int m = -2; m <= 2; m++) e[ax][m + 2] = a.e[p + m * stv[ax]] * a.dc[ax][qv[ax] + m];
   }
#pragma unroll
   for (int c = 0; c < 3; c++) {
      float acc = 0.f;
      for (int ax = 0; ax < a.naxes; ax++) {
         float d[7];
#pragma unroll
         for (int m = -3; m <= 3; m++) {
            const long long x = c * b.npts + p + m * stv[ax];
            if (a.adj && !in_q(b, i + (ax == 0) * m, j + (ax == 1) * m, k + (ax == 2) * m)) {
               d[m + 3] = 0.f;
               continue;
            }
            float d1, f1;
            two_sum(a.u[x], -a.um[x], d1, f1);
            d[m + 3] = d1 + (f1 + (a.u[x + lo] - a.um[x + lo]));
         }
         float s = 0.f;
#pragma unroll
         for (int m = -2; m <= 1; m++) {
            const float d3 = d[m + 5] - 3.f * d[m + 4] + 3.f * d[m + 3] - d[m + 2];
            s += kS6[m + 2] * (e[ax][m + 3] + e[ax][m + 2]) * d3;
         }
         acc += w[ax] * s;
      }
      const long long x = c * b.npts + p;
      float t, err, oh, ol;
      two_sum(a.out[x], birho * acc, t, err);
      fast_two_sum(t, err + a.out[x + lo], oh, ol);
      a.out[x] = oh;
      a.out[x + lo] = ol;
   }
}

__global__ void rho_jac_f32_kernel(long long n, const double* __restrict__ rho,
                                   const double* __restrict__ jac, float* __restrict__ e)
{
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x)
      e[q] = (float)(rho[q] * jac[q]);
}

}  // namespace

int launch_addsgd6c(const Box& b, double* up, const double* u, const double* um, const double* rho,
                    const double* dcx, const double* dcy, const double* strx, const double* stry,
                    const double* jac, const double* cox, const double* coy, double beta,
                    cudaStream_t s)
{
   if (beta == 0) return kOk;
   const int ni = b.ie - b.ib - 5, nj = b.je - b.jb - 5, nk = b.ke - b.kb - 5;
   if (ni < 1 || nj < 1 || nk < 1) return kOk;
   const dim3 blk(32, 8), g(blocks_for(ni, 32), blocks_for(nj, 8), nk);
   addsgd6c_kernel<<<g, blk, 0, s>>>(b, up, u, um, rho, dcx, dcy, strx, stry, jac, cox, coy, beta);
   return launch_status();
}

int launch_addsgd6_df(int naxes, const Box& b, float* out, const float* u, const float* um,
                      const float* e, const float* const dc[3], const float* const st[3],
                      const float* const co[3], double beta, cudaStream_t s, int adj)
{
   if (beta == 0) return kOk;
   if (naxes != 2 && naxes != 3) return kBadArgument;
   if (adj && naxes != 3) return kBadArgument;
   const int cut = adj ? 3 : 5;
   const int ni = b.ie - b.ib - cut, nj = b.je - b.jb - cut, nk = b.ke - b.kb - cut;
   if (ni < 1 || nj < 1 || nk < 1) return kOk;
   Sg6DF a;
   a.b = b;
   a.out = out;
   a.u = u;
   a.um = um;
   a.e = e;
   for (int q = 0; q < 3; q++) {
      a.dc[q] = dc[q];
      a.st[q] = st[q];
      a.co[q] = co[q];
   }
   a.naxes = naxes;
   a.beta = (float)beta;
   a.adj = adj;
   const dim3 blk(32, 8), g(blocks_for(ni, 32), blocks_for(nj, 8), nk);
   addsgd6_df_kernel<<<g, blk, 0, s>>>(a);
   return launch_status();
}

int launch_addsgd6_adj(const Box& b, double* up, const double* u, const double* um, const double* rho,
                       const double* const dc[3], const double* const st[3], const double* const co[3],
                       double beta, cudaStream_t s)
{
   if (beta == 0) return kOk;
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3, nk = b.ke - b.kb - 3;
   if (ni < 1 || nj < 1 || nk < 1) return kOk;
   Sg6Prof f;
   for (int q = 0; q < 3; q++) {
      f.dc[q] = dc[q];
      f.st[q] = st[q];
      f.co[q] = co[q];
   }
   const dim3 blk(32, 8), g(blocks_for(ni, 32), blocks_for(nj, 8), nk);
   addsgd6_adj_kernel<<<g, blk, 0, s>>>(b, up, u, um, rho, f, beta);
   return launch_status();
}

int launch_rho_jac_f32(long long n, const double* rho, const double* jac, float* e, cudaStream_t s)
{
   const long long g = (n + 255) / 256;
   rho_jac_f32_kernel<<<(int)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16), 256, 0, s>>>(n, rho, jac, e);
   return launch_status();
}

}  // namespace sw4g
