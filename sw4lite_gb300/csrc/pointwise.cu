// Pointwise time-level updates and supergrid damping, sm_103a.
//
//   predictor   up = 2u - um + dt^2/rho (lu + f)        src/ew-cfromfort.C:70-114
//   corrector   up += dt^4/(12 rho) (lu + f)            src/ew-cfromfort.C:40-67
//   dpdm        u2 = (up - 2u + um)/dt^2                 src/ew-cfromfort.C:116-142
//   addsgd4/6   4th/6th-order supergrid damping on up   src/ew-cfromfort.C:748-1158
//
// The pointwise kernels cover every array point, ghosts included, as the
// reference does; they are HBM-streaming kernels (grid-stride, coalesced).
#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

__global__ void pred_kernel(Box b, double* __restrict__ up, const double* __restrict__ u,
                            const double* __restrict__ um, const double* __restrict__ lu,
                            const double* __restrict__ fo, const double* __restrict__ rho,
                            double dt2)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const double c0 = dt2 / rho[p];
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = c * b.cs + b.ps * p;
         up[q] = 2 * u[q] - um[q] + c0 * (lu[q] + fo[q]);
      }
   }
}

__global__ void corr_kernel(Box b, double* __restrict__ up, const double* __restrict__ lu,
                            const double* __restrict__ fo, const double* __restrict__ rho,
                            double dt4i12)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const double c0 = dt4i12 / rho[p];
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = c * b.cs + b.ps * p;
         up[q] += c0 * (lu[q] + fo[q]);
      }
   }
}

__global__ void dpdm_kernel(long long n, const double* __restrict__ up,
                            const double* __restrict__ u, const double* __restrict__ um,
                            double* __restrict__ u2, double dt2i)
{
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x)
      u2[q] = dt2i * (up[q] - 2 * u[q] + um[q]);
}

struct SgArgs {
   Box b;
   double* __restrict__ up;
   const double* __restrict__ u;
   const double* __restrict__ um;
   const double* __restrict__ rho;
   const double* __restrict__ dc[3];
   const double* __restrict__ st[3];
   const double* __restrict__ co[3];
   double beta;
};

__device__ __forceinline__ int axis_off(const Box& b, int ax, int i, int j, int k)
{
   return ax == 0 ? i - b.ib : ax == 1 ? j - b.jb : k - b.kb;
}

// up -= beta/rho sum_axes str*co*co * D+D-( rho*dc * D+D-(u-um) )
__global__ void __launch_bounds__(256) addsgd4_kernel(SgArgs a)
{
   const Box& b = a.b;
   const int i = b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = b.kb + 2 + blockIdx.z;
   if (i > b.ie - 2 || j > b.je - 2) return;
   const double birho = a.beta / a.rho[pidx(b, i, j, k)];
   double w[3];
   w[0] = a.st[0][i - b.ib] * a.co[1][j - b.jb] * a.co[2][k - b.kb];
   w[1] = a.st[1][j - b.jb] * a.co[0][i - b.ib] * a.co[2][k - b.kb];
   w[2] = a.st[2][k - b.kb] * a.co[0][i - b.ib] * a.co[1][j - b.jb];
   double e[3][3];
   for (int ax = 0; ax < 3; ax++)
      for (int m = -1; m <= 1; m++) {
         const int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m, kk = k + (ax == 2) * m;
         e[ax][m + 1] = a.rho[pidx(b, ii, jj, kk)] * a.dc[ax][axis_off(b, ax, ii, jj, kk)];
      }
   for (int c = 0; c < 3; c++) {
      double tot = 0;
      for (int ax = 0; ax < 3; ax++) {
         double d[5];
         for (int m = -2; m <= 2; m++) {
            const long long q = cidx(b, c, i + (ax == 0) * m, j + (ax == 1) * m, k + (ax == 2) * m);
            d[m + 2] = a.u[q] - a.um[q];
         }
         const double s = e[ax][2] * (d[4] - 2 * d[3] + d[2]) - 2 * e[ax][1] * (d[3] - 2 * d[2] + d[1]) +
                          e[ax][0] * (d[2] - 2 * d[1] + d[0]);
         tot += w[ax] * s;
      }
      a.up[cidx(b, c, i, j, k)] -= birho * tot;
   }
}

// up += beta/(2 rho) sum_axes str*co*co * (6th-order damping), src/ew-cfromfort.C:1059-1158
__global__ void __launch_bounds__(256) addsgd6_kernel(SgArgs a)
{
   const Box& b = a.b;
   const int i = b.ib + 3 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + 3 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = b.kb + 3 + blockIdx.z;
   if (i > b.ie - 3 || j > b.je - 3) return;
   const double birho = 0.5 * a.beta / a.rho[pidx(b, i, j, k)];
   double w[3];
   w[0] = a.st[0][i - b.ib] * a.co[1][j - b.jb] * a.co[2][k - b.kb];
   w[1] = a.st[1][j - b.jb] * a.co[0][i - b.ib] * a.co[2][k - b.kb];
   w[2] = a.st[2][k - b.kb] * a.co[0][i - b.ib] * a.co[1][j - b.jb];
   double e[3][5];
   for (int ax = 0; ax < 3; ax++)
      for (int m = -2; m <= 2; m++) {
         const int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m, kk = k + (ax == 2) * m;
         e[ax][m + 2] = a.rho[pidx(b, ii, jj, kk)] * a.dc[ax][axis_off(b, ax, ii, jj, kk)];
      }
   for (int c = 0; c < 3; c++) {
      double tot = 0;
      for (int ax = 0; ax < 3; ax++) {
         double d[7];
         for (int m = -3; m <= 3; m++) {
            const long long q = cidx(b, c, i + (ax == 0) * m, j + (ax == 1) * m, k + (ax == 2) * m);
            d[m + 3] = a.u[q] - a.um[q];
         }
         // third differences at the half points -3/2 .. 3/2, weights -1, 3, -3, 1
         double s = 0;
         const double w4[4] = {-1, 3, -3, 1};
         for (int m = -2; m <= 1; m++) {
            const double d3 = d[m + 5] - 3 * d[m + 4] + 3 * d[m + 3] - d[m + 2];
            s += w4[m + 2] * (e[ax][m + 3] + e[ax][m + 2]) * d3;
         }
         tot += w[ax] * s;
      }
      a.up[cidx(b, c, i, j, k)] += birho * tot;
   }
}

// Ghost shell of a stage: every array point outside the interior box
// [ib+2,ie-2]x[jb+2,je-2]x[kb+2,ke-2] gets the stage update with Lu = F = 0, as
// the reference's pointwise predfort/corrfort do over the whole array
// (src/ew-cfromfort.C:40-114): predictor out = 2u - um, corrector out = up.
// Points are enumerated as the 4 outer k-planes, then the 4 outer j-rows of the
// inner planes, then the 4 outer i-columns of the inner rows.
// The shell point's update: corrector up, predictor 2u - um (FP64, or in double-float
// arithmetic on the FP32 pipe: TwoSum, then FastTwoSum of the error terms).
__device__ __forceinline__ void shell_update(const F64Field& out, const F64Field& u, const F64Field& um,
                                             const F64Field& up, long long x, int corrector)
{
   out.set(x, corrector ? up.get(x) : 2 * u.get(x) - um.get(x));
}

__device__ __forceinline__ void shell_update(const DFField& out, const DFField& u, const DFField& um,
                                             const DFField& up, long long x, int corrector)
{
   if (corrector) {
      out.h[x] = up.h[x];
      out.h[x + out.lo] = up.h[x + up.lo];
      return;
   }
   float s, e, oh, ol;
   two_sum(2.f * u.h[x], -um.h[x], s, e);
   fast_two_sum(s, e + (2.f * u.h[x + u.lo] - um.h[x + um.lo]), oh, ol);
   out.h[x] = oh;
   out.h[x + out.lo] = ol;
}

// The two-point shell of the array box around the centred rows: the two k-planes at
// each end (whole planes), the two j-rows at each end of the other planes, and the two
// i-points at each end of the remaining rows.  32-bit index arithmetic (the shell has
// O(N^2) points); on the i-faces four consecutive threads take the four shell points of
// one row, two adjacent pairs, so a warp's loads touch 16 sectors rather than 32.
template <class Field>
__global__ void ghost_shell_kernel(Box b, int corrector, Field out, Field u, Field um, Field up)
{
   const int ni = (int)b.ni, nj = b.je - b.jb + 1, nk = b.ke - b.kb + 1;
   const int nA = 4 * ni * nj, nB = 4 * ni * (nk - 4), nC = 4 * (nj - 4) * (nk - 4);
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nA + nB + nC; q += gridDim.x * blockDim.x) {
      int i, j, k;
      if (q < nA) {
         const int s = q / (ni * nj), r = q - s * ni * nj;
         k = s < 2 ? b.kb + s : b.ke - (3 - s);
         j = b.jb + r / ni;
         i = b.ib + r % ni;
      } else if (q < nA + nB) {
         const int r0 = q - nA;
         const int s = r0 / (ni * (nk - 4)), r = r0 - s * ni * (nk - 4);
         j = s < 2 ? b.jb + s : b.je - (3 - s);
         k = b.kb + 2 + r / ni;
         i = b.ib + r % ni;
      } else {
         const int r0 = q - nA - nB;
         const int s = r0 & 3, r = r0 >> 2;
         i = s < 2 ? b.ib + s : b.ie - (3 - s);
         k = b.kb + 2 + r / (nj - 4);
         j = b.jb + 2 + r % (nj - 4);
      }
#pragma unroll
      for (int c = 0; c < 3; c++) shell_update(out, u, um, up, cidx(b, c, i, j, k), corrector);
   }
}

int stream_grid(long long n)
{
   long long b = (n + 255) / 256;
   if (b > 152LL * 32) b = 152LL * 32;
   return (int)(b > 0 ? b : 1);
}

}  // namespace

int launch_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                    const double* u, const double* um, const double* lu, const double* fo,
                    const double* rho, double dt2, cudaStream_t s)
{
   Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   pred_kernel<<<stream_grid(b.npts), 256, 0, s>>>(b, up, u, um, lu, fo, rho, dt2);
   return launch_status();
}

int launch_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                    const double* lu, const double* fo, const double* rho, double dt4,
                    cudaStream_t s)
{
   Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   corr_kernel<<<stream_grid(b.npts), 256, 0, s>>>(b, up, lu, fo, rho, dt4 / 12);
   return launch_status();
}

int launch_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, const double* up,
                     const double* u, const double* um, double* u2, double dt2i, cudaStream_t s)
{
   const long long n = 3LL * (ie - ib + 1) * (je - jb + 1) * (ke - kb + 1);
   dpdm_kernel<<<stream_grid(n), 256, 0, s>>>(n, up, u, um, u2, dt2i);
   return launch_status();
}

int launch_ghost_shell(const Box& b, int corrector, double* out, const double* u,
                       const double* um, const double* up, cudaStream_t s)
{
   const long long ni = b.ni, nj = b.je - b.jb + 1, nk = b.ke - b.kb + 1;
   if (ni < 5 || nj < 5 || nk < 5) return kBadArgument;
   const long long n = 4 * ni * nj + 4 * ni * (nk - 4) + 4 * (nj - 4) * (nk - 4);
   if (n >= (1LL << 31)) return kNotSupported;  // the kernel indexes the shell in 32 bits
   ghost_shell_kernel<<<stream_grid(n), 256, 0, s>>>(b, corrector, F64Field{out},
                                                     F64Field{const_cast<double*>(u)},
                                                     F64Field{const_cast<double*>(um)},
                                                     F64Field{const_cast<double*>(up)});
   return launch_status();
}

int launch_ghost_shell_df(const Box& b, int corrector, float* out, const float* u, const float* um,
                          const float* up, cudaStream_t s)
{
   const long long ni = b.ni, nj = b.je - b.jb + 1, nk = b.ke - b.kb + 1;
   if (ni < 5 || nj < 5 || nk < 5) return kBadArgument;
   const long long n = 4 * ni * nj + 4 * ni * (nk - 4) + 4 * (nj - 4) * (nk - 4);
   if (n >= (1LL << 31)) return kNotSupported;  // the kernel indexes the shell in 32 bits
   const long long lo = 3 * b.npts;
   ghost_shell_kernel<<<stream_grid(n), 256, 0, s>>>(
       b, corrector, DFField{out, lo}, DFField{const_cast<float*>(u), lo},
       DFField{const_cast<float*>(um), lo}, DFField{const_cast<float*>(up), lo});
   return launch_status();
}

int launch_addsgd(int order, int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                  int klast, double* up, const double* u, const double* um, const double* rho,
                  const double* dcx, const double* dcy, const double* dcz, const double* strx,
                  const double* stry, const double* strz, const double* cox, const double* coy,
                  const double* coz, double beta, cudaStream_t s)
{
   if (beta == 0) return kOk;
   if (order != 4 && order != 6) return kBadArgument;
   SgArgs a;
   a.b = make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast);
   a.up = up;
   a.u = u;
   a.um = um;
   a.rho = rho;
   a.dc[0] = dcx; a.dc[1] = dcy; a.dc[2] = dcz;
   a.st[0] = strx; a.st[1] = stry; a.st[2] = strz;
   a.co[0] = cox; a.co[1] = coy; a.co[2] = coz;
   a.beta = beta;
   const int g = order == 4 ? 2 : 3;
   const int ni = ilast - ifirst + 1 - 2 * g, nj = jlast - jfirst + 1 - 2 * g,
             nk = klast - kfirst + 1 - 2 * g;
   if (ni <= 0 || nj <= 0 || nk <= 0) return kOk;
   const dim3 block(32, 8, 1), grid(blocks_for(ni, 32), blocks_for(nj, 8), nk);
   if (order == 4)
      addsgd4_kernel<<<grid, block, 0, s>>>(a);
   else
      addsgd6_kernel<<<grid, block, 0, s>>>(a);
   return launch_status();
}

}  // namespace sw4g
