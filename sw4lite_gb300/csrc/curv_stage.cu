// Fused stage kernels of the curvilinear grid (topography), sm_103a, FP64.
//
// The Cartesian fused design (stage_fused.cu) applied to the curvilinear operator
// of curv.cu (rhs4sgcurv, src/rhs4sgcurv_rev.C:34):
//   predictor  out = 2u - um + dt^2 K S(u)
//   corrector  out = up + dt^2/12 K S(up - 2u + um) - beta/(rho J) SG(u - um)
// with S the bracket of the operator (Lu = (sx sy / J) S) and K = sx sy / (J rho).
// Every time-invariant coefficient is computed once per run (curv_coef_kernel):
//   * the second-difference weights W1, W2 of the same-axis terms (p: two kinds,
//     q: two kinds, r: the six entries of the symmetric r-r matrix), with the
//     terms' 1/sx, 1/sy factors and the 1/6 folded in (those factors are constant
//     along the axis each weight acts on);
//   * the eight products mu m1^2, la m1^2, mu m2 m1, la m2 m1, mu m3 m1, la m3 m1,
//     mu m4 m1, la m4 m1 of the cross terms;
//   * K and 1/(rho J), rho J of the damping.
// Each cross term D_a(C D_b u) is an outer difference of per-point products
// G = C D_b u: G for the p (q) outer difference is staged in shared memory over
// the x (y) halo, G for the r outer difference rides a register queue, as in the
// Cartesian kernel.  The kernel covers the rows k = 7..nz under an SBP top; the six
// top rows and the ghost shell are done by curv_edge_kernel from the one-sided
// operator of curv.cu.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "sbp.h"
#include "stencil.cuh"

namespace sw4g {
namespace {

constexpr int TX = 32, TY = 8, HALO = 2;
constexpr int PX = TX + 2 * HALO;
constexpr int PY = TY + 2 * HALO;
constexpr int PLANE = PX * PY;
constexpr int NTHREADS = TX * TY;

// weight arrays: p-axis kinds 0 ((2mu+la) m1^2 sx), 1 (mu m1^2 sx); q-axis kinds
// 2 (mu m1^2 sy), 3 ((2mu+la) m1^2 sy); r-axis kinds 4..9 = A00, A11, A22, A01, A02, A12.
// Each kind has W1 (slot 2*kind) and W2 (slot 2*kind+1).
constexpr int kCurvKinds = 10;
// products: 0 mu m1^2, 1 la m1^2, 2 mu m2 m1, 3 la m2 m1, 4 mu m3 m1, 5 la m3 m1,
// 6 mu m4 m1, 7 la m4 m1
constexpr int kProducts = 8;

__global__ void curv_coef_kernel(Box b, const double* __restrict__ mu, const double* __restrict__ la,
                                 const double* __restrict__ rho, const double* __restrict__ met,
                                 const double* __restrict__ jac, const double* __restrict__ sx,
                                 const double* __restrict__ sy, CurvCoef c)
{
   const long long n = b.npts;
   const int nj = b.je - b.jb + 1;
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
        p += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(p % b.ni), j = b.jb + (int)((p / b.ni) % nj), k = b.kb + (int)(p / b.nij);
      const double m = mu[p], l = la[p], m1 = met[p], m2 = met[n + p], m3 = met[2 * n + p],
                   m4 = met[3 * n + p];
      c.prod[0][p] = m * m1 * m1;
      c.prod[1][p] = l * m1 * m1;
      c.prod[2][p] = m * m2 * m1;
      c.prod[3][p] = l * m2 * m1;
      c.prod[4][p] = m * m3 * m1;
      c.prod[5][p] = l * m3 * m1;
      c.prod[6][p] = m * m4 * m1;
      c.prod[7][p] = l * m4 * m1;
      const double sxi = sx[i - b.ib], syj = sy[j - b.jb];
      c.K[p] = sxi * syj / (jac[p] * rho[p]);
      c.rj[p] = rho[p] * jac[p];
      c.irj[p] = 1.0 / (rho[p] * jac[p]);
      const double istrx = 1 / sxi, istry = 1 / syj;
      // coefficient of kind t at offset q (points along the kind's axis)
      auto coefat = [&](int t, int q) -> double {
         long long pp;
         int ii = i, jj = j, kk = k;
         if (t < 2) ii = q;
         else if (t < 4) jj = q;
         else kk = q;
         pp = (long long)(ii - b.ib) + b.ni * (jj - b.jb) + b.nij * (long long)(kk - b.kb);
         const double mm = mu[pp], ll = la[pp], a1 = met[pp], a2 = met[n + pp] * sxi,
                      a3 = met[2 * n + pp] * syj, a4 = met[3 * n + pp];
         switch (t) {
            case 0: return (2 * mm + ll) * a1 * a1 * sx[ii - b.ib];
            case 1: return mm * a1 * a1 * sx[ii - b.ib];
            case 2: return mm * a1 * a1 * sy[jj - b.jb];
            case 3: return (2 * mm + ll) * a1 * a1 * sy[jj - b.jb];
            case 4: return (2 * mm + ll) * a2 * a2 + mm * (a3 * a3 + a4 * a4);
            case 5: return (2 * mm + ll) * a3 * a3 + mm * (a2 * a2 + a4 * a4);
            case 6: return (2 * mm + ll) * a4 * a4 + mm * (a2 * a2 + a3 * a3);
            case 7: return (mm + ll) * met[n + pp] * met[2 * n + pp];
            case 8: return (mm + ll) * met[n + pp] * met[3 * n + pp];
            default: return (mm + ll) * met[2 * n + pp] * met[3 * n + pp];
         }
      };
      const double scale[kCurvKinds] = {istry, istry, istrx, istrx, istrx * istry, istrx * istry,
                                        istrx * istry, 1.0, istry, istrx};
      for (int t = 0; t < kCurvKinds; t++) {
         const int q = t < 2 ? i : t < 4 ? j : k;
         const int lo = t < 2 ? b.ib : t < 4 ? b.jb : b.kb, hi = t < 2 ? b.ie : t < 4 ? b.je : b.ke;
         double w1 = 0, w2 = 0;
         if (q - 2 >= lo) {
            const double am2 = coefat(t, q - 2), am1 = coefat(t, q - 1), a0 = coefat(t, q);
            const double ap1 = q + 1 <= hi ? coefat(t, q + 1) : 0.0;
            w1 = am1 - 0.75 * (a0 + am2);
            if (q + 1 <= hi) w2 = am2 + ap1 + 3 * (a0 + am1);
         }
         c.w[2 * t][p] = w1 * scale[t] / 6;
         c.w[2 * t + 1][p] = w2 * scale[t] / 6;
      }
   }
}

struct StageArgs {
   Box b;
   int k1, k2, kchunk;
   const double* __restrict__ u;
   const double* __restrict__ um;
   const double* __restrict__ up;
   double* __restrict__ out;
   CurvCoef cc;
   const double* __restrict__ sx;
   const double* __restrict__ sy;
   const double* __restrict__ dcx;
   const double* __restrict__ dcy;
   const double* __restrict__ cox;
   const double* __restrict__ coy;
   double coef, beta;
};

__host__ __device__ constexpr int stage_smem(int corr)
{
   // V ring (5 x 3 planes) + [D plane (3) + RJ plane] + GX + GY
   return 15 * PLANE + (corr ? 4 * PLANE : 0) + 3 * TY * PX + 3 * PY * TX;
}

__device__ __forceinline__ int m5(int k) { return ((k % 5) + 5) % 5; }

template <int CORR>
__global__ void __launch_bounds__(NTHREADS, 2) curv_stage_kernel(StageArgs a)
{
   extern __shared__ double sm[];
   double* V = sm;                              // [5][3][PLANE]
   double* DP = V + 15 * PLANE;                 // [3][PLANE] (corrector, plane k)
   double* RJ = DP + (CORR ? 3 * PLANE : 0);    // [PLANE]    (corrector, plane k)
   double* GX = RJ + (CORR ? PLANE : 0);        // [3][TY][PX]
   double* GY = GX + 3 * TY * PX;               // [3][PY][TX]
   const Box& b = a.b;
   const long long n = b.npts;
   const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
   const int i0 = b.ib + 2 + blockIdx.x * TX, j0 = b.jb + 2 + blockIdx.y * TY;
   const int kbeg = a.k1 + blockIdx.z * a.kchunk;
   if (kbeg > a.k2) return;
   const int kend = min(kbeg + a.kchunk - 1, a.k2);
   const int i = i0 + tx, j = j0 + ty;
   const bool active = (i <= b.ie - 2) && (j <= b.je - 2);
   const int own = (ty + HALO) * PX + (tx + HALO);
   auto gidx = [&](int gi, int gj, int gk) -> long long {
      return (long long)(gi - b.ib) + b.ni * (gj - b.jb) + b.nij * (long long)(gk - b.kb);
   };
   auto load_plane = [&](int kk) {
      double* vs = V + m5(kk) * 3 * PLANE;
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int gi = i0 - HALO + idx % PX, gj = j0 - HALO + idx / PX;
         double v[3] = {0, 0, 0};
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, kk);
#pragma unroll
            for (int c = 0; c < 3; c++) {
               if (!CORR) v[c] = __ldg(a.u + p + c * n);
               else v[c] = (__ldg(a.up + p + c * n) - 2 * __ldg(a.u + p + c * n)) + __ldg(a.um + p + c * n);
            }
         }
#pragma unroll
         for (int c = 0; c < 3; c++) vs[c * PLANE + idx] = v[c];
      }
   };
   auto load_damping = [&](int kk) {
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int gi = i0 - HALO + idx % PX, gj = j0 - HALO + idx / PX;
         double d[3] = {0, 0, 0}, r = 0;
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, kk);
#pragma unroll
            for (int c = 0; c < 3; c++) d[c] = __ldg(a.u + p + c * n) - __ldg(a.um + p + c * n);
            r = __ldg(a.cc.rj + p);
         }
#pragma unroll
         for (int c = 0; c < 3; c++) DP[c * PLANE + idx] = d[c];
         RJ[idx] = r;
      }
   };
   const double sxi = active ? __ldg(a.sx + (i - b.ib)) : 1.0;
   const double syj = active ? __ldg(a.sy + (j - b.jb)) : 1.0;
   const double isxi = 1 / sxi, isyj = 1 / syj;
   auto P = [&](int t, long long p) { return __ldg(a.cc.prod[t] + p); };

   // r-outer products of the own column at plane kk (inner p and q differences)
   auto compute_gr = [&](int kk, double g[3]) {
      const double* vs = V + m5(kk) * 3 * PLANE;
      double dp[3], dq[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const double* f = vs + c * PLANE + own;
         dp[c] = d1c(f[-2], f[-1], f[1], f[2]);
         dq[c] = d1c(f[-2 * PX], f[-PX], f[PX], f[2 * PX]);
      }
      const long long p = gidx(i, j, kk);
      const double p21m = P(2, p), p21l = P(3, p), p31m = P(4, p), p31l = P(5, p), p41m = P(6, p),
                   p41l = P(7, p);
      g[0] = (2 * p21m + p21l) * sxi * isyj * dp[0] + p31m * dp[1] + p41m * isyj * dp[2] +
             p31m * syj * isxi * dq[0] + p21l * dq[1];
      g[1] = p31l * dp[0] + p21m * sxi * isyj * dp[1] + p21m * dq[0] +
             (2 * p31m + p31l) * syj * isxi * dq[1] + p41m * isxi * dq[2];
      g[2] = isyj * (p41l * dp[0] + p21m * sxi * dp[2]) + isxi * (p31m * syj * dq[2] + p41l * dq[1]);
   };

   double gz[5][3];
   for (int kk = kbeg - 2; kk <= kbeg + 1; kk++) load_plane(kk);
   __syncthreads();
   for (int kk = kbeg - 2; kk <= kbeg + 1; kk++)
      if (active) compute_gr(kk, gz[kk - kbeg + 3]);
   __syncthreads();

   for (int k = kbeg; k <= kend; k++) {
      load_plane(k + 2);
      if (CORR) load_damping(k);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
         for (int c = 0; c < 3; c++) gz[q][c] = gz[q + 1][c];
      if (active) compute_gr(k + 2, gz[4]);

      const double* vm2 = V + m5(k - 2) * 3 * PLANE;
      const double* vm1 = V + m5(k - 1) * 3 * PLANE;
      const double* v0 = V + m5(k) * 3 * PLANE;
      const double* vp1 = V + m5(k + 1) * 3 * PLANE;
      const double* vp2 = V + m5(k + 2) * 3 * PLANE;
      auto dr = [&](int c, int s) {
         return d1c(vm2[c * PLANE + s], vm1[c * PLANE + s], vp1[c * PLANE + s], vp2[c * PLANE + s]);
      };
      // p-outer products over the x-extended rows
      for (int idx = tid; idx < TY * PX; idx += NTHREADS) {
         const int li = idx % PX, ljr = idx / PX;
         const int s = (ljr + HALO) * PX + li;
         const int gi = i0 - HALO + li, gj = j0 + ljr;
         double g0 = 0, g1 = 0, g2 = 0;
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, k);
            const double sxx = __ldg(a.sx + (gi - b.ib)), syy = __ldg(a.sy + (gj - b.jb));
            const double isy = 1 / syy;
            double dq[3], drr[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const double* f = v0 + c * PLANE + s;
               dq[c] = d1c(f[-2 * PX], f[-PX], f[PX], f[2 * PX]);
               drr[c] = dr(c, s);
            }
            const double p11m = P(0, p), p11l = P(1, p), p21m = P(2, p), p21l = P(3, p),
                         p31m = P(4, p), p31l = P(5, p), p41m = P(6, p), p41l = P(7, p);
            g0 = p11l * dq[1] + isy * ((2 * p21m + p21l) * sxx * drr[0] + p31l * syy * drr[1] + p41l * drr[2]);
            g1 = p11m * dq[0] + p31m * drr[0] + p21m * sxx * isy * drr[1];
            g2 = isy * (p41m * drr[0] + p21m * sxx * drr[2]);
         }
         GX[idx] = g0;
         GX[TY * PX + idx] = g1;
         GX[2 * TY * PX + idx] = g2;
      }
      // q-outer products over the y-extended columns
      for (int idx = tid; idx < PY * TX; idx += NTHREADS) {
         const int lic = idx % TX, lj = idx / TX;
         const int s = lj * PX + lic + HALO;
         const int gi = i0 + lic, gj = j0 - HALO + lj;
         double g0 = 0, g1 = 0, g2 = 0;
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, k);
            const double sxx = __ldg(a.sx + (gi - b.ib)), syy = __ldg(a.sy + (gj - b.jb));
            const double isx = 1 / sxx;
            double dpp[3], drr[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const double* f = v0 + c * PLANE + s;
               dpp[c] = d1c(f[-2], f[-1], f[1], f[2]);
               drr[c] = dr(c, s);
            }
            const double p11m = P(0, p), p11l = P(1, p), p21m = P(2, p), p21l = P(3, p),
                         p31m = P(4, p), p31l = P(5, p), p41m = P(6, p), p41l = P(7, p);
            g0 = p11m * dpp[1] + p31m * syy * isx * drr[0] + p21m * drr[1];
            g1 = p11l * dpp[0] + p21l * drr[0] + (2 * p31m + p31l) * syy * isx * drr[1] + p41l * isx * drr[2];
            g2 = isx * (p31m * syy * drr[2] + p41m * drr[1]);
         }
         GY[idx] = g0;
         GY[PY * TX + idx] = g1;
         GY[2 * PY * TX + idx] = g2;
      }
      __syncthreads();

      if (active) {
         const long long p = gidx(i, j, k);
         const long long off[3] = {1, b.ni, b.nij};
         double s3[3] = {0, 0, 0};
         // same-axis p and q
#pragma unroll
         for (int ax = 0; ax < 2; ax++) {
            const long long o = off[ax];
#pragma unroll
            for (int t2 = 0; t2 < 2; t2++) {
               const int t = 2 * ax + t2;
               const double w0 = __ldg(a.cc.w[2 * t] + p), w1 = __ldg(a.cc.w[2 * t + 1] + p),
                            w2 = __ldg(a.cc.w[2 * t + 1] + p + o), w3 = __ldg(a.cc.w[2 * t] + p + 2 * o);
#pragma unroll
               for (int c = 0; c < 3; c++) {
                  // p-axis: kind 0 for c = 0, kind 1 for c = 1, 2; q-axis: kind 3 for c = 1
                  const bool use = ax == 0 ? ((c == 0) == (t2 == 0)) : ((c == 1) == (t2 == 1));
                  if (!use) continue;
                  const double* f = v0 + c * PLANE + own;
                  const int st = ax == 0 ? 1 : PX;
                  s3[c] += w0 * (f[-2 * st] - f[0]) + w1 * (f[-st] - f[0]) + w2 * (f[st] - f[0]) +
                           w3 * (f[2 * st] - f[0]);
               }
            }
         }
         // same-axis r: symmetric matrix A_cd
         const long long o = b.nij;
#pragma unroll
         for (int t = 4; t < 10; t++) {
            const int cc = t < 7 ? t - 4 : (t == 7 ? 0 : (t == 8 ? 0 : 1));
            const int dd = t < 7 ? t - 4 : (t == 7 ? 1 : 2);
            const double w0 = __ldg(a.cc.w[2 * t] + p), w1 = __ldg(a.cc.w[2 * t + 1] + p),
                         w2 = __ldg(a.cc.w[2 * t + 1] + p + o), w3 = __ldg(a.cc.w[2 * t] + p + 2 * o);
            auto rr = [&](int comp) {
               const int s = comp * PLANE + own;
               const double f0 = v0[s];
               return w0 * (vm2[s] - f0) + w1 * (vm1[s] - f0) + w2 * (vp1[s] - f0) + w3 * (vp2[s] - f0);
            };
            s3[cc] += rr(dd);
            if (cc != dd) s3[dd] += rr(cc);
         }
         // cross terms: outer differences of the staged products
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const double* gx = GX + c * TY * PX + ty * PX + tx;
            const double* gy = GY + c * PY * TX + ty * TX + tx;
            const double cx = d1c(gx[0], gx[1], gx[3], gx[4]);
            const double cy = d1c(gy[0], gy[TX], gy[3 * TX], gy[4 * TX]);
            const double cz = d1c(gz[0][c], gz[1][c], gz[3][c], gz[4][c]);
            s3[c] += (cx + cy + cz) * (1.0 / 144);
         }
         const double kk = a.coef * __ldg(a.cc.K + p);
         if (!CORR) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * n;
               a.out[q] = 2 * v0[c * PLANE + own] - __ldg(a.um + q) + kk * s3[c];
            }
         } else {
            double sg[3] = {0, 0, 0};
            if (a.beta != 0) {
               const double cxi = __ldg(a.cox + (i - b.ib)), cyj = __ldg(a.coy + (j - b.jb));
               const double dx0 = __ldg(a.dcx + (i - 1 - b.ib)), dx1 = __ldg(a.dcx + (i - b.ib)),
                            dx2 = __ldg(a.dcx + (i + 1 - b.ib));
               if (nonzero_bits(dx0) || nonzero_bits(dx1) || nonzero_bits(dx2)) {  // integer pipe
                  const double e0 = RJ[own - 1] * dx0, e1 = RJ[own] * dx1, e2 = RJ[own + 1] * dx2;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const double* d = DP + c * PLANE + own;
                     sg[c] += sxi * cyj * (e2 * (d[2] - 2 * d[1] + d[0]) - 2 * e1 * (d[1] - 2 * d[0] + d[-1]) +
                                           e0 * (d[0] - 2 * d[-1] + d[-2]));
                  }
               }
               const double dy0 = __ldg(a.dcy + (j - 1 - b.jb)), dy1 = __ldg(a.dcy + (j - b.jb)),
                            dy2 = __ldg(a.dcy + (j + 1 - b.jb));
               if (nonzero_bits(dy0) || nonzero_bits(dy1) || nonzero_bits(dy2)) {
                  const double e0 = RJ[own - PX] * dy0, e1 = RJ[own] * dy1, e2 = RJ[own + PX] * dy2;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const double* d = DP + c * PLANE + own;
                     sg[c] += syj * cxi * (e2 * (d[2 * PX] - 2 * d[PX] + d[0]) -
                                           2 * e1 * (d[PX] - 2 * d[0] + d[-PX]) +
                                           e0 * (d[0] - 2 * d[-PX] + d[-2 * PX]));
                  }
               }
            }
            const double birj = a.beta * __ldg(a.cc.irj + p);
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * n;
               a.out[q] = (__ldg(a.up + q) + kk * s3[c]) - birj * sg[c];
            }
         }
      }
      __syncthreads();
   }
}

// The ghost shell, where the reference's pointwise updates run with Lu = F = 0:
// predictor out = 2u - um, corrector out = up.
template <int CORR>
__global__ void curv_shell_kernel(Box b, int nz, const double* __restrict__ u,
                                  const double* __restrict__ um, const double* __restrict__ up,
                                  double* __restrict__ out)
{
   const long long n = b.npts;
   const int nj = b.je - b.jb + 1;
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
        p += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(p % b.ni), j = b.jb + (int)((p / b.ni) % nj), k = b.kb + (int)(p / b.nij);
      const bool col = i >= b.ib + 2 && i <= b.ie - 2 && j >= b.jb + 2 && j <= b.je - 2;
      if (col && k >= 1 && k <= nz) continue;
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = p + c * n;
         out[q] = CORR ? up[q] : 2 * u[q] - um[q];
      }
   }
}

__constant__ double t_acof[384];
__constant__ double t_bope[48];
__constant__ double t_ghcof[6];
bool g_top_tables[64] = {};

int upload_top_tables()
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kCudaError;
   if (g_top_tables[dev]) return kOk;
   double acof[384], ghcof[6], bope[48], sbop[5];
   sbp_coefficients(acof, ghcof, bope, sbop);
   if (cudaMemcpyToSymbol(t_acof, acof, sizeof(acof)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(t_bope, bope, sizeof(bope)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(t_ghcof, ghcof, sizeof(ghcof)) != cudaSuccess) return kCudaError;
   g_top_tables[dev] = true;
   return kOk;
}

// Per column, the r-r coefficients of the SBP top rows contracted with acof
// (src/rhs4sgcurv_rev.C:224-275): for kind t (A00, A11, A22, A01, A02, A12), row
// r = k-1 and plane q = 1..8, W = rs_t sum_m acof(k,q,m) A_t(m); q = 0 holds the
// ghost-point weight rs_t ghcof(k) A_t(1).  Slot (t*6 + r)*9 + q of `topw`.
constexpr int kTopSlots = 6 * 6 * 9;

__global__ void curv_topw_kernel(Box b, const double* __restrict__ mu, const double* __restrict__ la,
                                 const double* __restrict__ met, const double* __restrict__ sx,
                                 const double* __restrict__ sy, double* __restrict__ topw)
{
   const long long ncol = b.nij, n = b.npts;
   for (long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x; col < ncol;
        col += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(col % b.ni), j = b.jb + (int)(col / b.ni);
      const double sxc = sx[i - b.ib], syc = sy[j - b.jb];
      const double istrx = 1 / sxc, istry = 1 / syc;
      const double rs[6] = {istrx * istry, istrx * istry, istrx * istry, 1.0, istry, istrx};
      double A[6][8];
      for (int m = 1; m <= 8; m++) {
         const long long p = col + b.nij * (long long)(m - b.kb);
         const double mm = mu[p], ll = la[p], g2 = met[n + p], g3 = met[2 * n + p], g4 = met[3 * n + p];
         const double s2 = g2 * sxc, s3 = g3 * syc;
         A[0][m - 1] = (2 * mm + ll) * s2 * s2 + mm * (s3 * s3 + g4 * g4);
         A[1][m - 1] = (2 * mm + ll) * s3 * s3 + mm * (s2 * s2 + g4 * g4);
         A[2][m - 1] = (2 * mm + ll) * g4 * g4 + mm * (s2 * s2 + s3 * s3);
         A[3][m - 1] = (mm + ll) * g2 * g3;
         A[4][m - 1] = (mm + ll) * g2 * g4;
         A[5][m - 1] = (mm + ll) * g3 * g4;
      }
      for (int t = 0; t < 6; t++)
         for (int r = 0; r < 6; r++) {
            double* w = topw + ((long long)(t * 6 + r) * 9) * ncol + col;
            w[0] = rs[t] * t_ghcof[r] * A[t][0];
            for (int q = 1; q <= 8; q++) {
               double s = 0;
               for (int m = 1; m <= 8; m++) s += t_acof[r + 6 * (q - 1) + 48 * (m - 1)] * A[t][m - 1];
               w[(long long)q * ncol] = rs[t] * s;
            }
         }
   }
}

// Read-only views of a 3-component field: FP64, or a double-float level (hi at
// q, lo at q + lo) read as hi + lo in FP64.
struct RdF64 {
   const double* __restrict__ p;
   __device__ __forceinline__ double get(long long q) const { return __ldg(p + q); }
};
struct RdDF {
   const float* __restrict__ h;
   long long lo;
   __device__ __forceinline__ double get(long long q) const
   {
      return (double)__ldg(h + q) + (double)__ldg(h + q + lo);
   }
};

template <class RD, class WR, class SF>
struct TopArgs {
   Box b;   // the grid
   Box fb;  // the stage field's array (the grid, or a slab of planes kb..8)
   SF f;
   RD u, um, up;
   WR out;
   CurvCoef cc;
   const double* __restrict__ topw;
   // per column: one-sided r derivatives DR[(k-1)*3 + c] and r-outer sums
   // RO[(k-1)*3 + c] of rows k = 1..6 (curv_top_pre_kernel), 18 x ncol each
   const double* __restrict__ dr;
   const double* __restrict__ ro;
   // corrector, optional: u - um in FP64 over the stage field's planes (box fb)
   const double* __restrict__ dd;
   const double *sx, *sy, *dcx, *dcy, *cox, *coy;
   double coef, beta;
};

// Per column, the parts of the top rows that do not depend on the row's own
// position: the one-sided r derivatives sum_q bope(k,q) f(q) of the stage field
// (all columns; the p- and q-outer cross terms read them at the four neighbouring
// columns) and the r-outer cross terms sum_q bope(k,q) G(q) with G the PR + QR
// products at planes q = 1..8 (interior columns), for k = 1..6
// (src/rhs4sgcurv_rev.C:224-275).
template <class SF>
__global__ void __launch_bounds__(128) curv_top_pre_kernel(Box b, Box fb, SF f, CurvCoef cc,
                                                           const double* __restrict__ sx,
                                                           const double* __restrict__ sy,
                                                           double* __restrict__ dr,
                                                           double* __restrict__ ro)
{
   const long long ncol = b.nij;
   auto F = [&](int c, int ii, int jj, int kk) { return f.get(c * fb.npts + pidx(fb, ii, jj, kk)); };
   auto Pr = [&](int t, long long q) { return __ldg(cc.prod[t] + q); };
   const double i12 = 1.0 / 12;
   auto cd = [&](double fm2, double fm1, double fp1, double fp2) { return i12 * d1c(fm2, fm1, fp1, fp2); };
   for (long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x; col < ncol;
        col += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(col % b.ni), j = b.jb + (int)(col / b.ni);
#pragma unroll
      for (int c = 0; c < 3; c++) {
         double fq[8];
#pragma unroll
         for (int q = 1; q <= 8; q++) fq[q - 1] = F(c, i, j, q);
#pragma unroll
         for (int k = 1; k <= 6; k++) {
            double s = 0;
#pragma unroll
            for (int q = 1; q <= 8; q++) s += t_bope[(k - 1) + 6 * (q - 1)] * fq[q - 1];
            dr[((k - 1) * 3 + c) * ncol + col] = s;
         }
      }
      if (i < b.ib + 2 || i > b.ie - 2 || j < b.jb + 2 || j > b.je - 2) continue;
      const double sxc = __ldg(sx + (i - b.ib)), syc = __ldg(sy + (j - b.jb));
      const double istrx = 1 / sxc, istry = 1 / syc;
      double acc[6][3];
#pragma unroll
      for (int k = 0; k < 6; k++) acc[k][0] = acc[k][1] = acc[k][2] = 0;
#pragma unroll 1
      for (int qq = 1; qq <= 8; qq++) {
         const long long q = pidx(b, i, j, qq);
         double dp[3], dq[3];
#pragma unroll
         for (int c = 0; c < 3; c++) {
            dp[c] = cd(F(c, i - 2, j, qq), F(c, i - 1, j, qq), F(c, i + 1, j, qq), F(c, i + 2, j, qq));
            dq[c] = cd(F(c, i, j - 2, qq), F(c, i, j - 1, qq), F(c, i, j + 1, qq), F(c, i, j + 2, qq));
         }
         const double p21m = Pr(2, q), p21l = Pr(3, q), p31m = Pr(4, q), p31l = Pr(5, q),
                      p41m = Pr(6, q), p41l = Pr(7, q);
         const double g0 = (2 * p21m + p21l) * sxc * istry * dp[0] + p31m * dp[1] + p41m * istry * dp[2] +
                           p31m * syc * istrx * dq[0] + p21l * dq[1];
         const double g1 = p31l * dp[0] + p21m * sxc * istry * dp[1] + p21m * dq[0] +
                           (2 * p31m + p31l) * syc * istrx * dq[1] + p41m * istrx * dq[2];
         const double g2 = istry * (p41l * dp[0] + p21m * sxc * dp[2]) + istrx * (p31m * syc * dq[2] + p41l * dq[1]);
#pragma unroll
         for (int k = 0; k < 6; k++) {
            const double bw = t_bope[k + 6 * (qq - 1)];
            acc[k][0] += bw * g0;
            acc[k][1] += bw * g1;
            acc[k][2] += bw * g2;
         }
      }
#pragma unroll
      for (int k = 0; k < 6; k++)
#pragma unroll
         for (int c = 0; c < 3; c++) ro[(k * 3 + c) * ncol + col] = acc[k][c];
   }
}

// Rows k = 1..6 under the SBP top: the one-sided operator from precomputed
// coefficients, with the stage update (and the corrector's x/y damping) fused.
// FP64 throughout; the levels are FP64 or double-float (RD, WR).
template <int CORR, class RD, class WR, class SF>
__device__ __forceinline__ void curv_top_point(const TopArgs<RD, WR, SF>& a, int i, int j, int k)
{
   const Box& b = a.b;
   const Box& fb = a.fb;
   const long long n = b.npts, ncol = b.nij;
   const long long p = pidx(b, i, j, k), col = pidx(b, i, j, b.kb);
   auto F = [&](int c, int ii, int jj, int kk) { return a.f.get(c * fb.npts + pidx(fb, ii, jj, kk)); };
   auto Pr = [&](int t, long long q) { return __ldg(a.cc.prod[t] + q); };
   const double sxc = __ldg(a.sx + (i - b.ib)), syc = __ldg(a.sy + (j - b.jb));
   const double istrx = 1 / sxc, istry = 1 / syc;
   const double i12 = 1.0 / 12;
   auto cd = [&](double fm2, double fm1, double fp1, double fp2) { return i12 * d1c(fm2, fm1, fp1, fp2); };
   double s3[3] = {0, 0, 0};
   // same-axis p and q (precomputed weights, as the interior)
   {
      const long long off[2] = {1, b.ni};
#pragma unroll
      for (int ax = 0; ax < 2; ax++)
#pragma unroll
         for (int t2 = 0; t2 < 2; t2++) {
            const int t = 2 * ax + t2;
            const long long o = off[ax];
            const double w0 = __ldg(a.cc.w[2 * t] + p), w1 = __ldg(a.cc.w[2 * t + 1] + p),
                         w2 = __ldg(a.cc.w[2 * t + 1] + p + o), w3 = __ldg(a.cc.w[2 * t] + p + 2 * o);
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const bool use = ax == 0 ? ((c == 0) == (t2 == 0)) : ((c == 1) == (t2 == 1));
               if (!use) continue;
               const int di = ax == 0, dj = ax == 1;
               const double f0 = F(c, i, j, k);
               s3[c] += w0 * (F(c, i - 2 * di, j - 2 * dj, k) - f0) + w1 * (F(c, i - di, j - dj, k) - f0) +
                        w2 * (F(c, i + di, j + dj, k) - f0) + w3 * (F(c, i + 2 * di, j + 2 * dj, k) - f0);
            }
         }
   }
   // r-r: acof-contracted coefficients of this column
   {
      double fc[3][9];
#pragma unroll
      for (int c = 0; c < 3; c++)
#pragma unroll
         for (int q = 0; q <= 8; q++) fc[c][q] = F(c, i, j, q);
      const int cc[6] = {0, 1, 2, 0, 0, 1}, dd[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int t = 0; t < 6; t++) {
         const double* w = a.topw + ((long long)(t * 6 + (k - 1)) * 9) * ncol + col;
         double sd = 0, sc = 0;
#pragma unroll
         for (int q = 0; q <= 8; q++) {
            const double wq = __ldg(w + q * ncol);
            sd += wq * fc[dd[t]][q];
            if (cc[t] != dd[t]) sc += wq * fc[cc[t]][q];
         }
         s3[cc[t]] += sd;
         if (cc[t] != dd[t]) s3[dd[t]] += sc;
      }
   }
   // one-sided r derivative of component c at column (ii, jj), row k
   auto drb = [&](int c, int ii, int jj) {
      return __ldg(a.dr + ((k - 1) * 3 + c) * ncol + pidx(b, ii, jj, b.kb));
   };
   // p-outer: QP (central) + RP (one-sided r)
   {
      double G[3][4];
#pragma unroll
      for (int mm = 0; mm < 4; mm++) {
         const int ii = i + (mm < 2 ? mm - 2 : mm - 1);
         const long long q = pidx(b, ii, j, k);
         const double sxx = __ldg(a.sx + (ii - b.ib));
         double dq[3], dr[3];
#pragma unroll
         for (int c = 0; c < 3; c++) {
            dq[c] = cd(F(c, ii, j - 2, k), F(c, ii, j - 1, k), F(c, ii, j + 1, k), F(c, ii, j + 2, k));
            dr[c] = drb(c, ii, j);
         }
         G[0][mm] = Pr(1, q) * dq[1] + istry * ((2 * Pr(2, q) + Pr(3, q)) * sxx * dr[0] +
                                                 Pr(5, q) * syc * dr[1] + Pr(7, q) * dr[2]);
         G[1][mm] = Pr(0, q) * dq[0] + Pr(4, q) * dr[0] + Pr(2, q) * sxx * istry * dr[1];
         G[2][mm] = istry * (Pr(6, q) * dr[0] + Pr(2, q) * sxx * dr[2]);
      }
#pragma unroll
      for (int c = 0; c < 3; c++) s3[c] += cd(G[c][0], G[c][1], G[c][2], G[c][3]);
   }
   // q-outer: PQ (central) + RQ (one-sided r)
   {
      double G[3][4];
#pragma unroll
      for (int mm = 0; mm < 4; mm++) {
         const int jj = j + (mm < 2 ? mm - 2 : mm - 1);
         const long long q = pidx(b, i, jj, k);
         const double syy = __ldg(a.sy + (jj - b.jb));
         double dp[3], dr[3];
#pragma unroll
         for (int c = 0; c < 3; c++) {
            dp[c] = cd(F(c, i - 2, jj, k), F(c, i - 1, jj, k), F(c, i + 1, jj, k), F(c, i + 2, jj, k));
            dr[c] = drb(c, i, jj);
         }
         G[0][mm] = Pr(0, q) * dp[1] + Pr(4, q) * syy * istrx * dr[0] + Pr(2, q) * dr[1];
         G[1][mm] = Pr(1, q) * dp[0] + Pr(3, q) * dr[0] + (2 * Pr(4, q) + Pr(5, q)) * syy * istrx * dr[1] +
                    Pr(7, q) * istrx * dr[2];
         G[2][mm] = istrx * (Pr(4, q) * syy * dr[2] + Pr(6, q) * dr[1]);
      }
#pragma unroll
      for (int c = 0; c < 3; c++) s3[c] += cd(G[c][0], G[c][1], G[c][2], G[c][3]);
   }
   // r-outer (one-sided): PR + QR products at planes 1..8 of this column
#pragma unroll
   for (int c = 0; c < 3; c++) s3[c] += __ldg(a.ro + ((k - 1) * 3 + c) * ncol + col);
   const double kk = a.coef * __ldg(a.cc.K + p);
   if (!CORR) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = p + c * n;
         a.out.set(q, 2 * a.u.get(q) - a.um.get(q) + kk * s3[c]);
      }
   } else {
      double sg[3] = {0, 0, 0};
      if (a.beta != 0) {
         const long long st[2] = {1, b.ni};
         const double w[2] = {sxc * __ldg(a.coy + (j - b.jb)), syc * __ldg(a.cox + (i - b.ib))};
         const double* dcp[2] = {a.dcx + (i - b.ib), a.dcy + (j - b.jb)};
#pragma unroll
         for (int ax = 0; ax < 2; ax++) {
            const long long s = st[ax];
            const double e0 = a.cc.rj[p - s] * dcp[ax][-1], e1 = a.cc.rj[p] * dcp[ax][0],
                         e2 = a.cc.rj[p + s] * dcp[ax][1];
            if (e0 == 0 && e1 == 0 && e2 == 0) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * n;
               const long long qs = c * fb.npts + pidx(fb, i, j, k);
               double d[5];
#pragma unroll
               for (int m = -2; m <= 2; m++)
                  d[m + 2] = a.dd ? __ldg(a.dd + qs + m * s) : a.u.get(q + m * s) - a.um.get(q + m * s);
               sg[c] += w[ax] * (e2 * (d[4] - 2 * d[3] + d[2]) - 2 * e1 * (d[3] - 2 * d[2] + d[1]) +
                                 e0 * (d[2] - 2 * d[1] + d[0]));
            }
         }
      }
      const double birj = a.beta * __ldg(a.cc.irj + p);
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = p + c * n;
         a.out.set(q, (a.up.get(q) + kk * s3[c]) - birj * sg[c]);
      }
   }
}

// The gx x gy x 6 blocks of 32 x 4 points, strided over by the grid (one CTA per
// block, or a persistent grid beside the stage kernels).
template <int CORR, class RD, class WR, class SF>
__global__ void __launch_bounds__(128) curv_top_kernel(TopArgs<RD, WR, SF> a, int gx, int gy)
{
   const int nvb = gx * gy * 6;
   for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int i = a.b.ib + 2 + (vb % gx) * blockDim.x + threadIdx.x;
      const int j = a.b.jb + 2 + ((vb / gx) % gy) * blockDim.y + threadIdx.y;
      if (i > a.b.ie - 2 || j > a.b.je - 2) continue;
      curv_top_point<CORR>(a, i, j, 1 + vb / (gx * gy));
   }
}

int gsb(long long n, int threads = 256)
{
   long long b = (n + threads - 1) / threads;
   if (b > 152 * 16) b = 152 * 16;
   return (int)(b > 0 ? b : 1);
}

template <int CORR, class RD, class WR, class SF, class ST>
int launch_top(const ST& st, RD u, RD um, RD up, WR out, SF f, cudaStream_t s, const double* dd = nullptr,
               int ctas = 0)
{
   const Box& b = st.b;
   TopArgs<RD, WR, SF> t;
   t.b = b;
   t.fb = st.fbox;
   t.f = f;
   t.u = u;
   t.um = um;
   t.up = up;
   t.out = out;
   t.cc = st.cc;
   t.topw = st.cc.topw;
   t.dr = st.scratch;
   t.ro = st.scratch + 18 * b.nij;
   t.dd = dd;
   t.sx = st.sx;
   t.sy = st.sy;
   t.dcx = st.dcx;
   t.dcy = st.dcy;
   t.cox = st.cox;
   t.coy = st.coy;
   t.coef = CORR ? st.dt * st.dt / 12 : st.dt * st.dt;
   t.beta = st.beta;
   if (!st.scratch) return kBadArgument;
   curv_top_pre_kernel<<<ctas > 0 ? ctas : gsb(b.nij, 128), 128, 0, s>>>(b, st.fbox, f, st.cc, st.sx, st.sy,
                                                                         st.scratch, st.scratch + 18 * b.nij);
   SW4G_TRY(launch_status());
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3;
   const int gx = (ni + 31) / 32, gy = (nj + 3) / 4;
   const dim3 blk(32, 4), g(ctas > 0 ? std::min(ctas, gx * gy * 6) : gx * gy * 6);
   curv_top_kernel<CORR><<<g, blk, 0, s>>>(t, gx, gy);
   return launch_status();
}


}  // namespace

long long curv_coef_doubles(long long npts, long long ncol)
{
   return (2LL * kCurvKinds + kProducts + 3) * npts + (long long)kTopSlots * ncol;
}

int curv_coef_setup(const Box& b, const double* mu, const double* la, const double* rho,
                    const double* met, const double* jac, const double* sx, const double* sy,
                    double* store, CurvCoef* c, cudaStream_t s)
{
   const long long n = b.npts;
   for (int q = 0; q < 2 * kCurvKinds; q++) c->w[q] = store + q * n;
   for (int q = 0; q < kProducts; q++) c->prod[q] = store + (2 * kCurvKinds + q) * n;
   c->K = store + (2 * kCurvKinds + kProducts) * n;
   c->rj = c->K + n;
   c->irj = c->rj + n;
   c->topw = c->irj + n;
   SW4G_TRY(upload_top_tables());
   curv_coef_kernel<<<gsb(n), 256, 0, s>>>(b, mu, la, rho, met, jac, sx, sy, *c);
   SW4G_TRY(launch_status());
   curv_topw_kernel<<<gsb(b.nij), 256, 0, s>>>(b, mu, la, met, sx, sy, c->topw);
   return launch_status();
}

int launch_curv_top_df(const CurvStageDF& st, cudaStream_t s, int ctas)
{
   // the stage field (and the corrector's u - um) come as FP64 slabs over planes
   // kb..8: converting each double-float value once there keeps the float-to-double
   // conversions off the stencil loads
   const long long lo = 3 * st.b.npts;
   if (!st.f) return kBadArgument;
   if (st.corrector)
      return launch_top<1>(st, RdDF{st.u, lo}, RdDF{st.um, lo}, RdDF{st.up, lo}, DFField{st.out, lo},
                           RdF64{st.f}, s, st.dd, ctas);
   return launch_top<0>(st, RdDF{st.u, lo}, RdDF{st.um, lo}, RdDF{nullptr, lo}, DFField{st.out, lo},
                        RdF64{st.f}, s, nullptr, ctas);
}

int launch_curv_stage(const CurvStage& st, cudaStream_t s, int part, int ctas)
{
   const Box& b = st.b;
   StageArgs a;
   a.b = b;
   a.u = st.u;
   a.um = st.um;
   a.up = st.up;
   a.out = st.out;
   a.cc = st.cc;
   a.sx = st.sx;
   a.sy = st.sy;
   a.dcx = st.dcx;
   a.dcy = st.dcy;
   a.cox = st.cox;
   a.coy = st.coy;
   a.beta = st.beta;
   const int corr = st.corrector;
   a.coef = corr ? st.dt * st.dt / 12 : st.dt * st.dt;
   if (part != 2) {
      // the ghost shell
      if (corr) curv_shell_kernel<1><<<gsb(b.npts), 256, 0, s>>>(b, st.nz, st.u, st.um, st.up, st.out);
      else curv_shell_kernel<0><<<gsb(b.npts), 256, 0, s>>>(b, st.nz, st.u, st.um, st.up, st.out);
      SW4G_TRY(launch_status());
      // the SBP top rows k = 1..6
      if (corr)
         SW4G_TRY(launch_top<1>(st, RdF64{st.u}, RdF64{st.um}, RdF64{st.up}, F64Field{st.out}, RdF64{st.f}, s,
                                nullptr, ctas));
      else
         SW4G_TRY(launch_top<0>(st, RdF64{st.u}, RdF64{st.um}, RdF64{nullptr}, F64Field{st.out}, RdF64{st.f}, s,
                                nullptr, ctas));
   }
   if (part == 1) return kOk;
   a.coef = corr ? st.dt * st.dt / 12 : st.dt * st.dt;
   a.k1 = 7;
   a.k2 = st.nz;
   const int nk = a.k2 - a.k1 + 1;
   if (nk <= 0) return kOk;
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3;
   const int gx = blocks_for(ni, TX), gy = blocks_for(nj, TY);
   const size_t smem = stage_smem(corr) * sizeof(double);
   const void* kern = corr ? (const void*)curv_stage_kernel<1> : (const void*)curv_stage_kernel<0>;
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kCudaError;
   static bool attr[2][64] = {};
   static int resident[2][64] = {};
   if (!attr[corr][dev]) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
         return kCudaError;
      resident[corr][dev] = resident_ctas(kern, NTHREADS, smem);
      attr[corr][dev] = true;
   }
   a.kchunk = stage_kchunk((long long)gx * gy, nk, resident[corr][dev], 12);
   const dim3 grid(gx, gy, (nk + a.kchunk - 1) / a.kchunk), block(TX, TY, 1);
   if (corr) curv_stage_kernel<1><<<grid, block, smem, s>>>(a);
   else curv_stage_kernel<0><<<grid, block, smem, s>>>(a);
   return launch_status();
}

}  // namespace sw4g
