// Fused stage kernels of the curvilinear grid in the FP32-mixed form, sm_103a.
//
// The stages of curv_stage.cu,
//   predictor  out = 2u - um + dt^2 K S(u)
//   corrector  out = up + dt^2/12 K S(up - 2u + um) - beta/(rho J) SG(u - um)
// (S the bracket of the curvilinear operator, src/rhs4sgcurv_rev.C:34, K = sx sy /
// (J rho)) with the precisions of the Cartesian mixed form (stage_mixed.cu):
//   * the levels are double-float pairs (df.cuh); the time-level accumulation is
//     done with FP32 error-free transformations;
//   * the interior stencil (rows k = 7..nz) and the x/y damping run in FP32; the
//     predictor's stencil field is used as (hi, lo) in every difference, the
//     corrector's up - 2u + um is formed exactly in double-float and rounded once;
//   * every coefficient that combines the metric with the material -- the
//     second-difference weights of the same-axis terms, the cross-term products
//     mu m_a m1, la m_a m1, (2mu+la) m_a m1 and the scale K -- is computed in FP64
//     once per run (curv_coef_kernel) and kept as an FP32 (hi, lo) pair, so no
//     coefficient is rounded to FP32: each coefficient x field-difference product
//     is hi*d + lo*d;
//   * the constant 144 of the cross terms' two 4th-order first differences is
//     folded into the weights (x144) and K (/144) in FP64;
//   * the six SBP top rows, the curvilinear free-surface ghost plane and the
//     interface copy stay in FP64 over the double-float levels (curv_stage.cu,
//     curv.cu).
#include <algorithm>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "stencil.cuh"

namespace sw4g {
namespace {

constexpr int TX = 32, TY = 8, HALO = 2;
constexpr int PX = TX + 2 * HALO;
constexpr int PY = TY + 2 * HALO;
constexpr int PLANE = PX * PY;
constexpr int NTHREADS = TX * TY;

// product pairs: 0..7 as CurvCoef::prod, 8 (2mu+la) m2 m1, 9 (2mu+la) m3 m1
__global__ void curv_coef_df_kernel(long long n, CurvCoef c, CurvCoefDF d)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
        p += (long long)gridDim.x * blockDim.x) {
#pragma unroll
      for (int t = 0; t < 8; t++) df_split(c.prod[t][p], d.ph[t][p], d.pl[t][p]);
      df_split(2 * c.prod[2][p] + c.prod[3][p], d.ph[8][p], d.pl[8][p]);
      df_split(2 * c.prod[4][p] + c.prod[5][p], d.ph[9][p], d.pl[9][p]);
#pragma unroll
      for (int t = 0; t < 20; t++) df_split(144 * c.w[t][p], d.wh[t][p], d.wl[t][p]);
      df_split(c.K[p] / 144, d.Kh[p], d.Kl[p]);
      df_split(c.irj[p], d.irh[p], d.irl[p]);
      d.rj[p] = __double2float_rn(c.rj[p]);
   }
}

struct MArgs {
   Box b;
   int k1, k2, kchunk;
   const float* __restrict__ u;  // levels: hi at [c*npts + p], lo at 3*npts further
   const float* __restrict__ um;
   const float* __restrict__ up;
   float* __restrict__ out;
   CurvCoefDF cd;
   const float* __restrict__ sx;
   const float* __restrict__ sy;
   const float* __restrict__ dcx;
   const float* __restrict__ dcy;
   const float* __restrict__ cox;
   const float* __restrict__ coy;
   float ch, cl;  // dt^2 (predictor) or dt^2/12 (corrector) as a (hi, lo) pair
   float beta;
};

__host__ __device__ constexpr int mixed_smem_floats(int corr)
{
   // predictor: hi and lo rings (5 x 3 planes each); corrector: field ring, damping
   // plane (3) and rho J plane; both: GX, GY
   return (corr ? 19 * PLANE : 30 * PLANE) + 3 * TY * PX + 3 * PY * TX;
}

__device__ __forceinline__ int m5(int k) { return ((k % 5) + 5) % 5; }

template <int CORR>
__global__ void __launch_bounds__(NTHREADS, 3) curv_mixed_kernel(MArgs a)
{
   extern __shared__ float smf[];
   float* VH = smf;                       // [5][3][PLANE] stencil field (hi)
   float* VL = smf + 15 * PLANE;          // predictor: its lo half
   float* DP = smf + 15 * PLANE;          // corrector: u - um at plane k, [3][PLANE]
   float* RJ = DP + 3 * PLANE;            // corrector: rho J at plane k
   float* GX = smf + (CORR ? 19 : 30) * PLANE;  // [3][TY][PX]
   float* GY = GX + 3 * TY * PX;                // [3][PY][TX]
   const Box& b = a.b;
   const long long n = b.npts, lo = 3 * b.npts;
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
      float* vh = VH + m5(kk) * 3 * PLANE;
      float* vl = VL + m5(kk) * 3 * PLANE;
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int gi = i0 - HALO + idx % PX, gj = j0 - HALO + idx / PX;
         const bool in = gi <= b.ie && gj <= b.je;
         const long long p = in ? gidx(gi, gj, kk) : 0;
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const long long q = p + c * n;
            if (!CORR) {
               vh[c * PLANE + idx] = in ? __ldg(a.u + q) : 0.f;
               vl[c * PLANE + idx] = in ? __ldg(a.u + q + lo) : 0.f;
            } else {
               float v = 0.f;
               if (in) {
                  const float uph = __ldg(a.up + q), upl = __ldg(a.up + q + lo);
                  const float uh = __ldg(a.u + q), ul = __ldg(a.u + q + lo);
                  const float mh = __ldg(a.um + q), ml = __ldg(a.um + q + lo);
                  float s1, e1, s2, e2;
                  two_sum(uph, -2.f * uh, s1, e1);
                  two_sum(s1, mh, s2, e2);
                  v = s2 + ((e1 + e2) + ((upl - 2.f * ul) + ml));
               }
               vh[c * PLANE + idx] = v;
            }
         }
      }
   };
   auto load_damping = [&](int kk) {
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int gi = i0 - HALO + idx % PX, gj = j0 - HALO + idx / PX;
         float d[3] = {0.f, 0.f, 0.f}, r = 0.f;
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, kk);
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * n;
               float d1, f1;
               two_sum(__ldg(a.u + q), -__ldg(a.um + q), d1, f1);
               d[c] = d1 + (f1 + (__ldg(a.u + q + lo) - __ldg(a.um + q + lo)));
            }
            r = __ldg(a.cd.rj + p);
         }
#pragma unroll
         for (int c = 0; c < 3; c++) DP[c * PLANE + idx] = d[c];
         RJ[idx] = r;
      }
   };
   // 12 x the centred first difference f(-2) - 8 f(-1) + 8 f(1) - f(2) from four
   // staged samples (hi, and in the predictor lo)
   auto d1 = [&](const float* hm2, const float* hm1, const float* hp1, const float* hp2, int o,
                 int sm2, int sm1, int sp1, int sp2) -> float {
      if (CORR) return (hm2[sm2] - hp2[sp2]) + 8.f * (hp1[sp1] - hm1[sm1]);
      return ((hm2[sm2] - hp2[sp2]) + (hm2[sm2 + o] - hp2[sp2 + o])) +
             8.f * ((hp1[sp1] - hm1[sm1]) + (hp1[sp1 + o] - hm1[sm1 + o]));
   };
   const int LOFF = 15 * PLANE;  // VL - VH
   // in-plane first difference along x (st = 1) or y (st = PX) at staged index s
   auto d1p = [&](const float* v, int s, int st) {
      return d1(v, v, v, v, LOFF, s - 2 * st, s - st, s + st, s + 2 * st);
   };
   // coefficient pair t at point p times x: hi*x + lo*x
   auto pr = [&](int t, long long p, float x) {
      return fmaf(__ldg(a.cd.ph[t] + p), x, __ldg(a.cd.pl[t] + p) * x);
   };
   const float sxi = active ? __ldg(a.sx + (i - b.ib)) : 1.f;
   const float syj = active ? __ldg(a.sy + (j - b.jb)) : 1.f;
   const float isxi = 1.f / sxi, isyj = 1.f / syj;

   // r-outer products of the own column at plane kk (inner p and q differences)
   auto compute_gr = [&](int kk, float g[3]) {
      const float* vs = VH + m5(kk) * 3 * PLANE;
      float dp[3], dq[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
         dp[c] = d1p(vs + c * PLANE, own, 1);
         dq[c] = d1p(vs + c * PLANE, own, PX);
      }
      const long long p = gidx(i, j, kk);
      g[0] = pr(8, p, sxi * isyj * dp[0]) + pr(4, p, dp[1] + syj * isxi * dq[0]) +
             pr(6, p, isyj * dp[2]) + pr(3, p, dq[1]);
      g[1] = pr(5, p, dp[0]) + pr(2, p, sxi * isyj * dp[1] + dq[0]) + pr(9, p, syj * isxi * dq[1]) +
             pr(6, p, isxi * dq[2]);
      g[2] = pr(7, p, isyj * dp[0] + isxi * dq[1]) + pr(2, p, isyj * sxi * dp[2]) +
             pr(4, p, isxi * syj * dq[2]);
   };

   float gz[5][3];
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

      const float* vm2 = VH + m5(k - 2) * 3 * PLANE;
      const float* vm1 = VH + m5(k - 1) * 3 * PLANE;
      const float* v0 = VH + m5(k) * 3 * PLANE;
      const float* vp1 = VH + m5(k + 1) * 3 * PLANE;
      const float* vp2 = VH + m5(k + 2) * 3 * PLANE;
      auto dr = [&](int c, int s) {
         const int o = c * PLANE;
         return d1(vm2 + o, vm1 + o, vp1 + o, vp2 + o, LOFF, s, s, s, s);
      };
      // p-outer products over the x-extended rows
      for (int idx = tid; idx < TY * PX; idx += NTHREADS) {
         const int li = idx % PX, ljr = idx / PX;
         const int s = (ljr + HALO) * PX + li;
         const int gi = i0 - HALO + li, gj = j0 + ljr;
         float g0 = 0.f, g1 = 0.f, g2 = 0.f;
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, k);
            const float sxx = __ldg(a.sx + (gi - b.ib)), isy = 1.f / __ldg(a.sy + (gj - b.jb));
            float dq[3], drr[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
               dq[c] = d1p(v0 + c * PLANE, s, PX);
               drr[c] = dr(c, s);
            }
            g0 = pr(1, p, dq[1]) + pr(8, p, isy * sxx * drr[0]) + pr(5, p, drr[1]) + pr(7, p, isy * drr[2]);
            g1 = pr(0, p, dq[0]) + pr(4, p, drr[0]) + pr(2, p, sxx * isy * drr[1]);
            g2 = pr(6, p, isy * drr[0]) + pr(2, p, isy * sxx * drr[2]);
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
         float g0 = 0.f, g1 = 0.f, g2 = 0.f;
         if (gi <= b.ie && gj <= b.je) {
            const long long p = gidx(gi, gj, k);
            const float syy = __ldg(a.sy + (gj - b.jb)), isx = 1.f / __ldg(a.sx + (gi - b.ib));
            float dpp[3], drr[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
               dpp[c] = d1p(v0 + c * PLANE, s, 1);
               drr[c] = dr(c, s);
            }
            g0 = pr(0, p, dpp[1]) + pr(4, p, syy * isx * drr[0]) + pr(2, p, drr[1]);
            g1 = pr(1, p, dpp[0]) + pr(3, p, drr[0]) + pr(9, p, syy * isx * drr[1]) + pr(7, p, isx * drr[2]);
            g2 = pr(4, p, isx * syy * drr[2]) + pr(6, p, isx * drr[1]);
         }
         GY[idx] = g0;
         GY[PY * TX + idx] = g1;
         GY[2 * PY * TX + idx] = g2;
      }
      __syncthreads();

      if (active) {
         const long long p = gidx(i, j, k);
         const long long off[3] = {1, b.ni, b.nij};
         // f(s) - f(own) of component c in plane v (hi, and lo in the predictor)
         auto dlt = [&](const float* v, int c, int s) {
            const float* x = v + c * PLANE;
            if (CORR) return x[s] - v0[c * PLANE + own];
            return (x[s] - v0[c * PLANE + own]) + (x[s + LOFF] - v0[c * PLANE + own + LOFF]);
         };
         // weights W1(p), W2(p), W2(p+o), W1(p+2o) of kind t as pairs, applied to
         // four differences
         auto wsum = [&](int t, long long o, float dm2, float dm1, float dp1, float dp2) {
            const float* wh1 = a.cd.wh[2 * t];
            const float* wh2 = a.cd.wh[2 * t + 1];
            const float* wl1 = a.cd.wl[2 * t];
            const float* wl2 = a.cd.wl[2 * t + 1];
            const float sh = fmaf(__ldg(wh1 + p), dm2,
                                  fmaf(__ldg(wh2 + p), dm1, fmaf(__ldg(wh2 + p + o), dp1, __ldg(wh1 + p + 2 * o) * dp2)));
            const float sl = fmaf(__ldg(wl1 + p), dm2,
                                  fmaf(__ldg(wl2 + p), dm1, fmaf(__ldg(wl2 + p + o), dp1, __ldg(wl1 + p + 2 * o) * dp2)));
            return sh + sl;
         };
         float s3[3] = {0.f, 0.f, 0.f};
         // same-axis p (kind 0 for c = 0, 1 for c = 1, 2) and q (kind 3 for c = 1,
         // 2 for c = 0, 2)
#pragma unroll
         for (int c = 0; c < 3; c++) {
            s3[c] += wsum(c == 0 ? 0 : 1, off[0], dlt(v0, c, own - 2), dlt(v0, c, own - 1), dlt(v0, c, own + 1),
                          dlt(v0, c, own + 2));
            s3[c] += wsum(c == 1 ? 3 : 2, off[1], dlt(v0, c, own - 2 * PX), dlt(v0, c, own - PX),
                          dlt(v0, c, own + PX), dlt(v0, c, own + 2 * PX));
         }
         // same-axis r: the symmetric matrix A_cd (kinds 4..9 = A00, A11, A22, A01,
         // A02, A12)
#pragma unroll
         for (int t = 4; t < 10; t++) {
            const int cc = t < 7 ? t - 4 : (t == 9 ? 1 : 0);
            const int dd = t < 7 ? t - 4 : (t == 7 ? 1 : 2);
            auto rr = [&](int comp) {
               return wsum(t, off[2], dlt(vm2, comp, own), dlt(vm1, comp, own), dlt(vp1, comp, own),
                           dlt(vp2, comp, own));
            };
            s3[cc] += rr(dd);
            if (cc != dd) s3[dd] += rr(cc);
         }
         // cross terms: outer differences of the staged products (x144 scale)
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const float* gx = GX + c * TY * PX + ty * PX + tx;
            const float* gy = GY + c * PY * TX + ty * TX + tx;
            const float cx = (gx[0] - gx[4]) + 8.f * (gx[3] - gx[1]);
            const float cy = (gy[0] - gy[4 * TX]) + 8.f * (gy[3 * TX] - gy[TX]);
            const float cz = (gz[0][c] - gz[4][c]) + 8.f * (gz[3][c] - gz[1][c]);
            s3[c] += (cx + cy) + cz;
         }
         // per-point scale (ch + cl) (Kh + Kl) as a pair
         const float kh = __ldg(a.cd.Kh + p), kl = __ldg(a.cd.Kl + p);
         const float ph = a.ch * kh;
         const float pl = fmaf(a.ch, kh, -ph) + fmaf(a.ch, kl, a.cl * kh);
         auto scaled = [&](float x) { return fmaf(x, ph, x * pl); };
         if (!CORR) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * n;
               const float uh = v0[c * PLANE + own], ul = v0[c * PLANE + own + LOFF];
               const float mh = __ldg(a.um + q), ml = __ldg(a.um + q + lo);
               float s, e, t, e2, oh, ol;
               two_sum(2.f * uh, -mh, s, e);
               two_sum(s, scaled(s3[c]), t, e2);
               fast_two_sum(t, (e + e2) + (2.f * ul - ml), oh, ol);
               a.out[q] = oh;
               a.out[q + lo] = ol;
            }
         } else {
            float sg[3] = {0.f, 0.f, 0.f};
            if (a.beta != 0.f) {
               const float cxi = __ldg(a.cox + (i - b.ib)), cyj = __ldg(a.coy + (j - b.jb));
               const float dx0 = __ldg(a.dcx + (i - 1 - b.ib)), dx1 = __ldg(a.dcx + (i - b.ib)),
                           dx2 = __ldg(a.dcx + (i + 1 - b.ib));
               if (dx0 != 0.f || dx1 != 0.f || dx2 != 0.f) {
                  const float e0 = RJ[own - 1] * dx0, e1 = RJ[own] * dx1, e2 = RJ[own + 1] * dx2;
                  const float w = sxi * cyj;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const float* d = DP + c * PLANE + own;
                     sg[c] += w * (e2 * (d[2] - 2.f * d[1] + d[0]) - 2.f * e1 * (d[1] - 2.f * d[0] + d[-1]) +
                                   e0 * (d[0] - 2.f * d[-1] + d[-2]));
                  }
               }
               const float dy0 = __ldg(a.dcy + (j - 1 - b.jb)), dy1 = __ldg(a.dcy + (j - b.jb)),
                           dy2 = __ldg(a.dcy + (j + 1 - b.jb));
               if (dy0 != 0.f || dy1 != 0.f || dy2 != 0.f) {
                  const float e0 = RJ[own - PX] * dy0, e1 = RJ[own] * dy1, e2 = RJ[own + PX] * dy2;
                  const float w = syj * cxi;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const float* d = DP + c * PLANE + own;
                     sg[c] += w * (e2 * (d[2 * PX] - 2.f * d[PX] + d[0]) -
                                   2.f * e1 * (d[PX] - 2.f * d[0] + d[-PX]) +
                                   e0 * (d[0] - 2.f * d[-PX] + d[-2 * PX]));
                  }
               }
            }
            const float birj = a.beta * __ldg(a.cd.irh + p);
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * n;
               const float uph = __ldg(a.up + q), upl = __ldg(a.up + q + lo);
               float t, e, oh, ol;
               two_sum(uph, scaled(s3[c]) - birj * sg[c], t, e);
               fast_two_sum(t, e + upl, oh, ol);
               a.out[q] = oh;
               a.out[q + lo] = ol;
            }
         }
      }
      __syncthreads();
   }
}

int gsb(long long n)
{
   long long g = (n + 255) / 256;
   return (int)std::min<long long>(std::max<long long>(g, 1), 152LL * 16);
}

}  // namespace

long long curv_coef_df_floats(long long npts) { return (2LL * (10 + 20 + 2) + 3) * npts; }

int curv_coef_df_setup(long long npts, const CurvCoef& c, float* store, CurvCoefDF* d, cudaStream_t s)
{
   if (!store || !d) return kBadArgument;
   const long long n = npts;
   float* q = store;
   for (int t = 0; t < 10; t++) {
      d->ph[t] = q;
      d->pl[t] = q + n;
      q += 2 * n;
   }
   for (int t = 0; t < 20; t++) {
      d->wh[t] = q;
      d->wl[t] = q + n;
      q += 2 * n;
   }
   d->Kh = q;
   d->Kl = q + n;
   d->irh = q + 2 * n;
   d->irl = q + 3 * n;
   d->rj = q + 4 * n;
   curv_coef_df_kernel<<<gsb(n), 256, 0, s>>>(n, c, *d);
   return launch_status();
}

int launch_curv_stage_df(const CurvStageDF& st, cudaStream_t s, int part, int ctas)
{
   const Box& b = st.b;
   const int corr = st.corrector;
   if (!st.work1 || (corr && !st.work2)) return kBadArgument;
   if (part != 2) {
      // FP64 slabs of the top rows' stage field (and u - um) over planes kb..8
      CurvStageDF t = st;
      t.fbox = make_box(1, b.ib, b.ie, b.jb, b.je, b.kb, 8);
      t.f = st.work1;
      if (corr) {
         SW4G_TRY(launch_uacc_slab_df(b, b.kb, 8, st.up, st.u, st.um, st.work1, s));
         SW4G_TRY(launch_df_slab(b, b.kb, 8, st.u, st.um, st.work2, s));
         t.dd = st.work2;
      } else {
         SW4G_TRY(launch_df_slab(b, b.kb, 8, st.u, nullptr, st.work1, s));
      }
      // the ghost shell, then the SBP top rows k = 1..6 in FP64
      SW4G_TRY(launch_ghost_shell_df(b, corr, st.out, st.u, st.um, st.up, s));
      SW4G_TRY(launch_curv_top_df(t, s, ctas));
   }
   if (part == 1) return kOk;
   MArgs a;
   a.b = b;
   a.u = st.u;
   a.um = st.um;
   a.up = st.up;
   a.out = st.out;
   a.cd = st.cd;
   a.sx = st.sx32;
   a.sy = st.sy32;
   a.dcx = st.dcx32;
   a.dcy = st.dcy32;
   a.cox = st.cox32;
   a.coy = st.coy32;
   const double coef = corr ? st.dt * st.dt / 12 : st.dt * st.dt;
   a.ch = static_cast<float>(coef);
   a.cl = static_cast<float>(coef - (double)a.ch);
   a.beta = static_cast<float>(st.beta);
   a.k1 = 7;
   a.k2 = st.nz;
   const int nk = a.k2 - a.k1 + 1;
   if (nk <= 0) return kOk;
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3;
   const int gx = blocks_for(ni, TX), gy = blocks_for(nj, TY);
   const size_t smem = mixed_smem_floats(corr) * sizeof(float);
   const void* kern = corr ? (const void*)curv_mixed_kernel<1> : (const void*)curv_mixed_kernel<0>;
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
   if (corr) curv_mixed_kernel<1><<<grid, block, smem, s>>>(a);
   else curv_mixed_kernel<0><<<grid, block, smem, s>>>(a);
   return launch_status();
}

}  // namespace sw4g
