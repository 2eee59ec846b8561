// Fused stage kernels of the FP32-mixed form, sm_103a.
//
// Same stages as the FP64 form (stage_fused.cu):
//   predictor  out = 2u - um + dt^2/rho * L(u)
//   corrector  out = up + dt^2/12/rho * L(up - 2u + um) - beta/rho * SG(u - um)
//   adjoint    out = 2u - um + dt^2/rho * L(up) - beta/rho * SG(u - um)
// (the adjoint form is the scaled adjoint recursion of adjoint.cu; the predictor
// form with a replaced coefficient gives its first stage)
// with these precisions:
//   * solution levels are double-float pairs (df.cuh): 48-bit storage, so the
//     time-level accumulation keeps FP64-class precision, done with FP32
//     error-free transformations;
//   * the interior stencil L and the damping SG run in FP32 on FP32 material;
//   * the predictor's stencil field is used as (hi, lo): every difference the
//     stencil takes is (h_a - h_b) + (l_a - l_b), so FP32 rounding of u is not
//     fed to the second differences as noise;
//   * the corrector's stencil field up - 2u + um is formed exactly in
//     double-float and rounded once to FP32.
// Coefficients are kept at FP64 accuracy as FP32 (hi, lo) pairs: the
// second-difference weights (precomputed in FP64, split), mu, lambda and 1/rho, and
// the global scale dt^2/(144 h^2).  Each product coefficient x field-difference is
// formed as hi*d + lo*d.  Rounding a coefficient to FP32 would change the discrete
// wave speed by ~1e-7 everywhere at once, and that systematic error grows into a
// phase error proportional to the simulated time; the rounding left (FP32
// products and sums of field differences) varies from point to point and step
// to step.  One-sided rows, the free-surface ghost solve and forcing stay in
// FP64 (rhs4_direct.cu, bc.cu, forcing.cu).
#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

constexpr int TX = 32, TY = 8, HALO = 2;
constexpr int PX = TX + 2 * HALO;
constexpr int PY = TY + 2 * HALO;
constexpr int PLANE = PX * PY;
constexpr int NTHREADS = TX * TY;

struct MixedArgs {
   int ib, ie, jb, je, kb, ke;
   long long ni, nij, npts;
   int k1, k2, kchunk;
   const float* __restrict__ u;  // levels: hi at [c*npts + p], lo at 3*npts further
   const float* __restrict__ um;
   const float* __restrict__ up;
   float* __restrict__ out;
   const float2* __restrict__ mu2;  // mu, lambda, 1/rho as interleaved (hi, lo) pairs
   const float2* __restrict__ la2;
   const float2* __restrict__ ir2;
   const float* __restrict__ rho;   // FP32, supergrid damping only
   const float2* __restrict__ w2[kWeightArrays];  // second-difference weights (unscaled), pairs
   const float* __restrict__ sx;
   const float* __restrict__ sy;
   const float* __restrict__ sz;
   const float* __restrict__ dc[3];
   const float* __restrict__ co[3];
   float Kh, Kl;        // dt^2/(144 h^2) (predictor) or dt^2/(12*144 h^2) (corrector), as a pair
   float beta;
};

__host__ __device__ constexpr int smem_floats(int form)
{
   // predictor: hi and lo rings (5 x 3 planes each); corrector: field ring (5 x 3),
   // damping ring (3 x 3) and rho plane; adjoint: hi and lo rings, damping ring and rho
   // plane; all: mu, lambda (hi, lo) planes, GX, GY
   return (form == 1 ? 25 * PLANE : form == 2 ? 40 * PLANE : 30 * PLANE) + 4 * PLANE +
          3 * TY * PX + 3 * PY * TX;
}

__device__ __forceinline__ int mod5(int k) { return ((k % 5) + 5) % 5; }
__device__ __forceinline__ int mod3(int k) { return ((k % 3) + 3) % 3; }

template <int CORR>
__global__ void __launch_bounds__(NTHREADS, 3) mixed_stage_kernel(MixedArgs a)
{
   extern __shared__ float smf[];
   // predictor: VH | VL ; corrector: VH (the field) | DD | RH
   // CORR: 0 predictor, 1 corrector, 2 adjoint (stencil field up as (hi, lo), damping
   // of u - um, out = 2u - um + K L(up) - beta/rho SG(u - um))
   float* VH = smf;
   float* VL = smf + 15 * PLANE;                       // predictor and adjoint forms
   float* DD = smf + (CORR == 2 ? 30 : 15) * PLANE;    // corrector and adjoint forms
   float* RH = DD + 9 * PLANE;                         // corrector and adjoint forms
   float* MUH = smf + (CORR == 0 ? 30 : CORR == 1 ? 25 : 40) * PLANE;
   float* MUL = MUH + PLANE;
   float* LAH = MUL + PLANE;
   float* LAL = LAH + PLANE;
   float* GX = LAL + PLANE;                // [3][TY][PX]
   float* GY = GX + 3 * TY * PX;           // [3][PY][TX]

   const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
   const int i0 = a.ib + 2 + blockIdx.x * TX;
   const int j0 = a.jb + 2 + blockIdx.y * TY;
   const int kbeg = a.k1 + blockIdx.z * a.kchunk;
   if (kbeg > a.k2) return;
   const int kend = min(kbeg + a.kchunk - 1, a.k2);
   const int i = i0 + tx, j = j0 + ty;
   const bool active = (i <= a.ie - 2) && (j <= a.je - 2);
   const int own = (ty + HALO) * PX + (tx + HALO);
   const long long npts = a.npts, lo = 3 * a.npts;

   auto gidx = [&](int gi, int gj, int gk) -> long long {
      return (long long)(gi - a.ib) + a.ni * (gj - a.jb) + a.nij * (long long)(gk - a.kb);
   };

   auto load_plane = [&](int kk) {
      float* vh = VH + mod5(kk) * 3 * PLANE;
      float* vl = VL + mod5(kk) * 3 * PLANE;
      float* dd = DD + mod3(kk) * 3 * PLANE;
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int li = idx % PX, lj = idx / PX;
         const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
         const bool in = gi <= a.ie && gj <= a.je;
         const long long p = in ? gidx(gi, gj, kk) : 0;
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const long long q = p + c * npts;
            if (CORR != 1) {
               const float* src = CORR == 2 ? a.up : a.u;
               vh[c * PLANE + idx] = in ? __ldg(src + q) : 0.f;
               vl[c * PLANE + idx] = in ? __ldg(src + q + lo) : 0.f;
               if (CORR == 2) {
                  float d = 0.f;
                  if (in) {
                     float d1, f1;
                     two_sum(__ldg(a.u + q), -__ldg(a.um + q), d1, f1);
                     d = d1 + (f1 + (__ldg(a.u + q + lo) - __ldg(a.um + q + lo)));
                  }
                  dd[c * PLANE + idx] = d;
               }
            } else {
               float v = 0.f, d = 0.f;
               if (in) {
                  const float uph = __ldg(a.up + q), upl = __ldg(a.up + q + lo);
                  const float uh = __ldg(a.u + q), ul = __ldg(a.u + q + lo);
                  const float mh = __ldg(a.um + q), ml = __ldg(a.um + q + lo);
                  // (up - 2u + um) exactly in double-float, rounded once
                  float s1, e1, s2, e2;
                  two_sum(uph, -2.f * uh, s1, e1);
                  two_sum(s1, mh, s2, e2);
                  v = s2 + ((e1 + e2) + ((upl - 2.f * ul) + ml));
                  float d1, f1;
                  two_sum(uh, -mh, d1, f1);
                  d = d1 + (f1 + (ul - ml));
               }
               vh[c * PLANE + idx] = v;
               dd[c * PLANE + idx] = d;
            }
         }
      }
   };

   auto load_material = [&](int kk) {
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int li = idx % PX, lj = idx / PX;
         const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
         float mh = 0.f, ml = 0.f, lh = 0.f, ll = 0.f, r = 0.f;
         if (gi <= a.ie && gj <= a.je) {
            const long long p = gidx(gi, gj, kk);
            const float2 m2 = __ldg(a.mu2 + p), l2 = __ldg(a.la2 + p);
            mh = m2.x;
            ml = m2.y;
            lh = l2.x;
            ll = l2.y;
            if (CORR) r = __ldg(a.rho + p);
         }
         MUH[idx] = mh;
         MUL[idx] = ml;
         LAH[idx] = lh;
         LAL[idx] = ll;
         if (CORR) RH[idx] = r;
      }
   };

   // difference f(a) - f(b) of component c within one staged plane
   auto diff = [&](const float* vh, const float* vl, int ia, int ib_) -> float {
      if (CORR == 1) return vh[ia] - vh[ib_];
      return (vh[ia] - vh[ib_]) + (vl[ia] - vl[ib_]);
   };
   // 12h * centred first difference from 4 samples given as (plane, index) pairs
   auto d1 = [&](const float* hm2, const float* lm2, int im2, const float* hm1, const float* lm1,
                 int im1, const float* hp1, const float* lp1, int ip1, const float* hp2,
                 const float* lp2, int ip2) -> float {
      if (CORR == 1) return (hm2[im2] - hp2[ip2]) + 8.f * (hp1[ip1] - hm1[im1]);
      return ((hm2[im2] - hp2[ip2]) + (lm2[im2] - lp2[ip2])) +
             8.f * ((hp1[ip1] - hm1[im1]) + (lp1[ip1] - lm1[im1]));
   };

   const float sxi = active ? __ldg(a.sx + (i - a.ib)) : 0.f;
   const float syj = active ? __ldg(a.sy + (j - a.jb)) : 0.f;

   auto compute_gz = [&](int kk, float g[3]) {
      const float* vh = VH + mod5(kk) * 3 * PLANE;
      const float* vl = VL + mod5(kk) * 3 * PLANE;
      const float *hu = vh, *hv = vh + PLANE, *hw = vh + 2 * PLANE;
      const float *lu_ = vl, *lv = vl + PLANE, *lw = vl + 2 * PLANE;
      const float dxw = d1(hw, lw, own - 2, hw, lw, own - 1, hw, lw, own + 1, hw, lw, own + 2);
      const float dyw = d1(hw, lw, own - 2 * PX, hw, lw, own - PX, hw, lw, own + PX, hw, lw, own + 2 * PX);
      const float dxu = d1(hu, lu_, own - 2, hu, lu_, own - 1, hu, lu_, own + 1, hu, lu_, own + 2);
      const float dyv = d1(hv, lv, own - 2 * PX, hv, lv, own - PX, hv, lv, own + PX, hv, lv, own + 2 * PX);
      const long long p = gidx(i, j, kk);
      const float2 m2 = __ldg(a.mu2 + p), l2 = __ldg(a.la2 + p);
      const float mh = m2.x, ml = m2.y, lh = l2.x, ll = l2.y;
      const float x0 = sxi * dxw, x1 = syj * dyw, x2 = sxi * dxu + syj * dyv;
      g[0] = fmaf(mh, x0, ml * x0);
      g[1] = fmaf(mh, x1, ml * x1);
      g[2] = fmaf(lh, x2, ll * x2);
   };

   float gz[5][3], dq[5][3];

   // ---- prologue: planes kbeg-2 .. kbeg+1 ----
   for (int kk = kbeg - 2; kk <= kbeg; kk++) load_plane(kk);
   __syncthreads();
   for (int kk = kbeg - 2; kk <= kbeg; kk++) {
      const int q = kk - kbeg + 3;
      if (active) compute_gz(kk, gz[q]);
      if (CORR) {
         const float* dd = DD + mod3(kk) * 3 * PLANE;
#pragma unroll
         for (int c = 0; c < 3; c++) dq[q][c] = dd[c * PLANE + own];
      }
   }
   __syncthreads();
   load_plane(kbeg + 1);
   __syncthreads();
   if (active) compute_gz(kbeg + 1, gz[4]);
   if (CORR) {
      const float* dd = DD + mod3(kbeg + 1) * 3 * PLANE;
#pragma unroll
      for (int c = 0; c < 3; c++) dq[4][c] = dd[c * PLANE + own];
   }

   for (int k = kbeg; k <= kend; k++) {
      load_plane(k + 2);
      load_material(k);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 4; q++) {
#pragma unroll
         for (int c = 0; c < 3; c++) {
            gz[q][c] = gz[q + 1][c];
            if (CORR) dq[q][c] = dq[q + 1][c];
         }
      }
      if (active) compute_gz(k + 2, gz[4]);
      if (CORR) {
         const float* dd = DD + mod3(k + 2) * 3 * PLANE;
#pragma unroll
         for (int c = 0; c < 3; c++) dq[4][c] = dd[c * PLANE + own];
      }

      const float szk = __ldg(a.sz + (k - a.kb));
      const float* hm2 = VH + mod5(k - 2) * 3 * PLANE;
      const float* hm1 = VH + mod5(k - 1) * 3 * PLANE;
      const float* h0 = VH + mod5(k) * 3 * PLANE;
      const float* hp1 = VH + mod5(k + 1) * 3 * PLANE;
      const float* hp2 = VH + mod5(k + 2) * 3 * PLANE;
      const float* lm2 = VL + mod5(k - 2) * 3 * PLANE;
      const float* lm1 = VL + mod5(k - 1) * 3 * PLANE;
      const float* l0 = VL + mod5(k) * 3 * PLANE;
      const float* lp1 = VL + mod5(k + 1) * 3 * PLANE;
      const float* lp2 = VL + mod5(k + 2) * 3 * PLANE;
      auto dz = [&](int c, int s) {
         const int o = c * PLANE;
         return d1(hm2 + o, lm2 + o, s, hm1 + o, lm1 + o, s, hp1 + o, lp1 + o, s, hp2 + o, lp2 + o, s);
      };

      // x-outer products over 36 x 8, y-outer products over 32 x 12 (stage_fused.cu)
      for (int idx = tid; idx < TY * PX; idx += NTHREADS) {
         const int li = idx % PX, ljr = idx / PX;
         const int s = (ljr + HALO) * PX + li;
         const int gi = i0 - HALO + li, gj = j0 + ljr;
         float g0 = 0.f, g1 = 0.f, g2 = 0.f;
         if (gi <= a.ie && gj <= a.je) {
            const float syy = __ldg(a.sy + (gj - a.jb));
            const float *hu = h0, *hv = h0 + PLANE, *lu_ = l0, *lv = l0 + PLANE;
            const float dyv = d1(hv, lv, s - 2 * PX, hv, lv, s - PX, hv, lv, s + PX, hv, lv, s + 2 * PX);
            const float dyu = d1(hu, lu_, s - 2 * PX, hu, lu_, s - PX, hu, lu_, s + PX, hu, lu_, s + 2 * PX);
            const float dzw = dz(2, s), dzu = dz(0, s);
            const float mh = MUH[s], ml = MUL[s], lh = LAH[s], ll = LAL[s];
            const float x0 = syy * dyv + szk * dzw, x1 = syy * dyu, x2 = szk * dzu;
            g0 = fmaf(lh, x0, ll * x0);
            g1 = fmaf(mh, x1, ml * x1);
            g2 = fmaf(mh, x2, ml * x2);
         }
         GX[idx] = g0;
         GX[TY * PX + idx] = g1;
         GX[2 * TY * PX + idx] = g2;
      }
      for (int idx = tid; idx < PY * TX; idx += NTHREADS) {
         const int lic = idx % TX, lj = idx / TX;
         const int s = lj * PX + lic + HALO;
         const int gi = i0 + lic, gj = j0 - HALO + lj;
         float g0 = 0.f, g1 = 0.f, g2 = 0.f;
         if (gi <= a.ie && gj <= a.je) {
            const float sxx = __ldg(a.sx + (gi - a.ib));
            const float *hu = h0, *hv = h0 + PLANE, *lu_ = l0, *lv = l0 + PLANE;
            const float dxv = d1(hv, lv, s - 2, hv, lv, s - 1, hv, lv, s + 1, hv, lv, s + 2);
            const float dxu = d1(hu, lu_, s - 2, hu, lu_, s - 1, hu, lu_, s + 1, hu, lu_, s + 2);
            const float dzw = dz(2, s), dzv = dz(1, s);
            const float mh = MUH[s], ml = MUL[s], lh = LAH[s], ll = LAL[s];
            const float x0 = sxx * dxv, x1 = sxx * dxu + szk * dzw, x2 = szk * dzv;
            g0 = fmaf(mh, x0, ml * x0);
            g1 = fmaf(lh, x1, ll * x1);
            g2 = fmaf(mh, x2, ml * x2);
         }
         GY[idx] = g0;
         GY[PY * TX + idx] = g1;
         GY[2 * PY * TX + idx] = g2;
      }
      __syncthreads();

      if (active) {
         const long long p = gidx(i, j, k);
         // second-difference weights W1(q), W2(q), W2(q+1), W1(q+2) per axis and
         // coefficient type, as (hi, lo) pairs
         const long long off[3] = {1, a.ni, a.nij};
         float wth[3][2][4], wtl[3][2][4];
#pragma unroll
         for (int ax = 0; ax < 3; ax++)
#pragma unroll
            for (int t = 0; t < 2; t++) {
               const int s1 = ax * 4 + t * 2, s2 = s1 + 1;
               const long long o = off[ax];
               const float2 q0 = __ldg(a.w2[s1] + p), q1 = __ldg(a.w2[s2] + p),
                            q2 = __ldg(a.w2[s2] + p + o), q3 = __ldg(a.w2[s1] + p + 2 * o);
               wth[ax][t][0] = q0.x;
               wth[ax][t][1] = q1.x;
               wth[ax][t][2] = q2.x;
               wth[ax][t][3] = q3.x;
               wtl[ax][t][0] = q0.y;
               wtl[ax][t][1] = q1.y;
               wtl[ax][t][2] = q2.y;
               wtl[ax][t][3] = q3.y;
            }
         auto wsum = [&](int ax, int t, float dm2, float dm1, float dp1, float dp2) {
            const float* h = wth[ax][t];
            const float* l = wtl[ax][t];
            const float sh = fmaf(h[0], dm2, fmaf(h[1], dm1, fmaf(h[2], dp1, h[3] * dp2)));
            const float sl = fmaf(l[0], dm2, fmaf(l[1], dm1, fmaf(l[2], dp1, l[3] * dp2)));
            return sh + sl;
         };
         float xs[3];
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const float* ch = h0 + c * PLANE;
            const float* cl = l0 + c * PLANE;
            const int o = c * PLANE;
            const float sxx = wsum(0, c == 0, diff(ch, cl, own - 2, own), diff(ch, cl, own - 1, own),
                                   diff(ch, cl, own + 1, own), diff(ch, cl, own + 2, own));
            const float syy = wsum(1, c == 1, diff(ch, cl, own - 2 * PX, own),
                                   diff(ch, cl, own - PX, own), diff(ch, cl, own + PX, own),
                                   diff(ch, cl, own + 2 * PX, own));
            float dzm2, dzm1, dzp1, dzp2;
            if (CORR == 1) {
               dzm2 = hm2[o + own] - ch[own];
               dzm1 = hm1[o + own] - ch[own];
               dzp1 = hp1[o + own] - ch[own];
               dzp2 = hp2[o + own] - ch[own];
            } else {
               dzm2 = (hm2[o + own] - ch[own]) + (lm2[o + own] - cl[own]);
               dzm1 = (hm1[o + own] - ch[own]) + (lm1[o + own] - cl[own]);
               dzp1 = (hp1[o + own] - ch[own]) + (lp1[o + own] - cl[own]);
               dzp2 = (hp2[o + own] - ch[own]) + (lp2[o + own] - cl[own]);
            }
            const float szz = wsum(2, c == 2, dzm2, dzm1, dzp1, dzp2);
            const float* gx = GX + c * TY * PX + ty * PX + tx;
            const float* gy = GY + c * PY * TX + ty * TX + tx;
            const float cx = (gx[0] - gx[4]) + 8.f * (gx[3] - gx[1]);
            const float cy = (gy[0] - gy[4 * TX]) + 8.f * (gy[3 * TX] - gy[TX]);
            const float cz = (gz[0][c] - gz[4][c]) + 8.f * (gz[3][c] - gz[1][c]);
            // 144 h^2 L u = 24 * (second differences) + (mixed differences)
            const float sd = sxi * sxx + syj * syy + szk * szz;
            xs[c] = (16.f * sd + 8.f * sd) + (sxi * cx + syj * cy + szk * cz);
         }
         // per-point scale K/rho as a (hi, lo) pair: ph + pl = (Kh + Kl) * (irh + irl)
         const float2 ir = __ldg(a.ir2 + p);
         const float irh = ir.x, irl = ir.y;
         const float ph = a.Kh * irh;
         const float pl = fmaf(a.Kh, irh, -ph) + fmaf(a.Kh, irl, a.Kl * irh);
         auto scaled = [&](float x) { return fmaf(x, ph, x * pl); };
         if (!CORR) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * npts;
               const float uh = h0[c * PLANE + own], ul = l0[c * PLANE + own];
               const float mh = __ldg(a.um + q), ml = __ldg(a.um + q + lo);
               float s, e, t, e2, oh, ol;
               two_sum(2.f * uh, -mh, s, e);
               two_sum(s, scaled(xs[c]), t, e2);
               fast_two_sum(t, (e + e2) + (2.f * ul - ml), oh, ol);
               a.out[q] = oh;
               a.out[q + lo] = ol;
            }
         } else {
            float sg[3] = {0.f, 0.f, 0.f};
            if (a.beta != 0.f) {
               const float* dd = DD + mod3(k) * 3 * PLANE;
               const float cxi = __ldg(a.co[0] + (i - a.ib)), cyj = __ldg(a.co[1] + (j - a.jb)),
                           czk = __ldg(a.co[2] + (k - a.kb));
               const float dx0 = __ldg(a.dc[0] + (i - 1 - a.ib)), dx1 = __ldg(a.dc[0] + (i - a.ib)),
                           dx2 = __ldg(a.dc[0] + (i + 1 - a.ib));
               if (dx0 != 0.f || dx1 != 0.f || dx2 != 0.f) {
                  const float e0 = RH[own - 1] * dx0, e1 = RH[own] * dx1, e2 = RH[own + 1] * dx2;
                  const float w = sxi * cyj * czk;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const float* d = dd + c * PLANE + own;
                     sg[c] += w * (e2 * (d[2] - 2.f * d[1] + d[0]) - 2.f * e1 * (d[1] - 2.f * d[0] + d[-1]) +
                                   e0 * (d[0] - 2.f * d[-1] + d[-2]));
                  }
               }
               const float dy0 = __ldg(a.dc[1] + (j - 1 - a.jb)), dy1 = __ldg(a.dc[1] + (j - a.jb)),
                           dy2 = __ldg(a.dc[1] + (j + 1 - a.jb));
               if (dy0 != 0.f || dy1 != 0.f || dy2 != 0.f) {
                  const float e0 = RH[own - PX] * dy0, e1 = RH[own] * dy1, e2 = RH[own + PX] * dy2;
                  const float w = syj * cxi * czk;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const float* d = dd + c * PLANE + own;
                     sg[c] += w * (e2 * (d[2 * PX] - 2.f * d[PX] + d[0]) -
                                   2.f * e1 * (d[PX] - 2.f * d[0] + d[-PX]) +
                                   e0 * (d[0] - 2.f * d[-PX] + d[-2 * PX]));
                  }
               }
               const float dz0 = __ldg(a.dc[2] + (k - 1 - a.kb)), dz1 = __ldg(a.dc[2] + (k - a.kb)),
                           dz2 = __ldg(a.dc[2] + (k + 1 - a.kb));
               if (dz0 != 0.f || dz1 != 0.f || dz2 != 0.f) {
                  const float e0 = __ldg(a.rho + p - a.nij) * dz0, e1 = RH[own] * dz1,
                              e2 = __ldg(a.rho + p + a.nij) * dz2;
                  const float w = szk * cxi * cyj;
#pragma unroll
                  for (int c = 0; c < 3; c++)
                     sg[c] += w * (e2 * (dq[4][c] - 2.f * dq[3][c] + dq[2][c]) -
                                   2.f * e1 * (dq[3][c] - 2.f * dq[2][c] + dq[1][c]) +
                                   e0 * (dq[2][c] - 2.f * dq[1][c] + dq[0][c]));
               }
            }
            const float birho = a.beta * irh;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * npts;
               float t, e, oh, ol;
               if (CORR == 1) {
                  const float uph = __ldg(a.up + q), upl = __ldg(a.up + q + lo);
                  two_sum(uph, scaled(xs[c]) - birho * sg[c], t, e);
                  fast_two_sum(t, e + upl, oh, ol);
               } else {  // adjoint form: 2u - um + K L(up) - beta/rho SG(u - um)
                  const float uh = __ldg(a.u + q), ul = __ldg(a.u + q + lo);
                  const float mh = __ldg(a.um + q), ml = __ldg(a.um + q + lo);
                  float s2, e1, e2;
                  two_sum(2.f * uh, -mh, s2, e1);
                  two_sum(s2, scaled(xs[c]) - birho * sg[c], t, e2);
                  fast_two_sum(t, (e1 + e2) + (2.f * ul - ml), oh, ol);
               }
               a.out[q] = oh;
               a.out[q + lo] = ol;
            }
         }
      }
      __syncthreads();
   }
}

// Second-difference weights (stage_fused.cu's weights_kernel formula, unscaled) in
// FP64, stored as (hi, lo) FP32 pairs.
__global__ void weights_df_kernel(Box b, const double* __restrict__ mu, const double* __restrict__ la,
                                  const double* __restrict__ sx, const double* __restrict__ sy,
                                  const double* __restrict__ sz, WeightPtrsDF w)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(p % b.ni);
      const int j = b.jb + (int)((p / b.ni) % (b.je - b.jb + 1));
      const int k = b.kb + (int)(p / b.nij);
      const int qv[3] = {i, j, k}, lo_[3] = {b.ib, b.jb, b.kb}, hi_[3] = {b.ie, b.je, b.ke};
      const long long st[3] = {1, b.ni, b.nij};
      const double* sv[3] = {sx, sy, sz};
      for (int ax = 0; ax < 3; ax++) {
         double w1[2] = {0, 0}, w2[2] = {0, 0};
         const int q = qv[ax];
         if (q - 2 >= lo_[ax]) {
            double am[2][4];
            for (int m = -2; m <= 1; m++) {
               if (q + m > hi_[ax]) {
                  am[0][m + 2] = am[1][m + 2] = 0;
                  continue;
               }
               const long long pm = p + m * st[ax];
               const double s = sv[ax][q + m - lo_[ax]];
               am[0][m + 2] = mu[pm] * s;
               am[1][m + 2] = (2 * mu[pm] + la[pm]) * s;
            }
            for (int t = 0; t < 2; t++) {
               w1[t] = am[t][1] - 0.75 * (am[t][2] + am[t][0]);
               if (q + 1 <= hi_[ax]) w2[t] = am[t][0] + am[t][3] + 3 * (am[t][2] + am[t][1]);
            }
         }
         for (int t = 0; t < 2; t++) {
            float h1, l1, h2, l2;
            df_split(w1[t], h1, l1);
            df_split(w2[t], h2, l2);
            w.p[ax * 4 + t * 2][p] = make_float2(h1, l1);
            w.p[ax * 4 + t * 2 + 1][p] = make_float2(h2, l2);
         }
      }
   }
}

__global__ void df_from_f64_kernel(long long n, const double* __restrict__ x, float* __restrict__ h,
                                   float* __restrict__ l)
{
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x)
      df_split(x[q], h[q], l[q]);
}

__global__ void df2_from_f64_kernel(long long n, const double* __restrict__ x, float2* __restrict__ hl)
{
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x) {
      float h, l;
      df_split(x[q], h, l);
      hl[q] = make_float2(h, l);
   }
}

__global__ void df_to_f64_kernel(long long n, const float* __restrict__ h, const float* __restrict__ l,
                                 double* __restrict__ x)
{
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x)
      x[q] = df_value(h[q], l[q]);
}

__global__ void to_f32_kernel(long long n, const double* __restrict__ x, float* __restrict__ y)
{
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x)
      y[q] = __double2float_rn(x[q]);
}

int gs_blocks(long long n)
{
   long long g = (n + 255) / 256;
   return (int)std::min<long long>(std::max<long long>(g, 1), 152LL * 16);
}

}  // namespace

int launch_df2_from_f64(long long n, const double* x, float2* hl, cudaStream_t s)
{
   df2_from_f64_kernel<<<gs_blocks(n), 256, 0, s>>>(n, x, hl);
   return launch_status();
}

int launch_df_from_f64(long long n, const double* x, float* h, float* l, cudaStream_t s)
{
   df_from_f64_kernel<<<gs_blocks(n), 256, 0, s>>>(n, x, h, l);
   return launch_status();
}

int launch_df_to_f64(long long n, const float* h, const float* l, double* x, cudaStream_t s)
{
   df_to_f64_kernel<<<gs_blocks(n), 256, 0, s>>>(n, h, l, x);
   return launch_status();
}

int launch_weights_df(const Box& b, const double* mu, const double* la, const double* sx,
                      const double* sy, const double* sz, WeightPtrsDF w, cudaStream_t s)
{
   weights_df_kernel<<<gs_blocks(b.npts), 256, 0, s>>>(b, mu, la, sx, sy, sz, w);
   return launch_status();
}

int launch_to_f32(long long n, const double* x, float* y, cudaStream_t s)
{
   to_f32_kernel<<<gs_blocks(n), 256, 0, s>>>(n, x, y);
   return launch_status();
}

namespace {
std::atomic<int> g_mixed_tma{1};
}

void set_mixed_tma(int on) { g_mixed_tma.store(on ? 1 : 0); }
int mixed_tma_enabled() { return g_mixed_tma.load(); }
std::atomic<int> g_rows_overlap{1};
std::atomic<int> g_adj_pipe{1};
void set_adjoint_pipeline(int on) { g_adj_pipe.store(on ? 1 : 0); }
int adjoint_pipeline_enabled() { return g_adj_pipe.load(); }
void set_rows_overlap(int on) { g_rows_overlap.store(on ? 1 : 0); }
int rows_overlap_enabled() { return g_rows_overlap.load(); }

int launch_mixed_stage(const MixedStage& st, cudaStream_t stream)
{
   if (st.k2 < st.k1) return kOk;
   if (g_mixed_tma.load() && mixed_stage_tma_ok(st)) return launch_mixed_stage_tma(st, stream);
   const Box& b = st.b;
   MixedArgs a;
   a.ib = b.ib; a.ie = b.ie; a.jb = b.jb; a.je = b.je; a.kb = b.kb; a.ke = b.ke;
   a.ni = b.ni; a.nij = b.nij; a.npts = b.npts;
   a.k1 = st.k1;
   a.k2 = st.k2;
   a.u = st.u;
   a.um = st.um;
   a.up = st.up;
   a.out = st.out;
   a.mu2 = st.mu2;
   a.la2 = st.la2;
   a.rho = st.rho;
   a.ir2 = st.ir2;
   for (int q = 0; q < kWeightArrays; q++) {
      a.w2[q] = st.w2[q];
   }
   a.sx = st.st[0];
   a.sy = st.st[1];
   a.sz = st.st[2];
   for (int q = 0; q < 3; q++) {
      a.dc[q] = st.dc[q];
      a.co[q] = st.co[q];
   }
   if (st.corrector < 0 || st.corrector > 2) return kBadArgument;
   const double coef = st.coef != 0 ? st.coef : (st.corrector == 1 ? st.dt * st.dt / 12 : st.dt * st.dt);
   const double K = coef / (144 * st.h * st.h);
   a.Kh = (float)K;
   a.Kl = (float)(K - (double)a.Kh);
   a.beta = (float)st.beta;
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3, nk = st.k2 - st.k1 + 1;
   const int gx = blocks_for(ni, TX), gy = blocks_for(nj, TY);
   const size_t smem = smem_floats(st.corrector) * sizeof(float);
   const void* kern = st.corrector == 1   ? (const void*)mixed_stage_kernel<1>
                      : st.corrector == 2 ? (const void*)mixed_stage_kernel<2>
                                          : (const void*)mixed_stage_kernel<0>;
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kCudaError;
   static bool attr_set[3][64] = {};
   static int resident[3][64] = {};
   if (!attr_set[st.corrector][dev]) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
         return kCudaError;
      resident[st.corrector][dev] = resident_ctas(kern, NTHREADS, smem);
      attr_set[st.corrector][dev] = true;
   }
   a.kchunk = stage_kchunk((long long)gx * gy, nk, resident[st.corrector][dev], 12);
   const dim3 grid(gx, gy, (nk + a.kchunk - 1) / a.kchunk), block(TX, TY, 1);
   if (st.corrector == 1)
      mixed_stage_kernel<1><<<grid, block, smem, stream>>>(a);
   else if (st.corrector == 2)
      mixed_stage_kernel<2><<<grid, block, smem, stream>>>(a);
   else
      mixed_stage_kernel<0><<<grid, block, smem, stream>>>(a);
   return launch_status();
}

}  // namespace sw4g
