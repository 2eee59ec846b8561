// Fused stage kernels of the elastic time step on Cartesian grids, sm_103a, FP64.
//
// One launch computes, for every centred row k1..k2 of the interior,
//   predictor stage  out = 2u - um + dt^2/rho * L(u)
//   corrector stage  out = up + dt^2/12/rho * L(up - 2u + um) - beta/rho * SG(u - um)
// where L is the divergence-of-stress operator of the reference's rhs4sg
// (src/rhs4sg_rev.C:111-348) and SG its 4th-order supergrid damping
// (src/ew-cfromfort.C:952-1057).  These replace the reference's GPU phase
// sequence RHSPredCU_center / evalDpDmInTimeCU / RHSCorrCU_center /
// addSuperGridDampingCU_center (src/EW_cuda.C:1228-1509): each input field
// crosses HBM once per stage and no intermediate (Lu, Uacc, F) is written.
//
// Design for GB300's FP64 pipe, which bounds this kernel (~8 flop per byte):
//  * CTA = 32 x 8 columns; the CTA marches up z through a 5-plane ring of the
//    stage field (with a 2-point x/y halo) in shared memory.
//  * The variable-coefficient second differences use per-point weights
//    W1,W2 of mu*s and (2mu+lambda)*s that are precomputed once (material is
//    time-invariant): no FP64 work is spent rebuilding them every stage.
//  * Each mixed derivative (c f_b)_a is evaluated as an outer difference of a
//    per-point product G = c * D_b f computed once per point: G for the x (y)
//    outer difference is staged in shared memory over an x (y) halo, G for the
//    z outer difference rides a per-thread register queue.  The reference
//    recomputes the inner differences inside every outer term.
//  * The corrector stage forms (up - 2u + um) and (u - um) while staging the
//    plane; 1/dt^2 is folded into the update coefficient.
//  * A third form serves the discrete adjoint (adjoint.cu):
//      out = 2u - um + coef/rho * L(up) - beta/rho * SG(u - um)
//    (the stage field read from `up` directly).
#include <algorithm>
#include <atomic>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "stencil.cuh"

namespace sw4g {
namespace {

constexpr int TX = 32, TY = 8, HALO = 2;
constexpr int PX = TX + 2 * HALO;  // 36
constexpr int PY = TY + 2 * HALO;  // 12
constexpr int PLANE = PX * PY;     // 432
constexpr int NTHREADS = TX * TY;

struct FusedArgs {
   int ib, ie, jb, je, kb, ke;
   long long ni, nij, npts;
   int k1, k2, kchunk;
   const double* __restrict__ u;
   const double* __restrict__ um;
   const double* __restrict__ up;  // corrector input (predicted level)
   double* __restrict__ out;
   const double* __restrict__ mu;
   const double* __restrict__ la;
   const double* __restrict__ rho;
   const double* __restrict__ irho;
   const double* __restrict__ w[kWeightArrays];
   const double* __restrict__ ws[kWeightSums];
   const double* __restrict__ sx;
   const double* __restrict__ sy;
   const double* __restrict__ sz;
   const double* __restrict__ dc[3];
   const double* __restrict__ co[3];
   double cof144;  // 1/(144 h^2)
   double coef;    // dt^2 (predictor) or dt^2/12 (corrector)
   double beta;    // supergrid damping coefficient (corrector)
   int* emax;      // if set: atomicMax of the FP64 exponent fields written (corrector)
};

__host__ __device__ constexpr int smem_doubles(int corr)
{
   // V ring (5 planes x 3) + [D ring (3 planes x 3) + RHO plane] + MU, LA planes + GX + GY
   return 15 * PLANE + (corr ? 9 * PLANE + PLANE : 0) + 2 * PLANE + 3 * TY * PX + 3 * PY * TX;
}

// CORR: 0 predictor, 1 corrector, 2 adjoint stage (see the header)

__device__ __forceinline__ int mod5(int k) { return ((k % 5) + 5) % 5; }
__device__ __forceinline__ int mod3(int k) { return ((k % 3) + 3) % 3; }

// The centred first difference (fm2 - fp2) + 8 (fp1 - fm1) with its roundings
// spelled out, so that every copy of the code that forms it rounds alike.
__device__ __forceinline__ double d1r(double fm2, double fm1, double fp1, double fp2)
{
   return __fma_rn(8.0, __dsub_rn(fp1, fm1), __dsub_rn(fm2, fp2));
}

// x == 1.0 exactly, from the bit pattern (no FP64 instruction).
__device__ __forceinline__ bool is_one(double x)
{
   return __double_as_longlong(x) == 0x3ff0000000000000LL;
}

template <int CORR>
__global__ void __launch_bounds__(NTHREADS, 2) fused_stage_kernel(FusedArgs a)
{
   extern __shared__ double sm[];
   double* V = sm;                                   // [5 slots][3][PLANE]
   double* Dd = V + 15 * PLANE;                      // [3 slots][3][PLANE]   (corrector)
   double* RH = Dd + (CORR ? 9 * PLANE : 0);         // [PLANE]               (corrector)
   double* MU = RH + (CORR ? PLANE : 0);             // [PLANE]
   double* LA = MU + PLANE;                          // [PLANE]
   double* GX = LA + PLANE;                          // [3][TY][PX]
   double* GY = GX + 3 * TY * PX;                    // [3][PY][TX]

   const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
   const int i0 = a.ib + 2 + blockIdx.x * TX;
   const int j0 = a.jb + 2 + blockIdx.y * TY;
   const int kbeg = a.k1 + blockIdx.z * a.kchunk;
   if (kbeg > a.k2) return;
   const int kend = min(kbeg + a.kchunk - 1, a.k2);
   const int i = i0 + tx, j = j0 + ty;
   const bool active = (i <= a.ie - 2) && (j <= a.je - 2);
   const int own = (ty + HALO) * PX + (tx + HALO);
   const long long npts = a.npts;

   auto gidx = [&](int gi, int gj, int gk) -> long long {
      return (long long)(gi - a.ib) + a.ni * (gj - a.jb) + a.nij * (long long)(gk - a.kb);
   };

   // Damping (corrector and adjoint forms): an axis' term at a point is computed where
   // that axis' profile dc is nonzero at one of the point's three neighbours along the
   // axis; elsewhere it is exactly zero.  The x and y tests hold for the whole column;
   // need_d (uniform over the CTA) says whether any point of the CTA's columns and
   // planes has a term, and the damping field u - um is only formed where it does.
   bool dampx = false, dampy = false, need_d = false;
   if (CORR) {
      bool any = false;
      if (a.beta != 0) {
         if (active) {
            dampx = nonzero_bits(__ldg(a.dc[0] + (i - 1 - a.ib))) || nonzero_bits(__ldg(a.dc[0] + (i - a.ib))) ||
                    nonzero_bits(__ldg(a.dc[0] + (i + 1 - a.ib)));
            dampy = nonzero_bits(__ldg(a.dc[1] + (j - 1 - a.jb))) || nonzero_bits(__ldg(a.dc[1] + (j - a.jb))) ||
                    nonzero_bits(__ldg(a.dc[1] + (j + 1 - a.jb)));
         }
         any = dampx || dampy;
         for (int kk = kbeg - 1 + tid; kk <= kend + 1; kk += NTHREADS)
            any = any || nonzero_bits(__ldg(a.dc[2] + (kk - a.kb)));
      }
      need_d = __syncthreads_or(any) != 0;
   }

   // Stage plane kk (with halo) of the stage field, and for the corrector the
   // damping field u - um.  Points beyond the array edge are never read by an
   // active column and are zero-filled.
   auto load_plane = [&](int kk) {
      double* vs = V + mod5(kk) * 3 * PLANE;
      double* ds = Dd + mod3(kk) * 3 * PLANE;
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int li = idx % PX, lj = idx / PX;
         const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
         double v[3] = {0, 0, 0}, d[3] = {0, 0, 0};
         if (gi <= a.ie && gj <= a.je) {
            const long long p = gidx(gi, gj, kk);
#pragma unroll
            for (int c = 0; c < 3; c++) {
               if (CORR == 0) {
                  v[c] = __ldg(a.u + p + c * npts);
               } else if (CORR == 1) {
                  const double uu = __ldg(a.u + p + c * npts), uum = __ldg(a.um + p + c * npts);
                  v[c] = (__ldg(a.up + p + c * npts) - 2 * uu) + uum;
                  if (need_d) d[c] = uu - uum;
               } else {
                  v[c] = __ldg(a.up + p + c * npts);
                  if (need_d) d[c] = __ldg(a.u + p + c * npts) - __ldg(a.um + p + c * npts);
               }
            }
         }
#pragma unroll
         for (int c = 0; c < 3; c++) {
            vs[c * PLANE + idx] = v[c];
            if (CORR && need_d) ds[c * PLANE + idx] = d[c];
         }
      }
   };

   auto load_material = [&](int kk) {
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
         const int li = idx % PX, lj = idx / PX;
         const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
         double m = 0, l = 0, r = 0;
         if (gi <= a.ie && gj <= a.je) {
            const long long p = gidx(gi, gj, kk);
            m = __ldg(a.mu + p);
            l = __ldg(a.la + p);
            if (CORR) r = __ldg(a.rho + p);
         }
         MU[idx] = m;
         LA[idx] = l;
         if (CORR) RH[idx] = r;
      }
   };

   // The next plane (the stage field, and the corrector's u - um) and the next material
   // plane are loaded into registers before the current plane's arithmetic and stored
   // at the start of the next iteration, so their global-load latency overlaps the
   // arithmetic.  The corrector and adjoint forms spill a little to fit this in the
   // 128 registers of 2 CTAs per SM; measured a small net gain.
   constexpr int kPre = (PLANE + NTHREADS - 1) / NTHREADS;  // values per thread
   double pv[kPre][3], pm[kPre][2], pd[kPre][3];
   auto prefetch_plane = [&](int kk) {
      if (CORR == 0 || need_d) {
#pragma unroll
         for (int r = 0; r < kPre; r++) {
            const int idx = tid + r * NTHREADS;
            const int li = idx % PX, lj = idx / PX;
            const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
            const bool ok = idx < PLANE && gi <= a.ie && gj <= a.je;
            const long long p = ok ? gidx(gi, gj, kk) : 0;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               if (CORR == 0) {
                  pv[r][c] = ok ? __ldg(a.u + p + c * npts) : 0.0;
               } else {
                  const double uu = ok ? __ldg(a.u + p + c * npts) : 0.0, uum = ok ? __ldg(a.um + p + c * npts) : 0.0;
                  const double upp = ok ? __ldg(a.up + p + c * npts) : 0.0;
                  pv[r][c] = CORR == 1 ? (upp - 2 * uu) + uum : upp;
                  pd[r][c] = uu - uum;
               }
            }
         }
      } else {  // no damping in this CTA: the stage field alone
#pragma unroll
         for (int r = 0; r < kPre; r++) {
            const int idx = tid + r * NTHREADS;
            const int li = idx % PX, lj = idx / PX;
            const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
            const bool ok = idx < PLANE && gi <= a.ie && gj <= a.je;
            const long long p = ok ? gidx(gi, gj, kk) : 0;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const double upp = ok ? __ldg(a.up + p + c * npts) : 0.0;
               if (CORR == 1) {
                  const double uu = ok ? __ldg(a.u + p + c * npts) : 0.0, uum = ok ? __ldg(a.um + p + c * npts) : 0.0;
                  pv[r][c] = (upp - 2 * uu) + uum;
               } else {
                  pv[r][c] = upp;
               }
            }
         }
      }
   };
   auto store_plane = [&](int kk) {
      double* vs = V + mod5(kk) * 3 * PLANE;
      double* ds = Dd + mod3(kk) * 3 * PLANE;
#pragma unroll
      for (int r = 0; r < kPre; r++) {
         const int idx = tid + r * NTHREADS;
         if (idx < PLANE)
#pragma unroll
            for (int c = 0; c < 3; c++) {
               vs[c * PLANE + idx] = pv[r][c];
               if (CORR && need_d) ds[c * PLANE + idx] = pd[r][c];
            }
      }
   };
   auto prefetch_material = [&](int kk) {
#pragma unroll
      for (int r = 0; r < kPre; r++) {
         const int idx = tid + r * NTHREADS;
         const int li = idx % PX, lj = idx / PX;
         const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
         const bool ok = idx < PLANE && gi <= a.ie && gj <= a.je;
         const long long p = ok ? gidx(gi, gj, kk) : 0;
         pm[r][0] = ok ? __ldg(a.mu + p) : 0.0;
         pm[r][1] = ok ? __ldg(a.la + p) : 0.0;
      }
   };
   double prh[kPre];
   auto prefetch_rho = [&](int kk) {
#pragma unroll
      for (int r = 0; r < kPre; r++) {
         const int idx = tid + r * NTHREADS;
         const int li = idx % PX, lj = idx / PX;
         const int gi = i0 - HALO + li, gj = j0 - HALO + lj;
         const bool ok = idx < PLANE && gi <= a.ie && gj <= a.je;
         prh[r] = ok ? __ldg(a.rho + gidx(gi, gj, kk)) : 0.0;
      }
   };
   auto store_material = [&]() {
#pragma unroll
      for (int r = 0; r < kPre; r++) {
         const int idx = tid + r * NTHREADS;
         if (idx < PLANE) {
            MU[idx] = pm[r][0];
            LA[idx] = pm[r][1];
            if (CORR) RH[idx] = prh[r];
         }
      }
   };

   // Own-column stretching factors
   const double sxi = active ? __ldg(a.sx + (i - a.ib)) : 0.0;
   const double syj = active ? __ldg(a.sy + (j - a.jb)) : 0.0;

   // Away from the supergrid layers the stretching is exactly 1.  xu (yu): every
   // active column (row) of the CTA has s_x = 1 (s_y = 1); zu, per plane, s_z = 1.
   // Where they hold, the mixed-derivative products skip their multiplications by
   // the stretching.  Both forms round alike (x * 1 = x, fma(1, a, b) = a + b), so
   // the result does not depend on which form a CTA takes.
   bool xu, yu;
   {
      bool okx = true, oky = true;
      if (tid < TX && i0 + tid <= a.ie - 2) okx = is_one(__ldg(a.sx + (i0 + tid - a.ib)));
      if (tid < TY && j0 + tid <= a.je - 2) oky = is_one(__ldg(a.sy + (j0 + tid - a.jb)));
      xu = __syncthreads_and(okx) != 0;
      yu = __syncthreads_and(oky) != 0;
   }

   // z-outer products G_z at plane kk for the own column: components for
   // (mu w_x)_z, (mu w_y)_z and (lambda (u_x, v_y))_z.
   auto compute_gz = [&](int kk, double g[3]) {
      const double* vs = V + mod5(kk) * 3 * PLANE;
      const double* vu = vs;
      const double* vv = vs + PLANE;
      const double* vw = vs + 2 * PLANE;
      const double dxw = d1r(vw[own - 2], vw[own - 1], vw[own + 1], vw[own + 2]);
      const double dyw = d1r(vw[own - 2 * PX], vw[own - PX], vw[own + PX], vw[own + 2 * PX]);
      const double dxu = d1r(vu[own - 2], vu[own - 1], vu[own + 1], vu[own + 2]);
      const double dyv = d1r(vv[own - 2 * PX], vv[own - PX], vv[own + PX], vv[own + 2 * PX]);
      const long long p = gidx(i, j, kk);
      const double m = __ldg(a.mu + p), l = __ldg(a.la + p);
      if (xu && yu) {
         g[0] = __dmul_rn(m, dxw);
         g[1] = __dmul_rn(m, dyw);
         g[2] = __dmul_rn(l, __dadd_rn(dxu, dyv));
      } else {
         g[0] = __dmul_rn(__dmul_rn(m, sxi), dxw);
         g[1] = __dmul_rn(__dmul_rn(m, syj), dyw);
         g[2] = __dmul_rn(l, __fma_rn(sxi, dxu, __dmul_rn(syj, dyv)));
      }
   };

   double gz[5][3];   // G_z at planes k-2..k+2
   double dq[5][3];   // (u - um) own column at planes k-2..k+2 (corrector)

   // ---- prologue: planes kbeg-2 .. kbeg+1 ----
   for (int kk = kbeg - 2; kk <= kbeg; kk++) load_plane(kk);
   __syncthreads();
   for (int kk = kbeg - 2; kk <= kbeg; kk++) {
      const int q = kk - kbeg + 3;  // 1..3
      if (active) compute_gz(kk, gz[q]);
      if (CORR && need_d) {
         const double* ds = Dd + mod3(kk) * 3 * PLANE;
#pragma unroll
         for (int c = 0; c < 3; c++) dq[q][c] = ds[c * PLANE + own];
      }
   }
   __syncthreads();
   load_plane(kbeg + 1);
   __syncthreads();
   if (active) compute_gz(kbeg + 1, gz[4]);
   if (CORR && need_d) {
      const double* ds = Dd + mod3(kbeg + 1) * 3 * PLANE;
#pragma unroll
      for (int c = 0; c < 3; c++) dq[4][c] = ds[c * PLANE + own];
   }

   int em = 0;  // the largest exponent field written (a.emax)
   prefetch_plane(kbeg + 2);
   prefetch_material(kbeg);
   if (CORR) prefetch_rho(kbeg);
   for (int k = kbeg; k <= kend; k++) {
      store_plane(k + 2);
      store_material();
      __syncthreads();
      // planes up to kend + 2 are read (kend + 2 <= the last array plane)
      if (k < kend) {
         prefetch_plane(k + 3);
         prefetch_material(k + 1);
         if (CORR) prefetch_rho(k + 1);
      }

      // shift the register queues and append plane k+2
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
         for (int c = 0; c < 3; c++) {
            gz[q][c] = gz[q + 1][c];
            if (CORR) dq[q][c] = dq[q + 1][c];
         }
      if (active) compute_gz(k + 2, gz[4]);
      if (CORR && need_d) {
         const double* ds = Dd + mod3(k + 2) * 3 * PLANE;
#pragma unroll
         for (int c = 0; c < 3; c++) dq[4][c] = ds[c * PLANE + own];
      }

      const double szk = __ldg(a.sz + (k - a.kb));
      const bool zu = is_one(szk);
      const double* vm2 = V + mod5(k - 2) * 3 * PLANE;
      const double* vm1 = V + mod5(k - 1) * 3 * PLANE;
      const double* v0 = V + mod5(k) * 3 * PLANE;
      const double* vp1 = V + mod5(k + 1) * 3 * PLANE;
      const double* vp2 = V + mod5(k + 2) * 3 * PLANE;
      auto dz = [&](int c, int idx) {
         return d1r(vm2[c * PLANE + idx], vm1[c * PLANE + idx], vp1[c * PLANE + idx],
                    vp2[c * PLANE + idx]);
      };

      // x-outer products over the x-extended rows (all 36 columns, own 8 rows):
      //   G_x = { la (s_y v_y + s_z w_z),  mu s_y u_y,  mu s_z u_z }
      // (unit: s_y = s_z = 1 on the rows whose products are used)
      auto gx_products = [&](auto unit) {
         constexpr bool U = decltype(unit)::value;
         for (int idx = tid; idx < TY * PX; idx += NTHREADS) {
            const int li = idx % PX, ljr = idx / PX;
            const int s = (ljr + HALO) * PX + li;
            const int gi = i0 - HALO + li, gj = j0 + ljr;
            double g0 = 0, g1 = 0, g2 = 0;
            if (gi <= a.ie && gj <= a.je) {
               const double* vu = v0;
               const double* vv = v0 + PLANE;
               const double dyv = d1r(vv[s - 2 * PX], vv[s - PX], vv[s + PX], vv[s + 2 * PX]);
               const double dyu = d1r(vu[s - 2 * PX], vu[s - PX], vu[s + PX], vu[s + 2 * PX]);
               const double dzw = dz(2, s), dzu = dz(0, s);
               const double m = MU[s], l = LA[s];
               if (U) {
                  g0 = __dmul_rn(l, __dadd_rn(dyv, dzw));
                  g1 = __dmul_rn(m, dyu);
                  g2 = __dmul_rn(m, dzu);
               } else {
                  const double syy = __ldg(a.sy + (gj - a.jb));
                  g0 = __dmul_rn(l, __fma_rn(syy, dyv, __dmul_rn(szk, dzw)));
                  g1 = __dmul_rn(__dmul_rn(m, syy), dyu);
                  g2 = __dmul_rn(__dmul_rn(m, szk), dzu);
               }
            }
            GX[0 * TY * PX + idx] = g0;
            GX[1 * TY * PX + idx] = g1;
            GX[2 * TY * PX + idx] = g2;
         }
      };
      // y-outer products over the y-extended columns (own 32 columns, all 12 rows):
      //   G_y = { mu s_x v_x,  la (s_x u_x + s_z w_z),  mu s_z v_z }
      // (unit: s_x = s_z = 1 on the columns whose products are used)
      auto gy_products = [&](auto unit) {
         constexpr bool U = decltype(unit)::value;
         for (int idx = tid; idx < PY * TX; idx += NTHREADS) {
            const int lic = idx % TX, lj = idx / TX;
            const int s = lj * PX + lic + HALO;
            const int gi = i0 + lic, gj = j0 - HALO + lj;
            double g0 = 0, g1 = 0, g2 = 0;
            if (gi <= a.ie && gj <= a.je) {
               const double* vu = v0;
               const double* vv = v0 + PLANE;
               const double dxv = d1r(vv[s - 2], vv[s - 1], vv[s + 1], vv[s + 2]);
               const double dxu = d1r(vu[s - 2], vu[s - 1], vu[s + 1], vu[s + 2]);
               const double dzw = dz(2, s), dzv = dz(1, s);
               const double m = MU[s], l = LA[s];
               if (U) {
                  g0 = __dmul_rn(m, dxv);
                  g1 = __dmul_rn(l, __dadd_rn(dxu, dzw));
                  g2 = __dmul_rn(m, dzv);
               } else {
                  const double sxx = __ldg(a.sx + (gi - a.ib));
                  g0 = __dmul_rn(__dmul_rn(m, sxx), dxv);
                  g1 = __dmul_rn(l, __fma_rn(sxx, dxu, __dmul_rn(szk, dzw)));
                  g2 = __dmul_rn(__dmul_rn(m, szk), dzv);
               }
            }
            GY[0 * PY * TX + idx] = g0;
            GY[1 * PY * TX + idx] = g1;
            GY[2 * PY * TX + idx] = g2;
         }
      };
      if (yu && zu)
         gx_products(std::true_type{});
      else
         gx_products(std::false_type{});
      if (xu && zu)
         gy_products(std::true_type{});
      else
         gy_products(std::false_type{});
      __syncthreads();

      if (active) {
         const long long p = gidx(i, j, k);
         double lu[3];
         // variable-coefficient second differences with precomputed weights
         {
            const long long off[3] = {1, a.ni, a.nij};
            const double sc[3] = {sxi, syj, szk};
            const bool one[3] = {is_one(sxi), is_one(syj), zu};
            double acc[3] = {0, 0, 0};
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
               const long long o = off[ax];
               double wt[2][5];
#pragma unroll
               for (int t = 0; t < 2; t++) {
                  const double* w1 = a.w[ax * 4 + t * 2 + 0];
                  const double* w2 = a.w[ax * 4 + t * 2 + 1];
                  wt[t][0] = __ldg(w1 + p);
                  wt[t][1] = __ldg(w2 + p);
                  wt[t][2] = __ldg(w2 + p + o);
                  wt[t][3] = __ldg(w1 + p + 2 * o);
                  wt[t][4] = __ldg(a.ws[ax * 2 + t] + p);
               }
               auto second_differences = [&](auto unit) {
                  constexpr bool U = decltype(unit)::value;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     double f[5];
                     if (ax == 0) {
#pragma unroll
                        for (int m = -2; m <= 2; m++) f[m + 2] = v0[c * PLANE + own + m];
                     } else if (ax == 1) {
#pragma unroll
                        for (int m = -2; m <= 2; m++) f[m + 2] = v0[c * PLANE + own + m * PX];
                     } else {
                        f[0] = vm2[c * PLANE + own];
                        f[1] = vm1[c * PLANE + own];
                        f[2] = v0[c * PLANE + own];
                        f[3] = vp1[c * PLANE + own];
                        f[4] = vp2[c * PLANE + own];
                     }
                     // sum_m W_m (f_m - f_0) as sum_m W_m f_m - (sum_m W_m) f_0: five FMAs
                     // instead of four subtractions and four products
                     const double* wv = wt[ax == c ? 1 : 0];
                     if (U) {  // s = 1: the terms join the running sum, one FMA fewer
                        acc[c] = __fma_rn(-wv[4], f[2], __fma_rn(wv[3], f[4], __fma_rn(wv[2], f[3],
                                 __fma_rn(wv[1], f[1], __fma_rn(wv[0], f[0], acc[c])))));
                     } else {
                        const double s = fma(-wv[4], f[2], fma(wv[3], f[4], fma(wv[2], f[3],
                                                                              fma(wv[1], f[1], wv[0] * f[0]))));
                        acc[c] += sc[ax] * s;
                     }
                  }
               };
               // per point (not per CTA: the two forms round differently), so a point's
               // result does not depend on the tiling; predictor form only: the corrector
               // and adjoint forms sit at the register cap, where the second code path
               // costs more in spills than the FMA it saves
               if (CORR == 0 && one[ax])
                  second_differences(std::true_type{});
               else
                  second_differences(std::false_type{});
            }
            // mixed terms: outer differences of the staged products
            auto mixed_terms = [&](auto unit) {
               constexpr bool U = decltype(unit)::value;
#pragma unroll
               for (int c = 0; c < 3; c++) {
                  const double* gx = GX + c * TY * PX + ty * PX + tx;  // li = tx .. tx+4
                  const double* gy = GY + c * PY * TX + ty * TX + tx;  // lj = ty .. ty+4
                  const double cx = d1r(gx[0], gx[1], gx[3], gx[4]);
                  const double cy = d1r(gy[0], gy[TX], gy[3 * TX], gy[4 * TX]);
                  const double cz = d1r(gz[0][c], gz[1][c], gz[3][c], gz[4][c]);
                  const double t = U ? __dadd_rn(cx, __dadd_rn(cy, cz))
                                     : __fma_rn(sxi, cx, __fma_rn(syj, cy, __dmul_rn(szk, cz)));
                  lu[c] = __fma_rn(a.cof144, t, acc[c]);
               }
            };
            if (xu && yu && zu)
               mixed_terms(std::true_type{});
            else
               mixed_terms(std::false_type{});
         }
         const double ir = __ldg(a.irho + p);
         const double cr = a.coef * ir;
         if (!CORR) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * npts;
               a.out[q] = 2 * v0[c * PLANE + own] - __ldg(a.um + q) + cr * lu[c];
            }
         } else {
            double sg[3] = {0, 0, 0};
            // z: dc at k-1..k+1 (uniform over the CTA); x, y: the column's flags
            const bool dampz = need_d && (nonzero_bits(__ldg(a.dc[2] + (k - 1 - a.kb))) ||
                                          nonzero_bits(__ldg(a.dc[2] + (k - a.kb))) ||
                                          nonzero_bits(__ldg(a.dc[2] + (k + 1 - a.kb))));
            if (dampx || dampy || dampz) {
               const double* ds = Dd + mod3(k) * 3 * PLANE;
               const double cxi = __ldg(a.co[0] + (i - a.ib));
               const double cyj = __ldg(a.co[1] + (j - a.jb));
               const double czk = __ldg(a.co[2] + (k - a.kb));
               // x: e = rho*dc at i-1..i+1 (skipped where dc vanishes: the term is exactly 0)
               if (dampx) {
                  const double dx0 = __ldg(a.dc[0] + (i - 1 - a.ib)), dx1 = __ldg(a.dc[0] + (i - a.ib)),
                               dx2 = __ldg(a.dc[0] + (i + 1 - a.ib));
                  const double e0 = RH[own - 1] * dx0, e1 = RH[own] * dx1, e2 = RH[own + 1] * dx2;
                  const double wx = sxi * cyj * czk;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const double* d = ds + c * PLANE + own;
                     const double s = e2 * (d[2] - 2 * d[1] + d[0]) - 2 * e1 * (d[1] - 2 * d[0] + d[-1]) +
                                      e0 * (d[0] - 2 * d[-1] + d[-2]);
                     sg[c] += wx * s;
                  }
               }
               if (dampy) {
                  const double dy0 = __ldg(a.dc[1] + (j - 1 - a.jb)), dy1 = __ldg(a.dc[1] + (j - a.jb)),
                               dy2 = __ldg(a.dc[1] + (j + 1 - a.jb));
                  const double e0 = RH[own - PX] * dy0, e1 = RH[own] * dy1, e2 = RH[own + PX] * dy2;
                  const double wy = syj * cxi * czk;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const double* d = ds + c * PLANE + own;
                     const double s = e2 * (d[2 * PX] - 2 * d[PX] + d[0]) -
                                      2 * e1 * (d[PX] - 2 * d[0] + d[-PX]) +
                                      e0 * (d[0] - 2 * d[-PX] + d[-2 * PX]);
                     sg[c] += wy * s;
                  }
               }
               if (dampz) {
                  const double dz0 = __ldg(a.dc[2] + (k - 1 - a.kb)), dz1 = __ldg(a.dc[2] + (k - a.kb)),
                               dz2 = __ldg(a.dc[2] + (k + 1 - a.kb));
                  const double e0 = __ldg(a.rho + p - a.nij) * dz0, e1 = RH[own] * dz1,
                               e2 = __ldg(a.rho + p + a.nij) * dz2;
                  const double wz = szk * cxi * cyj;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const double s = e2 * (dq[4][c] - 2 * dq[3][c] + dq[2][c]) -
                                      2 * e1 * (dq[3][c] - 2 * dq[2][c] + dq[1][c]) +
                                      e0 * (dq[2][c] - 2 * dq[1][c] + dq[0][c]);
                     sg[c] += wz * s;
                  }
               }
            }
            const double birho = a.beta * ir;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * npts;
               const double v = CORR == 1 ? (__ldg(a.up + q) + cr * lu[c]) - birho * sg[c]
                                          : (2 * __ldg(a.u + q) - __ldg(a.um + q) + cr * lu[c]) - birho * sg[c];
               a.out[q] = v;
               em = max(em, (__double2hiint(v) >> 20) & 0x7ff);
            }
         }
      }
      __syncthreads();
   }
   if (a.emax) {  // uniform: every thread of a running CTA gets here
      em = __reduce_max_sync(0xffffffffu, em);
      if ((threadIdx.x & 31) == 0 && em > 0) atomicMax(a.emax, em);
   }
}

// Weights of the variable-coefficient second difference (src/rhs4sg_rev.C:114-136)
// along each axis, for coefficient mu*s (type 0) and (2mu+lambda)*s (type 1):
//   W1(q) = a(q-1) - 3/4 (a(q) + a(q-2))           (pair q-2, q)
//   W2(q) = a(q-2) + a(q+1) + 3 (a(q) + a(q-1))     (pair q-1, q)
// scaled by 1/(6 h^2); the operator at q uses W1(q), W2(q), W2(q+1), W1(q+2).
__global__ void weights_kernel(Box b, const double* __restrict__ mu, const double* __restrict__ la,
                               const double* __restrict__ sx, const double* __restrict__ sy,
                               const double* __restrict__ sz, double scale, WeightPtrs w)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(p % b.ni);
      const int j = b.jb + (int)((p / b.ni) % (b.je - b.jb + 1));
      const int k = b.kb + (int)(p / b.nij);
      const int qv[3] = {i, j, k}, lo[3] = {b.ib, b.jb, b.kb}, hi[3] = {b.ie, b.je, b.ke};
      const long long st[3] = {1, b.ni, b.nij};
      const double* sv[3] = {sx, sy, sz};
#pragma unroll
      for (int ax = 0; ax < 3; ax++) {
         double w1[2] = {0, 0}, w2[2] = {0, 0};
         const int q = qv[ax];
         if (q - 2 >= lo[ax]) {
            double am[2][4];  // offsets -2..+1
            for (int m = -2; m <= 1; m++) {
               if (q + m > hi[ax]) {
                  am[0][m + 2] = am[1][m + 2] = 0;
                  continue;
               }
               const long long pm = p + m * st[ax];
               const double s = sv[ax][q + m - lo[ax]];
               am[0][m + 2] = mu[pm] * s;
               am[1][m + 2] = (2 * mu[pm] + la[pm]) * s;
            }
            for (int t = 0; t < 2; t++) {
               w1[t] = am[t][1] - 0.75 * (am[t][2] + am[t][0]);
               if (q + 1 <= hi[ax]) w2[t] = am[t][0] + am[t][3] + 3 * (am[t][2] + am[t][1]);
            }
         }
         for (int t = 0; t < 2; t++) {
            w.p[ax * 4 + t * 2 + 0][p] = scale * w1[t];
            w.p[ax * 4 + t * 2 + 1][p] = scale * w2[t];
         }
      }
   }
}

__global__ void inverse_kernel(long long n, const double* __restrict__ x, double* __restrict__ y)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
        p += (long long)gridDim.x * blockDim.x)
      y[p] = 1.0 / x[p];
}

// (up - 2u + um) on a slab of planes [k0, k1] into a compact scratch array.
__global__ void uacc_slab_kernel(Box b, int k0, int k1, const double* __restrict__ up,
                                 const double* __restrict__ u, const double* __restrict__ um,
                                 double* __restrict__ out)
{
   const long long nslab = b.nij * (k1 - k0 + 1);
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < 3 * nslab;
        q += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(q / nslab);
      const long long r = q % nslab;
      const long long p = r + b.nij * (long long)(k0 - b.kb) + c * b.npts;
      out[q] = (up[p] - 2 * u[p]) + um[p];
   }
}

// Same for double-float levels (the slab itself is FP64).
__global__ void uacc_slab_df_kernel(Box b, int k0, int k1, DFField up, DFField u, DFField um,
                                    double* __restrict__ out)
{
   const long long nslab = b.nij * (k1 - k0 + 1);
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < 3 * nslab;
        q += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(q / nslab);
      const long long r = q % nslab;
      const long long p = r + b.nij * (long long)(k0 - b.kb) + c * b.npts;
      out[q] = (up.get(p) - 2 * u.get(p)) + um.get(p);
   }
}

// out = a (- b) in FP64 over planes k0..k1 of double-float levels (a
// component-major slab of 3 x nij x (k1 - k0 + 1) values)
__global__ void df_slab_kernel(Box bx, int k0, int k1, const float* __restrict__ a,
                               const float* __restrict__ bsub, double* __restrict__ out)
{
   const long long nslab = bx.nij * (k1 - k0 + 1), lo = 3 * bx.npts;
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < 3 * nslab;
        q += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(q / nslab);
      const long long p = q % nslab + bx.nij * (long long)(k0 - bx.kb) + c * bx.npts;
      double v = (double)a[p] + (double)a[p + lo];
      if (bsub) v -= (double)bsub[p] + (double)bsub[p + lo];
      out[q] = v;
   }
}

// Sums of the four weights each point's second difference applies along each axis
// (WeightPtrs::s); zero where the stencil would leave the array (never a stage point).
__global__ void weight_sums_kernel(Box b, WeightPtrs w)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      const int i = b.ib + (int)(p % b.ni);
      const int j = b.jb + (int)((p / b.ni) % (b.je - b.jb + 1));
      const int k = b.kb + (int)(p / b.nij);
      const int qv[3] = {i, j, k}, hi[3] = {b.ie, b.je, b.ke};
      const long long st[3] = {1, b.ni, b.nij};
#pragma unroll
      for (int ax = 0; ax < 3; ax++)
#pragma unroll
         for (int t = 0; t < 2; t++) {
            double s = 0;
            if (qv[ax] + 2 <= hi[ax]) {
               const double* w1 = w.p[ax * 4 + t * 2];
               const double* w2 = w.p[ax * 4 + t * 2 + 1];
               s = w1[p] + w2[p] + w2[p + st[ax]] + w1[p + 2 * st[ax]];
            }
            w.s[ax * 2 + t][p] = s;
         }
   }
}

int grid_stride_blocks(long long n)
{
   long long g = (n + 255) / 256;
   return (int)std::min<long long>(std::max<long long>(g, 1), 152LL * 16);
}

}  // namespace

int launch_weights_only(const Box& b, const double* mu, const double* la, const double* sx,
                        const double* sy, const double* sz, double h, WeightPtrs w, cudaStream_t s);

int launch_weights(const Box& b, const double* mu, const double* la, const double* sx,
                   const double* sy, const double* sz, double h, WeightPtrs w, cudaStream_t s)
{
   SW4G_TRY(launch_weights_only(b, mu, la, sx, sy, sz, h, w, s));
   weight_sums_kernel<<<grid_stride_blocks(b.npts), 256, 0, s>>>(b, w);
   return launch_status();
}

int launch_weights_only(const Box& b, const double* mu, const double* la, const double* sx,
                        const double* sy, const double* sz, double h, WeightPtrs w, cudaStream_t s)
{
   weights_kernel<<<grid_stride_blocks(b.npts), 256, 0, s>>>(b, mu, la, sx, sy, sz,
                                                             1.0 / (6 * h * h), w);
   return launch_status();
}

int launch_inverse(long long n, const double* x, double* y, cudaStream_t s)
{
   inverse_kernel<<<grid_stride_blocks(n), 256, 0, s>>>(n, x, y);
   return launch_status();
}

int launch_uacc_slab(const Box& b, int k0, int k1, const double* up, const double* u,
                     const double* um, double* out, cudaStream_t s)
{
   const long long n = 3 * b.nij * (k1 - k0 + 1);
   uacc_slab_kernel<<<grid_stride_blocks(n), 256, 0, s>>>(b, k0, k1, up, u, um, out);
   return launch_status();
}

int launch_df_slab(const Box& b, int k0, int k1, const float* a, const float* bsub, double* out,
                   cudaStream_t s)
{
   const long long n = 3 * b.nij * (k1 - k0 + 1);
   df_slab_kernel<<<grid_stride_blocks(n), 256, 0, s>>>(b, k0, k1, a, bsub, out);
   return launch_status();
}

int launch_uacc_slab_df(const Box& b, int k0, int k1, const float* up, const float* u,
                        const float* um, double* out, cudaStream_t s)
{
   const long long n = 3 * b.nij * (k1 - k0 + 1), lo = 3 * b.npts;
   uacc_slab_df_kernel<<<grid_stride_blocks(n), 256, 0, s>>>(
       b, k0, k1, DFField{const_cast<float*>(up), lo}, DFField{const_cast<float*>(u), lo},
       DFField{const_cast<float*>(um), lo}, out);
   return launch_status();
}

namespace {
std::atomic<int> g_stage_chunks{0};
}

int stage_chunks_override() { return g_stage_chunks.load(std::memory_order_relaxed); }
void set_stage_chunks_override(int chunks) { g_stage_chunks.store(chunks > 0 ? chunks : 0); }

int resident_ctas(const void* kernel, int threads, size_t smem)
{
   int n = 0;
   if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) {
      cudaGetLastError();
      return 1;
   }
   return n > 0 ? n : 1;
}

int stage_kchunk(long long cols, int nk, int resident, int min_planes)
{
   if (nk < 1) return 1;
   int sms = 0, dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
       sms < 1) {
      cudaGetLastError();
      sms = 152;
   }
   const long long slots = (long long)sms * std::max(1, resident);
   const int forced = stage_chunks_override();
   int chunks = 1;
   if (forced > 0) {
      chunks = std::min(forced, nk);
   } else {
      // among the counts that give at least 3.5 waves (fewer, longer CTAs measured
      // slower on the topography grids); the most chunks if none does
      const int most = std::max(1, nk / std::max(1, min_planes));
      double best = -1;
      chunks = most;
      for (int c = 1; c <= most; c++) {
         const int per = (nk + c - 1) / c;
         const long long ctas = cols * (long long)((nk + per - 1) / per);
         if (2 * ctas < 7 * slots) continue;
         const double cost = (double)((ctas + slots - 1) / slots) * (per + 2);
         if (best < 0 || cost < best * 0.999) {
            best = cost;
            chunks = c;
         }
      }
   }
   return (nk + chunks - 1) / chunks;
}

int launch_fused_stage(const FusedStage& st, cudaStream_t stream)
{
   if (st.k2 < st.k1) return kOk;
   const Box& b = st.b;
   if (b.cs != b.npts) return kNotSupported;  // SoA only
   FusedArgs a;
   a.ib = b.ib; a.ie = b.ie; a.jb = b.jb; a.je = b.je; a.kb = b.kb; a.ke = b.ke;
   a.ni = b.ni; a.nij = b.nij; a.npts = b.npts;
   a.k1 = st.k1;
   a.k2 = st.k2;
   a.u = st.u;
   a.um = st.um;
   a.up = st.up;
   a.out = st.out;
   a.mu = st.mu;
   a.la = st.la;
   a.rho = st.rho;
   a.irho = st.irho;
   for (int q = 0; q < kWeightArrays; q++) a.w[q] = st.w.p[q];
   for (int q = 0; q < kWeightSums; q++) a.ws[q] = st.w.s[q];
   a.sx = st.st[0];
   a.sy = st.st[1];
   a.sz = st.st[2];
   for (int q = 0; q < 3; q++) {
      a.dc[q] = st.dc[q];
      a.co[q] = st.co[q];
   }
   a.cof144 = 1.0 / (144 * st.h * st.h);
   a.coef = st.coef > 0 ? st.coef : (st.corrector ? st.dt * st.dt / 12 : st.dt * st.dt);
   a.beta = st.beta;
   a.emax = st.emax;
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3, nk = st.k2 - st.k1 + 1;
   const int gx = blocks_for(ni, TX), gy = blocks_for(nj, TY);
   const int form = st.corrector;  // 0, 1 or 2
   if (form < 0 || form > 2) return kBadArgument;
   const size_t smem = smem_doubles(form) * sizeof(double);
   const void* kern = form == 0 ? (const void*)fused_stage_kernel<0>
                      : form == 1 ? (const void*)fused_stage_kernel<1>
                                  : (const void*)fused_stage_kernel<2>;
   // the opt-in shared-memory size is a per-device function attribute
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kCudaError;
   static bool attr_set[3][64] = {};
   static int resident[3][64] = {};
   if (!attr_set[form][dev]) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
         return kCudaError;
      resident[form][dev] = resident_ctas(kern, NTHREADS, smem);
      attr_set[form][dev] = true;
   }
   a.kchunk = st.kchunk > 0 ? st.kchunk : stage_kchunk((long long)gx * gy, nk, resident[form][dev], 12);
   const dim3 grid(gx, gy, (nk + a.kchunk - 1) / a.kchunk), block(TX, TY, 1);
   if (form == 0)
      fused_stage_kernel<0><<<grid, block, smem, stream>>>(a);
   else if (form == 1)
      fused_stage_kernel<1><<<grid, block, smem, stream>>>(a);
   else
      fused_stage_kernel<2><<<grid, block, smem, stream>>>(a);
   return launch_status();
}

}  // namespace sw4g
