// One-thread-per-point sm_103a kernels for the Cartesian operator rhs4sg:
// the centred rows and the one-sided SBP boundary rows, AoS or SoA layout.
//
// They serve the kernel-level drop-in entry point (sw4g_rhs4sg, the replacement
// for the reference's rhs4sg / rhs4sg_rev, src/EW.C:141-149) for any bounds and
// onesided flags, and are the baseline the fused z-marching stage kernels
// (stage_fused.cu) are checked against.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "sbp.h"
#include "stencil.cuh"

namespace sw4g {
namespace {

__constant__ double k_acof[384];
__constant__ double k_bope[48];
__constant__ double k_ghcof[6];

struct OpArgs {
   Box b;   // material / output box
   Box bu;  // box of the field u (equal to b except for a scratch field slab)
   const double* __restrict__ u;
   const float* __restrict__ udf;  // double-float field instead of u when set (lo at 3*npts)
   const double* __restrict__ mu;
   const double* __restrict__ la;
   const double* __restrict__ sx;
   const double* __restrict__ sy;
   const double* __restrict__ sz;
   double* __restrict__ lu;
   double cof;
   int nk;
   // optional SBP z coefficients of the one-sided rows, per column (zcoef_kernel):
   // zc[((r*8 + q)*2 + t)*nij + column], row r=0..5, point q=0..7, t 0 mu, 1 2mu+lambda
   const double* __restrict__ zc;
   // optional per-column terms of the one-sided rows (rows_pre_kernel): the one-sided z
   // derivatives dzc[((kk-1)*3 + c)*nij + column] of every column and the z-differences
   // of the centred x/y products roc[((kk-1)*4 + t)*nij + column] of interior columns
   const double* __restrict__ dzc;
   const double* __restrict__ roc;
};

template <bool DF>
struct PtT {
   const OpArgs& a;
   __device__ PtT(const OpArgs& a_) : a(a_) {}
   __device__ __forceinline__ double u(int c, int i, int j, int k) const
   {
      const long long q = cidx(a.bu, c, i, j, k);
      if (DF) return (double)__ldg(a.udf + q) + (double)__ldg(a.udf + q + 3 * a.bu.npts);
      return __ldg(a.u + q);
   }
   __device__ __forceinline__ double mu(int i, int j, int k) const
   {
      return __ldg(a.mu + pidx(a.b, i, j, k));
   }
   __device__ __forceinline__ double la(int i, int j, int k) const
   {
      return __ldg(a.la + pidx(a.b, i, j, k));
   }
   __device__ __forceinline__ double s(int ax, int q) const
   {
      return ax == 0 ? __ldg(a.sx + q - a.b.ib) : ax == 1 ? __ldg(a.sy + q - a.b.jb)
                                                          : __ldg(a.sz + q - a.b.kb);
   }
};

using Pt = PtT<false>;

// (coef * f_ai)_ao times 144 h^2 with f = component c (src/rhs4sg_rev.C:221-347).
template <class P_>
__device__ __forceinline__ double mixed(const P_& P, bool la_coef, int ao, int ai, int c, int i,
                                        int j, int k)
{
   double s = 0;
#pragma unroll
   for (int m = -2; m <= 2; m++) {
      if (m == 0) continue;
      const int io = i + (ao == 0) * m, jo = j + (ao == 1) * m, ko = k + (ao == 2) * m;
      const int di = (ai == 0), dj = (ai == 1), dk = (ai == 2);
      const double inner =
          d1c(P.u(c, io - 2 * di, jo - 2 * dj, ko - 2 * dk), P.u(c, io - di, jo - dj, ko - dk),
              P.u(c, io + di, jo + dj, ko + dk), P.u(c, io + 2 * di, jo + 2 * dj, ko + 2 * dk));
      const double cf = la_coef ? P.la(io, jo, ko) : P.mu(io, jo, ko);
      const double w = (m == -2) ? 1.0 : (m == -1) ? -8.0 : (m == 1) ? 8.0 : -1.0;
      s += w * cf * inner;
   }
   return s;
}

// s_ax-stretched coefficient stencils along axis ax at (i,j,k): a = mu*s, b = (2mu+la)*s.
template <class P_>
__device__ __forceinline__ void coef_stencil(const P_& P, int ax, int i, int j, int k, double am[5],
                                             double bm[5])
{
#pragma unroll
   for (int m = -2; m <= 2; m++) {
      const int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m, kk = k + (ax == 2) * m;
      const double mu = P.mu(ii, jj, kk), la = P.la(ii, jj, kk);
      const double s = P.s(ax, ax == 0 ? ii : ax == 1 ? jj : kk);
      am[m + 2] = mu * s;
      bm[m + 2] = (2 * mu + la) * s;
   }
}

template <class P_>
__device__ __forceinline__ void field_stencil(const P_& P, int ax, int c, int i, int j, int k,
                                              double f[5])
{
#pragma unroll
   for (int m = -2; m <= 2; m++)
      f[m + 2] = P.u(c, i + (ax == 0) * m, j + (ax == 1) * m, k + (ax == 2) * m);
}

__global__ void __launch_bounds__(256) rhs4_center_kernel(OpArgs a, int k1)
{
   const int i = a.b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = a.b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   const int k = k1 + blockIdx.z;
   if (i > a.b.ie - 2 || j > a.b.je - 2) return;
   Pt P(a);
   const double i6 = 1.0 / 6, i144 = 1.0 / 144;
   const double sx = P.s(0, i), sy = P.s(1, j), sz = P.s(2, k);
   double am[3][5], bm[3][5];
   for (int ax = 0; ax < 3; ax++) coef_stencil(P, ax, i, j, k, am[ax], bm[ax]);
   double r[3];
   for (int c = 0; c < 3; c++) {
      double f[5], acc = 0;
      for (int ax = 0; ax < 3; ax++) {
         field_stencil(P, ax, c, i, j, k, f);
         const double sa = ax == 0 ? sx : ax == 1 ? sy : sz;
         acc += sa * d2var(ax == c ? bm[ax] : am[ax], f);
      }
      r[c] = i6 * acc;
   }
   r[0] += i144 * (sx * sy * (mixed(P, true, 0, 1, 1, i, j, k) + mixed(P, false, 1, 0, 1, i, j, k)) +
                   sx * sz * (mixed(P, true, 0, 2, 2, i, j, k) + mixed(P, false, 2, 0, 2, i, j, k)));
   r[1] += i144 * (sx * sy * (mixed(P, false, 0, 1, 0, i, j, k) + mixed(P, true, 1, 0, 0, i, j, k)) +
                   sy * sz * (mixed(P, true, 1, 2, 2, i, j, k) + mixed(P, false, 2, 1, 2, i, j, k)));
   r[2] += i144 * (sx * sz * (mixed(P, false, 0, 2, 0, i, j, k) + mixed(P, true, 2, 0, 0, i, j, k)) +
                   sy * sz * (mixed(P, false, 1, 2, 1, i, j, k) + mixed(P, true, 2, 1, 1, i, j, k)));
   for (int c = 0; c < 3; c++) a.lu[cidx(a.b, c, i, j, k)] = a.cof * r[c];
}

// One-sided rows.  Row r=0..5 is k=1+r (top) or k=nk-5+r (bottom); the SBP table
// row is kk = k (top) or nk-k+1 (bottom) and the z-stencil point q (1..8) sits at
// k=q (top) or nk-q+1 (bottom), with the first-derivative weights negated at the
// bottom (src/rhs4sg_rev.C:602-856).  strz is not applied on these rows.
// PRE: the per-column terms come from rows_pre_kernel (a.dzc, a.roc).
template <bool TOP, bool DF = false, bool PRE = false>
__device__ __forceinline__ void lu_bndry_point(const OpArgs& a, int i, int j, int k, double r[3])
{
   const int nk = a.nk;
   const int kk = TOP ? k : nk - k + 1;
   PtT<DF> P(a);
   const double i6 = 1.0 / 6, i12 = 1.0 / 12, i144 = 1.0 / 144;
   const double sx = P.s(0, i), sy = P.s(1, j);
   auto kq = [&](int q) { return TOP ? q : nk - q + 1; };  // q = 1..8
   auto wz = [&](int q) {
      const double w = k_bope[(kk - 1) + 6 * (q - 1)];
      return TOP ? w : -w;
   };

   double am[2][5], bm[2][5];
   for (int ax = 0; ax < 2; ax++) coef_stencil(P, ax, i, j, k, am[ax], bm[ax]);
   for (int c = 0; c < 3; c++) {
      double f[5], acc = 0;
      for (int ax = 0; ax < 2; ax++) {
         field_stencil(P, ax, c, i, j, k, f);
         acc += (ax == 0 ? sx : sy) * d2var(ax == c ? bm[ax] : am[ax], f);
      }
      // z: sum_q (sum_m acof(kk,q,m) coef(m)) u(q) + ghcof(kk) coef(bnd) u(ghost)
      const int t = c == 2 ? 1 : 0;
      double zz = 0;
      if (a.zc) {
         const long long col = (long long)(i - a.b.ib) + a.b.ni * (j - a.b.jb);
         const double* zr = a.zc + ((long long)(kk - 1) * 16 + t) * a.b.nij + col;
         for (int q = 1; q <= 8; q++) zz += __ldg(zr + (long long)(q - 1) * 2 * a.b.nij) * P.u(c, i, j, kq(q));
      } else {
         double cz[8];
         for (int m = 1; m <= 8; m++) {
            const double mu = P.mu(i, j, kq(m));
            cz[m - 1] = t ? 2 * mu + P.la(i, j, kq(m)) : mu;
         }
         for (int q = 1; q <= 8; q++) {
            double cq = 0;
            for (int m = 1; m <= 8; m++) cq += k_acof[(kk - 1) + 6 * (q - 1) + 48 * (m - 1)] * cz[m - 1];
            zz += cq * P.u(c, i, j, kq(q));
         }
      }
      const double mub = P.mu(i, j, TOP ? 1 : nk);
      const double cb = t ? 2 * mub + P.la(i, j, TOP ? 1 : nk) : mub;
      zz += k_ghcof[kk - 1] * cb * P.u(c, i, j, TOP ? 0 : nk + 1);
      r[c] = i6 * acc + zz;
   }
   // centred mixed x-y terms
   r[0] += sx * sy * i144 * (mixed(P, true, 0, 1, 1, i, j, k) + mixed(P, false, 1, 0, 1, i, j, k));
   r[1] += sx * sy * i144 * (mixed(P, false, 0, 1, 0, i, j, k) + mixed(P, true, 1, 0, 0, i, j, k));

   // (coef * Dz f)_a: outer centred difference along a of a one-sided z derivative
   auto outer_of_dz = [&](bool la_coef, int ax, int c) {
      double s = 0;
      for (int m = -2; m <= 2; m++) {
         if (m == 0) continue;
         const int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m;
         double dz = 0;
         if (PRE)
            dz = __ldg(a.dzc + ((long long)(kk - 1) * 3 + c) * a.b.nij + (ii - a.b.ib) +
                       a.b.ni * (long long)(jj - a.b.jb));
         else
#pragma unroll 1
            for (int q = 1; q <= 8; q++) dz += wz(q) * P.u(c, ii, jj, kq(q));
         const double cf = la_coef ? P.la(ii, jj, k) : P.mu(ii, jj, k);
         const double w = (m == -2) ? 1.0 : (m == -1) ? -8.0 : (m == 1) ? 8.0 : -1.0;
         s += w * cf * dz;
      }
      return s * i12;
   };
   // Dz(coef * f_a): one-sided z difference of a centred derivative along a
   auto dz_of_inner = [&](bool la_coef, int ax, int c) {
      double s = 0;
      const int di = ax == 0, dj = ax == 1;
      if (PRE) {
         const int t = la_coef ? 2 + ax : ax;
         return __ldg(a.roc + ((long long)(kk - 1) * 4 + t) * a.b.nij + (i - a.b.ib) +
                      a.b.ni * (long long)(j - a.b.jb));
      }
#pragma unroll 1
      for (int q = 1; q <= 8; q++) {
         const int kz = kq(q);
         const double inner = d1c(P.u(c, i - 2 * di, j - 2 * dj, kz), P.u(c, i - di, j - dj, kz),
                                  P.u(c, i + di, j + dj, kz), P.u(c, i + 2 * di, j + 2 * dj, kz));
         const double cf = la_coef ? P.la(i, j, kz) : P.mu(i, j, kz);
         s += wz(q) * cf * inner * i12;
      }
      return s;
   };
   r[0] += sx * outer_of_dz(true, 0, 2);
   r[0] += sx * dz_of_inner(false, 0, 2);
   r[1] += sy * outer_of_dz(true, 1, 2);
   r[1] += sy * dz_of_inner(false, 1, 2);
   r[2] += sx * outer_of_dz(false, 0, 0);
   r[2] += sy * outer_of_dz(false, 1, 1);
   r[2] += sx * dz_of_inner(true, 0, 0);
   r[2] += sy * dz_of_inner(true, 1, 1);
}

// Per column, the parts of the one-sided rows that do not depend on the row's own
// x/y position: the one-sided z derivatives sum_q wz(kk,q) u_c(q) of every column
// (the outer x/y differences of the rows read them at four neighbours), and for
// interior columns the z-differences sum_q wz(kk,q) coef(q) D_a u_c(q)/12 of the four
// centred products (mu D_x w, mu D_y w, la D_x u, la D_y v) of all six rows
// (src/rhs4sg_rev.C:349-600).
template <bool TOP>
__global__ void __launch_bounds__(128) rows_pre_kernel(OpArgs a, double* __restrict__ dzc,
                                                       double* __restrict__ roc)
{
   const long long nij = a.b.nij;
   const int nk = a.nk;
   Pt P(a);
   auto kq = [&](int q) { return TOP ? q : nk - q + 1; };
   auto wz = [&](int kk, int q) {
      const double w = k_bope[(kk - 1) + 6 * (q - 1)];
      return TOP ? w : -w;
   };
   const double i12 = 1.0 / 12;
   for (long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x; col < nij;
        col += (long long)gridDim.x * blockDim.x) {
      const int i = a.b.ib + (int)(col % a.b.ni), j = a.b.jb + (int)(col / a.b.ni);
#pragma unroll
      for (int c = 0; c < 3; c++) {
         double f[8];
#pragma unroll
         for (int q = 1; q <= 8; q++) f[q - 1] = P.u(c, i, j, kq(q));
#pragma unroll
         for (int kk = 1; kk <= 6; kk++) {
            double dz = 0;
#pragma unroll
            for (int q = 1; q <= 8; q++) dz += wz(kk, q) * f[q - 1];
            dzc[((long long)(kk - 1) * 3 + c) * nij + col] = dz;
         }
      }
      if (i < a.b.ib + 2 || i > a.b.ie - 2 || j < a.b.jb + 2 || j > a.b.je - 2) continue;
      // t: 0 mu D_x w, 1 mu D_y w, 2 la D_x u, 3 la D_y v
      double acc[6][4];
#pragma unroll
      for (int kk = 0; kk < 6; kk++) acc[kk][0] = acc[kk][1] = acc[kk][2] = acc[kk][3] = 0;
#pragma unroll 1
      for (int q = 1; q <= 8; q++) {
         const int kz = kq(q);
         const double mu = P.mu(i, j, kz), la = P.la(i, j, kz);
         double g[4];
#pragma unroll
         for (int t = 0; t < 4; t++) {
            const int ax = t & 1, c = t < 2 ? 2 : ax;
            const int di = ax == 0, dj = ax == 1;
            const double inner = d1c(P.u(c, i - 2 * di, j - 2 * dj, kz), P.u(c, i - di, j - dj, kz),
                                     P.u(c, i + di, j + dj, kz), P.u(c, i + 2 * di, j + 2 * dj, kz));
            g[t] = (t < 2 ? mu : la) * inner * i12;
         }
#pragma unroll
         for (int kk = 1; kk <= 6; kk++)
#pragma unroll
            for (int t = 0; t < 4; t++) acc[kk - 1][t] += wz(kk, q) * g[t];
      }
#pragma unroll
      for (int kk = 0; kk < 6; kk++)
#pragma unroll
         for (int t = 0; t < 4; t++) roc[((long long)kk * 4 + t) * nij + col] = acc[kk][t];
   }
}

template <bool TOP>
__global__ void __launch_bounds__(256) rhs4_bndry_kernel(OpArgs a)
{
   const int i = a.b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = a.b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   if (i > a.b.ie - 2 || j > a.b.je - 2) return;
   const int k = TOP ? 1 + (int)blockIdx.z : a.nk - 5 + (int)blockIdx.z;
   double r[3];
   lu_bndry_point<TOP>(a, i, j, k, r);
   for (int c = 0; c < 3; c++) a.lu[cidx(a.b, c, i, j, k)] = a.cof * r[c];
}

// Fused update on the one-sided rows (SoA fields):
//   predictor  out = 2u - um + dt^2/rho * L(u)
//   corrector  out = up + dt^2/12/rho * L(up - 2u + um) - beta/rho * SG(u - um)
//   adjoint    out = 2u - um + coef/rho * L(field) - beta/rho * SG(u - um)  (corrector 2,
//              the adjoint step's second stage)
// where the corrector's field (up - 2u + um) comes from a scratch slab (box a.bu)
// and SG is the 4th-order supergrid damping of src/ew-cfromfort.C:952-1057.
struct RowUpdate {
   int corrector;
   const double* __restrict__ u;
   const double* __restrict__ um;
   const double* __restrict__ up;
   double* __restrict__ out;
   // double-float levels (mixed form) used instead of the four above when set
   const float* __restrict__ udf;
   const float* __restrict__ umdf;
   const float* __restrict__ updf;
   float* __restrict__ outdf;
   long long lo;
   // optional FP64 slab of u - um (box ddb) read by the damping instead of u, um
   const double* __restrict__ dd;
   Box ddb;
   const double* __restrict__ irho;
   const double* __restrict__ rho;
   double coef;  // dt^2 (predictor) or dt^2/12 (corrector)
   double beta;
   const double* __restrict__ dc[3];
   const double* __restrict__ st[3];
   const double* __restrict__ co[3];
};

template <bool DF>
__device__ __forceinline__ double lvl(const double* d, const float* f, long long q, long long lo)
{
   if (DF) return (double)__ldg(f + q) + (double)__ldg(f + q + lo);
   return __ldg(d + q);
}

template <bool DF>
__device__ __forceinline__ double sg4_point(const Box& b, const RowUpdate& w, int c, int i, int j,
                                            int k)
{
   double tot = 0;
#pragma unroll
   for (int ax = 0; ax < 3; ax++) {
      const int di = ax == 0, dj = ax == 1, dk = ax == 2;
      double d[5];
#pragma unroll
      for (int m = -2; m <= 2; m++) {
         if (w.dd) {
            d[m + 2] = __ldg(w.dd + cidx(w.ddb, c, i + di * m, j + dj * m, k + dk * m));
            continue;
         }
         const long long q = cidx(b, c, i + di * m, j + dj * m, k + dk * m);
         d[m + 2] = lvl<DF>(w.u, w.udf, q, w.lo) - lvl<DF>(w.um, w.umdf, q, w.lo);
      }
      double e[3];
#pragma unroll
      for (int m = -1; m <= 1; m++) {
         const int ii = i + di * m, jj = j + dj * m, kk = k + dk * m;
         const int off = ax == 0 ? ii - b.ib : ax == 1 ? jj - b.jb : kk - b.kb;
         e[m + 1] = __ldg(w.rho + pidx(b, ii, jj, kk)) * __ldg(w.dc[ax] + off);
      }
      const double s = e[2] * (d[4] - 2 * d[3] + d[2]) - 2 * e[1] * (d[3] - 2 * d[2] + d[1]) +
                       e[0] * (d[2] - 2 * d[1] + d[0]);
      const double wgt = ax == 0 ? w.st[0][i - b.ib] * w.co[1][j - b.jb] * w.co[2][k - b.kb]
                       : ax == 1 ? w.st[1][j - b.jb] * w.co[0][i - b.ib] * w.co[2][k - b.kb]
                                 : w.st[2][k - b.kb] * w.co[0][i - b.ib] * w.co[1][j - b.jb];
      tot += wgt * s;
   }
   return tot;
}

// DF: the levels (and, when the stage field is not an FP64 slab, the field) are
// double-float pairs; FDF: the stage field is double-float.
// DF: the levels (and, when the stage field is not an FP64 slab, the field) are
// double-float pairs; FDF: the stage field is double-float.  The gx x gy x 6 blocks
// of 32 x 8 points are strided over by the grid (one CTA per block, or fewer CTAs,
// each taking several: a persistent grid beside a stage kernel).
template <bool TOP, bool DF, bool FDF, bool PRE>
__global__ void __launch_bounds__(256, 2) stage_rows_kernel(OpArgs a, RowUpdate w, int gx, int gy)
{
   const int nvb = gx * gy * 6;
   for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int i = a.b.ib + 2 + (vb % gx) * blockDim.x + threadIdx.x;
      const int j = a.b.jb + 2 + ((vb / gx) % gy) * blockDim.y + threadIdx.y;
      if (i > a.b.ie - 2 || j > a.b.je - 2) continue;
      const int bz = vb / (gx * gy);
      const int k = TOP ? 1 + bz : a.nk - 5 + bz;
      double r[3];
      lu_bndry_point<TOP, FDF, PRE>(a, i, j, k, r);
      const long long p = pidx(a.b, i, j, k);
      const double ir = w.irho ? __ldg(w.irho + p) : 1.0 / __ldg(w.rho + p);
      const double cr = w.coef * ir;
      const double birho = w.beta * ir;
      for (int c = 0; c < 3; c++) {
         const long long q = cidx(a.b, c, i, j, k);
         const double lu = a.cof * r[c];
         double v;
         if (w.corrector != 1)
            v = 2 * lvl<DF>(w.u, w.udf, q, w.lo) - lvl<DF>(w.um, w.umdf, q, w.lo) + cr * lu;
         else
            v = lvl<DF>(w.up, w.updf, q, w.lo) + cr * lu;
         if (w.corrector != 0 && w.beta != 0) v -= birho * sg4_point<DF>(a.b, w, c, i, j, k);
         if (DF) {
            const float hh = __double2float_rn(v);
            w.outdf[q] = hh;
            w.outdf[q + w.lo] = __double2float_rn(v - (double)hh);
         } else {
            w.out[q] = v;
         }
      }
   }
}

bool g_tables_uploaded[64] = {false};

}  // namespace

int upload_sbp_tables_direct()
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess) return kCudaError;
   if (dev < 0 || dev >= 64) return kBadArgument;
   if (g_tables_uploaded[dev]) return kOk;
   double acof[384], ghcof[6], bope[48], sbop[5];
   sbp_coefficients(acof, ghcof, bope, sbop);
   if (cudaMemcpyToSymbol(k_acof, acof, sizeof(acof)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(k_bope, bope, sizeof(bope)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(k_ghcof, ghcof, sizeof(ghcof)) != cudaSuccess) return kCudaError;
   g_tables_uploaded[dev] = true;
   return kOk;
}

int launch_rhs4sg_direct(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                         int klast, int nk, const int onesided[6], double* lu, const double* u,
                         const double* mu, const double* la, double h, const double* strx,
                         const double* stry, const double* strz, cudaStream_t stream)
{
   int st = upload_sbp_tables_direct();
   if (st != kOk) return st;
   OpArgs a;
   a.b = make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast);
   a.bu = a.b;
   a.u = u;
   a.udf = nullptr;
   a.zc = nullptr;
   a.dzc = a.roc = nullptr;
   a.mu = mu;
   a.la = la;
   a.sx = strx;
   a.sy = stry;
   a.sz = strz;
   a.lu = lu;
   a.cof = 1.0 / (h * h);
   a.nk = nk;
   const int ni = ilast - ifirst - 3, nj = jlast - jfirst - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const dim3 block(32, 8, 1);
   const int k1 = onesided[4] == 1 ? 7 : kfirst + 2;
   const int k2 = onesided[5] == 1 ? nk - 6 : klast - 2;
   if (k2 >= k1) {
      const dim3 grid(blocks_for(ni, 32), blocks_for(nj, 8), k2 - k1 + 1);
      rhs4_center_kernel<<<grid, block, 0, stream>>>(a, k1);
   }
   if (onesided[4] == 1) {
      const dim3 grid(blocks_for(ni, 32), blocks_for(nj, 8), 6);
      rhs4_bndry_kernel<true><<<grid, block, 0, stream>>>(a);
   }
   if (onesided[5] == 1) {
      const dim3 grid(blocks_for(ni, 32), blocks_for(nj, 8), 6);
      rhs4_bndry_kernel<false><<<grid, block, 0, stream>>>(a);
   }
   return launch_status();
}

int launch_stage_rows(int corrector, bool top, const Box& b, int nk, const double* field,
                      const Box& field_box, const double* mu, const double* la, double h,
                      const double* strx, const double* stry, const double* strz,
                      const double* u, const double* um, const double* up, double* out,
                      const double* rho, const double* irho, double coef, double beta,
                      const double* const dc[3], const double* const st[3],
                      const double* const co[3], const double* zc, cudaStream_t stream,
                      double* rscr, int ctas)
{
   int status = upload_sbp_tables_direct();
   if (status != kOk) return status;
   OpArgs a;
   a.zc = zc;
   a.dzc = a.roc = nullptr;
   a.b = b;
   a.bu = field_box;
   a.u = field;
   a.mu = mu;
   a.la = la;
   a.sx = strx;
   a.sy = stry;
   a.sz = strz;
   a.lu = nullptr;
   a.cof = 1.0 / (h * h);
   a.nk = nk;
   RowUpdate w;
   w.udf = w.umdf = w.updf = nullptr;
   w.outdf = nullptr;
   w.lo = 0;
   w.dd = nullptr;
   a.udf = nullptr;
   w.corrector = corrector;
   w.u = u;
   w.um = um;
   w.up = up;
   w.out = out;
   w.irho = irho;
   w.rho = rho;
   w.coef = coef;
   w.beta = beta;
   for (int q = 0; q < 3; q++) {
      w.dc[q] = dc[q];
      w.st[q] = st[q];
      w.co[q] = co[q];
   }
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const int gx = blocks_for(ni, 32), gy = blocks_for(nj, 8);
   const dim3 block(32, 8, 1), grid(ctas > 0 ? std::min(ctas, gx * gy * 6) : gx * gy * 6);
   if (rscr) {  // the per-column terms once, then the rows read them
      a.dzc = rscr;
      a.roc = rscr + 18 * b.nij;
      const int nb = ctas > 0 ? ctas : (int)std::min<long long>((b.nij + 127) / 128, 152LL * 16);
      if (top) rows_pre_kernel<true><<<nb, 128, 0, stream>>>(a, rscr, rscr + 18 * b.nij);
      else rows_pre_kernel<false><<<nb, 128, 0, stream>>>(a, rscr, rscr + 18 * b.nij);
      const int st = launch_status();
      if (st != kOk) return st;
   }
   const bool pre = rscr != nullptr;
   if (top) {
      if (pre) stage_rows_kernel<true, false, false, true><<<grid, block, 0, stream>>>(a, w, gx, gy);
      else stage_rows_kernel<true, false, false, false><<<grid, block, 0, stream>>>(a, w, gx, gy);
   } else {
      if (pre) stage_rows_kernel<false, false, false, true><<<grid, block, 0, stream>>>(a, w, gx, gy);
      else stage_rows_kernel<false, false, false, false><<<grid, block, 0, stream>>>(a, w, gx, gy);
   }
   return launch_status();
}

int launch_stage_rows_df(int corrector, bool top, const Box& b, int nz, const double* field_f64,
                         const float* field_df, const Box& field_box, const double* mu,
                         const double* la, double h, const double* strx, const double* stry,
                         const double* strz, const float* u, const float* um, const float* up,
                         float* out, const double* rho, const double* irho, double coef,
                         double beta, const double* const dc[3], const double* const st[3],
                         const double* const co[3], const double* zc, cudaStream_t stream,
                         const double* dd, double* rscr, int ctas)
{
   int status = upload_sbp_tables_direct();
   if (status != kOk) return status;
   OpArgs a;
   a.zc = zc;
   a.dzc = a.roc = nullptr;
   a.b = b;
   a.bu = field_box;
   a.u = field_f64;
   a.udf = field_df;
   a.mu = mu;
   a.la = la;
   a.sx = strx;
   a.sy = stry;
   a.sz = strz;
   a.lu = nullptr;
   a.cof = 1.0 / (h * h);
   a.nk = nz;
   RowUpdate w;
   w.corrector = corrector;
   w.u = w.um = w.up = nullptr;
   w.out = nullptr;
   w.udf = u;
   w.umdf = um;
   w.updf = up;
   w.outdf = out;
   w.lo = 3 * b.npts;
   w.dd = dd;
   w.ddb = field_box;
   w.irho = irho;
   w.rho = rho;
   w.coef = coef;
   w.beta = beta;
   for (int q = 0; q < 3; q++) {
      w.dc[q] = dc[q];
      w.st[q] = st[q];
      w.co[q] = co[q];
   }
   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3;
   if (ni <= 0 || nj <= 0) return kOk;
   const int gx = blocks_for(ni, 32), gy = blocks_for(nj, 8);
   const dim3 block(32, 8, 1), grid(ctas > 0 ? std::min(ctas, gx * gy * 6) : gx * gy * 6);
   if (rscr) {  // the per-column terms once, then the rows read them
      a.dzc = rscr;
      a.roc = rscr + 18 * b.nij;
      const int nb = ctas > 0 ? ctas : (int)std::min<long long>((b.nij + 127) / 128, 152LL * 16);
      if (top) rows_pre_kernel<true><<<nb, 128, 0, stream>>>(a, rscr, rscr + 18 * b.nij);
      else rows_pre_kernel<false><<<nb, 128, 0, stream>>>(a, rscr, rscr + 18 * b.nij);
      const int st = launch_status();
      if (st != kOk) return st;
   }
   const bool fdf = field_df != nullptr;
   if (top) {
      if (fdf) stage_rows_kernel<true, true, true, false><<<grid, block, 0, stream>>>(a, w, gx, gy);
      else if (rscr) stage_rows_kernel<true, true, false, true><<<grid, block, 0, stream>>>(a, w, gx, gy);
      else stage_rows_kernel<true, true, false, false><<<grid, block, 0, stream>>>(a, w, gx, gy);
   } else {
      if (fdf) stage_rows_kernel<false, true, true, false><<<grid, block, 0, stream>>>(a, w, gx, gy);
      else if (rscr) stage_rows_kernel<false, true, false, true><<<grid, block, 0, stream>>>(a, w, gx, gy);
      else stage_rows_kernel<false, true, false, false><<<grid, block, 0, stream>>>(a, w, gx, gy);
   }
   return launch_status();
}

namespace {
// SBP z coefficients of the 6 one-sided rows for every column (time-invariant):
// zc[((r*8 + q)*2 + t)*nij + col] = sum_m acof(r+1, q+1, m) * c_t(kq(m)), with
// c_0 = mu, c_1 = 2 mu + lambda and kq the row's stencil planes (top or bottom).
template <bool TOP>
__global__ void zcoef_kernel(Box b, int nk, const double* __restrict__ mu,
                             const double* __restrict__ la, double* __restrict__ zc)
{
   const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
   if (col >= b.nij) return;
   double cm[2][8];
   for (int m = 1; m <= 8; m++) {
      const int km = TOP ? m : nk - m + 1;
      const long long p = col + b.nij * (long long)(km - b.kb);
      cm[0][m - 1] = mu[p];
      cm[1][m - 1] = 2 * mu[p] + la[p];
   }
   for (int r = 0; r < 6; r++)
      for (int q = 0; q < 8; q++)
         for (int t = 0; t < 2; t++) {
            double v = 0;
            for (int m = 0; m < 8; m++) v += k_acof[r + 6 * q + 48 * m] * cm[t][m];
            zc[((long long)(r * 8 + q) * 2 + t) * b.nij + col] = v;
         }
}
}  // namespace

long long zcoef_len(const Box& b) { return 96LL * b.nij; }

int launch_zcoef(const Box& b, int nk, bool top, const double* mu, const double* la, double* zc,
                 cudaStream_t s)
{
   int status = upload_sbp_tables_direct();
   if (status != kOk) return status;
   if (top)
      zcoef_kernel<true><<<blocks_for(b.nij, 128), 128, 0, s>>>(b, nk, mu, la, zc);
   else
      zcoef_kernel<false><<<blocks_for(b.nij, 128), 128, 0, s>>>(b, nk, mu, la, zc);
   return launch_status();
}

}  // namespace sw4g
