// Grid-point weights of a point source on the Cartesian grid and on a Cartesian grid
// under a curvilinear grid, shared by the host set-up (setup.cpp) and the device
// discretisation (srcdisc.cu).  Both compile without FMA contraction, so the
// Cartesian weights give the same bits; the curvilinear ones also call exp and pow
// (topography, grid mapping), whose host and device results may differ in the last
// bit.
#pragma once

#include <cmath>

#include "setup.h"

#ifndef SW4G_HD
#ifdef __CUDACC__
#define SW4G_HD __host__ __device__
#else
#define SW4G_HD
#endif
#endif

namespace sw4g {

// 6-point delta weights at offsets -2..3 for a source at fractional position a
// (moments 0..4 exact), src/Source.C:553-584.
SW4G_HD inline void delta_weights(double a, double w[6])
{
   const double a2 = a * a, a3 = a2 * a, a4 = a3 * a, a5 = a4 * a;
   const double p5 = a5 * (5.0 / 3 - 7.0 / 24 * a - 17 / 12.0 * a2 + 1.125 * a3 - 0.25 * a4);
   w[0] = 1.0 / 24 * (2 * a - a2 - 2 * a3 - 19 * a4) + p5;
   w[1] = 1.0 / 6 * (-4 * a + 4 * a2 + a3) + 4 * a4 - 5 * p5;
   w[2] = 1 - 1.25 * a2 - 97.0 / 12 * a4 + 10 * p5;
   w[3] = 1.0 / 6 * (4 * a + 4 * a2 - a3 + 49 * a4) - 10 * p5;
   w[4] = 1.0 / 24 * (-2 * a - a2 + 2 * a3) - 4.125 * a4 + 5 * p5;
   w[5] = 5.0 / 6 * a4 - p5;
}

// 6-point delta' weights, src/Source.C:587-619.
SW4G_HD inline void ddelta_weights(double a, double w[6])
{
   const double a2 = a * a, a3 = a2 * a, a4 = a3 * a;
   const double p5 = a4 * (-25.0 / 12 - 0.75 * a + 59.0 / 12 * a2 - 4 * a3 + a4);
   w[0] = 1.0 / 12 * (-1 + a + 3 * a2 + 8 * a3) + p5;
   w[1] = 2.0 / 3 * (1 - 2 * a) - 0.5 * a2 - 3.5 * a3 - 5 * p5;
   w[2] = 2.5 * a + 22.0 / 3 * a3 + 10 * p5;
   w[3] = 2.0 / 3 * (-1 - 2 * a) + 0.5 * a2 - 23.0 / 3 * a3 - 10 * p5;
   w[4] = (1 + a) / 12 - 0.25 * a2 + 4 * a3 + 5 * p5;
   w[5] = -5.0 / 6 * a3 - p5;
}

// Five-point variants used next to the free surface when the source lies above
// the third grid plane (src/Source.C:622-679).
SW4G_HD inline void delta_weights_low(double a, double w[6])
{
   const double a2 = a * a, a3 = a2 * a, a4 = a3 * a;
   w[0] = (2 * a - a2 - 2 * a3 + a4) / 24;
   w[1] = (-4 * a + 4 * a2 + a3 - a4) / 6;
   w[2] = 1 - 1.25 * a2 + 0.25 * a4;
   w[3] = (4 * a + 4 * a2 - a3 - a4) / 6;
   w[4] = (-2 * a - a2 + 2 * a3 + a4) / 24;
   w[5] = 0;
}

SW4G_HD inline void ddelta_weights_low(double a, double w[6])
{
   const double a2 = a * a, a3 = a2 * a;
   w[0] = (-1 + a + 3 * a2 - 2 * a3) / 12;
   w[1] = (2 - 4 * a - 1.5 * a2 + 2 * a3) / 3;
   w[2] = 2.5 * a - a3;
   w[3] = (-2 - 4 * a + 1.5 * a2 + 2 * a3) / 3;
   w[4] = (1 + a - 3 * a2 - 2 * a3) / 12;
   w[5] = 0;
}

// The Cartesian grid's 6-point stencil of a source: centre indices (the stencil
// spans ic-2..ic+3, ...) and the delta / delta' weights per axis, with the five-point
// variants next to the free surface and the SBP quadrature normalisation near
// one-sided sides (src/Source.C:1145-1200, 1370-1440).
struct CartStencil {
   int ic, jc, kc;
   double wi[6], wj[6], wk[6], dwi[6], dwj[6], dwk[6];
};

SW4G_HD inline void cart_stencil(const GridSpec& g, bool top_os, bool bot_os, const SourceSpec& s,
                                 CartStencil& c)
{
   const double h = g.h;
   const int Ni = g.nx, Nj = g.ny, Nz = g.nz;
   const double q0 = s.x / h + 1, r0 = s.y / h + 1, s0 = (s.z - g.zmin) / h + 1;
   int ic = static_cast<int>(::floor(q0));
   int jc = static_cast<int>(::floor(r0));
   int kc = static_cast<int>(::floor(s0));
   // keep the 6-point stencil away from the ghost points (src/Source.C:1145-1200)
   if (ic <= 2) ic = 3;
   if (ic >= Ni - 2) ic = Ni - 3;
   if (jc <= 2) jc = 3;
   if (jc >= Nj - 2) jc = Nj - 3;
   if (kc >= Nz) kc = Nz - 1;
   if (kc < 1) kc = 1;
   if (kc <= 2) kc = 3;
   if (kc >= Nz - 2) kc = Nz - 3;
   const double ai = q0 - ic, bi = r0 - jc, ci = s0 - kc;
   delta_weights(ai, c.wi);
   delta_weights(bi, c.wj);
   delta_weights(ci, c.wk);
   ddelta_weights(ai, c.dwi);
   ddelta_weights(bi, c.dwj);
   ddelta_weights(ci, c.dwk);
   if (kc == 3 && ci <= 0) {
      delta_weights_low(ci, c.wk);
      ddelta_weights_low(ci, c.dwk);
   }
   const double normwgh[4] = {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0};
   if (top_os) {
      for (int k = 0; k <= 5; k++)
         if (1 <= k + kc - 2 && k + kc - 2 <= 4) {
            c.wk[k] /= normwgh[k + kc - 3];
            c.dwk[k] /= normwgh[k + kc - 3];
         }
   }
   if (bot_os) {
      for (int k = 0; k <= 5; k++)
         if (Nz - 3 <= k + kc - 2 && k + kc - 2 <= Nz) {
            c.wk[k] /= normwgh[Nz - k - kc + 2];
            c.dwk[k] /= normwgh[Nz - k - kc + 2];
         }
   }
   c.ic = ic;
   c.jc = jc;
   c.kc = kc;
}

// Entry t of the stencil, t = (k-kc+2) 36 + (j-jc+2) 6 + (i-ic+2) (the order the
// host adds them in): its grid point and amplitude (point force
// src/Source.C:1479-1530, moment tensor F = -M grad(delta) :1710-1930, 1/J = 1/h^3).
// False where no grid-point source is added.
SW4G_HD inline bool cart_entry(const GridSpec& g, const CartStencil& c, const SourceSpec& s, int t,
                               GridPointSource& p)
{
   const int i = c.ic - 2 + t % 6, j = c.jc - 2 + (t / 6) % 6, k = c.kc - 2 + t / 36;
   if (!(1 <= i && i <= g.nx && 1 <= j && j <= g.ny)) return false;
   const double h = g.h, hi = 1.0 / h, ih3 = 1.0 / (h * h * h);
   p.i = i;
   p.j = j;
   p.k = k;
   p.freq = s.freq;
   p.t0 = s.t0;
   p.kind = s.kind;
   const int a = i - c.ic + 2, b = j - c.jc + 2, d = k - c.kc + 2;
   if (!s.moment) {
      double wF = c.wi[a] * c.wj[b] * c.wk[d];
      if (wF == 0 || (s.f[0] == 0 && s.f[1] == 0 && s.f[2] == 0)) return false;
      wF *= ih3;
      for (int q = 0; q < 3; q++) p.amp[q] = wF * s.f[q];
   } else {
      const double wFx = hi * c.dwi[a] * c.wj[b] * c.wk[d];
      const double wFy = c.wi[a] * hi * c.dwj[b] * c.wk[d];
      const double wFz = c.wi[a] * c.wj[b] * hi * c.dwk[d];
      const double* M = s.m;  // xx, xy, xz, yy, yz, zz
      p.amp[0] = -(M[0] * wFx + M[1] * wFy + M[2] * wFz) * ih3;
      p.amp[1] = -(M[1] * wFx + M[3] * wFy + M[4] * wFz) * ih3;
      p.amp[2] = -(M[2] * wFx + M[4] * wFy + M[5] * wFz) * ih3;
   }
   return 1 <= k && k <= g.nz;
}


// ---- two grids: Cartesian below a curvilinear grid over topography ----

// 8-point interpolation weights at offsets -3..4 and their derivative, for the
// topography and its tangential derivatives at a source (src/Source.C:682-720; the
// same polynomials interpolate the topography, src/EW.C:5671-5690).
SW4G_HD inline void metric_weights(double a, double w[8], double dw[8])
{
   const double a2 = a * a, a3 = a2 * a, a4 = a3 * a, a5 = a4 * a, a6 = a5 * a, a7 = a6 * a;
   double pol = a7 * (-251 + 135 * a + 25 * a2 - 33 * a3 + 6 * a4) / 720;
   w[0] = -1.0 / 60 * a + 1.0 / 180 * a2 + 1.0 / 48 * a3 + 23.0 / 144 * a4 - (17.0 * a + 223.0) * a5 / 720 - pol;
   w[1] = 3.0 / 20 * a - 3.0 / 40 * a2 - 1.0 / 6 * a3 - 13.0 / 12 * a4 + 97.0 / 45 * a5 + 1.0 / 6 * a6 + 7 * pol;
   w[2] = -0.75 * a + 0.75 * a2 + (13.0 + 155 * a) * a3 / 48 - 103.0 / 16 * a5 - 121.0 / 240 * a6 - 21 * pol;
   w[3] = 1 - 49.0 / 36 * a2 - 49.0 / 9 * a4 + 385.0 / 36 * a5 + 61.0 / 72 * a6 + 35 * pol;
   w[4] = 0.75 * a + 0.75 * a2 - 13.0 / 48 * a3 + 89.0 / 16 * a4 - 1537.0 / 144 * a5 - 41.0 / 48 * a6 - 35 * pol;
   w[5] = -3.0 / 20 * a - 3.0 / 40 * a2 + 1.0 / 6 * a3 - 41.0 / 12 * a4 + 6.4 * a5 + 31.0 / 60 * a6 + 21 * pol;
   w[6] = 1.0 / 60 * a + 1.0 / 180 * a2 - 1.0 / 48 * a3 + 167.0 / 144 * a4 - 1537.0 / 720 * a5 - 25.0 / 144 * a6 - 7 * pol;
   w[7] = -1.0 / 6 * a4 + 11.0 / 36 * a5 + 1.0 / 40 * a6 + pol;
   pol = a6 * (-1757.0 / 720 + 1.5 * a + 0.3125 * a2 - (1.375 * a3 - 0.275 * a4) / 3);
   dw[0] = -1.0 / 60 + 1.0 / 90 * a + a2 / 16 + 23.0 / 36 * a3 - 223.0 / 144 * a4 - 17.0 / 120 * a5 - pol;
   dw[1] = 3.0 / 20 - 3.0 / 20 * a - 0.5 * a2 - 13.0 / 3 * a3 + 97.0 / 9 * a4 + a5 + 7 * pol;
   dw[2] = -0.75 + 1.5 * a + 13.0 / 16 * a2 + 155.0 * a3 / 12 - 103.0 * 5.0 / 16 * a4 - 121.0 / 40 * a5 - 21 * pol;
   dw[3] = -49.0 / 18 * a - 4 * 49.0 / 9.0 * a3 + 385.0 * 5.0 / 36 * a4 + 61.0 / 12 * a5 + 35 * pol;
   dw[4] = 0.75 + 1.5 * a - 13.0 / 16 * a2 + 89.0 / 4 * a3 - 1537.0 * 5 / 144.0 * a4 - 41.0 / 8 * a5 - 35 * pol;
   dw[5] = -3.0 / 20 - 3.0 / 20 * a + 0.5 * a2 - 41.0 / 3 * a3 + 32 * a4 + 3.1 * a5 + 21 * pol;
   dw[6] = 1.0 / 60 + 1.0 / 90 * a - 1.0 / 16 * a2 + 167.0 / 36 * a3 - 1537.0 / 144 * a4 - 25.0 / 24 * a5 - 7 * pol;
   dw[7] = -2.0 / 3 * a3 + 55.0 / 36 * a4 + 3.0 / 20 * a5 + pol;
}

// s of the point (q, r, z) on the curvilinear grid: Newton iteration on the grid
// mapping in the graded part, at most 10 iterations to 1e-9 (src/EW.C:5722-5782).
SW4G_HD inline bool invert_curvilinear_s(const CurvSourceGrid& c, double h, double q, double r, double z,
                                         double* s)
{
   const double ztopo = -c.elevation((q - 1) * h, (r - 1) * h);
   const int nz = c.nz;
   const double izb = 1.0 / c.zeta_break;
   double sun = 1 - (c.zmax - z) / ((nz - 1) * h);
   if (sun < c.zeta_break) {
      double err = 1e-9 + 1;
      for (int it = 0; it < 10 && err > 1e-9; it++) {
         double omsm = 1 - izb * sun;
         for (int l = 2; l <= c.order - 1; l++) omsm *= 1 - izb * sun;
         const double fp = h * (nz - 1) + izb * c.order * omsm * (c.zmax - (nz - 1) * h - ztopo);
         omsm *= 1 - izb * sun;
         const double f = c.zmax - (nz - 1) * h * (1 - sun) - omsm * (c.zmax - (nz - 1) * h - ztopo) - z;
         const double ds = f / fp;
         err = ::fabs(ds);
         sun -= ds;
      }
      if (err > 1e-9) return false;
   }
   *s = (nz - 1) * sun + 1;
   return true;
}

// z_q, z_r, z_s of the grid mapping at a source in the curvilinear grid from the
// topography at the 8 x 8 surrounding grid points (src/Source.C:2191-2330).
SW4G_HD inline void metric_at_source(const CurvSourceGrid& c, double h, double q, double r, double s,
                                     int ic, int jc, int kc, double* zq, double* zr, double* zs)
{
   const int nz = c.nz;
   *zq = *zr = 0;
   *zs = h;
   if (kc > nz - 3) return;  // the lowest grid lines are Cartesian
   const double zpar = (s - 1) / (c.zeta_break * (nz - 1));
   if (zpar >= 1) return;
   double wi[8], dwi[8], wj[8], dwj[8];
   metric_weights(q - ic, wi, dwi);
   metric_weights(r - jc, wj, dwj);
   const double kbreak = 1 + c.zeta_break * (nz - 1);
   const double pp = ::pow(1 - zpar, c.order - 1);
   const double powo = (1 - zpar) * pp, dpowo = -c.order * pp / c.zeta_break;
   double tavg = 0, tq = 0, tr = 0;
   for (int j = jc - 3; j <= jc + 4; j++)
      for (int i = ic - 3; i <= ic + 4; i++) {
         const double t = c.elevation((i - 1) * h, (j - 1) * h);
         tavg += wi[i - (ic - 3)] * wj[j - (jc - 3)] * t;
         tq += dwi[i - (ic - 3)] * wj[j - (jc - 3)] * t;
         tr += wi[i - (ic - 3)] * dwj[j - (jc - 3)] * t;
      }
   *zq = -tq * powo;
   *zr = -tr * powo;
   const double zmx = c.zmax - (nz - kbreak) * h;
   const double c1 = zmx + tavg - h * (kbreak - 1);
   *zs = h + c1 * (-dpowo) / (nz - 1);
}


// The stencil of a source in a two-grid set-up (src/Source.C:1074-1990 with the
// curvilinear branches): the grid of the source (the curvilinear grid at or above the
// interface), its mapped coordinates (s from the inverted grid mapping), the centre
// (not moved where the stencil reaches across the interface), the weights with the
// five-point and SBP boundary treatment, and the moment source's s-derivative of the
// mapping.
struct TopoStencil {
   bool in_curv, across;
   int ic, jc, kc, Nz;
   double wi[6], wj[6], wk[6], dwi[6], dwj[6], dwk[6];
   double sx0[3];
};

// 0, or 1 for a source above the topography, 2 if the mapping cannot be inverted.
SW4G_HD inline int topo_stencil(const GridSpec& g, const int onesided[6], const CurvSourceGrid& cv,
                                const SourceSpec& s, TopoStencil& st)
{
   const double h = g.h;
   const int Ni = g.nx, Nj = g.ny;
   // the grid of the source (src/EW.C:5149-5213); above the topography: refused
   // (src/Source.C:520-530)
   if (s.z < -cv.elevation(s.x, s.y) - 1e-9) return 1;
   st.in_curv = !(s.z > g.zmin);
   const int Nz = st.in_curv ? cv.nz : g.nz;
   st.Nz = Nz;
   // mapped coordinates (src/EW.C:5722-5782)
   const double q0 = s.x / h + 1, r0 = s.y / h + 1;
   double s0 = (s.z - g.zmin) / h + 1;
   if (st.in_curv && !invert_curvilinear_s(cv, h, q0, r0, s.z, &s0)) return 2;
   int ic = static_cast<int>(::floor(q0));
   int jc = static_cast<int>(::floor(r0));
   int kc = static_cast<int>(::floor(s0));
   // keep the 6-point stencil away from the ghost points (src/Source.C:1145-1200); a
   // stencil that reaches across the Cartesian/curvilinear interface is not moved
   if (ic <= 2) ic = 3;
   if (ic >= Ni - 2) ic = Ni - 3;
   if (jc <= 2) jc = 3;
   if (jc >= Nj - 2) jc = Nj - 3;
   if (kc >= Nz) kc = Nz - 1;
   if (kc < 1) kc = 1;
   const bool upper = kc >= 1 && kc <= 3, lower = kc >= Nz - 3 && kc <= Nz - 1;
   st.across = (upper && !st.in_curv) || (lower && st.in_curv);
   if (!st.across) {
      if (kc <= 2) kc = 3;
      if (kc >= Nz - 2) kc = Nz - 3;
   }
   const double ai = q0 - ic, bi = r0 - jc, ci = s0 - kc;
   delta_weights(ai, st.wi);
   delta_weights(bi, st.wj);
   delta_weights(ci, st.wk);
   ddelta_weights(ai, st.dwi);
   ddelta_weights(bi, st.dwj);
   ddelta_weights(ci, st.dwk);
   if (!st.across && kc == 3 && ci <= 0) {
      delta_weights_low(ci, st.wk);
      ddelta_weights_low(ci, st.dwk);
   }
   // SBP quadrature normalisation of the weights on the first/last 4 planes of a
   // one-sided side (src/Source.C:1410-1440); the curvilinear grid's top is the
   // free surface, its bottom the interface
   const double normwgh[4] = {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0};
   const bool top_os = st.in_curv ? true : onesided[4] != 0;
   const bool bot_os = st.in_curv ? false : onesided[5] != 0;
   if (top_os) {
      for (int k = 0; k <= 5; k++)
         if (1 <= k + kc - 2 && k + kc - 2 <= 4) {
            st.wk[k] /= normwgh[k + kc - 3];
            st.dwk[k] /= normwgh[k + kc - 3];
         }
   }
   if (bot_os) {
      for (int k = 0; k <= 5; k++)
         if (Nz - 3 <= k + kc - 2 && k + kc - 2 <= Nz) {
            st.wk[k] /= normwgh[Nz - k - kc + 2];
            st.dwk[k] /= normwgh[Nz - k - kc + 2];
         }
   }
   // the moment source's s-derivative of the mapping (src/Source.C:1603-1660): on the
   // Cartesian grid (0, 0, 1/h)
   const double hi = 1.0 / h;
   st.sx0[0] = 0;
   st.sx0[1] = 0;
   st.sx0[2] = hi;
   if (st.in_curv && s.moment) {
      double zq, zr, zs;
      metric_at_source(cv, h, q0, r0, s0, ic, jc, kc, &zq, &zr, &zs);
      st.sx0[0] = -zq / (h * zs);
      st.sx0[1] = -zr / (h * zs);
      st.sx0[2] = 1 / zs;
   }
   st.ic = ic;
   st.jc = jc;
   st.kc = kc;
   return 0;
}

// Entry t = (k-kc+2) 36 + (j-jc+2) 6 + (i-ic+2) of a two-grid stencil: bit 0 of the
// result when p goes to the source's own grid, bit 1 when q goes to the other grid
// (a stencil across the interface: the Cartesian plane k <= 1 is the curvilinear
// plane nz - 1 + k, the curvilinear plane k >= nz the Cartesian plane k - nz + 1).
SW4G_HD inline int topo_entry(const GridSpec& g, const CurvSourceGrid& cv, const SourceSpec& s,
                              const TopoStencil& st, int t, GridPointSource& p, GridPointSource& q)
{
   const int ic = st.ic, jc = st.jc, kc = st.kc, Nz = st.Nz;
   const int i = ic - 2 + t % 6, j = jc - 2 + (t / 6) % 6, k = kc - 2 + t / 36;
   if (!(1 <= i && i <= g.nx && 1 <= j && j <= g.ny)) return 0;
   const double h = g.h, hi = 1.0 / h, ih3 = 1.0 / (h * h * h);
   p.i = i;
   p.j = j;
   p.k = k;
   p.freq = s.freq;
   p.t0 = s.t0;
   p.kind = s.kind;
   // 1/J of the point (src/Source.C:1506-1509, :1810-1814)
   const double jaci = st.in_curv ? 1 / cv.J(i, j, k) : ih3;
   if (!s.moment) {
      // point force (src/Source.C:1479-1530)
      double wF = st.wi[i - ic + 2] * st.wj[j - jc + 2] * st.wk[k - kc + 2];
      if (wF == 0 || (s.f[0] == 0 && s.f[1] == 0 && s.f[2] == 0)) return 0;
      wF *= jaci;
      for (int c = 0; c < 3; c++) p.amp[c] = wF * s.f[c];
   } else {
      // moment tensor: F = -M grad(delta) (src/Source.C:1710-1930)
      double wFx = hi * st.dwi[i - ic + 2] * st.wj[j - jc + 2] * st.wk[k - kc + 2];
      double wFy = st.wi[i - ic + 2] * hi * st.dwj[j - jc + 2] * st.wk[k - kc + 2];
      double wFz = st.wi[i - ic + 2] * st.wj[j - jc + 2] * hi * st.dwk[k - kc + 2];
      if (st.in_curv) {
         const double w = st.wi[i - ic + 2] * st.wj[j - jc + 2] * st.dwk[k - kc + 2];
         wFx += w * st.sx0[0];
         wFy += w * st.sx0[1];
         wFz = w * st.sx0[2];
      }
      const double* M = s.m;  // xx, xy, xz, yy, yz, zz
      p.amp[0] = -(M[0] * wFx + M[1] * wFy + M[2] * wFz) * jaci;
      p.amp[1] = -(M[1] * wFx + M[3] * wFy + M[4] * wFz) * jaci;
      p.amp[2] = -(M[2] * wFx + M[4] * wFy + M[5] * wFz) * jaci;
   }
   int got = (1 <= k && k <= Nz) ? 1 : 0;
   if (st.across && !st.in_curv && k <= 1) {
      q = p;
      q.k = cv.nz - 1 + k;
      got |= 2;
   }
   if (st.across && st.in_curv && k >= Nz) {
      q = p;
      q.k = k - Nz + 1;
      got |= 2;
   }
   return got;
}

}  // namespace sw4g
