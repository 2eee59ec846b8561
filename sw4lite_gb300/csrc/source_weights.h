// Grid-point weights of a point source on the Cartesian grid, shared by the host
// set-up (setup.cpp) and the device discretisation (srcdisc.cu).  Both compile
// without FMA contraction, so the two give the same bits.
#pragma once

#include <cmath>

#include "setup.h"

#ifdef __CUDACC__
#define SW4G_HD __host__ __device__
#else
#define SW4G_HD
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

}  // namespace sw4g
