/*
 * CPU oracle: grid-point discretisation of a point source on a Cartesian grid --
 * TEST INFRASTRUCTURE ONLY (see sw4_oracle.h).
 *
 * Restates the Cartesian branch of Source::set_grid_point_sources4
 * (src/Source.C:1074-1530 for the stencil and its boundary treatment, :1479-1530
 * for point forces, :1591-1606 and :1710-1930 for moment tensors) with the weight
 * polynomials of getsourcewgh / getsourcedwgh (src/Source.C:553-619) and their
 * five-point free-surface variants getsourcewghlow / getsourcedwghlow (:622-679).
 *
 * The polynomials are stored here as monomial coefficient tables (exact integer
 * numerators expanded from the published formulas) and evaluated by Horner's rule
 * in extended precision, not in the grouped form the reference and the product use:
 * the two evaluations agree to rounding, so a parity test of the product against
 * this file checks the stencil logic (centre clamping, the five-point branch, the
 * SBP normalisation, the index order, which entries are emitted) rather than
 * repeating the product's arithmetic.
 * tests/test_oracle_sources.py checks the tables' defining moment conditions.
 */
#include <math.h>

#include "sw4_oracle.h"

/* Integer numerators of the monomial coefficients (a^0 first) over a common
 * denominator per table: delta (a^0..a^9) and its five-point variant (a^0..a^4) over
 * 24, delta' (a^0..a^8) and its five-point variant (a^0..a^3) over 12.  Weight m sits
 * at offset m - 2 from the stencil centre. */
static const double kDelta[6][10] = {  /* x 24 */
   {0, 2, -1, -2, -19, 40, -7, -34, 27, -6},
   {0, -16, 16, 4, 96, -200, 35, 170, -135, 30},
   {24, 0, -30, 0, -194, 400, -70, -340, 270, -60},
   {0, 16, 16, -4, 196, -400, 70, 340, -270, 60},
   {0, -2, -1, 2, -99, 200, -35, -170, 135, -30},
   {0, 0, 0, 0, 20, -40, 7, 34, -27, 6},
};
static const double kDDelta[6][9] = {  /* x 12 */
   {-1, 1, 3, 8, -25, -9, 59, -48, 12},
   {8, -16, -6, -42, 125, 45, -295, 240, -60},
   {0, 30, 0, 88, -250, -90, 590, -480, 120},
   {-8, -16, 6, -92, 250, 90, -590, 480, -120},
   {1, 1, -3, 48, -125, -45, 295, -240, 60},
   {0, 0, 0, -10, 25, 9, -59, 48, -12},
};
static const double kDeltaLow[6][5] = {  /* x 24 */
   {0, 2, -1, -2, 1},
   {0, -16, 16, 4, -4},
   {24, 0, -30, 0, 6},
   {0, 16, 16, -4, -4},
   {0, -2, -1, 2, 1},
   {0, 0, 0, 0, 0},
};
static const double kDDeltaLow[6][4] = {  /* x 12 */
   {-1, 1, 3, -2},
   {8, -16, -6, 8},
   {0, 30, 0, -12},
   {-8, -16, 6, 8},
   {1, 1, -3, -2},
   {0, 0, 0, 0},
};
static const double kDen[4] = {24, 12, 24, 12};

/* SBP quadrature weights of the first four points next to a one-sided side */
static const double kNorm[4] = {17.0 / 48, 59.0 / 48, 43.0 / 48, 49.0 / 48};

/* Horner's rule on the exact integer numerators in extended precision, divided by
 * the denominator at the end.  The alternating coefficients (up to 400/24 at a^5)
 * cancel strongly away from a = 0, and a clamped stencil centre next to a side puts
 * a near 2, where a double evaluation of the grouped published form loses about two
 * digits; this evaluation keeps the weights accurate to ~1e-17 there. */
static double horner(const double* c, int deg, double a, double den)
{
   long double s = c[deg];
   for (int d = deg - 1; d >= 0; d--) s = s * (long double)a + (long double)c[d];
   return (double)(s / den);
}

void sw4o_source_weights(int which, double a, double w[6])
{
   for (int m = 0; m < 6; m++) {
      switch (which) {
         case 0: w[m] = horner(kDelta[m], 9, a, kDen[0]); break;
         case 1: w[m] = horner(kDDelta[m], 8, a, kDen[1]); break;
         case 2: w[m] = horner(kDeltaLow[m], 4, a, kDen[2]); break;
         default: w[m] = horner(kDDeltaLow[m], 3, a, kDen[3]); break;
      }
   }
}

/* Stencil centre along one axis: floor of the grid coordinate, kept so that the
 * six points c-2..c+3 stay on interior points (src/Source.C:1145-1200). */
static int centre(double q, int n)
{
   int c = (int)floor(q);
   if (c <= 2) c = 3;
   if (c >= n - 2) c = n - 3;
   return c;
}

int sw4o_discretize_source(int nx, int ny, int nz, double h, double zmin, int top_onesided,
                           int bot_onesided, double x, double y, double z, int is_moment,
                           const double f[3], const double m[6], int cap, int* ijk, double* amp)
{
   const double q = x / h + 1, r = y / h + 1, s = (z - zmin) / h + 1;
   const int ic = centre(q, nx), jc = centre(r, ny);
   int kc = (int)floor(s);
   if (kc >= nz) kc = nz - 1;
   if (kc < 1) kc = 1;
   if (kc <= 2) kc = 3;
   if (kc >= nz - 2) kc = nz - 3;
   const double ai = q - ic, bi = r - jc, ci = s - kc;

   double wi[6], wj[6], wk[6], di[6], dj[6], dk[6];
   sw4o_source_weights(0, ai, wi);
   sw4o_source_weights(0, bi, wj);
   sw4o_source_weights(1, ai, di);
   sw4o_source_weights(1, bi, dj);
   if (kc == 3 && ci <= 0) {  /* the stencil would reach the ghost plane k = 0 */
      sw4o_source_weights(2, ci, wk);
      sw4o_source_weights(3, ci, dk);
   } else {
      sw4o_source_weights(0, ci, wk);
      sw4o_source_weights(1, ci, dk);
   }
   /* SBP normalisation of the points k = 1..4 (top) and nz-3..nz (bottom) */
   for (int t = 0; t < 6; t++) {
      const int k = kc - 2 + t;
      if (top_onesided && k >= 1 && k <= 4) {
         wk[t] /= kNorm[k - 1];
         dk[t] /= kNorm[k - 1];
      }
      if (bot_onesided && k >= nz - 3 && k <= nz) {
         wk[t] /= kNorm[nz - k];
         dk[t] /= kNorm[nz - k];
      }
   }

   const double vol = 1.0 / (h * h * h), hi = 1.0 / h;
   int n = 0;
   for (int tk = 0; tk < 6; tk++)
      for (int tj = 0; tj < 6; tj++)
         for (int ti = 0; ti < 6; ti++) {
            const int i = ic - 2 + ti, j = jc - 2 + tj, k = kc - 2 + tk;
            if (i < 1 || i > nx || j < 1 || j > ny || k < 1 || k > nz) continue;
            double a0, a1, a2;
            if (!is_moment) {
               const double w = wi[ti] * wj[tj] * wk[tk];
               if (w == 0 || (f[0] == 0 && f[1] == 0 && f[2] == 0)) continue;
               a0 = w * vol * f[0];
               a1 = w * vol * f[1];
               a2 = w * vol * f[2];
            } else {
               /* F = -M grad(delta): gradient weights in x, y, z */
               const double gx = hi * di[ti] * wj[tj] * wk[tk];
               const double gy = hi * wi[ti] * dj[tj] * wk[tk];
               const double gz = hi * wi[ti] * wj[tj] * dk[tk];
               /* m: xx, xy, xz, yy, yz, zz */
               a0 = -(m[0] * gx + m[1] * gy + m[2] * gz) * vol;
               a1 = -(m[1] * gx + m[3] * gy + m[4] * gz) * vol;
               a2 = -(m[2] * gx + m[4] * gy + m[5] * gz) * vol;
            }
            if (n >= cap) return -1;
            ijk[3 * n] = i;
            ijk[3 * n + 1] = j;
            ijk[3 * n + 2] = k;
            amp[3 * n] = a0;
            amp[3 * n + 1] = a1;
            amp[3 * n + 2] = a2;
            n++;
         }
   return n;
}
