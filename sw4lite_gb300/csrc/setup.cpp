// Host-side set-up for one Cartesian grid; see setup.h.
#include "setup.h"

#include "source_weights.h"

#include <algorithm>
#include <cmath>
#include <tuple>

namespace sw4g {

Bounds grid_bounds(const GridSpec& g)
{
   return Bounds{-1, g.nx + 2, -1, g.ny + 2, -1, g.nz + 2};
}

namespace {

// C5 smooth step of the supergrid taper (src/SuperGrid.C:148-176): 0 for xi<=0,
// 1 for xi>=1.  Evaluated as monomials in the same order as the reference: near
// xi=1 the polynomial cancels to ~1 and the stretching 1-(1-epsL)psi cancels
// again, so the evaluation order shows in dc = psi/phi at the 1e-9 level.
double psi0(double xi)
{
   if (xi <= 0.) return 0;
   if (xi >= 1.) return 1.0;
   return xi * xi * xi * xi * xi * xi *
          (462 - 1980 * xi + 3465 * xi * xi - 3080 * xi * xi * xi + 1386 * xi * xi * xi * xi -
           252 * xi * xi * xi * xi * xi);
}

struct Taper {
   bool left = false, right = false;
   double x0 = 0, x1 = 1, width = 0.1, trans = 0.05;
   static constexpr double epsL = 1e-4;

   double psi_aux(double x) const
   {
      if (left && x < x0 + width) return psi0((x0 + width - x) / width);
      if (right && x > x1 - width) return psi0((x - (x1 - width)) / width);
      return 0;
   }
   double psi_damp(double x) const
   {
      if (left && x < x0 + width) return psi0((x0 + width - x) / trans);
      if (right && x > x1 - width) return psi0((x - (x1 - width)) / trans);
      return 0;
   }
   double lin(double x) const
   {
      if (left && x < x0 + width) return (x0 + width - x) / width;
      if (right && x > x1 - width) return (x - (x1 - width)) / width;
      return 0;
   }
   double stretching(double x) const { return 1 - (1 - epsL) * psi_aux(x); }
   double damping(double x) const { return psi_damp(x) / stretching(x); }
   double corner(double x) const { return 1.0 - (1.0 - 0.33) * lin(x); }
};

Taper make_taper(bool left, double x0, bool right, double x1, double width)
{
   Taper t;
   t.left = left;
   t.right = right;
   t.x0 = x0;
   t.x1 = x1;
   t.width = width;
   t.trans = 0.5 * width;
   return t;
}

}  // namespace

SupergridProfiles supergrid_profiles(const GridSpec& g)
{
   SupergridProfiles p;
   const Bounds b = grid_bounds(g);
   const int first[3] = {b.ib, b.jb, b.kb}, last[3] = {b.ie, b.je, b.ke};
   for (int s = 0; s < 6; s++)
      if (g.bc[s] == kSuperGrid) p.used = true;
   const double width = g.sg_gp * g.h;
   const double xmax = (g.nx - 1) * g.h, ymax = (g.ny - 1) * g.h, zmax = g.zmin + (g.nz - 1) * g.h;
   Taper t[3];
   t[0] = make_taper(g.bc[0] == kSuperGrid, 0.0, g.bc[1] == kSuperGrid, xmax, width);
   t[1] = make_taper(g.bc[2] == kSuperGrid, 0.0, g.bc[3] == kSuperGrid, ymax, width);
   // Single Cartesian grid: the z taper starts at 0 as the reference's
   // define_taper(..., 0.0, ..., m_global_zmax, ...) (src/EW.C:4655-4658).
   t[2] = make_taper(g.bc[4] == kSuperGrid, 0.0, g.bc[5] == kSuperGrid, zmax, width);
   for (int ax = 0; ax < 3; ax++) {
      const int n = last[ax] - first[ax] + 1;
      p.dc[ax].resize(n);
      p.str[ax].resize(n);
      p.co[ax].resize(n);
      for (int q = first[ax]; q <= last[ax]; q++) {
         const double x = (ax == 2 ? g.zmin : 0.0) + (q - 1) * g.h;
         if (p.used) {
            p.dc[ax][q - first[ax]] = t[ax].damping(x);
            p.str[ax][q - first[ax]] = t[ax].stretching(x);
            p.co[ax][q - first[ax]] = t[ax].corner(x);
         } else {
            p.dc[ax][q - first[ax]] = 0;
            p.str[ax][q - first[ax]] = 1;
            p.co[ax][q - first[ax]] = 1;
         }
      }
   }
   return p;
}

SupergridProfiles subdomain_profiles(const GridSpec& global, const GridSpec& local, int ioff,
                                     int joff)
{
   const SupergridProfiles gp = supergrid_profiles(global);
   SupergridProfiles p;
   p.used = gp.used;
   const int off[3] = {ioff, joff, 0}, n[3] = {local.nx + 4, local.ny + 4, local.nz + 4};
   for (int ax = 0; ax < 3; ax++) {
      p.dc[ax].assign(gp.dc[ax].begin() + off[ax], gp.dc[ax].begin() + off[ax] + n[ax]);
      p.str[ax].assign(gp.str[ax].begin() + off[ax], gp.str[ax].begin() + off[ax] + n[ax]);
      p.co[ax].assign(gp.co[ax].begin() + off[ax], gp.co[ax].begin() + off[ax] + n[ax]);
   }
   return p;
}

void boundary_windows(const GridSpec& g, int wind[36], int npts[6])
{
   const Bounds b = grid_bounds(g);
   const int ng = 2;
   for (int s = 0; s < 6; s++) {
      npts[s] = 0;
      for (int q = 0; q < 6; q++) wind[6 * s + q] = (q % 2 == 0) ? 999 : -999;
      const int t = g.bc[s];
      if (!(t == kStressFree || t == kDirichlet || t == kSuperGrid || t == kPeriodic)) continue;
      int w[6] = {b.ib, b.ie, b.jb, b.je, b.kb, b.ke};
      const int layers = t == kStressFree ? 1 : ng;
      const int lo = 2 * (s / 2), hi = lo + 1;  // index pair of the side's axis in w
      if (s % 2 == 0) w[hi] = w[lo] + layers - 1;
      else w[lo] = w[hi] - (layers - 1);
      if (t == kStressFree) {
         // the boundary plane itself, just inside the ghost points
         if (s % 2 == 0) w[lo] += ng;
         else w[lo] -= ng;
         w[hi] = w[lo];
      }
      for (int q = 0; q < 6; q++) wind[6 * s + q] = w[q];
      npts[s] = (w[5] - w[4] + 1) * (w[3] - w[2] + 1) * (w[1] - w[0] + 1);
   }
}

void onesided_flags(const GridSpec& g, int onesided[6])
{
   for (int s = 0; s < 6; s++) onesided[s] = 0;
   // one grid: only a free surface (stress-free) side uses the SBP closure
   onesided[4] = g.bc[4] == kStressFree;
   onesided[5] = g.bc[5] == kStressFree;
}

double cfl_time_step(const GridSpec& g, const double* rho, const double* mu, const double* la,
                     double cfl, double tstart, double tmax, int* nsteps)
{
   const long long n = grid_bounds(g).npts();
   double eigmax = -1;
   for (long long p = 0; p < n; p++) {
      const double e = (4 * mu[p] + la[p]) / rho[p];
      eigmax = e > eigmax ? e : eigmax;
   }
   double dt = cfl * g.h * (1 / std::sqrt(eigmax));
   if (!((tmax - tstart) / dt < 2.0e9)) return -1;  // the step count would not fit an int
   int ns = static_cast<int>((tmax - tstart) / dt + 0.5);
   ns = ns == 0 ? 1 : ns;
   dt = (tmax - tstart) / ns;
   if (nsteps) *nsteps = ns;
   return dt;
}

namespace {

// 8-point interpolation weights at offsets -3..4 and their derivative, for the
// topography and its tangential derivatives at a source (src/Source.C:682-720; the
// same polynomials interpolate the topography, src/EW.C:5671-5690).
void metric_weights(double a, double w[8], double dw[8])
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
bool invert_curvilinear_s(const CurvSourceGrid& c, double h, double q, double r, double z, double* s)
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
         err = std::fabs(ds);
         sun -= ds;
      }
      if (err > 1e-9) return false;
   }
   *s = (nz - 1) * sun + 1;
   return true;
}

// z_q, z_r, z_s of the grid mapping at a source in the curvilinear grid from the
// topography at the 8 x 8 surrounding grid points (src/Source.C:2191-2330).
void metric_at_source(const CurvSourceGrid& c, double h, double q, double r, double s, int ic, int jc,
                      int kc, double* zq, double* zr, double* zs)
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
   const double pp = std::pow(1 - zpar, c.order - 1);
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

}  // namespace

void discretize_source(const GridSpec& g, const int onesided[6], const SourceSpec& s,
                       std::vector<GridPointSource>& out)
{
   CartStencil c;
   cart_stencil(g, onesided[4] != 0, onesided[5] != 0, s, c);
   for (int t = 0; t < 216; t++) {
      GridPointSource p;
      if (cart_entry(g, c, s, t, p)) out.push_back(p);
   }
}

int discretize_source_topo(const GridSpec& g, const int onesided[6], const CurvSourceGrid* cv,
                           const SourceSpec& s, std::vector<GridPointSource>& cart,
                           std::vector<GridPointSource>& curv)
{
   if (!cv) {  // one Cartesian grid (source_weights.h, shared with the device path)
      discretize_source(g, onesided, s, cart);
      return 0;
   }
   const double h = g.h;
   const int Ni = g.nx, Nj = g.ny;
   // the grid of the source (src/EW.C:5149-5213): the curvilinear grid at or above
   // the interface, a source above the topography is refused (src/Source.C:520-530)
   bool in_curv = false;
   if (cv) {
      if (s.z < -cv->elevation(s.x, s.y) - 1e-9) return 1;
      in_curv = !(s.z > g.zmin);
   }
   const int Nz = in_curv ? cv->nz : g.nz;
   // mapped coordinates (src/EW.C:5722-5782)
   const double q0 = s.x / h + 1, r0 = s.y / h + 1;
   double s0 = (s.z - g.zmin) / h + 1;
   if (in_curv && !invert_curvilinear_s(*cv, h, q0, r0, s.z, &s0)) return 2;
   int ic = static_cast<int>(std::floor(q0));
   int jc = static_cast<int>(std::floor(r0));
   int kc = static_cast<int>(std::floor(s0));
   // keep the 6-point stencil away from the ghost points (src/Source.C:1145-1200); a
   // stencil that reaches across the Cartesian/curvilinear interface is not moved
   if (ic <= 2) ic = 3;
   if (ic >= Ni - 2) ic = Ni - 3;
   if (jc <= 2) jc = 3;
   if (jc >= Nj - 2) jc = Nj - 3;
   if (kc >= Nz) kc = Nz - 1;
   if (kc < 1) kc = 1;
   const bool upper = kc >= 1 && kc <= 3, lower = kc >= Nz - 3 && kc <= Nz - 1;
   const bool across = cv && ((upper && !in_curv) || (lower && in_curv));
   if (!across) {
      if (kc <= 2) kc = 3;
      if (kc >= Nz - 2) kc = Nz - 3;
   }
   const double ai = q0 - ic, bi = r0 - jc, ci = s0 - kc;

   double wi[6], wj[6], wk[6], dwi[6], dwj[6], dwk[6];
   delta_weights(ai, wi);
   delta_weights(bi, wj);
   delta_weights(ci, wk);
   ddelta_weights(ai, dwi);
   ddelta_weights(bi, dwj);
   ddelta_weights(ci, dwk);
   if (!across && kc == 3 && ci <= 0) {
      delta_weights_low(ci, wk);
      ddelta_weights_low(ci, dwk);
   }
   // SBP quadrature normalisation of the weights on the first/last 4 planes of a
   // one-sided side (src/Source.C:1410-1440); the curvilinear grid's top is the
   // free surface, its bottom the interface
   const double normwgh[4] = {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0};
   const bool top_os = in_curv ? true : onesided[4] != 0, bot_os = in_curv ? false : onesided[5] != 0;
   if (top_os) {
      for (int k = 0; k <= 5; k++)
         if (1 <= k + kc - 2 && k + kc - 2 <= 4) {
            wk[k] /= normwgh[k + kc - 3];
            dwk[k] /= normwgh[k + kc - 3];
         }
   }
   if (bot_os) {
      for (int k = 0; k <= 5; k++)
         if (Nz - 3 <= k + kc - 2 && k + kc - 2 <= Nz) {
            wk[k] /= normwgh[Nz - k - kc + 2];
            dwk[k] /= normwgh[Nz - k - kc + 2];
         }
   }
   // the moment source's s-derivative of the mapping (src/Source.C:1603-1660): on the
   // Cartesian grid (0, 0, 1/h)
   const double hi = 1.0 / h;
   double sx0[3] = {0, 0, hi};
   if (in_curv && s.moment) {
      double zq, zr, zs;
      metric_at_source(*cv, h, q0, r0, s0, ic, jc, kc, &zq, &zr, &zs);
      sx0[0] = -zq / (h * zs);
      sx0[1] = -zr / (h * zs);
      sx0[2] = 1 / zs;
   }
   const double ih3 = 1.0 / (h * h * h);
   std::vector<GridPointSource>& own = in_curv ? curv : cart;
   for (int k = kc - 2; k <= kc + 3; k++)
      for (int j = jc - 2; j <= jc + 3; j++)
         for (int i = ic - 2; i <= ic + 3; i++) {
            if (!(1 <= i && i <= Ni && 1 <= j && j <= Nj)) continue;
            GridPointSource p;
            p.i = i;
            p.j = j;
            p.k = k;
            p.freq = s.freq;
            p.t0 = s.t0;
            p.kind = s.kind;
            // 1/J of the point (src/Source.C:1506-1509, :1810-1814)
            const double jaci = in_curv ? 1 / cv->J(i, j, k) : ih3;
            if (!s.moment) {
               // point force (src/Source.C:1479-1530)
               double wF = wi[i - ic + 2] * wj[j - jc + 2] * wk[k - kc + 2];
               if (wF == 0 || (s.f[0] == 0 && s.f[1] == 0 && s.f[2] == 0)) continue;
               wF *= jaci;
               for (int c = 0; c < 3; c++) p.amp[c] = wF * s.f[c];
            } else {
               // moment tensor: F = -M grad(delta) (src/Source.C:1710-1930)
               double wFx = hi * dwi[i - ic + 2] * wj[j - jc + 2] * wk[k - kc + 2];
               double wFy = wi[i - ic + 2] * hi * dwj[j - jc + 2] * wk[k - kc + 2];
               double wFz = wi[i - ic + 2] * wj[j - jc + 2] * hi * dwk[k - kc + 2];
               if (in_curv) {
                  const double w = wi[i - ic + 2] * wj[j - jc + 2] * dwk[k - kc + 2];
                  wFx += w * sx0[0];
                  wFy += w * sx0[1];
                  wFz = w * sx0[2];
               }
               const double* M = s.m;  // xx, xy, xz, yy, yz, zz
               p.amp[0] = -(M[0] * wFx + M[1] * wFy + M[2] * wFz) * jaci;
               p.amp[1] = -(M[1] * wFx + M[3] * wFy + M[4] * wFz) * jaci;
               p.amp[2] = -(M[2] * wFx + M[4] * wFy + M[5] * wFz) * jaci;
            }
            if (1 <= k && k <= Nz) own.push_back(p);
            // across the interface: the Cartesian plane k <= 1 is the curvilinear plane
            // nz - 1 + k, the curvilinear plane k >= nz the Cartesian plane k - nz + 1
            if (across && !in_curv && k <= 1) {
               GridPointSource q = p;
               q.k = cv->nz - 1 + k;
               curv.push_back(q);
            }
            if (across && in_curv && k >= Nz) {
               GridPointSource q = p;
               q.k = k - Nz + 1;
               cart.push_back(q);
            }
         }
   return 0;
}

void group_sources(std::vector<GridPointSource>& src, std::vector<int>& start)
{
   auto key = [](const GridPointSource& a) {
      return std::make_tuple(a.k, a.j, a.i);
   };
   std::stable_sort(src.begin(), src.end(),
                    [&](const GridPointSource& a, const GridPointSource& b) { return key(a) < key(b); });
   start.clear();
   start.push_back(0);
   for (size_t s = 1; s <= src.size(); s++)
      if (s == src.size() || key(src[s]) != key(src[s - 1])) start.push_back((int)s);
}

}  // namespace sw4g
