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
   // the stencil and its entries (source_weights.h, shared with the device path)
   TopoStencil st;
   const int rc = topo_stencil(g, onesided, *cv, s, st);
   if (rc != 0) return rc;
   std::vector<GridPointSource>& own = st.in_curv ? curv : cart;
   std::vector<GridPointSource>& other = st.in_curv ? cart : curv;
   for (int t = 0; t < 216; t++) {
      GridPointSource p, q;
      const int got = topo_entry(g, *cv, s, st, t, p, q);
      if (got & 1) own.push_back(p);
      if (got & 2) other.push_back(q);
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
