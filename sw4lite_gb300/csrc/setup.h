// Host-side set-up of one Cartesian grid for the elastic time step: supergrid
// profiles, boundary windows, one-sided flags, the CFL time step, and the
// discretisation of point sources into grid-point sources.  Everything here runs
// once before time stepping and is O(N^2) or less.
#pragma once

#include <cmath>
#include <vector>

#ifndef SW4G_HD
#ifdef __CUDACC__
#define SW4G_HD __host__ __device__
#else
#define SW4G_HD
#endif
#endif

namespace sw4g {

// Boundary condition kinds, numbered as the reference's boundaryConditionType
// (src/double/sw4.h:38).
enum Bc : int {
   kStressFree = 0,
   kDirichlet = 1,
   kSuperGrid = 2,
   kPeriodic = 3,
   kInterface = 4,  // bCCInterface: the top of a Cartesian grid below a curvilinear grid
   kProcessor = 7,  // bProcessor: a side shared with a neighbouring subdomain (halo exchange)
   kNone = 8
};

struct GridSpec {
   int nx = 0, ny = 0, nz = 0;  // interior points per axis
   double h = 0;                // grid spacing
   double zmin = 0;             // z of the first interior plane
   int bc[6] = {kSuperGrid, kSuperGrid, kSuperGrid, kSuperGrid, kStressFree, kSuperGrid};
   int sg_gp = 20;              // supergrid layer width in grid points (src/EW.C:176)
   double sg_damping = 0.02;    // supergrid damping coefficient (src/EW.C:174)
   int sg_order = 4;            // 4 or 6 (src/EW.C:1288-1305)
   int soa = 1;                 // component layout: 1 SoA (corder=1), 0 AoS
   int precision = 0;           // 0: FP64 throughout; 1: FP32-mixed (stage_mixed.cu)
};

// Array bounds of the grid: 2 ghost points per side.
struct Bounds {
   int ib, ie, jb, je, kb, ke;
   long long npts() const { return (long long)(ie - ib + 1) * (je - jb + 1) * (ke - kb + 1); }
};
Bounds grid_bounds(const GridSpec& g);

// 1-D supergrid coefficient profiles (damping dc, stretching str, corner taper co)
// along each axis, sampled at every array index (src/EW.C:4636-4803, src/SuperGrid.C).
struct SupergridProfiles {
   std::vector<double> dc[3], str[3], co[3];
   bool used = false;
};
SupergridProfiles supergrid_profiles(const GridSpec& g);
// The profiles of a subdomain: the global grid's profiles at the subdomain's array
// indices (local i = global i - ioff, local j = global j - joff).
SupergridProfiles subdomain_profiles(const GridSpec& global, const GridSpec& local, int ioff,
                                     int joff);

// Boundary windows and point counts per side (src/EW.C:3347-3444) and the
// one-sided flags of the top/bottom sides (src/EW.C:4863-4868).
void boundary_windows(const GridSpec& g, int wind[36], int npts[6]);
void onesided_flags(const GridSpec& g, int onesided[6]);

// dt = cfl * h / sqrt(max((4 mu + lambda)/rho)) over all array points, then
// adjusted to land on tmax (src/EW.C:5041-5146).  Returns dt; nsteps out.
double cfl_time_step(const GridSpec& g, const double* rho, const double* mu, const double* la,
                     double cfl, double tstart, double tmax, int* nsteps);

// One source: either a point force (fx,fy,fz) or a moment tensor (mxx..mzz).
struct SourceSpec {
   double x = 0, y = 0, z = 0;
   bool moment = false;
   double f[3] = {0, 0, 0};                  // fx, fy, fz
   double m[6] = {0, 0, 0, 0, 0, 0};         // mxx, mxy, mxz, myy, myz, mzz
   double freq = 1, t0 = 0;
   int kind = 0;                             // timefunc kind (forcing.cu)
};

struct GridPointSource {
   int i, j, k;
   double amp[3];
   double freq, t0;
   int kind;
};

// Cartesian single-grid source discretisation (src/Source.C:1074-1920):
// 6-point moment-exact delta / delta' weights per axis with the SBP boundary
// normalisation near one-sided boundaries.
void discretize_source(const GridSpec& g, const int onesided[6], const SourceSpec& s,
                       std::vector<GridPointSource>& out);

// The curvilinear grid of a two-grid set-up as the source discretisation sees it:
// nz planes from the surface (k = 1) to the interface (k = nz, z = zmax), a Gaussian
// hill elevation, the grid mapping's grading (zeta_break, order) and a host copy of
// its Jacobian over the array (bounds ib.., jb.., kb..).
struct CurvSourceGrid {
   int nz = 0;
   double zmax = 0;
   double amp = 0, xc = 0, yc = 0, lx = 1, ly = 1, zeta_break = 0.95;
   int order = 4;
   const double* jac = nullptr;
   int ib = 0, jb = 0, kb = 0;
   long long ni = 0, nij = 0;
   // jac: the Jacobian over the curvilinear array, in host memory for the host path and
   // in device memory for the device path
   SW4G_HD double elevation(double x, double y) const
   {
      return amp * ::exp(-((x - xc) / lx) * ((x - xc) / lx) - ((y - yc) / ly) * ((y - yc) / ly));
   }
   SW4G_HD double J(int i, int j, int k) const
   {
      return jac[(i - ib) + ni * (j - jb) + nij * (long long)(k - kb)];
   }
};

// Two-grid source discretisation (src/Source.C:1074-1990 with the curvilinear
// branches): the source goes to the curvilinear grid at or above the interface
// (s from the inverted grid mapping, weights divided by the Jacobian, the moment
// source's z-derivative through the mapping's metric at the source) or to the
// Cartesian grid below it; a stencil that reaches across the interface is split
// between the grids.  cv == nullptr: one Cartesian grid.  Returns 0, 1 if the
// source lies above the topography, 2 if the mapping cannot be inverted there.
int discretize_source_topo(const GridSpec& g, const int onesided[6], const CurvSourceGrid* cv,
                           const SourceSpec& s, std::vector<GridPointSource>& cart,
                           std::vector<GridPointSource>& curv);

// Sort grid-point sources by point and build the per-point groups
// (src/EW.C:6370-6433).  start has npoints+1 entries.
void group_sources(std::vector<GridPointSource>& src, std::vector<int>& start);

}  // namespace sw4g
