// The kernel-level bindings of INTEGRATION.md section 1 (Cartesian and curvilinear
// kernels), written into a class derived from the reference's own EW, so that they
// compile against the reference's EW.h / Sarray.h exactly as a maintainer would
// paste them into src/EW.C.  Each statement below the "// EW::" comments is a line of
// INTEGRATION.md (tests/test_integration_compile.py checks that they agree and
// compiles this file with the reference's headers, SW4_CUDA defined).  Locals the
// snippets name (ib..ke, up, u, um, lu, fo, rho, strx.., s) are declared around them
// from the EW members they stand for.
#include <cmath>
#include <cstdio>

#include "EW.h"
#include "EWCuda.h"
#include "sw4g.h"

struct Sw4gBinding : public EW {
   void eval_rhs(vector<Sarray>& a_U, vector<Sarray>& a_Mu, vector<Sarray>& a_Lambda,
                 vector<Sarray>& a_Uacc, int g)
   {
// EW::evalRHS, src/EW.C:3184-3203  (rhs4sg / rhs4sg_rev)
int st = sw4g_rhs4sg(m_corder, m_iStart[g], m_iEnd[g], m_jStart[g], m_jEnd[g],
                     m_kStart[g], m_kEnd[g], m_global_nz[g], m_onesided[g],
                     a_Uacc[g].dev_ptr(), a_U[g].dev_ptr(), a_Mu[g].dev_ptr(),
                     a_Lambda[g].dev_ptr(), mGridSize[g],
                     dev_sg_str_x[g], dev_sg_str_y[g], dev_sg_str_z[g],
                     m_cuobj->m_stream[0]);
if (st != SW4G_OK) { printf("rhs4sg: %s\n", sw4g_status_string(st)); /* handle */ }
   }

   void phases(int g, vector<Sarray>& a_Up, vector<Sarray>& a_U, vector<Sarray>& a_Um,
               vector<Sarray>& a_Lu, vector<Sarray>& a_F, vector<Sarray>& a_Rho,
               vector<Sarray>& a_Mu, vector<Sarray>& a_Lambda, vector<Sarray>& a_Uacc,
               double* bforce_dev[6])
   {
      const int ib = m_iStart[g], ie = m_iEnd[g], jb = m_jStart[g], je = m_jEnd[g];
      const int kb = m_kStart[g], ke = m_kEnd[g];
      double *up = a_Up[g].dev_ptr(), *u = a_U[g].dev_ptr(), *um = a_Um[g].dev_ptr();
      double *lu = a_Lu[g].dev_ptr(), *fo = a_F[g].dev_ptr(), *rho = a_Rho[g].dev_ptr();
      double *mu = a_Mu[g].dev_ptr(), *la = a_Lambda[g].dev_ptr(), *uacc = a_Uacc[g].dev_ptr();
      double *dcx = dev_sg_dc_x[g], *dcy = dev_sg_dc_y[g], *dcz = dev_sg_dc_z[g];
      double *strx = dev_sg_str_x[g], *stry = dev_sg_str_y[g], *strz = dev_sg_str_z[g];
      double *cox = dev_sg_corner_x[g], *coy = dev_sg_corner_y[g], *coz = dev_sg_corner_z[g];
      cudaStream_t s = m_cuobj->m_stream[0];
// EW::evalPredictor / evalCorrector / evalDpDmInTime, src/EW.C:3126-3172
sw4g_predfort(m_corder, ib, ie, jb, je, kb, ke, up, u, um, lu, fo, rho, mDt*mDt, s);
sw4g_corrfort(m_corder, ib, ie, jb, je, kb, ke, up, lu, fo, rho, pow(mDt,4), s);
sw4g_dpdmtfort(ib, ie, jb, je, kb, ke, up, u, um, uacc, 1/(mDt*mDt), s);

// EW::addSuperGridDamping, src/EW.C:3534-3637
sw4g_addsgd4fort(m_corder, ib, ie, jb, je, kb, ke, up, u, um, rho,
                 dcx, dcy, dcz, strx, stry, strz, cox, coy, coz,
                 m_supergrid_damping_coefficient, s);

// EW::enforceBC, src/EW.C:3446-3502  (bforce: host array of 6 device pointers or NULL)
sw4g_bcfortsg(m_corder, ib, ie, jb, je, kb, ke, m_BndryWindow[g], m_global_nx[g],
              m_global_ny[g], m_global_nz[g], u, mGridSize[g], (int*)m_bcType[g], m_sbop,
              mu, la, bforce_dev, strx, stry, s);
   }

   void curvilinear(int g, vector<Sarray>& a_Up, vector<Sarray>& a_U, vector<Sarray>& a_Um,
                    vector<Sarray>& a_Lu, vector<Sarray>& a_Rho, vector<Sarray>& a_Mu,
                    vector<Sarray>& a_Lambda, double* bforce_side4_dev)
   {
      const int ib = m_iStart[g], ie = m_iEnd[g], jb = m_jStart[g], je = m_jEnd[g];
      const int kb = m_kStart[g], ke = m_kEnd[g];
      const double h = mGridSize[g];
      double *up = a_Up[g].dev_ptr(), *u = a_U[g].dev_ptr(), *um = a_Um[g].dev_ptr();
      double *lu = a_Lu[g].dev_ptr(), *rho = a_Rho[g].dev_ptr();
      double *mu = a_Mu[g].dev_ptr(), *la = a_Lambda[g].dev_ptr();
      double *dcx = dev_sg_dc_x[g], *dcy = dev_sg_dc_y[g];
      double *strx = dev_sg_str_x[g], *stry = dev_sg_str_y[g];
      double *cox = dev_sg_corner_x[g], *coy = dev_sg_corner_y[g];
      cudaStream_t s = m_cuobj->m_stream[0];
// EW::evalRHS for the curvilinear grid, src/EW.C:3218-3240  (rhs4sgcurv / _rev)
sw4g_rhs4sgcurv(m_corder, ib, ie, jb, je, kb, ke, m_onesided[g], lu, u, mu, la,
                mMetric.dev_ptr(), mJ.dev_ptr(), strx, stry, s);
// EW::setup_metric, src/EW.C:6232-6288  (metric / metric_rev; synchronises)
sw4g_metric(m_corder, ib, ie, jb, je, kb, ke, h, mZ.dev_ptr(), mMetric.dev_ptr(), mJ.dev_ptr(), s);
// EW::enforceBC, top of the curvilinear grid, src/EW.C:3477-3497
sw4g_freesurfcurvisg(m_corder, ib, ie, jb, je, kb, ke, m_global_nz[g], 5, u, mu, la,
                     mMetric.dev_ptr(), m_sbop, bforce_side4_dev /*or NULL*/, strx, stry, s);
// EW::addSuperGridDamping, curvilinear grid, src/EW.C:3586-3611
sw4g_addsgd4cfort(m_corder, ib, ie, jb, je, kb, ke, up, u, um, rho, dcx, dcy, strx, stry,
                  mJ.dev_ptr(), cox, coy, m_supergrid_damping_coefficient, s);
// EW::computeDT, curvilinear part, src/EW.C:5066-5125 (replaces the LAPACK dspev loop)
double dtc; sw4g_curvilinear_time_step(m_corder, ib, ie, jb, je, kb, ke, rho, mu, la,
                                      mMetric.dev_ptr(), mJ.dev_ptr(), mCFL, &dtc, s);
// EW::generate_grid with topography input=gaussian, src/EW.C:6164
sw4g_gaussian_hill_grid(ib, ie, jb, je, kb, ke, m_global_nz[g], h, m_topo_zmax,
                        m_zetaBreak, m_grid_interpolation_order, m_GaussianAmp,
                        m_GaussianXc, m_GaussianYc, m_GaussianLx, m_GaussianLy, mZ.dev_ptr(), s);
   }
};
