// Test infrastructure only: C entry points onto the reference's OWN kernels,
// compiled from the read-only reference sources into oracle/_ref/libsw4ref.so by
// oracle/Makefile.  Nothing in the product links or loads this library; tests use
// it to pin the oracle restatement (oracle/sw4_oracle.c) and bench.py may time it
// as the CPU baseline when it has been built on the machine in question.
//
// The reference's pointwise, damping, boundary and metric kernels are non-virtual
// member functions of class EW (src/EW.h:220-290).  Their bodies read at most the
// member m_corder (src/ew-cfromfort.C:45, :75), so the shim calls them on a
// zero-filled block the size of EW with only m_corder set: the full EW
// constructor (src/EW.C:162) would parse an input deck and start MPI.
#include <cstring>
#include <new>
#include <vector>
#include "../oracle/sw4_oracle.h"
#include "sw4.h"
#include "EW.h"
#include "SuperGrid.h"
#include "time_functions.h"

// Free functions compiled from src/rhs4sg.C, rhs4sg_rev.C, rhs4sgcurv.C and
// rhs4sgcurv_rev.C; declarations as in src/EW.C:141-160.
void rhs4sg_rev(int, int, int, int, int, int, int, int*, float_sw4*, float_sw4*, float_sw4*,
                float_sw4*, float_sw4*, float_sw4*, float_sw4*, float_sw4, float_sw4*,
                float_sw4*, float_sw4*);
void rhs4sg(int, int, int, int, int, int, int, int*, float_sw4*, float_sw4*, float_sw4*,
            float_sw4*, float_sw4*, float_sw4*, float_sw4*, float_sw4, float_sw4*, float_sw4*,
            float_sw4*);
void rhs4sgcurv_rev(int, int, int, int, int, int, float_sw4*, float_sw4*, float_sw4*,
                    float_sw4*, float_sw4*, float_sw4*, int*, float_sw4*, float_sw4*,
                    float_sw4*, float_sw4*, float_sw4*);
void rhs4sgcurv(int, int, int, int, int, int, float_sw4*, float_sw4*, float_sw4*, float_sw4*,
                float_sw4*, float_sw4*, int*, float_sw4*, float_sw4*, float_sw4*, float_sw4*,
                float_sw4*);

namespace {
EW* kernel_host(int corder)
{
   static unsigned char storage[2][sizeof(EW)] __attribute__((aligned(64)));
   unsigned char* s = storage[corder ? 1 : 0];
   std::memset(s, 0, sizeof(EW));
   EW* ew = reinterpret_cast<EW*>(s);
   ew->m_corder = corder != 0;
   return ew;
}
}  // namespace

extern "C" {

void sw4ref_stencil_coefficients(double* acof, double* ghcof, double* bope, double* sbop)
{
   kernel_host(1)->GetStencilCoefficients(acof, ghcof, bope, sbop);
}

void sw4ref_rhs4sg(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                   int nk, int* onesided, double* acof, double* bope, double* ghcof, double* lu,
                   double* u, double* mu, double* la, double h, double* strx, double* stry,
                   double* strz)
{
   if (soa)
      rhs4sg_rev(ifirst, ilast, jfirst, jlast, kfirst, klast, nk, onesided, acof, bope, ghcof, lu,
                 u, mu, la, h, strx, stry, strz);
   else
      rhs4sg(ifirst, ilast, jfirst, jlast, kfirst, klast, nk, onesided, acof, bope, ghcof, lu, u,
             mu, la, h, strx, stry, strz);
}

void sw4ref_rhs4sgcurv(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                       int klast, double* u, double* mu, double* la, double* met, double* jac,
                       double* lu, int* onesided, double* acof, double* bope, double* ghcof,
                       double* strx, double* stry)
{
   if (soa)
      rhs4sgcurv_rev(ifirst, ilast, jfirst, jlast, kfirst, klast, u, mu, la, met, jac, lu,
                     onesided, acof, bope, ghcof, strx, stry);
   else
      rhs4sgcurv(ifirst, ilast, jfirst, jlast, kfirst, klast, u, mu, la, met, jac, lu, onesided,
                 acof, bope, ghcof, strx, stry);
}

void sw4ref_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                     double* u, double* um, double* lu, double* fo, double* rho, double dt2)
{
   kernel_host(soa)->predfort(ib, ie, jb, je, kb, ke, up, u, um, lu, fo, rho, dt2);
}

void sw4ref_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                     double* lu, double* fo, double* rho, double dt4)
{
   kernel_host(soa)->corrfort(ib, ie, jb, je, kb, ke, up, lu, fo, rho, dt4);
}

void sw4ref_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, double* up, double* u,
                      double* um, double* u2, double dt2i)
{
   kernel_host(1)->dpdmtfort(ib, ie, jb, je, kb, ke, up, u, um, u2, dt2i);
}

void sw4ref_addsgd4(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                    double* up, double* u, double* um, double* rho, double* dcx, double* dcy,
                    double* dcz, double* strx, double* stry, double* strz, double* cox,
                    double* coy, double* coz, double beta)
{
   EW* ew = kernel_host(soa);
   if (soa)
      ew->addsgd4fort_indrev(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                             dcy, dcz, strx, stry, strz, cox, coy, coz, beta);
   else
      ew->addsgd4fort(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx, dcy, dcz,
                      strx, stry, strz, cox, coy, coz, beta);
}

void sw4ref_addsgd6(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                    double* up, double* u, double* um, double* rho, double* dcx, double* dcy,
                    double* dcz, double* strx, double* stry, double* strz, double* cox,
                    double* coy, double* coz, double beta)
{
   EW* ew = kernel_host(soa);
   if (soa)
      ew->addsgd6fort_indrev(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                             dcy, dcz, strx, stry, strz, cox, coy, coz, beta);
   else
      ew->addsgd6fort(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx, dcy, dcz,
                      strx, stry, strz, cox, coy, coz, beta);
}

void sw4ref_addsgd4c(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                     int klast, double* up, double* u, double* um, double* rho, double* dcx,
                     double* dcy, double* strx, double* stry, double* jac, double* cox,
                     double* coy, double beta)
{
   EW* ew = kernel_host(soa);
   if (soa)
      ew->addsgd4cfort_indrev(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                              dcy, strx, stry, jac, cox, coy, beta);
   else
      ew->addsgd4cfort(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx, dcy,
                       strx, stry, jac, cox, coy, beta);
}

void sw4ref_addsgd6c(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                     int klast, double* up, double* u, double* um, double* rho, double* dcx,
                     double* dcy, double* strx, double* stry, double* jac, double* cox,
                     double* coy, double beta)
{
   EW* ew = kernel_host(soa);
   if (soa)
      ew->addsgd6cfort_indrev(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                              dcy, strx, stry, jac, cox, coy, beta);
   else
      ew->addsgd6cfort(ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx, dcy,
                       strx, stry, jac, cox, coy, beta);
}

void sw4ref_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, int* wind, int nx,
                     int ny, int nz, double* u, double h, const int* bccnd_int, double* sbop,
                     double* mu, double* la, double t, double* bf1, double* bf2, double* bf3,
                     double* bf4, double* bf5, double* bf6, double* strx, double* stry)
{
   boundaryConditionType bccnd[6];
   for (int s = 0; s < 6; s++) bccnd[s] = static_cast<boundaryConditionType>(bccnd_int[s]);
   EW* ew = kernel_host(soa);
   if (soa)
      ew->bcfortsg_indrev(ib, ie, jb, je, kb, ke, wind, nx, ny, nz, u, h, bccnd, sbop, mu, la, t,
                          bf1, bf2, bf3, bf4, bf5, bf6, 0.0, 0.0, 0.0, strx, stry);
   else
      ew->bcfortsg(ib, ie, jb, je, kb, ke, wind, nx, ny, nz, u, h, bccnd, sbop, mu, la, t, bf1,
                   bf2, bf3, bf4, bf5, bf6, 0.0, 0.0, 0.0, strx, stry);
}

int sw4ref_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* x, double* y,
                  double* z, double* met, double* jac)
{
   EW* ew = kernel_host(soa);
   if (soa) return ew->metric_rev(ib, ie, jb, je, kb, ke, x, y, z, met, jac);
   return ew->metric(ib, ie, jb, je, kb, ke, x, y, z, met, jac);
}

void sw4ref_metricexgh(int soa, int ib, int ie, int jb, int je, int kb, int ke, int nz, double* x,
                       double* y, double* z, double* met, double* jac, int order, double sb,
                       double zmax, double amp, double xc, double yc, double xl, double yl)
{
   EW* ew = kernel_host(soa);
   if (soa)
      ew->metricexgh_rev(ib, ie, jb, je, kb, ke, nz, x, y, z, met, jac, order, sb, zmax, amp, xc,
                         yc, xl, yl);
   else
      ew->metricexgh(ib, ie, jb, je, kb, ke, nz, x, y, z, met, jac, order, sb, zmax, amp, xc, yc,
                     xl, yl);
}

void sw4ref_freesurfcurvisg(int soa, int ib, int ie, int jb, int je, int kb, int ke, int nz,
                            int side, double* u, double* mu, double* la, double* met, double* sbop,
                            double* forcing, double* strx, double* stry)
{
   EW* ew = kernel_host(soa);
   if (soa)
      ew->freesurfcurvisg_rev(ib, ie, jb, je, kb, ke, nz, side, u, mu, la, met, sbop, forcing,
                              strx, stry);
   else
      ew->freesurfcurvisg(ib, ie, jb, je, kb, ke, nz, side, u, mu, la, met, sbop, forcing, strx,
                          stry);
}

// Supergrid profiles through the reference class (src/SuperGrid.C:52-198), sampled
// as in src/EW.C:4745-4781: x = (q-1)*h + xmin for q in [first,last].
void sw4ref_supergrid_profile(int first, int last, double h, double xmin, int left, int right,
                              double x0, double x1, double width, double* dc, double* str,
                              double* corner)
{
   SuperGrid sg;
   sg.define_taper(left != 0, x0, right != 0, x1, width);
   for (int q = first; q <= last; q++) {
      double x = (q - 1) * h + xmin;
      dc[q - first] = sg.dampingCoeff(x);
      str[q - first] = sg.stretching(x);
      corner[q - first] = sg.cornerTaper(x);
   }
}

// Source time functions (src/time_functions.C): kind 0 Gaussian, 1 C6SmoothBump.
// par[0] is the underflow cut-off exponent the reference's Source sets (-700,
// src/Source.C:2183-2187).
double sw4ref_timefunc(int kind, double freq, double t, int tt)
{
   double par[2] = {-700.0, 0.0};
   int ipar[1] = {0};
   if (kind == 0) return tt ? Gaussian_tt(freq, t, par, 2, ipar, 1) : Gaussian(freq, t, par, 2, ipar, 1);
   return tt ? C6SmoothBump_tt(freq, t, par, 2, ipar, 1) : C6SmoothBump(freq, t, par, 2, ipar, 1);
}

// One time step with the reference's own kernels, in the CPU phase order of
// EW::timesteploop (src/EW.C:2537-2756); forcing from the same grid-point source
// list the oracle uses (sw4o_force), boundary data zero.  Same contract as
// sw4o_step (oracle/sw4_oracle.h).
void sw4ref_step(const sw4o_problem* p, int soa, double t, double* up, const double* u,
                 const double* um, double* lu, double* f, double* uacc)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   kernel_host(soa)->GetStencilCoefficients(acof, ghcof, bope, sbop);
   const long npts = (long)(p->ie - p->ib + 1) * (p->je - p->jb + 1) * (p->ke - p->kb + 1);
   const double dt = p->dt;
   int onesided[6], wind[36];
   for (int s = 0; s < 6; s++) onesided[s] = p->onesided[s];
   for (int s = 0; s < 36; s++) wind[s] = p->wind[s];
   int npw[6];
   sw4o_boundary_windows(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nx, p->ny, p->nz, p->bccnd,
                         wind, npw);
   std::vector<std::vector<double>> bf(6);
   for (int s = 0; s < 6; s++) bf[s].assign(3 * (npw[s] > 0 ? npw[s] : 1), 0.0);
   auto bc = [&](double* w) {
      sw4ref_bcfortsg(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, wind, p->nx, p->ny, p->nz, w,
                      p->h, p->bccnd, sbop, const_cast<double*>(p->mu), const_cast<double*>(p->la), t + dt,
                      bf[0].data(), bf[1].data(), bf[2].data(), bf[3].data(), bf[4].data(),
                      bf[5].data(), const_cast<double*>(p->strx), const_cast<double*>(p->stry));
   };
   double* U = const_cast<double*>(u);
   double* UM = const_cast<double*>(um);
   EW* ew = kernel_host(soa);
   sw4o_force(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 0);
   std::memset(lu, 0, 3 * npts * sizeof(double));
   sw4ref_rhs4sg(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, onesided, acof, bope, ghcof,
                 lu, U, const_cast<double*>(p->mu), const_cast<double*>(p->la), p->h,
                 const_cast<double*>(p->strx), const_cast<double*>(p->stry),
                 const_cast<double*>(p->strz));
   ew->predfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, U, UM, lu, f,
                const_cast<double*>(p->rho), dt * dt);
   bc(up);
   sw4o_force(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 1);
   ew->dpdmtfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, U, UM, uacc, 1.0 / (dt * dt));
   sw4ref_rhs4sg(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, onesided, acof, bope, ghcof,
                 lu, uacc, const_cast<double*>(p->mu), const_cast<double*>(p->la), p->h,
                 const_cast<double*>(p->strx), const_cast<double*>(p->stry),
                 const_cast<double*>(p->strz));
   ew->corrfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, lu, f, const_cast<double*>(p->rho),
                dt * dt * dt * dt);
   if (p->sg_beta != 0) {
      double* pr[9] = {const_cast<double*>(p->dcx), const_cast<double*>(p->dcy),
                       const_cast<double*>(p->dcz), const_cast<double*>(p->strx),
                       const_cast<double*>(p->stry), const_cast<double*>(p->strz),
                       const_cast<double*>(p->cox), const_cast<double*>(p->coy),
                       const_cast<double*>(p->coz)};
      if (p->sg_order == 6)
         sw4ref_addsgd6(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, U, UM,
                        const_cast<double*>(p->rho), pr[0], pr[1], pr[2], pr[3], pr[4], pr[5],
                        pr[6], pr[7], pr[8], p->sg_beta);
      else
         sw4ref_addsgd4(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, U, UM,
                        const_cast<double*>(p->rho), pr[0], pr[1], pr[2], pr[3], pr[4], pr[5],
                        pr[6], pr[7], pr[8], p->sg_beta);
   }
   bc(up);
}


// The two-grid step of sw4o_step_topo with the reference's own kernels
// (rhs4sg_rev, rhs4sgcurv_rev, predfort, dpdmtfort, corrfort, addsgd4fort_indrev,
// addsgd4cfort_indrev, bcfortsg_indrev, freesurfcurvisg_rev) in the order of
// src/EW.C:2537-2756 and the interface copy of src/EW.C:3504.
void sw4ref_step_topo(const sw4o_problem* p, const sw4o_curv* cv, double t, double* up,
                      const double* u, const double* um, double* lu, double* f, double* uacc,
                      double* cup, const double* cu, const double* cum, double* clu, double* cf,
                      double* cuacc)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   EW* ew = kernel_host(1);
   ew->GetStencilCoefficients(acof, ghcof, bope, sbop);
   const long npts = (long)(p->ie - p->ib + 1) * (p->je - p->jb + 1) * (p->ke - p->kb + 1);
   const long cnpts = (long)(cv->ie - cv->ib + 1) * (cv->je - cv->jb + 1) * (cv->ke - cv->kb + 1);
   const double dt = p->dt;
   int onesided[6], onesided_c[6] = {0, 0, 0, 0, cv->bccnd[4] == 0, 0};
   for (int s = 0; s < 6; s++) onesided[s] = p->onesided[s];
   int wind[36], cwind[36], npw[6], cnpw[6];
   sw4o_boundary_windows(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nx, p->ny, p->nz, p->bccnd,
                         wind, npw);
   sw4o_boundary_windows(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cv->nx, cv->ny, cv->nz,
                         cv->bccnd, cwind, cnpw);
   std::vector<std::vector<double>> bf(6), cbf(6);
   for (int s = 0; s < 6; s++) {
      bf[s].assign(3 * (npw[s] > 0 ? npw[s] : 1), 0.0);
      cbf[s].assign(3 * (cnpw[s] > 0 ? cnpw[s] : 1), 0.0);
   }
   std::vector<double> fsforce(3 * (size_t)(cv->ie - cv->ib + 1) * (cv->je - cv->jb + 1), 0.0);
   auto D = [](const double* x) { return const_cast<double*>(x); };
   auto bc = [&](double* w, double* cw) {
      sw4ref_bcfortsg(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, wind, p->nx, p->ny, p->nz, w,
                      p->h, p->bccnd, sbop, D(p->mu), D(p->la), t + dt, bf[0].data(), bf[1].data(),
                      bf[2].data(), bf[3].data(), bf[4].data(), bf[5].data(), D(p->strx), D(p->stry));
      sw4ref_bcfortsg(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cwind, cv->nx, cv->ny,
                      cv->nz, cw, cv->h, cv->bccnd, sbop, D(cv->mu), D(cv->la), t + dt,
                      cbf[0].data(), cbf[1].data(), cbf[2].data(), cbf[3].data(), cbf[4].data(),
                      cbf[5].data(), D(cv->strx), D(cv->stry));
      if (cv->bccnd[4] == 0)
         ew->freesurfcurvisg_rev(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cv->nz, 5, cw,
                                 D(cv->mu), D(cv->la), D(cv->met), sbop, fsforce.data(),
                                 D(cv->strx), D(cv->stry));
      // enforceCartTopo, src/EW.C:3504-3530, with 2 ghost points
      const long ni = p->ie - p->ib + 1, nij = ni * (p->je - p->jb + 1);
      const long cni = cv->ie - cv->ib + 1, cnij = cni * (cv->je - cv->jb + 1);
      for (int j = p->jb; j <= p->je; j++)
         for (int i = p->ib; i <= p->ie; i++)
            for (int c = 0; c < 3; c++) {
               for (int q = 0; q < 2; q++)
                  w[c * npts + (i - p->ib) + ni * (j - p->jb) + nij * (p->kb + q - p->kb)] =
                      cw[c * cnpts + (i - cv->ib) + cni * (j - cv->jb) +
                         cnij * (cv->ke - 4 + q - cv->kb)];
               for (int q = 0; q <= 2; q++)
                  cw[c * cnpts + (i - cv->ib) + cni * (j - cv->jb) + cnij * (cv->ke - q - cv->kb)] =
                      w[c * npts + (i - p->ib) + ni * (j - p->jb) + nij * (p->kb + 4 - q - p->kb)];
            }
   };
   sw4o_force(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 0);
   sw4o_force(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cf, cv->nsrc, cv->src_ijk,
              cv->src_amp, cv->src_freq, cv->src_t0, cv->src_kind, t, 0);
   std::memset(lu, 0, 3 * npts * sizeof(double));
   std::memset(clu, 0, 3 * cnpts * sizeof(double));
   rhs4sg_rev(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, onesided, acof, bope, ghcof, lu,
              D(u), D(p->mu), D(p->la), p->h, D(p->strx), D(p->stry), D(p->strz));
   rhs4sgcurv_rev(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, D(cu), D(cv->mu), D(cv->la),
                  D(cv->met), D(cv->jac), clu, onesided_c, acof, bope, ghcof, D(cv->strx),
                  D(cv->stry));
   ew->predfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, D(u), D(um), lu, f, D(p->rho), dt * dt);
   ew->predfort(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, D(cu), D(cum), clu, cf,
                D(cv->rho), dt * dt);
   bc(up, cup);
   sw4o_force(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 1);
   sw4o_force(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cf, cv->nsrc, cv->src_ijk,
              cv->src_amp, cv->src_freq, cv->src_t0, cv->src_kind, t, 1);
   ew->dpdmtfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, D(u), D(um), uacc, 1.0 / (dt * dt));
   ew->dpdmtfort(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, D(cu), D(cum), cuacc,
                 1.0 / (dt * dt));
   rhs4sg_rev(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, onesided, acof, bope, ghcof, lu,
              uacc, D(p->mu), D(p->la), p->h, D(p->strx), D(p->stry), D(p->strz));
   rhs4sgcurv_rev(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cuacc, D(cv->mu), D(cv->la),
                  D(cv->met), D(cv->jac), clu, onesided_c, acof, bope, ghcof, D(cv->strx),
                  D(cv->stry));
   ew->corrfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, lu, f, D(p->rho), dt * dt * dt * dt);
   ew->corrfort(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, clu, cf, D(cv->rho),
                dt * dt * dt * dt);
   if (p->sg_beta != 0 && p->sg_order == 6) {
      ew->addsgd6fort_indrev(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, D(u), D(um), D(p->rho),
                             D(p->dcx), D(p->dcy), D(p->dcz), D(p->strx), D(p->stry), D(p->strz),
                             D(p->cox), D(p->coy), D(p->coz), p->sg_beta);
      ew->addsgd6cfort_indrev(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, D(cu), D(cum),
                              D(cv->rho), D(cv->dcx), D(cv->dcy), D(cv->strx), D(cv->stry),
                              D(cv->jac), D(cv->cox), D(cv->coy), p->sg_beta);
   } else if (p->sg_beta != 0) {
      ew->addsgd4fort_indrev(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, D(u), D(um), D(p->rho),
                             D(p->dcx), D(p->dcy), D(p->dcz), D(p->strx), D(p->stry), D(p->strz),
                             D(p->cox), D(p->coy), D(p->coz), p->sg_beta);
      ew->addsgd4cfort_indrev(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, D(cu), D(cum),
                              D(cv->rho), D(cv->dcx), D(cv->dcy), D(cv->strx), D(cv->stry),
                              D(cv->jac), D(cv->cox), D(cv->coy), p->sg_beta);
   }
   bc(up, cup);
}
}  // extern "C"
