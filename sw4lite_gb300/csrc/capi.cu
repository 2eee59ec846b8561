// extern "C" entry points of libsw4g.so (declared in include/sw4g.h).
#include <cmath>
#include <vector>
#include <cstring>
#include <exception>
#include <new>

#include "../../include/sw4g.h"
#include "ew.h"
#include "kernels.h"
#include "sbp.h"
#include "setup.h"

using namespace sw4g;

struct sw4g_ew {
   EW* impl;
};

namespace {

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

bool bounds_ok(int ib, int ie, int jb, int je, int kb, int ke)
{
   return ie >= ib && je >= jb && ke >= kb;
}

GridSpec to_spec(const sw4g_grid* g)
{
   GridSpec s;
   s.nx = g->nx;
   s.ny = g->ny;
   s.nz = g->nz;
   s.h = g->h;
   s.zmin = g->zmin;
   for (int q = 0; q < 6; q++) s.bc[q] = g->bc[q];
   s.sg_gp = g->sg_gp;
   s.sg_damping = g->sg_damping;
   s.sg_order = g->sg_order;
   s.soa = g->soa;
   s.precision = g->precision;
   return s;
}

SourceSpec to_source(const sw4g_source* s)
{
   SourceSpec o;
   o.x = s->x;
   o.y = s->y;
   o.z = s->z;
   o.moment = s->moment != 0;
   o.f[0] = s->fx;
   o.f[1] = s->fy;
   o.f[2] = s->fz;
   o.m[0] = s->mxx;
   o.m[1] = s->mxy;
   o.m[2] = s->mxz;
   o.m[3] = s->myy;
   o.m[4] = s->myz;
   o.m[5] = s->mzz;
   o.freq = s->freq;
   o.t0 = s->t0;
   o.kind = s->kind;
   return o;
}

}  // namespace

extern "C" {

const char* sw4g_version(void) { return "sw4g 0.1 (sm_103a)"; }

const char* sw4g_status_string(int status)
{
   switch (status) {
      case SW4G_OK: return "ok";
      case SW4G_BAD_ARGUMENT: return "bad argument";
      case SW4G_CUDA_ERROR: return "CUDA error";
      case SW4G_NAN_DETECTED: return "NaN detected";
      case SW4G_NOT_SUPPORTED: return "not supported";
      case SW4G_TIMEOUT: return "device wait timed out";
      default: return "unknown status";
   }
}

int sw4g_stencil_coefficients(double* acof, double* ghcof, double* bope, double* sbop)
{
   if (!acof || !ghcof || !bope || !sbop) return SW4G_BAD_ARGUMENT;
   sbp_coefficients(acof, ghcof, bope, sbop);
   return SW4G_OK;
}

int sw4g_rhs4sg(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                int nk, const int* onesided, double* lu, const double* u, const double* mu,
                const double* lambda, double h, const double* strx, const double* stry,
                const double* strz, void* stream)
{
   if (!onesided || !lu || !u || !mu || !lambda || !strx || !stry || !strz || !(h > 0))
      return SW4G_BAD_ARGUMENT;
   if (!bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast)) return SW4G_BAD_ARGUMENT;
   // one-sided rows read planes 0..8 (top) or nk-7..nk+1 (bottom)
   if (onesided[4] == 1 && (kfirst > 0 || klast < 8)) return SW4G_BAD_ARGUMENT;
   if (onesided[5] == 1 && (kfirst > nk - 7 || klast < nk + 1)) return SW4G_BAD_ARGUMENT;
   return launch_rhs4sg_direct(soa, ifirst, ilast, jfirst, jlast, kfirst, klast, nk, onesided, lu,
                               u, mu, lambda, h, strx, stry, strz, as_stream(stream));
}

int sw4g_rhs4sgcurv(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                    const int* onesided, double* lu, const double* u, const double* mu,
                    const double* lambda, const double* met, const double* jac, const double* strx,
                    const double* stry, void* stream)
{
   if (!onesided || !lu || !u || !mu || !lambda || !met || !jac || !strx || !stry)
      return SW4G_BAD_ARGUMENT;
   if (!bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast)) return SW4G_BAD_ARGUMENT;
   if (onesided[4] == 1 && (kfirst > 0 || klast < 8)) return SW4G_BAD_ARGUMENT;
   CurvSpec c;
   c.soa = soa;
   c.ib = ifirst; c.ie = ilast; c.jb = jfirst; c.je = jlast; c.kb = kfirst; c.ke = klast;
   c.u = u; c.mu = mu; c.la = lambda; c.met = met; c.jac = jac; c.strx = strx; c.stry = stry;
   return launch_rhs4sgcurv(c, onesided, lu, as_stream(stream));
}

int sw4g_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double h, const double* z,
                double* met, double* jac, void* stream)
{
   if (!z || !met || !jac || !(h > 0) || !bounds_ok(ib, ie, jb, je, kb, ke)) return SW4G_BAD_ARGUMENT;
   int* flag = nullptr;
   if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return SW4G_CUDA_ERROR;
   cudaStream_t s = as_stream(stream);
   int st = cudaMemsetAsync(flag, 0, sizeof(int), s) == cudaSuccess ? SW4G_OK : SW4G_CUDA_ERROR;
   if (st == SW4G_OK) st = launch_metric(soa, ib, ie, jb, je, kb, ke, h, z, met, jac, flag, s);
   int bad = 0;
   if (st == SW4G_OK &&
       (cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess))
      st = SW4G_CUDA_ERROR;
   cudaFree(flag);
   if (st == SW4G_OK && bad) st = SW4G_BAD_ARGUMENT;
   return st;
}

int sw4g_gaussian_hill_grid(int ib, int ie, int jb, int je, int kb, int ke, int nz, double h,
                            double zmax, double zeta_break, int order, double amp, double xc,
                            double yc, double lx, double ly, double* z, void* stream)
{
   if (!z || !(h > 0) || nz < 2 || order < 1 || !(zeta_break > 0) || !(lx > 0) || !(ly > 0) ||
       !bounds_ok(ib, ie, jb, je, kb, ke))
      return SW4G_BAD_ARGUMENT;
   return launch_gaussian_hill_z(ib, ie, jb, je, kb, ke, nz, h, zmax, zeta_break, order, amp, xc,
                                 yc, lx, ly, z, as_stream(stream));
}

int sw4g_freesurfcurvisg(int soa, int ib, int ie, int jb, int je, int kb, int ke, int nz, int side,
                         double* u, const double* mu, const double* lambda, const double* met,
                         const double* sbop, const double* forcing, const double* strx,
                         const double* stry, void* stream)
{
   if (!u || !mu || !lambda || !met || !sbop || !strx || !stry || !bounds_ok(ib, ie, jb, je, kb, ke))
      return SW4G_BAD_ARGUMENT;
   if (side != 5 && side != 6) return SW4G_BAD_ARGUMENT;
   const int k = side == 5 ? 1 : nz;
   if (k - 1 < kb || k + 1 > ke || (side == 5 && 4 > ke) || (side == 6 && nz - 3 < kb))
      return SW4G_BAD_ARGUMENT;
   CurvSpec c;
   c.soa = soa;
   c.ib = ib; c.ie = ie; c.jb = jb; c.je = je; c.kb = kb; c.ke = ke;
   c.u = u; c.mu = mu; c.la = lambda; c.met = met; c.strx = strx; c.stry = stry;
   return launch_freesurfcurvisg(c, nz, side, sbop, forcing, u, as_stream(stream));
}

int sw4g_addsgd4cfort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                      double* up, const double* u, const double* um, const double* rho,
                      const double* dcx, const double* dcy, const double* strx, const double* stry,
                      const double* jac, const double* cox, const double* coy, double beta,
                      void* stream)
{
   if (!up || !u || !um || !rho || !dcx || !dcy || !strx || !stry || !jac || !cox || !coy ||
       !bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast))
      return SW4G_BAD_ARGUMENT;
   return launch_addsgd4c(soa, ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                          dcy, strx, stry, jac, cox, coy, beta, as_stream(stream));
}

int sw4g_addsgd6cfort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                      double* up, const double* u, const double* um, const double* rho,
                      const double* dcx, const double* dcy, const double* strx, const double* stry,
                      const double* jac, const double* cox, const double* coy, double beta,
                      void* stream)
{
   if (!up || !u || !um || !rho || !dcx || !dcy || !strx || !stry || !jac || !cox || !coy ||
       !bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast))
      return SW4G_BAD_ARGUMENT;
   return launch_addsgd6c(make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast), up, u, um, rho,
                          dcx, dcy, strx, stry, jac, cox, coy, beta, as_stream(stream));
}

int sw4g_curvilinear_time_step(int soa, int ib, int ie, int jb, int je, int kb, int ke,
                               const double* rho, const double* mu, const double* lambda,
                               const double* met, const double* jac, double cfl, double* dt,
                               void* stream)
{
   if (!rho || !mu || !lambda || !met || !jac || !dt || !(cfl > 0) || !bounds_ok(ib, ie, jb, je, kb, ke))
      return SW4G_BAD_ARGUMENT;
   const long long n = (long long)(ie - ib + 1) * (je - jb + 1) * (ke - kb + 1);
   const int nb = 152 * 4;
   double* bm = nullptr;
   if (cudaMalloc(&bm, nb * sizeof(double)) != cudaSuccess) return SW4G_CUDA_ERROR;
   cudaStream_t s = as_stream(stream);
   std::vector<double> h(nb);
   int st = launch_curv_eig(soa, n, rho, mu, lambda, met, jac, bm, nb, s);
   if (st == SW4G_OK &&
       (cudaMemcpyAsync(h.data(), bm, nb * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess))
      st = SW4G_CUDA_ERROR;
   cudaFree(bm);
   if (st != SW4G_OK) return st;
   double e = -1;
   for (double v : h) e = v > e ? v : e;
   if (!(e > 0)) return SW4G_BAD_ARGUMENT;
   *dt = cfl / std::sqrt(e);
   return SW4G_OK;
}

int sw4g_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                  const double* u, const double* um, const double* lu, const double* fo,
                  const double* rho, double dt2, void* stream)
{
   if (!up || !u || !um || !lu || !fo || !rho || !bounds_ok(ib, ie, jb, je, kb, ke))
      return SW4G_BAD_ARGUMENT;
   return launch_predfort(soa, ib, ie, jb, je, kb, ke, up, u, um, lu, fo, rho, dt2,
                          as_stream(stream));
}

int sw4g_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                  const double* lu, const double* fo, const double* rho, double dt4, void* stream)
{
   if (!up || !lu || !fo || !rho || !bounds_ok(ib, ie, jb, je, kb, ke)) return SW4G_BAD_ARGUMENT;
   return launch_corrfort(soa, ib, ie, jb, je, kb, ke, up, lu, fo, rho, dt4, as_stream(stream));
}

int sw4g_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, const double* up,
                   const double* u, const double* um, double* u2, double dt2i, void* stream)
{
   if (!up || !u || !um || !u2 || !bounds_ok(ib, ie, jb, je, kb, ke)) return SW4G_BAD_ARGUMENT;
   return launch_dpdmtfort(ib, ie, jb, je, kb, ke, up, u, um, u2, dt2i, as_stream(stream));
}

static int addsgd_common(int order, int soa, int ifirst, int ilast, int jfirst, int jlast,
                         int kfirst, int klast, double* up, const double* u, const double* um,
                         const double* rho, const double* dcx, const double* dcy,
                         const double* dcz, const double* strx, const double* stry,
                         const double* strz, const double* cox, const double* coy,
                         const double* coz, double beta, void* stream)
{
   if (!up || !u || !um || !rho || !dcx || !dcy || !dcz || !strx || !stry || !strz || !cox ||
       !coy || !coz || !bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast))
      return SW4G_BAD_ARGUMENT;
   return launch_addsgd(order, soa, ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho,
                        dcx, dcy, dcz, strx, stry, strz, cox, coy, coz, beta, as_stream(stream));
}

int sw4g_addsgd4fort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                     double* up, const double* u, const double* um, const double* rho,
                     const double* dcx, const double* dcy, const double* dcz, const double* strx,
                     const double* stry, const double* strz, const double* cox, const double* coy,
                     const double* coz, double beta, void* stream)
{
   return addsgd_common(4, soa, ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                        dcy, dcz, strx, stry, strz, cox, coy, coz, beta, stream);
}

int sw4g_addsgd6fort(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                     double* up, const double* u, const double* um, const double* rho,
                     const double* dcx, const double* dcy, const double* dcz, const double* strx,
                     const double* stry, const double* strz, const double* cox, const double* coy,
                     const double* coz, double beta, void* stream)
{
   return addsgd_common(6, soa, ifirst, ilast, jfirst, jlast, kfirst, klast, up, u, um, rho, dcx,
                        dcy, dcz, strx, stry, strz, cox, coy, coz, beta, stream);
}

int sw4g_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int* wind,
                  int nx, int ny, int nz, double* u, double h, const int* bccnd, const double* sbop,
                  const double* mu, const double* lambda, const double* const* bforce,
                  const double* strx, const double* stry, void* stream)
{
   if (!wind || !u || !bccnd || !sbop || !mu || !lambda || !strx || !stry ||
       !bounds_ok(ib, ie, jb, je, kb, ke))
      return SW4G_BAD_ARGUMENT;
   return launch_bcfortsg(soa, ib, ie, jb, je, kb, ke, wind, nx, ny, nz, u, h, bccnd, sbop, mu,
                          lambda, bforce, strx, stry, as_stream(stream));
}

long long sw4g_corr_rows_scratch_len(int ifirst, int ilast, int jfirst, int jlast)
{
   if (ilast < ifirst || jlast < jfirst) return 0;
   return 3LL * 10 * ((long long)ilast - ifirst + 1) * ((long long)jlast - jfirst + 1);
}

namespace {
bool rows_args_ok(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int nz,
                  int side)
{
   if (!bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast)) return false;
   if (ilast - ifirst < 4 || jlast - jfirst < 4 || nz < 8) return false;
   if (side == 0) return kfirst <= -1 && klast >= 8;
   if (side == 1) return kfirst <= nz - 7 && klast >= nz + 2;
   return false;
}
}  // namespace

int sw4g_pred_rows(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int nz,
                   int side, double* out, const double* u, const double* um, const double* mu,
                   const double* lambda, const double* rho, const double* strx, const double* stry,
                   const double* strz, double h, double dt, void* stream)
{
   if (!rows_args_ok(ifirst, ilast, jfirst, jlast, kfirst, klast, nz, side) || !out || !u ||
       !um || !mu || !lambda || !rho || !strx || !stry || !strz || !(h > 0))
      return SW4G_BAD_ARGUMENT;
   const Box b = make_box(1, ifirst, ilast, jfirst, jlast, kfirst, klast);
   const double* none[3] = {strx, stry, strz};
   return launch_stage_rows(0, side == 0, b, nz, u, b, mu, lambda, h, strx, stry, strz, u, um,
                            nullptr, out, rho, nullptr, dt * dt, 0.0, none, none, none, nullptr,
                            as_stream(stream));
}

int sw4g_corr_rows(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int nz,
                   int side, double* out, const double* up, const double* u, const double* um,
                   const double* mu, const double* lambda, const double* rho, const double* strx,
                   const double* stry, const double* strz, const double* dcx, const double* dcy,
                   const double* dcz, const double* cox, const double* coy, const double* coz,
                   double h, double dt, double beta, double* scratch, long long scratch_len,
                   void* stream)
{
   if (!rows_args_ok(ifirst, ilast, jfirst, jlast, kfirst, klast, nz, side) || !out || !up ||
       !u || !um || !mu || !lambda || !rho || !strx || !stry || !strz || !dcx || !dcy || !dcz ||
       !cox || !coy || !coz || !scratch || !(h > 0))
      return SW4G_BAD_ARGUMENT;
   if (scratch_len < sw4g_corr_rows_scratch_len(ifirst, ilast, jfirst, jlast))
      return SW4G_BAD_ARGUMENT;
   const Box b = make_box(1, ifirst, ilast, jfirst, jlast, kfirst, klast);
   const int k0 = side == 0 ? -1 : nz - 7, k1 = side == 0 ? 8 : nz + 2;
   int st = launch_uacc_slab(b, k0, k1, up, u, um, scratch, as_stream(stream));
   if (st != SW4G_OK) return st;
   const Box sb = make_box(1, ifirst, ilast, jfirst, jlast, k0, k1);
   const double* dc[3] = {dcx, dcy, dcz};
   const double* sv[3] = {strx, stry, strz};
   const double* co[3] = {cox, coy, coz};
   return launch_stage_rows(1, side == 0, b, nz, scratch, sb, mu, lambda, h, strx, stry, strz, u,
                            um, up, out, rho, nullptr, dt * dt / 12, beta, dc, sv, co, nullptr,
                            as_stream(stream));
}

int sw4g_supergrid_profile(const sw4g_grid* g, int axis, double* dc, double* str, double* corner)
{
   if (!g || axis < 0 || axis > 2 || !dc || !str || !corner) return SW4G_BAD_ARGUMENT;
   const SupergridProfiles p = supergrid_profiles(to_spec(g));
   const size_t n = p.dc[axis].size();
   std::memcpy(dc, p.dc[axis].data(), n * sizeof(double));
   std::memcpy(str, p.str[axis].data(), n * sizeof(double));
   std::memcpy(corner, p.co[axis].data(), n * sizeof(double));
   return SW4G_OK;
}

int sw4g_boundary_windows(const sw4g_grid* g, int* wind, int* npts)
{
   if (!g || !wind || !npts) return SW4G_BAD_ARGUMENT;
   boundary_windows(to_spec(g), wind, npts);
   return SW4G_OK;
}

int sw4g_discretize_source(const sw4g_grid* g, const sw4g_source* s, int cap, int* ijk,
                           double* amp, int* n)
{
   if (!g || !s || !n || cap < 0 || (cap > 0 && (!ijk || !amp))) return SW4G_BAD_ARGUMENT;
   const GridSpec spec = to_spec(g);
   int onesided[6];
   onesided_flags(spec, onesided);
   std::vector<GridPointSource> out;
   discretize_source(spec, onesided, to_source(s), out);
   *n = (int)out.size();
   for (int q = 0; q < (int)out.size() && q < cap; q++) {
      ijk[3 * q] = out[q].i;
      ijk[3 * q + 1] = out[q].j;
      ijk[3 * q + 2] = out[q].k;
      for (int c = 0; c < 3; c++) amp[3 * q + c] = out[q].amp[c];
   }
   return SW4G_OK;
}

namespace {
void copy_sources(const std::vector<GridPointSource>& v, int cap, int* ijk, double* amp, int* n)
{
   *n = (int)v.size();
   for (int q = 0; q < (int)v.size() && q < cap; q++) {
      ijk[3 * q] = v[q].i;
      ijk[3 * q + 1] = v[q].j;
      ijk[3 * q + 2] = v[q].k;
      for (int c = 0; c < 3; c++) amp[3 * q + c] = v[q].amp[c];
   }
}
}  // namespace

int sw4g_discretize_source_topo(const sw4g_grid* g, const sw4g_topography* t, int nzc,
                                const double* jac, const sw4g_source* s, int cap, int* cart_ijk,
                                double* cart_amp, int* ncart, int* curv_ijk, double* curv_amp,
                                int* ncurv)
{
   if (!g || !t || !jac || !s || !ncart || !ncurv || cap < 0 || nzc < 8 ||
       (cap > 0 && (!cart_ijk || !cart_amp || !curv_ijk || !curv_amp)))
      return SW4G_BAD_ARGUMENT;
   const GridSpec spec = to_spec(g);
   int onesided[6];
   onesided_flags(spec, onesided);
   CurvSourceGrid cs;
   cs.nz = nzc;
   cs.zmax = spec.zmin;
   cs.amp = t->amp;
   cs.xc = t->xc;
   cs.yc = t->yc;
   cs.lx = t->lx;
   cs.ly = t->ly;
   cs.zeta_break = t->zeta_break;
   cs.order = t->order;
   cs.jac = jac;
   cs.ib = -1;
   cs.jb = -1;
   cs.kb = -1;
   cs.ni = spec.nx + 4;
   cs.nij = cs.ni * (spec.ny + 4);
   std::vector<GridPointSource> cart, curv;
   if (discretize_source_topo(spec, onesided, &cs, to_source(s), cart, curv) != 0) return SW4G_BAD_ARGUMENT;
   copy_sources(cart, cap, cart_ijk, cart_amp, ncart);
   copy_sources(curv, cap, curv_ijk, curv_amp, ncurv);
   return SW4G_OK;
}

int sw4g_ew_grid_point_sources(const sw4g_ew* ew, int grid, int cap, int* ijk, double* amp, int* n)
{
   if (!ew || !n || cap < 0 || (cap > 0 && (!ijk || !amp))) return SW4G_BAD_ARGUMENT;
   std::vector<GridPointSource> v;
   const int st = ew->impl->grid_point_sources(grid, &v);
   if (st != SW4G_OK) return st;
   copy_sources(v, cap, ijk, amp, n);
   return SW4G_OK;
}

int sw4g_ew_create(const sw4g_grid* g, void* stream, sw4g_ew** out)
{
   if (!g || !out) return SW4G_BAD_ARGUMENT;
   *out = nullptr;
   EW* e = new (std::nothrow) EW(to_spec(g), as_stream(stream));
   if (!e) return SW4G_BAD_ARGUMENT;
   int st = e->init();
   if (st != SW4G_OK) {
      delete e;
      return st;
   }
   sw4g_ew* h = new (std::nothrow) sw4g_ew{e};
   if (!h) {
      delete e;
      return SW4G_BAD_ARGUMENT;
   }
   *out = h;
   return SW4G_OK;
}

int sw4g_ew_create_subdomain(const sw4g_grid* global, int i0, int i1, int j0, int j1, void* stream,
                             sw4g_ew** out)
{
   if (!global || !out) return SW4G_BAD_ARGUMENT;
   *out = nullptr;
   const GridSpec gs = to_spec(global);
   if (i0 < 1 || j0 < 1 || i1 > gs.nx || j1 > gs.ny || i1 < i0 || j1 < j0) return SW4G_BAD_ARGUMENT;
   GridSpec ls = gs;
   ls.nx = i1 - i0 + 1;
   ls.ny = j1 - j0 + 1;
   const bool edge[4] = {i0 == 1, i1 == gs.nx, j0 == 1, j1 == gs.ny};
   for (int q = 0; q < 4; q++) {
      if (edge[q]) continue;
      // a periodic axis would need its wrap-around exchanged too
      if (gs.bc[q] == kPeriodic) return SW4G_NOT_SUPPORTED;
      ls.bc[q] = kProcessor;
   }
   EW* e = new (std::nothrow) EW(ls, as_stream(stream));
   if (!e) return SW4G_BAD_ARGUMENT;
   int st = e->set_subdomain(gs, i0 - 1, j0 - 1);
   if (st == SW4G_OK) st = e->init();
   if (st != SW4G_OK) {
      delete e;
      return st;
   }
   sw4g_ew* h = new (std::nothrow) sw4g_ew{e};
   if (!h) {
      delete e;
      return SW4G_BAD_ARGUMENT;
   }
   *out = h;
   return SW4G_OK;
}

int sw4g_ew_step_part(sw4g_ew* ew, int part)
{
   return ew ? ew->impl->step_part(part) : SW4G_BAD_ARGUMENT;
}

long long sw4g_ew_halo_bytes(const sw4g_ew* ew, int axis)
{
   if (!ew || (axis != 0 && axis != 1) || !ew->impl->is_subdomain()) return -1;
   return ew->impl->halo_bytes(axis);
}

int sw4g_ew_halo_pack(sw4g_ew* ew, int axis, int side, void* buf)
{
   return ew ? ew->impl->halo_pack(axis, side, buf) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_halo_unpack(sw4g_ew* ew, int axis, int side, const void* buf)
{
   return ew ? ew->impl->halo_unpack(axis, side, buf) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_step_group(sw4g_ew* const* subs, int n, const int* neighbors, int nsteps)
{
   if (!subs || n < 1 || n > 4096 || !neighbors) return SW4G_BAD_ARGUMENT;
   std::vector<EW*> v(n);
   for (int s = 0; s < n; s++) {
      if (!subs[s]) return SW4G_BAD_ARGUMENT;
      v[s] = subs[s]->impl;
   }
   return step_group(v.data(), n, neighbors, nsteps);
}

long long sw4g_halo_len(int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast, int axis)
{
   if (!bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast) || (axis != 0 && axis != 1)) return -1;
   return halo_len(make_box(1, ifirst, ilast, jfirst, jlast, kfirst, klast), axis, 3);
}

int sw4g_halo_pack(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                   int axis, int side, const double* u, double* buf, void* stream)
{
   if (!bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast) || !u || !buf) return SW4G_BAD_ARGUMENT;
   if (ilast - ifirst < 7 || jlast - jfirst < 7) return SW4G_BAD_ARGUMENT;
   return launch_halo_copy(make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast), axis, side, true,
                           false, 3, const_cast<double*>(u), buf, as_stream(stream));
}

int sw4g_halo_unpack(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                     int axis, int side, const double* buf, double* u, void* stream)
{
   if (!bounds_ok(ifirst, ilast, jfirst, jlast, kfirst, klast) || !u || !buf) return SW4G_BAD_ARGUMENT;
   if (ilast - ifirst < 7 || jlast - jfirst < 7) return SW4G_BAD_ARGUMENT;
   return launch_halo_copy(make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast), axis, side, false,
                           false, 3, u, const_cast<double*>(buf), as_stream(stream));
}

int sw4g_ew_create_topo(const sw4g_grid* g, const sw4g_topography* t, void* stream, sw4g_ew** out)
{
   if (!g || !t || !out) return SW4G_BAD_ARGUMENT;
   *out = nullptr;
   TopoSpec ts;
   ts.amp = t->amp;
   ts.xc = t->xc;
   ts.yc = t->yc;
   ts.lx = t->lx;
   ts.ly = t->ly;
   ts.zeta_break = t->zeta_break;
   ts.order = t->order;
   EW* e = new (std::nothrow) EW(to_spec(g), as_stream(stream), &ts);
   if (!e) return SW4G_BAD_ARGUMENT;
   int st = e->init();
   if (st != SW4G_OK) {
      delete e;
      return st;
   }
   sw4g_ew* h = new (std::nothrow) sw4g_ew{e};
   if (!h) {
      delete e;
      return SW4G_BAD_ARGUMENT;
   }
   *out = h;
   return SW4G_OK;
}

int sw4g_ew_gradient(sw4g_ew* ew, int nsteps, int checkpoint_every, const double* observed,
                     int obs_on_device, double* misfit, double* grad_rho, double* grad_mu,
                     double* grad_lambda, int grad_on_device)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   return ew->impl->gradient(nsteps, checkpoint_every, observed, obs_on_device != 0, misfit,
                             grad_rho, grad_mu, grad_lambda, grad_on_device != 0);
}

int sw4g_ew_write_checkpoint(sw4g_ew* ew, const char* path, int cycle)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   return ew->impl->write_checkpoint(path, cycle);
}

int sw4g_ew_read_checkpoint(sw4g_ew* ew, const char* path, int* cycle)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   return ew->impl->read_checkpoint(path, cycle);
}

int sw4g_ew_set_gradient_memory(sw4g_ew* ew, long long max_bytes)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   return ew->impl->set_gradient_memory(max_bytes);
}

int sw4g_ew_num_grids(const sw4g_ew* ew) { return ew ? ew->impl->num_grids() : -1; }

int sw4g_ew_grid_dims(const sw4g_ew* ew, int grid, int* nx, int* ny, int* nz, long long* npts)
{
   return ew ? ew->impl->grid_dims(grid, nx, ny, nz, npts) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_material_grid(sw4g_ew* ew, int grid, const double* rho, const double* mu,
                              const double* lambda, int on_device)
{
   return ew ? ew->impl->set_material_grid(grid, rho, mu, lambda, on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_fields_grid(sw4g_ew* ew, int grid, const double* u, const double* um, int on_device)
{
   return ew ? ew->impl->set_fields_grid(grid, u, um, on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_get_fields_grid(const sw4g_ew* ew, int grid, double* u, double* um, int on_device)
{
   return ew ? ew->impl->get_fields_grid(grid, u, um, on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_curvilinear_arrays(const sw4g_ew* ew, double* z, double* met, double* jac, int on_device)
{
   return ew ? ew->impl->curvilinear_arrays(z, met, jac, on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_destroy(sw4g_ew* ew)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   delete ew->impl;
   delete ew;
   return SW4G_OK;
}

long long sw4g_ew_npts(const sw4g_ew* ew) { return ew ? ew->impl->npts() : -1; }

int sw4g_ew_set_material(sw4g_ew* ew, const double* rho, const double* mu, const double* lambda,
                         int on_device)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   return ew->impl->set_material(rho, mu, lambda, on_device != 0);
}

int sw4g_ew_add_source(sw4g_ew* ew, const sw4g_source* s)
{
   if (!ew || !s) return SW4G_BAD_ARGUMENT;
   return ew->impl->add_source(to_source(s));
}

int sw4g_ew_add_grid_point_sources(sw4g_ew* ew, int n, const int* ijk, const double* amp,
                                   const double* freq, const double* t0, const int* kind)
{
   if (!ew) return SW4G_BAD_ARGUMENT;
   return ew->impl->add_grid_point_sources(n, ijk, amp, freq, t0, kind);
}

int sw4g_ew_clear_sources(sw4g_ew* ew) { return ew ? ew->impl->clear_sources() : SW4G_BAD_ARGUMENT; }

int sw4g_nearest_grid_point(const sw4g_grid* g, double x, double y, double z, int* ijk)
{
   if (!g || !ijk || !(g->h > 0)) return SW4G_BAD_ARGUMENT;
   // src/EW.C:5149-5177 for one Cartesian grid: round to the nearest point, a
   // point exactly half-way going to the lower index
   const double h = g->h;
   int i = (int)std::floor(x / h) + 1;
   if (x - ((i - 0.5) * h) > 0.) i++;
   int j = (int)std::floor(y / h) + 1;
   if (y - ((j - 0.5) * h) > 0.) j++;
   int k = (int)std::floor((z - g->zmin) / h) + 1;
   if (z - (g->zmin + (k - 0.5) * h) > 0.) k++;
   ijk[0] = i;
   ijk[1] = j;
   ijk[2] = k;
   return (i >= 1 && i <= g->nx && j >= 1 && j <= g->ny && k >= 1 && k <= g->nz) ? SW4G_OK
                                                                                : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_receivers(sw4g_ew* ew, int n, const int* ijk, const int* mode, int capacity)
{
   return ew ? ew->impl->set_receivers(n, ijk, mode, capacity) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_receivers_grid(sw4g_ew* ew, int n, const int* ijk, const int* mode, const int* grid,
                               int capacity)
{
   return ew ? ew->impl->set_receivers(n, ijk, mode, capacity, grid) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_nearest_grid_point(const sw4g_ew* ew, double x, double y, double z, int* ijk, int* grid)
{
   return ew ? ew->impl->nearest_grid_point(x, y, z, ijk, grid) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_topography_z(const sw4g_ew* ew, double x, double y, double* z)
{
   if (!ew || !z) return SW4G_BAD_ARGUMENT;
   *z = ew->impl->topography_z(x, y);
   return SW4G_OK;
}

int sw4g_ew_record_shape(const sw4g_ew* ew, int* rows, int* nvals)
{
   return ew ? ew->impl->record_shape(rows, nvals) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_get_records(const sw4g_ew* ew, double* out, int on_device)
{
   return ew ? ew->impl->get_records(out, on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_source_discretization(sw4g_ew* ew, int on_device)
{
   return ew ? ew->impl->set_source_discretization(on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_num_grid_point_sources(const sw4g_ew* ew)
{
   return ew ? ew->impl->num_grid_point_sources() : -1;
}

int sw4g_ew_set_time_step(sw4g_ew* ew, double dt, double t0)
{
   return ew ? ew->impl->set_time_step(dt, t0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_compute_time_step(sw4g_ew* ew, double cfl, double tmax, double* dt, int* nsteps)
{
   return ew ? ew->impl->compute_time_step(cfl, tmax, dt, nsteps) : SW4G_BAD_ARGUMENT;
}

double sw4g_ew_time(const sw4g_ew* ew) { return ew ? ew->impl->time() : 0.0; }

int sw4g_ew_set_graphs(sw4g_ew* ew, int on)
{
   return ew ? ew->impl->set_graphs(on != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_fields(sw4g_ew* ew, const double* u, const double* um, int on_device)
{
   return ew ? ew->impl->set_fields(u, um, on_device != 0) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_get_fields(const sw4g_ew* ew, double* u, double* um, int on_device)
{
   return ew ? ew->impl->get_fields(u, um, on_device != 0) : SW4G_BAD_ARGUMENT;
}

double* sw4g_ew_field(const sw4g_ew* ew, int which)
{
   if (!ew) return nullptr;
   return which == 0 ? ew->impl->field_u() : which == 1 ? ew->impl->field_um() : nullptr;
}

int sw4g_ew_step(sw4g_ew* ew, int nsteps, int mode)
{
   return ew ? ew->impl->step(nsteps, mode) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_set_nan_check(sw4g_ew* ew, int every)
{
   return ew ? ew->impl->set_nan_check(every) : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_nan_report(const sw4g_ew* ew, int* grid, int* c, int* i, int* j, int* k,
                       long long* count, double* t)
{
   if (!ew || !grid || !c || !i || !j || !k || !count || !t) return SW4G_BAD_ARGUMENT;
   const sw4g::EW::NanReport& r = ew->impl->nan_report();
   *grid = r.grid;
   *c = r.c;
   *i = r.i;
   *j = r.j;
   *k = r.k;
   *count = r.count;
   *t = r.t;
   return SW4G_OK;
}

int sw4g_ew_status(sw4g_ew* ew)
{
   return ew ? ew->impl->status() : SW4G_BAD_ARGUMENT;
}

int sw4g_ew_enforce_bc(sw4g_ew* ew, double* u)
{
   if (!ew || !u) return SW4G_BAD_ARGUMENT;
   return ew->impl->enforce_bc(u);
}

int sw4g_ew_launches_per_step(const sw4g_ew* ew, int mode)
{
   return ew ? ew->impl->launches_per_step(mode) : -1;
}

int sw4g_ew_profile_kernels(sw4g_ew* ew, int nrep, double* ms)
{
   if (!ew || !ms) return SW4G_BAD_ARGUMENT;
   return ew->impl->profile_kernels(nrep, ms);
}

int sw4g_dev_set_stage_chunks(int chunks)
{
   if (chunks < 0) return SW4G_BAD_ARGUMENT;
   set_stage_chunks_override(chunks);
   return SW4G_OK;
}

int sw4g_dev_set_mixed_tma(int on)
{
   if (on != 0 && on != 1) return SW4G_BAD_ARGUMENT;
   set_mixed_tma(on);
   return SW4G_OK;
}

int sw4g_dev_set_adjoint_pipeline(int on)
{
   if (on != 0 && on != 1) return SW4G_BAD_ARGUMENT;
   set_adjoint_pipeline(on);
   return SW4G_OK;
}

int sw4g_dev_set_rows_overlap(int on)
{
   if (on != 0 && on != 1) return SW4G_BAD_ARGUMENT;
   set_rows_overlap(on);
   return SW4G_OK;
}

int sw4g_dev_stage_kchunk(long long cols, int nk, int resident, int min_planes, int* planes)
{
   if (!planes || cols < 1 || nk < 1 || resident < 1 || min_planes < 1) return SW4G_BAD_ARGUMENT;
   *planes = stage_kchunk(cols, nk, resident, min_planes);
   return SW4G_OK;
}

}  // extern "C"
