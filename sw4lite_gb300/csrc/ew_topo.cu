// The curvilinear grid of an EW object with topography: set-up and its part of
// each time step (see ew.h).
//
// The reference keeps a list of grids, Cartesian below and one curvilinear grid
// on top (src/EW.C:2018-2046), and runs every phase of the time loop over all of
// them (src/EW.C:2537-2756).  The curvilinear grid's phases here:
//   predictor   rhs4sgcurv(U) with the SBP top rows, then predfort (no forcing:
//               sources lie in the Cartesian grid);
//   BC          bcfortsg on its x/y sides and flat free surface, the curvilinear
//               free-surface ghost plane (freesurfcurvisg) over it, then the
//               interface copy enforceCartTopo (src/EW.C:3446-3530);
//   corrector   dpdmtfort, rhs4sgcurv(Uacc), corrfort, addsgd4cfort.
// Its time levels rotate with the Cartesian grid's: the fused Cartesian
// corrector writes a fourth level, so the curvilinear corrector works in place
// and then swaps its buffer into that slot.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ew.h"
#include "source_weights.h"

namespace sw4g {

CurvGrid::~CurvGrid()
{
   auto f = [](void* p) {
      if (p) cudaFree(p);
   };
   f(z);
   f(met);
   f(jac);
   f(rhoj32);
   f(rho);
   f(mu);
   f(la);
   for (auto* p : lev) f(p);
   f(lu);
   f(uacc);
   f(fzero);
   f(coef);
   f(coefdf);
   f(topscr);
}

namespace {
CurvSpec curv_spec(const CurvGrid& c, const double* u, const double* strx, const double* stry)
{
   CurvSpec s;
   s.soa = 1;
   s.ib = c.b.ib; s.ie = c.b.ie; s.jb = c.b.jb; s.je = c.b.je; s.kb = c.b.kb; s.ke = c.b.ke;
   s.u = u;
   s.mu = c.mu;
   s.la = c.la;
   s.met = c.met;
   s.jac = c.jac;
   s.strx = strx;
   s.stry = stry;
   return s;
}
}  // namespace

int EW::init_topo()
{
   CurvGrid& c = *cv_;
   const TopoSpec& t = c.topo;
   if (!(t.lx > 0) || !(t.ly > 0) || !(t.zeta_break > 0) || t.order < 1) return kBadArgument;
   // topography z range over the array's (x, y) points; the curvilinear grid has
   // nz = 1 + round((zmax - avg)/h) points, avg the midpoint of that range
   // (src/EW.C:2018-2046)
   double zlo = 1e300, zhi = -1e300;
   for (int j = b_.jb; j <= b_.je; j++)
      for (int i = b_.ib; i <= b_.ie; i++) {
         const double x = (i - 1.0) * g_.h, y = (j - 1.0) * g_.h;
         const double zs = -t.amp * std::exp(-(x - t.xc) * (x - t.xc) / (t.lx * t.lx) -
                                             (y - t.yc) * (y - t.yc) / (t.ly * t.ly));
         zlo = std::min(zlo, zs);
         zhi = std::max(zhi, zs);
      }
   const double avg = 0.5 * (zlo + zhi);
   c.nz = 1 + static_cast<int>(std::lround((g_.zmin - avg) / g_.h));
   if (c.nz < 8) return kBadArgument;  // the SBP top rows need 8 planes
   c.b = Bounds{b_.ib, b_.ie, b_.jb, b_.je, -1, c.nz + 2};
   c.npts = c.b.npts();
   const int cbc[6] = {g_.bc[0], g_.bc[1], g_.bc[2], g_.bc[3], kStressFree, kInterface};
   GridSpec cg = g_;
   cg.nz = c.nz;
   for (int s = 0; s < 6; s++) c.bc[s] = cg.bc[s] = cbc[s];
   boundary_windows(cg, c.wind, c.bcpts);

   const size_t n = (size_t)c.npts;
   for (double** p : {&c.z, &c.jac, &c.rho, &c.mu, &c.la})
      SW4G_TRY(cuda_ok(cudaMalloc(p, n * sizeof(double))));
   SW4G_TRY(cuda_ok(cudaMalloc(&c.met, 4 * n * sizeof(double))));
   SW4G_TRY(cuda_ok(cudaMalloc(&c.topscr, 36 * (size_t)(b_.ie - b_.ib + 1) * (b_.je - b_.jb + 1) *
                                              sizeof(double))));
   for (double** p : {&c.lev[0], &c.lev[1], &c.lev[2], &c.lev[3], &c.lu, &c.uacc, &c.fzero}) {
      SW4G_TRY(cuda_ok(cudaMalloc(p, 3 * n * sizeof(double))));
      SW4G_TRY(cuda_ok(cudaMemsetAsync(*p, 0, 3 * n * sizeof(double), stream_)));
   }
   const Bounds& b = c.b;
   SW4G_TRY(launch_gaussian_hill_z(b.ib, b.ie, b.jb, b.je, b.kb, b.ke, c.nz, g_.h, g_.zmin,
                                   t.zeta_break, t.order, t.amp, t.xc, t.yc, t.lx, t.ly, c.z,
                                   stream_));
   int* flag = nullptr;
   SW4G_TRY(cuda_ok(cudaMalloc(&flag, sizeof(int))));
   int bad = 0;
   int st = cuda_ok(cudaMemsetAsync(flag, 0, sizeof(int), stream_));
   if (st == kOk)
      st = launch_metric(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, g_.h, c.z, c.met, c.jac, flag, stream_);
   if (st == kOk) st = cuda_ok(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, stream_));
   if (st == kOk) st = cuda_ok(cudaStreamSynchronize(stream_));
   cudaFree(flag);
   if (st != kOk) return st;
   if (bad) return kBadArgument;  // the grid folds (z_r <= 0): topography too steep for h
   c.hjac.resize(n);
   return cuda_ok(cudaMemcpy(c.hjac.data(), c.jac, n * sizeof(double), cudaMemcpyDeviceToHost));
}

// device: the Jacobian in device memory (the device discretisation), else its host copy
CurvSourceGrid EW::curv_source_grid(bool device) const
{
   const CurvGrid& c = *cv_;
   CurvSourceGrid cs;
   cs.nz = c.nz;
   cs.zmax = g_.zmin;
   cs.amp = c.topo.amp;
   cs.xc = c.topo.xc;
   cs.yc = c.topo.yc;
   cs.lx = c.topo.lx;
   cs.ly = c.topo.ly;
   cs.zeta_break = c.topo.zeta_break;
   cs.order = c.topo.order;
   cs.jac = device ? c.jac : c.hjac.data();
   cs.ib = c.b.ib;
   cs.jb = c.b.jb;
   cs.kb = c.b.kb;
   cs.ni = c.b.ie - c.b.ib + 1;
   cs.nij = cs.ni * (c.b.je - c.b.jb + 1);
   return cs;
}

double EW::topography_z(double x, double y) const
{
   return cv_ ? -curv_source_grid(false).elevation(x, y) : 0.0;
}

int EW::nearest_grid_point(double x, double y, double z, int ijk[3], int* grid) const
{
   if (!ijk || !grid) return kBadArgument;
   if (sub_) return kNotSupported;  // global indices: ask the whole grid's object
   // nearest (i, j); a point exactly half-way goes to the lower index
   const double h = g_.h;
   int i = (int)std::floor(x / h) + 1;
   if (x - ((i - 0.5) * h) > 0.) i++;
   int j = (int)std::floor(y / h) + 1;
   if (y - ((j - 0.5) * h) > 0.) j++;
   if (i < 1 || i > g_.nx || j < 1 || j > g_.ny) return kBadArgument;
   ijk[0] = i;
   ijk[1] = j;
   if (!cv_ || z > g_.zmin) {  // the Cartesian grid
      int k = (int)std::floor((z - g_.zmin) / h) + 1;
      if (z - (g_.zmin + (k - 0.5) * h) > 0.) k++;
      if (k < 1 || k > g_.nz) return kBadArgument;
      ijk[2] = k;
      *grid = 0;
      return kOk;
   }
   // the curvilinear grid: refused above the topography (with the reference's 1e-9
   // allowance); k from the inverted mapping, the surface where it cannot be inverted
   const CurvSourceGrid cs = curv_source_grid(false);
   if (z < -cs.elevation(x, y) - 1e-9) return kBadArgument;
   int k = 1;
   double s = 1;
   if (invert_curvilinear_s(cs, h, x / h + 1, y / h + 1, z, &s))
      k = std::min(std::max((int)std::lround(s), 1), cv_->nz);
   ijk[2] = k;
   *grid = 1;
   return kOk;
}

// Grid-point sources of the curvilinear grid into one of its levels (the reference
// adds F to every grid's predictor and corrector, src/EW.C:2537-2756).
int EW::curv_force(double* lev, int tt, double coef)
{
   if (dsrc_curv_.npoints == 0) return kOk;
   const Bounds& b = cv_->b;
   const double* clk = clocked_ ? dclock_ : nullptr;
   if (mixed_)
      return launch_force_update_df(b.ib, b.ie, b.jb, b.je, b.kb, b.ke, reinterpret_cast<float*>(lev),
                                    cv_->rho, dsrc_curv_, t_, tt, coef, stream_, clk);
   return launch_force_update(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, lev, cv_->rho, dsrc_curv_, t_, tt,
                              coef, stream_, clk);
}

int EW::grid_dims(int grid, int* nx, int* ny, int* nz, long long* npts) const
{
   if (grid < 0 || grid >= num_grids()) return kBadArgument;
   if (nx) *nx = g_.nx;
   if (ny) *ny = g_.ny;
   if (nz) *nz = grid == 0 ? g_.nz : cv_->nz;
   if (npts) *npts = grid == 0 ? npts_ : cv_->npts;
   return kOk;
}

int EW::set_material_grid(int grid, const double* rho, const double* mu, const double* la,
                          bool on_device)
{
   if (grid == 0) return set_material(rho, mu, la, on_device);
   if (grid != 1 || !cv_ || !ready_ || !rho || !mu || !la) return kBadArgument;
   const size_t bytes = (size_t)cv_->npts * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(cv_->rho, rho, bytes, kind, stream_)));
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(cv_->mu, mu, bytes, kind, stream_)));
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(cv_->la, la, bytes, kind, stream_)));
   if (!cv_->coef)
      SW4G_TRY(cuda_ok(cudaMalloc(&cv_->coef, curv_coef_doubles(cv_->npts, (long long)(cv_->b.ie - cv_->b.ib + 1) *
                                                                           (cv_->b.je - cv_->b.jb + 1)) *
                                                 sizeof(double))));
   const Bounds& cb = cv_->b;
   SW4G_TRY(curv_coef_setup(make_box(1, cb.ib, cb.ie, cb.jb, cb.je, cb.kb, cb.ke), cv_->mu, cv_->la,
                            cv_->rho, cv_->met, cv_->jac, dprof_[3], dprof_[4], cv_->coef, &cv_->cc,
                            stream_));
   if (mixed_) {
      if (!cv_->coefdf)
         SW4G_TRY(cuda_ok(cudaMalloc(&cv_->coefdf, curv_coef_df_floats(cv_->npts) * sizeof(float))));
      SW4G_TRY(curv_coef_df_setup(cv_->npts, cv_->cc, cv_->coefdf, &cv_->cd, stream_));
   }
   SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   cv_->material = true;
   cv_->rhoj32_ok = false;  // rho J of the mixed form's 6th-order damping, on next use
   return kOk;
}

int EW::set_fields_grid(int grid, const double* u, const double* um, bool on_device)
{
   if (grid == 0) return set_fields(u, um, on_device);
   if (grid != 1 || !cv_ || !ready_ || !u || !um) return kBadArgument;
   const size_t bytes = 3 * (size_t)cv_->npts * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
   if (!mixed_) {
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(cv_->lev[iu_], u, bytes, kind, stream_)));
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(cv_->lev[ium_], um, bytes, kind, stream_)));
   } else {
      // through the FP64 work array uacc, then split into (hi, lo)
      const long long n3 = 3 * cv_->npts;
      const double* src[2] = {u, um};
      const int dst[2] = {iu_, ium_};
      for (int q = 0; q < 2; q++) {
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(cv_->uacc, src[q], bytes, kind, stream_)));
         float* h = reinterpret_cast<float*>(cv_->lev[dst[q]]);
         SW4G_TRY(launch_df_from_f64(n3, cv_->uacc, h, h + n3, stream_));
      }
   }
   if (!on_device) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   return kOk;
}

int EW::get_fields_grid(int grid, double* u, double* um, bool on_device) const
{
   if (grid == 0) return get_fields(u, um, on_device);
   if (grid != 1 || !cv_ || !ready_) return kBadArgument;
   const size_t bytes = 3 * (size_t)cv_->npts * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
   if (!mixed_) {
      if (u) SW4G_TRY(cuda_ok(cudaMemcpyAsync(u, cv_->lev[iu_], bytes, kind, stream_)));
      if (um) SW4G_TRY(cuda_ok(cudaMemcpyAsync(um, cv_->lev[ium_], bytes, kind, stream_)));
   } else {
      // (hi, lo) -> FP64 in the work array uacc, then out
      const long long n3 = 3 * cv_->npts;
      double* dst[2] = {u, um};
      const int src[2] = {iu_, ium_};
      for (int q = 0; q < 2; q++) {
         if (!dst[q]) continue;
         const float* h = reinterpret_cast<const float*>(cv_->lev[src[q]]);
         SW4G_TRY(launch_df_to_f64(n3, h, h + n3, cv_->uacc, stream_));
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(dst[q], cv_->uacc, bytes, kind, stream_)));
      }
   }
   if (!on_device) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   return kOk;
}

int EW::curvilinear_arrays(double* z, double* met, double* jac, bool on_device) const
{
   if (!cv_ || !ready_) return kBadArgument;
   const size_t bytes = (size_t)cv_->npts * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
   if (z) SW4G_TRY(cuda_ok(cudaMemcpyAsync(z, cv_->z, bytes, kind, stream_)));
   if (met) SW4G_TRY(cuda_ok(cudaMemcpyAsync(met, cv_->met, 4 * bytes, kind, stream_)));
   if (jac) SW4G_TRY(cuda_ok(cudaMemcpyAsync(jac, cv_->jac, bytes, kind, stream_)));
   if (!on_device) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   return kOk;
}

namespace {
CurvStage curv_stage_args(const CurvGrid& c, double* const dprof[9], double dt, double beta)
{
   CurvStage st;
   st.b = make_box(1, c.b.ib, c.b.ie, c.b.jb, c.b.je, c.b.kb, c.b.ke);
   st.nz = c.nz;
   st.cc = c.cc;
   st.sx = dprof[3];
   st.sy = dprof[4];
   st.dcx = dprof[0];
   st.dcy = dprof[1];
   st.cox = dprof[6];
   st.coy = dprof[7];
   st.scratch = c.topscr;
   st.dt = dt;
   st.beta = beta;
   return st;
}
CurvStageDF curv_stage_args_df(const CurvGrid& c, double* const dprof[9], float* const prof32[9],
                               double dt, double beta)
{
   CurvStageDF st;
   st.b = make_box(1, c.b.ib, c.b.ie, c.b.jb, c.b.je, c.b.kb, c.b.ke);
   st.nz = c.nz;
   st.cc = c.cc;
   st.cd = c.cd;
   st.sx = dprof[3];
   st.sy = dprof[4];
   st.dcx = dprof[0];
   st.dcy = dprof[1];
   st.cox = dprof[6];
   st.coy = dprof[7];
   st.sx32 = prof32[3];
   st.sy32 = prof32[4];
   st.dcx32 = prof32[0];
   st.dcy32 = prof32[1];
   st.cox32 = prof32[6];
   st.coy32 = prof32[7];
   st.scratch = c.topscr;
   st.dt = dt;
   st.beta = beta;
   return st;
}

float* df(double* p) { return reinterpret_cast<float*>(p); }
}  // namespace

int EW::curv_pred(int ip) { return curv_pred_part(ip, 0, stream_, 0); }

// The curvilinear predictor in parts: 1 the ghost shell and the SBP top rows (on
// stream s, as a persistent grid of ctas CTAs when ctas > 0), 2 the stage kernel of
// rows 7..nz, 3 the forcing after both; 0 all three on the object's stream.
int EW::curv_pred_part(int ip, int part, cudaStream_t s, int ctas)
{
   CurvGrid& c = *cv_;
   if (part == 3) return curv_force(c.lev[ip], 0, dt_ * dt_);
   const int lp = part == 0 ? 0 : part;  // the launcher's part
   if (mixed_) {
      CurvStageDF st = curv_stage_args_df(c, dprof_, prof32_, dt_, 0.0);
      st.corrector = 0;
      st.u = df(c.lev[iu_]);
      st.um = df(c.lev[ium_]);
      st.out = df(c.lev[ip]);
      st.work1 = c.uacc;
      SW4G_TRY(launch_curv_stage_df(st, part == 1 ? s : stream_, lp, ctas));
   } else {
      // fused: the stage kernel (rows 7..nz), the top-row kernel (rows 1..6) and the
      // ghost shell
      CurvStage st = curv_stage_args(c, dprof_, dt_, 0.0);
      st.corrector = 0;
      st.u = c.lev[iu_];
      st.um = c.lev[ium_];
      st.out = c.lev[ip];
      st.f = c.lev[iu_];
      st.fbox = st.b;
      SW4G_TRY(launch_curv_stage(st, part == 1 ? s : stream_, lp, ctas));
   }
   return part == 0 ? curv_force(c.lev[ip], 0, dt_ * dt_) : kOk;
}

int EW::curv_corr(int ip, int iq) { return curv_corr_part(ip, iq, 0, stream_, 0); }

// The curvilinear corrector in parts as the predictor's (the parts apply to the
// fused form, ip != iq; part 3: the 6th-order damping pass and the forcing).
int EW::curv_corr_part(int ip, int iq, int part, cudaStream_t s, int ctas)
{
   CurvGrid& c = *cv_;
   const Bounds& b = c.b;
   const double dt = dt_;
   const double beta = (prof_.used && g_.sg_damping != 0) ? g_.sg_damping : 0.0;
   const double beta4 = g_.sg_order == 4 ? beta : 0.0;  // 6th order: a separate pass
   const Box cbox = make_box(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke);
   if (mixed_) {
      if (ip == iq) return kNotSupported;
      if (part != 3) {
         CurvStageDF st = curv_stage_args_df(c, dprof_, prof32_, dt, beta4);
         st.corrector = 1;
         st.up = df(c.lev[ip]);
         st.u = df(c.lev[iu_]);
         st.um = df(c.lev[ium_]);
         st.out = df(c.lev[iq]);
         st.work1 = c.uacc;
         st.work2 = c.lu;
         SW4G_TRY(launch_curv_stage_df(st, part == 1 ? s : stream_, part, ctas));
         if (part != 0) return kOk;
      }
      if (beta != 0 && g_.sg_order == 6) {
         if (!c.rhoj32) {
            SW4G_TRY(cuda_ok(cudaMalloc(&c.rhoj32, c.npts * sizeof(float))));
            c.rhoj32_ok = false;
         }
         if (!c.rhoj32_ok) {
            SW4G_TRY(launch_rho_jac_f32(c.npts, c.rho, c.jac, c.rhoj32, stream_));
            c.rhoj32_ok = true;
         }
         const float* dc32[3] = {prof32_[0], prof32_[1], nullptr};
         const float* st32[3] = {prof32_[3], prof32_[4], nullptr};
         const float* co32[3] = {prof32_[6], prof32_[7], nullptr};
         SW4G_TRY(launch_addsgd6_df(2, cbox, df(c.lev[iq]), df(c.lev[iu_]), df(c.lev[ium_]), c.rhoj32,
                                    dc32, st32, co32, beta, stream_));
      }
      return curv_force(c.lev[iq], 1, dt * dt * dt * dt / 12);
   }
   if (ip != iq) {
      // fused: the corrector reads level ip and writes level iq; the top rows read
      // up - 2u + um from a slab of planes kb..8
      if (part != 3) {
         cudaStream_t rs = part == 1 ? s : stream_;
         if (part != 2) {
            const Box full = make_box(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke);
            SW4G_TRY(launch_uacc_slab(full, b.kb, 8, c.lev[ip], c.lev[iu_], c.lev[ium_], c.uacc, rs));
         }
         CurvStage st = curv_stage_args(c, dprof_, dt, beta4);
         st.corrector = 1;
         st.up = c.lev[ip];
         st.u = c.lev[iu_];
         st.um = c.lev[ium_];
         st.out = c.lev[iq];
         st.f = c.uacc;
         st.fbox = make_box(1, b.ib, b.ie, b.jb, b.je, b.kb, 8);
         SW4G_TRY(launch_curv_stage(st, rs, part, ctas));
         if (part != 0) return kOk;
      }
      if (beta != 0 && g_.sg_order == 6)
         SW4G_TRY(launch_addsgd6c(cbox, c.lev[iq], c.lev[iu_], c.lev[ium_], c.rho, dprof_[0], dprof_[1],
                                  dprof_[3], dprof_[4], c.jac, dprof_[6], dprof_[7], beta, stream_));
      return curv_force(c.lev[iq], 1, dt * dt * dt * dt / 12);
   }
   // phase order (in place): the reference's kernel sequence
   const int onesided[6] = {0, 0, 0, 0, 1, 0};
   double *up = c.lev[ip], *u = c.lev[iu_], *um = c.lev[ium_];
   SW4G_TRY(launch_dpdmtfort(b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, u, um, c.uacc, 1 / (dt * dt),
                             stream_));
   SW4G_TRY(launch_rhs4sgcurv(curv_spec(c, c.uacc, dprof_[3], dprof_[4]), onesided, c.lu, stream_));
   SW4G_TRY(launch_corrfort(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, c.lu, c.fzero, c.rho,
                            dt * dt * dt * dt, stream_));
   SW4G_TRY(curv_force(up, 1, dt * dt * dt * dt / 12));
   if (beta != 0 && g_.sg_order == 6)
      SW4G_TRY(launch_addsgd6c(cbox, up, u, um, c.rho, dprof_[0], dprof_[1], dprof_[3], dprof_[4],
                               c.jac, dprof_[6], dprof_[7], beta, stream_));
   else if (beta != 0)
      SW4G_TRY(launch_addsgd4c(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, u, um, c.rho, dprof_[0],
                               dprof_[1], dprof_[3], dprof_[4], c.jac, dprof_[6], dprof_[7],
                               g_.sg_damping, stream_));
   return kOk;
}

int EW::curv_bc(double* ucart, double* ucurv)
{
   CurvGrid& c = *cv_;
   const Bounds& b = c.b;
   if (mixed_) {
      SW4G_TRY(launch_bcfortsg_df(b.ib, b.ie, b.jb, b.je, b.kb, b.ke, c.wind, g_.nx, g_.ny, c.nz, df(ucurv),
                                  g_.h, c.bc, sbop_, c.mu, c.la, dprof_[3], dprof_[4], stream_));
      SW4G_TRY(launch_freesurfcurvisg_df(curv_spec(c, nullptr, dprof_[3], dprof_[4]), c.nz, 5, sbop_,
                                         df(ucurv), stream_));
      return launch_cart_topo_df(make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke),
                                 make_box(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke), c.nz, df(ucart),
                                 df(ucurv), stream_);
   }
   SW4G_TRY(launch_bcfortsg(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, c.wind, g_.nx, g_.ny, c.nz, ucurv,
                            g_.h, c.bc, sbop_, c.mu, c.la, nullptr, dprof_[3], dprof_[4], stream_));
   SW4G_TRY(launch_freesurfcurvisg(curv_spec(c, ucurv, dprof_[3], dprof_[4]), c.nz, 5, sbop_,
                                   nullptr, ucurv, stream_));
   return launch_cart_topo(make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke),
                           make_box(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke), c.nz, ucart, ucurv,
                           stream_);
}

int EW::curv_time_step(double cfl, double* dt)
{
   CurvGrid& c = *cv_;
   if (!c.material) return kBadArgument;
   const int nb = 152 * 4;
   double* bm = nullptr;
   SW4G_TRY(cuda_ok(cudaMalloc(&bm, nb * sizeof(double))));
   std::vector<double> h(nb);
   int st = launch_curv_eig(1, c.npts, c.rho, c.mu, c.la, c.met, c.jac, bm, nb, stream_);
   if (st == kOk)
      st = cuda_ok(cudaMemcpyAsync(h.data(), bm, nb * sizeof(double), cudaMemcpyDeviceToHost, stream_));
   if (st == kOk) st = cuda_ok(cudaStreamSynchronize(stream_));
   cudaFree(bm);
   if (st != kOk) return st;
   double e = -1;
   for (double v : h) e = std::max(e, v);
   if (!(e > 0)) return kBadArgument;
   *dt = cfl / std::sqrt(e);
   return kOk;
}

int EW::curv_launches(int mode) const
{
   if (!cv_) return 0;
   int bc = 1 /* free surface */ + 1 /* interface copy */;
   for (int s = 0; s < 4; s++) {
      const int t = cv_->bc[s];
      if ((t == kDirichlet || t == kSuperGrid || t == kPeriodic) && cv_->bcpts[s] > 0) bc++;
   }
   bc++;  // flat free surface of bcfortsg on the top side
   const bool damp = prof_.used && g_.sg_damping != 0;
   // predictor (both modes): shell, top-row column pass, top rows, stage kernel;
   // the mixed form adds the FP64 slab of u
   const int pred = mixed_ ? 5 : 4;
   // corrector: slab, shell, top-row column pass, top rows, stage (the mixed form
   // adds the slab of u - um); phase order dpdm, two operator kernels, corrfort,
   // damping
   const int corr = mode == kModeFused ? (mixed_ ? 6 : 5) : 4 + (damp ? 1 : 0);
   const int force = hsrc_curv_.empty() ? 0 : 2;
   return pred + corr + 2 * bc + force;
}

}  // namespace sw4g
