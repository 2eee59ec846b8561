// Host-side time loop for one Cartesian grid; see ew.h.
#include "ew.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "sbp.h"
#include "source_weights.h"

namespace sw4g {

EW::EW(const GridSpec& g, cudaStream_t stream, const TopoSpec* topo) : g_(g), stream_(stream)
{
   if (topo) {
      cv_.reset(new CurvGrid());
      cv_->topo = *topo;
   }
}

EW::~EW()
{
   drop_graphs();
   drop_grad_cache();
   if (side_) {
      cudaStreamSynchronize(side_);
      cudaStreamDestroy(side_);
   }
   if (ev_fork_) cudaEventDestroy(ev_fork_);
   if (ev_join_) cudaEventDestroy(ev_join_);
   auto f = [](void* p) {
      if (p) cudaFree(p);
   };
   f(dclock_);
   f(dstat_);
   for (auto* p : xbuf_) f(p);
   f(rho_);
   f(mu_);
   f(la_);
   f(irho_);
   for (auto* p : dprof_) f(p);
   f(wstore_);
   for (auto* p : lev_) f(p);
   f(lu_);
   f(f_);
   f(uacc_);
   f(slab_);
   f(zc_[0]);
   f(zc_[1]);
   f(dsrc_mem_);
   f(dsrc_curv_mem_);
   f(rscr_);
   f(drec_mem_);
   f(records_);
   f(rho32_);
   f(mu32_);
   f(la32_);
   f(irho32_);
   f(wdf_);
   for (auto* p : prof32_) f(p);
   f(staging_);
}

int EW::init()
{
   if (g_.nx < 8 || g_.ny < 8 || g_.nz < 8 || !(g_.h > 0)) return kBadArgument;
   if (g_.soa != 1) return kNotSupported;  // the time loop keeps fields component-major
   for (int s = 0; s < 6; s++) {
      const int t = g_.bc[s];
      if (s == 4 && cv_) {
         if (t != kInterface) return kBadArgument;  // the top is the curvilinear grid
         continue;
      }
      if (t == kProcessor && sub_ && s < 4) continue;  // a side shared with a neighbour
      if (!(t == kStressFree || t == kDirichlet || t == kSuperGrid || t == kPeriodic)) return kBadArgument;
      if (t == kStressFree && s < 4) return kNotSupported;
   }
   if (g_.sg_order != 4 && g_.sg_order != 6) return kBadArgument;
   if (g_.precision != 0 && g_.precision != 1) return kBadArgument;
   mixed_ = g_.precision == 1;
   if ((g_.bc[4] == kStressFree && g_.nz < 14) || (g_.bc[5] == kStressFree && g_.nz < 14))
      return kBadArgument;  // the one-sided rows need 8 interior planes on each such side
   b_ = grid_bounds(g_);
   npts_ = b_.npts();
   boundary_windows(g_, wind_, bcpts_);
   onesided_flags(g_, onesided_);
   double acof[384], ghcof[6], bope[48];
   sbp_coefficients(acof, ghcof, bope, sbop_);
   prof_ = sub_ ? subdomain_profiles(global_, g_, ioff_, joff_) : supergrid_profiles(g_);

   const size_t n = (size_t)npts_;
   SW4G_TRY(cuda_ok(cudaGetDevice(&dev_)));
   if (sub_) {
      const size_t hb = (size_t)std::max(halo_bytes(0), halo_bytes(1));
      for (auto*& p : xbuf_) SW4G_TRY(cuda_ok(cudaMalloc(&p, hb)));
   }
   SW4G_TRY(cuda_ok(cudaMalloc(&dstat_, 4 * sizeof(unsigned long long))));
   {
      const unsigned long long init[4] = {0, 0, ~0ull, 0};
      SW4G_TRY(cuda_ok(cudaMemcpy(dstat_, init, sizeof init, cudaMemcpyHostToDevice)));
   }
   SW4G_TRY(cuda_ok(cudaMalloc(&rho_, n * sizeof(double))));
   SW4G_TRY(cuda_ok(cudaMalloc(&mu_, n * sizeof(double))));
   SW4G_TRY(cuda_ok(cudaMalloc(&la_, n * sizeof(double))));
   SW4G_TRY(cuda_ok(cudaMalloc(&irho_, n * sizeof(double))));
   if (!mixed_) {
      SW4G_TRY(cuda_ok(cudaMalloc(&wstore_, (kWeightArrays + kWeightSums) * n * sizeof(double))));
      for (int q = 0; q < kWeightArrays; q++) w_.p[q] = wstore_ + q * n;
      for (int q = 0; q < kWeightSums; q++) w_.s[q] = wstore_ + (kWeightArrays + q) * n;
   } else {
      SW4G_TRY(cuda_ok(cudaMalloc(&rho32_, n * sizeof(float))));
      SW4G_TRY(cuda_ok(cudaMalloc(&mu32_, 2 * n * sizeof(float))));
      SW4G_TRY(cuda_ok(cudaMalloc(&la32_, 2 * n * sizeof(float))));
      SW4G_TRY(cuda_ok(cudaMalloc(&irho32_, 2 * n * sizeof(float))));
      SW4G_TRY(cuda_ok(cudaMalloc(&wdf_, 2 * kWeightArrays * n * sizeof(float))));
      for (int q = 0; q < kWeightArrays; q++) wd_.p[q] = reinterpret_cast<float2*>(wdf_) + q * n;
   }
   // a level holds 3*npts doubles, or in the mixed form 3*npts hi + 3*npts lo floats
   // (the same bytes)
   for (int q = 0; q < 4; q++) {
      SW4G_TRY(cuda_ok(cudaMalloc(&lev_[q], 3 * n * sizeof(double))));
      SW4G_TRY(cuda_ok(cudaMemsetAsync(lev_[q], 0, 3 * n * sizeof(double), stream_)));
   }
   const int len[3] = {b_.ie - b_.ib + 1, b_.je - b_.jb + 1, b_.ke - b_.kb + 1};
   for (int w = 0; w < 3; w++)
      for (int ax = 0; ax < 3; ax++) {
         double*& d = dprof_[3 * w + ax];
         SW4G_TRY(cuda_ok(cudaMalloc(&d, len[ax] * sizeof(double))));
         const std::vector<double>& src = w == 0 ? prof_.dc[ax] : w == 1 ? prof_.str[ax] : prof_.co[ax];
         SW4G_TRY(cuda_ok(cudaMemcpy(d, src.data(), len[ax] * sizeof(double), cudaMemcpyHostToDevice)));
         if (mixed_) {
            float*& d32 = prof32_[3 * w + ax];
            SW4G_TRY(cuda_ok(cudaMalloc(&d32, len[ax] * sizeof(float))));
            SW4G_TRY(launch_to_f32(len[ax], d, d32, stream_));
         }
      }
   // slab for the corrector's stage field on the one-sided rows: planes kb..8
   // (top) or nz-7..ke (bottom)
   const long long nij = (long long)len[0] * len[1];
   slab_len_ = 3 * nij * 10;
   if (onesided_[4] || onesided_[5]) {  // the mixed form also keeps u - um slabs
      SW4G_TRY(cuda_ok(cudaMalloc(&slab_, (mixed_ ? 4 : 2) * slab_len_ * sizeof(double))));
      SW4G_TRY(cuda_ok(cudaMalloc(&rscr_, 42 * nij * sizeof(double))));
   }
   {
      const Box bx = make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke);
      for (int side = 0; side < 2; side++)
         if (onesided_[4 + side])
            SW4G_TRY(cuda_ok(cudaMalloc(&zc_[side], zcoef_len(bx) * sizeof(double))));
   }
   SW4G_TRY(upload_sbp_tables_direct());
   if (cv_) SW4G_TRY(init_topo());
   SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   // the rows' second stream, made here rather than inside a graph capture
   if (onesided_[4] || onesided_[5] || cv_) SW4G_TRY(side_stream());
   ready_ = true;
   return kOk;
}

const double* EW::profile(int which, int axis) const
{
   if (which < 0 || which > 2 || axis < 0 || axis > 2) return nullptr;
   return dprof_[3 * which + axis];
}

int EW::set_material(const double* rho, const double* mu, const double* la, bool on_device)
{
   if (!ready_ || !rho || !mu || !la) return kBadArgument;
   const size_t bytes = (size_t)npts_ * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(rho_, rho, bytes, kind, stream_)));
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(mu_, mu, bytes, kind, stream_)));
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(la_, la, bytes, kind, stream_)));
   SW4G_TRY(launch_inverse(npts_, rho_, irho_, stream_));
   Box b = make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke);
   for (int side = 0; side < 2; side++)
      if (zc_[side]) SW4G_TRY(launch_zcoef(b, g_.nz, side == 0, mu_, la_, zc_[side], stream_));
   if (!mixed_) {
      SW4G_TRY(launch_weights(b, mu_, la_, dprof_[3], dprof_[4], dprof_[5], g_.h, w_, stream_));
   } else {
      SW4G_TRY(launch_to_f32(npts_, rho_, rho32_, stream_));
      SW4G_TRY(launch_df2_from_f64(npts_, mu_, reinterpret_cast<float2*>(mu32_), stream_));
      SW4G_TRY(launch_df2_from_f64(npts_, la_, reinterpret_cast<float2*>(la32_), stream_));
      SW4G_TRY(launch_df2_from_f64(npts_, irho_, reinterpret_cast<float2*>(irho32_), stream_));
      SW4G_TRY(launch_weights_df(b, mu_, la_, dprof_[3], dprof_[4], dprof_[5], wd_, stream_));
   }
   SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   material_ = true;
   return kOk;
}

int EW::add_source(const SourceSpec& s)
{
   if (!ready_) return kBadArgument;
   if (s.kind < 0 || s.kind > 3 || !(s.freq > 0)) return kBadArgument;
   if (dev_src_) {  // discretised with the whole batch before the next step
      if (cv_) {
         // the same refusals as the host path: above the topography, or where the
         // grid mapping cannot be inverted (the stencil needs no Jacobian)
         const CurvSourceGrid cs = curv_source_grid(false);
         TopoStencil st;
         if (topo_stencil(g_, onesided_, cs, s, st) != 0) return kBadArgument;
      }
      specs_.push_back(s);
      src_dirty_ = true;
      return kOk;
   }
   if (cv_) {
      // two grids: the source may go to either, or straddle the interface
      const CurvSourceGrid cs = curv_source_grid(false);
      if (discretize_source_topo(g_, onesided_, &cs, s, hsrc_, hsrc_curv_) != 0) return kBadArgument;
   } else {
      discretize_into(s, hsrc_);
   }
   specs_.push_back(s);
   src_dirty_ = true;
   return kOk;
}

void EW::discretize_into(const SourceSpec& s, std::vector<GridPointSource>& out) const
{
   if (!sub_) {
      discretize_source(g_, onesided_, s, out);
      return;
   }
   // the global grid's grid-point sources, in the reference's order, on this
   // subdomain's interior points (src/Source.C: interior_point_in_proc)
   std::vector<GridPointSource> all;
   discretize_source(global_, onesided_, s, all);
   for (GridPointSource p : all) {
      p.i -= ioff_;
      p.j -= joff_;
      if (p.i >= 1 && p.i <= g_.nx && p.j >= 1 && p.j <= g_.ny) out.push_back(p);
   }
}

int EW::set_subdomain(const GridSpec& global, int ioff, int joff)
{
   if (ready_) return kBadArgument;
   if (ioff < 0 || joff < 0 || ioff + g_.nx > global.nx || joff + g_.ny > global.ny) return kBadArgument;
   global_ = global;
   ioff_ = ioff;
   joff_ = joff;
   sub_ = true;
   return kOk;
}

int EW::add_grid_point_sources(int n, const int* ijk, const double* amp, const double* freq,
                               const double* t0, const int* kind)
{
   if (!ready_ || n < 0 || (n > 0 && (!ijk || !amp || !freq || !t0 || !kind))) return kBadArgument;
   if (dev_src_) return kNotSupported;
   raw_src_ += n;
   for (int s = 0; s < n; s++) {
      GridPointSource p;
      p.i = ijk[3 * s];
      p.j = ijk[3 * s + 1];
      p.k = ijk[3 * s + 2];
      if (p.i < 1 || p.i > g_.nx || p.j < 1 || p.j > g_.ny || p.k < 1 || p.k > g_.nz)
         return kBadArgument;
      if (kind[s] < 0 || kind[s] > 3) return kBadArgument;
      for (int c = 0; c < 3; c++) p.amp[c] = amp[3 * s + c];
      p.freq = freq[s];
      p.t0 = t0[s];
      p.kind = kind[s];
      hsrc_.push_back(p);
   }
   src_dirty_ = true;
   return kOk;
}

int EW::clear_sources()
{
   hsrc_.clear();
   hsrc_curv_.clear();
   specs_.clear();
   raw_src_ = 0;
   src_dirty_ = true;
   return kOk;
}

int EW::set_source_discretization(bool on_device)
{
   if (!ready_) return kBadArgument;
   if (on_device && (raw_src_ > 0 || sub_)) return kNotSupported;
   if (on_device == dev_src_) return kOk;
   dev_src_ = on_device;
   if (!on_device) {  // the host lists from the sources added meanwhile
      hsrc_.clear();
      hsrc_curv_.clear();
      const CurvSourceGrid cs = cv_ ? curv_source_grid(false) : CurvSourceGrid{};
      for (const SourceSpec& s : specs_) {
         if (cv_)
            discretize_source_topo(g_, onesided_, &cs, s, hsrc_, hsrc_curv_);
         else
            discretize_into(s, hsrc_);
      }
   }
   src_dirty_ = true;
   return kOk;
}

int EW::num_grid_point_sources() const
{
   if (!dev_src_) return (int)hsrc_.size();
   std::vector<GridPointSource> v;
   return grid_point_sources(0, &v) == kOk ? (int)v.size() : -1;
}

namespace {
// One device block per source set: start | ijk | kind | amp | freq | t0 (ints first,
// then doubles, 8-aligned).
int pack_sources(std::vector<GridPointSource> src, SourceSet& ds, void*& mem)
{
   std::vector<int> start;
   group_sources(src, start);
   const int ns = (int)src.size(), np = (int)start.size() - 1;
   const size_t ints = (size_t)(np + 1) + 3 * (size_t)ns + ns;
   const size_t int_bytes = ((ints * sizeof(int) + 7) / 8) * 8;
   const size_t bytes = int_bytes + (5 * (size_t)ns) * sizeof(double);
   if (mem) {
      cudaFree(mem);
      mem = nullptr;
   }
   ds = SourceSet{};
   if (ns == 0) return kOk;
   std::vector<unsigned char> host(bytes, 0);
   int* hi = reinterpret_cast<int*>(host.data());
   for (int r = 0; r <= np; r++) hi[r] = start[r];
   int* hijk = hi + np + 1;
   int* hkind = hijk + 3 * ns;
   double* hd = reinterpret_cast<double*>(host.data() + int_bytes);
   double* hamp = hd;
   double* hfreq = hamp + 3 * ns;
   double* ht0 = hfreq + ns;
   for (int s = 0; s < ns; s++) {
      hijk[3 * s] = src[s].i;
      hijk[3 * s + 1] = src[s].j;
      hijk[3 * s + 2] = src[s].k;
      hkind[s] = src[s].kind;
      for (int c = 0; c < 3; c++) hamp[3 * s + c] = src[s].amp[c];
      hfreq[s] = src[s].freq;
      ht0[s] = src[s].t0;
   }
   SW4G_TRY(cuda_ok(cudaMalloc(&mem, bytes)));
   SW4G_TRY(cuda_ok(cudaMemcpy(mem, host.data(), bytes, cudaMemcpyHostToDevice)));
   unsigned char* base = static_cast<unsigned char*>(mem);
   const int* di = reinterpret_cast<const int*>(base);
   const double* dd = reinterpret_cast<const double*>(base + int_bytes);
   ds.npoints = np;
   ds.nsources = ns;
   ds.start = di;
   ds.ijk = di + np + 1;
   ds.kind = di + np + 1 + 3 * ns;
   ds.amp = dd;
   ds.freq = dd + 3 * ns;
   ds.t0 = dd + 4 * ns;
   return kOk;
}
}  // namespace

int EW::upload_sources()
{
   if (!src_dirty_) return kOk;
   drop_graphs();  // the graphs hold the old source list
   if (dsrc_mem_ || dsrc_curv_mem_) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   src_dirty_ = false;
   if (dev_src_ && cv_)
      return launch_discretize_sources_topo(g_, onesided_, curv_source_grid(true), (int)specs_.size(),
                                            specs_.data(), &dsrc_, &dsrc_mem_, &dsrc_curv_, &dsrc_curv_mem_,
                                            stream_);
   if (dev_src_)
      return launch_discretize_sources(g_, onesided_, (int)specs_.size(), specs_.data(), &dsrc_, &dsrc_mem_,
                                       stream_);
   SW4G_TRY(pack_sources(hsrc_, dsrc_, dsrc_mem_));
   return pack_sources(hsrc_curv_, dsrc_curv_, dsrc_curv_mem_);
}

int EW::grid_point_sources(int grid, std::vector<GridPointSource>* out) const
{
   if (grid < 0 || grid >= num_grids() || !out) return kBadArgument;
   if (!dev_src_) {
      *out = grid == 0 ? hsrc_ : hsrc_curv_;
      return kOk;
   }
   // the device list, grouped by grid point; discretised first if it is not yet (a
   // cache refresh: the object's observable state does not change)
   EW* self = const_cast<EW*>(this);
   SW4G_TRY(self->upload_sources());
   const SourceSet& ds = grid == 0 ? dsrc_ : dsrc_curv_;
   const int ns = ds.nsources;
   out->assign(ns, GridPointSource{});
   if (ns == 0) return kOk;
   std::vector<int> ijk(3 * (size_t)ns), kind(ns);
   std::vector<double> amp(3 * (size_t)ns), freq(ns), t0(ns);
   SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   SW4G_TRY(cuda_ok(cudaMemcpy(ijk.data(), ds.ijk, ijk.size() * sizeof(int), cudaMemcpyDeviceToHost)));
   SW4G_TRY(cuda_ok(cudaMemcpy(kind.data(), ds.kind, kind.size() * sizeof(int), cudaMemcpyDeviceToHost)));
   SW4G_TRY(cuda_ok(cudaMemcpy(amp.data(), ds.amp, amp.size() * sizeof(double), cudaMemcpyDeviceToHost)));
   SW4G_TRY(cuda_ok(cudaMemcpy(freq.data(), ds.freq, freq.size() * sizeof(double), cudaMemcpyDeviceToHost)));
   SW4G_TRY(cuda_ok(cudaMemcpy(t0.data(), ds.t0, t0.size() * sizeof(double), cudaMemcpyDeviceToHost)));
   for (int s = 0; s < ns; s++) {
      GridPointSource& p = (*out)[s];
      p.i = ijk[3 * s];
      p.j = ijk[3 * s + 1];
      p.k = ijk[3 * s + 2];
      for (int c = 0; c < 3; c++) p.amp[c] = amp[3 * s + c];
      p.freq = freq[s];
      p.t0 = t0[s];
      p.kind = kind[s];
   }
   return kOk;
}

int EW::set_time_step(double dt, double t0)
{
   if (!(dt > 0)) return kBadArgument;
   if (dt != dt_) drop_graphs();
   dt_ = dt;
   t_ = t0;
   return kOk;
}

int EW::compute_time_step(double cfl, double tmax, double* dt, int* nsteps)
{
   if (!material_ || !(cfl > 0)) return kBadArgument;
   const size_t n = (size_t)npts_;
   std::vector<double> r(n), m(n), l(n);
   SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   SW4G_TRY(cuda_ok(cudaMemcpy(r.data(), rho_, n * sizeof(double), cudaMemcpyDeviceToHost)));
   SW4G_TRY(cuda_ok(cudaMemcpy(m.data(), mu_, n * sizeof(double), cudaMemcpyDeviceToHost)));
   SW4G_TRY(cuda_ok(cudaMemcpy(l.data(), la_, n * sizeof(double), cudaMemcpyDeviceToHost)));
   int ns = 0;
   double d = cfl_time_step(g_, r.data(), m.data(), l.data(), cfl, t_, tmax, &ns);
   if (!(d > 0) || !(tmax > t_)) return kBadArgument;
   if (cv_) {
      // min over both grids of the raw limits, then land on tmax (src/EW.C:5041-5146)
      double eigmax = -1;
      for (size_t p = 0; p < n; p++) eigmax = std::max(eigmax, (4 * m[p] + l[p]) / r[p]);
      double dc = cfl * g_.h * (1 / std::sqrt(eigmax)), dv = 0;
      SW4G_TRY(curv_time_step(cfl, &dv));
      dc = std::min(dc, dv);
      if (!((tmax - t_) / dc < 2.0e9)) return kBadArgument;
      ns = static_cast<int>((tmax - t_) / dc + 0.5);
      ns = ns == 0 ? 1 : ns;
      d = (tmax - t_) / ns;
   }
   if (d != dt_) drop_graphs();
   dt_ = d;
   if (dt) *dt = d;
   if (nsteps) *nsteps = ns;
   return kOk;
}

int EW::ensure_staging()
{
   if (staging_) return kOk;
   return cuda_ok(cudaMalloc(&staging_, 3 * (size_t)npts_ * sizeof(double)));
}

int EW::set_fields(const double* u, const double* um, bool on_device)
{
   if (!ready_ || !u || !um) return kBadArgument;
   const size_t bytes = 3 * (size_t)npts_ * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
   if (!mixed_) {
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[iu_], u, bytes, kind, stream_)));
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[ium_], um, bytes, kind, stream_)));
      return kOk;
   }
   const long long n3 = 3 * npts_;
   const double* src[2] = {u, um};
   const int dst[2] = {iu_, ium_};
   for (int q = 0; q < 2; q++) {
      const double* from = src[q];
      if (!on_device) {
         SW4G_TRY(ensure_staging());
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(staging_, src[q], bytes, kind, stream_)));
         from = staging_;
      }
      float* h = reinterpret_cast<float*>(lev_[dst[q]]);
      SW4G_TRY(launch_df_from_f64(n3, from, h, h + n3, stream_));
   }
   return kOk;
}

int EW::get_fields(double* u, double* um, bool on_device) const
{
   if (!ready_) return kBadArgument;
   const size_t bytes = 3 * (size_t)npts_ * sizeof(double);
   const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
   if (!mixed_) {
      if (u) SW4G_TRY(cuda_ok(cudaMemcpyAsync(u, lev_[iu_], bytes, kind, stream_)));
      if (um) SW4G_TRY(cuda_ok(cudaMemcpyAsync(um, lev_[ium_], bytes, kind, stream_)));
   } else {
      const long long n3 = 3 * npts_;
      double* dst[2] = {u, um};
      const int srcl[2] = {iu_, ium_};
      for (int q = 0; q < 2; q++) {
         if (!dst[q]) continue;
         const float* h = reinterpret_cast<const float*>(lev_[srcl[q]]);
         if (on_device) {
            SW4G_TRY(launch_df_to_f64(n3, h, h + n3, dst[q], stream_));
         } else {
            SW4G_TRY(const_cast<EW*>(this)->ensure_staging());
            SW4G_TRY(launch_df_to_f64(n3, h, h + n3, staging_, stream_));
            SW4G_TRY(cuda_ok(cudaMemcpyAsync(dst[q], staging_, bytes, kind, stream_)));
         }
      }
   }
   if (!on_device) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   return kOk;
}

int EW::enforce_bc(double* u)
{
   if (mixed_)  // levels are double-float pairs in the mixed form
      return launch_bcfortsg_df(b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke, wind_, g_.nx, g_.ny, g_.nz,
                                reinterpret_cast<float*>(u), g_.h, g_.bc, sbop_, mu_, la_, dprof_[3],
                                dprof_[4], stream_);
   return launch_bcfortsg(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke, wind_, g_.nx, g_.ny, g_.nz,
                          u, g_.h, g_.bc, sbop_, mu_, la_, nullptr, dprof_[3], dprof_[4], stream_);
}

int EW::ensure_phase_arrays()
{
   if (lu_) return kOk;
   const size_t bytes = 3 * (size_t)npts_ * sizeof(double);
   SW4G_TRY(cuda_ok(cudaMalloc(&lu_, bytes)));
   SW4G_TRY(cuda_ok(cudaMalloc(&f_, bytes)));
   SW4G_TRY(cuda_ok(cudaMalloc(&uacc_, bytes)));
   SW4G_TRY(cuda_ok(cudaMemsetAsync(lu_, 0, bytes, stream_)));
   SW4G_TRY(cuda_ok(cudaMemsetAsync(uacc_, 0, bytes, stream_)));
   return kOk;
}

int EW::step(int nsteps, int mode)
{
   if (!ready_ || !material_ || !(dt_ > 0) || nsteps < 0) return kBadArgument;
   if (sub_) return kNotSupported;  // a subdomain steps by step_part with halo exchanges
   if (cv_ && !cv_->material) return kBadArgument;
   if (mode != kModePhases && mode != kModeFused) return kBadArgument;
   if (mixed_ && mode == kModePhases) return kNotSupported;
   if (drec_.n > 0 && rec_rows_ + (rec_initial_ ? 1 : 0) + nsteps > rec_cap_) return kBadArgument;
   SW4G_TRY(upload_sources());
   if (mode == kModePhases) SW4G_TRY(ensure_phase_arrays());
   if (drec_.n > 0 && rec_initial_) {
      SW4G_TRY(record(iu_, ium_, 1));
      rec_initial_ = false;
   }
   auto advance = [&](int k) -> int {
      if (mode == kModeFused && graphs_) return run_graphed(k);
      for (int n = 0; n < k; n++) SW4G_TRY(mode == kModePhases ? step_phases() : step_fused());
      return kOk;
   };
   if (nan_every_ <= 0) return advance(nsteps);
   for (int done = 0; done < nsteps;) {
      const int k = std::min(nan_every_, nsteps - done);
      SW4G_TRY(advance(k));
      done += k;
      SW4G_TRY(scan_levels());
   }
   return kOk;
}

int EW::set_nan_check(int every)
{
   if (!ready_ || every < 0) return kBadArgument;
   nan_every_ = every;
   nan_ = NanReport{};
   return kOk;
}

int EW::read_status(unsigned long long out[4])
{
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(out, dstat_, 4 * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, stream_)));
   return cuda_ok(cudaStreamSynchronize(stream_));
}

int EW::status()
{
   if (!ready_) return kBadArgument;
   unsigned long long h[4];
   SW4G_TRY(read_status(h));
   if (h[0] & (1ull << kTimeout)) {
      const unsigned long long zero = 0;
      SW4G_TRY(cuda_ok(cudaMemcpy(dstat_, &zero, sizeof zero, cudaMemcpyHostToDevice)));
      return kTimeout;
   }
   return kOk;
}

// Scans the current level of every grid (the level the last step wrote) for NaN and
// infinite values and reads the outcome: kNanDetected with nan_ filled in, kTimeout
// if a kernel's bounded wait gave up, else kOk.
int EW::scan_levels()
{
   const unsigned long long reset[2] = {0, ~0ull};
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(dstat_ + 1, reset, sizeof reset, cudaMemcpyHostToDevice, stream_)));
   const long long n0 = (mixed_ ? 6 : 3) * npts_;
   SW4G_TRY(launch_nonfinite_scan(lev_[iu_], n0, mixed_, 0, dstat_, stream_));
   if (cv_) {
      const long long n1 = (mixed_ ? 6 : 3) * cv_->npts;
      SW4G_TRY(launch_nonfinite_scan(cv_->lev[iu_], n1, mixed_, 1, dstat_, stream_));
   }
   unsigned long long h[4];
   SW4G_TRY(read_status(h));  // also orders the reset's host buffer before this frame ends
   if (h[0] & (1ull << kTimeout)) return kTimeout;
   if (h[1] == 0) return kOk;
   const int grid = (int)(h[2] >> kScanGridShift);
   long long off = (long long)(h[2] & ((1ull << kScanGridShift) - 1));
   const Bounds& b = grid == 0 ? b_ : cv_->b;
   const long long np = b.npts();
   off %= 3 * np;  // the mixed form's lo half holds the same points
   const long long ni = b.ie - b.ib + 1, nij = ni * (b.je - b.jb + 1);
   const long long p = off % np;
   nan_.grid = grid;
   nan_.c = (int)(off / np);
   nan_.i = b.ib + (int)(p % ni);
   nan_.j = b.jb + (int)((p / ni) % (b.je - b.jb + 1));
   nan_.k = b.kb + (int)(p / nij);
   nan_.count = (long long)h[1];
   nan_.t = t_;
   return kNanDetected;
}

int EW::record(int iup, int ium, int initial)
{
   // with the device clock the kernel takes its row from clock[1]
   const double* clk = clocked_ ? dclock_ : nullptr;
   double* row = clk ? records_ : records_ + (size_t)rec_rows_ * rec_nvals_;
   RecCurv rc;
   if (rec_curv_) {
      const Bounds& cb = cv_->b;
      rc.b = make_box(1, cb.ib, cb.ie, cb.jb, cb.je, cb.kb, cb.ke);
      rc.up = cv_->lev[iup];
      rc.um = cv_->lev[ium];
      rc.met = cv_->met;
      rc.jac = cv_->jac;
   }
   const Box b = make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke);
   if (mixed_)
      SW4G_TRY(launch_record_df(b, reinterpret_cast<const float*>(lev_[iup]),
                                reinterpret_cast<const float*>(lev_[ium]), drec_, row, dt_, g_.h, initial,
                                stream_, clk, rec_nvals_, rec_curv_ ? &rc : nullptr));
   else
      SW4G_TRY(launch_record(b, lev_[iup], lev_[ium], drec_, row, dt_, g_.h, initial, stream_, clk, rec_nvals_,
                             rec_curv_ ? &rc : nullptr));
   rec_rows_++;
   return kOk;
}

int EW::set_graphs(bool on)
{
   if (!ready_) return kBadArgument;
   if (on && !stream_) return kNotSupported;  // no stream capture on the legacy default stream
   if (on && !dclock_) SW4G_TRY(cuda_ok(cudaMalloc(&dclock_, 4 * sizeof(double))));
   if (!on) drop_graphs();
   graphs_ = on;
   return kOk;
}

void EW::drop_graphs()
{
   if (!graph_cache_.empty()) cudaStreamSynchronize(stream_);
   for (GraphKey& g : graph_cache_) cudaGraphExecDestroy(g.exec);
   graph_cache_.clear();
}

// The device clock from the host's time, record row and (adjoint) residual row.
int EW::sync_clock(double res_row)
{
   const double h[3] = {t_, (double)rec_rows_, res_row};
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(dclock_, h, sizeof(h), cudaMemcpyHostToDevice, stream_)));
   return cuda_ok(cudaStreamSynchronize(stream_));  // h lives on this stack frame
}

int EW::capture(const std::function<int()>& body, cudaGraphExec_t* exec)
{
   *exec = nullptr;
   SW4G_TRY(cuda_ok(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal)));
   const int st = body();
   cudaGraph_t g = nullptr;
   const cudaError_t e = cudaStreamEndCapture(stream_, &g);
   if (st != kOk || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return st != kOk ? st : kCudaError;
   }
   const cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
   cudaGraphDestroy(g);
   return ei == cudaSuccess ? kOk : kCudaError;
}

// Fused steps with the device clock; chunks of kGraphSteps steps that start in the
// level rotation's 3-cycle replay a graph cached by (rotation state, recording), the
// rest run directly.
int EW::run_graphed(int nsteps)
{
   if (!dclock_) return kBadArgument;
   if (!warm_ && nsteps > 0) {  // first launches (and their attribute set-up) outside capture
      SW4G_TRY(step_fused());
      warm_ = true;
      nsteps--;
   }
   SW4G_TRY(sync_clock());
   clocked_ = true;
   auto in_cycle = [&]() {
      return (iu_ == 2 && ium_ == 3) || (iu_ == 1 && ium_ == 2) || (iu_ == 3 && ium_ == 1);
   };
   int st = kOk;
   while (nsteps > 0 && st == kOk) {
      if (nsteps >= kGraphSteps && in_cycle()) {
         const int rec = drec_.n > 0 ? 1 : 0;
         cudaGraphExec_t ex = nullptr;
         for (const GraphKey& g : graph_cache_)
            if (g.iu == iu_ && g.ium == ium_ && g.rec == rec) ex = g.exec;
         if (ex) {
            st = cuda_ok(cudaGraphLaunch(ex, stream_));
            for (int q = 0; q < kGraphSteps; q++) {  // the host side of the replayed steps
               t_ += dt_;
               rec_rows_ += rec;
            }
         } else {
            const int iu0 = iu_, ium0 = ium_;
            st = capture([&]() -> int {
               for (int q = 0; q < kGraphSteps; q++) SW4G_TRY(step_fused());
               return kOk;
            }, &ex);
            if (st == kOk) {
               graph_cache_.push_back(GraphKey{iu0, ium0, rec, ex});
               st = cuda_ok(cudaGraphLaunch(ex, stream_));
            }
         }
         nsteps -= kGraphSteps;
      } else {
         st = step_fused();
         nsteps--;
      }
   }
   clocked_ = false;
   return st;
}

int EW::set_receivers(int n, const int* ijk, const int* mode, int capacity, const int* grid)
{
   if (!ready_ || n < 0 || (n > 0 && (!ijk || !mode || capacity < 1))) return kBadArgument;
   drop_graphs();  // the graphs hold the old receiver set
   std::vector<int> host(6 * (size_t)n);
   int nvals = 0;
   bool curv = false;
   for (int r = 0; r < n; r++) {
      const int i = ijk[3 * r], j = ijk[3 * r + 1], k = ijk[3 * r + 2];
      const int g = grid ? grid[r] : 0;
      if (g != 0 && !(g == 1 && cv_)) return kBadArgument;
      const Bounds& bb = g == 1 ? cv_->b : b_;
      const int nv = receiver_values(mode[r]);
      if (nv == 0) return kBadArgument;
      // the value itself needs (i,j,k) in the array; the differences need its neighbours
      const int m = (mode[r] == kRecDisplacement || mode[r] == kRecVelocity) ? 0 : 1;
      if (i - m < bb.ib || i + m > bb.ie || j - m < bb.jb || j + m > bb.je || k - m < bb.kb ||
          k + m > bb.ke)
         return kBadArgument;
      host[3 * r] = i;
      host[3 * r + 1] = j;
      host[3 * r + 2] = k;
      host[3 * n + r] = mode[r];
      host[4 * n + r] = nvals;
      host[5 * n + r] = g;
      curv = curv || g == 1;
      nvals += nv;
   }
   if (drec_mem_ || records_) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   if (drec_mem_) cudaFree(drec_mem_);
   if (records_) cudaFree(records_);
   drec_mem_ = nullptr;
   records_ = nullptr;
   drec_ = ReceiverSet{};
   rec_cap_ = rec_rows_ = rec_nvals_ = 0;
   rec_initial_ = false;
   rec_curv_ = false;
   if (n == 0) return kOk;
   SW4G_TRY(cuda_ok(cudaMalloc(&drec_mem_, host.size() * sizeof(int))));
   SW4G_TRY(cuda_ok(cudaMemcpy(drec_mem_, host.data(), host.size() * sizeof(int),
                               cudaMemcpyHostToDevice)));
   SW4G_TRY(cuda_ok(cudaMalloc(&records_, (size_t)capacity * nvals * sizeof(double))));
   SW4G_TRY(cuda_ok(cudaMemsetAsync(records_, 0, (size_t)capacity * nvals * sizeof(double), stream_)));
   const int* d = static_cast<const int*>(drec_mem_);
   drec_.n = n;
   drec_.ijk = d;
   drec_.mode = d + 3 * n;
   drec_.off = d + 4 * n;
   drec_.grid = curv ? d + 5 * n : nullptr;
   rec_cap_ = capacity;
   rec_nvals_ = nvals;
   rec_initial_ = true;
   rec_curv_ = curv;
   return kOk;
}

int EW::record_shape(int* rows, int* nvals) const
{
   if (!rows || !nvals) return kBadArgument;
   *rows = rec_rows_;
   *nvals = rec_nvals_;
   return kOk;
}

int EW::get_records(double* out, bool on_device) const
{
   if (!out) return kBadArgument;
   if (rec_rows_ == 0) return kOk;
   const size_t bytes = (size_t)rec_rows_ * rec_nvals_ * sizeof(double);
   SW4G_TRY(cuda_ok(cudaMemcpyAsync(out, records_, bytes,
                                    on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                    stream_)));
   if (!on_device) SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
   return kOk;
}

// The reference CPU phase order (src/EW.C:2537-2756) with the GPU kernels.
int EW::step_phases()
{
   const Bounds& b = b_;
   int ip = 0;
   while (ip == iu_ || ip == ium_) ip++;
   double *up = lev_[ip], *u = lev_[iu_], *um = lev_[ium_];
   const double dt = dt_;
   SW4G_TRY(launch_force_dense(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, f_, dsrc_, t_, 0, stream_));
   SW4G_TRY(launch_rhs4sg_direct(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, g_.nz, onesided_, lu_, u,
                                 mu_, la_, g_.h, dprof_[3], dprof_[4], dprof_[5], stream_));
   SW4G_TRY(launch_predfort(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, u, um, lu_, f_, rho_,
                            dt * dt, stream_));
   if (cv_) SW4G_TRY(curv_pred(ip));
   SW4G_TRY(enforce_bc(up));
   if (cv_) SW4G_TRY(curv_bc(up, cv_->lev[ip]));
   SW4G_TRY(launch_force_dense(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, f_, dsrc_, t_, 1, stream_));
   SW4G_TRY(launch_dpdmtfort(b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, u, um, uacc_, 1 / (dt * dt),
                             stream_));
   SW4G_TRY(launch_rhs4sg_direct(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, g_.nz, onesided_, lu_,
                                 uacc_, mu_, la_, g_.h, dprof_[3], dprof_[4], dprof_[5], stream_));
   SW4G_TRY(launch_corrfort(1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, lu_, f_, rho_,
                            dt * dt * dt * dt, stream_));
   if (prof_.used && g_.sg_damping != 0)
      SW4G_TRY(launch_addsgd(g_.sg_order, 1, b.ib, b.ie, b.jb, b.je, b.kb, b.ke, up, u, um, rho_,
                             dprof_[0], dprof_[1], dprof_[2], dprof_[3], dprof_[4], dprof_[5],
                             dprof_[6], dprof_[7], dprof_[8], g_.sg_damping, stream_));
   if (cv_) SW4G_TRY(curv_corr(ip, ip));
   SW4G_TRY(enforce_bc(up));
   if (cv_) SW4G_TRY(curv_bc(up, cv_->lev[ip]));
   if (drec_.n > 0) SW4G_TRY(record(ip, ium_, 0));
   ium_ = iu_;
   iu_ = ip;
   t_ += dt;
   return kOk;
}

// Fused stages: predictor kernel (+ one-sided rows, sparse forcing, BC), then the
// corrector kernel with supergrid damping (+ rows, forcing, BC).  A step is the
// pieces 0..5 in order: 0 predictor stage kernel, 1 predictor rows, 2 predictor
// forcing + BC, 3 corrector stage kernel, 4 corrector rows (+ 6th-order damping),
// 5 corrector forcing + BC; ip receives the predicted level, iq the new level.
int EW::fused_piece(int piece, int ip, int iq)
{
   const Bounds& bd = b_;
   Box b = make_box(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke);
   double *up = lev_[ip], *out = lev_[iq], *u = lev_[iu_], *um = lev_[ium_];
   const double dt = dt_, dt2 = dt * dt;
   const int nz = g_.nz;
   const double beta = (prof_.used && g_.sg_damping != 0) ? g_.sg_damping : 0.0;
   const double beta4 = g_.sg_order == 4 ? beta : 0.0;
   const double* dc[3] = {dprof_[0], dprof_[1], dprof_[2]};
   const double* st[3] = {dprof_[3], dprof_[4], dprof_[5]};
   const double* co[3] = {dprof_[6], dprof_[7], dprof_[8]};

   if (piece == 0 || piece == 3) {
      FusedStage fs;
      fs.b = b;
      fs.k1 = onesided_[4] ? 7 : 1;
      fs.k2 = onesided_[5] ? nz - 6 : nz;
      fs.mu = mu_;
      fs.la = la_;
      fs.rho = rho_;
      fs.irho = irho_;
      fs.w = w_;
      for (int q = 0; q < 3; q++) {
         fs.st[q] = st[q];
         fs.dc[q] = dc[q];
         fs.co[q] = co[q];
      }
      fs.h = g_.h;
      fs.dt = dt;
      fs.u = u;
      fs.um = um;
      if (piece == 0) {
         fs.corrector = 0;
         fs.up = nullptr;
         fs.out = up;
         fs.beta = 0;
      } else {
         fs.corrector = 1;
         fs.up = up;
         fs.out = out;
         fs.beta = beta4;
         fs.emax = stage_emax_;
      }
      return launch_fused_stage(fs, stream_);
   }
   if (piece == 1) {
      SW4G_TRY(launch_ghost_shell(b, 0, up, u, um, nullptr, stream_));
      for (int side = 0; side < 2; side++)
         if (onesided_[4 + side])
            SW4G_TRY(launch_stage_rows(0, side == 0, b, nz, u, b, mu_, la_, g_.h, st[0], st[1], st[2],
                                       u, um, nullptr, up, rho_, irho_, dt2, 0.0, dc, st, co,
                                       zc_[side], stream_, rscr_, rows_ctas_));
      return kOk;
   }
   if (piece == 2 || piece == kForcePred || piece == kBcPred) {
      if (piece != kBcPred)
         SW4G_TRY(launch_force_update(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, up, rho_, dsrc_, t_,
                                      0, dt2, stream_, clocked_ ? dclock_ : nullptr));
      return piece == kForcePred ? kOk : enforce_bc(up);
   }
   if (piece == 4) {
      SW4G_TRY(launch_ghost_shell(b, 1, out, u, um, up, stream_));
      for (int side = 0; side < 2; side++) {
         if (!onesided_[4 + side]) continue;
         const int k0 = side == 0 ? bd.kb : nz - 7, k1 = side == 0 ? 8 : bd.ke;
         double* slab = slab_ + side * slab_len_;
         SW4G_TRY(launch_uacc_slab(b, k0, k1, up, u, um, slab, stream_));
         Box sb = make_box(1, bd.ib, bd.ie, bd.jb, bd.je, k0, k1);
         SW4G_TRY(launch_stage_rows(1, side == 0, b, nz, slab, sb, mu_, la_, g_.h, st[0], st[1],
                                    st[2], u, um, up, out, rho_, irho_, dt2 / 12, beta4, dc, st, co,
                                    zc_[side], stream_, rscr_, rows_ctas_));
      }
      if (beta != 0 && g_.sg_order == 6)
         SW4G_TRY(launch_addsgd(6, 1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, out, u, um, rho_,
                                dc[0], dc[1], dc[2], st[0], st[1], st[2], co[0], co[1], co[2], beta,
                                stream_));
      return kOk;
   }
   if (piece == 5 || piece == kForceCorr || piece == kBcCorr) {
      if (piece != kBcCorr)
         SW4G_TRY(launch_force_update(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, out, rho_, dsrc_, t_,
                                      1, dt2 * dt2 / 12, stream_, clocked_ ? dclock_ : nullptr));
      return piece == kForceCorr ? kOk : enforce_bc(out);
   }
   return kBadArgument;
}

// The same six pieces for the FP32-mixed form: double-float levels, FP32 interior
// stage kernels, FP64 one-sided rows / free surface / forcing.
int EW::mixed_piece(int piece, int ip, int iq)
{
   const Bounds& bd = b_;
   Box b = make_box(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke);
   float* up = reinterpret_cast<float*>(lev_[ip]);
   float* out = reinterpret_cast<float*>(lev_[iq]);
   const float* u = reinterpret_cast<const float*>(lev_[iu_]);
   const float* um = reinterpret_cast<const float*>(lev_[ium_]);
   const double dt = dt_, dt2 = dt * dt;
   const int nz = g_.nz;
   const double beta = (prof_.used && g_.sg_damping != 0) ? g_.sg_damping : 0.0;
   const double* dc[3] = {dprof_[0], dprof_[1], dprof_[2]};
   const double* st[3] = {dprof_[3], dprof_[4], dprof_[5]};
   const double* co[3] = {dprof_[6], dprof_[7], dprof_[8]};
   if (piece == 0 || piece == 3) {
      MixedStage ms;
      ms.b = b;
      ms.k1 = onesided_[4] ? 7 : 1;
      ms.k2 = onesided_[5] ? nz - 6 : nz;
      ms.mu2 = reinterpret_cast<const float2*>(mu32_);
      ms.la2 = reinterpret_cast<const float2*>(la32_);
      ms.ir2 = reinterpret_cast<const float2*>(irho32_);
      ms.rho = rho32_;
      for (int q = 0; q < kWeightArrays; q++) ms.w2[q] = wd_.p[q];
      for (int q = 0; q < 3; q++) {
         ms.dc[q] = prof32_[q];
         ms.st[q] = prof32_[3 + q];
         ms.co[q] = prof32_[6 + q];
      }
      ms.h = g_.h;
      ms.dt = dt;
      ms.u = u;
      ms.um = um;
      ms.status = reinterpret_cast<int*>(dstat_);
      if (piece == 0) {
         ms.corrector = 0;
         ms.out = up;
         ms.beta = 0;
      } else {
         ms.corrector = 1;
         ms.up = up;
         ms.out = out;
         ms.beta = g_.sg_order == 4 ? beta : 0.0;  // 6th order: a separate pass in piece 4
      }
      return launch_mixed_stage(ms, stream_);
   }
   if (piece == 1) {
      SW4G_TRY(launch_ghost_shell_df(b, 0, up, u, um, nullptr, stream_));
      for (int side = 0; side < 2; side++) {
         if (!onesided_[4 + side]) continue;
         // the stage field as an FP64 slab: one conversion per value
         const int k0 = side == 0 ? bd.kb : nz - 7, k1 = side == 0 ? 8 : bd.ke;
         double* slab = slab_ + side * slab_len_;
         SW4G_TRY(launch_df_slab(b, k0, k1, u, nullptr, slab, stream_));
         Box sb = make_box(1, bd.ib, bd.ie, bd.jb, bd.je, k0, k1);
         SW4G_TRY(launch_stage_rows_df(0, side == 0, b, nz, slab, nullptr, sb, mu_, la_, g_.h, st[0],
                                       st[1], st[2], u, um, nullptr, up, rho_, irho_, dt2, 0.0, dc,
                                       st, co, zc_[side], stream_, nullptr, rscr_, rows_ctas_));
      }
      return kOk;
   }
   if (piece == 2 || piece == kForcePred || piece == kBcPred) {
      if (piece != kBcPred)
         SW4G_TRY(launch_force_update_df(bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, up, rho_, dsrc_, t_,
                                         0, dt2, stream_, clocked_ ? dclock_ : nullptr));
      if (piece == kForcePred) return kOk;
      return launch_bcfortsg_df(bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, wind_, g_.nx, g_.ny, g_.nz,
                                up, g_.h, g_.bc, sbop_, mu_, la_, dprof_[3], dprof_[4], stream_);
   }
   if (piece == 4) {
      const double beta4 = g_.sg_order == 4 ? beta : 0.0;
      SW4G_TRY(launch_ghost_shell_df(b, 1, out, u, um, up, stream_));
      for (int side = 0; side < 2; side++) {
         if (!onesided_[4 + side]) continue;
         const int k0 = side == 0 ? bd.kb : nz - 7, k1 = side == 0 ? 8 : bd.ke;
         double* slab = slab_ + side * slab_len_;
         double* dslab = slab_ + (2 + side) * slab_len_;  // u - um for the damping
         SW4G_TRY(launch_uacc_slab_df(b, k0, k1, up, u, um, slab, stream_));
         if (beta4 != 0) SW4G_TRY(launch_df_slab(b, k0, k1, u, um, dslab, stream_));
         Box sb = make_box(1, bd.ib, bd.ie, bd.jb, bd.je, k0, k1);
         SW4G_TRY(launch_stage_rows_df(1, side == 0, b, nz, slab, nullptr, sb, mu_, la_, g_.h, st[0],
                                       st[1], st[2], u, um, up, out, rho_, irho_, dt2 / 12, beta4,
                                       dc, st, co, zc_[side], stream_, beta4 != 0 ? dslab : nullptr,
                                       rscr_, rows_ctas_));
      }
      if (beta != 0 && g_.sg_order == 6) {
         const float* dc32[3] = {prof32_[0], prof32_[1], prof32_[2]};
         const float* st32[3] = {prof32_[3], prof32_[4], prof32_[5]};
         const float* co32[3] = {prof32_[6], prof32_[7], prof32_[8]};
         SW4G_TRY(launch_addsgd6_df(3, b, out, u, um, rho32_, dc32, st32, co32, beta, stream_));
      }
      return kOk;
   }
   if (piece == 5 || piece == kForceCorr || piece == kBcCorr) {
      if (piece != kBcCorr)
         SW4G_TRY(launch_force_update_df(bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, out, rho_, dsrc_, t_,
                                         1, dt2 * dt2 / 12, stream_, clocked_ ? dclock_ : nullptr));
      if (piece == kForceCorr) return kOk;
      return launch_bcfortsg_df(bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, wind_, g_.nx, g_.ny, g_.nz,
                                out, g_.h, g_.bc, sbop_, mu_, la_, dprof_[3], dprof_[4], stream_);
   }
   return kBadArgument;
}

int EW::side_stream()
{
   if (side_) return kOk;
   int dev = 0, lo = 0, hi = 0;
   SW4G_TRY(cuda_ok(cudaGetDevice(&dev)));
   SW4G_TRY(cuda_ok(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev)));
   // FP32-mixed form: the highest priority, so that the rows' persistent CTAs take
   // their place on every SM beside the (FP32, issue-bound) stage kernel's as soon as
   // they are launched.  FP64 form: the stage kernels and the rows both load the FP64
   // pipe, and the rows' own full grid at the default priority measured best.
   SW4G_TRY(cuda_ok(cudaDeviceGetStreamPriorityRange(&lo, &hi)));
   SW4G_TRY(cuda_ok(cudaStreamCreateWithPriority(&side_, cudaStreamNonBlocking, mixed_ ? hi : lo)));
   SW4G_TRY(cuda_ok(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming)));
   return cuda_ok(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
}

int EW::step_fused()
{
   int ip = 0;
   while (ip == iu_ || ip == ium_) ip++;
   int iq = ip + 1;
   while (iq == iu_ || iq == ium_) iq++;
   // The one-sided rows (pieces 1, 4) write planes 1..6 / nz-5..nz and the ghost
   // shell, the stage kernels (0, 3) the planes between, both from the same inputs:
   // the rows run beside the stage on a second stream, joined before the forcing and
   // boundary pieces; in the FP32-mixed form as a persistent grid of one CTA per SM (a
   // rows CTA fits beside a stage CTA on each SM) on a higher-priority stream.  Not
   // with 6th-order damping, whose pass in piece 4 covers every plane.
   const bool beta6 = g_.sg_order == 6 && prof_.used && g_.sg_damping != 0;
   const bool beside = rows_overlap_enabled() && (onesided_[4] || onesided_[5]) && !beta6;
   // With topography the curvilinear grid's top rows (its free surface, FP64) run
   // beside both grids' stage kernels in the same way, forked at the start of each
   // stage; its 6th-order damping pass and forcing follow the join.
   const bool cbeside = rows_overlap_enabled() && cv_ != nullptr;
   for (int which = 0; which < 6; which++) {
      if (beside && (which == 1 || which == 4)) continue;
      if ((beside || cbeside) && (which == 0 || which == 3)) {
         // fork point before the stages, stages first, then the rows, then the join
         SW4G_TRY(side_stream());
         SW4G_TRY(cuda_ok(cudaEventRecord(ev_fork_, stream_)));
         SW4G_TRY(piece(which, ip, iq));
         if (cbeside) SW4G_TRY(which == 0 ? curv_pred_part(ip, 2, stream_, 0) : curv_corr_part(ip, iq, 2, stream_, 0));
         SW4G_TRY(cuda_ok(cudaStreamWaitEvent(side_, ev_fork_, 0)));
         cudaStream_t own = stream_;
         stream_ = side_;
         rows_ctas_ = mixed_ ? sms_ : 0;
         int st = beside ? piece(which + 1, ip, iq) : kOk;
         if (st == kOk && cbeside)
            st = which == 0 ? curv_pred_part(ip, 1, side_, rows_ctas_) : curv_corr_part(ip, iq, 1, side_, rows_ctas_);
         rows_ctas_ = 0;
         stream_ = own;
         SW4G_TRY(st);
         SW4G_TRY(cuda_ok(cudaEventRecord(ev_join_, side_)));
         SW4G_TRY(cuda_ok(cudaStreamWaitEvent(stream_, ev_join_, 0)));
         if (cbeside) SW4G_TRY(which == 0 ? curv_pred_part(ip, 3, stream_, 0) : curv_corr_part(ip, iq, 3, stream_, 0));
      } else {
         SW4G_TRY(piece(which, ip, iq));
      }
      if (!cv_) continue;
      if (which == 0 && !cbeside) SW4G_TRY(curv_pred(ip));
      if (which == 2) SW4G_TRY(curv_bc(lev_[ip], cv_->lev[ip]));
      if (which == 3 && !cbeside) SW4G_TRY(curv_corr(ip, iq));
      if (which == 5) SW4G_TRY(curv_bc(lev_[iq], cv_->lev[iq]));
   }
   if (drec_.n > 0) SW4G_TRY(record(iq, ium_, 0));
   if (clocked_) SW4G_TRY(launch_clock_advance(dclock_, dt_, drec_.n > 0 ? 1.0 : 0.0, 0.0, stream_));
   ium_ = iu_;
   iu_ = iq;
   t_ += dt_;
   return kOk;
}

int EW::step_part(int part)
{
   if (!sub_ || part != part_) return kBadArgument;
   if (part == 0) {
      if (!ready_ || !material_ || !(dt_ > 0) || graphs_) return kBadArgument;
      if (drec_.n > 0 && rec_rows_ + (rec_initial_ ? 1 : 0) + 1 > rec_cap_) return kBadArgument;
      SW4G_TRY(upload_sources());
      if (drec_.n > 0 && rec_initial_) {
         SW4G_TRY(record(iu_, ium_, 1));
         rec_initial_ = false;
      }
      int ip = 0;
      while (ip == iu_ || ip == ium_) ip++;
      int iq = ip + 1;
      while (iq == iu_ || iq == ium_) iq++;
      split_ip_ = ip;
      split_iq_ = iq;
      SW4G_TRY(piece(0, ip, iq));
      SW4G_TRY(piece(1, ip, iq));
      SW4G_TRY(piece(kForcePred, ip, iq));
   } else if (part == 1) {
      SW4G_TRY(piece(kBcPred, split_ip_, split_iq_));
      SW4G_TRY(piece(3, split_ip_, split_iq_));
      SW4G_TRY(piece(4, split_ip_, split_iq_));
      SW4G_TRY(piece(kForceCorr, split_ip_, split_iq_));
   } else {
      SW4G_TRY(piece(kBcCorr, split_ip_, split_iq_));
      if (drec_.n > 0) SW4G_TRY(record(split_iq_, ium_, 0));
      ium_ = iu_;
      iu_ = split_iq_;
      t_ += dt_;
   }
   part_ = (part + 1) % 3;
   return kOk;
}

int EW::profile_kernels(int nrep, double ms[4])
{
   if (!ready_ || !material_ || !(dt_ > 0) || nrep < 1 || !ms) return kBadArgument;
   SW4G_TRY(upload_sources());
   int ip = 0;
   while (ip == iu_ || ip == ium_) ip++;
   int iq = ip + 1;
   while (iq == iu_ || iq == ium_) iq++;
   // one full fused step's pieces first, so every input level holds valid data
   for (int which = 0; which < 6; which++) SW4G_TRY(piece(which, ip, iq));
   const int groups[4][2] = {{0, -1}, {3, -1}, {1, 4}, {2, 5}};
   cudaEvent_t e0, e1;
   SW4G_TRY(cuda_ok(cudaEventCreate(&e0)));
   SW4G_TRY(cuda_ok(cudaEventCreate(&e1)));
   int status = kOk;
   for (int g = 0; g < 4 && status == kOk; g++) {
      cudaEventRecord(e0, stream_);
      for (int r = 0; r < nrep && status == kOk; r++)
         for (int q = 0; q < 2 && status == kOk; q++)
            if (groups[g][q] >= 0) status = piece(groups[g][q], ip, iq);
      cudaEventRecord(e1, stream_);
      if (cudaEventSynchronize(e1) != cudaSuccess) status = kCudaError;
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      ms[g] = t / nrep;
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   return status;
}

int EW::launches_per_step(int mode) const
{
   int bc = 0;
   for (int s = 0; s < 6; s++) {
      const int t = g_.bc[s];
      if ((t == kDirichlet || t == kSuperGrid || t == kPeriodic) && bcpts_[s] > 0) bc++;
      if (t == kStressFree) bc++;
   }
   const int rows = onesided_[4] + onesided_[5];
   const int src = hsrc_.empty() ? 0 : 1;
   const bool damp = prof_.used && g_.sg_damping != 0;
   const int rec = drec_.n > 0 ? 1 : 0;
   if (mode == kModePhases) {
      // force(memset+kernel), rhs (center + rows), pred, bc, force, dpdm, rhs, corr, addsgd, bc
      const int rhs = 1 + rows;
      return 2 * (1 + src) + 2 * rhs + 3 + (damp ? 1 : 0) + 2 * bc + rec + curv_launches(mode);
   }
   // per stage: stage kernel, ghost shell, one-sided rows, forcing, BC sides;
   // the corrector adds the rows' slab kernels (and 6th-order damping); the mixed
   // form adds an FP64 slab of the predictor's field and of the corrector's u - um
   const int mslabs = mixed_ ? rows * (1 + (damp ? 1 : 0)) : 0;
   // and each rows launch its per-column pass
   return 2 * (2 + 2 * rows + src + bc) + rows + (damp && g_.sg_order == 6 ? 1 : 0) + rec + mslabs +
          curv_launches(mode);
}

}  // namespace sw4g
