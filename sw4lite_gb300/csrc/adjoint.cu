// Discrete adjoint of the Cartesian time step and the material gradient of a
// receiver misfit, sm_103a: FP64, or the FP32-mixed form (double-float levels and
// adjoint variables, FP32 stages and gradient terms, FP64 gradient accumulation).
//
// The reference computes no material gradient (sw4lite has source-parameter
// gradients only, src/GridPointSource.C:659-760); this is the exact transpose of
// this library's own step for grids whose boundary sides are Dirichlet or
// supergrid with zero boundary data, so every ghost point is zero after each
// boundary pass and the state lives on the interior points I.  With R = 1/rho:
//   up = 2u - um + dt^2 R L(u) + dt^2 R F
//   u+ = up + dt^2/12 R L(up - 2u + um) - beta R SG(u - um) + dt^4/12 R F_tt
// Transposes: W L is symmetric for W = 1/(sx sy sz) (the stretched elastic
// operator is self-adjoint in the stretched volume), so L^T = W L W^-1; the
// damping is SG = sum_ax diag(w_ax) D2 (rho dc_ax) D2, so SG^T y = sum_ax
// D2 (rho dc_ax) D2 (w_ax y).  The adjoint recursion a^n = g^n + A^T a^{n+1} +
// B^T a^{n+2} becomes, with a1 = a^{n+1}, a2 = a^{n+2}:
//   s = L^T R a1,  m = a1 + dt^2/12 s,  t = L^T R m,
//   a^n = g^n + 2m + dt^2 t - dt^2/6 s - a2 - beta SG^T R (a1 - a2),
// two operator applications per step like the forward.  In the scaled variable
// b = W^-1 R a the recursion takes the forward's own form (the W factors commute
// with each axis' damping term, so W^-1 R SG^T R W = R SG):
//   mt = b1 + dt^2/12 R L(b1),
//   b^n = 2 b1 - b2 + dt^2 R L(mt) - beta R SG(b1 - b2) + W^-1 R g^n,
// which runs on the forward's fused stage kernels (predictor form with
// coefficient dt^2/12, and the adjoint form of stage_fused.cu).  The gradient of
// a1 . u+ at fixed (u, um) (a1 = rho W b1, m = rho W mt):
//   mu, lambda : G(dt^2/12 W b1, up - 2u + um) + G(dt^2 W mt, u), G(v, w) the
//                coefficient gradient of v . L(w).  The second differences have
//                symmetric edge weights, v . D2(a) w = -sum_q sum_{m=1,2}
//                W_m(q) (v(q+m)-v(q)) (w(q+m)-w(q)), so dG/da is 7 products of
//                forward differences; the mixed terms give minus products of
//                centred first differences;
//   rho        : -W [mt.(up - 2u + um) + b1.(u+ - up)] (the 1/rho factors and
//                the forcing) - beta dc D2(u - um) . D2(w W b1) (the damping's
//                rho dc factors).
// These sums run in adj_grad.cu: double-float arithmetic on the FP32 pipe for the
// FP64 form, FP32 for the mixed form.
// Free-surface z sides (the ghost plane solved from the interior by the traction
// condition, one-sided SBP rows): D L is symmetric for D = H W, H the SBP norm weights
// (17/48, 59/48, 43/48, 49/48 on the four planes next to the side), so the scaled
// adjoint is b = (H W)^-1 R a and the recursion keeps the forward's form, with the
// forward's one-sided rows (and an adjoint form of them) and free-surface ghost plane
// applied to b and mt.  This needs the z stretching to be 1 and the z damping zero on
// the planes next to the side (no supergrid layer there), which the call checks.  The
// gradient terms of the one-sided rows come from grad_rows (adj_grad.cu).
// Forward levels come from checkpoints every C steps, recomputed one segment
// at a time with every level and predicted level kept in HBM.
#include <algorithm>
#include <tuple>
#include <cmath>
#include <vector>

#include "df.cuh"
#include "ew.h"

namespace sw4g {
namespace {

template <class T>
struct ProfT {
   const T *dc[3], *st[3], *co[3];
};
using Prof = ProfT<double>;

template <class T>
__device__ __forceinline__ T sxyz(const Box& b, const ProfT<T>& f, int i, int j, int k)
{
   return f.st[0][i - b.ib] * f.st[1][j - b.jb] * f.st[2][k - b.kb];
}

// Receivers grouped by grid point: point u holds receivers rg.idx[rg.start[u] ..
// rg.start[u+1]) in increasing order (several receivers may share a point; one thread
// per point adds their residuals, in order, so the sum does not depend on scheduling).
struct RecGroups {
   int n = 0;  // points
   const int* start = nullptr;
   const int* idx = nullptr;
};

// residual sum of point u's receivers, component c, and the point's (i, j, k)
__device__ __forceinline__ double group_res(const RecGroups& rg, int u, const int* __restrict__ ijk,
                                            const double* __restrict__ res, int c)
{
   double acc = 0;
   for (int q = rg.start[u]; q < rg.start[u + 1]; q++) acc += res[3 * rg.idx[q] + c];
   return acc;
}

// b[receiver point] += (H W)^-1 R res (3 values per receiver; hz the SBP norm weights
// H of the z planes)
__global__ void adj_source_kernel(Box b, Prof f, RecGroups rg, const int* __restrict__ ijk,
                                  const double* __restrict__ res, const double* __restrict__ rho,
                                  const double* __restrict__ hz, double* __restrict__ an,
                                  const double* __restrict__ clk, int nval)
{
   const int u = blockIdx.x * blockDim.x + threadIdx.x;
   if (u >= rg.n) return;
   if (clk) res += (long long)clk[2] * nval;  // the residual row from the device clock
   const int r = rg.idx[rg.start[u]];
   const int i = ijk[3 * r], j = ijk[3 * r + 1], k = ijk[3 * r + 2];
   const long long p = pidx(b, i, j, k);
   const double s = sxyz(b, f, i, j, k) / (rho[p] * hz[k - b.kb]);
#pragma unroll
   for (int c = 0; c < 3; c++) an[c * b.npts + p] += s * group_res(rg, u, ijk, res, c);
}

// the adjoint source added to a double-float level (hi at q, lo at q + 3 npts) in FP64
__global__ void adj_source_df_kernel(Box b, Prof f, RecGroups rg, const int* __restrict__ ijk,
                                     const double* __restrict__ res, const double* __restrict__ rho,
                                     const double* __restrict__ hz, float* __restrict__ an,
                                     const double* __restrict__ clk, int nval)
{
   const int u = blockIdx.x * blockDim.x + threadIdx.x;
   if (u >= rg.n) return;
   if (clk) res += (long long)clk[2] * nval;
   const int r = rg.idx[rg.start[u]];
   const int i = ijk[3 * r], j = ijk[3 * r + 1], k = ijk[3 * r + 2];
   const long long p = pidx(b, i, j, k);
   const double s = sxyz(b, f, i, j, k) / (rho[p] * hz[k - b.kb]);
   const DFField a{an, 3 * b.npts};
#pragma unroll
   for (int c = 0; c < 3; c++)
      a.set(c * b.npts + p, a.get(c * b.npts + p) + s * group_res(rg, u, ijk, res, c));
}

}  // namespace

int EW::gradient(int nsteps, int ckpt, const double* obs, bool obs_on_device, double* misfit,
                 double* g_rho, double* g_mu, double* g_la, bool grad_on_device)
{
   if (!ready_ || !material_ || !(dt_ > 0) || nsteps < 1 || ckpt < 1 || !obs || !misfit || !g_rho ||
       !g_mu || !g_la)
      return kBadArgument;
   if (cv_ || (g_.sg_order != 4 && g_.sg_order != 6)) return kNotSupported;
   for (int s = 0; s < 6; s++)
      if (g_.bc[s] != kDirichlet && g_.bc[s] != kSuperGrid && !(s >= 4 && g_.bc[s] == kStressFree))
         return kNotSupported;
   // free-surface z sides: the symmetry D L = (D L)^T needs the z stretching 1 and the
   // z damping 0 on the ten planes next to the side (true without a layer there)
   const bool fs_top = onesided_[4] != 0, fs_bot = onesided_[5] != 0;
   if (fs_top || fs_bot) {
      const std::vector<double>& sz = prof_.str[2];
      const std::vector<double>& dz = prof_.dc[2];
      for (int k = b_.kb; k <= b_.ke; k++) {
         const bool near = (fs_top && k <= 10) || (fs_bot && k >= g_.nz - 9);
         const size_t q = (size_t)(k - b_.kb);
         if (near && ((q < sz.size() && sz[q] != 1.0) || (q < dz.size() && dz[q] != 0.0))) return kNotSupported;
      }
      if (g_.nz < 22) return kNotSupported;  // one-sided rows and centred rows apart
   }
   if (drec_.n == 0) return kBadArgument;
   // receivers grouped by grid point for the adjoint sources (start | idx)
   std::vector<int> rgroup;
   int ngroups = 0;
   {
      std::vector<int> modes(drec_.n), ijk(3 * (size_t)drec_.n);
      SW4G_TRY(cuda_ok(cudaMemcpy(modes.data(), drec_.mode, drec_.n * sizeof(int), cudaMemcpyDeviceToHost)));
      for (int m : modes)
         if (m != kRecDisplacement) return kNotSupported;
      SW4G_TRY(cuda_ok(cudaMemcpy(ijk.data(), drec_.ijk, ijk.size() * sizeof(int), cudaMemcpyDeviceToHost)));
      std::vector<int> ord(drec_.n);
      for (int r = 0; r < drec_.n; r++) ord[r] = r;
      auto key = [&](int r) {
         return std::make_tuple(ijk[3 * r + 2], ijk[3 * r + 1], ijk[3 * r]);
      };
      std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return key(x) < key(y); });
      std::vector<int> start;
      for (int q = 0; q < drec_.n; q++)
         if (q == 0 || key(ord[q]) != key(ord[q - 1])) start.push_back(q);
      ngroups = (int)start.size();
      start.push_back(drec_.n);
      rgroup = start;
      rgroup.insert(rgroup.end(), ord.begin(), ord.end());
   }
   const int nval = rec_nvals_;
   // the records of this run: the initial row and one per step, from row 0
   if (nsteps + 1 > rec_cap_) return kBadArgument;
   SW4G_TRY(upload_sources());

   const Bounds bd = b_;
   const Box b = make_box(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke);
   const size_t n3 = 3 * (size_t)npts_, lv = n3 * sizeof(double);
   const int nseg = (nsteps + ckpt - 1) / ckpt;
   const int seglen = std::min(ckpt, nsteps);
   const double dt = dt_;

   // device memory: checkpoints, one segment of levels and predicted levels, adjoint work
   // (kept from the previous call of the same shape)
   const size_t segbytes = (size_t)(2 * seglen + 2) * lv;
   const int nax[3] = {bd.ie - bd.ib + 1, bd.je - bd.jb + 1, bd.ke - bd.kb + 1};
   GradCache& gc = gcache_;
   int st = kOk;
   if (!(gc.npts == npts_ && gc.nsteps == nsteps && gc.ckpt == ckpt && gc.nval == nval &&
         gc.mixed == (int)mixed_ && gc.host_grad == (int)!grad_on_device && gc.budget == grad_store_bytes_)) {
      drop_grad_cache();
      auto alloc = [&](double** p, size_t bytes) {
         int s = cuda_ok(cudaMalloc(p, bytes));
         if (s == kOk) gc.mem.push_back(*p);
         return s;
      };
      st = alloc(&gc.ck, 2 * (size_t)nseg * lv);
      if (st == kOk) st = alloc(&gc.seg, (size_t)(seglen + 2) * lv);
      if (st == kOk) st = alloc(&gc.pred, (size_t)seglen * lv);
      if (st == kOk) st = alloc(&gc.work, 7 * lv);  // adjoint work (5) + the forward's final levels (2)
      if (st == kOk) st = alloc(&gc.resd, (size_t)(nsteps + 1) * nval * sizeof(double));
      // the gradient terms (adj_grad.cu): the step's levels in the kernels' number type
      // (5 levels of pairs, FP64 form, or of floats), the FP64 form's per-point sums (1
      // level), the edge sums (12 numbers per point), the 1-D profile pairs, the exponent
      // maxima (adjoint; forward per segment; the kept segments')
      if (st == kOk) st = alloc(&gc.dfw, mixed_ ? 5 * lv : 10 * lv);
      if (st == kOk) st = alloc(&gc.dfp, 4 * (size_t)(nax[0] + nax[1] + nax[2]) * sizeof(float2));
      if (st == kOk) st = alloc(&gc.dfe, ((size_t)nseg + 2) * sizeof(int) + sizeof(double));
      if (st == kOk) st = alloc(&gc.hz, (size_t)nax[2] * sizeof(double));
      if (st == kOk) st = alloc(&gc.rgrp, (2 * (size_t)nval / 3 + 1) * sizeof(int));
      if (st == kOk && !grad_on_device) st = alloc(&gc.gtmp, 3 * (size_t)npts_ * sizeof(double));
      // Segments kept from the forward run, whose recompute the backward sweep skips:
      // the last one in seg/pred, and before it as many as the store budget holds
      // (each 2C + 2 levels; by default the free device memory less a reserve).
      if (st == kOk && nseg > 1 && grad_store_bytes_ != 0) {
         size_t freeb = 0, totb = 0;
         if (cudaMemGetInfo(&freeb, &totb) == cudaSuccess) {
            const size_t reserve = std::max((size_t)4 << 30, totb / 32);
            size_t budget = freeb > reserve ? freeb - reserve : 0;
            if (grad_store_bytes_ > 0) budget = std::min(budget, (size_t)grad_store_bytes_);
            const int want = (int)std::min<size_t>((size_t)nseg - 1, budget / segbytes);
            for (int q = 0; q < want; q++) {
               double* x = nullptr;
               if (cudaMalloc(&x, segbytes) != cudaSuccess) {
                  cudaGetLastError();
                  break;
               }
               gc.mem.push_back(x);
               gc.xbuf.push_back(x);
            }
         }
      }
      if (st != kOk) {
         drop_grad_cache();
         return st;
      }
      gc.npts = npts_;
      gc.nsteps = nsteps;
      gc.ckpt = ckpt;
      gc.nval = nval;
      gc.mixed = (int)mixed_;
      gc.host_grad = (int)!grad_on_device;
      gc.budget = grad_store_bytes_;
   }
   double *ck = gc.ck, *seg = gc.seg, *pred = gc.pred, *work = gc.work, *resd = gc.resd, *dfw = gc.dfw,
          *dfp = gc.dfp, *dfe = gc.dfe, *hz = gc.hz;
   {  // the SBP norm weights of the z planes: 1 but next to free-surface sides
      static const double om[4] = {17.0 / 48, 59.0 / 48, 43.0 / 48, 49.0 / 48};
      std::vector<double> hh(nax[2], 1.0);
      for (int k = bd.kb; k <= bd.ke; k++) {
         if (fs_top && k >= 1 && k <= 4) hh[k - bd.kb] = om[k - 1];
         if (fs_bot && k <= g_.nz && k >= g_.nz - 3) hh[k - bd.kb] = om[g_.nz - k];
      }
      if (st == kOk) st = cuda_ok(cudaMemcpy(hz, hh.data(), hh.size() * sizeof(double), cudaMemcpyHostToDevice));
      if (st == kOk)
         st = cuda_ok(cudaMemcpy(gc.rgrp, rgroup.data(), rgroup.size() * sizeof(int), cudaMemcpyHostToDevice));
   }
   RecGroups rg;
   rg.n = ngroups;
   rg.start = reinterpret_cast<const int*>(gc.rgrp);
   rg.idx = rg.start + ngroups + 1;
   const std::vector<double*>& xbuf = gc.xbuf;
   double* gr_d = grad_on_device ? g_rho : gc.gtmp;
   double* gm_d = grad_on_device ? g_mu : gc.gtmp + npts_;
   double* gl_d = grad_on_device ? g_la : gc.gtmp + 2 * npts_;
   // A segment's adjoint steps run on two streams forked from the object's stream:
   // the stages (the critical path) on one of the highest priority and the gradient
   // terms of each step on one of the lowest, beside the next stages (they need the
   // step's mt and nothing after it needs them), so their CTAs take what the stage
   // kernels leave of each SM.  mt is double-buffered and events order its reuse.
   cudaStream_t hs = nullptr, gs = nullptr;
   cudaEvent_t ev_s0 = nullptr, ev_g[2] = {nullptr, nullptr}, ev_join = nullptr, ev_fork = nullptr,
               ev_back = nullptr;
   auto cleanup = [&]() {
      cudaStreamSynchronize(stream_);
      if (hs) cudaStreamSynchronize(hs);
      if (gs) cudaStreamSynchronize(gs);
      if (hs) cudaStreamDestroy(hs);
      if (gs) cudaStreamDestroy(gs);
      for (cudaEvent_t e : {ev_s0, ev_g[0], ev_g[1], ev_join, ev_fork, ev_back})
         if (e) cudaEventDestroy(e);
   };
   if (st == kOk) {
      int lo = 0, hi = 0;
      st = cuda_ok(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      if (st == kOk) st = cuda_ok(cudaStreamCreateWithPriority(&hs, cudaStreamNonBlocking, hi));
      if (st == kOk) st = cuda_ok(cudaStreamCreateWithPriority(&gs, cudaStreamNonBlocking, lo));
      for (cudaEvent_t* e : {&ev_s0, &ev_g[0], &ev_g[1], &ev_join, &ev_fork, &ev_back})
         if (st == kOk) st = cuda_ok(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
   }
   cudaStream_t sa = hs;  // the adjoint steps' stages
   if (st != kOk) {
      cleanup();
      return st;
   }
   const int nkept = 1 + (int)xbuf.size();
   std::vector<double> tseg(nseg);  // the time at each segment's start in the forward run
   auto kept = [&](int sg) { return sg >= nseg - nkept; };
   // buffers of segment sg: levels u^{s0-1..s1} and predicted levels up^{s0..s1-1}
   auto seg_of = [&](int sg) { return kept(sg) && sg < nseg - 1 ? xbuf[nseg - 2 - sg] : seg; };
   auto pred_of = [&](int sg) {
      return kept(sg) && sg < nseg - 1 ? xbuf[nseg - 2 - sg] + (size_t)(seglen + 2) * n3 : pred;
   };
   Prof pf;
   for (int a = 0; a < 3; a++) {
      pf.dc[a] = dprof_[a];
      pf.st[a] = dprof_[3 + a];
      pf.co[a] = dprof_[6 + a];
   }
   const double beta = (prof_.used && g_.sg_damping != 0) ? g_.sg_damping : 0.0;
   // the mixed form: double-float levels, FP32 stages and gradient terms
   MixedStage ms;
   if (mixed_) {
      ms.b = b;
      ms.k1 = 1;
      ms.k2 = g_.nz;
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
      ms.status = reinterpret_cast<int*>(dstat_);
      ms.k1 = fs_top ? 7 : 1;
      ms.k2 = fs_bot ? g_.nz - 6 : g_.nz;
   }
   auto F = [](double* x) { return reinterpret_cast<float*>(x); };
   GradDF gd;
   GradDFProfiles gp{};
   int* emax = reinterpret_cast<int*>(dfe);
   const double kmu = -(dt * dt / 12) / (144 * g_.h * g_.h);
   gd.b = b;
   if (mixed_) {  // FP32 numbers, added to the FP64 gradients every step
      float* f1 = reinterpret_cast<float*>(dfw);
      gd.db1 = f1;
      gd.dmt = f1 + n3;
      gd.dw1 = f1 + 2 * n3;
      gd.du = f1 + 3 * n3;
      gd.dum = f1 + 4 * n3;
      gd.ed = f1 + 5 * n3;
      gd.lo = (long long)n3;
      gd.gm64 = gm_d;
      gd.gl64 = gl_d;
      gd.gr64 = gr_d;
      gd.kmu = kmu;
   } else {
      float2* f2 = reinterpret_cast<float2*>(dfw);
      gd.db1 = f2;
      gd.dmt = f2 + n3;
      gd.dw1 = f2 + 2 * n3;
      gd.du = f2 + 3 * n3;
      gd.dum = f2 + 4 * n3;
      gd.am = f2 + 5 * n3;
      gd.al = f2 + 5 * n3 + npts_;
      gd.ar = f2 + 5 * n3 + 2 * npts_;
      gd.ed = f2 + 6 * n3;
      gd.emax = emax;
      // Each class's bound maps to 2^26..2^28: the largest products (x 1/(s_b s_c) <=
      // 2^32 in the supergrid layers, x 12, summed) stay below 2^110, and values down
      // to 2^-131 of the bound keep all 47 bits (FP32's lo word reaches 2^-103).
      int marg = 4;
      while ((1LL << (marg - 4)) < (long long)nsteps + 1) marg++;
      gd.marg_a = marg - 30;  // the adjoint level is at most (steps) x (largest injection)
      gd.marg_f = 4 - 32;     // w1 = up - 2u + um is at most 4 x the largest level
   }
   if (fs_top) gd.zlo = 6;
   if (fs_bot) gd.zhi = g_.nz - 5;
   gd.sg6 = g_.sg_order == 6;
   // sixth order: the stages carry no damping; the transposed damping pass follows
   const double beta4 = g_.sg_order == 4 ? beta : 0.0, beta6 = g_.sg_order == 6 ? beta : 0.0;
   const double* dcp6[3] = {dprof_[0], dprof_[1], dprof_[2]};
   const double* stp6[3] = {dprof_[3], dprof_[4], dprof_[5]};
   const double* cop6[3] = {dprof_[6], dprof_[7], dprof_[8]};
   GradRows gw;  // the one-sided rows' gradient terms
   gw.b = b;
   gw.nz = g_.nz;
   gw.sx = dprof_[3];
   gw.sy = dprof_[4];
   gw.sz = dprof_[5];
   gw.hz = hz;
   gw.c1 = dt * dt / 12;
   gw.c2 = dt * dt;
   gw.h = g_.h;
   gw.gm = gm_d;
   gw.gl = gl_d;
   gw.lo = (long long)n3;
   float2* pp = reinterpret_cast<float2*>(dfp);
   gp.beta = beta;
   gp.hz = hz;
   for (int a = 0; a < 3; a++) {
      gp.n[a] = nax[a];
      gp.st[a] = dprof_[3 + a];
      gp.co[a] = dprof_[6 + a];
      gp.dc[a] = dprof_[a];
      gp.st24[a] = pp;
      gp.ist[a] = pp + nax[a];
      gp.cist[a] = pp + 2 * nax[a];
      gp.bdc[a] = pp + 3 * nax[a];
      pp += 4 * nax[a];
      gd.st24[a] = gp.st24[a];
      gd.ist[a] = gp.ist[a];
      gd.cist[a] = gp.cist[a];
      gd.bdc[a] = gp.bdc[a];
   }
   // Fused steps n0..n1-1 with the level slots pointing into a segment's buffers, so
   // each level lands where the adjoint reads it: u^{n+1} in sq[n - n0 + 2], the
   // predicted level up^n in pq[n - n0] (sq[0], sq[1] hold u^{n0-1}, u^{n0} on
   // entry).  The object's own level buffers then get the last two levels back.
   auto steps_into = [&](int n0, int n1, double* sq, double* pq) -> int {
      double* own[4] = {lev_[0], lev_[1], lev_[2], lev_[3]};
      lev_[iu_] = sq + n3;
      lev_[ium_] = sq;
      int status = kOk;
      for (int n = n0; n < n1 && status == kOk; n++) {
         int ip = 0;
         while (ip == iu_ || ip == ium_) ip++;
         int iq = ip + 1;
         while (iq == iu_ || iq == ium_) iq++;
         lev_[ip] = pq + (size_t)(n - n0) * n3;
         lev_[iq] = sq + (size_t)(n - n0 + 2) * n3;
         status = step_fused();
      }
      for (int q = 0; q < 4; q++) lev_[q] = own[q];
      SW4G_TRY(status);
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[iu_], sq + (size_t)(n1 - n0 + 1) * n3, lv, cudaMemcpyDeviceToDevice,
                                       stream_)));
      return cuda_ok(cudaMemcpyAsync(lev_[ium_], sq + (size_t)(n1 - n0) * n3, lv, cudaMemcpyDeviceToDevice,
                                     stream_));
   };

   // The forward levels' shift of a segment: the largest exponent over its levels, of
   // the two it starts from here and of the others from the corrector stages that write
   // them (stage_emax_, set until the caller's steps end)
   auto forward_scale = [&](const double* sq, int* slot) -> int {
      if (mixed_) return kOk;
      SW4G_TRY(cuda_ok(cudaMemsetAsync(slot, 0, sizeof(int), stream_)));
      SW4G_TRY(launch_exp_max(sq, 2 * (long long)n3, slot, stream_));
      stage_emax_ = slot;
      return kOk;
   };

   auto run = [&]() -> int {
      SW4G_TRY(cuda_ok(cudaMemsetAsync(gr_d, 0, npts_ * sizeof(double), stream_)));
      SW4G_TRY(cuda_ok(cudaMemsetAsync(gm_d, 0, npts_ * sizeof(double), stream_)));
      SW4G_TRY(cuda_ok(cudaMemsetAsync(gl_d, 0, npts_ * sizeof(double), stream_)));
      // ghost points of the initial levels from the boundary conditions
      SW4G_TRY(enforce_bc(lev_[iu_]));
      SW4G_TRY(enforce_bc(lev_[ium_]));
      // forward with checkpoints; receivers record from row 0
      rec_rows_ = 0;
      rec_initial_ = true;
      for (int sg = 0; sg < nseg; sg++) {
         const int nn = sg * ckpt, s1 = std::min(nsteps, nn + ckpt);
         double* c0 = ck + 2 * (size_t)sg * n3;
         tseg[sg] = t_;  // the recompute restarts from this time, bit for bit
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(c0, lev_[iu_], lv, cudaMemcpyDeviceToDevice, stream_)));
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(c0 + n3, lev_[ium_], lv, cudaMemcpyDeviceToDevice, stream_)));
         if (!kept(sg)) {
            SW4G_TRY(step(s1 - nn, kModeFused));  // graphed when graphs are on
            continue;
         }
         // a kept segment: every level and predicted level into its buffers
         SW4G_TRY(step(0, kModeFused));  // sources uploaded, the initial record row
         double* sq = seg_of(sg);
         double* pq = pred_of(sg);
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(sq, lev_[ium_], lv, cudaMemcpyDeviceToDevice, stream_)));
         SW4G_TRY(cuda_ok(cudaMemcpyAsync(sq + n3, lev_[iu_], lv, cudaMemcpyDeviceToDevice, stream_)));
         SW4G_TRY(forward_scale(sq, emax + 2 + (nseg - 1 - sg)));
         const int status = steps_into(nn, s1, sq, pq);
         stage_emax_ = nullptr;
         SW4G_TRY(status);
      }
      const double t_end = t_;
      double* fin = work + 5 * n3;  // u^N, u^{N-1}: the recompute overwrites the levels
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(fin, lev_[iu_], lv, cudaMemcpyDeviceToDevice, stream_)));
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(fin + n3, lev_[ium_], lv, cudaMemcpyDeviceToDevice, stream_)));
      // misfit and residuals (host; rows x receivers is small)
      std::vector<double> rec((size_t)(nsteps + 1) * nval), ob((size_t)(nsteps + 1) * nval);
      SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
      SW4G_TRY(cuda_ok(cudaMemcpy(rec.data(), records_, rec.size() * sizeof(double), cudaMemcpyDeviceToHost)));
      SW4G_TRY(cuda_ok(cudaMemcpy(ob.data(), obs, ob.size() * sizeof(double),
                                  obs_on_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost)));
      double J = 0;
      for (size_t q = 0; q < rec.size(); q++) {
         rec[q] -= ob[q];
         J += 0.5 * rec[q] * rec[q];
      }
      *misfit = J;
      SW4G_TRY(cuda_ok(cudaMemcpy(resd, rec.data(), rec.size() * sizeof(double), cudaMemcpyHostToDevice)));
      SW4G_TRY(launch_grad_df_profiles(gp, stream_));
      if (!mixed_) {  // the adjoint level's shift from its sources; the per-point sums zeroed
         SW4G_TRY(cuda_ok(cudaMemsetAsync(dfe, 0, sizeof(double), stream_)));
         const double* stp[3] = {dprof_[3], dprof_[4], dprof_[5]};
         SW4G_TRY(launch_inj_exp(b, stp, drec_.n, drec_.ijk, resd, nsteps + 1, nval, rho_, hz, emax, stream_));
         SW4G_TRY(cuda_ok(cudaMemsetAsync(gd.am, 0, 3 * (size_t)npts_ * sizeof(float2), stream_)));
      }

      double* b1 = work;           // scaled adjoint b = W^-1 R a at n+1
      double* b2 = work + n3;      // at n+2
      double* bn = work + 2 * n3;  // at n
      double* mt = work + 3 * n3;  // b1 + dt^2/12 R L(b1)
      double* w1 = work + 4 * n3;  // the FP64 form's second mt slot
      SW4G_TRY(cuda_ok(cudaMemsetAsync(work, 0, 5 * lv, stream_)));  // not fin
      // b^N = (H W)^-1 R g^N
      if (mixed_)
         adj_source_df_kernel<<<blocks_for(rg.n, 64), 64, 0, stream_>>>(
             b, pf, rg, drec_.ijk, resd + (size_t)nsteps * nval, rho_, hz, F(b1), nullptr, nval);
      else
         adj_source_kernel<<<blocks_for(rg.n, 64), 64, 0, stream_>>>(
             b, pf, rg, drec_.ijk, resd + (size_t)nsteps * nval, rho_, hz, b1, nullptr, nval);
      SW4G_TRY(launch_status());
      // the free-surface ghost planes of an adjoint level
      auto fs_ghosts = [&](double* x, cudaStream_t s) -> int {
         for (int side = 4; side <= 5; side++)
            if (onesided_[side])
               SW4G_TRY(launch_free_surface_ghosts(b, g_.nz, side, mixed_, x, mu_, la_, dprof_[3], dprof_[4],
                                                   g_.h, sbop_, s));
         return kOk;
      };
      // the one-sided rows of an adjoint stage: corrector 0 (mt = u + coef R L(field),
      // u = um = field) or 2 (out = 2u - um + coef R L(field) - beta R SG(u - um))
      const double* dcp[3] = {dprof_[0], dprof_[1], dprof_[2]};
      const double* stp3[3] = {dprof_[3], dprof_[4], dprof_[5]};
      const double* cop[3] = {dprof_[6], dprof_[7], dprof_[8]};
      auto adj_rows = [&](int form, const double* field, const double* u, const double* um, double* out,
                          double coef, double bt, cudaStream_t s) -> int {
         for (int side = 0; side < 2; side++) {
            if (!onesided_[4 + side]) continue;
            if (mixed_) {
               auto CF = [](const double* x) { return reinterpret_cast<const float*>(x); };
               SW4G_TRY(launch_stage_rows_df(form, side == 0, b, g_.nz, nullptr, CF(field), b, mu_, la_, g_.h,
                                             stp3[0], stp3[1], stp3[2], CF(u), CF(um), nullptr, F(out), rho_,
                                             irho_, coef, bt, dcp, stp3, cop, zc_[side], s));
            } else {
               SW4G_TRY(launch_stage_rows(form, side == 0, b, g_.nz, field, b, mu_, la_, g_.h, stp3[0], stp3[1],
                                          stp3[2], u, um, nullptr, out, rho_, irho_, coef, bt, dcp, stp3, cop,
                                          zc_[side], s));
            }
         }
         return kOk;
      };
      SW4G_TRY(fs_ghosts(b1, stream_));
      FusedStage fs;
      fs.b = b;
      fs.k1 = fs_top ? 7 : 1;
      fs.k2 = fs_bot ? g_.nz - 6 : g_.nz;
      fs.mu = mu_;
      fs.la = la_;
      fs.rho = rho_;
      fs.irho = irho_;
      fs.w = w_;
      for (int q = 0; q < 3; q++) {
         fs.st[q] = dprof_[3 + q];
         fs.dc[q] = dprof_[q];
         fs.co[q] = dprof_[6 + q];
      }
      fs.h = g_.h;
      fs.dt = dt;
      const bool keep_rec = drec_.n > 0;
      const int saved_n = drec_.n;
      drec_.n = 0;  // no recording while segments are recomputed
      // one adjoint step nn of the segment starting at s0 (step nn maps u^nn, u^{nn-1}
      // to u^{nn+1}); with the device clock its residual row is clock[2]
      double* segp = seg;  // the buffers of the segment being swept
      double* predp = pred;
      auto adj_step = [&](int nn, int s0, double* b1, double* b2, double* bn, bool clocked, bool wait_g) -> int {
         const double* u = segp + (size_t)(nn - s0 + 1) * n3;
         const double* um = segp + (size_t)(nn - s0) * n3;
         const double* up = predp + (size_t)(nn - s0) * n3;
         const double* un = segp + (size_t)(nn - s0 + 2) * n3;
         const double* clk = clocked ? dclock_ : nullptr;
         const double* res = clocked ? resd : resd + (size_t)nn * nval;
         int status = kOk;
         if (mixed_) {  // double-float b, mt and levels; FP32 stages and gradient terms
            auto CF = [](const double* x) { return reinterpret_cast<const float*>(x); };
            double* mtb = (nn & 1) ? w1 : mt;
            if (wait_g) status = cuda_ok(cudaStreamWaitEvent(sa, ev_g[nn & 1], 0));
            MixedStage m = ms;  // mt = b1 + dt^2/12 R L(b1): predictor form, um = u
            m.corrector = 0;
            m.u = CF(b1);
            m.um = CF(b1);
            m.up = nullptr;
            m.out = F(mtb);
            m.beta = 0;
            m.coef = dt * dt / 12;
            if (status == kOk) status = launch_mixed_stage(m, sa);
            if (status == kOk) status = adj_rows(0, b1, b1, b1, mtb, dt * dt / 12, 0.0, sa);
            if (status == kOk) status = fs_ghosts(mtb, sa);
            if (status == kOk) status = cuda_ok(cudaEventRecord(ev_s0, sa));
            if (status == kOk) status = cuda_ok(cudaStreamWaitEvent(gs, ev_s0, 0));
            if (status == kOk) {
               GradDF g = gd;
               g.lb1 = CF(b1);
               g.lmt = CF(mtb);
               g.lup = CF(up);
               g.lu = CF(u);
               g.lum = CF(um);
               g.lun = CF(un);
               status = launch_grad_f1_step(g, gs);
            }
            for (int side = 0; side < 2 && status == kOk; side++) {
               if (!onesided_[4 + side]) continue;
               GradRows r = gw;
               r.top = side == 0;
               r.lb1 = CF(b1);
               r.lmt = CF(mtb);
               r.lup = CF(up);
               r.lu = CF(u);
               r.lum = CF(um);
               status = launch_grad_rows(r, gs);
            }
            if (status == kOk) status = cuda_ok(cudaEventRecord(ev_g[nn & 1], gs));
            m = ms;  // b^n = 2 b1 - b2 + dt^2 R L(mt) - beta R SG(b1 - b2): adjoint form
            m.corrector = 2;
            m.u = CF(b1);
            m.um = CF(b2);
            m.up = CF(mtb);
            m.out = F(bn);
            m.beta = beta4;
            if (status == kOk) status = launch_mixed_stage(m, sa);
            if (status == kOk) status = adj_rows(2, mtb, b1, b2, bn, dt * dt, beta4, sa);
            if (status == kOk && beta6 != 0) {
               const float* dc32[3] = {prof32_[0], prof32_[1], prof32_[2]};
               const float* st32[3] = {prof32_[3], prof32_[4], prof32_[5]};
               const float* co32[3] = {prof32_[6], prof32_[7], prof32_[8]};
               status = launch_addsgd6_df(3, b, F(bn), CF(b1), CF(b2), rho32_, dc32, st32, co32, beta6, sa, 1);
            }
            if (status == kOk) {
               adj_source_df_kernel<<<blocks_for(rg.n, 64), 64, 0, sa>>>(b, pf, rg, drec_.ijk, res, rho_, hz,
                                                                         F(bn), clk, nval);
               status = launch_status();
            }
            if (status == kOk) status = fs_ghosts(bn, sa);
         } else {
            // mt = b1 + dt^2/12 R L(b1): predictor form, um = u; into the slot whose
            // previous reader, the gradient terms two steps later, has finished
            double* mtb = (nn & 1) ? w1 : mt;
            if (wait_g) status = cuda_ok(cudaStreamWaitEvent(sa, ev_g[nn & 1], 0));
            fs.corrector = 0;
            fs.u = b1;
            fs.um = b1;
            fs.up = nullptr;
            fs.out = mtb;
            fs.beta = 0;
            fs.coef = dt * dt / 12;
            if (status == kOk) status = launch_fused_stage(fs, sa);
            if (status == kOk) status = adj_rows(0, b1, b1, b1, mtb, dt * dt / 12, 0.0, sa);
            if (status == kOk) status = fs_ghosts(mtb, sa);
            if (status == kOk) status = cuda_ok(cudaEventRecord(ev_s0, sa));
            if (status == kOk) status = cuda_ok(cudaStreamWaitEvent(gs, ev_s0, 0));
            if (status == kOk) {  // the gradient terms of the step (double-float sums)
               GradDF g = gd;
               g.b1 = b1;
               g.mt = mtb;
               g.up = up;
               g.u = u;
               g.um = um;
               g.un = un;
               status = launch_grad_df_step(g, gs);
            }
            for (int side = 0; side < 2 && status == kOk; side++) {
               if (!onesided_[4 + side]) continue;
               GradRows r = gw;
               r.top = side == 0;
               r.b1 = b1;
               r.mt = mtb;
               r.up = up;
               r.u = u;
               r.um = um;
               status = launch_grad_rows(r, gs);
            }
            if (status == kOk) status = cuda_ok(cudaEventRecord(ev_g[nn & 1], gs));
            if (status == kOk) {  // b^n = 2 b1 - b2 + dt^2 R L(mt) - beta R SG(b1 - b2)
               fs.corrector = 2;
               fs.u = b1;
               fs.um = b2;
               fs.up = mtb;
               fs.out = bn;
               fs.beta = beta4;
               fs.coef = dt * dt;
               status = launch_fused_stage(fs, sa);
            }
            if (status == kOk) status = adj_rows(2, mtb, b1, b2, bn, dt * dt, beta4, sa);
            if (status == kOk && beta6 != 0)
               status = launch_addsgd6_adj(b, bn, b1, b2, rho_, dcp6, stp6, cop6, beta6, sa);
            if (status == kOk) {
               adj_source_kernel<<<blocks_for(rg.n, 64), 64, 0, sa>>>(b, pf, rg, drec_.ijk, res, rho_, hz, bn,
                                                                     clk, nval);
               status = launch_status();
            }
            if (status == kOk) status = fs_ghosts(bn, sa);
         }
         if (status == kOk && clocked) status = launch_clock_advance(dclock_, 0.0, 0.0, -1.0, sa);
         return status;
      };
      // recompute the segment from its checkpoint: seg[q] = u^{s0-1+q}, pred[q] = up^{s0+q}
      auto recompute = [&](int s0, int s1) -> int {
         SW4G_TRY(forward_scale(seg, emax + 1));
         const int status = steps_into(s0, s1, seg, pred);
         stage_emax_ = nullptr;
         return status;
      };
      // the segment's double-float sums into the FP64 gradients
      auto flush = [&]() -> int {
         if (!mixed_) SW4G_TRY(launch_grad_df_flush(gd, kmu, gm_d, gl_d, gr_d, gs));
         SW4G_TRY(cuda_ok(cudaEventRecord(ev_join, gs)));
         SW4G_TRY(cuda_ok(cudaStreamWaitEvent(hs, ev_join, 0)));
         SW4G_TRY(cuda_ok(cudaEventRecord(ev_back, hs)));
         return cuda_ok(cudaStreamWaitEvent(stream_, ev_back, 0));
      };
      // a segment's adjoint steps start after everything before them on the object's stream
      auto fork = [&]() -> int {
         SW4G_TRY(cuda_ok(cudaEventRecord(ev_fork, stream_)));
         return cuda_ok(cudaStreamWaitEvent(hs, ev_fork, 0));
      };
      auto rotate = [&]() {
         double* tmp = b2;
         b2 = b1;
         b1 = bn;
         bn = tmp;
      };
      // CUDA graphs of full segments: one recompute graph (every full segment starts
      // in the same level rotation state) and one adjoint graph per rotation phase
      // of (b1, b2, bn); the first adjoint segment runs directly
      cudaGraphExec_t rgraph = nullptr;
      int r_iu = 0, r_ium = 0;
      struct AdjGraph {
         double* b1;
         double* seg;
         cudaGraphExec_t exec;
      };
      std::vector<AdjGraph> agraphs;
      bool adj_warm = false;
      int status = kOk;
      // Without graphs and with two or more kept segments, the backward sweep is
      // pipelined: each segment buffer freed by a finished sweep receives the recompute
      // of the next segment to recompute, on its own stream beside the next sweep (the
      // recompute's FP64 stages then share the GPU with the sweep's, and the gradient
      // terms find room beside the predictor-form stages of both).  The same kernels on
      // the same data in the same order per stream: results are bit-identical.
      const bool pipelined = !graphs_ && nkept >= 2 && nseg > nkept && adjoint_pipeline_enabled();
      if (pipelined) {
         struct Buf {
            double* sq;
            double* pq;
         };
         std::vector<Buf> bufof(nseg, Buf{nullptr, nullptr});
         for (int sg = nseg - nkept; sg < nseg; sg++) bufof[sg] = Buf{seg_of(sg), pred_of(sg)};
         std::vector<cudaEvent_t> ready(nseg, nullptr), swept(nseg, nullptr);
         cudaStream_t rcs = nullptr;
         int lo_pr = 0, hi_pr = 0;
         status = cuda_ok(cudaDeviceGetStreamPriorityRange(&lo_pr, &hi_pr));
         if (status == kOk) status = cuda_ok(cudaStreamCreateWithPriority(&rcs, cudaStreamNonBlocking, lo_pr));
         for (int sg = 0; sg < nseg && status == kOk; sg++) {
            status = cuda_ok(cudaEventCreateWithFlags(&ready[sg], cudaEventDisableTiming));
            if (status == kOk) status = cuda_ok(cudaEventCreateWithFlags(&swept[sg], cudaEventDisableTiming));
         }
         // recompute segment r into buffer bf on rcs (the object's stream swapped for the
         // enqueue), after the sweep that last used bf
         auto recompute_into = [&](int r, Buf bf, cudaEvent_t after) -> int {
            const int r0 = r * ckpt, r1 = std::min(nsteps, r0 + ckpt);
            SW4G_TRY(cuda_ok(cudaStreamWaitEvent(rcs, after, 0)));
            cudaStream_t own = stream_;
            stream_ = rcs;
            int st2 = kOk;
            const double* c0 = ck + 2 * (size_t)r * n3;
            st2 = cuda_ok(cudaMemcpyAsync(bf.sq, c0 + n3, lv, cudaMemcpyDeviceToDevice, stream_));
            if (st2 == kOk) st2 = cuda_ok(cudaMemcpyAsync(bf.sq + n3, c0, lv, cudaMemcpyDeviceToDevice, stream_));
            t_ = tseg[r];
            if (st2 == kOk) st2 = forward_scale(bf.sq, emax + 2 + (nseg - 1 - r));
            if (st2 == kOk) st2 = steps_into(r0, r1, bf.sq, bf.pq);
            stage_emax_ = nullptr;
            if (st2 == kOk) st2 = cuda_ok(cudaEventRecord(ready[r], stream_));
            stream_ = own;
            return st2;
         };
         int next_rc = nseg - nkept - 1;
         for (int sg = nseg - 1; sg >= 0 && status == kOk; sg--) {
            const int s0 = sg * ckpt, s1 = std::min(nsteps, s0 + ckpt);
            segp = bufof[sg].sq;
            predp = bufof[sg].pq;
            status = fork();
            if (status == kOk && !kept(sg)) status = cuda_ok(cudaStreamWaitEvent(hs, ready[sg], 0));
            // the forward levels' shift of this segment, from its own slot
            if (status == kOk && !mixed_)
               status = cuda_ok(cudaMemcpyAsync(emax + 1, emax + 2 + (nseg - 1 - sg), sizeof(int),
                                                cudaMemcpyDeviceToDevice, hs));
            for (int nn = s1 - 1; nn >= s0 && status == kOk; nn--) {
               status = adj_step(nn, s0, b1, b2, bn, false, nn + 2 <= s1 - 1);
               rotate();
            }
            if (status == kOk) status = flush();
            if (status == kOk) status = cuda_ok(cudaEventRecord(swept[sg], hs));
            if (status == kOk && next_rc >= 0) {
               bufof[next_rc] = bufof[sg];
               status = recompute_into(next_rc, bufof[sg], swept[sg]);
               next_rc--;
            }
         }
         if (rcs) {
            cudaStreamSynchronize(rcs);
            cudaStreamDestroy(rcs);
         }
         cudaStreamSynchronize(hs);
         for (int sg = 0; sg < nseg; sg++) {
            if (ready[sg]) cudaEventDestroy(ready[sg]);
            if (swept[sg]) cudaEventDestroy(swept[sg]);
         }
      }
      for (int sg = nseg - 1; sg >= 0 && status == kOk && !pipelined; sg--) {
         const int s0 = sg * ckpt, s1 = std::min(nsteps, s0 + ckpt);
         const bool full = graphs_ && s1 - s0 == ckpt;
         segp = seg_of(sg);
         predp = pred_of(sg);
         if (kept(sg)) {  // its forward levels' shift, from the forward run
            if (!mixed_)
               status = cuda_ok(cudaMemcpyAsync(emax + 1, emax + 2 + (nseg - 1 - sg), sizeof(int),
                                                cudaMemcpyDeviceToDevice, stream_));
         } else {
            if (full) {
               iu_ = 2;
               ium_ = 3;
            }
            double* c0 = ck + 2 * (size_t)sg * n3;
            status = cuda_ok(cudaMemcpyAsync(seg, c0 + n3, lv, cudaMemcpyDeviceToDevice, stream_));
            if (status == kOk) status = cuda_ok(cudaMemcpyAsync(seg + n3, c0, lv, cudaMemcpyDeviceToDevice, stream_));
            t_ = tseg[sg];
            if (status == kOk && full) {
               status = sync_clock();
               clocked_ = true;
               if (status == kOk && !rgraph) {
                  status = capture([&]() { return recompute(s0, s1); }, &rgraph);
                  r_iu = iu_;
                  r_ium = ium_;
                  if (status == kOk) status = cuda_ok(cudaGraphLaunch(rgraph, stream_));
               } else if (status == kOk) {
                  status = cuda_ok(cudaGraphLaunch(rgraph, stream_));
                  iu_ = r_iu;
                  ium_ = r_ium;
               }
               clocked_ = false;
            } else if (status == kOk) {
               status = recompute(s0, s1);
            }
         }
         if (status != kOk) break;
         if (full && adj_warm) {
            status = sync_clock((double)(s1 - 1));
            cudaGraphExec_t ex = nullptr;
            for (auto& g : agraphs)
               if (g.b1 == b1 && g.seg == segp) ex = g.exec;
            if (status == kOk && !ex) {
               double* key = b1;
               status = capture([&]() -> int {
                  SW4G_TRY(fork());
                  for (int nn = s1 - 1; nn >= s0; nn--) {
                     SW4G_TRY(adj_step(nn, s0, b1, b2, bn, true, nn + 2 <= s1 - 1));
                     rotate();
                  }
                  return flush();
               }, &ex);
               if (status == kOk) {
                  agraphs.push_back(AdjGraph{key, segp, ex});
                  status = cuda_ok(cudaGraphLaunch(ex, stream_));
               }
            } else if (status == kOk) {
               status = cuda_ok(cudaGraphLaunch(ex, stream_));
               for (int nn = s1 - 1; nn >= s0; nn--) rotate();
            }
         } else {
            status = fork();
            for (int nn = s1 - 1; nn >= s0 && status == kOk; nn--) {
               status = adj_step(nn, s0, b1, b2, bn, false, nn + 2 <= s1 - 1);
               rotate();
            }
            if (status == kOk) status = flush();
            adj_warm = true;
         }
      }
      if (rgraph || !agraphs.empty()) cudaStreamSynchronize(stream_);
      if (rgraph) cudaGraphExecDestroy(rgraph);
      for (auto& g : agraphs) cudaGraphExecDestroy(g.exec);
      drec_.n = keep_rec ? saved_n : 0;
      if (status != kOk) return status;
      // the object ends where the forward run ended
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[iu_], fin, lv, cudaMemcpyDeviceToDevice, stream_)));
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[ium_], fin + n3, lv, cudaMemcpyDeviceToDevice, stream_)));
      t_ = t_end;
      return kOk;
   };
   st = run();
   stage_emax_ = nullptr;
   if (st == kOk && !grad_on_device) {
      st = cuda_ok(cudaMemcpyAsync(g_rho, gr_d, npts_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
      if (st == kOk)
         st = cuda_ok(cudaMemcpyAsync(g_mu, gm_d, npts_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
      if (st == kOk)
         st = cuda_ok(cudaMemcpyAsync(g_la, gl_d, npts_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
   }
   // the mixed form's tensor-copy stages report a wait that gave up in the status block
   if (st == kOk && mixed_) st = status();
   cleanup();
   if (st != kOk) drop_grad_cache();
   return st;
}

void EW::drop_grad_cache()
{
   if (!gcache_.mem.empty()) cudaStreamSynchronize(stream_);
   for (void* p : gcache_.mem) cudaFree(p);
   gcache_ = GradCache{};
}

}  // namespace sw4g
