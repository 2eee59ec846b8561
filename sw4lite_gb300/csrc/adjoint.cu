// Discrete adjoint of the FP64 Cartesian time step and the material gradient of
// a receiver misfit, sm_103a.
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
// two operator applications per step like the forward.  The gradient of
// a1 . u+ at fixed (u, um):
//   mu, lambda : G(dt^2/12 R a1, up - 2u + um) + G(dt^2 R m, u), G(v, w) the
//                coefficient gradient of v . L(w) (a local gather: the derivative
//                of each second-difference row with respect to its five
//                coefficients, and minus products of first differences for the
//                mixed terms);
//   rho        : -(1/rho)[m.(up - 2u + um) + a1.(u+ - up)] (the 1/rho factors and
//                the forcing) - beta dc D2(u - um) . D2(w R a1) (the damping's
//                rho dc factors).
// Forward levels come from checkpoints every C steps, recomputed one segment
// at a time with every level and predicted level kept in HBM.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ew.h"

namespace sw4g {
namespace {

__device__ __forceinline__ bool inside(const Box& b, int i, int j, int k)
{
   return i >= b.ib + 2 && i <= b.ie - 2 && j >= b.jb + 2 && j <= b.je - 2 && k >= b.kb + 2 &&
          k <= b.ke - 2;
}

struct Prof {
   const double *dc[3], *st[3], *co[3];
};

__device__ __forceinline__ double sxyz(const Box& b, const Prof& f, int i, int j, int k)
{
   return f.st[0][i - b.ib] * f.st[1][j - b.jb] * f.st[2][k - b.kb];
}

__device__ __forceinline__ void grid_point(const Box& b, long long p, int& i, int& j, int& k)
{
   i = b.ib + (int)(p % b.ni);
   j = b.jb + (int)((p / b.ni) % (b.je - b.jb + 1));
   k = b.kb + (int)(p / b.nij);
}

// y = a * (sx sy sz) / rho on I, 0 elsewhere  (W^-1 R a)
__global__ void adj_scale_kernel(Box b, Prof f, const double* __restrict__ a,
                                 const double* __restrict__ rho, double* __restrict__ y)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      grid_point(b, p, i, j, k);
      const double s = inside(b, i, j, k) ? sxyz(b, f, i, j, k) / rho[p] : 0.0;
#pragma unroll
      for (int c = 0; c < 3; c++) y[c * b.npts + p] = s * a[c * b.npts + p];
   }
}

// s = W lu, m = a1 + dt^2/12 s, y = W^-1 R m  (on I; 0 elsewhere)
__global__ void adj_mid_kernel(Box b, Prof f, const double* __restrict__ lu,
                               const double* __restrict__ a1, const double* __restrict__ rho,
                               double c12, double* __restrict__ s, double* __restrict__ m,
                               double* __restrict__ y)
{
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      grid_point(b, p, i, j, k);
      const bool in = inside(b, i, j, k);
      const double iw = in ? sxyz(b, f, i, j, k) : 0.0;
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = c * b.npts + p;
         const double sv = in ? lu[q] / iw : 0.0;
         const double mv = in ? a1[q] + c12 * sv : 0.0;
         s[q] = sv;
         m[q] = mv;
         y[q] = in ? mv * iw / rho[p] : 0.0;
      }
   }
}

// a^n = 2m + dt^2 W lu - dt^2/6 s - a2 - beta SG^T R (a1 - a2) on I; 0 elsewhere
__global__ void adj_final_kernel(Box b, Prof f, const double* __restrict__ lu,
                                 const double* __restrict__ s, const double* __restrict__ m,
                                 const double* __restrict__ a1, const double* __restrict__ a2,
                                 const double* __restrict__ rho, double dt2, double beta,
                                 double* __restrict__ an)
{
   const long long st[3] = {1, b.ni, b.nij};
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < b.npts;
        p += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      grid_point(b, p, i, j, k);
      if (!inside(b, i, j, k)) {
#pragma unroll
         for (int c = 0; c < 3; c++) an[c * b.npts + p] = 0.0;
         continue;
      }
      const double w = 1.0 / sxyz(b, f, i, j, k);
      const int pc[3] = {i, j, k};
      const int lo[3] = {b.ib, b.jb, b.kb};
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const long long q = c * b.npts + p;
         double sg = 0;
         if (beta != 0) {
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
               double v[5];
#pragma unroll
               for (int mm = -2; mm <= 2; mm++) {
                  int qc[3] = {i, j, k};
                  qc[ax] += mm;
                  if (!inside(b, qc[0], qc[1], qc[2])) {
                     v[mm + 2] = 0;
                     continue;
                  }
                  const long long pq = p + mm * st[ax];
                  const int oi = qc[0] - b.ib, oj = qc[1] - b.jb, ok = qc[2] - b.kb;
                  const double wax = ax == 0   ? f.st[0][oi] * f.co[1][oj] * f.co[2][ok]
                                     : ax == 1 ? f.st[1][oj] * f.co[0][oi] * f.co[2][ok]
                                               : f.st[2][ok] * f.co[0][oi] * f.co[1][oj];
                  v[mm + 2] = wax * (a1[c * b.npts + pq] - a2[c * b.npts + pq]) / rho[pq];
               }
               const double* dc = f.dc[ax] + (pc[ax] - lo[ax]);
               const double e0 = rho[p - st[ax]] * dc[-1], e1 = rho[p] * dc[0],
                            e2 = rho[p + st[ax]] * dc[1];
               sg += e2 * (v[4] - 2 * v[3] + v[2]) - 2 * e1 * (v[3] - 2 * v[2] + v[1]) +
                     e0 * (v[2] - 2 * v[1] + v[0]);
            }
         }
         an[q] = 2 * m[q] + dt2 * w * lu[q] - dt2 / 6 * s[q] - a2[q] - beta * sg;
      }
   }
}

// an[receiver point] += residual row (receivers in order, 3 values each)
__global__ void adj_source_kernel(Box b, int nrec, const int* __restrict__ ijk,
                                  const double* __restrict__ res, double* __restrict__ an)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nrec) return;
   const long long p = pidx(b, ijk[3 * r], ijk[3 * r + 1], ijk[3 * r + 2]);
#pragma unroll
   for (int c = 0; c < 3; c++) an[c * b.npts + p] += res[3 * r + c];
}

__device__ constexpr double kDW[5] = {1, -8, 0, 8, -1};
// mixed terms of the operator: (equation, component, outer axis, inner axis, lambda?)
__device__ constexpr int kMix[12][5] = {{0, 1, 0, 1, 1}, {0, 1, 1, 0, 0}, {0, 2, 0, 2, 1},
                                        {0, 2, 2, 0, 0}, {1, 0, 0, 1, 0}, {1, 0, 1, 0, 1},
                                        {1, 2, 1, 2, 1}, {1, 2, 2, 1, 0}, {2, 0, 0, 2, 0},
                                        {2, 0, 2, 0, 1}, {2, 1, 1, 2, 0}, {2, 1, 2, 1, 1}};

struct GradArgs {
   Box b;
   Prof f;
   const double *a1, *m, *rho, *u, *um, *up, *un;
   double* gr;
   double* gm;
   double* gl;
   double c1, c2;  // dt^2/12 and dt^2: v1 = c1 R a1, v2 = c2 R m
   double ih2, beta;
};

// gradient of a1 . u+ at every array point (one thread per point)
__global__ void __launch_bounds__(128) adj_gradient_kernel(GradArgs g)
{
   const Box& b = g.b;
   const long long n = b.npts;
   const long long st[3] = {1, b.ni, b.nij};
   const int lo[3] = {b.ib, b.jb, b.kb}, hi[3] = {b.ie, b.je, b.ke};
   for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
        p += (long long)gridDim.x * blockDim.x) {
      int pc[3];
      grid_point(b, p, pc[0], pc[1], pc[2]);
      double gm = 0, gl = 0, gr = 0;
      // v of pair t at point q (component c); zero outside I
      auto vat = [&](int t, int c, long long q) {
         return (t == 0 ? g.c1 * g.a1[c * n + q] : g.c2 * g.m[c * n + q]) / g.rho[q];
      };
      // w of pair t at point q
      auto wat = [&](int t, int c, long long q) {
         return t == 0 ? g.up[c * n + q] - 2 * g.u[c * n + q] + g.um[c * n + q] : g.u[c * n + q];
      };
#pragma unroll
      for (int t = 0; t < 2; t++) {
         // same-axis second differences: rows q = p - nn e_ax
#pragma unroll
         for (int ax = 0; ax < 3; ax++)
#pragma unroll
            for (int nn = -2; nn <= 2; nn++) {
               int qc[3] = {pc[0], pc[1], pc[2]};
               qc[ax] -= nn;
               if (!inside(b, qc[0], qc[1], qc[2])) continue;
               const long long q = p - nn * st[ax];
               const double sq = g.f.st[ax][qc[ax] - lo[ax]], sp = g.f.st[ax][pc[ax] - lo[ax]];
#pragma unroll
               for (int c = 0; c < 3; c++) {
                  const double vq = vat(t, c, q);
                  double d[5];
#pragma unroll
                  for (int mm = -2; mm <= 2; mm++) d[mm + 2] = wat(t, c, q + mm * st[ax]) - wat(t, c, q);
                  double K;
                  if (nn == -2) K = -0.75 * d[0] + d[1];
                  else if (nn == -1) K = d[0] + 3 * d[1] + d[3];
                  else if (nn == 0) K = -0.75 * (d[0] + d[4]) + 3 * (d[1] + d[3]);
                  else if (nn == 1) K = d[1] + 3 * d[3] + d[4];
                  else K = d[3] - 0.75 * d[4];
                  const double fv = g.ih2 / 6 * vq * sq * K * sp;
                  if (c == ax) {
                     gm += 2 * fv;
                     gl += fv;
                  } else {
                     gm += fv;
                  }
               }
            }
         // mixed terms: -(1/144h^2) s_ai(p) (DW . w_d along ai)(p) (DW . (s_ao v_c) along ao)(p)
#pragma unroll
         for (int e = 0; e < 12; e++) {
            const int c = kMix[e][0], d = kMix[e][1], ao = kMix[e][2], ai = kMix[e][3];
            if (pc[ai] < lo[ai] + 2 || pc[ai] > hi[ai] - 2) continue;
            double inner = 0, outer = 0;
#pragma unroll
            for (int mm = -2; mm <= 2; mm++) {
               if (mm == 0) continue;
               inner += kDW[mm + 2] * wat(t, d, p + mm * st[ai]);
               int oc[3] = {pc[0], pc[1], pc[2]};
               oc[ao] += mm;
               if (oc[ao] < lo[ao] || oc[ao] > hi[ao] || !inside(b, oc[0], oc[1], oc[2])) continue;
               outer += kDW[mm + 2] * g.f.st[ao][oc[ao] - lo[ao]] * vat(t, c, p + mm * st[ao]);
            }
            const double gg = -g.ih2 / 144 * g.f.st[ai][pc[ai] - lo[ai]] * inner * outer;
            if (kMix[e][4]) gl += gg;
            else gm += gg;
         }
      }
      // rho: the 1/rho factors and forcing (interior points), and the damping's rho dc
      if (inside(b, pc[0], pc[1], pc[2])) {
         double s = 0;
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const long long q = c * n + p;
            s += g.m[q] * (g.up[q] - 2 * g.u[q] + g.um[q]) + g.a1[q] * (g.un[q] - g.up[q]);
         }
         gr -= s / g.rho[p];
      }
      if (g.beta != 0) {
         double sgr = 0;
#pragma unroll
         for (int ax = 0; ax < 3; ax++) {
            if (pc[ax] - 1 < lo[ax] || pc[ax] + 1 > hi[ax]) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               double vv[3], dd[3];
#pragma unroll
               for (int mm = -1; mm <= 1; mm++) {
                  int qc[3] = {pc[0], pc[1], pc[2]};
                  qc[ax] += mm;
                  const long long q = p + mm * st[ax];
                  dd[mm + 1] = g.u[c * n + q] - g.um[c * n + q];
                  if (inside(b, qc[0], qc[1], qc[2])) {
                     const int oi = qc[0] - b.ib, oj = qc[1] - b.jb, ok = qc[2] - b.kb;
                     const double wax = ax == 0   ? g.f.st[0][oi] * g.f.co[1][oj] * g.f.co[2][ok]
                                        : ax == 1 ? g.f.st[1][oj] * g.f.co[0][oi] * g.f.co[2][ok]
                                                  : g.f.st[2][ok] * g.f.co[0][oi] * g.f.co[1][oj];
                     vv[mm + 1] = wax * g.a1[c * n + q] / g.rho[q];
                  } else {
                     vv[mm + 1] = 0;
                  }
               }
               sgr += g.f.dc[ax][pc[ax] - lo[ax]] * (dd[2] - 2 * dd[1] + dd[0]) *
                      (vv[2] - 2 * vv[1] + vv[0]);
            }
         }
         gr -= g.beta * sgr;
      }
      g.gm[p] += gm;
      g.gl[p] += gl;
      g.gr[p] += gr;
   }
}

int gs_blocks(long long n, int threads)
{
   long long b = (n + threads - 1) / threads;
   if (b > 152 * 32) b = 152 * 32;
   return (int)(b > 0 ? b : 1);
}

}  // namespace

int EW::gradient(int nsteps, int ckpt, const double* obs, bool obs_on_device, double* misfit,
                 double* g_rho, double* g_mu, double* g_la, bool grad_on_device)
{
   if (!ready_ || !material_ || !(dt_ > 0) || nsteps < 1 || ckpt < 1 || !obs || !misfit || !g_rho ||
       !g_mu || !g_la)
      return kBadArgument;
   if (mixed_ || cv_ || g_.sg_order != 4) return kNotSupported;
   for (int s = 0; s < 6; s++)
      if (g_.bc[s] != kDirichlet && g_.bc[s] != kSuperGrid) return kNotSupported;
   if (drec_.n == 0) return kBadArgument;
   {
      std::vector<int> modes(drec_.n);
      SW4G_TRY(cuda_ok(cudaMemcpy(modes.data(), drec_.mode, drec_.n * sizeof(int), cudaMemcpyDeviceToHost)));
      for (int m : modes)
         if (m != kRecDisplacement) return kNotSupported;
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
   const double t0 = t_, dt = dt_;

   // device memory: checkpoints, one segment of levels and predicted levels, adjoint work
   std::vector<double*> bufs;
   auto alloc = [&](double** p, size_t bytes) {
      int st = cuda_ok(cudaMalloc(p, bytes));
      if (st == kOk) bufs.push_back(*p);
      return st;
   };
   double *ck = nullptr, *seg = nullptr, *pred = nullptr, *work = nullptr, *resd = nullptr;
   int st = alloc(&ck, 2 * (size_t)nseg * lv);
   if (st == kOk) st = alloc(&seg, (size_t)(seglen + 2) * lv);
   if (st == kOk) st = alloc(&pred, (size_t)seglen * lv);
   if (st == kOk) st = alloc(&work, 9 * lv);  // adjoint work (7) + the forward's final levels (2)
   if (st == kOk) st = alloc(&resd, (size_t)(nsteps + 1) * nval * sizeof(double));
   double* gr_d = g_rho;
   double* gm_d = g_mu;
   double* gl_d = g_la;
   double* gtmp = nullptr;
   if (st == kOk && !grad_on_device) {
      st = alloc(&gtmp, 3 * (size_t)npts_ * sizeof(double));
      gr_d = gtmp;
      gm_d = gtmp + npts_;
      gl_d = gtmp + 2 * npts_;
   }
   auto cleanup = [&]() {
      cudaStreamSynchronize(stream_);
      for (double* p : bufs) cudaFree(p);
   };
   if (st != kOk) {
      cleanup();
      return st;
   }
   const int blocks = gs_blocks(npts_, 256);
   Prof pf;
   for (int a = 0; a < 3; a++) {
      pf.dc[a] = dprof_[a];
      pf.st[a] = dprof_[3 + a];
      pf.co[a] = dprof_[6 + a];
   }
   const double beta = (prof_.used && g_.sg_damping != 0) ? g_.sg_damping : 0.0;
   const int onesided[6] = {0, 0, 0, 0, 0, 0};

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
      for (int nn = 0; nn < nsteps; nn++) {
         if (nn % ckpt == 0) {
            double* c0 = ck + 2 * (size_t)(nn / ckpt) * n3;
            SW4G_TRY(cuda_ok(cudaMemcpyAsync(c0, lev_[iu_], lv, cudaMemcpyDeviceToDevice, stream_)));
            SW4G_TRY(cuda_ok(cudaMemcpyAsync(c0 + n3, lev_[ium_], lv, cudaMemcpyDeviceToDevice, stream_)));
         }
         SW4G_TRY(step(1, kModeFused));
      }
      const double t_end = t_;
      double* fin = work + 7 * n3;  // u^N, u^{N-1}: the recompute overwrites the levels
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

      double* a1 = work;
      double* a2 = work + n3;
      double* an = work + 2 * n3;
      double* s = work + 3 * n3;
      double* m = work + 4 * n3;
      double* y = work + 5 * n3;
      double* lu = work + 6 * n3;
      SW4G_TRY(cuda_ok(cudaMemsetAsync(work, 0, 7 * lv, stream_)));  // not fin
      // a^N = g^N
      adj_source_kernel<<<blocks_for(drec_.n, 64), 64, 0, stream_>>>(b, drec_.n, drec_.ijk,
                                                                     resd + (size_t)nsteps * nval, a1);
      SW4G_TRY(launch_status());
      const bool keep_rec = drec_.n > 0;
      const int saved_n = drec_.n;
      drec_.n = 0;  // no recording while segments are recomputed
      int status = kOk;
      for (int sg = nseg - 1; sg >= 0 && status == kOk; sg--) {
         const int s0 = sg * ckpt, s1 = std::min(nsteps, s0 + ckpt);
         // recompute the segment: seg[q] = u^{s0-1+q}, pred[q] = up^{s0+q}
         double* c0 = ck + 2 * (size_t)sg * n3;
         status = cuda_ok(cudaMemcpyAsync(lev_[iu_], c0, lv, cudaMemcpyDeviceToDevice, stream_));
         if (status == kOk)
            status = cuda_ok(cudaMemcpyAsync(lev_[ium_], c0 + n3, lv, cudaMemcpyDeviceToDevice, stream_));
         if (status == kOk) status = cuda_ok(cudaMemcpyAsync(seg, c0 + n3, lv, cudaMemcpyDeviceToDevice, stream_));
         if (status == kOk) status = cuda_ok(cudaMemcpyAsync(seg + n3, c0, lv, cudaMemcpyDeviceToDevice, stream_));
         t_ = t0 + s0 * dt;
         for (int nn = s0; nn < s1 && status == kOk; nn++) {
            capture_pred_ = pred + (size_t)(nn - s0) * n3;
            status = step(1, kModeFused);
            capture_pred_ = nullptr;
            if (status == kOk)
               status = cuda_ok(cudaMemcpyAsync(seg + (size_t)(nn - s0 + 2) * n3, lev_[iu_], lv,
                                                cudaMemcpyDeviceToDevice, stream_));
         }
         // adjoint steps nn = s1-1 .. s0 (step nn maps u^nn, u^{nn-1} to u^{nn+1})
         for (int nn = s1 - 1; nn >= s0 && status == kOk; nn--) {
            const double* u = seg + (size_t)(nn - s0 + 1) * n3;
            const double* um = seg + (size_t)(nn - s0) * n3;
            const double* up = pred + (size_t)(nn - s0) * n3;
            const double* un = seg + (size_t)(nn - s0 + 2) * n3;
            adj_scale_kernel<<<blocks, 256, 0, stream_>>>(b, pf, a1, rho_, y);
            status = launch_status();
            if (status == kOk)
               status = launch_rhs4sg_direct(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, g_.nz,
                                             onesided, lu, y, mu_, la_, g_.h, dprof_[3], dprof_[4],
                                             dprof_[5], stream_);
            if (status == kOk) {
               adj_mid_kernel<<<blocks, 256, 0, stream_>>>(b, pf, lu, a1, rho_, dt * dt / 12, s, m, y);
               status = launch_status();
            }
            if (status == kOk)
               status = launch_rhs4sg_direct(1, bd.ib, bd.ie, bd.jb, bd.je, bd.kb, bd.ke, g_.nz,
                                             onesided, lu, y, mu_, la_, g_.h, dprof_[3], dprof_[4],
                                             dprof_[5], stream_);
            if (status == kOk) {
               GradArgs ga;
               ga.b = b;
               ga.f = pf;
               ga.a1 = a1;
               ga.m = m;
               ga.rho = rho_;
               ga.u = u;
               ga.um = um;
               ga.up = up;
               ga.un = un;
               ga.gr = gr_d;
               ga.gm = gm_d;
               ga.gl = gl_d;
               ga.c1 = dt * dt / 12;
               ga.c2 = dt * dt;
               ga.ih2 = 1 / (g_.h * g_.h);
               ga.beta = beta;
               adj_gradient_kernel<<<gs_blocks(npts_, 128), 128, 0, stream_>>>(ga);
               status = launch_status();
            }
            if (status == kOk) {
               adj_final_kernel<<<blocks, 256, 0, stream_>>>(b, pf, lu, s, m, a1, a2, rho_, dt * dt,
                                                             beta, an);
               status = launch_status();
            }
            if (status == kOk) {
               adj_source_kernel<<<blocks_for(saved_n, 64), 64, 0, stream_>>>(
                   b, saved_n, drec_.ijk, resd + (size_t)nn * nval, an);
               status = launch_status();
            }
            // rotate: a2 <- a1, a1 <- a^nn
            double* tmp = a2;
            a2 = a1;
            a1 = an;
            an = tmp;
         }
      }
      drec_.n = keep_rec ? saved_n : 0;
      if (status != kOk) return status;
      // the object ends where the forward run ended
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[iu_], fin, lv, cudaMemcpyDeviceToDevice, stream_)));
      SW4G_TRY(cuda_ok(cudaMemcpyAsync(lev_[ium_], fin + n3, lv, cudaMemcpyDeviceToDevice, stream_)));
      t_ = t_end;
      return kOk;
   };
   st = run();
   if (st == kOk && !grad_on_device) {
      st = cuda_ok(cudaMemcpyAsync(g_rho, gr_d, npts_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
      if (st == kOk)
         st = cuda_ok(cudaMemcpyAsync(g_mu, gm_d, npts_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
      if (st == kOk)
         st = cuda_ok(cudaMemcpyAsync(g_la, gl_d, npts_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
   }
   cleanup();
   return st;
}

}  // namespace sw4g
