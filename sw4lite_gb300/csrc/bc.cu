// Ghost-point closures on a Cartesian grid, sm_103a: the replacement for the
// reference's bcfortsg / bcfortsg_indrev (src/ew-cfromfort.C:205-746).
//
// Sides are processed in order 0..5 on the caller's stream, one launch per active
// side, because windows of later sides overlap earlier ones at edges and the
// free-surface solve reads ghost values written by the lateral sides.
//   bccnd 1 (Dirichlet) / 2 (supergrid): copy the boundary data into the 2 ghost
//     planes of the side's window (zero when no data array is given);
//   bccnd 3 (periodic): copy from the point one period inside;
//   bccnd 0 (free surface, sides 4/5): solve the ghost plane k=0 (k=nz+1) from
//     the traction condition with the one-sided boundary stencil sbop.
#include "common.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

struct Win {
   int i0, i1, j0, j1, k0, k1;
};

template <class Field>
__global__ void fill_window_kernel(Box b, Win w, Field u, const double* __restrict__ bforce)
{
   const long long idel = w.i1 - w.i0 + 1, ijdel = idel * (w.j1 - w.j0 + 1);
   const long long n = ijdel * (w.k1 - w.k0 + 1);
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x) {
      const int k = w.k0 + (int)(q / ijdel);
      const long long r = q % ijdel;
      const int j = w.j0 + (int)(r / idel);
      const int i = w.i0 + (int)(r % idel);
#pragma unroll
      for (int c = 0; c < 3; c++) u.set(cidx(b, c, i, j, k), bforce ? bforce[3 * q + c] : 0.0);
   }
}

template <class Field>
__global__ void periodic_window_kernel(Box b, Win w, Field u, int di, int dj, int dk)
{
   const long long idel = w.i1 - w.i0 + 1, ijdel = idel * (w.j1 - w.j0 + 1);
   const long long n = ijdel * (w.k1 - w.k0 + 1);
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x) {
      const int k = w.k0 + (int)(q / ijdel);
      const long long r = q % ijdel;
      const int j = w.j0 + (int)(r / idel);
      const int i = w.i0 + (int)(r % idel);
#pragma unroll
      for (int c = 0; c < 3; c++) u.set(cidx(b, c, i, j, k), u.get(cidx(b, c, i + di, j + dj, k + dk)));
   }
}

struct FreeSurf {
   double sbop[5];
};

// Ghost plane of a flat free surface (src/ew-cfromfort.C:415-476, :686-744).
template <class Field>
__global__ void free_surface_kernel(Box b, Field u, const double* __restrict__ mu,
                                    const double* __restrict__ la,
                                    const double* __restrict__ bforce,
                                    const double* __restrict__ strx,
                                    const double* __restrict__ stry, double h, int k, int kl,
                                    FreeSurf fs)
{
   const int i = b.ib + 2 + blockIdx.x * blockDim.x + threadIdx.x;
   const int j = b.jb + 2 + blockIdx.y * blockDim.y + threadIdx.y;
   if (i > b.ie - 2 || j > b.je - 2) return;
   const double d4a = 2.0 / 3.0, d4b = -1.0 / 12.0;
   const long long qq = (i - b.ib) + b.ni * (j - b.jb);
   const long long p = pidx(b, i, j, k);
   auto U = [&](int c, int ii, int jj, int kk) { return u.get(cidx(b, c, ii, jj, kk)); };
   const double sx = strx[i - b.ib], sy = stry[j - b.jb];
   const double wx = sx * (d4a * (U(2, i + 1, j, k) - U(2, i - 1, j, k)) +
                           d4b * (U(2, i + 2, j, k) - U(2, i - 2, j, k)));
   const double ux = sx * (d4a * (U(0, i + 1, j, k) - U(0, i - 1, j, k)) +
                           d4b * (U(0, i + 2, j, k) - U(0, i - 2, j, k)));
   const double wy = sy * (d4a * (U(2, i, j + 1, k) - U(2, i, j - 1, k)) +
                           d4b * (U(2, i, j + 2, k) - U(2, i, j - 2, k)));
   const double vy = sy * (d4a * (U(1, i, j + 1, k) - U(1, i, j - 1, k)) +
                           d4b * (U(1, i, j + 2, k) - U(1, i, j - 2, k)));
   double uz = 0, vz = 0, wz = 0;
#pragma unroll
   for (int q = 1; q <= 4; q++) {
      const int kq = k + kl * (q - 1);
      uz += fs.sbop[q] * U(0, i, j, kq);
      vz += fs.sbop[q] * U(1, i, j, kq);
      wz += fs.sbop[q] * U(2, i, j, kq);
   }
   const double f0 = bforce ? bforce[3 * qq] : 0.0;
   const double f1 = bforce ? bforce[3 * qq + 1] : 0.0;
   const double f2 = bforce ? bforce[3 * qq + 2] : 0.0;
   const double m = mu[p], l = la[p];
   u.set(cidx(b, 0, i, j, k - kl), (-uz - kl * wx + kl * h * f0 / m) / fs.sbop[0]);
   u.set(cidx(b, 1, i, j, k - kl), (-vz - kl * wy + kl * h * f1 / m) / fs.sbop[0]);
   u.set(cidx(b, 2, i, j, k - kl), (-wz + (-kl * l * (ux + vy) + kl * h * f2) / (2 * m + l)) / fs.sbop[0]);
}

int small_grid(long long n)
{
   long long g = (n + 255) / 256;
   if (g > 152LL * 8) g = 152LL * 8;
   return (int)(g > 0 ? g : 1);
}

}  // namespace

template <class Field>
int bc_sides(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int wind[36],
             int nx, int ny, int nz, Field u, double h, const int bccnd[6],
                    const double sbop[5], const double* mu, const double* la,
                    const double* const bforce[6], const double* strx, const double* stry,
                    cudaStream_t s)
{
   Box b = make_box(soa, ib, ie, jb, je, kb, ke);
   for (int side = 0; side < 6; side++) {
      const int* w6 = wind + 6 * side;
      Win w{w6[0], w6[1], w6[2], w6[3], w6[4], w6[5]};
      const int t = bccnd[side];
      if (t == 1 || t == 2 || t == 3) {
         if (w.i1 < w.i0 || w.j1 < w.j0 || w.k1 < w.k0) continue;
         if (w.i0 < ib || w.i1 > ie || w.j0 < jb || w.j1 > je || w.k0 < kb || w.k1 > ke)
            return kBadArgument;
         const long long n = (long long)(w.i1 - w.i0 + 1) * (w.j1 - w.j0 + 1) * (w.k1 - w.k0 + 1);
         if (t == 3) {
            const int di = side == 0 ? nx : side == 1 ? -nx : 0;
            const int dj = side == 2 ? ny : side == 3 ? -ny : 0;
            const int dk = side == 4 ? nz : side == 5 ? -nz : 0;
            periodic_window_kernel<<<small_grid(n), 256, 0, s>>>(b, w, u, di, dj, dk);
         } else {
            fill_window_kernel<<<small_grid(n), 256, 0, s>>>(b, w, u, bforce ? bforce[side] : nullptr);
         }
      } else if (t == 0) {
         if (side != 4 && side != 5) return kNotSupported;
         FreeSurf fs;
         for (int q = 0; q < 5; q++) fs.sbop[q] = sbop[q];
         const int k = side == 4 ? 1 : nz, kl = side == 4 ? 1 : -1;
         const dim3 block(32, 8), grid(blocks_for(ie - ib - 3, 32), blocks_for(je - jb - 3, 8));
         free_surface_kernel<<<grid, block, 0, s>>>(b, u, mu, la, bforce ? bforce[side] : nullptr,
                                                    strx, stry, h, k, kl, fs);
      }
   }
   return launch_status();
}

// The ghost plane of one free-surface z side (side 4 top, 5 bottom) from the
// homogeneous traction condition, on an FP64 level or a double-float level (df).
int launch_free_surface_ghosts(const Box& b, int nz, int side, bool df, void* u, const double* mu,
                               const double* la, const double* strx, const double* stry, double h,
                               const double sbop[5], cudaStream_t s)
{
   if ((side != 4 && side != 5) || !u) return kBadArgument;
   FreeSurf fs;
   for (int q = 0; q < 5; q++) fs.sbop[q] = sbop[q];
   const int k = side == 4 ? 1 : nz, kl = side == 4 ? 1 : -1;
   const dim3 block(32, 8), grid(blocks_for(b.ie - b.ib - 3, 32), blocks_for(b.je - b.jb - 3, 8));
   if (df)
      free_surface_kernel<<<grid, block, 0, s>>>(b, DFField{static_cast<float*>(u), 3 * b.npts}, mu, la,
                                                 nullptr, strx, stry, h, k, kl, fs);
   else
      free_surface_kernel<<<grid, block, 0, s>>>(b, F64Field{static_cast<double*>(u)}, mu, la, nullptr, strx,
                                                 stry, h, k, kl, fs);
   return launch_status();
}

int launch_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int wind[36],
                    int nx, int ny, int nz, double* u, double h, const int bccnd[6],
                    const double sbop[5], const double* mu, const double* la,
                    const double* const bforce[6], const double* strx, const double* stry,
                    cudaStream_t s)
{
   return bc_sides(soa, ib, ie, jb, je, kb, ke, wind, nx, ny, nz, F64Field{u}, h, bccnd, sbop, mu,
                   la, bforce, strx, stry, s);
}

int launch_bcfortsg_df(int ib, int ie, int jb, int je, int kb, int ke, const int wind[36], int nx,
                       int ny, int nz, float* uh, double h, const int bccnd[6], const double sbop[5],
                       const double* mu, const double* la, const double* strx, const double* stry,
                       cudaStream_t s)
{
   const Box b = make_box(1, ib, ie, jb, je, kb, ke);
   return bc_sides(1, ib, ie, jb, je, kb, ke, wind, nx, ny, nz, DFField{uh, 3 * b.npts}, h, bccnd,
                   sbop, mu, la, nullptr, strx, stry, s);
}

}  // namespace sw4g
