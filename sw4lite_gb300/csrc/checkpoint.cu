// Restart files in the reference's checkpoint format (src/CheckPoint.C:251-370 writes,
// :373-470 reads):
//   int precision (8), int number of grids, double time, int cycle,
//   per grid int[6] {1, nx, 1, ny, 1, nz},
//   per grid the previous level Um, then the current level U: the interior points
//   (i, j, k) = 1..n of each axis without ghost points, three components per point
//   (component fastest, then i, j, k), doubles.
// The time is the current level's.  On reading, the ghost points of both levels come
// from the boundary conditions (src/EW.C:2403-2415), by the same kernels a step uses,
// so a run restarted from a file continues bit for bit: every interior point and every
// ghost point a boundary condition sets.  (The outer ghost plane above a free surface
// is set by none and read by no stencil; it keeps what the pointwise update left
// there, in the reference as here.)  Grids: 0 the Cartesian grid, 1 the curvilinear
// grid when there is topography (the reference's grid order).
#include <cstdio>
#include <cstring>
#include <vector>

#include "ew.h"

namespace sw4g {
namespace {

struct FileCloser {
   FILE* f;
   ~FileCloser()
   {
      if (f) fclose(f);
   }
};

// interior points of grid level u (3 x npts, component-major over the array box with
// two ghost points per side) <-> the file's interior block (component fastest)
void pack_interior(const std::vector<double>& u, int nx, int ny, int nz, long long npts, double* out)
{
   const long long ni = nx + 4, nij = ni * (ny + 4);
   size_t q = 0;
   for (int k = 1; k <= nz; k++)
      for (int j = 1; j <= ny; j++)
         for (int i = 1; i <= nx; i++) {
            const long long p = (i + 1) + (j + 1) * ni + (k + 1) * nij;
            for (int c = 0; c < 3; c++) out[q++] = u[c * npts + p];
         }
}

void unpack_interior(const double* in, int nx, int ny, int nz, long long npts, std::vector<double>& u)
{
   const long long ni = nx + 4, nij = ni * (ny + 4);
   size_t q = 0;
   for (int k = 1; k <= nz; k++)
      for (int j = 1; j <= ny; j++)
         for (int i = 1; i <= nx; i++) {
            const long long p = (i + 1) + (j + 1) * ni + (k + 1) * nij;
            for (int c = 0; c < 3; c++) u[c * npts + p] = in[q++];
         }
}

}  // namespace

int EW::write_checkpoint(const char* path, int cycle)
{
   if (!ready_ || !path) return kBadArgument;
   const int ng = num_grids();
   FileCloser fc{fopen(path, "wb")};
   if (!fc.f) return kIoError;
   const int prec = 8;
   const double t = t_;
   bool ok = fwrite(&prec, sizeof(int), 1, fc.f) == 1 && fwrite(&ng, sizeof(int), 1, fc.f) == 1 &&
             fwrite(&t, sizeof(double), 1, fc.f) == 1 && fwrite(&cycle, sizeof(int), 1, fc.f) == 1;
   for (int g = 0; g < ng && ok; g++) {
      int nx, ny, nz;
      SW4G_TRY(grid_dims(g, &nx, &ny, &nz, nullptr));
      const int sizes[6] = {1, nx, 1, ny, 1, nz};
      ok = fwrite(sizes, sizeof(int), 6, fc.f) == 6;
   }
   for (int g = 0; g < ng && ok; g++) {
      int nx, ny, nz;
      long long npts;
      SW4G_TRY(grid_dims(g, &nx, &ny, &nz, &npts));
      std::vector<double> u(3 * (size_t)npts), um(3 * (size_t)npts);
      SW4G_TRY(get_fields_grid(g, u.data(), um.data(), false));
      SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));
      std::vector<double> block(3 * (size_t)nx * ny * nz);
      pack_interior(um, nx, ny, nz, npts, block.data());
      ok = fwrite(block.data(), sizeof(double), block.size(), fc.f) == block.size();
      pack_interior(u, nx, ny, nz, npts, block.data());
      ok = ok && fwrite(block.data(), sizeof(double), block.size(), fc.f) == block.size();
   }
   if (!ok) return kIoError;
   return fflush(fc.f) == 0 ? kOk : kIoError;
}

int EW::read_checkpoint(const char* path, int* cycle)
{
   if (!ready_ || !material_ || !path) return kBadArgument;
   if (cv_ && !cv_->material) return kBadArgument;
   const int ng = num_grids();
   FileCloser fc{fopen(path, "rb")};
   if (!fc.f) return kIoError;
   int prec = 0, ngf = 0, cyc = 0;
   double t = 0;
   if (fread(&prec, sizeof(int), 1, fc.f) != 1 || fread(&ngf, sizeof(int), 1, fc.f) != 1 ||
       fread(&t, sizeof(double), 1, fc.f) != 1 || fread(&cyc, sizeof(int), 1, fc.f) != 1)
      return kIoError;
   if (prec != 8 || ngf != ng) return kBadArgument;
   for (int g = 0; g < ng; g++) {
      int nx, ny, nz, sizes[6];
      SW4G_TRY(grid_dims(g, &nx, &ny, &nz, nullptr));
      if (fread(sizes, sizeof(int), 6, fc.f) != 6) return kIoError;
      if (sizes[0] != 1 || sizes[1] != nx || sizes[2] != 1 || sizes[3] != ny || sizes[4] != 1 || sizes[5] != nz)
         return kBadArgument;
   }
   std::vector<std::vector<double>> lev(2 * ng);
   for (int g = 0; g < ng; g++) {
      int nx, ny, nz;
      long long npts;
      SW4G_TRY(grid_dims(g, &nx, &ny, &nz, &npts));
      std::vector<double> block(3 * (size_t)nx * ny * nz);
      for (int q = 0; q < 2; q++) {  // Um, then U
         if (fread(block.data(), sizeof(double), block.size(), fc.f) != block.size()) return kIoError;
         std::vector<double>& u = lev[2 * g + q];
         u.assign(3 * (size_t)npts, 0.0);
         unpack_interior(block.data(), nx, ny, nz, npts, u);
      }
   }
   for (int g = 0; g < ng; g++) SW4G_TRY(set_fields_grid(g, lev[2 * g + 1].data(), lev[2 * g].data(), false));
   // the ghost points of both levels from the boundary conditions, in the step's order
   SW4G_TRY(enforce_bc(lev_[iu_]));
   if (cv_) SW4G_TRY(curv_bc(lev_[iu_], cv_->lev[iu_]));
   SW4G_TRY(enforce_bc(lev_[ium_]));
   if (cv_) SW4G_TRY(curv_bc(lev_[ium_], cv_->lev[ium_]));
   SW4G_TRY(cuda_ok(cudaStreamSynchronize(stream_)));  // the host vectors go out of scope
   t_ = t;
   if (cycle) *cycle = cyc;
   return kOk;
}

}  // namespace sw4g
