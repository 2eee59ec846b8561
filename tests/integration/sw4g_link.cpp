// A plain C++ caller of libsw4g.so, linked with -lsw4g (no Python, no ctypes): the
// shape of a host program that binds the library the way sw4lite would.  It reads a
// grid and fields from a binary file, runs sw4g_rhs4sg and sw4g_bcfortsg on the
// device through the C ABI, and writes the results back; tests/test_gpu_link.py
// compares them with the oracle.
//
// Input (little-endian): int32 soa, nx, ny, nz, onesided[6], bccnd[6], wind[36];
// float64 h, sbop[5], u[3n], mu[n], la[n], strx[nx+4], stry[ny+4], strz[nz+4], with
// n = (nx+4)(ny+4)(nz+4).  Output: float64 lu[3n] then the boundary-closed u[3n].
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "sw4g.h"

namespace {

bool read_all(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

int fail(const char* what, int st)
{
   std::fprintf(stderr, "%s: %d (%s)\n", what, st, sw4g_status_string(st));
   return 1;
}

double* upload(const std::vector<double>& h)
{
   double* d = nullptr;
   if (cudaMalloc(&d, h.size() * sizeof(double)) != cudaSuccess) return nullptr;
   cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
   return d;
}

}  // namespace

int main(int argc, char** argv)
{
   if (argc != 3) {
      std::fprintf(stderr, "usage: %s input output\n", argv[0]);
      return 2;
   }
   FILE* in = std::fopen(argv[1], "rb");
   if (!in) return 2;
   int hdr[4], onesided[6], bccnd[6], wind[36];
   double h, sbop[5];
   if (!read_all(in, hdr, sizeof hdr) || !read_all(in, onesided, sizeof onesided) ||
       !read_all(in, bccnd, sizeof bccnd) || !read_all(in, wind, sizeof wind) ||
       !read_all(in, &h, sizeof h) || !read_all(in, sbop, sizeof sbop))
      return 2;
   const int soa = hdr[0], nx = hdr[1], ny = hdr[2], nz = hdr[3];
   const int ib = -1, ie = nx + 2, jb = -1, je = ny + 2, kb = -1, ke = nz + 2;
   const size_t n = (size_t)(nx + 4) * (ny + 4) * (nz + 4);
   std::vector<double> u(3 * n), mu(n), la(n), sx(nx + 4), sy(ny + 4), sz(nz + 4);
   for (auto* v : {&u, &mu, &la, &sx, &sy, &sz})
      if (!read_all(in, v->data(), v->size() * sizeof(double))) return 2;
   std::fclose(in);

   double *du = upload(u), *dmu = upload(mu), *dla = upload(la), *dsx = upload(sx),
          *dsy = upload(sy), *dsz = upload(sz), *dlu = upload(std::vector<double>(3 * n, 0.0));
   if (!du || !dmu || !dla || !dsx || !dsy || !dsz || !dlu) return fail("cudaMalloc", SW4G_CUDA_ERROR);
   cudaStream_t s;
   cudaStreamCreate(&s);

   // EW::evalRHS (src/EW.C:3184-3203) in its sw4g form
   int st = sw4g_rhs4sg(soa, ib, ie, jb, je, kb, ke, nz, onesided, dlu, du, dmu, dla, h, dsx, dsy,
                        dsz, s);
   if (st != SW4G_OK) return fail("sw4g_rhs4sg", st);
   // EW::enforceBC (src/EW.C:3446-3502), no boundary forcing
   const double* bforce[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
   st = sw4g_bcfortsg(soa, ib, ie, jb, je, kb, ke, wind, nx, ny, nz, du, h, bccnd, sbop, dmu, dla,
                      bforce, dsx, dsy, s);
   if (st != SW4G_OK) return fail("sw4g_bcfortsg", st);
   if (cudaStreamSynchronize(s) != cudaSuccess) return fail("cudaStreamSynchronize", SW4G_CUDA_ERROR);

   std::vector<double> lu(3 * n);
   cudaMemcpy(lu.data(), dlu, lu.size() * sizeof(double), cudaMemcpyDeviceToHost);
   cudaMemcpy(u.data(), du, u.size() * sizeof(double), cudaMemcpyDeviceToHost);
   for (double* p : {du, dmu, dla, dsx, dsy, dsz, dlu}) cudaFree(p);
   cudaStreamDestroy(s);
   FILE* out = std::fopen(argv[2], "wb");
   if (!out) return 2;
   std::fwrite(lu.data(), sizeof(double), lu.size(), out);
   std::fwrite(u.data(), sizeof(double), u.size(), out);
   std::fclose(out);
   return 0;
}
