// An allocation-free variant of sw4g_corr_rows.
//
// Who needs it: callers that must not allocate device memory.  Examples are
// code running under a host-side allocator lock, tools that only intercept
// kernel launches, and embedding frameworks that forbid cudaMalloc after
// initialisation.  sw4g_corr_rows needs a scratch slab for the corrector's stage
// field (up - 2u + um) on 10 planes; those callers cannot provide one.  This entry
// point keeps that slab in a fixed-size array in device memory that belongs to
// the library, so it allocates nothing and frees nothing.
//
// Costs and limits:
//  * every GPU that loads libsw4g.so holds the array (64 MiB) until the process
//    exits;
//  * it covers at most kMaxScratchDoubles / 30 = 279,620 points per plane,
//    (ilast-ifirst+1)*(jlast-jfirst+1), e.g. a 528 x 528 plane with ghosts;
//    larger planes are rejected with SW4G_BAD_ARGUMENT before any device work;
//  * all calls on a device share the one array: calls whose work overlaps on the
//    GPU (different streams, or several host threads) race on it and give wrong
//    results; serialise them on one stream.  Every element the kernels read is
//    written earlier in the same call, so the array keeps the previous call's
//    contents without harm and nothing needs clearing;
//  * every call looks up the array's device address on the current device
//    (cudaGetSymbolAddress, a host-side table lookup) instead of caching it, so
//    an address never outlives a cudaDeviceReset or a re-created primary
//    context; the first call on a device also loads the library's device code
//    there, so make that first call before capturing a stream into a CUDA graph.

#include "../../include/sw4g.h"
#include "kernels.h"

namespace sw4g {
namespace {

constexpr long long kMaxScratchDoubles = 8LL << 20;  // 64 MiB of doubles

// Host code must not take this symbol's address directly: on the host it names a
// stand-in, not device memory.  Its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) double g_corr_rows_scratch[kMaxScratchDoubles];

// Device address of the scratch array on the current device, looked up afresh
// with that device current.
int scratch_address(double** out)
{
   void* p = nullptr;
   const cudaError_t e = cudaGetSymbolAddress(&p, g_corr_rows_scratch);
   if (e != cudaSuccess || p == nullptr) return kCudaError;
   *out = static_cast<double*>(p);
   return kOk;
}

}  // namespace
}  // namespace sw4g

extern "C" int sw4g_corr_rows_noalloc(int ifirst, int ilast, int jfirst, int jlast, int kfirst,
                                      int klast, int nz, int side, double* out, const double* up,
                                      const double* u, const double* um, const double* mu,
                                      const double* lambda, const double* rho,
                                      const double* strx, const double* stry,
                                      const double* strz, const double* dcx, const double* dcy,
                                      const double* dcz, const double* cox, const double* coy,
                                      const double* coz, double h, double dt, double beta,
                                      void* stream)
{
   const long long need = sw4g_corr_rows_scratch_len(ifirst, ilast, jfirst, jlast);
   if (need <= 0 || need > sw4g::kMaxScratchDoubles) return SW4G_BAD_ARGUMENT;
   double* scratch = nullptr;
   const int st = sw4g::scratch_address(&scratch);
   if (st != SW4G_OK) return st;
   return sw4g_corr_rows(ifirst, ilast, jfirst, jlast, kfirst, klast, nz, side, out, up, u, um, mu,
                         lambda, rho, strx, stry, strz, dcx, dcy, dcz, cox, coy, coz, h, dt, beta,
                         scratch, need, stream);
}
