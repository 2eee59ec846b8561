// Source discretisation on the device (replaces the host loop of
// Source::set_grid_point_sources4, src/Source.C:1074-1530, for the Cartesian grid):
// one CTA per source and one thread per stencil entry compute the grid-point sources
// of a whole batch of sources with the host's formulas (source_weights.h; this file
// compiles without FMA contraction, so the bits match the host's).  The entries are
// then grouped by grid point on the device: a radix sort on (grid point, entry order)
// keeps the host's order within a point (sources in the order added, each in its
// stencil order), so the forcing sums them in the same order and a run gives the same
// bits as with the host discretisation.  The result is the SourceSet the forcing
// kernels read, in one device block: start | ijk | kind | amp | freq | t0.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "common.cuh"
#include "kernels.h"
#include "source_weights.h"

namespace sw4g {
namespace {

constexpr int kStencil = 216;  // 6 x 6 x 6 entries per source
constexpr unsigned long long kNone = ~0ull;

// entry (s, t): key = point index << 32 | (s * 216 + t), or kNone where the host adds
// no grid-point source
__global__ void __launch_bounds__(kStencil) disc_kernel(GridSpec g, int top_os, int bot_os,
                                                       const SourceSpec* __restrict__ specs,
                                                       unsigned long long* __restrict__ keys,
                                                       unsigned* __restrict__ vals,
                                                       GridPointSource* __restrict__ ent)
{
   const int s = blockIdx.x, t = threadIdx.x;
   const SourceSpec sp = specs[s];
   CartStencil c;
   cart_stencil(g, top_os != 0, bot_os != 0, sp, c);
   GridPointSource p;
   const unsigned e = (unsigned)s * kStencil + t;
   unsigned long long key = kNone;
   if (cart_entry(g, c, sp, t, p)) {
      const long long ni = g.nx + 4, nij = ni * (g.ny + 4);
      const unsigned long long pt = (unsigned long long)((p.i + 1) + ni * (p.j + 1) + nij * (p.k + 1));
      key = (pt << 32) | e;
   }
   keys[e] = key;
   vals[e] = e;
   ent[e] = p;
}

// head[q] = 1 where a new grid point starts among the valid sorted entries
__global__ void heads_kernel(int n, const unsigned long long* __restrict__ keys, int* __restrict__ head,
                             int* __restrict__ nvalid)
{
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= n) return;
   const bool valid = keys[q] != kNone;
   head[q] = valid && (q == 0 || (keys[q] >> 32) != (keys[q - 1] >> 32)) ? 1 : 0;
   if (valid && (q + 1 == n || keys[q + 1] == kNone)) *nvalid = q + 1;
}

// the SourceSet arrays from the sorted entries
__global__ void gather_kernel(int n, const unsigned* __restrict__ vals, const int* __restrict__ head,
                              const int* __restrict__ pidx, const GridPointSource* __restrict__ ent,
                              int* __restrict__ start, int* __restrict__ ijk, int* __restrict__ kind,
                              double* __restrict__ amp, double* __restrict__ freq, double* __restrict__ t0,
                              const int* __restrict__ nvalid)
{
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   const int nv = *nvalid;
   if (q >= n || q >= nv) return;
   const GridPointSource& p = ent[vals[q]];
   ijk[3 * q] = p.i;
   ijk[3 * q + 1] = p.j;
   ijk[3 * q + 2] = p.k;
   kind[q] = p.kind;
   for (int c = 0; c < 3; c++) amp[3 * q + c] = p.amp[c];
   freq[q] = p.freq;
   t0[q] = p.t0;
   if (head[q]) start[pidx[q]] = q;
   if (q + 1 == nv) start[pidx[q] + head[q]] = nv;  // start[np] = number of sources
}

size_t align8(size_t b) { return (b + 7) / 8 * 8; }

}  // namespace

int launch_discretize_sources(const GridSpec& g, const int onesided[6], int nsrc, const SourceSpec* host_specs,
                              SourceSet* out, void** mem, cudaStream_t s)
{
   if (nsrc < 0 || !out || !mem || (nsrc > 0 && !host_specs)) return kBadArgument;
   if (*mem) {
      SW4G_TRY(cuda_ok(cudaStreamSynchronize(s)));
      cudaFree(*mem);
      *mem = nullptr;
   }
   *out = SourceSet{};
   if (nsrc == 0) return kOk;
   const int n = nsrc * kStencil;
   // work: specs, keys (2), vals (2), entries, heads, point indices, count, sort/scan temp
   size_t sort_bytes = 0, scan_bytes = 0;
   SW4G_TRY(cuda_ok(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (unsigned long long*)nullptr,
                                                    (unsigned long long*)nullptr, (unsigned*)nullptr,
                                                    (unsigned*)nullptr, n, 0, 64, s)));
   SW4G_TRY(cuda_ok(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (int*)nullptr, (int*)nullptr, n, s)));
   size_t off = 0;
   auto take = [&](size_t bytes) {
      const size_t at = off;
      off += align8(bytes);
      return at;
   };
   const size_t o_spec = take(nsrc * sizeof(SourceSpec)), o_k0 = take(n * 8ull), o_k1 = take(n * 8ull),
                o_v0 = take(n * 4ull), o_v1 = take(n * 4ull), o_ent = take(n * sizeof(GridPointSource)),
                o_head = take(n * 4ull), o_pidx = take(n * 4ull), o_nv = take(8), o_sort = take(sort_bytes),
                o_scan = take(scan_bytes);
   unsigned char* w = nullptr;
   SW4G_TRY(cuda_ok(cudaMalloc(&w, off)));
   // the SourceSet block, sized for every entry valid
   const size_t int_bytes = align8(((size_t)n + 1 + 3 * (size_t)n + n) * sizeof(int));
   const size_t set_bytes = int_bytes + 5 * (size_t)n * sizeof(double);
   unsigned char* set = nullptr;
   int st = cuda_ok(cudaMalloc(&set, set_bytes));
   auto at = [&](size_t o) { return w + o; };
   SourceSpec* dspec = reinterpret_cast<SourceSpec*>(at(o_spec));
   auto* k0 = reinterpret_cast<unsigned long long*>(at(o_k0));
   auto* k1 = reinterpret_cast<unsigned long long*>(at(o_k1));
   auto* v0 = reinterpret_cast<unsigned*>(at(o_v0));
   auto* v1 = reinterpret_cast<unsigned*>(at(o_v1));
   auto* ent = reinterpret_cast<GridPointSource*>(at(o_ent));
   int* head = reinterpret_cast<int*>(at(o_head));
   int* pidx = reinterpret_cast<int*>(at(o_pidx));
   int* nv = reinterpret_cast<int*>(at(o_nv));
   int* start = reinterpret_cast<int*>(set);
   int* ijk = start + n + 1;
   int* kind = ijk + 3 * n;
   double* amp = reinterpret_cast<double*>(set + int_bytes);
   double* freq = amp + 3 * (size_t)n;
   double* t0 = freq + n;
   if (st == kOk)
      st = cuda_ok(cudaMemcpyAsync(dspec, host_specs, nsrc * sizeof(SourceSpec), cudaMemcpyHostToDevice, s));
   if (st == kOk) st = cuda_ok(cudaMemsetAsync(nv, 0, sizeof(int), s));
   if (st == kOk) {
      disc_kernel<<<nsrc, kStencil, 0, s>>>(g, onesided[4], onesided[5], dspec, k0, v0, ent);
      st = launch_status();
   }
   if (st == kOk)
      st = cuda_ok(cub::DeviceRadixSort::SortPairs(at(o_sort), sort_bytes, k0, k1, v0, v1, n, 0, 64, s));
   if (st == kOk) {
      heads_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, k1, head, nv);
      st = launch_status();
   }
   if (st == kOk) st = cuda_ok(cub::DeviceScan::ExclusiveSum(at(o_scan), scan_bytes, head, pidx, n, s));
   if (st == kOk) {
      gather_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, v1, head, pidx, ent, start, ijk, kind, amp, freq, t0,
                                                       nv);
      st = launch_status();
   }
   // the counts for the forcing launches: sources and grid points
   int counts[2] = {0, 0};
   if (st == kOk) st = cuda_ok(cudaMemcpyAsync(&counts[0], nv, sizeof(int), cudaMemcpyDeviceToHost, s));
   if (st == kOk) st = cuda_ok(cudaStreamSynchronize(s));
   if (st == kOk && counts[0] > 0) {
      int last_pidx = 0, last_head = 0;
      st = cuda_ok(cudaMemcpy(&last_pidx, pidx + counts[0] - 1, sizeof(int), cudaMemcpyDeviceToHost));
      if (st == kOk) st = cuda_ok(cudaMemcpy(&last_head, head + counts[0] - 1, sizeof(int), cudaMemcpyDeviceToHost));
      counts[1] = last_pidx + last_head;
   }
   cudaFree(w);
   if (st != kOk) {
      if (set) cudaFree(set);
      return st;
   }
   if (counts[0] == 0) {
      cudaFree(set);
      return kOk;
   }
   *mem = set;
   out->npoints = counts[1];
   out->nsources = counts[0];
   out->start = start;
   out->ijk = ijk;
   out->kind = kind;
   out->amp = amp;
   out->freq = freq;
   out->t0 = t0;
   return kOk;
}

}  // namespace sw4g
