// Source discretisation on the device (replaces the host loop of
// Source::set_grid_point_sources4, src/Source.C:1074-1530, and its curvilinear
// branches, :1530-1990, for a Cartesian grid under a curvilinear grid):
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

// Two grids: entry (s, t) of a source may add a grid-point source to its own grid and,
// for a stencil across the interface, a copy to the other grid; each grid gets its own
// key array (kNone where the entry adds nothing there).
__global__ void __launch_bounds__(kStencil)
    disc_topo_kernel(GridSpec g, int top_os, int bot_os, CurvSourceGrid cv,
                     const SourceSpec* __restrict__ specs, unsigned long long* __restrict__ kcart,
                     unsigned long long* __restrict__ kcurv, unsigned* __restrict__ vals,
                     GridPointSource* __restrict__ ecart, GridPointSource* __restrict__ ecurv)
{
   __shared__ TopoStencil st;
   __shared__ int rc;
   const int s = blockIdx.x, t = threadIdx.x;
   const SourceSpec sp = specs[s];
   if (t == 0) {
      const int os[6] = {0, 0, 0, 0, top_os, bot_os};
      rc = topo_stencil(g, os, cv, sp, st);
   }
   __syncthreads();
   const unsigned e = (unsigned)s * kStencil + t;
   unsigned long long kc = kNone, kv = kNone;
   GridPointSource p, q;
   if (rc == 0) {
      const int got = topo_entry(g, cv, sp, st, t, p, q);
      const long long ni = g.nx + 4, nij = ni * (g.ny + 4);
      auto key = [&](const GridPointSource& x) {
         const unsigned long long pt = (unsigned long long)((x.i + 1) + ni * (x.j + 1) + nij * (x.k + 1));
         return (pt << 32) | e;
      };
      // own grid in p, the other grid in q
      if (got & 1) (st.in_curv ? kv : kc) = key(p);
      if (got & 2) (st.in_curv ? kc : kv) = key(q);
   }
   kcart[e] = kc;
   kcurv[e] = kv;
   vals[e] = e;
   ecart[e] = st.in_curv ? q : p;
   ecurv[e] = st.in_curv ? p : q;
}

size_t align8(size_t b) { return (b + 7) / 8 * 8; }

// Groups n entries (keys k0 = point << 32 | entry order, or kNone; vals v0 = entry
// index) by grid point into a SourceSet in one device block *mem.
int group_entries(int n, const unsigned long long* k0, const unsigned* v0, const GridPointSource* ent,
                  SourceSet* out, void** mem, cudaStream_t s)
{
   *out = SourceSet{};
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
   const size_t o_k1 = take(n * 8ull), o_v1 = take(n * 4ull), o_head = take(n * 4ull),
                o_pidx = take(n * 4ull), o_nv = take(8), o_sort = take(sort_bytes), o_scan = take(scan_bytes);
   unsigned char* w = nullptr;
   SW4G_TRY(cuda_ok(cudaMalloc(&w, off)));
   // the SourceSet block, sized for every entry valid
   const size_t int_bytes = align8(((size_t)n + 1 + 3 * (size_t)n + n) * sizeof(int));
   const size_t set_bytes = int_bytes + 5 * (size_t)n * sizeof(double);
   unsigned char* set = nullptr;
   int st = cuda_ok(cudaMalloc(&set, set_bytes));
   auto at = [&](size_t o) { return w + o; };
   auto* k1 = reinterpret_cast<unsigned long long*>(at(o_k1));
   auto* v1 = reinterpret_cast<unsigned*>(at(o_v1));
   int* head = reinterpret_cast<int*>(at(o_head));
   int* pidx = reinterpret_cast<int*>(at(o_pidx));
   int* nv = reinterpret_cast<int*>(at(o_nv));
   int* start = reinterpret_cast<int*>(set);
   int* ijk = start + n + 1;
   int* kind = ijk + 3 * n;
   double* amp = reinterpret_cast<double*>(set + int_bytes);
   double* freq = amp + 3 * (size_t)n;
   double* t0 = freq + n;
   if (st == kOk) st = cuda_ok(cudaMemsetAsync(nv, 0, sizeof(int), s));
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
   if (st != kOk || counts[0] == 0) {
      if (set) cudaFree(set);
      return st;
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

int release(void** mem, cudaStream_t s)
{
   if (*mem) {
      SW4G_TRY(cuda_ok(cudaStreamSynchronize(s)));
      cudaFree(*mem);
      *mem = nullptr;
   }
   return kOk;
}

}  // namespace

int launch_discretize_sources(const GridSpec& g, const int onesided[6], int nsrc, const SourceSpec* host_specs,
                              SourceSet* out, void** mem, cudaStream_t s)
{
   if (nsrc < 0 || !out || !mem || (nsrc > 0 && !host_specs)) return kBadArgument;
   SW4G_TRY(release(mem, s));
   *out = SourceSet{};
   if (nsrc == 0) return kOk;
   const int n = nsrc * kStencil;
   size_t off = 0;
   auto take = [&](size_t bytes) {
      const size_t at = off;
      off += align8(bytes);
      return at;
   };
   const size_t o_spec = take(nsrc * sizeof(SourceSpec)), o_k0 = take(n * 8ull), o_v0 = take(n * 4ull),
                o_ent = take(n * sizeof(GridPointSource));
   unsigned char* w = nullptr;
   SW4G_TRY(cuda_ok(cudaMalloc(&w, off)));
   auto* dspec = reinterpret_cast<SourceSpec*>(w + o_spec);
   auto* k0 = reinterpret_cast<unsigned long long*>(w + o_k0);
   auto* v0 = reinterpret_cast<unsigned*>(w + o_v0);
   auto* ent = reinterpret_cast<GridPointSource*>(w + o_ent);
   int st = cuda_ok(cudaMemcpyAsync(dspec, host_specs, nsrc * sizeof(SourceSpec), cudaMemcpyHostToDevice, s));
   if (st == kOk) {
      disc_kernel<<<nsrc, kStencil, 0, s>>>(g, onesided[4], onesided[5], dspec, k0, v0, ent);
      st = launch_status();
   }
   if (st == kOk) st = group_entries(n, k0, v0, ent, out, mem, s);
   cudaStreamSynchronize(s);
   cudaFree(w);
   return st;
}

int launch_discretize_sources_topo(const GridSpec& g, const int onesided[6], const CurvSourceGrid& cv,
                                   int nsrc, const SourceSpec* host_specs, SourceSet* cart, void** cart_mem,
                                   SourceSet* curv, void** curv_mem, cudaStream_t s)
{
   if (nsrc < 0 || !cart || !cart_mem || !curv || !curv_mem || (nsrc > 0 && !host_specs)) return kBadArgument;
   SW4G_TRY(release(cart_mem, s));
   SW4G_TRY(release(curv_mem, s));
   *cart = SourceSet{};
   *curv = SourceSet{};
   if (nsrc == 0) return kOk;
   const int n = nsrc * kStencil;
   size_t off = 0;
   auto take = [&](size_t bytes) {
      const size_t at = off;
      off += align8(bytes);
      return at;
   };
   const size_t o_spec = take(nsrc * sizeof(SourceSpec)), o_kc = take(n * 8ull), o_kv = take(n * 8ull),
                o_v0 = take(n * 4ull), o_ec = take(n * sizeof(GridPointSource)),
                o_ev = take(n * sizeof(GridPointSource));
   unsigned char* w = nullptr;
   SW4G_TRY(cuda_ok(cudaMalloc(&w, off)));
   auto* dspec = reinterpret_cast<SourceSpec*>(w + o_spec);
   auto* kc = reinterpret_cast<unsigned long long*>(w + o_kc);
   auto* kv = reinterpret_cast<unsigned long long*>(w + o_kv);
   auto* v0 = reinterpret_cast<unsigned*>(w + o_v0);
   auto* ec = reinterpret_cast<GridPointSource*>(w + o_ec);
   auto* ev = reinterpret_cast<GridPointSource*>(w + o_ev);
   int st = cuda_ok(cudaMemcpyAsync(dspec, host_specs, nsrc * sizeof(SourceSpec), cudaMemcpyHostToDevice, s));
   if (st == kOk) {
      disc_topo_kernel<<<nsrc, kStencil, 0, s>>>(g, onesided[4], onesided[5], cv, dspec, kc, kv, v0, ec, ev);
      st = launch_status();
   }
   if (st == kOk) st = group_entries(n, kc, v0, ec, cart, cart_mem, s);
   if (st == kOk) st = group_entries(n, kv, v0, ev, curv, curv_mem, s);
   cudaStreamSynchronize(s);
   cudaFree(w);
   return st;
}

}  // namespace sw4g
