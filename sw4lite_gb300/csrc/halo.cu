// Halo exchange of a decomposed Cartesian grid, sm_103a.
//
// The reference decomposes the grid in (i, j) over MPI ranks and, after the
// predictor and after the corrector of every step, sends the two interior planes
// next to each processor side into the neighbour's two ghost planes: x first, then
// y over the full i extent, so the corner columns travel too (EW::pack_HaloArrayCU_X/Y,
// communicate_arrayCU_X/Y and unpack_HaloArrayCU_X/Y, src/EW_cuda.C:1515-1900,
// called at src/EW.C:2596-2616 and 2728-2744).
//
// Here:
//  * halo_copy_kernel packs the two planes of one side into a contiguous buffer or
//    unpacks a buffer into the two ghost planes, for FP64 levels (3 components) and
//    for the mixed form's double-float levels (6 FP32 halves), either layout;
//  * an EW object made for a subdomain (EW::set_subdomain) stops its step at the two
//    exchange points (EW::step_part), exposes the level to exchange and packs /
//    unpacks it (EW::halo_pack / halo_unpack) in its own storage format;
//  * step_group runs several subdomains in lockstep inside one process, on one GPU
//    or several: the packed buffers go to the neighbour by device-to-device copies
//    into the receiving GPU's own memory (cudaMemcpyPeerAsync across devices), with
//    events ordering each pack before the neighbour's unpack and each unpack before
//    the sender reuses its buffer.  No TMA multicast and no peer loads in kernels.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "ew.h"
#include "kernels.h"

namespace sw4g {
namespace {

// Elements of one side's halo: 2 planes x the other tangential extent x nk x ncomp.
long long halo_elems(const Box& b, int axis, int ncomp)
{
   const long long nj = b.je - b.jb + 1, nk = b.ke - b.kb + 1;
   return 2LL * (axis == 0 ? nj : b.ni) * nk * ncomp;
}

// Buffer order: ((c * nk + k) * n_other + o) * 2 + t, t the plane (0 = lower index).
template <typename T>
__global__ void halo_copy_kernel(Box b, int axis, int first, int ncomp, T* __restrict__ field,
                                 T* __restrict__ buf, bool to_buf, long long n)
{
   const long long nj = b.je - b.jb + 1, nk = b.ke - b.kb + 1;
   const long long nother = axis == 0 ? nj : b.ni;
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x) {
      const int t = (int)(q & 1);
      long long r = q >> 1;
      const long long o = r % nother;
      r /= nother;
      const long long kk = r % nk;
      const int c = (int)(r / nk);
      const int i = axis == 0 ? first + t : b.ib + (int)o;
      const int j = axis == 0 ? b.jb + (int)o : first + t;
      const long long p = c * b.cs + b.ps * pidx(b, i, j, b.kb + (int)kk);
      if (to_buf)
         buf[q] = field[p];
      else
         field[p] = buf[q];
   }
}

int copy_grid(long long n)
{
   const long long g = (n + 255) / 256;
   return (int)std::min<long long>(std::max<long long>(g, 1), 152LL * 8);
}

}  // namespace

// First plane of the two that a side sends (pack) or receives (unpack).
int halo_first_plane(const Box& b, int axis, int side, bool pack)
{
   const int lo = axis == 0 ? b.ib : b.jb, hi = axis == 0 ? b.ie : b.je;
   if (pack) return side == 0 ? lo + 2 : hi - 3;  // the two interior planes next to the side
   return side == 0 ? lo : hi - 1;                // the two ghost planes
}

long long halo_len(const Box& b, int axis, int ncomp) { return halo_elems(b, axis, ncomp); }

int launch_halo_copy(const Box& b, int axis, int side, bool pack, bool is_float, int ncomp,
                     void* field, void* buf, cudaStream_t s)
{
   if ((axis != 0 && axis != 1) || (side != 0 && side != 1) || !field || !buf) return kBadArgument;
   const int first = halo_first_plane(b, axis, side, pack);
   const long long n = halo_elems(b, axis, ncomp);
   if (is_float)
      halo_copy_kernel<float><<<copy_grid(n), 256, 0, s>>>(b, axis, first, ncomp,
                                                           static_cast<float*>(field),
                                                           static_cast<float*>(buf), pack, n);
   else
      halo_copy_kernel<double><<<copy_grid(n), 256, 0, s>>>(b, axis, first, ncomp,
                                                            static_cast<double*>(field),
                                                            static_cast<double*>(buf), pack, n);
   return launch_status();
}

// ---- EW side ----
long long EW::halo_bytes(int axis) const
{
   const Box b = make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke);
   // FP64: 3 components of 8 bytes; mixed: 6 FP32 halves of 4 bytes (the same bytes)
   return halo_elems(b, axis, mixed_ ? 6 : 3) * (mixed_ ? 4 : 8);
}

int EW::halo_copy(int axis, int side, bool pack, void* buf)
{
   if (!sub_ || part_ == 0 || !buf) return kBadArgument;
   const int lev = part_ == 1 ? split_ip_ : split_iq_;  // the level the last part left
   const Box b = make_box(1, b_.ib, b_.ie, b_.jb, b_.je, b_.kb, b_.ke);
   return launch_halo_copy(b, axis, side, pack, mixed_, mixed_ ? 6 : 3, lev_[lev], buf, stream_);
}

// Steps a set of subdomain objects in lockstep.  nb[4 s + q] is the index of the
// neighbour of subdomain s across side q (0 x-low, 1 x-high, 2 y-low, 3 y-high), or -1.
int step_group(EW* const* subs, int n, const int* nb, int nsteps)
{
   if (n < 1 || !subs || !nb || nsteps < 0) return kBadArgument;
   for (int s = 0; s < n; s++) {
      if (!subs[s] || !subs[s]->is_subdomain()) return kBadArgument;
      for (int q = 0; q < 4; q++) {
         const int t = nb[4 * s + q];
         if (t < -1 || t >= n || t == s) return kBadArgument;
         // the neighbour across side q must name s across the opposite side
         if (t >= 0 && nb[4 * t + (q ^ 1)] != s) return kBadArgument;
      }
   }
   int dev0 = 0;
   SW4G_TRY(cuda_ok(cudaGetDevice(&dev0)));
   std::vector<cudaEvent_t> packed(n), unpacked(n);
   for (int s = 0; s < n; s++) {
      cudaSetDevice(subs[s]->device());
      cudaEventCreateWithFlags(&packed[s], cudaEventDisableTiming);
      cudaEventCreateWithFlags(&unpacked[s], cudaEventDisableTiming);
   }
   int st = kOk;
   auto on = [&](int s) { cudaSetDevice(subs[s]->device()); };
   // one exchange of the level every subdomain has just left, x first, then y
   auto exchange = [&]() -> int {
      for (int axis = 0; axis < 2; axis++) {
         for (int s = 0; s < n; s++) {
            on(s);
            for (int side = 0; side < 2; side++)
               if (nb[4 * s + 2 * axis + side] >= 0)
                  SW4G_TRY(subs[s]->halo_pack(axis, side, subs[s]->send_buffer(axis, side)));
            SW4G_TRY(cuda_ok(cudaEventRecord(packed[s], subs[s]->stream())));
         }
         for (int t = 0; t < n; t++) {
            on(t);
            for (int side = 0; side < 2; side++) {
               const int s = nb[4 * t + 2 * axis + side];
               if (s < 0) continue;
               SW4G_TRY(cuda_ok(cudaStreamWaitEvent(subs[t]->stream(), packed[s], 0)));
               // t's ghost planes across `side` hold s's interior planes across the
               // opposite side
               void* src = subs[s]->send_buffer(axis, side ^ 1);
               void* use = src;
               if (subs[s]->device() != subs[t]->device()) {
                  use = subs[t]->recv_buffer(axis, side);
                  SW4G_TRY(cuda_ok(cudaMemcpyPeerAsync(use, subs[t]->device(), src, subs[s]->device(),
                                                       (size_t)subs[t]->halo_bytes(axis),
                                                       subs[t]->stream())));
               }
               SW4G_TRY(subs[t]->halo_unpack(axis, side, use));
            }
            SW4G_TRY(cuda_ok(cudaEventRecord(unpacked[t], subs[t]->stream())));
         }
         // a sender reuses its buffers only after its neighbours have read them
         for (int s = 0; s < n; s++) {
            on(s);
            for (int q = 2 * axis; q < 2 * axis + 2; q++) {
               const int t = nb[4 * s + q];
               if (t >= 0) SW4G_TRY(cuda_ok(cudaStreamWaitEvent(subs[s]->stream(), unpacked[t], 0)));
            }
         }
      }
      return kOk;
   };
   for (int step = 0; step < nsteps && st == kOk; step++) {
      for (int part = 0; part < 3 && st == kOk; part++) {
         for (int s = 0; s < n && st == kOk; s++) {
            on(s);
            st = subs[s]->step_part(part);
         }
         if (st == kOk && part < 2) st = exchange();
      }
   }
   for (int s = 0; s < n; s++) {
      on(s);
      cudaEventDestroy(packed[s]);
      cudaEventDestroy(unpacked[s]);
   }
   cudaSetDevice(dev0);
   return st;
}

}  // namespace sw4g
