// Fused stage kernels of the FP32-mixed form fed by the Tensor Memory Accelerator,
// sm_103a.
//
// Same stages and arithmetic as stage_mixed.cu (predictor and corrector forms; see
// that file for the precision design), with a different way of moving data.  The
// synchronous kernel stages each plane by plain loads and reads its 24 coefficient
// pairs after the staging, so every plane's DRAM latency is exposed (it measured
// 28-31 % of HBM bandwidth with 5-9 long-scoreboard stalls per issue).  Here every
// input of a plane arrives by bulk tensor copies (cp.async.bulk.tensor) completed on
// shared-memory mbarriers, issued by one thread one or more planes ahead:
//
//  * F(m), the stage fields of plane m over the CTA's 36 x 12 halo tile: one 4-D box
//    {36, 12, 1, 6} per level (hi of the 3 components, then lo) lands as the
//    staged plane itself.  Predictor: a 6-slot ring of u planes (k-2..k+2 in use,
//    k+3 in flight).  Corrector: one raw slot of up, u, um, transformed into the
//    rounded stage field up - 2u + um (5-plane ring) and the damping field u - um
//    (3-plane ring) two planes ahead of the compute.  F(m) also brings mu, lambda
//    at the CTA's own points, for the z-flux G_z(m) computed right after it lands.
//  * M(m), everything plane m's compute reads once: mu, lambda (hi, lo) over the
//    halo tile, rho (corrector), the own points of the update level (up or um),
//    1/rho, and the twelve second-difference weight arrays over the extents each
//    axis needs (x: 34 columns, y: 10 rows, z: planes m..m+2).  Two stages: M(k+1)
//    is in flight while plane k computes.
//
// One CTA of 32 x 8 threads per SM (~205 KB of shared memory): the copies in
// flight, not resident warps, hide the DRAM latency.  Tensor copies need 16-byte
// aligned row strides, so the launcher takes this path when the array's i extent
// is a multiple of 4 and falls back to the synchronous kernel otherwise.  Every
// mbarrier wait gives up after one second: the kernel then records kTimeout in the
// caller's status word and its CTAs return at their next barrier.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

namespace sw4g {
namespace {

constexpr int TX = 32, TY = 8, HALO = 2;
constexpr int PX = TX + 2 * HALO;  // 36
constexpr int PY = TY + 2 * HALO;  // 12
constexpr int PLANE = PX * PY;     // 432
constexpr int NTHREADS = TX * TY;
constexpr int OWNP = PX * TY;      // 288: own rows of a tile with the x halo (columns 0..35)

constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s per mbarrier wait

// Tensor maps of one launch (encoded on the host, passed by value).
struct TmaMaps {
   CUtensorMap lev_halo[3];  // {36,12,1,6} boxes: corrector up,u,um; predictor u
   CUtensorMap lev_own;      // {36,8,1,6}: corrector up, predictor um
   CUtensorMap mu_halo, la_halo;  // {72,12,1}
   CUtensorMap mu_own, la_own;    // {72,8,1}
   CUtensorMap rho_halo;          // {36,12,1} (corrector)
   CUtensorMap ir_own;            // {72,8,1}
   CUtensorMap wx[4];             // {72,8,1}
   CUtensorMap wy[4];             // {72,10,1}
   CUtensorMap wz1[2];            // {72,8,3}: W1 of the z axis, types 0, 1
   CUtensorMap wz2[2];            // {72,8,2}: W2 of the z axis
};

struct TmaArgs {
   int ib, ie, jb, je, kb, ke;
   long long ni, nij, npts;
   int k1, k2, kchunk;
   float* __restrict__ out;
   const float* __restrict__ rho;  // z-damping neighbours (plain loads)
   const float* __restrict__ sx;
   const float* __restrict__ sy;
   const float* __restrict__ sz;
   const float* __restrict__ dc[3];
   const float* __restrict__ co[3];
   float Kh, Kl;
   float beta;
   int* status;  // kTimeout is or-ed in when a wait gives up (may be null)
};

// ---- shared-memory layout (byte offsets; every box 128-byte aligned) ----
constexpr int align128(int b) { return (b + 127) / 128 * 128; }
constexpr int kLevHaloB = 36 * 12 * 6 * 4;   // 10368
constexpr int kLevOwnB = 36 * 8 * 6 * 4;     // 6912
constexpr int kPairHaloB = 72 * 12 * 4;      // 3456
constexpr int kPairOwnB = 72 * 8 * 4;        // 2304
constexpr int kRhoHaloB = align128(36 * 12 * 4);  // 1792
constexpr int kWyB = align128(72 * 10 * 4);  // 2944
constexpr int kWz1B = 72 * 8 * 3 * 4;        // 6912
constexpr int kWz2B = 72 * 8 * 2 * 4;        // 4608

// M stage
template <int CORR>
struct MLayout {
   static constexpr int mu = 0;
   static constexpr int la = mu + kPairHaloB;
   static constexpr int rho = la + kPairHaloB;
   static constexpr int own = rho + (CORR ? kRhoHaloB : 0);
   static constexpr int ir = own + kLevOwnB;
   static constexpr int wx = ir + kPairOwnB;
   static constexpr int wy = wx + 4 * kPairOwnB;
   static constexpr int wz1 = wy + 4 * kWyB;
   static constexpr int wz2 = wz1 + 2 * kWz1B;
   static constexpr int bytes = wz2 + 2 * kWz2B;
   static constexpr unsigned tx_bytes = 2 * 72 * 12 * 4 + (CORR ? 36 * 12 * 4 : 0) + kLevOwnB +
                                        kPairOwnB + 4 * kPairOwnB + 4 * 72 * 10 * 4 +
                                        2 * kWz1B + 2 * kWz2B;
};

// whole CTA
template <int CORR>
struct Layout {
   using M = MLayout<CORR>;
   // F area: corrector one raw slot (3 levels), predictor a 6-slot ring of u planes
   static constexpr int fslots = CORR ? 3 : 6;
   static constexpr int f = 0;
   static constexpr int fown = f + fslots * kLevHaloB;      // mu, lambda own pairs
   static constexpr int m0 = fown + 2 * kPairOwnB;
   static constexpr int m1 = m0 + M::bytes;
   static constexpr int vh = m1 + M::bytes;                 // corrector: stage field ring
   static constexpr int dd = vh + (CORR ? 15 * PLANE * 4 : 0);
   static constexpr int gx = dd + (CORR ? 9 * PLANE * 4 : 0);
   static constexpr int gy = gx + 3 * TY * PX * 4;
   static constexpr int bar = align128(gy + 3 * PY * TX * 4);
   static constexpr int bytes = bar + 3 * 8 + 8;            // F barrier, M barriers, abort flag
   static constexpr unsigned f_tx = (CORR ? 3 : 1) * kLevHaloB + 2 * kPairOwnB;
};
static_assert(Layout<1>::bytes <= 227 * 1024, "corrector layout exceeds shared memory");
static_assert(Layout<0>::bytes <= 227 * 1024, "predictor layout exceeds shared memory");
static_assert(MLayout<1>::bytes % 128 == 0 && MLayout<0>::bytes % 128 == 0, "stage alignment");

// ---- PTX wrappers ----
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
   return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
   uint32_t ok;
   asm volatile(
       "{\n\t.reg .pred p;\n\t"
       "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
       "selp.u32 %0, 1, 0, p;\n\t}"
       : "=r"(ok)
       : "r"(bar), "r"(parity)
       : "memory");
   return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
   unsigned long long t;
   asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
   return t;
}

// Waits for the phase of the given parity to complete; false after kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
   if (mbar_try(bar, parity)) return true;
   const unsigned long long t0 = global_ns();
   while (!mbar_try(bar, parity))
      if (global_ns() - t0 > kWaitLimitNs) return false;
   return true;
}

__device__ __forceinline__ void tma3(uint32_t dst, const CUtensorMap* m, int x, int y, int z,
                                     uint32_t bar)
{
   asm volatile(
       "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
       " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
       "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(bar)
       : "memory");
}

__device__ __forceinline__ void tma4(uint32_t dst, const CUtensorMap* m, int x, int y, int z,
                                     int w, uint32_t bar)
{
   asm volatile(
       "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
       " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
       "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
       : "memory");
}

__device__ __forceinline__ void fence_async_shared()
{
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ int mod5(int k) { return ((k % 5) + 5) % 5; }
__device__ __forceinline__ int mod3(int k) { return ((k % 3) + 3) % 3; }
__device__ __forceinline__ int mod6(int k) { return ((k % 6) + 6) % 6; }

template <int CORR>
__global__ void __launch_bounds__(NTHREADS, 1)
    mixed_stage_tma_kernel(const __grid_constant__ TmaMaps tm, const TmaArgs a)
{
   using L = Layout<CORR>;
   using M = MLayout<CORR>;
   extern __shared__ __align__(128) unsigned char smb[];
   float* GX = reinterpret_cast<float*>(smb + L::gx);  // [3][TY][PX]
   float* GY = reinterpret_cast<float*>(smb + L::gy);  // [3][PY][TX]
   const uint32_t barF = smem_u32(smb + L::bar);
   const uint32_t barM0 = barF + 8;
   volatile int* abort_flag = reinterpret_cast<volatile int*>(smb + L::bar + 24);

   const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
   const int i0 = a.ib + 2 + blockIdx.x * TX;
   const int j0 = a.jb + 2 + blockIdx.y * TY;
   const int kbeg = a.k1 + blockIdx.z * a.kchunk;
   if (kbeg > a.k2) return;
   const int kend = min(kbeg + a.kchunk - 1, a.k2);
   const int i = i0 + tx, j = j0 + ty;
   const bool active = (i <= a.ie - 2) && (j <= a.je - 2);
   const int own = (ty + HALO) * PX + (tx + HALO);  // own point in a halo tile
   const int ownr = ty * PX + (tx + HALO);          // own point in an own-rows tile
   const long long npts = a.npts, lo = 3 * a.npts;
   // tensor coordinates of the CTA's tiles
   const int xt = blockIdx.x * TX;      // first column (i0 - 2) of the halo tile
   const int yh = blockIdx.y * TY;      // first row (j0 - 2) of the halo tile
   const int yo = yh + HALO;            // first own row (j0)

   auto gidx = [&](int gi, int gj, int gk) -> long long {
      return (long long)(gi - a.ib) + a.ni * (gj - a.jb) + a.nij * (long long)(gk - a.kb);
   };

   // ---- producers (thread 0) ----
   auto issue_F = [&](int m) {  // stage fields of plane m and the own mu, lambda pairs
      const int z = m - a.kb;
      const uint32_t slot = smem_u32(smb + L::f + (CORR ? 0 : mod6(m) * kLevHaloB));
      mbar_expect_tx(barF, L::f_tx);
      if (CORR) {
         for (int q = 0; q < 3; q++) tma4(slot + q * kLevHaloB, &tm.lev_halo[q], xt, yh, z, 0, barF);
      } else {
         tma4(slot, &tm.lev_halo[0], xt, yh, z, 0, barF);
      }
      const uint32_t fo = smem_u32(smb + L::fown);
      tma3(fo, &tm.mu_own, 2 * xt, yo, z, barF);
      tma3(fo + kPairOwnB, &tm.la_own, 2 * xt, yo, z, barF);
   };
   auto issue_M = [&](int m) {  // once-per-plane inputs of plane m
      const int z = m - a.kb;
      const uint32_t bar = barM0 + 8 * (m & 1);
      const uint32_t s = smem_u32(smb + ((m & 1) ? L::m1 : L::m0));
      mbar_expect_tx(bar, M::tx_bytes);
      tma3(s + M::mu, &tm.mu_halo, 2 * xt, yh, z, bar);
      tma3(s + M::la, &tm.la_halo, 2 * xt, yh, z, bar);
      if (CORR) tma3(s + M::rho, &tm.rho_halo, xt, yh, z, bar);
      tma4(s + M::own, &tm.lev_own, xt, yo, z, 0, bar);
      tma3(s + M::ir, &tm.ir_own, 2 * xt, yo, z, bar);
      for (int q = 0; q < 4; q++) {
         tma3(s + M::wx + q * kPairOwnB, &tm.wx[q], 2 * xt, yo, z, bar);
         tma3(s + M::wy + q * kWyB, &tm.wy[q], 2 * xt, yo, z, bar);
      }
      for (int t = 0; t < 2; t++) {
         tma3(s + M::wz1 + t * kWz1B, &tm.wz1[t], 2 * xt, yo, z, bar);
         tma3(s + M::wz2 + t * kWz2B, &tm.wz2[t], 2 * xt, yo, z, bar);
      }
   };

   if (tid == 0) {
      mbar_init(barF, 1);
      mbar_init(barM0, 1);
      mbar_init(barM0 + 8, 1);
      *abort_flag = 0;
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      fence_async_shared();
   }
   __syncthreads();

   uint32_t fphase = 0, mphase = 0;  // mphase bit s: parity of M stage s
   auto fail = [&]() {
      *abort_flag = 1;
      if (a.status) atomicOr(a.status, 1 << kTimeout);
   };
   auto wait_F = [&]() {
      if (!mbar_wait(barF, fphase)) fail();
      fphase ^= 1;
   };
   auto wait_M = [&](int m) {
      if (!mbar_wait(barM0 + 8 * (m & 1), (mphase >> (m & 1)) & 1)) fail();
      mphase ^= 1u << (m & 1);
   };

   // stage-field planes: hi/lo rings (predictor: the F ring itself) or the
   // transformed FP32 ring (corrector)
   auto vh_plane = [&](int kk) -> const float* {
      if (CORR) return reinterpret_cast<const float*>(smb + L::vh) + mod5(kk) * 3 * PLANE;
      return reinterpret_cast<const float*>(smb + L::f + mod6(kk) * kLevHaloB);
   };
   auto vl_plane = [&](int kk) -> const float* {  // predictor only
      return reinterpret_cast<const float*>(smb + L::f + mod6(kk) * kLevHaloB) + 3 * PLANE;
   };
   auto dd_plane = [&](int kk) -> float* {  // corrector only
      return reinterpret_cast<float*>(smb + L::dd) + mod3(kk) * 3 * PLANE;
   };

   // corrector: raw (up, u, um) slot -> rounded up - 2u + um and u - um
   auto transform = [&](int kk) {
      const float* raw = reinterpret_cast<const float*>(smb + L::f);
      float* vs = reinterpret_cast<float*>(smb + L::vh) + mod5(kk) * 3 * PLANE;
      float* ds = dd_plane(kk);
      for (int idx = tid; idx < PLANE; idx += NTHREADS) {
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const int q = c * PLANE + idx;
            const float uph = raw[q], upl = raw[q + 3 * PLANE];
            const float uh = raw[q + 6 * PLANE], ul = raw[q + 9 * PLANE];
            const float mh = raw[q + 12 * PLANE], ml = raw[q + 15 * PLANE];
            float s1, e1, s2, e2;
            two_sum(uph, -2.f * uh, s1, e1);
            two_sum(s1, mh, s2, e2);
            vs[q] = s2 + ((e1 + e2) + ((upl - 2.f * ul) + ml));
            float d1, f1;
            two_sum(uh, -mh, d1, f1);
            ds[q] = d1 + (f1 + (ul - ml));
         }
      }
   };

   auto diff = [&](const float* vh, const float* vl, int ia, int ib_) -> float {
      if (CORR == 1) return vh[ia] - vh[ib_];
      return (vh[ia] - vh[ib_]) + (vl[ia] - vl[ib_]);
   };
   auto d1 = [&](const float* hm2, const float* lm2, int im2, const float* hm1, const float* lm1,
                 int im1, const float* hp1, const float* lp1, int ip1, const float* hp2,
                 const float* lp2, int ip2) -> float {
      if (CORR == 1) return (hm2[im2] - hp2[ip2]) + 8.f * (hp1[ip1] - hm1[im1]);
      return ((hm2[im2] - hp2[ip2]) + (lm2[im2] - lp2[ip2])) +
             8.f * ((hp1[ip1] - hm1[im1]) + (lp1[ip1] - lm1[im1]));
   };

   const float sxi = active ? __ldg(a.sx + (i - a.ib)) : 0.f;
   const float syj = active ? __ldg(a.sy + (j - a.jb)) : 0.f;

   // own mu, lambda pairs of plane kk from the F area (read before the next F issue)
   float omh = 0.f, oml = 0.f, olh = 0.f, oll = 0.f;
   auto read_own_material = [&]() {
      const float* fo = reinterpret_cast<const float*>(smb + L::fown);
      omh = fo[2 * ownr];
      oml = fo[2 * ownr + 1];
      olh = fo[OWNP * 2 + 2 * ownr];
      oll = fo[OWNP * 2 + 2 * ownr + 1];
   };

   auto compute_gz = [&](int kk, float g[3]) {
      const float* vh = vh_plane(kk);
      const float* vl = CORR ? vh : vl_plane(kk);
      const float *hu = vh, *hv = vh + PLANE, *hw = vh + 2 * PLANE;
      const float *lu_ = vl, *lv = vl + PLANE, *lw = vl + 2 * PLANE;
      const float dxw = d1(hw, lw, own - 2, hw, lw, own - 1, hw, lw, own + 1, hw, lw, own + 2);
      const float dyw = d1(hw, lw, own - 2 * PX, hw, lw, own - PX, hw, lw, own + PX, hw, lw, own + 2 * PX);
      const float dxu = d1(hu, lu_, own - 2, hu, lu_, own - 1, hu, lu_, own + 1, hu, lu_, own + 2);
      const float dyv = d1(hv, lv, own - 2 * PX, hv, lv, own - PX, hv, lv, own + PX, hv, lv, own + 2 * PX);
      const float x0 = sxi * dxw, x1 = syj * dyw, x2 = sxi * dxu + syj * dyv;
      g[0] = fmaf(omh, x0, oml * x0);
      g[1] = fmaf(omh, x1, oml * x1);
      g[2] = fmaf(olh, x2, oll * x2);
   };

   float gz[5][3], dq[5][3];
   const int kfin = kend + 2;  // last plane the stencil reads

   // ---- prologue: planes kbeg-2 .. kbeg+1 into the rings, M(kbeg) in flight ----
   if (tid == 0) {
      issue_M(kbeg);
      issue_F(kbeg - 2);
   }
#pragma unroll
   for (int q = 1; q <= 4; q++) {  // slots 1..4 hold planes kbeg-2..kbeg+1
      const int kk = kbeg - 3 + q;
      wait_F();
      if (CORR) transform(kk);
      read_own_material();
      __syncthreads();
      if (*abort_flag) return;
      if (tid == 0) {
         fence_async_shared();
         issue_F(kk + 1);
      }
      if (active) compute_gz(kk, gz[q]);
      if (CORR) {
         const float* dd = dd_plane(kk);
#pragma unroll
         for (int c = 0; c < 3; c++) dq[q][c] = dd[c * PLANE + own];
      }
   }

   for (int k = kbeg; k <= kend; k++) {
      // F(k+2) landed: transform it (corrector), take the own material, free the slot
      wait_F();
      if (CORR) transform(k + 2);
      read_own_material();
      __syncthreads();  // (A)
      if (*abort_flag) return;
      if (tid == 0) {
         fence_async_shared();
         if (k + 3 <= kfin) issue_F(k + 3);
         if (k + 1 <= kend) issue_M(k + 1);
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
#pragma unroll
         for (int c = 0; c < 3; c++) {
            gz[q][c] = gz[q + 1][c];
            if (CORR) dq[q][c] = dq[q + 1][c];
         }
      }
      if (active) compute_gz(k + 2, gz[4]);
      if (CORR) {
         const float* dd = dd_plane(k + 2);
#pragma unroll
         for (int c = 0; c < 3; c++) dq[4][c] = dd[c * PLANE + own];
      }
      wait_M(k);
      const unsigned char* ms = smb + ((k & 1) ? L::m1 : L::m0);
      const float* MU2 = reinterpret_cast<const float*>(ms + M::mu);
      const float* LA2 = reinterpret_cast<const float*>(ms + M::la);

      const float szk = __ldg(a.sz + (k - a.kb));
      const float* hm2 = vh_plane(k - 2);
      const float* hm1 = vh_plane(k - 1);
      const float* h0 = vh_plane(k);
      const float* hp1 = vh_plane(k + 1);
      const float* hp2 = vh_plane(k + 2);
      const float* lm2 = CORR ? hm2 : vl_plane(k - 2);
      const float* lm1 = CORR ? hm1 : vl_plane(k - 1);
      const float* l0 = CORR ? h0 : vl_plane(k);
      const float* lp1 = CORR ? hp1 : vl_plane(k + 1);
      const float* lp2 = CORR ? hp2 : vl_plane(k + 2);
      auto dz = [&](int c, int s) {
         const int o = c * PLANE;
         return d1(hm2 + o, lm2 + o, s, hm1 + o, lm1 + o, s, hp1 + o, lp1 + o, s, hp2 + o, lp2 + o, s);
      };

      // x-outer products over 36 x 8, y-outer products over 32 x 12
      for (int idx = tid; idx < TY * PX; idx += NTHREADS) {
         const int li = idx % PX, ljr = idx / PX;
         const int s = (ljr + HALO) * PX + li;
         const int gi = i0 - HALO + li, gj = j0 + ljr;
         float g0 = 0.f, g1 = 0.f, g2 = 0.f;
         if (gi <= a.ie && gj <= a.je) {
            const float syy = __ldg(a.sy + (gj - a.jb));
            const float *hu = h0, *hv = h0 + PLANE, *lu_ = l0, *lv = l0 + PLANE;
            const float dyv = d1(hv, lv, s - 2 * PX, hv, lv, s - PX, hv, lv, s + PX, hv, lv, s + 2 * PX);
            const float dyu = d1(hu, lu_, s - 2 * PX, hu, lu_, s - PX, hu, lu_, s + PX, hu, lu_, s + 2 * PX);
            const float dzw = dz(2, s), dzu = dz(0, s);
            const float mh = MU2[2 * s], ml = MU2[2 * s + 1], lh = LA2[2 * s], ll = LA2[2 * s + 1];
            const float x0 = syy * dyv + szk * dzw, x1 = syy * dyu, x2 = szk * dzu;
            g0 = fmaf(lh, x0, ll * x0);
            g1 = fmaf(mh, x1, ml * x1);
            g2 = fmaf(mh, x2, ml * x2);
         }
         GX[idx] = g0;
         GX[TY * PX + idx] = g1;
         GX[2 * TY * PX + idx] = g2;
      }
      for (int idx = tid; idx < PY * TX; idx += NTHREADS) {
         const int lic = idx % TX, lj = idx / TX;
         const int s = lj * PX + lic + HALO;
         const int gi = i0 + lic, gj = j0 - HALO + lj;
         float g0 = 0.f, g1 = 0.f, g2 = 0.f;
         if (gi <= a.ie && gj <= a.je) {
            const float sxx = __ldg(a.sx + (gi - a.ib));
            const float *hu = h0, *hv = h0 + PLANE, *lu_ = l0, *lv = l0 + PLANE;
            const float dxv = d1(hv, lv, s - 2, hv, lv, s - 1, hv, lv, s + 1, hv, lv, s + 2);
            const float dxu = d1(hu, lu_, s - 2, hu, lu_, s - 1, hu, lu_, s + 1, hu, lu_, s + 2);
            const float dzw = dz(2, s), dzv = dz(1, s);
            const float mh = MU2[2 * s], ml = MU2[2 * s + 1], lh = LA2[2 * s], ll = LA2[2 * s + 1];
            const float x0 = sxx * dxv, x1 = sxx * dxu + szk * dzw, x2 = szk * dzv;
            g0 = fmaf(mh, x0, ml * x0);
            g1 = fmaf(lh, x1, ll * x1);
            g2 = fmaf(mh, x2, ml * x2);
         }
         GY[idx] = g0;
         GY[PY * TX + idx] = g1;
         GY[2 * PY * TX + idx] = g2;
      }
      __syncthreads();  // (B)
      if (*abort_flag) return;

      if (active) {
         const long long p = gidx(i, j, k);
         // W1(q), W2(q), W2(q+1), W1(q+2) per axis and coefficient type, as (hi, lo)
         const float2* wxs = reinterpret_cast<const float2*>(ms + M::wx);
         const float2* wys = reinterpret_cast<const float2*>(ms + M::wy);
         const float2* wz1 = reinterpret_cast<const float2*>(ms + M::wz1);
         const float2* wz2 = reinterpret_cast<const float2*>(ms + M::wz2);
         float wth[3][2][4], wtl[3][2][4];
#pragma unroll
         for (int t = 0; t < 2; t++) {
            const float2* x1 = wxs + (2 * t) * OWNP;      // W1 of the x axis
            const float2* x2 = wxs + (2 * t + 1) * OWNP;  // W2
            const float2 q0 = x1[ownr], q1 = x2[ownr], q2 = x2[ownr + 1], q3 = x1[ownr + 2];
            const float2* y1 = wys + (2 * t) * (kWyB / 8);
            const float2* y2 = wys + (2 * t + 1) * (kWyB / 8);
            const float2 r0 = y1[ownr], r1 = y2[ownr], r2 = y2[ownr + PX], r3 = y1[ownr + 2 * PX];
            const float2* z1 = wz1 + t * (kWz1B / 8);
            const float2* z2 = wz2 + t * (kWz2B / 8);
            const float2 s0 = z1[ownr], s1 = z2[ownr], s2 = z2[ownr + OWNP], s3 = z1[ownr + 2 * OWNP];
            wth[0][t][0] = q0.x; wth[0][t][1] = q1.x; wth[0][t][2] = q2.x; wth[0][t][3] = q3.x;
            wtl[0][t][0] = q0.y; wtl[0][t][1] = q1.y; wtl[0][t][2] = q2.y; wtl[0][t][3] = q3.y;
            wth[1][t][0] = r0.x; wth[1][t][1] = r1.x; wth[1][t][2] = r2.x; wth[1][t][3] = r3.x;
            wtl[1][t][0] = r0.y; wtl[1][t][1] = r1.y; wtl[1][t][2] = r2.y; wtl[1][t][3] = r3.y;
            wth[2][t][0] = s0.x; wth[2][t][1] = s1.x; wth[2][t][2] = s2.x; wth[2][t][3] = s3.x;
            wtl[2][t][0] = s0.y; wtl[2][t][1] = s1.y; wtl[2][t][2] = s2.y; wtl[2][t][3] = s3.y;
         }
         auto wsum = [&](int ax, int t, float dm2, float dm1, float dp1, float dp2) {
            const float* hh = wth[ax][t];
            const float* ll = wtl[ax][t];
            const float sh = fmaf(hh[0], dm2, fmaf(hh[1], dm1, fmaf(hh[2], dp1, hh[3] * dp2)));
            const float sl = fmaf(ll[0], dm2, fmaf(ll[1], dm1, fmaf(ll[2], dp1, ll[3] * dp2)));
            return sh + sl;
         };
         float xs[3];
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const float* ch = h0 + c * PLANE;
            const float* cl = l0 + c * PLANE;
            const int o = c * PLANE;
            const float sxx = wsum(0, c == 0, diff(ch, cl, own - 2, own), diff(ch, cl, own - 1, own),
                                   diff(ch, cl, own + 1, own), diff(ch, cl, own + 2, own));
            const float syy = wsum(1, c == 1, diff(ch, cl, own - 2 * PX, own),
                                   diff(ch, cl, own - PX, own), diff(ch, cl, own + PX, own),
                                   diff(ch, cl, own + 2 * PX, own));
            float dzm2, dzm1, dzp1, dzp2;
            if (CORR == 1) {
               dzm2 = hm2[o + own] - ch[own];
               dzm1 = hm1[o + own] - ch[own];
               dzp1 = hp1[o + own] - ch[own];
               dzp2 = hp2[o + own] - ch[own];
            } else {
               dzm2 = (hm2[o + own] - ch[own]) + (lm2[o + own] - cl[own]);
               dzm1 = (hm1[o + own] - ch[own]) + (lm1[o + own] - cl[own]);
               dzp1 = (hp1[o + own] - ch[own]) + (lp1[o + own] - cl[own]);
               dzp2 = (hp2[o + own] - ch[own]) + (lp2[o + own] - cl[own]);
            }
            const float szz = wsum(2, c == 2, dzm2, dzm1, dzp1, dzp2);
            const float* gxp = GX + c * TY * PX + ty * PX + tx;
            const float* gyp = GY + c * PY * TX + ty * TX + tx;
            const float cx = (gxp[0] - gxp[4]) + 8.f * (gxp[3] - gxp[1]);
            const float cy = (gyp[0] - gyp[4 * TX]) + 8.f * (gyp[3 * TX] - gyp[TX]);
            const float cz = (gz[0][c] - gz[4][c]) + 8.f * (gz[3][c] - gz[1][c]);
            const float sd = sxi * sxx + syj * syy + szk * szz;
            xs[c] = (16.f * sd + 8.f * sd) + (sxi * cx + syj * cy + szk * cz);
         }
         const float2 ir = reinterpret_cast<const float2*>(ms + M::ir)[ownr];
         const float irh = ir.x, irl = ir.y;
         const float ph = a.Kh * irh;
         const float pl = fmaf(a.Kh, irh, -ph) + fmaf(a.Kh, irl, a.Kl * irh);
         auto scaled = [&](float x) { return fmaf(x, ph, x * pl); };
         const float* ownlev = reinterpret_cast<const float*>(ms + M::own);  // [6][8][36]
         if (!CORR) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * npts;
               const float uh = h0[c * PLANE + own], ul = l0[c * PLANE + own];
               const float mh = ownlev[c * OWNP + ownr], ml = ownlev[(c + 3) * OWNP + ownr];
               float s, e, t, e2, oh, ol;
               two_sum(2.f * uh, -mh, s, e);
               two_sum(s, scaled(xs[c]), t, e2);
               fast_two_sum(t, (e + e2) + (2.f * ul - ml), oh, ol);
               a.out[q] = oh;
               a.out[q + lo] = ol;
            }
         } else {
            const float* RH = reinterpret_cast<const float*>(ms + M::rho);
            float sg[3] = {0.f, 0.f, 0.f};
            if (a.beta != 0.f) {
               const float* dd = dd_plane(k);
               const float cxi = __ldg(a.co[0] + (i - a.ib)), cyj = __ldg(a.co[1] + (j - a.jb)),
                           czk = __ldg(a.co[2] + (k - a.kb));
               const float dx0 = __ldg(a.dc[0] + (i - 1 - a.ib)), dx1 = __ldg(a.dc[0] + (i - a.ib)),
                           dx2 = __ldg(a.dc[0] + (i + 1 - a.ib));
               if (dx0 != 0.f || dx1 != 0.f || dx2 != 0.f) {
                  const float e0 = RH[own - 1] * dx0, e1 = RH[own] * dx1, e2 = RH[own + 1] * dx2;
                  const float w = sxi * cyj * czk;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const float* d = dd + c * PLANE + own;
                     sg[c] += w * (e2 * (d[2] - 2.f * d[1] + d[0]) - 2.f * e1 * (d[1] - 2.f * d[0] + d[-1]) +
                                   e0 * (d[0] - 2.f * d[-1] + d[-2]));
                  }
               }
               const float dy0 = __ldg(a.dc[1] + (j - 1 - a.jb)), dy1 = __ldg(a.dc[1] + (j - a.jb)),
                           dy2 = __ldg(a.dc[1] + (j + 1 - a.jb));
               if (dy0 != 0.f || dy1 != 0.f || dy2 != 0.f) {
                  const float e0 = RH[own - PX] * dy0, e1 = RH[own] * dy1, e2 = RH[own + PX] * dy2;
                  const float w = syj * cxi * czk;
#pragma unroll
                  for (int c = 0; c < 3; c++) {
                     const float* d = dd + c * PLANE + own;
                     sg[c] += w * (e2 * (d[2 * PX] - 2.f * d[PX] + d[0]) -
                                   2.f * e1 * (d[PX] - 2.f * d[0] + d[-PX]) +
                                   e0 * (d[0] - 2.f * d[-PX] + d[-2 * PX]));
                  }
               }
               const float dz0 = __ldg(a.dc[2] + (k - 1 - a.kb)), dz1 = __ldg(a.dc[2] + (k - a.kb)),
                           dz2 = __ldg(a.dc[2] + (k + 1 - a.kb));
               if (dz0 != 0.f || dz1 != 0.f || dz2 != 0.f) {
                  const float e0 = __ldg(a.rho + p - a.nij) * dz0, e1 = RH[own] * dz1,
                              e2 = __ldg(a.rho + p + a.nij) * dz2;
                  const float w = szk * cxi * cyj;
#pragma unroll
                  for (int c = 0; c < 3; c++)
                     sg[c] += w * (e2 * (dq[4][c] - 2.f * dq[3][c] + dq[2][c]) -
                                   2.f * e1 * (dq[3][c] - 2.f * dq[2][c] + dq[1][c]) +
                                   e0 * (dq[2][c] - 2.f * dq[1][c] + dq[0][c]));
               }
            }
            const float birho = a.beta * irh;
#pragma unroll
            for (int c = 0; c < 3; c++) {
               const long long q = p + c * npts;
               const float uph = ownlev[c * OWNP + ownr], upl = ownlev[(c + 3) * OWNP + ownr];
               float t, e, oh, ol;
               two_sum(uph, scaled(xs[c]) - birho * sg[c], t, e);
               fast_two_sum(t, e + upl, oh, ol);
               a.out[q] = oh;
               a.out[q + lo] = ol;
            }
         }
      }
      __syncthreads();  // (C): GX/GY, M stage k and the oldest ring slot are free
   }
}

// ---- host side: tensor-map encoding ----
PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
   static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
   static std::once_flag once;
   std::call_once(once, [] {
      void* p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                           &q) == cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
         fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
   });
   return fn;
}

// A float tensor of rank 3 or 4 over a level (x = i, y = j, z = k[, w = hi/lo comp])
// or a pair array (x = 2i + hi/lo).
struct MapKey {
   const void* ptr;
   int rank;
   unsigned long long dim[4], stride[3];
   unsigned box[4];
   bool operator<(const MapKey& o) const { return std::memcmp(this, &o, sizeof(MapKey)) < 0; }
};

// Encoded maps are cached by every argument of the encoding, so a cached map is
// always the map the arguments describe (also after the memory is freed and the
// address reused with the same shape).
int encode(const MapKey& key, CUtensorMap* out)
{
   static std::mutex mtx;
   static std::map<MapKey, CUtensorMap> cache;
   std::lock_guard<std::mutex> lock(mtx);
   auto it = cache.find(key);
   if (it != cache.end()) {
      *out = it->second;
      return kOk;
   }
   auto fn = encode_fn();
   if (!fn) return kCudaError;
   cuuint64_t dim[4], stride[3];
   cuuint32_t box[4], es[4] = {1, 1, 1, 1};
   for (int d = 0; d < key.rank; d++) {
      dim[d] = key.dim[d];
      box[d] = key.box[d];
      if (d < key.rank - 1) stride[d] = key.stride[d];
   }
   CUtensorMap m;
   const CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, key.rank, const_cast<void*>(key.ptr),
                         dim, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
   if (r != CUDA_SUCCESS) return kCudaError;
   if (cache.size() > 4096) cache.clear();
   cache.emplace(key, m);
   *out = m;
   return kOk;
}

MapKey level_key(const Box& b, const float* p, unsigned by)
{
   MapKey k;
   std::memset(&k, 0, sizeof k);
   k.ptr = p;
   k.rank = 4;
   k.dim[0] = b.ni;
   k.dim[1] = b.nij / b.ni;
   k.dim[2] = b.npts / b.nij;
   k.dim[3] = 6;
   k.stride[0] = b.ni * 4;
   k.stride[1] = b.nij * 4;
   k.stride[2] = b.npts * 4;
   k.box[0] = 36;
   k.box[1] = by;
   k.box[2] = 1;
   k.box[3] = 6;
   return k;
}

MapKey scalar_key(const Box& b, const void* p, int pairs, unsigned bx, unsigned by, unsigned bz)
{
   MapKey k;
   std::memset(&k, 0, sizeof k);
   k.ptr = p;
   k.rank = 3;
   k.dim[0] = b.ni * (pairs ? 2 : 1);
   k.dim[1] = b.nij / b.ni;
   k.dim[2] = b.npts / b.nij;
   k.stride[0] = k.dim[0] * 4;
   k.stride[1] = b.nij * (pairs ? 8 : 4);
   k.box[0] = bx;
   k.box[1] = by;
   k.box[2] = bz;
   return k;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

// The tensor-copy path applies when every row and plane stride is a multiple of 16
// bytes and every base address is 16-byte aligned.
bool mixed_stage_tma_ok(const MixedStage& st)
{
   if (st.corrector != 0 && st.corrector != 1) return false;
   if (st.b.ni % 4 != 0) return false;
   if (!encode_fn()) return false;
   const void* ptrs[] = {st.u, st.um, st.mu2, st.la2, st.ir2, st.corrector ? st.up : st.u,
                         st.corrector ? (const void*)st.rho : (const void*)st.u};
   for (const void* p : ptrs)
      if (!aligned16(p)) return false;
   for (int q = 0; q < kWeightArrays; q++)
      if (!aligned16(st.w2[q])) return false;
   return true;
}

int launch_mixed_stage_tma(const MixedStage& st, cudaStream_t stream)
{
   if (st.k2 < st.k1) return kOk;
   if (!mixed_stage_tma_ok(st)) return kBadArgument;
   const Box& b = st.b;
   const int corr = st.corrector;
   TmaMaps tm;
   std::memset(&tm, 0, sizeof tm);
   if (corr) {
      SW4G_TRY(encode(level_key(b, st.up, 12), &tm.lev_halo[0]));
      SW4G_TRY(encode(level_key(b, st.u, 12), &tm.lev_halo[1]));
      SW4G_TRY(encode(level_key(b, st.um, 12), &tm.lev_halo[2]));
      SW4G_TRY(encode(level_key(b, st.up, 8), &tm.lev_own));
      SW4G_TRY(encode(scalar_key(b, st.rho, 0, 36, 12, 1), &tm.rho_halo));
   } else {
      SW4G_TRY(encode(level_key(b, st.u, 12), &tm.lev_halo[0]));
      SW4G_TRY(encode(level_key(b, st.um, 8), &tm.lev_own));
   }
   SW4G_TRY(encode(scalar_key(b, st.mu2, 1, 72, 12, 1), &tm.mu_halo));
   SW4G_TRY(encode(scalar_key(b, st.la2, 1, 72, 12, 1), &tm.la_halo));
   SW4G_TRY(encode(scalar_key(b, st.mu2, 1, 72, 8, 1), &tm.mu_own));
   SW4G_TRY(encode(scalar_key(b, st.la2, 1, 72, 8, 1), &tm.la_own));
   SW4G_TRY(encode(scalar_key(b, st.ir2, 1, 72, 8, 1), &tm.ir_own));
   // weight arrays: index ax*4 + t*2 + (0: W1, 1: W2)
   for (int q = 0; q < 4; q++) {
      SW4G_TRY(encode(scalar_key(b, st.w2[q], 1, 72, 8, 1), &tm.wx[q]));
      SW4G_TRY(encode(scalar_key(b, st.w2[4 + q], 1, 72, 10, 1), &tm.wy[q]));
   }
   for (int t = 0; t < 2; t++) {
      SW4G_TRY(encode(scalar_key(b, st.w2[8 + 2 * t], 1, 72, 8, 3), &tm.wz1[t]));
      SW4G_TRY(encode(scalar_key(b, st.w2[9 + 2 * t], 1, 72, 8, 2), &tm.wz2[t]));
   }

   TmaArgs a;
   a.ib = b.ib; a.ie = b.ie; a.jb = b.jb; a.je = b.je; a.kb = b.kb; a.ke = b.ke;
   a.ni = b.ni; a.nij = b.nij; a.npts = b.npts;
   a.k1 = st.k1;
   a.k2 = st.k2;
   a.out = st.out;
   a.rho = st.rho;
   a.sx = st.st[0];
   a.sy = st.st[1];
   a.sz = st.st[2];
   for (int q = 0; q < 3; q++) {
      a.dc[q] = st.dc[q];
      a.co[q] = st.co[q];
   }
   const double coef = st.coef != 0 ? st.coef : (corr == 1 ? st.dt * st.dt / 12 : st.dt * st.dt);
   const double K = coef / (144 * st.h * st.h);
   a.Kh = (float)K;
   a.Kl = (float)(K - (double)a.Kh);
   a.beta = (float)st.beta;
   a.status = st.status;

   const int ni = b.ie - b.ib - 3, nj = b.je - b.jb - 3, nk = st.k2 - st.k1 + 1;
   const int gx = blocks_for(ni, TX), gy = blocks_for(nj, TY);
   const size_t smem = corr ? Layout<1>::bytes : Layout<0>::bytes;
   const void* kern = corr ? (const void*)mixed_stage_tma_kernel<1> : (const void*)mixed_stage_tma_kernel<0>;
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kCudaError;
   static bool attr_set[2][64] = {};
   static int resident[2][64] = {};
   static std::mutex amtx;
   {
      std::lock_guard<std::mutex> lock(amtx);
      if (!attr_set[corr][dev]) {
         if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
             cudaSuccess)
            return kCudaError;
         resident[corr][dev] = resident_ctas(kern, NTHREADS, smem);
         attr_set[corr][dev] = true;
      }
   }
   a.kchunk = stage_kchunk((long long)gx * gy, nk, resident[corr][dev], 12);
   const dim3 grid(gx, gy, (nk + a.kchunk - 1) / a.kchunk), block(TX, TY, 1);
   if (corr)
      mixed_stage_tma_kernel<1><<<grid, block, smem, stream>>>(tm, a);
   else
      mixed_stage_tma_kernel<0><<<grid, block, smem, stream>>>(tm, a);
   return launch_status();
}

}  // namespace sw4g
