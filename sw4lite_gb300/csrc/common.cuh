// Shared definitions for the sm_103a kernels of the sw4lite elastic time step.
//
// Index conventions are the reference's (src/EW.C:1921-1949, src/rhs4sg_rev.C:58-78):
// inclusive 1-based bounds [ib,ie]x[jb,je]x[kb,ke] that include 2 ghost points
// per side, i fastest.  A 3-component field is stored either component-major
// ("SoA", the reference's _rev/_indrev layout, u[c*npts + p]) or point-major
// ("AoS", u[3*p + c]); Box carries the two strides so one kernel serves both.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace sw4g {

struct Box {
   int ib, ie, jb, je, kb, ke;
   long long ni, nij, npts;
   long long cs;  // component stride: npts (SoA) or 1 (AoS)
   long long ps;  // point stride: 1 (SoA) or 3 (AoS)
};

inline Box make_box(int soa, int ib, int ie, int jb, int je, int kb, int ke)
{
   Box b;
   b.ib = ib; b.ie = ie; b.jb = jb; b.je = je; b.kb = kb; b.ke = ke;
   b.ni = ie - ib + 1;
   b.nij = b.ni * (je - jb + 1);
   b.npts = b.nij * (ke - kb + 1);
   b.cs = soa ? b.npts : 1;
   b.ps = soa ? 1 : 3;
   return b;
}

__host__ __device__ __forceinline__ long long pidx(const Box& b, int i, int j, int k)
{
   return (long long)(i - b.ib) + b.ni * (j - b.jb) + b.nij * (long long)(k - b.kb);
}

__host__ __device__ __forceinline__ long long cidx(const Box& b, int c, int i, int j, int k)
{
   return c * b.cs + b.ps * pidx(b, i, j, k);
}

// Field accessors for the kernels that run in FP64 arithmetic whatever the
// storage: plain FP64 arrays, or the mixed form's double-float pairs (hi at q,
// lo at q + lo_offset; see df.cuh).
struct F64Field {
   double* p;
   __device__ __forceinline__ double get(long long q) const { return p[q]; }
   __device__ __forceinline__ void set(long long q, double v) const { p[q] = v; }
   __device__ __forceinline__ static void copy(const F64Field& d, long long qd, const F64Field& s,
                                               long long qs)
   {
      d.p[qd] = s.p[qs];
   }
};

struct DFField {
   float* h;
   long long lo;  // offset of the lo half
   __device__ __forceinline__ double get(long long q) const
   {
      return (double)h[q] + (double)h[q + lo];
   }
   __device__ __forceinline__ void set(long long q, double v) const
   {
      const float a = __double2float_rn(v);
      h[q] = a;
      h[q + lo] = __double2float_rn(v - (double)a);
   }
   __device__ __forceinline__ static void copy(const DFField& d, long long qd, const DFField& s,
                                               long long qs)
   {
      d.h[qd] = s.h[qs];
      d.h[qd + d.lo] = s.h[qs + s.lo];
   }
};

// Status codes returned through the C ABI (include/sw4g.h).
enum Status : int {
   kOk = 0,
   kBadArgument = 1,
   kCudaError = 2,
   kNanDetected = 3,
   kNotSupported = 4,
   kTimeout = 5,
   kIoError = 6,
};

// Returns from the calling function with the status of expr unless it is kOk.
#define SW4G_TRY(expr)            \
   do {                           \
      int _st = (expr);           \
      if (_st != kOk) return _st; \
   } while (0)

inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? kOk : kCudaError; }

// Converts the sticky/launch error state into a status code.
inline int launch_status()
{
   cudaError_t e = cudaGetLastError();
   return e == cudaSuccess ? kOk : kCudaError;
}

inline int blocks_for(long long n, int threads)
{
   long long b = (n + threads - 1) / threads;
   return (int)(b > 0 ? b : 1);
}

// Planes per CTA of a stage kernel that marches along k over cols CTA columns of nk
// planes, with `resident` CTAs of it on each SM at once.  The launch runs in waves of
// resident x SMs CTAs and a last wave that fills only part of the GPU leaves the rest
// idle, so the chunk count minimises waves x (planes per chunk + the ring's warm-up,
// about two planes' work) over the counts that give at least 3.5 waves, with at
// least min_planes planes per chunk.  A positive
// stage_chunks_override() (sw4g_dev_set_stage_chunks) replaces the count.
int stage_kchunk(long long cols, int nk, int resident, int min_planes);
int stage_chunks_override();
void set_stage_chunks_override(int chunks);
// CTAs of `kernel` resident per SM at `threads` threads and `smem` dynamic bytes
int resident_ctas(const void* kernel, int threads, size_t smem);

}  // namespace sw4g
