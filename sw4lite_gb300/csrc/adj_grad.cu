// Material gradient of one FP64 adjoint step, in double-float arithmetic.
//
// The gradient of a1 . u+ with respect to (rho, mu, lambda) at fixed (u, um) is a
// sum of products of differences of an adjoint level (b1, or mt = b1 + dt^2/12 R
// L(b1)) and a forward level (w1 = up - 2u + um, or u).  The stretching factors
// cancel along every difference: with v = c W b (W = 1/(sx sy sz)),
//   (s_a v)(q + m e_a) - (s_a v)(q) = c / (s_b s_c) (b(q + m e_a) - b(q)),
// the factor constant along axis a.  So each step needs only plain differences and
// their products, and the profile factors enter once per point:
//   mu, lambda : K [ sum_a 24 s_a/(s_b s_c) S_a + sum_t M_t / s_t ],
//                K = -(dt^2/12) / (144 h^2),
//     S_a  the seven-edge combination of the same-axis second differences
//          (v . D2(a) w = -sum_q sum_{m=1,2} W_m(q) (v(q+m)-v(q)) (w(q+m)-w(q))),
//          summed over the pairs (b1, w1) and 12 x (mt, u);
//     M_t  the mixed terms whose two axes are not t: products of centred first
//          differences (lambda: the diagonal ones, mu: the off-diagonal ones);
//   rho        : -W [mt . w1 + b1 . (un - up)]  (interior points)
//                - beta sum_a dc_a co_b co_c/(s_b s_c) sum_c D2_a(u - um) D2_a(b1).
// The products run on the FP32 pipe in double-float arithmetic: a value is the
// unevaluated sum of two FP32 numbers (47 significant bits), sums use Knuth's
// TwoSum and Dekker's FastTwoSum, products FMA.  GB300 issues FP32 at 64 times its
// FP64 rate, so this costs a fraction of the FP64 form of the same sums.  Before the
// split every value is scaled by a power of two (adjoint levels by a bound from the
// injected residuals, forward levels by the maximum over the recomputed segment) that
// maps the level's largest value near 2^28: values down to about 2^-131 of it keep
// all 47 bits, values below 2^-154 of it count as zero.  Each point's sums go into
// double-float accumulators, added to the FP64 gradients once per segment.
//
// The cancellations that matter stay in FP64: w1 = (up - 2u) + um and un - up are
// formed from the FP64 levels before the split.
//
// Free-surface z sides: the state vector's norm gains the SBP weights H (17/48,
// 59/48, 43/48, 49/48 on the four planes next to the side), so the adjoint variable
// is b = (H W)^-1 R a and every term above carries H at its row.  The terms along x
// and y stay in their plane, so H joins the z profile factors (1/s_z, co_z/s_z).  The
// z-involving terms of the six one-sided rows next to the side differ from the centred
// form: the edge and combine kernels treat the adjoint values on those rows as zero for
// them (planes k <= zlo, k >= zhi), and grad_rows_kernel adds those rows' terms,
// differentiated term by term from the one-sided operator and the ghost plane's
// traction condition (src/rhs4sg_rev.C:349-856, src/ew-cfromfort.C:415-476), in FP64.
//
// The FP32-mixed form runs the same edge and combine kernels with single FP32 values
// (number type F1) on its double-float levels rounded to FP32 (w1 and un - up formed
// exactly from the pairs first), and adds each point's sums to the FP64 gradients
// every step.
#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "sbp.h"

namespace sw4g {
namespace {

struct DF {
   float h, l;
};

__device__ __forceinline__ DF df_zero() { return {0.f, 0.f}; }
__device__ __forceinline__ DF df_of(float2 a) { return {a.x, a.y}; }
__device__ __forceinline__ DF df_neg(DF a) { return {-a.h, -a.l}; }

// a - b: the leading difference exact (TwoSum), the trailing parts added once
__device__ __forceinline__ DF df_diff(DF a, DF b)
{
   float s, e;
   two_sum(a.h, -b.h, s, e);
   return {s, __fadd_rn(e, __fsub_rn(a.l, b.l))};
}

// a + b, renormalised
__device__ __forceinline__ DF df_add(DF a, DF b)
{
   float s, e;
   two_sum(a.h, b.h, s, e);
   e = __fadd_rn(e, __fadd_rn(a.l, b.l));
   DF r;
   fast_two_sum(s, e, r.h, r.l);
   return r;
}

// a * b to about 2^-46 relative (the lo * lo term dropped)
__device__ __forceinline__ DF df_mul(DF a, DF b)
{
   const float p = __fmul_rn(a.h, b.h);
   float e = __fmaf_rn(a.h, b.h, -p);
   e = __fmaf_rn(a.h, b.l, e);
   e = __fmaf_rn(a.l, b.h, e);
   return {p, e};
}

// a + b without the final renormalisation (the trailing part within a few ulp of
// the leading one): for sums that feed a product or another sum
__device__ __forceinline__ DF df_addf(DF a, DF b)
{
   float s, e;
   two_sum(a.h, b.h, s, e);
   return {s, __fadd_rn(e, __fadd_rn(a.l, b.l))};
}

// k a for a power of two k (exact)
__device__ __forceinline__ DF df_pow2(DF a, float k) { return {__fmul_rn(k, a.h), __fmul_rn(k, a.l)}; }

// k a for a small integer k (the rounding of k a.h kept)
__device__ __forceinline__ DF df_scale(DF a, float k)
{
   const float p = __fmul_rn(k, a.h);
   return {p, __fmaf_rn(k, a.l, __fmaf_rn(k, a.h, -p))};
}

// One FP32 value with the same operations (the mixed form's gradient terms).
struct F1 {
   float h;
};
__device__ __forceinline__ F1 df_neg(F1 a) { return {-a.h}; }
__device__ __forceinline__ F1 df_diff(F1 a, F1 b) { return {a.h - b.h}; }
__device__ __forceinline__ F1 df_add(F1 a, F1 b) { return {a.h + b.h}; }
__device__ __forceinline__ F1 df_addf(F1 a, F1 b) { return {a.h + b.h}; }
__device__ __forceinline__ F1 df_mul(F1 a, F1 b) { return {a.h * b.h}; }
__device__ __forceinline__ F1 df_pow2(F1 a, float k) { return {k * a.h}; }
__device__ __forceinline__ F1 df_scale(F1 a, float k) { return {k * a.h}; }

// storage and conversions of a number type: S the stored element of the level and
// edge arrays, of() a stored element, ofp() a profile pair, st() the stored form
template <class V>
struct Num;
template <>
struct Num<DF> {
   using S = float2;
   static __device__ __forceinline__ DF zero() { return {0.f, 0.f}; }
   static __device__ __forceinline__ DF of(float2 a) { return {a.x, a.y}; }
   static __device__ __forceinline__ DF ofp(float2 a) { return {a.x, a.y}; }
   static __device__ __forceinline__ float2 st(DF v) { return make_float2(v.h, v.l); }
};
template <>
struct Num<F1> {
   using S = float;
   static __device__ __forceinline__ F1 zero() { return {0.f}; }
   static __device__ __forceinline__ F1 of(float a) { return {a}; }
   static __device__ __forceinline__ F1 ofp(float2 a) { return {a.x + a.y}; }
   static __device__ __forceinline__ float st(F1 v) { return v.h; }
};
template <class V>
__device__ __forceinline__ const typename Num<V>::S* arr(const void* p)
{
   return static_cast<const typename Num<V>::S*>(p);
}

// the shift of a level class: 2^(emax - 1023 + margin) bounds its values
__device__ __forceinline__ int shift_of(int emax, int margin)
{
   return min(900, max(-800, emax - 1023 + margin));
}

// x 2^-sh as a pair (hi: the leading 24 bits, lo: the next 23, rounded) by integer
// operations on the FP64 bit pattern; kb = (896 + sh) << 20.  Values below
// 2^(sh - 126) give (0, 0); below 2^(sh - 103) the lo part is dropped.
__device__ __forceinline__ float2 to_df(double x, int kb)
{
   const int H = __double2hiint(x);
   const unsigned L = (unsigned)__double2loint(x);
   const int M = (H & 0x7fffffff) - kb;  // FP32 exponent field << 20 | top 20 mantissa bits
   if (M < (1 << 20)) return make_float2(0.f, 0.f);
   const unsigned sgn = (unsigned)H & 0x80000000u;
   const float hi = __uint_as_float(__funnelshift_l(L, (unsigned)M, 3) | sgn);
   const int eb = (M >> 20) - 23;  // exponent field of 2^(E - 23)
   float lo = 0.f;
   if (eb > 0) {
      // (r >> 6, rounded) 2^(E - 46) as 2^(E-23) (1 + r'/2^23) - 2^(E-23), exact
      const int base = eb << 23;
      const int r = (int)(((L & 0x1fffffffu) + 32u) >> 6);
      const float m = __int_as_float(base + r) - __int_as_float(base);
      lo = __uint_as_float(__float_as_uint(m) | sgn);
   }
   return make_float2(hi, lo);
}

__device__ __forceinline__ void acc_add(float2* a, long long p, DF v)
{
   const DF s = df_add(df_of(a[p]), v);
   a[p] = make_float2(s.h, s.l);
}

// the largest FP64 exponent field over n values, into *out (atomicMax)
__global__ void __launch_bounds__(256) exp_max_kernel(const double* __restrict__ x, long long n,
                                                      int* __restrict__ out)
{
   int m = 0;
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x)
      m = max(m, (__double2hiint(__ldg(x + q)) >> 20) & 0x7ff);
   m = __reduce_max_sync(0xffffffffu, m);
   if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, m);
}

// the largest exponent field of the injected adjoint sources sxyz/rho res over
// every residual row and receiver
__global__ void inj_exp_kernel(Box b, const double* __restrict__ s0, const double* __restrict__ s1,
                               const double* __restrict__ s2, int nrec, const int* __restrict__ ijk,
                               const double* __restrict__ res, long long rows, int nval,
                               const double* __restrict__ rho, const double* __restrict__ hz,
                               int* __restrict__ out)
{
   const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
   int m = 0;
   if (t < rows * nrec) {
      const int r = (int)(t % nrec);
      const long long row = t / nrec;
      const int i = ijk[3 * r], j = ijk[3 * r + 1], k = ijk[3 * r + 2];
      const double s = s0[i - b.ib] * s1[j - b.jb] * s2[k - b.kb] / (rho[pidx(b, i, j, k)] * (hz ? hz[k - b.kb] : 1.0));
      for (int c = 0; c < 3; c++)
         m = max(m, (__double2hiint(fabs(s * res[row * nval + 3 * r + c])) >> 20) & 0x7ff);
   }
   m = __reduce_max_sync(0xffffffffu, m);
   if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, m);
}

// per axis: 24 st, 1/st, co/st, beta dc as pairs
// (hz: the SBP norm weights of the z planes next to free-surface sides, for axis 2)
__global__ void grad_profiles_kernel(int n, const double* __restrict__ st, const double* __restrict__ co,
                                     const double* __restrict__ dc, double beta, float2* __restrict__ st24,
                                     float2* __restrict__ ist, float2* __restrict__ cist,
                                     float2* __restrict__ bdc, const double* __restrict__ hz)
{
   const int x = blockIdx.x * blockDim.x + threadIdx.x;
   if (x >= n) return;
   const double hw = hz ? hz[x] : 1.0;
   float h, l;
   df_split(24 * st[x], h, l);
   st24[x] = make_float2(h, l);
   df_split(hw / st[x], h, l);
   ist[x] = make_float2(h, l);
   df_split(hw * co[x] / st[x], h, l);
   cist[x] = make_float2(h, l);
   df_split(beta * dc[x], h, l);
   bdc[x] = make_float2(h, l);
}

// The step kernels: one thread per array point, kGradThreads consecutive points of
// a k plane (rows of i) per CTA, blockIdx.y the plane.  They run beside the FP64
// stage kernels, in the registers those leave free: the predictor-form stage (96
// registers x 512 threads per SM) leaves 16K, room for three 64-thread CTAs of
// grad_df_kernel (72 registers) but one of 128 threads.
constexpr int kGradThreads = 64;

// w1 = up - 2u + um; the pairs of b1, mt (adjoint shift) and w1, u, um (forward
// shift); the rho terms -W [mt . w1 + b1 . (un - up)] of the interior points
__global__ void __launch_bounds__(kGradThreads) grad_prep_kernel(GradDF g)
{
   const Box& b = g.b;
   const int t = blockIdx.x * kGradThreads + threadIdx.x;
   if (t >= (int)b.nij) return;
   const int i = b.ib + t % (int)b.ni, j = b.jb + t / (int)b.ni, k = b.kb + blockIdx.y;
   const long long n = b.npts;
   const long long p = t + (k - b.kb) * b.nij;
   const int ka = (896 + shift_of(g.emax[0], g.marg_a)) << 20;
   const int kf = (896 + shift_of(g.emax[1], g.marg_f)) << 20;
   const bool in = i >= b.ib + 2 && i <= b.ie - 2 && j >= b.jb + 2 && j <= b.je - 2 && k >= b.kb + 2 &&
                   k <= b.ke - 2;
   DF acc = df_zero();
#pragma unroll
   for (int c = 0; c < 3; c++) {
      const long long q = c * n + p;
      const double uq = __ldg(g.u + q), umq = __ldg(g.um + q), upq = __ldg(g.up + q);
      const double w1 = (upq - 2 * uq) + umq;
      // the adjoint is a vector on the interior: zero on the ghost points (a free
      // surface's ghost plane of b1 and mt holds the traction condition's values)
      const float2 vb = in ? to_df(__ldg(g.b1 + q), ka) : make_float2(0.f, 0.f);
      const float2 vm = in ? to_df(__ldg(g.mt + q), ka) : make_float2(0.f, 0.f);
      const float2 fw = to_df(w1, kf);
      static_cast<float2*>(g.db1)[q] = vb;
      static_cast<float2*>(g.dmt)[q] = vm;
      static_cast<float2*>(g.dw1)[q] = fw;
      static_cast<float2*>(g.du)[q] = to_df(uq, kf);
      static_cast<float2*>(g.dum)[q] = to_df(umq, kf);
      if (in) {
         const float2 d = to_df(__ldg(g.un + q) - upq, kf);
         acc = df_add(acc, df_add(df_mul(df_of(vm), df_of(fw)), df_mul(df_of(vb), df_of(d))));
      }
   }
   if (in) {
      const DF w = df_mul(df_mul(df_of(g.ist[0][i - b.ib]), df_of(g.ist[1][j - b.jb])),
                          df_of(g.ist[2][k - b.kb]));
      acc_add(static_cast<float2*>(g.ar), p, df_neg(df_mul(w, acc)));
   }
}

// The mixed form's step: its double-float levels (hi at q, lo at q + g.lo) rounded to
// FP32 values, w1 = up - 2u + um and un - up formed exactly first; the interior rho
// terms -W [mt . w1 + b1 . (un - up)] added to the FP64 gradient.
__device__ __forceinline__ float df_round(const float* x, long long q, long long lo)
{
   return __fadd_rn(__ldg(x + q), __ldg(x + q + lo));
}

__global__ void __launch_bounds__(kGradThreads) grad_prep_f1_kernel(GradDF g)
{
   const Box& b = g.b;
   const int t = blockIdx.x * kGradThreads + threadIdx.x;
   if (t >= (int)b.nij) return;
   const int i = b.ib + t % (int)b.ni, j = b.jb + t / (int)b.ni, k = b.kb + blockIdx.y;
   const long long n = b.npts, lo = g.lo;
   const long long p = t + (k - b.kb) * b.nij;
   const bool in = i >= b.ib + 2 && i <= b.ie - 2 && j >= b.jb + 2 && j <= b.je - 2 && k >= b.kb + 2 &&
                   k <= b.ke - 2;
   float acc = 0.f;
#pragma unroll
   for (int c = 0; c < 3; c++) {
      const long long q = c * n + p;
      // w1 = up - 2u + um exactly from the pairs, rounded once
      float s1, e1, s2, e2;
      two_sum(__ldg(g.lup + q), -2.f * __ldg(g.lu + q), s1, e1);
      two_sum(s1, __ldg(g.lum + q), s2, e2);
      const float w1 = s2 + ((e1 + e2) + ((__ldg(g.lup + q + lo) - 2.f * __ldg(g.lu + q + lo)) +
                                         __ldg(g.lum + q + lo)));
      const float vb = in ? df_round(g.lb1, q, lo) : 0.f, vm = in ? df_round(g.lmt, q, lo) : 0.f;
      static_cast<float*>(g.db1)[q] = vb;
      static_cast<float*>(g.dmt)[q] = vm;
      static_cast<float*>(g.dw1)[q] = w1;
      static_cast<float*>(g.du)[q] = df_round(g.lu, q, lo);
      static_cast<float*>(g.dum)[q] = df_round(g.lum, q, lo);
      if (in) {  // un - up exactly from the pairs
         float d, e;
         two_sum(__ldg(g.lun + q), -__ldg(g.lup + q), d, e);
         d = d + (e + (__ldg(g.lun + q + lo) - __ldg(g.lup + q + lo)));
         acc = fmaf(vm, w1, fmaf(vb, d, acc));
      }
   }
   if (in) {
      const float w = Num<F1>::ofp(g.ist[0][i - b.ib]).h * Num<F1>::ofp(g.ist[1][j - b.jb]).h *
                      Num<F1>::ofp(g.ist[2][k - b.kb]).h;
      g.gr64[p] -= (double)(w * acc);
   }
}


// the four edge sums {E1 mu, E1 lambda, E2 mu, E2 lambda} of the forward edges
// (q, q+1) and (q, q+2) along axis a, summed over the components (mu weight 2 for
// the component along a, lambda weight for it alone) and the pairs 12 x (mt, u) +
// (b1, w1).  CHECK: some of q, q+1, q+2 lie outside the array along a (values there
// count as zero; q may lie below the array).
template <class V, bool CHECK>
__device__ __forceinline__ void edges_body(const GradDF& g, long long n, int pq, bool ok0, bool ok1, bool ok2,
                                           bool ma0, bool ma1, bool ma2, int sd, int a, V E[4])
{
   using N = Num<V>;
   E[0] = E[1] = E[2] = E[3] = N::zero();
#pragma unroll
   for (int t = 0; t < 2; t++) {
      V s1 = N::zero(), s2 = N::zero(), a1 = N::zero(), a2 = N::zero();
#pragma unroll
      for (int c = 0; c < 3; c++) {
         const typename N::S* __restrict__ A = arr<V>(t == 0 ? g.dmt : g.db1) + c * n;
         const typename N::S* __restrict__ F = arr<V>(t == 0 ? g.du : g.dw1) + c * n;
         V x0, x1, x2, y0, y1, y2;
         if (CHECK) {
            x0 = ok0 && ma0 ? N::of(__ldg(A + pq)) : N::zero();
            y0 = ok0 ? N::of(__ldg(F + pq)) : N::zero();
            x1 = ok1 && ma1 ? N::of(__ldg(A + pq + sd)) : N::zero();
            y1 = ok1 ? N::of(__ldg(F + pq + sd)) : N::zero();
            x2 = ok2 && ma2 ? N::of(__ldg(A + pq + 2 * sd)) : N::zero();
            y2 = ok2 ? N::of(__ldg(F + pq + 2 * sd)) : N::zero();
         } else {
            x0 = N::of(__ldg(A + pq));
            y0 = N::of(__ldg(F + pq));
            x1 = N::of(__ldg(A + pq + sd));
            y1 = N::of(__ldg(F + pq + sd));
            x2 = N::of(__ldg(A + pq + 2 * sd));
            y2 = N::of(__ldg(F + pq + 2 * sd));
         }
         const V e1 = df_mul(df_diff(x1, x0), df_diff(y1, y0));
         const V e2 = df_mul(df_diff(x2, x0), df_diff(y2, y0));
         s1 = df_addf(s1, e1);
         s2 = df_addf(s2, e2);
         if (c == a) {
            a1 = e1;
            a2 = e2;
         }
      }
      const float wt = t == 0 ? 12.f : 1.f;
      E[0] = df_add(E[0], df_scale(df_addf(s1, a1), wt));
      E[1] = df_add(E[1], df_scale(a1, wt));
      E[2] = df_add(E[2], df_scale(df_addf(s2, a2), wt));
      E[3] = df_add(E[3], df_scale(a2, wt));
   }
}

// the adjoint value of plane k enters the z-involving terms (not a one-sided row)
__device__ __forceinline__ bool zrow(const GradDF& g, int k) { return k > g.zlo && k < g.zhi; }

template <class V>
__device__ __forceinline__ void edges_at(const GradDF& g, long long n, int pq, int xq, int xl, int xh, int sd,
                                         int a, V E[4])
{
   const bool m0 = a != 2 || zrow(g, xq), m1 = a != 2 || zrow(g, xq + 1), m2 = a != 2 || zrow(g, xq + 2);
   if (xq >= xl && xq + 2 <= xh && m0 && m1 && m2)
      edges_body<V, false>(g, n, pq, true, true, true, true, true, true, sd, a, E);
   else
      edges_body<V, true>(g, n, pq, xq >= xl, xq + 1 >= xl && xq + 1 <= xh, xq + 2 >= xl && xq + 2 <= xh, m0,
                          m1, m2, sd, a, E);
}

// the edge sums of every array point: ed[(a*4 + r) * npts + p]
template <class V>
__global__ void __launch_bounds__(kGradThreads) grad_edge_kernel(GradDF g)
{
   const Box& b = g.b;
   const int t = blockIdx.x * kGradThreads + threadIdx.x;
   if (t >= (int)b.nij) return;
   const int i = b.ib + t % (int)b.ni, j = b.jb + t / (int)b.ni, k = b.kb + (int)blockIdx.y;
   const long long n = b.npts;
   const int p = t + (k - b.kb) * (int)b.nij;
#pragma unroll 1
   for (int a = 0; a < 3; a++) {
      const int x = a == 0 ? i : a == 1 ? j : k;
      const int xl = a == 0 ? b.ib : a == 1 ? b.jb : b.kb, xh = a == 0 ? b.ie : a == 1 ? b.je : b.ke;
      const int sd = a == 0 ? 1 : a == 1 ? (int)b.ni : (int)b.nij;
      V E[4];
      edges_at<V>(g, n, p, x, xl, xh, sd, a, E);
#pragma unroll
      for (int r = 0; r < 4; r++)
         static_cast<typename Num<V>::S*>(g.ed)[(a * 4 + r) * n + p] = Num<V>::st(E[r]);
   }
}

// centred first differences (DW . f)(p) = f(p-2) - f(p+2) + 8 (f(p+1) - f(p-1)) of
// one component of A and F along an axis (x[m], y[m]: values at p + (m-2) sd)
template <class V>
__device__ __forceinline__ void first_diffs(const V x[5], const V y[5], bool inner, V& fa, V& fw)
{
   fa = df_addf(df_diff(x[0], x[4]), df_pow2(df_diff(x[3], x[1]), 8.f));
   fw = inner ? df_addf(df_diff(y[0], y[4]), df_pow2(df_diff(y[3], y[1]), 8.f)) : Num<V>::zero();
}

// the mu, lambda and damping rho sums of one point from the edge sums, the centred
// first differences and the damping's second differences
// SG6: sixth-order damping's rho term; ZM: free-surface sides (the one-sided rows'
// masks).  Both are template parameters so the common case carries neither.
template <class V, bool SG6, bool ZM>
__global__ void __launch_bounds__(kGradThreads) grad_df_kernel(GradDF g)
{
   using N = Num<V>;
   // centred first differences of the current pair, [slot][thread]: slot c*3 + a for
   // the adjoint level, 9 + c*3 + a for the forward level
   __shared__ typename N::S fd[18][kGradThreads];
   const int tid = threadIdx.x;
   const Box& b = g.b;
   const int t0 = blockIdx.x * kGradThreads + tid;
   if (t0 >= (int)b.nij) return;
   const int pc[3] = {b.ib + t0 % (int)b.ni, b.jb + t0 / (int)b.ni, b.kb + (int)blockIdx.y};
   const long long n = b.npts;
   const int off[3] = {pc[0] - b.ib, pc[1] - b.jb, pc[2] - b.kb};
   const int p = off[0] + off[1] * (int)b.ni + off[2] * (int)b.nij;
   V gm = N::zero(), gl = N::zero(), gr = N::zero();
   // same-axis second differences: the seven edges of each axis around p
#pragma unroll 1
   for (int a = 0; a < 3; a++) {
      const int a1 = a == 2 ? 0 : a + 1, a2 = a == 0 ? 2 : a - 1;
      const int x0 = a == 0 ? pc[0] : a == 1 ? pc[1] : pc[2];
      const int xl = a == 0 ? b.ib : a == 1 ? b.jb : b.kb, xh = a == 0 ? b.ie : a == 1 ? b.je : b.ke;
      const int sd = a == 0 ? 1 : a == 1 ? (int)b.ni : (int)b.nij;
      const int oa = x0 - xl, o1 = a1 == 0 ? off[0] : a1 == 1 ? off[1] : off[2],
                o2 = a2 == 0 ? off[0] : a2 == 1 ? off[1] : off[2];
      const typename N::S* __restrict__ ed = arr<V>(g.ed) + a * 4 * n;
      V E[4][4];  // edges starting at p-2 .. p+1
      if (x0 - 2 >= xl && x0 + 1 <= xh) {
#pragma unroll
         for (int m = 0; m < 4; m++)
#pragma unroll
            for (int r = 0; r < 4; r++) E[m][r] = N::of(__ldg(ed + r * n + p + (m - 2) * sd));
      } else {
#pragma unroll
         for (int m = 0; m < 4; m++) {
            const int x = x0 + m - 2;
            const int q = p + (m - 2) * sd;
            if (x > xh) {
               E[m][0] = E[m][1] = E[m][2] = E[m][3] = N::zero();
            } else if (x >= xl) {
#pragma unroll
               for (int r = 0; r < 4; r++) E[m][r] = N::of(__ldg(ed + r * n + q));
            } else {  // an edge from below the array (ghost-point gradients)
               edges_at<V>(g, n, q, x, xl, xh, sd, a, E[m]);
            }
         }
      }
      // E1(p+1) + E1(p-2) + E2(p-1) + 3 [E1(p-1) + E1(p) - (E2(p) + E2(p-2))/4]
      V T[2];
#pragma unroll
      for (int r = 0; r < 2; r++) {
         const V X = df_addf(df_addf(E[3][r], E[0][r]), E[1][2 + r]);
         const V Y = df_addf(df_addf(E[1][r], E[2][r]), df_pow2(df_addf(E[2][2 + r], E[0][2 + r]), -0.25f));
         T[r] = df_addf(X, df_scale(Y, 3.f));
      }
      const V qq = df_mul(df_mul(N::ofp(__ldg(g.st24[a] + oa)), N::ofp(__ldg(g.ist[a1] + o1))),
                           N::ofp(__ldg(g.ist[a2] + o2)));
      gm = df_addf(gm, df_mul(qq, T[0]));
      gl = df_addf(gl, df_mul(qq, T[1]));
   }
   // pair 0: (mt, u) with weight 12 (c2 = 12 c1) and the damping term; pair 1: (b1, w1)
#pragma unroll 1
   for (int t = 0; t < 2; t++) {
      const float wt = t == 0 ? 12.f : 1.f;
#pragma unroll 1
      for (int a = 0; a < 3; a++) {
         const int a1 = a == 2 ? 0 : a + 1, a2 = a == 0 ? 2 : a - 1;
         const int x0 = a == 0 ? pc[0] : a == 1 ? pc[1] : pc[2];
         const int xl = a == 0 ? b.ib : a == 1 ? b.jb : b.kb, xh = a == 0 ? b.ie : a == 1 ? b.je : b.ke;
         const int sd = a == 0 ? 1 : a == 1 ? (int)b.ni : (int)b.nij;
         const int oa = x0 - xl, o1 = a1 == 0 ? off[0] : a1 == 1 ? off[1] : off[2],
                   o2 = a2 == 0 ? off[0] : a2 == 1 ? off[1] : off[2];
         const bool inner = x0 - 2 >= xl && x0 + 2 <= xh;
         const float2 bd = t == 0 ? __ldg(g.bdc[a] + oa) : make_float2(0.f, 0.f);
         const bool damp = t == 0 && !SG6 && x0 - 1 >= xl && x0 + 1 <= xh && bd.x != 0.f;
         // sixth order: b1 is taken as zero outside the points three from every edge
         // (the damping's rows), so the other two coordinates must lie there
         const bool damp6 = SG6 && t == 0 && bd.x != 0.f && off[a1] >= 3 &&
                            (a1 == 0 ? b.ie - b.ib : a1 == 1 ? b.je - b.jb : b.ke - b.kb) - off[a1] >= 3 &&
                            off[a2] >= 3 &&
                            (a2 == 0 ? b.ie - b.ib : a2 == 1 ? b.je - b.jb : b.ke - b.kb) - off[a2] >= 3;
         V ds = N::zero();
#pragma unroll
         for (int c = 0; c < 3; c++) {
            const typename N::S* __restrict__ A = arr<V>(t == 0 ? g.dmt : g.db1) + c * n;
            const typename N::S* __restrict__ F = arr<V>(t == 0 ? g.du : g.dw1) + c * n;
            V x[5], y[5];
            if (inner) {
#pragma unroll
               for (int m = 0; m < 5; m++) {
                  if (m == 2) continue;
                  x[m] = N::of(__ldg(A + p + (m - 2) * sd));
                  y[m] = N::of(__ldg(F + p + (m - 2) * sd));
               }
            } else {
#pragma unroll
               for (int m = 0; m < 5; m++) {
                  if (m == 2) continue;
                  const bool ok = x0 + m - 2 >= xl && x0 + m - 2 <= xh;
                  x[m] = ok ? N::of(__ldg(A + p + (m - 2) * sd)) : N::zero();
                  y[m] = ok ? N::of(__ldg(F + p + (m - 2) * sd)) : N::zero();
               }
            }
            if (ZM && a == 2 && (x0 - 2 <= g.zlo || x0 + 2 >= g.zhi)) {
#pragma unroll
               for (int m = 0; m < 5; m++)
                  if (m != 2 && !zrow(g, x0 + m - 2)) x[m] = N::zero();
            }
            V fa, fw;
            first_diffs<V>(x, y, inner, fa, fw);
            fd[c * 3 + a][tid] = N::st(fa);
            fd[9 + c * 3 + a][tid] = N::st(fw);
            if (damp) {  // D2(u - um) D2(b1) along a (y holds u at p -+ 1)
               const typename N::S* __restrict__ um = arr<V>(g.dum) + c * n;
               const typename N::S* __restrict__ b1 = arr<V>(g.db1) + c * n;
               const V d0 = df_diff(y[1], N::of(__ldg(um + p - sd)));
               const V d1 = df_diff(N::of(__ldg(F + p)), N::of(__ldg(um + p)));
               const V d2 = df_diff(y[3], N::of(__ldg(um + p + sd)));
               const V d2u = df_addf(df_addf(d0, d2), df_pow2(d1, -2.f));
               const V d2b = df_addf(df_addf(N::of(__ldg(b1 + p - sd)), N::of(__ldg(b1 + p + sd))),
                                      df_pow2(N::of(__ldg(b1 + p)), -2.f));
               ds = df_addf(ds, df_mul(d2u, d2b));
            }
            if (SG6 && damp6) {  // T(b1) T(u - um) at the half points x0 -+ 1/2
               const typename N::S* __restrict__ um = arr<V>(g.dum) + c * n;
               const typename N::S* __restrict__ b1 = arr<V>(g.db1) + c * n;
               V bb[5], dd[5];
#pragma unroll
               for (int m = 0; m < 5; m++) {
                  const int xm = x0 + m - 2;
                  const long long q = p + (long long)(m - 2) * sd;
                  const bool in = xm >= xl && xm <= xh;
                  dd[m] = in ? df_diff(N::of(__ldg(F + q)), N::of(__ldg(um + q))) : N::zero();
                  bb[m] = xm >= xl + 3 && xm <= xh - 3 ? N::of(__ldg(b1 + q)) : N::zero();
               }
               // T = (a3 - a0) + 3 (a1 - a2) over four consecutive values a0..a3
               auto T3 = [](const V* v) { return df_addf(df_diff(v[3], v[0]), df_scale(df_diff(v[1], v[2]), 3.f)); };
               ds = df_addf(ds, df_addf(df_mul(T3(bb), T3(dd)), df_mul(T3(bb + 1), T3(dd + 1))));
            }
         }
         if (damp || damp6) {
            const V cc = df_mul(N::ofp(__ldg(g.cist[a1] + o1)), N::ofp(__ldg(g.cist[a2] + o2)));
            const V term = df_mul(df_mul(N::ofp(bd), cc), ds);
            gr = df_addf(gr, df_neg(damp6 ? df_pow2(term, 0.5f) : term));
         }
      }
      // mixed terms, grouped by the axis t3 that neither derivative takes:
      // lambda from the diagonal first differences, mu from the off-diagonal ones
#pragma unroll 1
      for (int t3 = 0; t3 < 3; t3++) {
         const int a1 = t3 == 2 ? 0 : t3 + 1, a2 = t3 == 0 ? 2 : t3 - 1;
         // the terms with a z derivative skip the one-sided rows' adjoint values: the
         // in-plane first differences of a one-sided row's plane drop out of them
         const bool zoff = ZM && t3 != 2 && !zrow(g, pc[2]);
         auto A_ = [&](int c, int a) { return zoff && a != 2 ? N::zero() : N::of(fd[c * 3 + a][tid]); };
         auto W_ = [&](int c, int a) { return N::of(fd[9 + c * 3 + a][tid]); };
         const V ml = df_addf(df_mul(W_(a2, a2), A_(a1, a1)), df_mul(W_(a1, a1), A_(a2, a2)));
         const V mm = df_addf(df_mul(W_(a2, a1), A_(a1, a2)), df_mul(W_(a1, a2), A_(a2, a1)));
         const int ot = t3 == 0 ? off[0] : t3 == 1 ? off[1] : off[2];
         const V f = df_scale(N::ofp(__ldg(g.ist[t3] + ot)), wt);
         gm = df_addf(gm, df_mul(f, mm));
         gl = df_addf(gl, df_mul(f, ml));
      }
   }
   if constexpr (sizeof(V) == sizeof(DF)) {  // per-segment double-float sums
      acc_add(static_cast<float2*>(g.am), p, gm);
      acc_add(static_cast<float2*>(g.al), p, gl);
      acc_add(static_cast<float2*>(g.ar), p, gr);
   } else {  // the FP64 gradients, every step
      g.gm64[p] += g.kmu * (double)Num<V>::st(gm);
      g.gl64[p] += g.kmu * (double)Num<V>::st(gl);
      g.gr64[p] += (double)Num<V>::st(gr);
   }
}

// ---- the one-sided rows next to a free-surface z side ----
__constant__ double kr_acof[384];  // acof[(k-1) + 6 (q-1) + 48 (m-1)]
__constant__ double kr_bope[48];   // bope[(k-1) + 6 (q-1)]
__constant__ double kr_sbop[5];
__constant__ double kr_gh;         // ghcof of row 1 (the other rows' are zero)

constexpr int kRowThreads = 64;

template <bool DF>
__device__ __forceinline__ double rlvl(const GradRows& g, const double* d, const float* f, long long q)
{
   if (DF) return (double)__ldg(f + q) + (double)__ldg(f + q + g.lo);
   return __ldg(d + q);
}

// One thread per interior column (i, j).  Rows kk = 1..6 from the side (plane kq(kk)),
// the material planes kq(1..8); term by term (the FP64 checker restates the same):
//   zz   sum_q (sum_m acof(kk,q,m) coef(m)) w(q) + ghcof coef(bnd) w(ghost), coef mu
//        (components 0, 1) or 2mu + lambda (component 2); the ghost plane through the
//        traction condition: u, v ghosts free of the material, (2mu + la) w_ghost =
//        -[(2mu + la) Sw + kl la (ux + vy)] / sbop0;
//   dz_of_inner  s_a Dz(coef D_a w) / 12 (coef on the column, planes kq(q));
//   outer_of_dz  s_a D_a(coef Dz w) / 12 (coef at the rows' neighbours along a, gathered
//        here from the rows that reach this column).
template <bool DF>
__global__ void __launch_bounds__(kRowThreads) grad_rows_kernel(GradRows g)
{
   const Box& b = g.b;
   const int nic = b.ie - b.ib - 3, njc = b.je - b.jb - 3;
   const int t = blockIdx.x * kRowThreads + threadIdx.x;
   if (t >= nic * njc) return;
   const int i = b.ib + 2 + t % nic, j = b.jb + 2 + t / nic;
   const bool top = g.top != 0;
   const int kl = top ? 1 : -1;
   const long long n = b.npts;
   const double cof = 1 / (g.h * g.h), DW[5] = {1, -8, 0, 8, -1};
   const double d4a = 2.0 / 3.0, d4b = -1.0 / 12.0;
   auto kq = [&](int q) { return top ? q : g.nz - q + 1; };  // q = 1..8
   auto wz = [&](int kk, int q) {
      const double v = kr_bope[(kk - 1) + 6 * (q - 1)];
      return top ? v : -v;
   };
   auto Wf = [&](int P, int c, int ii, int jj, int kk) -> double {
      const long long q = c * n + pidx(b, ii, jj, kk);
      if (P == 1) return rlvl<DF>(g, g.u, g.lu, q);
      return (rlvl<DF>(g, g.up, g.lup, q) - 2 * rlvl<DF>(g, g.u, g.lu, q)) + rlvl<DF>(g, g.um, g.lum, q);
   };
   auto Va = [&](int P, int c, int ii, int jj, int kk) -> double {
      if (ii < b.ib + 2 || ii > b.ie - 2 || jj < b.jb + 2 || jj > b.je - 2) return 0.0;
      const long long q = c * n + pidx(b, ii, jj, kk);
      const double x = P == 0 ? rlvl<DF>(g, g.b1, g.lb1, q) : rlvl<DF>(g, g.mt, g.lmt, q);
      const double s = __ldg(g.sx + ii - b.ib) * __ldg(g.sy + jj - b.jb) * __ldg(g.sz + kk - b.kb);
      return (P == 0 ? g.c1 : g.c2) * __ldg(g.hz + kk - b.kb) * x / s;
   };
   const double sxi = __ldg(g.sx + i - b.ib), syj = __ldg(g.sy + j - b.jb);
   double gmc[8], glc[8];
#pragma unroll
   for (int m = 0; m < 8; m++) gmc[m] = glc[m] = 0;
#pragma unroll 1
   for (int P = 0; P < 2; P++) {
      // zz rows, one component at a time
#pragma unroll 1
      for (int c = 0; c < 3; c++) {
         double Vk[6], wq[8];
#pragma unroll
         for (int kk = 0; kk < 6; kk++) Vk[kk] = Va(P, c, i, j, kq(kk + 1));
#pragma unroll
         for (int q = 0; q < 8; q++) wq[q] = Wf(P, c, i, j, kq(q + 1));
#pragma unroll
         for (int m = 0; m < 8; m++) {
            double tm = 0;
#pragma unroll
            for (int kk = 0; kk < 6; kk++) {
               double y = 0;
#pragma unroll
               for (int q = 0; q < 8; q++) y = fma(kr_acof[kk + 6 * q + 48 * m], wq[q], y);
               tm = fma(Vk[kk], y, tm);
            }
            gmc[m] += cof * (c == 2 ? 2 * tm : tm);
            if (c == 2) glc[m] += cof * tm;
         }
      }
      // the ghost plane (row 1)
      {
         const int k = kq(1);
         double S[3] = {0, 0, 0};
#pragma unroll
         for (int q = 1; q <= 4; q++)
#pragma unroll
            for (int c = 0; c < 3; c++) S[c] += kr_sbop[q] * Wf(P, c, i, j, k + kl * (q - 1));
         auto dxy = [&](int c, int ax) {
            const int di = ax == 0, dj = ax == 1;
            return (ax == 0 ? sxi : syj) *
                   (d4a * (Wf(P, c, i + di, j + dj, k) - Wf(P, c, i - di, j - dj, k)) +
                    d4b * (Wf(P, c, i + 2 * di, j + 2 * dj, k) - Wf(P, c, i - 2 * di, j - 2 * dj, k)));
         };
         const double wx = dxy(2, 0), wy = dxy(2, 1), ux = dxy(0, 0), vy = dxy(1, 1);
         const double s0 = kr_sbop[0];
         const double ugh = (-S[0] - kl * wx) / s0, vgh = (-S[1] - kl * wy) / s0;
         const double V0 = Va(P, 0, i, j, k), V1 = Va(P, 1, i, j, k), V2 = Va(P, 2, i, j, k);
         gmc[0] += cof * kr_gh * (V0 * ugh + V1 * vgh - 2 * V2 * S[2] / s0);
         glc[0] += cof * kr_gh * V2 * (-(S[2] + kl * (ux + vy)) / s0);
      }
      // dz_of_inner: this column's rows, the coefficient on planes kq(q)
      {
         double Bv[3][8];
#pragma unroll
         for (int c = 0; c < 3; c++)
#pragma unroll
            for (int q = 0; q < 8; q++) Bv[c][q] = 0;
#pragma unroll 1
         for (int kk = 1; kk <= 6; kk++) {
            const int k = kq(kk);
            const double V0 = Va(P, 0, i, j, k), V1 = Va(P, 1, i, j, k), V2 = Va(P, 2, i, j, k);
#pragma unroll
            for (int q = 0; q < 8; q++) {
               const double w = wz(kk, q + 1);
               Bv[0][q] = fma(w, V0, Bv[0][q]);
               Bv[1][q] = fma(w, V1, Bv[1][q]);
               Bv[2][q] = fma(w, V2, Bv[2][q]);
            }
         }
#pragma unroll 1
         for (int q = 0; q < 8; q++) {
            const int k = kq(q + 1);
            double dx0 = 0, dx2 = 0, dy1 = 0, dy2 = 0;
#pragma unroll
            for (int e = -2; e <= 2; e++) {
               if (e == 0) continue;
               dx0 += DW[e + 2] * Wf(P, 0, i + e, j, k);
               dx2 += DW[e + 2] * Wf(P, 2, i + e, j, k);
               dy1 += DW[e + 2] * Wf(P, 1, i, j + e, k);
               dy2 += DW[e + 2] * Wf(P, 2, i, j + e, k);
            }
            gmc[q] += cof / 12 * (Bv[0][q] * sxi * dx2 + Bv[1][q] * syj * dy2);
            glc[q] += cof / 12 * Bv[2][q] * (sxi * dx0 + syj * dy1);
         }
      }
      // outer_of_dz: the rows along x and y whose outer difference reaches this column
#pragma unroll 1
      for (int kk = 1; kk <= 6; kk++) {
         const int k = kq(kk);
         double dz[3] = {0, 0, 0};
#pragma unroll
         for (int q = 1; q <= 8; q++) {
            const double w = wz(kk, q);
#pragma unroll
            for (int c = 0; c < 3; c++) dz[c] = fma(w, Wf(P, c, i, j, kq(q)), dz[c]);
         }
         double tx0 = 0, ty1 = 0, tx2 = 0, ty2 = 0;
#pragma unroll
         for (int e = -2; e <= 2; e++) {
            if (e == 0) continue;
            const double sxe = __ldg(g.sx + i - e - b.ib), sye = __ldg(g.sy + j - e - b.jb);
            tx0 += DW[e + 2] * sxe * Va(P, 0, i - e, j, k);
            tx2 += DW[e + 2] * sxe * Va(P, 2, i - e, j, k);
            ty1 += DW[e + 2] * sye * Va(P, 1, i, j - e, k);
            ty2 += DW[e + 2] * sye * Va(P, 2, i, j - e, k);
         }
         glc[kk - 1] += cof / 12 * dz[2] * (tx0 + ty1);
         gmc[kk - 1] += cof / 12 * (dz[0] * tx2 + dz[1] * ty2);
      }
   }
#pragma unroll
   for (int m = 0; m < 8; m++) {
      const long long p = pidx(b, i, j, kq(m + 1));
      g.gm[p] += gmc[m];
      g.gl[p] += glc[m];
   }
}

bool g_row_tables[64] = {false};

int upload_row_tables()
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess) return kCudaError;
   if (dev < 0 || dev >= 64) return kBadArgument;
   if (g_row_tables[dev]) return kOk;
   double acof[384], ghcof[6], bope[48], sbop[5];
   sbp_coefficients(acof, ghcof, bope, sbop);
   if (cudaMemcpyToSymbol(kr_acof, acof, sizeof(acof)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(kr_bope, bope, sizeof(bope)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(kr_sbop, sbop, sizeof(sbop)) != cudaSuccess) return kCudaError;
   if (cudaMemcpyToSymbol(kr_gh, &ghcof[0], sizeof(double)) != cudaSuccess) return kCudaError;
   g_row_tables[dev] = true;
   return kOk;
}

// g += scale * acc (FP64), acc = 0
__global__ void __launch_bounds__(256) grad_flush_kernel(long long n, float2* __restrict__ am,
                                                         float2* __restrict__ al, float2* __restrict__ ar,
                                                         const int* __restrict__ emax, int marg_a, int marg_f,
                                                         double kmu, double* __restrict__ gm,
                                                         double* __restrict__ gl, double* __restrict__ gr)
{
   const double sc = ldexp(1.0, shift_of(emax[0], marg_a) + shift_of(emax[1], marg_f));
   const double km = kmu * sc;
   for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
        q += (long long)gridDim.x * blockDim.x) {
      const float2 m = am[q], l = al[q], r = ar[q];
      gm[q] += km * ((double)m.x + (double)m.y);
      gl[q] += km * ((double)l.x + (double)l.y);
      gr[q] += sc * ((double)r.x + (double)r.y);
      am[q] = al[q] = ar[q] = make_float2(0.f, 0.f);
   }
}

template <class V>
void launch_df_kernel(const GradDF& g, dim3 grid, cudaStream_t s)
{
   const bool zm = g.zlo > -(1 << 28) || g.zhi < (1 << 28);
   if (g.sg6 && zm) grad_df_kernel<V, true, true><<<grid, kGradThreads, 0, s>>>(g);
   else if (g.sg6) grad_df_kernel<V, true, false><<<grid, kGradThreads, 0, s>>>(g);
   else if (zm) grad_df_kernel<V, false, true><<<grid, kGradThreads, 0, s>>>(g);
   else grad_df_kernel<V, false, false><<<grid, kGradThreads, 0, s>>>(g);
}

int grid_stride_blocks(long long n, int threads)
{
   long long b = (n + threads - 1) / threads;
   if (b > 152 * 16) b = 152 * 16;
   return (int)(b > 0 ? b : 1);
}

}  // namespace

int launch_grad_df_profiles(const GradDFProfiles& p, cudaStream_t s)
{
   for (int a = 0; a < 3; a++) {
      grad_profiles_kernel<<<blocks_for(p.n[a], 128), 128, 0, s>>>(p.n[a], p.st[a], p.co[a], p.dc[a], p.beta,
                                                                   p.st24[a], p.ist[a], p.cist[a], p.bdc[a],
                                                                   a == 2 ? p.hz : nullptr);
      SW4G_TRY(launch_status());
   }
   return kOk;
}

int launch_exp_max(const double* x, long long n, int* out, cudaStream_t s)
{
   exp_max_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(x, n, out);
   return launch_status();
}

int launch_inj_exp(const Box& b, const double* const st[3], int nrec, const int* ijk, const double* res,
                   long long rows, int nval, const double* rho, const double* hz, int* out, cudaStream_t s)
{
   if (nrec <= 0 || rows <= 0) return kOk;
   inj_exp_kernel<<<blocks_for(rows * nrec, 128), 128, 0, s>>>(b, st[0], st[1], st[2], nrec, ijk, res, rows,
                                                               nval, rho, hz, out);
   return launch_status();
}

int launch_grad_df_step(const GradDF& g, cudaStream_t s)
{
   const Box& b = g.b;
   const dim3 grid(blocks_for(b.nij, kGradThreads), b.ke - b.kb + 1);
   grad_prep_kernel<<<grid, kGradThreads, 0, s>>>(g);
   SW4G_TRY(launch_status());
   grad_edge_kernel<DF><<<grid, kGradThreads, 0, s>>>(g);
   SW4G_TRY(launch_status());
   launch_df_kernel<DF>(g, grid, s);
   return launch_status();
}

int launch_grad_f1_step(const GradDF& g, cudaStream_t s)
{
   const Box& b = g.b;
   const dim3 grid(blocks_for(b.nij, kGradThreads), b.ke - b.kb + 1);
   grad_prep_f1_kernel<<<grid, kGradThreads, 0, s>>>(g);
   SW4G_TRY(launch_status());
   grad_edge_kernel<F1><<<grid, kGradThreads, 0, s>>>(g);
   SW4G_TRY(launch_status());
   launch_df_kernel<F1>(g, grid, s);
   return launch_status();
}

int launch_grad_rows(const GradRows& g, cudaStream_t s)
{
   SW4G_TRY(upload_row_tables());
   const Box& b = g.b;
   const long long cols = (long long)(b.ie - b.ib - 3) * (b.je - b.jb - 3);
   if (cols <= 0) return kOk;
   const int nb = (int)((cols + kRowThreads - 1) / kRowThreads);
   if (g.lb1)
      grad_rows_kernel<true><<<nb, kRowThreads, 0, s>>>(g);
   else
      grad_rows_kernel<false><<<nb, kRowThreads, 0, s>>>(g);
   return launch_status();
}

int launch_grad_df_flush(const GradDF& g, double kmu, double* gm, double* gl, double* gr, cudaStream_t s)
{
   grad_flush_kernel<<<grid_stride_blocks(g.b.npts, 256), 256, 0, s>>>(
       g.b.npts, static_cast<float2*>(g.am), static_cast<float2*>(g.al), static_cast<float2*>(g.ar), g.emax,
       g.marg_a, g.marg_f, kmu, gm, gl, gr);
   return launch_status();
}

}  // namespace sw4g
