// Double-float ("float-float") storage of the solution levels in the mixed form.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2,
// i.e. 48 significant bits.  The time-level accumulation
//   u^{n+1} = 2u^n - u^{n-1} + dt^2/rho (Lu + F)
// is carried out in this format with FP32 error-free transformations (Knuth's
// TwoSum and Dekker's FastTwoSum), so the accumulation keeps FP64-class precision
// while the stencil runs in FP32.  Components of a 3-component level are stored
// component-major: hi[c*npts + p], lo[c*npts + p] (lo = hi + 3*npts).
#pragma once

namespace sw4g {

// s + e == a + b exactly (Knuth TwoSum, 6 FP32 operations, no branch).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
   s = __fadd_rn(a, b);
   const float bb = __fsub_rn(s, a);
   e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e == a + b exactly when |a| >= |b| (Dekker FastTwoSum).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
   s = __fadd_rn(a, b);
   e = __fsub_rn(b, __fsub_rn(s, a));
}

// FP64 value -> (hi, lo).  Uses the FP64 pipe: only for O(N^2) work and set-up.
__device__ __forceinline__ void df_split(double v, float& h, float& l)
{
   h = __double2float_rn(v);
   l = __double2float_rn(v - (double)h);
}

__device__ __forceinline__ double df_value(float h, float l) { return (double)h + (double)l; }

}  // namespace sw4g
