// Device building blocks of the 4th-order SBP divergence-of-stress operator.
//
// The operator (src/rhs4sg_rev.C:44-864) is, per component,
//   Lu = (1/h^2) [ (1/6) sum_axes s_a (c_a u_x_a)_x_a          (variable-coefficient
//                                                              second differences)
//                + (1/144) sum_(a!=b) s_a s_b (c u_x_b)_x_a ]  (mixed differences)
// with c = mu or 2mu+lambda and s the supergrid stretching of each axis.  The
// helpers below evaluate those pieces on 5-point stencils; the kernels decide
// where the operands come from (global memory or shared memory).
#pragma once

namespace sw4g {

// Variable-coefficient second difference (a f')' on 5 points, times 6:
// a[0..4], f[0..4] are the coefficient and field at offsets -2..2.
template <typename R>
__device__ __forceinline__ R d2var(const R a[5], const R f[5])
{
   const R tf = R(0.75);
   const R wm2 = a[1] - tf * (a[2] + a[0]);
   const R wm1 = a[0] + a[3] + R(3) * (a[2] + a[1]);
   const R wp1 = a[1] + a[4] + R(3) * (a[3] + a[2]);
   const R wp2 = a[3] - tf * (a[2] + a[4]);
   return wm2 * (f[0] - f[2]) + wm1 * (f[1] - f[2]) + wp1 * (f[3] - f[2]) + wp2 * (f[4] - f[2]);
}

// 12h times the centred 4th-order first difference from values at -2,-1,+1,+2.
template <typename R>
__device__ __forceinline__ R d1c(R fm2, R fm1, R fp1, R fp2)
{
   return (fm2 - fp2) + R(8) * (fp1 - fm1);
}

// x != 0.0 for every double x (true for NaN, false for -0.0), tested on the bit pattern
// by the integer pipe: FP64-pipe-bound kernels keep their FP64 issue slots for the
// arithmetic.
__device__ __forceinline__ bool nonzero_bits(double x)
{
   return (__double_as_longlong(x) & 0x7fffffffffffffffLL) != 0;
}

}  // namespace sw4g
