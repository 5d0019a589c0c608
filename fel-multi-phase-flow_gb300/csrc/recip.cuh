// recip.cuh -- reciprocal and reciprocal square root of a positive normal double
// without a division or a square root.
#pragma once

namespace fmf {

// The Newton-Raphson iteration for 1/x, r <- r + r (1 - x r), doubles the number
// of correct bits per step (P. Markstein, IBM J. Res. Develop. 34 (1990) 111-119);
// it starts here from the PTX approximate reciprocal rcp.approx.ftz.f64, and two
// steps reach double precision.  Inputs must be positive normal numbers (no
// subnormals, zero, infinity or NaN).  fmf_check_reciprocal measures its error
// against the IEEE quotient 1.0 / x.
__device__ __forceinline__ double recip_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  r = fma(r, fma(-x, r, 1.0), r);
  return fma(r, fma(-x, r, 1.0), r);
}

// 1/sqrt(s): Newton-Raphson on f(y) = y^-2 - s, y <- y (3 - s y^2)/2, whose
// relative error squares per step, seeded with the PTX approximate reciprocal
// square root rsqrt.approx.ftz.f64; two steps reach FP64 rounding.  Seven FP64
// operations instead of a square root and a division.  Inputs: positive normal
// numbers.  fmf_check_rsqrt measures its error against 1.0 / sqrt(s).
__device__ __forceinline__ double rsqrt_nr(double s) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(s));
  const double h = 0.5 * s;
#pragma unroll
  for (int it = 0; it < 2; ++it) y = y * fma(-h * y, y, 1.5);
  return y;
}

}  // namespace fmf
