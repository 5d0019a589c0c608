// recip.cuh -- reciprocal of a positive normal double without a division.
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

}  // namespace fmf
