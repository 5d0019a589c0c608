// df64.cuh -- FP32-pair ("double-float") arithmetic for the FP64-accurate step on
// GB300's FP32 pipe.
//
// GB300 executes FP64 at 2 operations per clock per SM against 128 for FP32, so a
// stencil that needs FP64 accuracy runs faster as a few FP32 operations per FP64
// one.  A value is the unevaluated sum h + l of two floats (|l| <= ulp(h)/2 after
// renormalisation), about 49 significant bits, with float's exponent range.  The
// error-free transformations are the published ones:
//  * two_sum: Knuth, TAOCP vol. 2, 4.2.2 (Theorem B): s + e = a + b exactly, six
//    additions, no ordering condition;
//  * fast_two_sum: Dekker 1971 ("A floating-point technique for extending the
//    available precision"): s + e = a + b exactly when exponent(a) >= exponent(b);
//  * two_prod: with a fused multiply-add, e = fma(a, b, -p) is the exact error of
//    p = a * b (Ogita, Rump, Oishi 2005, "Accurate sum and dot product", Alg. 3.5);
// and the pair operations built from them follow Hida, Li, Bailey 2001 ("Algorithms
// for quad-double precision floating point arithmetic", the double-double "sloppy"
// addition and the FMA product).  Every float operation goes through an explicitly
// rounded intrinsic, so the compiler cannot contract a product into a following
// addition and break an error-free transformation.
//
// The header is also compiled by a host C++ compiler (without multiply-add
// contraction) to check the operations against long double on the CPU
// (tests/test_df64_host.py).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define DF_FN __host__ __device__ __forceinline__
#else
#define DF_FN inline
#endif

namespace fmf {
namespace df {

struct D {
  float h, l;
};

DF_FN float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DF_FN float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DF_FN float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
DF_FN float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}
DF_FN uint32_t fbits(float a) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(a);
#else
  uint32_t u;
  std::memcpy(&u, &a, 4);
  return u;
#endif
}
DF_FN float bitsf(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float a;
  std::memcpy(&a, &u, 4);
  return a;
#endif
}
// 2^k as a float, for -126 <= k <= 127
DF_FN float pow2f(int k) { return bitsf((uint32_t)(k + 127) << 23); }
// biased exponent field of a float (0: zero or subnormal)
DF_FN int fexp(float a) { return (int)((fbits(a) >> 23) & 0xffu); }

DF_FN D two_sum(float a, float b) {
  const float s = fadd(a, b);
  const float bb = fsub(s, a);
  const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
  return {s, e};
}
DF_FN D fast_two_sum(float a, float b) {
  const float s = fadd(a, b);
  return {s, fsub(b, fsub(s, a))};
}
DF_FN D neg(D x) { return {-x.h, -x.l}; }
// sloppy addition: absolute error below 2^-46 (|x| + |y|)
DF_FN D add(D x, D y) {
  const D s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, fadd(s.l, fadd(x.l, y.l)));
}
DF_FN D sub(D x, D y) { return add(x, neg(y)); }
// product (x.l y.l dropped): relative error below 2^-44 while the result and its
// low part are normal floats
DF_FN D mul(D x, D y) {
  const float p = fmul(x.h, y.h);
  float e = ffma(x.h, y.h, -p);
  e = ffma(x.h, y.l, e);
  e = ffma(x.l, y.h, e);
  return fast_two_sum(p, e);
}
// times a float (exact small integers such as 3, 7, 11 in the stencils)
DF_FN D mulf(D x, float f) {
  const float p = fmul(x.h, f);
  float e = ffma(x.h, f, -p);
  e = ffma(x.l, f, e);
  return fast_two_sum(p, e);
}
DF_FN D sqr(D x) {
  const float p = fmul(x.h, x.h);
  float e = ffma(x.h, x.h, -p);
  e = ffma(fadd(x.h, x.h), x.l, e);
  return fast_two_sum(p, e);
}
// times a power of two (exact while both parts stay normal floats)
DF_FN D scale(D x, float p2) { return {fmul(x.h, p2), fmul(x.l, p2)}; }

// float reciprocal to about one ulp: the hardware approximation refined by one
// Newton-Raphson step r + r (1 - d r) (on the host, the IEEE quotient)
DF_FN float recipf(float d) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
  const float e = ffma(-d, r, 1.0f);
  return ffma(r, e, r);
#else
  return 1.0f / d;
#endif
}
// n / d for a normal d: the float quotient q1 = n.h / d.h and one correction from
// the pair residual n - q1 d, relative error below 2^-43
DF_FN D div(D n, D d) {
  const float r = recipf(d.h);
  const float q1 = fmul(n.h, r);
  const D p = mulf(d, q1);  // q1 d
  // n - q1 d: n.h - p.h is exact (the two agree to a few ulps)
  const float rem = fsub(fadd(fsub(n.h, p.h), n.l), p.l);
  const float q2 = fmul(rem, r);
  return fast_two_sum(q1, q2);
}

// 1/sqrt(s) for a normal positive s: the float estimate r (hardware approximation
// and one Newton-Raphson step; on the host the IEEE value) corrected once with the
// pair residual, r + r (1 - s r^2) / 2, relative error below 2^-43
DF_FN float rsqrtf_(float s) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
  return fmul(r, ffma(fmul(-0.5f, s), fmul(r, r), 1.5f));
#else
  return 1.0f / __builtin_sqrtf(s);
#endif
}
DF_FN D rsqrt(D s) {
  const float r = rsqrtf_(s.h);
  const float rr = fmul(r, r);
  const D t = mul(s, D{rr, ffma(r, r, -rr)});  // s r^2 (r^2 exact as a pair)
  const float e = fsub(fsub(1.0f, t.h), t.l);
  return fast_two_sum(r, fmul(fmul(0.5f, r), e));
}

// The pair (h, l) of a double from its bits, without FP64 instructions: h is q's
// significand cut to float's 24 bits (toward zero), l the 29 bits below them as a
// float (rounded to 24), so h + l = q to 2^-48 of q while l is a normal float
// (|q| above about 2^-102; below that l is subnormal and adds up to 2^-150
// absolute).  Magnitudes below 2^-126 give (0, 0); above float's range +-inf (NaN
// for NaN) and l = 0.
DF_FN D split_double(double q) {
  uint64_t b;
#if defined(__CUDA_ARCH__)
  b = (uint64_t)__double_as_longlong(q);
#else
  std::memcpy(&b, &q, 8);
#endif
  const uint32_t hb = (uint32_t)(b >> 32);
  const uint32_t lb = (uint32_t)b;
  const int e = (int)((hb >> 20) & 0x7ffu);
  const uint32_t sg = hb & 0x80000000u;
  if (e < 897) return {bitsf(sg), bitsf(sg)};
  // beyond float's range: +-inf, NaN stays NaN (by bits: a double-to-float
  // conversion would take an FP64-pipe instruction on every call)
  if (e > 1150)
    return {bitsf(sg | (e == 2047 && ((hb & 0xfffffu) | lb) ? 0x7fc00000u : 0x7f800000u)), 0.0f};
  const float hi = bitsf(sg | ((uint32_t)(e - 896) << 23) | ((hb & 0xfffffu) << 3) | (lb >> 29));
  // q - hi = (low 29 bits) 2^(e - 1075), same sign as q.  The power of two is a
  // normal float for e >= 949; below that it is applied as 2^-64 2^(e - 1011)
  // L = the 29 low bits as a float, rounded once, without an integer-to-float
  // conversion (which GB300 issues on its FP64 pipe): the high 23 and low 6 bits
  // are exact floats by the 2^23 offset (2^23 + x has x in its significand for
  // x < 2^23), and one fused multiply-add joins them with a single rounding
  const uint32_t m29 = lb & 0x1fffffffu;
  const float fh = fsub(bitsf(0x4b000000u | (m29 >> 6)), 8388608.0f);
  const float fl = fsub(bitsf(0x4b000000u | (m29 & 63u)), 8388608.0f);
  const float L = ffma(fh, 64.0f, fl);
  const float lo = e >= 949 ? fmul(L, bitsf((uint32_t)(e - 948) << 23))
                            : fmul(fmul(L, 0x1p-64f), bitsf((uint32_t)(e - 884) << 23));
  return {hi, sg ? -lo : lo};
}

// A pair from a double, on the host (constants): h = (float)v, l = (float)(v - h)
DF_FN D from_double_host(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

#if defined(__CUDACC__)
// A float as a double from its bits, with integer operations only (a float-to-
// double conversion takes an FP64-pipe instruction), exactly: normal floats by
// their fields, a subnormal m 2^-149 normalised at its leading bit p
// (m 2^-149 = 1.f 2^(p - 149)), zeros, infinities and NaN as such.
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  const unsigned long long sg = (unsigned long long)(b & 0x80000000u) << 32;
  unsigned long long ed = e == 255 ? 2047ull : (unsigned long long)(e + 896);
  unsigned long long md = (unsigned long long)m << 29;
  if (e == 0) {
    const int p = 31 - __clz((int)m);  // -1 for m = 0
    ed = m ? (unsigned long long)(p + 874) : 0ull;
    md = m ? (((unsigned long long)m << (52 - p)) & 0xfffffffffffffull) : 0ull;
  }
  return __longlong_as_double((long long)(sg | (ed << 52) | md));
}
// a pair rounded to a double (one FP64 addition)
__device__ __forceinline__ double to_double(D a) { return f2d(a.h) + f2d(a.l); }
#endif

}  // namespace df
}  // namespace fmf
