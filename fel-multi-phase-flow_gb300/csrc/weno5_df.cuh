// weno5_df.cuh -- one directional WENO5 derivative of weno5.h:2-70 (times dxi) in
// FP32-pair arithmetic, for the FP64-accurate step (precision FMF_FP64E).
//
// Same quotient as the FP64 kernel's (the upwind side only, walked from its upwind
// end; weights m1 = (s2 s3)^2, m2 = 6 (s1 s3)^2, m3 = 3 (s1 s2)^2 and the additive
// 1e-80 of the reference):
//   Q = (X D1 + 6 Y D2 + 3 Z D3) / (X + 6 Y + 3 Z),  X = (s2 s3)^2, Y = (s1 s3)^2
//       + 1e-80/486, Z = (s1 s2)^2,  s_k = the reference's smoothness / 3,
//   D1 = 2 a5 - 7 a3 + 11 a1,  D2 = -a3 + 5 a1 + 2 b1,  D3 = 2 a1 + 5 b1 - b3,
//   result = |vsum| dxi/24 Q,
// which is the FP64 kernel's num/den with both multiplied by 6.  The weights scale
// like the 8th power of the differences, far outside float's exponent range, so
// the evaluation carries exponents explicitly, exactly (powers of two only):
//  * the five differences are multiplied by 2^-E', E' the exponent of the largest
//    (so the largest is in [1, 2)); Q is linear in them and is multiplied back;
//  * each s_k is split into a significand pair in [1, 2) and its exponent; X, Y, Z
//    are formed from the significands and scaled by 2^(2 (P - M)), P the exponent
//    sum of the pair of s that forms them and M the largest P, so the largest of
//    X, Y, Z is in [1, 16) and one below 2^-100 of it is dropped (its weight is
//    then below 2^-96);
//  * the reference's 1e-80/486 in these units is m_eps 2^(k_eps - 8 E' - 2 M):
//    added where that exponent is in [-110, 100], dropped below, and above it the
//    quotient is D2 (the other terms are then below 2^-96 of it), as it is where
//    every product is zero.
// A smoothness indicator below float's normal range (2^-126 in the scaled units:
// differences that agree to better than 2^-63 of the largest) counts as 0;
// differences all below 2^-99 give 0, as a zero velocity does.
#pragma once

#include "df64.cuh"

namespace fmf {
namespace df {

// b - a of two split pairs
DF_FN D pair_diff(D b, D a) {
  const D s = two_sum(b.h, -a.h);
  return fast_two_sum(s.h, fadd(s.l, fsub(b.l, a.l)));
}

// 1e-80/486 = kEpsM 2^kEpsK, kEpsM in [1, 2) as a pair
constexpr int kEpsK = -275;
constexpr double kEpsMd = 1.0e-80 / 486.0 * 0x1p275;

// q[0..5]: the stencil from its upwind end; vsum (nonzero) = 4 times the
// reference's vel; kx = dxi/24.  Returns the derivative term of weno5.h for this
// direction.
DF_FN D wdir_core(const D* q, D vsum, D kx) {
  D a5 = pair_diff(q[1], q[0]), a3 = pair_diff(q[2], q[1]), a1 = pair_diff(q[3], q[2]);
  D b1 = pair_diff(q[4], q[3]), b3 = pair_diff(q[5], q[4]);
  auto fa = [](float x) { return x < 0.0f ? -x : x; };
  auto fmx = [](float x, float y) { return x > y ? x : y; };
  const float m = fmx(fmx(fmx(fa(a5.h), fa(a3.h)), fmx(fa(a1.h), fa(b1.h))), fa(b3.h));
  const int Eb = fexp(m);
  if (Eb < 28) return {0.0f, 0.0f};
  const float sc = pow2f(127 - Eb);
  a5 = scale(a5, sc);
  a3 = scale(a3, sc);
  a1 = scale(a1, sc);
  b1 = scale(b1, sc);
  b3 = scale(b3, sc);
  const D c13 = {(float)(13.0 / 3.0), (float)(13.0 / 3.0 - (double)(float)(13.0 / 3.0))};
  // s/3 = (13/3) t1^2 + t2^2 (weno5.h's 13 t1^2 + 3 t2^2)
  D t1 = add(add(a5, a1), scale(a3, -2.0f));
  D t2 = add(add(a5, mulf(a1, 3.0f)), scale(a3, -4.0f));
  const D s1 = add(mul(sqr(t1), c13), sqr(t2));
  t1 = add(add(a3, b1), scale(a1, -2.0f));
  t2 = sub(a3, b1);
  const D s2 = add(mul(sqr(t1), c13), sqr(t2));
  t1 = add(add(a1, b3), scale(b1, -2.0f));
  t2 = add(add(b3, mulf(a1, 3.0f)), scale(b1, -4.0f));
  const D s3 = add(mul(sqr(t1), c13), sqr(t2));
  const D D1 = add(add(scale(a5, 2.0f), mulf(a3, -7.0f)), mulf(a1, 11.0f));
  const D D2 = add(add(neg(a3), mulf(a1, 5.0f)), scale(b1, 2.0f));
  const D D3 = add(add(scale(a1, 2.0f), mulf(b1, 5.0f)), neg(b3));
  // significands and exponents of the indicators
  const int e1 = fexp(s1.h), e2 = fexp(s2.h), e3 = fexp(s3.h);
  const D n1 = e1 ? scale(s1, pow2f(127 - e1)) : D{0.0f, 0.0f};
  const D n2 = e2 ? scale(s2, pow2f(127 - e2)) : D{0.0f, 0.0f};
  const D n3 = e3 ? scale(s3, pow2f(127 - e3)) : D{0.0f, 0.0f};
  const bool vx = e2 && e3, vy = e1 && e3, vz = e1 && e2;
  const int Px = e2 + e3, Py = e1 + e3, Pz = e1 + e2;
  int M = -100000;
  if (vx) M = Px;
  if (vy && Py > M) M = Py;
  if (vz && Pz > M) M = Pz;
  // the additive term's exponent in these units (biased exponents: s_k = n_k 2^(e_k - 127))
  const int K = kEpsK - 8 * (Eb - 127) - 2 * (M - 254);
  D Q;
  if (M == -100000 || K > 100) {
    Q = D2;
  } else {
    auto term = [&](bool v, int P, D na, D nb) {
      const int k2 = 2 * (P - M);
      if (!v || k2 < -100) return D{0.0f, 0.0f};
      return scale(sqr(mul(na, nb)), pow2f(k2));
    };
    const D Xh = term(vx, Px, n2, n3);
    D Yh = term(vy, Py, n1, n3);
    const D Zh = term(vz, Pz, n1, n2);
    if (K >= -110) {
      const D em = {(float)kEpsMd, (float)(kEpsMd - (double)(float)kEpsMd)};
      Yh = add(Yh, scale(em, pow2f(K)));
    }
    const D Y6 = mulf(Yh, 6.0f), Z3 = mulf(Zh, 3.0f);
    const D num = add(add(mul(Xh, D1), mul(Y6, D2)), mul(Z3, D3));
    const D den = add(add(Xh, Y6), Z3);
    Q = div(num, den);
  }
  const D va = vsum.h < 0.0f ? neg(vsum) : vsum;
  return scale(mul(mul(va, kx), Q), pow2f(Eb - 127));
}

}  // namespace df
}  // namespace fmf
