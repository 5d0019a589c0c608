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

// The reverse of the FP64 WENO5 walk (the adjoint's k_weno_T1) in FP32 pairs: from
// the walk's five differences e = (a5, a3, a1, b1, b3) (pairs of the FP64
// differences), R of the FP64 walk, num/den, and (grad) dR/de.  With wdir_core's
// scaling (differences times 2^(127 - Eb), indicators s_k = n_k 2^(e_k - 127),
// X, Y, Z scaled by a common power of two, one below 2^-100 of the largest dropped,
// eps = 1e-80/486 in those units) R = 2^(Eb - 127) Q, Q = (X D1 + 6 Y D2 + 3 Z D3) /
// den, den = X + 6 Y + 3 Z, and dR/de = dQ/de' (R is homogeneous of degree 1 in the
// differences, eps scaled with them), from
//   dQ/dD1 = X/den, dQ/dD2 = 6Y/den, dQ/dD3 = 3Z/den,
//   dQ/ds1 = 2 (gY + gZ)/s1, dQ/ds2 = 2 (gX + gZ)/s2, dQ/ds3 = 2 (gX + gY)/s3,
//   gX = X (D1 - Q)/den, gY = 6 (Y - eps)(D2 - Q)/den, gZ = 3 Z (D3 - Q)/den
// (a product that holds s_k is quadratic in it, so dQ/ds_k is 0 where s_k is 0) and
// s_k = (13/3) t1^2 + t2^2.  Where the differences are below 2^-99, or eps outweighs
// every product by more than 2^100, eps alone weighs in the FP64 walk: R = D2 and
// dR/de its coefficients (0, -1, 5, 2, 0).
DF_FN void wrev_core(D a5, D a3, D a1, D b1, D b3, bool grad, D& R, D* g) {
  const D zero{0.0f, 0.0f};
  auto d2_only = [&](float sc) {
    R = scale(add(add(neg(a3), mulf(a1, 5.0f)), scale(b1, 2.0f)), sc);
    g[0] = zero;
    g[1] = D{-1.0f, 0.0f};
    g[2] = D{5.0f, 0.0f};
    g[3] = D{2.0f, 0.0f};
    g[4] = zero;
  };
  auto fa = [](float x) { return x < 0.0f ? -x : x; };
  auto fmx = [](float x, float y) { return x > y ? x : y; };
  const float m = fmx(fmx(fmx(fa(a5.h), fa(a3.h)), fmx(fa(a1.h), fa(b1.h))), fa(b3.h));
  const int Eb = fexp(m);
  if (Eb < 28) {
    d2_only(1.0f);
    return;
  }
  const float sc = pow2f(127 - Eb);
  a5 = scale(a5, sc);
  a3 = scale(a3, sc);
  a1 = scale(a1, sc);
  b1 = scale(b1, sc);
  b3 = scale(b3, sc);
  const float back = pow2f(Eb - 127);
  const D c13 = {(float)(13.0 / 3.0), (float)(13.0 / 3.0 - (double)(float)(13.0 / 3.0))};
  const D t1a = add(add(a5, a1), scale(a3, -2.0f)), t2a = add(add(a5, mulf(a1, 3.0f)), scale(a3, -4.0f));
  const D t1b = add(add(a3, b1), scale(a1, -2.0f)), t2b = sub(a3, b1);
  const D t1c = add(add(a1, b3), scale(b1, -2.0f)), t2c = add(add(b3, mulf(a1, 3.0f)), scale(b1, -4.0f));
  const D s1 = add(mul(sqr(t1a), c13), sqr(t2a));
  const D s2 = add(mul(sqr(t1b), c13), sqr(t2b));
  const D s3 = add(mul(sqr(t1c), c13), sqr(t2c));
  const D D1 = add(add(scale(a5, 2.0f), mulf(a3, -7.0f)), mulf(a1, 11.0f));
  const D D2 = add(add(neg(a3), mulf(a1, 5.0f)), scale(b1, 2.0f));
  const D D3 = add(add(scale(a1, 2.0f), mulf(b1, 5.0f)), neg(b3));
  const int e1 = fexp(s1.h), e2 = fexp(s2.h), e3 = fexp(s3.h);
  const D n1 = e1 ? scale(s1, pow2f(127 - e1)) : zero;
  const D n2 = e2 ? scale(s2, pow2f(127 - e2)) : zero;
  const D n3 = e3 ? scale(s3, pow2f(127 - e3)) : zero;
  const bool vx = e2 && e3, vy = e1 && e3, vz = e1 && e2;
  const int Px = e2 + e3, Py = e1 + e3, Pz = e1 + e2;
  int M = -100000;
  if (vx) M = Px;
  if (vy && Py > M) M = Py;
  if (vz && Pz > M) M = Pz;
  const int K = kEpsK - 8 * (Eb - 127) - 2 * (M - 254);
  if (M == -100000 || K > 100) {
    d2_only(back);
    return;
  }
  auto term = [&](bool v, int P, D na, D nb) {
    const int k2 = 2 * (P - M);
    if (!v || k2 < -100) return zero;
    return scale(sqr(mul(na, nb)), pow2f(k2));
  };
  const D Xh = term(vx, Px, n2, n3), Y0 = term(vy, Py, n1, n3), Zh = term(vz, Pz, n1, n2);
  D Yh = Y0;
  if (K >= -110) {
    const D em = {(float)kEpsMd, (float)(kEpsMd - (double)(float)kEpsMd)};
    Yh = add(Yh, scale(em, pow2f(K)));
  }
  const D Y6 = mulf(Yh, 6.0f), Z3 = mulf(Zh, 3.0f);
  const D iden = div(D{1.0f, 0.0f}, add(add(Xh, Y6), Z3));
  const D Q = mul(add(add(mul(Xh, D1), mul(Y6, D2)), mul(Z3, D3)), iden);
  R = scale(Q, back);
  if (!grad) return;
  const D qD1 = mul(Xh, iden), qD2 = mul(Y6, iden), qD3 = mul(Z3, iden);
  const D gX = mul(mul(Xh, sub(D1, Q)), iden), gY = mul(mul(mulf(Y0, 6.0f), sub(D2, Q)), iden),
          gZ = mul(mul(Z3, sub(D3, Q)), iden);
  // dQ/ds_k with s_k = n_k 2^(e_k - 127) (e_k <= 137: every scaled difference is below 2)
  auto dS = [&](int ek, D nk, D gsum) { return ek ? scale(div(scale(gsum, 2.0f), nk), pow2f(127 - ek)) : zero; };
  const D P1 = dS(e1, n1, add(gY, gZ)), P2 = dS(e2, n2, add(gX, gZ)), P3 = dS(e3, n3, add(gX, gY));
  const D c26 = {(float)(26.0 / 3.0), (float)(26.0 / 3.0 - (double)(float)(26.0 / 3.0))};
  const D lt1a = mul(mul(P1, c26), t1a), lt2a = mul(scale(P1, 2.0f), t2a);
  const D lt1b = mul(mul(P2, c26), t1b), lt2b = mul(scale(P2, 2.0f), t2b);
  const D lt1c = mul(mul(P3, c26), t1c), lt2c = mul(scale(P3, 2.0f), t2c);
  g[0] = add(add(lt1a, lt2a), scale(qD1, 2.0f));
  g[1] = add(add(add(scale(lt1a, -2.0f), scale(lt2a, -4.0f)), add(lt1b, lt2b)), add(mulf(qD1, -7.0f), neg(qD2)));
  g[2] = add(add(add(add(lt1a, mulf(lt2a, 3.0f)), add(scale(lt1b, -2.0f), lt1c)), mulf(lt2c, 3.0f)),
             add(add(mulf(qD1, 11.0f), mulf(qD2, 5.0f)), scale(qD3, 2.0f)));
  g[3] = add(add(sub(lt1b, lt2b), add(scale(lt1c, -2.0f), scale(lt2c, -4.0f))), add(scale(qD2, 2.0f), mulf(qD3, 5.0f)));
  g[4] = sub(add(lt1c, lt2c), qD3);
}

}  // namespace df
}  // namespace fmf
