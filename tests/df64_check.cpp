// Host check of the FP32-pair arithmetic (fel-multi-phase-flow_gb300/csrc/df64.cuh)
// against long double: every pair operation on seeded inputs over many binades,
// and the bit-level split of a double into a pair.  Built by
// tests/test_df64_host.py with g++ -O2 -ffp-contract=off (no contraction of a
// product into an addition, which would break the error-free transformations);
// prints one line "name worst_error" per operation, each error in units of 2^-48
// of the operation's scale (|q| for the split, |x| + |y| for the addition, the
// exact result's magnitude for the others).
#include <cmath>
#include <cstdio>
#include <random>

#include "df64.cuh"

using fmf::df::D;
using LD = long double;

static LD val(D x) { return (LD)x.h + (LD)x.l; }

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> unit(-1.0, 1.0);
  // q = m 2^e with 1/2 <= |m| < 1: the pair format has float's exponent range,
  // so inputs stay within 2^+-30 where every product, quotient and low part is a
  // normal float (the stencils' values, differences and weights lie there too)
  auto rnd = [&](int lo, int hi) {
    std::uniform_int_distribution<int> e(lo, hi);
    double m = unit(rng);
    m = std::copysign(0.5 + 0.5 * std::fabs(m), m);
    return std::ldexp(m, e(rng));
  };
  const LD two48 = std::ldexp((LD)1, -48);
  double w_split = 0, w_add = 0, w_mul = 0, w_mulf = 0, w_sqr = 0, w_div = 0, w_rsqrt = 0, w_small = 0;
  const int N = 200000;
  for (int t = 0; t < N; ++t) {
    const double a = rnd(-30, 30), b = rnd(-30, 30);
    const D x = fmf::df::split_double(a), y = fmf::df::split_double(b);
    // split: h + l = q to 2^-48 of q
    w_split = std::fmax(w_split, (double)(std::fabs(val(x) - (LD)a) / (two48 * std::fabs((LD)a))));
    // sloppy addition: absolute, against |x| + |y|
    {
      const LD e = std::fabs(val(fmf::df::add(x, y)) - (val(x) + val(y)));
      w_add = std::fmax(w_add, (double)(e / (two48 * (std::fabs(val(x)) + std::fabs(val(y))))));
    }
    // products: relative
    {
      const LD p = val(x) * val(y);
      w_mul = std::fmax(w_mul, (double)(std::fabs(val(fmf::df::mul(x, y)) - p) / (two48 * std::fabs(p))));
      const float f = (float)(std::uniform_int_distribution<int>(1, 64)(rng));
      const LD q = val(x) * (LD)f;
      w_mulf = std::fmax(w_mulf, (double)(std::fabs(val(fmf::df::mulf(x, f)) - q) / (two48 * std::fabs(q))));
      const LD s = val(x) * val(x);
      w_sqr = std::fmax(w_sqr, (double)(std::fabs(val(fmf::df::sqr(x)) - s) / (two48 * s)));
    }
    // quotient and reciprocal square root: relative
    {
      const LD q = val(x) / val(y);
      w_div = std::fmax(w_div, (double)(std::fabs(val(fmf::df::div(x, y)) - q) / (two48 * std::fabs(q))));
      const D ax = {std::fabs(x.h), x.h < 0 ? -x.l : x.l};
      const LD r = 1.0L / std::sqrt(val(ax));
      w_rsqrt = std::fmax(w_rsqrt, (double)(std::fabs(val(fmf::df::rsqrt(ax)) - r) / (two48 * r)));
    }
  }
  // split below about 2^-97 (l subnormal): the pair holds q to 2^-48 of q plus
  // l's rounding to float's subnormal grid, 2^-150 absolute (bound taken as
  // 2^-48 |q| + 2^-149); below 2^-126 it is (0, 0)
  for (int t = 0; t < N; ++t) {
    const double a = rnd(-140, -96);
    const D x = fmf::df::split_double(a);
    if (std::fabs(a) < std::ldexp(1.0, -126)) {
      if (x.h != 0.0f || x.l != 0.0f) w_small = 1e30;
      continue;
    }
    w_small = std::fmax(w_small, (double)(std::fabs(val(x) - (LD)a) /
                                          (two48 * std::fabs((LD)a) + std::ldexp((LD)1, -149))));
  }
  // beyond float's range: +-inf with l = 0, NaN stays NaN
  int special_ok = 1;
  {
    const D p = fmf::df::split_double(std::ldexp(1.5, 130)), n = fmf::df::split_double(-std::ldexp(1.5, 200));
    const D z = fmf::df::split_double(NAN), zero = fmf::df::split_double(-0.0);
    special_ok &= std::isinf(p.h) && p.h > 0 && p.l == 0.0f;
    special_ok &= std::isinf(n.h) && n.h < 0 && n.l == 0.0f;
    special_ok &= std::isnan(z.h);
    special_ok &= zero.h == 0.0f && std::signbit(zero.h) && zero.l == 0.0f;
    // the largest double below 2^128: h is its significand cut to 24 bits, finite
    const D top = fmf::df::split_double(std::nextafter(std::ldexp(1.0, 128), 0.0));
    special_ok &= std::isfinite(top.h) && top.h == 3.4028234663852886e38f;
  }
  std::printf("split %.6g\nadd %.6g\nmul %.6g\nmulf %.6g\nsqr %.6g\ndiv %.6g\nrsqrt %.6g\nsplit_small %.6g\n"
              "special %d\n",
              w_split, w_add, w_mul, w_mulf, w_sqr, w_div, w_rsqrt, w_small, special_ok);
  return 0;
}
