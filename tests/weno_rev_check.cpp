// Host check of the FP32-pair WENO5 reverse core (csrc/weno5_df.cuh's wrev_core)
// against the FP64 reverse's formulas evaluated in long double (the forward walk
// R = num/den of the stencil's five differences and its gradient dR/de, as the
// adjoint's k_weno_T1 forms them: weno5.h's smoothness indicators and weights with
// the reference's additive 1e-80).  Stencils of six doubles in several regimes:
// smooth waves over magnitudes 1e-12 .. 1e10, small variations on a large mean,
// exactly linear and constant runs, jumps, random noise, values near the flat
// limit.  The differences are taken in double, as the device does.  Built by
// tests/test_df64_host.py with g++ -O2 -ffp-contract=off; prints per regime
// the worst error of R (over the largest |difference|) and of the gradient (over its
// largest entry), of the pair core and then of the same walk in double, and last
// the worst error of the forward pair core wdir_core (see there).
#include <cmath>
#include <cstdio>
#include <random>

#include "weno5_df.cuh"

using fmf::df::D;
using LD = long double;

static LD val(D x) { return (LD)x.h + (LD)x.l; }

// the FP64 walk in long double: R and dR/d(a5, a3, a1, b1, b3)
static void walk_ld(const LD* e, LD& R, LD* g) {
  const LD a5 = e[0], a3 = e[1], a1 = e[2], b1 = e[3], b3 = e[4];
  const LD c13 = 13.0L / 3.0L;
  const LD t1a = a5 + a1 - 2 * a3, t2a = a5 + 3 * a1 - 4 * a3;
  const LD t1b = a3 + b1 - 2 * a1, t2b = a3 - b1;
  const LD t1c = a1 + b3 - 2 * b1, t2c = b3 + 3 * a1 - 4 * b1;
  const LD s1 = c13 * t1a * t1a + t2a * t2a, s2 = c13 * t1b * t1b + t2b * t2b, s3 = c13 * t1c * t1c + t2c * t2c;
  const LD x = s2 * s3, y = s1 * s3, z = s1 * s2;
  const LD X = x * x, Y = y * y + 1.0e-80L / 486.0L, Z = z * z;
  const LD D1 = a1 * 11.0L / 6.0L - a3 * 7.0L / 6.0L + a5 / 3.0L;
  const LD d2 = 2 * b1 + 5 * a1 - a3;
  const LD D3 = 2.5L * b1 - 0.5L * b3 + a1;
  const LD den = X / 6 + Y + Z / 2;
  R = (X * D1 + Y * d2 + Z * D3) / den;
  const LD g4 = 4 / den;
  const LD lD1 = g4 * X, ld2 = g4 * Y, lD3 = g4 * Z;
  const LD lX = g4 * (D1 - R / 6), lY = g4 * (d2 - R), lZ = g4 * (D3 - R / 2);
  const LD lx = x * lX, ly = y * lY, lz = z * lZ;
  const LD S1 = ly * s3 + lz * s2, S2 = lx * s3 + lz * s1, S3 = lx * s2 + ly * s1;
  const LD lt1a = t1a * c13 * S1, lt2a = t2a * S1, lt1b = t1b * c13 * S2, lt2b = t2b * S2;
  const LD lt1c = t1c * c13 * S3, lt2c = t2c * S3;
  g[0] = lD1 / 12 + lt1a + lt2a;
  g[1] = -lD1 * 7 / 24 - ld2 / 4 - 2 * lt1a - 4 * lt2a + lt1b + lt2b;
  g[2] = lD1 * 11 / 24 + ld2 * 1.25L + lD3 / 4 + 3 * lt2a - 2 * lt1b + 3 * lt2c + lt1a + lt1c;
  g[3] = ld2 / 2 + lD3 * 0.625L - 2 * lt1c - 4 * lt2c + lt1b - lt2b;
  g[4] = -lD3 / 8 + lt1c + lt2c;
}

// the same walk in double, in the adjoint kernel's operation order (its fused
// multiply-adds written as fma, the reciprocal as a quotient): the FP64 reverse's
// own error, for comparison
static void walk_d(const double* e, double& R, double* g) {
  const double a5 = e[0], a3 = e[1], a1 = e[2], b1 = e[3], b3 = e[4];
  constexpr double c13 = 13.0 / 3.0;
  const double t1a = std::fma(a3, -2.0, a5 + a1), t2a = std::fma(a3, -4.0, std::fma(a1, 3.0, a5));
  const double t1b = std::fma(a1, -2.0, a3 + b1), t2b = a3 - b1;
  const double t1c = std::fma(b1, -2.0, a1 + b3), t2c = std::fma(b1, -4.0, std::fma(a1, 3.0, b3));
  const double s1 = std::fma(t1a * c13, t1a, t2a * t2a), s2 = std::fma(t1b * c13, t1b, t2b * t2b),
               s3 = std::fma(t1c * c13, t1c, t2c * t2c);
  const double x = s2 * s3, y = s1 * s3, z = s1 * s2;
  const double X = x * x, Y = std::fma(y, y, 1.0e-80 / 486.0), Z = z * z;
  const double D1 = std::fma(a1, 11.0 / 6.0, std::fma(a3, -7.0 / 6.0, a5 * (1.0 / 3.0)));
  const double d2 = std::fma(b1, 2.0, std::fma(a1, 5.0, -a3));
  const double D3 = std::fma(b1, 2.5, std::fma(b3, -0.5, a1));
  const double num = std::fma(Z, D3, std::fma(Y, d2, X * D1));
  const double iD = 1.0 / std::fma(X, 1.0 / 6.0, std::fma(Z, 0.5, Y));
  R = num * iD;
  const double g4 = 4.0 * iD;
  const double lD1 = g4 * X, ld2 = g4 * Y, lD3 = g4 * Z;
  const double lX = g4 * std::fma(R, -1.0 / 6.0, D1), lY = g4 * (d2 - R), lZ = g4 * std::fma(R, -0.5, D3);
  const double lx = x * lX, ly = y * lY, lz = z * lZ;
  const double S1 = std::fma(ly, s3, lz * s2), S2 = std::fma(lx, s3, lz * s1), S3 = std::fma(lx, s2, ly * s1);
  const double lt1a = (t1a * c13) * S1, lt2a = t2a * S1, lt1b = (t1b * c13) * S2, lt2b = t2b * S2;
  const double lt1c = (t1c * c13) * S3, lt2c = t2c * S3;
  g[0] = std::fma(lD1, 1.0 / 12.0, lt1a + lt2a);
  g[1] = std::fma(lD1, -7.0 / 24.0, std::fma(ld2, -0.25, std::fma(lt1a, -2.0, std::fma(lt2a, -4.0, lt1b + lt2b))));
  g[2] = std::fma(lD1, 11.0 / 24.0,
                  std::fma(ld2, 1.25, std::fma(lD3, 0.25, std::fma(lt2a, 3.0, std::fma(lt1b, -2.0,
                                                                                  std::fma(lt2c, 3.0, lt1a + lt1c))))));
  g[3] = std::fma(ld2, 0.5, std::fma(lD3, 0.625, std::fma(lt1c, -2.0, std::fma(lt2c, -4.0, lt1b - lt2b))));
  g[4] = std::fma(lD3, -0.125, lt1c + lt2c);
}

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const char* names[] = {"smooth", "offset", "linear", "jump", "noise", "tiny"};
  for (int regime = 0; regime < 6; ++regime) {
    double worst_r = 0, worst_g = 0, worst_r64 = 0, worst_g64 = 0, worst_f = 0;
    for (int t = 0; t < 40000; ++t) {
      double q[6];
      const double mag = std::pow(10.0, std::uniform_int_distribution<int>(-12, 10)(rng));
      const double w = 0.05 + 0.6 * std::fabs(U(rng)), ph = 3.0 * U(rng);
      for (int k = 0; k < 6; ++k) {
        switch (regime) {
          case 0: q[k] = mag * std::sin(w * k + ph); break;
          case 1: q[k] = mag * (1.0 + 1e-7 * std::sin(w * k + ph)); break;
          case 2: q[k] = (t % 3 == 0) ? mag : mag * (0.25 + 0.5 * k); break;  // constant or linear
          case 3: q[k] = mag * ((k + (t % 5)) >= 4 ? 1.0 : 0.0) + mag * 1e-3 * std::sin(w * k); break;
          case 4: q[k] = mag * U(rng); break;
          default: q[k] = 1e-28 * std::pow(10.0, -3.0 * std::fabs(U(rng))) * std::sin(w * k + ph); break;
        }
      }
      double e[5];
      for (int k = 0; k < 5; ++k) e[k] = q[k + 1] - q[k];
      LD el[5], Rl, gl[5];
      for (int k = 0; k < 5; ++k) el[k] = e[k];
      walk_ld(el, Rl, gl);
      D R, g[5];
      fmf::df::wrev_core(fmf::df::split_double(e[0]), fmf::df::split_double(e[1]), fmf::df::split_double(e[2]),
                         fmf::df::split_double(e[3]), fmf::df::split_double(e[4]), true, R, g);
      LD emax = 0, gmax = 0;
      for (int k = 0; k < 5; ++k) {
        emax = std::fmax(emax, std::fabs(el[k]));
        gmax = std::fmax(gmax, std::fabs(gl[k]));
      }
      if (emax > 0) worst_r = std::fmax(worst_r, (double)(std::fabs(val(R) - Rl) / emax));
      else if (val(R) != 0) worst_r = 1e30;
      LD ge = 0;
      for (int k = 0; k < 5; ++k) ge = std::fmax(ge, std::fabs(val(g[k]) - gl[k]));
      if (!std::isfinite((double)val(R))) worst_r = 1e30;
      for (int k = 0; k < 5; ++k)
        if (!std::isfinite((double)val(g[k]))) ge = 1e30;
      worst_g = std::fmax(worst_g, (double)(gmax > 0 ? ge / gmax : ge));
      // the forward pair core (the FP64-accurate step's WENO5) on the split values
      // themselves (vsum = 4 > 0: the walk from q[0], kx = 1, so it returns 4 R): its
      // differences are taken between split values, each within 2^-48 of its double,
      // and below 2^-99 it returns 0 (the FP64 walk: D2), so its error is taken over
      // 1e-12 of the largest difference + 4e-13 of the largest value + 2^-94
      {
        D w[6];
        LD qmax = 0;
        for (int k = 0; k < 6; ++k) {
          w[k] = fmf::df::split_double(q[k]);
          qmax = std::fmax(qmax, std::fabs((LD)q[k]));
        }
        const D f = fmf::df::wdir_core(w, D{4.0f, 0.0f}, D{1.0f, 0.0f});
        const LD scale = 1e-12L * emax + 4e-13L * qmax + std::ldexp((LD)1, -94);
        if (scale > 0) worst_f = std::fmax(worst_f, (double)(std::fabs(val(f) / 4 - Rl) / scale));
        if (!std::isfinite((double)val(f))) worst_f = 1e30;
      }
      double R64, g64[5];
      walk_d(e, R64, g64);
      if (emax > 0) worst_r64 = std::fmax(worst_r64, (double)(std::fabs((LD)R64 - Rl) / emax));
      LD ge64 = 0;
      for (int k = 0; k < 5; ++k) ge64 = std::fmax(ge64, std::fabs((LD)g64[k] - gl[k]));
      worst_g64 = std::fmax(worst_g64, (double)(gmax > 0 ? ge64 / gmax : ge64));
    }
    std::printf("%s %.3g %.3g %.3g %.3g %.3g\n", names[regime], worst_r, worst_g, worst_r64, worst_g64, worst_f);
  }
  return 0;
}
