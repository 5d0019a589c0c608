// adj_mom.cu -- adjoints of the WENO5 advection (cal_advu_weno5 + weno5.h) and of
// the CSF surface-tension force (cal_grad_p2a, calrn x4, calrkap, cal_grad_p2uvw,
// calfst).
#include "adj.cuh"
#include "fused.cuh"
#include "ops.cuh"
#include "recip.cuh"
#include "weno5_df.cuh"

namespace fmf {
namespace adj {

namespace {
// The forward derivative is fused_weno.cu's wdir: the five differences e taken
// walking from the upwind end of the stencil, and R(e) = num / den with
//   s_k/3 = (13/3) t1^2 + t2^2,  x = s2 s3, y = s1 s3, z = s1 s2,
//   X = x^2, Y = y^2 + 1e-80/486, Z = z^2,
//   num = X D1 + Y d2 + Z D3,  den = X/6 + Y + Z/2
// (D1 = d1/6, D3 = d3/2 of weno5.h), out += |vel|/6 * di * R(e).  Walk holds the
// forward quantities the reverse sweep reuses.
struct Walk {
  double t1a, t2a, t1b, t2b, t1c, t2c, s1, s2, s3, x, y, z, X, Y, Z, D1, d2, D3, iD, R;
};
__device__ __forceinline__ void walk_fwd(const double* __restrict__ q, long c, long st, Walk& W) {
  const double* p = q + c - 3 * st;
  const double q0 = p[0], q1 = p[st], q2 = p[2 * st], q3 = p[3 * st], q4 = p[4 * st], q5 = p[5 * st];
  const double a5 = q1 - q0, a3 = q2 - q1, a1 = q3 - q2, b1 = q4 - q3, b3 = q5 - q4;
  constexpr double c13 = 13.0 / 3.0;
  W.t1a = fma(a3, -2.0, a5 + a1);
  W.t2a = fma(a3, -4.0, fma(a1, 3.0, a5));
  W.t1b = fma(a1, -2.0, a3 + b1);
  W.t2b = a3 - b1;
  W.t1c = fma(b1, -2.0, a1 + b3);
  W.t2c = fma(b1, -4.0, fma(a1, 3.0, b3));
  W.s1 = fma(W.t1a * c13, W.t1a, W.t2a * W.t2a);
  W.s2 = fma(W.t1b * c13, W.t1b, W.t2b * W.t2b);
  W.s3 = fma(W.t1c * c13, W.t1c, W.t2c * W.t2c);
  W.x = W.s2 * W.s3;
  W.y = W.s1 * W.s3;
  W.z = W.s1 * W.s2;
  W.X = W.x * W.x;
  W.Y = fma(W.y, W.y, 1.0e-80 / 486.0);
  W.Z = W.z * W.z;
  W.D1 = fma(a1, 11.0 / 6.0, fma(a3, -7.0 / 6.0, a5 * (1.0 / 3.0)));
  W.d2 = fma(b1, 2.0, fma(a1, 5.0, -a3));
  W.D3 = fma(b1, 2.5, fma(b3, -0.5, a1));
  const double num = fma(W.Z, W.D3, fma(W.Y, W.d2, W.X * W.D1));
  W.iD = recip_nr(fma(W.X, 1.0 / 6.0, fma(W.Z, 0.5, W.Y)));
  W.R = num * W.iD;
}
// la[0..4] = lR dR/d(e) given g4 = 4 lR / den (lR the adjoint of R).  The factor
// 4 stands for the two factors 2 of d(x^2) = 2x dx and d(t^2) = 2t dt, so the
// smoothness-indicator terms need no constants; the terms through D1, d2, D3
// divide it out in their coefficients.
__device__ __forceinline__ void walk_rev(const Walk& W, double g4, double* la) {
  constexpr double c13 = 13.0 / 3.0;
  const double lD1 = g4 * W.X, ld2 = g4 * W.Y, lD3 = g4 * W.Z;  // 4 lR dR/d(D1, d2, D3)
  const double lX = g4 * fma(W.R, -1.0 / 6.0, W.D1), lY = g4 * (W.d2 - W.R), lZ = g4 * fma(W.R, -0.5, W.D3);
  const double lx = W.x * lX, ly = W.y * lY, lz = W.z * lZ;
  const double S1 = fma(ly, W.s3, lz * W.s2), S2 = fma(lx, W.s3, lz * W.s1), S3 = fma(lx, W.s2, ly * W.s1);
  // (t1 c13) is the forward's own product in s = fma(t1 c13, t1, t2^2)
  const double lt1a = (W.t1a * c13) * S1, lt2a = W.t2a * S1;
  const double lt1b = (W.t1b * c13) * S2, lt2b = W.t2b * S2;
  const double lt1c = (W.t1c * c13) * S3, lt2c = W.t2c * S3;
  la[0] = fma(lD1, 1.0 / 12.0, lt1a + lt2a);
  la[1] = fma(lD1, -7.0 / 24.0, fma(ld2, -0.25, fma(lt1a, -2.0, fma(lt2a, -4.0, lt1b + lt2b))));
  la[2] = fma(lD1, 11.0 / 24.0,
              fma(ld2, 1.25, fma(lD3, 0.25, fma(lt2a, 3.0, fma(lt1b, -2.0, fma(lt2c, 3.0, lt1a + lt1c))))));
  la[3] = fma(ld2, 0.5, fma(lD3, 0.625, fma(lt1c, -2.0, fma(lt2c, -4.0, lt1b - lt2b))));
  la[4] = fma(lD3, -0.125, lt1c + lt2c);
}
// adjoint of  out += wdir(q, c, S, 4 vel, di/24)  given lout: lD[0..5] = the
// adjoints of the six differences (dm5, dm3, dm1, dp1, dp3, dp5); returns lvel
__device__ double wline_T(const double* __restrict__ q, long c, long S, double vel, double lout, double di,
                          double* lD) {
  for (int m = 0; m < 6; ++m) lD[m] = 0.0;
  const double lr = lout * di;
  // zero and sign tested on the bits (no FP64-pipe comparison)
  if ((__double_as_longlong(lr) << 1) == 0) return 0.0;
  const long long vb = __double_as_longlong(vel);
  Walk A;
  if ((vb << 1) == 0) {
    // both sides enter d(out)/d(vel) of weno5.h, (R_minus + R_plus)/12, where the
    // walk from the plus end gives -R_plus; neither enters d(out)/d(q)
    Walk B;
    walk_fwd(q, c, S, A);
    walk_fwd(q, c, -S, B);
    return lr * (A.R - B.R) * (1.0 / 12.0);
  }
  const bool pos = vb > 0;
  walk_fwd(q, c, pos ? S : -S, A);
  // out = |vel|/6 di R, so lR = lr |vel| / 6 and g4 = 4 lR / den
  double la[5];
  walk_rev(A, (lr * fabs(vel)) * (2.0 / 3.0) * A.iD, la);
  // walk differences: (dm5, dm3, dm1, dp1, dp3) for vel > 0, -(dp5, dp3, dp1, dm1,
  // dm3) for vel < 0
  lD[0] = pos ? la[0] : 0.0;
  lD[1] = pos ? la[1] : -la[4];
  lD[2] = pos ? la[2] : -la[3];
  lD[3] = pos ? la[3] : -la[2];
  lD[4] = pos ? la[4] : -la[1];
  lD[5] = pos ? 0.0 : -la[0];
  // d(out)/d(vel) = sign(vel) di R / 6
  return lr * (pos ? A.R : -A.R) * (1.0 / 6.0);
}

// FP32 counterpart for handles whose forward runs the mixed-precision step
// (fused_weno.cu's k_weno2_f32): the same reverse sweep in float on the split pairs
// (hi, lo) of the velocity fields, a difference formed as (hi1 - hi0) + (lo1 -
// lo0), with the forward kernel's scaling -- the five differences divided by their
// largest magnitude s and the additive 1e-80/486 taken as 1e-80/486/s^8, clamped
// to [2^-126, 2^100] (the same PTX approximations of log2 and exp2).  R is
// homogeneous of degree 1 in the differences, so dR/de is the scaled quotient's
// derivative and R = s R'.  A stencil flatter than 2^-100 gives R = 0, as forward.
__device__ __forceinline__ float lg2_apx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_apx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
struct WalkF {
  float t1a, t2a, t1b, t2b, t1c, t2c, s1, s2, s3, x, y, z, X, Y, Z, D1, d2, D3, iD, R, sc;
};
// false where the stencil is flat (R = 0 and no derivative)
__device__ __forceinline__ bool walk_fwd_f32(const float2* __restrict__ q, long c, long st, WalkF& W) {
  const float2* p = q + c - 3 * st;
  const float2 q0 = __ldg(p), q1 = __ldg(p + st), q2 = __ldg(p + 2 * st), q3 = __ldg(p + 3 * st),
               q4 = __ldg(p + 4 * st), q5 = __ldg(p + 5 * st);
  float a5 = (q1.x - q0.x) + (q1.y - q0.y), a3 = (q2.x - q1.x) + (q2.y - q1.y), a1 = (q3.x - q2.x) + (q3.y - q2.y),
        b1 = (q4.x - q3.x) + (q4.y - q3.y), b3 = (q5.x - q4.x) + (q5.y - q4.y);
  const float s = fmaxf(fmaxf(fmaxf(fabsf(a5), fabsf(a3)), fmaxf(fabsf(a1), fabsf(b1))), fabsf(b3));
  W.R = 0.0f;
  W.sc = s;
  if (s < 0x1p-100f) return false;
  const float is = __fdividef(1.0f, s);
  a5 *= is;
  a3 *= is;
  a1 *= is;
  b1 *= is;
  b3 *= is;
  constexpr float c13 = 13.0f / 3.0f;
  W.t1a = fmaf(a3, -2.0f, a5 + a1);
  W.t2a = fmaf(a3, -4.0f, fmaf(a1, 3.0f, a5));
  W.t1b = fmaf(a1, -2.0f, a3 + b1);
  W.t2b = a3 - b1;
  W.t1c = fmaf(b1, -2.0f, a1 + b3);
  W.t2c = fmaf(b1, -4.0f, fmaf(a1, 3.0f, b3));
  W.s1 = fmaf(W.t1a * c13, W.t1a, W.t2a * W.t2a);
  W.s2 = fmaf(W.t1b * c13, W.t1b, W.t2b * W.t2b);
  W.s3 = fmaf(W.t1c * c13, W.t1c, W.t2c * W.t2c);
  // log2(1e-80 / 486) = -274.679
  const float eps = ex2_apx(fminf(fmaxf(-274.679f - 8.0f * lg2_apx(s), -126.0f), 100.0f));
  W.x = W.s2 * W.s3;
  W.y = W.s1 * W.s3;
  W.z = W.s1 * W.s2;
  W.X = W.x * W.x;
  W.Y = fmaf(W.y, W.y, eps);
  W.Z = W.z * W.z;
  W.D1 = fmaf(a1, 11.0f / 6.0f, fmaf(a3, -7.0f / 6.0f, a5 * (1.0f / 3.0f)));
  W.d2 = fmaf(b1, 2.0f, fmaf(a1, 5.0f, -a3));
  W.D3 = fmaf(b1, 2.5f, fmaf(b3, -0.5f, a1));
  const float num = fmaf(W.Z, W.D3, fmaf(W.Y, W.d2, W.X * W.D1));
  W.iD = __fdividef(1.0f, fmaf(W.X, 1.0f / 6.0f, fmaf(W.Z, 0.5f, W.Y)));
  W.R = num * W.iD;
  return true;
}
__device__ __forceinline__ void walk_rev_f32(const WalkF& W, float g4, float* la) {
  constexpr float c13 = 13.0f / 3.0f;
  const float lD1 = g4 * W.X, ld2 = g4 * W.Y, lD3 = g4 * W.Z;
  const float lX = g4 * fmaf(W.R, -1.0f / 6.0f, W.D1), lY = g4 * (W.d2 - W.R), lZ = g4 * fmaf(W.R, -0.5f, W.D3);
  const float lx = W.x * lX, ly = W.y * lY, lz = W.z * lZ;
  const float S1 = fmaf(ly, W.s3, lz * W.s2), S2 = fmaf(lx, W.s3, lz * W.s1), S3 = fmaf(lx, W.s2, ly * W.s1);
  const float lt1a = (W.t1a * c13) * S1, lt2a = W.t2a * S1;
  const float lt1b = (W.t1b * c13) * S2, lt2b = W.t2b * S2;
  const float lt1c = (W.t1c * c13) * S3, lt2c = W.t2c * S3;
  la[0] = fmaf(lD1, 1.0f / 12.0f, lt1a + lt2a);
  la[1] = fmaf(lD1, -7.0f / 24.0f, fmaf(ld2, -0.25f, fmaf(lt1a, -2.0f, fmaf(lt2a, -4.0f, lt1b + lt2b))));
  la[2] = fmaf(lD1, 11.0f / 24.0f,
               fmaf(ld2, 1.25f, fmaf(lD3, 0.25f, fmaf(lt2a, 3.0f, fmaf(lt1b, -2.0f, fmaf(lt2c, 3.0f, lt1a + lt1c))))));
  la[3] = fmaf(ld2, 0.5f, fmaf(lD3, 0.625f, fmaf(lt1c, -2.0f, fmaf(lt2c, -4.0f, lt1b - lt2b))));
  la[4] = fmaf(lD3, -0.125f, lt1c + lt2c);
}
// the adjoint of  out += |vsum| di/24 R  (vsum = 4 vel) given lr = lout di: lD =
// the adjoints of the six differences; returns the adjoint of vel
__device__ float wline_T_f32(const float2* __restrict__ q, long c, long S, float vsum, float lr, float* lD) {
  for (int m = 0; m < 6; ++m) lD[m] = 0.0f;
  if (lr == 0.0f) return 0.0f;
  WalkF A;
  if (vsum == 0.0f) {
    WalkF B;
    walk_fwd_f32(q, c, S, A);
    walk_fwd_f32(q, c, -S, B);
    return lr * (A.R * A.sc - B.R * B.sc) * (1.0f / 12.0f);
  }
  const bool pos = vsum > 0.0f;
  if (!walk_fwd_f32(q, c, pos ? S : -S, A)) return 0.0f;
  float la[5];
  walk_rev_f32(A, (lr * fabsf(vsum)) * (1.0f / 6.0f) * A.iD, la);
  lD[0] = pos ? la[0] : 0.0f;
  lD[1] = pos ? la[1] : -la[4];
  lD[2] = pos ? la[2] : -la[3];
  lD[3] = pos ? la[3] : -la[2];
  lD[4] = pos ? la[4] : -la[1];
  lD[5] = pos ? 0.0f : -la[0];
  return lr * (pos ? A.R : -A.R) * A.sc * (1.0f / 6.0f);
}

// FP32-pair counterpart for handles whose forward is the FP64 step: the walk's
// five differences taken in FP64 (exact for neighbouring values, as the forward's)
// and split into pairs, then R and dR/de in FP32-pair arithmetic
// (weno5_df.cuh's wrev_core).  Each line then costs about 25 FP64 operations (the
// advecting velocity, the differences, the rounding of the results, the products
// with lR) instead of about 100.
struct WalkP {
  df::D R;     // the forward's R
  df::D g[5];  // dR/d(a5, a3, a1, b1, b3)
};
__device__ __forceinline__ void walk_df(const double* __restrict__ q, long c, long st, bool grad, WalkP& W) {
  const double* p = q + c - 3 * st;
  const double q0 = __ldg(p), q1 = __ldg(p + st), q2 = __ldg(p + 2 * st), q3 = __ldg(p + 3 * st),
               q4 = __ldg(p + 4 * st), q5 = __ldg(p + 5 * st);
  using df::split_double;
  df::wrev_core(split_double(q1 - q0), split_double(q2 - q1), split_double(q3 - q2), split_double(q4 - q3),
                split_double(q5 - q4), grad, W.R, W.g);
}
// wline_T with the walks in FP32 pairs (FP64 handles): the same contract
__device__ double wline_T_df(const double* __restrict__ q, long c, long S, double vel, double lout, double di,
                             double* lD) {
  for (int m = 0; m < 6; ++m) lD[m] = 0.0;
  const double lr = lout * di;
  if ((__double_as_longlong(lr) << 1) == 0) return 0.0;
  const long long vb = __double_as_longlong(vel);
  WalkP A;
  if ((vb << 1) == 0) {
    WalkP B;
    walk_df(q, c, S, false, A);
    walk_df(q, c, -S, false, B);
    return lr * (df::to_double(A.R) - df::to_double(B.R)) * (1.0 / 12.0);
  }
  const bool pos = vb > 0;
  walk_df(q, c, pos ? S : -S, true, A);
  const double lR = (lr * __longlong_as_double(vb & 0x7fffffffffffffffLL)) * (1.0 / 6.0);
  double la[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) la[m] = lR * df::to_double(A.g[m]);
  lD[0] = pos ? la[0] : 0.0;
  lD[1] = pos ? la[1] : -la[4];
  lD[2] = pos ? la[2] : -la[3];
  lD[3] = pos ? la[3] : -la[2];
  lD[4] = pos ? la[4] : -la[1];
  lD[5] = pos ? 0.0 : -la[0];
  const double R = df::to_double(A.R);
  return lr * (pos ? R : -R) * (1.0 / 6.0);
}

// Offsets (relative to the cell) of the four velocity points that form the
// advecting velocity of line (component q, direction d); the line reads component d.
__constant__ signed char kVelOff[9][4][3] = {
    {{-1, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, 0, 0}},   {{0, -1, 0}, {1, -1, 0}, {0, 0, 0}, {1, 0, 0}},
    {{0, 0, -1}, {1, 0, -1}, {0, 0, 0}, {1, 0, 0}},  {{-1, 0, 0}, {-1, 1, 0}, {0, 0, 0}, {0, 1, 0}},
    {{0, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 1, 0}},   {{0, 0, -1}, {0, 1, -1}, {0, 0, 0}, {0, 1, 0}},
    {{-1, 0, 0}, {-1, 0, 1}, {0, 0, 0}, {0, 0, 1}},  {{0, -1, 0}, {0, -1, 1}, {0, 0, 0}, {0, 0, 1}},
    {{0, 0, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 1}}};

// Pass 1: per interior cell and each of the 9 lines (one thread per cell and
// line: grid z = 9 nk), the adjoints of the six differences (D, 54 arrays) and of
// the advecting velocity (V, 9 arrays).
__global__ void __launch_bounds__(256) k_weno_T1(Grid g, double dxi, double dyi, double dzi,
                                                 const double* __restrict__ u, const double* __restrict__ v,
                                                 const double* __restrict__ w, const double* __restrict__ la0,
                                                 const double* __restrict__ la1, const double* __restrict__ la2,
                                                 double* __restrict__ D, double* __restrict__ V) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int line = (int)blockIdx.z % 9, k = 1 + (int)blockIdx.z / 9;
  if (i > g.ni || j > g.nj) return;
  const int q = line / 3, d = line % 3;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  const double* vq = d == 0 ? u : (d == 1 ? v : w);
  const signed char(*o)[3] = kVelOff[line];
  const double a = vq[c + o[0][0] * X + o[0][1] * Y + o[0][2] * Z];
  const double b = vq[c + o[1][0] * X + o[1][1] * Y + o[1][2] * Z];
  const double e = vq[c + o[2][0] * X + o[2][1] * Y + o[2][2] * Z];
  const double f = vq[c + o[3][0] * X + o[3][1] * Y + o[3][2] * Z];
  const double vel = ((a + b) * 0.5 + (e + f) * 0.5) * 0.5;
  const double L = (q == 0 ? la0 : (q == 1 ? la1 : la2))[c];
  double lD[6];
  const double lvel = wline_T(q == 0 ? u : (q == 1 ? v : w), c, d == 0 ? X : (d == 1 ? Y : Z), vel, L,
                              d == 0 ? dxi : (d == 1 ? dyi : dzi), lD);
#pragma unroll
  for (int m = 0; m < 6; ++m) D[(long)(line * 6 + m) * n + c] = lD[m];
  V[(long)line * n + c] = lvel;
}
// Pass 1 in FP32 (handles with a mixed-precision forward): sp holds the split pairs
// of u, v, w (3 n float2); the advecting velocity is formed as the forward FP32
// kernel forms it (vsum = (a + b) + (c + d) of the pairs' high parts).  The
// adjoints are stored as double for pass 2.
__global__ void __launch_bounds__(256) k_weno_T1_f32(Grid g, float dxi, float dyi, float dzi,
                                                     const float2* __restrict__ sp, const double* __restrict__ la0,
                                                     const double* __restrict__ la1, const double* __restrict__ la2,
                                                     double* __restrict__ D, double* __restrict__ V) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int line = (int)blockIdx.z % 9, k = 1 + (int)blockIdx.z / 9;
  if (i > g.ni || j > g.nj) return;
  const int q = line / 3, d = line % 3;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  const float2* vq = sp + (long)d * n;
  const signed char(*o)[3] = kVelOff[line];
  auto h = [&](int t) { return __ldg(&vq[c + o[t][0] * X + o[t][1] * Y + o[t][2] * Z].x); };
  const float vsum = (h(0) + h(1)) + (h(2) + h(3));
  const float L = (float)(q == 0 ? la0 : (q == 1 ? la1 : la2))[c];
  float lD[6];
  const float lvel = wline_T_f32(sp + (long)q * n, c, d == 0 ? X : (d == 1 ? Y : Z), vsum,
                                 L * (d == 0 ? dxi : (d == 1 ? dyi : dzi)), lD);
#pragma unroll
  for (int m = 0; m < 6; ++m) D[(long)(line * 6 + m) * n + c] = (double)lD[m];
  V[(long)line * n + c] = (double)lvel;
}
// Pass 1 in FP32 pairs (FP64 handles): the advecting velocity as k_weno_T1 forms
// it, the walks through wline_T_df
__global__ void __launch_bounds__(256) k_weno_T1_df(Grid g, double dxi, double dyi, double dzi,
                                                    const double* __restrict__ u, const double* __restrict__ v,
                                                    const double* __restrict__ w,
                                                    const double* __restrict__ la0, const double* __restrict__ la1,
                                                    const double* __restrict__ la2, double* __restrict__ D,
                                                    double* __restrict__ V) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int line = (int)blockIdx.z % 9, k = 1 + (int)blockIdx.z / 9;
  if (i > g.ni || j > g.nj) return;
  const int q = line / 3, d = line % 3;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  const double* vq = d == 0 ? u : (d == 1 ? v : w);
  const signed char(*o)[3] = kVelOff[line];
  const double a = vq[c + o[0][0] * X + o[0][1] * Y + o[0][2] * Z];
  const double b = vq[c + o[1][0] * X + o[1][1] * Y + o[1][2] * Z];
  const double e = vq[c + o[2][0] * X + o[2][1] * Y + o[2][2] * Z];
  const double f = vq[c + o[3][0] * X + o[3][1] * Y + o[3][2] * Z];
  const double vel = ((a + b) * 0.5 + (e + f) * 0.5) * 0.5;
  const double L = (q == 0 ? la0 : (q == 1 ? la1 : la2))[c];
  double lD[6];
  const double lvel = wline_T_df(q == 0 ? u : (q == 1 ? v : w), c, d == 0 ? X : (d == 1 ? Y : Z), vel, L,
                                 d == 0 ? dxi : (d == 1 ? dyi : dzi), lD);
#pragma unroll
  for (int m = 0; m < 6; ++m) D[(long)(line * 6 + m) * n + c] = lD[m];
  V[(long)line * n + c] = lvel;
}
// Pass 2: every point gathers what the lines of the cells around it owe it.
__global__ void __launch_bounds__(256) k_weno_T2(Grid g, const double* __restrict__ D,
                                                 const double* __restrict__ V, double* __restrict__ lu,
                                                 double* __restrict__ lv, double* __restrict__ lw) {
  const int x = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int y = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int z = -2 + (int)blockIdx.z;
  if (x > g.ni + 3 || y > g.nj + 3) return;
  const long n = g.n;
  auto in = [&](int a, int b, int e) { return a >= 1 && a <= g.ni && b >= 1 && b <= g.nj && e >= 1 && e <= g.nk; };
  // point x sits at stencil position o (-3..3) of the cell x - o*S; its coefficient
  // there: o=-3: -D0, -2: D0-D1, -1: D1-D2, 0: D2-D3, 1: D3-D4, 2: D4-D5, 3: D5
  double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int p = 0; p < 3; ++p) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int line = p * 3 + d;
      const double* Dl = D + (long)line * 6 * n;
      for (int o = -3; o <= 3; ++o) {
        const int ci = x - (d == 0 ? o : 0), cj = y - (d == 1 ? o : 0), ck = z - (d == 2 ? o : 0);
        if (!in(ci, cj, ck)) continue;
        const long c = g.at(ci, cj, ck);
        const int m = o + 3;  // 0..6
        const double hi = m < 6 ? Dl[(long)m * n + c] : 0.0;     // + D_m
        const double lo = m > 0 ? Dl[(long)(m - 1) * n + c] : 0.0;  // - D_{m-1}
        acc[p] += lo - hi;
      }
    }
    // velocity points: lines (q, p) read component p at 4 offsets
    for (int q = 0; q < 3; ++q) {
      const int line = q * 3 + p;
      for (int t = 0; t < 4; ++t) {
        const int ci = x - kVelOff[line][t][0], cj = y - kVelOff[line][t][1], ck = z - kVelOff[line][t][2];
        if (!in(ci, cj, ck)) continue;
        acc[p] += 0.25 * V[(long)line * n + g.at(ci, cj, ck)];
      }
    }
  }
  const long c = g.at(x, y, z);
  lu[c] += acc[0];
  lv[c] += acc[1];
  lw[c] += acc[2];
}
}  // namespace

void weno_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
            const double* w, const double* const* ladv, double* lu, double* lv, double* lw, double* work,
            float2* split, bool pairs) {
  double* D = work;
  double* V = work + 54 * g.n;
  const dim3 grd((g.ni + 31) / 32, (g.nj + 7) / 8, 9 * g.nk), blk(32, 8);
  if (pairs) {
    k_weno_T1_df<<<grd, blk, 0, s>>>(g, dxi, dyi, dzi, u, v, w, ladv[0], ladv[1], ladv[2], D, V);
  } else if (split) {
    fused::split3(s, g, u, v, w, split);
    k_weno_T1_f32<<<grd, blk, 0, s>>>(g, (float)dxi, (float)dyi, (float)dzi, split, ladv[0], ladv[1], ladv[2], D, V);
  } else {
    k_weno_T1<<<grd, blk, 0, s>>>(g, dxi, dyi, dzi, u, v, w, ladv[0], ladv[1], ladv[2], D, V);
  }
  k_weno_T2<<<dim3((g.ni + 6 + 31) / 32, (g.nj + 6 + 7) / 8, g.nk + 6), dim3(32, 8), 0, s>>>(g, D, V, lu, lv, lw);
  count_launch(2);
}

// ---- CSF --------------------------------------------------------------------------
void csf_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double rhol, double rhog,
           double sigma, const double* phi, const double* const* lf, double* lphi, double* work) {
  const Grid G = g;
  const long n = g.n;
  double* Gv = work;             // vertex gradient (3n)
  double* rn = work + 3 * n;     // the four normal families (12n)
  double* kap = work + 15 * n;   // curvature at u, v, w points (3n)
  double* gq = work + 18 * n;    // face gradient of phi (3n)
  double* lG = work + 21 * n;    // adjoint of the vertex gradient (3n)
  double* lv = work + 24 * n;    // per normal family: adjoint of its 8-point mean (12n)
  double* lkap = work + 36 * n;  // adjoint of the curvature (3n)
  double* lgq = work + 39 * n;   // adjoint of the face gradient (3n)
  // Noise floor.  The normals N(v) = v/(|v| + vs) take vs = 1e-30 |grad| (calrn.f),
  // so where phi is flat to within rounding (the far tails of the interface
  // profile, phi = 1 - a few ulps) they are unit vectors of rounding noise with
  // O(1/dx) curvature.  The force there is ~0, but the exact linearisation of
  // those normals is O(1) and as random as the noise: it differs between any two
  // trajectories, and a central difference of any resolvable step does not see it
  // (the force is even in the step there).  So normals whose mean gradient is
  // below tau = 1e-6 |(dxi, dyi, dzi)| -- phi varying by under 1e-6 per cell, far
  // below the interface band's >= 1e-2 per cell and far above rounding -- are
  // taken as the constant 0: the curvature the transpose uses is formed from the
  // others (equal to the step's wherever the normals are resolved), and those
  // normals pass no adjoint to the vertex gradients.
  const double tau = 1.0e-6 * std::sqrt(dxi * dxi + dyi * dyi + dzi * dzi);
  const double vs = std::sqrt(dxi * dxi + dyi * dyi + dzi * dzi) * 1.0e-30;
  // forward recompute: vertex gradients, normals (calrn.f:45-87 with the floor),
  // curvature (calrkap.f) and face gradients
  fused::vertex_gradient(s, g, dxi, dyi, dzi, phi, Gv, Gv + n, Gv + 2 * n);
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const int ip = f == 0 || f == 3, jp = f == 0 || f == 2, kp = f == 0 || f == 1;
      double* out = rn + 3 * n * f + c;
      if (i < -2 + ip || j < -2 + jp || k < -2 + kp) {  // calrn does not write o
        out[0] = out[n] = out[2 * n] = 0.0;
        continue;
      }
      const long Xf = ip ? X : 0, Yf = jp ? Y : 0, Zf = kp ? Z : 0;
      const long b = c - Xf - Yf - Zf;
      double r[3];
#pragma unroll
      for (int q3 = 0; q3 < 3; ++q3) {
        const double* p = Gv + q3 * n + b;
        r[q3] = f == 0 ? (p[0] + p[Xf] + p[Yf] + p[Xf + Yf] + p[Zf] + p[Xf + Zf] + p[Yf + Zf] + p[Xf + Yf + Zf]) * 0.125
                       : (p[0] + p[Xf + Yf + Zf]) * 0.5;
      }
      const double s2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
      if (s2 <= tau * tau) {
        out[0] = out[n] = out[2 * n] = 0.0;
        continue;
      }
      // v/(|v| + vs) by Newton-Raphson reciprocals (s2 is a normal number here)
      const double ia = recip_nr(s2 * rsqrt_nr(s2) + vs);
      out[0] = r[0] * ia;
      out[n] = r[1] * ia;
      out[2 * n] = r[2] * ia;
    }
  });
  op::calrkap(s, g, dxi, dyi, dzi, rn, rn + 3 * n, rn + 6 * n, rn + 9 * n, kap);
  op::cal_grad_prs(s, g, dxi, dyi, dzi, phi, gq, gq + n, gq + 2 * n);
  // calfst: f_c = -st kap_c g_c
  const double st = 2.0 * sigma / (rhol + rhog);
  const double *lf0 = lf[0], *lf1 = lf[1], *lf2 = lf[2];
  flat(s, n, [=] __device__(long t) {
    const double L[3] = {lf0[t], lf1[t], lf2[t]};
    for (int q = 0; q < 3; ++q) {
      lkap[t + q * n] = -st * gq[t + q * n] * L[q];
      lgq[t + q * n] = L[q] != 0.0 ? -st * kap[t + q * n] * L[q] : 0.0;
    }
  });
  grad_prs_T(s, g, dxi, dyi, dzi, lgq, lgq + n, lgq + 2 * n, lphi);
  // calrkap and calrn reversed as two gathers (no atomics).
  // Families (calrkap's rn arguments): 0 = pp (offset 1,1,1), 1 = r12 (0,0,1),
  // 2 = r13 (0,1,0), 3 = r23 (1,0,0).  Family f's normal at o is N(v) = v/(|v| + vs)
  // of the mean v of Gv over o - {0,X_f} - {0,Y_f} - {0,Z_f} (X_f = 0 where the
  // offset is 0), written by calrn for o_i in [-2 + ip, ni+3] (same in j, k).
  // calrkap writes the u curvature where k >= -1, j >= -1, i <= ni+2, the v one where
  // k >= -1, j <= nj+2, i >= -1, the w one where k <= nk+2, j >= -1, i >= -1.
  // pass 1, per normal point o and family: the normal's adjoint gathered from the
  // curvatures that read it, then lv = (dN/dv)^T lrn
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    auto in = [&](int a, int b, int e) {
      return a >= -2 && a <= G.ni + 3 && b >= -2 && b <= G.nj + 3 && e >= -2 && e <= G.nk + 3;
    };
    auto ku = [&](int a, int b, int e, long o) {
      return in(a, b, e) && e >= -1 && b >= -1 && a <= G.ni + 2 ? lkap[o] : 0.0;
    };
    auto kv = [&](int a, int b, int e, long o) {
      return in(a, b, e) && e >= -1 && b <= G.nj + 2 && a >= -1 ? lkap[o + n] : 0.0;
    };
    auto kw = [&](int a, int b, int e, long o) {
      return in(a, b, e) && e <= G.nk + 2 && b >= -1 && a >= -1 ? lkap[o + 2 * n] : 0.0;
    };
    // kap_u = dxi (pp_x[+X] - pp_x) + dyi (r12_y - r12_y[-Y]) + dzi (r13_z - r13_z[-Z]),
    // kap_v = dxi (r12_x - r12_x[-X]) + dyi (pp_y[+Y] - pp_y) + dzi (r23_z - r23_z[-Z]),
    // kap_w = dxi (r13_x - r13_x[-X]) + dyi (r23_y - r23_y[-Y]) + dzi (pp_z[+Z] - pp_z)
    double L[4][3];
    L[0][0] = dxi * (ku(i - 1, j, k, c - X) - ku(i, j, k, c));
    L[0][1] = dyi * (kv(i, j - 1, k, c - Y) - kv(i, j, k, c));
    L[0][2] = dzi * (kw(i, j, k - 1, c - Z) - kw(i, j, k, c));
    L[1][0] = dxi * (kv(i, j, k, c) - kv(i + 1, j, k, c + X));
    L[1][1] = dyi * (ku(i, j, k, c) - ku(i, j + 1, k, c + Y));
    L[1][2] = 0.0;
    L[2][0] = dxi * (kw(i, j, k, c) - kw(i + 1, j, k, c + X));
    L[2][1] = 0.0;
    L[2][2] = dzi * (ku(i, j, k, c) - ku(i, j, k + 1, c + Z));
    L[3][0] = 0.0;
    L[3][1] = dyi * (kw(i, j, k, c) - kw(i, j + 1, k, c + Y));
    L[3][2] = dzi * (kv(i, j, k, c) - kv(i, j, k + 1, c + Z));
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const int ip = f == 0 || f == 3, jp = f == 0 || f == 2, kp = f == 0 || f == 1;
      if (i < -2 + ip || j < -2 + jp || k < -2 + kp) continue;  // calrn does not write o
      double* out = lv + 3 * n * f + c;
      const double lx = L[f][0], ly = L[f][1], lz = L[f][2];
      if (lx == 0.0 && ly == 0.0 && lz == 0.0) {
        out[0] = out[n] = out[2 * n] = 0.0;
        continue;
      }
      const long Xf = ip ? X : 0, Yf = jp ? Y : 0, Zf = kp ? Z : 0;
      const long b = c - Xf - Yf - Zf;
      double r[3];
#pragma unroll
      for (int q3 = 0; q3 < 3; ++q3) {
        const double* p = Gv + q3 * n + b;
        // family 0 averages 8 vertex gradients; families 1-3 (one offset only) the
        // two along that offset, each four times in the 8-term mean
        r[q3] = f == 0 ? (p[0] + p[Xf] + p[Yf] + p[Xf + Yf] + p[Zf] + p[Xf + Zf] + p[Yf + Zf] + p[Xf + Yf + Zf]) * 0.125
                       : (p[0] + p[Xf + Yf + Zf]) * 0.5;
      }
      // dN/dv = I/a - v v^T/(a^2 m) with m = |v|, a = m + vs:
      // lv = (l - v (v.l)/(m a)) / a, the factor formed as ((v.l)/m)/a, which stays
      // finite for any m > 0
      // (division-free reciprocals where s2 is a normal number; subnormal and zero
      // s2 take the library functions)
      const double s2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
      if (s2 <= tau * tau) {  // below the noise floor: a constant normal
        out[0] = out[n] = out[2 * n] = 0.0;
        continue;
      }
      double ia, t = 0.0;
      if (s2 >= 0x1p-1000) {
        const double im = rsqrt_nr(s2);
        ia = recip_nr(s2 * im + vs);
        t = ((r[0] * lx + r[1] * ly + r[2] * lz) * im) * ia;
      } else if (s2 > 0.0) {
        const double im = rsqrt(s2);
        ia = 1.0 / (s2 * im + vs);
        t = ((r[0] * lx + r[1] * ly + r[2] * lz) * im) * ia;
      } else {
        ia = 1.0 / vs;
      }
      out[0] = (lx - r[0] * t) * ia;
      out[n] = (ly - r[1] * t) * ia;
      out[2 * n] = (lz - r[2] * t) * ia;
    }
  });
  // pass 2, per vertex p: 0.125 lv over the (family, corner) pairs whose mean reads
  // p, i.e. o = p + {0,X_f} + {0,Y_f} + {0,Z_f} (families 1-3 read two points, four
  // times each)
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    auto ok = [&](int f, int a, int b, int e) {
      const int ip = f == 0 || f == 3, jp = f == 0 || f == 2, kp = f == 0 || f == 1;
      return a >= -2 + ip && a <= G.ni + 3 && b >= -2 + jp && b <= G.nj + 3 && e >= -2 + kp && e <= G.nk + 3;
    };
    const bool a1 = ok(1, i, j, k), b1 = ok(1, i, j, k + 1), a2 = ok(2, i, j, k), b2 = ok(2, i, j + 1, k),
               a3 = ok(3, i, j, k), b3 = ok(3, i + 1, j, k);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double* L0 = lv + q * n + c;
      double acc = 0.0;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int di = t & 1, dj = (t >> 1) & 1, dk = t >> 2;
        if (ok(0, i + di, j + dj, k + dk)) acc += L0[di * X + dj * Y + dk * Z];
      }
      const double* L1 = L0 + 3 * n;
      const double* L2 = L0 + 6 * n;
      const double* L3 = L0 + 9 * n;
      double acc4 = 0.0;
      if (a1) acc4 += L1[0];
      if (b1) acc4 += L1[Z];
      if (a2) acc4 += L2[0];
      if (b2) acc4 += L2[Y];
      if (a3) acc4 += L3[0];
      if (b3) acc4 += L3[X];
      lG[q * n + c] = 0.125 * (acc + 4.0 * acc4);
    }
  });
  grad_p2a_T(s, g, dxi, dyi, dzi, lG, lG + n, lG + 2 * n, lphi);
}

}  // namespace adj
}  // namespace fmf
