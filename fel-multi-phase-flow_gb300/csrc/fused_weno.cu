// fused_weno.cu -- WENO5 advection of both velocity levels in one kernel (the two
// cal_advu_weno5 calls of main.f90:532-533), compiled with multiply-add contraction.
//
// weno5.h forms both one-sided reconstructions and multiplies the unused one by
// vel-|vel| = 0 (or vel+|vel| = 0); here only the upwind side is evaluated, which
// gives the same value and halves the FP64 work.  The grid has one thread per
// interior cell (x fastest, 32 x 4 block, one k plane per grid z).
#include "fused.cuh"
#include "weno5_core.cuh"

namespace fmf {
namespace fused {

namespace {
// One-sided derivative: (a5,a3,a1,b1,b3) = (dfm5,dfm3,dfm1,dfp1,dfp3) for vel>0 and
// (dfp5,dfp3,dfp1,dfm1,dfm3) for vel<0 (weno5.h:2-70 with the sides exchanged).
template <class R>
__device__ __forceinline__ R weno_side(R a5, R a3, R a1, R b1, R b3) {
  const R d1 = a5 * (R)2 - a3 * (R)7 + a1 * (R)11;
  const R d2 = -a3 + a1 * (R)5 + b1 * (R)2;
  const R d3 = a1 * (R)2 + b1 * (R)5 - b3;
  R t1 = a5 - a3 * (R)2 + a1, t2 = a5 - a3 * (R)4 + a1 * (R)3;
  const R s1 = t1 * t1 * (R)13 + t2 * t2 * (R)3;
  t1 = a3 - a1 * (R)2 + b1;
  t2 = a3 - b1;
  const R s2 = t1 * t1 * (R)13 + t2 * t2 * (R)3;
  t1 = a1 - b1 * (R)2 + b3;
  t2 = a1 * (R)3 - b1 * (R)4 + b3;
  const R s3 = t1 * t1 * (R)13 + t2 * t2 * (R)3;
  R m1 = s2 * s3, m2 = s1 * s3, m3 = s1 * s2;
  m1 = m1 * m1;
  m2 = m2 * m2 * (R)6;
  m3 = m3 * m3 * (R)3;
  const R inv = (R)1 / (m1 + m2 + m3 + (R)1.0e-80);
  const R w1 = m1 * inv, w3 = m3 * inv;
  const R w2 = (R)1 - w1 - w3;
  return w1 * d1 + w2 * d2 + w3 * d3;
}

// derivative of q along stride S at c with advecting velocity vel
__device__ __forceinline__ double wdir(const double* __restrict__ q, long c, long S, double vel) {
  if (vel == 0.0) return 0.0;
  const double m3 = __ldg(q + c - 3 * S), m2 = __ldg(q + c - 2 * S), m1 = __ldg(q + c - S), z0 = __ldg(q + c),
               p1 = __ldg(q + c + S), p2 = __ldg(q + c + 2 * S), p3 = __ldg(q + c + 3 * S);
  const double dm5 = m2 - m3, dm3 = m1 - m2, dm1 = z0 - m1, dp1 = p1 - z0, dp3 = p2 - p1, dp5 = p3 - p2;
  // the upwind side's inputs chosen by selects: one inlined side, no divergence
  // where the velocity changes sign inside a warp
  const bool pos = vel > 0.0;
  const double r = weno_side<double>(pos ? dm5 : dp5, pos ? dm3 : dp3, pos ? dm1 : dp1, pos ? dp1 : dm1,
                                     pos ? dp3 : dm3);
  return (vel + vel) * r * (1.0 / 12.0);
}

// FP32 variant for the mixed-precision step.  The product-form weights scale like
// the 8th power of the differences, so float would underflow for smooth fields;
// the five differences are divided by their largest magnitude s first (the
// weights are unchanged by a common scale; the sum is multiplied back by s), and
// the reference's additive 1e-80 becomes 1e-80/s^8 in scaled units, evaluated as a
// power of two and clamped to [2^-126, 2^127].  The lower clamp is the smallest
// normal float: where all three smoothness indicators are 0 (data exactly linear
// in float) the denominator is that term alone and its reciprocal must stay finite
// (2^-149 gave 1/e = inf and 0 * inf = NaN); the weights are then 0, 1, 0 as in
// the reference's limit.
__device__ __forceinline__ float weno_side_f32(float a5, float a3, float a1, float b1, float b3) {
  const float s = fmaxf(fmaxf(fmaxf(fabsf(a5), fabsf(a3)), fmaxf(fabsf(a1), fabsf(b1))), fabsf(b3));
  if (s == 0.0f) return 0.0f;
  const float is = 1.0f / s;
  a5 *= is;
  a3 *= is;
  a1 *= is;
  b1 *= is;
  b3 *= is;
  const float d1 = a5 * 2.0f - a3 * 7.0f + a1 * 11.0f;
  const float d2 = -a3 + a1 * 5.0f + b1 * 2.0f;
  const float d3 = a1 * 2.0f + b1 * 5.0f - b3;
  float t1 = a5 - a3 * 2.0f + a1, t2 = a5 - a3 * 4.0f + a1 * 3.0f;
  const float s1 = t1 * t1 * 13.0f + t2 * t2 * 3.0f;
  t1 = a3 - a1 * 2.0f + b1;
  t2 = a3 - b1;
  const float s2 = t1 * t1 * 13.0f + t2 * t2 * 3.0f;
  t1 = a1 - b1 * 2.0f + b3;
  t2 = a1 * 3.0f - b1 * 4.0f + b3;
  const float s3 = t1 * t1 * 13.0f + t2 * t2 * 3.0f;
  float m1 = s2 * s3, m2 = s1 * s3, m3 = s1 * s2;
  m1 = m1 * m1;
  m2 = m2 * m2 * 6.0f;
  m3 = m3 * m3 * 3.0f;
  // 1e-80 / s^8 = 2^(log2(1e-80) - 8 log2 s)
  const float e = exp2f(fminf(fmaxf(-265.754f - 8.0f * log2f(s), -126.0f), 127.0f));
  const float inv = 1.0f / (m1 + m2 + m3 + e);
  const float w1 = m1 * inv, w3 = m3 * inv;
  const float w2 = 1.0f - w1 - w3;
  return (w1 * d1 + w2 * d2 + w3 * d3) * s;
}
__device__ __forceinline__ float wdir_f32(const double* __restrict__ q, long c, long S, float vel) {
  if (vel == 0.0f) return 0.0f;
  const double m3 = __ldg(q + c - 3 * S), m2 = __ldg(q + c - 2 * S), m1 = __ldg(q + c - S), z0 = __ldg(q + c),
               p1 = __ldg(q + c + S), p2 = __ldg(q + c + 2 * S), p3 = __ldg(q + c + 3 * S);
  // differences formed in double (cancellation-free), arithmetic in float
  const float dm5 = (float)(m2 - m3), dm3 = (float)(m1 - m2), dm1 = (float)(z0 - m1), dp1 = (float)(p1 - z0),
              dp3 = (float)(p2 - p1), dp5 = (float)(p3 - p2);
  const bool pos = vel > 0.0f;
  const float r = weno_side_f32(pos ? dm5 : dp5, pos ? dm3 : dp3, pos ? dm1 : dp1, pos ? dp1 : dm1, pos ? dp3 : dm3);
  return (vel + vel) * r * (1.0f / 12.0f);
}
__global__ void __launch_bounds__(128) k_weno2_f32(Grid g, double dxi_, double dyi_, double dzi_,
                                                   const double* __restrict__ u, const double* __restrict__ v,
                                                   const double* __restrict__ w, const double* __restrict__ uo,
                                                   const double* __restrict__ vo, const double* __restrict__ wo,
                                                   double* __restrict__ au, double* __restrict__ av,
                                                   double* __restrict__ aw, double* __restrict__ auo,
                                                   double* __restrict__ avo, double* __restrict__ awo) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const float dxi = (float)dxi_, dyi = (float)dyi_, dzi = (float)dzi_;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
#pragma unroll 1
  for (int lev = 0; lev < 2; ++lev) {
    const double* U = lev ? uo : u;
    const double* V = lev ? vo : v;
    const double* W = lev ? wo : w;
    const float u0 = (float)__ldg(U + c), uxm = (float)__ldg(U + c - X), uxp = (float)__ldg(U + c + X);
    const float v0 = (float)__ldg(V + c), vym = (float)__ldg(V + c - Y), vyp = (float)__ldg(V + c + Y);
    const float w0 = (float)__ldg(W + c), wzm = (float)__ldg(W + c - Z), wzp = (float)__ldg(W + c + Z);
    float vel, a;
    vel = ((uxm + u0) * 0.5f + (u0 + uxp) * 0.5f) * 0.5f;
    a = wdir_f32(U, c, X, vel) * dxi;
    vel = ((vym + (float)__ldg(V + c + X - Y)) * 0.5f + (v0 + (float)__ldg(V + c + X)) * 0.5f) * 0.5f;
    a += wdir_f32(U, c, Y, vel) * dyi;
    vel = ((wzm + (float)__ldg(W + c + X - Z)) * 0.5f + (w0 + (float)__ldg(W + c + X)) * 0.5f) * 0.5f;
    a += wdir_f32(U, c, Z, vel) * dzi;
    (lev ? auo : au)[c] = (double)a;
    vel = ((uxm + (float)__ldg(U + c - X + Y)) * 0.5f + (u0 + (float)__ldg(U + c + Y)) * 0.5f) * 0.5f;
    a = wdir_f32(V, c, X, vel) * dxi;
    vel = ((vym + v0) * 0.5f + (v0 + vyp) * 0.5f) * 0.5f;
    a += wdir_f32(V, c, Y, vel) * dyi;
    vel = ((wzm + (float)__ldg(W + c + Y - Z)) * 0.5f + (w0 + (float)__ldg(W + c + Y)) * 0.5f) * 0.5f;
    a += wdir_f32(V, c, Z, vel) * dzi;
    (lev ? avo : av)[c] = (double)a;
    vel = ((uxm + (float)__ldg(U + c - X + Z)) * 0.5f + (u0 + (float)__ldg(U + c + Z)) * 0.5f) * 0.5f;
    a = wdir_f32(W, c, X, vel) * dxi;
    vel = ((vym + (float)__ldg(V + c - Y + Z)) * 0.5f + (v0 + (float)__ldg(V + c + Z)) * 0.5f) * 0.5f;
    a += wdir_f32(W, c, Y, vel) * dyi;
    vel = ((wzm + w0) * 0.5f + (w0 + wzp) * 0.5f) * 0.5f;
    a += wdir_f32(W, c, Z, vel) * dzi;
    (lev ? awo : aw)[c] = (double)a;
  }
}

__global__ void __launch_bounds__(128) k_weno2(Grid g, double dxi, double dyi, double dzi, const double* __restrict__ u,
                                               const double* __restrict__ v, const double* __restrict__ w,
                                               const double* __restrict__ uo, const double* __restrict__ vo,
                                               const double* __restrict__ wo, double* __restrict__ au,
                                               double* __restrict__ av, double* __restrict__ aw,
                                               double* __restrict__ auo, double* __restrict__ avo,
                                               double* __restrict__ awo) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
#pragma unroll 1
  for (int lev = 0; lev < 2; ++lev) {
    const double* U = lev ? uo : u;
    const double* V = lev ? vo : v;
    const double* W = lev ? wo : w;
    const double u0 = __ldg(U + c), uxm = __ldg(U + c - X), uxp = __ldg(U + c + X);
    const double v0 = __ldg(V + c), vym = __ldg(V + c - Y), vyp = __ldg(V + c + Y);
    const double w0 = __ldg(W + c), wzm = __ldg(W + c - Z), wzp = __ldg(W + c + Z);
    double vel, a;
    // u (cal_advu_weno5.f:80-120)
    vel = ((uxm + u0) * 0.5 + (u0 + uxp) * 0.5) * 0.5;
    a = wdir(U, c, X, vel) * dxi;
    vel = ((vym + __ldg(V + c + X - Y)) * 0.5 + (v0 + __ldg(V + c + X)) * 0.5) * 0.5;
    a += wdir(U, c, Y, vel) * dyi;
    vel = ((wzm + __ldg(W + c + X - Z)) * 0.5 + (w0 + __ldg(W + c + X)) * 0.5) * 0.5;
    a += wdir(U, c, Z, vel) * dzi;
    (lev ? auo : au)[c] = a;
    // v (:147-187)
    vel = ((uxm + __ldg(U + c - X + Y)) * 0.5 + (u0 + __ldg(U + c + Y)) * 0.5) * 0.5;
    a = wdir(V, c, X, vel) * dxi;
    vel = ((vym + v0) * 0.5 + (v0 + vyp) * 0.5) * 0.5;
    a += wdir(V, c, Y, vel) * dyi;
    vel = ((wzm + __ldg(W + c + Y - Z)) * 0.5 + (w0 + __ldg(W + c + Y)) * 0.5) * 0.5;
    a += wdir(V, c, Z, vel) * dzi;
    (lev ? avo : av)[c] = a;
    // w (:214-254)
    vel = ((uxm + __ldg(U + c - X + Z)) * 0.5 + (u0 + __ldg(U + c + Z)) * 0.5) * 0.5;
    a = wdir(W, c, X, vel) * dxi;
    vel = ((vym + __ldg(V + c - Y + Z)) * 0.5 + (v0 + __ldg(V + c + Z)) * 0.5) * 0.5;
    a += wdir(W, c, Y, vel) * dyi;
    vel = ((wzm + w0) * 0.5 + (w0 + wzp) * 0.5) * 0.5;
    a += wdir(W, c, Z, vel) * dzi;
    (lev ? awo : aw)[c] = a;
  }
}
}  // namespace

// Both levels; only interior cells are written (the fused step never reads the
// halo of the advection terms, which cal_advu_weno5.f:44-52 sets to zero).
void weno5_both(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u,
                const double* v, const double* w, const double* uo, const double* vo, const double* wo,
                double* const* adv, double* const* advo, bool fp32) {
  dim3 b(32, 4, 1);
  dim3 gr((unsigned)((g.ni + 31) / 32), (unsigned)((g.nj + 3) / 4), (unsigned)g.nk);
  if (fp32)
    k_weno2_f32<<<gr, b, 0, s>>>(g, dxi, dyi, dzi, u, v, w, uo, vo, wo, adv[0], adv[1], adv[2], advo[0], advo[1],
                                 advo[2]);
  else
    k_weno2<<<gr, b, 0, s>>>(g, dxi, dyi, dzi, u, v, w, uo, vo, wo, adv[0], adv[1], adv[2], advo[0], advo[1], advo[2]);
  count_launch();
}

}  // namespace fused
}  // namespace fmf
