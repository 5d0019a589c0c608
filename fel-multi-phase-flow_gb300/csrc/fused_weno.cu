// fused_weno.cu -- WENO5 advection (the two cal_advu_weno5 calls of main.f90:532-533:
// both velocity levels in one kernel, or the (u, v, w) level alone where the step
// reuses the previous step's result for (uo, vo, wo)), compiled with multiply-add
// contraction.
//
// weno5.h forms both one-sided reconstructions and multiplies the unused one by
// vel-|vel| = 0 (or vel+|vel| = 0); here only the upwind side is evaluated, which
// gives the same value and halves the FP64 work, in a rearranged form of the same
// quotient (wdir) that needs about two thirds of the remaining FP64 operations.
// The grid has one thread per interior cell (x fastest, 32 x 4 block, one k plane
// per grid z).
#include <cstring>

#include "../../include/fmf_capi.h"
#include "fused.cuh"
#include "recip.cuh"
#include "weno5_df.cuh"

namespace fmf {
namespace fused {

namespace {
// One directional derivative of weno5.h:2-70 times dxi, from the upwind side
// only (the reference multiplies the other side by vel -/+ |vel| = 0).
//  * vsum = 4 vel exactly: the reference's ((a+b)*0.5 + (c+d)*0.5)*0.5 scales
//    (a+b) + (c+d) by powers of two only, so vsum = (a+b) + (c+d) and the term
//    (vel + |vel|)/12 * dxi (or vel - |vel|) is |vsum| * dxi/24 on the side used.
//  * The five differences are taken walking from the upwind end, q[c-3S]..q[c+2S]
//    for vel > 0 (dfm5, dfm3, dfm1, dfp1, dfp3) and q[c+3S]..q[c-2S] for vel < 0,
//    where they are -(dfp5, dfp3, dfp1, dfm1, dfm3); the reconstruction is odd in
//    its inputs, so the sign of vel cancels and one formula serves both sides.
//  * Weights: with the reference's m1 = (s2 s3)^2, m2 = 6 (s1 s3)^2,
//    m3 = 3 (s1 s2)^2, w1 = m1 / (m1 + m2 + m3 + 1e-80), w3 likewise and
//    w2 = 1 - w1 - w3, its sum w1 d1 + w2 d2 + w3 d3 equals
//    (m1 d1 + m2 d2 + m3 d3 + 1e-80 d2) / (m1 + m2 + m3 + 1e-80).  That quotient
//    is formed here with every s divided by 3 and every m by 486 (the factors 6
//    and 3 moved onto d1/6 and d3/2), the 1e-80 divided by 486 and added to m2:
//    the same value with fewer FP64 operations.
// kx = dxi / 24.
__device__ __forceinline__ double wdir(const double* __restrict__ q, long c, long S, double vsum, double kx) {
  // zero and sign tested on the bits (a double comparison would take an FP64-pipe
  // slot): +-0 return 0; a positive sign bit walks from c - 3S
  const long long vb = __double_as_longlong(vsum);
  if ((vb << 1) == 0) return 0.0;
  const long st = vb > 0 ? S : -S;
  const double* p = q + c - 3 * st;
  const double q0 = __ldg(p), q1 = __ldg(p + st), q2 = __ldg(p + 2 * st), q3 = __ldg(p + 3 * st),
               q4 = __ldg(p + 4 * st), q5 = __ldg(p + 5 * st);
  const double a5 = q1 - q0, a3 = q2 - q1, a1 = q3 - q2, b1 = q4 - q3, b3 = q5 - q4;
  constexpr double c13 = 13.0 / 3.0;
  // s/3 = (13/3) t1^2 + t2^2 (weno5.h's 13 t1^2 + 3 t2^2)
  double t1 = fma(a3, -2.0, a5 + a1), t2 = fma(a3, -4.0, fma(a1, 3.0, a5));
  const double s1 = fma(t1 * c13, t1, t2 * t2);
  t1 = fma(a1, -2.0, a3 + b1);
  t2 = a3 - b1;
  const double s2 = fma(t1 * c13, t1, t2 * t2);
  t1 = fma(b1, -2.0, a1 + b3);
  t2 = fma(b1, -4.0, fma(a1, 3.0, b3));
  const double s3 = fma(t1 * c13, t1, t2 * t2);
  const double x = s2 * s3, y = s1 * s3, z = s1 * s2;
  const double X = x * x, Y = fma(y, y, 1.0e-80 / 486.0), Z = z * z;
  // d1/6, d2, d3/2 of weno5.h (d1 = 2 a5 - 7 a3 + 11 a1, d2 = -a3 + 5 a1 + 2 b1,
  // d3 = 2 a1 + 5 b1 - b3)
  const double d1 = fma(a1, 11.0 / 6.0, fma(a3, -7.0 / 6.0, a5 * (1.0 / 3.0)));
  const double d2 = fma(b1, 2.0, fma(a1, 5.0, -a3));
  const double d3 = fma(b1, 2.5, fma(b3, -0.5, a1));
  const double num = fma(Z, d3, fma(Y, d2, X * d1));
  const double den = fma(X, 1.0 / 6.0, fma(Z, 0.5, Y));
  return (fabs(vsum) * kx) * (num * recip_nr(den));
}

// FP32 variant for the mixed-precision step.
//
// Inputs: the six velocity fields as float pairs (hi, lo) written once per step by
// k_split (split_pair: hi + lo holds q to about 2^-48).  A difference is formed as
// (hi1 - hi0) + (lo1 - lo0): accurate to float precision relative to the
// difference itself, as a double difference rounded to float would be, but
// on the FP32 pipe (converting each double where a stencil reads it put about
// thirteen conversions per point on GB300's FP64 pipe).
//
// The derivative is wdir's rearranged quotient in float.  The product-form
// weights scale like the 8th power of the differences, so float would underflow
// for smooth fields: the five differences are divided by their largest magnitude
// s first (the quotient is unchanged by a common scale; the result is multiplied
// back by s), and wdir's additive 1e-80/486 becomes 1e-80/486/s^8 in scaled
// units, evaluated as a power of two and clamped to [2^-126, 2^100].  The lower
// clamp keeps the denominator a normal float where all three smoothness
// indicators are 0 (data exactly linear in float: the quotient is then d2, the
// reference's limit); the upper keeps eps * d2 finite.  Differences below 2^-100
// (a flat stencil) give 0.
// The pair (hi, lo) of q from its bits, without FP64-pipe instructions (df::split_double:
// hi + lo holds q to about 2^-48 of q)
__device__ __forceinline__ float2 split_pair(double q) {
  const df::D d = df::split_double(q);
  return make_float2(d.h, d.l);
}
struct SplitSrc {
  const double* f[6];
};
// the split pairs of NF (3 or 6) fields, field f at out[f n ..]; the last three of
// six are skipped where *keep != 0 (their level's advection is carried over)
template <int NF>
__global__ void k_split(long n, SplitSrc src, float2* __restrict__ out, const int* __restrict__ keep) {
  const int nf = (NF == 6 && keep && *keep) ? 3 : NF;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int f = 0; f < NF; ++f)
      if (f < nf) out[f * n + t] = split_pair(__ldg(src.f[f] + t));
  }
}

__device__ __forceinline__ float lg2_approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float wdir_f32(const float2* __restrict__ q, long c, long S, float vsum, float kx) {
  if (vsum == 0.0f) return 0.0f;
  const long st = vsum > 0.0f ? S : -S;
  const float2* p = q + c - 3 * st;
  const float2 q0 = __ldg(p), q1 = __ldg(p + st), q2 = __ldg(p + 2 * st), q3 = __ldg(p + 3 * st),
               q4 = __ldg(p + 4 * st), q5 = __ldg(p + 5 * st);
  float a5 = (q1.x - q0.x) + (q1.y - q0.y), a3 = (q2.x - q1.x) + (q2.y - q1.y), a1 = (q3.x - q2.x) + (q3.y - q2.y),
        b1 = (q4.x - q3.x) + (q4.y - q3.y), b3 = (q5.x - q4.x) + (q5.y - q4.y);
  const float s = fmaxf(fmaxf(fmaxf(fabsf(a5), fabsf(a3)), fmaxf(fabsf(a1), fabsf(b1))), fabsf(b3));
  if (s < 0x1p-100f) return 0.0f;
  const float is = __fdividef(1.0f, s);
  a5 *= is;
  a3 *= is;
  a1 *= is;
  b1 *= is;
  b3 *= is;
  constexpr float c13 = 13.0f / 3.0f;
  float t1 = fmaf(a3, -2.0f, a5 + a1), t2 = fmaf(a3, -4.0f, fmaf(a1, 3.0f, a5));
  const float s1 = fmaf(t1 * c13, t1, t2 * t2);
  t1 = fmaf(a1, -2.0f, a3 + b1);
  t2 = a3 - b1;
  const float s2 = fmaf(t1 * c13, t1, t2 * t2);
  t1 = fmaf(b1, -2.0f, a1 + b3);
  t2 = fmaf(b1, -4.0f, fmaf(a1, 3.0f, b3));
  const float s3 = fmaf(t1 * c13, t1, t2 * t2);
  // log2(1e-80 / 486) = -274.679
  const float eps = ex2_approx(fminf(fmaxf(-274.679f - 8.0f * lg2_approx(s), -126.0f), 100.0f));
  const float x = s2 * s3, y = s1 * s3, z = s1 * s2;
  const float X = x * x, Y = fmaf(y, y, eps), Z = z * z;
  const float d1 = fmaf(a1, 11.0f / 6.0f, fmaf(a3, -7.0f / 6.0f, a5 * (1.0f / 3.0f)));
  const float d2 = fmaf(b1, 2.0f, fmaf(a1, 5.0f, -a3));
  const float d3 = fmaf(b1, 2.5f, fmaf(b3, -0.5f, a1));
  const float num = fmaf(Z, d3, fmaf(Y, d2, X * d1));
  const float den = fmaf(X, 1.0f / 6.0f, fmaf(Z, 0.5f, Y));
  return (fabsf(vsum) * kx) * (__fdividef(num, den) * s);
}
// sp: the split pair arrays of u, v, w (then uo, vo, wo for the second level); the
// second level is skipped where *keep != 0
__global__ void __launch_bounds__(128) k_weno2_f32(Grid g, int nlev, const int* __restrict__ keep, float kx,
                                                   float ky, float kz,
                                                   const float2* __restrict__ sp, double* __restrict__ au,
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
  for (int lev = 0; lev < nlev; ++lev) {
    if (lev == 1 && keep && *keep) break;
    const float2* U = sp + (long)(3 * lev) * g.n;
    const float2* V = U + g.n;
    const float2* W = V + g.n;
    auto h = [](const float2* a, long o) { return __ldg(&a[o].x); };
    const float u0 = h(U, c), uxm = h(U, c - X), uxp = h(U, c + X);
    const float v0 = h(V, c), vym = h(V, c - Y), vyp = h(V, c + Y);
    const float w0 = h(W, c), wzm = h(W, c - Z), wzp = h(W, c + Z);
    float a;
    a = wdir_f32(U, c, X, (uxm + u0) + (u0 + uxp), kx);
    a += wdir_f32(U, c, Y, (vym + h(V, c + X - Y)) + (v0 + h(V, c + X)), ky);
    a += wdir_f32(U, c, Z, (wzm + h(W, c + X - Z)) + (w0 + h(W, c + X)), kz);
    (lev ? auo : au)[c] = (double)a;
    a = wdir_f32(V, c, X, (uxm + h(U, c - X + Y)) + (u0 + h(U, c + Y)), kx);
    a += wdir_f32(V, c, Y, (vym + v0) + (v0 + vyp), ky);
    a += wdir_f32(V, c, Z, (wzm + h(W, c + Y - Z)) + (w0 + h(W, c + Y)), kz);
    (lev ? avo : av)[c] = (double)a;
    a = wdir_f32(W, c, X, (uxm + h(U, c - X + Z)) + (u0 + h(U, c + Z)), kx);
    a += wdir_f32(W, c, Y, (vym + h(V, c - Y + Z)) + (v0 + h(V, c + Z)), ky);
    a += wdir_f32(W, c, Z, (wzm + w0) + (w0 + wzp), kz);
    (lev ? awo : aw)[c] = (double)a;
  }
}

// One direction of the FP64-accurate step's WENO5 (df::wdir_core) on the split
// pairs of q; vsum as a pair
__device__ __forceinline__ df::D wdir_df(const float2* __restrict__ q, long c, long S, df::D vsum, df::D kx) {
  if (vsum.h == 0.0f) return {0.0f, 0.0f};
  const long st = vsum.h > 0.0f ? S : -S;
  const float2* p = q + c - 3 * st;
  df::D w[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const float2 v = __ldg(p + t * st);
    w[t] = {v.x, v.y};
  }
  return df::wdir_core(w, vsum, kx);
}
// The FP64-accurate step's WENO5 of one or both levels (as k_weno2) in FP32-pair
// arithmetic: sp holds the split pairs of u, v, w (then uo, vo, wo); each velocity
// sum and derivative is a pair, the three derivatives of a component are summed as
// pairs and the sum is rounded to a double once.  The nine (component, direction)
// derivatives of a level run as one loop that is not unrolled: fully inlined they
// made a loop body whose instruction fetch stalled the warps (the leading stall
// reason under ncu).  Line (q, d) advects component q along d with the velocity
// sum (Vd(c - Sd) + Vd(c - Sd + Sq)) + (Vd(c) + Vd(c + Sq)), Vd the d component,
// the same pairs in the same order as the unrolled form.
__global__ void __launch_bounds__(128) k_weno2_df(Grid g, int nlev, const int* __restrict__ keep, df::D kx,
                                                  df::D ky, df::D kz, const float2* __restrict__ sp,
                                                  double* __restrict__ au, double* __restrict__ av,
                                                  double* __restrict__ aw, double* __restrict__ auo,
                                                  double* __restrict__ avo, double* __restrict__ awo) {
  using df::add;
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
#pragma unroll 1
  for (int lev = 0; lev < nlev; ++lev) {
    if (lev == 1 && keep && *keep) break;
    const float2* U = sp + (long)(3 * lev) * g.n;
    const float2* V = U + g.n;
    const float2* W = V + g.n;
    auto h = [](const float2* a, long o) {
      const float2 v = __ldg(a + o);
      return df::D{v.x, v.y};
    };
    df::D a{0.0f, 0.0f};
#pragma unroll 1
    for (int line = 0; line < 9; ++line) {
      const int q = line / 3, d = line - 3 * q;
      const long Sq = q == 0 ? X : (q == 1 ? Y : Z), Sd = d == 0 ? X : (d == 1 ? Y : Z);
      const float2* Fd = d == 0 ? U : (d == 1 ? V : W);
      const df::D vsum = add(add(h(Fd, c - Sd), h(Fd, c - Sd + Sq)), add(h(Fd, c), h(Fd, c + Sq)));
      const df::D t = wdir_df(q == 0 ? U : (q == 1 ? V : W), c, Sd, vsum, d == 0 ? kx : (d == 1 ? ky : kz));
      a = d == 0 ? t : add(a, t);
      if (d == 2) {
        double* o = q == 0 ? (lev ? auo : au) : (q == 1 ? (lev ? avo : av) : (lev ? awo : aw));
        o[c] = df::to_double(a);
      }
    }
  }
}

__global__ void __launch_bounds__(128) k_weno2(Grid g, int nlev, const int* __restrict__ keep, double dxi,
                                               double dyi, double dzi,
                                               const double* __restrict__ u,
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
  const double kx = dxi * (1.0 / 24.0), ky = dyi * (1.0 / 24.0), kz = dzi * (1.0 / 24.0);
#pragma unroll 1
  for (int lev = 0; lev < nlev; ++lev) {
    if (lev == 1 && keep && *keep) break;
    const double* U = lev ? uo : u;
    const double* V = lev ? vo : v;
    const double* W = lev ? wo : w;
    const double u0 = __ldg(U + c), uxm = __ldg(U + c - X), uxp = __ldg(U + c + X);
    const double v0 = __ldg(V + c), vym = __ldg(V + c - Y), vyp = __ldg(V + c + Y);
    const double w0 = __ldg(W + c), wzm = __ldg(W + c - Z), wzp = __ldg(W + c + Z);
    double a;
    // u (cal_advu_weno5.f:80-120); each vsum is 4 times the reference's vel
    a = wdir(U, c, X, (uxm + u0) + (u0 + uxp), kx);
    a += wdir(U, c, Y, (vym + __ldg(V + c + X - Y)) + (v0 + __ldg(V + c + X)), ky);
    a += wdir(U, c, Z, (wzm + __ldg(W + c + X - Z)) + (w0 + __ldg(W + c + X)), kz);
    (lev ? auo : au)[c] = a;
    // v (:147-187)
    a = wdir(V, c, X, (uxm + __ldg(U + c - X + Y)) + (u0 + __ldg(U + c + Y)), kx);
    a += wdir(V, c, Y, (vym + v0) + (v0 + vyp), ky);
    a += wdir(V, c, Z, (wzm + __ldg(W + c + Y - Z)) + (w0 + __ldg(W + c + Y)), kz);
    (lev ? avo : av)[c] = a;
    // w (:214-254)
    a = wdir(W, c, X, (uxm + __ldg(U + c - X + Z)) + (u0 + __ldg(U + c + Z)), kx);
    a += wdir(W, c, Y, (vym + __ldg(V + c - Y + Z)) + (v0 + __ldg(V + c + Z)), ky);
    a += wdir(W, c, Z, (wzm + w0) + (w0 + wzp), kz);
    (lev ? awo : aw)[c] = a;
  }
}
}  // namespace

// One level (nlev = 1: u, v, w into adv) or both (nlev = 2: uo, vo, wo into advo as
// well); only interior cells are written (the fused step never reads the halo of
// the advection terms, which cal_advu_weno5.f:44-52 sets to zero).  prec: 0 FP64,
// 1 FP32, 2 FP32 pairs; the last two first write the split pairs of the 3 nlev
// fields into `split`.
static void weno5_levels(cudaStream_t s, const Grid& g, int nlev, double dxi, double dyi, double dzi,
                         const double* u, const double* v, const double* w, const double* uo, const double* vo,
                         const double* wo, double* const* adv, double* const* advo, int prec, float2* split,
                         const int* keep = nullptr) {
  dim3 b(32, 4, 1);
  dim3 gr((unsigned)((g.ni + 31) / 32), (unsigned)((g.nj + 3) / 4), (unsigned)g.nk);
  double* const ao[3] = {advo ? advo[0] : nullptr, advo ? advo[1] : nullptr, advo ? advo[2] : nullptr};
  if (prec == 1 || prec == 2) {
    if (!split) {
      set_status(FMF_ERR_ARG);
      return;
    }
    const SplitSrc src{{u, v, w, uo, vo, wo}};
    if (nlev == 2)
      k_split<6><<<152 * 8, 256, 0, s>>>(g.n, src, split, keep);
    else
      k_split<3><<<152 * 8, 256, 0, s>>>(g.n, src, split, nullptr);
    if (prec == 1)
      k_weno2_f32<<<gr, b, 0, s>>>(g, nlev, keep, (float)(dxi / 24.0), (float)(dyi / 24.0), (float)(dzi / 24.0),
                                   split, adv[0], adv[1], adv[2], ao[0], ao[1], ao[2]);
    else
      k_weno2_df<<<gr, b, 0, s>>>(g, nlev, keep, df::from_double_host(dxi / 24.0), df::from_double_host(dyi / 24.0),
                                  df::from_double_host(dzi / 24.0), split, adv[0], adv[1], adv[2], ao[0], ao[1],
                                  ao[2]);
    count_launch(2);
    return;
  }
  if (prec != 0) {
    set_status(FMF_ERR_ARG);
    return;
  }
  k_weno2<<<gr, b, 0, s>>>(g, nlev, keep, dxi, dyi, dzi, u, v, w, uo, vo, wo, adv[0], adv[1], adv[2], ao[0], ao[1],
                           ao[2]);
  count_launch();
}

void weno5_both(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u,
                const double* v, const double* w, const double* uo, const double* vo, const double* wo,
                double* const* adv, double* const* advo, int prec, float2* split) {
  weno5_levels(s, g, 2, dxi, dyi, dzi, u, v, w, uo, vo, wo, adv, advo, prec, split);
}

void weno5_one(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
               const double* w, double* const* adv, int prec, float2* split) {
  weno5_levels(s, g, 1, dxi, dyi, dzi, u, v, w, nullptr, nullptr, nullptr, adv, nullptr, prec, split);
}
void split3(cudaStream_t s, const Grid& g, const double* a, const double* b, const double* c, float2* out) {
  const SplitSrc src{{a, b, c, nullptr, nullptr, nullptr}};
  k_split<3><<<152 * 8, 256, 0, s>>>(g.n, src, out, nullptr);
  count_launch();
}

void weno5_keep(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
                const double* w, const double* uo, const double* vo, const double* wo, double* const* adv,
                double* const* advo, const int* keep, int prec, float2* split) {
  weno5_levels(s, g, 2, dxi, dyi, dzi, u, v, w, uo, vo, wo, adv, advo, prec, split, keep);
}

// n doubles of both signs spread over magnitudes 2^-96 .. 2^127 with pseudo-random
// significands; the largest |(hi + lo) - q| / |q| of their split pairs, as the
// ordered bits of a non-negative double
__global__ void k_check_split(long n, unsigned long long* worst) {
  unsigned long long m = 0;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    unsigned long long h = (unsigned long long)t * 0x9E3779B97F4A7C15ull;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    const long long e = 1023 - 96 + (long long)(t % 223);
    const long long sg = (t & 1) ? (1ll << 63) : 0;
    const double q = __longlong_as_double((long long)(sg | (e << 52) | (long long)(h & 0xFFFFFFFFFFFFFull)));
    const float2 p = split_pair(q);
    const double rel = fabs(((double)p.x + (double)p.y) - q) / fabs(q);
    const unsigned long long b = (unsigned long long)__double_as_longlong(rel);
    m = b > m ? b : m;
  }
  atomicMax(worst, m);
}

}  // namespace fused
}  // namespace fmf

// The split pairs of the mixed-precision WENO5 against the doubles they split:
// largest relative error of hi + lo over n values of 2^-96 .. 2^127 (both signs).
// Verification support; no counterpart in the reference.
extern "C" int fmf_check_split_pair(long long n, double* max_rel_err) {
  if (!max_rel_err || n <= 0) return FMF_ERR_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return FMF_ERR_NOMEM;
  cudaMemset(d, 0, sizeof(unsigned long long));
  fmf::fused::k_check_split<<<152 * 4, 256>>>((long)n, d);
  fmf::count_launch();
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return FMF_ERR_CUDA;
  std::memcpy(max_rel_err, &h, sizeof(double));
  return FMF_OK;
}
