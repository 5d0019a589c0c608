// fused_visc.cu -- the implicit viscous solve of the fused step (solu_sor4.f with
// the coefficients of cal_arith_coef_vis.f / cal_harm_coef_vis.f).
//
// The 45 coefficient arrays are products of six viscosities and constant grid
// factors (cal_arith_coef_vis.f:211-231): for u at (i+1/2,j,k) the x-viscosities
// are the cell values mu(i), mu(i+1) and the y/z ones are edge means shared with
// the neighbours.  k_edges stores the three edge means once per step (the same
// 4-cell sums, in the same order, as the reference) and k_src_ab, per component,
// A = 0.5/(rho00*D) and B = src/D with D = 1/dt + 0.5*a_p/rho00, so a point update
// of solu_sor4.f:150-170 becomes q_new = A*visn + B with visn the 14-neighbour sum.
// Colours are processed in their independent pairs (1,2) (3,4) (5,6) (7,8): two
// colours that differ in every index parity never read each other, so one launch
// per pair gives the sequential result.  The wall/halo refresh after every second
// colour (bndu + bnd_periodic of the swept component, solu_sor4.f:176-180) is one
// kernel (k_refresh; three ordered plane kernels on grids under 8 cells a side).
//
// The mixed-precision step solves the same system by one step of iterative
// refinement: the residual of the first sweep is formed in FP64 at u, then the
// sweeps run in FP32 on the correction d = un - u (FP32 storage and arithmetic),
// and un = u + d is formed in FP64 at the end.
#include <cstdlib>

#include "df64.cuh"
#include "fused.cuh"
#include "recip.cuh"
#include "refresh.cuh"

namespace fmf {
namespace fused {

namespace {
struct VP {
  double dtinv, dx2, dy2, dz2, dxy, dxz, dyz;
  int harmonic;
};

__device__ __forceinline__ double mean4(double a, double b, double c, double d, int harm) {
  if (!harm) return 0.25 * (a + b + c + d);
  return 4.0 / (1.0 / a + 1.0 / b + 1.0 / c + 1.0 / d);
}

// Edge viscosities over i,j,k in 0..n, then A/B per component over the interior.
// f[0..2] non-null: FP32 copies of the three edge arrays as well.
struct F3 {
  float* f[3];
};
__global__ void __launch_bounds__(256) k_edges(Grid g, VP p, const double* __restrict__ mu, double* __restrict__ exy,
                                               double* __restrict__ exz, double* __restrict__ eyz, F3 f) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double m0 = __ldg(mu + c), mx = __ldg(mu + c + X), my = __ldg(mu + c + Y), mz = __ldg(mu + c + Z);
  const double a = mean4(m0, mx, my, __ldg(mu + c + X + Y), p.harmonic);
  const double b = mean4(m0, mx, mz, __ldg(mu + c + X + Z), p.harmonic);
  const double d = mean4(m0, my, mz, __ldg(mu + c + Y + Z), p.harmonic);
  exy[c] = a;
  exz[c] = b;
  eyz[c] = d;
  if (f.f[0]) {
    f.f[0][c] = (float)a;
    f.f[1][c] = (float)b;
    f.f[2][c] = (float)d;
  }
}

// cal_srcu.f:53-137 fused with the update factors: src is formed in registers and
// only A = 0.5/(rho00*D), B = src/D are stored.  With T = 1/(rho00/dt + a_p/2)
// these are A = T/2 and B = (rho00*(explicit terms) - prs + vis/2)*T: one
// reciprocal per component (recip_nr: Newton-Raphson, no division).
struct SrcIn {
  const double *u, *v, *w, *rho, *rhon, *adv[3], *advo[3], *prs[3], *vis[3], *fst[3], *fstn[3];
  double grvb, grvp;
};
// Outputs: FP64 A and B per component, or (REFINE) FP32 A and the FP64 first-sweep
// residual R = A*visn(u) + B - u rounded to FP32 (the right-hand side of the
// correction sweeps of the mixed-precision solve).
struct ABOut {
  double *a[3], *b[3];
  float *af[3], *rf[3];
};
template <int COMP, class T>
__device__ __forceinline__ T visn_at(const Grid& g, const VP& p, long c, const T* __restrict__ mu,
                                     const T* __restrict__ exy, const T* __restrict__ exz,
                                     const T* __restrict__ eyz, const T* un, const T* vn, const T* wn);
template <bool REFINE>
__global__ void __launch_bounds__(256) k_src_ab(Grid g, VP p, SrcIn in, const double* __restrict__ mu,
                                                const double* __restrict__ exy, const double* __restrict__ exz,
                                                const double* __restrict__ eyz, ABOut out) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double r0 = __ldg(in.rho + c), n0 = __ldg(in.rhon + c);
  // rho00 * src
  auto rsrc = [&](int q, const double* vel, double r, double grav) {
    return r * (__ldg(vel + c) * p.dtinv - __ldg(in.adv[q] + c) * 1.5 + __ldg(in.advo[q] + c) * 0.5 +
                __ldg(in.fst[q] + c) * 0.5 + __ldg(in.fstn[q] + c) * 0.5 + grav) -
           __ldg(in.prs[q] + c) + __ldg(in.vis[q] + c) * 0.5;
  };
  auto store = [&](int q, double A, double B, double visn, const double* vel) {
    if (REFINE) {
      out.af[q][c] = (float)A;
      out.rf[q][c] = (float)(A * visn + B - __ldg(vel + c));
    } else {
      out.a[q][c] = A;
      out.b[q][c] = B;
    }
  };
  {
    const double r = (r0 + __ldg(in.rho + c + X) + n0 + __ldg(in.rhon + c + X)) * 0.25;
    const double ap = p.dz2 * __ldg(exz + c - Z) + p.dy2 * __ldg(exy + c - Y) + p.dx2 * __ldg(mu + c) * 2.0 +
                      p.dx2 * __ldg(mu + c + X) * 2.0 + p.dy2 * __ldg(exy + c) + p.dz2 * __ldg(exz + c);
    const double T = recip_nr(r * p.dtinv + ap * 0.5);
    const double vn = REFINE ? visn_at<0, double>(g, p, c, mu, exy, exz, eyz, in.u, in.v, in.w) : 0.0;
    store(0, 0.5 * T, rsrc(0, in.u, r, in.grvb) * T, vn, in.u);
  }
  if (j <= g.nj - 1) {
    const double r = (r0 + __ldg(in.rho + c + Y) + n0 + __ldg(in.rhon + c + Y)) * 0.25;
    const double ap = p.dz2 * __ldg(eyz + c - Z) + p.dy2 * __ldg(mu + c) * 2.0 + p.dx2 * __ldg(exy + c - X) +
                      p.dx2 * __ldg(exy + c) + p.dy2 * __ldg(mu + c + Y) * 2.0 + p.dz2 * __ldg(eyz + c);
    const double T = recip_nr(r * p.dtinv + ap * 0.5);
    const double vn = REFINE ? visn_at<1, double>(g, p, c, mu, exy, exz, eyz, in.u, in.v, in.w) : 0.0;
    store(1, 0.5 * T, rsrc(1, in.v, r, in.grvp) * T, vn, in.v);
  }
  {
    const double r = (r0 + __ldg(in.rho + c + Z) + n0 + __ldg(in.rhon + c + Z)) * 0.25;
    const double ap = p.dz2 * __ldg(mu + c) * 2.0 + p.dy2 * __ldg(eyz + c - Y) + p.dx2 * __ldg(exz + c - X) +
                      p.dx2 * __ldg(exz + c) + p.dy2 * __ldg(eyz + c) + p.dz2 * __ldg(mu + c + Z) * 2.0;
    const double T = recip_nr(r * p.dtinv + ap * 0.5);
    const double vn = REFINE ? visn_at<2, double>(g, p, c, mu, exy, exz, eyz, in.u, in.v, in.w) : 0.0;
    store(2, 0.5 * T, rsrc(2, in.w, r, 0.0) * T, vn, in.w);
  }
}

// k_src_ab with A and B in FP32-pair arithmetic (each double read split into a
// pair, A and B rounded to doubles once).  The FP64-accurate step (FMF_FP64E, REFINE
// false) stores them.  The mixed-precision step (REFINE true) forms the first-sweep
// residual R = A visn(u) + B - u from them in FP64, as k_src_ab<true> does: the
// viscous sum visn reads 20 doubles for about 25 operations, and with it in pairs
// as well the kernel measured 10.2 ms against 9.7 for k_src_ab<true> at
// 512x256x256 (the splits cost more than the FP64 operations they replace); in
// this form, 6.7 ms.  The momentum-factor denominator is
// grouped as dz2 (e(-Z) + e(0)) + dy2 (e(-Y) + e(0)) + 2 dx2 (mu(0) + mu(X)) (and
// likewise per component), the same sum.
struct VPS {
  df::D dtinv, dx2, dy2, dz2, dx2x2, dy2x2, dz2x2, grvb, grvp;
};
template <bool REFINE>
__global__ void __launch_bounds__(256) k_src_ab_e(Grid g, VPS p, VP pd, SrcIn in, const double* __restrict__ mu,
                                                  const double* __restrict__ exy, const double* __restrict__ exz,
                                                  const double* __restrict__ eyz, ABOut out) {
  using namespace df;
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  auto L = [&](const double* a, long o) { return split_double(__ldg(a + c + o)); };
  const D r0n0 = add(L(in.rho, 0), L(in.rhon, 0)), mu0 = L(mu, 0);
  // rho00 * src
  auto rsrc = [&](int q, const double* vel, D r, D grav) {
    D t = sub(mul(L(vel, 0), p.dtinv), mulf(L(in.adv[q], 0), 1.5f));
    t = add(t, scale(add(add(L(in.advo[q], 0), L(in.fst[q], 0)), L(in.fstn[q], 0)), 0.5f));
    t = add(t, grav);
    return add(sub(mul(r, t), L(in.prs[q], 0)), scale(L(in.vis[q], 0), 0.5f));
  };
  // A = T/2, B = rs T; REFINE: A and R = A visn + B - u (FP64) as floats
  auto store = [&](int q, D r, D ap, D rs, double vn, const double* vel) {
    const D T = div(D{1.0f, 0.0f}, add(mul(r, p.dtinv), scale(ap, 0.5f)));
    const double A = to_double(scale(T, 0.5f)), B = to_double(mul(rs, T));
    if (REFINE) {
      out.af[q][c] = (float)A;
      out.rf[q][c] = (float)(A * vn + B - __ldg(vel + c));
    } else {
      out.a[q][c] = A;
      out.b[q][c] = B;
    }
  };
  const D zero{0.0f, 0.0f};
  {
    const D r = scale(add(r0n0, add(L(in.rho, X), L(in.rhon, X))), 0.25f);
    D ap = mul(p.dz2, add(L(exz, -Z), L(exz, 0)));
    ap = add(ap, mul(p.dy2, add(L(exy, -Y), L(exy, 0))));
    ap = add(ap, mul(p.dx2x2, add(mu0, L(mu, X))));
    const double vn = REFINE ? visn_at<0, double>(g, pd, c, mu, exy, exz, eyz, in.u, in.v, in.w) : 0.0;
    store(0, r, ap, rsrc(0, in.u, r, p.grvb), vn, in.u);
  }
  if (j <= g.nj - 1) {
    const D r = scale(add(r0n0, add(L(in.rho, Y), L(in.rhon, Y))), 0.25f);
    D ap = mul(p.dz2, add(L(eyz, -Z), L(eyz, 0)));
    ap = add(ap, mul(p.dy2x2, add(mu0, L(mu, Y))));
    ap = add(ap, mul(p.dx2, add(L(exy, -X), L(exy, 0))));
    const double vn = REFINE ? visn_at<1, double>(g, pd, c, mu, exy, exz, eyz, in.u, in.v, in.w) : 0.0;
    store(1, r, ap, rsrc(1, in.v, r, p.grvp), vn, in.v);
  }
  {
    const D r = scale(add(r0n0, add(L(in.rho, Z), L(in.rhon, Z))), 0.25f);
    D ap = mul(p.dz2x2, add(mu0, L(mu, Z)));
    ap = add(ap, mul(p.dy2, add(L(eyz, -Y), L(eyz, 0))));
    ap = add(ap, mul(p.dx2, add(L(exz, -X), L(exz, 0))));
    const double vn = REFINE ? visn_at<2, double>(g, pd, c, mu, exy, exz, eyz, in.u, in.v, in.w) : 0.0;
    store(2, r, ap, rsrc(2, in.w, r, zero), vn, in.w);
  }
}

// The explicit viscous term 2 div(mu S) of main.f90:538-541 (calsij, cal_arith_tau,
// cal_div_tensor) for the interior u, v, w points, which are all the step reads.
// k_stress forms the six stresses over i, j, k in 0..n+1 (the points the interior
// divergence reads) straight from u, v, w and mu: tau_ii = 2 mu S_ii and, on the
// edges, tau_ij = 2 (mean of 4 mu) S_ij with S_ij = (du_i/dx_j + du_j/dx_i)/2,
// the factors 2, 1/2 and 1/4 folded into the constants; the strain never goes
// through memory.  k_div_stress takes its divergence on the interior.
// (sk, optional: the six strain components of calsij.f:28-139 at the same points,
// kept by the adjoint's record of the step)
__global__ void __launch_bounds__(256) k_stress(Grid g, double dxi, double dyi, double dzi,
                                                const double* __restrict__ u, const double* __restrict__ v,
                                                const double* __restrict__ w, const double* __restrict__ mu,
                                                double* __restrict__ tau, double* __restrict__ sk) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = (int)blockIdx.z;
  if (i > g.ni + 1 || j > g.nj + 1) return;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  const double m0 = __ldg(mu + c), mx = __ldg(mu + c + X), my = __ldg(mu + c + Y), mz = __ldg(mu + c + Z);
  const double u0 = __ldg(u + c), v0 = __ldg(v + c), w0 = __ldg(w + c);
  const double hx = 0.25 * dxi, hy = 0.25 * dyi, hz = 0.25 * dzi;
  tau[c] = (u0 - __ldg(u + c - X)) * m0 * (2.0 * dxi);
  tau[c + n] = (v0 - __ldg(v + c - Y)) * m0 * (2.0 * dyi);
  tau[c + 2 * n] = (w0 - __ldg(w + c - Z)) * m0 * (2.0 * dzi);
  tau[c + 3 * n] = ((__ldg(u + c + Y) - u0) * hy + (__ldg(v + c + X) - v0) * hx) *
                   ((m0 + mx) + (my + __ldg(mu + c + X + Y)));
  tau[c + 4 * n] = ((__ldg(u + c + Z) - u0) * hz + (__ldg(w + c + X) - w0) * hx) *
                   ((m0 + mx) + (mz + __ldg(mu + c + X + Z)));
  tau[c + 5 * n] = ((__ldg(v + c + Z) - v0) * hz + (__ldg(w + c + Y) - w0) * hy) *
                   ((m0 + my) + (mz + __ldg(mu + c + Y + Z)));
  if (sk) {
    sk[c] = (u0 - __ldg(u + c - X)) * dxi;
    sk[c + n] = (v0 - __ldg(v + c - Y)) * dyi;
    sk[c + 2 * n] = (w0 - __ldg(w + c - Z)) * dzi;
    sk[c + 3 * n] = ((__ldg(u + c + Y) - u0) * dyi + (__ldg(v + c + X) - v0) * dxi) * 0.5;
    sk[c + 4 * n] = ((__ldg(u + c + Z) - u0) * dzi + (__ldg(w + c + X) - w0) * dxi) * 0.5;
    sk[c + 5 * n] = ((__ldg(v + c + Z) - v0) * dzi + (__ldg(w + c + Y) - w0) * dyi) * 0.5;
  }
}
__global__ void __launch_bounds__(256) k_div_stress(Grid g, double dxi, double dyi, double dzi,
                                                    const double* __restrict__ t, double* __restrict__ vu,
                                                    double* __restrict__ vv, double* __restrict__ vw) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  const double* t1 = t;
  const double* t2 = t + n;
  const double* t3 = t + 2 * n;
  const double* t4 = t + 3 * n;
  const double* t5 = t + 4 * n;
  const double* t6 = t + 5 * n;
  const double a4 = __ldg(t4 + c), a5 = __ldg(t5 + c), a6 = __ldg(t6 + c);
  vu[c] = (__ldg(t1 + c + X) - __ldg(t1 + c)) * dxi + (a4 - __ldg(t4 + c - Y)) * dyi + (a5 - __ldg(t5 + c - Z)) * dzi;
  vv[c] = (a4 - __ldg(t4 + c - X)) * dxi + (__ldg(t2 + c + Y) - __ldg(t2 + c)) * dyi + (a6 - __ldg(t6 + c - Z)) * dzi;
  vw[c] = (a5 - __ldg(t5 + c - X)) * dxi + (a6 - __ldg(t6 + c - Y)) * dyi + (__ldg(t3 + c + Z) - __ldg(t3 + c)) * dzi;
}

// The FP64-accurate and mixed-precision steps: k_stress and k_div_stress in
// FP32-pair arithmetic (each double read split into a pair, each output rounded to
// a double once); the same sums in the same grouping.
// With sk (the adjoint's record of a mixed-precision step) the strain components
// are written as well, in FP64 as k_stress forms them.
struct VPT {
  df::D dxi2, dyi2, dzi2, hx, hy, hz, dxi, dyi, dzi;  // 2 dxi, ..., dxi/4, ..., dxi, ...
  double dxd, dyd, dzd;                               // dxi, dyi, dzi (the strain in FP64)
};
__global__ void __launch_bounds__(256) k_stress_e(Grid g, VPT p, const double* __restrict__ u,
                                                  const double* __restrict__ v, const double* __restrict__ w,
                                                  const double* __restrict__ mu, double* __restrict__ tau,
                                                  double* __restrict__ sk) {
  using namespace df;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = (int)blockIdx.z;
  if (i > g.ni + 1 || j > g.nj + 1) return;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  auto L = [&](const double* a, long o) { return split_double(__ldg(a + c + o)); };
  const D m0 = L(mu, 0), mx = L(mu, X), my = L(mu, Y), mz = L(mu, Z);
  const D u0 = L(u, 0), v0 = L(v, 0), w0 = L(w, 0);
  tau[c] = to_double(mul(mul(sub(u0, L(u, -X)), m0), p.dxi2));
  tau[c + n] = to_double(mul(mul(sub(v0, L(v, -Y)), m0), p.dyi2));
  tau[c + 2 * n] = to_double(mul(mul(sub(w0, L(w, -Z)), m0), p.dzi2));
  tau[c + 3 * n] = to_double(mul(add(mul(sub(L(u, Y), u0), p.hy), mul(sub(L(v, X), v0), p.hx)),
                                 add(add(m0, mx), add(my, L(mu, X + Y)))));
  tau[c + 4 * n] = to_double(mul(add(mul(sub(L(u, Z), u0), p.hz), mul(sub(L(w, X), w0), p.hx)),
                                 add(add(m0, mx), add(mz, L(mu, X + Z)))));
  tau[c + 5 * n] = to_double(mul(add(mul(sub(L(v, Z), v0), p.hz), mul(sub(L(w, Y), w0), p.hy)),
                                 add(add(m0, my), add(mz, L(mu, Y + Z)))));
  if (sk) {
    const double dxi = p.dxd, dyi = p.dyd, dzi = p.dzd;
    const double ud = __ldg(u + c), vd = __ldg(v + c), wd = __ldg(w + c);
    sk[c] = (ud - __ldg(u + c - X)) * dxi;
    sk[c + n] = (vd - __ldg(v + c - Y)) * dyi;
    sk[c + 2 * n] = (wd - __ldg(w + c - Z)) * dzi;
    sk[c + 3 * n] = ((__ldg(u + c + Y) - ud) * dyi + (__ldg(v + c + X) - vd) * dxi) * 0.5;
    sk[c + 4 * n] = ((__ldg(u + c + Z) - ud) * dzi + (__ldg(w + c + X) - wd) * dxi) * 0.5;
    sk[c + 5 * n] = ((__ldg(v + c + Z) - vd) * dzi + (__ldg(w + c + Y) - wd) * dyi) * 0.5;
  }
}
__global__ void __launch_bounds__(256) k_div_stress_e(Grid g, VPT p, const double* __restrict__ t,
                                                      double* __restrict__ vu, double* __restrict__ vv,
                                                      double* __restrict__ vw) {
  using namespace df;
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  auto L = [&](int q, long o) { return split_double(__ldg(t + q * n + c + o)); };
  const D a4 = L(3, 0), a5 = L(4, 0), a6 = L(5, 0);
  vu[c] = to_double(add(add(mul(sub(L(0, X), L(0, 0)), p.dxi), mul(sub(a4, L(3, -Y)), p.dyi)),
                        mul(sub(a5, L(4, -Z)), p.dzi)));
  vv[c] = to_double(add(add(mul(sub(a4, L(3, -X)), p.dxi), mul(sub(L(1, Y), L(1, 0)), p.dyi)),
                        mul(sub(a6, L(5, -Z)), p.dzi)));
  vw[c] = to_double(add(add(mul(sub(a5, L(4, -X)), p.dxi), mul(sub(a6, L(5, -Y)), p.dyi)),
                        mul(sub(L(2, Z), L(2, 0)), p.dzi)));
}

// One colour pair of one component.  Thread (a, b, kk) covers, for the pair whose
// first colour has parities (pi,pj,pk), the point (pi+2a, pj+2b, pk+2kk) and the
// point of the second colour (all parities flipped) at (pi'+2a, pj'+2b, pk'+2kk).
// T is the storage type of the iterates and coefficients and the arithmetic type.
//
// visn of component COMP at point c (solu_sor4.f:150-170 without the A/B factors)
template <int COMP, class T>
__device__ __forceinline__ T visn_at(const Grid& g, const VP& p, long c, const T* __restrict__ mu,
                                     const T* __restrict__ exy, const T* __restrict__ exz,
                                     const T* __restrict__ eyz, const T* un, const T* vn, const T* wn) {
  const long X = 1, Y = g.sy, Z = g.sz;
  const T dx2 = (T)p.dx2, dy2 = (T)p.dy2, dz2 = (T)p.dz2, dxy = (T)p.dxy, dxz = (T)p.dxz, dyz = (T)p.dyz;
  auto U = [&](long o) { return un[c + o]; };
  auto V = [&](long o) { return vn[c + o]; };
  auto W = [&](long o) { return wn[c + o]; };
  auto M = [&](const T* a, long o) { return __ldg(a + c + o); };
  if (COMP == 0) {
    const T ym = M(exy, -Y), yp = M(exy, 0), zm = M(exz, -Z), zp = M(exz, 0);
    return dz2 * (zm * U(-Z) + zp * U(Z)) + dy2 * (ym * U(-Y) + yp * U(Y)) +
           (T)2 * dx2 * (M(mu, 0) * U(-X) + M(mu, X) * U(X)) + dxy * (ym * (V(-Y) - V(X - Y)) + yp * (V(X) - V(0))) +
           dxz * (zm * (W(-Z) - W(X - Z)) + zp * (W(X) - W(0)));
  } else if (COMP == 1) {
    const T xm = M(exy, -X), xp = M(exy, 0), zm = M(eyz, -Z), zp = M(eyz, 0);
    return dz2 * (zm * V(-Z) + zp * V(Z)) + (T)2 * dy2 * (M(mu, 0) * V(-Y) + M(mu, Y) * V(Y)) +
           dx2 * (xm * V(-X) + xp * V(X)) + dxy * (xm * (U(-X) - U(-X + Y)) + xp * (U(Y) - U(0))) +
           dyz * (zm * (W(-Z) - W(Y - Z)) + zp * (W(Y) - W(0)));
  } else {
    const T xm = M(exz, -X), xp = M(exz, 0), ym = M(eyz, -Y), yp = M(eyz, 0);
    return (T)2 * dz2 * (M(mu, 0) * W(-Z) + M(mu, Z) * W(Z)) + dy2 * (ym * W(-Y) + yp * W(Y)) +
           dx2 * (xm * W(-X) + xp * W(X)) + dxz * (xm * (U(-X) - U(-X + Z)) + xp * (U(Z) - U(0))) +
           dyz * (ym * (V(-Y) - V(-Y + Z)) + yp * (V(Z) - V(0)));
  }
}

// T = double: the FP64 step, q_new = A*visn(q) + B on the velocity itself.
// T = float: the mixed-precision step, d_new = A*visn(d) + R on the correction
// d = un - u (R is the FP64 first-sweep residual; see refine_prep).
// part[block] = the block's sum of (q_new - q)^2.
template <int COMP, class T>
__global__ void __launch_bounds__(256) k_pair(Grid g, VP p, int pi, int pj, int pk, const T* __restrict__ mu,
                                              const T* __restrict__ exy, const T* __restrict__ exz,
                                              const T* __restrict__ eyz, const T* __restrict__ A,
                                              const T* __restrict__ B, T* un, T* vn, T* wn,
                                              double* __restrict__ part) {
  __shared__ T sh[8];
  const int jmax = COMP == 1 ? g.nj - 1 : g.nj;
  T* q = COMP == 0 ? un : (COMP == 1 ? vn : wn);
  T e = 0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = (h ? 3 - pi : pi) + 2 * (int)(blockIdx.x * 32 + threadIdx.x);
    const int j = (h ? 3 - pj : pj) + 2 * (int)(blockIdx.y * 8 + threadIdx.y);
    const int k = (h ? 3 - pk : pk) + 2 * (int)blockIdx.z;
    if (i > g.ni || j > jmax || k > g.nk) continue;
    const long c = g.at(i, j, k);
    const T visn = visn_at<COMP, T>(g, p, c, mu, exy, exz, eyz, un, vn, wn);
    const T qn = __ldg(A + c) * visn + __ldg(B + c);
    const T d = qn - q[c];
    q[c] = qn;
    e += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if (threadIdx.x == 0) sh[threadIdx.y] = e;
  __syncthreads();
  if (threadIdx.y == 0 && threadIdx.x == 0) {
    T t = 0;
    for (int w = 0; w < 8; ++w) t += sh[w];
    part[((long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = (double)t;
  }
}

// --- wall/halo refresh: bndu(un,vn,wn) then bnd_periodic(swept component) ----------
// k_wall_coef: Navier-slip coefficients c1, c2 per wall point (bndu.f:39-45), constant
// during the solve (phi, l1, l2 do not change).  Layout wc[side][k+2][i+2][2].
__global__ void __launch_bounds__(256) k_wall_coef(Grid g, double dy, const double* __restrict__ l1,
                                                   const double* __restrict__ l2, const double* __restrict__ phi,
                                                   double* __restrict__ wc) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int kk = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || kk > 2 * (g.nk + 6) - 3) return;
  const int side = kk >= g.nk + 4 ? 1 : 0;
  const int k = side ? kk - (g.nk + 6) : kk;
  const int jw = side ? g.nj : 1;
  const double pa = (phi[g.at(i, jw, k)] + phi[g.at((i + 1) % (g.ni + 3), jw, k)]) / 2.0;
  const double i1 = pa / l1[g.at(i, jw, k)], i2 = (1.0 - pa) / l2[g.at(i, jw, k)];
  const double ls = 1.0 / (i1 + i2);
  const long o = (((long)side * (g.nk + 6) + (k + 2)) * (g.ni + 6) + (i + 2)) * 2;
  wc[o] = (2.0 * dy) / (2.0 * ls + dy);
  wc[o + 1] = (2.0 * ls - dy) / (2.0 * ls + dy);
}
// The three refresh kernels issue every load of a thread before its first store: in
// each of them the points written and the points read are disjoint (ghost rows are
// written from interior rows; halo copies read rows the same kernel never writes),
// so this is the sequential result with one memory round trip per thread.
__global__ void __launch_bounds__(256) k_wall(Grid g, double uwall, const double* __restrict__ wc,
                                              double* __restrict__ uk, double* __restrict__ vk,
                                              double* __restrict__ wk) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int kk = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || kk > 2 * (g.nk + 6) - 3) return;
  const int side = kk >= g.nk + 4 ? 1 : 0;
  const int k = side ? kk - (g.nk + 6) : kk;
  const int NJ = g.nj;
  const long o = (((long)side * (g.nk + 6) + (k + 2)) * (g.ni + 6) + (i + 2)) * 2;
  const double c1 = wc[o], c2 = wc[o + 1];
  const long Y = g.sy;
  if (!side) {
    const long c = g.at(i, 1, k);
    const double u1 = uk[c], v1 = vk[c], v2 = vk[c + Y], w1 = wk[c];
    const double u0 = fma(c2, u1, c1 * (-uwall));  // one contraction, the same in k_refresh
    const double um1 = 2.0 * u0 - u1;
    uk[c - Y] = u0;
    uk[c - 2 * Y] = um1;
    uk[c - 3 * Y] = 2.0 * um1 - u0;
    vk[c - 3 * Y] = -v2;
    vk[c - 2 * Y] = -v1;
    vk[c - Y] = 0.0;
    const double w0 = c2 * w1;
    const double wm1 = 2.0 * w0 - w1;
    wk[c - Y] = w0;
    wk[c - 2 * Y] = wm1;
    wk[c - 3 * Y] = 2.0 * wm1 - w0;
  } else {
    const long c = g.at(i, NJ, k);
    const double u1 = uk[c], w1 = wk[c];
    const double vm1 = vk[c - Y], vm2 = vk[c - 2 * Y], vm3 = vk[c - 3 * Y];
    const double u0 = fma(c2, u1, c1 * uwall);
    const double up2 = 2.0 * u0 - u1;
    uk[c + Y] = u0;
    uk[c + 2 * Y] = up2;
    uk[c + 3 * Y] = 2.0 * up2 - u0;
    vk[c] = 0.0;
    vk[c + Y] = -vm1;
    vk[c + 2 * Y] = -vm2;
    vk[c + 3 * Y] = -vm3;
    const double w0 = c2 * w1;
    const double wp2 = 2.0 * w0 - w1;
    wk[c + Y] = w0;
    wk[c + 2 * Y] = wp2;
    wk[c + 3 * Y] = 2.0 * wp2 - w0;
  }
}
// x halos of all three components.  Bit c of `normal` set: component c gets the
// plain periodic copy (bnd_periodic applied after bndu overwrites bndu's halos);
// clear: bndu's copy, which for u is shifted by one (bndu.f:107-109).
__global__ void __launch_bounds__(256) k_halo_x(Grid g, int normal, double* __restrict__ uk,
                                                double* __restrict__ vk, double* __restrict__ wk) {
  const int j = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (j > g.nj + 3 || k > g.nk + 3) return;
  const int NI = g.ni;
  const long r = g.at(0, j, k);
  double* q[3] = {uk, vk, wk};
  const bool shifted = !(normal & 1);
  // sources of the destinations -2, -1, 0, ni+1, ni+2, ni+3 (offsets from r);
  // bndu's u: u(0)=u(ni+1), u(-1)=u(ni), u(-2)=u(ni-1), u(ni+1) untouched
  double t[3][6];
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    const double* a = q[cmp];
    const int sh = (cmp == 0 && shifted) ? 1 : 0;
    t[cmp][0] = a[r + NI - 2 + sh];
    t[cmp][1] = a[r + NI - 1 + sh];
    t[cmp][2] = a[r + NI + sh];
    t[cmp][3] = sh ? 0.0 : a[r + 1];
    t[cmp][4] = a[r + 2];
    t[cmp][5] = a[r + 3];
  }
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    double* a = q[cmp];
    a[r - 2] = t[cmp][0];
    a[r - 1] = t[cmp][1];
    a[r] = t[cmp][2];
    if (!(cmp == 0 && shifted)) a[r + NI + 1] = t[cmp][3];
    a[r + NI + 2] = t[cmp][4];
    a[r + NI + 3] = t[cmp][5];
  }
}
// z halos; for w bndu's copy is shifted by one (bndu.f:144-146).
__global__ void __launch_bounds__(256) k_halo_z(Grid g, int normal, double* __restrict__ uk,
                                                double* __restrict__ vk, double* __restrict__ wk) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || j > g.nj + 3) return;
  const int NK = g.nk;
  const long Z = g.sz;
  const long r = g.at(i, j, 0);
  double* q[3] = {uk, vk, wk};
  const bool shifted = !(normal & 4);
  // bndu's w: w(0)=w(nk+1), w(-1)=w(nk), w(-2)=w(nk-1), w(nk+1) untouched
  double t[3][6];
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    const double* a = q[cmp];
    const int sh = (cmp == 2 && shifted) ? 1 : 0;
    t[cmp][0] = a[r + (NK - 2 + sh) * Z];
    t[cmp][1] = a[r + (NK - 1 + sh) * Z];
    t[cmp][2] = a[r + (NK + sh) * Z];
    t[cmp][3] = sh ? 0.0 : a[r + Z];
    t[cmp][4] = a[r + 2 * Z];
    t[cmp][5] = a[r + 3 * Z];
  }
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    double* a = q[cmp];
    a[r - 2 * Z] = t[cmp][0];
    a[r - Z] = t[cmp][1];
    a[r] = t[cmp][2];
    if (!(cmp == 2 && shifted)) a[r + (NK + 1) * Z] = t[cmp][3];
    a[r + (NK + 2) * Z] = t[cmp][4];
    a[r + (NK + 3) * Z] = t[cmp][5];
  }
}
// k_halo_x for ni >= 8 with 8 lanes per (j, k, component): lanes 0-2 write the low
// ghosts -2..0, lanes 3-5 the high ghosts ni+1..ni+3, each from its interior source
// (none of which the kernel writes).  A warp then reads and writes a few contiguous
// runs instead of 32 rows, and the work spreads over every SM.
__global__ void __launch_bounds__(256) k_halo_x8(Grid g, int normal, double* __restrict__ uk,
                                                 double* __restrict__ vk, double* __restrict__ wk) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int m = (int)(t & 7);
  const long task = t >> 3;
  const long JK = (long)(g.nj + 6) * (g.nk + 6);
  if (m >= 6 || task >= 3 * JK) return;
  const int cmp = (int)(task / JK);
  const int rem = (int)(task % JK);
  double* a = cmp == 0 ? uk : (cmp == 1 ? vk : wk);
  const bool sh = cmp == 0 && !(normal & 1);  // bndu's u: u(-2..0) = u(ni-1..ni+1), u(ni+1) kept
  const long r = g.at(0, -2 + rem % (g.nj + 6), -2 + rem / (g.nj + 6));
  if (m < 3) {
    a[r + m - 2] = a[r + g.ni - 2 + m + (sh ? 1 : 0)];
  } else if (!(sh && m == 3)) {
    a[r + g.ni + m - 2] = a[r + m - 2];
  }
}
// k_wall, k_halo_x and k_halo_z in one pass (ni, nj, nk >= 8).  Composed, the three
// give every refreshed point as a function of points none of them writes: a ghost
// column (x or z destination) holds its source column's values, its wall rows
// included, and the wall rows of a column are the extrapolation of its source
// column's interior rows with that column's coefficients.  So the threads write
// their points in any order.  Blocks [0, nbW): the wall rows of every column, one
// thread per (column, wall); [nbW, nbW + nbX): the other rows of the x-ghost
// columns, one thread per (j, k, component) for its six ghost slots; the rest: the
// other rows of the z-ghost planes over the columns that are not x destinations,
// one thread per (i, j, component).  A thread reads all its sources before writing.
__global__ void __launch_bounds__(256) k_refresh(Grid g, int normal, double uwall, const double* __restrict__ wc,
                                                 double* __restrict__ uk, double* __restrict__ vk,
                                                 double* __restrict__ wk, int nbW, int nbX) {
  const int shu = !(normal & 1), shw = !(normal & 4);  // bndu's shifted copies: u along x, w along z
  const int NI = g.ni, NJ = g.nj, NK = g.nk;
  const long Y = g.sy;
  const int b = (int)blockIdx.x;
  if (b < nbW) {
    const long t = (long)b * 256 + threadIdx.x;
    const int W = NI + 6;
    if (t >= 2L * W * (NK + 6)) return;
    const int i = (int)(t % W) - 2;
    const int kk = (int)(t / W);
    const int side = kk >= NK + 6 ? 1 : 0;
    const int k = kk - side * (NK + 6) - 2;
    const int jw = side ? NJ : 1;
    auto wco = [&](int ci, int ck) { return (((long)side * (NK + 6) + (ck + 2)) * W + (ci + 2)) * 2; };
    // u from its source column
    const int iu = halo_src(i, NI, shu), ku = halo_src(k, NK, 0);
    const long ou = wco(iu, ku);
    const double u1 = uk[g.at(iu, jw, ku)];
    // v, w
    const int iv = halo_src(i, NI, 0), kv = halo_src(k, NK, 0);
    const int iw = halo_src(i, NI, 0), kw = halo_src(k, NK, shw);
    const double w1 = wk[g.at(iw, jw, kw)];
    const double c2w = wc[wco(iw, kw) + 1];
    const long cv = g.at(iv, jw, kv);
    double va, vb, vc = 0.0;
    if (!side) {
      va = vk[cv];
      vb = vk[cv + Y];
    } else {
      va = vk[cv - Y];
      vb = vk[cv - 2 * Y];
      vc = vk[cv - 3 * Y];
    }
    const double c1 = wc[ou], c2 = wc[ou + 1];
    const long c = g.at(i, jw, k);
    const long t1 = side ? Y : -Y;
    const double u0 = fma(c2, u1, c1 * (side ? uwall : -uwall));  // as k_wall
    const double um = 2.0 * u0 - u1;
    uk[c + t1] = u0;
    uk[c + 2 * t1] = um;
    uk[c + 3 * t1] = 2.0 * um - u0;
    const double w0 = c2w * w1;
    const double wm = 2.0 * w0 - w1;
    wk[c + t1] = w0;
    wk[c + 2 * t1] = wm;
    wk[c + 3 * t1] = 2.0 * wm - w0;
    if (!side) {  // v(0) = 0, v(-1) = -v(1), v(-2) = -v(2)
      vk[c - 3 * Y] = -vb;
      vk[c - 2 * Y] = -va;
      vk[c - Y] = 0.0;
    } else {  // v(nj) = 0, v(nj+m) = -v(nj-m)
      vk[c] = 0.0;
      vk[c + Y] = -va;
      vk[c + 2 * Y] = -vb;
      vk[c + 3 * Y] = -vc;
    }
    return;
  }
  if (b < nbW + nbX) {
    const long task = (long)(b - nbW) * 256 + threadIdx.x;
    if (task >= 3L * NJ * (NK + 6)) return;
    const int cmp = (int)(task / ((long)NJ * (NK + 6)));
    const int rem = (int)(task % ((long)NJ * (NK + 6)));
    const int j = 1 + rem % NJ, k = -2 + rem / NJ;
    if (cmp == 1 && j == NJ) return;  // a wall row of v
    const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
    const int ks = halo_src(k, NK, sz);
    double* a = cmp == 0 ? uk : (cmp == 1 ? vk : wk);
    double v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int d = halo_dest(m, NI, sx);
      v[m] = d == kNoHalo ? 0.0 : a[g.at(halo_src(d, NI, sx), j, ks)];
    }
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int d = halo_dest(m, NI, sx);
      if (d != kNoHalo) a[g.at(d, j, k)] = v[m];
    }
    return;
  }
  const long t = (long)(b - nbW - nbX) * 256 + threadIdx.x;
  const int i = 1 + (int)(t % (NI + 1));
  const long r = t / (NI + 1);
  const int j = 1 + (int)(r % NJ);
  const int cmp = (int)(r / NJ);
  if (cmp >= 3 || (cmp == 1 && j == NJ)) return;
  const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
  if (halo_src(i, NI, sx) != i) return;  // an x-ghost column: done above
  double* a = cmp == 0 ? uk : (cmp == 1 ? vk : wk);
  double v[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int d = halo_dest(m, NK, sz);
    v[m] = d == kNoHalo ? 0.0 : a[g.at(i, j, halo_src(d, NK, sz))];
  }
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int d = halo_dest(m, NK, sz);
    if (d != kNoHalo) a[g.at(i, j, d)] = v[m];
  }
}
// --- mixed precision: FP32 sweeps on the correction d = un - u ---------------------
// During the solve un = u + d holds at every point, halos and wall ghosts included:
// d starts at zero (un = u, main.f90:605-607) and every operation on un has an
// exact counterpart on d.  A sweep q_new = A*visn(q) + B becomes d_new = A*visn(d) + R
// with R = A*visn(u) + B - u; each wall/halo operation dst = f(src) is affine with
// fixed coefficients, so it becomes d_dst = f_lin(d_src) + gamma_dst with
// gamma_dst = f(u_src) - u_dst, formed once per step in FP64 from u.
//
// Wall constants per (side, k, i), 12 floats: c2, gamma_u[3], gamma_v[4], gamma_w[3], pad.
constexpr int kGW = 12;
// x-halo constants per (j, k) and z-halo constants per (i, j), 24 floats: the six
// destinations of the plain copy of u, v, w and the five of bndu's shifted copy
// (u in x: slots 6..10, v 12..17, w 18..23; z: u 0..5, v 6..11, w 12..17, shifted w 18..22).
constexpr int kGH = 24;

__device__ __forceinline__ long wall_slot(const Grid& g, int side, int k, int i) {
  return (((long)side * (g.nk + 6) + (k + 2)) * (g.ni + 6) + (i + 2));
}

__global__ void __launch_bounds__(256) k_gamma_wall(Grid g, double uwall, const double* __restrict__ wc,
                                                    const double* __restrict__ u, const double* __restrict__ v,
                                                    const double* __restrict__ w, float* __restrict__ gw) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int kk = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || kk > 2 * (g.nk + 6) - 3) return;
  const int side = kk >= g.nk + 4 ? 1 : 0;
  const int k = side ? kk - (g.nk + 6) : kk;
  const long o = wall_slot(g, side, k, i);
  const double c1 = wc[2 * o], c2 = wc[2 * o + 1];
  const long Y = g.sy;
  const long c = g.at(i, side ? g.nj : 1, k);
  const long t = side ? Y : -Y;  // towards the ghost rows
  float* G = gw + o * kGW;
  // u, w: q(g1) = K + c2 q(c), q(g2) = 2 q(g1) - q(c), q(g3) = 2 q(g2) - q(g1)
  auto lin = [&](const double* q, double K, float* out) {
    const double q1 = q[c], g1 = q[c + t], g2 = q[c + 2 * t], g3 = q[c + 3 * t];
    out[0] = (float)(K + c2 * q1 - g1);
    out[1] = (float)(2.0 * g1 - q1 - g2);
    out[2] = (float)(2.0 * g2 - g1 - g3);
  };
  G[0] = (float)c2;
  lin(u, side ? c1 * uwall : c1 * (-uwall), G + 1);
  lin(w, 0.0, G + 8);
  if (!side) {  // v(0) = 0, v(-1) = -v(1), v(-2) = -v(2)
    G[4] = (float)(-v[c - Y]);
    G[5] = (float)(-v[c] - v[c - 2 * Y]);
    G[6] = (float)(-v[c + Y] - v[c - 3 * Y]);
    G[7] = 0.f;
  } else {  // v(nj) = 0, v(nj+m) = -v(nj-m), m = 1..3
    G[4] = (float)(-v[c]);
    G[5] = (float)(-v[c - Y] - v[c + Y]);
    G[6] = (float)(-v[c - 2 * Y] - v[c + 2 * Y]);
    G[7] = (float)(-v[c - 3 * Y] - v[c + 3 * Y]);
  }
  G[11] = 0.f;
}
__global__ void __launch_bounds__(256) k_gamma_x(Grid g, const double* __restrict__ u, const double* __restrict__ v,
                                                 const double* __restrict__ w, float* __restrict__ gx) {
  const int j = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (j > g.nj + 3 || k > g.nk + 3) return;
  const int NI = g.ni;
  const long r = g.at(0, j, k);
  float* G = gx + ((long)(k + 2) * (g.nj + 6) + (j + 2)) * kGH;
  const int dst[6] = {-2, -1, 0, NI + 1, NI + 2, NI + 3};
  const int src[6] = {NI - 2, NI - 1, NI, 1, 2, 3};
  const double* q[3] = {u, v, w};
  const int base[3] = {0, 12, 18};
  for (int cmp = 0; cmp < 3; ++cmp)
    for (int t = 0; t < 6; ++t) G[base[cmp] + t] = (float)(q[cmp][r + src[t]] - q[cmp][r + dst[t]]);
  // bndu's u: destinations -2, -1, 0, ni+2, ni+3 from ni-1, ni, ni+1, 2, 3
  const int sd[5] = {-2, -1, 0, NI + 2, NI + 3};
  const int ss[5] = {NI - 1, NI, NI + 1, 2, 3};
  for (int t = 0; t < 5; ++t) G[6 + t] = (float)(u[r + ss[t]] - u[r + sd[t]]);
  G[11] = 0.f;
}
__global__ void __launch_bounds__(256) k_gamma_z(Grid g, const double* __restrict__ u, const double* __restrict__ v,
                                                 const double* __restrict__ w, float* __restrict__ gz) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || j > g.nj + 3) return;
  const int NK = g.nk;
  const long Z = g.sz;
  const long r = g.at(i, j, 0);
  float* G = gz + ((long)(j + 2) * (g.ni + 6) + (i + 2)) * kGH;
  const int dst[6] = {-2, -1, 0, NK + 1, NK + 2, NK + 3};
  const int src[6] = {NK - 2, NK - 1, NK, 1, 2, 3};
  const double* q[3] = {u, v, w};
  for (int cmp = 0; cmp < 3; ++cmp)
    for (int t = 0; t < 6; ++t) G[6 * cmp + t] = (float)(q[cmp][r + src[t] * Z] - q[cmp][r + dst[t] * Z]);
  const int sd[5] = {-2, -1, 0, NK + 2, NK + 3};
  const int ss[5] = {NK - 1, NK, NK + 1, 2, 3};
  for (int t = 0; t < 5; ++t) G[18 + t] = (float)(w[r + ss[t] * Z] - w[r + sd[t] * Z]);
  G[23] = 0.f;
}

// k_wall on the corrections
__global__ void __launch_bounds__(256) k_wall_d(Grid g, const float* __restrict__ gw, float* __restrict__ du,
                                                float* __restrict__ dv, float* __restrict__ dw) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int kk = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || kk > 2 * (g.nk + 6) - 3) return;
  const int side = kk >= g.nk + 4 ? 1 : 0;
  const int k = side ? kk - (g.nk + 6) : kk;
  const float4* G4 = reinterpret_cast<const float4*>(gw + wall_slot(g, side, k, i) * kGW);
  const float4 a = __ldg(G4), b = __ldg(G4 + 1), e = __ldg(G4 + 2);
  const float c2 = a.x;
  const long Y = g.sy;
  const long c = g.at(i, side ? g.nj : 1, k);
  const long t = side ? Y : -Y;
  const float u1 = du[c], w1 = dw[c];
  float v1, v2, v3;
  if (!side) {
    v1 = dv[c];
    v2 = dv[c + Y];
    v3 = 0.f;
  } else {
    v1 = dv[c - Y];
    v2 = dv[c - 2 * Y];
    v3 = dv[c - 3 * Y];
  }
  const float ug1 = c2 * u1 + a.y, ug2 = 2.f * ug1 - u1 + a.z, ug3 = 2.f * ug2 - ug1 + a.w;
  du[c + t] = ug1;
  du[c + 2 * t] = ug2;
  du[c + 3 * t] = ug3;
  const float wg1 = c2 * w1 + e.x, wg2 = 2.f * wg1 - w1 + e.y, wg3 = 2.f * wg2 - wg1 + e.z;
  dw[c + t] = wg1;
  dw[c + 2 * t] = wg2;
  dw[c + 3 * t] = wg3;
  if (!side) {
    dv[c - Y] = b.x;
    dv[c - 2 * Y] = -v1 + b.y;
    dv[c - 3 * Y] = -v2 + b.z;
  } else {
    dv[c] = b.x;
    dv[c + Y] = -v1 + b.y;
    dv[c + 2 * Y] = -v2 + b.z;
    dv[c + 3 * Y] = -v3 + b.w;
  }
}
// k_halo_x on the corrections
__global__ void __launch_bounds__(256) k_halo_x_d(Grid g, int normal, const float* __restrict__ gx,
                                                  float* __restrict__ du, float* __restrict__ dv,
                                                  float* __restrict__ dw) {
  const int j = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (j > g.nj + 3 || k > g.nk + 3) return;
  const int NI = g.ni;
  const long r = g.at(0, j, k);
  const float* G = gx + ((long)(k + 2) * (g.nj + 6) + (j + 2)) * kGH;
  float* q[3] = {du, dv, dw};
  const bool shifted = !(normal & 1);
  float t[3][6];
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    const float* a = q[cmp];
    const int sh = (cmp == 0 && shifted) ? 1 : 0;
    t[cmp][0] = a[r + NI - 2 + sh];
    t[cmp][1] = a[r + NI - 1 + sh];
    t[cmp][2] = a[r + NI + sh];
    t[cmp][3] = sh ? 0.f : a[r + 1];
    t[cmp][4] = a[r + 2];
    t[cmp][5] = a[r + 3];
  }
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    float* a = q[cmp];
    if (cmp == 0 && shifted) {
      const float* s = G + 6;
      a[r - 2] = t[0][0] + __ldg(s);
      a[r - 1] = t[0][1] + __ldg(s + 1);
      a[r] = t[0][2] + __ldg(s + 2);
      a[r + NI + 2] = t[0][4] + __ldg(s + 3);
      a[r + NI + 3] = t[0][5] + __ldg(s + 4);
    } else {
      const float* s = G + (cmp == 0 ? 0 : (cmp == 1 ? 12 : 18));
      a[r - 2] = t[cmp][0] + __ldg(s);
      a[r - 1] = t[cmp][1] + __ldg(s + 1);
      a[r] = t[cmp][2] + __ldg(s + 2);
      a[r + NI + 1] = t[cmp][3] + __ldg(s + 3);
      a[r + NI + 2] = t[cmp][4] + __ldg(s + 4);
      a[r + NI + 3] = t[cmp][5] + __ldg(s + 5);
    }
  }
}
// k_halo_z on the corrections
__global__ void __launch_bounds__(256) k_halo_z_d(Grid g, int normal, const float* __restrict__ gz,
                                                  float* __restrict__ du, float* __restrict__ dv,
                                                  float* __restrict__ dw) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || j > g.nj + 3) return;
  const int NK = g.nk;
  const long Z = g.sz;
  const long r = g.at(i, j, 0);
  const float* G = gz + ((long)(j + 2) * (g.ni + 6) + (i + 2)) * kGH;
  float* q[3] = {du, dv, dw};
  const bool shifted = !(normal & 4);
  float t[3][6];
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    const float* a = q[cmp];
    const int sh = (cmp == 2 && shifted) ? 1 : 0;
    t[cmp][0] = a[r + (NK - 2 + sh) * Z];
    t[cmp][1] = a[r + (NK - 1 + sh) * Z];
    t[cmp][2] = a[r + (NK + sh) * Z];
    t[cmp][3] = sh ? 0.f : a[r + Z];
    t[cmp][4] = a[r + 2 * Z];
    t[cmp][5] = a[r + 3 * Z];
  }
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    float* a = q[cmp];
    if (cmp == 2 && shifted) {
      const float* s = G + 18;
      a[r - 2 * Z] = t[2][0] + __ldg(s);
      a[r - Z] = t[2][1] + __ldg(s + 1);
      a[r] = t[2][2] + __ldg(s + 2);
      a[r + (NK + 2) * Z] = t[2][4] + __ldg(s + 3);
      a[r + (NK + 3) * Z] = t[2][5] + __ldg(s + 4);
    } else {
      const float* s = G + 6 * cmp;
      a[r - 2 * Z] = t[cmp][0] + __ldg(s);
      a[r - Z] = t[cmp][1] + __ldg(s + 1);
      a[r] = t[cmp][2] + __ldg(s + 2);
      a[r + (NK + 1) * Z] = t[cmp][3] + __ldg(s + 3);
      a[r + (NK + 2) * Z] = t[cmp][4] + __ldg(s + 4);
      a[r + (NK + 3) * Z] = t[cmp][5] + __ldg(s + 5);
    }
  }
}
// k_wall_d, k_halo_x_d and k_halo_z_d in one pass (ni, nj, nk >= 8), composed as
// k_refresh composes their FP64 counterparts, with the per-point constants added
// in the same order (wall extrapolation of the source column, then + the x
// constant of the source plane's row, then + the z constant of the final column's
// row), so the result is bit for bit that of the three kernels.  Blocks [0, nbW):
// the wall rows of every column, one thread per (column, wall); [nbW, nbW + nbX):
// the other rows of the x-ghost columns, one thread per (j, k, component);
// the rest: the other rows of the z-ghost planes of the columns that are not x
// destinations, one thread per (i, j, component).
__device__ __forceinline__ int gslot(int d, int N, int sh) { return d <= 0 ? d + 2 : d - N + 2 - sh; }
__global__ void __launch_bounds__(256) k_refresh_d(Grid g, int normal, const float* __restrict__ gw,
                                                   const float* __restrict__ gx, const float* __restrict__ gz,
                                                   float* __restrict__ du, float* __restrict__ dv,
                                                   float* __restrict__ dw, int nbW, int nbX) {
  const int shu = !(normal & 1), shw = !(normal & 4);
  const int NI = g.ni, NJ = g.nj, NK = g.nk;
  // constant slots: x (per (k, j)): u 0, shifted u 6, v 12, w 18; z (per (j, i)): u 0,
  // v 6, w 12, shifted w 18
  auto xb = [&](int cmp) { return cmp == 0 ? (shu ? 6 : 0) : 6 * cmp + 6; };
  auto zb = [&](int cmp) { return cmp == 2 ? (shw ? 18 : 12) : 6 * cmp; };
  auto GX = [&](int j, int k, int slot) { return __ldg(gx + ((long)(k + 2) * (NJ + 6) + (j + 2)) * kGH + slot); };
  auto GZ = [&](int i, int j, int slot) { return __ldg(gz + ((long)(j + 2) * (NI + 6) + (i + 2)) * kGH + slot); };
  const int b = (int)blockIdx.x;
  if (b < nbW) {
    const long t = (long)b * 256 + threadIdx.x;
    const int W = NI + 6;
    if (t >= 2L * W * (NK + 6)) return;
    const int i = (int)(t % W) - 2;
    const int kk = (int)(t / W);
    const int side = kk >= NK + 6 ? 1 : 0;
    const int k = kk - side * (NK + 6) - 2;
    const int jw = side ? NJ : 1, tj = side ? 1 : -1;
    // value of ghost row j of this column from the source column's value v
    auto compose = [&](float v, int cmp, int is, int ks, int j) {
      if (is != i) v = v + GX(j, ks, xb(cmp) + gslot(i, NI, cmp == 0 ? shu : 0));
      if (ks != k) v = v + GZ(i, j, zb(cmp) + gslot(k, NK, cmp == 2 ? shw : 0));
      return v;
    };
    // u and w: q(g1) = c2 q1 + G1, q(g2) = 2 q(g1) - q1 + G2, q(g3) = 2 q(g2) - q(g1) + G3
#pragma unroll
    for (int cmp = 0; cmp < 3; cmp += 2) {
      const int is = halo_src(i, NI, cmp == 0 ? shu : 0), ks = halo_src(k, NK, cmp == 2 ? shw : 0);
      const float4* G4 = reinterpret_cast<const float4*>(gw + wall_slot(g, side, ks, is) * kGW);
      const float4 a = __ldg(G4), e = __ldg(G4 + 2);
      float* q = cmp == 0 ? du : dw;
      const float q1 = q[g.at(is, jw, ks)];
      const float c2 = a.x;
      const float h1 = cmp == 0 ? a.y : e.x, h2 = cmp == 0 ? a.z : e.y, h3 = cmp == 0 ? a.w : e.z;
      const float g1 = c2 * q1 + h1, g2 = 2.f * g1 - q1 + h2, g3 = 2.f * g2 - g1 + h3;
      q[g.at(i, jw + tj, k)] = compose(g1, cmp, is, ks, jw + tj);
      q[g.at(i, jw + 2 * tj, k)] = compose(g2, cmp, is, ks, jw + 2 * tj);
      q[g.at(i, jw + 3 * tj, k)] = compose(g3, cmp, is, ks, jw + 3 * tj);
    }
    {
      const int is = halo_src(i, NI, 0), ks = halo_src(k, NK, 0);
      const float4 bb = __ldg(reinterpret_cast<const float4*>(gw + wall_slot(g, side, ks, is) * kGW) + 1);
      const long c = g.at(is, jw, ks);
      const long Y = g.sy;
      if (!side) {  // v(0), v(-1), v(-2)
        const float v1 = dv[c], v2 = dv[c + Y];
        dv[g.at(i, 0, k)] = compose(bb.x, 1, is, ks, 0);
        dv[g.at(i, -1, k)] = compose(-v1 + bb.y, 1, is, ks, -1);
        dv[g.at(i, -2, k)] = compose(-v2 + bb.z, 1, is, ks, -2);
      } else {  // v(nj), v(nj+1..nj+3)
        const float v1 = dv[c - Y], v2 = dv[c - 2 * Y], v3 = dv[c - 3 * Y];
        dv[g.at(i, NJ, k)] = compose(bb.x, 1, is, ks, NJ);
        dv[g.at(i, NJ + 1, k)] = compose(-v1 + bb.y, 1, is, ks, NJ + 1);
        dv[g.at(i, NJ + 2, k)] = compose(-v2 + bb.z, 1, is, ks, NJ + 2);
        dv[g.at(i, NJ + 3, k)] = compose(-v3 + bb.w, 1, is, ks, NJ + 3);
      }
    }
    return;
  }
  if (b < nbW + nbX) {
    const long task = (long)(b - nbW) * 256 + threadIdx.x;
    if (task >= 3L * NJ * (NK + 6)) return;
    const int cmp = (int)(task / ((long)NJ * (NK + 6)));
    const int rem = (int)(task % ((long)NJ * (NK + 6)));
    const int j = 1 + rem % NJ, k = -2 + rem / NJ;
    if (cmp == 1 && j == NJ) return;  // a wall row of v
    const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
    const int ks = halo_src(k, NK, sz);
    float* a = cmp == 0 ? du : (cmp == 1 ? dv : dw);
    float v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int d = halo_dest(m, NI, sx);
      if (d == kNoHalo) {
        v[m] = 0.f;
        continue;
      }
      v[m] = a[g.at(halo_src(d, NI, sx), j, ks)] + GX(j, ks, xb(cmp) + gslot(d, NI, sx));
      if (ks != k) v[m] = v[m] + GZ(d, j, zb(cmp) + gslot(k, NK, sz));
    }
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int d = halo_dest(m, NI, sx);
      if (d != kNoHalo) a[g.at(d, j, k)] = v[m];
    }
    return;
  }
  const long t = (long)(b - nbW - nbX) * 256 + threadIdx.x;
  const int i = 1 + (int)(t % (NI + 1));
  const long r = t / (NI + 1);
  const int j = 1 + (int)(r % NJ);
  const int cmp = (int)(r / NJ);
  if (cmp >= 3 || (cmp == 1 && j == NJ)) return;
  const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
  if (halo_src(i, NI, sx) != i) return;  // an x-ghost column: done above
  float* a = cmp == 0 ? du : (cmp == 1 ? dv : dw);
  float v[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int d = halo_dest(m, NK, sz);
    v[m] = d == kNoHalo ? 0.f : a[g.at(i, j, halo_src(d, NK, sz))] + GZ(i, j, zb(cmp) + gslot(d, NK, sz));
  }
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int d = halo_dest(m, NK, sz);
    if (d != kNoHalo) a[g.at(i, j, d)] = v[m];
  }
}
__global__ void k_to_float(long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}
// un = u + du, vn = v + dv, wn = w + dw at every point
__global__ void k_refine_finish(long n, const double* __restrict__ u, const double* __restrict__ v,
                                const double* __restrict__ w, const float* __restrict__ du,
                                const float* __restrict__ dv, const float* __restrict__ dw, double* __restrict__ un,
                                double* __restrict__ vn, double* __restrict__ wn) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    un[t] = u[t] + (double)du[t];
    vn[t] = v[t] + (double)dv[t];
    wn[t] = w[t] + (double)dw[t];
  }
}

__global__ void k_sum_parts2(const double* part, long n, double* out) {
  __shared__ double sh[256];
  double a = 0.0;
  for (long t = threadIdx.x; t < n; t += 256) a += part[t];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

// The one-pass refresh kernels where the grid allows them, unless FMF_REFRESH_ORDERED
// is set in the environment (then the ordered plane kernels, which give the same
// values: the tests compare the two).
bool one_pass_refresh(const Grid& g) {
  static const bool ordered = std::getenv("FMF_REFRESH_ORDERED") != nullptr;
  return !ordered && refresh_one_pass(g.ni, g.nj, g.nk);
}

VP make_vp(double dxinv, double dyinv, double dzinv, double dt, int harmonic) {
  VP p;
  p.dtinv = dt > 0.0 ? 1.0 / dt : 0.0;
  p.dx2 = dxinv * dxinv;
  p.dy2 = dyinv * dyinv;
  p.dz2 = dzinv * dzinv;
  p.dxy = dxinv * dyinv;
  p.dxz = dxinv * dzinv;
  p.dyz = dyinv * dzinv;
  p.harmonic = harmonic;
  return p;
}
const dim3 kB(32, 8, 1);
dim3 wall_grid(const Grid& g) { return dim3((g.ni + 6 + 31) / 32, (2 * (g.nk + 6) + 7) / 8); }
dim3 xh_grid(const Grid& g) { return dim3((g.nj + 6 + 31) / 32, (g.nk + 6 + 7) / 8); }
dim3 zh_grid(const Grid& g) { return dim3((g.ni + 6 + 31) / 32, (g.nj + 6 + 7) / 8); }
dim3 pair_grid(const Grid& g) {
  return dim3((unsigned)((g.ni / 2 + 31) / 32), (unsigned)((g.nj / 2 + 7) / 8), (unsigned)(g.nk / 2));
}
// first colour of each pair (solu_sor4.f:94-120): (1,1,1) (1,1,2) (1,2,1) (2,1,1)
const int kPi[4] = {1, 1, 1, 2}, kPj[4] = {1, 1, 2, 1}, kPk[4] = {1, 2, 1, 1};

// k_edges + k_src_ab<REFINE> + k_wall_coef
template <bool REFINE>
void src_prep(cudaStream_t s, const Grid& g, const VP& p, const double* u, const double* v, const double* w,
              const double* const* adv, const double* const* advo, const double* const* prs,
              const double* const* vis, const double* const* fst, const double* const* fstn, double grvb,
              double grvp, const double* mu, const double* rho, const double* rhon, double* const* E, F3 ef,
              ABOut out, const double* l1, const double* l2, const double* phi, double dy, double* wallc,
              bool pairs = false) {
  SrcIn in;
  in.u = u;
  in.v = v;
  in.w = w;
  in.rho = rho;
  in.rhon = rhon;
  for (int q = 0; q < 3; ++q) {
    in.adv[q] = adv[q];
    in.advo[q] = advo[q];
    in.prs[q] = prs[q];
    in.vis[q] = vis[q];
    in.fst[q] = fst[q];
    in.fstn[q] = fstn[q];
  }
  in.grvb = grvb;
  in.grvp = grvp;
  k_edges<<<dim3((g.ni + 1 + 31) / 32, (g.nj + 1 + 7) / 8, g.nk + 1), kB, 0, s>>>(g, p, mu, E[0], E[1], E[2], ef);
  if (pairs) {
    using df::split_double;
    VPS ps;
    ps.dtinv = split_double(p.dtinv);
    ps.dx2 = split_double(p.dx2);
    ps.dy2 = split_double(p.dy2);
    ps.dz2 = split_double(p.dz2);
    ps.dx2x2 = split_double(2.0 * p.dx2);
    ps.dy2x2 = split_double(2.0 * p.dy2);
    ps.dz2x2 = split_double(2.0 * p.dz2);
    ps.grvb = split_double(grvb);
    ps.grvp = split_double(grvp);
    k_src_ab_e<REFINE><<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), kB, 0, s>>>(g, ps, p, in, mu, E[0], E[1],
                                                                                 E[2], out);
  } else {
    k_src_ab<REFINE><<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), kB, 0, s>>>(g, p, in, mu, E[0], E[1], E[2], out);
  }
  k_wall_coef<<<wall_grid(g), kB, 0, s>>>(g, dy, l1, l2, phi, wallc);
  count_launch(3);
}

// The colour-pair sweeps of one outer iteration: per component 4 pairs, each
// followed by the wall/halo refresh; then the residual sum into errsum[0].
template <class T, class PairFn, class HaloFn>
void sweep_all(cudaStream_t s, const Grid& g, double* part, double* errsum, PairFn pair, HaloFn halo) {
  const long nb = (long)pair_grid(g).x * pair_grid(g).y * pair_grid(g).z;
  for (int comp = 0; comp < 3; ++comp) {
    for (int pr = 0; pr < 4; ++pr) {
      pair(comp, pr, part + (long)(comp * 4 + pr) * nb);
      count_launch();
      halo(1 << comp);
    }
  }
  k_sum_parts2<<<1, 256, 0, s>>>(part, nb * 12, errsum);
  count_launch();
}
}  // namespace

void src_visc_prep(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, int harmonic,
                   double grvb, double grvp, const double* u, const double* v, const double* w,
                   const double* const* adv, const double* const* advo, const double* const* prs,
                   const double* const* vis, const double* const* fst, const double* const* fstn, const double* mu,
                   const double* rho, const double* rhon, double* const* E, double* const* AB, const double* l1,
                   const double* l2, const double* phi, double dy, double* wallc, bool pairs) {
  ABOut out{};
  for (int q = 0; q < 3; ++q) {
    out.a[q] = AB[2 * q];
    out.b[q] = AB[2 * q + 1];
  }
  src_prep<false>(s, g, make_vp(dxinv, dyinv, dzinv, dt, harmonic), u, v, w, adv, advo, prs, vis, fst, fstn, grvb,
                  grvp, mu, rho, rhon, E, F3{{nullptr, nullptr, nullptr}}, out, l1, l2, phi, dy, wallc, pairs);
}

void wall_coef(cudaStream_t s, const Grid& g, double dy, const double* l1, const double* l2, const double* phi,
               double* wallc) {
  k_wall_coef<<<wall_grid(g), kB, 0, s>>>(g, dy, l1, l2, phi, wallc);
  count_launch();
}

void explicit_viscous(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* u,
                      const double* v, const double* w, const double* mu, double* tau, double* const* vis,
                      double* sk, bool pairs) {
  if (pairs) {
    using df::split_double;
    VPT p;
    p.dxd = dxinv;
    p.dyd = dyinv;
    p.dzd = dzinv;
    p.dxi2 = split_double(2.0 * dxinv);
    p.dyi2 = split_double(2.0 * dyinv);
    p.dzi2 = split_double(2.0 * dzinv);
    p.hx = split_double(0.25 * dxinv);
    p.hy = split_double(0.25 * dyinv);
    p.hz = split_double(0.25 * dzinv);
    p.dxi = split_double(dxinv);
    p.dyi = split_double(dyinv);
    p.dzi = split_double(dzinv);
    k_stress_e<<<dim3((g.ni + 2 + 31) / 32, (g.nj + 2 + 7) / 8, g.nk + 2), kB, 0, s>>>(g, p, u, v, w, mu, tau,
                                                                                                 sk);
    k_div_stress_e<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), kB, 0, s>>>(g, p, tau, vis[0], vis[1], vis[2]);
    count_launch(2);
    return;
  }
  k_stress<<<dim3((g.ni + 2 + 31) / 32, (g.nj + 2 + 7) / 8, g.nk + 2), kB, 0, s>>>(g, dxinv, dyinv, dzinv, u, v, w,
                                                                               mu, tau, sk);
  k_div_stress<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), kB, 0, s>>>(g, dxinv, dyinv, dzinv, tau, vis[0],
                                                                         vis[1], vis[2]);
  count_launch(2);
}

void wall_halo(cudaStream_t s, const Grid& g, int normal, double uwall, const double* wallc, double* un, double* vn,
               double* wn) {
  if (one_pass_refresh(g)) {
    const long tw = 2L * (g.ni + 6) * (g.nk + 6), tx = 3L * g.nj * (g.nk + 6), tz = 3L * (g.ni + 1) * g.nj;
    const int nbW = (int)((tw + 255) / 256), nbX = (int)((tx + 255) / 256), nbZ = (int)((tz + 255) / 256);
    k_refresh<<<nbW + nbX + nbZ, 256, 0, s>>>(g, normal, uwall, wallc, un, vn, wn, nbW, nbX);
    count_launch();
    return;
  }
  k_wall<<<wall_grid(g), kB, 0, s>>>(g, uwall, wallc, un, vn, wn);
  if (g.ni >= 8)
    k_halo_x8<<<(unsigned)((24L * (g.nj + 6) * (g.nk + 6) + 255) / 256), 256, 0, s>>>(g, normal, un, vn, wn);
  else
    k_halo_x<<<xh_grid(g), kB, 0, s>>>(g, normal, un, vn, wn);
  k_halo_z<<<zh_grid(g), kB, 0, s>>>(g, normal, un, vn, wn);
  count_launch(3);
}

void sor_iteration(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, int harmonic,
                   const double* mu, double* const* E, double* const* AB, double uwall, const double* wallc,
                   double* un, double* vn, double* wn, double* part, double* errsum) {
  const VP p = make_vp(dxinv, dyinv, dzinv, 0.0, harmonic);
  const dim3 grd = pair_grid(g);
  sweep_all<double>(
      s, g, part, errsum,
      [&](int comp, int pr, double* pp) {
#define FMF_PAIR(C) \
  k_pair<C, double><<<grd, kB, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], mu, E[0], E[1], E[2], AB[2 * C], AB[2 * C + 1], un, vn, wn, pp)
        if (comp == 0) FMF_PAIR(0);
        else if (comp == 1) FMF_PAIR(1);
        else FMF_PAIR(2);
#undef FMF_PAIR
      },
      [&](int normal) { wall_halo(s, g, normal, uwall, wallc, un, vn, wn); });
}

long refine_floats(const Grid& g, int part) {
  switch (part) {
    case 0: return 2L * (g.nk + 6) * (g.ni + 6) * kGW;
    case 1: return (long)(g.nj + 6) * (g.nk + 6) * kGH;
    default: return (long)(g.ni + 6) * (g.nj + 6) * kGH;
  }
}

void refine_prep(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, int harmonic,
                 double grvb, double grvp, const double* u, const double* v, const double* w,
                 const double* const* adv, const double* const* advo, const double* const* prs,
                 const double* const* vis, const double* const* fst, const double* const* fstn, const double* mu,
                 const double* rho, const double* rhon, double* const* E, const double* l1, const double* l2,
                 const double* phi, double dy, double uwall, double* wallc, const RefineBufs& rb) {
  ABOut out{};
  for (int q = 0; q < 3; ++q) {
    out.af[q] = rb.a[q];
    out.rf[q] = rb.r[q];
  }
  // A and B in FP32 pairs, the residual in FP64 (k_src_ab_e<true>)
  src_prep<true>(s, g, make_vp(dxinv, dyinv, dzinv, dt, harmonic), u, v, w, adv, advo, prs, vis, fst, fstn, grvb,
                 grvp, mu, rho, rhon, E, F3{{rb.e[0], rb.e[1], rb.e[2]}}, out, l1, l2, phi, dy, wallc, true);
  k_to_float<<<4 * 152, 256, 0, s>>>(g.n, mu, rb.mu);
  k_gamma_wall<<<wall_grid(g), kB, 0, s>>>(g, uwall, wallc, u, v, w, rb.gw);
  k_gamma_x<<<xh_grid(g), kB, 0, s>>>(g, u, v, w, rb.gx);
  k_gamma_z<<<zh_grid(g), kB, 0, s>>>(g, u, v, w, rb.gz);
  count_launch(4);
  for (int q = 0; q < 3; ++q) FMF_CUDA(cudaMemsetAsync(rb.d[q], 0, sizeof(float) * g.n, s));
}

void sor_iteration_refine(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                          const RefineBufs& rb, double* part, double* errsum) {
  const VP p = make_vp(dxinv, dyinv, dzinv, 0.0, 0);
  const dim3 grd = pair_grid(g);
  float *du = rb.d[0], *dv = rb.d[1], *dw = rb.d[2];
  sweep_all<float>(
      s, g, part, errsum,
      [&](int comp, int pr, double* pp) {
#define FMF_PAIR(C) \
  k_pair<C, float><<<grd, kB, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], rb.mu, rb.e[0], rb.e[1], rb.e[2], rb.a[C], rb.r[C], du, dv, dw, pp)
        if (comp == 0) FMF_PAIR(0);
        else if (comp == 1) FMF_PAIR(1);
        else FMF_PAIR(2);
#undef FMF_PAIR
      },
      [&](int normal) {
        if (one_pass_refresh(g)) {
          const long tw = 2L * (g.ni + 6) * (g.nk + 6), tx = 3L * g.nj * (g.nk + 6), tz = 3L * (g.ni + 1) * g.nj;
          const int nbW = (int)((tw + 255) / 256), nbX = (int)((tx + 255) / 256), nbZ = (int)((tz + 255) / 256);
          k_refresh_d<<<nbW + nbX + nbZ, 256, 0, s>>>(g, normal, rb.gw, rb.gx, rb.gz, du, dv, dw, nbW, nbX);
          count_launch();
          return;
        }
        k_wall_d<<<wall_grid(g), kB, 0, s>>>(g, rb.gw, du, dv, dw);
        k_halo_x_d<<<xh_grid(g), kB, 0, s>>>(g, normal, rb.gx, du, dv, dw);
        k_halo_z_d<<<zh_grid(g), kB, 0, s>>>(g, normal, rb.gz, du, dv, dw);
        count_launch(3);
      });
}

void refine_finish(cudaStream_t s, const Grid& g, const double* u, const double* v, const double* w,
                   const RefineBufs& rb, double* un, double* vn, double* wn) {
  k_refine_finish<<<4 * 152, 256, 0, s>>>(g.n, u, v, w, rb.d[0], rb.d[1], rb.d[2], un, vn, wn);
  count_launch();
}

long sor_parts(const Grid& g) {
  return (long)((g.ni / 2 + 31) / 32) * ((g.nj / 2 + 7) / 8) * (g.nk / 2) * 12;
}

}  // namespace fused
}  // namespace fmf
