// adj.cuh -- reverse-mode (adjoint) kernels of the FP64 time step.
//
// For every operation y = f(x) of the step the adjoint kernel adds J_f^T * ybar to
// xbar.  Conventions: "lq" is the adjoint of array q.  Operations that overwrite
// part of an array in place (boundary conditions) have in-place adjoints: the
// adjoint of each overwritten point is moved onto the points it was computed from
// and then cleared.  Scatters use FP64 atomicAdd, so sums are exact up to the order
// of additions (rounding-level nondeterminism).  Branches of the forward pass
// (band tests, upwind sides, clips, snaps, clamps) are taken as in the forward pass
// and differentiated on the branch that was executed.
#pragma once
#include <cmath>
#include <functional>
#include <map>
#include <utility>
#include <vector>

#include "../../include/fmf_capi.h"
#include "fmf_common.cuh"

namespace fmf {
// The product time step's state and walls (step.cu), for the forward steps of a
// rollout whose intermediates no reverse step reads.
double* ctx_field(fmf_ctx* c, int f);
void ctx_load_device(fmf_ctx* c, const double* const* state, const double* th, const double* ze,
                     const double* l1, const double* l2);
long ctx_sor_total(fmf_ctx* c);

namespace adj {

// Forward-mode number with N partial derivatives, for local Jacobians of small
// nonlinear point functions (contact-angle normals, slip coefficients, GNBC).
template <int N>
struct Dual {
  double v;
  double d[N];
  __host__ __device__ Dual() : v(0.0) {
    for (int t = 0; t < N; ++t) d[t] = 0.0;
  }
  __host__ __device__ Dual(double x) : v(x) {
    for (int t = 0; t < N; ++t) d[t] = 0.0;
  }
  __host__ __device__ static Dual var(double x, int slot) {
    Dual r(x);
    r.d[slot] = 1.0;
    return r;
  }
};
template <int N>
__host__ __device__ inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] + b.d[t];
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] - b.d[t];
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
  for (int t = 0; t < N; ++t) r.d[t] = -a.d[t];
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] * b.v + a.v * b.d[t];
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  const double q = a.v / b.v;
  Dual<N> r(q);
  for (int t = 0; t < N; ++t) r.d[t] = (a.d[t] - q * b.d[t]) / b.v;
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N>
__host__ __device__ inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N>
__host__ __device__ inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N>
__host__ __device__ inline Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r(a.v * b);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] * b;
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N>
__host__ __device__ inline Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N>
__host__ __device__ inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N>
__device__ inline Dual<N> dsqrt(const Dual<N>& a) {
  const double s = sqrt(a.v);
  Dual<N> r(s);
  for (int t = 0; t < N; ++t) r.d[t] = s > 0.0 ? a.d[t] * 0.5 / s : 0.0;
  return r;
}
template <int N>
__device__ inline Dual<N> dcos(const Dual<N>& a) {
  Dual<N> r(cos(a.v));
  const double ds = -sin(a.v);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] * ds;
  return r;
}
template <int N>
__device__ inline Dual<N> dsin(const Dual<N>& a) {
  Dual<N> r(sin(a.v));
  const double dc = cos(a.v);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] * dc;
  return r;
}
template <int N>
__device__ inline Dual<N> dexp(const Dual<N>& a) {
  const double e = exp(a.v);
  Dual<N> r(e);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] * e;
  return r;
}
template <int N>
__device__ inline Dual<N> dcosh(const Dual<N>& a) {
  Dual<N> r(cosh(a.v));
  const double sh = sinh(a.v);
  for (int t = 0; t < N; ++t) r.d[t] = a.d[t] * sh;
  return r;
}

__device__ __forceinline__ void aadd(double* p, double v) {
  if (v != 0.0) atomicAdd(p, v);
}

// ---- boundary conditions and copies (in place on the adjoint) -----------------
void periodic_T(cudaStream_t s, const Grid& g, double* lq);
void neumann_T(cudaStream_t s, const Grid& g, double* lq);
void avzero_T(cudaStream_t s, const Grid& g, double* lq);
// q0 = q1 everywhere, then clip of q0's interior to [0,1]: lq1 += lq0 (masked); lq0 = 0
void summation_T(cudaStream_t s, const Grid& g, const double* q1, double* lq0, double* lq1);
// theta from (u, w, theta0, zeta): adds to lu, lw, ltheta0, lzeta; ltheta is read
void gnbc_T(cudaStream_t s, const Grid& g, const double* u, const double* w, double uwall, const double* theta0,
            double sigma, const double* zeta, const double* ltheta, double* lu, double* lw, double* ltheta0,
            double* lzeta);
// ghosts of q from its wall rows and theta; q holds the forward input (wall rows)
void contact_angle_T(cudaStream_t s, const Grid& g, const double* q, const double* theta, double dx, double dy,
                     double dz, double* lq, double* ltheta);
// k_wall of the fused solve: ghosts of (u,v,w) from the wall rows and the slip
// coefficients wc; u, w hold the forward wall-row values; lwc accumulates (c1, c2)
void wall_T(cudaStream_t s, const Grid& g, double uwall, const double* wc, const double* u, const double* w,
            double* lu, double* lv, double* lw, double* lwc);
// x / z halo copies of (u, v, w); bit c of normal set: plain copy of component c
void halo_x_T(cudaStream_t s, const Grid& g, int normal, double* lu, double* lv, double* lw);
void halo_z_T(cudaStream_t s, const Grid& g, int normal, double* lu, double* lv, double* lw);
void wall_halo_T(cudaStream_t s, const Grid& g, int normal, double uwall, const double* wc, const double* u,
                 const double* w, double* lu, double* lv, double* lw, double* lwc);
// slip coefficients (c1, c2) from phi, l1, l2
void wall_coef_T(cudaStream_t s, const Grid& g, double dy, const double* l1, const double* l2, const double* phi,
                 const double* lwc, double* lphi, double* ll1, double* ll2);

// ---- linear stencils and pointwise maps ---------------------------------------
void grad_p2a_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lqx,
                const double* lqy, const double* lqz, double* lq);
void grad_prs_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lqx,
                const double* lqy, const double* lqz, double* lq);
// q = ql (1 - phi) + qg phi over all points
void mean_T(cudaStream_t s, const Grid& g, double ql, double qg, const double* lq, double* lphi);
void caldiv_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, const double* ldiv,
              double* lu, double* lv, double* lw);
void corunp_T(cudaStream_t s, const Grid& g, double rho, double dxi, double dyi, double dzi, double dt,
              const double* lun, const double* lvn, const double* lwn, const double* lpn, double* ldp,
              double* lphat);
void calsij_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lsk, double* lu,
              double* lv, double* lw);
void tau_T(cudaStream_t s, const Grid& g, const double* sk, const double* mu, const double* ltau, double* lsk,
           double* lmu);
void div_tensor_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lvu,
                  const double* lvv, const double* lvw, double* ltau);

// ---- transport ------------------------------------------------------------------
void mthinc1_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, double bet,
               const double* phi, const double* gx, const double* gy, const double* gz, const double* u,
               const double* v, const double* w, const double* lfx, const double* lfy, const double* lfz,
               double* lphi, double* lrn, double* lu, double* lv, double* lw, const int* list, const int* count,
               const double* newton);
// lrn (3 arrays of n: per cell the adjoint of the averaged vertex gradient) -> lgx..lgz
void rn_avg_T(cudaStream_t s, const Grid& g, const double* lrn, double* lgx, double* lgy, double* lgz);
void mthinc2_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, const double* u,
               const double* v, const double* w, const double* fx, const double* fy, const double* fz,
               const double* phi, const double* phin, double* lphin, double* lphi, double* lu, double* lv,
               double* lw, double* lfx, double* lfy, double* lfz, double* tmp);
// solphi_mthinc3: pb = its input pa after the band-test snap and clip; pass = 1
// where pb follows pa (gx..gz: vertex gradient of pa, as the forward pass used)
void mthinc3_record(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double bet, const double* gx,
                    const double* gy, const double* gz, const double* pa, double* pb, double* pass);
// adjoints of phin outside the interior (stale step-start values) -> lphin_start
void phin_stale_T(cudaStream_t s, const Grid& g, const double* pass, double* lphin, double* lphin_start);
// sums: (sum phi, sum pb, sum pb^2(1-pb)) of the forward pass; lphin in/out
// (interior), lphi += the volume-sum term; scal: >= 4 doubles of device scratch
void mthinc3_T(cudaStream_t s, const Grid& g, const double* pb, const double* pass, const double* sums,
               double* lphin, double* lphi, double* scal);

// ---- momentum ------------------------------------------------------------------
// work: >= 63n doubles (per-line adjoints of the differences and velocities);
// pairs: the reverse of the FP64 forward in FP32-pair arithmetic (an FP64 forward);
// else split (3n float2, or nullptr: FP64): the reverse of the forward's FP32
// kernel, in FP32 on the split pairs of u, v, w written there first (a
// mixed-precision forward)
void weno_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
            const double* w, const double* const* ladv, double* lu, double* lv, double* lw, double* work,
            float2* split = nullptr, bool pairs = false);
// CSF force of one field: lf (3 arrays) -> lphi; work: >= 42n doubles.  The
// normals and curvature are formed again from phi, normals of gradients at the
// rounding level taken as constants (the noise floor in adj_mom.cu)
void csf_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double rhol, double rhog,
           double sigma, const double* phi, const double* const* lf, double* lphi, double* work);

// ---- viscous solve -------------------------------------------------------------
struct SrcArgs {
  const double *u, *v, *w, *rho, *rhon, *mu;
  const double* E[3];  // exy, exz, eyz
  const double *adv[3], *advo[3], *prs[3], *vis[3], *fst[3], *fstn[3];
};
struct SrcAdj {
  double* u[3];  // adjoints of u, v, w
  double *adv[3], *advo[3], *prs[3], *vis[3], *fst[3], *fstn[3];
  double *rho, *rhon, *mu;
  double *ea[3], *eb[3];  // per component the two edge arrays of its diagonal (see src_ab_T)
};
// from lAB (Au Bu Av Bv Aw Bw adjoints)
void src_ab_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, double grvb,
              double grvp, const SrcArgs& a, const double* const* lAB, const SrcAdj& l);
void edges_T(cudaStream_t s, const Grid& g, int harmonic, const double* mu, const double* const* lE, double* lmu);
// the forward states before each of the 12 sweeps of one outer iteration started at
// ustar: snaps = 39n doubles (12 x 3 fields, then the running state)
void sor_replay(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* mu,
                double* const* E, double* const* AB, double uwall, const double* wallc, const double* const* ustar,
                double* snaps);
// CUDA graphs of one transposed iteration, keyed by the buffers they read and write
using GraphCache = std::map<std::vector<const void*>, std::pair<cudaGraphExec_t, long long>>;
// The executable graph of `body` for this set of buffers (key): captured on s the
// first time, then taken from the cache; nullptr when capture fails (the caller
// then runs body directly).  *per_launch = the kernels one replay launches.
cudaGraphExec_t cached_graph(cudaStream_t s, GraphCache* cache, const std::vector<const void*>& key,
                             const std::function<void()>& body, long long* per_launch);
// transposed fixed-point solve and gradient collection; lam: 3 output arrays (the
// converged adjoint of un*, consumed by the gradient pass); lAB, lmu, lE, lwc
// accumulate; work: >= 3n + 1026 doubles; host_norm: 2 pinned doubles; cache may
// be null (no graphs).  fb_out (3n) receives the feedback term G^T lam of the
// solve and *fb_norm its norm.  Where *fb_norm > 0 on entry, fb holds the previous
// solve's feedback term (and fb_prev, if not null, the one before): the solve
// starts from lout + fb, or lout + 2 fb - fb_prev (a warm start extrapolated in
// time), and its stop rule's scale is *fb_norm.  fb_out may be fb_prev's buffer.
// Returns the iterations used.
int sor_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* mu, double* const* E,
          double* const* AB, double uwall, const double* wallc, const double* const* ustar, const double* snaps,
          const double* const* lout, double* const* lam, double* const* lAB, double* lmu, double* const* lE,
          double* lwc, double tol, int maxit, double* work, double* host_norm, GraphCache* cache, double* fb,
          double* fb_norm, const double* fb_prev, double* fb_out);

}  // namespace adj
}  // namespace fmf
