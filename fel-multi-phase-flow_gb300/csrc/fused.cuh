// fused.cuh -- kernels of the fused time step (fmf_ctx_step).  These compute the
// same quantities as the drop-in kernels of ops.cuh but fuse reference
// subroutines, skip work whose result the step never reads, and let nvcc
// contract multiply-adds; they are checked against the oracle at 1e-10.
#pragma once
#include "fmf_common.cuh"

namespace fmf {
namespace fused {

// cal_advu_weno5 of (u, v, w) into adv and of (uo, vo, wo) into advo, interior
// cells.  prec 0: FP64; 1: FP32 arithmetic on the split pairs (hi, lo) of the six
// fields, written into `split` (6 n float2) first; 2: FP32-pair arithmetic on the
// same pairs (about 2^-42 of the stencil's values: the FP64-accurate step).
void weno5_both(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u,
                const double* v, const double* w, const double* uo, const double* vo, const double* wo,
                double* const* adv, double* const* advo, int prec = 0, float2* split = nullptr);
// cal_advu_weno5 of (u, v, w) alone into adv (prec 1, 2: split pairs of 3 fields, 3 n float2)
void weno5_one(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
               const double* w, double* const* adv, int prec = 0, float2* split = nullptr);
// the split pairs (hi, lo) of three fields (field f at out[f n ..]; hi + lo = q to
// about 2^-48), as the FP32 WENO5 reads them
void split3(cudaStream_t s, const Grid& g, const double* a, const double* b, const double* c, float2* out);
// both levels, the second (uo, vo, wo into advo) skipped on the device where *keep != 0
void weno5_keep(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
                const double* w, const double* uo, const double* vo, const double* wo, double* const* adv,
                double* const* advo, const int* keep, int prec = 0, float2* split = nullptr);

// cal_grad_p2a (the vertex gradients of q at (i+1/2, j+1/2, k+1/2), i, j, k in
// -2..n+2) in fewer FP64 operations than the reference's order
void vertex_gradient(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* q,
                     double* qx, double* qy, double* qz);

// solphi_mthinc1 for the faces solphi_mthinc2 reads (every face of rows 1..n in
// the two directions normal to it, faces 0..n along it); list/count: device scratch
// of >= (ni+2)(nj+2)(nk+2) ints and one int.  newton (optional, 2 (ni+2)(nj+2)(nk+2)
// doubles): per list entry e the Newton offset at [e] and its last step at
// [(ni+2)(nj+2)(nk+2) + e], for the adjoint.
void mthinc_fluxes(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, double bet,
                   const double* phi, const double* gx, const double* gy, const double* gz, const double* u,
                   const double* v, const double* w, double* fx, double* fy, double* fz, int* list, int* count,
                   bool fp32 = false, double* newton = nullptr);

// CSF force of one field on the interior u, v, w points (fu/fv/fw), replacing
// cal_grad_p2a + calrn x4 + calrkap + cal_grad_p2uvw + calfst; needs ni % 32 == 0
// and nj % 8 == 0 (csf_supported).  prec 0: FP64; 1: normals and curvature in
// FP32; 2: in FP32 pairs (the FP64-accurate step).  kap
// (optional, 3 arrays of n): the curvatures at the interior u, v, w points.
bool csf_supported(const Grid& g);
// skip (optional): a device int; where it is nonzero the kernel writes nothing
void csf_force(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double rhol, double rhog,
               double sigma, const double* phi, double* fu, double* fv, double* fw, int prec = 0,
               double* kap = nullptr, const int* skip = nullptr);

// The explicit viscous term (calsij, cal_arith_tau, cal_div_tensor) at the interior
// u, v, w points into vis[0..2]; tau: 6 n doubles of workspace; sk (optional, 6 n):
// the strain components at the points 0..n+1 the interior divergence reads
// (pairs: the stresses and their divergence in FP32-pair arithmetic, the strain
// still FP64; the FP64-accurate and the mixed-precision steps)
void explicit_viscous(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* u,
                      const double* v, const double* w, const double* mu, double* tau, double* const* vis,
                      double* sk = nullptr, bool pairs = false);

// Viscous solve.  src_visc_prep: edge viscosities E[0..2] (xy, xz, yz edges, i,j,k in
// 0..n), per-component A/B (AB[0..5] = Au Bu Av Bv Aw Bw) with the momentum
// right-hand side of cal_srcu formed in registers, and the Navier-slip wall
// coefficients wallc (2*(nk+6)*(ni+6)*2 doubles) from phi, l1, l2.
void src_visc_prep(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, int harmonic,
                   double grvb, double grvp, const double* u, const double* v, const double* w,
                   const double* const* adv, const double* const* advo, const double* const* prs,
                   const double* const* vis, const double* const* fst, const double* const* fstn, const double* mu,
                   const double* rho, const double* rhon, double* const* E, double* const* AB, const double* l1,
                   const double* l2, const double* phi, double dy, double* wallc, bool pairs = false);
// the Navier-slip coefficients wallc alone (as src_visc_prep computes them)
void wall_coef(cudaStream_t s, const Grid& g, double dy, const double* l1, const double* l2, const double* phi,
               double* wallc);
// bndu followed by bnd_periodic of the components whose bit is set in `normal`.
void wall_halo(cudaStream_t s, const Grid& g, int normal, double uwall, const double* wallc, double* un, double* vn,
               double* wn);
// one outer iteration (u, v, w sweeps of 4 colour pairs each); errsum[0] = sum du^2;
// part: sor_parts(g) doubles of scratch.  FP64 in the FP64-accurate step as well (a
// point update reads 23 doubles for about 30 operations; measured in FP32 pairs the
// splits cost more than the arithmetic saves)
void sor_iteration(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, int harmonic,
                   const double* mu, double* const* E, double* const* AB, double uwall, const double* wallc,
                   double* un, double* vn, double* wn, double* part, double* errsum);
long sor_parts(const Grid& g);

// The pressure Poisson solve (solp_fft_tdma1-3) on the half spectrum of the real
// divergence: div -> dp interior.  pr, pi: (ni/2+1) nj nk doubles each (the spectrum
// after the forward transform and the Thomas solve).
// coef (optional): the Thomas elimination factors of every mode (tdma_coef), formed
// once for the grid and rho; without it each solve forms them again.
void pressure_half(cudaStream_t s, const Grid& g, double rho, double dxinv, double dzinv, const double* as_f,
                   const double* an_f, const double* ap_f, const double* div, double* pr, double* pi, double* dp,
                   const double* coef = nullptr);
long tdma_coef_doubles(const Grid& g);
void tdma_coef(cudaStream_t s, const Grid& g, double rho, double dxinv, double dzinv, const double* as_f,
               const double* an_f, const double* ap_f, double* coef);

// corunp_explicit: un, vn, wn += dt/rho grad(dp) at the interior, pn = phat + dp
void project(cudaStream_t s, const Grid& g, double rho, double dxinv, double dyinv, double dzinv, double dt,
             const double* dp, const double* phat, double* un, double* vn, double* wn, double* pn);

// Mixed-precision viscous solve (one step of iterative refinement).  Buffers:
struct RefineBufs {
  float* d[3];  // corrections d = un - u, v, w (n floats each)
  float* a[3];  // A per component (n)
  float* r[3];  // R = A*visn(u) + B - u, formed in FP64 (A, B in FP32 pairs) (n)
  float* mu;    // mu (n)
  float* e[3];  // edge viscosities (n)
  float* gw;    // wall constants, refine_floats(g, 0)
  float* gx;    // x-halo constants, refine_floats(g, 1)
  float* gz;    // z-halo constants, refine_floats(g, 2)
};
long refine_floats(const Grid& g, int part);
// src_visc_prep's E and wallc, then rb.a, rb.r, rb.mu, rb.e, the wall/halo constants
// from u, v, w, and zero corrections
void refine_prep(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, int harmonic,
                 double grvb, double grvp, const double* u, const double* v, const double* w,
                 const double* const* adv, const double* const* advo, const double* const* prs,
                 const double* const* vis, const double* const* fst, const double* const* fstn, const double* mu,
                 const double* rho, const double* rhon, double* const* E, const double* l1, const double* l2,
                 const double* phi, double dy, double uwall, double* wallc, const RefineBufs& rb);
// one outer iteration on the corrections; errsum[0] = sum of squared increments
void sor_iteration_refine(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                          const RefineBufs& rb, double* part, double* errsum);
// un = u + d, vn = v + d_v, wn = w + d_w at every point
void refine_finish(cudaStream_t s, const Grid& g, const double* u, const double* v, const double* w,
                   const RefineBufs& rb, double* un, double* vn, double* wn);

}  // namespace fused
}  // namespace fmf
