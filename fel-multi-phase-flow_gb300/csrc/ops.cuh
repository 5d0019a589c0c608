// ops.cuh -- device-level implementations of the reference subroutines.
// Every function takes device pointers in the reference's Fortran layout and
// enqueues its kernels on stream s; none synchronises or allocates (scratch comes
// from fmf::scratch).  Each one reproduces exactly the write set of the
// subroutine it replaces (cited in the .cu file that defines it).
#pragma once
#include <cstdio>
#include "fmf_common.cuh"

namespace fmf {
namespace op {

// C1 MTHINC
void cal_grad_p2a(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                  const double* q, double* qx, double* qy, double* qz);
void solphi_mthinc1(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt,
                    double bet, const double* phi, const double* phix, const double* phiy,
                    const double* phiz, const double* u, const double* v, const double* w, double* flx,
                    double* fly, double* flz);
void solphi_mthinc2(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt,
                    const double* u, const double* v, const double* w, const double* flx,
                    const double* fly, const double* flz, const double* phi, double* phin);
// sums: device buffer of >= 4 doubles (scratch); returns nothing, phin updated in place
void solphi_mthinc3(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double bet,
                    const double* phix, const double* phiy, const double* phiz, const double* phi,
                    double* phin, double* sums);
void summation(cudaStream_t s, const Grid& g, double* q0, const double* q1);

// C5 walls / halos
void gnbc(cudaStream_t s, const Grid& g, const double* uk, const double* wk, double uwall,
          const double* theta0, double sigma, const double* zeta, double* theta);
void bnd_contact_angle(cudaStream_t s, const Grid& g, double* qk, const double* theta, double dx,
                       double dy, double dz);
void bndu(cudaStream_t s, const Grid& g, double* uk, double* vk, double* wk, double uwall, double dy,
          const double* l1, const double* l2, const double* phi);
void bnd_periodic(cudaStream_t s, const Grid& g, double* qk);
void bnd_neumann(cudaStream_t s, const Grid& g, double* qk);

// C2 WENO5
void cal_advu_weno5(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                    const double* u, const double* v, const double* w, double* au, double* av,
                    double* aw);

// C6 glue
void cal_arith_mean(cudaStream_t s, const Grid& g, const double* phi, double ql, double qg, double* q);
// rho, rhon, rmu, rmun = cal_arith_mean of (rhol, rhog) and (rmul, rmug) over phi0
// and phin0 in one pass (main.f90:526-529; the same values as the four calls)
void mixture_means(cudaStream_t s, const Grid& g, const double* phi0, const double* phin0, double rhol, double rhog,
                   double rmul, double rmug, double* rho, double* rhon, double* rmu, double* rmun);
void cal_harm_mean(cudaStream_t s, const Grid& g, const double* phi, double ql, double qg, double* q);
void calphat(cudaStream_t s, const Grid& g, const double* p, const double* po, double* phat);
void cal_grad_prs(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                  const double* q, double* qx, double* qy, double* qz);
void calsij(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* u,
            const double* v, const double* w, double* sk);
void cal_tau(cudaStream_t s, const Grid& g, const double* sk, const double* rmu, double* tau,
             bool harmonic);
void cal_div_tensor(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                    const double* tau, double* vu, double* vv, double* vw);
void calrn(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, int ip, int jp, int kp,
           const double* phix, const double* phiy, const double* phiz, double* rn);
void calrkap(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* rpp,
             const double* r12, const double* r13, const double* r23, double* rkap);
void calfst(cudaStream_t s, const Grid& g, double rhol, double rhog, double sigma, const double* gx,
            const double* gy, const double* gz, const double* rkap, double* fu, double* fv, double* fw);
void sum_fst(cudaStream_t s, const Grid& g, const double* fu, const double* fv, const double* fw,
             double* su, double* sv, double* sw);
void fill(cudaStream_t s, long n, double* q, double value);
void copy(cudaStream_t s, long n, const double* a, double* b);
// interior mean -> out[0] (device)
void cal_av(cudaStream_t s, const Grid& g, const double* q, double* out);
// Monitors (diag.cu), results in device memory, nothing read back:
// cal_vel.f:36-80 -- out[0..2] = vel, out[3..5] = re
void diag_vel(cudaStream_t s, const Grid& g, double radius, double rhol, double rmul, const double* u,
              const double* v, const double* w, const double* phi, double* out);
// cal_center.f:36-76 -- out[0] = sum phi, out[1..3] = sum phi * (x, y, z) with x
// unwrapped for (area_pre1, lap); delta = yl / svall
void diag_center_sums(cudaStream_t s, const Grid& g, int ID, double delta, double xl, int area_pre1, int lap,
                      const double* phi, double* out);
// find_interface_positions_upper.f90:13-24 -- the crossings of row nj in print order:
// xz[2c], xz[2c+1] = (x, z) for c < min(count, cap), *count = number of crossings
void diag_interface_upper(cudaStream_t s, const Grid& g, double dx, double dz, double xl, const double* phi,
                          double* xz, int* count, int cap);
// find_interface_positions_lower.f90:15-32 -- out[0] = -x_avg
void diag_interface_lower(cudaStream_t s, const Grid& g, double dx, double xl, const double* phi, double* out);
// Field output (vtk.cu).  vtk_ghosts: the ghost fill of mkvtk_*.f in place (kind 0
// phi: copies in y and z; 1 phil: zeros in y, copies in z; 2 p: copies in y,
// periodic in z; x periodic for all); vtk_vertex: the 8-point means at the
// (mi+1)(mj+1)(mk+1) vertices 0..m; vtk_q: mkvtk_q.f's two masked copies of q;
// slice: mk_slice_j.f (axis 1, fixed j) / mk_slice_k.f (axis 2, fixed k)
void vtk_ghosts(cudaStream_t s, const Grid& g, double* q, int kind);
void vtk_vertex(cudaStream_t s, const Grid& g, const double* q, double* out);
void vtk_q(cudaStream_t s, const Grid& g, const double* vorx, const double* q, double* out1, double* out2);
void slice(cudaStream_t s, const Grid& g, const double* q, int axis, int fixed, int ip, int jp, int kp, int st,
           double* out);
// host: Fortran Ew.d output (w characters + NUL), the VTK file, one '(20e20.10)' record
void fortran_e(char* out, double x, int w, int d);
int write_vtk(const char* fname, const char* scalar, int nstep, int nx, int ny, int nz, const double* origin,
              const double* spacing, const double* vals);
void write_e20(FILE* f, const double* v, int n);
void cal_srcu(cudaStream_t s, const Grid& g, double dt, double grvb, double grvp, const double* u,
              const double* v, const double* w, const double* rho, const double* rhon,
              const double* const* adv, const double* const* advo, const double* const* prs,
              const double* const* vis, const double* const* fst, const double* const* fstn,
              double* const* src);

// C3 viscous solve
void cal_coef_vis(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                  const double* rmu, double* const* coef, bool harmonic);
// One outer SOR iteration (3 components x 8 colours with the halo refresh after
// even colours).  errsum: device double receiving sum(du^2) of the iteration.
void sor_iteration(cudaStream_t s, const Grid& g, double dt, const double* rho, const double* rhon,
                   const double* const* coef, const double* const* src, double* un, double* vn, double* wn,
                   double uwall, double dy, const double* l1, const double* l2, const double* phi,
                   double* errsum);

// C4 pressure
void caldiv(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt,
            const double* u, const double* v, const double* w, double* div, double* err_out);
void fft_forward_planes(cudaStream_t s, const Grid& g, const double* div, double* pr, double* pi);
void tdma_modes(cudaStream_t s, const Grid& g, double rho, double dxinv, double dzinv, const double* as_f,
                const double* an_f, const double* ap_f, double* pr, double* pi);
void fft_inverse_planes(cudaStream_t s, const Grid& g, const double* pr, const double* pi, double* dp);
void bnd_avzero(cudaStream_t s, const Grid& g, double* q);
void corunp_explicit(cudaStream_t s, const Grid& g, double rho, double dxinv, double dyinv,
                     double dzinv, double dt, const double* dp, const double* phat, double* un,
                     double* vn, double* wn, double* pn);
// Poisson residual monitor: out[0]=sum(res^2), out[1]=sum(div^2)
void poisson_residual(cudaStream_t s, const Grid& g, double rho, double dxinv, double dyinv, double dzinv,
                      const double* div, const double* dp, double* out);

}  // namespace op
}  // namespace fmf
