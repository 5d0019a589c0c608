/*
 * fmf_oracle.h -- CPU oracle for the per-time-step two-phase update of
 * toruneko1129/fel-multi-phase-flow.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * entry point and the CPU-baseline leg of bench.py may load it.  The product
 * (the CUDA library under fel-multi-phase-flow_gb300/) never links or calls it.
 *
 * Each orc_<name> function restates the reference Fortran subroutine <name>
 * with the same argument list and order (every argument by pointer, arrays
 * column-major with origin -2), following the reference file:line cited at
 * its definition in fmf_oracle.cpp.  Arithmetic is IEEE double in the
 * reference's operation order; built with -ffp-contract=off and no
 * fast-math.  Reductions run in a fixed order (per k-plane partial sums added
 * in k order) so results do not depend on the OpenMP thread count.
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists in
 * this build environment, so the restatement is not pinned against the
 * reference's own outputs ("parity unpinned").  It is pinned against numpy's
 * FFT and against physical invariants (projection divergence, volume
 * conservation, Couette profile) in tests/test_oracle_*.py.
 */
#ifndef FMF_ORACLE_H
#define FMF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- C1 MTHINC transport ---------------------------------------------- */
void orc_cal_grad_p2a(const int* ID, const int* svall, const int* ni, const int* nj, const int* nk,
                      const double* dxinv, const double* dyinv_array, const double* dzinv,
                      const double* q, double* qx, double* qy, double* qz);
void orc_solphi_mthinc1(const int* ni, const int* nj, const int* nk,
                        const double* dxinv, const double* dyinv, const double* dzinv, const double* dt,
                        const double* bet_mthinc, const double* phi, const double* phix,
                        const double* phiy, const double* phiz, const double* u, const double* v,
                        const double* w, double* flphix, double* flphiy, double* flphiz);
void orc_solphi_mthinc2(const int* ni, const int* nj, const int* nk,
                        const double* dxinv, const double* dyinv, const double* dzinv, const double* dt,
                        const double* u, const double* v, const double* w, const double* flphix,
                        const double* flphiy, const double* flphiz, const double* phi, double* phin);
void orc_solphi_mthinc3(const int* ipara, const int* ni, const int* nj, const int* nk,
                        const double* dxinv, const double* dyinv, const double* dzinv,
                        const double* bet_mthinc, const double* phix, const double* phiy,
                        const double* phiz, const double* phi, double* phin);
void orc_summation(const int* ni, const int* nj, const int* nk, double* qk, const int* nbub);

/* ---- C5 wall / halo conditions ----------------------------------------- */
void orc_gnbc(const int* nID, const int* ni, const int* nj, const int* nk, const double* uk,
              const double* wk, const double* uwall, const double* theta_0_array,
              const double* surface_tension, const double* zeta_array, double* theta_array);
void orc_bnd_contact_angle(const int* nID, const int* ni, const int* nj, const int* nk, double* qk,
                           const double* theta_array, const double* dx, const double* dy,
                           const double* dz);
void orc_bndu(const int* nID, const int* ni, const int* nj, const int* nk, double* uk, double* vk,
              double* wk, const double* uwall, const double* dy, const double* l1, const double* l2,
              const double* phi);
void orc_bnd_periodic(const int* ni, const int* nj, const int* nk, double* qk);
void orc_bnd_neumann(const int* nID, const int* ni, const int* nj, const int* nk, double* qk);
void orc_bnd_comm(const int* ipara, const int* nID, const int* ni, const int* nj, const int* nk,
                  int* key, double* sendjb, double* recvjb, double* qk);

/* ---- C2 WENO5 ----------------------------------------------------------- */
void orc_cal_advu_weno5(const int* ni, const int* nj, const int* nk, const double* dxinv,
                        const double* dyinv, const double* dzinv, const double* u, const double* v,
                        const double* w, double* adv_u, double* adv_v, double* adv_w);

/* ---- C6 step glue ------------------------------------------------------- */
void orc_cal_arith_mean(const int* ni, const int* nj, const int* nk, const double* phik,
                        const double* ql, const double* qg, double* qk);
void orc_cal_harm_mean(const int* ni, const int* nj, const int* nk, const double* phik,
                       const double* ql, const double* qg, double* qk);
void orc_calphat(const int* ni, const int* nj, const int* nk, const double* p, const double* po,
                 double* phat);
void orc_cal_grad_prs(const int* ni, const int* nj, const int* nk, const double* dxinv,
                      const double* dyinv, const double* dzinv, const double* q, double* qx_u,
                      double* qy_v, double* qz_w);
void orc_calsij(const int* ni, const int* nj, const int* nk, const double* dxinv, const double* dyinv,
                const double* dzinv, const double* uk, const double* vk, const double* wk, double* sk);
void orc_cal_arith_tau(const int* ni, const int* nj, const int* nk, const double* s,
                       const double* rmu, double* tau);
void orc_cal_harm_tau(const int* ni, const int* nj, const int* nk, const double* s,
                      const double* rmu, double* tau);
void orc_cal_div_tensor(const int* ni, const int* nj, const int* nk, const double* dxinv,
                        const double* dyinv, const double* dzinv, const double* tauk, double* uk,
                        double* vk, double* wk);
void orc_calrn(const int* ni, const int* nj, const int* nk, const double* dxinv, const double* dyinv,
               const double* dzinv, const int* ip, const int* jp, const int* kp, const double* phix,
               const double* phiy, const double* phiz, double* rn);
void orc_calrkap(const int* ni, const int* nj, const int* nk, const double* dxinv,
                 const double* dyinv, const double* dzinv, const double* rn_pp, const double* rn_12,
                 const double* rn_13, const double* rn_23, double* rkap);
void orc_cal_grad_p2uvw(const int* ID, const int* svall, const int* ni, const int* nj, const int* nk,
                        const double* dxinv, const double* dyinv_array, const double* dzinv,
                        const double* q, double* qx_u, double* qy_v, double* qz_w);
void orc_calfst(const int* ni, const int* nj, const int* nk, const double* rhol, const double* rhog,
                const double* surface_tension, const double* phix_u, const double* phiy_v,
                const double* phiz_w, const double* rkap, double* fst_u, double* fst_v,
                double* fst_w);
void orc_sum_fst(const int* ni, const int* nj, const int* nk, const double* fst_u,
                 const double* fst_v, const double* fst_w, double* sum_fst_u, double* sum_fst_v,
                 double* sum_fst_w);
void orc_init_q(const int* ni, const int* nj, const int* nk, double* q1, double* q2, double* q3);
void orc_cal_av(const int* ipara, const int* ndiv, const int* ni, const int* nj, const int* nk,
                const double* q, double* av);
void orc_cal_srcu(const int* nID, const int* ni, const int* nj, const int* nk, const double* rho_av,
                  const double* dt, const double* grvb, const double* grvp, const double* u,
                  const double* v, const double* w, const double* rho, const double* rhon,
                  const double* adv_u, const double* adv_v, const double* adv_w,
                  const double* adv_uo, const double* adv_vo, const double* adv_wo,
                  const double* prs_u, const double* prs_v, const double* prs_w,
                  const double* vis_u, const double* vis_v, const double* vis_w,
                  const double* fst_u, const double* fst_v, const double* fst_w,
                  const double* fst_un, const double* fst_vn, const double* fst_wn,
                  double* src_u, double* src_v, double* src_w);
void orc_cpy(const int* ni, const int* nj, const int* nk, const double* q1, double* q2);

/* ---- C3 viscous solve --------------------------------------------------- */
/* coef[45] in the reference argument order (au_w_u ... av_tn_w) */
void orc_cal_arith_coef_vis_v(const int* ni, const int* nj, const int* nk, const double* dxinv,
                              const double* dyinv, const double* dzinv, const double* rmuk,
                              double* const* coef, int harmonic);
/* returns the number of outer iterations executed (lp+1); err ratio in *err_out */
int orc_solu_sor4_v(const int* nID, const int* ni, const int* nj, const int* nk, const double* dt,
                    const double* rho, const double* rhon, const double* const* coef,
                    const double* src_u, const double* src_v, const double* src_w, double* un,
                    double* vn, double* wn, const double* uwall, const double* dy,
                    const double* l1, const double* l2, const double* phi, double* err_out);
/* stop rule of the outer iteration: err/err0 <= tol within max_iter iterations
 * (the reference's 1e-3 and 21 unless changed) */
void orc_set_sor(double tol, int max_iter);

/* ---- C4 pressure ------------------------------------------------------- */
void orc_caldiv(const int* ipara, const int* ndiv, const int* ni, const int* nj, const int* nk,
                const double* dxinv, const double* dyinv, const double* dzinv, const double* dt,
                const double* uk, const double* vk, const double* wk, double* div, double* err_div);
void orc_cal_coef_prs(const int* nj, const double* rho, const double* dxinv, const double* dyinv,
                      const double* dzinv, double* aw_pk, double* ae_pk, double* as_pk,
                      double* an_pk, double* ab_pk, double* at_pk, double* ap_pk);
void orc_cal_coef_solp_fft(const int* nj, const double* as_p, const double* an_p, double* as_p_fft,
                           double* an_p_fft, double* ap_p_fft);
void orc_solp_fft_tdma1(const int* ni, const int* nj, const int* nk, double* fftdata,
                        const double* div, double* phir_r, double* phir_i);
void orc_trans_r2w(const int* ipara, const int* ID, const int* ndiv, const int* svall, int* key,
                   double* sendbuf, double* recvbuf, const double* r, double* w);
void orc_trans_w2r(const int* ipara, const int* ID, const int* ndiv, const int* svall, int* key,
                   double* sendbuf, double* recvbuf, const double* w, double* r);
void orc_solp_fft_tdma2(const int* ID, const int* ndiv, const int* svall, const double* rho,
                        const double* dxinv, const double* dzinv, const double* as_p_fft,
                        const double* an_p_fft, const double* ap_p_fft, double* atdma,
                        double* btdma_r, double* btdma_i, double* phiw_r, double* phiw_i);
void orc_solp_fft_tdma3(const int* ni, const int* nj, const int* nk, double* fftdata,
                        const double* phir_r, const double* phir_i, double* dp);
void orc_solp_fft_tdma4_v(const int* ni, const int* nj, const int* nk, const double* rho,
                          const double* dxinv, const double* dyinv, const double* dzinv,
                          const double* div, const double* dp, double* err_out, double* err0_out);
void orc_bnd_avzero(const int* ipara, const int* ndiv, const int* ni, const int* nj, const int* nk,
                    double* q);
void orc_corunp_explicit(const int* nID, const int* ni, const int* nj, const int* nk,
                         const double* rho, const double* dxinv, const double* dyinv,
                         const double* dzinv, const double* dt, const double* dp,
                         const double* phat, double* un, double* vn, double* wn, double* pn);

/* complex 2-D DFT used by the oracle's pressure solve: data is (n1 fastest, n2),
 * interleaved re/im, sign -1 or +1, unnormalised. */
void orc_fft2d(double* data, int n1, int n2, int sign);

/* ---- A1 objective ------------------------------------------------------ */
double orc_interface_lower(const int* ni, const int* nj, const int* nk, const double* phi,
                           const double* dx, const double* xl);

/* ---- monitors: cal_vel.f, cal_center.f, find_interface_positions_upper.f90 */
void orc_cal_vel(const int* ipara, const int* ni, const int* nj, const int* nk, const double* radius,
                 const double* rhol, const double* rmul, const double* u, const double* v, const double* w,
                 const double* phi, double* vel, double* re);
void orc_cal_center(const int* ipara, const int* ID, const int* svall, const int* ni, const int* nj,
                    const int* nk, const double* xl, const double* yl, const double* zl, const double* dt,
                    const double* rhog, const double* phi, double* center, double* center_pre1,
                    double* center_pre2, int* area_pre1, int* area_pre2, int* lap, double* velocity);
int orc_interface_upper(const int* ni, const int* nj, const int* nk, const double* phi, const double* dx,
                        const double* dz, const double* xl, double* xz, int cap);

/* ---- field output: mkvtk_*.f, mk_slice_j/k.f, mkuwp.h/mkuvp.h, mk_center.f, mk_vel.f
 * (files in the working directory; return 0 on success) */
void orc_format_e(char* buf, double x, int w, int d);
int orc_mkvtk(int kind, const int* svall, const int* nstep, const double* dx, const double* dy,
              const double* dz, double* q, const int* l);
int orc_mkvtk_q(const int* svall, const int* nstep, const double* dx, const double* dy,
                const double* dz, const double* vorx, const double* q);
void orc_mk_slice(int axis, const int* nID, const int* ni, const int* nj, const int* nk,
                  const int* fixed, const int* ip, const int* jp, const int* kp, const double* qk,
                  double* out);
int orc_write_slices(int kind, int nstep, const int* svall, double d1, double d2, const double* s1,
                     const double* s2, const double* s3);
int orc_mk_center(const double* time, const double* center, const double* velocity, const int* l);
int orc_mk_vel(const double* time, const double* vel, const double* re, const double* velocity,
               const int* l);

/* ---- the step driver: main.f90:473-697 ---------------------------------- */
typedef struct {
  int ni, nj, nk;
  double dx, dy, dz, dt;
  double rhol, rhog, rmul, rmug, sigma, uwall, grvb, grvp, bet_mthinc;
  int harmonic;      /* 0: cal_arith_coef_vis (as main.f90 calls), 1: cal_harm_coef_vis */
} orc_params;

/* state arrays (each (ni+6)(nj+6)(nk+6) doubles): u v w uo vo wo p po phi0 phi1 phin0 phin1
 * walls: theta0, zeta, l1, l2 as full 3-D arrays (only j=1 and j=nj planes are read).
 * The workspace persists between steps; create it once per run. */
typedef struct orc_ws orc_ws;
orc_ws* orc_ws_create(const orc_params* prm);
void orc_ws_destroy(orc_ws* ws);
/* one full time step; returns the SOR iteration count; diag[0]=err_div0, diag[1]=sor err ratio */
int orc_step(orc_ws* ws, double* const* state, const double* theta0, const double* zeta,
             const double* l1, const double* l2, double* diag);
/* the start-up boundary sequence of main.f90:322-366 applied to a state whose phi1 interior
 * (and u=v=w=... = 0) has been filled by the caller */
void orc_init_bc(orc_ws* ws, double* const* state, const double* theta0, const double* zeta,
                 const double* l1, const double* l2);

#ifdef __cplusplus
}
#endif
#endif
