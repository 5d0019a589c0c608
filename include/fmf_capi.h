/*
 * fmf_capi.h -- C-ABI of the GB300 (sm_103a) implementation of the per-time-step
 * two-phase update of toruneko1129/fel-multi-phase-flow.
 *
 * Part 1: drop-in replacements.  Each `<name>_` keeps the reference Fortran
 * subroutine's name (gfortran/ifx external-name mangling: lower case plus one
 * trailing underscore) and its argument list and order.  Every argument is passed
 * by reference, exactly as Fortran 77 passes it: integers are int32, reals are
 * double, arrays are the caller's host arrays, column-major with origin -2, i.e.
 * a pointer to element (-2,-2,-2) of a (-2:ni+3,-2:nj+3,-2:nk+3) array.
 * The routines return nothing, like the originals; a failure is recorded and
 * read with fmf_last_error().  The comment above each declaration cites the
 * reference file:line whose subroutine it replaces.
 *
 * Residency.  Host arrays are mirrored in HBM by a registry keyed by host
 * address.  In FMF_RESIDENT mode (default) the first call that sees an array
 * uploads it; afterwards the device copy is authoritative and consecutive calls
 * move no data between host and device.  Host code that reads an array (I/O,
 * diagnostics) calls fmf_sync_to_host(ptr) first; host code that writes one
 * calls fmf_sync_to_device(ptr) afterwards.  In FMF_COHERENT mode every call
 * uploads all of its array arguments and downloads every array it writes before
 * returning, so the routines behave exactly like the host originals.
 *
 * Scratch arguments of the reference (fftdata, atdma, btdma_*, key, sendjb,
 * recvjb, sendbuf, recvbuf) are accepted and not touched: the device code keeps
 * its own scratch.  With one rank (ipara=0) the reference's MPI routines are
 * in-device copies or no-ops (bnd_comm.f:18, trans_r2w.f:23-38).
 *
 * Part 2: device-pointer variants fmf_dev_<name>: the same arguments, but every
 * array is a device pointer (scalars stay host pointers), enqueued on the
 * library stream (fmf_set_stream).
 *
 * Part 3: the fused, device-resident time step (fmf_ctx_*), which runs the
 * whole of main.f90:473-697 on the GPU.
 *
 * Threading: one host thread drives the library at a time (the reference's
 * single-threaded caller contract).  All work goes to one CUDA stream.
 */
#ifndef FMF_CAPI_H
#define FMF_CAPI_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* status, residency                                                         */
/* ------------------------------------------------------------------------ */
enum {
  FMF_OK = 0,
  FMF_ERR_CUDA = 1,        /* a CUDA runtime call failed */
  FMF_ERR_ARG = 2,         /* invalid argument (size, null pointer, grid not a power of two) */
  FMF_ERR_NONFINITE = 3,   /* NaN/Inf met in a reduction (volume sum, SOR residual, mean) */
  FMF_ERR_ITER_CAP = 4,    /* the SOR hit its 21-iteration cap (reported, not fatal) */
  FMF_ERR_NOMEM = 5,       /* device allocation failed */
  FMF_ERR_UNSUPPORTED = 6  /* a multi-rank (ipara=1) argument on the one-GPU build */
};
enum { FMF_RESIDENT = 0, FMF_COHERENT = 1 };

int fmf_last_error(void);                 /* last status, then cleared */
const char* fmf_error_string(int code);
int fmf_set_mode(int mode);               /* FMF_RESIDENT or FMF_COHERENT */
int fmf_set_stream(void* cuda_stream);    /* NULL: the library's own stream */
int fmf_sync_to_host(void* host_ptr);     /* copy one mirrored array back */
int fmf_sync_to_device(void* host_ptr);   /* re-upload one mirrored array */
int fmf_sync_all_to_host(void);
int fmf_forget(void* host_ptr);           /* drop one mirror (host array about to be freed) */
int fmf_reset(void);                      /* drop every mirror */
int fmf_device_synchronize(void);
/* kernels this library launched since load (a counter kept by its launch helpers) */
long long fmf_kernel_launches(void);

/* ------------------------------------------------------------------------ */
/* Part 1: drop-in replacements of the reference subroutines                 */
/* ------------------------------------------------------------------------ */

/* srcs/cal_grad_p2a.f:1-76 (svall is svall(2), the global nj) */
void cal_grad_p2a_(int* ID, int* svall, int* ni, int* nj, int* nk, double* dxinv,
                   double* dyinv_array, double* dzinv, double* q, double* qx, double* qy,
                   double* qz);
/* srcs/solphi_mthinc1.f:1-292 */
void solphi_mthinc1_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                     double* dt, double* bet_mthinc, double* phi, double* phix, double* phiy,
                     double* phiz, double* u, double* v, double* w, double* flphix,
                     double* flphiy, double* flphiz);
/* srcs/solphi_mthinc2.f:1-48 */
void solphi_mthinc2_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                     double* dt, double* u, double* v, double* w, double* flphix, double* flphiy,
                     double* flphiz, double* phi, double* phin);
/* srcs/solphi_mthinc3.f:1-163 */
void solphi_mthinc3_(int* ipara, int* ni, int* nj, int* nk, double* dxinv, double* dyinv,
                     double* dzinv, double* bet_mthinc, double* phix, double* phiy, double* phiz,
                     double* phi, double* phin);
/* srcs/summation.f:1-54 (qk is the 4-D array qk(...,0:nbub)) */
void summation_(int* ni, int* nj, int* nk, double* qk, int* nbub);
/* srcs/gnbc.f90:1-100 */
void gnbc_(int* nID, int* ni, int* nj, int* nk, double* uk, double* wk, double* uwall,
           double* theta_0_array, double* surface_tension, double* zeta_array,
           double* theta_array);
/* srcs/bnd_contact_angle.f90:1-88 */
void bnd_contact_angle_(int* nID, int* ni, int* nj, int* nk, double* qk, double* theta_array,
                        double* dx, double* dy, double* dz);
/* srcs/bndu.f:1-161 */
void bndu_(int* nID, int* ni, int* nj, int* nk, double* uk, double* vk, double* wk,
           double* uwall, double* dy, double* l1, double* l2, double* phi);
/* srcs/bnd_periodic.f:1-44 */
void bnd_periodic_(int* ni, int* nj, int* nk, double* qk);
/* srcs/bnd_neumann.f:1-46 */
void bnd_neumann_(int* nID, int* ni, int* nj, int* nk, double* qk);
/* srcs/bnd_comm.f:1-121 (ipara=0: nothing to exchange on one GPU) */
void bnd_comm_(int* ipara, int* nID, int* ni, int* nj, int* nk, int* key, double* sendjb,
               double* recvjb, double* qk);
/* srcs/cal_advu_weno5.f:1-258 with srcs/weno5.h:1-71 */
void cal_advu_weno5_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                     double* u, double* v, double* w, double* adv_u, double* adv_v,
                     double* adv_w);
/* srcs/cal_arith_mean.f:1-29 */
void cal_arith_mean_(int* ni, int* nj, int* nk, double* phik, double* ql, double* qg, double* qk);
/* srcs/cal_harm_mean.f:30-58 */
void cal_harm_mean_(int* ni, int* nj, int* nk, double* phik, double* ql, double* qg, double* qk);
/* srcs/calphat.f:1-26 */
void calphat_(int* ni, int* nj, int* nk, double* p, double* po, double* phat);
/* srcs/cal_grad_prs.f:1-41 */
void cal_grad_prs_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                   double* q, double* qx_u, double* qy_v, double* qz_w);
/* srcs/calsij.f:1-143 (sk is sk(...,6)) */
void calsij_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* uk,
             double* vk, double* wk, double* sk);
/* srcs/cal_arith_tau.f:1-121 */
void cal_arith_tau_(int* ni, int* nj, int* nk, double* s, double* rmu, double* tau);
/* srcs/cal_harm_tau.f:1-121 */
void cal_harm_tau_(int* ni, int* nj, int* nk, double* s, double* rmu, double* tau);
/* srcs/cal_div_tensor.f:1-89 */
void cal_div_tensor_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                     double* tauk, double* uk, double* vk, double* wk);
/* srcs/calrn.f:1-91 (rn is rn(...,3)) */
void calrn_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, int* ip,
            int* jp, int* kp, double* phix, double* phiy, double* phiz, double* rn);
/* srcs/calrkap.f:1-101 */
void calrkap_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
              double* rn_pp, double* rn_12, double* rn_13, double* rn_23, double* rkap);
/* srcs/cal_grad_p2uvw.f:1-47 */
void cal_grad_p2uvw_(int* ID, int* svall, int* ni, int* nj, int* nk, double* dxinv,
                     double* dyinv_array, double* dzinv, double* q, double* qx_u, double* qy_v,
                     double* qz_w);
/* srcs/calfst.f:1-49 */
void calfst_(int* ni, int* nj, int* nk, double* rhol, double* rhog, double* surface_tension,
             double* phix_u, double* phiy_v, double* phiz_w, double* rkap, double* fst_u,
             double* fst_v, double* fst_w);
/* srcs/sum_fst.f:1-37 */
void sum_fst_(int* ni, int* nj, int* nk, double* fst_u, double* fst_v, double* fst_w,
              double* sum_fst_u, double* sum_fst_v, double* sum_fst_w);
/* srcs/init_q.f:1-29 */
void init_q_(int* ni, int* nj, int* nk, double* q1, double* q2, double* q3);
/* srcs/cal_av.f:1-40 */
void cal_av_(int* ipara, int* ndiv, int* ni, int* nj, int* nk, double* q, double* av);
/* srcs/cal_srcu.f:1-141 */
void cal_srcu_(int* nID, int* ni, int* nj, int* nk, double* rho_av, double* dt, double* grvb,
               double* grvp, double* u, double* v, double* w, double* rho, double* rhon,
               double* adv_u, double* adv_v, double* adv_w, double* adv_uo, double* adv_vo,
               double* adv_wo, double* prs_u, double* prs_v, double* prs_w, double* vis_u,
               double* vis_v, double* vis_w, double* fst_u, double* fst_v, double* fst_w,
               double* fst_un, double* fst_vn, double* fst_wn, double* src_u, double* src_v,
               double* src_w);
/* srcs/cpy.f:1-24 */
void cpy_(int* ni, int* nj, int* nk, double* q1, double* q2);
/* srcs/cal_arith_coef_vis.f:1-411 */
void cal_arith_coef_vis_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                         double* rmuk, double* au_w_uk, double* au_e_uk, double* au_s_uk,
                         double* au_n_uk, double* au_b_uk, double* au_t_uk, double* au_p_uk,
                         double* av_ws_uk, double* av_es_uk, double* av_wn_uk, double* av_en_uk,
                         double* aw_wb_uk, double* aw_eb_uk, double* aw_wt_uk, double* aw_et_uk,
                         double* av_w_vk, double* av_e_vk, double* av_s_vk, double* av_n_vk,
                         double* av_b_vk, double* av_t_vk, double* av_p_vk, double* au_sw_vk,
                         double* au_nw_vk, double* au_se_vk, double* au_ne_vk, double* aw_sb_vk,
                         double* aw_nb_vk, double* aw_st_vk, double* aw_nt_vk, double* aw_w_wk,
                         double* aw_e_wk, double* aw_s_wk, double* aw_n_wk, double* aw_b_wk,
                         double* aw_t_wk, double* aw_p_wk, double* au_bw_wk, double* au_tw_wk,
                         double* au_be_wk, double* au_te_wk, double* av_bs_wk, double* av_ts_wk,
                         double* av_bn_wk, double* av_tn_wk);
/* srcs/cal_harm_coef_vis.f:1-411 (same arguments) */
void cal_harm_coef_vis_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                        double* rmuk, double* au_w_uk, double* au_e_uk, double* au_s_uk,
                        double* au_n_uk, double* au_b_uk, double* au_t_uk, double* au_p_uk,
                        double* av_ws_uk, double* av_es_uk, double* av_wn_uk, double* av_en_uk,
                        double* aw_wb_uk, double* aw_eb_uk, double* aw_wt_uk, double* aw_et_uk,
                        double* av_w_vk, double* av_e_vk, double* av_s_vk, double* av_n_vk,
                        double* av_b_vk, double* av_t_vk, double* av_p_vk, double* au_sw_vk,
                        double* au_nw_vk, double* au_se_vk, double* au_ne_vk, double* aw_sb_vk,
                        double* aw_nb_vk, double* aw_st_vk, double* aw_nt_vk, double* aw_w_wk,
                        double* aw_e_wk, double* aw_s_wk, double* aw_n_wk, double* aw_b_wk,
                        double* aw_t_wk, double* aw_p_wk, double* au_bw_wk, double* au_tw_wk,
                        double* au_be_wk, double* au_te_wk, double* av_bs_wk, double* av_ts_wk,
                        double* av_bn_wk, double* av_tn_wk);
/* srcs/solu_sor4.f:1-308 */
void solu_sor4_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* key,
                double* sendjb, double* recvjb, int* nstep, int* imon_t, double* dt, double* rho,
                double* rhon, double* au_w_u, double* au_e_u, double* au_s_u, double* au_n_u,
                double* au_b_u, double* au_t_u, double* au_p_u, double* av_ws_u,
                double* av_es_u, double* av_wn_u, double* av_en_u, double* aw_wb_u,
                double* aw_eb_u, double* aw_wt_u, double* aw_et_u, double* av_w_v,
                double* av_e_v, double* av_s_v, double* av_n_v, double* av_b_v, double* av_t_v,
                double* av_p_v, double* au_sw_v, double* au_nw_v, double* au_se_v,
                double* au_ne_v, double* aw_sb_v, double* aw_nb_v, double* aw_st_v,
                double* aw_nt_v, double* aw_w_w, double* aw_e_w, double* aw_s_w, double* aw_n_w,
                double* aw_b_w, double* aw_t_w, double* aw_p_w, double* au_bw_w, double* au_tw_w,
                double* au_be_w, double* au_te_w, double* av_bs_w, double* av_ts_w,
                double* av_bn_w, double* av_tn_w, double* src_u, double* src_v, double* src_w,
                double* un, double* vn, double* wn, double* uwall, double* dy, double* l1,
                double* l2, double* phi);
/* srcs/caldiv.f:1-70 */
void caldiv_(int* ipara, int* ndiv, int* ni, int* nj, int* nk, double* dxinv, double* dyinv,
             double* dzinv, double* dt, double* uk, double* vk, double* wk, double* div,
             double* err_div);
/* srcs/cal_coef_prs.f:1-57 (1-D arrays (-2:nj+3)) */
void cal_coef_prs_(int* nj, double* rho, double* dxinv, double* dyinv, double* dzinv,
                   double* aw_pk, double* ae_pk, double* as_pk, double* an_pk, double* ab_pk,
                   double* at_pk, double* ap_pk);
/* srcs/cal_coef_solp_fft.f:1-42 */
void cal_coef_solp_fft_(int* nj, double* as_p, double* an_p, double* as_p_fft, double* an_p_fft,
                        double* ap_p_fft);
/* srcs/solp_fft_tdma1.f:1-50 (fftdata: scratch, not used) */
void solp_fft_tdma1_(int* ni, int* nj, int* nk, double* fftdata, double* div, double* phir_r,
                     double* phir_i);
/* srcs/trans_r2w.f:1-111 (serial branch :23-38) */
void trans_r2w_(int* ipara, int* ID, int* ndiv, int* svall, int* key, double* sendbuf,
                double* recvbuf, double* r, double* w);
/* srcs/trans_w2r.f:1-111 (serial branch :23-38) */
void trans_w2r_(int* ipara, int* ID, int* ndiv, int* svall, int* key, double* sendbuf,
                double* recvbuf, double* w, double* r);
/* srcs/solp_fft_tdma2.f:1-91 (atdma, btdma_r, btdma_i: scratch, not used) */
void solp_fft_tdma2_(int* ID, int* ndiv, int* svall, double* rho, double* dxinv, double* dzinv,
                     double* as_p_fft, double* an_p_fft, double* ap_p_fft, double* atdma,
                     double* btdma_r, double* btdma_i, double* phiw_r, double* phiw_i);
/* srcs/solp_fft_tdma3.f:1-48 */
void solp_fft_tdma3_(int* ni, int* nj, int* nk, double* fftdata, double* phir_r, double* phir_i,
                     double* dp);
/* srcs/solp_fft_tdma4.f:1-98 (prints the Err_solp monitor line every imon_t steps) */
void solp_fft_tdma4_(int* ipara, int* ID, int* ndiv, int* ni, int* nj, int* nk, int* nstep,
                     int* imon_t, double* rho, double* dxinv, double* dyinv, double* dzinv,
                     double* div, double* dp);
/* srcs/bnd_avzero.f:1-27 */
void bnd_avzero_(int* ipara, int* ndiv, int* ni, int* nj, int* nk, double* q);
/* srcs/corunp_explicit.f:1-78 */
void corunp_explicit_(int* nID, int* ni, int* nj, int* nk, double* rho, double* dxinv,
                      double* dyinv, double* dzinv, double* dt, double* dp, double* phat,
                      double* un, double* vn, double* wn, double* pn);
/* srcs/find_interface_positions_lower.f90:1-35 (prints -x_avg like the reference;
 * computed on the device, one double read back) */
void find_interface_positions_lower_(int* ni, int* nj, int* nk, double* phi, double* dx,
                                     double* dy, double* dz, double* xl);
/* srcs/find_interface_positions_upper.f90:1-26 (prints each crossing "x z" of the top
 * wall row in the reference's k-outer, i-inner order) */
void find_interface_positions_upper_(int* ni, int* nj, int* nk, double* phi, double* dx,
                                     double* dy, double* dz, double* xl);
/* srcs/find_interface_positions.f90:1-26 (the same routine as the upper one) */
void find_interface_positions_(int* ni, int* nj, int* nk, double* phi, double* dx, double* dy,
                               double* dz, double* xl);
/* srcs/cal_vel.f:1-82 (vel(3), re(3) out; ipara must be 0: one GPU holds the domain) */
void cal_vel_(int* ipara, int* ni, int* nj, int* nk, double* radius, double* rhol, double* rmul,
              double* u, double* v, double* w, double* phi, double* vel, double* re);
/* srcs/cal_center.f:1-121 (center(3), velocity out; center_pre1/2, area_pre1/2, lap
 * updated as the reference updates them; zl and rhog unused as in the reference) */
void cal_center_(int* ipara, int* ID, int* svall, int* ni, int* nj, int* nk, double* xl,
                 double* yl, double* zl, double* dt, double* rhog, double* phi, double* center,
                 double* center_pre1, double* center_pre2, int* area_pre1, int* area_pre2,
                 int* lap, double* velocity);

/* Field output.  The gathers and cell-to-vertex means run on the device; the files
 * are written by the host in the reference's formats (Fortran Ew.d numbers), in the
 * working directory, with the reference's names. */
/* srcs/mk_all.f:1-56 (one rank: qk_all = wrk_all = qk; ndiv must be 1) */
void mk_all_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, double* wrk_all,
             double* qk, double* qk_all);
/* srcs/mk_slice_j.f:1-60 (qk_slice(0:ni,0:nk) = 8-point means at row j; ndiv must be 1) */
void mk_slice_j_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* j,
                 int* ip, int* jp, int* kp, double* wrk_slice, double* qk, double* qk_slice);
/* srcs/mk_slice_k.f:1-60 (qk_slice(0:ni,0:nj) = 8-point means at plane k) */
void mk_slice_k_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* k,
                 int* ip, int* jp, int* kp, double* wrk_slice, double* qk, double* qk_slice);
/* srcs/mkvtk_phi.f:1-87 (fills q's ghosts in place as the reference does; phi_<nstep>.vtk) */
void mkvtk_phi_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* q);
/* srcs/mkvtk_phil.f:1-88 (phi<l>_<nstep>.vtk) */
void mkvtk_phil_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* q, int* l);
/* srcs/mkvtk_p.f:1-91 (p_<nstep>.vtk) */
void mkvtk_p_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* q);
/* srcs/mkvtk_q.f:1-79 (q1_<nstep>.vtk, q2_<nstep>.vtk) */
void mkvtk_q_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* vorx, double* q);
/* srcs/mk_center.f:1-23 (appends one record to center_<l>.dat) */
void mk_center_(int* nstep, double* time, double* center, double* velocity, int* l);
/* srcs/mk_vel.f:1-20 (appends one record to velocity_<l>.dat) */
void mk_vel_(int* nstep, double* time, double* vel, double* re, double* velocity, int* l);
/* The slice files the reference writes inline from srcs/mkuwp.h:1-23 (uwphi<nstep>: x, z,
 * u, w, phi over i 0..svall(1), k 0..svall(3)) and srcs/mkuvp.h:1-24 (uvwp<nstep>: x, y,
 * 0, u, v, phi over i 0..svall(1), j 0..svall(2)); the slices are host arrays as
 * mk_slice_j_/mk_slice_k_ return them.  Return FMF_OK or FMF_ERR_ARG. */
int fmf_write_uwphi(int nstep, const int* svall, double dx, double dz, const double* u_slice,
                    const double* w_slice, const double* phi_slice);
int fmf_write_uvwp(int nstep, const int* svall, double dx, double dy, const double* u_slice,
                   const double* v_slice, const double* phi_slice);
/* x as Fortran's Ew.d edit descriptor writes it (w characters and a NUL into buf,
 * bufsize >= w + 1); the formatter of the writers above.  Returns FMF_OK or
 * FMF_ERR_ARG. */
int fmf_format_fortran_e(char* buf, int bufsize, double x, int w, int d);

/* Monitors the reference prints, returned instead of printed (no counterpart
 * with this signature in the reference; the values are those of
 * srcs/solu_sor4.f:298-305 and srcs/solp_fft_tdma4.f:84-93). */
int fmf_last_sor_iterations(void);      /* lp+1 of the last solu_sor4_ call */
double fmf_last_sor_ratio(void);        /* err/err0 of the last solu_sor4_ call */
/* err and err0 (RMS Poisson residual and RMS div) of the last solp_fft_tdma4_
 * call that computed them (srcs/solp_fft_tdma4.f:84-93) */
int fmf_last_solp_residual(double* err, double* err0);
/* Stop rule of solu_sor4_: err/err0 <= tol within max_iter outer iterations (the
 * reference's 1e-3 and 21, srcs/solu_sor4.f:130,291 -- the defaults).  A call that
 * ends without meeting it leaves FMF_ERR_ITER_CAP in fmf_last_error() and keeps
 * the last iterate, as the reference does.  No counterpart in the reference. */
int fmf_set_sor(double tol, int max_iter);
double fmf_interface_lower(int ni, int nj, int nk, const double* phi_host, double dx,
                           double xl);

/* Interior mean of q (the value cal_av_ returns in av) for callers that must not
 * allocate device memory while they run: code working inside another
 * framework's memory pool or a fixed memory budget, or in the middle of its own
 * stream-ordered work.  No counterpart in the reference.  q (the
 * (-2:ni+3,-2:nj+3,-2:nk+3) field) and av (one double) are device pointers;
 * the work is enqueued on `stream` (NULL: the legacy default stream) and no
 * cudaMalloc/cudaFree or allocating library routine is called.  Its scratch is a
 * 512 KiB array compiled into the library, so ceil(nj/8)*nk must not exceed
 * 65536 and nk must not exceed 65535 (FMF_ERR_ARG otherwise, nothing launched).  All calls on a GPU share
 * that array: calls that overlap in time on one GPU race.  The first call on
 * each device looks up the array's address; make it before any stream capture.
 * Returns FMF_OK or an FMF_ERR_* code. */
int fmf_cal_av_noalloc(int ni, int nj, int nk, const double* q, double* av, void* stream);

/* ------------------------------------------------------------------------ */
/* Part 2: device-pointer variants (arrays are device pointers)             */
/* ------------------------------------------------------------------------ */
void fmf_dev_cal_advu_weno5(int ni, int nj, int nk, double dxinv, double dyinv, double dzinv,
                            const double* u, const double* v, const double* w, double* adv_u,
                            double* adv_v, double* adv_w);
/* the fused step's WENO5 of one velocity level in a context precision (FMF_FP64,
 * FMF_MIXED: FP32, FMF_FP64E: FP32 pairs), interior cells; returns a status */
int fmf_dev_weno5_fused(int precision, int ni, int nj, int nk, double dxinv, double dyinv,
                        double dzinv, const double* u, const double* v, const double* w,
                        double* adv_u, double* adv_v, double* adv_w);
/* the fused step's CSF force of one phi field in a context precision, interior u, v,
 * w points (ni % 32 == 0, nj % 8 == 0); returns a status */
int fmf_dev_csf_fused(int precision, int ni, int nj, int nk, double dx, double dy, double dz,
                      double rhol, double rhog, double sigma, const double* phi, double* fu,
                      double* fv, double* fw);
void fmf_dev_bnd_periodic(int ni, int nj, int nk, double* qk);
/* Monitors on device arrays, results left in device memory (nothing is read back,
 * no host synchronisation):
 * srcs/cal_vel.f:36-80 -- out6[0..2] = vel, out6[3..5] = re */
void fmf_dev_cal_vel(int ni, int nj, int nk, double radius, double rhol, double rmul,
                     const double* u, const double* v, const double* w, const double* phi,
                     double* out6);
/* srcs/cal_center.f:36-76 -- out4 = sum phi, sum phi*x, sum phi*y, sum phi*z with x
 * unwrapped for (area_pre1, lap) and delta = yl/svall; the caller keeps the
 * lap/area state (center = out4[1..3] / out4[0]) */
void fmf_dev_cal_center_sums(int ni, int nj, int nk, int ID, double delta, double xl,
                             int area_pre1, int lap, const double* phi, double* out4);
/* srcs/find_interface_positions_upper.f90:13-24 -- xz[2c], xz[2c+1] = (x, z) of the
 * crossings in print order for c < min(*count, cap); *count (device int) = their number */
void fmf_dev_interface_upper(int ni, int nj, int nk, const double* phi, double dx, double dz,
                             double xl, double* xz, int* count, int cap);
/* srcs/find_interface_positions_lower.f90:15-32 -- out1[0] = -x_avg */
void fmf_dev_interface_lower(int ni, int nj, int nk, const double* phi, double dx, double xl,
                             double* out1);

/* ------------------------------------------------------------------------ */
/* Part 3: the fused device-resident step (main.f90:473-697)                */
/* ------------------------------------------------------------------------ */
typedef struct {
  int ni, nj, nk;                 /* nj: the wall-normal count; all powers of two */
  double dx, dy, dz, dt;
  double rhol, rhog, rmul, rmug;  /* phi=0 fluid (l) and phi=1 fluid (g) */
  double sigma, uwall, grvb, grvp, bet_mthinc;
  int harmonic;                   /* 0: cal_arith_coef_vis (as main.f90 calls it), 1: harmonic */
  int precision;                  /* FMF_FP64, FMF_MIXED or FMF_FP64E */
} fmf_params;
/* FMF_FP64: every operation in FP64.  FMF_MIXED: FP32 WENO5, MTHINC, CSF and viscous
 * corrections (errors about 1e-6).  FMF_FP64E: the FP64 step with four of its
 * FP64-pipe-bound stages in FP32-pair arithmetic (a value is the sum of two
 * floats, about 48 significant bits) on the FP32 pipe: the WENO5 advection, the
 * CSF force, the viscous solve's momentum factors (A, B) and the explicit viscous
 * term; each stage reads doubles, splits them into pairs with integer operations
 * and rounds its outputs to doubles once.  The state, the viscous sweeps, the
 * pressure solve, the projection and the volume sums stay FP64, and the step
 * agrees with the oracle within the FP64 step's 1e-10 with the same viscous
 * iteration counts.  The WENO5 term agrees with FP64's to about 4e-13 of |vel|
 * dxi times the stencil's largest value (its differences are taken between split
 * values, each within 2^-48 of its double), and is 0 where the differences are
 * below 2^-99.  Contexts only (fmf_adj_create takes FMF_FP64 and FMF_MIXED). */
enum { FMF_FP64 = 0, FMF_MIXED = 1, FMF_FP64E = 2 };

typedef struct fmf_ctx fmf_ctx;
/* state order: u v w uo vo wo p po phi0 phi1 phin0 phin1, each (ni+6)(nj+6)(nk+6) doubles */
int fmf_ctx_create(const fmf_params* prm, fmf_ctx** out);
int fmf_ctx_destroy(fmf_ctx* ctx);
/* walls: theta0, zeta, l1, l2 as full 3-D host arrays (only the j=1 and j=nj planes are read) */
int fmf_ctx_set_walls(fmf_ctx* ctx, const double* theta0, const double* zeta, const double* l1,
                      const double* l2);
int fmf_ctx_upload(fmf_ctx* ctx, const double* const* state);   /* host -> device, async */
int fmf_ctx_download(fmf_ctx* ctx, double* const* state);       /* device -> host, async */
int fmf_ctx_init_bc(fmf_ctx* ctx);                  /* start-up boundary pass, main.f90:322-366 */
/* nsteps full time steps; returns FMF_ERR_ITER_CAP (after all nsteps) where a
 * step's viscous solve ended without meeting its stop rule -- the step carries on
 * with the last iterate, as the reference's does -- unless a worse error occurred.
 * The stop rule runs on the device, so the steps are enqueued without waiting for
 * the host; a residual that is not finite is reported (FMF_ERR_NONFINITE) after
 * the call's steps. */
int fmf_ctx_step(fmf_ctx* ctx, int nsteps);
/* the viscous solve's stop rule err/err0 <= tol within max_iter outer iterations
 * (default: the reference's 1e-3 and 21, srcs/solu_sor4.f:130,291) */
int fmf_ctx_set_sor(fmf_ctx* ctx, double tol, int max_iter);
/* One step from host buffers to host buffers: in[12] -> out[12] (the state layout
 * of fmf_ctx_upload; pinned host memory lets the copies overlap the step).  The
 * same result as fmf_ctx_upload + fmf_ctx_step(ctx, 1) + fmf_ctx_download: uo, vo,
 * wo, p, po go up while the step's first part runs (phin is not read: the step
 * writes it first), and the result fields that are final early (uo, vo, wo, po,
 * phi, phin) come back while the rest runs.  Returns after the result is in out.
 * No counterpart in the reference: the drop-in form of its time-step loop body. */
int fmf_ctx_step_host(fmf_ctx* ctx, const double* const* in, double* const* out);
int fmf_ctx_synchronize(fmf_ctx* ctx);
int fmf_ctx_set_stream(fmf_ctx* ctx, void* cuda_stream);
/* per-step SOR iteration counts of the last fmf_ctx_step call (up to cap entries) */
int fmf_ctx_sor_iterations(fmf_ctx* ctx, int* out, int cap);
/* device pointers of the state fields (for zero-copy consumers).  A step that
 * continues from the context's previous step reuses that step's advection of
 * (u, v, w) as its advection of (uo, vo, wo) and its surface tension of phin(1) as
 * that of phi(1); this call, fmf_ctx_upload, fmf_ctx_init_bc, fmf_ctx_set_walls
 * and fmf_ctx_step_host end that.  A caller that writes a state field through the
 * pointer must do so before its next fmf_ctx_step, or call this function again
 * after writing. */
int fmf_ctx_state_device_ptr(fmf_ctx* ctx, int field, void** out);
/* bytes of device memory held by the context */
long long fmf_ctx_device_bytes(fmf_ctx* ctx);
/* CUDA-event time of one stage of the step on the context stream (mean ms per
 * launch over reps): 0 WENO5 advection of both velocity levels, 1 one outer SOR
 * iteration, 2 pressure FFT+TDMA, 3 MTHINC fluxes, 4 WENO5 advection of (u, v, w)
 * alone (the level a continuing step computes).  Measurement support; no
 * counterpart in the reference. */
int fmf_ctx_time_stage(fmf_ctx* ctx, int stage, int reps, float* ms);
/* The next step's viscous solve (srcs/solu_sor4.f) measured against the FP64 stop
 * rule, on the current state, which is left as it was (the next step recomputes
 * the carried advection and surface tension).  Runs the step up to the solve and the
 * solve in the context's precision, then FP64 outer iterations on copies:
 *   out[0] outer iterations of the context's solve;
 *   out[1] err/err0 at its last iteration (in FMF_MIXED: of the FP32 correction);
 *   out[2] the RMS change of one FP64 outer iteration from the solve's result over
 *          the FP64 first-iteration change from un = u (the FP64 solve's err0);
 *   out[3] the same from the result of an FP64 solve run to the same rule;
 *   out[4] RMS(un - un_fp64) / RMS(un_fp64 - u) over the interior.
 * In FMF_FP64, out[2] = out[3] and out[4] = 0.  Measurement support; no
 * counterpart in the reference. */
int fmf_ctx_check_sor(fmf_ctx* ctx, double* out);
/* FMA throughput of this GPU in TFLOP/s (fp64=1: double, 0: float), from a
 * register-only kernel timed with CUDA events; the FP64 roofline denominator.
 * Measurement support; no counterpart in the reference. */
int fmf_measure_fma_rate(int fp64, double* tflops);
/* Largest relative error, over n positive normal doubles spread over 2^-1000 ..
 * 2^1000, of the division-free reciprocal the fused WENO5 kernel uses (Newton-
 * Raphson from an approximate reciprocal) against the IEEE quotient 1.0 / x.
 * Verification support; no counterpart in the reference. */
int fmf_check_reciprocal(long long n, double* max_rel_err);
/* The same for the division-free reciprocal square root of the fused CSF kernel
 * (Newton-Raphson from an approximate reciprocal square root) against
 * 1.0 / sqrt(x). */
int fmf_check_rsqrt(long long n, double* max_rel_err);
/* Largest relative error of the (hi, lo) float pairs the mixed-precision WENO5
 * splits each double into (hi + lo against the double), over n values of both
 * signs spread over 2^-96 .. 2^127.  Verification support; no counterpart in the
 * reference. */
int fmf_check_split_pair(long long n, double* max_rel_err);

/* ---- restart files (host code; no GPU needed) ---------------------------
 * One Fortran unformatted sequential record, as the reference writes it: u v w p
 * uo vo wo po (each (ni+6)(nj+6)(nk+6) doubles), phi(0:nbub), time (real*8),
 * nstep (integer*4), framed with gfortran's 4-byte record markers (subrecords of
 * at most 2^31-9 bytes).  fields: the 8 arrays in that order. */
int fmf_write_checkpoint(const char* path, int ni, int nj, int nk, int nbub, int nstep, double time,
                         const double* const* fields, const double* phi);
int fmf_read_checkpoint(const char* path, int ni, int nj, int nk, int nbub, int* nstep, double* time,
                        double* const* fields, double* phi);
/* dataou.f:1-46: writes x<nstep> (x<nstep>_<ID> if ipara = 1); mirrored arrays are
 * copied back from the device first */
void dataou_(int* ipara, int* ID, int* ni, int* nj, int* nk, int* nbub, int* nstep, double* time, double* u,
             double* v, double* w, double* p, double* uo, double* vo, double* wo, double* po, double* phi);
/* datain.f:1-46: reads x.inp (x.inp_<ID> if ipara = 1); mirrored arrays are
 * re-uploaded */
void datain_(int* ipara, int* ID, int* ni, int* nj, int* nk, int* nbub, int* nstep, double* time, double* u,
             double* v, double* w, double* p, double* uo, double* vo, double* wo, double* po, double* phi);

/* ===================================================================== part 4
 * Adjoint of the K-step rollout.  No counterpart in the reference (it has no
 * derivatives); the objective is its find_interface_positions_lower
 * (find_interface_positions_lower.f90:15-32): J = -mean over k of the first
 * phi(i,1,k) > 0.5 > phi(i+1,1,k) crossing of phi slice 0 after K steps, taken from
 * a state to which the start-up boundary pass (main.f90:322-366) is applied first.
 * The forward pass is the step of fmf_ctx_step in the handle's precision
 * (prm->precision: FMF_FP64, or FMF_MIXED for the mixed-precision forward) with
 * the viscous solve run to sor_tol; the reverse pass, in FP64, recomputes each step
 * from checkpoints taken every `every` steps (0: ceil(sqrt(K))) and differentiates
 * the FP64 step's operations at the states that forward produced.  In an FMF_MIXED
 * handle the reverse of the WENO5 advection runs in FP32, as its forward does
 * (environment FMF_ADJ_F32_REVERSE=0 at creation keeps it FP64); in an FMF_FP64
 * handle it runs in FP32-pair arithmetic on FP64 differences, to about 1e-11 of
 * the FP64 reverse (FMF_ADJ_PAIR_REVERSE=0 at creation keeps it FP64). */
typedef struct fmf_adj fmf_adj;
int fmf_adj_create(const fmf_params* prm, fmf_adj** out);
int fmf_adj_destroy(fmf_adj* adj);
/* viscous-solve stop rule err/err0 <= sor_tol within sor_max iterations (the
 * reference: 1e-3, 21) and the transposed solve's tolerance / cap: a reverse step's
 * transposed solve starts from the previous reverse step's solution and stops when
 * its change falls to adj_tol times the size of its feedback term (the first
 * reverse step of a rollout: of its first change) */
int fmf_adj_set_solver(fmf_adj* adj, double sor_tol, int sor_max, double adj_tol, int adj_max);
/* forward only: J after K steps; state_out (12 host fields) may be NULL */
int fmf_adj_forward(fmf_adj* adj, int K, const double* const* state0, const double* theta0,
                    const double* zeta, const double* l1, const double* l2, double* J,
                    double* const* state_out);
/* J and dJ/d(theta0, zeta, l1, l2, initial phi slice 1), each a host array of
 * (ni+6)(nj+6)(nk+6) doubles (NULL: not returned) */
int fmf_adj_rollout(fmf_adj* adj, int K, int every, const double* const* state0, const double* theta0,
                    const double* zeta, const double* l1, const double* l2, double* J, double* g_theta0,
                    double* g_zeta, double* g_l1, double* g_l2, double* g_phi);
/* viscous-solve iterations of the last call: forward (all recomputations) and transposed */
int fmf_adj_iterations(fmf_adj* adj, int* sor_total, int* adjoint_total);
/* device bytes the handle holds (work arrays, record slots, checkpoints, and those
 * of the second handle that recomputes segments beside the reverse) */
long long fmf_adj_device_bytes(fmf_adj* adj);
/* wall-clock seconds of the last fmf_adj_rollout: forward pass, segment
 * recomputation, reverse steps */
int fmf_adj_phase_seconds(fmf_adj* adj, double* seconds3);

#ifdef __cplusplus
}
#endif
#endif
