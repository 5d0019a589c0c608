// capi.cu -- the drop-in C-ABI (include/fmf_capi.h, parts 1 and 2).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/fmf_capi.h"
#include "fused.cuh"
#include "ops.cuh"
#include "runtime.cuh"

using namespace fmf;

namespace {
inline long n3(int ni, int nj, int nk) { return (long)(ni + 6) * (nj + 6) * (nk + 6); }
bool check_grid(int ni, int nj, int nk) {
  auto p2 = [](int n) { return n >= 4 && (n & (n - 1)) == 0; };
  if (!p2(ni) || !p2(nj) || !p2(nk)) {
    set_status(FMF_ERR_ARG);
    return false;
  }
  return true;
}
bool one_rank(const int* ipara) {
  if (ipara && *ipara != 0) {
    set_status(FMF_ERR_UNSUPPORTED);
    return false;
  }
  return true;
}
bool walls_only(const int* nID) {
  // one GPU holds the whole domain: both wall neighbours must be absent
  if (nID && (nID[1] >= 0 || nID[4] >= 0)) {
    set_status(FMF_ERR_UNSUPPORTED);
    return false;
  }
  return true;
}
// dyinv_array(dis), dis = j + nj*ID for j in -2..nj+2 (cal_grad_p2a.f:34-36): the device
// kernels take one dy; a non-uniform array is reported as unsupported.
bool uniform_dy(const double* a, int ID, int nj, double* out) {
  const double* base = a + 2 + (long)nj * ID;
  const double v = base[-2];
  for (int j = -2; j <= nj + 2; ++j)
    if (base[j] != v) {
      set_status(FMF_ERR_UNSUPPORTED);
      return false;
    }
  *out = v;
  return true;
}
int g_last_sor_iters = 0;
double g_last_sor_ratio = 0.0;
double g_last_solp[2] = {0.0, 0.0};  // err, err0 of the last solp_fft_tdma4_ monitor
double g_sor_tol = 1.0e-3;           // solu_sor4.f:291 stop rule, fmf_set_sor
int g_sor_max = 21;                  // solu_sor4.f:130 do lp=0,20
}  // namespace

// Every array argument is resolved (evaluated as a macro argument) before the
// launch; nothing is launched if any of them failed.
template <class F, class... A>
inline void launch_if(Call& call, F f, A... a) {
  if (call.ok) f(a...);
}
#define FMF_LAUNCH(fn, ...) launch_if(call, [&](auto... a_) { fn(a_...); }, __VA_ARGS__)

#define GRID3 \
  if (!check_grid(*ni, *nj, *nk)) return; \
  const Grid g(*ni, *nj, *nk);            \
  const long N3 = g.n;                    \
  cudaStream_t s = stream();              \
  Call call;

extern "C" {

int fmf_last_error(void) { return take_status(); }
const char* fmf_error_string(int code) {
  switch (code) {
    case FMF_OK: return "ok";
    case FMF_ERR_CUDA: return "CUDA runtime error";
    case FMF_ERR_ARG: return "invalid argument";
    case FMF_ERR_NONFINITE: return "non-finite value in a reduction";
    case FMF_ERR_ITER_CAP: return "SOR iteration cap reached";
    case FMF_ERR_NOMEM: return "device allocation failed";
    case FMF_ERR_UNSUPPORTED: return "unsupported on the one-GPU build";
    default: return "unknown error";
  }
}
int fmf_set_mode(int m) {
  if (m != FMF_RESIDENT && m != FMF_COHERENT) return FMF_ERR_ARG;
  set_mode(m);
  return 0;
}
int fmf_set_stream(void* st) {
  set_stream((cudaStream_t)st);
  return 0;
}
int fmf_sync_to_host(void* p) { return sync_to_host(p, 0); }
int fmf_sync_to_device(void* p) { return sync_to_device(p, 0); }
int fmf_sync_all_to_host(void) { return sync_all_to_host(); }
int fmf_forget(void* p) { return forget(p); }
int fmf_reset(void) { return reset_registry(); }
int fmf_device_synchronize(void) {
  FMF_CUDA(cudaStreamSynchronize(stream()));
  return take_status();
}
long long fmf_kernel_launches(void) { return launches(); }
int fmf_last_sor_iterations(void) { return g_last_sor_iters; }
double fmf_last_sor_ratio(void) { return g_last_sor_ratio; }
int fmf_last_solp_residual(double* err, double* err0) {
  if (!err || !err0) return FMF_ERR_ARG;
  *err = g_last_solp[0];
  *err0 = g_last_solp[1];
  return FMF_OK;
}
int fmf_set_sor(double tol, int max_iter) {
  if (!(tol > 0.0) || max_iter < 1 || max_iter > 100000) return FMF_ERR_ARG;
  g_sor_tol = tol;
  g_sor_max = max_iter;
  return FMF_OK;
}

// ---------------------------------------------------------------- C1
void cal_grad_p2a_(int* ID, int* svall, int* ni, int* nj, int* nk, double* dxinv, double* dyinv_array,
                   double* dzinv, double* q, double* qx, double* qy, double* qz) {
  (void)svall;
  GRID3;
  double dy;
  if (!uniform_dy(dyinv_array, *ID, *nj, &dy)) return;
  FMF_LAUNCH(op::cal_grad_p2a, s, g, *dxinv, dy, *dzinv, call.in(q, N3), call.out(qx, N3), call.out(qy, N3), call.out(qz, N3));
  call.finish();
}
void solphi_mthinc1_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* dt,
                     double* bet, double* phi, double* phix, double* phiy, double* phiz, double* u, double* v,
                     double* w, double* flx, double* fly, double* flz) {
  GRID3;
  FMF_LAUNCH(op::solphi_mthinc1, s, g, *dxinv, *dyinv, *dzinv, *dt, *bet, call.in(phi, N3), call.in(phix, N3),
                     call.in(phiy, N3), call.in(phiz, N3), call.in(u, N3), call.in(v, N3), call.in(w, N3),
                     call.out(flx, N3), call.out(fly, N3), call.out(flz, N3));
  call.finish();
}
void solphi_mthinc2_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* dt,
                     double* u, double* v, double* w, double* flx, double* fly, double* flz, double* phi,
                     double* phin) {
  GRID3;
  FMF_LAUNCH(op::solphi_mthinc2, s, g, *dxinv, *dyinv, *dzinv, *dt, call.in(u, N3), call.in(v, N3), call.in(w, N3),
                     call.in(flx, N3), call.in(fly, N3), call.in(flz, N3), call.in(phi, N3), call.out(phin, N3));
  call.finish();
}
void solphi_mthinc3_(int* ipara, int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
                     double* bet, double* phix, double* phiy, double* phiz, double* phi, double* phin) {
  if (!one_rank(ipara)) return;
  GRID3;
  double* sums = (double*)scratch(sizeof(double) * 4, 2);
  FMF_LAUNCH(op::solphi_mthinc3, s, g, *dxinv, *dyinv, *dzinv, *bet, call.in(phix, N3), call.in(phiy, N3),
                     call.in(phiz, N3), call.in(phi, N3), call.out(phin, N3), sums);
  call.finish();
}
void summation_(int* ni, int* nj, int* nk, double* qk, int* nbub) {
  GRID3;
  if (*nbub != 1) {
    set_status(FMF_ERR_UNSUPPORTED);
    return;
  }
  double* d = call.out(qk, 2 * N3);
  FMF_LAUNCH(op::summation, s, g, d, d + N3);
  call.finish();
}

// ---------------------------------------------------------------- C5
void gnbc_(int* nID, int* ni, int* nj, int* nk, double* uk, double* wk, double* uwall, double* theta0,
           double* sigma, double* zeta, double* theta) {
  if (!walls_only(nID)) return;
  GRID3;
  FMF_LAUNCH(op::gnbc, s, g, call.in(uk, N3), call.in(wk, N3), *uwall, call.in(theta0, N3), *sigma, call.in(zeta, N3),
           call.out(theta, N3));
  call.finish();
}
void bnd_contact_angle_(int* nID, int* ni, int* nj, int* nk, double* qk, double* theta, double* dx, double* dy,
                        double* dz) {
  if (!walls_only(nID)) return;
  GRID3;
  FMF_LAUNCH(op::bnd_contact_angle, s, g, call.out(qk, N3), call.in(theta, N3), *dx, *dy, *dz);
  call.finish();
}
void bndu_(int* nID, int* ni, int* nj, int* nk, double* uk, double* vk, double* wk, double* uwall, double* dy,
           double* l1, double* l2, double* phi) {
  if (!walls_only(nID)) return;
  GRID3;
  FMF_LAUNCH(op::bndu, s, g, call.out(uk, N3), call.out(vk, N3), call.out(wk, N3), *uwall, *dy, call.in(l1, N3),
           call.in(l2, N3), call.in(phi, N3));
  call.finish();
}
void bnd_periodic_(int* ni, int* nj, int* nk, double* qk) {
  GRID3;
  FMF_LAUNCH(op::bnd_periodic, s, g, call.out(qk, N3));
  call.finish();
}
void bnd_neumann_(int* nID, int* ni, int* nj, int* nk, double* qk) {
  if (!walls_only(nID)) return;
  GRID3;
  FMF_LAUNCH(op::bnd_neumann, s, g, call.out(qk, N3));
  call.finish();
}
void bnd_comm_(int* ipara, int*, int*, int*, int*, int*, double*, double*, double*) { one_rank(ipara); }

// ---------------------------------------------------------------- C2
void cal_advu_weno5_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* u,
                     double* v, double* w, double* au, double* av, double* aw) {
  GRID3;
  FMF_LAUNCH(op::cal_advu_weno5, s, g, *dxinv, *dyinv, *dzinv, call.in(u, N3), call.in(v, N3), call.in(w, N3),
                     call.out(au, N3), call.out(av, N3), call.out(aw, N3));
  call.finish();
}

// ---------------------------------------------------------------- C6
void cal_arith_mean_(int* ni, int* nj, int* nk, double* phik, double* ql, double* qg, double* qk) {
  GRID3;
  FMF_LAUNCH(op::cal_arith_mean, s, g, call.in(phik, N3), *ql, *qg, call.out(qk, N3));
  call.finish();
}
void cal_harm_mean_(int* ni, int* nj, int* nk, double* phik, double* ql, double* qg, double* qk) {
  GRID3;
  FMF_LAUNCH(op::cal_harm_mean, s, g, call.in(phik, N3), *ql, *qg, call.out(qk, N3));
  call.finish();
}
void calphat_(int* ni, int* nj, int* nk, double* p, double* po, double* phat) {
  GRID3;
  FMF_LAUNCH(op::calphat, s, g, call.in(p, N3), call.in(po, N3), call.out(phat, N3));
  call.finish();
}
void cal_grad_prs_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* q,
                   double* qx, double* qy, double* qz) {
  GRID3;
  FMF_LAUNCH(op::cal_grad_prs, s, g, *dxinv, *dyinv, *dzinv, call.in(q, N3), call.out(qx, N3), call.out(qy, N3),
                   call.out(qz, N3));
  call.finish();
}
void calsij_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* uk, double* vk,
             double* wk, double* sk) {
  GRID3;
  FMF_LAUNCH(op::calsij, s, g, *dxinv, *dyinv, *dzinv, call.in(uk, N3), call.in(vk, N3), call.in(wk, N3),
             call.out(sk, 6 * N3));
  call.finish();
}
void cal_arith_tau_(int* ni, int* nj, int* nk, double* sk, double* rmu, double* tau) {
  GRID3;
  FMF_LAUNCH(op::cal_tau, s, g, call.in(sk, 6 * N3), call.in(rmu, N3), call.out(tau, 6 * N3), false);
  call.finish();
}
void cal_harm_tau_(int* ni, int* nj, int* nk, double* sk, double* rmu, double* tau) {
  GRID3;
  FMF_LAUNCH(op::cal_tau, s, g, call.in(sk, 6 * N3), call.in(rmu, N3), call.out(tau, 6 * N3), true);
  call.finish();
}
void cal_div_tensor_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* tau,
                     double* uk, double* vk, double* wk) {
  GRID3;
  FMF_LAUNCH(op::cal_div_tensor, s, g, *dxinv, *dyinv, *dzinv, call.in(tau, 6 * N3), call.out(uk, N3), call.out(vk, N3),
                     call.out(wk, N3));
  call.finish();
}
void calrn_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, int* ip, int* jp, int* kp,
            double* phix, double* phiy, double* phiz, double* rn) {
  GRID3;
  if (*ip < 0 || *ip > 1 || *jp < 0 || *jp > 1 || *kp < 0 || *kp > 1) {
    set_status(FMF_ERR_ARG);
    return;
  }
  FMF_LAUNCH(op::calrn, s, g, *dxinv, *dyinv, *dzinv, *ip, *jp, *kp, call.in(phix, N3), call.in(phiy, N3),
            call.in(phiz, N3), call.out(rn, 3 * N3));
  call.finish();
}
void calrkap_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* rpp,
              double* r12, double* r13, double* r23, double* rkap) {
  GRID3;
  FMF_LAUNCH(op::calrkap, s, g, *dxinv, *dyinv, *dzinv, call.in(rpp, 3 * N3), call.in(r12, 3 * N3), call.in(r13, 3 * N3),
              call.in(r23, 3 * N3), call.out(rkap, 3 * N3));
  call.finish();
}
void cal_grad_p2uvw_(int* ID, int* svall, int* ni, int* nj, int* nk, double* dxinv, double* dyinv_array,
                     double* dzinv, double* q, double* qx, double* qy, double* qz) {
  (void)svall;
  GRID3;
  double dy;
  if (!uniform_dy(dyinv_array, *ID, *nj, &dy)) return;
  FMF_LAUNCH(op::cal_grad_prs, s, g, *dxinv, dy, *dzinv, call.in(q, N3), call.out(qx, N3), call.out(qy, N3),
                   call.out(qz, N3));
  call.finish();
}
void calfst_(int* ni, int* nj, int* nk, double* rhol, double* rhog, double* sigma, double* gx, double* gy,
             double* gz, double* rkap, double* fu, double* fv, double* fw) {
  GRID3;
  FMF_LAUNCH(op::calfst, s, g, *rhol, *rhog, *sigma, call.in(gx, N3), call.in(gy, N3), call.in(gz, N3),
             call.in(rkap, 3 * N3), call.out(fu, N3), call.out(fv, N3), call.out(fw, N3));
  call.finish();
}
void sum_fst_(int* ni, int* nj, int* nk, double* fu, double* fv, double* fw, double* su, double* sv,
              double* sw) {
  GRID3;
  FMF_LAUNCH(op::sum_fst, s, g, call.in(fu, N3), call.in(fv, N3), call.in(fw, N3), call.out(su, N3), call.out(sv, N3),
              call.out(sw, N3));
  call.finish();
}
void init_q_(int* ni, int* nj, int* nk, double* q1, double* q2, double* q3) {
  GRID3;
  FMF_LAUNCH(op::fill, s, N3, call.out(q1, N3), 0.0);
  FMF_LAUNCH(op::fill, s, N3, call.out(q2, N3), 0.0);
  FMF_LAUNCH(op::fill, s, N3, call.out(q3, N3), 0.0);
  call.finish();
}
void cal_av_(int* ipara, int* ndiv, int* ni, int* nj, int* nk, double* q, double* av) {
  if (!one_rank(ipara)) return;
  (void)ndiv;
  GRID3;
  double* d = (double*)scratch(sizeof(double) * 2, 3);
  FMF_LAUNCH(op::cal_av, s, g, call.in(q, N3), d);
  FMF_CUDA(cudaMemcpyAsync(av, d, sizeof(double), cudaMemcpyDeviceToHost, s));
  FMF_CUDA(cudaStreamSynchronize(s));
  if (!std::isfinite(*av)) set_status(FMF_ERR_NONFINITE);
  call.finish();
}
void cal_srcu_(int* nID, int* ni, int* nj, int* nk, double* rho_av, double* dt, double* grvb, double* grvp,
               double* u, double* v, double* w, double* rho, double* rhon, double* adv_u, double* adv_v,
               double* adv_w, double* adv_uo, double* adv_vo, double* adv_wo, double* prs_u, double* prs_v,
               double* prs_w, double* vis_u, double* vis_v, double* vis_w, double* fst_u, double* fst_v,
               double* fst_w, double* fst_un, double* fst_vn, double* fst_wn, double* src_u, double* src_v,
               double* src_w) {
  (void)rho_av;
  if (!walls_only(nID)) return;
  GRID3;
  const double* adv[3] = {call.in(adv_u, N3), call.in(adv_v, N3), call.in(adv_w, N3)};
  const double* advo[3] = {call.in(adv_uo, N3), call.in(adv_vo, N3), call.in(adv_wo, N3)};
  const double* prs[3] = {call.in(prs_u, N3), call.in(prs_v, N3), call.in(prs_w, N3)};
  const double* vis[3] = {call.in(vis_u, N3), call.in(vis_v, N3), call.in(vis_w, N3)};
  const double* fst[3] = {call.in(fst_u, N3), call.in(fst_v, N3), call.in(fst_w, N3)};
  const double* fstn[3] = {call.in(fst_un, N3), call.in(fst_vn, N3), call.in(fst_wn, N3)};
  double* src[3] = {call.out(src_u, N3), call.out(src_v, N3), call.out(src_w, N3)};
  FMF_LAUNCH(op::cal_srcu, s, g, *dt, *grvb, *grvp, call.in(u, N3), call.in(v, N3), call.in(w, N3), call.in(rho, N3),
               call.in(rhon, N3), adv, advo, prs, vis, fst, fstn, src);
  call.finish();
}
void cpy_(int* ni, int* nj, int* nk, double* q1, double* q2) {
  GRID3;
  FMF_LAUNCH(op::copy, s, N3, call.in(q1, N3), call.out(q2, N3));
  call.finish();
}

// ---------------------------------------------------------------- C3
static void coef_vis_impl(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* rmu,
                          double** c45, bool harmonic) {
  GRID3;
  double* d[45];
  for (int q = 0; q < 45; ++q) d[q] = call.out(c45[q], N3);
  FMF_LAUNCH(op::cal_coef_vis, s, g, *dxinv, *dyinv, *dzinv, call.in(rmu, N3), d, harmonic);
  call.finish();
}
#define C45_PARAMS                                                                                        \
  double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7,          \
      double *a8, double *a9, double *a10, double *a11, double *a12, double *a13, double *a14, double *a15, \
      double *a16, double *a17, double *a18, double *a19, double *a20, double *a21, double *a22,            \
      double *a23, double *a24, double *a25, double *a26, double *a27, double *a28, double *a29,            \
      double *a30, double *a31, double *a32, double *a33, double *a34, double *a35, double *a36,            \
      double *a37, double *a38, double *a39, double *a40, double *a41, double *a42, double *a43, double *a44
#define C45_ARRAY                                                                                         \
  {a0,  a1,  a2,  a3,  a4,  a5,  a6,  a7,  a8,  a9,  a10, a11, a12, a13, a14, a15, a16, a17, a18, a19, a20, a21, \
   a22, a23, a24, a25, a26, a27, a28, a29, a30, a31, a32, a33, a34, a35, a36, a37, a38, a39, a40, a41, a42, a43, a44}
void cal_arith_coef_vis_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* rmu,
                         C45_PARAMS) {
  double* c[45] = C45_ARRAY;
  coef_vis_impl(ni, nj, nk, dxinv, dyinv, dzinv, rmu, c, false);
}
void cal_harm_coef_vis_(int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv, double* rmu,
                        C45_PARAMS) {
  double* c[45] = C45_ARRAY;
  coef_vis_impl(ni, nj, nk, dxinv, dyinv, dzinv, rmu, c, true);
}
void solu_sor4_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* key, double* sendjb,
                double* recvjb, int* nstep, int* imon_t, double* dt, double* rho, double* rhon, C45_PARAMS,
                double* src_u, double* src_v, double* src_w, double* un, double* vn, double* wn, double* uwall,
                double* dy, double* l1, double* l2, double* phi) {
  (void)key;
  (void)sendjb;
  (void)recvjb;
  (void)ndiv;
  if (!one_rank(ipara) || !walls_only(nID)) return;
  GRID3;
  double* hc[45] = C45_ARRAY;
  const double* c[45];
  for (int q = 0; q < 45; ++q) c[q] = call.in(hc[q], N3);
  const double* src[3] = {call.in(src_u, N3), call.in(src_v, N3), call.in(src_w, N3)};
  double* du = call.out(un, N3);
  double* dv = call.out(vn, N3);
  double* dw = call.out(wn, N3);
  const double* dr = call.in(rho, N3);
  const double* drn = call.in(rhon, N3);
  const double* dl1 = call.in(l1, N3);
  const double* dl2 = call.in(l2, N3);
  const double* dphi = call.in(phi, N3);
  double* es = (double*)scratch(sizeof(double) * 2, 1);
  if (!call.ok || !es) return;
  double err = 0.0, err0 = 0.0;
  int lp;
  for (lp = 0; lp < g_sor_max; ++lp) {
    op::sor_iteration(s, g, *dt, dr, drn, c, src, du, dv, dw, *uwall, *dy, dl1, dl2, dphi, es);
    double e = 0.0;
    FMF_CUDA(cudaMemcpyAsync(&e, es, sizeof(double), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    if (!std::isfinite(e)) {
      set_status(FMF_ERR_NONFINITE);
      break;
    }
    err = std::sqrt(e / (double)g.cells()) + 1.0e-99;
    if (lp == 0) err0 = err;
    if (err / err0 <= g_sor_tol) break;
  }
  g_last_sor_iters = (lp < g_sor_max ? lp : g_sor_max - 1) + 1;
  g_last_sor_ratio = err0 > 0.0 ? err / err0 : 0.0;
  // the loop ended without meeting the stop rule (solu_sor4.f:130,291-293): the
  // reference carries on with the last iterate; reported, not fatal
  if (lp == g_sor_max && !get_status()) set_status(FMF_ERR_ITER_CAP);
  if (*ID == 0 && *imon_t > 0 && (*nstep % *imon_t) == 0)
    std::printf("Err_solu %10d%10d%20.10E%20.10E%20.10E\n", *nstep, lp, err / err0, err, err0);
  call.finish();
}

// ---------------------------------------------------------------- C4
void caldiv_(int* ipara, int* ndiv, int* ni, int* nj, int* nk, double* dxinv, double* dyinv, double* dzinv,
             double* dt, double* uk, double* vk, double* wk, double* div, double* err_div) {
  if (!one_rank(ipara)) return;
  (void)ndiv;
  GRID3;
  double* e = (double*)scratch(sizeof(double) * 2, 3);
  FMF_LAUNCH(op::caldiv, s, g, *dxinv, *dyinv, *dzinv, *dt, call.in(uk, N3), call.in(vk, N3), call.in(wk, N3),
             call.out(div, N3), e);
  FMF_CUDA(cudaMemcpyAsync(err_div, e, sizeof(double), cudaMemcpyDeviceToHost, s));
  FMF_CUDA(cudaStreamSynchronize(s));
  call.finish();
}
void cal_coef_prs_(int* nj, double* rho, double* dxinv, double* dyinv, double* dzinv, double* aw, double* ae,
                   double* as, double* an, double* ab, double* at, double* ap) {
  // 1-D, computed once before the time loop (main.f90:467): host arithmetic as the reference.
  const int NJ = *nj;
  const double r = *rho;
  for (int j = 1; j <= NJ; ++j) {
    const int t = j + 2;
    aw[t] = *dxinv * *dxinv / r;
    ae[t] = *dxinv * *dxinv / r;
    as[t] = *dyinv * *dyinv / r;
    an[t] = *dyinv * *dyinv / r;
    ab[t] = *dzinv * *dzinv / r;
    at[t] = *dzinv * *dzinv / r;
    ap[t] = aw[t] + ae[t] + as[t] + an[t] + ab[t] + at[t];
  }
  ap[3] = ap[3] - as[3];
  as[3] = 0.0;
  ap[NJ + 2] = ap[NJ + 2] - an[NJ + 2];
  an[NJ + 2] = 0.0;
  for (double* a : {aw, ae, as, an, ab, at, ap})
    if (mode() == FMF_RESIDENT) sync_to_device(a, 0);
}
void cal_coef_solp_fft_(int* nj, double* as_p, double* an_p, double* as_f, double* an_f, double* ap_f) {
  const int NJ = *nj;
  for (int j = 1; j <= NJ; ++j) {
    const int t = j + 2;
    as_f[t] = as_p[t];
    an_f[t] = an_p[t];
    ap_f[t] = as_f[t] + an_f[t];
  }
  ap_f[3] = ap_f[3] - as_f[3];
  as_f[3] = 0.0;
  ap_f[NJ + 2] = ap_f[NJ + 2] - an_f[NJ + 2];
  an_f[NJ + 2] = 0.0;
  for (double* a : {as_f, an_f, ap_f})
    if (mode() == FMF_RESIDENT) sync_to_device(a, 0);
}
void solp_fft_tdma1_(int* ni, int* nj, int* nk, double* fftdata, double* div, double* pr, double* pi) {
  (void)fftdata;
  GRID3;
  const long nm = g.cells();
  FMF_LAUNCH(op::fft_forward_planes, s, g, call.in(div, N3), call.out(pr, nm), call.out(pi, nm));
  call.finish();
}
void trans_r2w_(int* ipara, int* ID, int* ndiv, int* svall, int* key, double* sendbuf, double* recvbuf, double* r,
                double* w) {
  (void)ID;
  (void)key;
  (void)sendbuf;
  (void)recvbuf;
  if (!one_rank(ipara) || *ndiv != 1) return;
  const long nm = (long)svall[0] * svall[1] * svall[2];
  Call call;
  FMF_LAUNCH(op::copy, stream(), nm, call.in(r, nm), call.out(w, nm));
  call.finish();
}
void trans_w2r_(int* ipara, int* ID, int* ndiv, int* svall, int* key, double* sendbuf, double* recvbuf, double* w,
                double* r) {
  (void)ID;
  (void)key;
  (void)sendbuf;
  (void)recvbuf;
  if (!one_rank(ipara) || *ndiv != 1) return;
  const long nm = (long)svall[0] * svall[1] * svall[2];
  Call call;
  FMF_LAUNCH(op::copy, stream(), nm, call.in(w, nm), call.out(r, nm));
  call.finish();
}
void solp_fft_tdma2_(int* ID, int* ndiv, int* svall, double* rho, double* dxinv, double* dzinv, double* as_f,
                     double* an_f, double* ap_f, double* atdma, double* btdma_r, double* btdma_i, double* pr,
                     double* pi) {
  (void)atdma;
  (void)btdma_r;
  (void)btdma_i;
  if (*ndiv != 1 || *ID != 0) {
    set_status(FMF_ERR_UNSUPPORTED);
    return;
  }
  int ni = svall[0], nj = svall[1], nk = svall[2];
  if (!check_grid(ni, nj, nk)) return;
  const Grid g(ni, nj, nk);
  const long nm = g.cells();
  Call call;
  FMF_LAUNCH(op::tdma_modes, stream(), g, *rho, *dxinv, *dzinv, call.in(as_f, nj + 6), call.in(an_f, nj + 6),
                 call.in(ap_f, nj + 6), call.out(pr, nm), call.out(pi, nm));
  call.finish();
}
void solp_fft_tdma3_(int* ni, int* nj, int* nk, double* fftdata, double* pr, double* pi, double* dp) {
  (void)fftdata;
  GRID3;
  const long nm = g.cells();
  FMF_LAUNCH(op::fft_inverse_planes, s, g, call.in(pr, nm), call.in(pi, nm), call.out(dp, N3));
  call.finish();
}
void solp_fft_tdma4_(int* ipara, int* ID, int* ndiv, int* ni, int* nj, int* nk, int* nstep, int* imon_t,
                     double* rho, double* dxinv, double* dyinv, double* dzinv, double* div, double* dp) {
  if (!one_rank(ipara)) return;
  (void)ndiv;
  if (*imon_t <= 0 || (*nstep % *imon_t) != 0) return;
  GRID3;
  double* d = (double*)scratch(sizeof(double) * 2, 3);
  FMF_LAUNCH(op::poisson_residual, s, g, *rho, *dxinv, *dyinv, *dzinv, call.in(div, N3), call.in(dp, N3), d);
  double h[2];
  FMF_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  FMF_CUDA(cudaStreamSynchronize(s));
  const double N = (double)g.cells();
  const double err = std::sqrt(h[0] / N) + 1.0e-99, err0 = std::sqrt(h[1] / N) + 1.0e-99;
  g_last_solp[0] = err;
  g_last_solp[1] = err0;
  if (*ID == 0) std::printf("Err_solp %10d%20.10E%20.10E%20.10E\n", *nstep, err / err0, err, err0);
  call.finish();
}
void bnd_avzero_(int* ipara, int* ndiv, int* ni, int* nj, int* nk, double* q) {
  if (!one_rank(ipara)) return;
  (void)ndiv;
  GRID3;
  FMF_LAUNCH(op::bnd_avzero, s, g, call.out(q, N3));
  call.finish();
}
void corunp_explicit_(int* nID, int* ni, int* nj, int* nk, double* rho, double* dxinv, double* dyinv,
                      double* dzinv, double* dt, double* dp, double* phat, double* un, double* vn, double* wn,
                      double* pn) {
  if (!walls_only(nID)) return;
  GRID3;
  FMF_LAUNCH(op::corunp_explicit, s, g, *rho, *dxinv, *dyinv, *dzinv, *dt, call.in(dp, N3), call.in(phat, N3),
                      call.out(un, N3), call.out(vn, N3), call.out(wn, N3), call.out(pn, N3));
  call.finish();
}

double fmf_interface_lower(int ni, int nj, int nk, const double* phi, double dx, double xl) {
  const Grid g(ni, nj, nk);
  double sum_x = 0.0;
  for (int k = 1; k <= nk; ++k) {
    double xk = 0.0;
    for (int i = 1; i <= ni; ++i) {
      const double p1 = phi[g.at(i, 1, k)], p2 = phi[g.at(i + 1, 1, k)];
      if (p1 > 0.5 && p2 < 0.5) {
        xk = ((double)i - 0.5) * dx + (0.5 - p1) * dx / (p2 - p1) - xl * 0.75;
        break;
      }
    }
    sum_x = sum_x + xk;
  }
  return -(sum_x / (double)nk);
}
void find_interface_positions_lower_(int* ni, int* nj, int* nk, double* phi, double* dx, double* dy, double* dz,
                                     double* xl) {
  (void)dy;
  (void)dz;
  GRID3;
  double* d = (double*)scratch(sizeof(double) * 2, 3);
  FMF_LAUNCH(op::diag_interface_lower, s, g, *dx, *xl, call.in(phi, N3), d);
  double v = 0.0;
  if (call.ok) {
    FMF_CUDA(cudaMemcpyAsync(&v, d, sizeof(double), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    std::printf(" Lower Interface Position (Average over k):\n %.15E\n", v);
  }
  call.finish();
}

// find_interface_positions_upper.f90:1-26: every crossing of the top wall row,
// printed as "x z" lines in the reference's order
void find_interface_positions_upper_(int* ni, int* nj, int* nk, double* phi, double* dx, double* dy, double* dz,
                                     double* xl) {
  (void)dy;
  GRID3;
  const int cap = *ni * *nk;
  double* xz = (double*)scratch(sizeof(double) * (2L * cap + 1), 13);
  int* cnt = (int*)(xz + 2L * cap);
  FMF_LAUNCH(op::diag_interface_upper, s, g, *dx, *dz, *xl, call.in(phi, N3), xz, cnt, cap);
  if (call.ok) {
    int c = 0;
    FMF_CUDA(cudaMemcpyAsync(&c, cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    if (c > cap) c = cap;  // cannot happen: at most one crossing per (i, k)
    std::vector<double> h(2L * (c > 0 ? c : 1));
    if (c > 0) {
      FMF_CUDA(cudaMemcpyAsync(h.data(), xz, sizeof(double) * 2 * c, cudaMemcpyDeviceToHost, s));
      FMF_CUDA(cudaStreamSynchronize(s));
    }
    for (int t = 0; t < c; ++t) std::printf(" %23.15E %23.15E\n", h[2 * t], h[2 * t + 1]);
  }
  call.finish();
}
// find_interface_positions.f90:1-26 is the same routine as the upper one
void find_interface_positions_(int* ni, int* nj, int* nk, double* phi, double* dx, double* dy, double* dz,
                               double* xl) {
  find_interface_positions_upper_(ni, nj, nk, phi, dx, dy, dz, xl);
}

// cal_vel.f:1-82: vel = sum(phi u)/sum(phi) (and v, w), re = rhol vel 2 radius / rmul
void cal_vel_(int* ipara, int* ni, int* nj, int* nk, double* radius, double* rhol, double* rmul, double* u,
              double* v, double* w, double* phi, double* vel, double* re) {
  if (!one_rank(ipara)) return;
  GRID3;
  double* d = (double*)scratch(sizeof(double) * 6, 3);
  FMF_LAUNCH(op::diag_vel, s, g, *radius, *rhol, *rmul, call.in(u, N3), call.in(v, N3), call.in(w, N3),
             call.in(phi, N3), d);
  if (call.ok) {
    double h[6];
    FMF_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    for (int q = 0; q < 3; ++q) {
      vel[q] = h[q];
      re[q] = h[3 + q];
    }
    if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2])) set_status(FMF_ERR_NONFINITE);
  }
  call.finish();
}

// cal_center.f:1-121: centre of mass of phi with x unwrapped across the periodic
// direction, its x velocity, and the (center_pre, area_pre, lap) state update;
// the four sums run on the device, the scalar bookkeeping on the host
void cal_center_(int* ipara, int* ID, int* svall, int* ni, int* nj, int* nk, double* xl, double* yl, double* zl,
                 double* dt, double* rhog, double* phi, double* center, double* center_pre1, double* center_pre2,
                 int* area_pre1, int* area_pre2, int* lap, double* velocity) {
  (void)zl;
  (void)rhog;
  if (!one_rank(ipara)) return;
  GRID3;
  const double L = *xl;
  if (*svall <= 0 || !(L > 0.0)) {
    set_status(FMF_ERR_ARG);
    return;
  }
  const double delta = *yl / (double)*svall;
  const double sensor1 = L * 0.25, sensor2 = L * 0.75;
  if (*area_pre1 == 1 && *area_pre2 == 3) *lap = *lap + 1;
  double* d = (double*)scratch(sizeof(double) * 4, 3);
  FMF_LAUNCH(op::diag_center_sums, s, g, *ID, delta, L, *area_pre1, *lap, call.in(phi, N3), d);
  if (call.ok) {
    double h[4];
    FMF_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    for (int q = 0; q < 3; ++q) center[q] = h[1 + q] / h[0];
    *velocity = (center[0] - *center_pre1) / *dt;
    *center_pre2 = *center_pre1;
    *center_pre1 = center[0];
    double cc = center[0];
    *area_pre2 = *area_pre1;
    if (cc > L && std::isfinite(cc)) {  // the reference's loop never ends on inf
      for (;;) {
        cc = cc - L;
        if (cc < L) break;
      }
    }
    if (cc < sensor1) *area_pre1 = 1;
    if (cc > sensor2) *area_pre1 = 3;
    if (sensor1 <= cc && cc <= sensor2) *area_pre1 = 2;
    if (!std::isfinite(center[0])) set_status(FMF_ERR_NONFINITE);
  }
  call.finish();
}

// ---------------------------------------------------------------- output (f3)
// mk_all.f:1-56: qk_all = wrk_all = qk over rows jst..jen (the whole array on one GPU)
void mk_all_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, double* wrk_all, double* qk,
             double* qk_all) {
  (void)ID;
  if (!one_rank(ipara) || !walls_only(nID)) return;
  if (*ndiv != 1) {
    set_status(FMF_ERR_UNSUPPORTED);
    return;
  }
  GRID3;
  const double* q = call.in(qk, N3);
  double* a = call.out(qk_all, N3);
  double* w = call.out(wrk_all, N3);
  if (call.ok) {
    FMF_CUDA(cudaMemcpyAsync(a, q, sizeof(double) * N3, cudaMemcpyDeviceToDevice, s));
    FMF_CUDA(cudaMemcpyAsync(w, q, sizeof(double) * N3, cudaMemcpyDeviceToDevice, s));
  }
  call.finish();
}
}  // extern "C"
namespace {
void mk_slice(int axis, int* ipara, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* fixed, int* ip, int* jp,
              int* kp, double* wrk_slice, double* qk, double* qk_slice) {
  if (!one_rank(ipara)) return;
  if (*ndiv != 1) {
    set_status(FMF_ERR_UNSUPPORTED);
    return;
  }
  GRID3;
  const int lim = axis == 1 ? *nj : *nk;
  if (*fixed < -2 || *fixed > lim + 2 || *ip < 0 || *ip > 1 || *jp < 0 || *jp > 1 || *kp < 0 || *kp > 1) {
    set_status(FMF_ERR_ARG);
    return;
  }
  // rows from 0 where the domain ends below (nID(Z_MINUS) / nID(Y_MINUS) < 0), else 1
  const int st = (nID ? nID[axis == 1 ? 2 : 1] : -1) < 0 ? 0 : 1;
  const long ns = (long)(*ni + 1) * ((axis == 1 ? *nk : *nj) + 1);
  const double* q = call.in(qk, N3);
  double* o = call.out(qk_slice, ns);
  double* w = call.out(wrk_slice, ns);
  FMF_LAUNCH(op::slice, s, g, q, axis, *fixed, *ip, *jp, *kp, st, o);
  if (call.ok) FMF_CUDA(cudaMemcpyAsync(w, o, sizeof(double) * ns, cudaMemcpyDeviceToDevice, s));
  call.finish();
}
// mkvtk_phi.f / mkvtk_phil.f / mkvtk_p.f: ghosts in place, vertex means, one file
void mkvtk(int kind, const char* fname, const char* scalar, int* svall, int* nstep, double* dx, double* dy,
           double* dz, double* qk) {
  int ni_ = svall[0], nj_ = svall[1], nk_ = svall[2];
  int *ni = &ni_, *nj = &nj_, *nk = &nk_;
  GRID3;
  const long nv = (long)(ni_ + 1) * (nj_ + 1) * (nk_ + 1);
  double* q = call.out(qk, N3);
  double* v = (double*)scratch(sizeof(double) * nv, 14);
  FMF_LAUNCH(op::vtk_ghosts, s, g, q, kind);
  FMF_LAUNCH(op::vtk_vertex, s, g, q, v);
  if (call.ok) {
    std::vector<double> h((size_t)nv);
    FMF_CUDA(cudaMemcpyAsync(h.data(), v, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    const double org[3] = {0.0, 0.0, 0.0}, sp[3] = {*dx, *dy, *dz};
    if (!get_status()) {
      const int st = op::write_vtk(fname, scalar, *nstep, ni_ + 1, nj_ + 1, nk_ + 1, org, sp, h.data());
      if (st) set_status(st);
    }
  }
  call.finish();
}
}  // namespace
extern "C" {
// mk_slice_j.f:1-60 (8-point means at row j over i 0..ni, k 0..nk)
void mk_slice_j_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* j, int* ip, int* jp,
                 int* kp, double* wrk_slice, double* qk, double* qk_slice) {
  (void)ID;
  mk_slice(1, ipara, nID, ndiv, ni, nj, nk, j, ip, jp, kp, wrk_slice, qk, qk_slice);
}
// mk_slice_k.f:1-60 (8-point means at plane k over i 0..ni, j 0..nj)
void mk_slice_k_(int* ipara, int* ID, int* nID, int* ndiv, int* ni, int* nj, int* nk, int* k, int* ip, int* jp,
                 int* kp, double* wrk_slice, double* qk, double* qk_slice) {
  (void)ID;
  mk_slice(2, ipara, nID, ndiv, ni, nj, nk, k, ip, jp, kp, wrk_slice, qk, qk_slice);
}
// mkvtk_phi.f:1-87 -> phi_<nstep>.vtk
void mkvtk_phi_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* q) {
  char f[48];
  std::snprintf(f, sizeof(f), "phi_%07d.vtk", *nstep);
  mkvtk(0, f, "phi", svall, nstep, dx, dy, dz, q);
}
// mkvtk_phil.f:1-88 -> phi<l>_<nstep>.vtk
void mkvtk_phil_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* q, int* l) {
  char f[48];
  std::snprintf(f, sizeof(f), "phi%02d_%07d.vtk", *l, *nstep);
  mkvtk(1, f, "p", svall, nstep, dx, dy, dz, q);
}
// mkvtk_p.f:1-91 -> p_<nstep>.vtk
void mkvtk_p_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* q) {
  char f[48];
  std::snprintf(f, sizeof(f), "p_%07d.vtk", *nstep);
  mkvtk(2, f, "p", svall, nstep, dx, dy, dz, q);
}
// mkvtk_q.f:1-79 -> q1_<nstep>.vtk (q where the x-vorticity is > 0), q2_ (< 0)
void mkvtk_q_(int* svall, int* nstep, double* dx, double* dy, double* dz, double* vorx, double* q) {
  int ni_ = svall[0], nj_ = svall[1], nk_ = svall[2];
  int *ni = &ni_, *nj = &nj_, *nk = &nk_;
  GRID3;
  const long nc = (long)ni_ * nj_ * nk_;
  const double* vx = call.in(vorx, N3);
  const double* qq = call.in(q, N3);
  double* o = (double*)scratch(sizeof(double) * 2 * nc, 14);
  FMF_LAUNCH(op::vtk_q, s, g, vx, qq, o, o + nc);
  if (call.ok) {
    std::vector<double> h((size_t)(2 * nc));
    FMF_CUDA(cudaMemcpyAsync(h.data(), o, sizeof(double) * 2 * nc, cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    const double org[3] = {*dx * 0.5, *dy * 0.5, *dz * 0.5}, sp[3] = {*dx, *dy, *dz};
    for (int t = 0; t < 2 && !get_status(); ++t) {
      char f[48];
      std::snprintf(f, sizeof(f), "q%d_%07d.vtk", t + 1, *nstep);
      const int st = op::write_vtk(f, "p", *nstep, ni_, nj_, nk_, org, sp, h.data() + t * nc);
      if (st) set_status(st);
    }
  }
  call.finish();
}

}  // extern "C"
namespace {
// the slice files of mkuwp.h / mkuvp.h: rows of (a, b, [0,] u, v, phi) with values
// below 1e-40 in magnitude written as 0, a blank record after each row
int write_slice(const char* fname, int n1, int n2, double d1, double d2, bool zero_col, const double* s1,
                const double* s2, const double* s3) {
  FILE* f = std::fopen(fname, "w");
  if (!f) return FMF_ERR_ARG;
  auto clip = [](double x) { return std::fabs(x) < 1.0e-40 ? 0.0 : x; };
  for (int b = 0; b <= n2; ++b) {
    for (int a = 0; a <= n1; ++a) {
      const long o = (long)b * (n1 + 1) + a;
      double v[6];
      int m = 0;
      v[m++] = (double)a * d1;
      v[m++] = (double)b * d2;
      if (zero_col) v[m++] = 0.0;
      v[m++] = clip(s1[o]);
      v[m++] = clip(s2[o]);
      v[m++] = clip(s3[o]);
      op::write_e20(f, v, m);
    }
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  if (ok) std::printf(" output %s\n", fname);
  return ok ? 0 : FMF_ERR_ARG;
}
int append_log(const char* fname, const double* v, int n) {
  FILE* f = std::fopen(fname, "a");
  if (!f) return FMF_ERR_ARG;
  op::write_e20(f, v, n);
  return std::fclose(f) == 0 ? 0 : FMF_ERR_ARG;
}
}  // namespace
extern "C" {
int fmf_write_uwphi(int nstep, const int* svall, double dx, double dz, const double* u_slice, const double* w_slice,
                    const double* phi_slice) {
  if (!svall || !u_slice || !w_slice || !phi_slice) return FMF_ERR_ARG;
  char f[48];
  std::snprintf(f, sizeof(f), "uwphi%07d", nstep);
  return write_slice(f, svall[0], svall[2], dx, dz, false, u_slice, w_slice, phi_slice);
}
int fmf_write_uvwp(int nstep, const int* svall, double dx, double dy, const double* u_slice, const double* v_slice,
                   const double* phi_slice) {
  if (!svall || !u_slice || !v_slice || !phi_slice) return FMF_ERR_ARG;
  char f[48];
  std::snprintf(f, sizeof(f), "uvwp%07d", nstep);
  return write_slice(f, svall[0], svall[1], dx, dy, true, u_slice, v_slice, phi_slice);
}
// mk_center.f:1-23: appends time, center(3), velocity, |(cx, cz) - (0.5, 0.5)| to center_<l>.dat
void mk_center_(int* nstep, double* time, double* center, double* velocity, int* l) {
  (void)nstep;
  char f[48];
  std::snprintf(f, sizeof(f), "center_%02d.dat", *l);
  const double a = center[0] - 0.5, b = center[2] - 0.5;
  const double v[6] = {*time, center[0], center[1], center[2], *velocity, std::sqrt(a * a + b * b)};
  const int st = append_log(f, v, 6);
  if (st) set_status(st);
}
// mk_vel.f:1-20: appends time, vel(3), re(1), re(2), velocity to velocity_<l>.dat
void mk_vel_(int* nstep, double* time, double* vel, double* re, double* velocity, int* l) {
  (void)nstep;
  char f[48];
  std::snprintf(f, sizeof(f), "velocity_%02d.dat", *l);
  const double v[7] = {*time, vel[0], vel[1], vel[2], re[0], re[1], *velocity};
  const int st = append_log(f, v, 7);
  if (st) set_status(st);
}
int fmf_format_fortran_e(char* buf, int bufsize, double x, int w, int d) {
  if (!buf || w < 1 || d < 1 || d > 30 || bufsize < w + 1) return FMF_ERR_ARG;
  op::fortran_e(buf, x, w, d);
  return 0;
}

// ---------------------------------------------------------------- part 2
void fmf_dev_cal_advu_weno5(int ni, int nj, int nk, double dxinv, double dyinv, double dzinv, const double* u,
                            const double* v, const double* w, double* au, double* av, double* aw) {
  if (!check_grid(ni, nj, nk)) return;
  if (!u || !v || !w || !au || !av || !aw) {
    set_status(FMF_ERR_ARG);
    return;
  }
  op::cal_advu_weno5(stream(), Grid(ni, nj, nk), dxinv, dyinv, dzinv, u, v, w, au, av, aw);
  FMF_CUDA(cudaGetLastError());
}
// The fused step's WENO5 of one velocity level (cal_advu_weno5.f:1-258 as the fused
// step evaluates it) in the arithmetic of a context precision: FMF_FP64,
// FMF_MIXED (FP32) or FMF_FP64E (FP32 pairs); interior cells of adv written.
int fmf_dev_weno5_fused(int precision, int ni, int nj, int nk, double dxinv, double dyinv, double dzinv,
                        const double* u, const double* v, const double* w, double* au, double* av, double* aw) {
  if (!check_grid(ni, nj, nk)) return take_status();
  if (!u || !v || !w || !au || !av || !aw || precision < FMF_FP64 || precision > FMF_FP64E) return FMF_ERR_ARG;
  const Grid g(ni, nj, nk);
  float2* split = nullptr;
  if (precision != FMF_FP64) {
    split = (float2*)scratch(sizeof(float2) * 3 * g.n, 6);
    if (!split) return take_status();
  }
  double* adv[3] = {au, av, aw};
  fused::weno5_one(stream(), g, dxinv, dyinv, dzinv, u, v, w, adv, precision, split);
  FMF_CUDA(cudaGetLastError());
  return take_status();
}
// The fused step's CSF force of one volume-fraction field (main.f90:548-567 as the
// fused step evaluates it: cal_grad_p2a, calrn x4, calrkap, cal_grad_p2uvw, calfst)
// in the arithmetic of a context precision; interior u, v, w points of f written.
// Needs ni % 32 == 0 and nj % 8 == 0.
int fmf_dev_csf_fused(int precision, int ni, int nj, int nk, double dx, double dy, double dz, double rhol,
                      double rhog, double sigma, const double* phi, double* fu, double* fv, double* fw) {
  if (!check_grid(ni, nj, nk)) return take_status();
  const Grid g(ni, nj, nk);
  if (!phi || !fu || !fv || !fw || precision < FMF_FP64 || precision > FMF_FP64E || !fused::csf_supported(g))
    return FMF_ERR_ARG;
  fused::csf_force(stream(), g, 1.0 / dx, 1.0 / dy, 1.0 / dz, rhol, rhog, sigma, phi, fu, fv, fw, precision);
  FMF_CUDA(cudaGetLastError());
  return take_status();
}
void fmf_dev_bnd_periodic(int ni, int nj, int nk, double* qk) {
  if (!check_grid(ni, nj, nk)) return;
  if (!qk) {
    set_status(FMF_ERR_ARG);
    return;
  }
  op::bnd_periodic(stream(), Grid(ni, nj, nk), qk);
  FMF_CUDA(cudaGetLastError());
}
void fmf_dev_cal_vel(int ni, int nj, int nk, double radius, double rhol, double rmul, const double* u,
                     const double* v, const double* w, const double* phi, double* out6) {
  if (!check_grid(ni, nj, nk)) return;
  if (!u || !v || !w || !phi || !out6) {
    set_status(FMF_ERR_ARG);
    return;
  }
  op::diag_vel(stream(), Grid(ni, nj, nk), radius, rhol, rmul, u, v, w, phi, out6);
  FMF_CUDA(cudaGetLastError());
}
void fmf_dev_cal_center_sums(int ni, int nj, int nk, int ID, double delta, double xl, int area_pre1, int lap,
                             const double* phi, double* out4) {
  if (!check_grid(ni, nj, nk)) return;
  if (!phi || !out4) {
    set_status(FMF_ERR_ARG);
    return;
  }
  op::diag_center_sums(stream(), Grid(ni, nj, nk), ID, delta, xl, area_pre1, lap, phi, out4);
  FMF_CUDA(cudaGetLastError());
}
void fmf_dev_interface_upper(int ni, int nj, int nk, const double* phi, double dx, double dz, double xl,
                             double* xz, int* count, int cap) {
  if (!check_grid(ni, nj, nk)) return;
  if (!phi || !count || cap < 0 || (cap > 0 && !xz)) {
    set_status(FMF_ERR_ARG);
    return;
  }
  op::diag_interface_upper(stream(), Grid(ni, nj, nk), dx, dz, xl, phi, xz, count, cap);
  FMF_CUDA(cudaGetLastError());
}
void fmf_dev_interface_lower(int ni, int nj, int nk, const double* phi, double dx, double xl, double* out1) {
  if (!check_grid(ni, nj, nk)) return;
  if (!phi || !out1) {
    set_status(FMF_ERR_ARG);
    return;
  }
  op::diag_interface_lower(stream(), Grid(ni, nj, nk), dx, xl, phi, out1);
  FMF_CUDA(cudaGetLastError());
}

}  // extern "C"
