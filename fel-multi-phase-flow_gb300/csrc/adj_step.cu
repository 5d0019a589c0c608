// adj_step.cu -- the adjoint of the K-step rollout (include/fmf_capi.h part 4).
//
// Objective: J = find_interface_positions_lower (find_interface_positions_lower.f90:
// 15-32) of phi slice 0 after K steps, started from a state to which the start-up
// boundary pass (main.f90:322-366) is applied first.  Parameters: the per-wall-cell
// static angle theta0, the GNBC coefficient zeta, the slip lengths l1, l2 (all four as
// full arrays, read on the wall planes) and the initial phi (slice 1).
//
// Forward: the FP64 step of step.cu written out with its intermediates kept
// (record_step), with the viscous solve run to a configurable tolerance.  Reverse:
// for each step, newest first, the step is recomputed from its start state and the
// adjoint kernels of adj_*.cu run in the opposite order.  Start states are
// checkpointed every C steps and recomputed between checkpoints (C ~ sqrt(K)).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <functional>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fmf_capi.h"
#include "adj.cuh"
#include "fused.cuh"
#include "ops.cuh"
#include "runtime.cuh"

using namespace fmf;

namespace {
enum { SU, SV, SW, SUO, SVO, SWO, SP, SPO, SPHI0, SPHI1, SPHIN0, SPHIN1, NSTATE };
}

// Per-stage device time of the reverse steps (FMF_ADJ_TIME set: CUDA events at the
// stage boundaries, summed per stage and printed to stderr when the handle closes)
struct StageTimer {
  bool on = std::getenv("FMF_ADJ_TIME") != nullptr;
  std::vector<cudaEvent_t> ev;
  std::vector<const char*> name;
  size_t used = 0;
  std::map<std::string, double> ms;
  void mark(cudaStream_t s, const char* stage) {
    if (!on) return;
    if (used == ev.size()) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      ev.push_back(e);
      name.push_back(nullptr);
    }
    name[used] = stage;
    cudaEventRecord(ev[used++], s);
  }
  void flush(cudaStream_t s) {
    if (!on || used == 0) return;
    cudaStreamSynchronize(s);
    for (size_t t = 1; t < used; ++t) {
      float v = 0.0f;
      if (cudaEventElapsedTime(&v, ev[t - 1], ev[t]) == cudaSuccess) ms[name[t]] += v;
    }
    used = 0;
  }
  ~StageTimer() {
    if (on && !ms.empty()) {
      double tot = 0.0;
      for (auto& e : ms) tot += e.second;
      for (auto& e : ms) std::fprintf(stderr, "adjoint stage %-10s %10.3f ms  %5.1f %%\n", e.first.c_str(), e.second, 100.0 * e.second / tot);
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
};

struct fmf_adj {
  fmf_params prm;
  Grid g;
  // precision FMF_MIXED: the forward (and recomputed) steps run the mixed-precision
  // kernels of the product step (FP32 WENO5, MTHINC Newton and fluxes, CSF, viscous
  // corrections); the record keeps what they produced and the reverse is FP64
  bool mixed = false;
  fused::RefineBufs rb{};    // FP32 buffers of the mixed viscous solve
  float2* wsplit = nullptr;  // split pairs of the velocity fields for the FP32 WENO5
  long long bytes = 0;       // device bytes this handle allocated
  cudaStream_t s = nullptr;
  void* scr = nullptr;
  std::vector<void*> allocs;
  StageTimer stimer;
  double sor_tol = 1.0e-3;
  int sor_max = 21;
  double adj_tol = 1.0e-12;
  int adj_max = 200;
  // walls
  double *theta0, *zeta, *l1, *l2;
  // working state (the step runs in place on it)
  double* S[NSTATE];
  // record of one step
  double *gx1[3], *fl[3], *pa, *gxn[3], *pb, *pass, *sums, *pc, *theta, *phn1f;
  double *rho, *rhon, *rmu, *rmun, *adv[3], *advo[3], *phat, *prs[3], *sk, *tau, *vis[3];
  double *sfst[3], *sfstn[3], *E[3], *AB[6], *wallc, *ustar[3], *un2[3], *snaps, *sorpart;
  double *un[3], *pn, *dp, *div, *pr, *pi, *as_f, *an_f, *ap_f, *red;
  double* csfwork;  // forward CSF chain (drop-in): G(3n) rn(12n) kap(3n) g(3n) f(3n)
  int* band;        // MTHINC band-cell list and its length
  double* newton;   // per band-list entry: Newton offset, last Newton step
  // adjoints
  double* lS[NSTATE];  // adjoint of the step-start state (in/out of reverse_step)
  double *lgx[3], *lfl[3], *lrn, *ltheta, *lphn0, *lphn1, *lrho, *lrhon, *lrmu, *lrmun;
  double *ladv[3], *ladvo[3], *lphat, *lprs[3], *lsk, *ltau, *lvis[3], *lsfst[3], *lsfstn[3];
  double *lE[3], *lAB[6], *lwc, *lun[3], *lam[3], *lpn, *ldp, *ldiv, *lpre, *work;
  double *gtheta0, *gzeta, *gl1, *gl2;  // parameter gradients
  // init_bc record
  double *ib_theta1, *ib_theta2, *ib_phi1, *ib_phi0, *ib_u, *ib_w, *ib_wallc;
  // checkpoints
  std::vector<double*> ckpt;
  std::vector<double*> seg;
  int sor_total = 0, adj_total = 0;
  double t_phase[3] = {0.0, 0.0, 0.0};  // seconds: forward, segment recomputation, reverse
  // record slots: what reverse_step reads of one step (its intermediates and its
  // start state), one slot per step of a checkpoint segment when memory allows
  struct Rec {
    double *gx1[3], *fl[3], *pb, *pass, *pc, *theta, *phn1f, *rho, *rhon, *rmu, *rmun;
    double *adv[3], *advo[3], *prs[3], *vis[3], *sfst[3], *sfstn[3], *sk, *E[3], *AB[6], *ustar[3], *un2[3];
    double *wallc, *sums, *state, *newton;
    int* band;
  };
  std::vector<Rec> recs;
  std::vector<void*> rec_blocks;
  double* lblock = nullptr;  // the intermediate adjoints (one memset per reverse step)
  long lblock_n = 0;
  adj::GraphCache graphs;      // transposed viscous iterations, one per record slot
  adj::GraphCache fgraphs;     // forward viscous iterations, one per record slot
  adj::GraphCache rgraphs;     // replays of the last forward viscous cycle, one per record slot
  adj::GraphCache pgraphs;     // the parts before and after the viscous solve of steps not recorded
  bool rec_warm = false;       // a step has run on this handle (scratch sized for capture)
  // The state continues from this handle's previous record_step (cont): that step's
  // advection of (u, v, w) is this step's of (uo, vo, wo), and its surface tension
  // of phin(1) this step's of phi(1); where they were written
  bool cont = false;
  bool no_carry = false;  // FMF_STEP_CACHE=0 at creation: recompute both levels every step
  double *prev_adv[3] = {nullptr, nullptr, nullptr}, *prev_sfstn[3] = {nullptr, nullptr, nullptr};
  // The reverse counterpart: the transposed advection and surface tension are linear
  // in the adjoint they receive, and step t's (uo, vo, wo) and phi(1) are step t-1's
  // (u, v, w) and phin(1).  reverse_step(t) leaves the adjoints of step t's advo and
  // sfst in lcarry (6n doubles: ladvo, then lsfst) instead of transposing them;
  // reverse_step(t-1) adds them to its adv and sfstn adjoints before their
  // transposes (carry_in).
  double* lcarry = nullptr;
  bool carry_in = false;
  double* host_norm = nullptr;  // pinned
  double* tdma = nullptr;       // the pressure solve's Thomas factors (fused::tdma_coef)
  fmf_adj* worker = nullptr;    // recomputes the next segment while this handle reverses one
  // The product step (graph-replayed, pointer rotation, no record copies) for the
  // forward steps whose intermediates no reverse step reads: the rollout's steps
  // before its last segment and every step of fmf_adj_forward.  It runs the same
  // kernels in the same order as record_step, so the states are the same bits.
  // FMF_ADJ_RECORD_ALL set at creation: record_step for every step instead.
  fmf_ctx* plain = nullptr;
  bool record_all = false;
  // The transposed viscous solve of reverse step t starts from that of step t+1:
  // lam = lout + fb, fb the feedback term G^T lam of the previous solve (3n), whose
  // norm fb_norm (0: none yet, a cold start) also scales the stop rule.
  // FMF_ADJ_WARM=0 at creation: every solve starts cold.
  // The last two solves' feedback terms (fb[fb_latest] the latest; fb_count of them
  // valid): from two on, the start is extrapolated linearly in time, lout + 2 fb -
  // fb_prev (FMF_ADJ_EXTRAP=0 at creation: lout + fb).
  double* fb[2] = {nullptr, nullptr};
  int fb_latest = 0, fb_count = 0;
  bool extrap = true;
  double fb_norm = 0.0;
  bool warm = true;
  // With a mixed-precision forward the reverse of its FP32 WENO5 runs in FP32
  // (FMF_ADJ_F32_REVERSE=0 at creation: FP64)
  bool f32_reverse = true;
  // With an FP64 forward the WENO5 reverse runs in FP32-pair arithmetic
  // (FMF_ADJ_PAIR_REVERSE=0 at creation: FP64)
  bool pair_reverse = true;
};

namespace {
double* dalloc(fmf_adj* a, long n) {
  void* p = nullptr;
  if (!FMF_CUDA(cudaMalloc(&p, sizeof(double) * n))) {
    set_status(FMF_ERR_NOMEM);
    return nullptr;
  }
  FMF_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * n, a->s));
  a->allocs.push_back(p);
  a->bytes += (long long)sizeof(double) * n;
  return (double*)p;
}
float* falloc(fmf_adj* a, long n) { return (float*)dalloc(a, (n + 1) / 2); }
struct Scope {
  explicit Scope(void* set) : prev(scratch_set_use(set)) {}
  ~Scope() { scratch_set_use(prev); }
  void* prev;
};
void zero(fmf_adj* a, double* p, long n) { FMF_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * n, a->s)); }
// dst[q] += src[q], q = 0..2, n points each
void add3(cudaStream_t s, long n, double* const* src, double* const* dst) {
  const double *s0 = src[0], *s1 = src[1], *s2 = src[2];
  double *d0 = dst[0], *d1 = dst[1], *d2 = dst[2];
  flat(s, n, [=] __device__(long t) {
    d0[t] += s0[t];
    d1[t] += s1[t];
    d2[t] += s2[t];
  });
}

// the record fields of a point at slot r
void set_rec(fmf_adj* a, const fmf_adj::Rec& r) {
  for (int q = 0; q < 3; ++q) {
    a->gx1[q] = r.gx1[q];
    a->fl[q] = r.fl[q];
    a->adv[q] = r.adv[q];
    a->advo[q] = r.advo[q];
    a->prs[q] = r.prs[q];
    a->vis[q] = r.vis[q];
    a->sfst[q] = r.sfst[q];
    a->sfstn[q] = r.sfstn[q];
    a->E[q] = r.E[q];
    a->ustar[q] = r.ustar[q];
    a->un2[q] = r.un2[q];
  }
  for (int q = 0; q < 6; ++q) a->AB[q] = r.AB[q];
  a->pb = r.pb;
  a->pass = r.pass;
  a->pc = r.pc;
  a->theta = r.theta;
  a->phn1f = r.phn1f;
  a->rho = r.rho;
  a->rhon = r.rhon;
  a->rmu = r.rmu;
  a->rmun = r.rmun;
  a->sk = r.sk;
  a->wallc = r.wallc;
  a->sums = r.sums;
  a->band = r.band;
  a->newton = r.newton;
}
long nwall(const Grid& g) { return 4L * (g.nk + 6) * (g.ni + 6); }
long nband_d(const Grid& g) { return ((long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2) + 2) / 2 + 1; }
long nband(const Grid& g) { return (long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2); }
long slot_doubles(const Grid& g) { return 66 * g.n + nwall(g) + 8 + 2 * nband(g) + nband_d(g) + 16; }
// carve one slot out of a block of slot_doubles(g) doubles
fmf_adj::Rec carve(const Grid& g, double* p) {
  const long n = g.n;
  fmf_adj::Rec r;
  auto take = [&](long k) {
    double* q = p;
    p += k;
    return q;
  };
  for (int q = 0; q < 3; ++q) {
    r.gx1[q] = take(n);
    r.fl[q] = take(n);
    r.adv[q] = take(n);
    r.advo[q] = take(n);
    r.prs[q] = take(n);
    r.vis[q] = take(n);
    r.sfst[q] = take(n);
    r.sfstn[q] = take(n);
    r.E[q] = take(n);
    r.ustar[q] = take(n);
    r.un2[q] = take(n);
  }
  for (int q = 0; q < 6; ++q) r.AB[q] = take(n);
  r.pb = take(n);
  r.pass = take(n);
  r.pc = take(n);
  r.theta = take(n);
  r.phn1f = take(n);
  r.rho = take(n);
  r.rhon = take(n);
  r.rmu = take(n);
  r.rmun = take(n);
  r.sk = take(6 * n);
  r.state = take(12 * n);
  r.wallc = take(nwall(g));
  r.sums = take(8);
  r.newton = take(2 * nband(g));
  r.band = (int*)take(nband_d(g));
  return r;
}
// grow the record slots to `want` (at least one), keeping 2 GiB of the device free
void grow_recs(fmf_adj* a, int want) {
  const size_t bytes = sizeof(double) * (size_t)slot_doubles(a->g);
  while ((int)a->recs.size() < want) {
    size_t fr = 0, tot = 0;
    FMF_CUDA(cudaMemGetInfo(&fr, &tot));
    if (!a->recs.empty() && fr < bytes + (2ull << 30)) break;
    void* p = nullptr;
    if (!FMF_CUDA(cudaMalloc(&p, bytes))) break;
    FMF_CUDA(cudaMemsetAsync(p, 0, bytes, a->s));
    a->bytes += (long long)bytes;
    a->rec_blocks.push_back(p);
    a->recs.push_back(carve(a->g, (double*)p));
  }
}
void dcopy(fmf_adj* a, const double* src, double* dst, long n) {
  FMF_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, a->s));
}

// objective and its gradient on phi (slice 0): one thread per k finds the first
// crossing phi(i,1,k) > 0.5 > phi(i+1,1,k); out[0] = J; lphi (zeroed by the caller)
// receives dJ/dphi at the two crossing points
__global__ void k_interface(Grid g, const double* phi, double dx, double xl, double* xk, double* lphi) {
  const int k = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (k > g.nk) return;
  double x = 0.0;
  const double w = -1.0 / (double)g.nk;
  for (int i = 1; i <= g.ni; ++i) {
    const double p1 = phi[g.at(i, 1, k)], p2 = phi[g.at(i + 1, 1, k)];
    if (p1 > 0.5 && p2 < 0.5) {
      const double d = p2 - p1;
      x = ((double)i - 0.5) * dx + (0.5 - p1) * dx / d - xl * 0.75;
      if (lphi) {
        lphi[g.at(i, 1, k)] = w * dx * (0.5 - p2) / (d * d);
        lphi[g.at(i + 1, 1, k)] = -w * dx * (0.5 - p1) / (d * d);
      }
      break;
    }
  }
  xk[k - 1] = x;
}
__global__ void k_mean_neg(const double* xk, int nk, double* out) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int k = 0; k < nk; ++k) s = s + xk[k];
  out[0] = -(s / (double)nk);
}

__global__ void k_nonfinite(const double* p, long n, int* flag) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    if (!isfinite(p[t])) {
      *flag = 1;
      return;
    }
}
// With FMF_ADJ_CHECK set in the environment: after each stage of the reverse step,
// report on stderr the first stage that left a non-finite adjoint value.
void check_stage(fmf_adj* a, const char* stage) {
  a->stimer.mark(a->s, stage);
  static const bool on = std::getenv("FMF_ADJ_CHECK") != nullptr;
  static bool reported = false;
  if (!on || reported) return;
  const long n = a->g.n;
  int* flag = (int*)(a->sums + 6);
  FMF_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), a->s));
  std::vector<std::pair<const char*, double*>> arrs = {
      {"lS.u", a->lS[SU]},     {"lS.v", a->lS[SV]},   {"lS.w", a->lS[SW]},     {"lS.uo", a->lS[SUO]},
      {"lS.p", a->lS[SP]},     {"lS.phi0", a->lS[SPHI0]}, {"lS.phi1", a->lS[SPHI1]}, {"lun0", a->lun[0]},
      {"lun1", a->lun[1]},     {"lun2", a->lun[2]},   {"ldp", a->ldp},         {"ldiv", a->ldiv},
      {"lphat", a->lphat},     {"lAB0", a->lAB[0]},   {"lAB1", a->lAB[1]},     {"lrmun", a->lrmun},
      {"lrho", a->lrho},       {"lsfst0", a->lsfst[0]}, {"lphn0", a->lphn0},   {"lphn1", a->lphn1},
      {"ltheta", a->ltheta},   {"lfl0", a->lfl[0]},   {"gtheta0", a->gtheta0}, {"gzeta", a->gzeta},
      {"gl1", a->gl1}};
  for (auto& e : arrs) {
    k_nonfinite<<<256, 256, 0, a->s>>>(e.second, n, flag);
    int h = 0;
    FMF_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, a->s));
    FMF_CUDA(cudaStreamSynchronize(a->s));
    if (h) {
      std::fprintf(stderr, "adjoint: non-finite value in %s after stage %s\n", e.first, stage);
      reported = true;
      return;
    }
  }
}

double objective(fmf_adj* a, const double* phi0, double* lphi) {
  const Grid& g = a->g;
  const double xl = a->prm.dx * a->prm.ni;
  if (lphi) zero(a, lphi, g.n);
  k_interface<<<(g.nk + 127) / 128, 128, 0, a->s>>>(g, phi0, a->prm.dx, xl, a->red + 16, lphi);
  k_mean_neg<<<1, 32, 0, a->s>>>(a->red + 16, g.nk, a->red + 8);
  count_launch(2);
  double J = 0.0;
  FMF_CUDA(cudaMemcpyAsync(&J, a->red + 8, sizeof(double), cudaMemcpyDeviceToHost, a->s));
  FMF_CUDA(cudaStreamSynchronize(a->s));
  return J;
}
}  // namespace

namespace {
// main.f90:322-366 on the working state, keeping what its adjoint reads
void init_bc_fwd(fmf_adj* a) {
  a->cont = false;
  const fmf_params& P = a->prm;
  const Grid& g = a->g;
  cudaStream_t s = a->s;
  const long n = g.n;
  double** S = a->S;
  op::gnbc(s, g, S[SU], S[SW], P.uwall, a->theta0, P.sigma, a->zeta, a->ib_theta1);
  op::bnd_contact_angle(s, g, S[SPHI1], a->ib_theta1, P.dx, P.dy, P.dz);
  op::bnd_periodic(s, g, S[SPHI1]);
  dcopy(a, S[SPHI1], a->ib_phi1, n);
  op::summation(s, g, S[SPHI0], S[SPHI1]);
  fused::wall_coef(s, g, P.dy, a->l1, a->l2, S[SPHI1], a->ib_wallc);
  op::bndu(s, g, S[SU], S[SV], S[SW], P.uwall, P.dy, a->l1, a->l2, S[SPHI1]);
  op::bndu(s, g, S[SUO], S[SVO], S[SWO], P.uwall, P.dy, a->l1, a->l2, S[SPHI1]);
  for (int f : {SU, SV, SW, SUO, SVO, SWO}) op::bnd_periodic(s, g, S[f]);
  dcopy(a, S[SU], a->ib_u, n);
  dcopy(a, S[SW], a->ib_w, n);
  op::gnbc(s, g, S[SU], S[SW], P.uwall, a->theta0, P.sigma, a->zeta, a->ib_theta2);
  op::bnd_contact_angle(s, g, S[SPHI0], a->ib_theta2, P.dx, P.dy, P.dz);
  dcopy(a, S[SPHI0], a->ib_phi0, n);
  op::bnd_periodic(s, g, S[SPHI0]);
}

// the CSF force of one field through the drop-in chain (main.f90:548-567)
void csf_fwd(fmf_adj* a, const double* phi, double* const* f) {
  const fmf_params& P = a->prm;
  const Grid& g = a->g;
  cudaStream_t s = a->s;
  const long n = g.n;
  const double dxi = 1.0 / P.dx, dyi = 1.0 / P.dy, dzi = 1.0 / P.dz;
  double* G = a->csfwork;
  double* rn = G + 3 * n;
  double* kap = G + 15 * n;
  double* gq = G + 18 * n;
  static const int offs[4][3] = {{1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  op::cal_grad_p2a(s, g, dxi, dyi, dzi, phi, G, G + n, G + 2 * n);
  for (int q = 0; q < 4; ++q)
    op::calrn(s, g, dxi, dyi, dzi, offs[q][0], offs[q][1], offs[q][2], G, G + n, G + 2 * n, rn + 3 * n * q);
  op::calrkap(s, g, dxi, dyi, dzi, rn, rn + 3 * n, rn + 6 * n, rn + 9 * n, kap);
  op::cal_grad_prs(s, g, dxi, dyi, dzi, phi, gq, gq + n, gq + 2 * n);
  for (int q = 0; q < 3; ++q) op::fill(s, n, f[q], 0.0);
  op::calfst(s, g, P.rhol, P.rhog, P.sigma, gq, gq + n, gq + 2 * n, kap, G, G + n, G + 2 * n);
  op::sum_fst(s, g, G, G + n, G + 2 * n, f[0], f[1], f[2]);
}

// Runs one part of a step: eagerly, or, for a step whose record is not kept
// (graphs), as a CUDA graph captured at the handle's first such call with the
// current buffers (keyed by them) and replayed afterwards.  The handle's first step
// runs eagerly, which sizes the scratch buffers the captured kernels use.
void run_part(fmf_adj* a, bool graphs, int id, const std::function<void()>& body) {
  if (!graphs || !a->rec_warm) {
    body();
    return;
  }
  long long per_launch = 0;
  const cudaGraphExec_t exec = adj::cached_graph(
      a->s, &a->pgraphs,
      {(const void*)(intptr_t)(id + 1 + (a->cont ? 100 : 0)), a->gx1[0], a->adv[0], a->E[0], a->ustar[0],
       a->S[0], a->un[0], a->prev_adv[0], a->prev_sfstn[0]},
      body, &per_launch);
  if (!exec) {
    body();
    return;
  }
  FMF_CUDA(cudaGraphLaunch(exec, a->s));
  count_launch((int)per_launch);
}

// one FP64 step on a->S (main.f90:473-697), recording the intermediates
int record_step(fmf_adj* a, bool graphs) {
  const fmf_params& P = a->prm;
  const Grid& g = a->g;
  cudaStream_t s = a->s;
  const long n = g.n;
  const double dxi = 1.0 / P.dx, dyi = 1.0 / P.dy, dzi = 1.0 / P.dz, dt = P.dt;
  double** S = a->S;
  double *phi0 = S[SPHI0], *phi1 = S[SPHI1], *phn0 = S[SPHIN0], *phn1 = S[SPHIN1];
  const bool carry = a->cont;
  const bool csf_fused = fused::csf_supported(g);
  // the step before the viscous solve
  auto pre = [&]() {
    if (carry) {
      // the previous step's terms, copied before this step overwrites them where
      // both steps use the same record slot
      for (int q = 0; q < 3; ++q) {
        dcopy(a, a->prev_adv[q], a->advo[q], n);
        dcopy(a, a->prev_sfstn[q], a->sfst[q], n);
      }
    }
    // :491-503
    fused::vertex_gradient(s, g, dxi, dyi, dzi, phi1, a->gx1[0], a->gx1[1], a->gx1[2]);
    {
      const long nb = (long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2);
      fused::mthinc_fluxes(s, g, dxi, dyi, dzi, dt, P.bet_mthinc, phi1, a->gx1[0], a->gx1[1], a->gx1[2], S[SU],
                           S[SV], S[SW], a->fl[0], a->fl[1], a->fl[2], a->band, a->band + nb, a->mixed, a->newton);
    }
    op::solphi_mthinc2(s, g, dxi, dyi, dzi, dt, S[SU], S[SV], S[SW], a->fl[0], a->fl[1], a->fl[2], phi1, phn1);
    dcopy(a, phn1, a->pa, n);
    fused::vertex_gradient(s, g, dxi, dyi, dzi, phn1, a->gxn[0], a->gxn[1], a->gxn[2]);
    adj::mthinc3_record(s, g, dxi, dyi, dzi, P.bet_mthinc, a->gxn[0], a->gxn[1], a->gxn[2], a->pa, a->pb, a->pass);
    op::solphi_mthinc3(s, g, dxi, dyi, dzi, P.bet_mthinc, a->gxn[0], a->gxn[1], a->gxn[2], phi1, phn1, a->sums);
    dcopy(a, phn1, a->pc, n);
    op::gnbc(s, g, S[SU], S[SW], P.uwall, a->theta0, P.sigma, a->zeta, a->theta);
    op::bnd_contact_angle(s, g, phn1, a->theta, P.dx, P.dy, P.dz);
    op::bnd_periodic(s, g, phn1);
    dcopy(a, phn1, a->phn1f, n);
    // :509-517
    op::summation(s, g, phn0, phn1);
    op::bnd_neumann(s, g, phn0);
    op::bnd_contact_angle(s, g, phi0, a->theta, P.dx, P.dy, P.dz);
    op::bnd_periodic(s, g, phn0);
    // :526-541
    op::mixture_means(s, g, phi0, phn0, P.rhol, P.rhog, P.rmul, P.rmug, a->rho, a->rhon, a->rmu, a->rmun);
    if (carry)
      fused::weno5_one(s, g, dxi, dyi, dzi, S[SU], S[SV], S[SW], a->adv, a->mixed, a->wsplit);
    else
      fused::weno5_both(s, g, dxi, dyi, dzi, S[SU], S[SV], S[SW], S[SUO], S[SVO], S[SWO], a->adv, a->advo, a->mixed,
                        a->wsplit);
    op::calphat(s, g, S[SP], S[SPO], a->phat);
    op::cal_grad_prs(s, g, dxi, dyi, dzi, a->phat, a->prs[0], a->prs[1], a->prs[2]);
    // in FP32 pairs with a mixed-precision forward, as the product step forms it
    fused::explicit_viscous(s, g, dxi, dyi, dzi, S[SU], S[SV], S[SW], a->rmu, a->tau, a->vis, a->sk, a->mixed);
    // :545-573 (the fused kernel where the grid tiles; csf_T differentiates the same
    // sequence of reference subroutines either way)
    if (csf_fused) {
      if (!carry)
        fused::csf_force(s, g, dxi, dyi, dzi, P.rhol, P.rhog, P.sigma, phi1, a->sfst[0], a->sfst[1], a->sfst[2],
                         a->mixed);
      fused::csf_force(s, g, dxi, dyi, dzi, P.rhol, P.rhog, P.sigma, phn1, a->sfstn[0], a->sfstn[1], a->sfstn[2],
                       a->mixed);
    } else {
      if (!carry) csf_fwd(a, phi1, a->sfst);
      csf_fwd(a, phn1, a->sfstn);
    }
    // :579-623
    const double* advp[3] = {a->adv[0], a->adv[1], a->adv[2]};
    const double* advop[3] = {a->advo[0], a->advo[1], a->advo[2]};
    const double* prsp[3] = {a->prs[0], a->prs[1], a->prs[2]};
    const double* visp[3] = {a->vis[0], a->vis[1], a->vis[2]};
    const double* fstp[3] = {a->sfst[0], a->sfst[1], a->sfst[2]};
    const double* fstnp[3] = {a->sfstn[0], a->sfstn[1], a->sfstn[2]};
    // the FP64 factors A, B the reverse differentiates (the viscous solve's fixed
    // point is un* = A visn(un*) + B in either precision)
    fused::src_visc_prep(s, g, dxi, dyi, dzi, dt, P.harmonic, P.grvb, P.grvp, S[SU], S[SV], S[SW], advp, advop, prsp,
                         visp, fstp, fstnp, a->rmun, a->rho, a->rhon, a->E, a->AB, a->l1, a->l2, phi1, P.dy, a->wallc);
    if (a->mixed)
      // the mixed solve's FP64 first-sweep residual, FP32 factors and wall/halo
      // constants; un = u through zero corrections
      fused::refine_prep(s, g, dxi, dyi, dzi, dt, P.harmonic, P.grvb, P.grvp, S[SU], S[SV], S[SW], advp, advop, prsp,
                         visp, fstp, fstnp, a->rmun, a->rho, a->rhon, a->E, a->l1, a->l2, phi1, P.dy, P.uwall,
                         a->wallc, a->rb);
    else
      for (int q = 0; q < 3; ++q) dcopy(a, S[SU + q], a->un[q], n);
  };
  run_part(a, graphs, 0, pre);
  // one outer iteration (12 colour-pair sweeps and their refreshes), replayed as a
  // CUDA graph per record slot
  auto iteration = [&]() {
    if (a->mixed)
      fused::sor_iteration_refine(s, g, dxi, dyi, dzi, a->rb, a->sorpart, a->red + 4);
    else
      fused::sor_iteration(s, g, dxi, dyi, dzi, P.harmonic, a->rmun, a->E, a->AB, P.uwall, a->wallc, a->un[0],
                           a->un[1], a->un[2], a->sorpart, a->red + 4);
  };
  long long per_launch = 0;
  const cudaGraphExec_t exec =
      adj::cached_graph(s, &a->fgraphs,
                        {a->rmun, a->E[0], a->E[1], a->E[2], a->AB[0], a->AB[1], a->AB[2], a->AB[3], a->AB[4],
                         a->AB[5], a->wallc, a->un[0], a->un[1], a->un[2], a->sorpart, a->red},
                        iteration, &per_launch);
  double err0 = 0.0;
  int lp;
  for (lp = 0; lp < a->sor_max; ++lp) {
    if (exec) {
      FMF_CUDA(cudaGraphLaunch(exec, s));
      count_launch((int)per_launch);
    } else {
      iteration();
    }
    double e = 0.0;
    FMF_CUDA(cudaMemcpyAsync(&e, a->red + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    if (!std::isfinite(e)) {
      set_status(FMF_ERR_NONFINITE);
      break;
    }
    const double err = std::sqrt(e / (double)g.cells()) + 1.0e-99;
    if (lp == 0) err0 = err;
    if (err / err0 <= a->sor_tol) break;
  }
  a->sor_total += lp + 1;
  // the step after the viscous solve
  auto post = [&]() {
    if (a->mixed) fused::refine_finish(s, g, S[SU], S[SV], S[SW], a->rb, a->un[0], a->un[1], a->un[2]);
    for (int q = 0; q < 3; ++q) dcopy(a, a->un[q], a->ustar[q], n);
    // :625-661
    fused::wall_halo(s, g, 7, P.uwall, a->wallc, a->un[0], a->un[1], a->un[2]);
    op::caldiv(s, g, dxi, dyi, dzi, dt, a->un[0], a->un[1], a->un[2], a->div, nullptr);
    fused::pressure_half(s, g, P.rhog, dxi, dzi, a->as_f, a->an_f, a->ap_f, a->div, a->pr, a->pi, a->dp, a->tdma);
    op::bnd_avzero(s, g, a->dp);
    op::bnd_neumann(s, g, a->dp);
    op::bnd_periodic(s, g, a->dp);
    fused::project(s, g, P.rhog, dxi, dyi, dzi, dt, a->dp, a->phat, a->un[0], a->un[1], a->un[2], a->pn);
    for (int q = 0; q < 3; ++q) dcopy(a, a->un[q], a->un2[q], n);
    fused::wall_halo(s, g, 7, P.uwall, a->wallc, a->un[0], a->un[1], a->un[2]);
    op::bnd_avzero(s, g, a->pn);
    op::bnd_neumann(s, g, a->pn);
    op::bnd_periodic(s, g, a->pn);
    // :686-697 rotation (copies: the record keeps the step's inputs in the arrays above)
    for (int q = 0; q < 3; ++q) {
      dcopy(a, S[SU + q], S[SUO + q], n);
      dcopy(a, a->un[q], S[SU + q], n);
    }
    dcopy(a, S[SP], S[SPO], n);
    dcopy(a, a->pn, S[SP], n);
    dcopy(a, phn0, phi0, n);
    dcopy(a, phn1, phi1, n);
  };
  run_part(a, graphs, 1, post);
  a->rec_warm = true;
  FMF_CUDA(cudaGetLastError());
  for (int q = 0; q < 3; ++q) {
    a->prev_adv[q] = a->adv[q];
    a->prev_sfstn[q] = a->sfstn[q];
  }
  a->cont = get_status() == 0 && !a->no_carry;
  return get_status();
}

void save_state(fmf_adj* a, double* dst) {
  for (int f = 0; f < NSTATE; ++f) dcopy(a, a->S[f], dst + (long)f * a->g.n, a->g.n);
}
void load_state(fmf_adj* a, const double* src) {
  a->cont = false;
  for (int f = 0; f < NSTATE; ++f) dcopy(a, src + (long)f * a->g.n, a->S[f], a->g.n);
}

// The product step for forward steps whose record no reverse step reads, created on
// first use on this handle's stream (nullptr: record_step runs them).
fmf_ctx* plain_ctx(fmf_adj* a) {
  if (a->record_all || get_status()) return nullptr;
  if (!a->plain) {
    fmf_ctx* c = nullptr;
    if (fmf_ctx_create(&a->prm, &c) != 0) return nullptr;
    if (fmf_ctx_set_stream(c, a->s) != 0) {
      fmf_ctx_destroy(c);
      return nullptr;
    }
    a->plain = c;
    a->bytes += fmf_ctx_device_bytes(c);
  }
  fmf_ctx_set_sor(a->plain, a->sor_tol, a->sor_max);
  return a->plain;
}

// Steps [t, t1) of a forward pass from a->S on the product step, the state copied
// back into a->S after them; with every > 0 the state at each multiple of `every`
// is saved into its checkpoint first.
void plain_steps(fmf_adj* a, fmf_ctx* c, int t, int t1, int every) {
  const long n = a->g.n;
  ctx_load_device(c, a->S, a->theta0, a->zeta, a->l1, a->l2);
  while (t < t1 && !get_status()) {
    int m = t1 - t;
    if (every > 0) {
      if (t % every == 0)
        for (int f = 0; f < NSTATE; ++f) dcopy(a, ctx_field(c, f), a->ckpt[t / every] + (long)f * n, n);
      m = std::min(m, every - t % every);
    }
    const int st = fmf_ctx_step(c, m);  // its iteration cap is no error here, as in record_step
    if (st != FMF_OK && st != FMF_ERR_ITER_CAP) {
      set_status(st);
      break;
    }
    a->sor_total += (int)ctx_sor_total(c);
    t += m;
  }
  for (int f = 0; f < NSTATE; ++f) dcopy(a, ctx_field(c, f), a->S[f], n);
  a->cont = false;
}

// Reverse of one step.  On entry lS holds the adjoint of the state after the step;
// on exit the adjoint of the state before it.  The record of the step (record_step
// run from that start state) must be current; the step-start state itself is passed
// in st (NSTATE fields).  defer: the next reverse_step is that of the previous step
// of the same rollout, which then transposes this step's (uo, vo, wo) advection and
// phi(1) surface tension together with its own (u, v, w) and phin(1) ones.
void reverse_step(fmf_adj* a, const double* st, bool defer) {
  const fmf_params& P = a->prm;
  const Grid& g = a->g;
  cudaStream_t s = a->s;
  const long n = g.n;
  const double dxi = 1.0 / P.dx, dyi = 1.0 / P.dy, dzi = 1.0 / P.dz, dt = P.dt;
  auto ST = [&](int f) { return st + (long)f * n; };
  double** lS = a->lS;
  a->stimer.mark(s, "begin");
  // :686-697 rotation: u' = un, uo' = u, p' = pn, po' = p, phi' = phin' = phin (phin'
  // is the same phin: its adjoint adds); one pass over the 12 adjoint fields
  {
    double *lu = lS[SU], *lv = lS[SV], *lw = lS[SW], *luo = lS[SUO], *lvo = lS[SVO], *lwo = lS[SWO];
    double *lp = lS[SP], *lpo = lS[SPO], *lf0 = lS[SPHI0], *lf1 = lS[SPHI1], *ln0 = lS[SPHIN0],
           *ln1 = lS[SPHIN1];
    double *o0 = a->lun[0], *o1 = a->lun[1], *o2 = a->lun[2], *opn = a->lpn, *oh0 = a->lphn0, *oh1 = a->lphn1;
    flat(s, n, [=] __device__(long t) {
      o0[t] = lu[t];
      o1[t] = lv[t];
      o2[t] = lw[t];
      lu[t] = luo[t];
      lv[t] = lvo[t];
      lw[t] = lwo[t];
      luo[t] = 0.0;
      lvo[t] = 0.0;
      lwo[t] = 0.0;
      opn[t] = lp[t];
      lp[t] = lpo[t];
      lpo[t] = 0.0;
      oh0[t] = lf0[t] + ln0[t];
      oh1[t] = lf1[t] + ln1[t];
      lf0[t] = 0.0;
      lf1[t] = 0.0;
      ln0[t] = 0.0;
      ln1[t] = 0.0;
    });
  }
  // clear the intermediate adjoints
  zero(a, a->lblock, a->lblock_n);
  // :655-661 pn boundary conditions, wall/halo of un
  adj::periodic_T(s, g, a->lpn);
  adj::neumann_T(s, g, a->lpn);
  adj::avzero_T(s, g, a->lpn);
  adj::wall_halo_T(s, g, 7, P.uwall, a->wallc, a->un2[0], a->un2[2], a->lun[0], a->lun[1], a->lun[2], a->lwc);
  check_stage(a, "post-bc");
  // :648-653 projection and pn = phat + dp
  adj::corunp_T(s, g, P.rhog, dxi, dyi, dzi, dt, a->lun[0], a->lun[1], a->lun[2], a->lpn, a->ldp, a->lphat);
  // :642-646 dp boundary conditions, then the Poisson solve (symmetric: the same solve)
  adj::periodic_T(s, g, a->ldp);
  adj::neumann_T(s, g, a->ldp);
  adj::avzero_T(s, g, a->ldp);
  fused::pressure_half(s, g, P.rhog, dxi, dzi, a->as_f, a->an_f, a->ap_f, a->ldp, a->pr, a->pi, a->ldiv,
                       a->tdma);
  adj::caldiv_T(s, g, dxi, dyi, dzi, dt, a->ldiv, a->lun[0], a->lun[1], a->lun[2]);
  check_stage(a, "poisson");
  adj::wall_halo_T(s, g, 7, P.uwall, a->wallc, a->ustar[0], a->ustar[2], a->lun[0], a->lun[1], a->lun[2], a->lwc);
  // :605-623 the viscous solve
  {  // the 12 sweep snapshots of the fixed point, replayed as a CUDA graph per record slot
    auto replay = [&]() {
      adj::sor_replay(s, g, dxi, dyi, dzi, a->rmun, a->E, a->AB, P.uwall, a->wallc, a->ustar, a->snaps);
    };
    long long per_launch = 0;
    const cudaGraphExec_t exec =
        adj::cached_graph(s, &a->rgraphs,
                          {a->rmun, a->E[0], a->E[1], a->E[2], a->AB[0], a->AB[1], a->AB[2], a->AB[3], a->AB[4],
                           a->AB[5], a->wallc, a->ustar[0], a->ustar[1], a->ustar[2], a->snaps},
                          replay, &per_launch);
    if (exec) {
      FMF_CUDA(cudaGraphLaunch(exec, s));
      count_launch((int)per_launch);
    } else {
      replay();
    }
  }
  check_stage(a, "replay");
  const double* lout[3] = {a->lun[0], a->lun[1], a->lun[2]};
  a->adj_total += adj::sor_T(s, g, dxi, dyi, dzi, a->rmun, a->E, a->AB, P.uwall, a->wallc, a->ustar, a->snaps,
                             lout, a->lam, a->lAB, a->lrmun, a->lE, a->lwc, a->adj_tol, a->adj_max, a->work,
                             a->host_norm, &a->graphs, a->fb[a->fb_latest], &a->fb_norm,
                             a->fb_count >= 2 && a->extrap ? a->fb[1 - a->fb_latest] : nullptr,
                             a->fb[1 - a->fb_latest]);
  a->fb_latest = 1 - a->fb_latest;
  ++a->fb_count;
  if (!a->warm) {
    a->fb_norm = 0.0;
    a->fb_count = 0;
  }
  check_stage(a, "sor");
  // :579-603 momentum factors, edge viscosities, slip coefficients
  {
    adj::SrcArgs A;
    A.u = ST(SU);
    A.v = ST(SV);
    A.w = ST(SW);
    A.rho = a->rho;
    A.rhon = a->rhon;
    A.mu = a->rmun;
    for (int q = 0; q < 3; ++q) {
      A.E[q] = a->E[q];
      A.adv[q] = a->adv[q];
      A.advo[q] = a->advo[q];
      A.prs[q] = a->prs[q];
      A.vis[q] = a->vis[q];
      A.fst[q] = a->sfst[q];
      A.fstn[q] = a->sfstn[q];
    }
    adj::SrcAdj L;
    for (int q = 0; q < 3; ++q) {
      L.u[q] = lS[SU + q];
      L.adv[q] = a->ladv[q];
      L.advo[q] = a->ladvo[q];
      L.prs[q] = a->lprs[q];
      L.vis[q] = a->lvis[q];
      L.fst[q] = a->lsfst[q];
      L.fstn[q] = a->lsfstn[q];
    }
    L.rho = a->lrho;
    L.rhon = a->lrhon;
    L.mu = a->lrmun;
    // diagonal edge pairs: u (exz, exy), v (eyz, exy), w (eyz, exz)
    L.ea[0] = a->lE[1];
    L.eb[0] = a->lE[0];
    L.ea[1] = a->lE[2];
    L.eb[1] = a->lE[0];
    L.ea[2] = a->lE[2];
    L.eb[2] = a->lE[1];
    const double* lab[6] = {a->lAB[0], a->lAB[1], a->lAB[2], a->lAB[3], a->lAB[4], a->lAB[5]};
    adj::src_ab_T(s, g, dxi, dyi, dzi, dt, P.grvb, P.grvp, A, lab, L);
    const double* le[3] = {a->lE[0], a->lE[1], a->lE[2]};
    adj::edges_T(s, g, P.harmonic, a->rmun, le, a->lrmun);
    adj::wall_coef_T(s, g, P.dy, a->l1, a->l2, ST(SPHI1), a->lwc, lS[SPHI1], a->gl1, a->gl2);
  check_stage(a, "src");
  }
  // :545-573 surface tension of phi(1) and phin(1)
  double* const cadv[3] = {a->lcarry, a->lcarry + n, a->lcarry + 2 * n};
  double* const cfst[3] = {a->lcarry + 3 * n, a->lcarry + 4 * n, a->lcarry + 5 * n};
  {
    // the next step's carried adjoint is consumed before this step's replaces it
    if (a->carry_in) add3(s, n, cfst, a->lsfstn);
    if (defer) {
      for (int q = 0; q < 3; ++q) dcopy(a, a->lsfst[q], cfst[q], n);
    } else {
      const double* lf[3] = {a->lsfst[0], a->lsfst[1], a->lsfst[2]};
      adj::csf_T(s, g, dxi, dyi, dzi, P.rhol, P.rhog, P.sigma, ST(SPHI1), lf, lS[SPHI1], a->work + 3 * n + 1024);
    }
    const double* lfn[3] = {a->lsfstn[0], a->lsfstn[1], a->lsfstn[2]};
    adj::csf_T(s, g, dxi, dyi, dzi, P.rhol, P.rhog, P.sigma, a->phn1f, lfn, a->lphn1, a->work + 3 * n + 1024);
  }
  check_stage(a, "csf");
  // :536-541 explicit viscous term, pressure gradient, advection
  adj::div_tensor_T(s, g, dxi, dyi, dzi, a->lvis[0], a->lvis[1], a->lvis[2], a->ltau);
  adj::tau_T(s, g, a->sk, a->rmu, a->ltau, a->lsk, a->lrmu);
  adj::calsij_T(s, g, dxi, dyi, dzi, a->lsk, lS[SU], lS[SV], lS[SW]);
  check_stage(a, "visc");
  adj::grad_prs_T(s, g, dxi, dyi, dzi, a->lprs[0], a->lprs[1], a->lprs[2], a->lphat);
  {
    const Grid G = g;
    double *lp = lS[SP], *lpo = lS[SPO];
    const double* lph = a->lphat;
    range3(s, -1, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
      const long c = G.at(i, j, k);
      lp[c] += 2.0 * lph[c];
      lpo[c] -= lph[c];
    });
  }
  {
    if (a->carry_in) add3(s, n, cadv, a->ladv);
    const double* la[3] = {a->ladv[0], a->ladv[1], a->ladv[2]};
    // a mixed-precision forward (FP32 WENO5): its reverse in FP32 as well; an FP64
    // forward: its reverse in FP32 pairs
    float2* wsp = a->mixed && a->f32_reverse ? a->wsplit : nullptr;
    const bool wpairs = !a->mixed && a->pair_reverse;
    adj::weno_T(s, g, dxi, dyi, dzi, ST(SU), ST(SV), ST(SW), la, lS[SU], lS[SV], lS[SW], a->work + 3 * n + 1024,
                wsp, wpairs);
    if (defer) {
      for (int q = 0; q < 3; ++q) dcopy(a, a->ladvo[q], cadv[q], n);
    } else {
      const double* lao[3] = {a->ladvo[0], a->ladvo[1], a->ladvo[2]};
      adj::weno_T(s, g, dxi, dyi, dzi, ST(SUO), ST(SVO), ST(SWO), lao, lS[SUO], lS[SVO], lS[SWO],
                  a->work + 3 * n + 1024, wsp, wpairs);
    }
  }
  a->carry_in = defer;
  check_stage(a, "weno");
  // :526-529 mixture properties (phi0 after its contact-angle ghosts, phin0)
  adj::mean_T(s, g, P.rhol, P.rhog, a->lrho, lS[SPHI0]);
  adj::mean_T(s, g, P.rmul, P.rmug, a->lrmu, lS[SPHI0]);
  adj::mean_T(s, g, P.rhol, P.rhog, a->lrhon, a->lphn0);
  adj::mean_T(s, g, P.rmul, P.rmug, a->lrmun, a->lphn0);
  // :509-517
  adj::periodic_T(s, g, a->lphn0);
  adj::contact_angle_T(s, g, ST(SPHI0), a->theta, P.dx, P.dy, P.dz, lS[SPHI0], a->ltheta);
  adj::neumann_T(s, g, a->lphn0);
  adj::summation_T(s, g, a->phn1f, a->lphn0, a->lphn1);
  check_stage(a, "means");
  // :496-503
  adj::periodic_T(s, g, a->lphn1);
  adj::contact_angle_T(s, g, a->pc, a->theta, P.dx, P.dy, P.dz, a->lphn1, a->ltheta);
  adj::gnbc_T(s, g, ST(SU), ST(SW), P.uwall, a->theta0, P.sigma, a->zeta, a->ltheta, lS[SU], lS[SW], a->gtheta0,
              a->gzeta);
  check_stage(a, "gnbc");
  adj::mthinc3_T(s, g, a->pb, a->pass, a->sums, a->lphn1, lS[SPHI1], a->sums + 4);
  adj::phin_stale_T(s, g, a->pass, a->lphn1, lS[SPHIN1]);
  check_stage(a, "mthinc3");
  adj::mthinc2_T(s, g, dxi, dyi, dzi, dt, ST(SU), ST(SV), ST(SW), a->fl[0], a->fl[1], a->fl[2], ST(SPHI1), a->pa,
                 a->lphn1, lS[SPHI1], lS[SU], lS[SV], lS[SW], a->lfl[0], a->lfl[1], a->lfl[2], a->lpre);
  check_stage(a, "mthinc2");
  adj::mthinc1_T(s, g, dxi, dyi, dzi, dt, P.bet_mthinc, ST(SPHI1), a->gx1[0], a->gx1[1], a->gx1[2], ST(SU), ST(SV),
                 ST(SW), a->lfl[0], a->lfl[1], a->lfl[2], lS[SPHI1], a->lrn, lS[SU], lS[SV], lS[SW], a->band,
                 a->band + nband(g), a->newton);
  adj::rn_avg_T(s, g, a->lrn, a->lgx[0], a->lgx[1], a->lgx[2]);
  check_stage(a, "mthinc");
  adj::grad_p2a_T(s, g, dxi, dyi, dzi, a->lgx[0], a->lgx[1], a->lgx[2], lS[SPHI1]);
  check_stage(a, "gradp2a");
  a->stimer.flush(s);
  FMF_CUDA(cudaGetLastError());
}

// reverse of init_bc_fwd; on entry lS = adjoint of the state it produced
void reverse_init_bc(fmf_adj* a) {
  const fmf_params& P = a->prm;
  const Grid& g = a->g;
  cudaStream_t s = a->s;
  const long n = g.n;
  double** lS = a->lS;
  zero(a, a->ltheta, n);
  zero(a, a->lwc, 4L * (g.nk + 6) * (g.ni + 6));
  adj::periodic_T(s, g, lS[SPHI0]);
  adj::contact_angle_T(s, g, a->ib_phi0, a->ib_theta2, P.dx, P.dy, P.dz, lS[SPHI0], a->ltheta);
  adj::gnbc_T(s, g, a->ib_u, a->ib_w, P.uwall, a->theta0, P.sigma, a->zeta, a->ltheta, lS[SU], lS[SW], a->gtheta0,
              a->gzeta);
  zero(a, a->ltheta, n);
  for (int f : {SU, SV, SW, SUO, SVO, SWO}) adj::periodic_T(s, g, lS[f]);
  // bndu = wall ghosts, x halos (u shifted), z halos (w shifted); the velocity
  // ghosts read the initial (zero) wall rows
  for (int base : {SUO, SU}) {
    adj::halo_z_T(s, g, 3, lS[base], lS[base + 1], lS[base + 2]);
    adj::halo_x_T(s, g, 6, lS[base], lS[base + 1], lS[base + 2]);
    adj::wall_T(s, g, P.uwall, a->ib_wallc, a->S[base], a->S[base + 2], lS[base], lS[base + 1], lS[base + 2],
                a->lwc);
  }
  adj::wall_coef_T(s, g, P.dy, a->l1, a->l2, a->ib_phi1, a->lwc, lS[SPHI1], a->gl1, a->gl2);
  adj::summation_T(s, g, a->ib_phi1, lS[SPHI0], lS[SPHI1]);
  adj::periodic_T(s, g, lS[SPHI1]);
  adj::contact_angle_T(s, g, a->ib_phi1, a->ib_theta1, P.dx, P.dy, P.dz, lS[SPHI1], a->ltheta);
  adj::gnbc_T(s, g, a->S[SU], a->S[SW], P.uwall, a->theta0, P.sigma, a->zeta, a->ltheta, lS[SU], lS[SW],
              a->gtheta0, a->gzeta);
  FMF_CUDA(cudaGetLastError());
}

void upload_inputs(fmf_adj* a, const double* const* st, const double* th, const double* ze, const double* l1,
                   const double* l2) {
  const size_t b = sizeof(double) * a->g.n;
  a->cont = false;
  for (int f = 0; f < NSTATE; ++f) FMF_CUDA(cudaMemcpyAsync(a->S[f], st[f], b, cudaMemcpyHostToDevice, a->s));
  FMF_CUDA(cudaMemcpyAsync(a->theta0, th, b, cudaMemcpyHostToDevice, a->s));
  FMF_CUDA(cudaMemcpyAsync(a->zeta, ze, b, cudaMemcpyHostToDevice, a->s));
  FMF_CUDA(cudaMemcpyAsync(a->l1, l1, b, cudaMemcpyHostToDevice, a->s));
  FMF_CUDA(cudaMemcpyAsync(a->l2, l2, b, cudaMemcpyHostToDevice, a->s));
}
}  // namespace

extern "C" {

int fmf_adj_create(const fmf_params* prm, fmf_adj** out) {
  if (!prm || !out) return FMF_ERR_ARG;
  auto p2 = [](int v) { return v >= 4 && (v & (v - 1)) == 0; };
  if (!p2(prm->ni) || !p2(prm->nj) || !p2(prm->nk) || prm->ni < 16) return FMF_ERR_ARG;
  if (prm->precision != FMF_FP64 && prm->precision != FMF_MIXED) return FMF_ERR_ARG;
  fmf_adj* a = new fmf_adj();
  a->prm = *prm;
  a->mixed = prm->precision == FMF_MIXED;
  if (const char* e = std::getenv("FMF_STEP_CACHE")) a->no_carry = std::atoi(e) == 0;
  a->record_all = std::getenv("FMF_ADJ_RECORD_ALL") != nullptr;
  if (const char* e = std::getenv("FMF_ADJ_WARM")) a->warm = std::atoi(e) != 0;
  if (const char* e = std::getenv("FMF_ADJ_EXTRAP")) a->extrap = std::atoi(e) != 0;
  if (const char* e = std::getenv("FMF_ADJ_F32_REVERSE")) a->f32_reverse = std::atoi(e) != 0;
  if (const char* e = std::getenv("FMF_ADJ_PAIR_REVERSE")) a->pair_reverse = std::atoi(e) != 0;
  a->g = Grid(prm->ni, prm->nj, prm->nk);
  a->scr = scratch_set_create();
  // the highest stream priority: the reverse steps are the critical path when a
  // worker recomputes the next segment beside them (the worker runs at the lowest)
  int least = 0, greatest = 0;
  FMF_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  if (!FMF_CUDA(cudaStreamCreateWithPriority(&a->s, cudaStreamNonBlocking, greatest))) {
    delete a;
    return FMF_ERR_CUDA;
  }
  const long n = a->g.n;
  for (double** p : {&a->theta0, &a->zeta, &a->l1, &a->l2}) *p = dalloc(a, n);
  for (int f = 0; f < NSTATE; ++f) a->S[f] = dalloc(a, n);
  for (int q = 0; q < 3; ++q)
    for (double** p : {&a->gxn[q], &a->un[q], &a->lun[q], &a->lam[q]}) *p = dalloc(a, n);
  for (double** p : {&a->pa, &a->phat, &a->pn, &a->dp, &a->div, &a->lphn0, &a->lphn1, &a->lpn, &a->lpre,
                     &a->gtheta0, &a->gzeta, &a->gl1, &a->gl2, &a->ib_theta1, &a->ib_theta2, &a->ib_phi1,
                     &a->ib_phi0, &a->ib_u, &a->ib_w})
    *p = dalloc(a, n);
  a->red = dalloc(a, 64 + prm->nk);
  a->tau = dalloc(a, 6 * n);
  a->lrn = dalloc(a, 4 * n);  // 3 normal adjoints + the band-cell marks of mthinc1_T
  const long nwc = 4L * (prm->nk + 6) * (prm->ni + 6);
  // the intermediate adjoints cleared at the start of every reverse step, in one block
  a->lblock_n = 53 * n + nwc;
  {
    double* p = dalloc(a, a->lblock_n);
    a->lblock = p;
    auto take = [&](long k) {
      double* q = p;
      p += k;
      return q;
    };
    for (int q = 0; q < 3; ++q)
      for (double** f : {&a->lgx[q], &a->lfl[q], &a->ladv[q], &a->ladvo[q], &a->lprs[q], &a->lvis[q], &a->lsfst[q],
                         &a->lsfstn[q], &a->lE[q]})
        *f = take(n);
    for (int q = 0; q < 6; ++q) a->lAB[q] = take(n);
    for (double** f : {&a->ltheta, &a->lrho, &a->lrhon, &a->lrmu, &a->lrmun, &a->lphat, &a->ldp, &a->ldiv})
      *f = take(n);
    a->lsk = take(6 * n);
    a->ltau = take(6 * n);
    a->lwc = take(nwc);
  }
  a->ib_wallc = dalloc(a, nwc);
  a->snaps = dalloc(a, 39 * n);
  a->sorpart = dalloc(a, fused::sor_parts(a->g));
  a->csfwork = dalloc(a, 21 * n);
  a->work = dalloc(a, 3 * n + 1024 + 63 * n);  // SOR adjoint, then CSF (42n) or WENO5 (63n) adjoints
  a->fb[0] = dalloc(a, 3 * n);
  a->fb[1] = dalloc(a, 3 * n);
  a->lcarry = dalloc(a, 6 * n);
  if (a->mixed) {
    fused::RefineBufs& rb = a->rb;
    for (int q = 0; q < 3; ++q) {
      rb.d[q] = falloc(a, n);
      rb.a[q] = falloc(a, n);
      rb.r[q] = falloc(a, n);
      rb.e[q] = falloc(a, n);
    }
    rb.mu = falloc(a, n);
    rb.gw = falloc(a, fused::refine_floats(a->g, 0));
    rb.gx = falloc(a, fused::refine_floats(a->g, 1));
    rb.gz = falloc(a, fused::refine_floats(a->g, 2));
    a->wsplit = (float2*)dalloc(a, 6 * n);
  }
  FMF_CUDA(cudaMallocHost(&a->host_norm, sizeof(double) * 2));
  grow_recs(a, 1);  // the record of the current step
  if (a->recs.empty()) {
    fmf_adj_destroy(a);
    return FMF_ERR_NOMEM;
  }
  set_rec(a, a->recs[0]);
  for (int f = 0; f < NSTATE; ++f) a->lS[f] = dalloc(a, n);
  const long nm = a->g.cells();
  a->pr = dalloc(a, nm);
  a->pi = dalloc(a, nm);
  const int NJ = prm->nj;
  a->as_f = dalloc(a, NJ + 6);
  a->an_f = dalloc(a, NJ + 6);
  a->ap_f = dalloc(a, NJ + 6);
  if (get_status()) {
    fmf_adj_destroy(a);
    return take_status();
  }
  // cal_coef_prs.f:28-54 + cal_coef_solp_fft.f:25-39, as fmf_ctx_create
  std::vector<double> as(NJ + 6, 0.0), an(NJ + 6, 0.0), ap(NJ + 6, 0.0);
  const double dyinv = 1.0 / prm->dy;
  for (int j = 1; j <= NJ; ++j) {
    as[j + 2] = dyinv * dyinv / prm->rhog;
    an[j + 2] = dyinv * dyinv / prm->rhog;
    ap[j + 2] = as[j + 2] + an[j + 2];
  }
  ap[3] = ap[3] - as[3];
  as[3] = 0.0;
  ap[NJ + 2] = ap[NJ + 2] - an[NJ + 2];
  an[NJ + 2] = 0.0;
  FMF_CUDA(cudaMemcpyAsync(a->as_f, as.data(), sizeof(double) * (NJ + 6), cudaMemcpyHostToDevice, a->s));
  FMF_CUDA(cudaMemcpyAsync(a->an_f, an.data(), sizeof(double) * (NJ + 6), cudaMemcpyHostToDevice, a->s));
  FMF_CUDA(cudaMemcpyAsync(a->ap_f, ap.data(), sizeof(double) * (NJ + 6), cudaMemcpyHostToDevice, a->s));
  // the Thomas elimination factors of the pressure solve and its transpose
  a->tdma = dalloc(a, fused::tdma_coef_doubles(a->g));
  if (a->tdma)
    fused::tdma_coef(a->s, a->g, prm->rhog, 1.0 / prm->dx, 1.0 / prm->dz, a->as_f, a->an_f, a->ap_f, a->tdma);
  FMF_CUDA(cudaStreamSynchronize(a->s));
  *out = a;
  return take_status();
}

int fmf_adj_destroy(fmf_adj* a) {
  if (!a) return 0;
  if (a->worker) fmf_adj_destroy(a->worker);
  if (a->s) cudaStreamSynchronize(a->s);
  if (a->plain) fmf_ctx_destroy(a->plain);
  for (double* p : a->ckpt) cudaFree(p);
  for (double* p : a->seg) cudaFree(p);
  for (void* p : a->rec_blocks) cudaFree(p);
  for (auto& e : a->graphs) cudaGraphExecDestroy(e.second.first);
  for (auto& e : a->fgraphs) cudaGraphExecDestroy(e.second.first);
  for (auto& e : a->pgraphs) cudaGraphExecDestroy(e.second.first);
  for (auto& e : a->rgraphs) cudaGraphExecDestroy(e.second.first);
  if (a->host_norm) cudaFreeHost(a->host_norm);
  for (void* p : a->allocs) cudaFree(p);
  scratch_set_destroy(a->scr);
  if (a->s) cudaStreamDestroy(a->s);
  delete a;
  return take_status();
}

int fmf_adj_set_solver(fmf_adj* a, double sor_tol, int sor_max, double adj_tol, int adj_max) {
  if (!a || !(sor_tol > 0.0) || sor_max < 1 || !(adj_tol > 0.0) || adj_max < 1) return FMF_ERR_ARG;
  a->sor_tol = sor_tol;
  a->sor_max = sor_max;
  a->adj_tol = adj_tol;
  a->adj_max = adj_max;
  return 0;
}

int fmf_adj_forward(fmf_adj* a, int K, const double* const* state0, const double* theta0, const double* zeta,
                    const double* l1, const double* l2, double* J, double* const* state_out) {
  if (!a || K < 0 || !state0 || !theta0 || !zeta || !l1 || !l2 || !J) return FMF_ERR_ARG;
  Scope scope(a->scr);
  upload_inputs(a, state0, theta0, zeta, l1, l2);
  init_bc_fwd(a);
  a->sor_total = 0;
  if (fmf_ctx* c = plain_ctx(a))
    plain_steps(a, c, 0, K, 0);
  else
    for (int t = 0; t < K && !get_status(); ++t) record_step(a, true);
  *J = objective(a, a->S[SPHI0], nullptr);
  if (state_out)
    for (int f = 0; f < NSTATE; ++f)
      FMF_CUDA(cudaMemcpyAsync(state_out[f], a->S[f], sizeof(double) * a->g.n, cudaMemcpyDeviceToHost, a->s));
  FMF_CUDA(cudaStreamSynchronize(a->s));
  return take_status();
}

// The handle that recomputes segment c-1 (on its own stream, scratch set and record
// slots, from a host thread of its own) while `a` reverses segment c; nullptr where
// its slots do not fit or FMF_ADJ_SERIAL is set.  The walls are copied from `a`.
static fmf_adj* overlap_worker(fmf_adj* a, int every) {
  if (std::getenv("FMF_ADJ_SERIAL")) return nullptr;
  if (!a->worker) {
    if (fmf_adj_create(&a->prm, &a->worker) != 0) {
      a->worker = nullptr;
      take_status();
      return nullptr;
    }
    // the worker's stream at the lowest priority: it fills what the reverse leaves idle
    fmf_adj* w = a->worker;
    int least = 0, greatest = 0;
    cudaStream_t ls = nullptr;
    if (FMF_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest)) &&
        FMF_CUDA(cudaStreamCreateWithPriority(&ls, cudaStreamNonBlocking, least))) {
      FMF_CUDA(cudaStreamSynchronize(w->s));
      FMF_CUDA(cudaStreamDestroy(w->s));
      w->s = ls;
    }
  }
  fmf_adj* w = a->worker;
  w->sor_tol = a->sor_tol;
  w->sor_max = a->sor_max;
  {
    Scope sc(w->scr);
    grow_recs(w, every);
  }
  if ((int)w->recs.size() < every) return nullptr;
  const size_t b = sizeof(double) * a->g.n;
  const double* src[4] = {a->theta0, a->zeta, a->l1, a->l2};
  double* dst[4] = {w->theta0, w->zeta, w->l1, w->l2};
  for (int q = 0; q < 4; ++q) FMF_CUDA(cudaMemcpyAsync(dst[q], src[q], b, cudaMemcpyDeviceToDevice, a->s));
  FMF_CUDA(cudaStreamSynchronize(a->s));
  w->sor_total = 0;
  return get_status() ? nullptr : w;
}

int fmf_adj_rollout(fmf_adj* a, int K, int every, const double* const* state0, const double* theta0,
                    const double* zeta, const double* l1, const double* l2, double* J, double* g_theta0,
                    double* g_zeta, double* g_l1, double* g_l2, double* g_phi) {
  if (!a || K < 1 || !state0 || !theta0 || !zeta || !l1 || !l2 || !J) return FMF_ERR_ARG;
  Scope scope(a->scr);
  const long n = a->g.n;
  if (every <= 0) every = (int)std::ceil(std::sqrt((double)K));
  const int nck = (K + every - 1) / every;
  // checkpoints, and one record slot per step of a segment where memory allows
  // (else segment start states only, each step recorded again before its reverse)
  while ((int)a->ckpt.size() < nck) {
    void* p = nullptr;
    if (!FMF_CUDA(cudaMalloc(&p, sizeof(double) * NSTATE * n))) return take_status();
    a->ckpt.push_back((double*)p);
    a->bytes += (long long)sizeof(double) * NSTATE * n;
  }
  grow_recs(a, every);
  const bool slots = (int)a->recs.size() >= every;
  while (!slots && (int)a->seg.size() < every) {
    void* p = nullptr;
    if (!FMF_CUDA(cudaMalloc(&p, sizeof(double) * NSTATE * n))) return take_status();
    a->seg.push_back((double*)p);
    a->bytes += (long long)sizeof(double) * NSTATE * n;
  }
  upload_inputs(a, state0, theta0, zeta, l1, l2);
  for (double* p : {a->gtheta0, a->gzeta, a->gl1, a->gl2}) zero(a, p, n);
  fmf_adj* w = slots && nck > 1 ? overlap_worker(a, every) : nullptr;
  // forward with checkpoints
  init_bc_fwd(a);
  a->sor_total = 0;
  a->adj_total = 0;
  set_rec(a, a->recs[0]);
  using clk = std::chrono::steady_clock;
  auto lap = [&](clk::time_point& t0) {
    FMF_CUDA(cudaStreamSynchronize(a->s));
    const clk::time_point t1 = clk::now();
    const double dt = std::chrono::duration<double>(t1 - t0).count();
    t0 = t1;
    return dt;
  };
  for (double& t : a->t_phase) t = 0.0;
  clk::time_point tp = clk::now();
  // the last segment is recorded into its slots on the way (it is reversed first);
  // the steps before it (all steps where no slots fit) need no record
  const int tlast = (nck - 1) * every;
  const int tplain = slots ? tlast : K;
  int t = 0;
  if (tplain > 0)
    if (fmf_ctx* pc = plain_ctx(a)) {
      plain_steps(a, pc, 0, tplain, every);
      t = tplain;
    }
  for (; t < K && !get_status(); ++t) {
    if (t % every == 0) save_state(a, a->ckpt[t / every]);
    const bool kept = slots && t >= tlast;
    if (kept) {
      set_rec(a, a->recs[t - tlast]);
      save_state(a, a->recs[t - tlast].state);
    }
    record_step(a, !kept);
  }
  if (get_status()) return take_status();
  *J = objective(a, a->S[SPHI0], a->lS[SPHI0]);
  for (int f = 0; f < NSTATE; ++f)
    if (f != SPHI0) zero(a, a->lS[f], n);
  a->t_phase[0] += lap(tp);
  // reverse, segment by segment
  a->carry_in = false;
  a->fb_norm = 0.0;
  a->fb_count = 0;
  for (int c = nck - 1; c >= 0 && !get_status(); --c) {
    const int t0 = c * every, t1 = std::min(K, t0 + every);
    if (w) {
      // a->recs holds segment c (recorded during the forward pass or by the worker
      // in the previous iteration); the worker records segment c-1 into its own slots
      double t_rec = 0.0;
      std::thread th;
      if (c >= 1) {
        th = std::thread([a, w, c, every, &t_rec]() {
          Scope sc(w->scr);
          const clk::time_point ta = clk::now();
          const int u0 = (c - 1) * every;
          load_state(w, a->ckpt[c - 1]);
          for (int t = u0; t < u0 + every && !get_status(); ++t) {
            set_rec(w, w->recs[t - u0]);
            save_state(w, w->recs[t - u0].state);
            record_step(w, false);
          }
          FMF_CUDA(cudaStreamSynchronize(w->s));
          t_rec = std::chrono::duration<double>(clk::now() - ta).count();
        });
      }
      for (int t = t1 - 1; t >= t0 && !get_status(); --t) {
        set_rec(a, a->recs[t - t0]);
        reverse_step(a, a->recs[t - t0].state, t > 0 && !a->no_carry);
      }
      a->t_phase[2] += lap(tp);
      if (th.joinable()) {
        th.join();
        a->t_phase[1] += t_rec;  // overlapped with the reverse steps above
        a->t_phase[2] += lap(tp);  // the wait for the worker, if it finished last
        std::swap(a->recs, w->recs);
      }
    } else if (slots) {
      if (c != nck - 1) {
        load_state(a, a->ckpt[c]);
        for (int t = t0; t < t1; ++t) {
          set_rec(a, a->recs[t - t0]);
          save_state(a, a->recs[t - t0].state);
          record_step(a, false);
        }
      }
      a->t_phase[1] += lap(tp);
      for (int t = t1 - 1; t >= t0 && !get_status(); --t) {
        set_rec(a, a->recs[t - t0]);
        reverse_step(a, a->recs[t - t0].state, t > 0 && !a->no_carry);
      }
      a->t_phase[2] += lap(tp);
    } else {
      load_state(a, a->ckpt[c]);
      set_rec(a, a->recs[0]);
      for (int t = t0; t < t1; ++t) {
        save_state(a, a->seg[t - t0]);
        if (t + 1 < t1) record_step(a, false);
      }
      a->t_phase[1] += lap(tp);
      for (int t = t1 - 1; t >= t0 && !get_status(); --t) {
        load_state(a, a->seg[t - t0]);
        record_step(a, false);
        a->t_phase[1] += lap(tp);
        reverse_step(a, a->seg[t - t0], t > 0 && !a->no_carry);
        a->t_phase[2] += lap(tp);
      }
    }
  }
  if (w) a->sor_total += w->sor_total;
  set_rec(a, a->recs[0]);
  // the start-up pass: recompute its record from the uploaded state
  for (int f = 0; f < NSTATE; ++f)
    FMF_CUDA(cudaMemcpyAsync(a->S[f], state0[f], sizeof(double) * n, cudaMemcpyHostToDevice, a->s));
  init_bc_fwd(a);
  for (int f = 0; f < NSTATE; ++f)
    FMF_CUDA(cudaMemcpyAsync(a->S[f], state0[f], sizeof(double) * n, cudaMemcpyHostToDevice, a->s));
  reverse_init_bc(a);
  const size_t b = sizeof(double) * n;
  if (g_theta0) FMF_CUDA(cudaMemcpyAsync(g_theta0, a->gtheta0, b, cudaMemcpyDeviceToHost, a->s));
  if (g_zeta) FMF_CUDA(cudaMemcpyAsync(g_zeta, a->gzeta, b, cudaMemcpyDeviceToHost, a->s));
  if (g_l1) FMF_CUDA(cudaMemcpyAsync(g_l1, a->gl1, b, cudaMemcpyDeviceToHost, a->s));
  if (g_l2) FMF_CUDA(cudaMemcpyAsync(g_l2, a->gl2, b, cudaMemcpyDeviceToHost, a->s));
  if (g_phi) FMF_CUDA(cudaMemcpyAsync(g_phi, a->lS[SPHI1], b, cudaMemcpyDeviceToHost, a->s));
  FMF_CUDA(cudaStreamSynchronize(a->s));
  return take_status();
}

int fmf_adj_iterations(fmf_adj* a, int* sor_total, int* adjoint_total) {
  if (!a) return FMF_ERR_ARG;
  if (sor_total) *sor_total = a->sor_total;
  if (adjoint_total) *adjoint_total = a->adj_total;
  return 0;
}

long long fmf_adj_device_bytes(fmf_adj* a) {
  if (!a) return 0;
  return a->bytes + (a->worker ? a->worker->bytes : 0);
}

int fmf_adj_phase_seconds(fmf_adj* a, double* seconds3) {
  if (!a || !seconds3) return FMF_ERR_ARG;
  for (int t = 0; t < 3; ++t) seconds3[t] = a->t_phase[t];
  return 0;
}

}  // extern "C"
