// step.cu -- the device-resident time step (include/fmf_capi.h part 3).
//
// fmf_ctx_step runs main.f90:473-697 on the GPU with every field resident in HBM:
// the state rotation of :686-697 is a pointer rotation, the MPI calls of the
// reference are absent (one rank), and the stop test of solu_sor4.f:291-293 runs
// on the device in graph-replayed steps (a conditional loop in the solve's graph;
// the iteration counts are read once per call), so a call enqueues its steps
// without host round trips (an eager step reads the 8-byte residual after each
// outer iteration instead).
//
// Work carried from one step to the next.  After the rotation (:686-697), (uo, vo,
// wo) of step n+1 is bit for bit (u, v, w) of step n (nothing writes u, v, w after
// the step reads them), and phi slice 1 of step n+1 is phin slice 1 of step n,
// untouched since that step's surface tension read it (:695-697 copies it, and
// :509-516 of the next step writes slice 0 only).  So the advection of (uo, vo, wo)
// (:533) is the previous step's advection of (u, v, w) (:532), and the surface
// tension of phi(1) (:547-566) the previous step's of phin(1): the step swaps
// those buffers instead of recomputing them, and computes one WENO5 level and one
// CSF force.  The carried terms are valid while the state continues from this
// context's previous step (`cont`); uploading, the start-up pass, new walls or a
// request for a state pointer clear it (FMF_STEP_CACHE=0 in the environment at
// creation turns the reuse off).  The host-buffer step uploads the caller's state:
// there the uploaded uo, vo, wo and phi(1) are compared bit for bit with the
// device's copies, and the kernels of the two carried terms read the outcome from
// device flags (no host synchronisation): equal inputs (a caller that passes back
// the previous step's result) keep the carried terms, any other inputs recompute
// them.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <utility>
#include <vector>

#include "../../include/fmf_capi.h"
#include "fused.cuh"
#include "ops.cuh"
#include "runtime.cuh"

using namespace fmf;

struct GraphKey {
  int seg;
  const double* p[16];
  bool operator<(const GraphKey& o) const {
    if (seg != o.seg) return seg < o.seg;
    for (int t = 0; t < 16; ++t)
      if (p[t] != o.p[t]) return p[t] < o.p[t];
    return false;
  }
};
struct GraphEntry {
  cudaGraphExec_t exec;
  long long launches;
};

struct fmf_ctx {
  bool graphs = true;  // replay captured CUDA graphs (FMF_GRAPHS=0 disables)
  bool warm = false;   // the first step runs eagerly (allocates scratch, twiddle tables)
  bool reuse = true;   // carry advo and sfst over from the previous step (FMF_STEP_CACHE=0 disables)
  bool cont = false;   // the state continues from this context's previous step
  bool verify = false; // this step decides on the device whether the carried terms hold (same[])
  int* same = nullptr; // device: [0] uploaded uo, vo, wo equal the carried ones; [1] phi(1) likewise
  void* scr = nullptr; // this context's scratch set
  std::map<GraphKey, GraphEntry> cache;
  fmf_params prm;
  Grid g;
  cudaStream_t s = nullptr;
  bool own_stream = false;
  cudaStream_t cs = nullptr;                        // copies overlapping the step (fmf_ctx_step_host)
  // inputs up (u, v, w; phi(0); the rest); first part of the step done
  cudaEvent_t ev_in = nullptr, ev_in_phi0 = nullptr, ev_in2 = nullptr, ev_pre = nullptr;
  std::vector<void*> allocs;
  long long bytes = 0;
  // state
  double *u, *v, *w, *uo, *vo, *wo, *p, *po;
  double *phi, *phin;  // two slices each: [0] = slice 0, [n] = slice 1
  double *un, *vn, *wn, *pn;
  // walls
  double *theta0, *zeta, *l1, *l2, *theta;
  // work
  double *phix, *phiy, *phiz, *flx, *fly, *flz, *rho, *rhon, *rmu, *rmun;
  double *adv[3], *advo[3], *phat, *prs[3], *tau, *vis[3];
  double *rn[4], *rnn[4], *rkap, *rkapn, *fst[3], *fstn[3], *sfst[3], *sfstn[3], *src[3];
  double *edge[3], *ab[6], *wallc, *sorpart;  // fused viscous solve (fused_visc.cu)
  double *dp, *div, *pr, *pi;
  double *as_f, *an_f, *ap_f;
  double* red;  // small reduction outputs
  int* band;    // MTHINC band-cell list, then its length
  bool mixed = false;        // precision == FMF_MIXED
  int wprec = 0;             // WENO5 arithmetic: 0 FP64, 1 FP32 (FMF_MIXED), 2 FP32 pairs (FMF_FP64E)
  fused::RefineBufs rb{};    // FP32 buffers of the mixed-precision viscous solve
  float2* wsplit = nullptr;  // mixed: split pairs of u, v, w, uo, vo, wo for the FP32 WENO5 (6 n)
  double* host_err = nullptr;  // pinned
  double* tdma = nullptr;       // the pressure solve's Thomas factors (fused::tdma_coef)
  std::vector<int> sor_iters;
  double sor_tol = 1.0e-3;  // solu_sor4.f:291 stop rule (fmf_ctx_set_sor)
  int sor_max = 21;         // solu_sor4.f:130 do lp=0,20
  int capped = 0;           // steps of the last call whose viscous solve hit sor_max
  // The stop rule on the device, for graph-replayed steps: a CUDA graph whose WHILE
  // conditional node runs outer iterations until k_sor_ctl ends it, so no step
  // waits for the host.  Each solve's iteration count goes to sorlog, read back
  // after the call's steps.  FMF_DEVICE_LOOP=0 at creation: the host applies the
  // rule after every iteration.
  bool dev_loop = true;
  struct SorLoop* loop = nullptr;  // device
  int* sorlog = nullptr;           // device, kSorLog entries
  int pending = 0;                 // solves logged on the device since the last read
  long long per_iter = 0;          // kernels of one outer iteration (the loop body)
};

// The device side of the stop rule (solu_sor4.f:130,291-293 as step_once applies
// it on the host): err = sqrt(e / cells) + 1e-99 after each outer iteration,
// err0 = that of the first, stop at err/err0 <= tol or after maxit iterations.
struct SorLoop {
  double tol, cells, err0, pad;
  int maxit, it, nlog, flags;
};
constexpr int kSorLog = 4096;
constexpr int kLogCapped = 1 << 20, kLogNonfinite = 1 << 21;

namespace {
// *same = 0 where any of the nf field pairs a[f], b[f] (n doubles each) differ in a bit
struct Pairs3 {
  const double* a[3];
  const double* b[3];
};
__global__ void k_same(long n, int nf, Pairs3 p, int* same) {
  bool eq = true;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    for (int f = 0; f < nf; ++f)
      eq = eq && __double_as_longlong(p.a[f][t]) == __double_as_longlong(p.b[f][t]);
  if (__syncthreads_and(eq) == 0 && threadIdx.x == 0) *same = 0;
}
// b[f] = a[f] unless *same (then they are equal already)
__global__ void k_copy_unless(long n, int nf, Pairs3 p, const int* same) {
  if (*same) return;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    for (int f = 0; f < nf; ++f) const_cast<double*>(p.b[f])[t] = p.a[f][t];
}
// staged copies of nf fields (src) against their destinations (dst): same[0] = 1 if
// every bit agrees, else 0 and the destinations take the staged values
void verify_upload(cudaStream_t s, long n, int nf, const double* const* src, double* const* dst, int* same) {
  Pairs3 p{};
  for (int f = 0; f < nf; ++f) {
    p.a[f] = src[f];
    p.b[f] = dst[f];
  }
  FMF_CUDA(cudaMemsetAsync(same, 0xff, sizeof(int), s));
  k_same<<<152 * 8, 256, 0, s>>>(n, nf, p, same);
  k_copy_unless<<<152 * 8, 256, 0, s>>>(n, nf, p, same);
  count_launch(2);
}

__global__ void k_sor_rule(SorLoop* L, double tol, int maxit, double cells) {
  L->tol = tol;
  L->maxit = maxit;
  L->cells = cells;
}
__global__ void k_sor_log_reset(SorLoop* L) {
  L->nlog = 0;
  L->flags = 0;
}
__global__ void k_sor_begin(SorLoop* L) { L->it = 0; }
// After one outer iteration (its residual sum at *esum): the rule, the log entry of
// a finished solve (iterations, capped and non-finite bits), and the condition of
// the WHILE node (0 ends the loop).  The iteration count is bounded by maxit, itself
// clamped to the 100000 fmf_ctx_set_sor allows, whatever the loop state holds.
__global__ void k_sor_ctl(cudaGraphConditionalHandle h, const double* esum, SorLoop* L, int* log) {
  const double e = *esum;
  const int mx = min(max(L->maxit, 1), 100000);
  const int it = L->it + 1;
  L->it = it;
  int entry = it;
  bool done = it >= mx || it < 1;
  if (!isfinite(e)) {
    entry |= kLogNonfinite;
    done = true;
  } else {
    const double err = sqrt(e / L->cells) + 1.0e-99;
    if (it == 1) L->err0 = err;
    if (err / L->err0 <= L->tol)
      done = true;
    else if (done)
      entry |= kLogCapped;
  }
  if (done) {
    if (L->nlog < kSorLog) log[L->nlog] = entry;
    L->nlog += 1;
  }
  cudaGraphSetConditional(h, done ? 0u : 1u);
}

// acc[0] += sum over interior points of |a - b|^2, acc[1] += |b - c|^2 (three
// components each); one thread per (i, j) of a k-plane
struct Vel3 {
  const double* q[3];
};
__global__ void __launch_bounds__(256) k_diff2(Grid g, Vel3 a, Vel3 b, Vel3 c, double* acc) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  double s0 = 0.0, s1 = 0.0;
  if (i <= g.ni && j <= g.nj) {
    const long x = g.at(i, j, k);
    for (int f = 0; f < 3; ++f) {
      const double d0 = a.q[f][x] - b.q[f][x], d1 = b.q[f][x] - c.q[f][x];
      s0 = fma(d0, d0, s0);
      s1 = fma(d1, d1, s1);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0 && (s0 != 0.0 || s1 != 0.0)) {
    atomicAdd(acc, s0);
    atomicAdd(acc + 1, s1);
  }
}

double* alloc(fmf_ctx* c, long n) {
  void* p = nullptr;
  if (!FMF_CUDA(cudaMalloc(&p, sizeof(double) * n))) {
    set_status(FMF_ERR_NOMEM);
    return nullptr;
  }
  FMF_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * n, c->s));
  c->allocs.push_back(p);
  c->bytes += (long long)sizeof(double) * n;
  return (double*)p;
}
float* allocf(fmf_ctx* c, long n) { return (float*)alloc(c, (n + 1) / 2); }
}  // namespace

extern "C" {

int fmf_ctx_create(const fmf_params* prm, fmf_ctx** out) {
  if (!prm || !out) return FMF_ERR_ARG;
  auto p2 = [](int n) { return n >= 4 && (n & (n - 1)) == 0; };
  if (!p2(prm->ni) || !p2(prm->nj) || !p2(prm->nk) || prm->ni < 16) return FMF_ERR_ARG;
  if (prm->precision != FMF_FP64 && prm->precision != FMF_MIXED && prm->precision != FMF_FP64E)
    return FMF_ERR_ARG;
  fmf_ctx* c = new fmf_ctx();
  c->prm = *prm;
  if (const char* e = std::getenv("FMF_GRAPHS")) c->graphs = std::atoi(e) != 0;
  if (const char* e = std::getenv("FMF_STEP_CACHE")) c->reuse = std::atoi(e) != 0;
  c->scr = scratch_set_create();
  c->g = Grid(prm->ni, prm->nj, prm->nk);
  if (!FMF_CUDA(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking))) {
    delete c;
    return FMF_ERR_CUDA;
  }
  c->own_stream = true;
  const long n = c->g.n, nm = c->g.cells();
  double** f3[] = {&c->u, &c->v, &c->w, &c->uo, &c->vo, &c->wo, &c->p, &c->po, &c->un, &c->vn, &c->wn, &c->pn,
                   &c->theta0, &c->zeta, &c->l1, &c->l2, &c->theta, &c->phix, &c->phiy, &c->phiz, &c->flx,
                   &c->fly, &c->flz, &c->rho, &c->rhon, &c->rmu, &c->rmun, &c->phat, &c->dp, &c->div};
  for (auto f : f3) *f = alloc(c, n);
  c->phi = alloc(c, 2 * n);
  c->phin = alloc(c, 2 * n);
  for (int q = 0; q < 3; ++q) {
    c->adv[q] = alloc(c, n);
    c->advo[q] = alloc(c, n);
    c->prs[q] = alloc(c, n);
    c->vis[q] = alloc(c, n);
    c->fst[q] = alloc(c, n);
    c->fstn[q] = alloc(c, n);
    c->sfst[q] = alloc(c, n);
    c->sfstn[q] = alloc(c, n);
    c->src[q] = alloc(c, n);
  }
  c->tau = alloc(c, 6 * n);
  for (int q = 0; q < 4; ++q) {
    c->rn[q] = alloc(c, 3 * n);
    c->rnn[q] = alloc(c, 3 * n);
  }
  c->rkap = alloc(c, 3 * n);
  c->rkapn = alloc(c, 3 * n);
  for (int q = 0; q < 3; ++q) c->edge[q] = alloc(c, n);
  for (int q = 0; q < 6; ++q) c->ab[q] = alloc(c, n);
  c->wallc = alloc(c, 4L * (prm->nk + 6) * (prm->ni + 6));
  c->sorpart = alloc(c, fused::sor_parts(c->g));
  c->pr = alloc(c, nm);
  c->pi = alloc(c, nm);
  c->as_f = alloc(c, prm->nj + 6);
  c->an_f = alloc(c, prm->nj + 6);
  c->ap_f = alloc(c, prm->nj + 6);
  c->red = alloc(c, 64);
  c->same = (int*)alloc(c, 1);
  c->mixed = prm->precision == FMF_MIXED;
  if (c->mixed) {
    fused::RefineBufs& rb = c->rb;
    for (int q = 0; q < 3; ++q) {
      rb.d[q] = allocf(c, n);
      rb.a[q] = allocf(c, n);
      rb.r[q] = allocf(c, n);
      rb.e[q] = allocf(c, n);
    }
    rb.mu = allocf(c, n);
    rb.gw = allocf(c, fused::refine_floats(c->g, 0));
    rb.gx = allocf(c, fused::refine_floats(c->g, 1));
    rb.gz = allocf(c, fused::refine_floats(c->g, 2));
    c->wsplit = (float2*)alloc(c, 6 * n);
  }
  c->wprec = c->mixed ? 1 : prm->precision == FMF_FP64E ? 2 : 0;
  if (c->wprec == 2) c->wsplit = (float2*)alloc(c, 6 * n);
  {
    const long nb = (long)(prm->ni + 2) * (prm->nj + 2) * (prm->nk + 2) + 1;
    c->band = (int*)alloc(c, (nb + 1) / 2);
  }
  FMF_CUDA(cudaMallocHost(&c->host_err, sizeof(double) * 8));
  if (const char* e = std::getenv("FMF_DEVICE_LOOP")) c->dev_loop = std::atoi(e) != 0;
  c->loop = (SorLoop*)alloc(c, (sizeof(SorLoop) + 7) / 8);
  c->sorlog = (int*)alloc(c, kSorLog / 2);
  if (c->loop) {
    k_sor_rule<<<1, 1, 0, c->s>>>(c->loop, c->sor_tol, c->sor_max, (double)c->g.cells());
    k_sor_log_reset<<<1, 1, 0, c->s>>>(c->loop);
    count_launch(2);
  }
  if (get_status()) {
    fmf_ctx_destroy(c);
    return take_status();
  }
  // cal_coef_prs.f:28-54 + cal_coef_solp_fft.f:25-39 (main.f90:467-468), on the host
  const int NJ = prm->nj;
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
  FMF_CUDA(cudaMemcpyAsync(c->as_f, as.data(), sizeof(double) * (NJ + 6), cudaMemcpyHostToDevice, c->s));
  FMF_CUDA(cudaMemcpyAsync(c->an_f, an.data(), sizeof(double) * (NJ + 6), cudaMemcpyHostToDevice, c->s));
  FMF_CUDA(cudaMemcpyAsync(c->ap_f, ap.data(), sizeof(double) * (NJ + 6), cudaMemcpyHostToDevice, c->s));
  // the Thomas elimination factors of the pressure solve, fixed for the context
  c->tdma = alloc(c, fused::tdma_coef_doubles(c->g));
  if (c->tdma) fused::tdma_coef(c->s, c->g, prm->rhog, 1.0 / prm->dx, 1.0 / prm->dz, c->as_f, c->an_f, c->ap_f, c->tdma);
  FMF_CUDA(cudaStreamSynchronize(c->s));
  *out = c;
  return take_status();
}

int fmf_ctx_destroy(fmf_ctx* c) {
  if (!c) return 0;
  if (c->s) cudaStreamSynchronize(c->s);
  if (c->cs) {
    cudaStreamSynchronize(c->cs);
    cudaStreamDestroy(c->cs);
  }
  if (c->ev_in) cudaEventDestroy(c->ev_in);
  if (c->ev_in_phi0) cudaEventDestroy(c->ev_in_phi0);
  if (c->ev_in2) cudaEventDestroy(c->ev_in2);
  if (c->ev_pre) cudaEventDestroy(c->ev_pre);
  for (auto& e : c->cache) cudaGraphExecDestroy(e.second.exec);
  scratch_set_destroy(c->scr);
  for (void* p : c->allocs) cudaFree(p);
  if (c->host_err) cudaFreeHost(c->host_err);
  if (c->own_stream && c->s) cudaStreamDestroy(c->s);
  delete c;
  return take_status();
}

int fmf_ctx_set_stream(fmf_ctx* c, void* st) {
  if (!c) return FMF_ERR_ARG;
  cudaStreamSynchronize(c->s);
  if (c->own_stream) cudaStreamDestroy(c->s);
  if (st) {
    c->s = (cudaStream_t)st;
    c->own_stream = false;
  } else {
    FMF_CUDA(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return take_status();
}

int fmf_ctx_set_walls(fmf_ctx* c, const double* th, const double* ze, const double* l1, const double* l2) {
  if (!c || !th || !ze || !l1 || !l2) return FMF_ERR_ARG;
  const size_t b = sizeof(double) * c->g.n;
  c->cont = false;
  FMF_CUDA(cudaMemcpyAsync(c->theta0, th, b, cudaMemcpyHostToDevice, c->s));
  FMF_CUDA(cudaMemcpyAsync(c->zeta, ze, b, cudaMemcpyHostToDevice, c->s));
  FMF_CUDA(cudaMemcpyAsync(c->l1, l1, b, cudaMemcpyHostToDevice, c->s));
  FMF_CUDA(cudaMemcpyAsync(c->l2, l2, b, cudaMemcpyHostToDevice, c->s));
  return take_status();
}

// Routes fmf::scratch to the context's own scratch set while the context works.
struct ScratchScope {
  explicit ScratchScope(void* set) : prev(scratch_set_use(set)) {}
  ~ScratchScope() { scratch_set_use(prev); }
  void* prev;
};

static double* field_ptr(fmf_ctx* c, int f) {
  const long n = c->g.n;
  switch (f) {
    case 0: return c->u;
    case 1: return c->v;
    case 2: return c->w;
    case 3: return c->uo;
    case 4: return c->vo;
    case 5: return c->wo;
    case 6: return c->p;
    case 7: return c->po;
    case 8: return c->phi;
    case 9: return c->phi + n;
    case 10: return c->phin;
    case 11: return c->phin + n;
    default: return nullptr;
  }
}

int fmf_ctx_upload(fmf_ctx* c, const double* const* st) {
  if (!c || !st) return FMF_ERR_ARG;
  const size_t b = sizeof(double) * c->g.n;
  c->cont = false;
  for (int f = 0; f < 12; ++f) FMF_CUDA(cudaMemcpyAsync(field_ptr(c, f), st[f], b, cudaMemcpyHostToDevice, c->s));
  return take_status();
}
int fmf_ctx_download(fmf_ctx* c, double* const* st) {
  if (!c || !st) return FMF_ERR_ARG;
  const size_t b = sizeof(double) * c->g.n;
  for (int f = 0; f < 12; ++f) FMF_CUDA(cudaMemcpyAsync(st[f], field_ptr(c, f), b, cudaMemcpyDeviceToHost, c->s));
  return take_status();
}
int fmf_ctx_state_device_ptr(fmf_ctx* c, int f, void** out) {
  if (!c || !out || f < 0 || f > 11) return FMF_ERR_ARG;
  c->cont = false;  // the caller may write through the pointer before the next step
  *out = field_ptr(c, f);
  return 0;
}
long long fmf_ctx_device_bytes(fmf_ctx* c) { return c ? c->bytes : 0; }
int fmf_ctx_synchronize(fmf_ctx* c) {
  if (!c) return FMF_ERR_ARG;
  FMF_CUDA(cudaStreamSynchronize(c->s));
  return take_status();
}
int fmf_ctx_sor_iterations(fmf_ctx* c, int* out, int cap) {
  if (!c) return 0;
  const int n = (int)c->sor_iters.size();
  for (int t = 0; t < n && t < cap; ++t) out[t] = c->sor_iters[t];
  return n;
}

// main.f90:322-366 (start-up boundary pass) on the uploaded state
int fmf_ctx_init_bc(fmf_ctx* c) {
  if (!c) return FMF_ERR_ARG;
  c->cont = false;
  ScratchScope scope(c->scr);
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  const long n = g.n;
  double* phi0 = c->phi;
  double* phi1 = c->phi + n;
  op::gnbc(s, g, c->u, c->w, P.uwall, c->theta0, P.sigma, c->zeta, c->theta);
  op::bnd_contact_angle(s, g, phi1, c->theta, P.dx, P.dy, P.dz);
  op::bnd_periodic(s, g, phi1);
  op::summation(s, g, phi0, phi1);
  op::copy(s, n, c->u, c->un);
  op::copy(s, n, c->v, c->vn);
  op::copy(s, n, c->w, c->wn);
  op::bndu(s, g, c->u, c->v, c->w, P.uwall, P.dy, c->l1, c->l2, phi1);
  op::bndu(s, g, c->uo, c->vo, c->wo, P.uwall, P.dy, c->l1, c->l2, phi1);
  op::bndu(s, g, c->un, c->vn, c->wn, P.uwall, P.dy, c->l1, c->l2, phi1);
  for (double* q : {c->u, c->v, c->w, c->uo, c->vo, c->wo, c->un, c->vn, c->wn}) op::bnd_periodic(s, g, q);
  op::gnbc(s, g, c->u, c->w, P.uwall, c->theta0, P.sigma, c->zeta, c->theta);
  op::bnd_contact_angle(s, g, phi0, c->theta, P.dx, P.dy, P.dz);
  op::bnd_periodic(s, g, phi0);
  FMF_CUDA(cudaGetLastError());
  return take_status();
}

// ---- the step in three segments ---------------------------------------------
// seg_pre: main.f90:489-607 (transport, properties, right-hand side, solver set-up)
// seg_iter: one outer iteration of solu_sor4 (its residual lands in red[8])
// seg_post: main.f90:625-697 (pressure solve, projection, boundary conditions, rotation
// of phin into phi).  The pointer rotation of u/uo/un, p/po/pn and phi/phin is done
// on the host between steps.
static void csf_one(fmf_ctx* c, const double* phi, double* const* f);

// The first part in three pieces, so that the host-buffer step can start it while
// inputs are still on their way: (a) reads phi(1) only, (b) u, v, w as well, (c)
// phi(0) as well.  phin is final after (b).
static void seg_pre_a(fmf_ctx* c) {
  const fmf_params& P = c->prm;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz;
  // :491 (the vertex gradients of phi(1))
  fused::vertex_gradient(c->s, c->g, dxinv, dyinv, dzinv, c->phi + c->g.n, c->phix, c->phiy, c->phiz);
}
static void seg_pre_b(fmf_ctx* c) {
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  const long n = g.n;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz, dt = P.dt;
  double* phi1 = c->phi + n;
  double* phin0 = c->phin;
  double* phin1 = c->phin + n;
  // :491-503 transport
  {
    const long nb = (long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2);
    fused::mthinc_fluxes(s, g, dxinv, dyinv, dzinv, dt, P.bet_mthinc, phi1, c->phix, c->phiy, c->phiz, c->u, c->v,
                         c->w, c->flx, c->fly, c->flz, c->band, c->band + nb, P.precision == FMF_MIXED);
  }
  op::solphi_mthinc2(s, g, dxinv, dyinv, dzinv, dt, c->u, c->v, c->w, c->flx, c->fly, c->flz, phi1, phin1);
  fused::vertex_gradient(s, g, dxinv, dyinv, dzinv, phin1, c->phix, c->phiy, c->phiz);
  op::solphi_mthinc3(s, g, dxinv, dyinv, dzinv, P.bet_mthinc, c->phix, c->phiy, c->phiz, phi1, phin1, c->red);
  op::gnbc(s, g, c->u, c->w, P.uwall, c->theta0, P.sigma, c->zeta, c->theta);
  op::bnd_contact_angle(s, g, phin1, c->theta, P.dx, P.dy, P.dz);
  op::bnd_periodic(s, g, phin1);
  // :509-517 on phin (the contact-angle pass on phi(0) of :515, independent of
  // these, follows in part c)
  op::summation(s, g, phin0, phin1);
  op::bnd_neumann(s, g, phin0);
  op::bnd_periodic(s, g, phin0);
}
static void seg_pre_c(fmf_ctx* c) {
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  double* phi0 = c->phi;
  op::bnd_contact_angle(c->s, g, phi0, c->theta, P.dx, P.dy, P.dz);  // gnbc result unchanged since :498
  // :526-529
  op::mixture_means(c->s, g, phi0, c->phin, P.rhol, P.rhog, P.rmul, P.rmug, c->rho, c->rhon, c->rmu, c->rmun);
}
static void seg_pre(fmf_ctx* c) {
  seg_pre_a(c);
  seg_pre_b(c);
  seg_pre_c(c);
}

// The rest of the step before the viscous solve: reads uo, vo, wo, p, po (the
// first part reads u, v, w and phi only).
static void seg_pre2(fmf_ctx* c) {
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  k_sor_begin<<<1, 1, 0, s>>>(c->loop);  // the device stop rule's iteration count
  count_launch();
  const long n = g.n;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz, dt = P.dt;
  double* phi1 = c->phi + n;
  double* phin1 = c->phin + n;
  // :532-541 (advo carried over from the previous step where the state continues)
  if (c->verify)
    fused::weno5_keep(s, g, dxinv, dyinv, dzinv, c->u, c->v, c->w, c->uo, c->vo, c->wo, c->adv, c->advo, c->same,
                      c->wprec, c->wsplit);
  else if (c->cont)
    fused::weno5_one(s, g, dxinv, dyinv, dzinv, c->u, c->v, c->w, c->adv, c->wprec, c->wsplit);
  else
    fused::weno5_both(s, g, dxinv, dyinv, dzinv, c->u, c->v, c->w, c->uo, c->vo, c->wo, c->adv, c->advo, c->wprec,
                      c->wsplit);
  op::calphat(s, g, c->p, c->po, c->phat);
  op::cal_grad_prs(s, g, dxinv, dyinv, dzinv, c->phat, c->prs[0], c->prs[1], c->prs[2]);
  fused::explicit_viscous(s, g, dxinv, dyinv, dzinv, c->u, c->v, c->w, c->rmu, c->tau, c->vis, nullptr,
                          c->wprec != 0);
  // :545-570 surface tension (sfst carried over from the previous step's sfstn where
  // the state continues)
  if (c->verify && fused::csf_supported(g))
    fused::csf_force(s, g, dxinv, dyinv, dzinv, P.rhol, P.rhog, P.sigma, phi1, c->sfst[0], c->sfst[1], c->sfst[2],
                     c->wprec, nullptr, c->same + 1);
  else if (!c->cont || c->verify)
    csf_one(c, phi1, c->sfst);
  csf_one(c, phin1, c->sfstn);
  // :579-603 (cal_av of rho/rhon at :571-573 feeds nothing downstream)
  const double* advp[3] = {c->adv[0], c->adv[1], c->adv[2]};
  const double* advop[3] = {c->advo[0], c->advo[1], c->advo[2]};
  const double* prsp[3] = {c->prs[0], c->prs[1], c->prs[2]};
  const double* visp[3] = {c->vis[0], c->vis[1], c->vis[2]};
  const double* fstp[3] = {c->sfst[0], c->sfst[1], c->sfst[2]};
  const double* fstnp[3] = {c->sfstn[0], c->sfstn[1], c->sfstn[2]};
  // :579-603: cal_srcu and the coefficients (as edge viscosities) folded into the
  // per-point update factors of the viscous solve
  if (c->mixed) {
    // the FP64 residual at u and the wall/halo constants of the correction solve;
    // un = u (:605-607) holds implicitly through zero corrections
    fused::refine_prep(s, g, dxinv, dyinv, dzinv, dt, P.harmonic, P.grvb, P.grvp, c->u, c->v, c->w, advp, advop,
                       prsp, visp, fstp, fstnp, c->rmun, c->rho, c->rhon, c->edge, c->l1, c->l2, phi1, P.dy, P.uwall,
                       c->wallc, c->rb);
    return;
  }
  fused::src_visc_prep(s, g, dxinv, dyinv, dzinv, dt, P.harmonic, P.grvb, P.grvp, c->u, c->v, c->w, advp, advop,
                       prsp, visp, fstp, fstnp, c->rmun, c->rho, c->rhon, c->edge, c->ab, c->l1, c->l2, phi1, P.dy,
                       c->wallc, c->wprec == 2);
  // :605-607
  op::copy(s, n, c->u, c->un);
  op::copy(s, n, c->v, c->vn);
  op::copy(s, n, c->w, c->wn);
}

// The surface tension of one field (the force on the u, v, w points): the fused
// kernel, or the reference's sequence of subroutines on grids it does not tile (ni
// not a multiple of 32 or nj not a multiple of 8).
static void csf_one(fmf_ctx* c, const double* phi, double* const* f) {
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  const long n = g.n;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz;
  if (fused::csf_supported(g)) {
    fused::csf_force(s, g, dxinv, dyinv, dzinv, P.rhol, P.rhog, P.sigma, phi, f[0], f[1], f[2], c->wprec);
    return;
  }
  for (int q = 0; q < 3; ++q) op::fill(s, n, f[q], 0.0);
  static const int offs[4][3] = {{1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  fused::vertex_gradient(s, g, dxinv, dyinv, dzinv, phi, c->phix, c->phiy, c->phiz);
  for (int q = 0; q < 4; ++q)
    op::calrn(s, g, dxinv, dyinv, dzinv, offs[q][0], offs[q][1], offs[q][2], c->phix, c->phiy, c->phiz, c->rn[q]);
  op::calrkap(s, g, dxinv, dyinv, dzinv, c->rn[0], c->rn[1], c->rn[2], c->rn[3], c->rkap);
  op::cal_grad_prs(s, g, dxinv, dyinv, dzinv, phi, c->phix, c->phiy, c->phiz);
  op::calfst(s, g, P.rhol, P.rhog, P.sigma, c->phix, c->phiy, c->phiz, c->rkap, c->fst[0], c->fst[1], c->fst[2]);
  op::sum_fst(s, g, c->fst[0], c->fst[1], c->fst[2], f[0], f[1], f[2]);
}

// one outer iteration of the viscous solve; its residual sum lands in red[8]
static void iter_kernels(fmf_ctx* c) {
  const fmf_params& P = c->prm;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz;
  if (c->mixed)
    fused::sor_iteration_refine(c->s, c->g, dxinv, dyinv, dzinv, c->rb, c->sorpart, c->red + 8);
  else
    fused::sor_iteration(c->s, c->g, dxinv, dyinv, dzinv, P.harmonic, c->rmun, c->edge, c->ab, P.uwall, c->wallc,
                         c->un, c->vn, c->wn, c->sorpart, c->red + 8);
}
// the same, with the residual sum copied to the host (the host applies the rule)
static void seg_iter(fmf_ctx* c) {
  iter_kernels(c);
  FMF_CUDA(cudaMemcpyAsync(c->host_err, c->red + 8, sizeof(double), cudaMemcpyDeviceToHost, c->s));
}

// The whole viscous solve as one executable graph: a WHILE conditional node whose
// body is one outer iteration followed by k_sor_ctl, which applies the stop rule
// and ends the loop; captured once per set of rotating buffers.  nullptr (and the
// host-side rule from then on) where the runtime builds no such graph.
static cudaGraphExec_t solve_exec(fmf_ctx* c) {
  GraphKey key{4, {c->u, c->v, c->w, c->uo, c->vo, c->wo, c->un, c->vn, c->wn, c->p, c->po, c->pn, c->phi, c->phin,
                   c->adv[0], c->sfst[0]}};
  auto it = c->cache.find(key);
  if (it != c->cache.end()) return it->second.exec;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams cp{};
  cudaGraphNode_t node;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
            cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  if (ok) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const long long l0 = launches();
    ok = cudaStreamBeginCaptureToGraph(c->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) ==
         cudaSuccess;
    if (ok) {
      iter_kernels(c);
      k_sor_ctl<<<1, 1, 0, c->s>>>(h, c->red + 8, c->loop, c->sorlog);
      count_launch();
      cudaGraph_t captured = nullptr;
      ok = cudaStreamEndCapture(c->s, &captured) == cudaSuccess;
    }
    const long long nl = launches() - l0;
    count_launch((int)-nl);  // counted per iteration when the log is read
    c->per_iter = nl;
    if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
  }
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();  // the host-side rule runs the same iterations
    if (exec) cudaGraphExecDestroy(exec);
    c->dev_loop = false;
    return nullptr;
  }
  c->cache.emplace(key, GraphEntry{exec, 0});
  return exec;
}

// The solves the device logged since the last read: their iteration counts into
// sor_iters, the capped ones into capped, a non-finite residual into the status,
// and their kernels into the launch count.
static void read_sor_log(fmf_ctx* c) {
  if (!c->pending) return;
  SorLoop h{};
  std::vector<int> lg((size_t)std::min(c->pending, kSorLog));
  FMF_CUDA(cudaMemcpyAsync(&h, c->loop, sizeof(SorLoop), cudaMemcpyDeviceToHost, c->s));
  FMF_CUDA(cudaMemcpyAsync(lg.data(), c->sorlog, sizeof(int) * lg.size(), cudaMemcpyDeviceToHost, c->s));
  k_sor_log_reset<<<1, 1, 0, c->s>>>(c->loop);
  count_launch();
  FMF_CUDA(cudaStreamSynchronize(c->s));
  if (h.nlog != c->pending) set_status(FMF_ERR_CUDA);  // a solve that did not finish
  long long its = 0;
  for (int e : lg) {
    const int n = e & (kLogCapped - 1);
    c->sor_iters.push_back(n);
    its += n;
    if (e & kLogCapped) ++c->capped;
    if (e & kLogNonfinite) set_status(FMF_ERR_NONFINITE);
  }
  count_launch((int)(its * c->per_iter));
  c->pending = 0;
}

static void seg_post(fmf_ctx* c) {
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  const long n = g.n;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz, dt = P.dt;
  if (c->mixed) fused::refine_finish(s, g, c->u, c->v, c->w, c->rb, c->un, c->vn, c->wn);
  // :625-646
  fused::wall_halo(s, g, 7, P.uwall, c->wallc, c->un, c->vn, c->wn);
  op::caldiv(s, g, dxinv, dyinv, dzinv, dt, c->un, c->vn, c->wn, c->div, nullptr);
  fused::pressure_half(s, g, P.rhog, dxinv, dzinv, c->as_f, c->an_f, c->ap_f, c->div, c->pr, c->pi, c->dp,
                        c->tdma);
  op::bnd_avzero(s, g, c->dp);
  op::bnd_neumann(s, g, c->dp);
  op::bnd_periodic(s, g, c->dp);
  // :648-661
  fused::project(s, g, P.rhog, dxinv, dyinv, dzinv, dt, c->dp, c->phat, c->un, c->vn, c->wn, c->pn);
  fused::wall_halo(s, g, 7, P.uwall, c->wallc, c->un, c->vn, c->wn);
  op::bnd_avzero(s, g, c->pn);
  op::bnd_neumann(s, g, c->pn);
  op::bnd_periodic(s, g, c->pn);
  // :695-697 phi(l) = phin(l); phin keeps its values (cpy leaves the source intact),
  // so after the pointer swap below the new phin must equal the new phi
  op::copy(s, 2 * n, c->phin, c->phi);
}

// Runs one segment: eagerly, or as a CUDA graph captured the first time this
// segment is met with the current set of rotating buffer pointers and replayed
// afterwards (the rotation cycles through six pointer sets).
static void run_segment(fmf_ctx* c, int id, void (*fn)(fmf_ctx*)) {
  if (!c->graphs) {
    fn(c);
    return;
  }
  GraphKey key{id + (c->cont ? 100 : 0) + (c->verify ? 200 : 0),
               {c->u, c->v, c->w, c->uo, c->vo, c->wo, c->un, c->vn, c->wn, c->p, c->po, c->pn, c->phi, c->phin,
                c->adv[0], c->sfst[0]}};
  auto it = c->cache.find(key);
  if (it == c->cache.end()) {
    const long long l0 = launches();
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (!FMF_CUDA(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeRelaxed))) return;
    fn(c);
    if (!FMF_CUDA(cudaStreamEndCapture(c->s, &graph))) return;
    if (!FMF_CUDA(cudaGraphInstantiate(&exec, graph, 0))) {
      cudaGraphDestroy(graph);
      return;
    }
    cudaGraphDestroy(graph);
    const long long nl = launches() - l0;
    count_launch((int)-nl);  // counted again at every replay below
    it = c->cache.emplace(key, GraphEntry{exec, nl}).first;
  }
  FMF_CUDA(cudaGraphLaunch(it->second.exec, c->s));
  count_launch((int)it->second.launches);
}

// One step.  The optional host callbacks run between its parts (fmf_ctx_step_host:
// waits for inputs, copies of results final early): before_b once part a is
// enqueued, after_b once part b is (phin is final from there on), before_c, and
// before_pre2 ahead of the second segment.
struct StepHooks {
  std::function<void()> before_b, after_b, before_c, before_pre2;
};
static int step_once(fmf_ctx* c, const StepHooks* hk = nullptr) {
  const Grid& g = c->g;
  auto hook = [&](const std::function<void()> StepHooks::*f) {
    if (hk && hk->*f) (hk->*f)();
  };
  run_segment(c, 0, seg_pre_a);
  hook(&StepHooks::before_b);
  run_segment(c, 5, seg_pre_b);
  hook(&StepHooks::after_b);
  hook(&StepHooks::before_c);
  run_segment(c, 6, seg_pre_c);
  hook(&StepHooks::before_pre2);
  run_segment(c, 3, seg_pre2);
  const cudaGraphExec_t sx = c->graphs && c->dev_loop ? solve_exec(c) : nullptr;
  if (sx) {
    // the rule on the device; the counts are read after the call's steps
    FMF_CUDA(cudaGraphLaunch(sx, c->s));
    ++c->pending;
  } else {
    read_sor_log(c);  // counts of earlier device-side solves first, in step order
    double err = 0.0, err0 = 0.0;
    int lp;
    for (lp = 0; lp < c->sor_max; ++lp) {
      run_segment(c, 1, seg_iter);
      FMF_CUDA(cudaStreamSynchronize(c->s));
      const double e = c->host_err[0];
      if (!std::isfinite(e)) {
        set_status(FMF_ERR_NONFINITE);
        break;
      }
      err = std::sqrt(e / (double)g.cells()) + 1.0e-99;
      if (lp == 0) err0 = err;
      if (err / err0 <= c->sor_tol) break;
    }
    c->sor_iters.push_back((lp < c->sor_max ? lp : c->sor_max - 1) + 1);
    if (lp == c->sor_max) ++c->capped;  // reported after the call; the step carries on
  }
  run_segment(c, 2, seg_post);
  // :686-697 rotation by pointer
  double* t;
  t = c->uo; c->uo = c->u; c->u = c->un; c->un = t;
  t = c->vo; c->vo = c->v; c->v = c->vn; c->vn = t;
  t = c->wo; c->wo = c->w; c->w = c->wn; c->wn = t;
  t = c->po; c->po = c->p; c->p = c->pn; c->pn = t;
  t = c->phi; c->phi = c->phin; c->phin = t;
  // the next step's advo and sfst: this step's adv and sfstn
  for (int q = 0; q < 3; ++q) {
    std::swap(c->adv[q], c->advo[q]);
    std::swap(c->sfst[q], c->sfstn[q]);
  }
  FMF_CUDA(cudaGetLastError());
  c->cont = c->reuse && get_status() == 0;
  return get_status();
}

// Times one stage of the step on the context's stream with CUDA events, reps
// launches after one warm-up launch, on the current state (the state is not
// advanced: stages write only work arrays).  Stage 0: WENO5 advection of both
// levels, (u,v,w) and (uo,vo,wo); 1: one outer SOR iteration on copies of the
// velocity; 2: pressure FFT+TDMA+inverse; 3: MTHINC fluxes; 4: WENO5 advection of
// (u,v,w) alone (what a step that continues from the previous one runs).  *ms =
// mean milliseconds per launch of the stage.
int fmf_ctx_time_stage(fmf_ctx* c, int stage, int reps, float* ms) {
  if (!c || !ms || reps <= 0 || stage < 0 || stage > 4) return FMF_ERR_ARG;
  ScratchScope scope(c->scr);
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz;
  const long n = g.n;
  const bool mixed = P.precision == FMF_MIXED;
  auto run = [&]() {
    switch (stage) {
      case 0:
        fused::weno5_both(s, g, dxinv, dyinv, dzinv, c->u, c->v, c->w, c->uo, c->vo, c->wo, c->adv, c->advo,
                          c->wprec, c->wsplit);
        break;
      case 1:
        if (mixed)
          fused::sor_iteration_refine(s, g, dxinv, dyinv, dzinv, c->rb, c->sorpart, c->red + 8);
        else
          fused::sor_iteration(s, g, dxinv, dyinv, dzinv, P.harmonic, c->rmun, c->edge, c->ab, P.uwall, c->wallc,
                               c->un, c->vn, c->wn, c->sorpart, c->red + 8);
        break;
      case 2:
        fused::pressure_half(s, g, P.rhog, dxinv, dzinv, c->as_f, c->an_f, c->ap_f, c->div, c->pr, c->pi, c->dp,
                        c->tdma);
        break;
      case 3:
        fused::mthinc_fluxes(s, g, dxinv, dyinv, dzinv, P.dt, P.bet_mthinc, c->phi + n, c->phix, c->phiy,
                             c->phiz, c->u, c->v, c->w, c->flx, c->fly, c->flz, c->band,
                             c->band + (long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2), mixed);
        break;
      case 4:  // writes adv only: the carried advo stays valid
        fused::weno5_one(s, g, dxinv, dyinv, dzinv, c->u, c->v, c->w, c->adv, c->wprec, c->wsplit);
        break;
    }
  };
  if (stage == 1) {
    op::copy(s, n, c->u, c->un);
    op::copy(s, n, c->v, c->vn);
    op::copy(s, n, c->w, c->wn);
  }
  run();
  cudaEvent_t e0, e1;
  FMF_CUDA(cudaEventCreate(&e0));
  FMF_CUDA(cudaEventCreate(&e1));
  FMF_CUDA(cudaEventRecord(e0, s));
  for (int r = 0; r < reps; ++r) run();
  FMF_CUDA(cudaEventRecord(e1, s));
  FMF_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  FMF_CUDA(cudaEventElapsedTime(&t, e0, e1));
  *ms = t / (float)reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return take_status();
}

// The next step's viscous solve against the FP64 stop rule (fmf_capi.h), on the
// current state: the step up to its solve and the solve as fmf_ctx_step runs them
// (eagerly), then FP64 outer iterations of solu_sor4 on copies of the velocity.
int fmf_ctx_check_sor(fmf_ctx* c, double* out) {
  if (!c || !out) return FMF_ERR_ARG;
  ScratchScope scope(c->scr);
  const fmf_params& P = c->prm;
  const Grid& g = c->g;
  cudaStream_t s = c->s;
  const long n = g.n;
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz;
  double* q = (double*)scratch(sizeof(double) * (10 * n + 2), 15);
  if (!q) return take_status();
  // phi and phin (written by the step's first part: phin, and the contact-angle
  // ghosts of phi(0)) are put back at the end; both advection levels and both
  // surface-tension forces are computed here and again by the next step
  double* keep_phi = q + 6 * n;
  op::copy(s, 2 * n, c->phi, keep_phi);
  op::copy(s, 2 * n, c->phin, keep_phi + 2 * n);
  c->cont = false;
  seg_pre(c);
  seg_pre2(c);
  auto rms = [&](double e) { return std::sqrt(e / (double)g.cells()) + 1.0e-99; };
  auto read_err = [&]() {
    FMF_CUDA(cudaStreamSynchronize(s));
    const double e = c->host_err[0];
    if (!std::isfinite(e)) set_status(FMF_ERR_NONFINITE);
    return rms(e);
  };
  // the context's own solve (FP32 correction sweeps in the mixed precision)
  double err0 = 0.0, err = 0.0;
  int lp;
  for (lp = 0; lp < c->sor_max && !get_status(); ++lp) {
    seg_iter(c);
    err = read_err();
    if (lp == 0) err0 = err;
    if (err / err0 <= c->sor_tol) break;
  }
  out[0] = (double)std::min(lp + 1, c->sor_max);
  out[1] = err / err0;
  if (c->mixed) {
    fused::refine_finish(s, g, c->u, c->v, c->w, c->rb, c->un, c->vn, c->wn);
    // the FP64 factors of the same system
    const double* advp[3] = {c->adv[0], c->adv[1], c->adv[2]};
    const double* advop[3] = {c->advo[0], c->advo[1], c->advo[2]};
    const double* prsp[3] = {c->prs[0], c->prs[1], c->prs[2]};
    const double* visp[3] = {c->vis[0], c->vis[1], c->vis[2]};
    const double* fstp[3] = {c->sfst[0], c->sfst[1], c->sfst[2]};
    const double* fstnp[3] = {c->sfstn[0], c->sfstn[1], c->sfstn[2]};
    fused::src_visc_prep(s, g, dxinv, dyinv, dzinv, P.dt, P.harmonic, P.grvb, P.grvp, c->u, c->v, c->w, advp, advop,
                         prsp, visp, fstp, fstnp, c->rmun, c->rho, c->rhon, c->edge, c->ab, c->l1, c->l2,
                         c->phi + n, P.dy, c->wallc);
  }
  double *q64[3] = {q, q + n, q + 2 * n}, *qx[3] = {q + 3 * n, q + 4 * n, q + 5 * n};
  double* acc = q + 10 * n;
  const double* uvw[3] = {c->u, c->v, c->w};
  const double* unp[3] = {c->un, c->vn, c->wn};
  auto iter64 = [&](double* const* v) {
    fused::sor_iteration(s, g, dxinv, dyinv, dzinv, P.harmonic, c->rmun, c->edge, c->ab, P.uwall, c->wallc, v[0],
                         v[1], v[2], c->sorpart, c->red + 8);
    FMF_CUDA(cudaMemcpyAsync(c->host_err, c->red + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
    return read_err();
  };
  auto copy3 = [&](const double* const* a, double* const* b) {
    for (int f = 0; f < 3; ++f) op::copy(s, n, a[f], b[f]);
  };
  // the FP64 solve from un = u to the same rule
  copy3(uvw, q64);
  double e0 = 0.0;
  for (int l = 0; l < c->sor_max && !get_status(); ++l) {
    const double e = iter64(q64);
    if (l == 0) e0 = e;
    if (e / e0 <= c->sor_tol) break;
  }
  // one more FP64 iteration from each result
  copy3(unp, qx);
  out[2] = iter64(qx) / e0;
  copy3(q64, qx);
  out[3] = iter64(qx) / e0;
  FMF_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s));
  k_diff2<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), dim3(32, 8), 0, s>>>(
      g, Vel3{{c->un, c->vn, c->wn}}, Vel3{{q64[0], q64[1], q64[2]}}, Vel3{{c->u, c->v, c->w}}, acc);
  count_launch();
  double h[2] = {0.0, 0.0};
  FMF_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
  op::copy(s, 2 * n, keep_phi, c->phi);
  op::copy(s, 2 * n, keep_phi + 2 * n, c->phin);
  FMF_CUDA(cudaStreamSynchronize(s));
  out[4] = std::sqrt(h[0]) / (std::sqrt(h[1]) + 1.0e-300);
  return take_status();
}

// One step from host buffers to host buffers (fmf_capi.h).  The copies run on a
// second stream beside the step: the step's first part starts once phi(1) is up
// (its vertex gradients), goes on once u, v, w are (transport and the volume fix),
// and once phi(0) is (its contact-angle pass, the mixture properties); uo, vo, wo,
// p, po follow while that runs (phin is not an input: the step writes it before
// reading it).  After the pointer rotation the result's uo, vo, wo, po are this
// step's inputs u, v, w, p (their buffers are only read during the step) and its
// phi and phin both hold phin, final once the first part has run: those eight
// fields go back on the second stream while the rest of the step runs; u, v, w, p
// follow the step.
int fmf_ctx_step_host(fmf_ctx* c, const double* const* in, double* const* out) {
  if (!c || !in || !out) return FMF_ERR_ARG;
  ScratchScope scope(c->scr);
  if (!c->cs) {
    if (!FMF_CUDA(cudaStreamCreateWithFlags(&c->cs, cudaStreamNonBlocking)) ||
        !FMF_CUDA(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming)) ||
        !FMF_CUDA(cudaEventCreateWithFlags(&c->ev_in_phi0, cudaEventDisableTiming)) ||
        !FMF_CUDA(cudaEventCreateWithFlags(&c->ev_in2, cudaEventDisableTiming)) ||
        !FMF_CUDA(cudaEventCreateWithFlags(&c->ev_pre, cudaEventDisableTiming)))
      return take_status();
  }
  const long n = c->g.n;
  const size_t b = sizeof(double) * n;
  auto h2d = [&](int f, cudaStream_t st) {
    FMF_CUDA(cudaMemcpyAsync(field_ptr(c, f), in[f], b, cudaMemcpyHostToDevice, st));
  };
  auto d2h = [&](int f, const double* src, cudaStream_t st) {
    FMF_CUDA(cudaMemcpyAsync(out[f], src, b, cudaMemcpyDeviceToHost, st));
  };
  // Where this context's last step produced the device state, its carried advection
  // of (uo, vo, wo) and surface tension of phi(1) hold if the caller passes those
  // fields back unchanged: they go up into free work arrays (div; un, vn, wn, written
  // by the step only after its first two parts) and are compared with the device's
  // copies there.
  c->verify = c->cont;
  c->cont = false;
  // the step's stream: phi(1)
  if (c->verify) {
    FMF_CUDA(cudaMemcpyAsync(c->div, in[9], b, cudaMemcpyHostToDevice, c->s));
    const double* src[1] = {c->div};
    double* dst[1] = {field_ptr(c, 9)};
    verify_upload(c->s, n, 1, src, dst, c->same + 1);
  } else {
    h2d(9, c->s);
  }
  // the copy stream: u, v, w, then phi(0), then uo, vo, wo, p, po
  for (int f : {0, 1, 2}) h2d(f, c->cs);
  FMF_CUDA(cudaEventRecord(c->ev_in, c->cs));
  h2d(8, c->cs);
  FMF_CUDA(cudaEventRecord(c->ev_in_phi0, c->cs));
  if (c->verify) {
    double* st[3] = {c->un, c->vn, c->wn};
    for (int f = 0; f < 3; ++f) FMF_CUDA(cudaMemcpyAsync(st[f], in[3 + f], b, cudaMemcpyHostToDevice, c->cs));
    const double* src[3] = {c->un, c->vn, c->wn};
    double* dst[3] = {c->uo, c->vo, c->wo};
    verify_upload(c->cs, n, 3, src, dst, c->same);
  } else {
    for (int f : {3, 4, 5}) h2d(f, c->cs);  // uo, vo, wo
  }
  for (int f : {6, 7}) h2d(f, c->cs);  // p, po
  FMF_CUDA(cudaEventRecord(c->ev_in2, c->cs));
  // the result's uo, vo, wo, po: this step's u, v, w, p
  d2h(3, c->u, c->cs);
  d2h(4, c->v, c->cs);
  d2h(5, c->w, c->cs);
  d2h(7, c->p, c->cs);
  c->sor_iters.clear();
  c->capped = 0;
  const bool gr = c->graphs;
  if (!c->warm) c->graphs = false;
  double* phin = c->phin;
  StepHooks hk;
  hk.before_b = [&]() { FMF_CUDA(cudaStreamWaitEvent(c->s, c->ev_in, 0)); };
  hk.after_b = [&]() {
    FMF_CUDA(cudaEventRecord(c->ev_pre, c->s));
    FMF_CUDA(cudaStreamWaitEvent(c->cs, c->ev_pre, 0));
    for (int f = 8; f < 12; ++f) d2h(f, phin + (f % 2) * n, c->cs);
  };
  hk.before_c = [&]() { FMF_CUDA(cudaStreamWaitEvent(c->s, c->ev_in_phi0, 0)); };
  hk.before_pre2 = [&]() { FMF_CUDA(cudaStreamWaitEvent(c->s, c->ev_in2, 0)); };
  const int st = step_once(c, &hk);
  c->verify = false;
  c->graphs = gr;
  c->warm = true;
  for (int f : {0, 1, 2, 6}) d2h(f, field_ptr(c, f), c->s);
  read_sor_log(c);
  FMF_CUDA(cudaStreamSynchronize(c->s));
  FMF_CUDA(cudaStreamSynchronize(c->cs));
  const int st2 = st ? st : take_status();
  return st2 ? st2 : (c->capped ? FMF_ERR_ITER_CAP : FMF_OK);
}

int fmf_ctx_step(fmf_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return FMF_ERR_ARG;
  ScratchScope scope(c->scr);
  c->sor_iters.clear();
  c->capped = 0;
  for (int t = 0; t < nsteps; ++t) {
    const bool g = c->graphs;
    if (!c->warm) c->graphs = false;  // first step eager: scratch and tables get allocated here
    const int st = step_once(c);
    c->graphs = g;
    c->warm = true;
    if (st) break;
    if (c->pending >= kSorLog) read_sor_log(c);
  }
  read_sor_log(c);
  const int st = take_status();
  return st ? st : (c->capped ? FMF_ERR_ITER_CAP : FMF_OK);
}

int fmf_ctx_set_sor(fmf_ctx* c, double tol, int max_iter) {
  if (!c || !(tol > 0.0) || max_iter < 1 || max_iter > 100000) return FMF_ERR_ARG;
  c->sor_tol = tol;
  c->sor_max = max_iter;
  k_sor_rule<<<1, 1, 0, c->s>>>(c->loop, tol, max_iter, (double)c->g.cells());
  count_launch();
  return take_status();
}

}  // extern "C"

namespace fmf {
// For the adjoint's forward pass: the context's current array of state field f
// (fmf_ctx_upload's order) without ending the carry, and a state and walls loaded
// from device arrays on the context's stream (the carry ends).
double* ctx_field(fmf_ctx* c, int f) { return field_ptr(c, f); }
void ctx_load_device(fmf_ctx* c, const double* const* state, const double* th, const double* ze,
                     const double* l1, const double* l2) {
  const size_t b = sizeof(double) * c->g.n;
  c->cont = false;
  for (int f = 0; f < 12; ++f)
    FMF_CUDA(cudaMemcpyAsync(field_ptr(c, f), state[f], b, cudaMemcpyDeviceToDevice, c->s));
  const double* src[4] = {th, ze, l1, l2};
  double* dst[4] = {c->theta0, c->zeta, c->l1, c->l2};
  for (int q = 0; q < 4; ++q) FMF_CUDA(cudaMemcpyAsync(dst[q], src[q], b, cudaMemcpyDeviceToDevice, c->s));
}
// the viscous-solve iteration counts of the last fmf_ctx_step call, summed
long ctx_sor_total(fmf_ctx* c) {
  long t = 0;
  for (int k : c->sor_iters) t += k;
  return t;
}
}  // namespace fmf
