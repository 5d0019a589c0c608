// adj_visc.cu -- adjoint of the implicit viscous solve and of its coefficients
// (solu_sor4.f, cal_arith_coef_vis.f / cal_harm_coef_vis.f, cal_srcu.f), in the
// A/B/edge-viscosity form of fused_visc.cu.
//
// The forward solve iterates un <- G(un) (one outer iteration: 12 colour-pair
// sweeps, each followed by the wall/halo refresh) to its fixed point un*.  Its
// adjoint is the transposed fixed-point iteration  l <- lout + G'(un*)^T l  on the
// same sweep structure run backwards (each sweep transposed: the adjoint at the
// swept points is scattered to their 14 neighbours and cleared), followed by one
// more backward sweep that collects the gradients with respect to A, B, the edge
// viscosities, mu and the slip coefficients.  The forward states before each sweep
// of one cycle at the fixed point are replayed from un* (12 snapshots).
#include "../../include/fmf_capi.h"
#include "adj.cuh"
#include "fused.cuh"
#include "runtime.cuh"

namespace fmf {
namespace adj {

namespace {
struct VPa {
  double dx2, dy2, dz2, dxy, dxz, dyz;
};
VPa make_vpa(double dxi, double dyi, double dzi) {
  VPa p;
  p.dx2 = dxi * dxi;
  p.dy2 = dyi * dyi;
  p.dz2 = dzi * dzi;
  p.dxy = dxi * dyi;
  p.dxz = dxi * dzi;
  p.dyz = dyi * dzi;
  return p;
}
// The 14 terms of visn for component COMP at c: term t reads array arr[t] (0 u,
// 1 v, 2 w) at c + off[t] with coefficient mult[t] * coefficient cf[t], where the
// coefficient is mu (ca[t] = 0) or edge array ca[t]-1 at index ci[t].
struct Sten {
  int arr[14], ca[14];
  long off[14], ci[14];
  double mult[14];
};
template <int COMP>
__device__ void stencil(const Grid& g, const VPa& p, long c, Sten& S) {
  const long X = 1, Y = g.sy, Z = g.sz;
  int t = 0;
  auto put = [&](int arr, long off, double mult, int ca, long ci) {
    S.arr[t] = arr;
    S.off[t] = off;
    S.mult[t] = mult;
    S.ca[t] = ca;
    S.ci[t] = ci;
    ++t;
  };
  // edge arrays: 1 = exy, 2 = exz, 3 = eyz
  if (COMP == 0) {
    put(0, -Z, p.dz2, 2, c - Z);
    put(0, Z, p.dz2, 2, c);
    put(0, -Y, p.dy2, 1, c - Y);
    put(0, Y, p.dy2, 1, c);
    put(0, -X, 2.0 * p.dx2, 0, c);
    put(0, X, 2.0 * p.dx2, 0, c + X);
    put(1, -Y, p.dxy, 1, c - Y);
    put(1, X - Y, -p.dxy, 1, c - Y);
    put(1, X, p.dxy, 1, c);
    put(1, 0, -p.dxy, 1, c);
    put(2, -Z, p.dxz, 2, c - Z);
    put(2, X - Z, -p.dxz, 2, c - Z);
    put(2, X, p.dxz, 2, c);
    put(2, 0, -p.dxz, 2, c);
  } else if (COMP == 1) {
    put(1, -Z, p.dz2, 3, c - Z);
    put(1, Z, p.dz2, 3, c);
    put(1, -Y, 2.0 * p.dy2, 0, c);
    put(1, Y, 2.0 * p.dy2, 0, c + Y);
    put(1, -X, p.dx2, 1, c - X);
    put(1, X, p.dx2, 1, c);
    put(0, -X, p.dxy, 1, c - X);
    put(0, -X + Y, -p.dxy, 1, c - X);
    put(0, Y, p.dxy, 1, c);
    put(0, 0, -p.dxy, 1, c);
    put(2, -Z, p.dyz, 3, c - Z);
    put(2, Y - Z, -p.dyz, 3, c - Z);
    put(2, Y, p.dyz, 3, c);
    put(2, 0, -p.dyz, 3, c);
  } else {
    put(2, -Z, 2.0 * p.dz2, 0, c);
    put(2, Z, 2.0 * p.dz2, 0, c + Z);
    put(2, -Y, p.dy2, 3, c - Y);
    put(2, Y, p.dy2, 3, c);
    put(2, -X, p.dx2, 2, c - X);
    put(2, X, p.dx2, 2, c);
    put(0, -X, p.dxz, 2, c - X);
    put(0, -X + Z, -p.dxz, 2, c - X);
    put(0, Z, p.dxz, 2, c);
    put(0, 0, -p.dxz, 2, c);
    put(1, -Y, p.dyz, 3, c - Y);
    put(1, -Y + Z, -p.dyz, 3, c - Y);
    put(1, Z, p.dyz, 3, c);
    put(1, 0, -p.dyz, 3, c);
  }
}
struct Arr3 {
  double* a[3];
};
struct CArr4 {
  const double* a[4];  // mu, exy, exz, eyz
};
struct Arr4 {
  double* a[4];
};
struct CArr3 {
  const double* a[3];
};

// transposed sweep of one colour pair: l_C at the swept points is scattered to the
// 14 neighbours (times A) and cleared
template <int COMP>
__global__ void __launch_bounds__(256) k_pair_T(Grid g, VPa p, int pi, int pj, int pk, CArr4 cf,
                                                const double* __restrict__ A, Arr3 l) {
  const int jmax = COMP == 1 ? g.nj - 1 : g.nj;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = (h ? 3 - pi : pi) + 2 * (int)(blockIdx.x * 32 + threadIdx.x);
    const int j = (h ? 3 - pj : pj) + 2 * (int)(blockIdx.y * 8 + threadIdx.y);
    const int k = (h ? 3 - pk : pk) + 2 * (int)blockIdx.z;
    if (i > g.ni || j > jmax || k > g.nk) continue;
    const long c = g.at(i, j, k);
    const double m = l.a[COMP][c];
    if (m == 0.0) continue;
    l.a[COMP][c] = 0.0;
    Sten S;
    stencil<COMP>(g, p, c, S);
    const double ma = m * A[c];
    for (int t = 0; t < 14; ++t) aadd(l.a[S.arr[t]] + c + S.off[t], ma * S.mult[t] * cf.a[S.ca[t]][S.ci[t]]);
  }
}
// gradient collection of one pair at the fixed point: lB += l, lA += l * visn(q),
// and the coefficient adjoints (q = the forward state before this sweep)
template <int COMP>
__global__ void __launch_bounds__(256) k_pair_grad(Grid g, VPa p, int pi, int pj, int pk, CArr4 cf,
                                                   const double* __restrict__ A, CArr3 q, Arr3 l, double* lA,
                                                   double* lB, Arr4 lcf) {
  const int jmax = COMP == 1 ? g.nj - 1 : g.nj;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = (h ? 3 - pi : pi) + 2 * (int)(blockIdx.x * 32 + threadIdx.x);
    const int j = (h ? 3 - pj : pj) + 2 * (int)(blockIdx.y * 8 + threadIdx.y);
    const int k = (h ? 3 - pk : pk) + 2 * (int)blockIdx.z;
    if (i > g.ni || j > jmax || k > g.nk) continue;
    const long c = g.at(i, j, k);
    const double m = l.a[COMP][c];
    if (m == 0.0) continue;
    Sten S;
    stencil<COMP>(g, p, c, S);
    double visn = 0.0;
    for (int t = 0; t < 14; ++t) {
      const double qv = q.a[S.arr[t]][c + S.off[t]];
      visn += S.mult[t] * cf.a[S.ca[t]][S.ci[t]] * qv;
      aadd(lcf.a[S.ca[t]] + S.ci[t], m * A[c] * S.mult[t] * qv);
    }
    lB[c] += m;
    lA[c] += m * visn;
  }
}
// the forward sweep (same arithmetic role as fused k_pair<.., double>, without the residual)
template <int COMP>
__global__ void __launch_bounds__(256) k_pair_fwd(Grid g, VPa p, int pi, int pj, int pk, CArr4 cf,
                                                  const double* __restrict__ A, const double* __restrict__ B,
                                                  Arr3 q) {
  const int jmax = COMP == 1 ? g.nj - 1 : g.nj;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = (h ? 3 - pi : pi) + 2 * (int)(blockIdx.x * 32 + threadIdx.x);
    const int j = (h ? 3 - pj : pj) + 2 * (int)(blockIdx.y * 8 + threadIdx.y);
    const int k = (h ? 3 - pk : pk) + 2 * (int)blockIdx.z;
    if (i > g.ni || j > jmax || k > g.nk) continue;
    const long c = g.at(i, j, k);
    Sten S;
    stencil<COMP>(g, p, c, S);
    double visn = 0.0;
    for (int t = 0; t < 14; ++t) visn += S.mult[t] * cf.a[S.ca[t]][S.ci[t]] * q.a[S.arr[t]][c + S.off[t]];
    q.a[COMP][c] = A[c] * visn + B[c];
  }
}
const int kPi[4] = {1, 1, 1, 2}, kPj[4] = {1, 1, 2, 1}, kPk[4] = {1, 2, 1, 1};
dim3 pgrid(const Grid& g) {
  return dim3((unsigned)((g.ni / 2 + 31) / 32), (unsigned)((g.nj / 2 + 7) / 8), (unsigned)(g.nk / 2));
}
__global__ void k_copy3(long n, Arr3 a, double* __restrict__ b) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    b[t] = a.a[0][t];
    b[t + n] = a.a[1][t];
    b[t + 2 * n] = a.a[2][t];
  }
}
// l holds G^T l_old: fb = l (the feedback term), l += lout; part[block] = sum of
// (l - prev)^2, part[512 + block] = sum of fb^2 (gridDim.x <= 512)
__global__ void k_add_diff3(long n, Arr3 l, CArr3 o, const double* __restrict__ prev, double* part,
                            double* __restrict__ fb) {
  __shared__ double sh[2][256];
  double acc = 0.0, acf = 0.0;
  for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += (long)gridDim.x * 256) {
    for (int c = 0; c < 3; ++c) {
      const double f = l.a[c][t];
      fb[t + c * n] = f;
      acf += f * f;
      const double v = f + o.a[c][t];
      l.a[c][t] = v;
      const double d = v - prev[t + c * n];
      acc += d * d;
    }
  }
  sh[0][threadIdx.x] = acc;
  sh[1][threadIdx.x] = acf;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + st];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sh[0][0];
    part[512 + blockIdx.x] = sh[1][0];
  }
}
// l = lout + fb (the warm start), or lout + 2 fb - fb2 (fb2 the feedback term one
// solve earlier: linear extrapolation in time)
__global__ void k_warm3(long n, Arr3 l, CArr3 o, const double* __restrict__ fb, const double* __restrict__ fb2) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    for (int c = 0; c < 3; ++c) {
      const double f = fb[t + c * n];
      l.a[c][t] = o.a[c][t] + (fb2 ? f + (f - fb2[t + c * n]) : f);
    }
}
// out[0] = sum of part[0..n), out[1] = sum of part[512..512+n)
__global__ void k_sum_small(const double* part, int n, double* out) {
  __shared__ double sh[2][256];
  double acc = 0.0, acf = 0.0;
  for (int t = threadIdx.x; t < n; t += 256) {
    acc += part[t];
    acf += part[512 + t];
  }
  sh[0][threadIdx.x] = acc;
  sh[1][threadIdx.x] = acf;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + st];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sh[0][0];
    out[1] = sh[1][0];
  }
}
}  // namespace

// Momentum factors of k_src_ab: per component T = 1/(r/dt + ap/2), A = T/2,
// B = rs T with r the 4-point density mean, ap the 6-term viscous diagonal and rs
// = r*(u/dt - 1.5 adv + 0.5 advo + 0.5 fst + 0.5 fstn + grav) - prs + 0.5 vis.
void src_ab_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, double grvb,
              double grvp, const SrcArgs& a, const double* const* lAB, const SrcAdj& l) {
  const Grid G = g;
  const VPa p = make_vpa(dxi, dyi, dzi);
  const double dtinv = 1.0 / dt;
  const SrcArgs A = a;
  const SrcAdj L = l;
  const double *lA0 = lAB[0], *lB0 = lAB[1], *lA1 = lAB[2], *lB1 = lAB[3], *lA2 = lAB[4], *lB2 = lAB[5];
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    const double* mu = A.mu;
    const double *exy = A.E[0], *exz = A.E[1], *eyz = A.E[2];
    // q: component, o: its unit offset, lAq/lBq: adjoints; ap terms (array, index, factor)
    auto comp = [&](int q, long o, double lAq, double lBq, const double* vel, double grav, const double* ea,
                    long ia0, long ia1, double fa, const double* eb, long ib0, long ib1, double fb, double fm) {
      if (lAq == 0.0 && lBq == 0.0) return;
      const double r = (A.rho[c] + A.rho[c + o] + A.rhon[c] + A.rhon[c + o]) * 0.25;
      const double ap = fa * ea[ia0] + fb * eb[ib0] + fm * mu[c] * 2.0 + fm * mu[c + o] * 2.0 + fa * ea[ia1] +
                        fb * eb[ib1];
      const double Dd = r * dtinv + ap * 0.5, T = 1.0 / Dd;
      const double ex = vel[c] * dtinv - A.adv[q][c] * 1.5 + A.advo[q][c] * 0.5 + A.fst[q][c] * 0.5 +
                        A.fstn[q][c] * 0.5 + grav;
      const double rs = r * ex - A.prs[q][c] + A.vis[q][c] * 0.5;
      const double lT = 0.5 * lAq + rs * lBq, lrs = T * lBq;
      const double lD = -T * T * lT;
      const double lr = dtinv * lD + lrs * ex, lap = 0.5 * lD;
      aadd(L.u[q] + c, lrs * r * dtinv);
      L.adv[q][c] += -1.5 * r * lrs;
      L.advo[q][c] += 0.5 * r * lrs;
      L.fst[q][c] += 0.5 * r * lrs;
      L.fstn[q][c] += 0.5 * r * lrs;
      L.prs[q][c] += -lrs;
      L.vis[q][c] += 0.5 * lrs;
      aadd(L.rho + c, 0.25 * lr);
      aadd(L.rho + c + o, 0.25 * lr);
      aadd(L.rhon + c, 0.25 * lr);
      aadd(L.rhon + c + o, 0.25 * lr);
      aadd(L.ea[q] + ia0, fa * lap);
      aadd(L.ea[q] + ia1, fa * lap);
      aadd(L.eb[q] + ib0, fb * lap);
      aadd(L.eb[q] + ib1, fb * lap);
      aadd(L.mu + c, 2.0 * fm * lap);
      aadd(L.mu + c + o, 2.0 * fm * lap);
    };
    // u: ap = dz2 exz(-Z) + dy2 exy(-Y) + 2dx2 mu + 2dx2 mu(+X) + dy2 exy + dz2 exz
    comp(0, X, lA0[c], lB0[c], A.u, grvb, exz, c - Z, c, p.dz2, exy, c - Y, c, p.dy2, p.dx2);
    // v: dz2 eyz(-Z) + 2dy2 mu + dx2 exy(-X) + dx2 exy + 2dy2 mu(+Y) + dz2 eyz
    if (j <= G.nj - 1) comp(1, Y, lA1[c], lB1[c], A.v, grvp, eyz, c - Z, c, p.dz2, exy, c - X, c, p.dx2, p.dy2);
    // w: 2dz2 mu + dy2 eyz(-Y) + dx2 exz(-X) + dx2 exz + dy2 eyz + 2dz2 mu(+Z)
    comp(2, Z, lA2[c], lB2[c], A.w, 0.0, eyz, c - Y, c, p.dy2, exz, c - X, c, p.dx2, p.dz2);
  });
}

// k_edges: E(c) = 4-cell mean of mu over i,j,k in 0..n (arithmetic or harmonic)
void edges_T(cudaStream_t s, const Grid& g, int harmonic, const double* mu, const double* const* lE, double* lmu) {
  const Grid G = g;
  const double *l0 = lE[0], *l1 = lE[1], *l2 = lE[2];
  range3(s, 0, g.ni, 0, g.nj, 0, g.nk, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    auto one = [&](double L, long a, long b, long d, long e) {
      if (L == 0.0) return;
      if (!harmonic) {
        aadd(lmu + a, 0.25 * L);
        aadd(lmu + b, 0.25 * L);
        aadd(lmu + d, 0.25 * L);
        aadd(lmu + e, 0.25 * L);
      } else {
        const double sm = 1.0 / mu[a] + 1.0 / mu[b] + 1.0 / mu[d] + 1.0 / mu[e];
        const double f = 4.0 / (sm * sm) * L;  // d(4/sm)/d(mu_p) = 4/sm^2 / mu_p^2
        aadd(lmu + a, f / (mu[a] * mu[a]));
        aadd(lmu + b, f / (mu[b] * mu[b]));
        aadd(lmu + d, f / (mu[d] * mu[d]));
        aadd(lmu + e, f / (mu[e] * mu[e]));
      }
    };
    one(l0[c], c, c + X, c + Y, c + X + Y);
    one(l1[c], c, c + X, c + Z, c + X + Z);
    one(l2[c], c, c + Y, c + Z, c + Y + Z);
  });
}

void sor_replay(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* mu,
                double* const* E, double* const* AB, double uwall, const double* wallc, const double* const* ustar,
                double* snaps) {
  const VPa p = make_vpa(dxi, dyi, dzi);
  const long n = g.n;
  const CArr4 cf{{mu, E[0], E[1], E[2]}};
  double* q[3] = {snaps + 36 * n, snaps + 37 * n, snaps + 38 * n};  // running state
  for (int c = 0; c < 3; ++c) FMF_CUDA(cudaMemcpyAsync(q[c], ustar[c], sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  const dim3 grd = pgrid(g), blk(32, 8);
  for (int comp = 0; comp < 3; ++comp)
    for (int pr = 0; pr < 4; ++pr) {
      const int idx = comp * 4 + pr;
      for (int c = 0; c < 3; ++c)
        FMF_CUDA(cudaMemcpyAsync(snaps + (3 * idx + c) * n, q[c], sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      const Arr3 Q{{q[0], q[1], q[2]}};
      if (comp == 0) k_pair_fwd<0><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[0], AB[1], Q);
      else if (comp == 1) k_pair_fwd<1><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[2], AB[3], Q);
      else k_pair_fwd<2><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[4], AB[5], Q);
      count_launch();
      fused::wall_halo(s, g, 1 << comp, uwall, wallc, q[0], q[1], q[2]);
    }
}

cudaGraphExec_t cached_graph(cudaStream_t s, GraphCache* cache, const std::vector<const void*>& key,
                             const std::function<void()>& body, long long* per_launch) {
  auto itc = cache->find(key);
  if (itc != cache->end()) {
    *per_launch = itc->second.second;
    return itc->second.first;
  }
  *per_launch = 0;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  const long long l0 = launches();
  if (!FMF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed))) return nullptr;
  body();
  // the captured launches did not run: they are counted when the graph is replayed
  const long long captured = launches() - l0;
  count_launch((int)-captured);
  if (FMF_CUDA(cudaStreamEndCapture(s, &graph)) && FMF_CUDA(cudaGraphInstantiate(&exec, graph, 0))) {
    *per_launch = captured;
    (*cache)[key] = {exec, captured};
  } else {
    exec = nullptr;
  }
  if (graph) cudaGraphDestroy(graph);
  return exec;
}

int sor_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* mu, double* const* E,
          double* const* AB, double uwall, const double* wallc, const double* const* ustar, const double* snaps,
          const double* const* lout, double* const* lam, double* const* lAB, double* lmu, double* const* lE,
          double* lwc, double tol, int maxit, double* work, double* host_norm, GraphCache* cache, double* fb,
          double* fb_norm, const double* fb_prev, double* fb_out) {
  const VPa p = make_vpa(dxi, dyi, dzi);
  const long n = g.n;
  const CArr4 cf{{mu, E[0], E[1], E[2]}};
  const dim3 grd = pgrid(g), blk(32, 8);
  double* prev = work;               // 3n
  double* part = work + 3 * n;       // 1024
  double* nrm = work + 3 * n + 1024; // 2 doubles
  const Arr3 L3{{lam[0], lam[1], lam[2]}};
  const CArr3 O3{{lout[0], lout[1], lout[2]}};
  // l = lout, or lout plus the previous solve's feedback term
  const bool warm = *fb_norm > 0.0;
  if (warm) {
    k_warm3<<<608, 256, 0, s>>>(n, L3, O3, fb, fb_prev);
    count_launch();
  } else {
    for (int c = 0; c < 3; ++c)
      FMF_CUDA(cudaMemcpyAsync(lam[c], lout[c], sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  }
  auto backward_cycle = [&](bool grad) {
    const Arr3 L{{lam[0], lam[1], lam[2]}};
    for (int comp = 2; comp >= 0; --comp)
      for (int pr = 3; pr >= 0; --pr) {
        const int idx = comp * 4 + pr;
        // transposed refresh; the slip-coefficient adjoint only in the gradient pass
        wall_halo_T(s, g, 1 << comp, uwall, wallc, ustar[0], ustar[2], lam[0], lam[1], lam[2],
                    grad ? lwc : nullptr);
        if (grad) {
          const CArr3 dq{{snaps + (3 * idx) * n, snaps + (3 * idx + 1) * n, snaps + (3 * idx + 2) * n}};
          const Arr4 lcf{{lmu, lE[0], lE[1], lE[2]}};
          if (comp == 0) k_pair_grad<0><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[0], dq, L, lAB[0], lAB[1], lcf);
          else if (comp == 1) k_pair_grad<1><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[2], dq, L, lAB[2], lAB[3], lcf);
          else k_pair_grad<2><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[4], dq, L, lAB[4], lAB[5], lcf);
          count_launch();
        }
        if (comp == 0) k_pair_T<0><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[0], L);
        else if (comp == 1) k_pair_T<1><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[2], L);
        else k_pair_T<2><<<grd, blk, 0, s>>>(g, p, kPi[pr], kPj[pr], kPk[pr], cf, AB[4], L);
        count_launch();
      }
  };
  // one iteration l <- lout + G^T l, |l_new - l_old|^2 and |G^T l|^2 into nrm and
  // the feedback term G^T l into fb: 51 kernels, replayed as a CUDA graph (one per
  // set of buffers)
  auto iteration = [&]() {
    k_copy3<<<608, 256, 0, s>>>(n, L3, prev);
    backward_cycle(false);
    k_add_diff3<<<512, 256, 0, s>>>(n, L3, O3, prev, part, fb_out);
    k_sum_small<<<1, 256, 0, s>>>(part, 512, nrm);
    count_launch(3);
  };
  long long per_launch = 0;
  cudaGraphExec_t exec =
      cache ? cached_graph(s, cache,
                           {lam[0], lam[1], lam[2], lout[0], lout[1], lout[2], mu, E[0], E[1], E[2], AB[0], AB[2],
                            AB[4], wallc, ustar[0], ustar[2], work, fb_out},
                           iteration, &per_launch)
            : nullptr;
  // The stop rule's scale: the change of the first iteration from l = lout (the
  // size of the feedback term G^T lout); from a warm start, the previous solve's
  // feedback norm, the same quantity one step later.
  double n0 = warm ? *fb_norm : -1.0;
  int it = 0;
  for (it = 0; it < maxit; ++it) {
    if (exec) {
      FMF_CUDA(cudaGraphLaunch(exec, s));
      count_launch((int)per_launch);
    } else {
      iteration();
    }
    FMF_CUDA(cudaMemcpyAsync(host_norm, nrm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
    const double d = std::sqrt(host_norm[0]);
    if (!std::isfinite(d) || !std::isfinite(host_norm[1])) {
      set_status(FMF_ERR_NONFINITE);
      break;
    }
    *fb_norm = std::sqrt(host_norm[1]);
    if (n0 < 0.0) n0 = d;
    if (!(d > tol * (n0 + 1e-300))) break;
  }
  // gradient pass at the converged adjoint
  backward_cycle(true);
  return it + 1;
}

}  // namespace adj
}  // namespace fmf
