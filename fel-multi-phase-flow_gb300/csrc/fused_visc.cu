// fused_visc.cu -- the implicit viscous solve of the fused step (solu_sor4.f with
// the coefficients of cal_arith_coef_vis.f / cal_harm_coef_vis.f).
//
// The 45 coefficient arrays are products of six viscosities and constant grid
// factors (cal_arith_coef_vis.f:211-231): for u at (i+1/2,j,k) the x-viscosities
// are the cell values mu(i), mu(i+1) and the y/z ones are edge means shared with
// the neighbours.  k_prep stores the three edge means once per step (the same
// 4-cell sums, in the same order, as the reference) together with, per component,
// A = 0.5/(rho00*D) and B = src/D with D = 1/dt + 0.5*a_p/rho00, so a point update
// of solu_sor4.f:150-170 becomes q_new = A*visn + B with visn the 14-neighbour sum.
// Colours are processed in their independent pairs (1,2) (3,4) (5,6) (7,8): two
// colours that differ in every index parity never read each other, so one launch
// per pair gives the sequential result.  The wall/halo refresh after every second
// colour (bndu + bnd_periodic of the swept component, solu_sor4.f:176-180) is three
// ordered plane kernels.
#include "fused.cuh"

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
__global__ void __launch_bounds__(256) k_edges(Grid g, VP p, const double* __restrict__ mu, double* __restrict__ exy,
                                               double* __restrict__ exz, double* __restrict__ eyz) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double m0 = __ldg(mu + c), mx = __ldg(mu + c + X), my = __ldg(mu + c + Y), mz = __ldg(mu + c + Z);
  exy[c] = mean4(m0, mx, my, __ldg(mu + c + X + Y), p.harmonic);
  exz[c] = mean4(m0, mx, mz, __ldg(mu + c + X + Z), p.harmonic);
  eyz[c] = mean4(m0, my, mz, __ldg(mu + c + Y + Z), p.harmonic);
}

__global__ void __launch_bounds__(256) k_ab(Grid g, VP p, const double* __restrict__ mu,
                                            const double* __restrict__ exy, const double* __restrict__ exz,
                                            const double* __restrict__ eyz, const double* __restrict__ rho,
                                            const double* __restrict__ rhon, const double* __restrict__ su,
                                            const double* __restrict__ sv, const double* __restrict__ sw,
                                            double* __restrict__ au, double* __restrict__ bu, double* __restrict__ av,
                                            double* __restrict__ bv, double* __restrict__ aw, double* __restrict__ bw) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double r0 = __ldg(rho + c), n0 = __ldg(rhon + c);
  {  // u: a_p = 2dx2(mu_i + mu_i+1) + dy2(exy_j-1 + exy_j) + dz2(exz_k-1 + exz_k)
    const double r = (r0 + __ldg(rho + c + X) + n0 + __ldg(rhon + c + X)) * 0.25;
    const double ap = p.dz2 * __ldg(exz + c - Z) + p.dy2 * __ldg(exy + c - Y) + p.dx2 * __ldg(mu + c) * 2.0 +
                      p.dx2 * __ldg(mu + c + X) * 2.0 + p.dy2 * __ldg(exy + c) + p.dz2 * __ldg(exz + c);
    const double D = p.dtinv + ap / r * 0.5;
    au[c] = 0.5 / (r * D);
    bu[c] = __ldg(su + c) / D;
  }
  if (j <= g.nj - 1) {  // v
    const double r = (r0 + __ldg(rho + c + Y) + n0 + __ldg(rhon + c + Y)) * 0.25;
    const double ap = p.dz2 * __ldg(eyz + c - Z) + p.dy2 * __ldg(mu + c) * 2.0 + p.dx2 * __ldg(exy + c - X) +
                      p.dx2 * __ldg(exy + c) + p.dy2 * __ldg(mu + c + Y) * 2.0 + p.dz2 * __ldg(eyz + c);
    const double D = p.dtinv + ap / r * 0.5;
    av[c] = 0.5 / (r * D);
    bv[c] = __ldg(sv + c) / D;
  }
  {  // w
    const double r = (r0 + __ldg(rho + c + Z) + n0 + __ldg(rhon + c + Z)) * 0.25;
    const double ap = p.dz2 * __ldg(mu + c) * 2.0 + p.dy2 * __ldg(eyz + c - Y) + p.dx2 * __ldg(exz + c - X) +
                      p.dx2 * __ldg(exz + c) + p.dy2 * __ldg(eyz + c) + p.dz2 * __ldg(mu + c + Z) * 2.0;
    const double D = p.dtinv + ap / r * 0.5;
    aw[c] = 0.5 / (r * D);
    bw[c] = __ldg(sw + c) / D;
  }
}

// cal_srcu.f:53-137 fused with the update factors: src is formed in registers
// (1/rho00 taken once per face) and only A = 0.5/(rho00*D), B = src/D are stored.
struct SrcIn {
  const double *u, *v, *w, *rho, *rhon, *adv[3], *advo[3], *prs[3], *vis[3], *fst[3], *fstn[3];
  double grvb, grvp;
};
__global__ void __launch_bounds__(256) k_src_ab(Grid g, VP p, SrcIn in, const double* __restrict__ mu,
                                                const double* __restrict__ exy, const double* __restrict__ exz,
                                                const double* __restrict__ eyz, double* __restrict__ au,
                                                double* __restrict__ bu, double* __restrict__ av, double* __restrict__ bv,
                                                double* __restrict__ aw, double* __restrict__ bw) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double r0 = __ldg(in.rho + c), n0 = __ldg(in.rhon + c);
  auto src = [&](int q, const double* vel, double rinv, double grav) {
    return __ldg(vel + c) * p.dtinv - __ldg(in.adv[q] + c) * 1.5 + __ldg(in.advo[q] + c) * 0.5 -
           __ldg(in.prs[q] + c) * rinv + __ldg(in.vis[q] + c) * rinv * 0.5 + __ldg(in.fst[q] + c) * 0.5 +
           __ldg(in.fstn[q] + c) * 0.5 + grav;
  };
  {
    const double r = (r0 + __ldg(in.rho + c + X) + n0 + __ldg(in.rhon + c + X)) * 0.25, ri = 1.0 / r;
    const double ap = p.dz2 * __ldg(exz + c - Z) + p.dy2 * __ldg(exy + c - Y) + p.dx2 * __ldg(mu + c) * 2.0 +
                      p.dx2 * __ldg(mu + c + X) * 2.0 + p.dy2 * __ldg(exy + c) + p.dz2 * __ldg(exz + c);
    const double Di = 1.0 / (p.dtinv + ap * ri * 0.5);
    au[c] = 0.5 * ri * Di;
    bu[c] = src(0, in.u, ri, in.grvb) * Di;
  }
  if (j <= g.nj - 1) {
    const double r = (r0 + __ldg(in.rho + c + Y) + n0 + __ldg(in.rhon + c + Y)) * 0.25, ri = 1.0 / r;
    const double ap = p.dz2 * __ldg(eyz + c - Z) + p.dy2 * __ldg(mu + c) * 2.0 + p.dx2 * __ldg(exy + c - X) +
                      p.dx2 * __ldg(exy + c) + p.dy2 * __ldg(mu + c + Y) * 2.0 + p.dz2 * __ldg(eyz + c);
    const double Di = 1.0 / (p.dtinv + ap * ri * 0.5);
    av[c] = 0.5 * ri * Di;
    bv[c] = src(1, in.v, ri, in.grvp) * Di;
  }
  {
    const double r = (r0 + __ldg(in.rho + c + Z) + n0 + __ldg(in.rhon + c + Z)) * 0.25, ri = 1.0 / r;
    const double ap = p.dz2 * __ldg(mu + c) * 2.0 + p.dy2 * __ldg(eyz + c - Y) + p.dx2 * __ldg(exz + c - X) +
                      p.dx2 * __ldg(exz + c) + p.dy2 * __ldg(eyz + c) + p.dz2 * __ldg(mu + c + Z) * 2.0;
    const double Di = 1.0 / (p.dtinv + ap * ri * 0.5);
    aw[c] = 0.5 * ri * Di;
    bw[c] = src(2, in.w, ri, 0.0) * Di;
  }
}

// One colour pair of one component.  Thread (a, b, kk) covers, for the pair whose
// first colour has parities (pi,pj,pk), the point (pi+2a, pj+2b, pk+2kk) and the
// point of the second colour (all parities flipped) at (pi'+2a, pj'+2b, pk'+2kk).
// R = double: the FP64 step.  R = float: the mixed-precision step -- the iterates
// stay in double storage, the 14-neighbour sum and the update are formed in float,
// and the increment d = q_new - q and the residual sum are taken in double.
template <int COMP, class R>
__global__ void __launch_bounds__(256) k_pair(Grid g, VP p, int pi, int pj, int pk, const double* __restrict__ mu,
                                              const double* __restrict__ exy, const double* __restrict__ exz,
                                              const double* __restrict__ eyz, const double* __restrict__ A,
                                              const double* __restrict__ B, double* un, double* vn, double* wn,
                                              double* __restrict__ part) {
  __shared__ double sh[256];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int jmax = COMP == 1 ? g.nj - 1 : g.nj;
  const long X = 1, Y = g.sy, Z = g.sz;
  const R dx2 = (R)p.dx2, dy2 = (R)p.dy2, dz2 = (R)p.dz2, dxy = (R)p.dxy, dxz = (R)p.dxz, dyz = (R)p.dyz;
  double e = 0.0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = (h ? 3 - pi : pi) + 2 * (int)(blockIdx.x * 32 + threadIdx.x);
    const int j = (h ? 3 - pj : pj) + 2 * (int)(blockIdx.y * 8 + threadIdx.y);
    const int k = (h ? 3 - pk : pk) + 2 * (int)blockIdx.z;
    if (i > g.ni || j > jmax || k > g.nk) continue;
    const long c = g.at(i, j, k);
    auto U = [&](long o) { return (R)un[c + o]; };
    auto V = [&](long o) { return (R)vn[c + o]; };
    auto W = [&](long o) { return (R)wn[c + o]; };
    auto M = [&](const double* a, long o) { return (R)__ldg(a + c + o); };
    R visn;
    double q;
    if (COMP == 0) {
      const R ym = M(exy, -Y), yp = M(exy, 0), zm = M(exz, -Z), zp = M(exz, 0);
      visn = dz2 * (zm * U(-Z) + zp * U(Z)) + dy2 * (ym * U(-Y) + yp * U(Y)) +
             (R)2 * dx2 * (M(mu, 0) * U(-X) + M(mu, X) * U(X)) + dxy * (ym * (V(-Y) - V(X - Y)) + yp * (V(X) - V(0))) +
             dxz * (zm * (W(-Z) - W(X - Z)) + zp * (W(X) - W(0)));
      q = un[c];
    } else if (COMP == 1) {
      const R xm = M(exy, -X), xp = M(exy, 0), zm = M(eyz, -Z), zp = M(eyz, 0);
      visn = dz2 * (zm * V(-Z) + zp * V(Z)) + (R)2 * dy2 * (M(mu, 0) * V(-Y) + M(mu, Y) * V(Y)) +
             dx2 * (xm * V(-X) + xp * V(X)) + dxy * (xm * (U(-X) - U(-X + Y)) + xp * (U(Y) - U(0))) +
             dyz * (zm * (W(-Z) - W(Y - Z)) + zp * (W(Y) - W(0)));
      q = vn[c];
    } else {
      const R xm = M(exz, -X), xp = M(exz, 0), ym = M(eyz, -Y), yp = M(eyz, 0);
      visn = (R)2 * dz2 * (M(mu, 0) * W(-Z) + M(mu, Z) * W(Z)) + dy2 * (ym * W(-Y) + yp * W(Y)) +
             dx2 * (xm * W(-X) + xp * W(X)) + dxz * (xm * (U(-X) - U(-X + Z)) + xp * (U(Z) - U(0))) +
             dyz * (ym * (V(-Y) - V(-Y + Z)) + yp * (V(Z) - V(0)));
      q = wn[c];
    }
    const double qn = (double)(M(A, 0) * visn + M(B, 0));
    const double d = qn - q;
    if (COMP == 0) un[c] = qn;
    else if (COMP == 1) vn[c] = qn;
    else wn[c] = qn;
    e += d * d;
  }
  sh[tid] = e;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (tid < st) sh[tid] += sh[tid + st];
    __syncthreads();
  }
  if (tid == 0) part[((long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = sh[0];
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
__global__ void __launch_bounds__(256) k_wall(Grid g, double uwall, const double* __restrict__ wc, double* uk,
                                              double* vk, double* wk) {
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
    const double u1 = uk[c];
    const double u0 = c1 * (-uwall) + c2 * u1;
    const double um1 = 2.0 * u0 - u1;
    uk[c - Y] = u0;
    uk[c - 2 * Y] = um1;
    uk[c - 3 * Y] = 2.0 * um1 - u0;
    vk[c - 3 * Y] = -vk[c + Y];
    vk[c - 2 * Y] = -vk[c];
    vk[c - Y] = 0.0;
    const double w1 = wk[c];
    const double w0 = c2 * w1;
    const double wm1 = 2.0 * w0 - w1;
    wk[c - Y] = w0;
    wk[c - 2 * Y] = wm1;
    wk[c - 3 * Y] = 2.0 * wm1 - w0;
  } else {
    const long c = g.at(i, NJ, k);
    const double u1 = uk[c];
    const double u0 = c1 * uwall + c2 * u1;
    const double up2 = 2.0 * u0 - u1;
    uk[c + Y] = u0;
    uk[c + 2 * Y] = up2;
    uk[c + 3 * Y] = 2.0 * up2 - u0;
    const double vm1 = vk[c - Y], vm2 = vk[c - 2 * Y], vm3 = vk[c - 3 * Y];
    vk[c] = 0.0;
    vk[c + Y] = -vm1;
    vk[c + 2 * Y] = -vm2;
    vk[c + 3 * Y] = -vm3;
    const double w1 = wk[c];
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
__global__ void __launch_bounds__(256) k_halo_x(Grid g, int normal, double* uk, double* vk, double* wk) {
  const int j = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (j > g.nj + 3 || k > g.nk + 3) return;
  const int NI = g.ni;
  const long r = g.at(0, j, k);
  double* q[3] = {uk, vk, wk};
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    double* a = q[cmp];
    if (cmp == 0 && !(normal & 1)) {  // bndu's u: u(0)=u(ni+1), u(-1)=u(ni), u(-2)=u(ni-1), u(ni+1) untouched
      a[r] = a[r + NI + 1];
      a[r - 1] = a[r + NI];
      a[r - 2] = a[r + NI - 1];
      a[r + NI + 2] = a[r + 2];
      a[r + NI + 3] = a[r + 3];
    } else {
      a[r - 2] = a[r + NI - 2];
      a[r - 1] = a[r + NI - 1];
      a[r] = a[r + NI];
      a[r + NI + 1] = a[r + 1];
      a[r + NI + 2] = a[r + 2];
      a[r + NI + 3] = a[r + 3];
    }
  }
}
// z halos; for w bndu's copy is shifted by one (bndu.f:144-146).
__global__ void __launch_bounds__(256) k_halo_z(Grid g, int normal, double* uk, double* vk, double* wk) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || j > g.nj + 3) return;
  const int NK = g.nk;
  const long Z = g.sz;
  const long r = g.at(i, j, 0);
  double* q[3] = {uk, vk, wk};
#pragma unroll
  for (int cmp = 0; cmp < 3; ++cmp) {
    double* a = q[cmp];
    if (cmp == 2 && !(normal & 4)) {  // bndu's w: w(0)=w(nk+1), ..., w(nk+1) untouched
      a[r] = a[r + (NK + 1) * Z];
      a[r - Z] = a[r + NK * Z];
      a[r - 2 * Z] = a[r + (NK - 1) * Z];
      a[r + (NK + 2) * Z] = a[r + 2 * Z];
      a[r + (NK + 3) * Z] = a[r + 3 * Z];
    } else {
      a[r - 2 * Z] = a[r + (NK - 2) * Z];
      a[r - Z] = a[r + (NK - 1) * Z];
      a[r] = a[r + NK * Z];
      a[r + (NK + 1) * Z] = a[r + Z];
      a[r + (NK + 2) * Z] = a[r + 2 * Z];
      a[r + (NK + 3) * Z] = a[r + 3 * Z];
    }
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
}  // namespace

void visc_prep(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, int harmonic,
               const double* mu, const double* rho, const double* rhon, const double* const* src, double* const* E,
               double* const* AB, const double* l1, const double* l2, const double* phi, double dy, double* wallc) {
  VP p;
  p.dtinv = 1.0 / dt;
  p.dx2 = dxinv * dxinv;
  p.dy2 = dyinv * dyinv;
  p.dz2 = dzinv * dzinv;
  p.dxy = dxinv * dyinv;
  p.dxz = dxinv * dzinv;
  p.dyz = dyinv * dzinv;
  p.harmonic = harmonic;
  dim3 b(32, 8, 1);
  k_edges<<<dim3((g.ni + 1 + 31) / 32, (g.nj + 1 + 7) / 8, g.nk + 1), b, 0, s>>>(g, p, mu, E[0], E[1], E[2]);
  k_ab<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), b, 0, s>>>(g, p, mu, E[0], E[1], E[2], rho, rhon, src[0], src[1],
                                                                 src[2], AB[0], AB[1], AB[2], AB[3], AB[4], AB[5]);
  k_wall_coef<<<dim3((g.ni + 6 + 31) / 32, (2 * (g.nk + 6) + 7) / 8), b, 0, s>>>(g, dy, l1, l2, phi, wallc);
  count_launch(3);
}

void src_visc_prep(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, int harmonic,
                   double grvb, double grvp, const double* u, const double* v, const double* w,
                   const double* const* adv, const double* const* advo, const double* const* prs,
                   const double* const* vis, const double* const* fst, const double* const* fstn, const double* mu,
                   const double* rho, const double* rhon, double* const* E, double* const* AB, const double* l1,
                   const double* l2, const double* phi, double dy, double* wallc) {
  VP p;
  p.dtinv = 1.0 / dt;
  p.dx2 = dxinv * dxinv;
  p.dy2 = dyinv * dyinv;
  p.dz2 = dzinv * dzinv;
  p.dxy = dxinv * dyinv;
  p.dxz = dxinv * dzinv;
  p.dyz = dyinv * dzinv;
  p.harmonic = harmonic;
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
  dim3 b(32, 8, 1);
  k_edges<<<dim3((g.ni + 1 + 31) / 32, (g.nj + 1 + 7) / 8, g.nk + 1), b, 0, s>>>(g, p, mu, E[0], E[1], E[2]);
  k_src_ab<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), b, 0, s>>>(g, p, in, mu, E[0], E[1], E[2], AB[0], AB[1],
                                                                     AB[2], AB[3], AB[4], AB[5]);
  k_wall_coef<<<dim3((g.ni + 6 + 31) / 32, (2 * (g.nk + 6) + 7) / 8), b, 0, s>>>(g, dy, l1, l2, phi, wallc);
  count_launch(3);
}

void wall_halo(cudaStream_t s, const Grid& g, int normal, double uwall, const double* wallc, double* un, double* vn,
               double* wn) {
  dim3 b(32, 8, 1);
  k_wall<<<dim3((g.ni + 6 + 31) / 32, (2 * (g.nk + 6) + 7) / 8), b, 0, s>>>(g, uwall, wallc, un, vn, wn);
  k_halo_x<<<dim3((g.nj + 6 + 31) / 32, (g.nk + 6 + 7) / 8), b, 0, s>>>(g, normal, un, vn, wn);
  k_halo_z<<<dim3((g.ni + 6 + 31) / 32, (g.nj + 6 + 7) / 8), b, 0, s>>>(g, normal, un, vn, wn);
  count_launch(3);
}

void sor_iteration(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, int harmonic,
                   const double* mu, double* const* E, double* const* AB, double uwall, const double* wallc,
                   double* un, double* vn, double* wn, double* part, double* errsum, bool fp32) {
  VP p;
  p.dtinv = 0.0;
  p.dx2 = dxinv * dxinv;
  p.dy2 = dyinv * dyinv;
  p.dz2 = dzinv * dzinv;
  p.dxy = dxinv * dyinv;
  p.dxz = dxinv * dzinv;
  p.dyz = dyinv * dzinv;
  p.harmonic = harmonic;
  // first colour of each pair (solu_sor4.f:94-120): (1,1,1) (1,1,2) (1,2,1) (2,1,1)
  static const int pi_[4] = {1, 1, 1, 2}, pj_[4] = {1, 1, 2, 1}, pk_[4] = {1, 2, 1, 1};
  const dim3 blk(32, 8, 1);
  const dim3 grd((unsigned)((g.ni / 2 + 31) / 32), (unsigned)((g.nj / 2 + 7) / 8), (unsigned)(g.nk / 2));
  const long nb = (long)grd.x * grd.y * grd.z;
  for (int comp = 0; comp < 3; ++comp) {
    for (int pr = 0; pr < 4; ++pr) {
      double* pp = part + (long)(comp * 4 + pr) * nb;
#define FMF_PAIR(C, R)                                                                                      \
  k_pair<C, R><<<grd, blk, 0, s>>>(g, p, pi_[pr], pj_[pr], pk_[pr], mu, E[0], E[1], E[2], AB[2 * C], AB[2 * C + 1], \
                                   un, vn, wn, pp)
      if (fp32) {
        if (comp == 0) FMF_PAIR(0, float);
        else if (comp == 1) FMF_PAIR(1, float);
        else FMF_PAIR(2, float);
      } else {
        if (comp == 0) FMF_PAIR(0, double);
        else if (comp == 1) FMF_PAIR(1, double);
        else FMF_PAIR(2, double);
      }
#undef FMF_PAIR
      count_launch();
      wall_halo(s, g, 1 << comp, uwall, wallc, un, vn, wn);
    }
  }
  k_sum_parts2<<<1, 256, 0, s>>>(part, nb * 12, errsum);
  count_launch();
}

long sor_parts(const Grid& g) {
  return (long)((g.ni / 2 + 31) / 32) * ((g.nj / 2 + 7) / 8) * (g.nk / 2) * 12;
}

}  // namespace fused
}  // namespace fmf
