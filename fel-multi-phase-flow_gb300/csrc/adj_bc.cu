// adj_bc.cu -- adjoints of the boundary conditions, copies and linear stencils of
// the step (k_bc.cu, k_glue.cu, k_press.cu, fused_visc.cu wall/halo kernels).
#include "adj.cuh"
#include "refresh.cuh"

namespace fmf {
namespace adj {

namespace {
// out[0] = sum of a[0..n-1] (two-stage tree; partials in scratch slot 11)
__global__ void k_sum_stage(const double* a, long n, double* part) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += (long)gridDim.x * 256) acc += a[t];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
void sum_all(cudaStream_t s, long n, const double* a, double* out) {
  const int nb = 152 * 4;
  double* part = (double*)scratch(sizeof(double) * nb, 11);
  k_sum_stage<<<nb, 256, 0, s>>>(a, n, part);
  k_sum_stage<<<1, 256, 0, s>>>(part, nb, out);
  count_launch(2);
}
}  // namespace

// Transposed copy along one line (stride S, N interior points): the adjoints of the
// destinations -2, -1, 0, N+1, N+2, N+3 are added to their sources and cleared.
// SHIFT: bndu's copy of the normal component (-2, -1, 0 from N-1, N, N+1; N+1 not
// written).  The destination loads are issued together; the source updates run
// one after another (sources can coincide when N = 4).
template <bool SHIFT>
__device__ __forceinline__ void line_T(double* __restrict__ a, long r, long S, int N) {
  const long sh = SHIFT ? S : 0;
  const double L0 = a[r - 2 * S], L1 = a[r - S], L2 = a[r], L4 = a[r + (N + 2) * S], L5 = a[r + (N + 3) * S];
  const double L3 = SHIFT ? 0.0 : a[r + (N + 1) * S];
  if (N >= 8) {  // six distinct sources: every load first, then every store
    const double s0 = a[r + (N - 2) * S + sh], s1 = a[r + (N - 1) * S + sh], s2 = a[r + N * S + sh];
    const double s3 = SHIFT ? 0.0 : a[r + S], s4 = a[r + 2 * S], s5 = a[r + 3 * S];
    a[r - 2 * S] = 0.0;
    a[r - S] = 0.0;
    a[r] = 0.0;
    if (!SHIFT) a[r + (N + 1) * S] = 0.0;
    a[r + (N + 2) * S] = 0.0;
    a[r + (N + 3) * S] = 0.0;
    a[r + (N - 2) * S + sh] = s0 + L0;
    a[r + (N - 1) * S + sh] = s1 + L1;
    a[r + N * S + sh] = s2 + L2;
    if (!SHIFT) a[r + S] = s3 + L3;
    a[r + 2 * S] = s4 + L4;
    a[r + 3 * S] = s5 + L5;
    return;
  }
  a[r - 2 * S] = 0.0;
  a[r - S] = 0.0;
  a[r] = 0.0;
  if (!SHIFT) a[r + (N + 1) * S] = 0.0;
  a[r + (N + 2) * S] = 0.0;
  a[r + (N + 3) * S] = 0.0;
  a[r + (N - 2) * S + sh] += L0;
  a[r + (N - 1) * S + sh] += L1;
  a[r + N * S + sh] += L2;
  if (!SHIFT) a[r + S] += L3;
  a[r + 2 * S] += L4;
  a[r + 3 * S] += L5;
}
// x lines (one thread per (j,k)), normal: bit c set = plain copy of component c
__global__ void __launch_bounds__(256) k_halo_x_T(Grid g, int normal, double* __restrict__ lu,
                                                  double* __restrict__ lv, double* __restrict__ lw) {
  const int j = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (j > g.nj + 3 || k > g.nk + 3) return;
  const long r = g.at(0, j, k);
  if (normal & 1) line_T<false>(lu, r, 1, g.ni);
  else line_T<true>(lu, r, 1, g.ni);
  if (lv) line_T<false>(lv, r, 1, g.ni);
  if (lw) line_T<false>(lw, r, 1, g.ni);
}
// z lines (one thread per (i,j)); w is the shifted component
__global__ void __launch_bounds__(256) k_halo_z_T(Grid g, int normal, double* __restrict__ lu,
                                                  double* __restrict__ lv, double* __restrict__ lw) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 3 || j > g.nj + 3) return;
  const long r = g.at(i, j, 0);
  if (lu) line_T<false>(lu, r, g.sz, g.nk);
  if (lv) line_T<false>(lv, r, g.sz, g.nk);
  if (lw) {
    if (normal & 4) line_T<false>(lw, r, g.sz, g.nk);
    else line_T<true>(lw, r, g.sz, g.nk);
  }
}
// k_halo_x_T for ni >= 8 with 8 lanes per (j, k, component): lanes 0-2 move the
// adjoints of the low ghosts -2..0 to their sources, lanes 3-5 those of ni+1..ni+3;
// no lane's destination is another lane's source, so the lanes are independent.
__global__ void __launch_bounds__(256) k_halo_x_T8(Grid g, int normal, double* __restrict__ lu,
                                                   double* __restrict__ lv, double* __restrict__ lw) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int m = (int)(t & 7);
  const long task = t >> 3;
  const long JK = (long)(g.nj + 6) * (g.nk + 6);
  if (m >= 6 || task >= 3 * JK) return;
  const int cmp = (int)(task / JK);
  const int rem = (int)(task % JK);
  double* a = cmp == 0 ? lu : (cmp == 1 ? lv : lw);
  if (!a) return;
  const bool sh = cmp == 0 && !(normal & 1);
  const long r = g.at(0, -2 + rem % (g.nj + 6), -2 + rem / (g.nj + 6));
  long dst, src;
  if (m < 3) {
    dst = r + m - 2;
    src = r + g.ni - 2 + m + (sh ? 1 : 0);
  } else {
    if (sh && m == 3) return;  // the shifted copy does not write ni+1
    dst = r + g.ni + m - 2;
    src = r + m - 2;
  }
  const double L = a[dst], v = a[src];
  a[dst] = 0.0;
  a[src] = v + L;
}
dim3 xh_grid(const Grid& g) { return dim3((g.nj + 6 + 31) / 32, (g.nk + 6 + 7) / 8); }
dim3 zh_grid(const Grid& g) { return dim3((g.ni + 6 + 31) / 32, (g.nj + 6 + 7) / 8); }
void launch_halo_x_T(cudaStream_t s, const Grid& g, int normal, double* lu, double* lv, double* lw) {
  if (g.ni >= 8)
    k_halo_x_T8<<<(unsigned)((24L * (g.nj + 6) * (g.nk + 6) + 255) / 256), 256, 0, s>>>(g, normal, lu, lv, lw);
  else
    k_halo_x_T<<<xh_grid(g), dim3(32, 8), 0, s>>>(g, normal, lu, lv, lw);
}

// bnd_periodic: x copies over every (j,k) then z copies over every (i,j); the adjoint
// runs z first.
void periodic_T(cudaStream_t s, const Grid& g, double* lq) {
  k_halo_z_T<<<zh_grid(g), dim3(32, 8), 0, s>>>(g, 4, nullptr, nullptr, lq);
  launch_halo_x_T(s, g, 1, lq, nullptr, nullptr);
  count_launch(2);
}

void neumann_T(cudaStream_t s, const Grid& g, double* lq) {
  const Grid G = g;
  range2(s, -2, g.ni + 3, -2, g.nk + 3, [=] __device__(int i, int k) {
    const int NJ = G.nj;
    const long Y = G.sy, r = G.at(i, 0, k);
    // destinations j = -2, -1, 0, NJ+1, NJ+2, NJ+3 from 3, 2, 1, NJ, NJ-1, NJ-2
    const double L0 = lq[r - 2 * Y], L1 = lq[r - Y], L2 = lq[r], L3 = lq[r + (NJ + 1) * Y], L4 = lq[r + (NJ + 2) * Y],
                 L5 = lq[r + (NJ + 3) * Y];
    lq[r - 2 * Y] = 0.0;
    lq[r - Y] = 0.0;
    lq[r] = 0.0;
    lq[r + (NJ + 1) * Y] = 0.0;
    lq[r + (NJ + 2) * Y] = 0.0;
    lq[r + (NJ + 3) * Y] = 0.0;
    lq[r + 3 * Y] += L0;
    lq[r + 2 * Y] += L1;
    lq[r + Y] += L2;
    lq[r + NJ * Y] += L3;
    lq[r + (NJ - 1) * Y] += L4;
    lq[r + (NJ - 2) * Y] += L5;
  });
}

// q -= mean(interior q) at every point: lq[interior] -= sum(lq)/cells
void avzero_T(cudaStream_t s, const Grid& g, double* lq) {
  const Grid G = g;
  double* S = (double*)scratch(sizeof(double) * 2, 12);
  sum_all(s, g.n, lq, S);
  const double inv = 1.0 / (double)g.cells();
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) { lq[G.at(i, j, k)] -= S[0] * inv; });
}

void summation_T(cudaStream_t s, const Grid& g, const double* q1, double* lq0, double* lq1) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    const bool in = i >= 1 && i <= G.ni && j >= 1 && j <= G.nj && k >= 1 && k <= G.nk;
    const double x = q1[c];
    const double m = (!in || (x >= 0.0 && x <= 1.0)) ? 1.0 : 0.0;
    lq1[c] += m * lq0[c];
    lq0[c] = 0.0;
  });
}

void gnbc_T(cudaStream_t s, const Grid& g, const double* uk, const double* wk, double uwall, const double* theta0,
            double sigma, const double* zeta, const double* ltheta, double* lu, double* lw, double* ltheta0,
            double* lzeta) {
  const Grid G = g;
  const double pi = std::acos(-1.0);
  range2(s, -2, g.ni + 3, -2, 2 * (g.nk + 6) - 3, [=] __device__(int i, int kk) {
    const int side = kk >= G.nk + 4 ? 1 : 0;
    const int k = side ? kk - (G.nk + 6) : kk;
    const int ja = side ? G.nj : 0, jb = ja + 1, jw = side ? G.nj : 1;
    const long c = G.at(i, jw, k);
    const double lt = ltheta[c];
    if (lt == 0.0) return;
    const double us = side ? -uwall : uwall;
    const int mi = (i + G.ni + 2) % (G.ni + 3);
    const long p0 = G.at(mi, ja, k), p1 = G.at(mi, jb, k), p2 = G.at(i, ja, k), p3 = G.at(i, jb, k);
    const double ucx = (uk[p0] + uk[p1] + uk[p2] + uk[p3]) / 4.0 + us;
    const double ucz = (wk[p0] + wk[p1] + wk[p2] + wk[p3]) / 4.0;
    const double r = sqrt(ucx * ucx + ucz * ucz + 1.0e-12);
    const double sg = signbit(ucx) ? -1.0 : 1.0;
    double ucl = sg * r;
    const double flip = (i <= G.ni / 2) ? -1.0 : 1.0;
    ucl *= flip;
    const double th0 = theta0[c] * (pi / 180.0);
    const double ct = cos(th0) - zeta[c] * ucl / sigma;
    if (!(ct > -1.0 && ct < 1.0)) return;  // clamped: no dependence
    const double L = lt * (-(180.0 / pi) / sqrt(1.0 - ct * ct));
    ltheta0[c] += L * (-sin(th0)) * (pi / 180.0);
    lzeta[c] += L * (-ucl / sigma);
    const double lucl = L * (-zeta[c] / sigma) * flip;
    const double lr = sg * lucl;
    const double lx = lr * ucx / r * 0.25, lz = lr * ucz / r * 0.25;
    const long ps[4] = {p0, p1, p2, p3};
    for (int t = 0; t < 4; ++t) {
      aadd(lu + ps[t], lx);
      aadd(lw + ps[t], lz);
    }
  });
}

void contact_angle_T(cudaStream_t s, const Grid& g, const double* qk, const double* theta, double dx, double dy,
                     double dz, double* lq, double* ltheta) {
  const Grid G = g;
  const double pi = std::acos(-1.0), ax = dy / dx, az = dy / dz;
  range2(s, -1, g.ni + 2, -1, 2 * (g.nk + 4) - 2, [=] __device__(int i, int kk) {
    const int side = kk >= G.nk + 3 ? 1 : 0;
    const int k = side ? kk - (G.nk + 4) : kk;
    const int jw = side ? G.nj : 1;
    const long g0 = side ? G.at(i, G.nj + 1, k) : G.at(i, 0, k);
    const long g1 = side ? G.at(i, G.nj + 2, k) : G.at(i, -1, k);
    const long g2 = side ? G.at(i, G.nj + 3, k) : G.at(i, -2, k);
    const double L0 = lq[g0], L1 = lq[g1], L2 = lq[g2];
    lq[g0] = 0.0;
    lq[g1] = 0.0;
    lq[g2] = 0.0;
    if (L0 == 0.0 && L1 == 0.0 && L2 == 0.0) return;
    const double eps = 1.0e-20;
    using D1 = Dual<1>;
    const long cw = G.at(i, jw, k);
    const D1 th = D1::var(theta[cw], 0) * (pi / 180.0);
    const D1 ct = dcos(th), sn = dsin(th);
    const double sg = (i - G.ni / 2) >= 0 ? 1.0 : -1.0;
    D1 nx = sn * (sg * ax), nz = sn * (sg * az), ny = ct;
    const D1 nrm = dsqrt(nx * nx + ny * ny + nz * nz + eps);
    nx = nx / nrm;
    ny = ny / nrm;
    nz = nz / nrm;
    const D1 A = ny / (nx + eps) * (0.5 * ax), B = ny / (nz + eps) * (0.5 * az);
    const double Dx = qk[G.at(i + 1, jw, k)] - qk[G.at(i - 1, jw, k)];
    const double Dz = qk[G.at(i, jw, k + 1)] - qk[G.at(i, jw, k - 1)];
    // gh = q1 - A Dx - B Dz; ghosts gh, 2gh - q1, 3gh - 2q1
    const double lgh = L0 + 2.0 * L1 + 3.0 * L2;
    aadd(lq + cw, L0 + L1 + L2);  // q1: through gh (lgh) and directly (-L1 - 2 L2)
    aadd(lq + G.at(i + 1, jw, k), -A.v * lgh);
    aadd(lq + G.at(i - 1, jw, k), A.v * lgh);
    aadd(lq + G.at(i, jw, k + 1), -B.v * lgh);
    aadd(lq + G.at(i, jw, k - 1), B.v * lgh);
    ltheta[cw] += (-Dx * lgh) * A.d[0] + (-Dz * lgh) * B.d[0];
  });
}

__global__ void __launch_bounds__(256) k_wall_T(Grid G, double uwall, const double* __restrict__ wc,
                                                const double* __restrict__ uk, const double* __restrict__ wk,
                                                double* __restrict__ lu, double* __restrict__ lv,
                                                double* __restrict__ lw, double* __restrict__ lwc) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int kk = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > G.ni + 3 || kk > 2 * (G.nk + 6) - 3) return;
  {
    const int side = kk >= G.nk + 4 ? 1 : 0;
    const int k = side ? kk - (G.nk + 6) : kk;
    const long o = (((long)side * (G.nk + 6) + (k + 2)) * (G.ni + 6) + (i + 2)) * 2;
    const double c2 = wc[o + 1];
    const long Y = G.sy;
    const long c = G.at(i, side ? G.nj : 1, k);
    const long t = side ? Y : -Y;
    // every load first (ghost rows and the wall rows they came from are disjoint)
    const double L1 = lu[c + t], L2 = lu[c + 2 * t], L3 = lu[c + 3 * t], U0 = lu[c];
    const double M1 = lw[c + t], M2 = lw[c + 2 * t], M3 = lw[c + 3 * t], W0 = lw[c];
    // v: side 0 ghosts 0, -1, -2 from -, 1, 2; side 1 ghosts nj, nj+1..3 from -, nj-1..3
    const double va = lv[c + (side ? Y : -2 * Y)], vb = lv[c + (side ? 2 * Y : -3 * Y)];
    const double vd = side ? lv[c + 3 * Y] : 0.0;
    const double V0 = lv[c + (side ? -Y : 0)], V1 = lv[c + (side ? -2 * Y : Y)];
    const double V2 = side ? lv[c - 3 * Y] : 0.0;
    lu[c + t] = lu[c + 2 * t] = lu[c + 3 * t] = 0.0;
    lw[c + t] = lw[c + 2 * t] = lw[c + 3 * t] = 0.0;
    lu[c] = U0 + c2 * L1 + (2.0 * c2 - 1.0) * L2 + (3.0 * c2 - 2.0) * L3;
    lw[c] = W0 + c2 * M1 + (2.0 * c2 - 1.0) * M2 + (3.0 * c2 - 2.0) * M3;
    const double SL = L1 + 2.0 * L2 + 3.0 * L3, SM = M1 + 2.0 * M2 + 3.0 * M3;
    if (lwc) {
      lwc[o] += (side ? uwall : -uwall) * SL;
      lwc[o + 1] += uk[c] * SL + wk[c] * SM;
    }
    if (!side) {  // v(0) = 0, v(-1) = -v(1), v(-2) = -v(2)
      lv[c - Y] = lv[c - 2 * Y] = lv[c - 3 * Y] = 0.0;
      lv[c] = V0 - va;
      lv[c + Y] = V1 - vb;
    } else {  // v(nj) = 0, v(nj+m) = -v(nj-m)
      lv[c] = lv[c + Y] = lv[c + 2 * Y] = lv[c + 3 * Y] = 0.0;
      lv[c - Y] = V0 - va;
      lv[c - 2 * Y] = V1 - vb;
      lv[c - 3 * Y] = V2 - vd;
    }
  }
}
// The owned rows of one source column next to wall SIDE (side 0: rows -2..2, side 1:
// rows nj-3..nj+3) with its x, z and corner images gathered in, the wall transpose
// applied and the images cleared; returns L1 + 2 L2 + 3 L3 of u or w (the weight of
// the slip coefficient), 0 for v.  Every load is issued before the first store.
template <int SIDE>
__device__ __forceinline__ double wall_col_T(const Grid& G, double* __restrict__ a, int cmp, int i, int k, int ix,
                                             int kz, double c2) {
  constexpr int NR = SIDE ? 7 : 5;
  const int j0 = SIDE ? G.nj - 3 : -2;
  const long Y = G.sy;
  const bool hx = ix != kNoHalo, hz = kz != kNoHalo;
  const long c0 = G.at(i, j0, k), cx = hx ? G.at(ix, j0, k) : c0, cz = hz ? G.at(i, j0, kz) : c0,
             cxz = hx && hz ? G.at(ix, j0, kz) : c0;
  double gv[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) gv[r] = a[c0 + r * Y];
  // the images one column at a time (most source columns have none): few registers
  // live, which keeps the occupancy of the whole kernel up
#pragma unroll 1
  for (int q = 0; q < 3; ++q) {
    const bool has = q == 0 ? hx : (q == 1 ? hz : hx && hz);
    if (!has) continue;
    const long ci = q == 0 ? cx : (q == 1 ? cz : cxz);
    double v[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) v[r] = a[ci + r * Y];
#pragma unroll
    for (int r = 0; r < NR; ++r) gv[r] += v[r];
  }
  double S = 0.0;
  if (cmp != 1) {  // u, w: the wall row is r = 3 (j = 1 or nj), its ghosts on the far side
    constexpr int t1 = SIDE ? 1 : -1;
    const double L1 = gv[3 + t1], L2 = gv[3 + 2 * t1], L3 = gv[3 + 3 * t1];
    gv[3] += c2 * L1 + (2.0 * c2 - 1.0) * L2 + (3.0 * c2 - 2.0) * L3;
    gv[3 + t1] = gv[3 + 2 * t1] = gv[3 + 3 * t1] = 0.0;
    S = L1 + 2.0 * L2 + 3.0 * L3;
  } else {
    if constexpr (SIDE == 0) {  // v(0) = 0, v(-1) = -v(1), v(-2) = -v(2); rows -2..2 are r = 0..4
      gv[3] -= gv[1];
      gv[4] -= gv[0];
      gv[0] = gv[1] = gv[2] = 0.0;
    } else {  // v(nj) = 0, v(nj+m) = -v(nj-m); rows nj-3..nj+3 are r = 0..6
      gv[2] -= gv[4];
      gv[1] -= gv[5];
      gv[0] -= gv[6];
      gv[3] = gv[4] = gv[5] = gv[6] = 0.0;
    }
  }
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    a[c0 + r * Y] = gv[r];
    if (hx) a[cx + r * Y] = 0.0;
    if (hz) a[cz + r * Y] = 0.0;
    if (hx && hz) a[cxz + r * Y] = 0.0;
  }
  return S;
}
// Transpose of the one-pass refresh (ni, nj, nk >= 8): the same result as halo_z_T,
// halo_x_T and k_wall_T in that order.  Every ghost column is a copy of its source
// column, so the adjoint of a source column is its own plus that of its images (the
// x, z and corner destinations that copy it); the wall transpose then runs on the
// source column only (on the cleared ghost columns it moves zeros).  Blocks [0, nbW):
// one thread per (column, wall, component) owning rows -2..2 (or nj-3..nj+3) of a
// source column and its images: gathers them, applies the wall transpose, clears
// the images;
// [nbW, nbW + nb1): rows 3..nj-4 of the x-source columns, one thread per (j, k,
// component) for its six slots, with the z and corner images where k has one; the
// rest: rows 3..nj-4 of the columns with a z image only, one thread per (i, j,
// component).  Each point has one owner.
__global__ void __launch_bounds__(256) k_refresh_T(Grid G, int normal, double uwall, const double* __restrict__ wc,
                                                   const double* __restrict__ uk, const double* __restrict__ wk,
                                                   double* __restrict__ lu, double* __restrict__ lv,
                                                   double* __restrict__ lw, double* __restrict__ lwc, int nbW,
                                                   int nb1) {
  const int shu = !(normal & 1), shw = !(normal & 4);
  const int NI = G.ni, NJ = G.nj, NK = G.nk;
  const int b = (int)blockIdx.x;
  if (b < nbW) {
    const long t = (long)b * 256 + threadIdx.x;
    const int W = NI + 6;
    if (t >= 6L * W * (NK + 6)) return;
    const int i = (int)(t % W) - 2;
    const long r = t / W;
    const int kk = (int)(r % (2 * (NK + 6)));
    const int cmp = (int)(r / (2 * (NK + 6)));
    const int side = kk >= NK + 6 ? 1 : 0;
    const int k = kk - side * (NK + 6) - 2;
    const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
    if (halo_src(i, NI, sx) != i || halo_src(k, NK, sz) != k) return;  // a ghost column of this component
    const long o = (((long)side * (NK + 6) + (k + 2)) * W + (i + 2)) * 2;
    const double c2 = wc[o + 1];
    double* a = cmp == 0 ? lu : (cmp == 1 ? lv : lw);
    const int ix = halo_image(i, NI, sx), kz = halo_image(k, NK, sz);
    const double S = side ? wall_col_T<1>(G, a, cmp, i, k, ix, kz, c2) : wall_col_T<0>(G, a, cmp, i, k, ix, kz, c2);
    if (lwc && cmp != 1 && S != 0.0) {
      // u and w of a column both feed lwc[o + 1]: atomic there
      const long c = G.at(i, side ? NJ : 1, k);
      if (cmp == 0) lwc[o] += (side ? uwall : -uwall) * S;
      atomicAdd(lwc + o + 1, (cmp == 0 ? uk[c] : wk[c]) * S);
    }
    return;
  }
  // Parts 1 and 2 take the six halo slots of a row (or column) in one thread: each
  // slot's source and image are points no other slot touches, so every load is
  // issued before any store (one memory round trip per thread).
  if (b < nbW + nb1) {
    const long task = (long)(b - nbW) * 256 + threadIdx.x;
    const int nj2 = NJ - 6;  // rows 3..nj-4
    if (task >= 3L * nj2 * (NK + 6)) return;
    const int cmp = (int)(task / ((long)nj2 * (NK + 6)));
    const int rem = (int)(task % ((long)nj2 * (NK + 6)));
    const int j = 3 + rem % nj2, k = -2 + rem / nj2;
    const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
    if (halo_src(k, NK, sz) != k) return;  // a z destination: gathered by its source
    const int kz = halo_image(k, NK, sz);
    double* a = cmp == 0 ? lu : (cmp == 1 ? lv : lw);
    double v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int d = halo_dest(m, NI, sx);
      v[m] = d == kNoHalo ? 0.0 : a[G.at(halo_src(d, NI, sx), j, k)] + a[G.at(d, j, k)];
    }
    if (kz != kNoHalo) {
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const int d = halo_dest(m, NI, sx);
        if (d != kNoHalo) v[m] += a[G.at(halo_src(d, NI, sx), j, kz)] + a[G.at(d, j, kz)];
      }
    }
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int d = halo_dest(m, NI, sx);
      if (d == kNoHalo) continue;
      const int is = halo_src(d, NI, sx);
      a[G.at(d, j, k)] = 0.0;
      if (kz != kNoHalo) {
        a[G.at(is, j, kz)] = 0.0;
        a[G.at(d, j, kz)] = 0.0;
      }
      a[G.at(is, j, k)] = v[m];
    }
    return;
  }
  const long t = (long)(b - nbW - nb1) * 256 + threadIdx.x;
  const int nj2 = NJ - 6;
  const int i = 1 + (int)(t % (NI + 1));
  const long r = t / (NI + 1);
  const int j = 3 + (int)(r % nj2);
  const int cmp = (int)(r / nj2);
  if (cmp >= 3) return;
  const int sx = cmp == 0 ? shu : 0, sz = cmp == 2 ? shw : 0;
  if (halo_src(i, NI, sx) != i || halo_image(i, NI, sx) != kNoHalo) return;  // x ghost, or done with its x image
  double* a = cmp == 0 ? lu : (cmp == 1 ? lv : lw);
  double v[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int d = halo_dest(m, NK, sz);
    v[m] = d == kNoHalo ? 0.0 : a[G.at(i, j, halo_src(d, NK, sz))] + a[G.at(i, j, d)];
  }
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int d = halo_dest(m, NK, sz);
    if (d == kNoHalo) continue;
    a[G.at(i, j, halo_src(d, NK, sz))] = v[m];
    a[G.at(i, j, d)] = 0.0;
  }
}
void wall_T(cudaStream_t s, const Grid& g, double uwall, const double* wc, const double* uk, const double* wk,
            double* lu, double* lv, double* lw, double* lwc) {
  k_wall_T<<<dim3((g.ni + 6 + 31) / 32, (2 * (g.nk + 6) + 7) / 8), dim3(32, 8), 0, s>>>(g, uwall, wc, uk, wk, lu, lv,
                                                                                       lw, lwc);
  count_launch();
}

void halo_x_T(cudaStream_t s, const Grid& g, int normal, double* lu, double* lv, double* lw) {
  launch_halo_x_T(s, g, normal, lu, lv, lw);
  count_launch();
}

void halo_z_T(cudaStream_t s, const Grid& g, int normal, double* lu, double* lv, double* lw) {
  k_halo_z_T<<<zh_grid(g), dim3(32, 8), 0, s>>>(g, normal, lu, lv, lw);
  count_launch();
}

void wall_halo_T(cudaStream_t s, const Grid& g, int normal, double uwall, const double* wc, const double* u,
                 const double* w, double* lu, double* lv, double* lw, double* lwc) {
  if (refresh_one_pass(g.ni, g.nj, g.nk)) {
    const long tw = 6L * (g.ni + 6) * (g.nk + 6), t1 = 3L * (g.nj - 6) * (g.nk + 6),
               t2 = 3L * (g.ni + 1) * (g.nj - 6);
    const int nbW = (int)((tw + 255) / 256), nb1 = (int)((t1 + 255) / 256), nb2 = (int)((t2 + 255) / 256);
    k_refresh_T<<<nbW + nb1 + nb2, 256, 0, s>>>(g, normal, uwall, wc, u, w, lu, lv, lw, lwc, nbW, nb1);
    count_launch();
    return;
  }
  halo_z_T(s, g, normal, lu, lv, lw);
  halo_x_T(s, g, normal, lu, lv, lw);
  wall_T(s, g, uwall, wc, u, w, lu, lv, lw, lwc);
}

void wall_coef_T(cudaStream_t s, const Grid& g, double dy, const double* l1, const double* l2, const double* phi,
                 const double* lwc, double* lphi, double* ll1, double* ll2) {
  const Grid G = g;
  range2(s, -2, g.ni + 3, -2, 2 * (g.nk + 6) - 3, [=] __device__(int i, int kk) {
    const int side = kk >= G.nk + 4 ? 1 : 0;
    const int k = side ? kk - (G.nk + 6) : kk;
    const int jw = side ? G.nj : 1;
    const long o = (((long)side * (G.nk + 6) + (k + 2)) * (G.ni + 6) + (i + 2)) * 2;
    const double lc1 = lwc[o], lc2 = lwc[o + 1];
    if (lc1 == 0.0 && lc2 == 0.0) return;
    using D3 = Dual<3>;
    const long ca = G.at(i, jw, k), cb = G.at((i + 1) % (G.ni + 3), jw, k);
    const D3 pa = D3::var((phi[ca] + phi[cb]) / 2.0, 0);
    const D3 L1 = D3::var(l1[ca], 1), L2 = D3::var(l2[ca], 2);
    const D3 i1 = pa / L1, i2 = (1.0 - pa) / L2;
    const D3 ls = 1.0 / (i1 + i2);
    const D3 c1 = (2.0 * dy) / (2.0 * ls + dy), c2 = (2.0 * ls - dy) / (2.0 * ls + dy);
    const double lpa = lc1 * c1.d[0] + lc2 * c2.d[0];
    aadd(lphi + ca, 0.5 * lpa);
    aadd(lphi + cb, 0.5 * lpa);
    ll1[ca] += lc1 * c1.d[1] + lc2 * c2.d[1];
    ll2[ca] += lc1 * c1.d[2] + lc2 * c2.d[2];
  });
}

// ---- linear stencils ----------------------------------------------------------
void grad_p2a_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lqx,
                const double* lqy, const double* lqz, double* lq) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int x, int y, int z) {
    double acc = 0.0;
    for (int c = 0; c < 2; ++c)
      for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a) {
          const int i = x - a, j = y - b, k = z - c;
          if (i < -2 || i > G.ni + 2 || j < -2 || j > G.nj + 2 || k < -2 || k > G.nk + 2) continue;
          const long v = G.at(i, j, k);
          acc += 0.25 * ((a ? dxi : -dxi) * lqx[v] + (b ? dyi : -dyi) * lqy[v] + (c ? dzi : -dzi) * lqz[v]);
        }
    lq[G.at(x, y, z)] += acc;
  });
}

void grad_prs_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lqx,
                const double* lqy, const double* lqz, double* lq) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    auto in = [&](int a, int b, int c) {
      return a >= -2 && a <= G.ni + 2 && b >= -2 && b <= G.nj + 2 && c >= -2 && c <= G.nk + 2;
    };
    double acc = 0.0;
    if (in(i, j, k)) {
      const long c = G.at(i, j, k);
      acc -= dxi * lqx[c] + dyi * lqy[c] + dzi * lqz[c];
    }
    if (in(i - 1, j, k)) acc += dxi * lqx[G.at(i - 1, j, k)];
    if (in(i, j - 1, k)) acc += dyi * lqy[G.at(i, j - 1, k)];
    if (in(i, j, k - 1)) acc += dzi * lqz[G.at(i, j, k - 1)];
    lq[G.at(i, j, k)] += acc;
  });
}

void mean_T(cudaStream_t s, const Grid& g, double ql, double qg, const double* lq, double* lphi) {
  const double f = qg - ql;
  flat(s, g.n, [=] __device__(long t) { lphi[t] += f * lq[t]; });
}

void caldiv_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, const double* ldiv,
              double* lu, double* lv, double* lw) {
  const Grid G = g;
  const double f = 1.0 / dt;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    auto D = [&](int a, int b, int c) {
      return (a >= -1 && b >= -1 && c >= -1 && a <= G.ni + 3 && b <= G.nj + 3 && c <= G.nk + 3)
                 ? ldiv[G.at(a, b, c)] * f
                 : 0.0;
    };
    const long c = G.at(i, j, k);
    const double d0 = D(i, j, k);
    lu[c] += dxi * (d0 - D(i + 1, j, k));
    lv[c] += dyi * (d0 - D(i, j + 1, k));
    lw[c] += dzi * (d0 - D(i, j, k + 1));
  });
}

void corunp_T(cudaStream_t s, const Grid& g, double rho, double dxi, double dyi, double dzi, double dt,
              const double* lun, const double* lvn, const double* lwn, const double* lpn, double* ldp,
              double* lphat) {
  const Grid G = g;
  const double f = dt / rho;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    auto in = [&](int a, int b, int c) { return a >= 1 && a <= G.ni && b >= 1 && b <= G.nj && c >= 1 && c <= G.nk; };
    auto inv_ = [&](int a, int b, int c) { return in(a, b, c) && b <= G.nj - 1; };
    const long c = G.at(i, j, k);
    double acc = 0.0;  // velocity corrections that read dp(c)
    if (in(i, j, k)) acc += dxi * lun[c] + dzi * lwn[c];
    if (inv_(i, j, k)) acc += dyi * lvn[c];
    if (in(i - 1, j, k)) acc -= dxi * lun[c - 1];
    if (inv_(i, j - 1, k)) acc -= dyi * lvn[c - G.sy];
    if (in(i, j, k - 1)) acc -= dzi * lwn[c - G.sz];
    const double lp = in(i, j, k) ? lpn[c] : 0.0;  // pn = phat + dp
    ldp[c] += f * acc + lp;
    lphat[c] += lp;
  });
}

void calsij_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lsk, double* lu,
              double* lv, double* lw) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    double L;
    if (i >= -1 && (L = lsk[c]) != 0.0) {
      aadd(lu + c, dxi * L);
      aadd(lu + c - X, -dxi * L);
    }
    if (j >= -1 && (L = lsk[c + n]) != 0.0) {
      aadd(lv + c, dyi * L);
      aadd(lv + c - Y, -dyi * L);
    }
    if (i >= -1 && j >= -1 && k >= -1 && (L = lsk[c + 2 * n]) != 0.0) {
      aadd(lw + c, dzi * L);
      aadd(lw + c - Z, -dzi * L);
    }
    if (j <= G.nj + 2 && i <= G.ni + 2 && (L = 0.5 * lsk[c + 3 * n]) != 0.0) {
      aadd(lu + c + Y, dyi * L);
      aadd(lu + c, -dyi * L);
      aadd(lv + c + X, dxi * L);
      aadd(lv + c, -dxi * L);
    }
    if (k <= G.nk + 2 && i <= G.ni + 2 && (L = 0.5 * lsk[c + 4 * n]) != 0.0) {
      aadd(lu + c + Z, dzi * L);
      aadd(lu + c, -dzi * L);
      aadd(lw + c + X, dxi * L);
      aadd(lw + c, -dxi * L);
    }
    if (k <= G.nk + 2 && j <= G.nj + 2 && (L = 0.5 * lsk[c + 5 * n]) != 0.0) {
      aadd(lv + c + Z, dzi * L);
      aadd(lv + c, -dzi * L);
      aadd(lw + c + Y, dyi * L);
      aadd(lw + c, -dyi * L);
    }
  });
}

// arithmetic edge means only (the step's cal_arith_tau)
void tau_T(cudaStream_t s, const Grid& g, const double* sk, const double* mu, const double* ltau, double* lsk,
           double* lmu) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    double lm = 0.0;
    for (int l = 0; l < 3; ++l) {
      const double L = ltau[c + l * n];
      lsk[c + l * n] += L * mu[c] * 2.0;
      lm += L * sk[c + l * n] * 2.0;
    }
    aadd(lmu + c, lm);
    auto edge = [&](int l, long a, long b, long d, long e) {
      const double L = ltau[c + l * n];
      if (L == 0.0) return;
      const double m4 = 0.25 * mu[a] + 0.25 * mu[b] + 0.25 * mu[d] + 0.25 * mu[e];
      lsk[c + l * n] += L * m4 * 2.0;
      const double lm4 = L * sk[c + l * n] * 2.0 * 0.25;
      aadd(lmu + a, lm4);
      aadd(lmu + b, lm4);
      aadd(lmu + d, lm4);
      aadd(lmu + e, lm4);
    };
    if (j <= G.nj + 2 && i <= G.ni + 2) edge(3, c, c + X, c + Y, c + X + Y);
    if (k <= G.nk + 2 && i <= G.ni + 2) edge(4, c, c + X, c + Z, c + X + Z);
    if (k <= G.nk + 2 && j <= G.nj + 2) edge(5, c, c + Y, c + Z, c + Y + Z);
  });
}

void div_tensor_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* lvu,
                  const double* lvv, const double* lvw, double* lt) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    double* t1 = lt;
    double* t2 = lt + n;
    double* t3 = lt + 2 * n;
    double* t4 = lt + 3 * n;
    double* t5 = lt + 4 * n;
    double* t6 = lt + 5 * n;
    double L;
    if (k >= -1 && j >= -1 && i <= G.ni + 2 && (L = lvu[c]) != 0.0) {
      aadd(t1 + c + X, dxi * L);
      aadd(t1 + c, -dxi * L);
      aadd(t4 + c, dyi * L);
      aadd(t4 + c - Y, -dyi * L);
      aadd(t5 + c, dzi * L);
      aadd(t5 + c - Z, -dzi * L);
    }
    if (k >= -1 && j <= G.nj + 2 && i >= -1 && (L = lvv[c]) != 0.0) {
      aadd(t4 + c, dxi * L);
      aadd(t4 + c - X, -dxi * L);
      aadd(t2 + c + Y, dyi * L);
      aadd(t2 + c, -dyi * L);
      aadd(t6 + c, dzi * L);
      aadd(t6 + c - Z, -dzi * L);
    }
    if (k <= G.nk + 2 && j >= -1 && i >= -1 && (L = lvw[c]) != 0.0) {
      aadd(t5 + c, dxi * L);
      aadd(t5 + c - X, -dxi * L);
      aadd(t6 + c, dyi * L);
      aadd(t6 + c - Y, -dyi * L);
      aadd(t3 + c + Z, dzi * L);
      aadd(t3 + c, -dzi * L);
    }
  });
}

}  // namespace adj
}  // namespace fmf
