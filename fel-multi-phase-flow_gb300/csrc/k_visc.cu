// k_visc.cu -- C3: viscous coefficients and the 8-colour Gauss-Seidel sweep
// (drop-in kernels, coefficients read from the 45 arrays).
#include "ops.cuh"

namespace fmf {
namespace op {

namespace {
struct P45 {
  double* c[45];
};
}  // namespace

// cal_arith_coef_vis.f:82-408 / cal_harm_coef_vis.f (harmonic 4-point edge means).
// coef[] in the reference argument order au_w_u ... av_tn_w.
void cal_coef_vis(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                  const double* rmu, double* const* coef, bool harmonic) {
  P45 cp;
  for (int t = 0; t < 45; ++t) cp.c[t] = coef[t];
  const Grid G = g;
  const bool hm = harmonic;
  flat(s, g.n, [=] __device__(long t) {
#pragma unroll
    for (int q = 0; q < 45; ++q) cp.c[q][t] = 0.0;
  });
  const double dx2 = dxinv * dxinv, dy2 = dyinv * dyinv, dz2 = dzinv * dzinv;
  const double dxy = dxinv * dyinv, dxz = dxinv * dzinv, dyz = dyinv * dzinv;
  range3(s, -1, g.ni + 2, -1, g.nj + 2, -1, g.nk + 2, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long t = G.at(i, j, k);
    const double* r = rmu;
    auto m4 = [&](long a, long b, long c, long d) {
      if (!hm) return 0.25 * (r[a] + r[b] + r[c] + r[d]);
      return 4.0 / (1.0 / r[a] + 1.0 / r[b] + 1.0 / r[c] + 1.0 / r[d]);
    };
    double* const* C = cp.c;
    {
      const double xm = r[t], xp = r[t + X];
      const double ym = m4(t - Y, t + X - Y, t, t + X), yp = m4(t, t + X, t + Y, t + X + Y);
      const double zm = m4(t - Z, t + X - Z, t, t + X), zp = m4(t, t + X, t + Z, t + X + Z);
      const double b = dz2 * zm, sn = dy2 * ym, w = dx2 * xm * 2.0, e = dx2 * xp * 2.0, nn = dy2 * yp, tt = dz2 * zp;
      C[0][t] = w; C[1][t] = e; C[2][t] = sn; C[3][t] = nn; C[4][t] = b; C[5][t] = tt;
      C[6][t] = b + sn + w + e + nn + tt;
      C[7][t] = dxy * ym; C[8][t] = -(dxy * ym); C[9][t] = -(dxy * yp); C[10][t] = dxy * yp;
      C[11][t] = dxz * zm; C[12][t] = -(dxz * zm); C[13][t] = -(dxz * zp); C[14][t] = dxz * zp;
    }
    {
      const double xm = m4(t - X, t, t - X + Y, t + Y), xp = m4(t, t + X, t + Y, t + X + Y);
      const double ym = r[t], yp = r[t + Y];
      const double zm = m4(t - Z, t + Y - Z, t, t + Y), zp = m4(t, t + Y, t + Z, t + Y + Z);
      const double b = dz2 * zm, sn = dy2 * ym * 2.0, w = dx2 * xm, e = dx2 * xp, nn = dy2 * yp * 2.0, tt = dz2 * zp;
      C[15][t] = w; C[16][t] = e; C[17][t] = sn; C[18][t] = nn; C[19][t] = b; C[20][t] = tt;
      C[21][t] = b + sn + w + e + nn + tt;
      C[22][t] = dxy * xm; C[23][t] = -(dxy * xm); C[24][t] = -(dxy * xp); C[25][t] = dxy * xp;
      C[26][t] = dyz * zm; C[27][t] = -(dyz * zm); C[28][t] = -(dyz * zp); C[29][t] = dyz * zp;
    }
    {
      const double xm = m4(t - X, t, t - X + Z, t + Z), xp = m4(t, t + X, t + Z, t + X + Z);
      const double ym = m4(t - Y, t, t - Y + Z, t + Z), yp = m4(t, t + Y, t + Z, t + Y + Z);
      const double zm = r[t], zp = r[t + Z];
      const double b = dz2 * zm * 2.0, sn = dy2 * ym, w = dx2 * xm, e = dx2 * xp, nn = dy2 * yp, tt = dz2 * zp * 2.0;
      C[30][t] = w; C[31][t] = e; C[32][t] = sn; C[33][t] = nn; C[34][t] = b; C[35][t] = tt;
      C[36][t] = b + sn + w + e + nn + tt;
      C[37][t] = dxz * xm; C[38][t] = -(dxz * xm); C[39][t] = -(dxz * xp); C[40][t] = dxz * xp;
      C[41][t] = dyz * ym; C[42][t] = -(dyz * ym); C[43][t] = -(dyz * yp); C[44][t] = dyz * yp;
    }
  });
}

namespace {
struct Coef15 {
  const double* c[15];
};

// One colour of one component (solu_sor4.f:134-175 / :184-225 / :234-275).
// comp 0: u, 1: v, 2: w.  Each block writes the partial sum of du^2 of its points.
template <int COMP>
__global__ void __launch_bounds__(256) k_sor_colour(Grid g, int is, int js, int ks, int jmax, double dtinv,
                                                    const double* __restrict__ rho,
                                                    const double* __restrict__ rhon, Coef15 cf,
                                                    const double* __restrict__ src, double* un, double* vn,
                                                    double* wn, double* part) {
  __shared__ double sh[256];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int i = is + 2 * (int)(blockIdx.x * 32 + threadIdx.x);
  const int j = js + 2 * (int)(blockIdx.y * 8 + threadIdx.y);
  const int k = ks + 2 * (int)blockIdx.z;
  double e = 0.0;
  if (i <= g.ni && j <= jmax) {
    const long X = 1, Y = g.sy, Z = g.sz;
    const long t = g.at(i, j, k);
    const long so = COMP == 0 ? X : (COMP == 1 ? Y : Z);
    const double r = (rho[t] + rho[t + so] + rhon[t] + rhon[t + so]) * 0.25;
    const double* const* c = cf.c;
    double visn, q;
    if (COMP == 0) {
      visn = (c[4][t] * un[t - Z] + c[2][t] * un[t - Y] + c[0][t] * un[t - X] + c[1][t] * un[t + X] +
              c[3][t] * un[t + Y] + c[5][t] * un[t + Z] + c[7][t] * vn[t - Y] + c[8][t] * vn[t + X - Y] +
              c[9][t] * vn[t] + c[10][t] * vn[t + X] + c[11][t] * wn[t - Z] + c[12][t] * wn[t + X - Z] +
              c[13][t] * wn[t] + c[14][t] * wn[t + X]) / r;
      q = un[t];
    } else if (COMP == 1) {
      visn = (c[4][t] * vn[t - Z] + c[2][t] * vn[t - Y] + c[0][t] * vn[t - X] + c[1][t] * vn[t + X] +
              c[3][t] * vn[t + Y] + c[5][t] * vn[t + Z] + c[7][t] * un[t - X] + c[9][t] * un[t] +
              c[8][t] * un[t - X + Y] + c[10][t] * un[t + Y] + c[11][t] * wn[t - Z] + c[12][t] * wn[t + Y - Z] +
              c[13][t] * wn[t] + c[14][t] * wn[t + Y]) / r;
      q = vn[t];
    } else {
      visn = (c[4][t] * wn[t - Z] + c[2][t] * wn[t - Y] + c[0][t] * wn[t - X] + c[1][t] * wn[t + X] +
              c[3][t] * wn[t + Y] + c[5][t] * wn[t + Z] + c[7][t] * un[t - X] + c[9][t] * un[t] +
              c[8][t] * un[t - X + Z] + c[10][t] * un[t + Z] + c[11][t] * vn[t - Y] + c[13][t] * vn[t] +
              c[12][t] * vn[t - Y + Z] + c[14][t] * vn[t + Z]) / r;
      q = wn[t];
    }
    const double d = (visn * 0.5 + src[t]) / (dtinv + c[6][t] / r * 0.5) - q;
    const double qn = q + d;
    if (COMP == 0) un[t] = qn;
    else if (COMP == 1) vn[t] = qn;
    else wn[t] = qn;
    e = d * d;
  }
  sh[tid] = e;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (tid < st) sh[tid] += sh[tid + st];
    __syncthreads();
  }
  if (tid == 0) part[((long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void k_sum_parts(const double* part, long n, double* out) {
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

// solu_sor4.f:133-281 -- one outer iteration; errsum[0] = sum of du^2 over the 24 sweeps.
void sor_iteration(cudaStream_t s, const Grid& g, double dt, const double* rho, const double* rhon,
                   const double* const* coef, const double* const* src, double* un, double* vn, double* wn,
                   double uwall, double dy, const double* l1, const double* l2, const double* phi,
                   double* errsum) {
  static const int isor[8] = {1, 2, 1, 2, 1, 2, 2, 1};
  static const int jsor[8] = {1, 2, 1, 2, 2, 1, 1, 2};
  static const int ksor[8] = {1, 2, 2, 1, 1, 2, 1, 2};
  const double dtinv = 1.0 / dt;
  const dim3 blk(32, 8, 1);
  const dim3 grd((unsigned)((g.ni / 2 + 31) / 32), (unsigned)((g.nj / 2 + 7) / 8), (unsigned)((g.nk + 1) / 2));
  const long nb = (long)grd.x * grd.y * grd.z;
  double* part = (double*)scratch(sizeof(double) * nb * 24, 6);
  for (int comp = 0; comp < 3; ++comp) {
    Coef15 cf;
    for (int q = 0; q < 15; ++q) cf.c[q] = coef[15 * comp + q];
    const int jmax = comp == 1 ? g.nj - 1 : g.nj;
    for (int col = 0; col < 8; ++col) {
      double* pp = part + (long)(comp * 8 + col) * nb;
      if (comp == 0)
        k_sor_colour<0><<<grd, blk, 0, s>>>(g, isor[col], jsor[col], ksor[col], jmax, dtinv, rho, rhon, cf, src[0], un, vn, wn, pp);
      else if (comp == 1)
        k_sor_colour<1><<<grd, blk, 0, s>>>(g, isor[col], jsor[col], ksor[col], jmax, dtinv, rho, rhon, cf, src[1], un, vn, wn, pp);
      else
        k_sor_colour<2><<<grd, blk, 0, s>>>(g, isor[col], jsor[col], ksor[col], jmax, dtinv, rho, rhon, cf, src[2], un, vn, wn, pp);
      count_launch();
      if (col % 2 == 1) {
        bndu(s, g, un, vn, wn, uwall, dy, l1, l2, phi);
        bnd_periodic(s, g, comp == 0 ? un : (comp == 1 ? vn : wn));
      }
    }
  }
  k_sum_parts<<<1, 256, 0, s>>>(part, nb * 24, errsum);
  count_launch();
}

}  // namespace op
}  // namespace fmf
