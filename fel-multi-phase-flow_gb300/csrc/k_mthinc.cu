// k_mthinc.cu -- C1: MTHINC volume-fraction transport (drop-in kernels).
//
// Arithmetic follows the reference operation by operation (this file is compiled
// with -fmad=false so no multiply-add is fused), so results differ from the host
// original only through the device exp/cosh/tanh.
#include "recip.cuh"
#include "ops.cuh"

namespace fmf {
namespace op {

// cal_grad_p2a.f:30-71 -- vertex gradient over -2..n+2 (uniform dy: dyinv_array is
// 1/dy at every index, main.f90:215-224).
void cal_grad_p2a(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                  const double* q, double* qx, double* qy, double* qz) {
  const Grid G = g;
  range3(s, -2, g.ni + 2, -2, g.nj + 2, -2, g.nk + 2, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    const long X = 1, Y = G.sy, Z = G.sz;
    const double q000 = q[c], qp00 = q[c + X], q0p0 = q[c + Y], qpp0 = q[c + X + Y], q00p = q[c + Z],
                 qp0p = q[c + X + Z], q0pp = q[c + Y + Z], qppp = q[c + X + Y + Z];
    const double gx = -q000 + qp00 - q0p0 + qpp0 - q00p + qp0p - q0pp + qppp;
    const double gy = -q000 - qp00 + q0p0 + qpp0 - q00p - qp0p + q0pp + qppp;
    const double gz = -q000 - qp00 - q0p0 - qpp0 + q00p + qp0p + q0pp + qppp;
    qx[c] = gx * 0.25 * dxinv;
    qy[c] = gy * 0.25 * dyinv;
    qz[c] = gz * 0.25 * dzinv;
  });
}

namespace {
struct GP8 {
  double a[8];  // x111 x211 x121 x221 x112 x212 x122 x222
};
// mthinc_x.h:1-14
__device__ __forceinline__ GP8 gauss_x(double rnx, double rny, double rnz, double xg1, double xg2,
                                       double yg1, double yg2, double zg1, double zg2) {
  const double x1 = rnx * xg1, x2 = rnx * xg2, y1 = rny * yg1, y2 = rny * yg2, z1 = rnz * zg1,
               z2 = rnz * zg2;
  GP8 g;
  g.a[0] = x1 + y1 + z1;
  g.a[1] = x2 + y1 + z1;
  g.a[2] = x1 + y2 + z1;
  g.a[3] = x2 + y2 + z1;
  g.a[4] = x1 + y1 + z2;
  g.a[5] = x2 + y1 + z2;
  g.a[6] = x1 + y2 + z2;
  g.a[7] = x2 + y2 + z2;
  return g;
}
// mthinc_tanh.h:1-9
__device__ __forceinline__ double sig8(const GP8& g, double wght, double bet, double ddd) {
  const double m = -2.0 * bet;
  double s = wght / (1.0 + exp(m * (g.a[0] + ddd)));
#pragma unroll
  for (int t = 1; t < 8; ++t) s = s + wght / (1.0 + exp(m * (g.a[t] + ddd)));
  return s;
}
__device__ __forceinline__ double avg8(const double* p, long c, long X, long Y, long Z) {
  // (i-1,j-1,k-1) (i,j-1,k-1) (i-1,j,k-1) (i,j,k-1) (i-1,j-1,k) (i,j-1,k) (i-1,j,k) (i,j,k)
  return (p[c - X - Y - Z] + p[c - Y - Z] + p[c - X - Z] + p[c - Z] + p[c - X - Y] + p[c - Y] + p[c - X] +
          p[c]) *
         0.125;
}
struct MthincConst {
  double gp1, gp2, dcellinv, eps_mthinc, eps_trunc;
};
MthincConst mthinc_const(double dxinv, double dyinv, double dzinv, double bet) {
  MthincConst m;
  const double dx = 1.0 / dxinv, dy = 1.0 / dyinv, dz = 1.0 / dzinv;
  m.gp1 = -0.5 / std::sqrt(3.0);
  m.gp2 = 0.5 / std::sqrt(3.0);
  m.dcellinv = 1.0 / std::sqrt((dx * dx + dy * dy + dz * dz) / 3.0);
  const double ch = std::cosh(-bet * 1.5);
  m.eps_mthinc = bet / (2.0 * (ch * ch));
  m.eps_trunc = 0.5 * (std::tanh(-bet * 2.5) + 1.0);
  return m;
}
}  // namespace

// solphi_mthinc1.f:115-366
void solphi_mthinc1(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt,
                    double bet, const double* phi, const double* phix, const double* phiy,
                    const double* phiz, const double* u, const double* v, const double* w, double* flx,
                    double* fly, double* flz) {
  const Grid G = g;
  range3(s, -1, g.ni + 1, -1, g.nj + 1, -1, g.nk + 1, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    flx[c] = 0.0;
    fly[c] = 0.0;
    flz[c] = 0.0;
  });
  const MthincConst M = mthinc_const(dxinv, dyinv, dzinv, bet);
  range3(s, 0, g.ni + 1, 0, g.nj + 1, 0, g.nk + 1, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    double rnx = avg8(phix, c, X, Y, Z), rny = avg8(phiy, c, X, Y, Z), rnz = avg8(phiz, c, X, Y, Z);
    const double q00 = sqrt(rnx * rnx + rny * rny + rnz * rnz);
    const double uw = u[c - X], ue = u[c], vs = v[c - Y], vn = v[c], wb = w[c - Z], wt = w[c];
    if (q00 <= M.eps_mthinc * M.dcellinv) {
      double phi00 = phi[c];
      if (phi00 <= M.eps_trunc) phi00 = 0.0;
      if (1.0 - phi00 <= M.eps_trunc) phi00 = 1.0;
      if (uw <= 0.0) flx[c - X] = uw * phi00 * dt * dxinv;
      if (ue >= 0.0) flx[c] = ue * phi00 * dt * dxinv;
      if (vs <= 0.0) fly[c - Y] = vs * phi00 * dt * dyinv;
      if (vn >= 0.0) fly[c] = vn * phi00 * dt * dyinv;
      if (wb <= 0.0) flz[c - Z] = wb * phi00 * dt * dzinv;
      if (wt >= 0.0) flz[c] = wt * phi00 * dt * dzinv;
      return;
    }
    const double coef = 1.0 / q00;
    rnx = rnx * coef;
    rny = rny * coef;
    rnz = rnz * coef;
    const double gp1 = M.gp1, gp2 = M.gp2;
    const GP8 gg = gauss_x(rnx, rny, rnz, gp1, gp2, gp1, gp2, gp1, gp2);
    const double ph = phi[c];
    double ddd = 0.0;
    for (int inr = 0; inr < 10; ++inr) {
      const double f = sig8(gg, 0.125, bet, ddd) - ph;
      double acc = 0.0;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const double ch = cosh(bet * (gg.a[t] + ddd));
        acc = acc + 0.125 / (ch * ch);
      }
      const double df = 0.5 * bet * acc;
      ddd = ddd - f * df / (df * df + 1.0e-99);
    }
    if (uw < 0.0) {
      const double vd = uw * dt * dxinv, st = -0.5, en = -0.5 - vd;
      const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
      flx[c - X] = sig8(gauss_x(rnx, rny, rnz, a1, a2, gp1, gp2, gp1, gp2), 0.125 * vd, bet, ddd);
    }
    if (ue > 0.0) {
      const double vd = ue * dt * dxinv, st = 0.5 - vd, en = 0.5;
      const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
      flx[c] = sig8(gauss_x(rnx, rny, rnz, a1, a2, gp1, gp2, gp1, gp2), 0.125 * vd, bet, ddd);
    }
    if (vs < 0.0) {
      const double vd = vs * dt * dyinv, st = -0.5, en = -0.5 - vd;
      const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
      fly[c - Y] = sig8(gauss_x(rnx, rny, rnz, gp1, gp2, a1, a2, gp1, gp2), 0.125 * vd, bet, ddd);
    }
    if (vn > 0.0) {
      const double vd = vn * dt * dyinv, st = 0.5 - vd, en = 0.5;
      const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
      fly[c] = sig8(gauss_x(rnx, rny, rnz, gp1, gp2, a1, a2, gp1, gp2), 0.125 * vd, bet, ddd);
    }
    if (wb < 0.0) {
      const double vd = wb * dt * dzinv, st = -0.5, en = -0.5 - vd;
      const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
      flz[c - Z] = sig8(gauss_x(rnx, rny, rnz, gp1, gp2, gp1, gp2, a1, a2), 0.125 * vd, bet, ddd);
    }
    if (wt > 0.0) {
      const double vd = wt * dt * dzinv, st = 0.5 - vd, en = 0.5;
      const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
      flz[c] = sig8(gauss_x(rnx, rny, rnz, gp1, gp2, gp1, gp2, a1, a2), 0.125 * vd, bet, ddd);
    }
  });
}

// solphi_mthinc2.f:19-45
void solphi_mthinc2(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt,
                    const double* u, const double* v, const double* w, const double* flx,
                    const double* fly, const double* flz, const double* phi, double* phin) {
  const Grid G = g;
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    const double div00 = (-u[c - X] + u[c]) * dxinv + (-v[c - Y] + v[c]) * dyinv + (-w[c - Z] + w[c]) * dzinv;
    double p = phi[c] * (1.0 + dt * div00) + flx[c - X] - flx[c] + fly[c - Y] - fly[c] + flz[c - Z] - flz[c];
    p = fmin(p, 1.0);
    phin[c] = fmax(p, 0.0);
  });
}

// solphi_mthinc3.f:84-209
namespace {
// solphi_mthinc3.f:138-160: phin += offset phin^2 (1 - phin), clipped, over the
// interior; the offset (sums[2] >= 0: the Newton-Raphson reciprocal, no division)
// formed once per block
__global__ void __launch_bounds__(256) k_mthinc3_offset(Grid g, const double* __restrict__ sums,
                                                        double* __restrict__ phin) {
  __shared__ double off;
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  const bool in = i <= g.ni && j <= g.nj;
  const long c = in ? g.at(i, j, k) : 0;
  double p = in ? phin[c] : 0.0;  // in flight while the offset is formed
  if (threadIdx.x == 0 && threadIdx.y == 0) off = (sums[0] - sums[1]) * recip_nr(sums[2] + 1.0e-99);
  __syncthreads();
  if (!in) return;
  const double offset = off;
  p = p + offset * (p * p) * (1.0 - p);
  p = fmin(p, 1.0);
  phin[c] = fmax(p, 0.0);
}
}  // namespace

void solphi_mthinc3(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double bet,
                    const double* phix, const double* phiy, const double* phiz, const double* phi,
                    double* phin, double* sums) {
  const Grid G = g;
  const MthincConst M = mthinc_const(dxinv, dyinv, dzinv, bet);
  // the band test sqrt(q2) <= lim decided on q2 against lim^2 where q2 is clearly on
  // one side, with the square root only within 1e-12 of it
  const double lim = M.eps_mthinc * M.dcellinv;
  const double lim2lo = lim * lim * (1.0 - 1.0e-12), lim2hi = lim * lim * (1.0 + 1.0e-12);
  // the snap of :61-112 over 0..n+1, and on the interior the clip of :113-120 of
  // the snapped value (the two passes of the reference touch each point alone)
  range3(s, 0, g.ni + 1, 0, g.nj + 1, 0, g.nk + 1, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    const double rnx = avg8(phix, c, X, Y, Z), rny = avg8(phiy, c, X, Y, Z), rnz = avg8(phiz, c, X, Y, Z);
    const double q2 = rnx * rnx + rny * rny + rnz * rnz;
    const bool outside = q2 < lim2lo ? true : (q2 > lim2hi ? false : sqrt(q2) <= lim);
    const bool interior = i >= 1 && i <= G.ni && j >= 1 && j <= G.nj && k >= 1 && k <= G.nk;
    if (outside || interior) {
      double p = phin[c];
      if (outside) {
        if (p <= M.eps_trunc) p = 0.0;
        if (1.0 - p <= M.eps_trunc) p = 1.0;
      }
      if (interior) p = fmax(fmin(p, 1.0), 0.0);
      phin[c] = p;
    }
  });
  reduce_interior<3>(
      s, g,
      [=] __device__(int i, int j, int k, double* r) {
        const long c = G.at(i, j, k);
        const double p = phin[c];
        r[0] = phi[c];
        r[1] = p;
        r[2] = p * p * (1.0 - p);
      },
      sums);
  k_mthinc3_offset<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), dim3(32, 8), 0, s>>>(g, sums, phin);
  count_launch();
}

// summation.f:222-264 (nbub=1): q0 = q1 over the whole array, then clip the interior.
void summation(cudaStream_t s, const Grid& g, double* q0, const double* q1) {
  const Grid G = g;
  flat(s, g.n, [=] __device__(long t) { q0[t] = q1[t]; });
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    q0[c] = fmin(fmax(q0[c], 0.0), 1.0);
  });
}

}  // namespace op
}  // namespace fmf
