// fused_mthinc.cu -- MTHINC fluxes (solphi_mthinc1.f) for the fused step.
//
// Two kernels instead of one thread per cell on the full 0..n+1 range:
//   k_classify: every cell forms its normal from the 8 vertex gradients; cells
//     outside the interface band write their truncated upwind fluxes at once,
//     band cells are appended to a compact list;
//   k_band: one thread per band cell (list entry) runs the 10 Newton steps and
//     writes the swept-volume fluxes.
// A warp then carries band cells only, instead of idling on the bulk cells that
// share its x-run.  The sigmoid derivative uses 1/cosh^2(a) = 4 s (1 - s) with
// s = 1/(1 + exp(-2a)) (same function, one exp per Gauss point).
//
// Face ownership: a face is written by its donor cell (u>0: the west cell, u<0:
// the east cell) or left zero; cells write their east/north/top face when u>=0
// and their west/south/bottom face when u<0, so every face in 0..n of every
// interior row gets exactly one writer (solphi_mthinc1.f:121-130 zeroes first;
// faces nobody donates through hold the zero written by k_classify's owner).
#include "fused.cuh"
#include "recip.cuh"

namespace fmf {
namespace fused {

namespace {
struct MC {
  double gp1, gp2, lim, eps_trunc, bet, dt, dxi, dyi, dzi;
  double lim2lo, lim2hi;  // lim^2 (1 -/+ 1e-12)
  double dtdx, dtdy, dtdz;  // dt dxinv etc.
};

__device__ __forceinline__ double avg8(const double* __restrict__ p, long c, long X, long Y, long Z) {
  return (__ldg(p + c - X - Y - Z) + __ldg(p + c - Y - Z) + __ldg(p + c - X - Z) + __ldg(p + c - Z) +
          __ldg(p + c - X - Y) + __ldg(p + c - Y) + __ldg(p + c - X) + __ldg(p + c)) *
         0.125;
}

__device__ __forceinline__ double ex(double x) { return exp(x); }
__device__ __forceinline__ float ex(float x) { return expf(fminf(x, 80.0f)); }

// 1/(1+e) for e >= 0: the division-free reciprocal in double (an overflowed e gives
// exactly 0, as the quotient does; NaN stays NaN), the quotient in float
__device__ __forceinline__ double inv1p(double e) {
  const double a = 1.0 + e;
  return (__double2hiint(a) == 0x7ff00000 && __double2loint(a) == 0) ? 0.0 : recip_nr(a);
}
__device__ __forceinline__ float inv1p(float e) { return 1.0f / (1.0f + e); }

// The sum over the 8 Gauss points t of w/(1+exp(m2b (a_t + d))) (m2b = -2 bet) and,
// optionally, the sum of s(1-s) (1-s = e/(1+e), exact in relative terms for any
// a_t), with exp(m2b (a_t + d)) factorised: a_t = x + y + z over the Gauss
// offsets of the three axes, so exp(m2b a_t) = X Y Z of per-axis factors (E_t,
// gexp8) and only exp(m2b d) changes with d.  Every factor is bounded by the
// normal's unit length times the Gauss offsets; where exp(m2b d) overflows or
// underflows, so does the unfactorised exponential.  Six exponentials per cell
// and one per Newton step instead of eight per step.
template <class R>
__device__ __forceinline__ R sig8f(const R* E, R w, R ed, R* sd) {
  R s = 0, q = 0;
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const R e = E[t] * ed;
    const R r = inv1p(e);
    s += r;
    if (sd) q += e * r * r;
  }
  if (sd) *sd = q;
  return w * s;
}
// E_t over the 8 Gauss points, x fastest, then y, then z: factors X1 X2, Y1 Y2, Z1 Z2
template <class R>
__device__ __forceinline__ void gexp8(R* E, R X1, R X2, R Y1, R Y2, R Z1, R Z2) {
  const R a = X1 * Y1, b = X2 * Y1, c = X1 * Y2, d = X2 * Y2;
  E[0] = a * Z1;
  E[1] = b * Z1;
  E[2] = c * Z1;
  E[3] = d * Z1;
  E[4] = a * Z2;
  E[5] = b * Z2;
  E[6] = c * Z2;
  E[7] = d * Z2;
}
__global__ void __launch_bounds__(256) k_classify(Grid g, MC m, const double* __restrict__ phi,
                                                  const double* __restrict__ gx, const double* __restrict__ gy,
                                                  const double* __restrict__ gz, const double* __restrict__ u,
                                                  const double* __restrict__ v, const double* __restrict__ w,
                                                  double* __restrict__ fx, double* __restrict__ fy,
                                                  double* __restrict__ fz, int* __restrict__ list,
                                                  int* __restrict__ count) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = (int)blockIdx.z;
  if (i > g.ni + 1 || j > g.nj + 1) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double rnx = avg8(gx, c, X, Y, Z), rny = avg8(gy, c, X, Y, Z), rnz = avg8(gz, c, X, Y, Z);
  const double q2 = rnx * rnx + rny * rny + rnz * rnz;
  const double uw = __ldg(u + c - X), ue = __ldg(u + c), vs = __ldg(v + c - Y), vn = __ldg(v + c),
               wb = __ldg(w + c - Z), wt = __ldg(w + c);
  // the band test sqrt(q2) <= lim of the reference: decided on q2 against lim^2
  // where q2 is clearly on one side (compared as bit patterns: all three are
  // non-negative), with the square root only within 1e-12 of it
  const long long qb = __double_as_longlong(q2);
  const bool band = qb < __double_as_longlong(m.lim2lo)
                        ? false
                        : (qb > __double_as_longlong(m.lim2hi) ? true : !(sqrt(q2) <= m.lim));
  if (band) {
    const int slot = atomicAdd(count, 1);
    list[slot] = (int)c;
  }
  double phi00 = 0.0;
  if (!band) {
    phi00 = __ldg(phi + c);
    if (phi00 <= m.eps_trunc) phi00 = 0.0;
    if (1.0 - phi00 <= m.eps_trunc) phi00 = 1.0;
  }
  // owned faces: east/north/top when the velocity there is >= 0 (this cell donates or
  // the flux is zero), west/south/bottom when < 0; band cells leave the donated
  // faces to k_band but still zero the owned faces they do not donate through.
  // Signs are read from the bits: nonneg(v) is v >= 0 (so true for -0 as well; it
  // differs from the comparison only for NaN).  Fluxes are v phi dt/dx with dt/dx
  // formed once.
  auto nonneg = [](double v) { return __double_as_longlong(v) >= 0 || (__double_as_longlong(v) << 1) == 0; };
  const double pdx = phi00 * m.dtdx, pdy = phi00 * m.dtdy, pdz = phi00 * m.dtdz;
  const bool e_ = nonneg(ue), w_ = nonneg(uw), n_ = nonneg(vn), s_ = nonneg(vs), t_ = nonneg(wt), b_ = nonneg(wb);
  if (e_) fx[c] = band ? 0.0 : ue * pdx;
  if (!w_) fx[c - X] = band ? 0.0 : uw * pdx;
  if (n_) fy[c] = band ? 0.0 : vn * pdy;
  if (!s_) fy[c - Y] = band ? 0.0 : vs * pdy;
  if (t_) fz[c] = band ? 0.0 : wt * pdz;
  if (!b_) fz[c - Z] = band ? 0.0 : wb * pdz;
  // west/south/bottom faces of the first cells with no in-range donor stay zero
  if (i == 0 && w_) fx[c - X] = 0.0;
  if (j == 0 && s_) fy[c - Y] = 0.0;
  if (k == 0 && b_) fz[c - Z] = 0.0;
  if (i == g.ni + 1 && !e_) fx[c] = 0.0;
  if (j == g.nj + 1 && !n_) fy[c] = 0.0;
  if (k == g.nk + 1 && !t_) fz[c] = 0.0;
}

// R = double: the FP64 step.  R = float: the mixed-precision step (normal, band
// test and the fluxes' storage stay double; the Newton solve and the Gauss-point
// integrals run in float with the exponent argument clamped to the float range
// and the Newton regularisation 1e-99 raised to 1e-30).
template <class R>
__global__ void __launch_bounds__(128) k_band(Grid g, MC m, const double* __restrict__ phi,
                                              const double* __restrict__ gx, const double* __restrict__ gy,
                                              const double* __restrict__ gz, const double* __restrict__ u,
                                              const double* __restrict__ v, const double* __restrict__ w,
                                              double* __restrict__ fx, double* __restrict__ fy,
                                              double* __restrict__ fz, const int* __restrict__ list,
                                              const int* __restrict__ count, double* __restrict__ newton,
                                              long cap) {
  const int n = *count;
  const long X = 1, Y = g.sy, Z = g.sz;
  const R m2b = (R)(-2.0 * m.bet), gp1 = (R)m.gp1, gp2 = (R)m.gp2, bet = (R)m.bet, dtt = (R)m.dt;
  const R reg = sizeof(R) == 8 ? (R)1.0e-99 : (R)1.0e-30;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const long c = list[e];
    double nx = avg8(gx, c, X, Y, Z), ny = avg8(gy, c, X, Y, Z), nz = avg8(gz, c, X, Y, Z);
    const double q00 = sqrt(nx * nx + ny * ny + nz * nz);
    const double coef = 1.0 / q00;
    const R rnx = (R)(nx * coef), rny = (R)(ny * coef), rnz = (R)(nz * coef);
    // per-axis factors exp(m2b n gp) of the centred Gauss points
    const R X1 = ex(m2b * rnx * gp1), X2 = ex(m2b * rnx * gp2), Y1 = ex(m2b * rny * gp1),
            Y2 = ex(m2b * rny * gp2), Z1 = ex(m2b * rnz * gp1), Z2 = ex(m2b * rnz * gp2);
    R E[8];
    gexp8<R>(E, X1, X2, Y1, Y2, Z1, Z2);
    const R ph = (R)__ldg(phi + c);
    R ddd = 0, step = 0;
#pragma unroll 1
    for (int it = 0; it < 10; ++it) {
      R sd;
      const R f = sig8f<R>(E, (R)0.125, ex(m2b * ddd), &sd) - ph;
      // df = 0.5 bet sum 0.125/cosh^2 = 0.5 bet * 0.125 * 4 * sum s(1-s)
      const R df = (R)0.25 * bet * sd;
      step = sizeof(R) == 8 ? (R)((double)(f * df) * recip_nr((double)(df * df + reg))) : f * df / (df * df + reg);
      const R dn = ddd - step;
      // once d no longer changes, every remaining iteration recomputes the same
      // f, df and step: stopping here is the ten-step result bit for bit.  In
      // float the iterate can dither in its last bit instead; there a step below
      // float precision ends the loop.
      if (dn == ddd) break;
      ddd = dn;
      if (sizeof(R) == 4 && fabs((double)step) <= 1.0e-7 * (1.0 + fabs((double)ddd))) break;
    }
    if (newton) {
      newton[e] = (double)ddd;
      newton[cap + e] = (double)step;
    }
    const double uw = __ldg(u + c - X), ue = __ldg(u + c), vs = __ldg(v + c - Y), vn = __ldg(v + c),
                 wb = __ldg(w + c - Z), wt = __ldg(w + c);
    const R edf = ex(m2b * ddd);  // exp(m2b d) at the offset found
    auto side = [&](double vel, double dinv, int axis, bool minus, double* out) {
      const R vd = (R)vel * dtt * (R)dinv;
      const R st = minus ? (R)-0.5 : (R)0.5 - vd, en = minus ? (R)-0.5 - vd : (R)0.5;
      const R g1 = (st + en) * (R)0.5 + (-st + en) * gp1, g2 = (st + en) * (R)0.5 + (-st + en) * gp2;
      // the flux axis takes the swept interval's Gauss points, the others the centred ones
      R Eb[8];
      if (axis == 0) gexp8<R>(Eb, ex(m2b * rnx * g1), ex(m2b * rnx * g2), Y1, Y2, Z1, Z2);
      else if (axis == 1) gexp8<R>(Eb, X1, X2, ex(m2b * rny * g1), ex(m2b * rny * g2), Z1, Z2);
      else gexp8<R>(Eb, X1, X2, Y1, Y2, ex(m2b * rnz * g1), ex(m2b * rnz * g2));
      *out = (double)sig8f<R>(Eb, (R)0.125 * vd, edf, nullptr);
    };
    if (uw < 0.0) side(uw, m.dxi, 0, true, fx + c - X);
    if (ue > 0.0) side(ue, m.dxi, 0, false, fx + c);
    if (vs < 0.0) side(vs, m.dyi, 1, true, fy + c - Y);
    if (vn > 0.0) side(vn, m.dyi, 1, false, fy + c);
    if (wb < 0.0) side(wb, m.dzi, 2, true, fz + c - Z);
    if (wt > 0.0) side(wt, m.dzi, 2, false, fz + c);
  }
}
// cal_grad_p2a.f:46-60 for the fused step: the vertex gradient at (i+1/2, j+1/2,
// k+1/2), i, j, k in -2..n+2, from the 8 surrounding points.  Per (i, j) corner the
// sum s and difference d of the two k planes; with ta = s(+,+) - s(0,0) and
// tb = s(+,0) - s(0,+) the x sum is ta + tb, the y sum ta - tb and the z sum the
// four differences: 18 FP64 operations per point instead of the reference's 27.
__global__ void __launch_bounds__(256) k_vertex_grad(Grid g, double cx, double cy, double cz,
                                                     const double* __restrict__ q, double* __restrict__ qx,
                                                     double* __restrict__ qy, double* __restrict__ qz) {
  const int i = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = -2 + (int)blockIdx.z;
  if (i > g.ni + 2 || j > g.nj + 2) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double q000 = __ldg(q + c), qp00 = __ldg(q + c + X), q0p0 = __ldg(q + c + Y), qpp0 = __ldg(q + c + X + Y),
               q00p = __ldg(q + c + Z), qp0p = __ldg(q + c + X + Z), q0pp = __ldg(q + c + Y + Z),
               qppp = __ldg(q + c + X + Y + Z);
  const double s00 = q000 + q00p, sp0 = qp00 + qp0p, s0p = q0p0 + q0pp, spp = qpp0 + qppp;
  const double ta = spp - s00, tb = sp0 - s0p;
  qx[c] = (ta + tb) * cx;
  qy[c] = (ta - tb) * cy;
  qz[c] = ((q00p - q000) + (qp0p - qp00) + ((q0pp - q0p0) + (qppp - qpp0))) * cz;
}
}  // namespace

void vertex_gradient(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* q,
                     double* qx, double* qy, double* qz) {
  const dim3 b(32, 8, 1), gr((unsigned)((g.ni + 5 + 31) / 32), (unsigned)((g.nj + 5 + 7) / 8), (unsigned)(g.nk + 5));
  k_vertex_grad<<<gr, b, 0, s>>>(g, 0.25 * dxinv, 0.25 * dyinv, 0.25 * dzinv, q, qx, qy, qz);
  count_launch();
}

void mthinc_fluxes(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, double bet,
                   const double* phi, const double* gx, const double* gy, const double* gz, const double* u,
                   const double* v, const double* w, double* fx, double* fy, double* fz, int* list, int* count,
                   bool fp32, double* newton) {
  MC m;
  const double dx = 1.0 / dxinv, dy = 1.0 / dyinv, dz = 1.0 / dzinv;
  m.gp1 = -0.5 / std::sqrt(3.0);
  m.gp2 = 0.5 / std::sqrt(3.0);
  const double dcellinv = 1.0 / std::sqrt((dx * dx + dy * dy + dz * dz) / 3.0);
  const double ch = std::cosh(-bet * 1.5);
  m.lim = bet / (2.0 * (ch * ch)) * dcellinv;
  m.lim2lo = m.lim * m.lim * (1.0 - 1.0e-12);
  m.lim2hi = m.lim * m.lim * (1.0 + 1.0e-12);
  m.eps_trunc = 0.5 * (std::tanh(-bet * 2.5) + 1.0);
  m.bet = bet;
  m.dt = dt;
  m.dxi = dxinv;
  m.dyi = dyinv;
  m.dzi = dzinv;
  m.dtdx = dt * dxinv;
  m.dtdy = dt * dyinv;
  m.dtdz = dt * dzinv;
  FMF_CUDA(cudaMemsetAsync(count, 0, sizeof(int), s));
  dim3 b(32, 8, 1);
  dim3 gr((unsigned)((g.ni + 2 + 31) / 32), (unsigned)((g.nj + 2 + 7) / 8), (unsigned)(g.nk + 2));
  k_classify<<<gr, b, 0, s>>>(g, m, phi, gx, gy, gz, u, v, w, fx, fy, fz, list, count);
  const long cap = (long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2);
  if (fp32)
    k_band<float><<<152 * 8, 128, 0, s>>>(g, m, phi, gx, gy, gz, u, v, w, fx, fy, fz, list, count, newton, cap);
  else
    k_band<double><<<152 * 8, 128, 0, s>>>(g, m, phi, gx, gy, gz, u, v, w, fx, fy, fz, list, count, newton, cap);
  count_launch(2);
}

}  // namespace fused
}  // namespace fmf
