// adj_mom.cu -- adjoints of the WENO5 advection (cal_advu_weno5 + weno5.h) and of
// the CSF surface-tension force (cal_grad_p2a, calrn x4, calrkap, cal_grad_p2uvw,
// calfst).
#include "adj.cuh"
#include "ops.cuh"

namespace fmf {
namespace adj {

namespace {
// One side of weno5.h: r = w1 d1 + w2 d2 + w3 d3 with the product-form weights, and
// its reverse sweep (la[0..4] += dr/d(a5, a3, a1, b1, b3) * lr).  The weights are
// formed with one reciprocal of the denominator (iD), which the reverse sweep reuses:
// an adjoint needs the derivative, not the forward's last bit.
struct Side {
  double d1, d2, d3, t[6], s1, s2, s3, P1, P2, P3, iD, w1, w3, r;
};
__device__ __forceinline__ void side_fwd(double a5, double a3, double a1, double b1, double b3, Side& S) {
  S.d1 = a5 * 2.0 - a3 * 7.0 + a1 * 11.0;
  S.d2 = -a3 + a1 * 5.0 + b1 * 2.0;
  S.d3 = a1 * 2.0 + b1 * 5.0 - b3;
  S.t[0] = a5 - a3 * 2.0 + a1;
  S.t[1] = a5 - a3 * 4.0 + a1 * 3.0;
  S.t[2] = a3 - a1 * 2.0 + b1;
  S.t[3] = a3 - b1;
  S.t[4] = a1 - b1 * 2.0 + b3;
  S.t[5] = a1 * 3.0 - b1 * 4.0 + b3;
  S.s1 = S.t[0] * S.t[0] * 13.0 + S.t[1] * S.t[1] * 3.0;
  S.s2 = S.t[2] * S.t[2] * 13.0 + S.t[3] * S.t[3] * 3.0;
  S.s3 = S.t[4] * S.t[4] * 13.0 + S.t[5] * S.t[5] * 3.0;
  S.P1 = S.s2 * S.s3;
  S.P2 = S.s1 * S.s3;
  S.P3 = S.s1 * S.s2;
  const double m1 = S.P1 * S.P1, m2 = S.P2 * S.P2 * 6.0, m3 = S.P3 * S.P3 * 3.0;
  S.iD = 1.0 / (m1 + m2 + m3 + 1.0e-80);
  S.w1 = m1 * S.iD;
  S.w3 = m3 * S.iD;
  S.r = S.w1 * S.d1 + (1.0 - S.w1 - S.w3) * S.d2 + S.w3 * S.d3;
}
__device__ __forceinline__ void side_rev(const Side& S, double lr, double* la) {
  const double w2 = 1.0 - S.w1 - S.w3;
  const double ld1 = lr * S.w1, ld2 = lr * w2, ld3 = lr * S.w3;
  const double lw1 = lr * (S.d1 - S.d2), lw3 = lr * (S.d3 - S.d2);
  const double G = lw1 * S.w1 + lw3 * S.w3;
  const double lm1 = (lw1 - G) * S.iD, lm2 = -G * S.iD, lm3 = (lw3 - G) * S.iD;
  const double lP1 = 2.0 * S.P1 * lm1, lP2 = 12.0 * S.P2 * lm2, lP3 = 6.0 * S.P3 * lm3;
  const double ls1 = lP2 * S.s3 + lP3 * S.s2, ls2 = lP1 * S.s3 + lP3 * S.s1, ls3 = lP1 * S.s2 + lP2 * S.s1;
  const double lt0 = 26.0 * S.t[0] * ls1, lt1 = 6.0 * S.t[1] * ls1;
  const double lt2 = 26.0 * S.t[2] * ls2, lt3 = 6.0 * S.t[3] * ls2;
  const double lt4 = 26.0 * S.t[4] * ls3, lt5 = 6.0 * S.t[5] * ls3;
  la[0] += 2.0 * ld1 + lt0 + lt1;
  la[1] += -7.0 * ld1 - ld2 - 2.0 * lt0 - 4.0 * lt1 + lt2 + lt3;
  la[2] += 11.0 * ld1 + 5.0 * ld2 + 2.0 * ld3 + lt0 + 3.0 * lt1 - 2.0 * lt2 + lt4 + 3.0 * lt5;
  la[3] += 2.0 * ld2 + 5.0 * ld3 + lt2 - lt3 - 2.0 * lt4 - 4.0 * lt5;
  la[4] += -ld3 + lt4 + lt5;
}
// adjoint of  out += weno5_line(q, c, S, vel) * di  given lout: lD[0..5] = the
// adjoints of the six differences (dm5, dm3, dm1, dp1, dp3, dp5); returns lvel
__device__ double wline_T(const double* __restrict__ q, long c, long S, double vel, double lout, double di,
                          double* lD) {
  for (int m = 0; m < 6; ++m) lD[m] = 0.0;
  const double lr = lout * di;
  if (lr == 0.0) return 0.0;
  const double m3 = q[c - 3 * S], m2 = q[c - 2 * S], m1 = q[c - S], z0 = q[c], p1 = q[c + S], p2 = q[c + 2 * S],
               p3 = q[c + 3 * S];
  const double dm5 = -m3 + m2, dm3 = -m2 + m1, dm1 = -m1 + z0, dp1 = -z0 + p1, dp3 = -p1 + p2, dp5 = -p2 + p3;
  // the upwind side (the other one carries the weight 0 in weno5.h), its inputs
  // mirrored by selects so that one inlined copy serves both signs of vel
  const bool neg = vel < 0.0;
  Side A;
  side_fwd(neg ? dp5 : dm5, neg ? dp3 : dm3, neg ? dp1 : dm1, neg ? dm1 : dp1, neg ? dm3 : dp3, A);
  if (vel == 0.0) {  // both sides enter d(out)/d(vel); neither enters d(out)/d(q)
    Side B;
    side_fwd(dp5, dp3, dp1, dm1, dm3, B);
    return lr * (A.r + B.r) / 12.0;
  }
  double la[5] = {0, 0, 0, 0, 0};
  side_rev(A, lr * 2.0 * vel / 12.0, la);
  lD[0] = neg ? 0.0 : la[0];
  lD[1] = neg ? la[4] : la[1];
  lD[2] = neg ? la[3] : la[2];
  lD[3] = neg ? la[2] : la[3];
  lD[4] = neg ? la[1] : la[4];
  lD[5] = neg ? la[0] : 0.0;
  return lr * 2.0 * A.r / 12.0;
}

// Offsets (relative to the cell) of the four velocity points that form the
// advecting velocity of line (component q, direction d); the line reads component d.
__constant__ signed char kVelOff[9][4][3] = {
    {{-1, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, 0, 0}},   {{0, -1, 0}, {1, -1, 0}, {0, 0, 0}, {1, 0, 0}},
    {{0, 0, -1}, {1, 0, -1}, {0, 0, 0}, {1, 0, 0}},  {{-1, 0, 0}, {-1, 1, 0}, {0, 0, 0}, {0, 1, 0}},
    {{0, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 1, 0}},   {{0, 0, -1}, {0, 1, -1}, {0, 0, 0}, {0, 1, 0}},
    {{-1, 0, 0}, {-1, 0, 1}, {0, 0, 0}, {0, 0, 1}},  {{0, -1, 0}, {0, -1, 1}, {0, 0, 0}, {0, 0, 1}},
    {{0, 0, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 1}}};

// Pass 1: per interior cell and each of the 9 lines (one thread per cell and
// line: grid z = 9 nk), the adjoints of the six differences (D, 54 arrays) and of
// the advecting velocity (V, 9 arrays).
__global__ void __launch_bounds__(256) k_weno_T1(Grid g, double dxi, double dyi, double dzi,
                                                 const double* __restrict__ u, const double* __restrict__ v,
                                                 const double* __restrict__ w, const double* __restrict__ la0,
                                                 const double* __restrict__ la1, const double* __restrict__ la2,
                                                 double* __restrict__ D, double* __restrict__ V) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int line = (int)blockIdx.z % 9, k = 1 + (int)blockIdx.z / 9;
  if (i > g.ni || j > g.nj) return;
  const int q = line / 3, d = line % 3;
  const long X = 1, Y = g.sy, Z = g.sz, n = g.n;
  const long c = g.at(i, j, k);
  const double* vq = d == 0 ? u : (d == 1 ? v : w);
  const signed char(*o)[3] = kVelOff[line];
  const double a = vq[c + o[0][0] * X + o[0][1] * Y + o[0][2] * Z];
  const double b = vq[c + o[1][0] * X + o[1][1] * Y + o[1][2] * Z];
  const double e = vq[c + o[2][0] * X + o[2][1] * Y + o[2][2] * Z];
  const double f = vq[c + o[3][0] * X + o[3][1] * Y + o[3][2] * Z];
  const double vel = ((a + b) * 0.5 + (e + f) * 0.5) * 0.5;
  const double L = (q == 0 ? la0 : (q == 1 ? la1 : la2))[c];
  double lD[6];
  const double lvel = wline_T(q == 0 ? u : (q == 1 ? v : w), c, d == 0 ? X : (d == 1 ? Y : Z), vel, L,
                              d == 0 ? dxi : (d == 1 ? dyi : dzi), lD);
#pragma unroll
  for (int m = 0; m < 6; ++m) D[(long)(line * 6 + m) * n + c] = lD[m];
  V[(long)line * n + c] = lvel;
}
// Pass 2: every point gathers what the lines of the cells around it owe it.
__global__ void __launch_bounds__(256) k_weno_T2(Grid g, const double* __restrict__ D,
                                                 const double* __restrict__ V, double* __restrict__ lu,
                                                 double* __restrict__ lv, double* __restrict__ lw) {
  const int x = -2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int y = -2 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int z = -2 + (int)blockIdx.z;
  if (x > g.ni + 3 || y > g.nj + 3) return;
  const long n = g.n;
  auto in = [&](int a, int b, int e) { return a >= 1 && a <= g.ni && b >= 1 && b <= g.nj && e >= 1 && e <= g.nk; };
  // point x sits at stencil position o (-3..3) of the cell x - o*S; its coefficient
  // there: o=-3: -D0, -2: D0-D1, -1: D1-D2, 0: D2-D3, 1: D3-D4, 2: D4-D5, 3: D5
  double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int p = 0; p < 3; ++p) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int line = p * 3 + d;
      const double* Dl = D + (long)line * 6 * n;
      for (int o = -3; o <= 3; ++o) {
        const int ci = x - (d == 0 ? o : 0), cj = y - (d == 1 ? o : 0), ck = z - (d == 2 ? o : 0);
        if (!in(ci, cj, ck)) continue;
        const long c = g.at(ci, cj, ck);
        const int m = o + 3;  // 0..6
        const double hi = m < 6 ? Dl[(long)m * n + c] : 0.0;     // + D_m
        const double lo = m > 0 ? Dl[(long)(m - 1) * n + c] : 0.0;  // - D_{m-1}
        acc[p] += lo - hi;
      }
    }
    // velocity points: lines (q, p) read component p at 4 offsets
    for (int q = 0; q < 3; ++q) {
      const int line = q * 3 + p;
      for (int t = 0; t < 4; ++t) {
        const int ci = x - kVelOff[line][t][0], cj = y - kVelOff[line][t][1], ck = z - kVelOff[line][t][2];
        if (!in(ci, cj, ck)) continue;
        acc[p] += 0.25 * V[(long)line * n + g.at(ci, cj, ck)];
      }
    }
  }
  const long c = g.at(x, y, z);
  lu[c] += acc[0];
  lv[c] += acc[1];
  lw[c] += acc[2];
}
}  // namespace

void weno_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u, const double* v,
            const double* w, const double* const* ladv, double* lu, double* lv, double* lw, double* work) {
  double* D = work;
  double* V = work + 54 * g.n;
  k_weno_T1<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, 9 * g.nk), dim3(32, 8), 0, s>>>(g, dxi, dyi, dzi, u, v, w, ladv[0],
                                                                               ladv[1], ladv[2], D, V);
  k_weno_T2<<<dim3((g.ni + 6 + 31) / 32, (g.nj + 6 + 7) / 8, g.nk + 6), dim3(32, 8), 0, s>>>(g, D, V, lu, lv, lw);
  count_launch(2);
}

// ---- CSF --------------------------------------------------------------------------
void csf_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double rhol, double rhog,
           double sigma, const double* phi, const double* const* lf, double* lphi, double* work,
           const double* kap_rec) {
  const Grid G = g;
  const long n = g.n;
  double* Gv = work;             // vertex gradient (3n)
  double* rn = work + 3 * n;     // the four normal families (12n)
  double* kap = work + 15 * n;   // curvature at u, v, w points (3n)
  double* gq = work + 18 * n;    // face gradient of phi (3n)
  double* lG = work + 21 * n;    // adjoint of the vertex gradient (3n)
  double* lv = work + 24 * n;    // per normal family: adjoint of its 8-point mean (12n)
  double* lkap = work + 36 * n;  // adjoint of the curvature (3n)
  double* lgq = work + 39 * n;   // adjoint of the face gradient (3n)
  static const int offs[4][3] = {{1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  // forward recompute
  op::cal_grad_p2a(s, g, dxi, dyi, dzi, phi, Gv, Gv + n, Gv + 2 * n);
  if (!kap_rec) {
    for (int q = 0; q < 4; ++q)
      op::calrn(s, g, dxi, dyi, dzi, offs[q][0], offs[q][1], offs[q][2], Gv, Gv + n, Gv + 2 * n, rn + 3 * n * q);
    op::calrkap(s, g, dxi, dyi, dzi, rn, rn + 3 * n, rn + 6 * n, rn + 9 * n, kap);
  } else {
    kap = (double*)kap_rec;  // read only; valid where the force adjoints can be non-zero
  }
  op::cal_grad_prs(s, g, dxi, dyi, dzi, phi, gq, gq + n, gq + 2 * n);
  // calfst: f_c = -st kap_c g_c
  const double st = 2.0 * sigma / (rhol + rhog);
  const double *lf0 = lf[0], *lf1 = lf[1], *lf2 = lf[2];
  flat(s, n, [=] __device__(long t) {
    const double L[3] = {lf0[t], lf1[t], lf2[t]};
    for (int q = 0; q < 3; ++q) {
      lkap[t + q * n] = -st * gq[t + q * n] * L[q];
      lgq[t + q * n] = L[q] != 0.0 ? -st * kap[t + q * n] * L[q] : 0.0;
    }
  });
  grad_prs_T(s, g, dxi, dyi, dzi, lgq, lgq + n, lgq + 2 * n, lphi);
  // calrkap and calrn reversed as two gathers (no atomics).
  // Families (calrkap's rn arguments): 0 = pp (offset 1,1,1), 1 = r12 (0,0,1),
  // 2 = r13 (0,1,0), 3 = r23 (1,0,0).  Family f's normal at o is N(v) = v/(|v| + vs)
  // of the mean v of Gv over o - {0,X_f} - {0,Y_f} - {0,Z_f} (X_f = 0 where the
  // offset is 0), written by calrn for o_i in [-2 + ip, ni+3] (same in j, k).
  // calrkap writes the u curvature where k >= -1, j >= -1, i <= ni+2, the v one where
  // k >= -1, j <= nj+2, i >= -1, the w one where k <= nk+2, j >= -1, i >= -1.
  const double vs = std::sqrt(dxi * dxi + dyi * dyi + dzi * dzi) * 1.0e-30;
  // pass 1, per normal point o and family: the normal's adjoint gathered from the
  // curvatures that read it, then lv = (dN/dv)^T lrn
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    auto in = [&](int a, int b, int e) {
      return a >= -2 && a <= G.ni + 3 && b >= -2 && b <= G.nj + 3 && e >= -2 && e <= G.nk + 3;
    };
    auto ku = [&](int a, int b, int e, long o) {
      return in(a, b, e) && e >= -1 && b >= -1 && a <= G.ni + 2 ? lkap[o] : 0.0;
    };
    auto kv = [&](int a, int b, int e, long o) {
      return in(a, b, e) && e >= -1 && b <= G.nj + 2 && a >= -1 ? lkap[o + n] : 0.0;
    };
    auto kw = [&](int a, int b, int e, long o) {
      return in(a, b, e) && e <= G.nk + 2 && b >= -1 && a >= -1 ? lkap[o + 2 * n] : 0.0;
    };
    // kap_u = dxi (pp_x[+X] - pp_x) + dyi (r12_y - r12_y[-Y]) + dzi (r13_z - r13_z[-Z]),
    // kap_v = dxi (r12_x - r12_x[-X]) + dyi (pp_y[+Y] - pp_y) + dzi (r23_z - r23_z[-Z]),
    // kap_w = dxi (r13_x - r13_x[-X]) + dyi (r23_y - r23_y[-Y]) + dzi (pp_z[+Z] - pp_z)
    double L[4][3];
    L[0][0] = dxi * (ku(i - 1, j, k, c - X) - ku(i, j, k, c));
    L[0][1] = dyi * (kv(i, j - 1, k, c - Y) - kv(i, j, k, c));
    L[0][2] = dzi * (kw(i, j, k - 1, c - Z) - kw(i, j, k, c));
    L[1][0] = dxi * (kv(i, j, k, c) - kv(i + 1, j, k, c + X));
    L[1][1] = dyi * (ku(i, j, k, c) - ku(i, j + 1, k, c + Y));
    L[1][2] = 0.0;
    L[2][0] = dxi * (kw(i, j, k, c) - kw(i + 1, j, k, c + X));
    L[2][1] = 0.0;
    L[2][2] = dzi * (ku(i, j, k, c) - ku(i, j, k + 1, c + Z));
    L[3][0] = 0.0;
    L[3][1] = dyi * (kw(i, j, k, c) - kw(i, j + 1, k, c + Y));
    L[3][2] = dzi * (kv(i, j, k, c) - kv(i, j, k + 1, c + Z));
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const int ip = f == 0 || f == 3, jp = f == 0 || f == 2, kp = f == 0 || f == 1;
      if (i < -2 + ip || j < -2 + jp || k < -2 + kp) continue;  // calrn does not write o
      double* out = lv + 3 * n * f + c;
      const double lx = L[f][0], ly = L[f][1], lz = L[f][2];
      if (lx == 0.0 && ly == 0.0 && lz == 0.0) {
        out[0] = out[n] = out[2 * n] = 0.0;
        continue;
      }
      const long Xf = ip ? X : 0, Yf = jp ? Y : 0, Zf = kp ? Z : 0;
      const long b = c - Xf - Yf - Zf;
      double r[3];
#pragma unroll
      for (int q3 = 0; q3 < 3; ++q3) {
        const double* p = Gv + q3 * n + b;
        r[q3] = (p[0] + p[Xf] + p[Yf] + p[Xf + Yf] + p[Zf] + p[Xf + Zf] + p[Yf + Zf] + p[Xf + Yf + Zf]) * 0.125;
      }
      // dN/dv = I/a - v v^T/(a^2 m) with m = |v|, a = m + vs:
      // lv = (l - v (v.l)/(m a)) / a, the factor formed as ((v.l)/m)/a, which stays
      // finite for any m > 0
      const double s2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
      double ia, t = 0.0;
      if (s2 > 0.0) {
        const double im = rsqrt(s2);
        ia = 1.0 / (s2 * im + vs);
        t = ((r[0] * lx + r[1] * ly + r[2] * lz) * im) * ia;
      } else {
        ia = 1.0 / vs;
      }
      out[0] = (lx - r[0] * t) * ia;
      out[n] = (ly - r[1] * t) * ia;
      out[2 * n] = (lz - r[2] * t) * ia;
    }
  });
  // pass 2, per vertex p: 0.125 lv over the (family, corner) pairs whose mean reads
  // p, i.e. o = p + {0,X_f} + {0,Y_f} + {0,Z_f} (families 1-3 read two points, four
  // times each)
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    auto ok = [&](int f, int a, int b, int e) {
      const int ip = f == 0 || f == 3, jp = f == 0 || f == 2, kp = f == 0 || f == 1;
      return a >= -2 + ip && a <= G.ni + 3 && b >= -2 + jp && b <= G.nj + 3 && e >= -2 + kp && e <= G.nk + 3;
    };
    const bool a1 = ok(1, i, j, k), b1 = ok(1, i, j, k + 1), a2 = ok(2, i, j, k), b2 = ok(2, i, j + 1, k),
               a3 = ok(3, i, j, k), b3 = ok(3, i + 1, j, k);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double* L0 = lv + q * n + c;
      double acc = 0.0;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int di = t & 1, dj = (t >> 1) & 1, dk = t >> 2;
        if (ok(0, i + di, j + dj, k + dk)) acc += L0[di * X + dj * Y + dk * Z];
      }
      const double* L1 = L0 + 3 * n;
      const double* L2 = L0 + 6 * n;
      const double* L3 = L0 + 9 * n;
      double acc4 = 0.0;
      if (a1) acc4 += L1[0];
      if (b1) acc4 += L1[Z];
      if (a2) acc4 += L2[0];
      if (b2) acc4 += L2[Y];
      if (a3) acc4 += L3[0];
      if (b3) acc4 += L3[X];
      lG[q * n + c] = 0.125 * (acc + 4.0 * acc4);
    }
  });
  grad_p2a_T(s, g, dxi, dyi, dzi, lG, lG + n, lG + 2 * n, lphi);
}

}  // namespace adj
}  // namespace fmf
