// adj_transport.cu -- adjoints of the MTHINC transport (solphi_mthinc1/2/3).
//
// solphi_mthinc1: a band cell's Newton offset d(n, phi) is differentiated at its
// root where the forward pass's iteration converged (implicit function: the
// derivatives of the 8-point Gauss sum by hand), else through the ten iterations
// (forward-mode numbers seeded with the unit normal and phi); each outflow-face
// flux through its 8-point Gauss sum by hand (with respect to n, d and the swept
// fraction vd).  Bulk cells: flux = u phi00 dt/dx with phi00 snapped (zero
// derivative) inside eps_trunc of 0 or 1.
#include "recip.cuh"
#include "adj.cuh"
#include "ops.cuh"

namespace fmf {
namespace adj {

namespace {
struct MC {
  double gp1, gp2, dcellinv, eps_mthinc, eps_trunc;
};
MC mconst(double dxi, double dyi, double dzi, double bet) {
  MC m;
  const double dx = 1.0 / dxi, dy = 1.0 / dyi, dz = 1.0 / dzi;
  m.gp1 = -0.5 / std::sqrt(3.0);
  m.gp2 = 0.5 / std::sqrt(3.0);
  m.dcellinv = 1.0 / std::sqrt((dx * dx + dy * dy + dz * dz) / 3.0);
  const double ch = std::cosh(-bet * 1.5);
  m.eps_mthinc = bet / (2.0 * (ch * ch));
  m.eps_trunc = 0.5 * (std::tanh(-bet * 2.5) + 1.0);
  return m;
}
__device__ __forceinline__ double avg8(const double* p, long c, long X, long Y, long Z) {
  return (p[c - X - Y - Z] + p[c - Y - Z] + p[c - X - Z] + p[c - Z] + p[c - X - Y] + p[c - Y] + p[c - X] + p[c]) *
         0.125;
}
// w / (1 + exp(x)) with the derivative taken as 0 where exp(x) overflows (the
// forward value is 0 there too)
template <int N>
__device__ __forceinline__ Dual<N> sigw(const Dual<N>& w, const Dual<N>& x) {
  if (x.v > 700.0) return Dual<N>(0.0);
  const double e = exp(x.v), s = 1.0 / (1.0 + e), ds = -e * s * s;
  Dual<N> r(w.v * s);
  for (int t = 0; t < N; ++t) r.d[t] = w.d[t] * s + w.v * ds * x.d[t];
  return r;
}
// 1 / cosh(x)^2, 0 (with zero derivative) where cosh(x)^2 overflows
template <int N>
__device__ __forceinline__ Dual<N> sech2(const Dual<N>& x) {
  if (fabs(x.v) > 350.0) return Dual<N>(0.0);
  const double c = cosh(x.v), v = 1.0 / (c * c), dv = -2.0 * tanh(x.v) * v;
  Dual<N> r(v);
  for (int t = 0; t < N; ++t) r.d[t] = dv * x.d[t];
  return r;
}
// the 8 Gauss-point offsets of mthinc_x.h for positions (x1,x2) (y1,y2) (z1,z2)
template <class T>
__device__ void gauss8(const T& nx, const T& ny, const T& nz, const T& xa, const T& xb, const T& ya, const T& yb,
                       const T& za, const T& zb, T* a) {
  const T x1 = nx * xa, x2 = nx * xb, y1 = ny * ya, y2 = ny * yb, z1 = nz * za, z2 = nz * zb;
  a[0] = x1 + y1 + z1;
  a[1] = x2 + y1 + z1;
  a[2] = x1 + y2 + z1;
  a[3] = x2 + y2 + z1;
  a[4] = x1 + y1 + z2;
  a[5] = x2 + y1 + z2;
  a[6] = x1 + y2 + z2;
  a[7] = x2 + y2 + z2;
}
template <class T>
__device__ T sig8(const T* a, const T& wght, double bet, const T& d) {
  const double m = -2.0 * bet;
  T s = sigw(wght, (a[0] + d) * m);
  for (int t = 1; t < 8; ++t) s = s + sigw(wght, (a[t] + d) * m);
  return s;
}
// Newton offset of solphi_mthinc1.f:161-176 (10 iterations from d = 0)
template <class T>
__device__ T newton_d(const T& nx, const T& ny, const T& nz, const T& ph, const MC& M, double bet) {
  T a[8];
  const T g1(M.gp1), g2(M.gp2);
  gauss8(nx, ny, nz, g1, g2, g1, g2, g1, g2, a);
  T d(0.0);
  for (int it = 0; it < 10; ++it) {
    const T f = sig8(a, T(0.125), bet, d) - ph;
    T acc(0.0);
    for (int t = 0; t < 8; ++t) acc = acc + sech2((a[t] + d) * bet) * 0.125;
    const T df = acc * (0.5 * bet);
    d = d - f * df / (df * df + 1.0e-99);
  }
  return d;
}
}  // namespace

namespace {
// Logistic sums over the 8 Gauss points with the exponentials factorised: point t
// (gauss8's order, x index fastest) has z_t = m (x_i + y_j + z_k + d), and with the
// per-axis factors eX[i] = exp(m n_x p_x[i]) (likewise y, z) and ed = exp(m d),
// e_t = exp(z_t) = eX[i] eY[j] eZ[k] ed.  s_t = 1/(1 + e_t) and ds_t = ds/dz =
// -e_t s_t^2 (both 0 where e_t overflows, as sigw takes them).  Returns the sum of
// s_t and, per axis and Gauss index, the sum of ds_t over the points with it.
struct GSums {
  double s, sx[2], sy[2], sz[2];
};
__device__ __forceinline__ GSums gsums(const double* eX, const double* eY, const double* eZ, double ed) {
  GSums G = {0.0, {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const double e = eX[i] * eY[j] * eZ[k] * ed;
        double r = 0.0, ds = 0.0;
        if (e < INFINITY) {  // 1 + e >= 1: the Newton-Raphson reciprocal, no division
          r = recip_nr(1.0 + e);
          ds = -(e * r) * r;
        }
        G.s += r;
        G.sx[i] += ds;
        G.sy[j] += ds;
        G.sz[k] += ds;
      }
  return G;
}

// band cells (the compact list of the forward pass's k_classify): the Newton offset
// and the outflow-face fluxes, differentiated by hand (analytic derivatives of the
// Gauss-point sums); the offsets that did not converge through forward-mode numbers
__global__ void __launch_bounds__(128) k_band_T(Grid g, MC M, double sx, double sy, double sz, double bet,
                                                const double* __restrict__ phi, const double* __restrict__ gx,
                                                const double* __restrict__ gy, const double* __restrict__ gz,
                                                const double* __restrict__ u, const double* __restrict__ v,
                                                const double* __restrict__ w, const double* __restrict__ lfx,
                                                const double* __restrict__ lfy, const double* __restrict__ lfz,
                                                double* lphi, double* __restrict__ lrn, double* lu, double* lv,
                                                double* lw, const int* __restrict__ list,
                                                const int* __restrict__ count, const double* __restrict__ newton,
                                                long cap) {
  const int nb = *count;
  const long n = g.n;
  const long X = 1, Y = g.sy, Z = g.sz;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb; e += gridDim.x * blockDim.x) {
    const long c = list[e];
    double L[6], U[6];
    bool any = false;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const long o = (f & 1) ? c : c - (f < 2 ? X : (f < 4 ? Y : Z));
      const double* lf = f < 2 ? lfx : (f < 4 ? lfy : lfz);
      const double* vl = f < 2 ? u : (f < 4 ? v : w);
      L[f] = lf[o];
      U[f] = vl[o];
      any = any || ((f & 1) ? U[f] > 0.0 : U[f] < 0.0) && L[f] != 0.0;
    }
    if (!any) continue;
    const double rnx = avg8(gx, c, X, Y, Z), rny = avg8(gy, c, X, Y, Z), rnz = avg8(gz, c, X, Y, Z);
    const double q00 = sqrt(rnx * rnx + rny * rny + rnz * rnz);
    const double coef = 1.0 / q00;
    const double nx = rnx * coef, ny = rny * coef, nz = rnz * coef;
    using D4 = Dual<4>;
    D4 dd;
    // per-axis factors of the centred Gauss points (m = -2 bet)
    const double mb = -2.0 * bet;
    const double eX[2] = {exp(mb * nx * M.gp1), exp(mb * nx * M.gp2)},
                 eY[2] = {exp(mb * ny * M.gp1), exp(mb * ny * M.gp2)},
                 eZ[2] = {exp(mb * nz * M.gp1), exp(mb * nz * M.gp2)};
    {
      // d and the last of the forward pass's ten Newton steps (recorded per list
      // entry); where that step moved d by less than 1e-13 (1 + |d|) the iteration
      // has converged and dd/dv = -F_v/F_d at d (F = the 8-point mean - phi), else
      // the derivatives are carried through the ten steps
      const double dv = newton[e], last = newton[cap + e];
      if (fabs(last) <= 1.0e-13 * (1.0 + fabs(dv))) {
        // F = 0.125 sum s_t - phi: F_d = 0.125 m sum ds, F_n = 0.125 m sum ds p_n, F_phi = -1
        const GSums S = gsums(eX, eY, eZ, exp(mb * dv));
        const double Fd = 0.125 * mb * (S.sx[0] + S.sx[1]);
        dd.v = dv;
        dd.d[0] = -0.125 * mb * (S.sx[0] * M.gp1 + S.sx[1] * M.gp2) / Fd;
        dd.d[1] = -0.125 * mb * (S.sy[0] * M.gp1 + S.sy[1] * M.gp2) / Fd;
        dd.d[2] = -0.125 * mb * (S.sz[0] * M.gp1 + S.sz[1] * M.gp2) / Fd;
        dd.d[3] = 1.0 / Fd;
      } else {
        dd = newton_d(D4::var(nx, 0), D4::var(ny, 1), D4::var(nz, 2), D4::var(phi[c], 3), M, bet);
      }
    }
    double ln[3] = {0.0, 0.0, 0.0}, ld = 0.0;
    const double edf = exp(mb * dd.v);
    for (int f = 0; f < 6; ++f) {
      const bool own = (f & 1) ? (U[f] > 0.0) : (U[f] < 0.0);
      if (!own || L[f] == 0.0) continue;
      const int dir = f / 2, side = f & 1;
      const double sc = f < 2 ? sx : (f < 4 ? sy : sz);
      const double vd = U[f] * sc;
      // face_flux: the flux axis's Gauss points over the swept interval [st, en]
      const double st = side ? 0.5 - vd : -0.5, en = side ? 0.5 : -0.5 - vd;
      const double pf[2] = {(st + en) * 0.5 + (-st + en) * M.gp1, (st + en) * 0.5 + (-st + en) * M.gp2};
      const double dpf[2] = {side ? -0.5 + M.gp1 : -0.5 - M.gp1, side ? -0.5 + M.gp2 : -0.5 - M.gp2};  // d pf / d vd
      const double nd = dir == 0 ? nx : (dir == 1 ? ny : nz);
      const double eF[2] = {exp(mb * nd * pf[0]), exp(mb * nd * pf[1])};
      const GSums S = gsums(dir == 0 ? eF : eX, dir == 1 ? eF : eY, dir == 2 ? eF : eZ, edf);
      // flux = w sum s_t (w = vd/8): d/dd = w m sum ds; d/dn_a = w m sum ds p_a;
      // d/dvd = sum s / 8 + w m n_dir sum ds dp_dir/dvd
      const double wm = 0.125 * vd * mb, Lf = L[f];
      const double px0 = dir == 0 ? pf[0] : M.gp1, px1 = dir == 0 ? pf[1] : M.gp2;
      const double py0 = dir == 1 ? pf[0] : M.gp1, py1 = dir == 1 ? pf[1] : M.gp2;
      const double pz0 = dir == 2 ? pf[0] : M.gp1, pz1 = dir == 2 ? pf[1] : M.gp2;
      ln[0] += Lf * wm * (S.sx[0] * px0 + S.sx[1] * px1);
      ln[1] += Lf * wm * (S.sy[0] * py0 + S.sy[1] * py1);
      ln[2] += Lf * wm * (S.sz[0] * pz0 + S.sz[1] * pz1);
      ld += Lf * wm * (S.sx[0] + S.sx[1]);
      const double* sF = dir == 0 ? S.sx : (dir == 1 ? S.sy : S.sz);
      const double lvd = 0.125 * S.s + wm * nd * (sF[0] * dpf[0] + sF[1] * dpf[1]);
      const long o = side ? c : c - (dir == 0 ? X : (dir == 1 ? Y : Z));
      aadd((dir == 0 ? lu : (dir == 1 ? lv : lw)) + o, Lf * lvd * sc);
    }
    for (int q = 0; q < 3; ++q) ln[q] += ld * dd.d[q];
    aadd(lphi + c, ld * dd.d[3]);
    // n = r/|r|: lr = (ln - n (n.ln)) / |r|
    const double dot = ln[0] * nx + ln[1] * ny + ln[2] * nz;
    lrn[c] = (ln[0] - nx * dot) * coef;
    lrn[c + n] = (ln[1] - ny * dot) * coef;
    lrn[c + 2 * n] = (ln[2] - nz * dot) * coef;
  }
}
__global__ void k_mark(const int* __restrict__ list, const int* __restrict__ count, double* __restrict__ flag) {
  const int nb = *count;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb; e += gridDim.x * blockDim.x) flag[list[e]] = 1.0;
}
}  // namespace

void mthinc1_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, double bet,
               const double* phi, const double* gx, const double* gy, const double* gz, const double* u,
               const double* v, const double* w, const double* lfx, const double* lfy, const double* lfz,
               double* lphi, double* lrn, double* lu, double* lv, double* lw, const int* list, const int* count,
               const double* newton) {
  const Grid G = g;
  const MC M = mconst(dxi, dyi, dzi, bet);
  const long n = g.n;
  // lrn[3n + c] = 1 marks the band cells of the forward pass (its classification,
  // not a recomputed one)
  FMF_CUDA(cudaMemsetAsync(lrn, 0, sizeof(double) * 4 * n, s));
  k_mark<<<152 * 4, 256, 0, s>>>(list, count, lrn + 3 * n);
  count_launch();
  range3(s, 0, g.ni + 1, 0, g.nj + 1, 0, g.nk + 1, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    // faces in the order x-, x+, y-, y+, z-, z+: flux adjoints, velocities, scales
    const long fo[6] = {c - X, c, c - Y, c, c - Z, c};
    const double* lf[3] = {lfx, lfy, lfz};
    const double* vel[3] = {u, v, w};
    double* lvel[3] = {lu, lv, lw};
    const double sc[3] = {dt * dxi, dt * dyi, dt * dzi};
    double L[6], U[6];
    bool any = false;
    for (int f = 0; f < 6; ++f) {
      L[f] = lf[f / 2][fo[f]];
      U[f] = vel[f / 2][fo[f]];
      any = any || L[f] != 0.0;
    }
    if (!any) return;
    // bulk cells: those the forward pass did not put on its band list
    if (lrn[c + 3 * n] == 0.0) {
      double phi00 = phi[c];
      double dsnap = 1.0;
      if (phi00 <= M.eps_trunc) {
        phi00 = 0.0;
        dsnap = 0.0;
      }
      if (1.0 - phi00 <= M.eps_trunc) {
        phi00 = 1.0;
        dsnap = 0.0;
      }
      double lp = 0.0;
      for (int f = 0; f < 6; ++f) {
        // owner of the face: the lower face if its velocity <= 0, the upper one if > 0
        const bool own = (f & 1) ? (U[f] > 0.0) : (U[f] <= 0.0);
        if (!own || L[f] == 0.0) continue;
        aadd(lvel[f / 2] + fo[f], L[f] * phi00 * sc[f / 2]);
        lp += L[f] * U[f] * sc[f / 2];
      }
      aadd(lphi + c, lp * dsnap);
    }
    // band cells: k_band_T over the forward pass's band list
  });
  k_band_T<<<152 * 8, 128, 0, s>>>(g, M, dt * dxi, dt * dyi, dt * dzi, bet, phi, gx, gy, gz, u, v, w, lfx, lfy, lfz,
                                   lphi, lrn, lu, lv, lw, list, count, newton,
                                   (long)(g.ni + 2) * (g.nj + 2) * (g.nk + 2));
  count_launch();
}

// cell (i,j,k) averages the vertex gradients (i-1..i, j-1..j, k-1..k); gather over
// the cells 0..n+1 that use vertex v
void rn_avg_T(cudaStream_t s, const Grid& g, const double* lrn, double* lgx, double* lgy, double* lgz) {
  const Grid G = g;
  const long n = g.n;
  range3(s, -2, g.ni + 2, -2, g.nj + 2, -2, g.nk + 2, [=] __device__(int a, int b, int e) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int dc = 0; dc < 2; ++dc)
      for (int db = 0; db < 2; ++db)
        for (int da = 0; da < 2; ++da) {
          const int i = a + da, j = b + db, k = e + dc;
          if (i < 0 || i > G.ni + 1 || j < 0 || j > G.nj + 1 || k < 0 || k > G.nk + 1) continue;
          const long c = G.at(i, j, k);
          sx += lrn[c];
          sy += lrn[c + n];
          sz += lrn[c + 2 * n];
        }
    const long v = G.at(a, b, e);
    lgx[v] += 0.125 * sx;
    lgy[v] += 0.125 * sy;
    lgz[v] += 0.125 * sz;
  });
}

void mthinc2_T(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double dt, const double* u,
               const double* v, const double* w, const double* fx, const double* fy, const double* fz,
               const double* phi, const double* phin, double* lphin, double* lphi, double* lu, double* lv,
               double* lw, double* lfx, double* lfy, double* lfz, double* lpre) {
  const Grid G = g;
  (void)phin;
  // lpre = adjoint of the unclipped value (zero outside the interior)
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    if (i < 1 || i > G.ni || j < 1 || j > G.nj || k < 1 || k > G.nk) {
      lpre[c] = 0.0;
      return;
    }
    // the forward value before its clip, rounded operation by operation as
    // solphi_mthinc2 computes it (this file contracts multiply-adds elsewhere)
    const double div00 = __dadd_rn(__dadd_rn(__dmul_rn(-u[c - X] + u[c], dxi), __dmul_rn(-v[c - Y] + v[c], dyi)),
                                   __dmul_rn(-w[c - Z] + w[c], dzi));
    const double p = __dmul_rn(phi[c], __dadd_rn(1.0, __dmul_rn(dt, div00))) + fx[c - X] - fx[c] + fy[c - Y] -
                     fy[c] + fz[c - Z] - fz[c];
    const double L = (p >= 0.0 && p <= 1.0) ? lphin[c] : 0.0;
    lphin[c] = 0.0;
    lpre[c] = L;
    lphi[c] += L * (1.0 + dt * div00);
  });
  range3(s, -2, g.ni + 2, -2, g.nj + 2, -2, g.nk + 2, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    const double p0 = lpre[c], px = lpre[c + X], py = lpre[c + Y], pz = lpre[c + Z];
    lu[c] += dt * dxi * (phi[c] * p0 - phi[c + X] * px);
    lv[c] += dt * dyi * (phi[c] * p0 - phi[c + Y] * py);
    lw[c] += dt * dzi * (phi[c] * p0 - phi[c + Z] * pz);
    lfx[c] += px - p0;
    lfy[c] += py - p0;
    lfz[c] += pz - p0;
  });
}

// ---- solphi_mthinc3 -----------------------------------------------------------
// Record: pb = pa after the band-test snap and the clip, pass = 1 where pb moved
// with pa (not snapped, not clipped).
void mthinc3_record(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, double bet, const double* gx,
                    const double* gy, const double* gz, const double* pa, double* pb, double* pass) {
  const Grid G = g;
  const MC M = mconst(dxi, dyi, dzi, bet);
  // the snap covers cells 0..n+1 (the ring outside the interior holds the stale
  // values of phin that bnd_contact_angle later reads); the clip the interior only
  range3(s, 0, g.ni + 1, 0, g.nj + 1, 0, g.nk + 1, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    const bool in = i >= 1 && i <= G.ni && j >= 1 && j <= G.nj && k >= 1 && k <= G.nk;
    const double rnx = avg8(gx, c, X, Y, Z), rny = avg8(gy, c, X, Y, Z), rnz = avg8(gz, c, X, Y, Z);
    // the band test of solphi_mthinc3 rounded operation by operation as it computes it
    const double q00 = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(rnx, rnx), __dmul_rn(rny, rny)), __dmul_rn(rnz, rnz)));
    double p = pa[c];
    double m = 1.0;
    if (q00 <= M.eps_mthinc * M.dcellinv) {
      if (p <= M.eps_trunc) {
        p = 0.0;
        m = 0.0;
      }
      if (1.0 - p <= M.eps_trunc) {
        p = 1.0;
        m = 0.0;
      }
    }
    if (in) {
      if (p > 1.0 || p < 0.0) m = 0.0;
      p = fmax(fmin(p, 1.0), 0.0);
    }
    pb[c] = p;
    pass[c] = m;
  });
}

// phin outside the interior is not written by solphi_mthinc2: there it holds the
// values phin had at the start of the step (after the band-test snap of
// solphi_mthinc3 on cells 0..n+1).  Their adjoints go to the step-start phin.
void phin_stale_T(cudaStream_t s, const Grid& g, const double* pass, double* lphin, double* lphin_start) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    if (i >= 1 && i <= G.ni && j >= 1 && j <= G.nj && k >= 1 && k <= G.nk) return;
    const bool ring = i >= 0 && i <= G.ni + 1 && j >= 0 && j <= G.nj + 1 && k >= 0 && k <= G.nk + 1;
    lphin_start[c] += lphin[c] * (ring ? pass[c] : 1.0);
    lphin[c] = 0.0;
  });
}

// sums[0..2] = (sum phi, sum pb, sum pb^2 (1-pb)) as left by op::solphi_mthinc3;
// scal: device scratch of >= 4 doubles
void mthinc3_T(cudaStream_t s, const Grid& g, const double* pb, const double* pass, const double* sums,
               double* lphin, double* lphi, double* scal) {
  const Grid G = g;
  // lambda_off = sum lc * pass_c * pb^2 (1-pb), pass_c: the final clip did not bind
  reduce_interior<1>(
      s, g,
      [=] __device__(int i, int j, int k, double* r) {
        const long c = G.at(i, j, k);
        const double off = (sums[0] - sums[1]) / (sums[2] + 1.0e-99);
        const double p = pb[c];
        const double gp = p * p * (1.0 - p);
        const double q = p + off * gp;
        r[0] = (q >= 0.0 && q <= 1.0) ? lphin[c] * gp : 0.0;
      },
      scal, 10);
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    const double den = sums[2] + 1.0e-99;
    const double off = (sums[0] - sums[1]) / den;
    const double loff = scal[0];
    const double lS1 = loff / den, lS2 = -loff / den, lDn = -loff * off / den;
    const double p = pb[c];
    const double gp = p * p * (1.0 - p), dg = 2.0 * p - 3.0 * p * p;
    const double q = p + off * gp;
    const double lc = (q >= 0.0 && q <= 1.0) ? lphin[c] : 0.0;
    const double lb = lc * (1.0 + off * dg) + lS2 + lDn * dg;
    lphin[c] = lb * pass[c];
    lphi[c] += lS1;
  });
}

}  // namespace adj
}  // namespace fmf
