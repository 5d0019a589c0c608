// fmf_oracle.cpp -- CPU oracle (test infrastructure; see fmf_oracle.h).
//
// A line-faithful C++ restatement of the reference's per-step subroutines.  Every
// function names the reference file:line it restates.  Arrays are Fortran-ordered
// (i fastest) with origin -2 in each direction; F(a,i,j,k) addresses element (i,j,k).
// Compiled with -O2 -fopenmp -ffp-contract=off: no FMA contraction, no fast-math,
// so every + - * / and sqrt is one correctly rounded IEEE double operation in the
// reference's left-to-right order.  Transcendentals come from the C library.
#include "fmf_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Dim {
  int ni, nj, nk;
  long nx, ny, nz;
  Dim(int a, int b, int c) : ni(a), nj(b), nk(c), nx(a + 6), ny(b + 6), nz(c + 6) {}
  inline long at(int i, int j, int k) const {
    return (long)(i + 2) + nx * ((long)(j + 2) + ny * (long)(k + 2));
  }
  long size() const { return nx * ny * nz; }
};

#define F(a, i, j, k) a[D.at((i), (j), (k))]
#define F4(a, i, j, k, l) a[D.at((i), (j), (k)) + (long)((l)-1) * D.size()]

inline double sq(double x) { return x * x; }

double g_sor_tol = 1.0e-3;  // solu_sor4.f:291-293
int g_sor_max = 21;

// Fixed-order reduction: one partial per k plane (computed in i-fastest order),
// summed in increasing k.  Deterministic for any thread count.
template <class Fn>
double plane_sum(const Dim& D, Fn fn) {
  std::vector<double> part(D.nk + 1, 0.0);
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k) {
    double s = 0.0;
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) s = s + fn(i, j, k);
    part[k] = s;
  }
  double s = 0.0;
  for (int k = 1; k <= D.nk; ++k) s = s + part[k];
  return s;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// cal_grad_p2a.f:1-76 -- vertex gradient of q, range -2..n+2 in each direction.
void orc_cal_grad_p2a(const int* ID, const int* svall, const int* ni, const int* nj, const int* nk,
                      const double* dxinv, const double* dyinv_array, const double* dzinv,
                      const double* q, double* qx, double* qy, double* qz) {
  (void)svall;
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dzi = *dzinv;
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= D.nk + 2; ++k)
    for (int j = -2; j <= D.nj + 2; ++j)
      for (int i = -2; i <= D.ni + 2; ++i) {
        const int dis = j + D.nj * (*ID);
        const double dyi = dyinv_array[dis + 2];
        const double q000 = F(q, i, j, k), qp00 = F(q, i + 1, j, k), q0p0 = F(q, i, j + 1, k),
                     qpp0 = F(q, i + 1, j + 1, k), q00p = F(q, i, j, k + 1),
                     qp0p = F(q, i + 1, j, k + 1), q0pp = F(q, i, j + 1, k + 1),
                     qppp = F(q, i + 1, j + 1, k + 1);
        double gx = -q000 + qp00 - q0p0 + qpp0 - q00p + qp0p - q0pp + qppp;
        double gy = -q000 - qp00 + q0p0 + qpp0 - q00p - qp0p + q0pp + qppp;
        double gz = -q000 - qp00 - q0p0 - qpp0 + q00p + qp0p + q0pp + qppp;
        F(qx, i, j, k) = gx * 0.25 * dxi;
        F(qy, i, j, k) = gy * 0.25 * dyi;
        F(qz, i, j, k) = gz * 0.25 * dzi;
      }
}

// ---------------------------------------------------------------------------
// mthinc_x.h:1-14 and mthinc_tanh.h:1-9: Gauss-point offsets and the 8-point
// sigmoid average.
namespace {
struct GP8 {
  double x111, x211, x121, x221, x112, x212, x122, x222;
};
inline GP8 mthinc_x(double rnx, double rny, double rnz, double xg1, double xg2, double yg1,
                    double yg2, double zg1, double zg2) {
  const double x1 = rnx * xg1, x2 = rnx * xg2, y1 = rny * yg1, y2 = rny * yg2, z1 = rnz * zg1,
               z2 = rnz * zg2;
  GP8 g;
  g.x111 = x1 + y1 + z1;
  g.x211 = x2 + y1 + z1;
  g.x121 = x1 + y2 + z1;
  g.x221 = x2 + y2 + z1;
  g.x112 = x1 + y1 + z2;
  g.x212 = x2 + y1 + z2;
  g.x122 = x1 + y2 + z2;
  g.x222 = x2 + y2 + z2;
  return g;
}
inline double mthinc_tanh(const GP8& g, double wght, double bet, double ddd) {
  const double m = -2.0 * bet;
  return wght / (1.0 + std::exp(m * (g.x111 + ddd))) + wght / (1.0 + std::exp(m * (g.x211 + ddd))) +
         wght / (1.0 + std::exp(m * (g.x121 + ddd))) + wght / (1.0 + std::exp(m * (g.x221 + ddd))) +
         wght / (1.0 + std::exp(m * (g.x112 + ddd))) + wght / (1.0 + std::exp(m * (g.x212 + ddd))) +
         wght / (1.0 + std::exp(m * (g.x122 + ddd))) + wght / (1.0 + std::exp(m * (g.x222 + ddd)));
}
inline double isech2(double wght, double a) {
  const double c = std::cosh(a);
  return wght / (c * c);
}
}  // namespace

// solphi_mthinc1.f:1-292 -- MTHINC face fluxes (volume fractions x u dt/dx).
void orc_solphi_mthinc1(const int* ni, const int* nj, const int* nk, const double* dxinv,
                        const double* dyinv, const double* dzinv, const double* dt,
                        const double* bet_mthinc, const double* phi, const double* phix,
                        const double* phiy, const double* phiz, const double* u, const double* v,
                        const double* w, double* flphix, double* flphiy, double* flphiz) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv, dtt = *dt;
  const double dx = 1.0 / dxi, dy = 1.0 / dyi, dz = 1.0 / dzi;
  // :44-53 zero the fluxes
#pragma omp parallel for schedule(static)
  for (int k = -1; k <= D.nk + 1; ++k)
    for (int j = -1; j <= D.nj + 1; ++j)
      for (int i = -1; i <= D.ni + 1; ++i) {
        F(flphix, i, j, k) = 0.0;
        F(flphiy, i, j, k) = 0.0;
        F(flphiz, i, j, k) = 0.0;
      }
  const double bet = *bet_mthinc;
  const double gp1 = -0.5 / std::sqrt(3.0), gp2 = 0.5 / std::sqrt(3.0);
  const double dcellinv = 1.0 / std::sqrt((dx * dx + dy * dy + dz * dz) / 3.0);
  const double ch = std::cosh(-bet * 1.5);
  const double eps_mthinc = bet / (2.0 * (ch * ch));
  const double eps_trunc = 0.5 * (std::tanh(-bet * 2.5) + 1.0);
  // Cells write only the faces they donate through; a face is written by at most
  // one cell (u<0 -> east cell, u>0 -> west cell, u==0 -> both write 0), so the
  // k-parallel loop is race free (solphi_mthinc1.f:77-288).
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= D.nk + 1; ++k)
    for (int j = 0; j <= D.nj + 1; ++j)
      for (int i = 0; i <= D.ni + 1; ++i) {
        double rnx = (F(phix, i - 1, j - 1, k - 1) + F(phix, i, j - 1, k - 1) + F(phix, i - 1, j, k - 1) +
                      F(phix, i, j, k - 1) + F(phix, i - 1, j - 1, k) + F(phix, i, j - 1, k) +
                      F(phix, i - 1, j, k) + F(phix, i, j, k)) * 0.125;
        double rny = (F(phiy, i - 1, j - 1, k - 1) + F(phiy, i, j - 1, k - 1) + F(phiy, i - 1, j, k - 1) +
                      F(phiy, i, j, k - 1) + F(phiy, i - 1, j - 1, k) + F(phiy, i, j - 1, k) +
                      F(phiy, i - 1, j, k) + F(phiy, i, j, k)) * 0.125;
        double rnz = (F(phiz, i - 1, j - 1, k - 1) + F(phiz, i, j - 1, k - 1) + F(phiz, i - 1, j, k - 1) +
                      F(phiz, i, j, k - 1) + F(phiz, i - 1, j - 1, k) + F(phiz, i, j - 1, k) +
                      F(phiz, i - 1, j, k) + F(phiz, i, j, k)) * 0.125;
        const double q00 = std::sqrt(rnx * rnx + rny * rny + rnz * rnz);
        if (q00 <= eps_mthinc * dcellinv) {
          // :110-135 truncated first-order upwinding
          double phi00 = F(phi, i, j, k);
          if (phi00 <= eps_trunc) phi00 = 0.0;
          if (1.0 - phi00 <= eps_trunc) phi00 = 1.0;
          if (F(u, i - 1, j, k) <= 0.0) F(flphix, i - 1, j, k) = F(u, i - 1, j, k) * phi00 * dtt * dxi;
          if (F(u, i, j, k) >= 0.0) F(flphix, i, j, k) = F(u, i, j, k) * phi00 * dtt * dxi;
          if (F(v, i, j - 1, k) <= 0.0) F(flphiy, i, j - 1, k) = F(v, i, j - 1, k) * phi00 * dtt * dyi;
          if (F(v, i, j, k) >= 0.0) F(flphiy, i, j, k) = F(v, i, j, k) * phi00 * dtt * dyi;
          if (F(w, i, j, k - 1) <= 0.0) F(flphiz, i, j, k - 1) = F(w, i, j, k - 1) * phi00 * dtt * dzi;
          if (F(w, i, j, k) >= 0.0) F(flphiz, i, j, k) = F(w, i, j, k) * phi00 * dtt * dzi;
        } else {
          const double coef = 1.0 / q00;
          rnx = rnx * coef;
          rny = rny * coef;
          rnz = rnz * coef;
          // :161-176 Newton iterations for the offset d
          GP8 g = mthinc_x(rnx, rny, rnz, gp1, gp2, gp1, gp2, gp1, gp2);
          const double wght = 0.125;
          double ddd = 0.0;
          const double ph = F(phi, i, j, k);
          for (int inr = 1; inr <= 10; ++inr) {
            const double f = mthinc_tanh(g, wght, bet, ddd) - ph;
            const double df =
                0.5 * bet *
                (isech2(wght, bet * (g.x111 + ddd)) + isech2(wght, bet * (g.x211 + ddd)) +
                 isech2(wght, bet * (g.x121 + ddd)) + isech2(wght, bet * (g.x221 + ddd)) +
                 isech2(wght, bet * (g.x112 + ddd)) + isech2(wght, bet * (g.x212 + ddd)) +
                 isech2(wght, bet * (g.x122 + ddd)) + isech2(wght, bet * (g.x222 + ddd)));
            ddd = ddd - f * df / (df * df + 1.0e-99);
          }
          // :182-282 swept-volume fluxes through the outflow faces
          const double uw = F(u, i - 1, j, k), ue = F(u, i, j, k);
          const double vs = F(v, i, j - 1, k), vn = F(v, i, j, k);
          const double wb = F(w, i, j, k - 1), wt = F(w, i, j, k);
          if (uw < 0.0) {
            const double vd = uw * dtt * dxi;
            const double st = -0.5, en = -0.5 - vd;
            const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
            GP8 h = mthinc_x(rnx, rny, rnz, a1, a2, gp1, gp2, gp1, gp2);
            F(flphix, i - 1, j, k) = mthinc_tanh(h, 0.125 * vd, bet, ddd);
          }
          if (ue > 0.0) {
            const double vd = ue * dtt * dxi;
            const double st = 0.5 - vd, en = 0.5;
            const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
            GP8 h = mthinc_x(rnx, rny, rnz, a1, a2, gp1, gp2, gp1, gp2);
            F(flphix, i, j, k) = mthinc_tanh(h, 0.125 * vd, bet, ddd);
          }
          if (vs < 0.0) {
            const double vd = vs * dtt * dyi;
            const double st = -0.5, en = -0.5 - vd;
            const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
            GP8 h = mthinc_x(rnx, rny, rnz, gp1, gp2, a1, a2, gp1, gp2);
            F(flphiy, i, j - 1, k) = mthinc_tanh(h, 0.125 * vd, bet, ddd);
          }
          if (vn > 0.0) {
            const double vd = vn * dtt * dyi;
            const double st = 0.5 - vd, en = 0.5;
            const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
            GP8 h = mthinc_x(rnx, rny, rnz, gp1, gp2, a1, a2, gp1, gp2);
            F(flphiy, i, j, k) = mthinc_tanh(h, 0.125 * vd, bet, ddd);
          }
          if (wb < 0.0) {
            const double vd = wb * dtt * dzi;
            const double st = -0.5, en = -0.5 - vd;
            const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
            GP8 h = mthinc_x(rnx, rny, rnz, gp1, gp2, gp1, gp2, a1, a2);
            F(flphiz, i, j, k - 1) = mthinc_tanh(h, 0.125 * vd, bet, ddd);
          }
          if (wt > 0.0) {
            const double vd = wt * dtt * dzi;
            const double st = 0.5 - vd, en = 0.5;
            const double a1 = (st + en) * 0.5 + (-st + en) * gp1, a2 = (st + en) * 0.5 + (-st + en) * gp2;
            GP8 h = mthinc_x(rnx, rny, rnz, gp1, gp2, gp1, gp2, a1, a2);
            F(flphiz, i, j, k) = mthinc_tanh(h, 0.125 * vd, bet, ddd);
          }
        }
      }
}

// solphi_mthinc2.f:1-48 -- conservative update and clip.
void orc_solphi_mthinc2(const int* ni, const int* nj, const int* nk, const double* dxinv,
                        const double* dyinv, const double* dzinv, const double* dt, const double* u,
                        const double* v, const double* w, const double* flphix,
                        const double* flphiy, const double* flphiz, const double* phi,
                        double* phin) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv, dtt = *dt;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        const double div00 = (-F(u, i - 1, j, k) + F(u, i, j, k)) * dxi +
                             (-F(v, i, j - 1, k) + F(v, i, j, k)) * dyi +
                             (-F(w, i, j, k - 1) + F(w, i, j, k)) * dzi;
        double p = F(phi, i, j, k) * (1.0 + dtt * div00) + F(flphix, i - 1, j, k) - F(flphix, i, j, k) +
                   F(flphiy, i, j - 1, k) - F(flphiy, i, j, k) + F(flphiz, i, j, k - 1) -
                   F(flphiz, i, j, k);
        p = std::fmin(p, 1.0);
        p = std::fmax(p, 0.0);
        F(phin, i, j, k) = p;
      }
}

// solphi_mthinc3.f:1-163 -- band-test snap on the new field, clip, volume-restoring
// offset phin += offset*phin^2*(1-phin).
void orc_solphi_mthinc3(const int* ipara, const int* ni, const int* nj, const int* nk,
                        const double* dxinv, const double* dyinv, const double* dzinv,
                        const double* bet_mthinc, const double* phix, const double* phiy,
                        const double* phiz, const double* phi, double* phin) {
  (void)ipara;
  Dim D(*ni, *nj, *nk);
  const double dx = 1.0 / *dxinv, dy = 1.0 / *dyinv, dz = 1.0 / *dzinv;
  const double bet = *bet_mthinc;
  const double dcellinv = 1.0 / std::sqrt((dx * dx + dy * dy + dz * dz) / 3.0);
  const double ch = std::cosh(-bet * 1.5);
  const double eps_mthinc = bet / (2.0 * (ch * ch));
  const double eps_trunc = 0.5 * (std::tanh(-bet * 2.5) + 1.0);
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= D.nk + 1; ++k)
    for (int j = 0; j <= D.nj + 1; ++j)
      for (int i = 0; i <= D.ni + 1; ++i) {
        const double rnx = (F(phix, i - 1, j - 1, k - 1) + F(phix, i, j - 1, k - 1) + F(phix, i - 1, j, k - 1) +
                            F(phix, i, j, k - 1) + F(phix, i - 1, j - 1, k) + F(phix, i, j - 1, k) +
                            F(phix, i - 1, j, k) + F(phix, i, j, k)) * 0.125;
        const double rny = (F(phiy, i - 1, j - 1, k - 1) + F(phiy, i, j - 1, k - 1) + F(phiy, i - 1, j, k - 1) +
                            F(phiy, i, j, k - 1) + F(phiy, i - 1, j - 1, k) + F(phiy, i, j - 1, k) +
                            F(phiy, i - 1, j, k) + F(phiy, i, j, k)) * 0.125;
        const double rnz = (F(phiz, i - 1, j - 1, k - 1) + F(phiz, i, j - 1, k - 1) + F(phiz, i - 1, j, k - 1) +
                            F(phiz, i, j, k - 1) + F(phiz, i - 1, j - 1, k) + F(phiz, i, j - 1, k) +
                            F(phiz, i - 1, j, k) + F(phiz, i, j, k)) * 0.125;
        const double q00 = std::sqrt(rnx * rnx + rny * rny + rnz * rnz);
        if (q00 <= eps_mthinc * dcellinv) {
          if (F(phin, i, j, k) <= eps_trunc) F(phin, i, j, k) = 0.0;
          if (1.0 - F(phin, i, j, k) <= eps_trunc) F(phin, i, j, k) = 1.0;
        }
      }
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        double p = std::fmin(F(phin, i, j, k), 1.0);
        F(phin, i, j, k) = std::fmax(p, 0.0);
      }
  // :150-174 the four sums (a 4-double allreduce in the MPI build)
  const double sum1 = plane_sum(D, [&](int i, int j, int k) { return F(phi, i, j, k); });
  const double sum2 = plane_sum(D, [&](int i, int j, int k) { return F(phin, i, j, k); });
  const double den2 = plane_sum(D, [&](int i, int j, int k) {
    const double p = F(phin, i, j, k);
    return p * p * (1.0 - p);
  });
  const double offset = (sum1 - sum2) / (den2 + 1.0e-99);
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        double p = F(phin, i, j, k);
        p = p + offset * (p * p) * (1.0 - p);
        p = std::fmin(p, 1.0);
        F(phin, i, j, k) = std::fmax(p, 0.0);
      }
}

// summation.f:1-53 with nbub=1: qk(:,:,:,0) = qk(:,:,:,1) everywhere, clip interior.
void orc_summation(const int* ni, const int* nj, const int* nk, double* qk, const int* nbub) {
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
  double* q0 = qk;
  std::memcpy(q0, qk + n, sizeof(double) * n);
  for (int l = 2; l <= *nbub; ++l)
    for (long t = 0; t < n; ++t) q0[t] = q0[t] + qk[t + l * n];
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) F(q0, i, j, k) = std::fmin(std::fmax(F(q0, i, j, k), 0.0), 1.0);
}

// ---------------------------------------------------------------------------
// gnbc.f90:1-100 -- dynamic contact angle on the two wall planes.
void orc_gnbc(const int* nID, const int* ni, const int* nj, const int* nk, const double* uk,
              const double* wk, const double* uwall, const double* theta_0_array,
              const double* surface_tension, const double* zeta_array, double* theta_array) {
  Dim D(*ni, *nj, *nk);
  const double pi = std::acos(-1.0), eps = 1.0e-12, uw = *uwall, st = *surface_tension;
  for (int side = 0; side < 2; ++side) {
    if (nID[side == 0 ? 1 : 4] >= 0) continue;  // Y_MINUS=2, Y_PLUS=5 (1-based)
    const int ja = side == 0 ? 0 : D.nj, jb = side == 0 ? 1 : D.nj + 1;
    const int jw = side == 0 ? 1 : D.nj;
    const double us = side == 0 ? uw : -uw;
    for (int k = -2; k <= D.nk + 3; ++k)
      for (int i = -2; i <= D.ni + 3; ++i) {
        const int mi = (i + D.ni + 2) % (D.ni + 3);
        const double ucx = (F(uk, mi, ja, k) + F(uk, mi, jb, k) + F(uk, i, ja, k) + F(uk, i, jb, k)) / 4.0 + us;
        const double ucz = (F(wk, mi, ja, k) + F(wk, mi, jb, k) + F(wk, i, ja, k) + F(wk, i, jb, k)) / 4.0;
        double ucl = std::copysign(std::sqrt(ucx * ucx + ucz * ucz + eps), ucx);
        if (i <= D.ni / 2) ucl = -ucl;
        const double th0 = F(theta_0_array, i, jw, k) * (pi / 180.0);
        const double c0 = std::cos(th0);
        double ct = c0 - F(zeta_array, i, jw, k) * ucl / st;
        ct = std::fmin(1.0, std::fmax(-1.0, ct));
        F(theta_array, i, jw, k) = std::acos(ct) * (180.0 / pi);
      }
  }
}

// bnd_contact_angle.f90:1-88 -- contact-angle extrapolation of the wall ghosts.
// Columns i=-2, ni+3 and planes k=-2, nk+3 are left unchanged: there the reference
// reads outside its array (i-1=-3, i+1=ni+4, k+-1 beyond the halo); every call site
// re-applies bnd_periodic afterwards, which overwrites exactly those cells
// (main.f90:327-329, 500-502; the phi0 call at :514 leaves them unread downstream).
void orc_bnd_contact_angle(const int* nID, const int* ni, const int* nj, const int* nk, double* qk,
                           const double* theta_array, const double* dx, const double* dy,
                           const double* dz) {
  Dim D(*ni, *nj, *nk);
  const double pi = std::acos(-1.0), eps = 1.0e-20;
  const double ax = *dy / *dx, az = *dy / *dz;
  for (int side = 0; side < 2; ++side) {
    if (nID[side == 0 ? 1 : 4] >= 0) continue;
    for (int k = -1; k <= D.nk + 2; ++k)
      for (int i = -1; i <= D.ni + 2; ++i) {
        const int jw = side == 0 ? 1 : D.nj;
        const double th = F(theta_array, i, jw, k) * pi / 180.0;
        const double ct = std::cos(th), s = std::sin(th);
        const double sg = (i - D.ni / 2) >= 0 ? 1.0 : -1.0;
        double nx = sg * s * ax, nz = sg * s * az, ny = ct;
        const double nrm = std::sqrt(nx * nx + ny * ny + nz * nz + eps);
        nx = nx / nrm;
        ny = ny / nrm;
        nz = nz / nrm;
        const double g = F(qk, i, jw, k) -
                         (ny / (nx + eps)) * (F(qk, i + 1, jw, k) - F(qk, i - 1, jw, k)) * 0.5 * ax -
                         (ny / (nz + eps)) * (F(qk, i, jw, k + 1) - F(qk, i, jw, k - 1)) * 0.5 * az;
        if (side == 0) {
          F(qk, i, 0, k) = g;
          F(qk, i, -1, k) = 2.0 * F(qk, i, 0, k) - F(qk, i, 1, k);
          F(qk, i, -2, k) = 2.0 * F(qk, i, -1, k) - F(qk, i, 0, k);
        } else {
          F(qk, i, D.nj + 1, k) = g;
          F(qk, i, D.nj + 2, k) = 2.0 * F(qk, i, D.nj + 1, k) - F(qk, i, D.nj, k);
          F(qk, i, D.nj + 3, k) = 2.0 * F(qk, i, D.nj + 2, k) - F(qk, i, D.nj + 1, k);
        }
      }
  }
}

// bndu.f:1-161 -- Navier-slip wall ghosts, then the x and z halos with the
// reference's staggered index shift for u (x) and w (z).
void orc_bndu(const int* nID, const int* ni, const int* nj, const int* nk, double* uk, double* vk,
              double* wk, const double* uwall, const double* dy, const double* l1, const double* l2,
              const double* phi) {
  Dim D(*ni, *nj, *nk);
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  const double uw = *uwall, ddy = *dy;
  if (nID[1] < 0) {
    for (int k = -2; k <= NK + 3; ++k)
      for (int i = -2; i <= NI + 3; ++i) {
        const double pa = (F(phi, i, 1, k) + F(phi, (i + 1) % (NI + 3), 1, k)) / 2.0;
        const double i1 = pa / F(l1, i, 1, k), i2 = (1.0 - pa) / F(l2, i, 1, k);
        const double ls = 1.0 / (i1 + i2);
        const double c1 = (2.0 * ddy) / (2.0 * ls + ddy), c2 = (2.0 * ls - ddy) / (2.0 * ls + ddy);
        F(uk, i, 0, k) = c1 * (-uw) + c2 * F(uk, i, 1, k);
        F(uk, i, -1, k) = 2.0 * F(uk, i, 0, k) - F(uk, i, 1, k);
        F(uk, i, -2, k) = 2.0 * F(uk, i, -1, k) - F(uk, i, 0, k);
        F(vk, i, -2, k) = -F(vk, i, 2, k);
        F(vk, i, -1, k) = -F(vk, i, 1, k);
        F(vk, i, 0, k) = 0.0;
        F(wk, i, 0, k) = c2 * F(wk, i, 1, k);
        F(wk, i, -1, k) = 2.0 * F(wk, i, 0, k) - F(wk, i, 1, k);
        F(wk, i, -2, k) = 2.0 * F(wk, i, -1, k) - F(wk, i, 0, k);
      }
  }
  if (nID[4] < 0) {
    for (int k = -2; k <= NK + 3; ++k)
      for (int i = -2; i <= NI + 3; ++i) {
        const double pa = (F(phi, i, NJ, k) + F(phi, (i + 1) % (NI + 3), NJ, k)) / 2.0;
        const double i1 = pa / F(l1, i, NJ, k), i2 = (1.0 - pa) / F(l2, i, NJ, k);
        const double ls = 1.0 / (i1 + i2);
        const double c1 = (2.0 * ddy) / (2.0 * ls + ddy), c2 = (2.0 * ls - ddy) / (2.0 * ls + ddy);
        F(uk, i, NJ + 1, k) = c1 * uw + c2 * F(uk, i, NJ, k);
        F(uk, i, NJ + 2, k) = 2.0 * F(uk, i, NJ + 1, k) - F(uk, i, NJ, k);
        F(uk, i, NJ + 3, k) = 2.0 * F(uk, i, NJ + 2, k) - F(uk, i, NJ + 1, k);
        F(vk, i, NJ, k) = 0.0;
        F(vk, i, NJ + 1, k) = -F(vk, i, NJ - 1, k);
        F(vk, i, NJ + 2, k) = -F(vk, i, NJ - 2, k);
        F(vk, i, NJ + 3, k) = -F(vk, i, NJ - 3, k);
        F(wk, i, NJ + 1, k) = c2 * F(wk, i, NJ, k);
        F(wk, i, NJ + 2, k) = 2.0 * F(wk, i, NJ + 1, k) - F(wk, i, NJ, k);
        F(wk, i, NJ + 3, k) = 2.0 * F(wk, i, NJ + 2, k) - F(wk, i, NJ + 1, k);
      }
  }
  // bndu.f:98-128 x halos (u shifted by one: u(0)=u(ni+1), u(ni+1) untouched)
  for (int j = -2; j <= NJ + 3; ++j)
    for (int k = -2; k <= NK + 3; ++k) {
      F(uk, 0, j, k) = F(uk, NI + 1, j, k);
      F(uk, -1, j, k) = F(uk, NI, j, k);
      F(uk, -2, j, k) = F(uk, NI - 1, j, k);
      F(vk, 0, j, k) = F(vk, NI, j, k);
      F(vk, -1, j, k) = F(vk, NI - 1, j, k);
      F(vk, -2, j, k) = F(vk, NI - 2, j, k);
      F(wk, 0, j, k) = F(wk, NI, j, k);
      F(wk, -1, j, k) = F(wk, NI - 1, j, k);
      F(wk, -2, j, k) = F(wk, NI - 2, j, k);
      F(uk, NI + 2, j, k) = F(uk, 2, j, k);
      F(uk, NI + 3, j, k) = F(uk, 3, j, k);
      F(vk, NI + 1, j, k) = F(vk, 1, j, k);
      F(vk, NI + 2, j, k) = F(vk, 2, j, k);
      F(vk, NI + 3, j, k) = F(vk, 3, j, k);
      F(wk, NI + 1, j, k) = F(wk, 1, j, k);
      F(wk, NI + 2, j, k) = F(wk, 2, j, k);
      F(wk, NI + 3, j, k) = F(wk, 3, j, k);
    }
  // bndu.f:131-158 z halos (w shifted by one: w(0)=w(nk+1), w(nk+1) untouched)
  for (int i = -2; i <= NI + 3; ++i)
    for (int j = -2; j <= NJ + 3; ++j) {
      F(uk, i, j, 0) = F(uk, i, j, NK);
      F(uk, i, j, -1) = F(uk, i, j, NK - 1);
      F(uk, i, j, -2) = F(uk, i, j, NK - 2);
      F(vk, i, j, 0) = F(vk, i, j, NK);
      F(vk, i, j, -1) = F(vk, i, j, NK - 1);
      F(vk, i, j, -2) = F(vk, i, j, NK - 2);
      F(wk, i, j, 0) = F(wk, i, j, NK + 1);
      F(wk, i, j, -1) = F(wk, i, j, NK);
      F(wk, i, j, -2) = F(wk, i, j, NK - 1);
      F(uk, i, j, NK + 1) = F(uk, i, j, 1);
      F(uk, i, j, NK + 2) = F(uk, i, j, 2);
      F(uk, i, j, NK + 3) = F(uk, i, j, 3);
      F(vk, i, j, NK + 1) = F(vk, i, j, 1);
      F(vk, i, j, NK + 2) = F(vk, i, j, 2);
      F(vk, i, j, NK + 3) = F(vk, i, j, 3);
      F(wk, i, j, NK + 2) = F(wk, i, j, 2);
      F(wk, i, j, NK + 3) = F(wk, i, j, 3);
    }
}

// bnd_periodic.f:1-44 -- x then z periodic halos over the full other extents.
void orc_bnd_periodic(const int* ni, const int* nj, const int* nk, double* qk) {
  Dim D(*ni, *nj, *nk);
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  for (int k = -2; k <= NK + 3; ++k)
    for (int j = -2; j <= NJ + 3; ++j) {
      F(qk, -2, j, k) = F(qk, NI - 2, j, k);
      F(qk, -1, j, k) = F(qk, NI - 1, j, k);
      F(qk, 0, j, k) = F(qk, NI, j, k);
      F(qk, NI + 1, j, k) = F(qk, 1, j, k);
      F(qk, NI + 2, j, k) = F(qk, 2, j, k);
      F(qk, NI + 3, j, k) = F(qk, 3, j, k);
    }
  for (int j = -2; j <= NJ + 3; ++j)
    for (int i = -2; i <= NI + 3; ++i) {
      F(qk, i, j, -2) = F(qk, i, j, NK - 2);
      F(qk, i, j, -1) = F(qk, i, j, NK - 1);
      F(qk, i, j, 0) = F(qk, i, j, NK);
      F(qk, i, j, NK + 1) = F(qk, i, j, 1);
      F(qk, i, j, NK + 2) = F(qk, i, j, 2);
      F(qk, i, j, NK + 3) = F(qk, i, j, 3);
    }
}

// bnd_neumann.f:1-46 -- even reflection across the walls.
void orc_bnd_neumann(const int* nID, const int* ni, const int* nj, const int* nk, double* qk) {
  Dim D(*ni, *nj, *nk);
  const int NJ = D.nj;
  for (int k = -2; k <= D.nk + 3; ++k)
    for (int i = -2; i <= D.ni + 3; ++i) {
      if (nID[1] < 0) {
        F(qk, i, -2, k) = F(qk, i, 3, k);
        F(qk, i, -1, k) = F(qk, i, 2, k);
        F(qk, i, 0, k) = F(qk, i, 1, k);
      }
      if (nID[4] < 0) {
        F(qk, i, NJ + 1, k) = F(qk, i, NJ, k);
        F(qk, i, NJ + 2, k) = F(qk, i, NJ - 1, k);
        F(qk, i, NJ + 3, k) = F(qk, i, NJ - 2, k);
      }
    }
}

// bnd_comm.f:18 -- with one rank (ipara=0) the y-halo exchange does nothing.
void orc_bnd_comm(const int* ipara, const int*, const int*, const int*, const int*, int*, double*,
                  double*, double*) {
  (void)ipara;
}

// ---------------------------------------------------------------------------
// weno5.h:1-70 -- the WENO5-JS directional derivative (product-form weights).
namespace {
inline double weno5(double vel00, double dfm5, double dfm3, double dfm1, double dfp1, double dfp3,
                    double dfp5) {
  const double verysmall = 1.0e-80, d1_12 = 1.0 / 12.0;
  const double dfm_1 = dfm5 * 2.0 - dfm3 * 7.0 + dfm1 * 11.0;
  const double dfm_2 = -dfm3 + dfm1 * 5.0 + dfp1 * 2.0;
  const double dfm_3 = dfm1 * 2.0 + dfp1 * 5.0 - dfp3;
  const double dfp_1 = dfp5 * 2.0 - dfp3 * 7.0 + dfp1 * 11.0;
  const double dfp_2 = -dfp3 + dfp1 * 5.0 + dfm1 * 2.0;
  const double dfp_3 = dfp1 * 2.0 + dfm1 * 5.0 - dfm3;
  const double sm_1 = sq(dfm5 - dfm3 * 2.0 + dfm1) * 13.0 + sq(dfm5 - dfm3 * 4.0 + dfm1 * 3.0) * 3.0;
  const double sm_2 = sq(dfm3 - dfm1 * 2.0 + dfp1) * 13.0 + sq(dfm3 - dfp1) * 3.0;
  const double sm_3 = sq(dfm1 - dfp1 * 2.0 + dfp3) * 13.0 + sq(dfm1 * 3.0 - dfp1 * 4.0 + dfp3) * 3.0;
  const double sp_1 = sq(dfp5 - dfp3 * 2.0 + dfp1) * 13.0 + sq(dfp5 - dfp3 * 4.0 + dfp1 * 3.0) * 3.0;
  const double sp_2 = sq(dfp3 - dfp1 * 2.0 + dfm1) * 13.0 + sq(dfp3 - dfm1) * 3.0;
  const double sp_3 = sq(dfp1 - dfm1 * 2.0 + dfm3) * 13.0 + sq(dfp1 * 3.0 - dfm1 * 4.0 + dfm3) * 3.0;
  double am_1 = sm_2 * sm_3, am_2 = sm_1 * sm_3, am_3 = sm_1 * sm_2;
  double ap_1 = sp_2 * sp_3, ap_2 = sp_1 * sp_3, ap_3 = sp_1 * sp_2;
  am_1 = am_1 * am_1;
  am_2 = am_2 * am_2;
  am_3 = am_3 * am_3;
  ap_1 = ap_1 * ap_1;
  ap_2 = ap_2 * ap_2;
  ap_3 = ap_3 * ap_3;
  am_2 = am_2 * 6.0;
  am_3 = am_3 * 3.0;
  ap_2 = ap_2 * 6.0;
  ap_3 = ap_3 * 3.0;
  const double dam = 1.0 / (am_1 + am_2 + am_3 + verysmall);
  const double dap = 1.0 / (ap_1 + ap_2 + ap_3 + verysmall);
  const double wgm_1 = am_1 * dam, wgm_3 = am_3 * dam;
  const double wgp_1 = ap_1 * dap, wgp_3 = ap_3 * dap;
  const double wgm_2 = 1.0 - wgm_1 - wgm_3;
  const double wgp_2 = 1.0 - wgp_1 - wgp_3;
  const double velab = std::fabs(vel00);
  const double velm1 = vel00 + velab, velp1 = vel00 - velab;
  return (velm1 * (wgm_1 * dfm_1 + wgm_2 * dfm_2 + wgm_3 * dfm_3) +
          velp1 * (wgp_1 * dfp_1 + wgp_2 * dfp_2 + wgp_3 * dfp_3)) *
         d1_12;
}
}  // namespace

// cal_advu_weno5.f:1-258 -- WENO5 advection of u, v, w on their staggered points.
void orc_cal_advu_weno5(const int* ni, const int* nj, const int* nk, const double* dxinv,
                        const double* dyinv, const double* dzinv, const double* u, const double* v,
                        const double* w, double* adv_u, double* adv_v, double* adv_w) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  const long n = D.size();
  std::memset(adv_u, 0, sizeof(double) * n);
  std::memset(adv_v, 0, sizeof(double) * n);
  std::memset(adv_w, 0, sizeof(double) * n);
  // line-difference helpers along x (sx), y (sy), z (sz)
  const long sx = 1, sy = D.nx, sz = D.nx * D.ny;
  auto dir = [&](const double* q, long c, long s, double vel) {
    return weno5(vel, -q[c - 3 * s] + q[c - 2 * s], -q[c - 2 * s] + q[c - s], -q[c - s] + q[c],
                 -q[c] + q[c + s], -q[c + s] + q[c + 2 * s], -q[c + 2 * s] + q[c + 3 * s]);
  };
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        const long c = D.at(i, j, k);
        double vel, a;
        // u (:80-120)
        vel = ((F(u, i - 1, j, k) + F(u, i, j, k)) * 0.5 + (F(u, i, j, k) + F(u, i + 1, j, k)) * 0.5) * 0.5;
        a = dir(u, c, sx, vel) * dxi;
        vel = ((F(v, i, j - 1, k) + F(v, i + 1, j - 1, k)) * 0.5 + (F(v, i, j, k) + F(v, i + 1, j, k)) * 0.5) * 0.5;
        a = a + dir(u, c, sy, vel) * dyi;
        vel = ((F(w, i, j, k - 1) + F(w, i + 1, j, k - 1)) * 0.5 + (F(w, i, j, k) + F(w, i + 1, j, k)) * 0.5) * 0.5;
        a = a + dir(u, c, sz, vel) * dzi;
        adv_u[c] = a;
        // v (:147-187)
        vel = ((F(u, i - 1, j, k) + F(u, i - 1, j + 1, k)) * 0.5 + (F(u, i, j, k) + F(u, i, j + 1, k)) * 0.5) * 0.5;
        a = dir(v, c, sx, vel) * dxi;
        vel = ((F(v, i, j - 1, k) + F(v, i, j, k)) * 0.5 + (F(v, i, j, k) + F(v, i, j + 1, k)) * 0.5) * 0.5;
        a = a + dir(v, c, sy, vel) * dyi;
        vel = ((F(w, i, j, k - 1) + F(w, i, j + 1, k - 1)) * 0.5 + (F(w, i, j, k) + F(w, i, j + 1, k)) * 0.5) * 0.5;
        a = a + dir(v, c, sz, vel) * dzi;
        adv_v[c] = a;
        // w (:214-254)
        vel = ((F(u, i - 1, j, k) + F(u, i - 1, j, k + 1)) * 0.5 + (F(u, i, j, k) + F(u, i, j, k + 1)) * 0.5) * 0.5;
        a = dir(w, c, sx, vel) * dxi;
        vel = ((F(v, i, j - 1, k) + F(v, i, j - 1, k + 1)) * 0.5 + (F(v, i, j, k) + F(v, i, j, k + 1)) * 0.5) * 0.5;
        a = a + dir(w, c, sy, vel) * dyi;
        vel = ((F(w, i, j, k - 1) + F(w, i, j, k)) * 0.5 + (F(w, i, j, k) + F(w, i, j, k + 1)) * 0.5) * 0.5;
        a = a + dir(w, c, sz, vel) * dzi;
        adv_w[c] = a;
        (void)sx;
      }
}

// ---------------------------------------------------------------------------
// cal_arith_mean.f:4-29 -- q = ql*(1-phi) + qg*phi on the full halo.
void orc_cal_arith_mean(const int* ni, const int* nj, const int* nk, const double* phik,
                        const double* ql, const double* qg, double* qk) {
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
  const double a = *ql, b = *qg;
#pragma omp parallel for schedule(static)
  for (long t = 0; t < n; ++t) qk[t] = a * (1.0 - phik[t]) + b * phik[t];
}
// cal_harm_mean.f:33-58 -- q = 1/((1-phi)/ql + phi/qg).
void orc_cal_harm_mean(const int* ni, const int* nj, const int* nk, const double* phik,
                       const double* ql, const double* qg, double* qk) {
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
  const double a = *ql, b = *qg;
#pragma omp parallel for schedule(static)
  for (long t = 0; t < n; ++t) qk[t] = 1.0 / ((1.0 - phik[t]) / a + phik[t] / b);
}

// calphat.f:1-26 -- phat = 2p - po (i from -1: column -2 is left as it was).
void orc_calphat(const int* ni, const int* nj, const int* nk, const double* p, const double* po,
                 double* phat) {
  Dim D(*ni, *nj, *nk);
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= D.nk + 3; ++k)
    for (int j = -2; j <= D.nj + 3; ++j)
      for (int i = -1; i <= D.ni + 3; ++i) F(phat, i, j, k) = F(p, i, j, k) * 2.0 - F(po, i, j, k);
}

// cal_grad_prs.f:1-41 -- face gradients over -2..n+2.
void orc_cal_grad_prs(const int* ni, const int* nj, const int* nk, const double* dxinv,
                      const double* dyinv, const double* dzinv, const double* q, double* qx_u,
                      double* qy_v, double* qz_w) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= D.nk + 2; ++k)
    for (int j = -2; j <= D.nj + 2; ++j)
      for (int i = -2; i <= D.ni + 2; ++i) {
        const double q0 = F(q, i, j, k);
        F(qx_u, i, j, k) = (-q0 + F(q, i + 1, j, k)) * dxi;
        F(qy_v, i, j, k) = (-q0 + F(q, i, j + 1, k)) * dyi;
        F(qz_w, i, j, k) = (-q0 + F(q, i, j, k + 1)) * dzi;
      }
}
// cal_grad_p2uvw.f:1-47 -- same stencil as cal_grad_prs, dy from dyinv_array.
void orc_cal_grad_p2uvw(const int* ID, const int* svall, const int* ni, const int* nj, const int* nk,
                        const double* dxinv, const double* dyinv_array, const double* dzinv,
                        const double* q, double* qx_u, double* qy_v, double* qz_w) {
  (void)svall;
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dzi = *dzinv;
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= D.nk + 2; ++k)
    for (int j = -2; j <= D.nj + 2; ++j)
      for (int i = -2; i <= D.ni + 2; ++i) {
        const double dyi = dyinv_array[j + D.nj * (*ID) + 2];
        const double q0 = F(q, i, j, k);
        F(qx_u, i, j, k) = (-q0 + F(q, i + 1, j, k)) * dxi;
        F(qy_v, i, j, k) = (-q0 + F(q, i, j + 1, k)) * dyi;
        F(qz_w, i, j, k) = (-q0 + F(q, i, j, k + 1)) * dzi;
      }
}

// calsij.f:5-143 -- strain-rate components on their own ranges.
void orc_calsij(const int* ni, const int* nj, const int* nk, const double* dxinv, const double* dyinv,
                const double* dzinv, const double* uk, const double* vk, const double* wk, double* sk) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= NK + 3; ++k)
    for (int j = -2; j <= NJ + 3; ++j)
      for (int i = -2; i <= NI + 3; ++i) {
        if (i >= -1) F4(sk, i, j, k, 1) = (-F(uk, i - 1, j, k) + F(uk, i, j, k)) * dxi;
        if (j >= -1) F4(sk, i, j, k, 2) = (-F(vk, i, j - 1, k) + F(vk, i, j, k)) * dyi;
        if (i >= -1 && j >= -1 && k >= -1) F4(sk, i, j, k, 3) = (-F(wk, i, j, k - 1) + F(wk, i, j, k)) * dzi;
        if (j <= NJ + 2 && i <= NI + 2)
          F4(sk, i, j, k, 4) =
              ((-F(uk, i, j, k) + F(uk, i, j + 1, k)) * dyi + (-F(vk, i, j, k) + F(vk, i + 1, j, k)) * dxi) * 0.5;
        if (k <= NK + 2 && i <= NI + 2)
          F4(sk, i, j, k, 5) =
              ((-F(uk, i, j, k) + F(uk, i, j, k + 1)) * dzi + (-F(wk, i, j, k) + F(wk, i + 1, j, k)) * dxi) * 0.5;
        if (k <= NK + 2 && j <= NJ + 2)
          F4(sk, i, j, k, 6) =
              ((-F(vk, i, j, k) + F(vk, i, j, k + 1)) * dzi + (-F(wk, i, j, k) + F(wk, i, j + 1, k)) * dyi) * 0.5;
      }
}

// cal_arith_tau.f:7-121 -- tau = 2 mu S, off-diagonal mu the 4-cell arithmetic mean;
// cal_harm_tau.f:7-121 -- the same with the harmonic 4-cell mean 1/(sum 0.25/mu).
static void tau_impl(const int* ni, const int* nj, const int* nk, const double* s, const double* rmu,
                     double* tau, bool harm);
void orc_cal_arith_tau(const int* ni, const int* nj, const int* nk, const double* s,
                       const double* rmu, double* tau) {
  tau_impl(ni, nj, nk, s, rmu, tau, false);
}
void orc_cal_harm_tau(const int* ni, const int* nj, const int* nk, const double* s,
                      const double* rmu, double* tau) {
  tau_impl(ni, nj, nk, s, rmu, tau, true);
}
static void tau_impl(const int* ni, const int* nj, const int* nk, const double* s, const double* rmu,
                     double* tau, bool harm) {
  Dim D(*ni, *nj, *nk);
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  auto m4 = [&](double a, double b, double c, double d) {
    if (!harm) return 0.25 * a + 0.25 * b + 0.25 * c + 0.25 * d;
    return 1.0 / (0.25 / a + 0.25 / b + 0.25 / c + 0.25 / d);
  };
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= NK + 3; ++k)
    for (int j = -2; j <= NJ + 3; ++j)
      for (int i = -2; i <= NI + 3; ++i) {
        for (int l = 1; l <= 3; ++l) F4(tau, i, j, k, l) = F4(s, i, j, k, l) * F(rmu, i, j, k) * 2.0;
        if (j <= NJ + 2 && i <= NI + 2) {
          const double m = m4(F(rmu, i, j, k), F(rmu, i + 1, j, k), F(rmu, i, j + 1, k), F(rmu, i + 1, j + 1, k));
          F4(tau, i, j, k, 4) = F4(s, i, j, k, 4) * m * 2.0;
        }
        if (k <= NK + 2 && i <= NI + 2) {
          const double m = m4(F(rmu, i, j, k), F(rmu, i + 1, j, k), F(rmu, i, j, k + 1), F(rmu, i + 1, j, k + 1));
          F4(tau, i, j, k, 5) = F4(s, i, j, k, 5) * m * 2.0;
        }
        if (k <= NK + 2 && j <= NJ + 2) {
          const double m = m4(F(rmu, i, j, k), F(rmu, i, j + 1, k), F(rmu, i, j, k + 1), F(rmu, i, j + 1, k + 1));
          F4(tau, i, j, k, 6) = F4(s, i, j, k, 6) * m * 2.0;
        }
      }
}

// cal_div_tensor.f:1-89 -- divergence of tau on u, v, w points.
void orc_cal_div_tensor(const int* ni, const int* nj, const int* nk, const double* dxinv,
                        const double* dyinv, const double* dzinv, const double* tauk, double* uk,
                        double* vk, double* wk) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  const long n = D.size();
  std::memset(uk, 0, sizeof(double) * n);
  std::memset(vk, 0, sizeof(double) * n);
  std::memset(wk, 0, sizeof(double) * n);
  const double* t = tauk;
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= NK + 3; ++k)
    for (int j = -2; j <= NJ + 3; ++j)
      for (int i = -2; i <= NI + 3; ++i) {
        if (k >= -1 && j >= -1 && i <= NI + 2)
          F(uk, i, j, k) = (-F4(t, i, j, k, 1) + F4(t, i + 1, j, k, 1)) * dxi +
                           (-F4(t, i, j - 1, k, 4) + F4(t, i, j, k, 4)) * dyi +
                           (-F4(t, i, j, k - 1, 5) + F4(t, i, j, k, 5)) * dzi;
        if (k >= -1 && j <= NJ + 2 && i >= -1)
          F(vk, i, j, k) = (-F4(t, i - 1, j, k, 4) + F4(t, i, j, k, 4)) * dxi +
                           (-F4(t, i, j, k, 2) + F4(t, i, j + 1, k, 2)) * dyi +
                           (-F4(t, i, j, k - 1, 6) + F4(t, i, j, k, 6)) * dzi;
        if (k <= NK + 2 && j >= -1 && i >= -1)
          F(wk, i, j, k) = (-F4(t, i - 1, j, k, 5) + F4(t, i, j, k, 5)) * dxi +
                           (-F4(t, i, j - 1, k, 6) + F4(t, i, j, k, 6)) * dyi +
                           (-F4(t, i, j, k, 3) + F4(t, i, j, k + 1, 3)) * dzi;
      }
}

// calrn.f:1-91 -- unit normal averaged over the 8 (ip,jp,kp)-offset vertices.
void orc_calrn(const int* ni, const int* nj, const int* nk, const double* dxinv, const double* dyinv,
               const double* dzinv, const int* ip, const int* jp, const int* kp, const double* phix,
               const double* phiy, const double* phiz, double* rn) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  const double verysmall = std::sqrt(dxi * dxi + dyi * dyi + dzi * dzi) * 1.0e-30;
  std::memset(rn, 0, sizeof(double) * 3 * D.size());
  const int IP = *ip, JP = *jp, KP = *kp;
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= D.nk + 3 - KP; ++k)
    for (int j = -2; j <= D.nj + 3 - JP; ++j)
      for (int i = -2; i <= D.ni + 3 - IP; ++i) {
        const int ii = i + IP, jj = j + JP, kk = k + KP;
        const double rx = (F(phix, i, j, k) + F(phix, ii, j, k) + F(phix, i, jj, k) + F(phix, ii, jj, k) +
                           F(phix, i, j, kk) + F(phix, ii, j, kk) + F(phix, i, jj, kk) + F(phix, ii, jj, kk)) * 0.125;
        const double ry = (F(phiy, i, j, k) + F(phiy, ii, j, k) + F(phiy, i, jj, k) + F(phiy, ii, jj, k) +
                           F(phiy, i, j, kk) + F(phiy, ii, j, kk) + F(phiy, i, jj, kk) + F(phiy, ii, jj, kk)) * 0.125;
        const double rz = (F(phiz, i, j, k) + F(phiz, ii, j, k) + F(phiz, i, jj, k) + F(phiz, ii, jj, k) +
                           F(phiz, i, j, kk) + F(phiz, ii, j, kk) + F(phiz, i, jj, kk) + F(phiz, ii, jj, kk)) * 0.125;
        const double a = std::sqrt(rx * rx + ry * ry + rz * rz) + verysmall;
        const double ainv = 1.0 / a;
        F4(rn, ii, jj, kk, 1) = rx * ainv;
        F4(rn, ii, jj, kk, 2) = ry * ainv;
        F4(rn, ii, jj, kk, 3) = rz * ainv;
      }
}

// calrkap.f:1-101 -- curvature (divergence of the normal) on u, v, w points.
void orc_calrkap(const int* ni, const int* nj, const int* nk, const double* dxinv,
                 const double* dyinv, const double* dzinv, const double* rn_pp, const double* rn_12,
                 const double* rn_13, const double* rn_23, double* rkap) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  std::memset(rkap, 0, sizeof(double) * 3 * D.size());
#pragma omp parallel for schedule(static)
  for (int k = -2; k <= NK + 3; ++k)
    for (int j = -2; j <= NJ + 3; ++j)
      for (int i = -2; i <= NI + 3; ++i) {
        if (k >= -1 && j >= -1 && i <= NI + 2)
          F4(rkap, i, j, k, 1) = (-F4(rn_pp, i, j, k, 1) + F4(rn_pp, i + 1, j, k, 1)) * dxi +
                                 (-F4(rn_12, i, j - 1, k, 2) + F4(rn_12, i, j, k, 2)) * dyi +
                                 (-F4(rn_13, i, j, k - 1, 3) + F4(rn_13, i, j, k, 3)) * dzi;
        if (k >= -1 && j <= NJ + 2 && i >= -1)
          F4(rkap, i, j, k, 2) = (-F4(rn_12, i - 1, j, k, 1) + F4(rn_12, i, j, k, 1)) * dxi +
                                 (-F4(rn_pp, i, j, k, 2) + F4(rn_pp, i, j + 1, k, 2)) * dyi +
                                 (-F4(rn_23, i, j, k - 1, 3) + F4(rn_23, i, j, k, 3)) * dzi;
        if (k <= NK + 2 && j >= -1 && i >= -1)
          F4(rkap, i, j, k, 3) = (-F4(rn_13, i - 1, j, k, 1) + F4(rn_13, i, j, k, 1)) * dxi +
                                 (-F4(rn_23, i, j - 1, k, 2) + F4(rn_23, i, j, k, 2)) * dyi +
                                 (-F4(rn_pp, i, j, k, 3) + F4(rn_pp, i, j, k + 1, 3)) * dzi;
      }
}

// calfst.f:7-49 -- CSF force -(2 sigma/(rhol+rhog)) kappa grad(phi).
void orc_calfst(const int* ni, const int* nj, const int* nk, const double* rhol, const double* rhog,
                const double* surface_tension, const double* phix_u, const double* phiy_v,
                const double* phiz_w, const double* rkap, double* fst_u, double* fst_v,
                double* fst_w) {
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
  const double st = 2.0 * (*surface_tension) / (*rhol + *rhog);
#pragma omp parallel for schedule(static)
  for (long t = 0; t < n; ++t) {
    fst_u[t] = -st * rkap[t] * phix_u[t];
    fst_v[t] = -st * rkap[t + n] * phiy_v[t];
    fst_w[t] = -st * rkap[t + 2 * n] * phiz_w[t];
  }
}
// sum_fst.f:1-37
void orc_sum_fst(const int* ni, const int* nj, const int* nk, const double* fst_u,
                 const double* fst_v, const double* fst_w, double* sum_fst_u, double* sum_fst_v,
                 double* sum_fst_w) {
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
#pragma omp parallel for schedule(static)
  for (long t = 0; t < n; ++t) {
    sum_fst_u[t] = sum_fst_u[t] + fst_u[t];
    sum_fst_v[t] = sum_fst_v[t] + fst_v[t];
    sum_fst_w[t] = sum_fst_w[t] + fst_w[t];
  }
}
// init_q.f:1-29
void orc_init_q(const int* ni, const int* nj, const int* nk, double* q1, double* q2, double* q3) {
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
  std::memset(q1, 0, sizeof(double) * n);
  std::memset(q2, 0, sizeof(double) * n);
  std::memset(q3, 0, sizeof(double) * n);
}
// cal_av.f:1-40 -- interior mean (a 1-double allreduce in the MPI build).
void orc_cal_av(const int* ipara, const int* ndiv, const int* ni, const int* nj, const int* nk,
                const double* q, double* av) {
  (void)ipara;
  Dim D(*ni, *nj, *nk);
  const double s = plane_sum(D, [&](int i, int j, int k) { return F(q, i, j, k); });
  *av = s / (double)((long)D.ni * D.nj * D.nk * (*ndiv));
}

// cal_srcu.f:1-141 -- momentum right-hand side (AB2 advection, CN viscosity, CSF).
void orc_cal_srcu(const int* nID, const int* ni, const int* nj, const int* nk, const double* rho_av,
                  const double* dt, const double* grvb, const double* grvp, const double* u,
                  const double* v, const double* w, const double* rho, const double* rhon,
                  const double* adv_u, const double* adv_v, const double* adv_w,
                  const double* adv_uo, const double* adv_vo, const double* adv_wo,
                  const double* prs_u, const double* prs_v, const double* prs_w,
                  const double* vis_u, const double* vis_v, const double* vis_w,
                  const double* fst_u, const double* fst_v, const double* fst_w,
                  const double* fst_un, const double* fst_vn, const double* fst_wn,
                  double* src_u, double* src_v, double* src_w) {
  (void)rho_av;
  Dim D(*ni, *nj, *nk);
  const int jen = nID[4] < 0 ? D.nj - 1 : D.nj;
  const double dtinv = 1.0 / (*dt), gb = *grvb, gp = *grvp;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        const long c = D.at(i, j, k);
        double r = (F(rho, i, j, k) + F(rho, i + 1, j, k) + F(rhon, i, j, k) + F(rhon, i + 1, j, k)) * 0.25;
        src_u[c] = u[c] * dtinv - adv_u[c] * 1.5 + adv_uo[c] * 0.5 - prs_u[c] / r + vis_u[c] / r * 0.5 +
                   fst_u[c] * 0.5 + fst_un[c] * 0.5 + gb;
        if (j <= jen) {
          r = (F(rho, i, j, k) + F(rho, i, j + 1, k) + F(rhon, i, j, k) + F(rhon, i, j + 1, k)) * 0.25;
          src_v[c] = v[c] * dtinv - adv_v[c] * 1.5 + adv_vo[c] * 0.5 - prs_v[c] / r + vis_v[c] / r * 0.5 +
                     fst_v[c] * 0.5 + fst_vn[c] * 0.5 + gp;
        }
        r = (F(rho, i, j, k) + F(rho, i, j, k + 1) + F(rhon, i, j, k) + F(rhon, i, j, k + 1)) * 0.25;
        src_w[c] = w[c] * dtinv - adv_w[c] * 1.5 + adv_wo[c] * 0.5 - prs_w[c] / r + vis_w[c] / r * 0.5 +
                   fst_w[c] * 0.5 + fst_wn[c] * 0.5;
      }
}

// cpy.f:1-24
void orc_cpy(const int* ni, const int* nj, const int* nk, const double* q1, double* q2) {
  Dim D(*ni, *nj, *nk);
  std::memcpy(q2, q1, sizeof(double) * D.size());
}

// ---------------------------------------------------------------------------
// cal_arith_coef_vis.f:6-411 (harmonic=0) / cal_harm_coef_vis.f (harmonic=1):
// the 45 viscous coefficient arrays, coef[] in the reference argument order.
void orc_cal_arith_coef_vis_v(const int* ni, const int* nj, const int* nk, const double* dxinv,
                              const double* dyinv, const double* dzinv, const double* rmuk,
                              double* const* coef, int harmonic) {
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  const long n = D.size();
  for (int c = 0; c < 45; ++c) std::memset(coef[c], 0, sizeof(double) * n);
  auto m4 = [&](double a, double b, double c, double d) {
    if (!harmonic) return 0.25 * (a + b + c + d);
    return 4.0 / (1.0 / a + 1.0 / b + 1.0 / c + 1.0 / d);
  };
  const double dx2 = dxi * dxi, dy2 = dyi * dyi, dz2 = dzi * dzi;
  const double dxy = dxi * dyi, dxz = dxi * dzi, dyz = dyi * dzi;
#pragma omp parallel for schedule(static)
  for (int k = -1; k <= D.nk + 2; ++k)
    for (int j = -1; j <= D.nj + 2; ++j)
      for (int i = -1; i <= D.ni + 2; ++i) {
        const long t = D.at(i, j, k);
        const double* r = rmuk;
        // u coefficients (:184-235)
        {
          const double xm = F(r, i, j, k), xp = F(r, i + 1, j, k);
          const double ym = m4(F(r, i, j - 1, k), F(r, i + 1, j - 1, k), F(r, i, j, k), F(r, i + 1, j, k));
          const double yp = m4(F(r, i, j, k), F(r, i + 1, j, k), F(r, i, j + 1, k), F(r, i + 1, j + 1, k));
          const double zm = m4(F(r, i, j, k - 1), F(r, i + 1, j, k - 1), F(r, i, j, k), F(r, i + 1, j, k));
          const double zp = m4(F(r, i, j, k), F(r, i + 1, j, k), F(r, i, j, k + 1), F(r, i + 1, j, k + 1));
          const double b = dz2 * zm, s = dy2 * ym, w = dx2 * xm * 2.0, e = dx2 * xp * 2.0, nn = dy2 * yp,
                       tt = dz2 * zp;
          coef[0][t] = w; coef[1][t] = e; coef[2][t] = s; coef[3][t] = nn; coef[4][t] = b; coef[5][t] = tt;
          coef[6][t] = b + s + w + e + nn + tt;
          coef[7][t] = dxy * ym; coef[8][t] = -(dxy * ym); coef[9][t] = -(dxy * yp); coef[10][t] = dxy * yp;
          coef[11][t] = dxz * zm; coef[12][t] = -(dxz * zm); coef[13][t] = -(dxz * zp); coef[14][t] = dxz * zp;
        }
        // v coefficients (:270-321)
        {
          const double xm = m4(F(r, i - 1, j, k), F(r, i, j, k), F(r, i - 1, j + 1, k), F(r, i, j + 1, k));
          const double xp = m4(F(r, i, j, k), F(r, i + 1, j, k), F(r, i, j + 1, k), F(r, i + 1, j + 1, k));
          const double ym = F(r, i, j, k), yp = F(r, i, j + 1, k);
          const double zm = m4(F(r, i, j, k - 1), F(r, i, j + 1, k - 1), F(r, i, j, k), F(r, i, j + 1, k));
          const double zp = m4(F(r, i, j, k), F(r, i, j + 1, k), F(r, i, j, k + 1), F(r, i, j + 1, k + 1));
          const double b = dz2 * zm, s = dy2 * ym * 2.0, w = dx2 * xm, e = dx2 * xp, nn = dy2 * yp * 2.0,
                       tt = dz2 * zp;
          coef[15][t] = w; coef[16][t] = e; coef[17][t] = s; coef[18][t] = nn; coef[19][t] = b; coef[20][t] = tt;
          coef[21][t] = b + s + w + e + nn + tt;
          coef[22][t] = dxy * xm; coef[23][t] = -(dxy * xm); coef[24][t] = -(dxy * xp); coef[25][t] = dxy * xp;
          coef[26][t] = dyz * zm; coef[27][t] = -(dyz * zm); coef[28][t] = -(dyz * zp); coef[29][t] = dyz * zp;
        }
        // w coefficients (:356-407)
        {
          const double xm = m4(F(r, i - 1, j, k), F(r, i, j, k), F(r, i - 1, j, k + 1), F(r, i, j, k + 1));
          const double xp = m4(F(r, i, j, k), F(r, i + 1, j, k), F(r, i, j, k + 1), F(r, i + 1, j, k + 1));
          const double ym = m4(F(r, i, j - 1, k), F(r, i, j, k), F(r, i, j - 1, k + 1), F(r, i, j, k + 1));
          const double yp = m4(F(r, i, j, k), F(r, i, j + 1, k), F(r, i, j, k + 1), F(r, i, j + 1, k + 1));
          const double zm = F(r, i, j, k), zp = F(r, i, j, k + 1);
          const double b = dz2 * zm * 2.0, s = dy2 * ym, w = dx2 * xm, e = dx2 * xp, nn = dy2 * yp,
                       tt = dz2 * zp * 2.0;
          coef[30][t] = w; coef[31][t] = e; coef[32][t] = s; coef[33][t] = nn; coef[34][t] = b; coef[35][t] = tt;
          coef[36][t] = b + s + w + e + nn + tt;
          coef[37][t] = dxz * xm; coef[38][t] = -(dxz * xm); coef[39][t] = -(dxz * xp); coef[40][t] = dxz * xp;
          coef[41][t] = dyz * ym; coef[42][t] = -(dyz * ym); coef[43][t] = -(dyz * yp); coef[44][t] = dyz * yp;
        }
      }
}

// solu_sor4.f:1-308 -- 8-colour Gauss-Seidel (omega=1) sweeps for u, then v, then w,
// with the wall/halo refresh after every even colour; at most 21 outer iterations,
// stop when the RMS update falls to 1e-3 of the first iteration's.
int orc_solu_sor4_v(const int* nID, const int* ni, const int* nj, const int* nk, const double* dt,
                    const double* rho, const double* rhon, const double* const* cf,
                    const double* src_u, const double* src_v, const double* src_w, double* un,
                    double* vn, double* wn, const double* uwall, const double* dy,
                    const double* l1, const double* l2, const double* phi, double* err_out) {
  Dim D(*ni, *nj, *nk);
  static const int isor[8] = {1, 2, 1, 2, 1, 2, 2, 1};
  static const int jsor[8] = {1, 2, 1, 2, 2, 1, 1, 2};
  static const int ksor[8] = {1, 2, 2, 1, 1, 2, 1, 2};
  const double dtinv = 1.0 / (*dt);
  const int jen = nID[4] < 0 ? D.nj - 1 : D.nj;
  const long sx = 1, sy = D.nx, sz = D.nx * D.ny;
  double err0 = 0.0, err = 0.0;
  int lp;
  const int lmax = g_sor_max - 1;
  std::vector<double> part(D.nk + 1);
  for (lp = 0; lp <= lmax; ++lp) {
    double esum = 0.0;
    for (int comp = 0; comp < 3; ++comp) {
      double* q = comp == 0 ? un : (comp == 1 ? vn : wn);
      const double* src = comp == 0 ? src_u : (comp == 1 ? src_v : src_w);
      const long so = comp == 0 ? sx : (comp == 1 ? sy : sz);  // rho averaging offset
      const double* const* c = cf + 15 * comp;
      const int jmax = comp == 1 ? jen : D.nj;
      for (int col = 0; col < 8; ++col) {
        std::fill(part.begin(), part.end(), 0.0);
#pragma omp parallel for schedule(static)
        for (int k = ksor[col]; k <= D.nk; k += 2) {
          double es = 0.0;
          for (int j = jsor[col]; j <= jmax; j += 2)
            for (int i = isor[col]; i <= D.ni; i += 2) {
              const long t = D.at(i, j, k);
              const double r = (rho[t] + rho[t + so] + rhon[t] + rhon[t + so]) * 0.25;
              double visn;
              if (comp == 0) {
                visn = (c[4][t] * un[t - sz] + c[2][t] * un[t - sy] + c[0][t] * un[t - sx] + c[1][t] * un[t + sx] +
                        c[3][t] * un[t + sy] + c[5][t] * un[t + sz] + c[7][t] * vn[t - sy] +
                        c[8][t] * vn[t + sx - sy] + c[9][t] * vn[t] + c[10][t] * vn[t + sx] +
                        c[11][t] * wn[t - sz] + c[12][t] * wn[t + sx - sz] + c[13][t] * wn[t] +
                        c[14][t] * wn[t + sx]) / r;
              } else if (comp == 1) {
                visn = (c[4][t] * vn[t - sz] + c[2][t] * vn[t - sy] + c[0][t] * vn[t - sx] + c[1][t] * vn[t + sx] +
                        c[3][t] * vn[t + sy] + c[5][t] * vn[t + sz] + c[7][t] * un[t - sx] + c[9][t] * un[t] +
                        c[8][t] * un[t - sx + sy] + c[10][t] * un[t + sy] + c[11][t] * wn[t - sz] +
                        c[12][t] * wn[t + sy - sz] + c[13][t] * wn[t] + c[14][t] * wn[t + sy]) / r;
              } else {
                visn = (c[4][t] * wn[t - sz] + c[2][t] * wn[t - sy] + c[0][t] * wn[t - sx] + c[1][t] * wn[t + sx] +
                        c[3][t] * wn[t + sy] + c[5][t] * wn[t + sz] + c[7][t] * un[t - sx] + c[9][t] * un[t] +
                        c[8][t] * un[t - sx + sz] + c[10][t] * un[t + sz] + c[11][t] * vn[t - sy] +
                        c[13][t] * vn[t] + c[12][t] * vn[t - sy + sz] + c[14][t] * vn[t + sz]) / r;
              }
              const double d = (visn * 0.5 + src[t]) / (dtinv + c[6][t] / r * 0.5) - q[t];
              q[t] = q[t] + d;
              es = es + d * d;
            }
          part[k] = es;
        }
        for (int k = 1; k <= D.nk; ++k) esum = esum + part[k];
        if (col % 2 == 1) {
          orc_bndu(nID, ni, nj, nk, un, vn, wn, uwall, dy, l1, l2, phi);
          orc_bnd_periodic(ni, nj, nk, q);
        }
      }
    }
    err = std::sqrt(esum / (double)((long)D.ni * D.nj * D.nk)) + 1.0e-99;
    if (lp == 0) err0 = err;
    if (err / err0 <= g_sor_tol) break;
  }
  if (err_out) *err_out = err / err0;
  return (lp <= lmax ? lp : lmax) + 1;
}

// The stop rule of solu_sor4.f:291-293 is err/err0 <= 1e-3 within 21 iterations;
// the adjoint's finite-difference checks need the solve converged much further.
void orc_set_sor(double tol, int max_iter) {
  g_sor_tol = tol;
  g_sor_max = max_iter;
}

// ---------------------------------------------------------------------------
// caldiv.f:1-70 -- div/dt over -1..n+3 and its interior RMS.
void orc_caldiv(const int* ipara, const int* ndiv, const int* ni, const int* nj, const int* nk,
                const double* dxinv, const double* dyinv, const double* dzinv, const double* dt,
                const double* uk, const double* vk, const double* wk, double* div, double* err_div) {
  (void)ipara;
  Dim D(*ni, *nj, *nk);
  const double dxi = *dxinv, dyi = *dyinv, dzi = *dzinv, dtinv = 1.0 / (*dt);
#pragma omp parallel for schedule(static)
  for (int k = -1; k <= D.nk + 3; ++k)
    for (int j = -1; j <= D.nj + 3; ++j)
      for (int i = -1; i <= D.ni + 3; ++i)
        F(div, i, j, k) = ((-F(uk, i - 1, j, k) + F(uk, i, j, k)) * dxi + (-F(vk, i, j - 1, k) + F(vk, i, j, k)) * dyi +
                           (-F(wk, i, j, k - 1) + F(wk, i, j, k)) * dzi) * dtinv;
  const double s = plane_sum(D, [&](int i, int j, int k) { return sq(F(div, i, j, k)); });
  *err_div = std::sqrt(s / (double)((long)D.ni * D.nj * D.nk * (*ndiv))) + 1.0e-99;
}

// cal_coef_prs.f:5-57
void orc_cal_coef_prs(const int* nj, const double* rho, const double* dxinv, const double* dyinv,
                      const double* dzinv, double* aw, double* ae, double* as, double* an,
                      double* ab, double* at, double* ap) {
  const int NJ = *nj;
  const double r = *rho, dxi = *dxinv, dyi = *dyinv, dzi = *dzinv;
  for (int j = 1; j <= NJ; ++j) {
    const int t = j + 2;
    aw[t] = dxi * dxi / r;
    ae[t] = dxi * dxi / r;
    as[t] = dyi * dyi / r;
    an[t] = dyi * dyi / r;
    ab[t] = dzi * dzi / r;
    at[t] = dzi * dzi / r;
    ap[t] = aw[t] + ae[t] + as[t] + an[t] + ab[t] + at[t];
  }
  ap[1 + 2] = ap[1 + 2] - as[1 + 2];
  as[1 + 2] = 0.0;
  ap[NJ + 2] = ap[NJ + 2] - an[NJ + 2];
  an[NJ + 2] = 0.0;
}
// cal_coef_solp_fft.f:5-42
void orc_cal_coef_solp_fft(const int* nj, const double* as_p, const double* an_p, double* as_f,
                           double* an_f, double* ap_f) {
  const int NJ = *nj;
  for (int j = 1; j <= NJ; ++j) {
    const int t = j + 2;
    as_f[t] = as_p[t];
    an_f[t] = an_p[t];
    ap_f[t] = as_f[t] + an_f[t];
  }
  ap_f[1 + 2] = ap_f[1 + 2] - as_f[1 + 2];
  as_f[1 + 2] = 0.0;
  ap_f[NJ + 2] = ap_f[NJ + 2] - an_f[NJ + 2];
  an_f[NJ + 2] = 0.0;
}

// The oracle's own FFT (the reference calls the vendored Numerical Recipes fourn.f,
// whose arithmetic is the DFT X_m = sum_n x_n exp(sign*2*pi*i*m*n/N); this is an
// independent radix-2 decimation-in-time restatement of that DFT, pinned against
// numpy.fft in tests/test_oracle_pins.py).
namespace {
void fft1d(double* re, double* im, int n, int sign) {
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  const double two_pi = 6.283185307179586476925286766559;
  for (int len = 2; len <= n; len <<= 1) {
    const int h = len >> 1;
    for (int m = 0; m < h; ++m) {
      const double ang = sign * two_pi * (double)m / (double)len;
      const double wr = std::cos(ang), wi = std::sin(ang);
      for (int s = 0; s < n; s += len) {
        const int a = s + m, b = a + h;
        const double tr = wr * re[b] - wi * im[b];
        const double ti = wr * im[b] + wi * re[b];
        re[b] = re[a] - tr;
        im[b] = im[a] - ti;
        re[a] = re[a] + tr;
        im[a] = im[a] + ti;
      }
    }
  }
}
}  // namespace

void orc_fft2d(double* data, int n1, int n2, int sign) {
  std::vector<double> re(std::max(n1, n2)), im(std::max(n1, n2));
  for (int r = 0; r < n2; ++r) {
    for (int c = 0; c < n1; ++c) {
      re[c] = data[2 * ((long)r * n1 + c)];
      im[c] = data[2 * ((long)r * n1 + c) + 1];
    }
    fft1d(re.data(), im.data(), n1, sign);
    for (int c = 0; c < n1; ++c) {
      data[2 * ((long)r * n1 + c)] = re[c];
      data[2 * ((long)r * n1 + c) + 1] = im[c];
    }
  }
  for (int c = 0; c < n1; ++c) {
    for (int r = 0; r < n2; ++r) {
      re[r] = data[2 * ((long)r * n1 + c)];
      im[r] = data[2 * ((long)r * n1 + c) + 1];
    }
    fft1d(re.data(), im.data(), n2, sign);
    for (int r = 0; r < n2; ++r) {
      data[2 * ((long)r * n1 + c)] = re[r];
      data[2 * ((long)r * n1 + c) + 1] = im[r];
    }
  }
}

// solp_fft_tdma1.f:4-50 -- per y-plane forward 2-D DFT of div over (x,z), /(ni*nk),
// stored at centred wavenumbers phir(-ni/2:ni/2-1, 1:nj, -nk/2:nk/2-1).
void orc_solp_fft_tdma1(const int* ni, const int* nj, const int* nk, double* fftdata,
                        const double* div, double* phir_r, double* phir_i) {
  Dim D(*ni, *nj, *nk);
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  const long pl = 2L * NI * NK;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= NJ; ++j) {
    double* fd = fftdata + (long)(j - 1) * pl;
    for (int k = 0; k < NK; ++k)
      for (int i = 0; i < NI; ++i) {
        const long l = (long)NI * k + i;
        fd[2 * l] = F(div, i + 1, j, k + 1);
        fd[2 * l + 1] = 0.0;
      }
    orc_fft2d(fd, NI, NK, -1);
    for (int k = -NK / 2; k <= NK / 2 - 1; ++k) {
      const int kk = (k + NK) % NK;
      for (int i = -NI / 2; i <= NI / 2 - 1; ++i) {
        const int ii = (i + NI) % NI;
        const long l = (long)NI * kk + ii;
        const long t = (long)(i + NI / 2) + (long)NI * ((long)(j - 1) + (long)NJ * (long)(k + NK / 2));
        phir_r[t] = fd[2 * l] / (double)((long)NI * NK);
        phir_i[t] = fd[2 * l + 1] / (double)((long)NI * NK);
      }
    }
  }
}

// trans_r2w.f:23-38 / trans_w2r.f:23-38 -- the serial (ipara=0) branch: a relabelling
// k -> k - nk/2 - 1 of the third index; with one rank phir and phiw hold the same
// numbers in the same order, so this is a plain copy.
void orc_trans_r2w(const int* ipara, const int*, const int* ndiv, const int* svall, int*, double*,
                   double*, const double* r, double* w) {
  (void)ipara;
  (void)ndiv;
  const long n = (long)svall[0] * svall[1] * svall[2];
  std::memcpy(w, r, sizeof(double) * n);
}
void orc_trans_w2r(const int* ipara, const int*, const int* ndiv, const int* svall, int*, double*,
                   double*, const double* w, double* r) {
  (void)ipara;
  (void)ndiv;
  const long n = (long)svall[0] * svall[1] * svall[2];
  std::memcpy(r, w, sizeof(double) * n);
}

// solp_fft_tdma2.f:4-91 -- per (kx,kz) mode, Thomas solve along y with the
// regularised pivot -d/(d^2+1e-99) (phiw layout (-ni/2:ni/2-1, nj, nk)).
void orc_solp_fft_tdma2(const int* ID, const int* ndiv, const int* svall, const double* rho,
                        const double* dxinv, const double* dzinv, const double* as_f,
                        const double* an_f, const double* ap_f, double* atdma, double* btdma_r,
                        double* btdma_i, double* phiw_r, double* phiw_i) {
  (void)atdma;
  (void)btdma_r;
  (void)btdma_i;
  const int NI = svall[0], NJ = svall[1], NK = svall[2] / (*ndiv);
  const double pi = std::atan(1.0) * 4.0;
  const double dx2r = (*dxinv) * (*dxinv) / (*rho), dz2r = (*dzinv) * (*dzinv) / (*rho);
  const double pi2_ni = pi * 2.0 / (double)svall[0], pi2_nk = pi * 2.0 / (double)svall[2];
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= NK; ++k) {
    std::vector<double> at(NJ + 2), br(NJ + 2), bi(NJ + 2);
    for (int i = -NI / 2; i <= NI / 2 - 1; ++i) {
      const double c1x = std::cos((double)i * pi2_ni) * 2.0;
      const double c1z = std::cos((double)(k + (*ID) * NK - svall[2] / 2 - 1) * pi2_nk) * 2.0;
      at[0] = 0.0;
      br[0] = 0.0;
      bi[0] = 0.0;
      auto P = [&](int j) { return (long)(i + NI / 2) + (long)NI * ((long)(j - 1) + (long)NJ * (long)(k - 1)); };
      for (int j = 1; j <= NJ; ++j) {
        const double ap = ap_f[j + 2] + dx2r * (2.0 - c1x) + dz2r * (2.0 - c1z);
        const double d00 = -ap + as_f[j + 2] * at[j - 1];
        const double apinv = -d00 / (d00 * d00 + 1.0e-99);
        at[j] = apinv * an_f[j + 2];
        br[j] = apinv * (-phiw_r[P(j)] + as_f[j + 2] * br[j - 1]);
        bi[j] = apinv * (-phiw_i[P(j)] + as_f[j + 2] * bi[j - 1]);
      }
      phiw_r[P(NJ)] = br[NJ];
      phiw_i[P(NJ)] = bi[NJ];
      for (int j = NJ - 1; j >= 1; --j) {
        phiw_r[P(j)] = br[j] + at[j] * phiw_r[P(j + 1)];
        phiw_i[P(j)] = bi[j] + at[j] * phiw_i[P(j + 1)];
      }
    }
  }
}

// solp_fft_tdma3.f:4-48 -- inverse 2-D DFT (sign +1, unnormalised); real part -> dp.
void orc_solp_fft_tdma3(const int* ni, const int* nj, const int* nk, double* fftdata,
                        const double* phir_r, const double* phir_i, double* dp) {
  Dim D(*ni, *nj, *nk);
  const int NI = D.ni, NJ = D.nj, NK = D.nk;
  const long pl = 2L * NI * NK;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= NJ; ++j) {
    double* fd = fftdata + (long)(j - 1) * pl;
    for (int k = -NK / 2; k <= NK / 2 - 1; ++k) {
      const int kk = (k + NK) % NK;
      for (int i = -NI / 2; i <= NI / 2 - 1; ++i) {
        const int ii = (i + NI) % NI;
        const long l = (long)NI * kk + ii;
        const long t = (long)(i + NI / 2) + (long)NI * ((long)(j - 1) + (long)NJ * (long)(k + NK / 2));
        fd[2 * l] = phir_r[t];
        fd[2 * l + 1] = phir_i[t];
      }
    }
    orc_fft2d(fd, NI, NK, +1);
    for (int k = 0; k < NK; ++k)
      for (int i = 0; i < NI; ++i) F(dp, i + 1, j, k + 1) = fd[2 * ((long)NI * k + i)];
  }
}

// solp_fft_tdma4.f:4-98 -- RMS Poisson residual vs RMS rhs (monitor only).
void orc_solp_fft_tdma4_v(const int* ni, const int* nj, const int* nk, const double* rho,
                          const double* dxinv, const double* dyinv, const double* dzinv,
                          const double* div, const double* dp, double* err_out, double* err0_out) {
  Dim D(*ni, *nj, *nk);
  const double r = *rho;
  const double aw = (*dxinv) * (*dxinv) / r, ae = aw, as = (*dyinv) * (*dyinv) / r, an = as,
               ab = (*dzinv) * (*dzinv) / r, at = ab;
  const double ap = aw + ae + as + an + ab + at;
  const double e0 = plane_sum(D, [&](int i, int j, int k) { return sq(F(div, i, j, k)); });
  const double e = plane_sum(D, [&](int i, int j, int k) {
    const double d = F(dp, i, j, k - 1) * ab + F(dp, i, j - 1, k) * as + F(dp, i - 1, j, k) * aw -
                     F(dp, i, j, k) * ap + F(dp, i + 1, j, k) * ae + F(dp, i, j + 1, k) * an +
                     F(dp, i, j, k + 1) * at - F(div, i, j, k);
    return d * d;
  });
  const double N = (double)((long)D.ni * D.nj * D.nk);
  *err0_out = std::sqrt(e0 / N) + 1.0e-99;
  *err_out = std::sqrt(e / N) + 1.0e-99;
}

// bnd_avzero.f:1-27 -- subtract the interior mean from every element.
void orc_bnd_avzero(const int* ipara, const int* ndiv, const int* ni, const int* nj, const int* nk,
                    double* q) {
  double av;
  orc_cal_av(ipara, ndiv, ni, nj, nk, q, &av);
  Dim D(*ni, *nj, *nk);
  const long n = D.size();
#pragma omp parallel for schedule(static)
  for (long t = 0; t < n; ++t) q[t] = q[t] - av;
}

// corunp_explicit.f:1-78 -- velocity correction and pn = phat + dp.
void orc_corunp_explicit(const int* nID, const int* ni, const int* nj, const int* nk,
                         const double* rho, const double* dxinv, const double* dyinv,
                         const double* dzinv, const double* dt, const double* dp,
                         const double* phat, double* un, double* vn, double* wn, double* pn) {
  Dim D(*ni, *nj, *nk);
  const int jen = nID[4] < 0 ? D.nj - 1 : D.nj;
  const double r = *rho, dxi = *dxinv, dyi = *dyinv, dzi = *dzinv, dtt = *dt;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        const long c = D.at(i, j, k);
        un[c] = un[c] + (dp[c] - F(dp, i + 1, j, k)) / r * dxi * dtt;
        if (j <= jen) vn[c] = vn[c] + (dp[c] - F(dp, i, j + 1, k)) / r * dyi * dtt;
        wn[c] = wn[c] + (dp[c] - F(dp, i, j, k + 1)) / r * dzi * dtt;
        pn[c] = phat[c] + dp[c];
      }
}

// find_interface_positions_lower.f90:1-35 -- mean lower-wall contact-line position
// (the value the reference prints, i.e. -x_avg).
double orc_interface_lower(const int* ni, const int* nj, const int* nk, const double* phi,
                           const double* dx, const double* xl) {
  Dim D(*ni, *nj, *nk);
  double sum_x = 0.0;
  for (int k = 1; k <= D.nk; ++k) {
    double xk = 0.0;
    for (int i = 1; i <= D.ni; ++i) {
      const double p1 = F(phi, i, 1, k), p2 = F(phi, i + 1, 1, k);
      if (p1 > 0.5 && p2 < 0.5) {
        xk = ((double)i - 0.5) * (*dx) + (0.5 - p1) * (*dx) / (p2 - p1) - (*xl) * 0.75;
        break;
      }
    }
    sum_x = sum_x + xk;
  }
  return -(sum_x / (double)D.nk);
}

// cal_vel.f:1-82 -- phi-weighted mean velocity of the dispersed phase and its
// Reynolds numbers (the four sums are a 4-double allreduce in the MPI build).
void orc_cal_vel(const int* ipara, const int* ni, const int* nj, const int* nk, const double* radius,
                 const double* rhol, const double* rmul, const double* u, const double* v, const double* w,
                 const double* phi, double* vel, double* re) {
  (void)ipara;
  Dim D(*ni, *nj, *nk);
  double sp = 0.0, su = 0.0, sv = 0.0, sw = 0.0;
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        const double p = F(phi, i, j, k);
        sp = sp + p;
        su = su + p * F(u, i, j, k);
        sv = sv + p * F(v, i, j, k);
        sw = sw + p * F(w, i, j, k);
      }
  vel[0] = su / sp;
  vel[1] = sv / sp;
  vel[2] = sw / sp;
  const double dia = (*radius) * 2.0;
  for (int q = 0; q < 3; ++q) re[q] = (*rhol) * vel[q] * dia / (*rmul);
}

// cal_center.f:1-121 -- centre of mass of phi with the x position unwrapped across
// the periodic direction (lap counts the passes; area 1/2/3 = x below xl/4, between,
// above 3xl/4), the x velocity from the previous centre, and the state update.
void orc_cal_center(const int* ipara, const int* ID, const int* svall, const int* ni, const int* nj,
                    const int* nk, const double* xl, const double* yl, const double* zl, const double* dt,
                    const double* rhog, const double* phi, double* center, double* center_pre1,
                    double* center_pre2, int* area_pre1, int* area_pre2, int* lap, double* velocity) {
  (void)ipara;
  (void)zl;
  (void)rhog;
  Dim D(*ni, *nj, *nk);
  const double L = *xl;
  const double delta = (*yl) / (double)(*svall);
  const double sensor1 = L * 0.25, sensor2 = L * 0.75;
  if (*area_pre1 == 1 && *area_pre2 == 3) *lap = *lap + 1;
  double wt = 0.0, wx = 0.0, wy = 0.0, wz = 0.0;
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) {
        const double p = F(phi, i, j, k);
        wt = wt + p;
        double x = delta * ((double)i - 0.5);
        const double y = delta * ((double)(j + (*ID) * D.nj) - 0.5);
        const double z = delta * ((double)k - 0.5);
        if (*area_pre1 == 3 && x < sensor1) x = x + L;
        if (*area_pre1 == 1 && x > sensor2) x = x - L;
        x = x + L * (double)(*lap);
        wx = wx + p * x;
        wy = wy + p * y;
        wz = wz + p * z;
      }
  center[0] = wx / wt;
  center[1] = wy / wt;
  center[2] = wz / wt;
  *velocity = (center[0] - *center_pre1) / (*dt);
  *center_pre2 = *center_pre1;
  *center_pre1 = center[0];
  double cc = center[0];
  *area_pre2 = *area_pre1;
  if (cc > L && L > 0.0 && std::isfinite(cc)) {  // the reference's loop never ends on inf
    for (;;) {
      cc = cc - L;
      if (cc < L) break;
    }
  }
  if (cc < sensor1) *area_pre1 = 1;
  if (cc > sensor2) *area_pre1 = 3;
  if (sensor1 <= cc && cc <= sensor2) *area_pre1 = 2;
}

// find_interface_positions_upper.f90:1-26 (find_interface_positions.f90 is the same
// routine): every crossing phi(i,nj,k) > 0.5 > phi(i+1,nj,k) of the top wall row, in
// the reference's print order (k outer, i inner).  Writes up to cap (x, z) pairs and
// returns the number of crossings.
int orc_interface_upper(const int* ni, const int* nj, const int* nk, const double* phi, const double* dx,
                        const double* dz, const double* xl, double* xz, int cap) {
  Dim D(*ni, *nj, *nk);
  int c = 0;
  for (int k = 1; k <= D.nk; ++k) {
    const double z = ((double)k - 0.5) * (*dz);
    for (int i = 1; i <= D.ni; ++i) {
      const double p1 = F(phi, i, D.nj, k), p2 = F(phi, i + 1, D.nj, k);
      if (p1 > 0.5 && p2 < 0.5) {
        if (c < cap) {
          xz[2 * c] = ((double)i - 0.5) * (*dx) + (0.5 - p1) * (*dx) / (p2 - p1) - (*xl) * 0.75;
          xz[2 * c + 1] = z;
        }
        ++c;
      }
    }
  }
  return c;
}

// ---------------------------------------------------------------------------
// Field output: mkvtk_phi.f / mkvtk_phil.f / mkvtk_p.f / mkvtk_q.f, mk_slice_j.f /
// mk_slice_k.f, the slice files of mkuwp.h / mkuvp.h, mk_center.f, mk_vel.f.

// Fortran Ew.d output (scale factor 0): optional sign, "0.", d digits of the value
// rounded to nearest, exponent as E+dd (|e| <= 99) or +ddd (|e| <= 999); when the
// field is one character too short the optional 0 goes; a field that still does
// not fit prints w asterisks.
static std::string orc_fe(double x, int w, int d) {
  std::string r;
  if (x != x) {
    r = "NaN";
  } else if (std::isinf(x)) {
    r = x < 0 ? (w >= 9 ? "-Infinity" : "-Inf") : (w >= 8 ? "Infinity" : "Inf");
  } else {
    // d significant decimal digits of |x| and the decimal exponent of the first one
    char t[80];
    std::snprintf(t, sizeof(t), "%.*e", d - 1, std::fabs(x));
    std::string mant;
    const char* p = t;
    for (; *p && *p != 'e'; ++p)
      if (*p >= '0' && *p <= '9') mant += *p;
    const int e10 = std::atoi(p + 1);
    const bool allzero = mant.find_first_not_of('0') == std::string::npos;
    const int ex = allzero ? 0 : e10 + 1;  // 0.d1d2.. x 10^ex
    const bool neg = std::signbit(x);
    std::string expo;
    const int m = ex < 0 ? -ex : ex;
    char b[16];
    if (m < 100) {
      std::snprintf(b, sizeof(b), "E%c%d%d", ex < 0 ? '-' : '+', m / 10, m % 10);
      expo = b;
    } else if (m < 1000) {
      std::snprintf(b, sizeof(b), "%c%d", ex < 0 ? '-' : '+', m);
      expo = b;
    }
    if (expo.empty()) return std::string((size_t)w, '*');
    r = (neg ? "-0." : "0.") + mant + expo;
    if ((int)r.size() == w + 1) r = (neg ? "-." : ".") + mant + expo;
  }
  if ((int)r.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)r.size()), ' ') + r;
}
void orc_format_e(char* buf, double x, int w, int d) {
  const std::string s = orc_fe(x, w, d);
  std::memcpy(buf, s.c_str(), s.size() + 1);
}

static int orc_vtk_file(const char* fname, const char* scalar, int nstep, int nx, int ny, int nz, const double* o,
                        const double* a, const std::vector<double>& v) {
  FILE* f = std::fopen(fname, "w");
  if (!f) return 1;
  std::string s = "# vtk DataFile Version 2.0\nt=" + std::to_string(nstep) + "\nASCII\nDATASET STRUCTURED_POINTS\n";
  s += "DIMENSIONS " + std::to_string(nx) + " " + std::to_string(ny) + " " + std::to_string(nz) + "\n";
  s += "ORIGIN " + orc_fe(o[0], 11, 4) + " " + orc_fe(o[1], 11, 4) + " " + orc_fe(o[2], 11, 4) + "\n";
  s += "ASPECT_RATIO " + orc_fe(a[0], 11, 4) + " " + orc_fe(a[1], 11, 4) + " " + orc_fe(a[2], 11, 4) + "\n\n";
  s += "POINT_DATA " + std::to_string((long)nx * ny * nz) + "\nSCALARS " + scalar + " float\nLOOKUP_TABLE default\n";
  std::fputs(s.c_str(), f);
  for (double x : v) std::fprintf(f, "%s\n", orc_fe(x, 10, 3).c_str());
  return std::fclose(f) == 0 ? 0 : 1;
}

// mkvtk_phi.f (kind 0), mkvtk_phil.f (kind 1, file phi<l>_), mkvtk_p.f (kind 2):
// the ghost fill of q in place, then the 8-point vertex means
int orc_mkvtk(int kind, const int* svall, const int* nstep, const double* dx, const double* dy, const double* dz,
              double* q, const int* l) {
  Dim D(svall[0], svall[1], svall[2]);
  const int mi = D.ni, mj = D.nj, mk = D.nk;
  for (int k = 0; k <= mk + 1; ++k)
    for (int j = 0; j <= mj + 1; ++j) {
      F(q, 0, j, k) = F(q, mi, j, k);
      F(q, mi + 1, j, k) = F(q, 1, j, k);
    }
  for (int k = 0; k <= mk + 1; ++k)
    for (int i = 0; i <= mi + 1; ++i) {
      F(q, i, 0, k) = kind == 1 ? 0.0 : F(q, i, 1, k);
      F(q, i, mj + 1, k) = kind == 1 ? 0.0 : F(q, i, mj, k);
    }
  for (int j = 0; j <= mj + 1; ++j)
    for (int i = 0; i <= mi + 1; ++i) {
      F(q, i, j, 0) = kind == 2 ? F(q, i, j, mk) : F(q, i, j, 1);
      F(q, i, j, mk + 1) = kind == 2 ? F(q, i, j, 1) : F(q, i, j, mk);
    }
  std::vector<double> v;
  v.reserve((size_t)(mi + 1) * (mj + 1) * (mk + 1));
  for (int k = 0; k <= mk; ++k)
    for (int j = 0; j <= mj; ++j)
      for (int i = 0; i <= mi; ++i)
        v.push_back((+F(q, i, j, k) + F(q, i + 1, j, k) + F(q, i, j + 1, k) + F(q, i + 1, j + 1, k) +
                     F(q, i, j, k + 1) + F(q, i + 1, j, k + 1) + F(q, i, j + 1, k + 1) + F(q, i + 1, j + 1, k + 1)) *
                    0.125);
  char fname[48];
  if (kind == 1) std::snprintf(fname, sizeof(fname), "phi%02d_%07d.vtk", *l, *nstep);
  else std::snprintf(fname, sizeof(fname), kind == 0 ? "phi_%07d.vtk" : "p_%07d.vtk", *nstep);
  const double o[3] = {0.0, 0.0, 0.0}, a[3] = {*dx, *dy, *dz};
  return orc_vtk_file(fname, kind == 0 ? "phi" : "p", *nstep, mi + 1, mj + 1, mk + 1, o, a, v);
}

// mkvtk_q.f: q at the cells where the mean of the 4 surrounding x-vorticities is
// > 0 (q1_ file) or < 0 (q2_ file), 0 elsewhere
int orc_mkvtk_q(const int* svall, const int* nstep, const double* dx, const double* dy, const double* dz,
                const double* vorx, const double* q) {
  Dim D(svall[0], svall[1], svall[2]);
  const double o[3] = {*dx * 0.5, *dy * 0.5, *dz * 0.5}, a[3] = {*dx, *dy, *dz};
  for (int t = 1; t <= 2; ++t) {
    std::vector<double> v;
    for (int k = 1; k <= D.nk; ++k)
      for (int j = 1; j <= D.nj; ++j)
        for (int i = 1; i <= D.ni; ++i) {
          const double vm =
              (F(vorx, i, j - 1, k - 1) + F(vorx, i, j, k - 1) + F(vorx, i, j - 1, k) + F(vorx, i, j, k)) * 0.25;
          double q00 = F(q, i, j, k);
          if (t == 1 ? vm <= 0.0 : vm >= 0.0) q00 = 0.0;
          v.push_back(q00);
        }
    char fname[48];
    std::snprintf(fname, sizeof(fname), "q%d_%07d.vtk", t, *nstep);
    if (orc_vtk_file(fname, "p", *nstep, D.ni, D.nj, D.nk, o, a, v)) return 1;
  }
  return 0;
}

// mk_slice_j.f (axis 1: fixed j, rows k) and mk_slice_k.f (axis 2: fixed k, rows j)
// with one rank: out(0:ni, 0:n), rows below the start zero
void orc_mk_slice(int axis, const int* nID, const int* ni, const int* nj, const int* nk, const int* fixed,
                  const int* ip, const int* jp, const int* kp, const double* qk, double* out) {
  Dim D(*ni, *nj, *nk);
  const int n = axis == 1 ? D.nk : D.nj;
  const int st = nID[axis == 1 ? 2 : 1] < 0 ? 0 : 1;
  for (int r = 0; r <= n; ++r)
    for (int i = 0; i <= D.ni; ++i) {
      double v = 0.0;
      if (r >= st) {
        const int j = axis == 1 ? *fixed : r, k = axis == 1 ? r : *fixed;
        const int a = *ip, b = *jp, c = *kp;
        v = (F(qk, i, j, k) + F(qk, i + a, j, k) + F(qk, i, j + b, k) + F(qk, i + a, j + b, k) + F(qk, i, j, k + c) +
             F(qk, i + a, j, k + c) + F(qk, i, j + b, k + c) + F(qk, i + a, j + b, k + c)) *
            0.125;
      }
      out[(long)r * (D.ni + 1) + i] = v;
    }
}

// mkuwp.h (kind 0: uwphi<nstep>, x z u w phi) and mkuvp.h (kind 1: uvwp<nstep>,
// x y 0 u v phi): one '(20e20.10)' record per point, a blank record per row
int orc_write_slices(int kind, int nstep, const int* svall, double d1, double d2, const double* s1, const double* s2,
                     const double* s3) {
  char fname[48];
  std::snprintf(fname, sizeof(fname), kind == 0 ? "uwphi%07d" : "uvwp%07d", nstep);
  FILE* f = std::fopen(fname, "w");
  if (!f) return 1;
  const int n1 = svall[0], n2 = kind == 0 ? svall[2] : svall[1];
  for (int b = 0; b <= n2; ++b) {
    for (int a = 0; a <= n1; ++a) {
      const long o = (long)b * (n1 + 1) + a;
      double u = s1[o], v = s2[o], q = s3[o];
      if (std::fabs(u) < 1.0e-40) u = 0.0;
      if (std::fabs(v) < 1.0e-40) v = 0.0;
      if (std::fabs(q) < 1.0e-40) q = 0.0;
      std::string line = orc_fe((double)a * d1, 20, 10) + orc_fe((double)b * d2, 20, 10);
      if (kind == 1) line += orc_fe(0.0, 20, 10);
      line += orc_fe(u, 20, 10) + orc_fe(v, 20, 10) + orc_fe(q, 20, 10);
      std::fprintf(f, "%s\n", line.c_str());
    }
    std::fputc('\n', f);
  }
  return std::fclose(f) == 0 ? 0 : 1;
}

// mk_center.f / mk_vel.f: append one '(20e20.10)' record
int orc_mk_center(const double* time, const double* center, const double* velocity, const int* l) {
  char fname[48];
  std::snprintf(fname, sizeof(fname), "center_%02d.dat", *l);
  FILE* f = std::fopen(fname, "a");
  if (!f) return 1;
  const double v[6] = {*time, center[0], center[1], center[2], *velocity,
                       std::sqrt((center[0] - 0.5) * (center[0] - 0.5) + (center[2] - 0.5) * (center[2] - 0.5))};
  std::string line;
  for (double x : v) line += orc_fe(x, 20, 10);
  std::fprintf(f, "%s\n", line.c_str());
  return std::fclose(f) == 0 ? 0 : 1;
}
int orc_mk_vel(const double* time, const double* vel, const double* re, const double* velocity, const int* l) {
  char fname[48];
  std::snprintf(fname, sizeof(fname), "velocity_%02d.dat", *l);
  FILE* f = std::fopen(fname, "a");
  if (!f) return 1;
  const double v[7] = {*time, vel[0], vel[1], vel[2], re[0], re[1], *velocity};
  std::string line;
  for (double x : v) line += orc_fe(x, 20, 10);
  std::fprintf(f, "%s\n", line.c_str());
  return std::fclose(f) == 0 ? 0 : 1;
}

// ---------------------------------------------------------------------------
// The step driver.
struct orc_ws {
  orc_params p;
  int ni, nj, nk;
  long n;
  std::vector<double> phix, phiy, phiz, flx, fly, flz, theta, rho, rhon, rmu, rmun;
  std::vector<double> adv[3], advo[3], phat, prs[3], s, tau, vis[3];
  std::vector<double> rn[4], rnn[4], rkap, rkapn, fst[3], fstn[3], sfst[3], sfstn[3], src[3];
  std::vector<double> coef[45];
  std::vector<double> un, vn, wn, pn, dp, div, fftdata, phir_r, phir_i, phiw_r, phiw_i;
  std::vector<double> dyinv_array, as_p, an_p, aw_p, ae_p, ab_p, at_p, ap_p, as_f, an_f, ap_f;
};

orc_ws* orc_ws_create(const orc_params* prm) {
  orc_ws* ws = new orc_ws();
  ws->p = *prm;
  ws->ni = prm->ni;
  ws->nj = prm->nj;
  ws->nk = prm->nk;
  const long n = (long)(prm->ni + 6) * (prm->nj + 6) * (prm->nk + 6);
  ws->n = n;
  for (auto* v : {&ws->phix, &ws->phiy, &ws->phiz, &ws->flx, &ws->fly, &ws->flz, &ws->theta, &ws->rho,
                  &ws->rhon, &ws->rmu, &ws->rmun, &ws->phat, &ws->rkap, &ws->rkapn, &ws->un, &ws->vn,
                  &ws->wn, &ws->pn, &ws->dp, &ws->div})
    v->assign(n, 0.0);
  for (int c = 0; c < 3; ++c)
    for (auto* v : {&ws->adv[c], &ws->advo[c], &ws->prs[c], &ws->vis[c], &ws->fst[c], &ws->fstn[c],
                    &ws->sfst[c], &ws->sfstn[c], &ws->src[c]})
      v->assign(n, 0.0);
  ws->s.assign(6 * n, 0.0);
  ws->tau.assign(6 * n, 0.0);
  ws->rkap.assign(3 * n, 0.0);
  ws->rkapn.assign(3 * n, 0.0);
  for (int c = 0; c < 4; ++c) {
    ws->rn[c].assign(3 * n, 0.0);
    ws->rnn[c].assign(3 * n, 0.0);
  }
  for (int c = 0; c < 45; ++c) ws->coef[c].assign(n, 0.0);
  const long nm = (long)prm->ni * prm->nj * prm->nk;
  ws->fftdata.assign(2 * nm, 0.0);
  for (auto* v : {&ws->phir_r, &ws->phir_i, &ws->phiw_r, &ws->phiw_i}) v->assign(nm, 0.0);
  const int nj6 = prm->nj + 6;
  for (auto* v : {&ws->dyinv_array, &ws->as_p, &ws->an_p, &ws->aw_p, &ws->ae_p, &ws->ab_p, &ws->at_p,
                  &ws->ap_p, &ws->as_f, &ws->an_f, &ws->ap_f})
    v->assign(nj6, 0.0);
  for (int t = 0; t < nj6; ++t) ws->dyinv_array[t] = 1.0 / prm->dy;  // main.f90:215-224
  const double dxinv = 1.0 / prm->dx, dyinv = 1.0 / prm->dy, dzinv = 1.0 / prm->dz;
  // main.f90:467-468
  orc_cal_coef_prs(&prm->nj, &prm->rhog, &dxinv, &dyinv, &dzinv, ws->aw_p.data(), ws->ae_p.data(),
                   ws->as_p.data(), ws->an_p.data(), ws->ab_p.data(), ws->at_p.data(), ws->ap_p.data());
  orc_cal_coef_solp_fft(&prm->nj, ws->as_p.data(), ws->an_p.data(), ws->as_f.data(), ws->an_f.data(),
                        ws->ap_f.data());
  return ws;
}

void orc_ws_destroy(orc_ws* ws) { delete ws; }

namespace {
const int kNID[6] = {-1, -1, -1, -1, -1, -1};  // one rank: no neighbours anywhere
// summation.f:14-51 for nbub=1 with the two slices given as separate pointers.
void summation_slices(const int* ni, const int* nj, const int* nk, double* q0, const double* q1) {
  Dim D(*ni, *nj, *nk);
  std::memcpy(q0, q1, sizeof(double) * D.size());
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= D.nk; ++k)
    for (int j = 1; j <= D.nj; ++j)
      for (int i = 1; i <= D.ni; ++i) F(q0, i, j, k) = std::fmin(std::fmax(F(q0, i, j, k), 0.0), 1.0);
}
}

void orc_init_bc(orc_ws* ws, double* const* S, const double* theta0, const double* zeta,
                 const double* l1, const double* l2) {
  const orc_params& P = ws->p;
  const int *ni = &P.ni, *nj = &P.nj, *nk = &P.nk;
  double *u = S[0], *v = S[1], *w = S[2], *uo = S[3], *vo = S[4], *wo = S[5];
  double *phi0 = S[8], *phi1 = S[9];
  const int nbub = 1;
  // main.f90:322-331
  orc_gnbc(kNID, ni, nj, nk, u, w, &P.uwall, theta0, &P.sigma, zeta, ws->theta.data());
  orc_bnd_contact_angle(kNID, ni, nj, nk, phi1, ws->theta.data(), &P.dx, &P.dy, &P.dz);
  orc_bnd_periodic(ni, nj, nk, phi1);
  // :335
  (void)nbub;
  summation_slices(ni, nj, nk, phi0, phi1);
  // :337-357 (bndu's phi argument: slice 1, see orc_step)
  double* un = ws->un.data();
  double* vn = ws->vn.data();
  double* wn = ws->wn.data();
  orc_cpy(ni, nj, nk, u, un);  // main.f90:304-306
  orc_cpy(ni, nj, nk, v, vn);
  orc_cpy(ni, nj, nk, w, wn);
  orc_bndu(kNID, ni, nj, nk, u, v, w, &P.uwall, &P.dy, l1, l2, phi1);
  orc_bndu(kNID, ni, nj, nk, uo, vo, wo, &P.uwall, &P.dy, l1, l2, phi1);
  orc_bndu(kNID, ni, nj, nk, un, vn, wn, &P.uwall, &P.dy, l1, l2, phi1);
  for (double* q : {u, v, w, uo, vo, wo, un, vn, wn}) orc_bnd_periodic(ni, nj, nk, q);
  // :361-366
  orc_gnbc(kNID, ni, nj, nk, u, w, &P.uwall, theta0, &P.sigma, zeta, ws->theta.data());
  orc_bnd_contact_angle(kNID, ni, nj, nk, phi0, ws->theta.data(), &P.dx, &P.dy, &P.dz);
  orc_bnd_periodic(ni, nj, nk, phi0);
}

// main.f90:473-697 with nbub=1.  State order: u v w uo vo wo p po phi0 phi1 phin0 phin1.
// Deviation D1: bndu's phi argument is phi(:,:,:,1) (the reference passes slice
// l=nbub+1, one past the end of phi(:,:,:,0:nbub), after its do-l loops).
int orc_step(orc_ws* ws, double* const* S, const double* theta0, const double* zeta,
             const double* l1, const double* l2, double* diag) {
  const orc_params& P = ws->p;
  const int *ni = &P.ni, *nj = &P.nj, *nk = &P.nk;
  const int ID = 0, ipara = 0, ndiv = 1;
  const int svall[3] = {P.ni, P.nj, P.nk};
  const double dxinv = 1.0 / P.dx, dyinv = 1.0 / P.dy, dzinv = 1.0 / P.dz, dt = P.dt;
  double *u = S[0], *v = S[1], *w = S[2], *uo = S[3], *vo = S[4], *wo = S[5], *p = S[6], *po = S[7];
  double *phi = S[8], *phi1 = S[9], *phin = S[10], *phin1 = S[11];
  (void)phin;
  double* dya = ws->dyinv_array.data();
  double *phix = ws->phix.data(), *phiy = ws->phiy.data(), *phiz = ws->phiz.data();
  double* theta = ws->theta.data();
  // :491-503 MTHINC transport of phi(1)
  orc_cal_grad_p2a(&ID, &svall[1], ni, nj, nk, &dxinv, dya, &dzinv, phi1, phix, phiy, phiz);
  orc_solphi_mthinc1(ni, nj, nk, &dxinv, &dyinv, &dzinv, &dt, &P.bet_mthinc, phi1, phix, phiy, phiz, u, v, w,
                     ws->flx.data(), ws->fly.data(), ws->flz.data());
  orc_solphi_mthinc2(ni, nj, nk, &dxinv, &dyinv, &dzinv, &dt, u, v, w, ws->flx.data(), ws->fly.data(),
                     ws->flz.data(), phi1, phin1);
  orc_cal_grad_p2a(&ID, &svall[1], ni, nj, nk, &dxinv, dya, &dzinv, phin1, phix, phiy, phiz);
  orc_solphi_mthinc3(&ipara, ni, nj, nk, &dxinv, &dyinv, &dzinv, &P.bet_mthinc, phix, phiy, phiz, phi1, phin1);
  orc_gnbc(kNID, ni, nj, nk, u, w, &P.uwall, theta0, &P.sigma, zeta, theta);
  orc_bnd_contact_angle(kNID, ni, nj, nk, phin1, theta, &P.dx, &P.dy, &P.dz);
  orc_bnd_periodic(ni, nj, nk, phin1);
  // :509-517
  summation_slices(ni, nj, nk, S[10], phin1);
  orc_bnd_neumann(kNID, ni, nj, nk, S[10]);
  orc_gnbc(kNID, ni, nj, nk, u, w, &P.uwall, theta0, &P.sigma, zeta, theta);
  orc_bnd_contact_angle(kNID, ni, nj, nk, phi, theta, &P.dx, &P.dy, &P.dz);
  orc_bnd_periodic(ni, nj, nk, S[10]);
  // :526-529 (4-D arrays passed to 3-D dummies resolve to slice 0)
  double *rho = ws->rho.data(), *rhon = ws->rhon.data(), *rmu = ws->rmu.data(), *rmun = ws->rmun.data();
  orc_cal_arith_mean(ni, nj, nk, phi, &P.rhol, &P.rhog, rho);
  orc_cal_arith_mean(ni, nj, nk, S[10], &P.rhol, &P.rhog, rhon);
  orc_cal_arith_mean(ni, nj, nk, phi, &P.rmul, &P.rmug, rmu);
  orc_cal_arith_mean(ni, nj, nk, S[10], &P.rmul, &P.rmug, rmun);
  // :532-541
  orc_cal_advu_weno5(ni, nj, nk, &dxinv, &dyinv, &dzinv, u, v, w, ws->adv[0].data(), ws->adv[1].data(),
                     ws->adv[2].data());
  orc_cal_advu_weno5(ni, nj, nk, &dxinv, &dyinv, &dzinv, uo, vo, wo, ws->advo[0].data(), ws->advo[1].data(),
                     ws->advo[2].data());
  orc_calphat(ni, nj, nk, p, po, ws->phat.data());
  orc_cal_grad_prs(ni, nj, nk, &dxinv, &dyinv, &dzinv, ws->phat.data(), ws->prs[0].data(), ws->prs[1].data(),
                   ws->prs[2].data());
  orc_calsij(ni, nj, nk, &dxinv, &dyinv, &dzinv, u, v, w, ws->s.data());
  orc_cal_arith_tau(ni, nj, nk, ws->s.data(), rmu, ws->tau.data());
  orc_cal_div_tensor(ni, nj, nk, &dxinv, &dyinv, &dzinv, ws->tau.data(), ws->vis[0].data(), ws->vis[1].data(),
                     ws->vis[2].data());
  // :545-573 surface tension
  orc_init_q(ni, nj, nk, ws->sfst[0].data(), ws->sfst[1].data(), ws->sfst[2].data());
  orc_init_q(ni, nj, nk, ws->sfstn[0].data(), ws->sfstn[1].data(), ws->sfstn[2].data());
  static const int offs[4][3] = {{1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  orc_cal_grad_p2a(&ID, &svall[1], ni, nj, nk, &dxinv, dya, &dzinv, phi1, phix, phiy, phiz);
  for (int c = 0; c < 4; ++c)
    orc_calrn(ni, nj, nk, &dxinv, &dyinv, &dzinv, &offs[c][0], &offs[c][1], &offs[c][2], phix, phiy, phiz,
              ws->rn[c].data());
  orc_cal_grad_p2a(&ID, &svall[1], ni, nj, nk, &dxinv, dya, &dzinv, phin1, phix, phiy, phiz);
  for (int c = 0; c < 4; ++c)
    orc_calrn(ni, nj, nk, &dxinv, &dyinv, &dzinv, &offs[c][0], &offs[c][1], &offs[c][2], phix, phiy, phiz,
              ws->rnn[c].data());
  orc_calrkap(ni, nj, nk, &dxinv, &dyinv, &dzinv, ws->rn[0].data(), ws->rn[1].data(), ws->rn[2].data(),
              ws->rn[3].data(), ws->rkap.data());
  orc_calrkap(ni, nj, nk, &dxinv, &dyinv, &dzinv, ws->rnn[0].data(), ws->rnn[1].data(), ws->rnn[2].data(),
              ws->rnn[3].data(), ws->rkapn.data());
  orc_cal_grad_p2uvw(&ID, &svall[1], ni, nj, nk, &dxinv, dya, &dzinv, phi1, phix, phiy, phiz);
  orc_calfst(ni, nj, nk, &P.rhol, &P.rhog, &P.sigma, phix, phiy, phiz, ws->rkap.data(), ws->fst[0].data(),
             ws->fst[1].data(), ws->fst[2].data());
  orc_cal_grad_p2uvw(&ID, &svall[1], ni, nj, nk, &dxinv, dya, &dzinv, phin1, phix, phiy, phiz);
  orc_calfst(ni, nj, nk, &P.rhol, &P.rhog, &P.sigma, phix, phiy, phiz, ws->rkapn.data(), ws->fstn[0].data(),
             ws->fstn[1].data(), ws->fstn[2].data());
  orc_sum_fst(ni, nj, nk, ws->fst[0].data(), ws->fst[1].data(), ws->fst[2].data(), ws->sfst[0].data(),
              ws->sfst[1].data(), ws->sfst[2].data());
  orc_sum_fst(ni, nj, nk, ws->fstn[0].data(), ws->fstn[1].data(), ws->fstn[2].data(), ws->sfstn[0].data(),
              ws->sfstn[1].data(), ws->sfstn[2].data());
  double rho_av, rhon_av;
  orc_cal_av(&ipara, &ndiv, ni, nj, nk, rho, &rho_av);
  orc_cal_av(&ipara, &ndiv, ni, nj, nk, rhon, &rhon_av);
  rho_av = (rho_av + rhon_av) * 0.5;
  // :579-603
  orc_cal_srcu(kNID, ni, nj, nk, &rho_av, &dt, &P.grvb, &P.grvp, u, v, w, rho, rhon, ws->adv[0].data(),
               ws->adv[1].data(), ws->adv[2].data(), ws->advo[0].data(), ws->advo[1].data(), ws->advo[2].data(),
               ws->prs[0].data(), ws->prs[1].data(), ws->prs[2].data(), ws->vis[0].data(), ws->vis[1].data(),
               ws->vis[2].data(), ws->sfst[0].data(), ws->sfst[1].data(), ws->sfst[2].data(), ws->sfstn[0].data(),
               ws->sfstn[1].data(), ws->sfstn[2].data(), ws->src[0].data(), ws->src[1].data(), ws->src[2].data());
  double* cf[45];
  for (int c = 0; c < 45; ++c) cf[c] = ws->coef[c].data();
  orc_cal_arith_coef_vis_v(ni, nj, nk, &dxinv, &dyinv, &dzinv, rmun, cf, P.harmonic);
  // :605-623
  double *un = ws->un.data(), *vn = ws->vn.data(), *wn = ws->wn.data(), *pn = ws->pn.data();
  orc_cpy(ni, nj, nk, u, un);
  orc_cpy(ni, nj, nk, v, vn);
  orc_cpy(ni, nj, nk, w, wn);
  double sor_err = 0.0;
  const int nsor = orc_solu_sor4_v(kNID, ni, nj, nk, &dt, rho, rhon, cf, ws->src[0].data(), ws->src[1].data(),
                                   ws->src[2].data(), un, vn, wn, &P.uwall, &P.dy, l1, l2, phi1, &sor_err);
  // :625-631
  orc_bndu(kNID, ni, nj, nk, un, vn, wn, &P.uwall, &P.dy, l1, l2, phi1);
  orc_bnd_periodic(ni, nj, nk, un);
  orc_bnd_periodic(ni, nj, nk, vn);
  orc_bnd_periodic(ni, nj, nk, wn);
  // :633-646 pressure
  double err_div0;
  orc_caldiv(&ipara, &ndiv, ni, nj, nk, &dxinv, &dyinv, &dzinv, &dt, un, vn, wn, ws->div.data(), &err_div0);
  orc_solp_fft_tdma1(ni, nj, nk, ws->fftdata.data(), ws->div.data(), ws->phir_r.data(), ws->phir_i.data());
  int key[8];
  orc_trans_r2w(&ipara, &ID, &ndiv, svall, key, nullptr, nullptr, ws->phir_r.data(), ws->phiw_r.data());
  orc_trans_r2w(&ipara, &ID, &ndiv, svall, key, nullptr, nullptr, ws->phir_i.data(), ws->phiw_i.data());
  orc_solp_fft_tdma2(&ID, &ndiv, svall, &P.rhog, &dxinv, &dzinv, ws->as_f.data(), ws->an_f.data(),
                     ws->ap_f.data(), nullptr, nullptr, nullptr, ws->phiw_r.data(), ws->phiw_i.data());
  orc_trans_w2r(&ipara, &ID, &ndiv, svall, key, nullptr, nullptr, ws->phiw_r.data(), ws->phir_r.data());
  orc_trans_w2r(&ipara, &ID, &ndiv, svall, key, nullptr, nullptr, ws->phiw_i.data(), ws->phir_i.data());
  double* dp = ws->dp.data();
  orc_solp_fft_tdma3(ni, nj, nk, ws->fftdata.data(), ws->phir_r.data(), ws->phir_i.data(), dp);
  orc_bnd_avzero(&ipara, &ndiv, ni, nj, nk, dp);
  orc_bnd_neumann(kNID, ni, nj, nk, dp);
  orc_bnd_periodic(ni, nj, nk, dp);
  // :648-661
  orc_corunp_explicit(kNID, ni, nj, nk, &P.rhog, &dxinv, &dyinv, &dzinv, &dt, dp, ws->phat.data(), un, vn, wn,
                      pn);
  orc_bndu(kNID, ni, nj, nk, un, vn, wn, &P.uwall, &P.dy, l1, l2, phi1);
  orc_bnd_periodic(ni, nj, nk, un);
  orc_bnd_periodic(ni, nj, nk, vn);
  orc_bnd_periodic(ni, nj, nk, wn);
  orc_bnd_avzero(&ipara, &ndiv, ni, nj, nk, pn);
  orc_bnd_neumann(kNID, ni, nj, nk, pn);
  orc_bnd_periodic(ni, nj, nk, pn);
  if (diag) {
    diag[0] = err_div0;
    diag[1] = sor_err;
  }
  // :686-697 rotation
  orc_cpy(ni, nj, nk, u, uo);
  orc_cpy(ni, nj, nk, v, vo);
  orc_cpy(ni, nj, nk, w, wo);
  orc_cpy(ni, nj, nk, p, po);
  orc_cpy(ni, nj, nk, un, u);
  orc_cpy(ni, nj, nk, vn, v);
  orc_cpy(ni, nj, nk, wn, w);
  orc_cpy(ni, nj, nk, pn, p);
  orc_cpy(ni, nj, nk, S[10], S[8]);
  orc_cpy(ni, nj, nk, S[11], S[9]);
  return nsor;
}

}  // extern "C"
