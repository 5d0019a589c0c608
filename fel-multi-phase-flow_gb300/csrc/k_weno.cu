// k_weno.cu -- C2: WENO5 momentum advection (drop-in kernel).
#include "ops.cuh"
#include "weno5_core.cuh"

namespace fmf {
namespace op {

// cal_advu_weno5.f:38-255 -- zero the three outputs on the full halo, then the
// nine directional derivatives per interior cell (u, v, w each along x, y, z).
void cal_advu_weno5(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                    const double* u, const double* v, const double* w, double* au, double* av,
                    double* aw) {
  const Grid G = g;
  flat(s, g.n, [=] __device__(long t) {
    au[t] = 0.0;
    av[t] = 0.0;
    aw[t] = 0.0;
  });
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    double vel, a;
    vel = ((u[c - X] + u[c]) * 0.5 + (u[c] + u[c + X]) * 0.5) * 0.5;
    a = weno5_line<double>(u, c, X, vel) * dxinv;
    vel = ((v[c - Y] + v[c + X - Y]) * 0.5 + (v[c] + v[c + X]) * 0.5) * 0.5;
    a = a + weno5_line<double>(u, c, Y, vel) * dyinv;
    vel = ((w[c - Z] + w[c + X - Z]) * 0.5 + (w[c] + w[c + X]) * 0.5) * 0.5;
    a = a + weno5_line<double>(u, c, Z, vel) * dzinv;
    au[c] = a;
    vel = ((u[c - X] + u[c - X + Y]) * 0.5 + (u[c] + u[c + Y]) * 0.5) * 0.5;
    a = weno5_line<double>(v, c, X, vel) * dxinv;
    vel = ((v[c - Y] + v[c]) * 0.5 + (v[c] + v[c + Y]) * 0.5) * 0.5;
    a = a + weno5_line<double>(v, c, Y, vel) * dyinv;
    vel = ((w[c - Z] + w[c + Y - Z]) * 0.5 + (w[c] + w[c + Y]) * 0.5) * 0.5;
    a = a + weno5_line<double>(v, c, Z, vel) * dzinv;
    av[c] = a;
    vel = ((u[c - X] + u[c - X + Z]) * 0.5 + (u[c] + u[c + Z]) * 0.5) * 0.5;
    a = weno5_line<double>(w, c, X, vel) * dxinv;
    vel = ((v[c - Y] + v[c - Y + Z]) * 0.5 + (v[c] + v[c + Z]) * 0.5) * 0.5;
    a = a + weno5_line<double>(w, c, Y, vel) * dyinv;
    vel = ((w[c - Z] + w[c]) * 0.5 + (w[c] + w[c + Z]) * 0.5) * 0.5;
    a = a + weno5_line<double>(w, c, Z, vel) * dzinv;
    aw[c] = a;
  });
}

}  // namespace op
}  // namespace fmf
