// k_bc.cu -- C5: contact line and wall / halo conditions (plane kernels).
// With one GPU the reference's MPI halo exchange (bnd_comm.f) has nothing to do;
// periodic and wall halos are these in-device plane kernels.
#include "ops.cuh"

namespace fmf {
namespace op {

// gnbc.f90:24-97 -- dynamic contact angle from the wall slip speed, both walls.
void gnbc(cudaStream_t s, const Grid& g, const double* uk, const double* wk, double uwall,
          const double* theta0, double sigma, const double* zeta, double* theta) {
  const Grid G = g;
  const double pi = std::acos(-1.0);
  range2(s, -2, g.ni + 3, -2, 2 * (g.nk + 6) - 3, [=] __device__(int i, int kk) {
    const int side = kk >= G.nk + 4 ? 1 : 0;
    const int k = side ? kk - (G.nk + 6) : kk;
    const int ja = side ? G.nj : 0, jb = ja + 1, jw = side ? G.nj : 1;
    const double us = side ? -uwall : uwall;
    const int mi = (i + G.ni + 2) % (G.ni + 3);
    const double ucx = (uk[G.at(mi, ja, k)] + uk[G.at(mi, jb, k)] + uk[G.at(i, ja, k)] + uk[G.at(i, jb, k)]) / 4.0 + us;
    const double ucz = (wk[G.at(mi, ja, k)] + wk[G.at(mi, jb, k)] + wk[G.at(i, ja, k)] + wk[G.at(i, jb, k)]) / 4.0;
    double ucl = copysign(sqrt(ucx * ucx + ucz * ucz + 1.0e-12), ucx);
    if (i <= G.ni / 2) ucl = -ucl;
    const long c = G.at(i, jw, k);
    const double c0 = cos(theta0[c] * (pi / 180.0));
    double ct = c0 - zeta[c] * ucl / sigma;
    ct = fmin(1.0, fmax(-1.0, ct));
    theta[c] = acos(ct) * (180.0 / pi);
  });
}

// bnd_contact_angle.f90:25-85 -- ghost extrapolation along the contact-angle normal.
// Columns i=-2,ni+3 and planes k=-2,nk+3 are left unchanged (there the reference
// reads outside its array; every call site overwrites them with bnd_periodic).
void bnd_contact_angle(cudaStream_t s, const Grid& g, double* qk, const double* theta, double dx,
                       double dy, double dz) {
  const Grid G = g;
  const double pi = std::acos(-1.0), ax = dy / dx, az = dy / dz;
  range2(s, -1, g.ni + 2, -1, 2 * (g.nk + 4) - 2, [=] __device__(int i, int kk) {
    const int side = kk >= G.nk + 3 ? 1 : 0;
    const int k = side ? kk - (G.nk + 4) : kk;
    const int jw = side ? G.nj : 1;
    const double eps = 1.0e-20;
    const double th = theta[G.at(i, jw, k)] * pi / 180.0;
    const double ct = cos(th), sn = sin(th);
    const double sg = (i - G.ni / 2) >= 0 ? 1.0 : -1.0;
    double nx = sg * sn * ax, nz = sg * sn * az, ny = ct;
    const double nrm = sqrt(nx * nx + ny * ny + nz * nz + eps);
    nx = nx / nrm;
    ny = ny / nrm;
    nz = nz / nrm;
    const double q1 = qk[G.at(i, jw, k)];
    const double gh = q1 - (ny / (nx + eps)) * (qk[G.at(i + 1, jw, k)] - qk[G.at(i - 1, jw, k)]) * 0.5 * ax -
                      (ny / (nz + eps)) * (qk[G.at(i, jw, k + 1)] - qk[G.at(i, jw, k - 1)]) * 0.5 * az;
    if (!side) {
      const double g1 = 2.0 * gh - q1;
      qk[G.at(i, 0, k)] = gh;
      qk[G.at(i, -1, k)] = g1;
      qk[G.at(i, -2, k)] = 2.0 * g1 - gh;
    } else {
      const double g1 = 2.0 * gh - q1;
      qk[G.at(i, G.nj + 1, k)] = gh;
      qk[G.at(i, G.nj + 2, k)] = g1;
      qk[G.at(i, G.nj + 3, k)] = 2.0 * g1 - gh;
    }
  });
}

// bndu.f:29-158 -- Navier-slip ghosts at both walls, then x halos (u shifted by
// one), then z halos (w shifted by one), as three ordered plane kernels.
void bndu(cudaStream_t s, const Grid& g, double* uk, double* vk, double* wk, double uwall, double dy,
          const double* l1, const double* l2, const double* phi) {
  const Grid G = g;
  range2(s, -2, g.ni + 3, -2, 2 * (g.nk + 6) - 3, [=] __device__(int i, int kk) {
    const int side = kk >= G.nk + 4 ? 1 : 0;
    const int k = side ? kk - (G.nk + 6) : kk;
    const int NJ = G.nj;
    const int jw = side ? NJ : 1;
    const double pa = (phi[G.at(i, jw, k)] + phi[G.at((i + 1) % (G.ni + 3), jw, k)]) / 2.0;
    const double i1 = pa / l1[G.at(i, jw, k)], i2 = (1.0 - pa) / l2[G.at(i, jw, k)];
    const double ls = 1.0 / (i1 + i2);
    const double c1 = (2.0 * dy) / (2.0 * ls + dy), c2 = (2.0 * ls - dy) / (2.0 * ls + dy);
    if (!side) {
      const double u1 = uk[G.at(i, 1, k)];
      const double u0 = c1 * (-uwall) + c2 * u1;
      const double um1 = 2.0 * u0 - u1;
      uk[G.at(i, 0, k)] = u0;
      uk[G.at(i, -1, k)] = um1;
      uk[G.at(i, -2, k)] = 2.0 * um1 - u0;
      vk[G.at(i, -2, k)] = -vk[G.at(i, 2, k)];
      vk[G.at(i, -1, k)] = -vk[G.at(i, 1, k)];
      vk[G.at(i, 0, k)] = 0.0;
      const double w1 = wk[G.at(i, 1, k)];
      const double w0 = c2 * w1;
      const double wm1 = 2.0 * w0 - w1;
      wk[G.at(i, 0, k)] = w0;
      wk[G.at(i, -1, k)] = wm1;
      wk[G.at(i, -2, k)] = 2.0 * wm1 - w0;
    } else {
      const double u1 = uk[G.at(i, NJ, k)];
      const double u0 = c1 * uwall + c2 * u1;
      const double up2 = 2.0 * u0 - u1;
      uk[G.at(i, NJ + 1, k)] = u0;
      uk[G.at(i, NJ + 2, k)] = up2;
      uk[G.at(i, NJ + 3, k)] = 2.0 * up2 - u0;
      const double vm1 = vk[G.at(i, NJ - 1, k)], vm2 = vk[G.at(i, NJ - 2, k)], vm3 = vk[G.at(i, NJ - 3, k)];
      vk[G.at(i, NJ, k)] = 0.0;
      vk[G.at(i, NJ + 1, k)] = -vm1;
      vk[G.at(i, NJ + 2, k)] = -vm2;
      vk[G.at(i, NJ + 3, k)] = -vm3;
      const double w1 = wk[G.at(i, NJ, k)];
      const double w0 = c2 * w1;
      const double wp2 = 2.0 * w0 - w1;
      wk[G.at(i, NJ + 1, k)] = w0;
      wk[G.at(i, NJ + 2, k)] = wp2;
      wk[G.at(i, NJ + 3, k)] = 2.0 * wp2 - w0;
    }
  });
  range2(s, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int j, int k) {
    const int NI = G.ni;
    const long r = G.at(0, j, k);  // (0,j,k); i offsets relative to it
    uk[r] = uk[r + NI + 1];
    uk[r - 1] = uk[r + NI];
    uk[r - 2] = uk[r + NI - 1];
    vk[r] = vk[r + NI];
    vk[r - 1] = vk[r + NI - 1];
    vk[r - 2] = vk[r + NI - 2];
    wk[r] = wk[r + NI];
    wk[r - 1] = wk[r + NI - 1];
    wk[r - 2] = wk[r + NI - 2];
    uk[r + NI + 2] = uk[r + 2];
    uk[r + NI + 3] = uk[r + 3];
    vk[r + NI + 1] = vk[r + 1];
    vk[r + NI + 2] = vk[r + 2];
    vk[r + NI + 3] = vk[r + 3];
    wk[r + NI + 1] = wk[r + 1];
    wk[r + NI + 2] = wk[r + 2];
    wk[r + NI + 3] = wk[r + 3];
  });
  range2(s, -2, g.ni + 3, -2, g.nj + 3, [=] __device__(int i, int j) {
    const int NK = G.nk;
    const long Z = G.sz;
    const long r = G.at(i, j, 0);
    uk[r] = uk[r + NK * Z];
    uk[r - Z] = uk[r + (NK - 1) * Z];
    uk[r - 2 * Z] = uk[r + (NK - 2) * Z];
    vk[r] = vk[r + NK * Z];
    vk[r - Z] = vk[r + (NK - 1) * Z];
    vk[r - 2 * Z] = vk[r + (NK - 2) * Z];
    wk[r] = wk[r + (NK + 1) * Z];
    wk[r - Z] = wk[r + NK * Z];
    wk[r - 2 * Z] = wk[r + (NK - 1) * Z];
    uk[r + (NK + 1) * Z] = uk[r + Z];
    uk[r + (NK + 2) * Z] = uk[r + 2 * Z];
    uk[r + (NK + 3) * Z] = uk[r + 3 * Z];
    vk[r + (NK + 1) * Z] = vk[r + Z];
    vk[r + (NK + 2) * Z] = vk[r + 2 * Z];
    vk[r + (NK + 3) * Z] = vk[r + 3 * Z];
    wk[r + (NK + 2) * Z] = wk[r + 2 * Z];
    wk[r + (NK + 3) * Z] = wk[r + 3 * Z];
  });
}

// bnd_periodic.f:173-205 -- x halos over every (j,k), then z halos over every (i,j).
void bnd_periodic(cudaStream_t s, const Grid& g, double* qk) {
  const Grid G = g;
  range2(s, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int j, int k) {
    const int NI = G.ni;
    const long r = G.at(0, j, k);
    qk[r - 2] = qk[r + NI - 2];
    qk[r - 1] = qk[r + NI - 1];
    qk[r] = qk[r + NI];
    qk[r + NI + 1] = qk[r + 1];
    qk[r + NI + 2] = qk[r + 2];
    qk[r + NI + 3] = qk[r + 3];
  });
  range2(s, -2, g.ni + 3, -2, g.nj + 3, [=] __device__(int i, int j) {
    const int NK = G.nk;
    const long Z = G.sz;
    const long r = G.at(i, j, 0);
    qk[r - 2 * Z] = qk[r + (NK - 2) * Z];
    qk[r - Z] = qk[r + (NK - 1) * Z];
    qk[r] = qk[r + NK * Z];
    qk[r + (NK + 1) * Z] = qk[r + Z];
    qk[r + (NK + 2) * Z] = qk[r + 2 * Z];
    qk[r + (NK + 3) * Z] = qk[r + 3 * Z];
  });
}

// bnd_neumann.f:222-252 -- even reflection across both walls.
void bnd_neumann(cudaStream_t s, const Grid& g, double* qk) {
  const Grid G = g;
  range2(s, -2, g.ni + 3, -2, g.nk + 3, [=] __device__(int i, int k) {
    const int NJ = G.nj;
    qk[G.at(i, -2, k)] = qk[G.at(i, 3, k)];
    qk[G.at(i, -1, k)] = qk[G.at(i, 2, k)];
    qk[G.at(i, 0, k)] = qk[G.at(i, 1, k)];
    qk[G.at(i, NJ + 1, k)] = qk[G.at(i, NJ, k)];
    qk[G.at(i, NJ + 2, k)] = qk[G.at(i, NJ - 1, k)];
    qk[G.at(i, NJ + 3, k)] = qk[G.at(i, NJ - 2, k)];
  });
}

}  // namespace op
}  // namespace fmf
