// k_glue.cu -- C6: mixture properties, explicit viscous stress, CSF surface tension,
// momentum right-hand side (drop-in kernels).
#include "ops.cuh"

namespace fmf {
namespace op {

// cal_arith_mean.f:13-27
void cal_arith_mean(cudaStream_t s, const Grid& g, const double* phi, double ql, double qg, double* q) {
  flat(s, g.n, [=] __device__(long t) { q[t] = ql * (1.0 - phi[t]) + qg * phi[t]; });
}
// The four cal_arith_mean calls of main.f90:526-529 in one pass: rho, rhon from
// (rhol, rhog) and rmu, rmun from (rmul, rmug) over phi0 and phin0 -- the same
// expression per point, two points per thread per pass so that four loads are in
// flight (the single-field pass keeps one and runs at a third of HBM's rate).
namespace {
__global__ void __launch_bounds__(256) k_means4(long n, const double* __restrict__ p0, const double* __restrict__ p1,
                                                double rl, double rg, double ml, double mg, double* __restrict__ rho,
                                                double* __restrict__ rhon, double* __restrict__ rmu,
                                                double* __restrict__ rmun) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += 2 * stride) {
    const long t2 = t + stride;
    const bool two = t2 < n;
    const double a = p0[t], b = p1[t];
    const double a2 = two ? p0[t2] : 0.0, b2 = two ? p1[t2] : 0.0;
    rho[t] = rl * (1.0 - a) + rg * a;
    rhon[t] = rl * (1.0 - b) + rg * b;
    rmu[t] = ml * (1.0 - a) + mg * a;
    rmun[t] = ml * (1.0 - b) + mg * b;
    if (two) {
      rho[t2] = rl * (1.0 - a2) + rg * a2;
      rhon[t2] = rl * (1.0 - b2) + rg * b2;
      rmu[t2] = ml * (1.0 - a2) + mg * a2;
      rmun[t2] = ml * (1.0 - b2) + mg * b2;
    }
  }
}
}  // namespace
void mixture_means(cudaStream_t s, const Grid& g, const double* phi0, const double* phin0, double rhol, double rhog,
                   double rmul, double rmug, double* rho, double* rhon, double* rmu, double* rmun) {
  k_means4<<<152 * 8, 256, 0, s>>>(g.n, phi0, phin0, rhol, rhog, rmul, rmug, rho, rhon, rmu, rmun);
  count_launch();
}
// cal_harm_mean.f:42-56
void cal_harm_mean(cudaStream_t s, const Grid& g, const double* phi, double ql, double qg, double* q) {
  flat(s, g.n, [=] __device__(long t) { q[t] = 1.0 / ((1.0 - phi[t]) / ql + phi[t] / qg); });
}
// calphat.f:10-23 (i from -1)
void calphat(cudaStream_t s, const Grid& g, const double* p, const double* po, double* phat) {
  const Grid G = g;
  range3(s, -1, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    phat[c] = p[c] * 2.0 - po[c];
  });
}
// cal_grad_prs.f:16-38
void cal_grad_prs(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                  const double* q, double* qx, double* qy, double* qz) {
  const Grid G = g;
  range3(s, -2, g.ni + 2, -2, g.nj + 2, -2, g.nk + 2, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    const double q0 = q[c];
    qx[c] = (-q0 + q[c + 1]) * dxinv;
    qy[c] = (-q0 + q[c + G.sy]) * dyinv;
    qz[c] = (-q0 + q[c + G.sz]) * dzinv;
  });
}
// calsij.f:22-139 -- six components, each on its own range
void calsij(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* u,
            const double* v, const double* w, double* sk) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    if (i >= -1) sk[c] = (-u[c - X] + u[c]) * dxinv;
    if (j >= -1) sk[c + n] = (-v[c - Y] + v[c]) * dyinv;
    if (i >= -1 && j >= -1 && k >= -1) sk[c + 2 * n] = (-w[c - Z] + w[c]) * dzinv;
    if (j <= G.nj + 2 && i <= G.ni + 2)
      sk[c + 3 * n] = ((-u[c] + u[c + Y]) * dyinv + (-v[c] + v[c + X]) * dxinv) * 0.5;
    if (k <= G.nk + 2 && i <= G.ni + 2)
      sk[c + 4 * n] = ((-u[c] + u[c + Z]) * dzinv + (-w[c] + w[c + X]) * dxinv) * 0.5;
    if (k <= G.nk + 2 && j <= G.nj + 2)
      sk[c + 5 * n] = ((-v[c] + v[c + Z]) * dzinv + (-w[c] + w[c + Y]) * dyinv) * 0.5;
  });
}
// cal_arith_tau.f:21-117 / cal_harm_tau.f:21-117
void cal_tau(cudaStream_t s, const Grid& g, const double* sk, const double* rmu, double* tau,
             bool harmonic) {
  const Grid G = g;
  const bool hm = harmonic;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    for (int l = 0; l < 3; ++l) tau[c + l * n] = sk[c + l * n] * rmu[c] * 2.0;
    auto m4 = [&](long a, long b, long d, long e) {
      if (!hm) return 0.25 * rmu[a] + 0.25 * rmu[b] + 0.25 * rmu[d] + 0.25 * rmu[e];
      return 1.0 / (0.25 / rmu[a] + 0.25 / rmu[b] + 0.25 / rmu[d] + 0.25 / rmu[e]);
    };
    if (j <= G.nj + 2 && i <= G.ni + 2) tau[c + 3 * n] = sk[c + 3 * n] * m4(c, c + X, c + Y, c + X + Y) * 2.0;
    if (k <= G.nk + 2 && i <= G.ni + 2) tau[c + 4 * n] = sk[c + 4 * n] * m4(c, c + X, c + Z, c + X + Z) * 2.0;
    if (k <= G.nk + 2 && j <= G.nj + 2) tau[c + 5 * n] = sk[c + 5 * n] * m4(c, c + Y, c + Z, c + Y + Z) * 2.0;
  });
}
// cal_div_tensor.f:14-86
void cal_div_tensor(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv,
                    const double* t, double* vu, double* vv, double* vw) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    const double* t1 = t;
    const double* t2 = t + n;
    const double* t3 = t + 2 * n;
    const double* t4 = t + 3 * n;
    const double* t5 = t + 4 * n;
    const double* t6 = t + 5 * n;
    double a = 0.0, b = 0.0, d = 0.0;
    if (k >= -1 && j >= -1 && i <= G.ni + 2)
      a = (-t1[c] + t1[c + X]) * dxinv + (-t4[c - Y] + t4[c]) * dyinv + (-t5[c - Z] + t5[c]) * dzinv;
    if (k >= -1 && j <= G.nj + 2 && i >= -1)
      b = (-t4[c - X] + t4[c]) * dxinv + (-t2[c] + t2[c + Y]) * dyinv + (-t6[c - Z] + t6[c]) * dzinv;
    if (k <= G.nk + 2 && j >= -1 && i >= -1)
      d = (-t5[c - X] + t5[c]) * dxinv + (-t6[c - Y] + t6[c]) * dyinv + (-t3[c] + t3[c + Z]) * dzinv;
    vu[c] = a;
    vv[c] = b;
    vw[c] = d;
  });
}
// calrn.f:18-88 -- zero, then the 8-vertex averaged unit normal at (i+ip, j+jp, k+kp)
void calrn(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, int ip, int jp, int kp,
           const double* phix, const double* phiy, const double* phiz, double* rn) {
  const Grid G = g;
  const double vs = std::sqrt(dxinv * dxinv + dyinv * dyinv + dzinv * dzinv) * 1.0e-30;
  flat(s, 3 * g.n, [=] __device__(long t) { rn[t] = 0.0; });
  range3(s, -2, g.ni + 3 - ip, -2, g.nj + 3 - jp, -2, g.nk + 3 - kp, [=] __device__(int i, int j, int k) {
    const long n = G.n;
    const long c = G.at(i, j, k);
    const long X = ip, Y = jp ? G.sy : 0, Z = kp ? G.sz : 0;
    auto avg = [&](const double* p) {
      return (p[c] + p[c + X] + p[c + Y] + p[c + X + Y] + p[c + Z] + p[c + X + Z] + p[c + Y + Z] + p[c + X + Y + Z]) *
             0.125;
    };
    const double rx = avg(phix), ry = avg(phiy), rz = avg(phiz);
    const double a = sqrt(rx * rx + ry * ry + rz * rz) + vs;
    const double ainv = 1.0 / a;
    const long o = c + X + Y + Z;
    rn[o] = rx * ainv;
    rn[o + n] = ry * ainv;
    rn[o + 2 * n] = rz * ainv;
  });
}
// calrkap.f:15-98
void calrkap(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, const double* pp,
             const double* r12, const double* r13, const double* r23, double* rkap) {
  const Grid G = g;
  range3(s, -2, g.ni + 3, -2, g.nj + 3, -2, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz, n = G.n;
    const long c = G.at(i, j, k);
    double a = 0.0, b = 0.0, d = 0.0;
    if (k >= -1 && j >= -1 && i <= G.ni + 2)
      a = (-pp[c] + pp[c + X]) * dxinv + (-r12[c - Y + n] + r12[c + n]) * dyinv +
          (-r13[c - Z + 2 * n] + r13[c + 2 * n]) * dzinv;
    if (k >= -1 && j <= G.nj + 2 && i >= -1)
      b = (-r12[c - X] + r12[c]) * dxinv + (-pp[c + n] + pp[c + Y + n]) * dyinv +
          (-r23[c - Z + 2 * n] + r23[c + 2 * n]) * dzinv;
    if (k <= G.nk + 2 && j >= -1 && i >= -1)
      d = (-r13[c - X] + r13[c]) * dxinv + (-r23[c - Y + n] + r23[c + n]) * dyinv +
          (-pp[c + 2 * n] + pp[c + Z + 2 * n]) * dzinv;
    rkap[c] = a;
    rkap[c + n] = b;
    rkap[c + 2 * n] = d;
  });
}
// calfst.f:25-46
void calfst(cudaStream_t s, const Grid& g, double rhol, double rhog, double sigma, const double* gx,
            const double* gy, const double* gz, const double* rkap, double* fu, double* fv, double* fw) {
  const long n = g.n;
  const double st = 2.0 * sigma / (rhol + rhog);
  flat(s, n, [=] __device__(long t) {
    fu[t] = -st * rkap[t] * gx[t];
    fv[t] = -st * rkap[t + n] * gy[t];
    fw[t] = -st * rkap[t + 2 * n] * gz[t];
  });
}
// sum_fst.f:19-34
void sum_fst(cudaStream_t s, const Grid& g, const double* fu, const double* fv, const double* fw,
             double* su, double* sv, double* sw) {
  flat(s, g.n, [=] __device__(long t) {
    su[t] = su[t] + fu[t];
    sv[t] = sv[t] + fv[t];
    sw[t] = sw[t] + fw[t];
  });
}
void fill(cudaStream_t s, long n, double* q, double value) {
  flat(s, n, [=] __device__(long t) { q[t] = value; });
}
void copy(cudaStream_t s, long n, const double* a, double* b) {
  FMF_CUDA(cudaMemcpyAsync(b, a, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
}
// cal_av.f:13-37 -- interior mean into out[0]
void cal_av(cudaStream_t s, const Grid& g, const double* q, double* out) {
  const Grid G = g;
  reduce_interior<1>(s, g, [=] __device__(int i, int j, int k, double* r) { r[0] = q[G.at(i, j, k)]; }, out);
  const double inv = (double)g.cells();
  flat(s, 1, [=] __device__(long) { out[0] = out[0] / inv; });
}
// cal_srcu.f:53-137 (src_v only for j<=nj-1: the upper wall face is not solved)
void cal_srcu(cudaStream_t s, const Grid& g, double dt, double grvb, double grvp, const double* u,
              const double* v, const double* w, const double* rho, const double* rhon,
              const double* const* adv, const double* const* advo, const double* const* prs,
              const double* const* vis, const double* const* fst, const double* const* fstn,
              double* const* src) {
  const Grid G = g;
  const double dtinv = 1.0 / dt;
  const double *a0 = adv[0], *a1 = adv[1], *a2 = adv[2], *o0 = advo[0], *o1 = advo[1], *o2 = advo[2];
  const double *p0 = prs[0], *p1 = prs[1], *p2 = prs[2], *v0 = vis[0], *v1 = vis[1], *v2 = vis[2];
  const double *f0 = fst[0], *f1 = fst[1], *f2 = fst[2], *n0 = fstn[0], *n1 = fstn[1], *n2 = fstn[2];
  double *s0 = src[0], *s1 = src[1], *s2 = src[2];
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long X = 1, Y = G.sy, Z = G.sz;
    const long c = G.at(i, j, k);
    double r = (rho[c] + rho[c + X] + rhon[c] + rhon[c + X]) * 0.25;
    s0[c] = u[c] * dtinv - a0[c] * 1.5 + o0[c] * 0.5 - p0[c] / r + v0[c] / r * 0.5 + f0[c] * 0.5 + n0[c] * 0.5 + grvb;
    if (j <= G.nj - 1) {
      r = (rho[c] + rho[c + Y] + rhon[c] + rhon[c + Y]) * 0.25;
      s1[c] = v[c] * dtinv - a1[c] * 1.5 + o1[c] * 0.5 - p1[c] / r + v1[c] / r * 0.5 + f1[c] * 0.5 + n1[c] * 0.5 + grvp;
    }
    r = (rho[c] + rho[c + Z] + rhon[c] + rhon[c + Z]) * 0.25;
    s2[c] = w[c] * dtinv - a2[c] * 1.5 + o2[c] * 0.5 - p2[c] / r + v2[c] / r * 0.5 + f2[c] * 0.5 + n2[c] * 0.5;
  });
}

}  // namespace op
}  // namespace fmf
