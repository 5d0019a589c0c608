// diag.cu -- the reference's run-time monitors on device arrays: cal_vel.f,
// cal_center.f, find_interface_positions_upper.f90 / _lower.f90.  Every result
// lands in device memory; the drop-ins read back a few doubles, the fmf_dev_*
// variants read back nothing.
#include "ops.cuh"

namespace fmf {
namespace op {

namespace {
// out[0..2] = su/sp, sv/sp, sw/sp; out[3..5] = rhol vel diameter / rmul (cal_vel.f:72-78)
__global__ void k_vel_finish(const double* sums, double dia, double rhol, double rmul, double* out) {
  const double sp = sums[0];
  for (int q = 0; q < 3; ++q) {
    const double v = sums[1 + q] / sp;
    out[q] = v;
    out[3 + q] = rhol * v * dia / rmul;
  }
}

// The crossing of row j between i and i+1 (phi(i) > 0.5 > phi(i+1)), interpolated
// linearly, shifted by -3/4 xl (find_interface_positions_*.f90)
__device__ __forceinline__ bool crossing(const Grid& g, const double* phi, int i, int j, int k, double dx,
                                         double xl, double* x) {
  const double p1 = phi[g.at(i, j, k)], p2 = phi[g.at(i + 1, j, k)];
  if (!(p1 > 0.5 && p2 < 0.5)) return false;
  *x = ((double)i - 0.5) * dx + (0.5 - p1) * dx / (p2 - p1) - xl * 0.75;
  return true;
}

// One block: thread t owns the k planes [1 + t c, t c + c] (c = ceil(nk / threads)),
// counts its crossings, a scan over the block gives each its first output slot, and
// the crossings are written in (k, i) order.
__global__ void __launch_bounds__(1024) k_iface_upper(Grid g, double dx, double dz, double xl, const double* phi,
                                                      double* xz, int* count, int cap) {
  __shared__ int sc[1024];
  const int T = (int)blockDim.x, t = (int)threadIdx.x;
  const int chunk = (g.nk + T - 1) / T;
  const int k0 = 1 + t * chunk, k1 = min(g.nk, k0 + chunk - 1);
  int c = 0;
  double x;
  for (int k = k0; k <= k1; ++k)
    for (int i = 1; i <= g.ni; ++i) c += crossing(g, phi, i, g.nj, k, dx, xl, &x) ? 1 : 0;
  sc[t] = c;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int q = 0; q < T; ++q) {
      const int v = sc[q];
      sc[q] = acc;
      acc += v;
    }
    *count = acc;
  }
  __syncthreads();
  int o = sc[t];
  for (int k = k0; k <= k1; ++k) {
    const double z = ((double)k - 0.5) * dz;
    for (int i = 1; i <= g.ni; ++i)
      if (crossing(g, phi, i, g.nj, k, dx, xl, &x)) {
        if (o < cap) {
          xz[2L * o] = x;
          xz[2L * o + 1] = z;
        }
        ++o;
      }
  }
}

// One block: per k the first crossing of row 1 (0 where there is none), summed over
// k in a fixed order; out[0] = -(sum / nk)
__global__ void __launch_bounds__(1024) k_iface_lower(Grid g, double dx, double xl, const double* phi,
                                                      double* out) {
  __shared__ double sh[1024];
  const int t = (int)threadIdx.x;
  double acc = 0.0;
  for (int k = 1 + t; k <= g.nk; k += (int)blockDim.x) {
    double xk = 0.0, x;
    for (int i = 1; i <= g.ni; ++i)
      if (crossing(g, phi, i, 1, k, dx, xl, &x)) {
        xk = x;
        break;
      }
    acc += xk;
  }
  sh[t] = acc;
  __syncthreads();
  for (int st = (int)blockDim.x / 2; st > 0; st >>= 1) {
    if (t < st) sh[t] += sh[t + st];
    __syncthreads();
  }
  if (t == 0) out[0] = -(sh[0] / (double)g.nk);
}
}  // namespace

void diag_vel(cudaStream_t s, const Grid& g, double radius, double rhol, double rmul, const double* u,
              const double* v, const double* w, const double* phi, double* out) {
  const Grid G = g;
  double* sums = (double*)scratch(sizeof(double) * 4, 9);
  reduce_interior<4>(
      s, g,
      [=] __device__(int i, int j, int k, double* r) {
        const long c = G.at(i, j, k);
        const double p = phi[c];
        r[0] = p;
        r[1] = p * u[c];
        r[2] = p * v[c];
        r[3] = p * w[c];
      },
      sums);
  k_vel_finish<<<1, 1, 0, s>>>(sums, radius * 2.0, rhol, rmul, out);
  count_launch();
}

void diag_center_sums(cudaStream_t s, const Grid& g, int ID, double delta, double xl, int area_pre1, int lap,
                      const double* phi, double* out) {
  const Grid G = g;
  const double sensor1 = xl * 0.25, sensor2 = xl * 0.75, shift = xl * (double)lap;
  const int joff = ID * g.nj;
  reduce_interior<4>(
      s, g,
      [=] __device__(int i, int j, int k, double* r) {
        const double p = phi[G.at(i, j, k)];
        double x = delta * ((double)i - 0.5);
        if (area_pre1 == 3 && x < sensor1) x = x + xl;
        if (area_pre1 == 1 && x > sensor2) x = x - xl;
        x = x + shift;
        r[0] = p;
        r[1] = p * x;
        r[2] = p * (delta * ((double)(j + joff) - 0.5));
        r[3] = p * (delta * ((double)k - 0.5));
      },
      out);
}

void diag_interface_upper(cudaStream_t s, const Grid& g, double dx, double dz, double xl, const double* phi,
                          double* xz, int* count, int cap) {
  const int threads = g.nk >= 1024 ? 1024 : ((g.nk + 31) / 32) * 32;
  k_iface_upper<<<1, threads, 0, s>>>(g, dx, dz, xl, phi, xz, count, cap);
  count_launch();
}

void diag_interface_lower(cudaStream_t s, const Grid& g, double dx, double xl, const double* phi, double* out) {
  k_iface_lower<<<1, 1024, 0, s>>>(g, dx, xl, phi, out);
  count_launch();
}

}  // namespace op
}  // namespace fmf
