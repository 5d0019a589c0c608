// k_press.cu -- C4: divergence, FFT + Thomas pressure Poisson solve, projection.
//
// The reference transforms each y-plane with the vendored Numerical Recipes fourn
// (solp_fft_tdma1.f:35, solp_fft_tdma3.f:36).  Here the same 2-D DFT (sign -1
// forward, /(ni*nk); sign +1 inverse, unnormalised) is computed by radix-2
// decimation-in-time FFTs in shared memory: one block per x-line, then one block
// per tile of 16 x-wavenumbers for the z-lines.
#include <map>
#include <vector>

#include "fft.cuh"
#include "recip.cuh"
#include "ops.cuh"

namespace fmf {
namespace op {

// caldiv.f:25-67 -- div over -1..n+3 and sqrt(sum(div^2)/N)+1e-99 into err_out[0].
void caldiv(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt,
            const double* u, const double* v, const double* w, double* div, double* err_out) {
  const Grid G = g;
  const double dtinv = 1.0 / dt;
  range3(s, -1, g.ni + 3, -1, g.nj + 3, -1, g.nk + 3, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    div[c] = ((-u[c - 1] + u[c]) * dxinv + (-v[c - G.sy] + v[c]) * dyinv + (-w[c - G.sz] + w[c]) * dzinv) * dtinv;
  });
  if (err_out) {
    reduce_interior<1>(s, g, [=] __device__(int i, int j, int k, double* r) {
      const double d = div[G.at(i, j, k)];
      r[0] = d * d;
    }, err_out);
    const double N = (double)g.cells();
    flat(s, 1, [=] __device__(long) { err_out[0] = sqrt(err_out[0] / N) + 1.0e-99; });
  }
}

namespace {
// x-lines: one block per (j,k) row.  Forward: real div -> complex T(kx, j, k).
__global__ void __launch_bounds__(256) k_fft_x_fwd(Grid g, const double* div, double* tr, double* ti,
                                                   const double2* tw) {
  extern __shared__ double sm[];
  const int L = g.ni;
  double* re = sm;
  double* im = sm + L;
  const int j = 1 + blockIdx.x, k = 1 + blockIdx.y;
  const long c0 = g.at(1, j, k);
  for (int a = threadIdx.x; a < L; a += blockDim.x) {
    re[a] = div[c0 + a];
    im[a] = 0.0;
  }
  __syncthreads();
  group_fft(re, im, L, -1.0, threadIdx.x, blockDim.x, tw);
  const long o = ((long)(k - 1) * g.nj + (j - 1)) * L;
  for (int a = threadIdx.x; a < L; a += blockDim.x) {
    tr[o + a] = re[a];
    ti[o + a] = im[a];
  }
}
// Inverse x: complex T(kx, j, k) -> real part into dp(1..ni, j, k).
__global__ void __launch_bounds__(256) k_fft_x_inv(Grid g, const double* tr, const double* ti, double* dp,
                                                   const double2* tw) {
  extern __shared__ double sm[];
  const int L = g.ni;
  double* re = sm;
  double* im = sm + L;
  const int j = 1 + blockIdx.x, k = 1 + blockIdx.y;
  const long o = ((long)(k - 1) * g.nj + (j - 1)) * L;
  for (int a = threadIdx.x; a < L; a += blockDim.x) {
    re[a] = tr[o + a];
    im[a] = ti[o + a];
  }
  __syncthreads();
  group_fft(re, im, L, +1.0, threadIdx.x, blockDim.x, tw);
  const long c0 = g.at(1, j, k);
  for (int a = threadIdx.x; a < L; a += blockDim.x) dp[c0 + a] = re[a];
}

constexpr int kTile = 16;  // x-wavenumbers per z-line block (16 threads per column)

// z-lines forward: T(kx, j, k) for kx in a tile -> phir(ix, j, iz) / (ni*nk), centred.
__global__ void __launch_bounds__(256) k_fft_z_fwd(Grid g, const double* tr, const double* ti, double* pr,
                                                   double* pi, const double2* tw) {
  extern __shared__ double sm[];
  const int L = g.nk, NI = g.ni, NJ = g.nj;
  const int j = 1 + blockIdx.y;
  const int kx0 = blockIdx.x * kTile;
  for (int e = threadIdx.x; e < L * kTile; e += blockDim.x) {
    const int col = e % kTile, kz = e / kTile;
    const long o = ((long)kz * NJ + (j - 1)) * NI + kx0 + col;
    sm[col * 2 * L + kz] = tr[o];
    sm[col * 2 * L + L + kz] = ti[o];
  }
  __syncthreads();
  const int col = threadIdx.x / 16;
  group_fft(sm + col * 2 * L, sm + col * 2 * L + L, L, -1.0, threadIdx.x % 16, 16, tw);
  const double scale = (double)((long)NI * g.nk);
  for (int e = threadIdx.x; e < L * kTile; e += blockDim.x) {
    const int cl = e % kTile, kz = e / kTile;
    const int ii = kx0 + cl;
    const int ix = (ii + NI / 2) % NI, iz = (kz + L / 2) % L;
    const long o = (long)ix + (long)NI * ((long)(j - 1) + (long)NJ * iz);
    pr[o] = sm[cl * 2 * L + kz] / scale;
    pi[o] = sm[cl * 2 * L + L + kz] / scale;
  }
}
// z-lines inverse: phir(ix, j, iz) -> T(kx, j, k)
__global__ void __launch_bounds__(256) k_fft_z_inv(Grid g, const double* pr, const double* pi, double* tr,
                                                   double* ti, const double2* tw) {
  extern __shared__ double sm[];
  const int L = g.nk, NI = g.ni, NJ = g.nj;
  const int j = 1 + blockIdx.y;
  const int kx0 = blockIdx.x * kTile;
  for (int e = threadIdx.x; e < L * kTile; e += blockDim.x) {
    const int cl = e % kTile, kz = e / kTile;
    const int ii = kx0 + cl;
    const int ix = (ii + NI / 2) % NI, iz = (kz + L / 2) % L;
    const long o = (long)ix + (long)NI * ((long)(j - 1) + (long)NJ * iz);
    sm[cl * 2 * L + kz] = pr[o];
    sm[cl * 2 * L + L + kz] = pi[o];
  }
  __syncthreads();
  const int col = threadIdx.x / 16;
  group_fft(sm + col * 2 * L, sm + col * 2 * L + L, L, +1.0, threadIdx.x % 16, 16, tw);
  for (int e = threadIdx.x; e < L * kTile; e += blockDim.x) {
    const int cl = e % kTile, kz = e / kTile;
    const long o = ((long)kz * NJ + (j - 1)) * NI + kx0 + cl;
    tr[o] = sm[cl * 2 * L + kz];
    ti[o] = sm[cl * 2 * L + L + kz];
  }
}
}  // namespace

// (cos, sin)(2 pi m / L) for m < L/2 in device memory, one table per length,
// kept for the life of the library.
const double2* fft_twiddles(int L) {
  static std::map<int, double2*> cache;
  auto it = cache.find(L);
  if (it != cache.end()) return it->second;
  std::vector<double2> h(L / 2 > 0 ? L / 2 : 1);
  const double two_pi = 6.283185307179586476925286766559;
  for (int m = 0; m < L / 2; ++m) {
    const double ang = two_pi * (double)m / (double)L;
    h[m] = make_double2(std::cos(ang), std::sin(ang));
  }
  double2* d = nullptr;
  if (!FMF_CUDA(cudaMalloc(&d, sizeof(double2) * h.size()))) return nullptr;
  FMF_CUDA(cudaMemcpy(d, h.data(), sizeof(double2) * h.size(), cudaMemcpyHostToDevice));
  cache[L] = d;
  return d;
}

// solp_fft_tdma1.f:20-48 (with trans_r2w's serial relabelling folded into the layout)
void fft_forward_planes(cudaStream_t s, const Grid& g, const double* div, double* pr, double* pi) {
  const long nm = g.cells();
  double* t = (double*)scratch(sizeof(double) * 2 * nm, 5);
  const double2 *twx = fft_twiddles(g.ni), *twz = fft_twiddles(g.nk);
  k_fft_x_fwd<<<dim3(g.nj, g.nk), 256, sizeof(double) * 2 * g.ni, s>>>(g, div, t, t + nm, twx);
  const size_t smz = sizeof(double) * 2 * g.nk * kTile;
  cudaFuncSetAttribute(k_fft_z_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz);
  k_fft_z_fwd<<<dim3(g.ni / kTile, g.nj), 256, smz, s>>>(g, t, t + nm, pr, pi, twz);
  count_launch(2);
}
// solp_fft_tdma3.f:20-45
void fft_inverse_planes(cudaStream_t s, const Grid& g, const double* pr, const double* pi, double* dp) {
  const long nm = g.cells();
  double* t = (double*)scratch(sizeof(double) * 2 * nm, 5);
  const double2 *twx = fft_twiddles(g.ni), *twz = fft_twiddles(g.nk);
  const size_t smz = sizeof(double) * 2 * g.nk * kTile;
  cudaFuncSetAttribute(k_fft_z_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz);
  k_fft_z_inv<<<dim3(g.ni / kTile, g.nj), 256, smz, s>>>(g, pr, pi, t, t + nm, twz);
  k_fft_x_inv<<<dim3(g.nj, g.nk), 256, sizeof(double) * 2 * g.ni, s>>>(g, t, t + nm, dp, twx);
  count_launch(2);
}

namespace {
// solp_fft_tdma2.f:46-86 -- one thread per (kx, kz) mode; the forward sweep leaves
// b in place and a in scratch, then back-substitution.
__global__ void __launch_bounds__(128) k_tdma(Grid g, double dx2r, double dz2r, double pi2_ni, double pi2_nk,
                                              const double* as_f, const double* an_f, const double* ap_f,
                                              double* pr, double* pi, double* at) {
  const int NI = g.ni, NJ = g.nj, NK = g.nk;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = 1 + blockIdx.y;
  if (ix >= NI) return;
  const int i = ix - NI / 2;
  const double c1x = cos((double)i * pi2_ni) * 2.0;
  const double c1z = cos((double)(k - NK / 2 - 1) * pi2_nk) * 2.0;
  const long base = ix + (long)NI * (long)NJ * (k - 1);
  const long mode = ix + (long)NI * (k - 1), nmode = (long)NI * NK;
  double a_prev = 0.0, br = 0.0, bi = 0.0;
  for (int j = 1; j <= NJ; ++j) {
    const double ap = ap_f[j + 2] + dx2r * (2.0 - c1x) + dz2r * (2.0 - c1z);
    const double d00 = -ap + as_f[j + 2] * a_prev;
    const double apinv = -d00 * recip_nr(fma(d00, d00, 1.0e-99));  // Newton-Raphson, no division
    const double a = apinv * an_f[j + 2];
    const long o = base + (long)NI * (j - 1);
    br = apinv * (-pr[o] + as_f[j + 2] * br);
    bi = apinv * (-pi[o] + as_f[j + 2] * bi);
    pr[o] = br;
    pi[o] = bi;
    at[(long)(j - 1) * nmode + mode] = a;
    a_prev = a;
  }
  double xr = pr[base + (long)NI * (NJ - 1)], xi = pi[base + (long)NI * (NJ - 1)];
  for (int j = NJ - 1; j >= 1; --j) {
    const long o = base + (long)NI * (j - 1);
    const double a = at[(long)(j - 1) * nmode + mode];
    xr = pr[o] + a * xr;
    xi = pi[o] + a * xi;
    pr[o] = xr;
    pi[o] = xi;
  }
}
}  // namespace

void tdma_modes(cudaStream_t s, const Grid& g, double rho, double dxinv, double dzinv, const double* as_f,
                const double* an_f, const double* ap_f, double* pr, double* pi) {
  const double pi_ = std::atan(1.0) * 4.0;
  const double dx2r = dxinv * dxinv / rho, dz2r = dzinv * dzinv / rho;
  const double pi2_ni = pi_ * 2.0 / (double)g.ni, pi2_nk = pi_ * 2.0 / (double)g.nk;
  double* at = (double*)scratch(sizeof(double) * g.cells(), 4);
  k_tdma<<<dim3((g.ni + 127) / 128, g.nk), 128, 0, s>>>(g, dx2r, dz2r, pi2_ni, pi2_nk, as_f, an_f, ap_f, pr, pi, at);
  count_launch();
}

// bnd_avzero.f:10-24
void bnd_avzero(cudaStream_t s, const Grid& g, double* q) {
  double* av = (double*)scratch(sizeof(double) * 2, 3);
  cal_av(s, g, q, av);
  flat(s, g.n, [=] __device__(long t) { q[t] = q[t] - av[0]; });
}

// corunp_explicit.f:21-75
void corunp_explicit(cudaStream_t s, const Grid& g, double rho, double dxinv, double dyinv,
                     double dzinv, double dt, const double* dp, const double* phat, double* un,
                     double* vn, double* wn, double* pn) {
  const Grid G = g;
  range3(s, 1, g.ni, 1, g.nj, 1, g.nk, [=] __device__(int i, int j, int k) {
    const long c = G.at(i, j, k);
    un[c] = un[c] + (dp[c] - dp[c + 1]) / rho * dxinv * dt;
    if (j <= G.nj - 1) vn[c] = vn[c] + (dp[c] - dp[c + G.sy]) / rho * dyinv * dt;
    wn[c] = wn[c] + (dp[c] - dp[c + G.sz]) / rho * dzinv * dt;
    pn[c] = phat[c] + dp[c];
  });
}

// solp_fft_tdma4.f:30-72
void poisson_residual(cudaStream_t s, const Grid& g, double rho, double dxinv, double dyinv, double dzinv,
                      const double* div, const double* dp, double* out) {
  const Grid G = g;
  const double aw = dxinv * dxinv / rho, ae = aw, as = dyinv * dyinv / rho, an = as, ab = dzinv * dzinv / rho,
               at = ab;
  const double ap = aw + ae + as + an + ab + at;
  reduce_interior<2>(s, g, [=] __device__(int i, int j, int k, double* r) {
    const long c = G.at(i, j, k);
    const double d = dp[c - G.sz] * ab + dp[c - G.sy] * as + dp[c - 1] * aw - dp[c] * ap + dp[c + 1] * ae +
                     dp[c + G.sy] * an + dp[c + G.sz] * at - div[c];
    r[0] = d * d;
    r[1] = div[c] * div[c];
  }, out);
}

}  // namespace op
}  // namespace fmf
