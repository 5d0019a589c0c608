// fused_press.cu -- the pressure Poisson solve of the fused step on the half
// spectrum (solp_fft_tdma1-3, main.f90:636-647).
//
// The reference transforms the real divergence with a complex 2-D DFT (sign -1,
// divided by ni*nk), solves a tridiagonal system in y per (kx, kz) mode, and takes
// the real part of the unnormalised inverse.  The input is real, so the spectrum is
// Hermitian, X(-kx, -kz) = conj X(kx, kz), and the per-mode systems of a mode and its
// mirror have the same real matrix: the modes kx = 0..ni/2 carry everything.  Here:
//  * x, forward (real to half complex): z[n] = x[2n] + i x[2n+1] through an
//    M = ni/2 point complex FFT, then E = (Z[m] + conj Z[M-m])/2,
//    O = (Z[m] - conj Z[M-m])/(2i), X[m] = E + exp(-2 pi i m/ni) O, m = 0..M;
//  * z, both directions: the ni/2+1 columns, complex FFT of length nk;
//  * y: the Thomas solve per mode (kx = 0..ni/2, kz = 0..nk-1) with the modified
//    wavenumbers of solp_fft_tdma2.f:46-86 (cos is even and periodic, so natural
//    wavenumbers give the reference's centred ones);
//  * x, inverse (half complex to real): Y[m] = (X[m] + conj X[M-m])
//    + i (X[m] - conj X[M-m]) exp(+2 pi i m/ni), an unnormalised M-point inverse
//    FFT, x[2n] = Re, x[2n+1] = Im -- the real part of the full inverse.
// Half the FFT and Thomas work of the full-spectrum drop-in path (op::fft_*,
// op::tdma_modes), which keeps the reference's full spectra for the C-ABI.
// Spectrum layout: (kx, j, kz) at kx + H ((j-1) + nj kz), H = ni/2 + 1.
#include "../../include/fmf_capi.h"
#include "fft.cuh"
#include "fused.cuh"
#include "recip.cuh"

namespace fmf {
namespace fused {

namespace {
constexpr int kRows = 4, kRowThreads = 64;  // x transforms: 4 rows of 64 threads per block
constexpr int kTileZ = 16;                  // z transforms: 16 columns of 16 threads per block

__global__ void __launch_bounds__(256) k_rfft_x_fwd(Grid g, const double* __restrict__ div, double* __restrict__ tr,
                                                    double* __restrict__ ti, const double2* __restrict__ twM,
                                                    const double2* __restrict__ twN) {
  extern __shared__ double sm[];
  const int M = g.ni / 2, H = M + 1;
  const int rl = threadIdx.x / kRowThreads, t = threadIdx.x % kRowThreads;
  const int r = blockIdx.x * kRows + rl;  // row (j, k), nj nk rows in all (a multiple of 4)
  const int j = 1 + r % g.nj, k = 1 + r / g.nj;
  double* re = sm + rl * 2 * M;
  double* im = re + M;
  const long c0 = g.at(1, j, k);
  for (int n = t; n < M; n += kRowThreads) {
    re[n] = div[c0 + 2 * n];
    im[n] = div[c0 + 2 * n + 1];
  }
  __syncthreads();
  group_fft(re, im, M, -1.0, t, kRowThreads, twM);
  const long o = ((long)(k - 1) * g.nj + (j - 1)) * H;
  for (int m = t; m < H; m += kRowThreads) {
    const int a = m % M, b = (M - m) % M;
    const double zr = re[a], zi = im[a], cr = re[b], ci = -im[b];  // Z[m], conj Z[M-m]
    const double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
    const double orr = 0.5 * (zi - ci), oi = -0.5 * (zr - cr);  // (Z - conj Z')/(2i)
    double wr = -1.0, wi = 0.0;                                  // exp(-2 pi i m/ni), m = M: -1
    if (m < M) {
      const double2 w = __ldg(twN + m);
      wr = w.x;
      wi = -w.y;
    }
    tr[o + m] = er + (wr * orr - wi * oi);
    ti[o + m] = ei + (wr * oi + wi * orr);
  }
}

__global__ void __launch_bounds__(256) k_rfft_x_inv(Grid g, const double* __restrict__ tr,
                                                    const double* __restrict__ ti, double* __restrict__ dp,
                                                    const double2* __restrict__ twM, const double2* __restrict__ twN) {
  extern __shared__ double sm[];
  const int M = g.ni / 2, H = M + 1;
  const int rl = threadIdx.x / kRowThreads, t = threadIdx.x % kRowThreads;
  const int r = blockIdx.x * kRows + rl;
  const int j = 1 + r % g.nj, k = 1 + r / g.nj;
  double* xr = sm + rl * (2 * H + 2 * M);
  double* xi = xr + H;
  double* yr = xi + H;
  double* yi = yr + M;
  const long o = ((long)(k - 1) * g.nj + (j - 1)) * H;
  for (int m = t; m < H; m += kRowThreads) {
    xr[m] = tr[o + m];
    xi[m] = ti[o + m];
  }
  __syncthreads();
  for (int m = t; m < M; m += kRowThreads) {
    const double ar = xr[m] + xr[M - m], ai = xi[m] - xi[M - m];  // X[m] + conj X[M-m]
    const double br = xr[m] - xr[M - m], bi = xi[m] + xi[M - m];  // X[m] - conj X[M-m]
    const double2 w = __ldg(twN + m);                               // exp(+2 pi i m/ni)
    const double cr = br * w.x - bi * w.y, ci = br * w.y + bi * w.x;
    yr[m] = ar - ci;
    yi[m] = ai + cr;
  }
  __syncthreads();
  group_fft(yr, yi, M, +1.0, t, kRowThreads, twM);
  const long c0 = g.at(1, j, k);
  for (int n = t; n < M; n += kRowThreads) {
    dp[c0 + 2 * n] = yr[n];
    dp[c0 + 2 * n + 1] = yi[n];
  }
}

// z transform of the half spectrum, 16 columns kx per block, one j per grid y;
// in and out in the spectrum layout (in place allowed), scaled by `scale`
__global__ void __launch_bounds__(256) k_fft_z_half(Grid g, const double* tr, const double* ti, double* pr,
                                                    double* pi, const double2* __restrict__ tw, double sgn,
                                                    double scale) {
  extern __shared__ double sm[];
  const int L = g.nk, H = g.ni / 2 + 1, NJ = g.nj;
  const int j = blockIdx.y;
  const int kx0 = blockIdx.x * kTileZ;
  for (int e = threadIdx.x; e < L * kTileZ; e += blockDim.x) {
    const int col = e % kTileZ, kz = e / kTileZ, kx = kx0 + col;
    const long o = ((long)kz * NJ + j) * H + kx;
    sm[col * 2 * L + kz] = kx < H ? tr[o] : 0.0;
    sm[col * 2 * L + L + kz] = kx < H ? ti[o] : 0.0;
  }
  __syncthreads();
  const int col = threadIdx.x / 16;
  group_fft(sm + col * 2 * L, sm + col * 2 * L + L, L, sgn, threadIdx.x % 16, 16, tw);
  for (int e = threadIdx.x; e < L * kTileZ; e += blockDim.x) {
    const int cl = e % kTileZ, kz = e / kTileZ, kx = kx0 + cl;
    if (kx >= H) continue;
    const long o = ((long)kz * NJ + j) * H + kx;
    pr[o] = sm[cl * 2 * L + kz] * scale;
    pi[o] = sm[cl * 2 * L + L + kz] * scale;
  }
}

// solp_fft_tdma2.f:46-86 per half-spectrum mode (kx, kz): one thread each; the
// forward sweep leaves b in place and a in `at`, then back-substitution
__global__ void __launch_bounds__(128) k_tdma_half(Grid g, double dx2r, double dz2r, double pi2_ni, double pi2_nk,
                                                   const double* __restrict__ as_f, const double* __restrict__ an_f,
                                                   const double* __restrict__ ap_f, double* pr, double* pi,
                                                   double* __restrict__ at) {
  const int H = g.ni / 2 + 1, NJ = g.nj;
  const int kx = blockIdx.x * blockDim.x + threadIdx.x;
  const int kz = blockIdx.y;
  if (kx >= H) return;
  const double c1x = cos((double)kx * pi2_ni) * 2.0;
  const double c1z = cos((double)kz * pi2_nk) * 2.0;
  const long mode = kx + (long)H * kz, nmode = (long)H * g.nk;
  const long base = kx + (long)H * NJ * kz;
  double a_prev = 0.0, br = 0.0, bi = 0.0;
  for (int j = 1; j <= NJ; ++j) {
    const double ap = ap_f[j + 2] + dx2r * (2.0 - c1x) + dz2r * (2.0 - c1z);
    const double d00 = -ap + as_f[j + 2] * a_prev;
    const double apinv = -d00 * recip_nr(fma(d00, d00, 1.0e-99));
    const double a = apinv * an_f[j + 2];
    const long o = base + (long)H * (j - 1);
    br = apinv * (-pr[o] + as_f[j + 2] * br);
    bi = apinv * (-pi[o] + as_f[j + 2] * bi);
    pr[o] = br;
    pi[o] = bi;
    at[(long)(j - 1) * nmode + mode] = a;
    a_prev = a;
  }
  double xr = pr[base + (long)H * (NJ - 1)], xi = pi[base + (long)H * (NJ - 1)];
  for (int j = NJ - 1; j >= 1; --j) {
    const long o = base + (long)H * (j - 1);
    const double a = at[(long)(j - 1) * nmode + mode];
    xr = pr[o] + a * xr;
    xi = pi[o] + a * xi;
    pr[o] = xr;
    pi[o] = xi;
  }
}

// The matrix of every mode's system is fixed by the grid and rho_g, so its
// elimination factors are formed once (k_tdma_coef: apinv and a of the forward
// sweep above, by the same expressions) and the solves only apply them
// (k_tdma_pre).  coef: [apinv | a], each (ni/2+1) nk nj doubles, index
// (j-1) nmode + mode.
__global__ void __launch_bounds__(128) k_tdma_coef(Grid g, double dx2r, double dz2r, double pi2_ni, double pi2_nk,
                                                   const double* __restrict__ as_f, const double* __restrict__ an_f,
                                                   const double* __restrict__ ap_f, double* __restrict__ coef) {
  const int H = g.ni / 2 + 1, NJ = g.nj;
  const int kx = blockIdx.x * blockDim.x + threadIdx.x;
  const int kz = blockIdx.y;
  if (kx >= H) return;
  const double c1x = cos((double)kx * pi2_ni) * 2.0;
  const double c1z = cos((double)kz * pi2_nk) * 2.0;
  const long mode = kx + (long)H * kz, nmode = (long)H * g.nk, nh = nmode * NJ;
  double a_prev = 0.0;
  for (int j = 1; j <= NJ; ++j) {
    const double ap = ap_f[j + 2] + dx2r * (2.0 - c1x) + dz2r * (2.0 - c1z);
    const double d00 = -ap + as_f[j + 2] * a_prev;
    const double apinv = -d00 * recip_nr(fma(d00, d00, 1.0e-99));
    const double a = apinv * an_f[j + 2];
    coef[(long)(j - 1) * nmode + mode] = apinv;
    coef[nh + (long)(j - 1) * nmode + mode] = a;
    a_prev = a;
  }
}
__global__ void __launch_bounds__(128) k_tdma_pre(Grid g, const double* __restrict__ as_f,
                                                  const double* __restrict__ coef, double* pr, double* pi) {
  const int H = g.ni / 2 + 1, NJ = g.nj;
  const int kx = blockIdx.x * blockDim.x + threadIdx.x;
  const int kz = blockIdx.y;
  if (kx >= H) return;
  const long mode = kx + (long)H * kz, nmode = (long)H * g.nk, nh = nmode * NJ;
  const long base = kx + (long)H * NJ * kz;
  double br = 0.0, bi = 0.0;
  for (int j = 1; j <= NJ; ++j) {
    const double apinv = __ldg(coef + (long)(j - 1) * nmode + mode);
    const long o = base + (long)H * (j - 1);
    br = apinv * (-pr[o] + as_f[j + 2] * br);
    bi = apinv * (-pi[o] + as_f[j + 2] * bi);
    pr[o] = br;
    pi[o] = bi;
  }
  double xr = br, xi = bi;
  for (int j = NJ - 1; j >= 1; --j) {
    const long o = base + (long)H * (j - 1);
    const double a = __ldg(coef + nh + (long)(j - 1) * nmode + mode);
    xr = pr[o] + a * xr;
    xi = pi[o] + a * xi;
    pr[o] = xr;
    pi[o] = xi;
  }
}

// corunp_explicit.f:26-75 with the constant dt dxinv / rho formed once on the host
// (the reference divides by rho at every point)
__global__ void __launch_bounds__(256) k_project(Grid g, double cx, double cy, double cz,
                                                 const double* __restrict__ dp, const double* __restrict__ phat,
                                                 double* __restrict__ un, double* __restrict__ vn,
                                                 double* __restrict__ wn, double* __restrict__ pn) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long c = g.at(i, j, k);
  const double d0 = __ldg(dp + c);
  un[c] = fma(d0 - __ldg(dp + c + 1), cx, un[c]);
  if (j <= g.nj - 1) vn[c] = fma(d0 - __ldg(dp + c + g.sy), cy, vn[c]);
  wn[c] = fma(d0 - __ldg(dp + c + g.sz), cz, wn[c]);
  pn[c] = __ldg(phat + c) + d0;
}
}  // namespace

long tdma_coef_doubles(const Grid& g) { return 2L * (g.ni / 2 + 1) * g.nj * g.nk; }

void tdma_coef(cudaStream_t s, const Grid& g, double rho, double dxinv, double dzinv, const double* as_f,
               const double* an_f, const double* ap_f, double* coef) {
  const int H = g.ni / 2 + 1;
  const double pi_ = 3.141592653589793238462643383279502884;
  k_tdma_coef<<<dim3((unsigned)((H + 127) / 128), (unsigned)g.nk), 128, 0, s>>>(
      g, dxinv * dxinv / rho, dzinv * dzinv / rho, pi_ * 2.0 / (double)g.ni, pi_ * 2.0 / (double)g.nk, as_f, an_f,
      ap_f, coef);
  count_launch();
}

void pressure_half(cudaStream_t s, const Grid& g, double rho, double dxinv, double dzinv, const double* as_f,
                   const double* an_f, const double* ap_f, const double* div, double* pr, double* pi, double* dp,
                   const double* coef) {
  const long nh = (long)(g.ni / 2 + 1) * g.nj * g.nk;
  double* tr = (double*)scratch(sizeof(double) * 2 * nh, 5);
  double* ti = tr + nh;
  double* at = coef ? nullptr : (double*)scratch(sizeof(double) * nh, 4);
  const int M = g.ni / 2, H = M + 1;
  const double2 *twM = op::fft_twiddles(M), *twN = op::fft_twiddles(g.ni), *twz = op::fft_twiddles(g.nk);
  const int rows = g.nj * g.nk;  // a multiple of kRows for power-of-two nj, nk >= 4
  const size_t smf = sizeof(double) * kRows * 2 * M, smi = sizeof(double) * kRows * (2 * H + 2 * M);
  const size_t smz = sizeof(double) * 2 * g.nk * kTileZ;
  // shared memory per block: 227 KB at most on this GPU (ni up to 1024, nk up to 512)
  if (smi > 232448 || smz > 232448) {
    set_status(FMF_ERR_ARG);
    return;
  }
  cudaFuncSetAttribute(k_rfft_x_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf);
  cudaFuncSetAttribute(k_rfft_x_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smi);
  k_rfft_x_fwd<<<rows / kRows, 256, smf, s>>>(g, div, tr, ti, twM, twN);
  cudaFuncSetAttribute(k_fft_z_half, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz);
  const dim3 gz((unsigned)((H + kTileZ - 1) / kTileZ), (unsigned)g.nj);
  k_fft_z_half<<<gz, 256, smz, s>>>(g, tr, ti, pr, pi, twz, -1.0, 1.0 / ((double)g.ni * (double)g.nk));
  const double pi_ = 3.141592653589793238462643383279502884;
  const double dx2r = dxinv * dxinv / rho, dz2r = dzinv * dzinv / rho;
  if (coef)
    k_tdma_pre<<<dim3((unsigned)((H + 127) / 128), (unsigned)g.nk), 128, 0, s>>>(g, as_f, coef, pr, pi);
  else
    k_tdma_half<<<dim3((unsigned)((H + 127) / 128), (unsigned)g.nk), 128, 0, s>>>(
        g, dx2r, dz2r, pi_ * 2.0 / (double)g.ni, pi_ * 2.0 / (double)g.nk, as_f, an_f, ap_f, pr, pi, at);
  k_fft_z_half<<<gz, 256, smz, s>>>(g, pr, pi, tr, ti, twz, +1.0, 1.0);
  k_rfft_x_inv<<<rows / kRows, 256, smi, s>>>(g, tr, ti, dp, twM, twN);
  count_launch(5);
}

void project(cudaStream_t s, const Grid& g, double rho, double dxinv, double dyinv, double dzinv, double dt,
             const double* dp, const double* phat, double* un, double* vn, double* wn, double* pn) {
  k_project<<<dim3((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk), dim3(32, 8), 0, s>>>(
      g, dt * dxinv / rho, dt * dyinv / rho, dt * dzinv / rho, dp, phat, un, vn, wn, pn);
  count_launch();
}

}  // namespace fused
}  // namespace fmf
