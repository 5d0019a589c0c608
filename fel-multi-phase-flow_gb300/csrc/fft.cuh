// fft.cuh -- the shared-memory FFT of the pressure solve's x and z transforms.
#pragma once
#include <cuda_runtime.h>

namespace fmf {

// In-place radix-2 decimation-in-time FFT of L complex values in shared memory
// (re, im), run by the nthr threads t = 0..nthr-1 of a group; every thread of the
// block reaches the same __syncthreads.  tw[m] = (cos, sin)(2 pi m / L), m < L/2,
// computed on the host; stage len uses tw[m * L/len] (the same angle as
// 2 pi m / len), sign -1 forward, +1 inverse.
__device__ __forceinline__ void group_fft(double* re, double* im, int L, double sgn, int t, int nthr,
                                          const double2* __restrict__ tw) {
  int lg = 0;
  while ((1 << lg) < L) ++lg;
  for (int a = t; a < L; a += nthr) {
    const int b = (int)(__brev((unsigned)a) >> (32 - lg));
    if (a < b) {
      const double t0 = re[a], t1 = im[a];
      re[a] = re[b];
      im[a] = im[b];
      re[b] = t0;
      im[b] = t1;
    }
  }
  __syncthreads();
  for (int len = 2, step = L / 2; len <= L; len <<= 1, step >>= 1) {
    const int h = len >> 1;
    for (int q = t; q < L / 2; q += nthr) {
      const int m = q & (h - 1), a = (q - m) * 2 + m, b = a + h;
      const double2 w = __ldg(tw + m * step);
      const double wr = w.x, wi = sgn * w.y;
      const double xr = wr * re[b] - wi * im[b];
      const double xi = wr * im[b] + wi * re[b];
      re[b] = re[a] - xr;
      im[b] = im[a] - xi;
      re[a] = re[a] + xr;
      im[a] = im[a] + xi;
    }
    __syncthreads();
  }
}

namespace op {
// (cos, sin)(2 pi m / L) for m < L/2 in device memory, one table per length, kept
// for the life of the library.
const double2* fft_twiddles(int L);
}  // namespace op

}  // namespace fmf
