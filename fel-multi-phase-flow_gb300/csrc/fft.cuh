// fft.cuh -- the shared-memory FFT of the pressure solve's x and z transforms.
#pragma once
#include <cuda_runtime.h>

namespace fmf {

// In-place decimation-in-time FFT of L complex values (L a power of two) in shared
// memory (re, im), run by the nthr threads t = 0..nthr-1 of a group; every thread
// of the block reaches the same __syncthreads.  tw[m] = (cos, sin)(2 pi m / L),
// m < L/2, computed on the host; sign sgn = -1 forward, +1 inverse.  After the
// bit-reversal permutation the radix-2 stages are taken two at a time (radix
// 2^2): with span h, the four points x0..x3 at a, a+h, a+2h, a+3h (m = a mod h)
// and w = W_4h^m,
//   t1 = w^2 x1, t2 = w x2, t3 = w^3 x3,
//   X0 = x0 + t1 + (t2 + t3),  X2 = x0 + t1 - (t2 + t3),
//   X1 = x0 - t1 + sgn i (t2 - t3),  X3 = x0 - t1 - sgn i (t2 - t3),
// which is the two radix-2 stages of spans h and 2h (W_4h^h = sgn i) with three
// twiddle products instead of four and one pass over shared memory instead of
// two; a single radix-2 stage first where log2 L is odd.
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
  int h = 1;
  if (lg & 1) {
    // span 1: twiddles 1
    for (int q = t; q < L / 2; q += nthr) {
      const int a = 2 * q, b = a + 1;
      const double ar = re[a], ai = im[a], br = re[b], bi = im[b];
      re[a] = ar + br;
      im[a] = ai + bi;
      re[b] = ar - br;
      im[b] = ai - bi;
    }
    __syncthreads();
    h = 2;
  }
  for (; h < L; h <<= 2) {
    const int step = L / (4 * h);  // W_4h^k = tw[k step] (k < 2h)
    for (int q = t; q < L / 4; q += nthr) {
      const int m = q & (h - 1), a = (q - m) * 4 + m;
      const double x0r = re[a], x0i = im[a], x1r = re[a + h], x1i = im[a + h];
      const double x2r = re[a + 2 * h], x2i = im[a + 2 * h], x3r = re[a + 3 * h], x3i = im[a + 3 * h];
      double t1r = x1r, t1i = x1i, t2r = x2r, t2i = x2i, t3r = x3r, t3i = x3i;
      if (m) {
        const double2 w1 = __ldg(tw + m * step), w2 = __ldg(tw + 2 * m * step);
        const int k3 = 3 * m;
        double2 w3;
        double s3 = 1.0;
        if (k3 < 2 * h) {
          w3 = __ldg(tw + k3 * step);
        } else {  // W^k = -W^(k - 2h)
          w3 = __ldg(tw + (k3 - 2 * h) * step);
          s3 = -1.0;
        }
        const double c1 = w1.x, s1 = sgn * w1.y, c2 = w2.x, s2 = sgn * w2.y, c3 = s3 * w3.x, sn3 = s3 * sgn * w3.y;
        t1r = c2 * x1r - s2 * x1i;  // w^2 x1
        t1i = c2 * x1i + s2 * x1r;
        t2r = c1 * x2r - s1 * x2i;  // w x2
        t2i = c1 * x2i + s1 * x2r;
        t3r = c3 * x3r - sn3 * x3i;  // w^3 x3
        t3i = c3 * x3i + sn3 * x3r;
      }
      const double s0r = x0r + t1r, s0i = x0i + t1i, d0r = x0r - t1r, d0i = x0i - t1i;
      const double s1r = t2r + t3r, s1i = t2i + t3i, d1r = t2r - t3r, d1i = t2i - t3i;
      re[a] = s0r + s1r;
      im[a] = s0i + s1i;
      re[a + 2 * h] = s0r - s1r;
      im[a + 2 * h] = s0i - s1i;
      // sgn i d1 = (-sgn d1i, sgn d1r)
      re[a + h] = d0r - sgn * d1i;
      im[a + h] = d0i + sgn * d1r;
      re[a + 3 * h] = d0r + sgn * d1i;
      im[a + 3 * h] = d0i - sgn * d1r;
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
