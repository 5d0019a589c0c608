// probe.cu -- arithmetic-rate probe used as the FP64/FP32 roofline denominators.
//
// The measured-peaks file of the run gives the HBM copy rate and the bf16 tensor
// rate; the kernels of this library are bounded by FP64 (non-tensor) throughput,
// so bench.py measures that rate live: 152*8 blocks of 256 threads, each thread
// 8 independent multiply-add chains (enough independent work to fill every FP64
// pipe), timed with CUDA events after a warm-up launch.  Reads no memory; writes
// one value per thread so the chains are not removed.  Also here: the error
// checks of the division-free reciprocal and reciprocal square root (recip.cuh)
// against CUDA's own 1.0 / x and 1.0 / sqrt(x).
#include <cstring>

#include "../../include/fmf_capi.h"
#include "fmf_common.cuh"
#include "recip.cuh"

namespace {
// explicit fused multiply-add (this file is built without automatic contraction)
__device__ __forceinline__ double mad(double x, double a, double b) { return fma(x, a, b); }
__device__ __forceinline__ float mad(float x, float a, float b) { return fmaf(x, a, b); }

template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3, x4 = x0 + (T)4, x5 = x0 + (T)5,
    x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int t = 0; t < iters; ++t) {
    x0 = mad(x0, a, b);
    x1 = mad(x1, a, b);
    x2 = mad(x2, a, b);
    x3 = mad(x3, a, b);
    x4 = mad(x4, a, b);
    x5 = mad(x5, a, b);
    x6 = mad(x6, a, b);
    x7 = mad(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template <class T>
int measure(int iters, double* tflops) {
  const int blocks = 152 * 8, thr = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * thr) != cudaSuccess) return FMF_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<T><<<blocks, thr>>>(out, 16, (T)0.999, (T)1e-3);
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, thr>>>(out, iters, (T)0.999, (T)1e-3);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  fmf::count_launch(2);
  *tflops = 2.0 * 8.0 * (double)iters * blocks * thr / (ms * 1e-3) / 1e12;
  return cudaGetLastError() == cudaSuccess ? FMF_OK : FMF_ERR_CUDA;
}

// n positive normal doubles spread over exponents 2^-1000 .. 2^1000 with
// pseudo-random mantissas (a 64-bit mix of the index); the largest relative error
// of recip_nr (which = 0) against the IEEE quotient 1.0 / x, or of rsqrt_nr
// (which = 1) against 1.0 / sqrt(x), as ordered bits of a non-negative double.
__global__ void k_check_recip(long n, int which, unsigned long long* worst) {
  unsigned long long m = 0;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    unsigned long long h = (unsigned long long)t * 0x9E3779B97F4A7C15ull;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    const long long e = 1023 + (long long)(t % 2001) - 1000;
    const double x = __longlong_as_double((long long)((e << 52) | (h & 0xFFFFFFFFFFFFFull)));
    const double q = which ? 1.0 / sqrt(x) : 1.0 / x, r = which ? fmf::rsqrt_nr(x) : fmf::recip_nr(x);
    const double rel = fabs(r - q) / q;
    const unsigned long long b = (unsigned long long)__double_as_longlong(rel);
    m = b > m ? b : m;
  }
  atomicMax(worst, m);
}
int check_recip(long long n, int which, double* max_rel_err) {
  if (!max_rel_err || n <= 0) return FMF_ERR_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return FMF_ERR_NOMEM;
  cudaMemset(d, 0, sizeof(unsigned long long));
  k_check_recip<<<152 * 4, 256>>>((long)n, which, d);
  fmf::count_launch();
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return FMF_ERR_CUDA;
  std::memcpy(max_rel_err, &h, sizeof(double));
  return FMF_OK;
}
}  // namespace

extern "C" int fmf_check_reciprocal(long long n, double* max_rel_err) { return check_recip(n, 0, max_rel_err); }
extern "C" int fmf_check_rsqrt(long long n, double* max_rel_err) { return check_recip(n, 1, max_rel_err); }

extern "C" int fmf_measure_fma_rate(int fp64, double* tflops) {
  if (!tflops) return FMF_ERR_ARG;
  return fp64 ? measure<double>(2000, tflops) : measure<float>(20000, tflops);
}
