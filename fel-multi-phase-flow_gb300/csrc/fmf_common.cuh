// fmf_common.cuh -- shared definitions of the sm_103a kernels.
//
// Field layout in HBM: the reference's own Fortran layout, so host arrays move to
// and from the device with one contiguous copy: element (i,j,k) of a
// (-2:ni+3, -2:nj+3, -2:nk+3) array sits at (i+2) + nx*((j+2) + ny*(k+2)) with
// nx = ni+6, ny = nj+6 (i fastest; a warp reads 32 consecutive i = 256 B).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

namespace fmf {

struct Grid {
  int ni, nj, nk;
  int nx, ny, nz;     // padded extents ni+6, nj+6, nk+6
  long sy, sz, n;     // strides in elements and the element count
  __host__ __device__ Grid() {}
  __host__ __device__ Grid(int a, int b, int c)
      : ni(a), nj(b), nk(c), nx(a + 6), ny(b + 6), nz(c + 6), sy(a + 6), sz((long)(a + 6) * (b + 6)),
        n((long)(a + 6) * (b + 6) * (c + 6)) {}
  __host__ __device__ __forceinline__ long at(int i, int j, int k) const {
    return (long)(i + 2) + sy * (long)(j + 2) + sz * (long)(k + 2);
  }
  __host__ __device__ long cells() const { return (long)ni * nj * nk; }
};

// ---- status --------------------------------------------------------------
void set_status(int code);
int get_status();
bool cuda_ok(cudaError_t e, const char* where);
#define FMF_CUDA(call) ::fmf::cuda_ok((call), #call)
void count_launch(int n = 1);
cudaStream_t stream();
void* scratch(size_t bytes, int slot);  // per-slot growable device scratch (library owned)

// ---- index-range launcher ------------------------------------------------
// fn(i,j,k) for i in [i0,i1], j in [j0,j1], k in [k0,k1]; 32x8 threads per block,
// one k plane per grid z index.
template <class Fn>
__global__ void __launch_bounds__(256) k_range3(int i0, int i1, int j0, int j1, int k0, Fn fn) {
  const int i = i0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = k0 + (int)blockIdx.z;
  if (i <= i1 && j <= j1) fn(i, j, k);
}
template <class Fn>
inline void range3(cudaStream_t s, int i0, int i1, int j0, int j1, int k0, int k1, Fn fn) {
  if (i1 < i0 || j1 < j0 || k1 < k0) return;
  dim3 b(32, 8, 1);
  dim3 g((unsigned)((i1 - i0 + 32) / 32), (unsigned)((j1 - j0 + 8) / 8), (unsigned)(k1 - k0 + 1));
  k_range3<<<g, b, 0, s>>>(i0, i1, j0, j1, k0, fn);
  count_launch();
}
// fn(a,b) over a 2-D index range (plane kernels)
template <class Fn>
__global__ void __launch_bounds__(256) k_range2(int a0, int a1, int b0, int b1, Fn fn) {
  const int a = a0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int b = b0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (a <= a1 && b <= b1) fn(a, b);
}
template <class Fn>
inline void range2(cudaStream_t s, int a0, int a1, int b0, int b1, Fn fn) {
  if (a1 < a0 || b1 < b0) return;
  dim3 bl(32, 8, 1);
  dim3 g((unsigned)((a1 - a0 + 32) / 32), (unsigned)((b1 - b0 + 8) / 8), 1);
  k_range2<<<g, bl, 0, s>>>(a0, a1, b0, b1, fn);
  count_launch();
}
// fn(t) over a flat element range
template <class Fn>
__global__ void __launch_bounds__(256) k_flat(long n, Fn fn) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) fn(t);
}
template <class Fn>
inline void flat(cudaStream_t s, long n, Fn fn) {
  if (n <= 0) return;
  long blocks = (n + 255) / 256;
  if (blocks > 152L * 16) blocks = 152L * 16;
  k_flat<<<(unsigned)blocks, 256, 0, s>>>(n, fn);
  count_launch();
}

// ---- deterministic interior reductions ----------------------------------
// Sum of fn(i,j,k) over the interior, in a fixed order: one partial per (k, 8-row
// j chunk) from a fixed-shape block tree, then a single block adds the partials
// in index order.  out[slot] receives the sum (device memory).
template <int NV, class Fn>
__global__ void __launch_bounds__(256) k_reduce_rows(Grid g, Fn fn, double* part) {
  __shared__ double sh[NV][256];
  const int tid = threadIdx.x;
  const int k = 1 + blockIdx.y;
  const int j0 = 1 + blockIdx.x * 8;
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
  for (int jj = 0; jj < 8; ++jj) {
    const int j = j0 + jj;
    if (j > g.nj) break;
    for (int i = 1 + tid; i <= g.ni; i += 256) {
      double r[NV];
      fn(i, j, k, r);
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] += r[v];
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) sh[v][tid] = acc[v];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (tid < s) {
#pragma unroll
      for (int v = 0; v < NV; ++v) sh[v][tid] += sh[v][tid + s];
    }
    __syncthreads();
  }
  if (tid == 0) {
    const long b = (long)blockIdx.y * gridDim.x + blockIdx.x;
    const long nb = (long)gridDim.x * gridDim.y;
#pragma unroll
    for (int v = 0; v < NV; ++v) part[v * nb + b] = sh[v][0];
  }
}
template <int NV>
__global__ void __launch_bounds__(256) k_reduce_final(const double* part, long nb, double* out) {
  __shared__ double sh[NV][256];
  const int tid = threadIdx.x;
  for (int v = 0; v < NV; ++v) {
    double a = 0.0;
    for (long b = tid; b < nb; b += 256) a += part[v * nb + b];
    sh[v][tid] = a;
  }
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (tid < s)
      for (int v = 0; v < NV; ++v) sh[v][tid] += sh[v][tid + s];
    __syncthreads();
  }
  if (tid == 0)
    for (int v = 0; v < NV; ++v) out[v] = sh[v][0];
}
// fn(i,j,k, double r[NV]); writes NV sums to out[0..NV-1] (device)
template <int NV, class Fn>
inline void reduce_interior(cudaStream_t s, const Grid& g, Fn fn, double* out, int slot = 7) {
  dim3 gr((unsigned)((g.nj + 7) / 8), (unsigned)g.nk);
  const long nb = (long)gr.x * gr.y;
  double* part = (double*)scratch(sizeof(double) * NV * nb, slot);
  k_reduce_rows<NV><<<gr, 256, 0, s>>>(g, fn, part);
  k_reduce_final<NV><<<1, 256, 0, s>>>(part, nb, out);
  count_launch(2);
}

}  // namespace fmf
