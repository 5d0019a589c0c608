// noalloc.cu -- an interior-mean entry point that allocates no device memory.
//
// Who needs it: code that already owns every device buffer it may use and is not
// allowed to allocate more while it runs -- a solver embedded in another
// framework's memory pool or arena (where a stray cudaMalloc would fragment or
// exceed the pool), a caller in the middle of its own stream-ordered work that
// cannot afford the device-wide synchronisation cudaMalloc/cudaFree can imply,
// or a long-running service with a fixed memory budget.  The regular cal_av_
// (cal_av.f) takes host arrays and lets the library's registry and scratch
// allocator create device memory on demand; this variant takes device pointers
// for the input field and the result, and keeps its only scratch -- the per-block
// partial sums of the reduction -- in a fixed array compiled into the library.
//
// Limits and sharing:
//  * the partial-sum array holds kMaxPartials doubles (512 KiB); a grid needs
//    ceil(nj/8) * nk of them, so nj*nk up to about 524,288 (e.g. nj = nk = 512 at
//    the reduction's 8 rows per block), and nk at most 65535 (one block row per k
//    plane); larger grids are rejected with FMF_ERR_ARG before anything is
//    launched;
//  * the array lives in device memory of every GPU that loads the library, for
//    as long as the library stays loaded;
//  * all calls on one GPU share it and it keeps the last call's partial sums;
//    every partial is rewritten by each call before it is read, so nothing has
//    to be cleared between calls;
//  * two calls whose kernels overlap in time on the same GPU (different streams
//    or threads) race on the shared array; serialise them on one stream.
//  * set-up: the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and caches it (threads that
//    race on that first call store the same address); make that first call before
//    the caller starts any stream capture of its own.
//  * errors: each launch's own status is checked (cudaLaunchKernel); an error the
//    caller left pending in the runtime is neither reported as this call's nor
//    cleared.
#include <atomic>

#include "../../include/fmf_capi.h"
#include "fmf_common.cuh"

namespace {
constexpr long kMaxPartials = 65536;
constexpr int kMaxGridY = 65535;
__device__ __align__(256) double g_noalloc_partials[kMaxPartials];

constexpr int kMaxDevices = 64;
std::atomic<void*> g_partials_addr[kMaxDevices];  // static storage: starts as nullptr

__global__ void k_mean_finish(double* av, double cells) { av[0] = av[0] / cells; }

// a kernel launch that returns its own status
template <class... P, class... A>
cudaError_t launch(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t s, A... a) {
  void* args[] = {(void*)&a...};
  return cudaLaunchKernel((const void*)k, grid, block, args, 0, s);
}
}  // namespace

extern "C" int fmf_cal_av_noalloc(int ni, int nj, int nk, const double* q, double* av, void* stream) {
  auto p2 = [](int n) { return n >= 4 && (n & (n - 1)) == 0; };
  if (!p2(ni) || !p2(nj) || !p2(nk) || !q || !av) return FMF_ERR_ARG;
  const fmf::Grid g(ni, nj, nk);
  const dim3 grid((unsigned)((nj + 7) / 8), (unsigned)nk);
  const long nb = (long)grid.x * grid.y;
  if (nb > kMaxPartials || nk > kMaxGridY) {
    std::fprintf(stderr,
                 "fmf_cal_av_noalloc: grid %dx%dx%d needs %ld partial sums and %d block rows; the fixed array "
                 "holds %ld (nj*nk <= %ld) and nk may not exceed %d; use cal_av_ instead\n",
                 ni, nj, nk, nb, nk, kMaxPartials, kMaxPartials * 8, kMaxGridY);
    return FMF_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FMF_ERR_CUDA;
  void* addr = g_partials_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_partials);
    if (e != cudaSuccess || !addr) {
      std::fprintf(stderr, "fmf_cal_av_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return FMF_ERR_CUDA;
    }
    g_partials_addr[dev].store(addr, std::memory_order_release);
  }
  double* part = (double*)addr;
  cudaStream_t s = (cudaStream_t)stream;
  // the same two-stage fixed-order reduction as cal_av_ (one partial per k plane
  // and 8-row j chunk, then one block adds them in index order), then /N
  auto rowsum = [=] __device__(int i, int j, int k, double* r) { r[0] = q[g.at(i, j, k)]; };
  cudaError_t e = launch(fmf::k_reduce_rows<1, decltype(rowsum)>, grid, dim3(256), s, g, rowsum, part);
  if (e == cudaSuccess) e = launch(fmf::k_reduce_final<1>, dim3(1), dim3(256), s, (const double*)part, nb, av);
  if (e == cudaSuccess) e = launch(k_mean_finish, dim3(1), dim3(1), s, av, (double)g.cells());
  if (e != cudaSuccess) {
    std::fprintf(stderr, "fmf_cal_av_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return FMF_ERR_CUDA;
  }
  fmf::count_launch(3);
  return FMF_OK;
}
