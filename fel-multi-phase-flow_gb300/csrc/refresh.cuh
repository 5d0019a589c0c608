// refresh.cuh -- index maps of the wall/halo refresh (bndu.f + bnd_periodic.f) for
// the one-pass refresh kernel and its transpose.  Along a periodic direction with N
// interior points the destinations are -2, -1, 0 (from N-2..N) and N+1, N+2, N+3
// (from 1..3); bndu's shifted copy (sh = 1) takes -2..0 from N-1..N+1 and keeps N+1.
// For N >= 8 the map is injective and its sources are never destinations.
#pragma once

namespace fmf {

// the source of index i (i itself when i is not a destination)
__host__ __device__ __forceinline__ int halo_src(int i, int N, int sh) {
  if (i <= 0) return N + sh + i;
  if (i >= N + 2 || (i == N + 1 && !sh)) return i - N;
  return i;
}
// destination slot s in 0..5 -> -2, -1, 0, N+1, N+2, N+3; kNoHalo for N+1 under the
// shifted copy
constexpr int kNoHalo = -100;
__host__ __device__ __forceinline__ int halo_dest(int s, int N, int sh) {
  if (s < 3) return s - 2;
  if (s == 3 && sh) return kNoHalo;
  return N + s - 2;
}
// the destination whose source is i, or kNoHalo
__host__ __device__ __forceinline__ int halo_image(int i, int N, int sh) {
  if (i >= N - 2 + sh && i <= N + sh) return i - N - sh;
  if (i >= 1 + sh && i <= 3) return i + N;
  return kNoHalo;
}
// the one-pass kernels need the maps above to be injective and row ranges -2..2,
// 3..nj-4, nj-3..nj+3 to be disjoint
__host__ __device__ __forceinline__ bool refresh_one_pass(int ni, int nj, int nk) {
  return ni >= 8 && nj >= 8 && nk >= 8;
}

}  // namespace fmf
