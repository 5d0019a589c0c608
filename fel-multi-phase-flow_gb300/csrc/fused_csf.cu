// fused_csf.cu -- CSF surface-tension force of one volume-fraction field in one
// pass (main.f90:548-567: cal_grad_p2a, calrn x4, calrkap, cal_grad_p2uvw, calfst).
//
// Per interior cell the force on the u, v, w faces is
//   f_u = -(2 sigma/(rho_l+rho_g)) * kappa_u * (phi(i+1)-phi(i))/dx   (calfst.f:40-42)
// with kappa_u the divergence of the unit normal over the u control volume
// (calrkap.f:45-98), built from four families of normals (calrn.f:45-87):
//   npp at cell centres  = N(mean of the 8 vertex gradients around the cell),
//   n12 at (i+1/2,j+1/2,k) = N(mean of vertex gradients k-1/2, k+1/2),
//   n13 at (i+1/2,j,k+1/2) = N(mean over j-1/2, j+1/2),
//   n23 at (i,j+1/2,k+1/2) = N(mean over i-1/2, i+1/2),
// N(v) = v/(|v| + 1e-30*|dxinv|) and vertex gradients from cal_grad_p2a.f:46-60.
//
// A block owns a 32 x 8 tile of (i,j) columns and marches over a chunk of k planes.
// Vertex gradients G of planes k, k+1 and the normals of planes k-1..k+1 live in
// shared memory; H(k+1) = G(k)+G(k+1) gives both n12(k+1) and, summed over the
// four surrounding (i,j), npp(k+1).  Each normal is formed once per block.
//
// Three instantiations: R = double (the FP64 step; phi read straight from global
// memory), R = float (the mixed-precision step; each phi plane is converted once
// into a shared-memory ring of three planes, everything after that is FP32 and the
// three forces are widened to double on the store) and R = Pr, an FP32 pair (the
// FP64-accurate step FMF_FP64E: phi planes split into pairs in the same ring, the
// arithmetic in FP32-pair operations on the FP32 pipe, the forces rounded to double).
#include <algorithm>
#include <type_traits>

#include "df64.cuh"
#include "fused.cuh"
#include "recip.cuh"

namespace fmf {
namespace fused {

namespace {
constexpr int TX = 32, TY = 8;
constexpr int GX = TX + 2, GY = TY + 2;  // G and H region: i in [I0-1, I0+TX], j in [J0-1, J0+TY]
constexpr int NX = TX + 1, NY = TY + 1;  // normal regions
constexpr int GP = GX * GY, NP = NX * NY;
constexpr int QX = GX + 1, QY = GY + 1;  // staged phi plane: i in [I0-1, I0+TX+1], j in [J0-1, J0+TY+1]
constexpr int QP = QX * QY;

// FP32 pair (df64.cuh) with the arithmetic operators the kernel's template uses
struct Pr {
  df::D v;
  Pr() = default;
  __host__ __device__ Pr(df::D d) : v(d) {}
  __host__ __device__ explicit Pr(double q) : v(df::split_double(q)) {}
  __device__ explicit operator double() const { return df::to_double(v); }
};
__host__ __device__ __forceinline__ Pr operator+(Pr a, Pr b) { return df::add(a.v, b.v); }
__host__ __device__ __forceinline__ Pr operator-(Pr a, Pr b) { return df::sub(a.v, b.v); }
__host__ __device__ __forceinline__ Pr operator*(Pr a, Pr b) { return df::mul(a.v, b.v); }
__host__ __device__ __forceinline__ Pr operator-(Pr a) { return df::neg(a.v); }

template <class R>
constexpr bool kStaged = !std::is_same<R, double>::value;

template <class R>
struct CsfP {
  R dxi, dyi, dzi, gx, gy, gz, vs2, vs8;  // vs2 = 2 vs, vs8 = 8 vs
  R fx, fy, fz;                           // -(2 sigma/(rho_l + rho_g)) dxinv etc. (calfst.f:40-42)
};

template <class R>
struct Smem {
  R G[2][3][GP];    // vertex gradients, two planes (ring)
  R H[3][GP];       // G(k) + G(k+1)
  R pp[2][3][NP];   // npp, planes k and k+1 (ring); region i in [I0, I0+TX], j in [J0, J0+TY]
  R a12[2][2][NP];  // n12 (x, y), planes k and k+1; region i in [I0-1, I0+TX-1], j in [J0-1, J0+TY-1]
  R a13[2][2][NP];  // n13 (x, z), planes k-1 and k; same region
  R a23[2][2][NP];  // n23 (y, z), planes k-1 and k; same region
  R Q[kStaged<R> ? 3 : 1][kStaged<R> ? QP : 1];  // staged phi planes, slot = plane % 3
};

// N(v) = v/(|v| + vs).  Where |v| exceeds vs by more than 1e12 the relative
// correction vs/|v| is below 1e-12 and 1/|v| is used; smaller |v| (including zero
// gradients) takes the exact expression.  Callers pass v scaled by 1/c (a sum
// instead of a mean) with vs scaled by 1/c: N(c w) = w/(|w| + vs/c).
__device__ __forceinline__ void unit(double x, double y, double z, double vs, double* o) {
  const double s = x * x + y * y + z * z;
  const double big = vs * 1.0e12;
  // s > big^2 compared on the bit patterns (both non-negative; no FP64-pipe compare)
  const bool far = __double_as_longlong(s) > __double_as_longlong(big * big);
  const double inv = far ? rsqrt_nr(s) : 1.0 / (sqrt(s) + vs);
  o[0] = x * inv;
  o[1] = y * inv;
  o[2] = z * inv;
}
// FP32: where |v| < 1e-15 the squares would leave the normal range, so numerator
// and denominator are both scaled by 2^64 first (an exact power-of-two scaling).
__device__ __forceinline__ void unit(float x, float y, float z, float vs, float* o) {
  float s = x * x + y * y + z * z;
  if (s < 1.0e-30f) {
    const float c = 18446744073709551616.0f;  // 2^64
    x *= c;
    y *= c;
    z *= c;
    vs *= c;
    s = x * x + y * y + z * z;
  }
  const float inv = 1.0f / (sqrtf(s) + vs);
  o[0] = x * inv;
  o[1] = y * inv;
  o[2] = z * inv;
}

// FP32 pairs.  Where |v| is below about 2^-50 the squares approach float's normal
// range, so v and vs are scaled by 2^64 first (exact; N is unchanged); a sum of
// squares below 2^-126 after that counts as 0 (|v| + vs = vs).
__device__ __forceinline__ void unit(Pr x, Pr y, Pr z, Pr vs, Pr* o) {
  using namespace df;
  D X = x.v, Y = y.v, Z = z.v, V = vs.v;
  D s = add(add(sqr(X), sqr(Y)), sqr(Z));
  if (s.h < 0x1p-100f) {
    const float c = 0x1p64f;
    X = scale(X, c);
    Y = scale(Y, c);
    Z = scale(Z, c);
    V = scale(V, c);
    s = add(add(sqr(X), sqr(Y)), sqr(Z));
  }
  const float big = fmul(V.h, 1.0e12f);
  D inv;
  if (s.h > fmul(big, big))
    inv = rsqrt(s);
  else if (fexp(s.h) == 0)
    inv = div(D{1.0f, 0.0f}, V);
  else
    inv = div(D{1.0f, 0.0f}, add(mul(s, rsqrt(s)), V));
  o[0] = mul(X, inv);
  o[1] = mul(Y, inv);
  o[2] = mul(Z, inv);
}

// vertex gradient at (i+1/2, j+1/2, k+1/2), straight from phi in global memory
__device__ void grad_plane(const Grid& g, const CsfP<double>& p, const double* __restrict__ phi, int I0, int J0,
                           int k, double (*G)[GP]) {
  const long X = 1, Y = g.sy, Z = g.sz;
  for (int e = threadIdx.x; e < GP; e += blockDim.x) {
    const int a = e % GX, b = e / GX;
    const int i = I0 - 1 + a, j = J0 - 1 + b;
    const long c = g.at(i, j, k);
    const double q000 = __ldg(phi + c), qp00 = __ldg(phi + c + X), q0p0 = __ldg(phi + c + Y),
                 qpp0 = __ldg(phi + c + X + Y), q00p = __ldg(phi + c + Z), qp0p = __ldg(phi + c + X + Z),
                 q0pp = __ldg(phi + c + Y + Z), qppp = __ldg(phi + c + X + Y + Z);
    // per (i, j) corner the sum and the difference of the two k planes; with
    // ta = s(+,+) - s(0,0) and tb = s(+,0) - s(0,+), the x sum is ta + tb, the y sum ta - tb
    // and the z sum the four differences (18 operations instead of 24)
    const double s00 = q000 + q00p, sp0 = qp00 + qp0p, s0p = q0p0 + q0pp, spp = qpp0 + qppp;
    const double d00 = q00p - q000, dp0 = qp0p - qp00, d0p = q0pp - q0p0, dpp = qppp - qpp0;
    const double ta = spp - s00, tb = sp0 - s0p;
    G[0][e] = (ta + tb) * p.gx;
    G[1][e] = (ta - tb) * p.gy;
    G[2][e] = ((d00 + dp0) + (d0p + dpp)) * p.gz;
  }
}
// the same from two staged planes (Qa = plane k, Qb = plane k+1)
template <class R>
__device__ void grad_staged(const CsfP<R>& p, const R* Qa, const R* Qb, R (*G)[GP]) {
  for (int e = threadIdx.x; e < GP; e += blockDim.x) {
    const int a = e % GX, b = e / GX;
    const int c = b * QX + a;
    const R q000 = Qa[c], qp00 = Qa[c + 1], q0p0 = Qa[c + QX], qpp0 = Qa[c + QX + 1];
    const R q00p = Qb[c], qp0p = Qb[c + 1], q0pp = Qb[c + QX], qppp = Qb[c + QX + 1];
    if constexpr (std::is_same<R, Pr>::value) {
      // the FP64 path's sums and differences of the two planes (15 pair additions)
      const R s00 = q000 + q00p, sp0 = qp00 + qp0p, s0p = q0p0 + q0pp, spp = qpp0 + qppp;
      const R d00 = q00p - q000, dp0 = qp0p - qp00, d0p = q0pp - q0p0, dpp = qppp - qpp0;
      const R ta = spp - s00, tb = sp0 - s0p;
      G[0][e] = (ta + tb) * p.gx;
      G[1][e] = (ta - tb) * p.gy;
      G[2][e] = ((d00 + dp0) + (d0p + dpp)) * p.gz;
    } else {
      G[0][e] = (-q000 + qp00 - q0p0 + qpp0 - q00p + qp0p - q0pp + qppp) * p.gx;
      G[1][e] = (-q000 - qp00 + q0p0 + qpp0 - q00p - qp0p + q0pp + qppp) * p.gy;
      G[2][e] = (-q000 - qp00 - q0p0 - qpp0 + q00p + qp0p + q0pp + qppp) * p.gz;
    }
  }
}
// phi plane k (i in [I0-1, I0+TX+1], j in [J0-1, J0+TY+1]) into Q, converted to R
template <class R>
__device__ void stage_plane(const Grid& g, const double* __restrict__ phi, int I0, int J0, int k, R* Q) {
  for (int e = threadIdx.x; e < QP; e += blockDim.x) {
    const int a = e % QX, b = e / QX;
    Q[e] = (R)__ldg(phi + g.at(I0 - 1 + a, J0 - 1 + b, k));
  }
}
// n13 and n23 of plane k from G(k) (slot gk) into ring slot s
template <class R>
__device__ void side_normals(const CsfP<R>& p, Smem<R>& S, int gk, int s) {
  for (int e = threadIdx.x; e < NP; e += blockDim.x) {
    const int a = e % NX, b = e / NX;  // normal point (I0-1+a, J0-1+b)
    const int ga = a, gb = b;          // same point in the G region (offset -1,-1)
    const int c0 = gb * GX + ga;
    R o[3];
    // n13(i,j): mean of G(i, j-1) and G(i, j) (the sum, with 2 vs)
    const int cm = (gb - 1) * GX + ga;
    if (gb >= 1) {
      unit(S.G[gk][0][cm] + S.G[gk][0][c0], S.G[gk][1][cm] + S.G[gk][1][c0], S.G[gk][2][cm] + S.G[gk][2][c0], p.vs2,
           o);
      S.a13[s][0][e] = o[0];
      S.a13[s][1][e] = o[2];
    }
    // n23(i,j): mean of G(i-1, j) and G(i, j)
    if (ga >= 1) {
      const int cw = gb * GX + ga - 1;
      unit(S.G[gk][0][cw] + S.G[gk][0][c0], S.G[gk][1][cw] + S.G[gk][1][c0], S.G[gk][2][cw] + S.G[gk][2][c0], p.vs2,
           o);
      S.a23[s][0][e] = o[1];
      S.a23[s][1][e] = o[2];
    }
  }
}
// H = G(gk) + G(gk1); then npp (slot s) and n12 (slot s) of the plane of G(gk1)
template <class R>
__device__ void centre_normals(const CsfP<R>& p, Smem<R>& S, int gk, int gk1, int s) {
  for (int e = threadIdx.x; e < GP; e += blockDim.x)
    for (int q = 0; q < 3; ++q) S.H[q][e] = S.G[gk][q][e] + S.G[gk1][q][e];
  __syncthreads();
  for (int e = threadIdx.x; e < NP; e += blockDim.x) {
    const int a = e % NX, b = e / NX;
    R o[3];
    // npp at (I0+a, J0+b): H over (i-1..i, j-1..j) = G region (a..a+1, b..b+1), the
    // sum of the 8 vertex gradients with 8 vs
    const int h00 = b * GX + a, h10 = h00 + 1, h01 = h00 + GX, h11 = h01 + 1;
    unit(S.H[0][h00] + S.H[0][h10] + S.H[0][h01] + S.H[0][h11], S.H[1][h00] + S.H[1][h10] + S.H[1][h01] + S.H[1][h11],
         S.H[2][h00] + S.H[2][h10] + S.H[2][h01] + S.H[2][h11], p.vs8, o);
    S.pp[s][0][e] = o[0];
    S.pp[s][1][e] = o[1];
    S.pp[s][2][e] = o[2];
    // n12 at (I0-1+a, J0-1+b): H at the same point
    unit(S.H[0][h00], S.H[1][h00], S.H[2][h00], p.vs2, o);
    S.a12[s][0][e] = o[0];
    S.a12[s][1][e] = o[1];
  }
}

template <class R>
__global__ void __launch_bounds__(256) k_csf(Grid g, CsfP<R> p, int kchunk, const double* __restrict__ phi,
                                             double* __restrict__ fu, double* __restrict__ fv,
                                             double* __restrict__ fw, double* __restrict__ kap,
                                             const int* __restrict__ skip) {
  if (skip && *skip) return;  // the whole block leaves before any barrier
  extern __shared__ double smraw[];
  Smem<R>& S = *reinterpret_cast<Smem<R>*>(smraw);
  const int I0 = 1 + blockIdx.x * TX, J0 = 1 + blockIdx.y * TY;
  const int kb = 1 + blockIdx.z * kchunk, ke = min(g.nk, kb + kchunk - 1);
  int gA = 0, gB = 1;  // G slots: gA holds plane k, gB the next
  int sp = 0;          // pp/n12 slot of plane k
  int sm = 0;          // n13/n23 slot of plane k-1
  // warm-up: G(kb-1) -> gB, G(kb) -> gA; n13/n23(kb-1) from gB; npp/n12(kb) from both
  if constexpr (kStaged<R>) {
    for (int q = kb - 1; q <= kb + 1; ++q) stage_plane(g, phi, I0, J0, q, S.Q[q % 3]);
    __syncthreads();
    grad_staged(p, S.Q[(kb - 1) % 3], S.Q[kb % 3], S.G[gB]);
    grad_staged(p, S.Q[kb % 3], S.Q[(kb + 1) % 3], S.G[gA]);
  } else {
    grad_plane(g, p, phi, I0, J0, kb - 1, S.G[gB]);
    grad_plane(g, p, phi, I0, J0, kb, S.G[gA]);
  }
  __syncthreads();
  side_normals(p, S, gB, sm);
  centre_normals(p, S, gB, gA, sp);
  __syncthreads();
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int i = I0 + tx, j = J0 + ty;
  for (int k = kb; k <= ke; ++k) {
    // G(k+1) -> gB; n13/n23(k) from gA; npp/n12(k+1)
    if constexpr (kStaged<R>) {
      stage_plane(g, phi, I0, J0, k + 2, S.Q[(k + 2) % 3]);  // the slot of plane k-1, unused from here on
      __syncthreads();
      grad_staged(p, S.Q[(k + 1) % 3], S.Q[(k + 2) % 3], S.G[gB]);
    } else {
      grad_plane(g, p, phi, I0, J0, k + 1, S.G[gB]);
    }
    __syncthreads();
    side_normals(p, S, gA, sm ^ 1);
    centre_normals(p, S, gA, gB, sp ^ 1);
    __syncthreads();
    if (i <= g.ni && j <= g.nj) {
      const long c = g.at(i, j, k);
      const int e = ty * NX + tx;            // npp point (i, j)
      const int f = (ty + 1) * NX + tx + 1;  // n12/n13/n23 point (i, j)
      const R ku = (S.pp[sp][0][e + 1] - S.pp[sp][0][e]) * p.dxi + (S.a12[sp][1][f] - S.a12[sp][1][f - NX]) * p.dyi +
                   (S.a13[sm ^ 1][1][f] - S.a13[sm][1][f]) * p.dzi;
      const R kv = (S.a12[sp][0][f] - S.a12[sp][0][f - 1]) * p.dxi + (S.pp[sp][1][e + NX] - S.pp[sp][1][e]) * p.dyi +
                   (S.a23[sm ^ 1][1][f] - S.a23[sm][1][f]) * p.dzi;
      const R kw = (S.a13[sm ^ 1][0][f] - S.a13[sm ^ 1][0][f - 1]) * p.dxi +
                   (S.a23[sm ^ 1][0][f] - S.a23[sm ^ 1][0][f - NX]) * p.dyi + (S.pp[sp ^ 1][2][e] - S.pp[sp][2][e]) * p.dzi;
      R ph, px, py, pz;
      if constexpr (kStaged<R>) {
        const int cq = (ty + 1) * QX + tx + 1;
        const R* Qk = S.Q[k % 3];
        ph = Qk[cq];
        px = Qk[cq + 1];
        py = Qk[cq + QX];
        pz = S.Q[(k + 1) % 3][cq];
      } else {
        ph = __ldg(phi + c);
        px = __ldg(phi + c + 1);
        py = __ldg(phi + c + g.sy);
        pz = __ldg(phi + c + g.sz);
      }
      fu[c] = (double)(ku * (px - ph) * p.fx);
      fv[c] = (double)(kv * (py - ph) * p.fy);
      fw[c] = (double)(kw * (pz - ph) * p.fz);
      if (kap) {  // the curvatures at the u, v, w points, kept for the adjoint
        kap[c] = (double)ku;
        kap[c + g.n] = (double)kv;
        kap[c + 2 * g.n] = (double)kw;
      }
    }
    __syncthreads();
    gA ^= 1;
    gB ^= 1;
    sp ^= 1;
    sm ^= 1;
  }
}

// k planes per block.  A block of c planes costs about c + 1 plane passes (the
// first plane's gradients and side normals are formed twice), and blocks run in
// waves of (SMs x resident blocks per SM); the chunk minimises waves x (c + 1)
// over 4 <= c <= nk (nk itself on small grids), so the last wave is not left
// mostly empty.  Occupancy and SM count are queried once per kernel and device.
int csf_chunk(const Grid& g, const void* fn, size_t smem) {
  static thread_local const void* cached_fn = nullptr;
  static thread_local int cached_dev = -1, cached_cap = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (fn != cached_fn || dev != cached_dev) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem);
    cached_fn = fn;
    cached_dev = dev;
    cached_cap = std::max(1, sms * per_sm);
  }
  if (g.nk < 16) return g.nk;
  const long tiles = (long)(g.ni / TX) * (g.nj / TY);
  int best = 16;
  long best_cost = -1;
  for (int c = 4; c <= g.nk; ++c) {
    const long blocks = tiles * ((g.nk + c - 1) / c);
    const long cost = ((blocks + cached_cap - 1) / cached_cap) * (c + 1);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = c;
    }
  }
  return best;
}

template <class R>
void launch_csf(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double rhol, double rhog,
                double sigma, const double* phi, double* fu, double* fv, double* fw, double* kap, const int* skip) {
  CsfP<R> p;
  p.dxi = (R)dxinv;
  p.dyi = (R)dyinv;
  p.dzi = (R)dzinv;
  p.gx = (R)(0.25 * dxinv);
  p.gy = (R)(0.25 * dyinv);
  p.gz = (R)(0.25 * dzinv);
  const double vs = std::sqrt(dxinv * dxinv + dyinv * dyinv + dzinv * dzinv) * 1.0e-30;
  p.vs2 = (R)(2.0 * vs);
  p.vs8 = (R)(8.0 * vs);
  const double st = 2.0 * sigma / (rhol + rhog);
  p.fx = (R)(-st * dxinv);
  p.fy = (R)(-st * dyinv);
  p.fz = (R)(-st * dzinv);
  const size_t smem = sizeof(Smem<R>);
  cudaFuncSetAttribute(k_csf<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int kchunk = csf_chunk(g, (const void*)k_csf<R>, smem);
  dim3 gr((unsigned)(g.ni / TX), (unsigned)(g.nj / TY), (unsigned)((g.nk + kchunk - 1) / kchunk));
  k_csf<R><<<gr, 256, smem, s>>>(g, p, kchunk, phi, fu, fv, fw, kap, skip);
  count_launch();
}
}  // namespace

bool csf_supported(const Grid& g) { return g.ni % TX == 0 && g.nj % TY == 0; }

void csf_force(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double rhol, double rhog,
               double sigma, const double* phi, double* fu, double* fv, double* fw, int prec, double* kap,
               const int* skip) {
  if (prec == 1)
    launch_csf<float>(s, g, dxinv, dyinv, dzinv, rhol, rhog, sigma, phi, fu, fv, fw, kap, skip);
  else if (prec == 2)
    launch_csf<Pr>(s, g, dxinv, dyinv, dzinv, rhol, rhog, sigma, phi, fu, fv, fw, kap, skip);
  else
    launch_csf<double>(s, g, dxinv, dyinv, dzinv, rhol, rhog, sigma, phi, fu, fv, fw, kap, skip);
}

}  // namespace fused
}  // namespace fmf
