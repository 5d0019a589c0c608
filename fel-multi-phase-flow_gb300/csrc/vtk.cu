// vtk.cu -- the reference's field output: the gathers (mk_all.f, mk_slice_j.f,
// mk_slice_k.f), the VTK writers (mkvtk_phi.f, mkvtk_phil.f, mkvtk_p.f,
// mkvtk_q.f), the slice files of mkuwp.h / mkuvp.h and the logs of mk_center.f /
// mk_vel.f.  Ghost fills and the cell-to-vertex averages run on the device; one
// device-to-host copy of the averaged values feeds a host writer that formats
// numbers as Fortran's Ew.d edit descriptor does.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/fmf_capi.h"
#include "ops.cuh"

namespace fmf {
namespace op {

namespace {
// x periodic over j, k in 0..m+1 (the first loop of every mkvtk_*.f)
__global__ void k_vtk_x(Grid g, double* q) {
  const int j = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (j > g.nj + 1 || k > g.nk + 1) return;
  q[g.at(0, j, k)] = q[g.at(g.ni, j, k)];
  q[g.at(g.ni + 1, j, k)] = q[g.at(1, j, k)];
}
// y over i, k in 0..m+1: kind 0 copies the wall rows (phi, p), kind 1 writes 0 (phil)
__global__ void k_vtk_y(Grid g, double* q, int kind) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 1 || k > g.nk + 1) return;
  q[g.at(i, 0, k)] = kind == 1 ? 0.0 : q[g.at(i, 1, k)];
  q[g.at(i, g.nj + 1, k)] = kind == 1 ? 0.0 : q[g.at(i, g.nj, k)];
}
// z over i, j in 0..m+1: periodic (p) or copies of the end planes (phi, phil)
__global__ void k_vtk_z(Grid g, double* q, bool periodic) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (i > g.ni + 1 || j > g.nj + 1) return;
  q[g.at(i, j, 0)] = q[g.at(i, j, periodic ? g.nk : 1)];
  q[g.at(i, j, g.nk + 1)] = q[g.at(i, j, periodic ? 1 : g.nk)];
}
// vertex (i, j, k) in 0..m: the mean of the 8 cells around it, summed in the
// reference's order; out is (mi+1)(mj+1)(mk+1), i fastest
__global__ void k_vtk_vertex(Grid g, const double* __restrict__ q, double* __restrict__ out) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long X = 1, Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  out[((long)k * (g.nj + 1) + j) * (g.ni + 1) + i] =
      (q[c] + q[c + X] + q[c + Y] + q[c + X + Y] + q[c + Z] + q[c + X + Z] + q[c + Y + Z] + q[c + X + Y + Z]) *
      0.125;
}
// mkvtk_q.f: q at cells 1..m where the mean vorticity of the 4 x-edges around the
// cell is > 0 (out1) or < 0 (out2), else 0; out is mi mj mk, i fastest
__global__ void k_vtk_q(Grid g, const double* __restrict__ vorx, const double* __restrict__ q, double* out1,
                        double* out2) {
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = 1 + (int)blockIdx.z;
  if (i > g.ni || j > g.nj) return;
  const long Y = g.sy, Z = g.sz;
  const long c = g.at(i, j, k);
  const double vm = (vorx[c - Y - Z] + vorx[c - Z] + vorx[c - Y] + vorx[c]) * 0.25;
  const long o = ((long)(k - 1) * g.nj + (j - 1)) * g.ni + (i - 1);
  out1[o] = vm <= 0.0 ? 0.0 : q[c];
  out2[o] = vm >= 0.0 ? 0.0 : q[c];
}
// slice of the 8-point means with offsets (ip, jp, kp) at a fixed j (axis 1) or k
// (axis 2); out is (ni+1) x (n+1) with the other index from st..n (rows below st
// are zeroed, as the reference zeroes its work slice first)
__global__ void k_slice(Grid g, const double* __restrict__ q, int axis, int fixed, int ip, int jp, int kp, int st,
                        double* __restrict__ out) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int r = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int nr = axis == 1 ? g.nk : g.nj;
  if (i > g.ni || r > nr) return;
  double v = 0.0;
  if (r >= st) {
    const int j = axis == 1 ? fixed : r, k = axis == 1 ? r : fixed;
    const long X = ip, Y = jp ? g.sy : 0, Z = kp ? g.sz : 0;
    const long c = g.at(i, j, k);
    v = (q[c] + q[c + X] + q[c + Y] + q[c + X + Y] + q[c + Z] + q[c + X + Z] + q[c + Y + Z] + q[c + X + Y + Z]) *
        0.125;
  }
  out[(long)r * (g.ni + 1) + i] = v;
}
dim3 b2() { return dim3(32, 8); }
dim3 g2(int a, int b) { return dim3((unsigned)((a + 31) / 32), (unsigned)((b + 7) / 8)); }
}  // namespace

void vtk_ghosts(cudaStream_t s, const Grid& g, double* q, int kind) {
  k_vtk_x<<<g2(g.nj + 2, g.nk + 2), b2(), 0, s>>>(g, q);
  k_vtk_y<<<g2(g.ni + 2, g.nk + 2), b2(), 0, s>>>(g, q, kind == 1 ? 1 : 0);
  k_vtk_z<<<g2(g.ni + 2, g.nj + 2), b2(), 0, s>>>(g, q, kind == 2);
  count_launch(3);
}
void vtk_vertex(cudaStream_t s, const Grid& g, const double* q, double* out) {
  dim3 gr = g2(g.ni + 1, g.nj + 1);
  gr.z = (unsigned)(g.nk + 1);
  k_vtk_vertex<<<gr, b2(), 0, s>>>(g, q, out);
  count_launch();
}
void vtk_q(cudaStream_t s, const Grid& g, const double* vorx, const double* q, double* out1, double* out2) {
  dim3 gr = g2(g.ni, g.nj);
  gr.z = (unsigned)g.nk;
  k_vtk_q<<<gr, b2(), 0, s>>>(g, vorx, q, out1, out2);
  count_launch();
}
void slice(cudaStream_t s, const Grid& g, const double* q, int axis, int fixed, int ip, int jp, int kp, int st,
           double* out) {
  const int nr = axis == 1 ? g.nk : g.nj;
  k_slice<<<g2(g.ni + 1, nr + 1), b2(), 0, s>>>(g, q, axis, fixed, ip, jp, kp, st, out);
  count_launch();
}

// ---- host writers ---------------------------------------------------------------
// Fortran Ew.d output of x into out (w characters and a terminating NUL): sign,
// "0.", d digits rounded to nearest (the C library's decimal conversion), then
// E+dd for exponents up to 99 or +ddd up to 999; the optional leading 0 is dropped
// when the field is one character short, and a field that still does not fit is w
// asterisks.  NaN and infinities are right-justified words.
void fortran_e(char* out, double x, int w, int d) {
  std::string r;
  if (std::isnan(x)) {
    r = "NaN";
  } else if (std::isinf(x)) {
    r = x < 0 ? (w >= 9 ? "-Infinity" : "-Inf") : (w >= 8 ? "Infinity" : "Inf");
  } else {
    char t[64];
    std::snprintf(t, sizeof(t), "%+.*e", d - 1, x);  // +D.DDDe+XX, d significant digits
    const bool neg = t[0] == '-';
    std::string dig(1, t[1]);
    if (d > 1) dig += std::string(t + 3, t + 3 + (d - 1));
    const char* e = std::strchr(t, 'e');
    int ex = std::atoi(e + 1);
    const bool zero = dig.find_first_not_of('0') == std::string::npos;
    ex = zero ? 0 : ex + 1;
    const int ae = ex < 0 ? -ex : ex;
    char ef[16];
    if (ae <= 99) std::snprintf(ef, sizeof(ef), "E%c%02d", ex < 0 ? '-' : '+', ae);
    else if (ae <= 999) std::snprintf(ef, sizeof(ef), "%c%03d", ex < 0 ? '-' : '+', ae);
    else ef[0] = 0;
    if (!ef[0]) {
      r = std::string((size_t)w, '*');
    } else {
      r = std::string(neg ? "-" : "") + "0." + dig + ef;
      if ((int)r.size() > w) r = std::string(neg ? "-" : "") + "." + dig + ef;
    }
  }
  if ((int)r.size() > w) r = std::string((size_t)w, '*');
  std::snprintf(out, (size_t)w + 1, "%*s", w, r.c_str());
}

int write_vtk(const char* fname, const char* scalar, int nstep, int nx, int ny, int nz, const double* origin,
              const double* spacing, const double* vals) {
  FILE* f = std::fopen(fname, "w");
  if (!f) return FMF_ERR_ARG;
  char a[3][32], b[3][32];
  for (int q = 0; q < 3; ++q) {
    fortran_e(a[q], origin[q], 11, 4);
    fortran_e(b[q], spacing[q], 11, 4);
  }
  std::fprintf(f, "# vtk DataFile Version 2.0\nt=%d\nASCII\nDATASET STRUCTURED_POINTS\n", nstep);
  std::fprintf(f, "DIMENSIONS %d %d %d\n", nx, ny, nz);
  std::fprintf(f, "ORIGIN %s %s %s\nASPECT_RATIO %s %s %s\n\n", a[0], a[1], a[2], b[0], b[1], b[2]);
  const long n = (long)nx * ny * nz;
  std::fprintf(f, "POINT_DATA %ld\nSCALARS %s float\nLOOKUP_TABLE default\n", n, scalar);
  char v[32];
  for (long t = 0; t < n; ++t) {
    fortran_e(v, vals[t], 10, 3);
    std::fputs(v, f);
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  if (ok) std::printf(" output %s\n", fname);
  return ok ? 0 : FMF_ERR_ARG;
}

// one '(20e20.10)' record of n values
void write_e20(FILE* f, const double* v, int n) {
  char b[32];
  for (int t = 0; t < n; ++t) {
    fortran_e(b, v[t], 20, 10);
    std::fputs(b, f);
  }
  std::fputc('\n', f);
}

}  // namespace op
}  // namespace fmf
