// checkpoint.cu -- the reference's restart files (dataou.f:1-46, datain.f:1-46),
// host code only.
//
// One Fortran unformatted sequential record holding u v w p uo vo wo po, phi(0:nbub)
// (each the full halo'd array, i fastest), time (real*8) and nstep (integer*4),
// framed as gfortran frames it (default 4-byte record markers): the record is cut
// into subrecords of at most 2^31-9 bytes, each written as [head][bytes][tail]
// where head = -length if more subrecords follow (else +length) and tail = -length
// if a subrecord precedes it (else +length).  A record under 2 GiB is therefore
// [L][bytes][L].
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/fmf_capi.h"
#include "runtime.cuh"

using namespace fmf;

namespace {
long long max_subrecord() {
  // FMF_RECORD_CHUNK (bytes) overrides the subrecord size; used to exercise the
  // framing of >2 GiB records on small files
  if (const char* e = std::getenv("FMF_RECORD_CHUNK")) {
    const long long v = std::atoll(e);
    if (v > 0 && v <= 2147483639LL) return v;
  }
  return 2147483639LL;
}
struct Seg {
  char* p;
  long long n;
};
// the byte segments of the record in file order
std::vector<Seg> segments(long n, int nbub, double* const* f, double* phi, double* time, int32_t* nstep) {
  std::vector<Seg> s;
  for (int q = 0; q < 8; ++q) s.push_back({(char*)f[q], (long long)sizeof(double) * n});
  s.push_back({(char*)phi, (long long)sizeof(double) * n * (nbub + 1)});
  s.push_back({(char*)time, 8});
  s.push_back({(char*)nstep, 4});
  return s;
}
int write_record(const char* path, const std::vector<Seg>& segs) {
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return FMF_ERR_ARG;
  long long total = 0;
  for (const Seg& s : segs) total += s.n;
  const long long chunk = max_subrecord();
  long long done = 0;
  size_t si = 0;
  long long off = 0;
  bool ok = true, first = true;
  while (ok && (done < total || first)) {
    const long long len = total - done < chunk ? total - done : chunk;
    const bool more = done + len < total;
    const int32_t head = (int32_t)(more ? -len : len), tail = (int32_t)(first ? len : -len);
    ok = ok && std::fwrite(&head, 4, 1, fp) == 1;
    long long left = len;
    while (ok && left > 0) {
      const long long take = segs[si].n - off < left ? segs[si].n - off : left;
      ok = ok && std::fwrite(segs[si].p + off, 1, (size_t)take, fp) == (size_t)take;
      off += take;
      left -= take;
      if (off == segs[si].n) {
        ++si;
        off = 0;
      }
    }
    ok = ok && std::fwrite(&tail, 4, 1, fp) == 1;
    done += len;
    first = false;
  }
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? 0 : FMF_ERR_ARG;
}
int read_record(const char* path, const std::vector<Seg>& segs) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return FMF_ERR_ARG;
  long long total = 0;
  for (const Seg& s : segs) total += s.n;
  long long got = 0;
  size_t si = 0;
  long long off = 0;
  bool ok = true, more = true;
  while (ok && more) {
    int32_t head = 0, tail = 0;
    ok = std::fread(&head, 4, 1, fp) == 1;
    if (!ok) break;
    const long long len = head < 0 ? -(long long)head : (long long)head;
    more = head < 0;
    if (got + len > total) {
      ok = false;
      break;
    }
    long long left = len;
    while (ok && left > 0) {
      const long long take = segs[si].n - off < left ? segs[si].n - off : left;
      ok = std::fread(segs[si].p + off, 1, (size_t)take, fp) == (size_t)take;
      off += take;
      left -= take;
      if (off == segs[si].n) {
        ++si;
        off = 0;
      }
    }
    ok = ok && std::fread(&tail, 4, 1, fp) == 1 && (tail == (int32_t)len || tail == -(int32_t)len);
    got += len;
  }
  std::fclose(fp);
  return (ok && got == total) ? 0 : FMF_ERR_ARG;
}
}  // namespace

extern "C" {

int fmf_write_checkpoint(const char* path, int ni, int nj, int nk, int nbub, int nstep, double time,
                         const double* const* fields, const double* phi) {
  if (!path || !fields || !phi || ni < 1 || nj < 1 || nk < 1 || nbub < 0) return FMF_ERR_ARG;
  for (int q = 0; q < 8; ++q)
    if (!fields[q]) return FMF_ERR_ARG;
  const long n = (long)(ni + 6) * (nj + 6) * (nk + 6);
  double t = time;
  int32_t s = nstep;
  return write_record(path, segments(n, nbub, (double* const*)fields, (double*)phi, &t, &s));
}

int fmf_read_checkpoint(const char* path, int ni, int nj, int nk, int nbub, int* nstep, double* time,
                        double* const* fields, double* phi) {
  if (!path || !fields || !phi || !nstep || !time || ni < 1 || nj < 1 || nk < 1 || nbub < 0) return FMF_ERR_ARG;
  for (int q = 0; q < 8; ++q)
    if (!fields[q]) return FMF_ERR_ARG;
  const long n = (long)(ni + 6) * (nj + 6) * (nk + 6);
  int32_t s = 0;
  const int st = read_record(path, segments(n, nbub, fields, phi, time, &s));
  if (st == 0) *nstep = s;
  return st;
}

// dataou.f:1-46: file x<nstep> (x<nstep>_<ID> when ipara = 1) in the working directory
void dataou_(int* ipara, int* ID, int* ni, int* nj, int* nk, int* nbub, int* nstep, double* time, double* u,
             double* v, double* w, double* p, double* uo, double* vo, double* wo, double* po, double* phi) {
  char fname[64];
  if (*ipara == 1)
    std::snprintf(fname, sizeof(fname), "x%07d_%04d", *nstep, *ID);
  else
    std::snprintf(fname, sizeof(fname), "x%07d", *nstep);
  double* f[8] = {u, v, w, p, uo, vo, wo, po};
  if (mode() == FMF_RESIDENT) {
    // every device mirror inside each array (none for arrays the library never
    // saw; phi's slices may have been registered one by one)
    const size_t b = sizeof(double) * (size_t)(*ni + 6) * (*nj + 6) * (*nk + 6);
    for (double* q : f) sync_range_to_host(q, b);
    sync_range_to_host(phi, b * (size_t)(*nbub + 1));
  }
  const int st = fmf_write_checkpoint(fname, *ni, *nj, *nk, *nbub, *nstep, *time, f, phi);
  if (st) set_status(st);
  else std::printf(" output %s\n", fname);
}

// datain.f:1-46: file x.inp (x.inp_<ID> when ipara = 1)
void datain_(int* ipara, int* ID, int* ni, int* nj, int* nk, int* nbub, int* nstep, double* time, double* u,
             double* v, double* w, double* p, double* uo, double* vo, double* wo, double* po, double* phi) {
  char fname[64];
  if (*ipara == 1)
    std::snprintf(fname, sizeof(fname), "x.inp_%04d", *ID);
  else
    std::snprintf(fname, sizeof(fname), "x.inp");
  double* f[8] = {u, v, w, p, uo, vo, wo, po};
  const int st = fmf_read_checkpoint(fname, *ni, *nj, *nk, *nbub, nstep, time, f, phi);
  if (st) {
    set_status(st);
    return;
  }
  if (mode() == FMF_RESIDENT) {
    const size_t b = sizeof(double) * (size_t)(*ni + 6) * (*nj + 6) * (*nk + 6);
    for (double* q : f) sync_range_to_device(q, b);
    sync_range_to_device(phi, b * (size_t)(*nbub + 1));
  }
  std::printf(" input %s\n", fname);
}

}  // extern "C"
