// runtime.cuh -- library runtime shared by the C-ABI translation units.
#pragma once
#include <cstdint>
#include <vector>

#include "fmf_common.cuh"

namespace fmf {

int take_status();
long long launches();
void set_stream(cudaStream_t s);
int mode();
void set_mode(int m);
void* mirror(const void* host, size_t bytes, bool* fresh, std::vector<uintptr_t>* protect);
int sync_to_host(const void* host, size_t bytes_or_0);
int sync_to_device(const void* host, size_t bytes_or_0);
// every mirror overlapping [host, host + bytes), for the overlapping bytes
int sync_range_to_host(const void* host, size_t bytes);
int sync_range_to_device(const void* host, size_t bytes);
int sync_all_to_host();
int forget(const void* host);
int reset_registry();
void* scratch_set_create();
void scratch_set_destroy(void* set);
// Makes `set` this thread's scratch set (nullptr: the library-wide set) and returns
// the one it replaces, so that nested scopes restore their caller's.
void* scratch_set_use(void* set);

// The array arguments of one drop-in call.  arr() returns the device copy of a
// host array: in resident mode the registry mirror (uploaded when first seen),
// in coherent mode a temporary buffer uploaded now.  An entry point resolves all
// of its arrays first and launches only if ok is still true; finish() downloads
// the written arrays in coherent mode and frees the temporaries.
struct Call {
  struct Out {
    void* host;
    void* dev;
    size_t bytes;
  };
  std::vector<Out> outs;
  std::vector<uintptr_t> protect;
  std::vector<double*> temps;
  bool ok = true;
  double* arr(void* host, size_t ndouble, bool written);
  double* in(void* host, size_t ndouble) { return arr(host, ndouble, false); }
  double* out(void* host, size_t ndouble) { return arr(host, ndouble, true); }
  void finish();
  void release();
  ~Call() { release(); }
};

}  // namespace fmf
