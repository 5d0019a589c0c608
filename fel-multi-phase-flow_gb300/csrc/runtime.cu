// runtime.cu -- library runtime: status, stream, scratch, and the host-array
// registry that mirrors the caller's arrays in HBM.
#include <atomic>
#include <map>
#include <mutex>
#include <vector>

#include "runtime.cuh"

namespace fmf {

// atomic: the adjoint rollout runs a second host thread
static std::atomic<int> g_status{0};
static std::atomic<long long> g_launches{0};
static cudaStream_t g_stream = nullptr;
static bool g_own_stream = false;
static int g_mode = 0;  // FMF_RESIDENT

void set_status(int code) {
  if (code != 0) g_status = code;
}
int get_status() { return g_status; }
int take_status() { return g_status.exchange(0); }
bool cuda_ok(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return true;
  std::fprintf(stderr, "fmf: CUDA error %s (%s) at %s\n", cudaGetErrorName(e), cudaGetErrorString(e), where);
  set_status(1);
  return false;
}
void count_launch(int n) { g_launches += n; }
long long launches() { return g_launches; }

cudaStream_t stream() {
  if (!g_stream) {
    if (FMF_CUDA(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking))) g_own_stream = true;
  }
  return g_stream;
}
void set_stream(cudaStream_t s) {
  if (s) {
    g_stream = s;
    g_own_stream = false;
  } else {
    g_stream = nullptr;
    stream();
  }
}
int mode() { return g_mode; }
void set_mode(int m) { g_mode = m; }

// ---- scratch ----------------------------------------------------------------
struct Slot {
  void* p = nullptr;
  size_t bytes = 0;
};
struct ScratchSet {
  Slot slots[16];
};
static ScratchSet g_global_set;
// A time-step context owns its scratch: graphs captured from it keep pointing at
// buffers that no other caller can grow or free.
static thread_local ScratchSet* g_set = nullptr;
void* scratch_set_create() { return new ScratchSet(); }
void scratch_set_destroy(void* p) {
  ScratchSet* s = (ScratchSet*)p;
  if (!s) return;
  for (Slot& sl : s->slots)
    if (sl.p) cudaFree(sl.p);
  delete s;
}
void* scratch_set_use(void* p) {
  ScratchSet* old = g_set;
  g_set = (ScratchSet*)p;
  return old;
}
void* scratch(size_t bytes, int slot) {
  Slot& s = (g_set ? g_set : &g_global_set)->slots[slot];
  if (s.bytes >= bytes) return s.p;
  if (s.p) {
    FMF_CUDA(cudaStreamSynchronize(stream()));
    FMF_CUDA(cudaFree(s.p));
  }
  s.p = nullptr;
  s.bytes = 0;
  if (!FMF_CUDA(cudaMalloc(&s.p, bytes))) {
    set_status(5);
    return nullptr;
  }
  s.bytes = bytes;
  return s.p;
}

// ---- host-array registry -------------------------------------------------
// Entries are keyed by host start address and never overlap: a request that
// overlaps existing mirrors without being contained in one of them merges them
// into one mirror covering the union (device contents of the old mirrors win
// over host contents; the rest of the union is uploaded from the host).
struct Entry {
  uintptr_t end;
  char* dev;
};
static std::map<uintptr_t, Entry> g_reg;
static std::mutex g_mu;

static char* lookup_locked(uintptr_t a, uintptr_t b, bool* fresh, const std::vector<uintptr_t>* protect) {
  *fresh = false;
  auto it = g_reg.upper_bound(a);
  if (it != g_reg.begin()) {
    auto pv = std::prev(it);
    if (pv->first <= a && pv->second.end >= b) return pv->second.dev + (a - pv->first);
  }
  // collect overlapping entries
  uintptr_t lo = a, hi = b;
  std::vector<std::map<uintptr_t, Entry>::iterator> ov;
  it = g_reg.upper_bound(a);
  if (it != g_reg.begin()) {
    auto pv = std::prev(it);
    if (pv->second.end > a) ov.push_back(pv);
  }
  for (; it != g_reg.end() && it->first < b; ++it) ov.push_back(it);
  for (auto& e : ov) {
    lo = std::min(lo, e->first);
    hi = std::max(hi, e->second.end);
    // a mirror already handed to this call must stay where it is
    if (protect)
      for (uintptr_t key : *protect)
        if (key == e->first) {
          std::fprintf(stderr, "fmf: arguments of one call overlap partially in host memory; register the "
                               "enclosing array first (fmf_sync_to_device)\n");
          set_status(2);
          return nullptr;
        }
  }
  char* dev = nullptr;
  if (!FMF_CUDA(cudaMalloc(&dev, hi - lo))) {
    set_status(5);
    return nullptr;
  }
  cudaStream_t s = stream();
  FMF_CUDA(cudaMemcpyAsync(dev, (const void*)lo, hi - lo, cudaMemcpyHostToDevice, s));
  for (auto& e : ov) {
    FMF_CUDA(cudaMemcpyAsync(dev + (e->first - lo), e->second.dev, e->second.end - e->first,
                             cudaMemcpyDeviceToDevice, s));
  }
  FMF_CUDA(cudaStreamSynchronize(s));
  for (auto& e : ov) {
    FMF_CUDA(cudaFree(e->second.dev));
    g_reg.erase(e);
  }
  g_reg[lo] = Entry{hi, dev};
  *fresh = true;
  return dev + (a - lo);
}

void* mirror(const void* host, size_t bytes, bool* fresh, std::vector<uintptr_t>* protect) {
  std::lock_guard<std::mutex> lk(g_mu);
  const uintptr_t a = (uintptr_t)host;
  char* d = lookup_locked(a, a + bytes, fresh, protect);
  if (d && protect) {
    auto it = std::prev(g_reg.upper_bound(a));
    protect->push_back(it->first);
  }
  return d;
}

int sync_to_host(const void* host, size_t bytes_or_0) {
  std::lock_guard<std::mutex> lk(g_mu);
  const uintptr_t a = (uintptr_t)host;
  auto it = g_reg.upper_bound(a);
  if (it == g_reg.begin()) return 2;
  --it;
  if (a >= it->second.end) return 2;
  const size_t n = bytes_or_0 ? bytes_or_0 : (size_t)(it->second.end - a);
  FMF_CUDA(cudaMemcpyAsync((void*)a, it->second.dev + (a - it->first), n, cudaMemcpyDeviceToHost, stream()));
  FMF_CUDA(cudaStreamSynchronize(stream()));
  return get_status();
}
int sync_to_device(const void* host, size_t bytes_or_0) {
  std::lock_guard<std::mutex> lk(g_mu);
  const uintptr_t a = (uintptr_t)host;
  auto it = g_reg.upper_bound(a);
  if (it == g_reg.begin()) return 2;
  --it;
  if (a >= it->second.end) return 2;
  const size_t n = bytes_or_0 ? bytes_or_0 : (size_t)(it->second.end - a);
  FMF_CUDA(cudaMemcpyAsync(it->second.dev + (a - it->first), (const void*)a, n, cudaMemcpyHostToDevice, stream()));
  FMF_CUDA(cudaStreamSynchronize(stream()));
  return get_status();
}
// Every mirror that overlaps [host, host + bytes), for the overlapping part: an
// array whose pieces were registered separately (3-D slices of a 4-D array passed
// to different calls) is synchronised whole.
static int sync_range(const void* host, size_t bytes, bool to_host) {
  std::lock_guard<std::mutex> lk(g_mu);
  const uintptr_t a = (uintptr_t)host, b = a + bytes;
  auto it = g_reg.upper_bound(a);
  if (it != g_reg.begin() && std::prev(it)->second.end > a) --it;
  for (; it != g_reg.end() && it->first < b; ++it) {
    const uintptr_t lo = std::max(a, it->first), hi = std::min(b, it->second.end);
    if (lo >= hi) continue;
    char* d = it->second.dev + (lo - it->first);
    if (to_host)
      FMF_CUDA(cudaMemcpyAsync((void*)lo, d, hi - lo, cudaMemcpyDeviceToHost, stream()));
    else
      FMF_CUDA(cudaMemcpyAsync(d, (const void*)lo, hi - lo, cudaMemcpyHostToDevice, stream()));
  }
  FMF_CUDA(cudaStreamSynchronize(stream()));
  return get_status();
}
int sync_range_to_host(const void* host, size_t bytes) { return sync_range(host, bytes, true); }
int sync_range_to_device(const void* host, size_t bytes) { return sync_range(host, bytes, false); }
int sync_all_to_host() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& e : g_reg)
    FMF_CUDA(cudaMemcpyAsync((void*)e.first, e.second.dev, e.second.end - e.first, cudaMemcpyDeviceToHost, stream()));
  FMF_CUDA(cudaStreamSynchronize(stream()));
  return get_status();
}
int forget(const void* host) {
  std::lock_guard<std::mutex> lk(g_mu);
  const uintptr_t a = (uintptr_t)host;
  auto it = g_reg.upper_bound(a);
  if (it == g_reg.begin()) return 0;
  --it;
  if (a >= it->second.end) return 0;
  FMF_CUDA(cudaStreamSynchronize(stream()));
  FMF_CUDA(cudaFree(it->second.dev));
  g_reg.erase(it);
  return 0;
}
int reset_registry() {
  std::lock_guard<std::mutex> lk(g_mu);
  FMF_CUDA(cudaStreamSynchronize(stream()));
  for (auto& e : g_reg) FMF_CUDA(cudaFree(e.second.dev));
  g_reg.clear();
  return 0;
}

// ---- one call's argument set -----------------------------------------------
// Resident mode: registry mirrors; a mirror handed out earlier in this call is
// protected from merges.  Coherent mode: a temporary device buffer per argument,
// uploaded now and (if written) downloaded and freed in finish(); nothing persists.
double* Call::arr(void* host, size_t ndouble, bool written) {
  if (!host || !ok) {
    if (!host) set_status(2);
    ok = false;
    return nullptr;
  }
  const size_t bytes = ndouble * sizeof(double);
  double* d = nullptr;
  if (mode() == 1) {
    if (!FMF_CUDA(cudaMalloc((void**)&d, bytes))) {
      set_status(5);
      ok = false;
      return nullptr;
    }
    temps.push_back(d);
    FMF_CUDA(cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, stream()));
  } else {
    bool fresh = false;
    d = (double*)mirror(host, bytes, &fresh, &protect);
    if (!d) {
      ok = false;
      return nullptr;
    }
  }
  if (written) outs.push_back(Out{host, d, bytes});
  return d;
}
void Call::finish() {
  cudaStream_t s = stream();
  FMF_CUDA(cudaGetLastError());
  if (mode() == 1) {
    if (ok)
      for (auto& o : outs) FMF_CUDA(cudaMemcpyAsync(o.host, o.dev, o.bytes, cudaMemcpyDeviceToHost, s));
    FMF_CUDA(cudaStreamSynchronize(s));
  }
  release();
}
void Call::release() {
  if (temps.empty()) return;
  FMF_CUDA(cudaStreamSynchronize(stream()));
  for (double* t : temps) FMF_CUDA(cudaFree(t));
  temps.clear();
}

}  // namespace fmf
