// runtime.cu -- error reporting, launch accounting and per-stream workspace.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "ntt.cuh"

namespace pp {

namespace {
thread_local char t_err[512] = "";
std::atomic<uint64_t> g_launches{0};
std::atomic<uint64_t> g_allocs{0};
std::atomic<uint64_t> g_alloc_bytes{0};

struct WsKey {
  int dev;
  cudaStream_t stream;
  int slot;
  bool operator<(const WsKey &o) const {
    return std::tie(dev, stream, slot) < std::tie(o.dev, o.stream, o.slot);
  }
};
struct WsBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_ws_mu;
std::map<WsKey, WsBuf> g_ws;
}  // namespace

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
}
const char *last_error() { return t_err; }

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_alloc(size_t bytes) {
  g_allocs.fetch_add(1, std::memory_order_relaxed);
  g_alloc_bytes.fetch_add(bytes, std::memory_order_relaxed);
}

int device_sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return 152;
  if (!cached[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

void *workspace_get(size_t bytes, cudaStream_t stream, int slot, int *status) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *status = PP_E_CUDA;
    set_error("cudaGetDevice failed");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_ws_mu);
  WsBuf &b = g_ws[WsKey{dev, stream, slot}];
  if (b.bytes >= bytes) {
    *status = PP_OK;
    return b.ptr;
  }
  if (b.ptr) {
    // the old buffer may still be in use by queued work on this stream
    cudaStreamSynchronize(stream);
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  PP_COUNT_ALLOC(bytes);
  cudaError_t e = cudaMalloc(&b.ptr, bytes);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    *status = PP_E_NOMEM;
    set_error("workspace of %zu bytes: %s", bytes, cudaGetErrorString(e));
    cudaGetLastError();
    return nullptr;
  }
  b.bytes = bytes;
  *status = PP_OK;
  return b.ptr;
}

// frees the workspaces of one stream (before the stream is destroyed); a
// later stream may reuse the handle value, so stale entries must not stay
void workspace_release_stream(cudaStream_t stream) {
  std::lock_guard<std::mutex> lk(g_ws_mu);
  for (auto it = g_ws.begin(); it != g_ws.end();) {
    if (it->first.stream == stream) {
      cudaStreamSynchronize(stream);
      cudaFree(it->second.ptr);
      it = g_ws.erase(it);
    } else {
      ++it;
    }
  }
}

int release_all() {
  cudaDeviceSynchronize();
  {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    for (auto &kv : g_ws) cudaFree(kv.second.ptr);
    g_ws.clear();
  }
  ntt_release_tables();
  host_many_release();
  return PP_OK;
}

}  // namespace pp

extern "C" {

const char *pp_status_string(int s) {
  switch (s) {
    case PP_OK: return "ok";
    case PP_E_INVAL: return "invalid argument";
    case PP_E_NOMEM: return "out of device memory";
    case PP_E_CUDA: return "CUDA error";
    case PP_E_TIMEOUT: return "bounded wait timed out";
    case PP_E_UNSUPPORTED: return "unsupported size";
    case PP_E_CANCELLED: return "cancelled";
    case PP_E_BUSY: return "busy";
    default: return "unknown status";
  }
}

const char *pp_last_error(void) { return pp::last_error(); }

const char *pp_version(void) { return "ppfr 0.1 (sm_103a)"; }

uint64_t pp_launch_count(void) { return pp::g_launches.load(); }

uint64_t pp_device_alloc_count(void) { return pp::g_allocs.load(); }

uint64_t pp_device_alloc_bytes(void) { return pp::g_alloc_bytes.load(); }

int pp_release(void) { return pp::release_all(); }

}  // extern "C"

// Synchronous device -> host copy for callers without their own CUDA binding
// (e.g. reading serving results from Python).
extern "C" int pp_copy_to_host(void *h_dst, const void *d_src, uint64_t bytes) {
  if (!bytes) return PP_OK;
  if (!h_dst || !d_src) {
    pp::set_error("pp_copy_to_host: null pointer");
    return PP_E_INVAL;
  }
  PP_CUDA_TRY(cudaMemcpy(h_dst, d_src, bytes, cudaMemcpyDeviceToHost));
  return PP_OK;
}
