// common.cuh -- shared helpers of the Fr operator library (status codes, checks,
// launch geometry, device-memory workspace).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pp_ops.h"
#include "fr.cuh"

namespace pp {

// number of SMs of the current device (cached per device)
int device_sm_count();

// last error message of the calling thread (set by every failing entry point)
void set_error(const char *fmt, ...);
const char *last_error();

#define PP_CUDA_TRY(call)                                                              \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      ::pp::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                      __LINE__);                                                       \
      return PP_E_CUDA;                                                                \
    }                                                                                  \
  } while (0)

#define PP_LAUNCH_CHECK()                                                                   \
  do {                                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                    \
    if (e_ != cudaSuccess) {                                                                \
      ::pp::set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, \
                      __LINE__);                                                            \
      return PP_E_CUDA;                                                                     \
    }                                                                                       \
  } while (0)

// 16-byte vector loads/stores of a field element (global memory)
__device__ __forceinline__ fr ld_fr(const fr *p) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  uint4 a = q[0], b = q[1];
  return fr{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
}
__device__ __forceinline__ fr ldg_fr(const fr *p) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  uint4 a = __ldg(q), b = __ldg(q + 1);
  return fr{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
}
// streaming load (read once: do not keep in L1)
__device__ __forceinline__ fr ldcs_fr(const fr *p) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  uint4 a = __ldcs(q), b = __ldcs(q + 1);
  return fr{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
}
__device__ __forceinline__ void st_fr(fr *p, const fr &v) {
  uint4 *q = reinterpret_cast<uint4 *>(p);
  q[0] = make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
  q[1] = make_uint4(v.v[4], v.v[5], v.v[6], v.v[7]);
}

// Device-memory workspace that grows on demand and is reused between calls.
// One buffer per (device, stream, slot): work queued on one stream is ordered,
// so calls on that stream may reuse it; different streams never share one.
void *workspace_get(size_t bytes, cudaStream_t stream, int slot, int *status);
// frees every workspace of `stream` (call before destroying the stream)
void workspace_release_stream(cudaStream_t stream);
// destroys pp_ntt_host_many's cached copy streams and events (pp_release)
void host_many_release();

// counts kernel launches issued by this library (pp_launch_count)
void count_launch();
#define PP_COUNT_LAUNCH() ::pp::count_launch()
// every device allocation this library requests (cudaMalloc, cudaMallocAsync,
// cudaMallocFromPoolAsync) is counted with its size; pp_device_alloc_count()
// and pp_device_alloc_bytes() read the totals
void count_alloc(size_t bytes);
#define PP_COUNT_ALLOC(bytes) ::pp::count_alloc(bytes)

}  // namespace pp
