// syncedmem.cpp -- lazy host/device synchronisation (state machine of the
// reference's caffe/syncedmem.cpp:37-117, 180-230, re-implemented).
#include "syncedmem.h"

#include <cstring>
#include <string>

#include "pp_ops.h"

namespace pp {

void check(int status, const char *what) {
  if (status != PP_OK)
    throw Error(status, std::string(what) + ": " + pp_status_string(status) + ": " + pp_last_error());
}

void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(PP_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

SyncedMemoryKernel::SyncedMemoryKernel(size_t size) : size_(size) {}

SyncedMemoryKernel::~SyncedMemoryKernel() {
  if (cpu_ && own_cpu_) cudaFreeHost(cpu_);
  if (gpu_ && own_gpu_) {
    int cur = -1;
    cudaGetDevice(&cur);
    if (device_ >= 0 && cur != device_) cudaSetDevice(device_);
    cudaFree(gpu_);
    if (device_ >= 0 && cur != device_) cudaSetDevice(cur);
  }
}

void SyncedMemoryKernel::to_cpu(cudaStream_t s, bool async) {
  switch (head_) {
    case UNINITIALIZED:
      check_cuda(cudaMallocHost(&cpu_, size_ ? size_ : 1), "cudaMallocHost");
      std::memset(cpu_, 0, size_);
      own_cpu_ = true;
      head_ = HEAD_AT_CPU;
      break;
    case HEAD_AT_GPU:
      if (!cpu_) {
        check_cuda(cudaMallocHost(&cpu_, size_ ? size_ : 1), "cudaMallocHost");
        own_cpu_ = true;
      }
      if (async) {
        check_cuda(cudaMemcpyAsync(cpu_, gpu_, size_, cudaMemcpyDeviceToHost, s), "D2H copy");
      } else {
        check_cuda(cudaMemcpy(cpu_, gpu_, size_, cudaMemcpyDeviceToHost), "D2H copy");
      }
      head_ = SYNCED;
      break;
    case HEAD_AT_CPU:
    case SYNCED:
      break;
  }
}

void SyncedMemoryKernel::to_gpu(cudaStream_t s, bool async) {
  switch (head_) {
    case UNINITIALIZED:
      check_cuda(cudaMalloc(&gpu_, size_ ? size_ : 1), "cudaMalloc");
      cudaGetDevice(&device_);
      own_gpu_ = true;
      if (async) {
        check_cuda(cudaMemsetAsync(gpu_, 0, size_, s), "cudaMemsetAsync");
      } else {
        check_cuda(cudaMemset(gpu_, 0, size_), "cudaMemset");
      }
      head_ = HEAD_AT_GPU;
      break;
    case HEAD_AT_CPU:
      if (!gpu_) {
        check_cuda(cudaMalloc(&gpu_, size_ ? size_ : 1), "cudaMalloc");
        cudaGetDevice(&device_);
        own_gpu_ = true;
      }
      if (async) {
        check_cuda(cudaMemcpyAsync(gpu_, cpu_, size_, cudaMemcpyHostToDevice, s), "H2D copy");
      } else {
        check_cuda(cudaMemcpy(gpu_, cpu_, size_, cudaMemcpyHostToDevice), "H2D copy");
      }
      head_ = SYNCED;
      break;
    case HEAD_AT_GPU:
    case SYNCED:
      break;
  }
}

const void *SyncedMemoryKernel::cpu_data() {
  to_cpu(0, false);
  return cpu_;
}
const void *SyncedMemoryKernel::gpu_data() {
  to_gpu(0, false);
  return gpu_;
}
void *SyncedMemoryKernel::mutable_cpu_data() {
  to_cpu(0, false);
  head_ = HEAD_AT_CPU;
  return cpu_;
}
void *SyncedMemoryKernel::mutable_gpu_data() {
  to_gpu(0, false);
  head_ = HEAD_AT_GPU;
  return gpu_;
}
void *SyncedMemoryKernel::mutable_cpu_data_async(cudaStream_t s) {
  to_cpu(s, true);
  head_ = HEAD_AT_CPU;
  return cpu_;
}
void *SyncedMemoryKernel::mutable_gpu_data_async(cudaStream_t s) {
  to_gpu(s, true);
  head_ = HEAD_AT_GPU;
  return gpu_;
}
void SyncedMemoryKernel::set_cpu_data(void *p) {
  if (cpu_ && own_cpu_) cudaFreeHost(cpu_);
  cpu_ = p;
  head_ = HEAD_AT_CPU;
  own_cpu_ = false;
}
void SyncedMemoryKernel::set_gpu_data(void *p) {
  if (gpu_ && own_gpu_) cudaFree(gpu_);
  gpu_ = p;
  head_ = HEAD_AT_GPU;
  own_gpu_ = false;
}
void SyncedMemoryKernel::async_gpu_push(cudaStream_t s) {
  if (head_ != HEAD_AT_CPU) return;
  if (!gpu_) {
    check_cuda(cudaMalloc(&gpu_, size_ ? size_ : 1), "cudaMalloc");
    cudaGetDevice(&device_);
    own_gpu_ = true;
  }
  check_cuda(cudaMemcpyAsync(gpu_, cpu_, size_, cudaMemcpyHostToDevice, s), "H2D copy");
  head_ = SYNCED;
}

}  // namespace pp
