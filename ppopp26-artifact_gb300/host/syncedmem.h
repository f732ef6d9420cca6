// syncedmem.h -- SyncedMemory-compatible buffer handle for the Fr operators.
//
// Mirrors the reference's buffer type (caffe/interface.hpp:7-29,
// caffe/syncedmem.hpp:47-86): a shared handle (copies alias the same storage)
// to a byte buffer that lives in pinned host memory, device memory or both,
// synchronised lazily by a head state.  size() is in bytes (Fr count =
// size() / 32).  Uninitialised storage reads as zeros on either side, as in
// the reference (syncedmem.cpp:37-117).
//
// Differences, by design:
//  * CUDA failures throw pp::Error (status + message) instead of printing and
//    calling exit(1) (caffe/common.hpp:23-30); uncaught, it still ends the
//    program.
//  * Accessors on a null handle throw instead of returning garbage
//    (caffe/interface.cpp:18-64 falls off the end of non-void functions).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>

namespace pp {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &msg) : std::runtime_error(msg), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

// throws pp::Error for a non-zero PP_* status (message from pp_last_error)
void check(int status, const char *what);
void check_cuda(cudaError_t e, const char *what);

class SyncedMemoryKernel {
 public:
  enum Head { UNINITIALIZED, HEAD_AT_CPU, HEAD_AT_GPU, SYNCED };
  explicit SyncedMemoryKernel(size_t size);
  ~SyncedMemoryKernel();
  SyncedMemoryKernel(const SyncedMemoryKernel &) = delete;
  SyncedMemoryKernel &operator=(const SyncedMemoryKernel &) = delete;

  const void *cpu_data();
  const void *gpu_data();
  void *mutable_cpu_data();
  void *mutable_gpu_data();
  void *mutable_cpu_data_async(cudaStream_t s);
  void *mutable_gpu_data_async(cudaStream_t s);
  void set_cpu_data(void *p);
  void set_gpu_data(void *p);
  void async_gpu_push(cudaStream_t s);
  Head head() const { return head_; }
  size_t size() const { return size_; }

 private:
  void to_cpu(cudaStream_t s, bool async);
  void to_gpu(cudaStream_t s, bool async);
  void *cpu_ = nullptr;
  void *gpu_ = nullptr;
  size_t size_ = 0;
  Head head_ = UNINITIALIZED;
  bool own_cpu_ = false;
  bool own_gpu_ = false;
  int device_ = -1;
};

}  // namespace pp

class SyncedMemory {
 public:
  enum SyncedHead { UNINITIALIZED, HEAD_AT_CPU, HEAD_AT_GPU, SYNCED };
  std::shared_ptr<pp::SyncedMemoryKernel> kernel;
  bool type_flag = true;  // true: Fr (the reference's Fq flag is not used on this path)

  SyncedMemory() = default;
  explicit SyncedMemory(size_t size) : kernel(std::make_shared<pp::SyncedMemoryKernel>(size)) {}
  SyncedMemory(size_t size, bool flag)
      : kernel(std::make_shared<pp::SyncedMemoryKernel>(size)), type_flag(flag) {}

  const void *cpu_data() { return k()->cpu_data(); }
  const void *gpu_data() { return k()->gpu_data(); }
  void set_cpu_data(void *p) { k()->set_cpu_data(p); }
  void set_gpu_data(void *p) { k()->set_gpu_data(p); }
  void *mutable_cpu_data() { return k()->mutable_cpu_data(); }
  void *mutable_gpu_data() { return k()->mutable_gpu_data(); }
  void *mutable_cpu_data_async(cudaStream_t s) { return k()->mutable_cpu_data_async(s); }
  void *mutable_gpu_data_async(cudaStream_t s) { return k()->mutable_gpu_data_async(s); }
  void async_gpu_push(const cudaStream_t &s) { k()->async_gpu_push(s); }
  SyncedHead head() const { return kernel ? (SyncedHead)kernel->head() : UNINITIALIZED; }
  size_t size() const { return kernel ? kernel->size() : 0; }

 private:
  pp::SyncedMemoryKernel *k() const {
    if (!kernel) throw pp::Error(1, "SyncedMemory: use of an empty handle");
    return kernel.get();
  }
};
