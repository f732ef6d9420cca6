// ref_harness.cpp -- TEST INFRASTRUCTURE: exposes the reference's own CPU code
// for this path through a C ABI so that the oracle can be pinned against it.
//
// It is linked with objects compiled, unmodified, from the reference sources:
//   miss_ops.cu            naive_gp (:34-47), naive_div (:49-87)
//   caffe/*.cpp            SyncedMemory, the buffer type those functions use
//   PLONK/blst/src/assembly.S  the blst field assembly behind
//                          cpu::BLS12_381_Fr_G1 (PLONK/utils/mont/cpu/ff/bls12-381.hpp)
// The machine that builds it has no GPU, so the few CUDA runtime calls the
// reference's CPU path touches are replaced by host fakes below: pinned host
// allocation becomes malloc/free, and every device call reports
// cudaErrorNoDevice.  The reference's GPU operators referenced by its main()
// are never called here and abort if they were.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "caffe/interface.hpp"
#include "PLONK/utils/mont/cpu/ff/bls12-381.hpp"

SyncedMemory naive_gp(int lg_N, SyncedMemory input);
SyncedMemory naive_div(int lg_N, SyncedMemory input, SyncedMemory divisor);

// ---- host fakes of the CUDA runtime entry points the CPU path links -------
extern "C" {
cudaError_t cudaMallocHost(void **ptr, size_t size) {
  *ptr = std::malloc(size ? size : 1);
  return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFreeHost(void *ptr) {
  std::free(ptr);
  return cudaSuccess;
}
cudaError_t cudaMalloc(void **, size_t) { return cudaErrorNoDevice; }
cudaError_t cudaFree(void *) { return cudaErrorNoDevice; }
cudaError_t cudaMemcpy(void *, const void *, size_t, enum cudaMemcpyKind) { return cudaErrorNoDevice; }
cudaError_t cudaMemcpyAsync(void *, const void *, size_t, enum cudaMemcpyKind, cudaStream_t) {
  return cudaErrorNoDevice;
}
cudaError_t cudaMemset(void *, int, size_t) { return cudaErrorNoDevice; }
cudaError_t cudaMemsetAsync(void *, int, size_t, cudaStream_t) { return cudaErrorNoDevice; }
const char *cudaGetErrorString(cudaError_t) { return "CUDA runtime faked by the CPU oracle harness"; }
cudaError_t cudaEventCreate(cudaEvent_t *) { return cudaErrorNoDevice; }
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaErrorNoDevice; }
cudaError_t cudaEventElapsedTime(float *, cudaEvent_t, cudaEvent_t) { return cudaErrorNoDevice; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaErrorNoDevice; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaErrorNoDevice; }
static void *fake_fatbin_handle[4];
void **__cudaRegisterFatBinary(void *) { return fake_fatbin_handle; }
void __cudaRegisterFatBinaryEnd(void **) {}
void __cudaUnregisterFatBinary(void **) {}
void __cudaRegisterVar(void **, char *, char *, const char *, int, size_t, int, int) {}
}

SyncedMemory poly_div_poly(SyncedMemory, SyncedMemory) { std::abort(); }
SyncedMemory accumulate_mul_poly(SyncedMemory, cudaStream_t) { std::abort(); }
SyncedMemory evaluate(SyncedMemory, SyncedMemory) { std::abort(); }

// ---- C ABI used by oracle/oracle.py ---------------------------------------
using Fr = cpu::BLS12_381_Fr_G1;

extern "C" {
void ref_fr_mul(const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    Fr x, y;
    std::memcpy(&x, a + 4 * i, 32);
    std::memcpy(&y, b + 4 * i, 32);
    Fr z = x * y;
    std::memcpy(out + 4 * i, &z, 32);
  }
}
void ref_fr_add(const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    Fr x, y;
    std::memcpy(&x, a + 4 * i, 32);
    std::memcpy(&y, b + 4 * i, 32);
    x += y;
    std::memcpy(out + 4 * i, &x, 32);
  }
}
void ref_fr_sub(const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    Fr x, y;
    std::memcpy(&x, a + 4 * i, 32);
    std::memcpy(&y, b + 4 * i, 32);
    x -= y;
    std::memcpy(out + 4 * i, &x, 32);
  }
}
// 1/x exactly as naive_div computes divisor_leading_inv (miss_ops.cu:67)
void ref_fr_inv(const uint64_t *a, uint64_t *out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    Fr x;
    std::memcpy(&x, a + 4 * i, 32);
    Fr z = 1 / x;
    std::memcpy(out + 4 * i, &z, 32);
  }
}
// the reference's naive_gp on 2^lg_n elements; out receives 2^lg_n elements
void ref_naive_gp(int lg_n, const uint64_t *in, uint64_t *out) {
  const size_t bytes = (size_t{1} << lg_n) * 32;
  SyncedMemory input(bytes);
  std::memcpy(input.mutable_cpu_data(), in, bytes);
  SyncedMemory res = naive_gp(lg_n, input);
  std::memcpy(out, res.mutable_cpu_data(), bytes);
}
// the reference's naive_div by [c, one] = X + c; quotient has 2^lg_n - 1 entries
void ref_naive_div(int lg_n, const uint64_t *in, const uint64_t *c, uint64_t *quotient) {
  const size_t n = size_t{1} << lg_n;
  SyncedMemory input(n * 32);
  std::memcpy(input.mutable_cpu_data(), in, n * 32);
  SyncedMemory divisor(64);
  uint64_t *d = reinterpret_cast<uint64_t *>(divisor.mutable_cpu_data());
  std::memcpy(d, c, 32);
  const uint64_t one[4] = {0x00000001fffffffeULL, 0x5884b7fa00034802ULL, 0x998c4fefecbc4ff5ULL,
                           0x1824b159acc5056fULL};
  std::memcpy(d + 4, one, 32);
  SyncedMemory q = naive_div(lg_n, input, divisor);
  std::memcpy(quotient, q.mutable_cpu_data(), (n - 1) * 32);
}
}
