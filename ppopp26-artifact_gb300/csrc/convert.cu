// convert.cu -- data-format operators on either side of the path: Montgomery
// encoding and decoding of raw element files, and a canonical-form check.
//
// The reference reads and writes raw files of 32-byte little-endian
// Montgomery elements (miss_ops.cu:8-24 read_file, lde.cu:222-231
// read_file_exact) and converts with to_mont / to_base
// (PLONK/utils/function.cu:5-21 -> mont_arithmetic.cu:57-71, :222-238, :372-411;
// mont_t::to() / from() at mont_t.cuh:473, :503).  Each element costs one
// Montgomery multiply against 64 bytes, about 4 multiply instructions per
// byte: near the machine balance, so these run close to both roofs.
#include "common.cuh"

namespace pp {
namespace {

constexpr int kThreads = 256;

// a -> a * R mod r (to Montgomery form), for any 256-bit input: the multiply
// by R^2 mod r (< r) keeps a * b < r * 2^256, so the result is canonical
__global__ void __launch_bounds__(kThreads) k_to_mont(const fr *in, fr *out, uint64_t n) {
  const fr rr = fr_rr();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    st_fr(out + i, fr_mul(ldcs_fr(in + i), rr));
}

// a -> a * R^-1 mod r (from Montgomery form): a Montgomery multiply by 1
__global__ void __launch_bounds__(kThreads) k_to_base(const fr *in, fr *out, uint64_t n) {
  fr one = fr_zero();
  one.v[0] = 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    st_fr(out + i, fr_mul(ldcs_fr(in + i), one));
}

__device__ __forceinline__ bool geq_r(const fr &a) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
#pragma unroll
  for (int k = 7; k >= 0; --k)
    if (a.v[k] != r[k]) return a.v[k] > r[k];
  return true;
}

// number of elements >= r (not canonical): per-warp counts, one atomic each
__global__ void __launch_bounds__(kThreads) k_count_noncanonical(const fr *in, uint64_t n,
                                                                 unsigned long long *count) {
  unsigned long long c = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    c += geq_r(ldcs_fr(in + i)) ? 1 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

bool aligned16(const void *p) { return p && (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// one thread per element (the loops stride only past 2^31 - 1 blocks), as
// for the element-wise operators, where capping the grid at 8 blocks per SM
// cost 3-6 %
unsigned grid_for(uint64_t n) {
  const uint64_t want = (n + kThreads - 1) / kThreads;
  const uint64_t cap = 0x7fffffffull;
  return (unsigned)(want < cap ? want : cap);
}

template <bool TO_MONT>
int convert(const void *d_in, void *d_out, uint64_t n, void *stream, const char *who) {
  if (n == 0) return PP_OK;
  if (!aligned16(d_in) || !aligned16(d_out)) {
    set_error("%s: buffers must be 16-byte aligned device pointers", who);
    return PP_E_INVAL;
  }
  const fr *in = static_cast<const fr *>(d_in);
  fr *out = static_cast<fr *>(d_out);
  if (TO_MONT)
    k_to_mont<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(in, out, n);
  else
    k_to_base<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(in, out, n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

}  // namespace
}  // namespace pp

extern "C" int pp_to_mont(const void *d_in, void *d_out, uint64_t n, void *stream) {
  return pp::convert<true>(d_in, d_out, n, stream, "pp_to_mont");
}

extern "C" int pp_to_base(const void *d_in, void *d_out, uint64_t n, void *stream) {
  return pp::convert<false>(d_in, d_out, n, stream, "pp_to_base");
}

extern "C" int pp_count_noncanonical(const void *d_in, uint64_t n, uint64_t *d_count,
                                     void *stream) {
  if (!d_count || (reinterpret_cast<uintptr_t>(d_count) & 7)) {
    pp::set_error("pp_count_noncanonical: d_count must be an 8-byte aligned device pointer");
    return PP_E_INVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PP_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
  if (n == 0) return PP_OK;
  if (!pp::aligned16(d_in)) {
    pp::set_error("pp_count_noncanonical: input must be a 16-byte aligned device pointer");
    return PP_E_INVAL;
  }
  pp::k_count_noncanonical<<<pp::grid_for(n), pp::kThreads, 0, s>>>(
      static_cast<const pp::fr *>(d_in), n, reinterpret_cast<unsigned long long *>(d_count));
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}
