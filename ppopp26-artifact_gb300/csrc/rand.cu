// rand.cu -- seeded canonical random Fr elements on the device.
//
// Element (first + i), limb j, attempt t is the SplitMix64 output (Steele,
// Lea, Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
// at counter ((first + i) << 8 | t << 2 | j) of the stream seeded with
// `seed`; bit 255 is cleared and the attempt is accepted when the value is
// below r (acceptance ~0.9 per attempt).  The accepted value is stored as the
// Montgomery representation, a bijection on [0, r), so the elements are
// uniform.  The benchmark and tests generate their inputs this way.
#include "common.cuh"

namespace pp {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__global__ void k_random_fr(fr *out, uint64_t n, uint64_t seed, uint64_t first) {
  const uint64_t R64[4] = {0xffffffff00000001ULL, 0x53bda402fffe5bfeULL, 0x3339d80809a1d805ULL,
                           0x73eda753299d7d48ULL};
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t idx = first + i;
    uint64_t v[4] = {0, 0, 0, 0};
    bool ok = false;
    for (uint64_t t = 0; t < 64 && !ok; ++t) {
#pragma unroll
      for (uint64_t j = 0; j < 4; ++j) {
        const uint64_t ctr = (idx << 8) | (t << 2) | j;
        v[j] = mix64(seed + (ctr + 1) * 0x9E3779B97F4A7C15ULL);
      }
      v[3] &= 0x7fffffffffffffffULL;
      // v < r ?
      bool lt = false, decided = false;
      for (int k = 3; k >= 0 && !decided; --k) {
        if (v[k] != R64[k]) {
          lt = v[k] < R64[k];
          decided = true;
        }
      }
      ok = decided && lt;
    }
    if (!ok) {  // v < 2^255 < 2r: subtract r once
      uint64_t br = 0;
      for (int k = 0; k < 4; ++k) {
        const uint64_t d = v[k] - R64[k] - br;
        br = (v[k] < R64[k] || (v[k] == R64[k] && br)) ? 1 : 0;
        v[k] = d;
      }
    }
    uint4 *q = reinterpret_cast<uint4 *>(out + i);
    q[0] = make_uint4((uint32_t)v[0], (uint32_t)(v[0] >> 32), (uint32_t)v[1], (uint32_t)(v[1] >> 32));
    q[1] = make_uint4((uint32_t)v[2], (uint32_t)(v[2] >> 32), (uint32_t)v[3], (uint32_t)(v[3] >> 32));
  }
}

}  // namespace pp

extern "C" int pp_random_fr(void *d_out, uint64_t n, uint64_t seed, uint64_t first_index,
                            void *stream) {
  if (n == 0) return PP_OK;
  if (!d_out || (reinterpret_cast<uintptr_t>(d_out) & 15)) {
    pp::set_error("pp_random_fr: output must be a 16-byte aligned device pointer");
    return PP_E_INVAL;
  }
  const int threads = 256;
  const uint64_t want = (n + threads - 1) / threads;
  const uint64_t cap = (uint64_t)pp::device_sm_count() * 16;
  const unsigned blocks = (unsigned)(want < cap ? want : cap);
  pp::k_random_fr<<<blocks, threads, 0, (cudaStream_t)stream>>>(static_cast<pp::fr *>(d_out), n,
                                                                seed, first_index);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}
