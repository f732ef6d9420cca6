// tune.cu -- radix-split autotuner for the NTT and its persisted cache.
//
// A transform of 2^L points can be split into passes of 2^k_1 ... 2^k_P
// points in many ways (3 <= k_p <= 11).  The split trades the number of HBM
// passes and layer-twiddle multiplies (fewer, larger passes) against tile
// width and shared-memory rounds (smaller passes give wider, better-coalesced
// tiles).  The tuner times every balanced ordered split on the current GPU
// with CUDA events and keeps the fastest; results are cached per GPU name in
// a small JSON file:
//   {"gpu": "NVIDIA GB300", "ntt": {"24": [8, 8, 8], "26": [9, 9, 8]}}
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "ntt.cuh"

namespace pp {
namespace {

void enumerate(uint32_t remaining, uint32_t parts_left, std::vector<uint32_t> &cur,
               std::vector<std::vector<uint32_t>> &out) {
  if (parts_left == 0) {
    if (remaining == 0) out.push_back(cur);
    return;
  }
  for (uint32_t k = 3; k <= 11 && k <= remaining; ++k) {
    cur.push_back(k);
    enumerate(remaining - k, parts_left - 1, cur, out);
    cur.pop_back();
  }
}

std::vector<std::vector<uint32_t>> candidates(uint32_t lg) {
  std::vector<std::vector<uint32_t>> all, keep;
  if (lg <= 11) {
    all.push_back({lg});
    return all;
  }
  std::vector<uint32_t> cur;
  const uint32_t pmin = (lg + 10) / 11;
  for (uint32_t P = pmin; P <= 4 && P <= lg / 3; ++P) enumerate(lg, P, cur, all);
  for (auto &c : all) {
    uint32_t mn = 99, mx = 0;
    for (uint32_t k : c) {
      mn = k < mn ? k : mn;
      mx = k > mx ? k : mx;
    }
    if (mx - mn <= 3) keep.push_back(c);
  }
  return keep;
}

}  // namespace
}  // namespace pp

extern "C" int pp_ntt_set_split(uint32_t lg_n, const uint32_t *bits) {
  if (lg_n > PP_MAX_LG_N) return PP_E_UNSUPPORTED;
  const int st = pp::ntt_set_split(lg_n, bits);
  if (st) pp::set_error("pp_ntt_set_split: invalid split for 2^%u (parts must be 3..11 and sum to %u)", lg_n,
                        lg_n);
  return st;
}

extern "C" int pp_ntt_get_split(uint32_t lg_n, uint32_t *bits4) {
  if (!bits4 || lg_n > PP_MAX_LG_N) return PP_E_INVAL;
  uint32_t np = 0, b[4] = {0, 0, 0, 0};
  pp::ntt_get_split(lg_n, b, &np);
  for (int i = 0; i < 4; ++i) bits4[i] = i < (int)np ? b[i] : 0;
  return PP_OK;
}

extern "C" int pp_ntt_autotune(uint32_t lg_n, int reps, uint32_t *best_bits4, float *best_ms) {
  if (lg_n < 12 || lg_n > 28) {
    // single-pass sizes have nothing to tune; very large sizes are left to the caller
    if (best_bits4) pp_ntt_get_split(lg_n, best_bits4);
    if (best_ms) *best_ms = 0.f;
    return lg_n > PP_MAX_LG_N ? PP_E_UNSUPPORTED : PP_OK;
  }
  if (reps < 1) reps = 3;
  const uint64_t n = 1ull << lg_n;
  void *x = nullptr, *y = nullptr;
  PP_COUNT_ALLOC(n * sizeof(pp::fr));
  PP_CUDA_TRY(cudaMalloc(&x, n * sizeof(pp::fr)));
  PP_COUNT_ALLOC(n * sizeof(pp::fr));
  cudaError_t e = cudaMalloc(&y, n * sizeof(pp::fr));
  if (e != cudaSuccess) {
    cudaFree(x);
    pp::set_error("autotune: %s", cudaGetErrorString(e));
    return PP_E_NOMEM;
  }
  int st = pp_random_fr(x, n, 0x7u, 0, nullptr);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  std::vector<uint32_t> best_split;
  for (const auto &c : pp::candidates(lg_n)) {
    if (st) break;
    uint32_t b[5] = {0, 0, 0, 0, 0};
    for (size_t i = 0; i < c.size(); ++i) b[i] = c[i];
    if (pp::ntt_set_split(lg_n, b) != PP_OK) continue;
    if ((st = pp_ntt(x, y, lg_n, 0, nullptr))) break;  // builds the tables
    cudaDeviceSynchronize();
    cudaEventRecord(e0, 0);
    for (int r = 0; r < reps && !st; ++r) st = pp_ntt(x, y, lg_n, 0, nullptr);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= reps;
    if (!st && ms < best) {
      best = ms;
      best_split = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(y);
  if (st) return st;
  uint32_t b[5] = {0, 0, 0, 0, 0};
  for (size_t i = 0; i < best_split.size(); ++i) b[i] = best_split[i];
  st = pp::ntt_set_split(lg_n, best_split.empty() ? nullptr : b);
  if (best_bits4)
    for (int i = 0; i < 4; ++i) best_bits4[i] = b[i];
  if (best_ms) *best_ms = best;
  return st;
}

// JSON cache: {"gpu": "<name>", "ntt": {"<lg>": [k1, k2, ...], ...}}
extern "C" int pp_tune_save(const char *path) {
  if (!path) return PP_E_INVAL;
  cudaDeviceProp prop;
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  PP_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
  FILE *f = std::fopen(path, "w");
  if (!f) {
    pp::set_error("pp_tune_save: cannot write %s", path);
    return PP_E_INVAL;
  }
  std::fprintf(f, "{\"gpu\": \"%s\", \"ntt\": {", prop.name);
  bool first = true;
  for (uint32_t lg = 12; lg <= 28; ++lg) {
    uint32_t b[4];
    pp_ntt_get_split(lg, b);
    std::fprintf(f, "%s\"%u\": [", first ? "" : ", ", lg);
    for (int i = 0; i < 4 && b[i]; ++i) std::fprintf(f, "%s%u", i ? ", " : "", b[i]);
    std::fprintf(f, "]");
    first = false;
  }
  std::fprintf(f, "}}\n");
  std::fclose(f);
  return PP_OK;
}

// applies a cache written by pp_tune_save if it was made on a GPU of the same
// name; returns PP_OK with no change otherwise
extern "C" int pp_tune_load(const char *path) {
  if (!path) return PP_E_INVAL;
  FILE *f = std::fopen(path, "r");
  if (!f) {
    pp::set_error("pp_tune_load: cannot read %s", path);
    return PP_E_INVAL;
  }
  std::string s;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, got);
  std::fclose(f);
  cudaDeviceProp prop;
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  PP_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
  if (s.find(std::string("\"gpu\": \"") + prop.name + "\"") == std::string::npos) return PP_OK;
  const size_t ntt = s.find("\"ntt\"");
  if (ntt == std::string::npos) return PP_E_INVAL;
  size_t pos = ntt + 5;  // past "ntt"
  while (pos < s.size()) {
    const size_t q = s.find('"', pos);
    if (q == std::string::npos) break;
    const size_t q2 = s.find('"', q + 1);
    const size_t lb = s.find('[', q2);
    const size_t rb = s.find(']', lb);
    if (q2 == std::string::npos || lb == std::string::npos || rb == std::string::npos) break;
    const uint32_t lg = (uint32_t)std::strtoul(s.c_str() + q + 1, nullptr, 10);
    uint32_t b[5] = {0, 0, 0, 0, 0};
    int nb = 0;
    const char *p = s.c_str() + lb + 1;
    while (p < s.c_str() + rb && nb < 4) {
      char *end = nullptr;
      const unsigned long v = std::strtoul(p, &end, 10);
      if (end == p) break;
      b[nb++] = (uint32_t)v;
      p = end;
      while (p < s.c_str() + rb && (*p == ',' || *p == ' ')) ++p;
    }
    if (lg >= 12 && lg <= 28 && nb > 0) pp::ntt_set_split(lg, b);
    pos = rb + 1;
  }
  return PP_OK;
}

// ---------------------------------------------------------------------------
// Integer-pipe microbenchmark: the measured denominators of the integer
// roofline.  Every launch fills each SM with 2048 threads; each thread runs
// kIntChains independent dependency chains of one instruction kind, so the
// pipe, not latency, bounds it.  Rates are lane operations per second (one
// warp instruction = 32 lane operations).
// ---------------------------------------------------------------------------
namespace pp {
namespace {

constexpr int kIntChains = 8;
constexpr int kIntIters = 4096;

template <int KIND>
__global__ void __launch_bounds__(256) k_int_rate(uint32_t seed, uint32_t *sink) {
  uint32_t acc[kIntChains];
  uint64_t wide[kIntChains];
  const uint32_t a = seed ^ (threadIdx.x * 0x9e3779b9u), b = seed + blockIdx.x;
#pragma unroll
  for (int k = 0; k < kIntChains; ++k) {
    acc[k] = a + k;
    wide[k] = ((uint64_t)b << 32) ^ k;
  }
#pragma unroll 1
  for (int it = 0; it < kIntIters; ++it) {
#pragma unroll
    for (int k = 0; k < kIntChains; ++k) {
      if (KIND == 0) {
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(acc[k]) : "r"(a), "r"(b));
      } else if (KIND == 1) {
        asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(acc[k]) : "r"(a), "r"(b));
      } else if (KIND == 2) {
        // 32 x 32 -> 64-bit product with a 64-bit addend: the row product of
        // the Montgomery multiply
        // the multiplicand is the accumulator's low word, so the product
        // depends on the chain and cannot be hoisted out of the loop
        asm volatile("{\n\t.reg .u32 l, h;\n\tmov.b64 {l, h}, %0;\n\tmad.wide.u32 %0, l, %1, %0;\n\t}"
                     : "+l"(wide[k]) : "r"(a));
      } else if (KIND == 3) {
        // the same product without the addend
        asm volatile("{\n\t.reg .u32 l, h;\n\tmov.b64 {l, h}, %0;\n\tmul.wide.u32 %0, l, %1;\n\t}"
                     : "+l"(wide[k]) : "r"(a));
      } else {
        // the product without the addend, then the addend as a 64-bit add
        asm volatile("{\n\t.reg .u32 l, h;\n\t.reg .u64 p;\n\tmov.b64 {l, h}, %0;\n\t"
                     "mul.wide.u32 p, l, %1;\n\tadd.u64 %0, %0, p;\n\t}"
                     : "+l"(wide[k]) : "r"(a));
      }
    }
  }
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kIntChains; ++k) s ^= acc[k] ^ (uint32_t)wide[k] ^ (uint32_t)(wide[k] >> 32);
  if (s == 0x12345678u) sink[0] = s;  // keeps the chains live
}

// vals[i] = the Montgomery form of i + 1, i < n
__global__ void k_fill_small(fr *vals, int n) {
  if ((int)threadIdx.x >= n) return;
  fr v = fr_one();
  for (uint32_t k = 0; k < threadIdx.x; ++k) v = fr_add(v, fr_one());
  st_fr(vals + threadIdx.x, v);
}

__global__ void __launch_bounds__(256) k_mm_rate(const fr *in, fr *sink, int iters) {
  fr x = ld_fr(in + (threadIdx.x & 7)), y = ld_fr(in + 8 + (threadIdx.x & 7));
  const fr w = ld_fr(in + 16);
#pragma unroll 1
  for (int it = 0; it < iters; ++it) {
    x = fr_mul(x, w);
    y = fr_mul(y, w);
  }
  if (fr_is_zero(x) && fr_is_zero(y)) st_fr(sink, x);  // keeps the chains live
}

}  // namespace
}  // namespace pp

// out[0]: mad.lo.u32, out[1]: mad.hi.u32, out[2]: mad.wide.u32 lane operations
// per second; out[3]: Montgomery multiplies per second (two independent chains
// per thread, the standalone rate of the field multiply); out[4]: mul.wide.u32
// (no addend) lane operations per second; out[5]: mul.wide.u32 followed by a
// dependent add.u64, per second.  Uses a 1 KiB workspace; about 40 ms of GPU
// time.
extern "C" int pp_measure_int_rates(double out[4]) {
  double all[6];
  const int st = pp_measure_int_rates_ex(all, 6);
  if (st == PP_OK)
    for (int i = 0; i < 4; ++i) out[i] = all[i];
  return st;
}

extern "C" int pp_measure_int_rates_ex(double *out, int n) {
  if (!out || n < 4 || n > 6) return PP_E_INVAL;
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  const int sms = pp::device_sm_count();
  const uint32_t blocks = (uint32_t)sms * 8;
  int st = PP_OK;
  auto *ws = static_cast<uint32_t *>(pp::workspace_get(1024, nullptr, 9, &st));
  if (st) return st;
  cudaEvent_t e0, e1;
  PP_CUDA_TRY(cudaEventCreate(&e0));
  PP_CUDA_TRY(cudaEventCreate(&e1));
  const double lane_ops = (double)blocks * 256 * pp::kIntIters * pp::kIntChains;
  static const int kKindSlot[5] = {0, 1, 2, 4, 5};
  for (int kind = 0; kind < 5 && st == PP_OK; ++kind) {
    const int slot = kKindSlot[kind];
    if (slot >= n) continue;
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
      cudaEventRecord(e0, nullptr);
      if (kind == 0) pp::k_int_rate<0><<<blocks, 256>>>(0x1234u + rep, ws);
      else if (kind == 1) pp::k_int_rate<1><<<blocks, 256>>>(0x1234u + rep, ws);
      else if (kind == 2) pp::k_int_rate<2><<<blocks, 256>>>(0x1234u + rep, ws);
      else if (kind == 3) pp::k_int_rate<3><<<blocks, 256>>>(0x1234u + rep, ws);
      else pp::k_int_rate<4><<<blocks, 256>>>(0x1234u + rep, ws);
      PP_COUNT_LAUNCH();
      cudaEventRecord(e1, nullptr);
      if (cudaEventSynchronize(e1) != cudaSuccess) st = PP_E_CUDA;
      cudaEventElapsedTime(&ms, e0, e1);
    }
    out[slot] = lane_ops / (ms * 1e-3);
  }
  if (st == PP_OK) {
    // field-multiply rate: inputs are 17 small Montgomery values
    auto *vals = reinterpret_cast<pp::fr *>(ws + 64);
    pp::k_fill_small<<<1, 32>>>(vals, 17);
    PP_COUNT_LAUNCH();
    const int iters = 256;
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, nullptr);
      pp::k_mm_rate<<<blocks, 256>>>(vals, vals + 17, iters);
      PP_COUNT_LAUNCH();
      cudaEventRecord(e1, nullptr);
      if (cudaEventSynchronize(e1) != cudaSuccess) st = PP_E_CUDA;
      cudaEventElapsedTime(&ms, e0, e1);
    }
    out[3] = (double)blocks * 256 * 2 * iters / (ms * 1e-3);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != PP_OK) {
    cudaGetLastError();
    pp::set_error("pp_measure_int_rates: a microbenchmark launch failed");
  }
  return st;
}
