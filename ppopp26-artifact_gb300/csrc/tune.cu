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
  PP_COUNT_ALLOC();
  PP_CUDA_TRY(cudaMalloc(&x, n * sizeof(pp::fr)));
  PP_COUNT_ALLOC();
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
