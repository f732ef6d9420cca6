// function.cpp -- the reference's operator entry points over libppfr.so.
#include "function.h"

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "pp_ops.h"

namespace {

constexpr size_t kFr = 32;

size_t fr_count(SyncedMemory &m, const char *what) {
  if (m.size() % kFr) throw pp::Error(PP_E_INVAL, std::string(what) + ": size is not a multiple of 32 bytes");
  return m.size() / kFr;
}

int lg_of(size_t n, const char *what) {
  int lg = 0;
  while ((size_t{1} << lg) < n) ++lg;
  if ((size_t{1} << lg) != n) throw pp::Error(PP_E_INVAL, std::string(what) + ": length is not a power of two");
  return lg;
}

// device staging buffers of the host-resident drivers, grown on demand
struct Staging {
  std::mutex mu;
  void *in = nullptr, *out = nullptr;
  size_t in_bytes = 0, out_bytes = 0;
  void *get(void **p, size_t *have, size_t want) {
    if (*have < want) {
      if (*p) cudaFree(*p);
      *p = nullptr;
      *have = 0;
      pp::check_cuda(cudaMalloc(p, want), "cudaMalloc (staging)");
      *have = want;
    }
    return *p;
  }
};
Staging g_stage;
SyncedMemory g_last_lde;

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// host buffer -> device -> transform (pp_ntt or pp_lde) -> host buffer
float host_roundtrip(const void *host_in, size_t in_bytes, void *host_out, size_t out_bytes,
                     const char *what, int (*op)(void *, void *, void *), void *ctx) {
  std::lock_guard<std::mutex> lk(g_stage.mu);
  void *din = g_stage.get(&g_stage.in, &g_stage.in_bytes, in_bytes);
  void *dout = g_stage.get(&g_stage.out, &g_stage.out_bytes, out_bytes);
  cudaEvent_t e0, e1;
  pp::check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
  pp::check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
  cudaDeviceSynchronize();
  cudaEventRecord(e0, 0);
  pp::check_cuda(cudaMemcpyAsync(din, host_in, in_bytes, cudaMemcpyHostToDevice, 0), "H2D");
  pp::check(op(din, dout, ctx), what);
  pp::check_cuda(cudaMemcpyAsync(host_out, dout, out_bytes, cudaMemcpyDeviceToHost, 0), "D2H");
  cudaEventRecord(e1, 0);
  pp::check_cuda(cudaEventSynchronize(e1), what);
  const float ms = elapsed(e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

struct NttCtx {
  uint32_t lg;
  int inverse;
};
int ntt_op(void *din, void *dout, void *ctx) {
  const NttCtx *c = static_cast<const NttCtx *>(ctx);
  return pp_ntt(din, dout, c->lg, c->inverse, nullptr);
}
struct LdeCtx {
  uint32_t lg, lambda, mode;
};
int lde_op(void *din, void *dout, void *ctx) {
  const LdeCtx *c = static_cast<const LdeCtx *>(ctx);
  return pp_lde(din, dout, c->lg, c->lambda, c->mode, nullptr);
}
int ntt_host_op(void *hin, void *hout, void *ctx) {
  const NttCtx *c = static_cast<const NttCtx *>(ctx);
  return pp_ntt_host(hin, hout, c->lg, c->inverse, nullptr);
}
int lde_host_op(void *hin, void *hout, void *ctx) {
  const LdeCtx *c = static_cast<const LdeCtx *>(ctx);
  return pp_lde_host(hin, hout, c->lg, c->lambda, c->mode, nullptr);
}

bool page_locked(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost && at.devicePointer != nullptr;
}

// page-locked host buffer in, page-locked host buffer out, no staging copy:
// the transform's first pass reads host memory and its last pass writes it
float host_direct(void *host_in, void *host_out, const char *what, int (*op)(void *, void *, void *),
                  void *ctx) {
  cudaEvent_t e0, e1;
  pp::check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
  pp::check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
  cudaDeviceSynchronize();
  cudaEventRecord(e0, 0);
  pp::check(op(host_in, host_out, ctx), what);
  cudaEventRecord(e1, 0);
  pp::check_cuda(cudaEventSynchronize(e1), what);
  const float ms = elapsed(e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

}  // namespace

// ------------------------------------------------------------- miss_ops ---
SyncedMemory accumulate_mul_poly(SyncedMemory product, cudaStream_t stream) {
  const size_t n = fr_count(product, "accumulate_mul_poly");
  if (n == 0) return product;
  void *d = product.mutable_gpu_data_async(stream);
  pp::check(pp_gp_prefix(d, n, stream), "accumulate_mul_poly");
  return product;
}

void accumulate_mul_poly_(SyncedMemory product, SyncedMemory output, cudaStream_t stream) {
  const size_t n = fr_count(product, "accumulate_mul_poly_");
  if (output.size() < product.size())
    throw pp::Error(PP_E_INVAL, "accumulate_mul_poly_: output smaller than product");
  if (n == 0) return;
  void *d = product.mutable_gpu_data_async(stream);
  void *o = output.mutable_gpu_data_async(stream);
  pp::check(pp_gp_scan(d, d, o, n, stream), "accumulate_mul_poly_");
}

SyncedMemory evaluate(SyncedMemory poly, SyncedMemory x) {
  SyncedMemory y(kFr);
  const size_t n = poly.size() / kFr;
  void *dy = y.mutable_gpu_data();
  if (n == 0) {
    pp::check(pp_eval(nullptr, 0, nullptr, dy, nullptr), "evaluate");
    return y;
  }
  if (x.size() < kFr) throw pp::Error(PP_E_INVAL, "evaluate: point buffer holds no element");
  pp::check(pp_eval(poly.mutable_gpu_data(), n, x.mutable_gpu_data(), dy, nullptr), "evaluate");
  return y;
}

SyncedMemory poly_div_poly(SyncedMemory divid, SyncedMemory c) {
  const size_t n = fr_count(divid, "poly_div_poly");
  if (n == 0) return divid;
  if (c.size() < kFr) throw pp::Error(PP_E_INVAL, "poly_div_poly: constant buffer holds no element");
  pp::check(pp_div_xplusc(divid.mutable_gpu_data(), n, c.mutable_gpu_data(), nullptr), "poly_div_poly");
  return divid;
}

// ------------------------------------------------------------------ NTT ---
Ntt::Ntt(int domain_size, cudaStream_t) : max_lg_(domain_size) {
  if (domain_size < 0 || domain_size > 32) throw pp::Error(PP_E_INVAL, "Ntt: domain size out of range");
}

SyncedMemory Ntt::forward(SyncedMemory input, cudaStream_t stream) {
  SyncedMemory output(input.size());
  forward_(input, output, stream);
  return output;
}

void Ntt::forward_(SyncedMemory input, SyncedMemory output, cudaStream_t stream) {
  const size_t n = fr_count(input, "Ntt::forward");
  const int lg = lg_of(n, "Ntt::forward");
  if (lg > max_lg_) throw pp::Error(PP_E_UNSUPPORTED, "Ntt::forward: larger than the domain of this Ntt");
  if (output.size() < input.size()) throw pp::Error(PP_E_INVAL, "Ntt::forward_: output too small");
  const void *din = input.mutable_gpu_data_async(stream);
  void *dout = output.mutable_gpu_data_async(stream);
  pp::check(pp_ntt(din, dout, (uint32_t)lg, inverse_ ? 1 : 0, stream), "Ntt::forward");
}

Intt::Intt(int domain_size, cudaStream_t stream) : Ntt(domain_size, stream) { inverse_ = true; }

void Intt::_forward_(SyncedMemory input, cudaStream_t stream) { forward_(input, input, stream); }

// ------------------------------------------------- host-resident drivers ---
void our_ntt(SyncedMemory input, int lg_N, int, int, int, int, int, Ntt ntt, const StageIndexMap *) {
  const size_t n = fr_count(input, "our_ntt");
  if (n != (size_t{1} << lg_N)) throw pp::Error(PP_E_INVAL, "our_ntt: buffer length is not 2^lg_N");
  if (lg_N > ntt.max_lg()) throw pp::Error(PP_E_UNSUPPORTED, "our_ntt: larger than the Ntt domain");
  // SyncedMemory's host side is page-locked: transform it where it lies
  void *h = input.mutable_cpu_data();
  NttCtx ctx{(uint32_t)lg_N, 0};
  const float ms = page_locked(h) ? host_direct(h, h, "our_ntt", ntt_host_op, &ctx)
                                  : host_roundtrip(h, n * kFr, h, n * kFr, "our_ntt", ntt_op, &ctx);
  std::printf("our-ntt execution time: %g ms\n", ms);
}

void standard4_ntt(SyncedMemory input, int lg_N, int, int, int, int, Ntt ntt) {
  const size_t n = fr_count(input, "standard4_ntt");
  if (n != (size_t{1} << lg_N)) throw pp::Error(PP_E_INVAL, "standard4_ntt: buffer length is not 2^lg_N");
  if (lg_N > ntt.max_lg()) throw pp::Error(PP_E_UNSUPPORTED, "standard4_ntt: larger than the Ntt domain");
  void *h = input.mutable_cpu_data();
  NttCtx ctx{(uint32_t)lg_N, 0};
  const float ms = host_roundtrip(h, n * kFr, h, n * kFr, "standard4_ntt", ntt_op, &ctx);
  std::printf("standard4-ntt execution time: %g ms\n", ms);
}

static float lde_driver(cpu::BLS12_381_Fr_G1 *input, int lg_N, int lambda, uint32_t mode, Ntt &ntt,
                        const char *what, bool direct_ok) {
  if (lg_N < 0 || lambda < 0 || lg_N + lambda > ntt.max_lg())
    throw pp::Error(PP_E_UNSUPPORTED, std::string(what) + ": 2^(lg_N+lambda) exceeds the Ntt domain");
  const size_t n = size_t{1} << lg_N, m = n << lambda;
  g_last_lde = SyncedMemory(m * kFr);
  void *hout = g_last_lde.mutable_cpu_data();
  LdeCtx ctx{(uint32_t)lg_N, (uint32_t)lambda, mode};
  // a page-locked caller buffer is read in place; a pageable one is staged
  if (direct_ok && page_locked(input)) return host_direct(input, hout, what, lde_host_op, &ctx);
  return host_roundtrip(input, n * kFr, hout, m * kFr, what, lde_op, &ctx);
}

float our_lde(cpu::BLS12_381_Fr_G1 *input, int lg_N, int lambda, int, int, int, Ntt &ntt) {
  const float ms = lde_driver(input, lg_N, lambda, PP_LDE_COEFFS, ntt, "our_lde", true);
  std::printf("our-lde execution time: %g ms\n", ms);
  return ms;
}

float naive_lde(cpu::BLS12_381_Fr_G1 *input, int lg_N, int lambda, int, int, int, Ntt &ntt) {
  const float ms = lde_driver(input, lg_N, lambda, PP_LDE_SPREAD, ntt, "naive_lde", false);
  std::printf("naive-lde execution time: %g ms\n", ms);
  return ms;
}

SyncedMemory last_lde_output() { return g_last_lde; }

// ------------------------------------------------------------------- MSM ---
SyncedMemory multi_scalar_mult(SyncedMemory points, SyncedMemory scalars, cudaStream_t stream) {
  if (points.size() % 96 || scalars.size() % 32)
    throw pp::Error(PP_E_INVAL, "multi_scalar_mult: sizes are not whole points / scalars");
  const uint64_t np = points.size() / 96, ns = scalars.size() / 32;
  const uint64_t n = np < ns ? np : ns;
  SyncedMemory out(3 * 48);
  void *o = out.mutable_gpu_data_async(stream);
  const void *p = n ? points.mutable_gpu_data_async(stream) : nullptr;
  const void *s = n ? scalars.mutable_gpu_data_async(stream) : nullptr;
  pp::check(pp_msm_g1(p, s, n, o, stream), "multi_scalar_mult");
  return out;
}
