// transform_api.cu -- C ABI of the transforms: NTT/INTT and the coset LDE.
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "ntt.cuh"

using pp::fr;

namespace {
bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
}  // namespace

extern "C" int pp_ntt(const void *d_in, void *d_out, uint32_t lg_n, int inverse, void *stream) {
  if (!d_in || !d_out || !aligned16(d_in) || !aligned16(d_out)) {
    pp::set_error("pp_ntt: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  if (lg_n > PP_MAX_LG_N) {
    pp::set_error("pp_ntt: lg_n = %u exceeds %d", lg_n, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  pp::NttInputDesc in;
  return pp::ntt_run(static_cast<const fr *>(d_in), static_cast<fr *>(d_out), lg_n, inverse != 0,
                     in, (cudaStream_t)stream);
}

namespace {
// the three LDE forms; in_host / out_host: the input / output is page-locked
// host memory, read by the first pass / written by the last pass directly
int lde_run(const fr *in, fr *out, uint32_t lg_n, uint32_t lambda, uint32_t mode, cudaStream_t s,
            bool in_host, bool out_host) {
  const uint32_t L = lg_n + lambda;
  pp::NttInputDesc desc;
  desc.n_valid = 1ull << lg_n;
  desc.in_host = in_host;
  desc.out_host = out_host;
  int st = PP_OK;
  if (mode == PP_LDE_SPREAD) {
    // inputs at i << lambda, no coset factor: X_k = sum_i a_i w_L^(i 2^lambda k)
    // = NTT_N(a)[k mod N] -- one N-point transform, then 2^lambda - 1 copies
    // of it (the same values as the 2^L-point transform of the spread input)
    const uint64_t n = 1ull << lg_n;
    pp::NttInputDesc plain;
    plain.in_host = in_host;
    fr *first = out;
    if (out_host) {
      first = static_cast<fr *>(pp::workspace_get(sizeof(fr) << lg_n, s, 2, &st));
      if (st) return st;
    }
    st = pp::ntt_run(in, first, lg_n, false, plain, s);
    if (st) return st;
    for (uint64_t r = out_host ? 0 : 1; r < (1ull << lambda); ++r)
      PP_CUDA_TRY(cudaMemcpyAsync(out + r * n, first, sizeof(fr) * n, cudaMemcpyDefault, s));
    return PP_OK;
  }
  if (mode == PP_LDE_COEFFS) {
    // coefficient i scaled by (7^(2^lambda))^i
    const fr h = pp::host_pow(pp::host_mont_small(7), 1ull << lambda);
    desc.kind = pp::NTT_IN_DIAG;
    desc.diag = pp::pow_table(h, lg_n, &st);
    if (st) return st;
    return pp::ntt_run(in, out, L, false, desc, s);
  }
  // evaluations: INTT into coefficients, then coefficient i * 7^i.  With a
  // host output the coefficients go to device scratch (slot 2) instead of the
  // first 2^lg_n outputs.
  fr *coef = out;
  if (out_host) {
    coef = static_cast<fr *>(pp::workspace_get(sizeof(fr) << lg_n, s, 2, &st));
    if (st) return st;
  }
  pp::NttInputDesc inv;
  inv.in_host = in_host;
  st = pp::ntt_run(in, coef, lg_n, true, inv, s);
  if (st) return st;
  desc.kind = pp::NTT_IN_DIAG;
  desc.in_host = false;
  desc.diag = pp::pow_table(pp::host_mont_small(7), lg_n, &st);
  if (st) return st;
  return pp::ntt_run(coef, out, L, false, desc, s);
}
}  // namespace

extern "C" int pp_lde(const void *d_in, void *d_out, uint32_t lg_n, uint32_t lambda, uint32_t mode,
                      void *stream) {
  if (!d_in || !d_out || !aligned16(d_in) || !aligned16(d_out)) {
    pp::set_error("pp_lde: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  if (lambda > 8 || mode > PP_LDE_SPREAD) {
    pp::set_error("pp_lde: lambda %u / mode %u not supported", lambda, mode);
    return PP_E_INVAL;
  }
  if (lg_n + lambda > PP_MAX_LG_N) {
    pp::set_error("pp_lde: 2^(%u+%u) exceeds the supported size", lg_n, lambda);
    return PP_E_UNSUPPORTED;
  }
  return lde_run(static_cast<const fr *>(d_in), static_cast<fr *>(d_out), lg_n, lambda, mode,
                 (cudaStream_t)stream, false, false);
}

extern "C" int pp_ntt_prepare(uint32_t lg_n, int inverse) {
  return pp::ntt_prepare(lg_n, inverse != 0);
}

// ------------------------------------------------- host-resident transforms
// The input and output live in page-locked host memory.  The first pass reads
// the input straight from host memory and the last pass writes the output
// there (over NVLink-C2C on Grace hosts); only the intermediate passes touch
// HBM.  There is no staging copy and no host-side permutation.
namespace {
// Device-visible address of a page-locked host buffer.  Pageable or device
// memory is refused on the host, before any kernel could touch the address.
int host_view(const void *h, const char *who, const char *what, const void **dev) {
  if (!h || !aligned16(h)) {
    pp::set_error("%s: %s must be a 16-byte aligned page-locked host buffer", who, what);
    return PP_E_INVAL;
  }
  cudaPointerAttributes at;
  const cudaError_t e = cudaPointerGetAttributes(&at, h);
  if (e != cudaSuccess) {
    cudaGetLastError();
    pp::set_error("%s: %s: %s", who, what, cudaGetErrorString(e));
    return PP_E_INVAL;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) {
    pp::set_error("%s: %s is not page-locked host memory (cudaHostAlloc / cudaHostRegister)", who,
                  what);
    return PP_E_INVAL;
  }
  *dev = at.devicePointer;
  return PP_OK;
}
}  // namespace

extern "C" int pp_ntt_host(const void *h_in, void *h_out, uint32_t lg_n, int inverse,
                           void *stream) {
  if (lg_n > PP_MAX_LG_N) {
    pp::set_error("pp_ntt_host: lg_n = %u exceeds %d", lg_n, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  const void *din = nullptr, *dout = nullptr;
  int st = host_view(h_in, "pp_ntt_host", "input", &din);
  if (!st) st = host_view(h_out, "pp_ntt_host", "output", &dout);
  if (st) return st;
  pp::NttInputDesc in;
  in.in_host = true;
  in.out_host = true;
  return pp::ntt_run(static_cast<const fr *>(din), static_cast<fr *>(const_cast<void *>(dout)),
                     lg_n, inverse != 0, in, (cudaStream_t)stream);
}

extern "C" int pp_ntt_out_of_core(const void *h_in, void *h_out, void *h_scratch, uint32_t lg_n,
                                  int inverse, void *stream) {
  if (lg_n > PP_MAX_LG_N) {
    pp::set_error("pp_ntt_out_of_core: lg_n = %u exceeds %d", lg_n, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  const void *din = nullptr, *dout = nullptr, *dtmp = nullptr;
  int st = host_view(h_in, "pp_ntt_out_of_core", "input", &din);
  if (!st) st = host_view(h_out, "pp_ntt_out_of_core", "output", &dout);
  if (!st) st = host_view(h_scratch, "pp_ntt_out_of_core", "scratch", &dtmp);
  if (st) return st;
  if (h_in == h_out || h_in == h_scratch || h_out == h_scratch) {
    pp::set_error("pp_ntt_out_of_core: input, output and scratch must be three distinct buffers");
    return PP_E_INVAL;
  }
  return pp::ntt_run_host_passes(static_cast<const fr *>(din), static_cast<fr *>(const_cast<void *>(dout)),
                                 static_cast<fr *>(const_cast<void *>(dtmp)), lg_n, inverse != 0,
                                 (cudaStream_t)stream);
}

namespace {
// dst[i] = src[i], 16-byte words; stream-ordered (a host-to-host
// cudaMemcpyAsync may run on the CPU ahead of the stream's kernels)
__global__ void k_copy16(uint4 *__restrict__ dst, const uint4 *__restrict__ src, uint64_t n16) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16;
       i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// the diagonal h^i, i < 2^lg_n, of an LDE's first pass: one table up to 2^11
// points, else two of about 2^(lg_n / 2) entries (h^j, h^(j 2^k))
int lde_diag(const fr &h, uint32_t lg_n, uint32_t L, pp::NttInputDesc *d) {
  int st = PP_OK;
  d->kind = pp::NTT_IN_DIAG;
  d->n_valid = 1ull << lg_n;
  if (L <= 11) {
    d->diag = pp::pow_table(h, lg_n, &st);
    return st;
  }
  const uint32_t k = (lg_n + 1) / 2;
  d->diag = pp::pow_table(h, k, &st);
  if (st) return st;
  d->diag_hi = pp::pow_table(pp::host_pow(h, 1ull << k), lg_n - k, &st);
  d->diag_lgh = k;
  return st;
}
}  // namespace

extern "C" int pp_lde_out_of_core(const void *h_in, void *h_out, void *h_scratch, uint32_t lg_n,
                                  uint32_t lambda, uint32_t mode, void *stream) {
  if (lambda > 8 || mode > PP_LDE_SPREAD) {
    pp::set_error("pp_lde_out_of_core: lambda %u / mode %u not supported", lambda, mode);
    return PP_E_INVAL;
  }
  const uint32_t L = lg_n + lambda;
  if (L > PP_MAX_LG_N) {
    pp::set_error("pp_lde_out_of_core: 2^(%u+%u) exceeds the supported size", lg_n, lambda);
    return PP_E_UNSUPPORTED;
  }
  const void *din = nullptr, *dout = nullptr, *dtmp = nullptr;
  int st = host_view(h_in, "pp_lde_out_of_core", "input", &din);
  if (!st) st = host_view(h_out, "pp_lde_out_of_core", "output", &dout);
  if (!st) st = host_view(h_scratch, "pp_lde_out_of_core", "scratch", &dtmp);
  if (st) return st;
  if (h_in == h_out || h_in == h_scratch || h_out == h_scratch) {
    pp::set_error("pp_lde_out_of_core: input, output and scratch must be three distinct buffers");
    return PP_E_INVAL;
  }
  const cudaStream_t s = (cudaStream_t)stream;
  const fr *in = static_cast<const fr *>(din);
  fr *out = static_cast<fr *>(const_cast<void *>(dout)), *tmp = static_cast<fr *>(const_cast<void *>(dtmp));
  if (mode == PP_LDE_SPREAD) {
    // the N-point transform into out[0, N), then 2^lambda - 1 copies of it
    st = pp::ntt_run_host_passes(in, out, tmp, lg_n, false, s);
    if (st || lambda == 0) return st;
    const uint64_t n16 = 2ull << lg_n;  // 16-byte words of N elements
    for (uint64_t r = 1; r < (1ull << lambda); ++r) {
      k_copy16<<<pp::device_sm_count() * 4, 256, 0, s>>>(reinterpret_cast<uint4 *>(out) + r * n16,
                                                          reinterpret_cast<const uint4 *>(out), n16);
      PP_COUNT_LAUNCH();
      PP_LAUNCH_CHECK();
    }
    return PP_OK;
  }
  pp::NttInputDesc desc;
  if (mode == PP_LDE_COEFFS) {
    // coefficient i scaled by (7^(2^lambda))^i
    st = lde_diag(pp::host_pow(pp::host_mont_small(7), 1ull << lambda), lg_n, L, &desc);
    if (st) return st;
    return pp::ntt_run_host_passes(in, out, tmp, L, false, desc, s);
  }
  // evaluations: the INTT's coefficients go to the buffer the main
  // transform's first pass does not write (pass j writes out or scratch
  // alternately, ending in out), and the main transform reads them from there
  uint32_t P = 1;
  st = pp::ntt_host_plan_passes(L, &P);
  if (st) return st;
  fr *coef = tmp, *other = out;
  if (P >= 2 && ((P - 2) & 1) == 0) {  // pass 1 writes scratch
    coef = out;
    other = tmp;
  }
  st = pp::ntt_run_host_passes(in, coef, other, lg_n, true, s);
  if (st) return st;
  st = lde_diag(pp::host_mont_small(7), lg_n, L, &desc);
  if (st) return st;
  return pp::ntt_run_host_passes(coef, out, tmp, L, false, desc, s);
}

extern "C" int pp_lde_host(const void *h_in, void *h_out, uint32_t lg_n, uint32_t lambda,
                           uint32_t mode, void *stream) {
  if (lambda > 8 || mode > PP_LDE_SPREAD) {
    pp::set_error("pp_lde_host: lambda %u / mode %u not supported", lambda, mode);
    return PP_E_INVAL;
  }
  if (lg_n + lambda > PP_MAX_LG_N) {
    pp::set_error("pp_lde_host: 2^(%u+%u) exceeds the supported size", lg_n, lambda);
    return PP_E_UNSUPPORTED;
  }
  const void *din = nullptr, *dout = nullptr;
  int st = host_view(h_in, "pp_lde_host", "input", &din);
  if (!st) st = host_view(h_out, "pp_lde_host", "output", &dout);
  if (st) return st;
  return lde_run(static_cast<const fr *>(din), static_cast<fr *>(const_cast<void *>(dout)), lg_n,
                 lambda, mode, (cudaStream_t)stream, true, true);
}

// ------------------------------------------- many host-resident polynomials
// Each polynomial is copied to HBM by a copy engine, transformed there and
// copied back, with the copies of neighbouring polynomials overlapping the
// transforms: host-to-device copies on one internal stream, the transforms
// on the caller's stream, device-to-host copies on another.  Three rotating
// device buffers keep the transform the bound: a buffer is held for one
// polynomial's two copies and its transform (about 9.6 ms at 2^24 over a
// 200 GB/s host link), under three transforms of 4.3 ms.  The buffers are
// workspace slots 5-7 of the caller's stream, and the call ends by making
// the caller's stream wait for the last copy, so later work on that stream
// (and a workspace reallocation, which synchronises it) is ordered after
// every copy.
namespace {
// pp_ntt_host_many's copy streams and events for one (device, caller stream)
struct HostManyCtx {
  std::mutex mu;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev_start = nullptr, ev_done = nullptr;
  cudaEvent_t ev_in[3] = {}, ev_cmp[3] = {}, ev_out[3] = {};
};
std::mutex g_many_mu;
std::map<std::pair<int, cudaStream_t>, HostManyCtx *> g_many;

int host_many_ctx(cudaStream_t s, HostManyCtx **out) {
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_many_mu);
  auto it = g_many.find({dev, s});
  if (it != g_many.end()) {
    *out = it->second;
    return PP_OK;
  }
  auto *c = new HostManyCtx();
  cudaError_t e = cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming);
  for (int b = 0; b < 3 && e == cudaSuccess; ++b) {
    e = cudaEventCreateWithFlags(&c->ev_in[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_cmp[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out[b], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    // a partly built context is kept out of the map and leaks its handles
    cudaGetLastError();
    pp::set_error("pp_ntt_host_many: stream or event creation failed: %s", cudaGetErrorString(e));
    return PP_E_CUDA;
  }
  g_many[{dev, s}] = c;
  *out = c;
  return PP_OK;
}
}  // namespace

namespace pp {
void host_many_release() {
  std::lock_guard<std::mutex> lk(g_many_mu);
  for (auto &kv : g_many) {
    HostManyCtx *c = kv.second;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(kv.first.first);
    cudaStreamSynchronize(c->s_in);
    cudaStreamSynchronize(c->s_out);
    cudaStreamDestroy(c->s_in);
    cudaStreamDestroy(c->s_out);
    cudaEventDestroy(c->ev_start);
    cudaEventDestroy(c->ev_done);
    for (int b = 0; b < 3; ++b) {
      cudaEventDestroy(c->ev_in[b]);
      cudaEventDestroy(c->ev_cmp[b]);
      cudaEventDestroy(c->ev_out[b]);
    }
    cudaSetDevice(cur);
    delete c;
  }
  g_many.clear();
  cudaGetLastError();
}
}  // namespace pp

extern "C" int pp_ntt_host_many(const void *const *h_in, void *const *h_out, uint32_t count,
                                uint32_t lg_n, int inverse, void *stream) {
  if (lg_n > PP_MAX_LG_N) {
    pp::set_error("pp_ntt_host_many: lg_n = %u exceeds %d", lg_n, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  if (count == 0) return PP_OK;
  if (!h_in || !h_out) {
    pp::set_error("pp_ntt_host_many: the input and output pointer arrays are required");
    return PP_E_INVAL;
  }
  const void *dev = nullptr;
  for (uint32_t j = 0; j < count; ++j) {
    int st = host_view(h_in[j], "pp_ntt_host_many", "an input", &dev);
    if (!st) st = host_view(h_out[j], "pp_ntt_host_many", "an output", &dev);
    if (st) return st;
  }
  constexpr int kBufs = 3;
  const cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = sizeof(fr) << lg_n;
  fr *buf[kBufs];
  for (int b = 0; b < kBufs; ++b) {
    int st = PP_OK;
    buf[b] = static_cast<fr *>(pp::workspace_get(bytes, s, 5 + b, &st));
    if (st) return st;
  }
  int st = pp::ntt_prepare(lg_n, inverse != 0);
  if (st) return st;
  // the copy streams and events belong to the (device, caller stream) pair:
  // created on its first call and reused, so a call creates nothing
  HostManyCtx *c = nullptr;
  st = host_many_ctx(s, &c);
  if (st) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  // the copy streams start after the work already queued on the caller's stream
  cudaError_t e = cudaEventRecord(c->ev_start, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->s_in, c->ev_start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->s_out, c->ev_start, 0);
  pp::NttInputDesc desc;
  for (uint32_t j = 0; j < count && e == cudaSuccess && st == PP_OK; ++j) {
    const int b = (int)(j % kBufs);
    if (j >= (uint32_t)kBufs) e = cudaStreamWaitEvent(c->s_in, c->ev_out[b], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf[b], h_in[j], bytes, cudaMemcpyHostToDevice, c->s_in);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_in[b], c->s_in);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_in[b], 0);
    if (e != cudaSuccess) break;
    st = pp::ntt_run(buf[b], buf[b], lg_n, inverse != 0, desc, s);
    if (st) break;
    e = cudaEventRecord(c->ev_cmp[b], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->s_out, c->ev_cmp[b], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_out[j], buf[b], bytes, cudaMemcpyDeviceToHost, c->s_out);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_out[b], c->s_out);
  }
  if (st || e != cudaSuccess) {
    // copies already queued may still read h_in or write h_out: finish them
    // before the caller can free those buffers on seeing the error
    cudaStreamSynchronize(c->s_in);
    cudaStreamSynchronize(c->s_out);
    cudaGetLastError();
    if (st) return st;
    pp::set_error("pp_ntt_host_many: %s", cudaGetErrorString(e));
    return PP_E_CUDA;
  }
  // the caller's stream waits for the last device-to-host copy (the copies
  // run in order on one stream, so that one covers them all)
  e = cudaEventRecord(c->ev_done, c->s_out);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_done, 0);
  if (e != cudaSuccess) {
    pp::set_error("pp_ntt_host_many: %s", cudaGetErrorString(e));
    cudaGetLastError();
    return PP_E_CUDA;
  }
  return PP_OK;
}
