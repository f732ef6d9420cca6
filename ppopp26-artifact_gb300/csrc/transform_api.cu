// transform_api.cu -- C ABI of the transforms: NTT/INTT and the coset LDE.
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
