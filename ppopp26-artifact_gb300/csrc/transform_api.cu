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
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t L = lg_n + lambda;
  const fr *in = static_cast<const fr *>(d_in);
  fr *out = static_cast<fr *>(d_out);
  pp::NttInputDesc desc;
  desc.n_valid = 1ull << lg_n;
  int st = PP_OK;
  if (mode == PP_LDE_SPREAD) {
    desc.kind = pp::NTT_IN_SPREAD;
    desc.spread = lambda;
    desc.n_valid = 0;
    return pp::ntt_run(in, out, L, false, desc, s);
  }
  if (mode == PP_LDE_COEFFS) {
    // coefficient i scaled by (7^(2^lambda))^i
    const fr h = pp::host_pow(pp::host_mont_small(7), 1ull << lambda);
    desc.kind = pp::NTT_IN_DIAG;
    desc.diag = pp::pow_table(h, lg_n, &st);
    if (st) return st;
    return pp::ntt_run(in, out, L, false, desc, s);
  }
  // evaluations: INTT into the first 2^lg_n outputs, then coefficient i * 7^i
  st = pp::ntt_run(in, out, lg_n, true, pp::NttInputDesc(), s);
  if (st) return st;
  desc.kind = pp::NTT_IN_DIAG;
  desc.diag = pp::pow_table(pp::host_mont_small(7), lg_n, &st);
  if (st) return st;
  return pp::ntt_run(out, out, L, false, desc, s);
}

extern "C" int pp_ntt_prepare(uint32_t lg_n, int inverse) {
  return pp::ntt_prepare(lg_n, inverse != 0);
}
