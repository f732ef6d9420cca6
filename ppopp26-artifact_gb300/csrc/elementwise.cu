// elementwise.cu -- element-wise Fr operators over vectors: the reference's
// add_mod / sub_mod / mul_mod / div_mod with their _scalar and in-place forms,
// neg_mod, inv_mod, exp_mod, gen_sequence and repeat_to_poly
// (PLONK/utils/function.cu:23-170 -> PLONK/utils/mont/cuda/mont_arithmetic.cu:
// 6-52, 414-520 and mont_arithmetic.cuh:17-95).
//
// They move 64-96 bytes per element for at most one Montgomery multiply, so
// HBM bounds them; grid-stride loops of 16-byte accesses.  Division and
// inversion differ: the reference inverts each element (mont_t::reciprocal,
// ff/mont_t.cuh:1117); here runs of kInvRun elements share one inversion
// (Montgomery's simultaneous inversion: 3 multiplies per element).  As in
// the reference, the inverse of 0 is taken as 0.
#include "common.cuh"

namespace pp {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kInvRun = 32;

unsigned grid_for(uint64_t work) {
  const uint64_t want = (work + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)device_sm_count() * 8;
  return (unsigned)(want < cap ? (want ? want : 1) : cap);
}

bool aligned16(const void *p) { return p && (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// c = a op b, or a op b[0] when b_scalar
__global__ void __launch_bounds__(kThreads)
    k_fr_binary(uint32_t op, const fr *a, const fr *b, fr *c, uint64_t n, int b_scalar) {
  const fr s = b_scalar ? ld_fr(b) : fr_zero();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const fr x = ld_fr(a + i), y = b_scalar ? s : ld_fr(b + i);
    fr r;
    if (op == PP_FR_ADD) r = fr_add(x, y);
    else if (op == PP_FR_SUB) r = fr_sub(x, y);
    else r = fr_mul(x, y);
    st_fr(c + i, r);
  }
}

// c_i = a_i / b_i (1 / b_i without a), 0 where b_i = 0.  The forward pass keeps
// the run's running products of the non-zero b in pre[]; the backward pass
// reads each b_i and a_i before it writes c_i, so c may alias a or b.
__global__ void __launch_bounds__(kThreads)
    k_fr_div(const fr *a, const fr *b, fr *c, uint64_t n) {
  const uint64_t runs = (n + kInvRun - 1) / kInvRun;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < runs;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = r * kInvRun, hi = lo + kInvRun < n ? lo + kInvRun : n;
    fr pre[kInvRun];
    fr acc = fr_one();
    for (uint64_t j = lo; j < hi; ++j) {
      const fr v = ld_fr(b + j);
      if (!fr_is_zero(v)) acc = fr_mul(acc, v);
      pre[j - lo] = acc;
    }
    fr inv = fr_inv_binary(acc);  // a product of non-zero values
    for (uint64_t j = hi; j > lo; --j) {
      const fr v = ld_fr(b + j - 1);
      fr q = fr_zero();
      if (!fr_is_zero(v)) {
        q = fr_mul(inv, j - 1 > lo ? pre[j - 2 - lo] : fr_one());  // 1 / b
        inv = fr_mul(inv, v);
        if (a) q = fr_mul(ld_fr(a + j - 1), q);
      }
      st_fr(c + j - 1, q);
    }
  }
}

// out[0] = 1 / x[0] (0 for 0)
__global__ void k_fr_inv1(const fr *x, fr *out) { st_fr(out, fr_inv_binary(ld_fr(x))); }

__global__ void __launch_bounds__(kThreads) k_fr_neg(const fr *a, fr *c, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    st_fr(c + i, fr_sub(fr_zero(), ld_fr(a + i)));
}

__global__ void __launch_bounds__(kThreads) k_fr_pow(const fr *a, fr *c, uint64_t n, uint64_t e) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    st_fr(c + i, fr_pow_u64(ld_fr(a + i), e));
}

// out[i] = x^i: one thread per run of kInvRun, starting from x^lo
__global__ void __launch_bounds__(kThreads) k_fr_powers(const fr *x, fr *out, uint64_t n) {
  const fr b = ld_fr(x);
  const uint64_t runs = (n + kInvRun - 1) / kInvRun;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < runs;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = r * kInvRun, hi = lo + kInvRun < n ? lo + kInvRun : n;
    fr p = fr_pow_u64(b, lo);
    for (uint64_t j = lo; j < hi; ++j) {
      st_fr(out + j, p);
      p = fr_mul(p, b);
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_fr_fill(const fr *x, fr *out, uint64_t n) {
  const fr v = ld_fr(x);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    st_fr(out + i, v);
}

bool overlaps(const void *p, size_t pn, const void *q, size_t qn) {
  const char *a = static_cast<const char *>(p), *b = static_cast<const char *>(q);
  return a < b + qn && b < a + pn;
}

}  // namespace
}  // namespace pp

using pp::fr;

extern "C" int pp_fr_binary(uint32_t op, const void *d_a, const void *d_b, void *d_c, uint64_t n,
                            int b_is_scalar, void *stream) {
  if (op > PP_FR_DIV) {
    pp::set_error("pp_fr_binary: op %u unknown", op);
    return PP_E_INVAL;
  }
  if (n == 0) return PP_OK;
  if (!pp::aligned16(d_a) || !pp::aligned16(d_b) || !pp::aligned16(d_c)) {
    pp::set_error("pp_fr_binary: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  if (b_is_scalar && pp::overlaps(d_b, sizeof(fr), d_c, n * sizeof(fr))) {
    pp::set_error("pp_fr_binary: the scalar operand must not overlap the output");
    return PP_E_INVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const fr *a = static_cast<const fr *>(d_a), *b = static_cast<const fr *>(d_b);
  fr *c = static_cast<fr *>(d_c);
  if (op == PP_FR_DIV) {
    if (!b_is_scalar) {
      pp::k_fr_div<<<pp::grid_for((n + pp::kInvRun - 1) / pp::kInvRun), pp::kThreads, 0, s>>>(a, b, c,
                                                                                             n);
      PP_COUNT_LAUNCH();
      PP_LAUNCH_CHECK();
      return PP_OK;
    }
    // a / b[0] = a * (1 / b[0]): one inversion, then a scalar multiply
    int st = PP_OK;
    fr *inv = static_cast<fr *>(pp::workspace_get(sizeof(fr), s, 4, &st));
    if (st) return st;
    pp::k_fr_inv1<<<1, 1, 0, s>>>(b, inv);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    b = inv;
    op = PP_FR_MUL;
  }
  pp::k_fr_binary<<<pp::grid_for(n), pp::kThreads, 0, s>>>(op, a, b, c, n, b_is_scalar);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_fr_unary(uint32_t op, const void *d_a, void *d_c, uint64_t n, void *stream) {
  if (op > PP_FR_INV) {
    pp::set_error("pp_fr_unary: op %u unknown", op);
    return PP_E_INVAL;
  }
  if (n == 0) return PP_OK;
  if (!pp::aligned16(d_a) || !pp::aligned16(d_c)) {
    pp::set_error("pp_fr_unary: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const fr *a = static_cast<const fr *>(d_a);
  fr *c = static_cast<fr *>(d_c);
  if (op == PP_FR_NEG) {
    pp::k_fr_neg<<<pp::grid_for(n), pp::kThreads, 0, s>>>(a, c, n);
  } else {
    pp::k_fr_div<<<pp::grid_for((n + pp::kInvRun - 1) / pp::kInvRun), pp::kThreads, 0, s>>>(nullptr, a,
                                                                                           c, n);
  }
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_fr_pow(const void *d_a, void *d_c, uint64_t n, uint64_t exponent, void *stream) {
  if (n == 0) return PP_OK;
  if (!pp::aligned16(d_a) || !pp::aligned16(d_c)) {
    pp::set_error("pp_fr_pow: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  pp::k_fr_pow<<<pp::grid_for(n), pp::kThreads, 0, (cudaStream_t)stream>>>(
      static_cast<const fr *>(d_a), static_cast<fr *>(d_c), n, exponent);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_fr_powers(const void *d_x, void *d_out, uint64_t n, void *stream) {
  if (n == 0) return PP_OK;
  if (!pp::aligned16(d_x) || !pp::aligned16(d_out) ||
      pp::overlaps(d_x, sizeof(fr), d_out, n * sizeof(fr))) {
    pp::set_error("pp_fr_powers: aligned device buffers, x not inside the output");
    return PP_E_INVAL;
  }
  pp::k_fr_powers<<<pp::grid_for((n + pp::kInvRun - 1) / pp::kInvRun), pp::kThreads, 0,
                    (cudaStream_t)stream>>>(static_cast<const fr *>(d_x), static_cast<fr *>(d_out), n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_fr_fill(const void *d_x, void *d_out, uint64_t n, void *stream) {
  if (n == 0) return PP_OK;
  if (!pp::aligned16(d_x) || !pp::aligned16(d_out) ||
      pp::overlaps(d_x, sizeof(fr), d_out, n * sizeof(fr))) {
    pp::set_error("pp_fr_fill: aligned device buffers, x not inside the output");
    return PP_E_INVAL;
  }
  pp::k_fr_fill<<<pp::grid_for(n), pp::kThreads, 0, (cudaStream_t)stream>>>(
      static_cast<const fr *>(d_x), static_cast<fr *>(d_out), n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}
