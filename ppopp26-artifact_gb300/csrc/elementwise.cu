// elementwise.cu -- element-wise Fr operators over vectors: the reference's
// add_mod / sub_mod / mul_mod / div_mod with their _scalar and in-place forms,
// neg_mod, inv_mod, exp_mod, gen_sequence and repeat_to_poly
// (PLONK/utils/function.cu:23-170 -> PLONK/utils/mont/cuda/mont_arithmetic.cu:
// 6-52, 414-520 and mont_arithmetic.cuh:17-95).
//
// They move 64-96 bytes per element for at most one Montgomery multiply, so
// HBM bounds them; grid-stride loops of 16-byte accesses.  Division and
// inversion differ: the reference inverts each element (mont_t::reciprocal,
// ff/mont_t.cuh:1117); here a warp's 1024 elements share one inversion
// (Montgomery's simultaneous inversion: about 3 multiplies per element).  An
// inversion costs thousands of dependent instructions, so fewer of them is
// what counts: with binary-GCD inversions 2^24 divisions took 3.71 ms with
// one divergent inversion per lane and 32 elements, 5.09 ms with one per
// warp and 256 elements in registers (118 registers), 1.81 ms as here; with
// the divstep inversion (modinv.cuh) 1.73 ms.  As in the reference, the
// inverse of 0 is taken as 0.
#include "common.cuh"

namespace pp {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kPowRun = 128;  // powers: elements per thread after one x^lo

// one thread per unit of work, the loops striding only past 2^31 - 1 blocks:
// at 2^24 add / mul / x^5 take 0.228 / 0.336 / 1.255 ms, against 0.243 /
// 0.348 / 1.289 ms with the grid capped at 8 blocks per SM
unsigned grid_for(uint64_t work) {
  const uint64_t want = (work + kThreads - 1) / kThreads;
  const uint64_t cap = 0x7fffffffull;
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

__device__ __forceinline__ fr shfl_up_fr(const fr &v, int o) {
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = __shfl_up_sync(0xffffffffu, v.v[i], o);
  return r;
}
__device__ __forceinline__ fr shfl_down_fr(const fr &v, int o) {
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = __shfl_down_sync(0xffffffffu, v.v[i], o);
  return r;
}
__device__ __forceinline__ fr shfl_fr(const fr &v, int src) {
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = __shfl_sync(0xffffffffu, v.v[i], src);
  return r;
}

// c_i = a_i / b_i (1 / b_i without a), 0 where b_i = 0.  Each lane takes a
// run of kDivRun elements and keeps the running products of its non-zero b;
// the warp combines the 32 run products with a prefix and a suffix
// scan, so one inversion -- the same value in every lane, no divergence --
// serves 32 kDivRun elements.  Each b_i and a_i is read before c_i is written,
// so c may alias a or b.  Every lane of a warp runs the same number of loop
// trips (the shuffles need all 32).
constexpr uint32_t kDivRun = 32;

// at most 64 registers: four blocks per SM (with the divstep inversion inlined
// the compiler would otherwise take 100 and fit two)
__global__ void __launch_bounds__(kThreads, 4)
    k_fr_div(const fr *a, const fr *b, fr *c, uint64_t n) {
  const int lane = threadIdx.x & 31;
  const uint64_t per_warp = 32ull * kDivRun;
  const uint64_t warps = (n + per_warp - 1) / per_warp;
  const uint64_t warp0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t wstride = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = warp0; w < warps; w += wstride) {
    const uint64_t lo = w * per_warp + (uint64_t)lane * kDivRun;
    fr pre[kDivRun];  // in local memory: a rolled loop keeps registers for occupancy
    fr acc = fr_one();
#pragma unroll 1
    for (uint32_t j = 0; j < kDivRun; ++j) {
      if (lo + j < n) {
        const fr v = ld_fr(b + lo + j);
        if (!fr_is_zero(v)) acc = fr_mul(acc, v);
      }
      pre[j] = acc;
    }
    // inclusive prefix and exclusive suffix products of the lanes' runs
    fr incl = acc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const fr u = shfl_up_fr(incl, o);
      if (lane >= o) incl = fr_mul(u, incl);
    }
    const fr total = shfl_fr(incl, 31);
    fr s = acc;  // inclusive suffix, then shifted to exclusive
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const fr u = shfl_down_fr(s, o);
      if (lane + o < 32) s = fr_mul(s, u);
    }
    fr suf = shfl_down_fr(s, 1);
    if (lane == 31) suf = fr_one();
    const fr excl = shfl_up_fr(incl, 1);
    // 1 / (this run's product) = (1 / total) * (runs before) * (runs after)
    fr inv = fr_mul(fr_inv_fast(total), suf);
    if (lane > 0) inv = fr_mul(inv, excl);
#pragma unroll 1
    for (int j = (int)kDivRun - 1; j >= 0; --j) {
      if (lo + j < n) {
        const fr v = ld_fr(b + lo + j);
        fr q = fr_zero();
        if (!fr_is_zero(v)) {
          q = j > 0 ? fr_mul(inv, pre[j - 1]) : inv;  // 1 / b
          inv = fr_mul(inv, v);
          if (a) q = fr_mul(ld_fr(a + lo + j), q);
        }
        st_fr(c + lo + j, q);
      }
    }
  }
}

// out[0] = 1 / x[0] (0 for 0)
__global__ void k_fr_inv1(const fr *x, fr *out) { st_fr(out, fr_inv_fast(ld_fr(x))); }

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

// out[i] = x^i: one thread per run of kPowRun, starting from x^lo
__global__ void __launch_bounds__(kThreads) k_fr_powers(const fr *x, fr *out, uint64_t n) {
  const fr b = ld_fr(x);
  const uint64_t runs = (n + kPowRun - 1) / kPowRun;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < runs;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = r * kPowRun, hi = lo + kPowRun < n ? lo + kPowRun : n;
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
      pp::k_fr_div<<<pp::grid_for((n + pp::kDivRun - 1) / pp::kDivRun), pp::kThreads, 0, s>>>(a, b, c,
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
    pp::k_fr_div<<<pp::grid_for((n + pp::kDivRun - 1) / pp::kDivRun), pp::kThreads, 0, s>>>(nullptr, a,
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
  pp::k_fr_powers<<<pp::grid_for((n + pp::kPowRun - 1) / pp::kPowRun), pp::kThreads, 0,
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
