// constraint.cu -- PLONK quotient-constraint operators: element-wise terms
// over the points of the extended domain, computed from the LDE outputs.
//
// Each output point costs 18 (permutation, fused) to ~105 (gate) Montgomery
// multiplies against 448 / 736 bytes of HBM traffic, so both kernels are
// integer-multiply bound by a factor of 5-40 over HBM.  They are plain
// element-wise loops: one thread per point, scalars staged once per block.
#include "common.cuh"

namespace pp {
namespace {

constexpr int kThreads = 256;

struct PermArgs {
  const fr *x, *w[4], *z, *z_next, *sigma[4], *mod, *l1;
  const fr *alpha, *beta, *gamma, *k[3], *one;
};

enum : int { kIdentity = 1, kCopy = 2, kTermOne = 4, kAll = 7 };

// prod_j (u_j * beta * c_j + w_j + gamma): the identity product uses u_j = x
// and c = (1, k1, k2, k3); the copy product u_j = sigma_j and c_j = 1
__device__ __forceinline__ fr identity_product(const PermArgs &a, uint64_t i, const fr &beta,
                                               const fr &gamma, const fr k[3]) {
  const fr xb = fr_mul(ldcs_fr(a.x + i), beta);
  fr acc = fr_add(fr_add(xb, ldcs_fr(a.w[0] + i)), gamma);
#pragma unroll
  for (int j = 1; j < 4; ++j)
    acc = fr_mul(acc, fr_add(fr_add(fr_mul(xb, k[j - 1]), ldcs_fr(a.w[j] + i)), gamma));
  return acc;
}

__device__ __forceinline__ fr copy_product(const PermArgs &a, uint64_t i, const fr &beta,
                                           const fr &gamma) {
  fr acc = fr_add(fr_add(fr_mul(ldcs_fr(a.sigma[0] + i), beta), ldcs_fr(a.w[0] + i)), gamma);
#pragma unroll
  for (int j = 1; j < 4; ++j)
    acc = fr_mul(acc, fr_add(fr_add(fr_mul(ldcs_fr(a.sigma[j] + i), beta), ldcs_fr(a.w[j] + i)),
                             gamma));
  return acc;
}

template <int TERMS>
__global__ void __launch_bounds__(kThreads) k_perm_quotient(const PermArgs a, fr *result,
                                                            uint64_t n) {
  const fr alpha = ldg_fr(a.alpha), beta = ldg_fr(a.beta), gamma = ldg_fr(a.gamma);
  fr k[3];
  if (TERMS & kIdentity) {
#pragma unroll
    for (int j = 0; j < 3; ++j) k[j] = ldg_fr(a.k[j]);
  }
  const fr one = (TERMS & kTermOne) ? ldg_fr(a.one) : fr_zero();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    fr r;
    if (TERMS == kAll) {
      // (id * z - cp * z_next) * alpha + mod + (z - one) * l1: alpha once
      const fr z = ldcs_fr(a.z + i);
      const fr id = fr_mul(identity_product(a, i, beta, gamma, k), z);
      const fr cp = fr_mul(copy_product(a, i, beta, gamma), ldcs_fr(a.z_next + i));
      r = fr_add(fr_mul(fr_sub(id, cp), alpha), ldcs_fr(a.mod + i));
      r = fr_add(r, fr_mul(fr_sub(z, one), ldcs_fr(a.l1 + i)));
    } else if (TERMS == kIdentity) {
      r = fr_mul(fr_mul(identity_product(a, i, beta, gamma, k), ldcs_fr(a.z + i)), alpha);
    } else if (TERMS == kCopy) {
      const fr cp = fr_mul(fr_mul(copy_product(a, i, beta, gamma), ldcs_fr(a.z_next + i)), alpha);
      r = fr_sub(fr_add(ld_fr(result + i), ldcs_fr(a.mod + i)), cp);
    } else {
      r = fr_add(ld_fr(result + i), fr_mul(fr_sub(ldcs_fr(a.z + i), one), ldcs_fr(a.l1 + i)));
    }
    st_fr(result + i, r);
  }
}

// ------------------------------------------------------------------- gate
struct GateArgs {
  const fr *v[PP_GATE_NV];
  const fr *s[PP_GATE_NS];
  uint32_t sbox_alpha;  // 2 <= sbox_alpha < 2^31
};

// x^e for 2 <= e < 2^31, square and multiply from the top set bit
__device__ __forceinline__ fr pow_small(const fr &x, uint32_t e) {
  fr r = x;
  for (int b = 30 - __clz(e); b >= 0; --b) {
    r = fr_mul(r, r);
    if ((e >> b) & 1) r = fr_mul(r, x);
  }
  return r;
}

// x^4 * three * one * two: the reference's x (x three)((x one)(x two))
__device__ __forceinline__ fr delta4(const fr &x, const fr &k312) {
  const fr x2 = fr_mul(x, x);
  return fr_mul(fr_mul(x2, x2), k312);
}

// small multiples by additions (exact, like any field identity)
__device__ __forceinline__ fr dbl(const fr &x) { return fr_add(x, x); }
__device__ __forceinline__ fr mul3(const fr &x) { return fr_add(dbl(x), x); }
__device__ __forceinline__ fr mul4(const fr &x) { return dbl(dbl(x)); }
__device__ __forceinline__ fr mul6(const fr &x) { return dbl(mul3(x)); }
__device__ __forceinline__ fr mul9(const fr &x) { return fr_add(dbl(mul4(x)), x); }
__device__ __forceinline__ fr mul18(const fr &x) { return dbl(mul9(x)); }
__device__ __forceinline__ fr mul36(const fr &x) { return dbl(mul18(x)); }
__device__ __forceinline__ fr mul81(const fr &x) { return mul9(mul9(x)); }
__device__ __forceinline__ fr mul83(const fr &x) { return fr_add(mul81(x), dbl(x)); }

// 6 x^4 (delta4 with three one two = 6)
__device__ __forceinline__ fr delta4_6(const fr &x) {
  const fr x2 = fr_mul(x, x);
  return mul6(fr_mul(x2, x2));
}

// The gate runs as three launches so that each keeps its live values in
// fewer registers (more resident warps): the range and logic terms are
// written first, then the arithmetic and public-input terms and the fixed-
// and variable-base group additions are added.

// The scalars as the gate kernels use them, prepared once per call by
// k_gate_prepare: the PP_GATE_NS scalars, then three one two, then whether
// four, one, two, three, nine, eighteen, eightyone and eightythree hold
// those integers, as the prover passes them.  Then the kernels take
// SMALL = true: multiplies by them become additions and one one / three one
// two drop out, with the same field values (range and logic 47 -> 27
// multiplies per point, groups 38 -> 35).  Any other values take SMALL =
// false, the expression as written.
struct GateScalars {
  fr s[PP_GATE_NS + 1];
  int small;
};

__global__ void k_gate_prepare(const GateArgs a, GateScalars *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  fr sc[PP_GATE_NS + 1];
  for (int j = 0; j < PP_GATE_NS; ++j) sc[j] = ldg_fr(a.s[j]);
  sc[PP_GATE_NS] = fr_mul(fr_mul(sc[PP_GATE_S_THREE], sc[PP_GATE_S_ONE]), sc[PP_GATE_S_TWO]);
  const fr one = fr_one();
  out->small = fr_eq(sc[PP_GATE_S_ONE], one) && fr_eq(sc[PP_GATE_S_TWO], dbl(one)) &&
               fr_eq(sc[PP_GATE_S_THREE], mul3(one)) && fr_eq(sc[PP_GATE_S_FOUR], mul4(one)) &&
               fr_eq(sc[PP_GATE_S_NINE], mul9(one)) && fr_eq(sc[PP_GATE_S_EIGHTEEN], mul18(one)) &&
               fr_eq(sc[PP_GATE_S_EIGHTYONE], mul81(one)) &&
               fr_eq(sc[PP_GATE_S_EIGHTYTHREE], mul83(one));
  for (int j = 0; j <= PP_GATE_NS; ++j) st_fr(out->s + j, sc[j]);
}

// copies the prepared scalars to shared memory
__device__ __forceinline__ void stage_scalars(const GateScalars *g, fr *sc) {
  if (threadIdx.x <= PP_GATE_NS) sc[threadIdx.x] = ldg_fr(g->s + threadIdx.x);
  __syncthreads();
}

#define S(name) sc[PP_GATE_S_##name]
#define V(name) ldcs_fr(a.v[PP_GATE_V_##name] + i)

// The host launches both forms; the one whose SMALL does not match the
// scalars returns at once.
template <bool SMALL>
__global__ void __launch_bounds__(kThreads, 2) k_gate_range_logic(const GateArgs a,
                                                               const GateScalars *gs, fr *out,
                                                               uint64_t n) {
  if ((__ldg(&gs->small) != 0) != SMALL) return;
  __shared__ __align__(16) fr sc[PP_GATE_NS + 1];
  stage_scalars(gs, sc);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const fr k312 = sc[PP_GATE_NS];
    const fr a_ = V(A), b = V(B), c = V(C), d = V(D), dn = V(D_NEXT);
    fr a4, b4, c4, d4;
    if constexpr (SMALL) {
      a4 = mul4(a_), b4 = mul4(b), c4 = mul4(c), d4 = mul4(d);
    } else {
      const fr four = S(FOUR);
      a4 = fr_mul(a_, four), b4 = fr_mul(b, four), c4 = fr_mul(c, four), d4 = fr_mul(d, four);
    }
    auto quad = [&](const fr &x) { return SMALL ? delta4_6(x) : delta4(x, k312); };

    // range gate: four 2-bit quads
    fr t = fr_mul(quad(fr_sub(a4, dn)), S(KAPPA_CU_RANGE));
    t = fr_add(t, fr_mul(quad(fr_sub(a_, b4)), S(KAPPA_SQ_RANGE)));
    t = fr_add(t, quad(fr_sub(c, d4)));
    t = fr_add(t, fr_mul(quad(fr_sub(b, c4)), S(KAPPA_RANGE)));
    fr acc = fr_mul(fr_mul(t, S(RANGE_CHALLENGE)), V(RANGE));

    // logic gate
    const fr da = fr_sub(a4, V(A_NEXT)), db = fr_sub(b4, V(B_NEXT));
    const fr w = fr_add(da, db), e = fr_sub(dn, d4);
    const fr da2 = fr_mul(da, da);
    fr inner, A, B, da4;
    if constexpr (SMALL) {
      inner = fr_sub(mul81(w), fr_add(fr_mul(c, mul81(fr_sub(c4, mul18(w)))), mul36(da2)));
      A = fr_sub(mul3(fr_add(e, w)), dbl(fr_mul(c, mul83(inner))));
      B = fr_mul(V(Q_C), fr_sub(mul9(e), mul3(w)));
      da4 = mul6(fr_mul(da2, da2));
    } else {
      inner = fr_sub(fr_mul(w, S(EIGHTYONE)),
                     fr_add(fr_mul(c, fr_mul(fr_sub(c4, fr_mul(w, S(EIGHTEEN))), S(EIGHTYONE))),
                            fr_mul(fr_add(da2, da2), S(EIGHTEEN))));
      A = fr_sub(fr_mul(fr_add(e, w), S(THREE)),
                 fr_mul(fr_mul(c, fr_mul(inner, S(EIGHTYTHREE))), S(TWO)));
      B = fr_mul(V(Q_C), fr_sub(fr_mul(e, S(NINE)), fr_mul(w, S(THREE))));
      da4 = fr_mul(fr_mul(da2, da2), k312);
    }
    fr l = fr_mul(fr_add(A, B), S(KAPPA_QU_LOGIC));
    l = fr_add(l, fr_mul(fr_sub(c, fr_mul(da, db)), S(KAPPA_CU_LOGIC)));
    l = fr_add(l, quad(e));
    l = fr_add(l, da4);
    l = fr_add(l, quad(db));
    acc = fr_add(acc, fr_mul(fr_mul(l, S(LOGIC_CHALLENGE)), V(LOGIC)));
    st_fr(out + i, acc);
  }
}

__global__ void __launch_bounds__(kThreads, 2) k_gate_arith(const GateArgs a, fr *out, uint64_t n) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const fr a_ = V(A), b = V(B), c = V(C), d = V(D);
    // arithmetic gate (with the x^alpha S-box terms) and public inputs
    fr ar = fr_mul(pow_small(d, a.sbox_alpha), V(Q_H4));
    ar = fr_add(ar, fr_mul(pow_small(b, a.sbox_alpha), V(Q_HR)));
    ar = fr_add(ar, fr_mul(pow_small(a_, a.sbox_alpha), V(Q_HL)));
    ar = fr_add(ar, fr_mul(d, V(Q_4)));
    ar = fr_add(ar, fr_mul(c, V(Q_O)));
    ar = fr_add(ar, fr_mul(b, V(Q_R)));
    ar = fr_add(ar, fr_mul(fr_mul(a_, b), V(Q_M)));
    ar = fr_add(ar, fr_mul(a_, V(Q_L)));
    ar = fr_add(ar, V(Q_C));
    const fr acc = fr_add(fr_add(ld_fr(out + i), fr_mul(ar, V(Q_ARITH))), V(PI));
    st_fr(out + i, acc);
  }
}

template <bool SMALL>
__global__ void __launch_bounds__(kThreads, 2) k_gate_groups(const GateArgs a,
                                                          const GateScalars *gs, fr *out,
                                                          uint64_t n) {
  if ((__ldg(&gs->small) != 0) != SMALL) return;
  __shared__ __align__(16) fr sc[PP_GATE_NS + 1];
  stage_scalars(gs, sc);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const fr a_ = V(A), b = V(B), c = V(C), d = V(D);
    const fr an = V(A_NEXT), bn = V(B_NEXT), dn = V(D_NEXT);
    const fr pd = S(P_D);
    const fr bc = fr_mul(b, c);
    // fixed-base group addition
    fr f;
    {
      const fr abc = fr_mul(a_, bc);
      const fr dn2 = fr_mul(dn, dn);
      // one one = 1 when SMALL
      const fr one2 = SMALL ? fr_one() : fr_mul(S(ONE), S(ONE));
      const fr qr2 = SMALL ? fr_mul(V(Q_R), dn2) : fr_mul(fr_mul(V(Q_R), dn2), one2);
      const fr qldn = fr_mul(V(Q_L), dn);
      f = fr_mul(fr_sub(c, fr_mul(V(Q_C), dn)), S(KAPPA_FB));
      f = fr_add(f, fr_mul(fr_sub(fr_sub(bn, fr_mul(fr_mul(abc, bn), pd)),
                                  fr_sub(fr_mul(b, qr2), fr_mul(a_, fr_mul(qldn, S(P_A))))),
                           S(KAPPA_CU_FB)));
      f = fr_add(f, SMALL ? fr_mul(dn2, dn) : fr_mul(fr_mul(dn2, dn), one2));
      f = fr_add(f, fr_mul(fr_sub(fr_add(an, fr_mul(fr_mul(abc, an), pd)),
                                  fr_add(fr_mul(b, qldn), fr_mul(a_, qr2))),
                           S(KAPPA_SQ_FB)));
      f = fr_mul(fr_mul(f, S(FB_CHALLENGE)), V(FIXED_GROUP_ADD));
    }
    // variable-base group addition
    fr v1 = fr_sub(fr_sub(fr_mul(b, d), fr_mul(fr_mul(a_, c), S(P_A))),
                   fr_sub(bn, fr_mul(bc, fr_mul(dn, fr_mul(bn, pd)))));
    v1 = fr_mul(v1, S(KAPPA_SQ_VB));
    fr v2 = fr_sub(fr_add(dn, bc), fr_add(an, fr_mul(bc, fr_mul(dn, fr_mul(an, pd)))));
    v2 = fr_add(fr_sub(dn, fr_mul(a_, d)), fr_mul(v2, S(KAPPA_VB)));
    const fr vb = fr_mul(fr_mul(fr_add(v1, v2), S(VB_CHALLENGE)), V(VARIABLE_GROUP_ADD));
    st_fr(out + i, fr_add(fr_add(ld_fr(out + i), f), vb));
  }
}
#undef S
#undef V

bool aligned16(const void *p) { return p && (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// capped: at most 8 blocks per SM, each striding over points; otherwise one
// thread per point, as every kernel here launches (the permutation terms:
// 2^22 points in 1.45 ms, against 1.85 ms with the cap)
unsigned grid_for(uint64_t n, bool capped = true) {
  const uint64_t want = (n + kThreads - 1) / kThreads;
  const uint64_t cap = capped ? (uint64_t)device_sm_count() * 8 : 0x7fffffffull;
  return (unsigned)(want < cap ? want : cap);
}

// which fields each term reads
int check_perm(const pp_perm_quotient_args *a, int terms, const void *result, const char *who) {
  if (!a || !aligned16(result)) {
    set_error("%s: arguments and a 16-byte aligned result are required", who);
    return PP_E_INVAL;
  }
  bool ok = aligned16(a->alpha) || !(terms & (kIdentity | kCopy));
  if (terms & (kIdentity | kCopy)) ok = ok && aligned16(a->beta) && aligned16(a->gamma);
  for (int j = 0; j < 4; ++j) {
    if (terms & (kIdentity | kCopy)) ok = ok && aligned16(a->w[j]);
    if (terms & kCopy) ok = ok && aligned16(a->sigma[j]);
  }
  if (terms & kIdentity) {
    ok = ok && aligned16(a->x) && aligned16(a->z);
    for (int j = 0; j < 3; ++j) ok = ok && aligned16(a->k[j]);
  }
  if (terms & kCopy) ok = ok && aligned16(a->mod) && aligned16(a->z_next);
  if (terms & kTermOne) ok = ok && aligned16(a->z) && aligned16(a->l1) && aligned16(a->one);
  if (!ok) {
    set_error("%s: a required input is missing or not 16-byte aligned", who);
    return PP_E_INVAL;
  }
  return PP_OK;
}

template <int TERMS>
int perm_launch(const pp_perm_quotient_args *a, void *result, uint64_t n, void *stream,
                const char *who) {
  if (n == 0) return PP_OK;
  const int st = check_perm(a, TERMS, result, who);
  if (st) return st;
  PermArgs p;
  p.x = static_cast<const fr *>(a->x);
  for (int j = 0; j < 4; ++j) {
    p.w[j] = static_cast<const fr *>(a->w[j]);
    p.sigma[j] = static_cast<const fr *>(a->sigma[j]);
  }
  p.z = static_cast<const fr *>(a->z);
  p.z_next = static_cast<const fr *>(a->z_next);
  p.mod = static_cast<const fr *>(a->mod);
  p.l1 = static_cast<const fr *>(a->l1);
  p.alpha = static_cast<const fr *>(a->alpha);
  p.beta = static_cast<const fr *>(a->beta);
  p.gamma = static_cast<const fr *>(a->gamma);
  for (int j = 0; j < 3; ++j) p.k[j] = static_cast<const fr *>(a->k[j]);
  p.one = static_cast<const fr *>(a->one);
  k_perm_quotient<TERMS><<<grid_for(n, false), kThreads, 0, (cudaStream_t)stream>>>(
      p, static_cast<fr *>(result), n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

}  // namespace
}  // namespace pp

extern "C" int pp_quotient_identity(const pp_perm_quotient_args *a, void *d_result, uint64_t n,
                                    void *stream) {
  return pp::perm_launch<pp::kIdentity>(a, d_result, n, stream, "pp_quotient_identity");
}

extern "C" int pp_quotient_copy(const pp_perm_quotient_args *a, void *d_result, uint64_t n,
                                void *stream) {
  return pp::perm_launch<pp::kCopy>(a, d_result, n, stream, "pp_quotient_copy");
}

extern "C" int pp_quotient_term_one(const pp_perm_quotient_args *a, void *d_result, uint64_t n,
                                    void *stream) {
  return pp::perm_launch<pp::kTermOne>(a, d_result, n, stream, "pp_quotient_term_one");
}

extern "C" int pp_quotient_permutation(const pp_perm_quotient_args *a, void *d_result, uint64_t n,
                                       void *stream) {
  return pp::perm_launch<pp::kAll>(a, d_result, n, stream, "pp_quotient_permutation");
}

extern "C" int pp_gate_constraint(const pp_gate_args *a, void *d_out, uint64_t n, void *stream) {
  if (n == 0) return PP_OK;
  if (!a || !pp::aligned16(d_out)) {
    pp::set_error("pp_gate_constraint: arguments and a 16-byte aligned output are required");
    return PP_E_INVAL;
  }
  if (a->sbox_alpha < 2 || a->sbox_alpha >= (int64_t{1} << 31)) {
    pp::set_error("pp_gate_constraint: sbox_alpha = %lld outside [2, 2^31)",
                  (long long)a->sbox_alpha);
    return PP_E_INVAL;
  }
  pp::GateArgs g;
  for (int j = 0; j < PP_GATE_NV; ++j) {
    if (!pp::aligned16(a->v[j])) {
      pp::set_error("pp_gate_constraint: vector %d is missing or not 16-byte aligned", j);
      return PP_E_INVAL;
    }
    g.v[j] = static_cast<const pp::fr *>(a->v[j]);
  }
  for (int j = 0; j < PP_GATE_NS; ++j) {
    if (!pp::aligned16(a->s[j])) {
      pp::set_error("pp_gate_constraint: scalar %d is missing or not 16-byte aligned", j);
      return PP_E_INVAL;
    }
    g.s[j] = static_cast<const pp::fr *>(a->s[j]);
  }
  g.sbox_alpha = (uint32_t)a->sbox_alpha;
  cudaStream_t s = (cudaStream_t)stream;
  int st = PP_OK;
  auto *gs = static_cast<pp::GateScalars *>(pp::workspace_get(sizeof(pp::GateScalars), s, 8, &st));
  if (st) return st;
  pp::k_gate_prepare<<<1, 32, 0, s>>>(g, gs);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  // one thread per point; of each pair, the form that does not match the
  // scalars returns at once
  const unsigned grid = pp::grid_for(n, false);
  pp::fr *out = static_cast<pp::fr *>(d_out);
  pp::k_gate_range_logic<true><<<grid, pp::kThreads, 0, s>>>(g, gs, out, n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_gate_range_logic<false><<<grid, pp::kThreads, 0, s>>>(g, gs, out, n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_gate_arith<<<grid, pp::kThreads, 0, s>>>(g, out, n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_gate_groups<true><<<grid, pp::kThreads, 0, s>>>(g, gs, out, n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_gate_groups<false><<<grid, pp::kThreads, 0, s>>>(g, gs, out, n);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}
