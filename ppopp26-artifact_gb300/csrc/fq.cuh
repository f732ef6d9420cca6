// fq.cuh -- BLS12-381 base field Fq (381-bit) for the G1 multi-scalar
// multiplication: Montgomery form with R = 2^384, canonical (< q), 12 x
// 32-bit little-endian limbs -- the same bytes as the reference's 6 x 64-bit
// limbs (PLONK/utils/mont/cuda/ff/bls12-381.hpp BLS12_381_P, BLS12_381_RR,
// one).  Usable on host and device (the carry primitives of fr.cuh are
// emulated on the host), so the formulas are unit-tested on the CPU.
#pragma once
#include "fr.cuh"

namespace pp {

struct fq {
  uint32_t v[12];
};

// q, least significant limb first
#define PP_Q0 0xffffaaabu
#define PP_Q1 0xb9feffffu
#define PP_Q2 0xb153ffffu
#define PP_Q3 0x1eabfffeu
#define PP_Q4 0xf6b0f624u
#define PP_Q5 0x6730d2a0u
#define PP_Q6 0xf38512bfu
#define PP_Q7 0x64774b84u
#define PP_Q8 0x434bacd7u
#define PP_Q9 0x4b1ba7b6u
#define PP_Q10 0x397fe69au
#define PP_Q11 0x1a0111eau
#define PP_QP 0xfffcfffdu  // -q^-1 mod 2^32

PP_HD fq fq_zero() {
  fq r;
#pragma unroll
  for (int i = 0; i < 12; ++i) r.v[i] = 0;
  return r;
}

// R mod q: the Montgomery form of 1
PP_HD fq fq_one() {
  return fq{{0x0002fffdu, 0x76090000u, 0xc40c0002u, 0xebf4000bu, 0x53c758bau, 0x5f489857u,
             0x70525745u, 0x77ce5853u, 0xa256ec6du, 0x5c071a97u, 0xfa80e493u, 0x15f65ec3u}};
}

PP_HD bool fq_is_zero(const fq &a) {
  uint32_t o = 0;
#pragma unroll
  for (int i = 0; i < 12; ++i) o |= a.v[i];
  return o == 0;
}

PP_HD bool fq_eq(const fq &a, const fq &b) {
  uint32_t o = 0;
#pragma unroll
  for (int i = 0; i < 12; ++i) o |= a.v[i] ^ b.v[i];
  return o == 0;
}

// x - q if x >= q (x < 2q), branch-free selection
PP_HD void fq_reduce_once(uint32_t x[12]) {
  const uint32_t q[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                          PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
  uint32_t d[12];
  d[0] = sub_cc(x[0], q[0]);
#pragma unroll
  for (int i = 1; i < 12; ++i) d[i] = subc_cc(x[i], q[i]);
  const uint32_t borrow = subc(0, 0);  // all ones when x < q
#pragma unroll
  for (int i = 0; i < 12; ++i) x[i] = borrow ? x[i] : d[i];
}

PP_HD fq fq_add(const fq &a, const fq &b) {
  fq r;
  r.v[0] = add_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int i = 1; i < 12; ++i) r.v[i] = addc_cc(a.v[i], b.v[i]);
  // a + b < 2q < 2^383: no carry out of the top limb
  fq_reduce_once(r.v);
  return r;
}

PP_HD fq fq_sub(const fq &a, const fq &b) {
  const uint32_t q[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                          PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
  fq r;
  r.v[0] = sub_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int i = 1; i < 12; ++i) r.v[i] = subc_cc(a.v[i], b.v[i]);
  const uint32_t borrow = subc(0, 0);
  r.v[0] = add_cc(r.v[0], q[0] & borrow);
#pragma unroll
  for (int i = 1; i < 12; ++i) r.v[i] = addc_cc(r.v[i], q[i] & borrow);
  return r;
}

PP_HD fq fq_dbl(const fq &a) { return fq_add(a, a); }

PP_HD fq fq_neg(const fq &a) { return fq_sub(fq_zero(), a); }

// Montgomery product a b R^-1 mod q: CIOS with the rows of Fr's variant 9
// (independent wide products per row, one add chain), m_i = t_0 * q' per row.
PP_HD void fq_row_ab(uint32_t t[14], uint32_t ai, const uint32_t b[12]) {
  uint32_t lo[12], hi[12];
#pragma unroll
  for (int j = 0; j < 12; ++j) {
    const uint64_t s = (uint64_t)ai * b[j] + t[j];
    lo[j] = (uint32_t)s;
    hi[j] = (uint32_t)(s >> 32);
  }
  t[0] = lo[0];
  t[1] = add_cc(lo[1], hi[0]);
#pragma unroll
  for (int j = 2; j < 12; ++j) t[j] = addc_cc(lo[j], hi[j - 1]);
  t[12] = addc_cc(t[12], hi[11]);
  t[13] = addc(t[13], 0);
}

PP_HD void fq_row_red(uint32_t t[14]) {
  const uint32_t q[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                          PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
  const uint32_t m = t[0] * PP_QP;
  uint32_t lo[12], hi[12];
#pragma unroll
  for (int j = 0; j < 12; ++j) {
    const uint64_t s = (uint64_t)m * q[j] + t[j];
    lo[j] = (uint32_t)s;
    hi[j] = (uint32_t)(s >> 32);
  }
  // lo[0] = 0 by the choice of m; word j+1 collects lo[j+1] + hi[j]
  uint32_t u[13];
  u[0] = add_cc(lo[1], hi[0]);
#pragma unroll
  for (int j = 1; j < 11; ++j) u[j] = addc_cc(lo[j + 1], hi[j]);
  u[11] = addc_cc(t[12], hi[11]);
  u[12] = addc(t[13], 0);
#pragma unroll
  for (int j = 0; j < 13; ++j) t[j] = u[j];
  t[13] = 0;
}

// The same rows with bare wide products and two add chains (low words, then
// high words).  A wide multiply with a 64-bit addend holds the integer-
// multiply pipe about 1.4 times as long as a bare one; the second add chain
// runs on the ALU pipe instead.
PP_HD void fq_row_ab_wide(uint32_t t[14], uint32_t ai, const uint32_t b[12]) {
  uint32_t lo[12], hi[12];
#pragma unroll
  for (int j = 0; j < 12; ++j) {
    const uint64_t p = (uint64_t)ai * b[j];
    lo[j] = (uint32_t)p;
    hi[j] = (uint32_t)(p >> 32);
  }
  t[0] = add_cc(t[0], lo[0]);
#pragma unroll
  for (int j = 1; j < 12; ++j) t[j] = addc_cc(t[j], lo[j]);
  t[12] = addc_cc(t[12], 0);
  t[13] = addc(t[13], 0);
  t[1] = add_cc(t[1], hi[0]);
#pragma unroll
  for (int j = 1; j < 12; ++j) t[j + 1] = addc_cc(t[j + 1], hi[j]);
  t[13] = addc(t[13], 0);
}

PP_HD void fq_row_red_wide(uint32_t t[14]) {
  const uint32_t q[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                          PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
  const uint32_t m = t[0] * PP_QP;
  uint32_t lo[12], hi[12];
#pragma unroll
  for (int j = 0; j < 12; ++j) {
    const uint64_t p = (uint64_t)m * q[j];
    lo[j] = (uint32_t)p;
    hi[j] = (uint32_t)(p >> 32);
  }
  (void)add_cc(t[0], lo[0]);  // 0 by the choice of m; keeps the carry
#pragma unroll
  for (int j = 1; j < 12; ++j) t[j] = addc_cc(t[j], lo[j]);
  t[12] = addc_cc(t[12], 0);
  t[13] = addc(t[13], 0);
  t[1] = add_cc(t[1], hi[0]);
#pragma unroll
  for (int j = 1; j < 12; ++j) t[j + 1] = addc_cc(t[j + 1], hi[j]);
  t[13] = addc(t[13], 0);
#pragma unroll
  for (int k = 0; k < 13; ++k) t[k] = t[k + 1];
  t[13] = 0;
}

// Row forms: AB / RED = 0 for the single-chain rows above, 1 for bare wide
// products.  Every form leaves the same 14-word window after each row.  The
// MSM's bucket sums keep the integer-multiply pipe ~84 % busy and the ALU
// pipe ~32 %, so moving the product rows' additions to the ALU pays there:
// the 2^20 MSM took 15.21 ms with (0, 0), 14.02 with (1, 0), 14.73 with
// (0, 1) and 14.84 with (1, 1) on GB300.
#ifndef PP_FQ_AB
#define PP_FQ_AB 1
#endif
#ifndef PP_FQ_RED
#define PP_FQ_RED 0
#endif
// the squaring's product rows: 0 single chain, 1 bare wide products (the
// same 2^20 MSM time, 14.13 against 14.12 ms)
#ifndef PP_FQ_SQ_WIDE
#define PP_FQ_SQ_WIDE 0
#endif

template <int AB, int RED>
PP_HD fq fq_mul_rows(const fq &a, const fq &b) {
  uint32_t t[14];
#pragma unroll
  for (int j = 0; j < 14; ++j) t[j] = 0;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    if (AB) fq_row_ab_wide(t, a.v[i], b.v);
    else fq_row_ab(t, a.v[i], b.v);
    if (RED) fq_row_red_wide(t);
    else fq_row_red(t);
  }
  // t < 2q < 2^383: t[12] = 0
  fq_reduce_once(t);
  fq r;
#pragma unroll
  for (int i = 0; i < 12; ++i) r.v[i] = t[i];
  return r;
}

// One out-of-line copy per translation unit: the point formulas call it
// ~10-14 times per addition, and with every call inlined the bucket-sum
// kernels outgrew the instruction cache (instruction-fetch stalls led; the
// 2^20 MSM ran in 25.5 ms against 18.8 ms with calls).
#ifdef __CUDACC__
#define PP_FQ_MUL static __host__ __device__ __noinline__
#else
#define PP_FQ_MUL static inline
#endif
PP_FQ_MUL fq fq_mul(const fq &a, const fq &b) { return fq_mul_rows<PP_FQ_AB, PP_FQ_RED>(a, b); }

// ---- squaring: a^2 = sum_i a_i C_i 2^(64 i) with C_i = a_i + 2^32 D_i and
// D_i = 2 floor(a / 2^(32 (i + 1))), so row i multiplies a_i by the 13 - i
// words of C_i instead of all 12 words of a: 78 wide products instead of 144
// before the (unchanged) reduction rows.  After i reduction rows the CIOS
// window has moved i words, so row i's term starts at window word i.
// A2 = 2a in 13 words; D_i's words are A2[i + 1 ..] with the bit that a_i
// shifted in cleared.
// the same row with bare wide products and two add chains
template <int I>
PP_HD void fq_row_sq_wide(uint32_t t[14], uint32_t ai, const uint32_t A2[13]) {
  constexpr int L = I < 11 ? 13 - I : 1;  // words I .. 12 (I = 11: word 11 only)
  uint32_t lo[13], hi[13];
  uint64_t p = (uint64_t)ai * ai;
  lo[0] = (uint32_t)p;
  hi[0] = (uint32_t)(p >> 32);
#pragma unroll
  for (int k = 1; k + 1 < L; ++k) {
    const uint32_t dk = k == 1 ? (A2[I + 1] & ~1u) : A2[I + k];
    p = (uint64_t)ai * dk;
    lo[k] = (uint32_t)p;
    hi[k] = (uint32_t)(p >> 32);
  }
  if constexpr (L > 1) {  // word 12: a_i times the top bit of 2a, no high word
    lo[L - 1] = A2[12] ? ai : 0u;
    hi[L - 1] = 0;
  }
  t[I] = add_cc(t[I], lo[0]);
#pragma unroll
  for (int k = 1; k < L; ++k) t[I + k] = addc_cc(t[I + k], lo[k]);
#pragma unroll
  for (int k = I + L; k < 13; ++k) t[k] = addc_cc(t[k], 0);
  t[13] = addc(t[13], 0);
  // high words land on I + 1 .. 12 for every row (the select's is 0)
  t[I + 1] = add_cc(t[I + 1], hi[0]);
#pragma unroll
  for (int k = 1; k + 1 < L; ++k) t[I + 1 + k] = addc_cc(t[I + 1 + k], hi[k]);
  t[13] = addc(t[13], 0);
}

template <int I>
PP_HD void fq_row_sq(uint32_t t[14], uint32_t ai, const uint32_t A2[13]) {
  uint32_t lo[13], hi[13];
  uint64_t s = (uint64_t)ai * ai + t[I];
  lo[0] = (uint32_t)s;
  hi[0] = (uint32_t)(s >> 32);
  if constexpr (I == 11) {  // C_11 = a_11
    t[11] = lo[0];
    t[12] = add_cc(t[12], hi[0]);
    t[13] = addc(t[13], 0);
  } else {
    constexpr int L = 13 - I;  // words I .. 12
#pragma unroll
    for (int k = 1; k + 1 < L; ++k) {  // a_i D_i[k - 1] at word I + k
      const uint32_t dk = k == 1 ? (A2[I + 1] & ~1u) : A2[I + k];
      s = (uint64_t)ai * dk + t[I + k];
      lo[k] = (uint32_t)s;
      hi[k] = (uint32_t)(s >> 32);
    }
    s = (uint64_t)(A2[12] ? ai : 0u) + t[12];  // a_i times the top bit of 2a
    lo[L - 1] = (uint32_t)s;
    hi[L - 1] = (uint32_t)(s >> 32);
    t[I] = lo[0];
    t[I + 1] = add_cc(lo[1], hi[0]);
#pragma unroll
    for (int k = 2; k < L; ++k) t[I + k] = addc_cc(lo[k], hi[k - 1]);
    t[13] = addc(t[13], hi[L - 1]);
  }
}

template <int I>
PP_HD void fq_sq_rows(uint32_t t[14], const fq &a, const uint32_t A2[13]) {
  if (PP_FQ_SQ_WIDE) fq_row_sq_wide<I>(t, a.v[I], A2);
  else fq_row_sq<I>(t, a.v[I], A2);
  if (PP_FQ_RED) fq_row_red_wide(t);
  else fq_row_red(t);
  if constexpr (I < 11) fq_sq_rows<I + 1>(t, a, A2);
}

// a^2 R^-1 mod q for a < q (same result as fq_mul(a, a)); the window stays
// below 2^448 (row 0 adds up to 2^417) and ends below 2q
PP_FQ_MUL fq fq_sqr(const fq &a) {
  uint32_t A2[13];
  A2[0] = a.v[0] << 1;
#pragma unroll
  for (int k = 1; k < 12; ++k) A2[k] = (a.v[k] << 1) | (a.v[k - 1] >> 31);
  A2[12] = a.v[11] >> 31;
  uint32_t t[14];
#pragma unroll
  for (int j = 0; j < 14; ++j) t[j] = 0;
  fq_sq_rows<0>(t, a, A2);
  fq_reduce_once(t);
  fq r;
#pragma unroll
  for (int i = 0; i < 12; ++i) r.v[i] = t[i];
  return r;
}

// ---- binary extended-GCD inverse: shifts and subtractions instead of the
// ~480 dependent multiplies of a Fermat chain (for single-thread use)
PP_HD bool fq_words_is_one(const uint32_t a[12]) {
  uint32_t o = a[0] ^ 1u;
#pragma unroll
  for (int i = 1; i < 12; ++i) o |= a[i];
  return o == 0;
}
PP_HD bool fq_words_lt(const uint32_t a[12], const uint32_t b[12]) {
  for (int i = 11; i >= 0; --i)
    if (a[i] != b[i]) return a[i] < b[i];
  return false;
}
PP_HD void fq_words_shr1(uint32_t a[12]) {
#pragma unroll
  for (int i = 0; i < 11; ++i) a[i] = (a[i] >> 1) | (a[i + 1] << 31);
  a[11] >>= 1;
}
PP_HD void fq_words_sub(uint32_t a[12], const uint32_t b[12]) {
  a[0] = sub_cc(a[0], b[0]);
#pragma unroll
  for (int i = 1; i < 12; ++i) a[i] = subc_cc(a[i], b[i]);
}
// x / 2 mod q for x < q: (x + q) / 2 when x is odd (x + q < 2^383)
PP_HD void fq_half(uint32_t x[12]) {
  const uint32_t q[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                          PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
  const uint32_t mask = 0u - (x[0] & 1u);
  x[0] = add_cc(x[0], q[0] & mask);
#pragma unroll
  for (int i = 1; i < 12; ++i) x[i] = addc_cc(x[i], q[i] & mask);
  fq_words_shr1(x);
}

// a^-1 in Montgomery form (0 -> 0).  The GCD inverts the raw word value
// A = a R; the result A^-1 times R^3 under one Montgomery multiply is
// a^-1 R.
PP_HD fq fq_inv(const fq &a) {
  if (fq_is_zero(a)) return fq_zero();
  uint32_t u[12], v[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                           PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
  fq x1 = fq_zero(), x2 = fq_zero();
  x1.v[0] = 1;
#pragma unroll
  for (int i = 0; i < 12; ++i) u[i] = a.v[i];
  // at most ~2 * 384 halvings and 384 subtractions for canonical input; the
  // bounds only guard against non-canonical input
  for (int guard = 0; guard < 1536 && !fq_words_is_one(u) && !fq_words_is_one(v); ++guard) {
    for (int k = 0; k < 384 && !(u[0] & 1u); ++k) {
      fq_words_shr1(u);
      fq_half(x1.v);
    }
    for (int k = 0; k < 384 && !(v[0] & 1u); ++k) {
      fq_words_shr1(v);
      fq_half(x2.v);
    }
    if (!fq_words_lt(u, v)) {
      fq_words_sub(u, v);
      x1 = fq_sub(x1, x2);
    } else {
      fq_words_sub(v, u);
      x2 = fq_sub(x2, x1);
    }
  }
  const fq y = fq_words_is_one(u) ? x1 : x2;
  // R^3 mod q
  const fq r3 = {{0xd94ca1e0u, 0xed48ac6bu, 0x03a7adf8u, 0x315f831eu, 0x615e29ddu, 0x9a53352au,
                  0x921e1761u, 0x34c04e5eu, 0x65724728u, 0x2512d435u, 0x91755d4du, 0x0aa63460u}};
  return fq_mul(y, r3);
}

// q in B-bit limbs and q^-1 mod 2^B
template <typename L>
PP_HD ModulusB<L, (381 + LimbTraits<L>::B) / LimbTraits<L>::B> fq_modulus_limbs();
template <>
PP_HD ModulusB<int32_t, 13> fq_modulus_limbs<int32_t>() {
  return {{0x3fffaaab, 0x27fbffff, 0x153ffffb, 0x2affffac, 0x30f6241e, 0x034a83da, 0x112bf673,
           0x12e13ce1, 0x2cd76477, 0x1ed90d2e, 0x29a4b1ba, 0x3a8e5ff9, 0x001a0111},
          0x00030003u};
}
template <>
PP_HD ModulusB<int64_t, 7> fq_modulus_limbs<int64_t>() {
  return {{0x39feffffffffaaabll, 0x3aaffffac54ffffell, 0x330d2a0f6b0f6241ll, 0x1dd2e13ce144afd9ll,
           0x1ba7b6434bacd764ll, 0x0447a8e5ff9a692cll, 0x00000000000001a0ll},
          0x360c000300030003ull};
}

// the same inverse by divsteps (modinv.cuh): at most 37 batches of 30 steps
// (or 18 of 62) instead of the binary GCD's ~1150 steps on 12-word numbers
template <typename L>
PP_HD fq fq_inv_divsteps(const fq &a) {
  constexpr int B = LimbTraits<L>::B, NL = (381 + B) / B;
  if (fq_is_zero(a)) return fq_zero();
  const ModulusB<L, NL> M = fq_modulus_limbs<L>();
  const SLimbs<L, NL> y =
      modinv_divsteps<L, NL>(words_to_limbs<L, 12, NL>(a.v), M, (1101 + B - 1) / B);
  fq out;
  limbs_to_words<L, 12, NL>(y, out.v);
  const fq r3 = {{0xd94ca1e0u, 0xed48ac6bu, 0x03a7adf8u, 0x315f831eu, 0x615e29ddu, 0x9a53352au,
                  0x921e1761u, 0x34c04e5eu, 0x65724728u, 0x2512d435u, 0x91755d4du, 0x0aa63460u}};
  return fq_mul(out, r3);
}

PP_HD fq fq_inv_fast(const fq &a) {
#ifdef __CUDA_ARCH__
  return fq_inv_divsteps<int32_t>(a);
#else
  return fq_inv_divsteps<int64_t>(a);
#endif
}

}  // namespace pp
