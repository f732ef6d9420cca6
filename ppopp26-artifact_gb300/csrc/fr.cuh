// fr.cuh -- BLS12-381 scalar field Fr on 8 x 32-bit limbs, Montgomery form.
//
// Storage is the reference's: 4 little-endian uint64 limbs (= 8 little-endian
// uint32 limbs), Montgomery representation with R = 2^256, canonical (< r)
// (PLONK/utils/mont/cuda/ff/bls12-381.hpp:7-45, mont_t.cuh:34).
//
// Arithmetic is written once over "carry-chain primitives" that map 1:1 onto
// PTX integer instructions with the condition-code carry (add.cc, addc,
// mad.lo.cc, madc.hi ...).  On the device they are inline PTX; on the host the
// same functions emulate the carry flag exactly, so every multiply variant is
// unit-tested on the CPU against the oracle before it runs on a GPU.
//
// Multiplication is Montgomery CIOS (Koc, Acar, Kaliski, "Analyzing and
// comparing Montgomery multiplication algorithms", IEEE Micro 1996) on 32-bit
// words.  r = 1 (mod 2^32) gives -r^-1 = 0xffffffff, so each row's m is a
// negation, and the two lowest words of r (1 and 0xffffffff) make m*r[0] and
// m*r[1] multiply-free: each row costs 16 + 12 integer multiplies instead of
// 16 + 16.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PP_HD __host__ __device__ __forceinline__
#else
#define PP_HD inline
#endif

namespace pp {

// r, 32-bit limbs, least significant first
#define PP_R0 0x00000001u
#define PP_R1 0xffffffffu
#define PP_R2 0xfffe5bfeu
#define PP_R3 0x53bda402u
#define PP_R4 0x09a1d805u
#define PP_R5 0x3339d808u
#define PP_R6 0x299d7d48u
#define PP_R7 0x73eda753u

struct fr {
  uint32_t v[8];
};

// ---------------------------------------------------------------------------
// carry-chain primitives
// ---------------------------------------------------------------------------
#if !defined(__CUDA_ARCH__)
inline uint32_t &host_cf() {
  static thread_local uint32_t cf = 0;
  return cf;
}
#endif

#if defined(__CUDA_ARCH__)
#define PP_ASM1(op, a, b)                                                     \
  uint32_t r;                                                                 \
  asm volatile(op " %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));                 \
  return r
#define PP_ASM2(op, a, b, c)                                                  \
  uint32_t r;                                                                 \
  asm volatile(op " %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));     \
  return r
#endif

PP_HD uint32_t add_cc(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  PP_ASM1("add.cc.u32", a, b);
#else
  uint64_t s = (uint64_t)a + b;
  host_cf() = (uint32_t)(s >> 32);
  return (uint32_t)s;
#endif
}
PP_HD uint32_t addc_cc(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  PP_ASM1("addc.cc.u32", a, b);
#else
  uint64_t s = (uint64_t)a + b + host_cf();
  host_cf() = (uint32_t)(s >> 32);
  return (uint32_t)s;
#endif
}
PP_HD uint32_t addc(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  PP_ASM1("addc.u32", a, b);
#else
  return (uint32_t)((uint64_t)a + b + host_cf());
#endif
}
PP_HD uint32_t sub_cc(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  PP_ASM1("sub.cc.u32", a, b);
#else
  host_cf() = a < b;
  return a - b;
#endif
}
PP_HD uint32_t subc_cc(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  PP_ASM1("subc.cc.u32", a, b);
#else
  uint64_t bb = (uint64_t)b + host_cf();
  host_cf() = (uint64_t)a < bb;
  return (uint32_t)((uint64_t)a - bb);
#endif
}
PP_HD uint32_t subc(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  PP_ASM1("subc.u32", a, b);
#else
  return (uint32_t)((uint64_t)a - b - host_cf());
#endif
}
PP_HD uint32_t mullo(uint32_t a, uint32_t b) { return a * b; }
PP_HD uint32_t mulhi(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
PP_HD uint32_t madlo_cc(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
  PP_ASM2("mad.lo.cc.u32", a, b, c);
#else
  uint64_t s = (uint64_t)(uint32_t)(a * b) + c;
  host_cf() = (uint32_t)(s >> 32);
  return (uint32_t)s;
#endif
}
PP_HD uint32_t madloc_cc(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
  PP_ASM2("madc.lo.cc.u32", a, b, c);
#else
  uint64_t s = (uint64_t)(uint32_t)(a * b) + c + host_cf();
  host_cf() = (uint32_t)(s >> 32);
  return (uint32_t)s;
#endif
}
PP_HD uint32_t madloc(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
  PP_ASM2("madc.lo.u32", a, b, c);
#else
  return (uint32_t)((uint64_t)(uint32_t)(a * b) + c + host_cf());
#endif
}
PP_HD uint32_t madhi_cc(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
  PP_ASM2("mad.hi.cc.u32", a, b, c);
#else
  uint64_t s = (((uint64_t)a * b) >> 32) + c;
  host_cf() = (uint32_t)(s >> 32);
  return (uint32_t)s;
#endif
}
PP_HD uint32_t madhic_cc(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
  PP_ASM2("madc.hi.cc.u32", a, b, c);
#else
  uint64_t s = (((uint64_t)a * b) >> 32) + c + host_cf();
  host_cf() = (uint32_t)(s >> 32);
  return (uint32_t)s;
#endif
}
PP_HD uint32_t madhic(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
  PP_ASM2("madc.hi.u32", a, b, c);
#else
  return (uint32_t)((((uint64_t)a * b) >> 32) + c + host_cf());
#endif
}

// ---------------------------------------------------------------------------
// constants
// ---------------------------------------------------------------------------
PP_HD fr fr_zero() { return fr{{0, 0, 0, 0, 0, 0, 0, 0}}; }
// R mod r (Montgomery one)
PP_HD fr fr_one() {
  return fr{{0xfffffffeu, 0x00000001u, 0x00034802u, 0x5884b7fau, 0xecbc4ff5u, 0x998c4fefu,
             0xacc5056fu, 0x1824b159u}};
}
// R^2 mod r
PP_HD fr fr_rr() {
  return fr{{0xf3f29c6du, 0xc999e990u, 0x87925c23u, 0x2b6cedcbu, 0x7254398fu, 0x05d31496u,
             0x9f59ff11u, 0x0748d9d9u}};
}

PP_HD bool fr_is_zero(const fr &a) {
  return (a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5] | a.v[6] | a.v[7]) == 0;
}
PP_HD bool fr_eq(const fr &a, const fr &b) {
  uint32_t d = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) d |= a.v[i] ^ b.v[i];
  return d == 0;
}

// x - r if x >= r else x, for x < 2^256 (x < 2r)
PP_HD void fr_reduce_once(uint32_t x[8]) {
  uint32_t t[8];
  t[0] = sub_cc(x[0], PP_R0);
  t[1] = subc_cc(x[1], PP_R1);
  t[2] = subc_cc(x[2], PP_R2);
  t[3] = subc_cc(x[3], PP_R3);
  t[4] = subc_cc(x[4], PP_R4);
  t[5] = subc_cc(x[5], PP_R5);
  t[6] = subc_cc(x[6], PP_R6);
  t[7] = subc_cc(x[7], PP_R7);
  uint32_t borrow = subc(0, 0);  // 0xffffffff if x < r
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = borrow ? x[i] : t[i];
}

PP_HD fr fr_add(const fr &a, const fr &b) {
  fr s;
  s.v[0] = add_cc(a.v[0], b.v[0]);
  s.v[1] = addc_cc(a.v[1], b.v[1]);
  s.v[2] = addc_cc(a.v[2], b.v[2]);
  s.v[3] = addc_cc(a.v[3], b.v[3]);
  s.v[4] = addc_cc(a.v[4], b.v[4]);
  s.v[5] = addc_cc(a.v[5], b.v[5]);
  s.v[6] = addc_cc(a.v[6], b.v[6]);
  s.v[7] = addc(a.v[7], b.v[7]);  // a + b < 2r < 2^256
  fr_reduce_once(s.v);
  return s;
}

PP_HD fr fr_sub(const fr &a, const fr &b) {
  fr d;
  d.v[0] = sub_cc(a.v[0], b.v[0]);
  d.v[1] = subc_cc(a.v[1], b.v[1]);
  d.v[2] = subc_cc(a.v[2], b.v[2]);
  d.v[3] = subc_cc(a.v[3], b.v[3]);
  d.v[4] = subc_cc(a.v[4], b.v[4]);
  d.v[5] = subc_cc(a.v[5], b.v[5]);
  d.v[6] = subc_cc(a.v[6], b.v[6]);
  d.v[7] = subc_cc(a.v[7], b.v[7]);
  uint32_t mask = subc(0, 0);  // all ones on borrow
  d.v[0] = add_cc(d.v[0], PP_R0 & mask);
  d.v[1] = addc_cc(d.v[1], PP_R1 & mask);
  d.v[2] = addc_cc(d.v[2], PP_R2 & mask);
  d.v[3] = addc_cc(d.v[3], PP_R3 & mask);
  d.v[4] = addc_cc(d.v[4], PP_R4 & mask);
  d.v[5] = addc_cc(d.v[5], PP_R5 & mask);
  d.v[6] = addc_cc(d.v[6], PP_R6 & mask);
  d.v[7] = addc(d.v[7], PP_R7 & mask);
  return d;
}

PP_HD fr fr_neg(const fr &a) { return fr_sub(fr_zero(), a); }

// ---------------------------------------------------------------------------
// Montgomery multiplication, a * b * 2^-256 mod r
// ---------------------------------------------------------------------------
// One CIOS row on the running sum t[0..9] (t[9] receives the top carry):
// t += ai * b; m = -t[0]; t += m * r; t >>= 32.
// Variant "s" (special): uses r[0] = 1, r[1] = 2^32 - 1.
PP_HD void cios_row_s(uint32_t t[10], uint32_t ai, const uint32_t b[8]) {
  // t[0..8] += lo(ai*b[j]) at j, carry into t[9]
  t[0] = madlo_cc(ai, b[0], t[0]);
  t[1] = madloc_cc(ai, b[1], t[1]);
  t[2] = madloc_cc(ai, b[2], t[2]);
  t[3] = madloc_cc(ai, b[3], t[3]);
  t[4] = madloc_cc(ai, b[4], t[4]);
  t[5] = madloc_cc(ai, b[5], t[5]);
  t[6] = madloc_cc(ai, b[6], t[6]);
  t[7] = madloc_cc(ai, b[7], t[7]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(0, 0);
  // t[1..9] += hi(ai*b[j]) at j+1
  t[1] = madhi_cc(ai, b[0], t[1]);
  t[2] = madhic_cc(ai, b[1], t[2]);
  t[3] = madhic_cc(ai, b[2], t[3]);
  t[4] = madhic_cc(ai, b[3], t[4]);
  t[5] = madhic_cc(ai, b[4], t[5]);
  t[6] = madhic_cc(ai, b[5], t[6]);
  t[7] = madhic_cc(ai, b[6], t[7]);
  t[8] = madhic_cc(ai, b[7], t[8]);
  t[9] = addc(t[9], 0);
  // m = -t0 (mod 2^32).  m*r[0] + m*r[1]*2^32 = m + (m << 32) - m*... :
  //   lo(m*1) = m       -> t0 + m == 0 (mod 2^32), carry out = (t0 != 0)
  //   lo(m*(2^32-1)) = -m = t0,  hi(m*(2^32-1)) = m - (m != 0)
  const uint32_t t0 = t[0];
  const uint32_t m = 0u - t0;
  uint32_t h1;
  (void)sub_cc(0, m);  // borrow = (m != 0)
  h1 = subc(m, 0);     // m - (m != 0)
  (void)add_cc(t0, 0xffffffffu);  // carry = (t0 != 0): the carry out of t0 + m
  t[1] = addc_cc(t[1], t0);
  t[2] = madloc_cc(m, PP_R2, t[2]);
  t[3] = madloc_cc(m, PP_R3, t[3]);
  t[4] = madloc_cc(m, PP_R4, t[4]);
  t[5] = madloc_cc(m, PP_R5, t[5]);
  t[6] = madloc_cc(m, PP_R6, t[6]);
  t[7] = madloc_cc(m, PP_R7, t[7]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(t[9], 0);
  t[2] = add_cc(t[2], h1);
  t[3] = madhic_cc(m, PP_R2, t[3]);
  t[4] = madhic_cc(m, PP_R3, t[4]);
  t[5] = madhic_cc(m, PP_R4, t[5]);
  t[6] = madhic_cc(m, PP_R5, t[6]);
  t[7] = madhic_cc(m, PP_R6, t[7]);
  t[8] = madhic_cc(m, PP_R7, t[8]);
  t[9] = addc(t[9], 0);
  // shift down one word (t[0] is zero now)
#pragma unroll
  for (int k = 0; k < 9; ++k) t[k] = t[k + 1];
  t[9] = 0;
}

// Variant "g" (generic CIOS rows, no use of the shape of r).
PP_HD void cios_row_g(uint32_t t[10], uint32_t ai, const uint32_t b[8]) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  t[0] = madlo_cc(ai, b[0], t[0]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j] = madloc_cc(ai, b[j], t[j]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(0, 0);
  t[1] = madhi_cc(ai, b[0], t[1]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j + 1] = madhic_cc(ai, b[j], t[j + 1]);
  t[9] = addc(t[9], 0);
  const uint32_t m = t[0] * 0xffffffffu;
  t[0] = madlo_cc(m, r[0], t[0]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j] = madloc_cc(m, r[j], t[j]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(t[9], 0);
  t[1] = madhi_cc(m, r[0], t[1]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j + 1] = madhic_cc(m, r[j], t[j + 1]);
  t[9] = addc(t[9], 0);
#pragma unroll
  for (int k = 0; k < 9; ++k) t[k] = t[k + 1];
  t[9] = 0;
}

template <int VARIANT>
PP_HD fr fr_mul_v(const fr &a, const fr &b) {
  uint32_t t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (VARIANT == 0)
      cios_row_s(t, a.v[i], b.v);
    else
      cios_row_g(t, a.v[i], b.v);
  }
  // t < 2r < 2^256 (t[8] == 0)
  fr_reduce_once(t);
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[i];
  return out;
}

// Variant "w": CIOS in plain C over 64-bit products (compiler-chosen wide
// multiply-adds), also using r[0] = 1.
PP_HD fr fr_mul_w(const fr &a, const fr &b) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  uint32_t t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      uint64_t s = (uint64_t)a.v[i] * b.v[j] + t[j] + c;
      t[j] = (uint32_t)s;
      c = s >> 32;
    }
    uint64_t s = (uint64_t)t[8] + c;
    t[8] = (uint32_t)s;
    t[9] = (uint32_t)(s >> 32);
    const uint32_t m = 0u - t[0];
    c = ((uint64_t)m + t[0]) >> 32;
#pragma unroll
    for (int j = 1; j < 8; ++j) {
      s = (uint64_t)m * r[j] + t[j] + c;
      t[j - 1] = (uint32_t)s;
      c = s >> 32;
    }
    s = (uint64_t)t[8] + c;
    t[7] = (uint32_t)s;
    t[8] = t[9] + (uint32_t)(s >> 32);
  }
  fr_reduce_once(t);
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[i];
  return out;
}

// ---------------------------------------------------------------------------
// Karatsuba product + word-serial Montgomery reduction (variants 3 and 4).
// A 32x32->64 multiply costs two to three times an add on the integer pipes
// of sm_103a, so trading products for additions pays: one Karatsuba level
// turns the 64 products of an 8x8-limb schoolbook into 48, two levels into 36.
// Carries are tracked in 64-bit C arithmetic (the compiler picks the wide
// multiply-add forms); the same code runs on the host for testing.
// ---------------------------------------------------------------------------
// r[0..2n) = a[0..n) * b[0..n), schoolbook
template <int NL>
PP_HD void mul_school(uint32_t *r, const uint32_t *a, const uint32_t *b) {
#pragma unroll
  for (int k = 0; k < 2 * NL; ++k) r[k] = 0;
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < NL; ++j) {
      const uint64_t s = (uint64_t)a[i] * b[j] + r[i + j] + c;
      r[i + j] = (uint32_t)s;
      c = s >> 32;
    }
    r[i + NL] = (uint32_t)c;
  }
}

// r[0..2n) = a * b via one Karatsuba level on top of MUL (n = 2h)
template <int NL, bool DEEP>
PP_HD void mul_kara(uint32_t *r, const uint32_t *a, const uint32_t *b) {
  constexpr int H = NL / 2;
  uint32_t sa[H], sb[H];
  uint64_t c = 0;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    c += (uint64_t)a[i] + a[i + H];
    sa[i] = (uint32_t)c;
    c >>= 32;
  }
  const uint32_t ca = (uint32_t)c;
  c = 0;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    c += (uint64_t)b[i] + b[i + H];
    sb[i] = (uint32_t)c;
    c >>= 32;
  }
  const uint32_t cb = (uint32_t)c;
  uint32_t z0[NL], z2[NL], z1[NL];
  if constexpr (DEEP && (H % 2 == 0)) {
    mul_kara<H, false>(z0, a, b);
    mul_kara<H, false>(z2, a + H, b + H);
    mul_kara<H, false>(z1, sa, sb);
  } else {
    mul_school<H>(z0, a, b);
    mul_school<H>(z2, a + H, b + H);
    mul_school<H>(z1, sa, sb);
  }
  // z1 (NL+1 limbs) += ca*sb<<H*32 + cb*sa<<H*32 + ca*cb<<NL*32
  const uint32_t ma = 0u - ca, mb = 0u - cb;
  uint32_t z1top = ca & cb;
  c = 0;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    c += (uint64_t)z1[i + H] + (sb[i] & ma) + (sa[i] & mb);
    z1[i + H] = (uint32_t)c;
    c >>= 32;
  }
  z1top += (uint32_t)c;
  // z1 -= z0 + z2 (the middle term is non-negative)
  int64_t br = 0;
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    const int64_t d = (int64_t)z1[i] - z0[i] - z2[i] + br;
    z1[i] = (uint32_t)d;
    br = d >> 32;  // arithmetic: -2, -1 or 0
  }
  z1top = (uint32_t)((int64_t)z1top + br);
  // r = z0 + z1 << (H*32) + z2 << (NL*32)
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    r[i] = z0[i];
    r[i + NL] = z2[i];
  }
  c = 0;
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    c += (uint64_t)r[i + H] + z1[i];
    r[i + H] = (uint32_t)c;
    c >>= 32;
  }
  c += (uint64_t)r[NL + H] + z1top;
  r[NL + H] = (uint32_t)c;
  c >>= 32;
#pragma unroll
  for (int i = NL + H + 1; i < 2 * NL; ++i) {
    c += r[i];
    r[i] = (uint32_t)c;
    c >>= 32;
  }
}

// Word-serial Montgomery reduction of t[0..16) (t < r * 2^256):
// t * 2^-256 mod r.  Round i adds m * r * 2^(32 i) with m = -t[i]; r[0] = 1
// and r[1] = 2^32 - 1 make the first two word products shifts and adds
// (m * (2^32 - 1) = (m << 32) - m), so a round costs 6 wide products.  The
// carry out of round i's top word (i + 8) is kept as one bit and added with
// round i+1's carry into word i + 9, so no carry ripples to the top.
PP_HD fr mont_redc16(uint32_t t[16]) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  uint32_t hc = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t m = 0u - t[i];
    uint64_t c = ((uint64_t)m + t[i]) >> 32;  // word i becomes 0
    uint64_t s = ((uint64_t)m << 32) - m + t[i + 1] + c;
    t[i + 1] = (uint32_t)s;
    c = s >> 32;
#pragma unroll
    for (int j = 2; j < 8; ++j) {
      s = (uint64_t)m * r[j] + t[i + j] + c;
      t[i + j] = (uint32_t)s;
      c = s >> 32;
    }
    s = (uint64_t)t[i + 8] + c + hc;
    t[i + 8] = (uint32_t)s;
    hc = (uint32_t)(s >> 32);
  }
  // result t[8..16) < 2r < 2^256 (hc == 0)
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[8 + i];
  fr_reduce_once(out.v);
  return out;
}

// variant 3: one Karatsuba level; variant 4: two levels
template <bool DEEP>
PP_HD fr fr_mul_kara(const fr &a, const fr &b) {
  uint32_t t[16];
  mul_kara<8, DEEP>(t, a.v, b.v);
  return mont_redc16(t);
}

#ifndef PP_MUL_VARIANT
#define PP_MUL_VARIANT 0
#endif

// ---------------------------------------------------------------------------
// Variants 6-8: bare 32x32->64 products (mul.wide, no addend) whose halves
// are summed by explicit add-with-carry chains.  On sm_103a a wide multiply
// with a 64-bit addend occupies the integer-multiply pipe ~1.4x longer than a
// bare one, while carry-chain adds can issue on the ALU pipe; splitting the
// two moves work off the multiply pipe, which bounds every other variant.
// ---------------------------------------------------------------------------
// t[0..9] += ai * b (one CIOS row, product part) with bare wide products
PP_HD void row_ab_wide(uint32_t t[10], uint32_t ai, const uint32_t b[8]) {
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint64_t p = (uint64_t)ai * b[j];
    lo[j] = (uint32_t)p;
    hi[j] = (uint32_t)(p >> 32);
  }
  t[0] = add_cc(t[0], lo[0]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j] = addc_cc(t[j], lo[j]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(t[9], 0);
  t[1] = add_cc(t[1], hi[0]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j + 1] = addc_cc(t[j + 1], hi[j]);
  t[9] = addc(t[9], 0);
}

// same product part with lo/hi multiply-add carry chains (as variant 0)
PP_HD void row_ab_madc(uint32_t t[10], uint32_t ai, const uint32_t b[8]) {
  t[0] = madlo_cc(ai, b[0], t[0]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j] = madloc_cc(ai, b[j], t[j]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(t[9], 0);
  t[1] = madhi_cc(ai, b[0], t[1]);
#pragma unroll
  for (int j = 1; j < 8; ++j) t[j + 1] = madhic_cc(ai, b[j], t[j + 1]);
  t[9] = addc(t[9], 0);
}

// reduction part of a CIOS row (m = -t0, r[0] = 1, r[1] = 2^32 - 1), then the
// one-word shift; bare wide products for m * r[2..7]
PP_HD void row_red_wide(uint32_t t[10]) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  const uint32_t t0 = t[0];
  const uint32_t m = 0u - t0;
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int j = 2; j < 8; ++j) {
    const uint64_t p = (uint64_t)m * r[j];
    lo[j] = (uint32_t)p;
    hi[j] = (uint32_t)(p >> 32);
  }
  (void)sub_cc(0, m);
  const uint32_t h1 = subc(m, 0);  // hi(m * (2^32 - 1)) = m - (m != 0)
  (void)add_cc(t0, 0xffffffffu);   // carry out of t0 + m
  t[1] = addc_cc(t[1], t0);        // lo(m * (2^32 - 1)) = -m = t0
#pragma unroll
  for (int j = 2; j < 8; ++j) t[j] = addc_cc(t[j], lo[j]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(t[9], 0);
  t[2] = add_cc(t[2], h1);
#pragma unroll
  for (int j = 2; j < 8; ++j) t[j + 1] = addc_cc(t[j + 1], hi[j]);
  t[9] = addc(t[9], 0);
#pragma unroll
  for (int k = 0; k < 9; ++k) t[k] = t[k + 1];
  t[9] = 0;
}

// the same reduction part with multiply-add carry chains
PP_HD void row_red_madc(uint32_t t[10]) {
  const uint32_t t0 = t[0];
  const uint32_t m = 0u - t0;
  (void)sub_cc(0, m);
  const uint32_t h1 = subc(m, 0);
  (void)add_cc(t0, 0xffffffffu);
  t[1] = addc_cc(t[1], t0);
  t[2] = madloc_cc(m, PP_R2, t[2]);
  t[3] = madloc_cc(m, PP_R3, t[3]);
  t[4] = madloc_cc(m, PP_R4, t[4]);
  t[5] = madloc_cc(m, PP_R5, t[5]);
  t[6] = madloc_cc(m, PP_R6, t[6]);
  t[7] = madloc_cc(m, PP_R7, t[7]);
  t[8] = addc_cc(t[8], 0);
  t[9] = addc(t[9], 0);
  t[2] = add_cc(t[2], h1);
  t[3] = madhic_cc(m, PP_R2, t[3]);
  t[4] = madhic_cc(m, PP_R3, t[4]);
  t[5] = madhic_cc(m, PP_R4, t[5]);
  t[6] = madhic_cc(m, PP_R5, t[6]);
  t[7] = madhic_cc(m, PP_R6, t[7]);
  t[8] = madhic_cc(m, PP_R7, t[8]);
  t[9] = addc(t[9], 0);
#pragma unroll
  for (int k = 0; k < 9; ++k) t[k] = t[k + 1];
  t[9] = 0;
}

// AB: 0 = multiply-add chains, 1 = bare wide products; RED likewise
template <int AB, int RED>
PP_HD fr fr_mul_split(const fr &a, const fr &b) {
  uint32_t t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (AB) row_ab_wide(t, a.v[i], b.v);
    else row_ab_madc(t, a.v[i], b.v);
    if (RED) row_red_wide(t);
    else row_red_madc(t);
  }
  fr_reduce_once(t);
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[i];
  return out;
}

// ---------------------------------------------------------------------------
// Variant 9: each row's products absorb only the row's own 32-bit word,
//   s_j = a_i * b_j + t_j   (< 2^64, independent across j),
// and one add-with-carry chain joins lo(s_j) with hi(s_{j-1}).  The products
// of a row carry no dependency on each other, and the only addend a wide
// multiply sees is a zero-extended 32-bit word.
// ---------------------------------------------------------------------------
PP_HD void row9_ab(uint32_t t[10], uint32_t ai, const uint32_t b[8]) {
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint64_t s = (uint64_t)ai * b[j] + t[j];
    lo[j] = (uint32_t)s;
    hi[j] = (uint32_t)(s >> 32);
  }
  t[0] = lo[0];
  t[1] = add_cc(lo[1], hi[0]);
#pragma unroll
  for (int j = 2; j < 8; ++j) t[j] = addc_cc(lo[j], hi[j - 1]);
  t[8] = addc_cc(t[8], hi[7]);
  t[9] = addc(t[9], 0);
}

PP_HD void row9_red(uint32_t t[10]) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  const uint32_t t0 = t[0];
  const uint32_t m = 0u - t0;
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int j = 2; j < 8; ++j) {
    const uint64_t s = (uint64_t)m * r[j] + t[j];
    lo[j] = (uint32_t)s;
    hi[j] = (uint32_t)(s >> 32);
  }
  (void)sub_cc(0, m);
  const uint32_t h1 = subc(m, 0);      // hi(m * (2^32 - 1))
  (void)add_cc(t0, 0xffffffffu);       // carry out of word 0 (t0 + m)
  const uint32_t u1 = addc_cc(t[1], t0);  // + lo(m * (2^32 - 1)) = t0
  const uint32_t u2 = addc_cc(lo[2], h1);
  const uint32_t u3 = addc_cc(lo[3], hi[2]);
  const uint32_t u4 = addc_cc(lo[4], hi[3]);
  const uint32_t u5 = addc_cc(lo[5], hi[4]);
  const uint32_t u6 = addc_cc(lo[6], hi[5]);
  const uint32_t u7 = addc_cc(lo[7], hi[6]);
  const uint32_t u8 = addc_cc(t[8], hi[7]);
  const uint32_t u9 = addc(t[9], 0);
  t[0] = u1;
  t[1] = u2;
  t[2] = u3;
  t[3] = u4;
  t[4] = u5;
  t[5] = u6;
  t[6] = u7;
  t[7] = u8;
  t[8] = u9;
  t[9] = 0;
}

// LAZY: skip the final subtraction.  For b < r and any 256-bit a the result
// is < 2r: every row keeps t < b + r, and at the end
// t = (a b + m r) / R < (R r + R r) / R = 2r.
template <bool LAZY = false>
PP_HD fr fr_mul_row9(const fr &a, const fr &b) {
  uint32_t t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    row9_ab(t, a.v[i], b.v);
    row9_red(t);
  }
  if (!LAZY) fr_reduce_once(t);
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[i];
  return out;
}

// ---------------------------------------------------------------------------
// Variants 11-13: variant 9's rows for part of the multiply and bare wide
// products with two add chains for the rest.  A wide multiply with an addend
// holds the integer-multiply pipe ~1.4x longer than a bare one, and the second
// add chain runs on the ALU pipe, so the mix trades multiply-pipe cycles for
// ALU cycles.  AB / RED choose the rows: 0 = variant 9, 1 = bare products,
// 2 = bare on odd rows only.  Both row forms keep the same t[0..10) invariant.
// ---------------------------------------------------------------------------
template <int AB, int RED>
PP_HD fr fr_mul_mix(const fr &a, const fr &b) {
  uint32_t t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (AB == 1 || (AB == 2 && (i & 1))) row_ab_wide(t, a.v[i], b.v);
    else row9_ab(t, a.v[i], b.v);
    if (RED == 1 || (RED == 2 && (i & 1))) row_red_wide(t);
    else row9_red(t);
  }
  fr_reduce_once(t);
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[i];
  return out;
}

// ---------------------------------------------------------------------------
// Variant 10: variant 9's row structure inside a one-level Karatsuba product
// (3 products of 4x4 limbs = 48 wide products instead of 64) followed by a
// word-serial reduction of the 512-bit product with the same row structure.
// ---------------------------------------------------------------------------
// r[0..8) = a[0..4) * b[0..4), rows of independent products + one chain
PP_HD void mul4_rows(uint32_t r[8], const uint32_t a[4], const uint32_t b[4]) {
#pragma unroll
  for (int k = 0; k < 8; ++k) r[k] = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t lo[4], hi[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint64_t s = (uint64_t)a[i] * b[j] + r[i + j];
      lo[j] = (uint32_t)s;
      hi[j] = (uint32_t)(s >> 32);
    }
    r[i] = lo[0];
    r[i + 1] = add_cc(lo[1], hi[0]);
    r[i + 2] = addc_cc(lo[2], hi[1]);
    r[i + 3] = addc_cc(lo[3], hi[2]);
    r[i + 4] = addc(hi[3], 0);
  }
}

PP_HD void mul8_kara_rows(uint32_t r[16], const uint32_t a[8], const uint32_t b[8]) {
  uint32_t sa[4], sb[4];
  sa[0] = add_cc(a[0], a[4]);
  sa[1] = addc_cc(a[1], a[5]);
  sa[2] = addc_cc(a[2], a[6]);
  sa[3] = addc_cc(a[3], a[7]);
  const uint32_t ca = addc(0, 0);
  sb[0] = add_cc(b[0], b[4]);
  sb[1] = addc_cc(b[1], b[5]);
  sb[2] = addc_cc(b[2], b[6]);
  sb[3] = addc_cc(b[3], b[7]);
  const uint32_t cb = addc(0, 0);
  uint32_t z0[8], z2[8], z1[8];
  mul4_rows(z0, a, b);
  mul4_rows(z2, a + 4, b + 4);
  mul4_rows(z1, sa, sb);
  // z1 += (ca * sb + cb * sa) << 128, top word z1t
  const uint32_t ma = 0u - ca, mb = 0u - cb;
  z1[4] = add_cc(z1[4], sb[0] & ma);
  z1[5] = addc_cc(z1[5], sb[1] & ma);
  z1[6] = addc_cc(z1[6], sb[2] & ma);
  z1[7] = addc_cc(z1[7], sb[3] & ma);
  uint32_t z1t = addc(ca & cb, 0);
  z1[4] = add_cc(z1[4], sa[0] & mb);
  z1[5] = addc_cc(z1[5], sa[1] & mb);
  z1[6] = addc_cc(z1[6], sa[2] & mb);
  z1[7] = addc_cc(z1[7], sa[3] & mb);
  z1t = addc(z1t, 0);
  // z1 -= z0 + z2 (non-negative middle term a0*b1 + a1*b0)
  z1[0] = sub_cc(z1[0], z0[0]);
#pragma unroll
  for (int i = 1; i < 8; ++i) z1[i] = subc_cc(z1[i], z0[i]);
  z1t = subc(z1t, 0);
  z1[0] = sub_cc(z1[0], z2[0]);
#pragma unroll
  for (int i = 1; i < 8; ++i) z1[i] = subc_cc(z1[i], z2[i]);
  z1t = subc(z1t, 0);
  // r = z0 + z1 << 128 + z2 << 256
#pragma unroll
  for (int i = 0; i < 4; ++i) r[i] = z0[i];
  r[4] = add_cc(z0[4], z1[0]);
  r[5] = addc_cc(z0[5], z1[1]);
  r[6] = addc_cc(z0[6], z1[2]);
  r[7] = addc_cc(z0[7], z1[3]);
  r[8] = addc_cc(z2[0], z1[4]);
  r[9] = addc_cc(z2[1], z1[5]);
  r[10] = addc_cc(z2[2], z1[6]);
  r[11] = addc_cc(z2[3], z1[7]);
  r[12] = addc_cc(z2[4], z1t);
  r[13] = addc_cc(z2[5], 0);
  r[14] = addc_cc(z2[6], 0);
  r[15] = addc(z2[7], 0);
}

// word-serial Montgomery reduction of t[0..16) with variant 9's rows; the
// carry out of round i's top word (i + 8) is added at round i+1's top word
template <bool LAZY = false>
PP_HD fr mont_redc16_rows(uint32_t t[16]) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  uint32_t hc = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t t0 = t[i];
    const uint32_t m = 0u - t0;
    uint32_t lo[8], hi[8];
#pragma unroll
    for (int j = 2; j < 8; ++j) {
      const uint64_t s = (uint64_t)m * r[j] + t[i + j];
      lo[j] = (uint32_t)s;
      hi[j] = (uint32_t)(s >> 32);
    }
    (void)sub_cc(0, m);
    const uint32_t h1 = subc(m, 0);
    (void)add_cc(t0, 0xffffffffu);
    t[i + 1] = addc_cc(t[i + 1], t0);
    t[i + 2] = addc_cc(lo[2], h1);
#pragma unroll
    for (int j = 3; j < 8; ++j) t[i + j] = addc_cc(lo[j], hi[j - 1]);
    t[i + 8] = addc_cc(t[i + 8], hi[7]);
    const uint32_t c1 = addc(0, 0);
    t[i + 8] = add_cc(t[i + 8], hc);
    hc = addc(c1, 0);
  }
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = t[8 + i];
  if (!LAZY) fr_reduce_once(out.v);
  return out;
}

PP_HD fr fr_mul_kara_rows(const fr &a, const fr &b) {
  uint32_t t[16];
  mul8_kara_rows(t, a.v, b.v);
  return mont_redc16_rows(t);
}

// variant 5: schoolbook product + the same reduction (separated operand scanning)
PP_HD fr fr_mul_sos(const fr &a, const fr &b) {
  uint32_t t[16];
  mul_school<8>(t, a.v, b.v);
  return mont_redc16(t);
}

PP_HD fr fr_mul(const fr &a, const fr &b) {
#if PP_MUL_VARIANT == 2
  return fr_mul_w(a, b);
#elif PP_MUL_VARIANT == 3
  return fr_mul_kara<false>(a, b);
#elif PP_MUL_VARIANT == 4
  return fr_mul_kara<true>(a, b);
#elif PP_MUL_VARIANT == 5
  return fr_mul_sos(a, b);
#elif PP_MUL_VARIANT == 6
  return fr_mul_split<1, 1>(a, b);
#elif PP_MUL_VARIANT == 7
  return fr_mul_split<1, 0>(a, b);
#elif PP_MUL_VARIANT == 8
  return fr_mul_split<0, 1>(a, b);
#elif PP_MUL_VARIANT == 9
  return fr_mul_row9(a, b);
#elif PP_MUL_VARIANT == 10
  return fr_mul_kara_rows(a, b);
#elif PP_MUL_VARIANT == 11
  return fr_mul_mix<0, 1>(a, b);
#elif PP_MUL_VARIANT == 12
  return fr_mul_mix<1, 0>(a, b);
#elif PP_MUL_VARIANT == 13
  return fr_mul_mix<0, 2>(a, b);
#else
  return fr_mul_v<PP_MUL_VARIANT>(a, b);
#endif
}

// r[0..16) = a^2 for a < 2^255: the 28 cross products a_i a_j (i < j) in rows
// of independent products (row i: a_i times a_(i+1..7), each row's top word
// new), doubled, plus the 8 squares a_i^2 in one add-with-carry chain: 36 wide
// products where a general product needs 64.
PP_HD void sqr8_rows(uint32_t r[16], const uint32_t a[8]) {
#pragma unroll
  for (int k = 0; k < 16; ++k) r[k] = 0;
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    const int n = 7 - i;  // partners a[i + 1 .. 7] at words 2i + 1 .. i + 7
    uint32_t lo[7], hi[7];
#pragma unroll
    for (int j = 0; j < n; ++j) {
      const uint64_t s = (uint64_t)a[i] * a[i + 1 + j] + r[2 * i + 1 + j];
      lo[j] = (uint32_t)s;
      hi[j] = (uint32_t)(s >> 32);
    }
    r[2 * i + 1] = lo[0];
    if (n == 1) {
      r[2 * i + 2] = hi[0];
    } else {
      r[2 * i + 2] = add_cc(lo[1], hi[0]);
#pragma unroll
      for (int j = 2; j < n; ++j) r[2 * i + 1 + j] = addc_cc(lo[j], hi[j - 1]);
      r[i + 8] = addc(hi[n - 1], 0);
    }
  }
  // 2 x (the cross products) < a^2 < 2^510: the shift loses no bit
#pragma unroll
  for (int k = 15; k > 0; --k) r[k] = (r[k] << 1) | (r[k - 1] >> 31);
  r[0] <<= 1;
  uint32_t sl[8], sh[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint64_t s = (uint64_t)a[i] * a[i];
    sl[i] = (uint32_t)s;
    sh[i] = (uint32_t)(s >> 32);
  }
  r[0] = add_cc(r[0], sl[0]);
  r[1] = addc_cc(r[1], sh[0]);
#pragma unroll
  for (int i = 1; i < 7; ++i) {
    r[2 * i] = addc_cc(r[2 * i], sl[i]);
    r[2 * i + 1] = addc_cc(r[2 * i + 1], sh[i]);
  }
  r[14] = addc_cc(r[14], sl[7]);
  r[15] = addc(r[15], sh[7]);
}

// a^2 for canonical a (a^2 < r 2^256, as the reduction needs): the square's
// 36 wide products, then the row-form Montgomery reduction (48)
PP_HD fr fr_sqr(const fr &a) {
  uint32_t t[16];
  sqr8_rows(t, a.v);
  return mont_redc16_rows(t);
}

// ---- lazy arithmetic on [0, 2r) for the NTT's inner rounds: values stay
// below 2r and are made canonical once, when the transform stores its
// result.  fr_mul_lazy takes a < 2r and b < r (the twiddle) and returns a
// value < 2r.
PP_HD fr fr_mul_lazy(const fr &a, const fr &b) {
#if PP_MUL_VARIANT == 9
  return fr_mul_row9<true>(a, b);
#else
  fr c = a;
  fr_reduce_once(c.v);
  return fr_mul(c, b);
#endif
}

// The transform's twiddle multiply: a < 2r, b < r (a twiddle), result < 2r.
// PP_NTT_MUL selects its formulation (9: fr_mul_lazy's rows; 10: one
// Karatsuba level for the product, 48 wide products instead of 64, then the
// same row-wise reduction without the final subtraction: for a < 2r, b < r
// the reduced value (a b + m r) / R < (2 r^2 + R r) / R < 2r).
#ifndef PP_NTT_MUL
#define PP_NTT_MUL 9
#endif
PP_HD fr fr_mul_twiddle(const fr &a, const fr &b) {
#if PP_NTT_MUL == 10
  uint32_t t[16];
  mul8_kara_rows(t, a.v, b.v);
  return mont_redc16_rows<true>(t);
#else
  return fr_mul_lazy(a, b);
#endif
}

// 2r, least significant limb first
#define PP_2R0 0x00000002u
#define PP_2R1 0xfffffffeu
#define PP_2R2 0xfffcb7fdu
#define PP_2R3 0xa77b4805u
#define PP_2R4 0x1343b00au
#define PP_2R5 0x6673b010u
#define PP_2R6 0x533afa90u
#define PP_2R7 0xe7db4ea6u

// a + b mod 2r for a, b < 2r: a + b < 4r may carry out of 256 bits
PP_HD fr fr_add_lazy(const fr &a, const fr &b) {
  uint32_t s[8], d[8];
  s[0] = add_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int i = 1; i < 8; ++i) s[i] = addc_cc(a.v[i], b.v[i]);
  const uint32_t carry = addc(0, 0);
  d[0] = sub_cc(s[0], PP_2R0);
  d[1] = subc_cc(s[1], PP_2R1);
  d[2] = subc_cc(s[2], PP_2R2);
  d[3] = subc_cc(s[3], PP_2R3);
  d[4] = subc_cc(s[4], PP_2R4);
  d[5] = subc_cc(s[5], PP_2R5);
  d[6] = subc_cc(s[6], PP_2R6);
  d[7] = subc_cc(s[7], PP_2R7);
  const uint32_t borrow = subc(0, 0);        // all ones when s < 2r (as 256 bits)
  const uint32_t keep = borrow & (carry - 1u);  // ... and there was no carry
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = keep ? s[i] : d[i];
  return r;
}

// a - b mod 2r for a, b < 2r
PP_HD fr fr_sub_lazy(const fr &a, const fr &b) {
  fr d;
  d.v[0] = sub_cc(a.v[0], b.v[0]);
#pragma unroll
  for (int i = 1; i < 8; ++i) d.v[i] = subc_cc(a.v[i], b.v[i]);
  const uint32_t mask = subc(0, 0);  // all ones on borrow
  d.v[0] = add_cc(d.v[0], PP_2R0 & mask);
  d.v[1] = addc_cc(d.v[1], PP_2R1 & mask);
  d.v[2] = addc_cc(d.v[2], PP_2R2 & mask);
  d.v[3] = addc_cc(d.v[3], PP_2R3 & mask);
  d.v[4] = addc_cc(d.v[4], PP_2R4 & mask);
  d.v[5] = addc_cc(d.v[5], PP_2R5 & mask);
  d.v[6] = addc_cc(d.v[6], PP_2R6 & mask);
  d.v[7] = addc(d.v[7], PP_2R7 & mask);
  return d;
}

// canonical form of a value < 2r
PP_HD fr fr_canon(const fr &a) {
  fr r = a;
  fr_reduce_once(r.v);
  return r;
}

// ---------------------------------------------------------------------------
// Dot products with one reduction per group of terms (Horner's chunks).  A
// sum of G products of canonical values is below G r^2, so it is accumulated
// in 17 words without reducing each product, and one Montgomery reduction of
// the 17-word sum (below G r / 2 + r after it) plus a few conditional
// subtractions gives the canonical result: 64 wide products per term and one
// reduction per group, where a multiply per term costs 112.
// ---------------------------------------------------------------------------
// r[0..16) = a * b, rows of independent products + one add chain per row
PP_HD void mul8_rows(uint32_t r[16], const uint32_t a[8], const uint32_t b[8]) {
#pragma unroll
  for (int k = 0; k < 16; ++k) r[k] = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uint32_t lo[8], hi[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint64_t s = (uint64_t)a[i] * b[j] + r[i + j];
      lo[j] = (uint32_t)s;
      hi[j] = (uint32_t)(s >> 32);
    }
    r[i] = lo[0];
    r[i + 1] = add_cc(lo[1], hi[0]);
#pragma unroll
    for (int j = 2; j < 8; ++j) r[i + j] = addc_cc(lo[j], hi[j - 1]);
    r[i + 8] = addc(hi[7], 0);
  }
}

// acc[0..17) += a * b
PP_HD void fr_mac17(uint32_t acc[17], const fr &a, const fr &b) {
  uint32_t p[16];
  mul8_rows(p, a.v, b.v);
  acc[0] = add_cc(acc[0], p[0]);
#pragma unroll
  for (int k = 1; k < 16; ++k) acc[k] = addc_cc(acc[k], p[k]);
  acc[16] = addc(acc[16], 0);
}

// x - k r if x >= k r (x: 9 words)
PP_HD void sub_if_ge9(uint32_t x[9], const uint32_t kr[9]) {
  uint32_t t[9];
  t[0] = sub_cc(x[0], kr[0]);
#pragma unroll
  for (int i = 1; i < 9; ++i) t[i] = subc_cc(x[i], kr[i]);
  const uint32_t borrow = subc(0, 0);  // 0xffffffff if x < k r
#pragma unroll
  for (int i = 0; i < 9; ++i) x[i] = borrow ? x[i] : t[i];
}

// acc * 2^-256 mod r, canonical, for acc < 2^543 whose reduction is below
// 16 r (a sum of at most 16 products of canonical values: acc < 16 r^2, so
// the reduced value is below 16 r^2 / 2^256 + r < 8.3 r)
PP_HD fr fr_redc17(uint32_t t[17]) {
  const uint32_t r[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  uint32_t hc = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    // round i: t += m r 2^(32 i) with m = -t[i] (r = 1 mod 2^32), as
    // mont_redc16_rows; the carry out of word i + 8 rides into round i + 1
    const uint32_t t0 = t[i];
    const uint32_t m = 0u - t0;
    uint32_t lo[8], hi[8];
#pragma unroll
    for (int j = 2; j < 8; ++j) {
      const uint64_t s = (uint64_t)m * r[j] + t[i + j];
      lo[j] = (uint32_t)s;
      hi[j] = (uint32_t)(s >> 32);
    }
    (void)sub_cc(0, m);
    const uint32_t h1 = subc(m, 0);
    (void)add_cc(t0, 0xffffffffu);
    t[i + 1] = addc_cc(t[i + 1], t0);
    t[i + 2] = addc_cc(lo[2], h1);
#pragma unroll
    for (int j = 3; j < 8; ++j) t[i + j] = addc_cc(lo[j], hi[j - 1]);
    t[i + 8] = addc_cc(t[i + 8], hi[7]);
    const uint32_t c1 = addc(0, 0);
    t[i + 8] = add_cc(t[i + 8], hc);
    hc = addc(c1, 0);
  }
  t[16] += hc;  // the value t[8..17) is below 2^260: no carry leaves word 16
  uint32_t x[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) x[i] = t[8 + i];
  // k r for k = 8, 4, 2, 1
  uint32_t kr[9];
#pragma unroll
  for (int sh = 3; sh >= 0; --sh) {
    uint64_t c = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      c += (uint64_t)r[i] << sh;
      kr[i] = (uint32_t)c;
      c >>= 32;
    }
    kr[8] = (uint32_t)c;
    sub_if_ge9(x, kr);
  }
  fr out;
#pragma unroll
  for (int i = 0; i < 8; ++i) out.v[i] = x[i];
  return out;
}

// a^e for a 64-bit exponent (square and multiply, most significant bit first)
PP_HD fr fr_pow_u64(const fr &a, uint64_t e) {
  fr acc = fr_one();
  bool started = false;
  for (int bit = 63; bit >= 0; --bit) {
    if (started) acc = fr_sqr(acc);
    if ((e >> bit) & 1) {
      acc = started ? fr_mul(acc, a) : a;
      started = true;
    }
  }
  return acc;
}

// a^(r-2) = a^-1 (0 -> 0), Fermat; e = r - 2 as 32-bit limbs, least significant first
PP_HD fr fr_inv(const fr &a) {
  const uint32_t e[8] = {0xffffffffu, 0xfffffffeu, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  fr acc = fr_one();
  // 4-bit fixed window
  fr tab[16];
  tab[0] = fr_one();
  tab[1] = a;
  for (int i = 2; i < 16; ++i) tab[i] = fr_mul(tab[i - 1], a);
  for (int w = 7; w >= 0; --w) {
    for (int nib = 7; nib >= 0; --nib) {
      if (!(w == 7 && nib == 7)) {
        acc = fr_sqr(acc);
        acc = fr_sqr(acc);
        acc = fr_sqr(acc);
        acc = fr_sqr(acc);
      }
      const uint32_t d = (e[w] >> (4 * nib)) & 15u;
      acc = fr_mul(acc, tab[d]);
    }
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Inverse by the binary extended Euclidean algorithm (Knuth TAOCP vol. 2,
// 4.5.2; Menezes et al., Handbook of Applied Cryptography, Alg. 14.61 for an
// odd modulus): a few hundred shift / subtract steps on 8-limb words instead
// of the ~320 dependent Montgomery multiplies of a Fermat exponentiation.
// Variable time (fine for public prover data).  Input and output are in
// Montgomery form: the plain inverse y of the representative a*R is
// R^-1 a^-1, so the result is y * R^3 * R^-1 = (a^-1) R.  0 maps to 0.
// ---------------------------------------------------------------------------
PP_HD bool lt_words(const uint32_t a[8], const uint32_t b[8]) {
  for (int i = 7; i >= 0; --i)
    if (a[i] != b[i]) return a[i] < b[i];
  return false;
}
PP_HD bool is_one_words(const uint32_t a[8]) {
  return a[0] == 1 && (a[1] | a[2] | a[3] | a[4] | a[5] | a[6] | a[7]) == 0;
}
// x = x / 2 (mod r) for x < r
PP_HD void half_mod(uint32_t x[8]) {
  const uint32_t odd = 0u - (x[0] & 1u);
  uint32_t c;
  x[0] = add_cc(x[0], PP_R0 & odd);
  x[1] = addc_cc(x[1], PP_R1 & odd);
  x[2] = addc_cc(x[2], PP_R2 & odd);
  x[3] = addc_cc(x[3], PP_R3 & odd);
  x[4] = addc_cc(x[4], PP_R4 & odd);
  x[5] = addc_cc(x[5], PP_R5 & odd);
  x[6] = addc_cc(x[6], PP_R6 & odd);
  x[7] = addc_cc(x[7], PP_R7 & odd);
  c = addc(0, 0);
#pragma unroll
  for (int i = 0; i < 7; ++i) x[i] = (x[i] >> 1) | (x[i + 1] << 31);
  x[7] = (x[7] >> 1) | (c << 31);
}
PP_HD void shr1_words(uint32_t x[8]) {
#pragma unroll
  for (int i = 0; i < 7; ++i) x[i] = (x[i] >> 1) | (x[i + 1] << 31);
  x[7] >>= 1;
}
PP_HD void sub_words(uint32_t a[8], const uint32_t b[8]) {
  a[0] = sub_cc(a[0], b[0]);
#pragma unroll
  for (int i = 1; i < 7; ++i) a[i] = subc_cc(a[i], b[i]);
  a[7] = subc(a[7], b[7]);
}

PP_HD fr fr_inv_binary(const fr &a) {
  if (fr_is_zero(a)) return fr_zero();
  uint32_t u[8], v[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};
  fr x1 = fr_zero(), x2 = fr_zero();
  x1.v[0] = 1;
#pragma unroll
  for (int i = 0; i < 8; ++i) u[i] = a.v[i];
  // at most ~2 * 256 halvings and 256 subtractions for canonical input; the
  // bounds only guard against non-canonical input (u or v reaching 0)
  for (int guard = 0; guard < 1024 && !is_one_words(u) && !is_one_words(v); ++guard) {
    for (int k = 0; k < 256 && !(u[0] & 1u); ++k) {
      shr1_words(u);
      half_mod(x1.v);
    }
    for (int k = 0; k < 256 && !(v[0] & 1u); ++k) {
      shr1_words(v);
      half_mod(x2.v);
    }
    if (!lt_words(u, v)) {
      sub_words(u, v);
      x1 = fr_sub(x1, x2);
    } else {
      sub_words(v, u);
      x2 = fr_sub(x2, x1);
    }
  }
  const fr y = is_one_words(u) ? x1 : x2;
  // R^3 mod r
  const fr r3 = {{0x439b73afu, 0xc62c1807u, 0x8cf06990u, 0x1b3e0d18u,
                  0xc7b5f418u, 0x73d13c71u, 0xc8db33e9u, 0x6e2a5bb9u}};
  return fr_mul(y, r3);
}

}  // namespace pp

#include "modinv.cuh"

namespace pp {

// r in B-bit limbs and r^-1 mod 2^B
template <typename L>
PP_HD ModulusB<L, (255 + LimbTraits<L>::B) / LimbTraits<L>::B> fr_modulus_limbs();
template <>
PP_HD ModulusB<int32_t, 9> fr_modulus_limbs<int32_t>() {
  return {{0x00000001, 0x3ffffffc, 0x3fe5bfef, 0x2f6900bf, 0x21d80553, 0x27602026, 0x17d48333,
           0x29d4ca67, 0x000073ed},
          0x00000001u};
}
template <>
PP_HD ModulusB<int64_t, 5> fr_modulus_limbs<int64_t>() {
  return {{0x3fffffff00000001ll, 0x0ef6900bfff96ffbll, 0x339d80809a1d8055ll,
           0x3b69d4ca675f520cll, 0x0000000000000073ll},
          0x0000000100000001ull};
}

// a^-1 in Montgomery form (0 -> 0) by divsteps (modinv.cuh) on B-bit limbs:
// 25 batches of 30 steps (or 12 of 62) at most, instead of the binary GCD's
// ~770 steps on 8-word numbers.  As for fr_inv_binary, the plain inverse of
// the word value a R is R^-1 a^-1, and a multiply by R^3 gives a^-1 R.
template <typename L>
PP_HD fr fr_inv_divsteps(const fr &a) {
  constexpr int B = LimbTraits<L>::B, NL = (255 + B) / B;
  if (fr_is_zero(a)) return fr_zero();
  const ModulusB<L, NL> M = fr_modulus_limbs<L>();
  const SLimbs<L, NL> y =
      modinv_divsteps<L, NL>(words_to_limbs<L, 8, NL>(a.v), M, (741 + B - 1) / B);
  fr out;
  limbs_to_words<L, 8, NL>(y, out.v);
  const fr r3 = {{0x439b73afu, 0xc62c1807u, 0x8cf06990u, 0x1b3e0d18u,
                  0xc7b5f418u, 0x73d13c71u, 0xc8db33e9u, 0x6e2a5bb9u}};
  return fr_mul(out, r3);
}

// 30-bit limbs on the GPU, 62-bit ones on a 64-bit host
PP_HD fr fr_inv_fast(const fr &a) {
#ifdef __CUDA_ARCH__
  return fr_inv_divsteps<int32_t>(a);
#else
  return fr_inv_divsteps<int64_t>(a);
#endif
}

}  // namespace pp
