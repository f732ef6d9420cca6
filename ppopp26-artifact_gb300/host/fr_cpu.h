// fr_cpu.h -- the reference's host-side Fr element type, cpu::BLS12_381_Fr_G1
// (PLONK/utils/mont/cpu/ff/bls12-381.hpp:28-32 over blst_256_t,
// PLONK/blst/include/blst_t.hpp:307-470), with the operators the reference's
// host code applies to it: miss_ops.cu:34-87 (naive_gp's `*=`, naive_div's
// `1/x`, `*`, `-=`, `is_zero()`), and the rest of blst_256_t's arithmetic
// surface (`+`, `-`, unary `-`, `^`, `/`, `==`, `one()`, `to()`, `from()`).
//
// Layout: 4 little-endian 64-bit limbs in Montgomery form (R = 2^256), 32 bytes,
// the same bytes the GPU operators read and write.  Values are kept canonical
// (< r), as blst keeps them.
//
// The arithmetic is portable C++ (no assembly, unsigned __int128 products;
// gcc and clang on x86-64 and AArch64): a word-serial Montgomery product
// (CIOS, Koc-Acar-Kaliski 1996) with n0' = -r^-1 mod 2^64 = 0xfffffffeffffffff,
// and inversion by Fermat's little theorem (x^(r-2); the inverse of 0 is 0, as
// blst's constant-time inversion gives).  It is host code for callers'
// bookkeeping, not a hot path: the GPU operators never use it.
#pragma once
#include <cstddef>
#include <cstdint>
#include <ostream>

namespace cpu {

class BLS12_381_Fr_G1 {
  uint64_t val[4];

  using u128 = unsigned __int128;
  static constexpr uint64_t kMod[4] = {0xffffffff00000001ull, 0x53bda402fffe5bfeull,
                                       0x3339d80809a1d805ull, 0x73eda753299d7d48ull};
  static constexpr uint64_t kOne[4] = {0x00000001fffffffeull, 0x5884b7fa00034802ull,
                                       0x998c4fefecbc4ff5ull, 0x1824b159acc5056full};
  static constexpr uint64_t kRR[4] = {0xc999e990f3f29c6dull, 0x2b6cedcb87925c23ull,
                                      0x05d314967254398full, 0x0748d9d99f59ff11ull};
  static constexpr uint64_t kN0 = 0xfffffffeffffffffull;

  // t (5 words, t < 2r) -> t mod r
  static void reduce_once(uint64_t out[4], const uint64_t t[4], uint64_t hi) {
    uint64_t d[4];
    uint64_t borrow = 0;
    for (int i = 0; i < 4; ++i) {
      u128 x = (u128)t[i] - kMod[i] - borrow;
      d[i] = (uint64_t)x;
      borrow = (uint64_t)(x >> 64) & 1;
    }
    const bool keep_t = hi == 0 && borrow;  // t < r
    for (int i = 0; i < 4; ++i) out[i] = keep_t ? t[i] : d[i];
  }

  static void mont_mul(uint64_t out[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
      uint64_t carry = 0;
      for (int j = 0; j < 4; ++j) {
        u128 s = (u128)a[j] * b[i] + t[j] + carry;
        t[j] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
      }
      u128 s = (u128)t[4] + carry;
      t[4] = (uint64_t)s;
      t[5] = (uint64_t)(s >> 64);
      const uint64_t m = t[0] * kN0;
      s = (u128)m * kMod[0] + t[0];
      carry = (uint64_t)(s >> 64);
      for (int j = 1; j < 4; ++j) {
        s = (u128)m * kMod[j] + t[j] + carry;
        t[j - 1] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
      }
      s = (u128)t[4] + carry;
      t[3] = (uint64_t)s;
      t[4] = t[5] + (uint64_t)(s >> 64);
    }
    reduce_once(out, t, t[4]);
  }

  static void add_mod(uint64_t out[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[4];
    uint64_t carry = 0;
    for (int i = 0; i < 4; ++i) {
      u128 s = (u128)a[i] + b[i] + carry;
      t[i] = (uint64_t)s;
      carry = (uint64_t)(s >> 64);
    }
    reduce_once(out, t, carry);
  }

  static void sub_mod(uint64_t out[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[4];
    uint64_t borrow = 0;
    for (int i = 0; i < 4; ++i) {
      u128 x = (u128)a[i] - b[i] - borrow;
      t[i] = (uint64_t)x;
      borrow = (uint64_t)(x >> 64) & 1;
    }
    uint64_t carry = 0;
    for (int i = 0; i < 4; ++i) {  // add r back when a < b
      u128 s = (u128)t[i] + (borrow ? kMod[i] : 0) + carry;
      out[i] = (uint64_t)s;
      carry = (uint64_t)(s >> 64);
    }
  }

 public:
  using mem_t = BLS12_381_Fr_G1;
  static const size_t n = 4;
  static const size_t nbits = 255;
  static constexpr size_t bit_length() { return 255; }

  BLS12_381_Fr_G1() = default;
  // the Montgomery form of the integer a (blst_t.hpp:333-338)
  BLS12_381_Fr_G1(uint64_t a) : val{a, 0, 0, 0} {
    if (a) to();
  }
  BLS12_381_Fr_G1(int a) : BLS12_381_Fr_G1((uint64_t)a) {}
  // raw Montgomery limbs
  explicit BLS12_381_Fr_G1(const uint64_t p[4]) : val{p[0], p[1], p[2], p[3]} {}

  operator const uint64_t *() const { return val; }
  operator uint64_t *() { return val; }
  uint64_t &operator[](size_t i) { return val[i]; }
  const uint64_t &operator[](size_t i) const { return val[i]; }

  static const BLS12_381_Fr_G1 &one() {
    static const BLS12_381_Fr_G1 o(kOne);
    return o;
  }
  // integer -> Montgomery form, in place
  BLS12_381_Fr_G1 &to() {
    mont_mul(val, val, kRR);
    return *this;
  }
  // Montgomery form -> integer, in place
  BLS12_381_Fr_G1 &from() {
    static const uint64_t unit[4] = {1, 0, 0, 0};
    mont_mul(val, val, unit);
    return *this;
  }
  void store(uint64_t *p) const {
    for (int i = 0; i < 4; ++i) p[i] = val[i];
  }

  int is_zero() const { return (val[0] | val[1] | val[2] | val[3]) == 0; }
  bool is_one() const { return *this == one(); }
  void zero() { val[0] = val[1] = val[2] = val[3] = 0; }

  BLS12_381_Fr_G1 &operator+=(const BLS12_381_Fr_G1 &b) {
    add_mod(val, val, b.val);
    return *this;
  }
  friend BLS12_381_Fr_G1 operator+(BLS12_381_Fr_G1 a, const BLS12_381_Fr_G1 &b) { return a += b; }
  BLS12_381_Fr_G1 &operator-=(const BLS12_381_Fr_G1 &b) {
    sub_mod(val, val, b.val);
    return *this;
  }
  friend BLS12_381_Fr_G1 operator-(BLS12_381_Fr_G1 a, const BLS12_381_Fr_G1 &b) { return a -= b; }
  friend BLS12_381_Fr_G1 operator-(const BLS12_381_Fr_G1 &a) {
    BLS12_381_Fr_G1 z;
    z.zero();
    return z -= a;
  }
  BLS12_381_Fr_G1 &operator*=(const BLS12_381_Fr_G1 &b) {
    mont_mul(val, val, b.val);
    return *this;
  }
  friend BLS12_381_Fr_G1 operator*(BLS12_381_Fr_G1 a, const BLS12_381_Fr_G1 &b) { return a *= b; }
  friend BLS12_381_Fr_G1 sqr(const BLS12_381_Fr_G1 &a) { return a * a; }

  // a^p by square-and-multiply; mind the ^ operator's precedence (as in blst_t.hpp)
  friend BLS12_381_Fr_G1 operator^(const BLS12_381_Fr_G1 &a, unsigned p) {
    BLS12_381_Fr_G1 acc = one(), base = a;
    for (; p; p >>= 1) {
      if (p & 1) acc *= base;
      base *= base;
    }
    return acc;
  }
  BLS12_381_Fr_G1 &operator^=(unsigned p) { return *this = *this ^ p; }
  BLS12_381_Fr_G1 operator()(unsigned p) const { return *this ^ p; }

  // multiplicative inverse, x^(r-2); the inverse of 0 is 0
  BLS12_381_Fr_G1 reciprocal() const {
    static const uint64_t e[4] = {kMod[0] - 2, kMod[1], kMod[2], kMod[3]};
    BLS12_381_Fr_G1 acc = one();
    for (int w = 3; w >= 0; --w)
      for (int b = 63; b >= 0; --b) {
        acc *= acc;
        if ((e[w] >> b) & 1) acc *= *this;
      }
    return acc;
  }
  // `1 / a` (blst_t.hpp: operator/(int one, a)); the numerator must be 1
  friend BLS12_381_Fr_G1 operator/(int one_, const BLS12_381_Fr_G1 &a) {
    BLS12_381_Fr_G1 r = a.reciprocal();
    if (one_ != 1) r *= BLS12_381_Fr_G1((uint64_t)one_);
    return r;
  }
  friend BLS12_381_Fr_G1 operator/(const BLS12_381_Fr_G1 &a, const BLS12_381_Fr_G1 &b) {
    return a * b.reciprocal();
  }
  BLS12_381_Fr_G1 &operator/=(const BLS12_381_Fr_G1 &b) { return *this = *this / b; }

  friend bool operator==(const BLS12_381_Fr_G1 &a, const BLS12_381_Fr_G1 &b) {
    return a.val[0] == b.val[0] && a.val[1] == b.val[1] && a.val[2] == b.val[2] &&
           a.val[3] == b.val[3];
  }
  friend bool operator!=(const BLS12_381_Fr_G1 &a, const BLS12_381_Fr_G1 &b) { return !(a == b); }

  friend std::ostream &operator<<(std::ostream &os, const BLS12_381_Fr_G1 &x) {
    static const char *hex = "0123456789abcdef";
    char buf[67];
    buf[0] = '0';
    buf[1] = 'x';
    for (int i = 0; i < 64; ++i) buf[2 + i] = hex[(x.val[3 - i / 16] >> (60 - 4 * (i % 16))) & 15];
    buf[66] = 0;
    return os << buf;
  }
};

static_assert(sizeof(BLS12_381_Fr_G1) == 32, "an Fr element is 32 bytes");

}  // namespace cpu
