// Host-side check of the device field code: compiles csrc/fr.cuh without a GPU
// (the PTX carry-chain primitives run as their exact host emulation) and
// compares every multiply variant, add, sub and inverse with the oracle.
// Built and run by tests/test_fr_host.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../ppopp26-artifact_gb300/csrc/fr.cuh"
extern "C" {
#include "../oracle/pp_oracle.h"
}

using pp::fr;

static fr load(const uint64_t *p) {
  fr a;
  std::memcpy(a.v, p, 32);
  return a;
}

static const uint32_t kR[8] = {PP_R0, PP_R1, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7};

// a + r for a < r (the other representative of a below 2r)
static fr plus_r(const fr &a) {
  fr s;
  uint64_t c = 0;
  for (int i = 0; i < 8; ++i) {
    c += (uint64_t)a.v[i] + kR[i];
    s.v[i] = (uint32_t)c;
    c >>= 32;
  }
  return s;
}

static bool below_2r(const fr &a) {
  // compare a with 2r from the top limb down
  uint32_t two_r[8];
  uint64_t c = 0;
  for (int i = 0; i < 8; ++i) {
    c += 2ull * kR[i];
    two_r[i] = (uint32_t)c;
    c >>= 32;
  }
  for (int i = 7; i >= 0; --i)
    if (a.v[i] != two_r[i]) return a.v[i] < two_r[i];
  return false;
}

// the lazy form must stay below 2r and be congruent to the canonical answer
static bool lazy_ok(const fr &lazy, const uint64_t want[4]) {
  const fr c = pp::fr_canon(lazy);
  return below_2r(lazy) && std::memcmp(c.v, want, 32) == 0;
}

int main(int argc, char **argv) {
  const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 20000;
  uint64_t *a = new uint64_t[4 * n], *b = new uint64_t[4 * n];
  or_random_fr(a, n, 0x1234, 0);
  or_random_fr(b, n, 0x5678, 0);
  // edge values
  const uint64_t rm1[4] = {0xffffffff00000000ULL, 0x53bda402fffe5bfeULL, 0x3339d80809a1d805ULL,
                           0x73eda753299d7d48ULL};
  std::memset(a, 0, 32);
  std::memcpy(b + 4, rm1, 32);
  std::memcpy(a + 8, rm1, 32);
  std::memcpy(b + 8, rm1, 32);
  or_fr_one(a + 12);
  // r - 1 at odd indices: the lazy operands there reach 2r - 1
  std::memcpy(a + 20, rm1, 32);
  std::memcpy(b + 20, rm1, 32);
  std::memcpy(a + 28, rm1, 32);
  std::memcpy(b + 28, rm1, 32);
  // inversion edges (raw word values): 1, 2, 3, 2^k for k = 1 .. 254 in steps
  // of 23, r - 2, r - 2^32, 2^64 - 1
  if (n >= 40) {
    for (int k = 0; k < 3; ++k) {
      std::memset(a + 4 * (10 + k), 0, 32);
      a[4 * (10 + k)] = (uint64_t)k + 1;
    }
    for (int j = 0, k = 1; k < 255; ++j, k += 23) {
      uint64_t *p = a + 4 * (13 + j);
      std::memset(p, 0, 32);
      p[k / 64] = 1ull << (k % 64);
    }
    uint64_t *p = a + 4 * 25;
    std::memcpy(p, rm1, 32);
    p[0] -= 1;  // r - 2
    p = a + 4 * 26;
    std::memcpy(p, rm1, 32);
    p[0] = 1;  // r - 2^32
    p = a + 4 * 27;
    std::memset(p, 0, 32);
    p[0] = ~0ull;
  }
  long bad = 0;
  {
    // the largest accumulation: 16 products of (r - 1)^2
    uint32_t acc[17] = {0};
    uint64_t want_dot[4] = {0, 0, 0, 0};
    for (int k = 0; k < 16; ++k) {
      pp::fr_mac17(acc, load(rm1), load(rm1));
      uint64_t prod[4], sum[4];
      or_fr_mul(rm1, rm1, prod);
      or_fr_add(want_dot, prod, sum);
      std::memcpy(want_dot, sum, 32);
    }
    const fr got = pp::fr_redc17(acc);
    if (std::memcmp(got.v, want_dot, 32)) {
      bad++;
      std::printf("dot product mismatch for 16 (r - 1)^2\n");
    }
  }
  for (uint64_t i = 0; i < n; ++i) {
    fr x = load(a + 4 * i), y = load(b + 4 * i);
    uint64_t want[4];
    or_fr_mul(a + 4 * i, b + 4 * i, want);
    fr m0 = pp::fr_mul_v<0>(x, y), m1 = pp::fr_mul_v<1>(x, y), m2 = pp::fr_mul_w(x, y);
    fr m3 = pp::fr_mul_kara<false>(x, y), m4 = pp::fr_mul_kara<true>(x, y), m5 = pp::fr_mul_sos(x, y);
    fr m6 = pp::fr_mul_split<1, 1>(x, y), m7 = pp::fr_mul_split<1, 0>(x, y), m8 = pp::fr_mul_split<0, 1>(x, y);
    fr m9 = pp::fr_mul_row9(x, y), m10 = pp::fr_mul_kara_rows(x, y);
    fr m11 = pp::fr_mul_mix<0, 1>(x, y), m12 = pp::fr_mul_mix<1, 0>(x, y), m13 = pp::fr_mul_mix<0, 2>(x, y);
    if (std::memcmp(m0.v, want, 32) || std::memcmp(m1.v, want, 32) || std::memcmp(m2.v, want, 32) ||
        std::memcmp(m3.v, want, 32) || std::memcmp(m4.v, want, 32) || std::memcmp(m5.v, want, 32) ||
        std::memcmp(m6.v, want, 32) || std::memcmp(m7.v, want, 32) || std::memcmp(m8.v, want, 32) ||
        std::memcmp(m9.v, want, 32) || std::memcmp(m10.v, want, 32) || std::memcmp(m11.v, want, 32) ||
        std::memcmp(m12.v, want, 32) || std::memcmp(m13.v, want, 32)) {
      if (bad++ < 5) std::printf("mul mismatch at %llu\n", (unsigned long long)i);
    }
    // the dedicated square against the oracle's product of a value with itself
    {
      uint64_t want_sq[4];
      or_fr_mul(a + 4 * i, a + 4 * i, want_sq);
      const fr sq = pp::fr_sqr(x);
      if (std::memcmp(sq.v, want_sq, 32)) {
        if (bad++ < 5) std::printf("square mismatch at %llu\n", (unsigned long long)i);
      }
    }
    // dot products of up to 16 terms with one reduction (fr_mac17 + fr_redc17)
    if (i % 16 == 15) {
      const int G = 1 + (int)((i / 16) % 16);
      uint32_t acc[17] = {0};
      uint64_t want_dot[4] = {0, 0, 0, 0};
      for (int k = 0; k < G; ++k) {
        const uint64_t *pa = a + 4 * (i - k), *pb = b + 4 * (i - k);
        pp::fr_mac17(acc, load(pa), load(pb));
        uint64_t prod[4], sum[4];
        or_fr_mul(pa, pb, prod);
        or_fr_add(want_dot, prod, sum);
        std::memcpy(want_dot, sum, 32);
      }
      const fr got = pp::fr_redc17(acc);
      if (std::memcmp(got.v, want_dot, 32)) {
        if (bad++ < 5) std::printf("dot product mismatch at %llu (G = %d)\n", (unsigned long long)i, G);
      }
    }
    // lazy operands: either representative below 2r
    const fr xl = (i & 1) ? plus_r(x) : x, yl = (i & 2) ? plus_r(y) : y;
    const fr ml = pp::fr_mul_lazy(xl, y), mc = pp::fr_mul_row9(xl, y);
    if (!lazy_ok(ml, want) || std::memcmp(mc.v, want, 32)) {
      if (bad++ < 5) std::printf("lazy mul mismatch at %llu\n", (unsigned long long)i);
    }
    // the transform's Karatsuba twiddle multiply (PP_NTT_MUL = 10), lazy
    {
      uint32_t t[16];
      pp::mul8_kara_rows(t, xl.v, y.v);
      if (!lazy_ok(pp::mont_redc16_rows<true>(t), want)) {
        if (bad++ < 5) std::printf("lazy Karatsuba mul mismatch at %llu\n", (unsigned long long)i);
      }
    }
    or_fr_add(a + 4 * i, b + 4 * i, want);
    fr s = pp::fr_add(x, y);
    if (std::memcmp(s.v, want, 32) || !lazy_ok(pp::fr_add_lazy(xl, yl), want)) {
      if (bad++ < 5) std::printf("add mismatch at %llu\n", (unsigned long long)i);
    }
    or_fr_sub(a + 4 * i, b + 4 * i, want);
    fr d = pp::fr_sub(x, y);
    if (std::memcmp(d.v, want, 32) || !lazy_ok(pp::fr_sub_lazy(xl, yl), want)) {
      if (bad++ < 5) std::printf("sub mismatch at %llu\n", (unsigned long long)i);
    }
    if (i < 200) {
      or_fr_inv(a + 4 * i, want);
      fr v = pp::fr_inv(x);
      if (std::memcmp(v.v, want, 32)) {
        if (bad++ < 5) std::printf("inv mismatch at %llu\n", (unsigned long long)i);
      }
      fr vb = pp::fr_inv_binary(x);
      if (std::memcmp(vb.v, want, 32)) {
        if (bad++ < 5) std::printf("binary inv mismatch at %llu\n", (unsigned long long)i);
      }
    }
    if (i < 20000) {
      or_fr_inv(a + 4 * i, want);
      // both limb widths: 62 bits (the host form) and 30 bits (the GPU form)
      fr vf = pp::fr_inv_divsteps<int64_t>(x), vg = pp::fr_inv_divsteps<int32_t>(x);
      if (std::memcmp(vf.v, want, 32) || std::memcmp(vg.v, want, 32)) {
        if (bad++ < 5) std::printf("divstep inv mismatch at %llu\n", (unsigned long long)i);
      }
    }
    if (i < 200) {
      uint64_t e[4] = {i * 7919 + 3, 0, 0, 0};
      or_fr_pow(a + 4 * i, e, want);
      fr p = pp::fr_pow_u64(x, e[0]);
      if (std::memcmp(p.v, want, 32)) {
        if (bad++ < 5) std::printf("pow mismatch at %llu\n", (unsigned long long)i);
      }
    }
  }
  std::printf("checked %llu, mismatches %ld\n", (unsigned long long)n, bad);
  return bad ? 1 : 0;
}
