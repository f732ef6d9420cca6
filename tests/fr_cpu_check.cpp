// fr_cpu_check.cpp -- checks the host field element cpu::BLS12_381_Fr_G1
// (ppopp26-artifact_gb300/host/fr_cpu.h) against the oracle's C field code, on
// seeded random elements and edge values, and runs the reference's naive_gp /
// naive_div loops (miss_ops.cu:34-87, restated here on plain arrays) against
// the oracle's or_naive_gp / or_naive_div.  Prints "mismatches N".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fr_cpu.h"

extern "C" {
#include "pp_oracle.h"
}

using Fr = cpu::BLS12_381_Fr_G1;

static int bad = 0;

static void expect(const Fr &got, const uint64_t want[4], const char *what, size_t i) {
  if (std::memcmp((const uint64_t *)got, want, 32) != 0) {
    if (bad < 10) std::printf("mismatch %s at %zu\n", what, i);
    ++bad;
  }
}

int main(int argc, char **argv) {
  const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 10000;
  std::vector<uint64_t> a(4 * n), b(4 * n);
  or_random_fr(a.data(), n, 0xF5C0FFEEull, 0);
  or_random_fr(b.data(), n, 0xF5C0FFEFull, 0);
  // edge values: 0, 1, r - 1 (Montgomery forms of the integers)
  uint64_t one[4], minus_one[4], zero[4] = {0, 0, 0, 0};
  or_fr_one(one);
  or_fr_neg(one, minus_one);
  std::memcpy(&a[0], zero, 32);
  std::memcpy(&a[4], one, 32);
  std::memcpy(&a[8], minus_one, 32);
  std::memcpy(&b[12], minus_one, 32);
  for (size_t i = 0; i < n; ++i) {
    Fr x(&a[4 * i]), y(&b[4 * i]);
    uint64_t w[4];
    or_fr_mul(&a[4 * i], &b[4 * i], w);
    expect(x * y, w, "mul", i);
    Fr t = x;
    t *= y;
    expect(t, w, "mul=", i);
    or_fr_add(&a[4 * i], &b[4 * i], w);
    expect(x + y, w, "add", i);
    or_fr_sub(&a[4 * i], &b[4 * i], w);
    expect(x - y, w, "sub", i);
    t = x;
    t -= y;
    expect(t, w, "sub=", i);
    or_fr_neg(&a[4 * i], w);
    expect(-x, w, "neg", i);
    if (i % 16 == 0) {
      or_fr_inv(&a[4 * i], w);
      expect(1 / x, w, "inv", i);
      const uint64_t e[4] = {(uint64_t)(i * 2654435761u) & 0xffffffffu, 0, 0, 0};
      or_fr_pow(&a[4 * i], e, w);
      expect(x ^ (unsigned)e[0], w, "pow", i);
    }
    if (x.is_zero() != (std::memcmp(&a[4 * i], zero, 32) == 0)) {
      std::printf("is_zero wrong at %zu\n", i);
      ++bad;
    }
  }
  // integer -> Montgomery conversion
  for (uint64_t v : {0ull, 1ull, 2ull, 7ull, 0xffffffffffffffffull}) {
    uint64_t plain[4] = {v, 0, 0, 0}, w[4];
    or_fr_to_mont(plain, w);
    expect(Fr(v), w, "to_mont", (size_t)v);
    Fr back = Fr(v);
    back.from();
    expect(back, plain, "from_mont", (size_t)v);
  }
  // naive_gp as miss_ops.cu:34-47 computes it: out[i] = prod_{j<=i} in[j] for
  // i < N-1 (the inclusive product), out[N-1] left as the zero-filled buffer.
  const size_t m = n < 4096 ? n : 4096;
  std::vector<uint64_t> gp(4 * m), want(4 * m);
  {
    Fr state = Fr::one();
    std::memcpy(&gp[0], (const uint64_t *)state, 32);
    for (size_t i = 0; i + 1 < m; ++i) {
      state *= Fr(&b[4 * i]);
      std::memcpy(&gp[4 * i], (const uint64_t *)state, 32);
    }
    or_naive_gp(b.data(), m, want.data());
    for (size_t i = 0; i < m; ++i) expect(Fr(&gp[4 * i]), &want[4 * i], "naive_gp", i);
  }
  // naive_div by [c, 1] (miss_ops.cu:49-87)
  {
    std::vector<uint64_t> rem(b.begin(), b.begin() + 4 * m), q(4 * (m - 1), 0), qw(4 * (m - 1));
    const Fr c(&a[4 * 7]);
    const Fr lead_inv = 1 / Fr::one();
    size_t len = m;
    Fr *r = reinterpret_cast<Fr *>(rem.data());
    Fr *qq = reinterpret_cast<Fr *>(q.data());
    const Fr div[2] = {c, Fr::one()};
    while (len >= 2) {
      Fr coef = r[len - 1] * lead_inv;
      qq[len - 2] = coef;
      for (int k = 0; k < 2; ++k) r[len - 2 + k] -= coef * div[k];
      while (len > 0 && r[len - 1].is_zero()) --len;
    }
    or_naive_div(b.data(), m, &a[4 * 7], qw.data());
    for (size_t i = 0; i + 1 < m; ++i) expect(qq[i], &qw[4 * i], "naive_div", i);
  }
  std::printf("checked %zu elements, mismatches %d\n", n, bad);
  return bad ? 1 : 0;
}
