// Host-side check of the device G1 code: compiles csrc/g1.cuh (and fq.cuh)
// without a GPU, the carry chains running as their host emulation.
//   g1_host_check msm <points.bin> <scalars.bin> <n> <out.bin>
//       sum_i s_i P_i by per-point double-and-add in XYZZ, to affine
//   g1_host_check add <n>
//       random P, Q from the oracle: P + Q (affine and XYZZ forms), P + P and
//       P + (-P) against the oracle's Jacobian arithmetic; prints mismatches
// Built and run by tests/test_g1_host.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../ppopp26-artifact_gb300/csrc/g1.cuh"
extern "C" {
#include "../oracle/pp_oracle.h"
}

using namespace pp;

static g1a load_aff(const uint64_t *p) {
  g1a a;
  std::memcpy(a.x.v, p, 48);
  std::memcpy(a.y.v, p + 6, 48);
  return a;
}
static void store_aff(const g1a &a, uint64_t *p) {
  std::memcpy(p, a.x.v, 48);
  std::memcpy(p + 6, a.y.v, 48);
}

static g1x mul(const g1a &p, const uint64_t s[4]) {
  g1x r = g1x_inf();
  for (int w = 3; w >= 0; --w)
    for (int b = 63; b >= 0; --b) {
      r = g1x_dbl(r);
      if ((s[w] >> b) & 1) r = g1x_add_affine(r, p);
    }
  return r;
}

static std::vector<uint64_t> read_words(const char *path, size_t n) {
  std::vector<uint64_t> v(n);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), 8, n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

int main(int argc, char **argv) {
  if (argc >= 6 && !std::strcmp(argv[1], "msm")) {
    const size_t n = std::strtoull(argv[4], nullptr, 10);
    auto P = read_words(argv[2], 12 * n), S = read_words(argv[3], 4 * n);
    g1x acc = g1x_inf();
    for (size_t i = 0; i < n; ++i) acc = g1x_add(acc, mul(load_aff(&P[12 * i]), &S[4 * i]));
    uint64_t out[12];
    store_aff(g1x_to_affine(acc), out);
    FILE *f = std::fopen(argv[5], "wb");
    std::fwrite(out, 8, 12, f);
    std::fclose(f);
    std::printf("msm done\n");
    return 0;
  }
  if (argc >= 3 && !std::strcmp(argv[1], "add")) {
    const size_t n = std::strtoull(argv[2], nullptr, 10);
    std::vector<uint64_t> k(8 * n), pts(24 * n);
    or_random_fr(k.data(), 2 * n, 0x61, 0);
    or_g1_mul_gen(k.data(), 2 * n, pts.data(), 0);
    long bad = 0;
    for (size_t i = 0; i < n; ++i) {
      const uint64_t *a = &pts[24 * i], *b = &pts[24 * i + 12];
      uint64_t want[12], got[12];
      or_g1_add(a, b, want);
      const g1a pa = load_aff(a), pb = load_aff(b);
      store_aff(g1x_to_affine(g1x_add_affine(g1x_from_affine(pa), pb)), got);
      bad += std::memcmp(got, want, 96) != 0;
      store_aff(g1x_to_affine(g1x_add(g1x_from_affine(pa), g1x_dbl_affine(pb))), got);
      uint64_t b2[12];
      or_g1_add(b, b, b2);
      or_g1_add(a, b2, want);
      bad += std::memcmp(got, want, 96) != 0;
      // P + P through the addition formulas (equal-x case) and P + (-P)
      store_aff(g1x_to_affine(g1x_add_affine(g1x_from_affine(pa), pa)), got);
      or_g1_add(a, a, want);
      bad += std::memcmp(got, want, 96) != 0;
      store_aff(g1x_to_affine(g1x_add_affine(g1x_from_affine(pa), g1a_neg(pa))), got);
      for (int j = 0; j < 12; ++j) bad += got[j] != 0;
      // the dedicated squaring against the multiply, on the coordinates
      for (const fq *v : {&pa.x, &pa.y, &pb.x, &pb.y}) {
        const fq s1 = fq_sqr(*v), s2 = fq_mul(*v, *v);
        bad += std::memcmp(s1.v, s2.v, 48) != 0;
      }
      // every row form of the multiply gives the same product
      {
        const fq m00 = fq_mul_rows<0, 0>(pa.x, pb.y), m01 = fq_mul_rows<0, 1>(pa.x, pb.y);
        const fq m10 = fq_mul_rows<1, 0>(pa.x, pb.y), m11 = fq_mul_rows<1, 1>(pa.x, pb.y);
        bad += std::memcmp(m00.v, m01.v, 48) != 0;
        bad += std::memcmp(m00.v, m10.v, 48) != 0;
        bad += std::memcmp(m00.v, m11.v, 48) != 0;
      }
    }
    // squaring edge values: 0, 1, q - 1, q - 2, all-ones low limbs
    {
      fq e[5] = {fq_zero(), fq_one(), fq_zero(), fq_zero(), fq_zero()};
      const uint32_t q[12] = {PP_Q0, PP_Q1, PP_Q2, PP_Q3, PP_Q4, PP_Q5,
                              PP_Q6, PP_Q7, PP_Q8, PP_Q9, PP_Q10, PP_Q11};
      for (int j = 0; j < 12; ++j) e[2].v[j] = e[3].v[j] = q[j];
      e[2].v[0] -= 1;
      e[3].v[0] -= 2;
      for (int j = 0; j < 11; ++j) e[4].v[j] = 0xffffffffu;
      e[4].v[11] = q[11] - 1;
      for (const fq &v : e) {
        const fq s1 = fq_sqr(v), s2 = fq_mul(v, v);
        bad += std::memcmp(s1.v, s2.v, 48) != 0;
        // both inverses agree (0 -> 0), and v * v^-1 = 1 otherwise
        const fq i1 = fq_inv(v), i2 = fq_inv_divsteps<int64_t>(v);
        const fq i3 = fq_inv_divsteps<int32_t>(v);
        bad += std::memcmp(i1.v, i2.v, 48) != 0;
        bad += std::memcmp(i1.v, i3.v, 48) != 0;
        if (!fq_is_zero(v)) bad += !fq_eq(fq_mul(v, i2), fq_one());
      }
    }
    // the divstep inverse against the binary GCD on the points' coordinates
    for (size_t i = 0; i < n; ++i) {
      const g1a pa = load_aff(&pts[24 * i]);
      for (const fq *v : {&pa.x, &pa.y}) {
        const fq i1 = fq_inv(*v), i2 = fq_inv_divsteps<int64_t>(*v);
        const fq i3 = fq_inv_divsteps<int32_t>(*v);
        bad += std::memcmp(i1.v, i2.v, 48) != 0;
        bad += std::memcmp(i1.v, i3.v, 48) != 0;
        bad += !fq_eq(fq_mul(*v, i2), fq_one());
      }
    }
    std::printf("mismatches %ld\n", bad);
    return bad ? 1 : 0;
  }
  std::fprintf(stderr, "usage: %s msm|add ...\n", argv[0]);
  return 2;
}
