/*
 * pp_oracle.c -- CPU oracle for the Fr prover-operator path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C over
 * unsigned __int128, what the reference computes on this path, so that the
 * CUDA implementation can be checked against it.  Nothing in the product
 * links it; only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it (through oracle/oracle.py).
 *
 * Field: BLS12-381 Fr, r = 0x73eda753...ffffffff00000001, Montgomery form with
 * R = 2^256 (reference: PLONK/utils/mont/cpu/ff/bls12-381.hpp:6-32, the same
 * constants as PLONK/utils/mont/cuda/ff/bls12-381.hpp:7-45).  Multiplication
 * is word-serial Montgomery (CIOS, Koc/Acar/Kaliski 1996) over 64-bit words
 * with n0' = -r^-1 mod 2^64 = 0xfffffffeffffffff (bls12-381.hpp:26).
 */
#include "pp_oracle.h"
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
typedef uint64_t u64;

static const u64 R_MOD[4] = {0xffffffff00000001ULL, 0x53bda402fffe5bfeULL,
                             0x3339d80809a1d805ULL, 0x73eda753299d7d48ULL};
static const u64 R_ONE[4] = {0x00000001fffffffeULL, 0x5884b7fa00034802ULL,
                             0x998c4fefecbc4ff5ULL, 0x1824b159acc5056fULL};
static const u64 R_RR[4] = {0xc999e990f3f29c6dULL, 0x2b6cedcb87925c23ULL,
                            0x05d314967254398fULL, 0x0748d9d99f59ff11ULL};
static const u64 N0 = 0xfffffffeffffffffULL;

static inline int geq_r(const u64 t[4]) {
  for (int i = 3; i >= 0; --i) {
    if (t[i] > R_MOD[i]) return 1;
    if (t[i] < R_MOD[i]) return 0;
  }
  return 1;
}

static inline void sub_r(u64 t[4]) {
  u64 borrow = 0;
  for (int i = 0; i < 4; ++i) {
    u128 d = (u128)t[i] - R_MOD[i] - borrow;
    t[i] = (u64)d;
    borrow = (u64)(d >> 64) & 1;
  }
}

static inline void mmul(u64 out[4], const u64 a[4], const u64 b[4]) {
  u64 t[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    u64 c = 0;
    for (int j = 0; j < 4; ++j) {
      u128 uv = (u128)a[j] * b[i] + t[j] + c;
      t[j] = (u64)uv;
      c = (u64)(uv >> 64);
    }
    u128 uv = (u128)t[4] + c;
    t[4] = (u64)uv;
    t[5] = (u64)(uv >> 64);
    u64 m = t[0] * N0;
    uv = (u128)m * R_MOD[0] + t[0];
    c = (u64)(uv >> 64);
    for (int j = 1; j < 4; ++j) {
      uv = (u128)m * R_MOD[j] + t[j] + c;
      t[j - 1] = (u64)uv;
      c = (u64)(uv >> 64);
    }
    uv = (u128)t[4] + c;
    t[3] = (u64)uv;
    t[4] = t[5] + (u64)(uv >> 64);
  }
  /* r < 2^254.9 so the CIOS result is < 2r < 2^256: t[4] == 0 */
  u64 res[4] = {t[0], t[1], t[2], t[3]};
  if (geq_r(res)) sub_r(res);
  memcpy(out, res, sizeof(res));
}

static inline void madd(u64 out[4], const u64 a[4], const u64 b[4]) {
  u64 s[4];
  u64 c = 0;
  for (int i = 0; i < 4; ++i) {
    u128 x = (u128)a[i] + b[i] + c;
    s[i] = (u64)x;
    c = (u64)(x >> 64);
  }
  /* a + b < 2r < 2^256, no carry out */
  if (geq_r(s)) sub_r(s);
  memcpy(out, s, sizeof(s));
}

static inline void msub(u64 out[4], const u64 a[4], const u64 b[4]) {
  u64 d[4];
  u64 borrow = 0;
  for (int i = 0; i < 4; ++i) {
    u128 x = (u128)a[i] - b[i] - borrow;
    d[i] = (u64)x;
    borrow = (u64)(x >> 64) & 1;
  }
  if (borrow) {
    u64 c = 0;
    for (int i = 0; i < 4; ++i) {
      u128 x = (u128)d[i] + R_MOD[i] + c;
      d[i] = (u64)x;
      c = (u64)(x >> 64);
    }
  }
  memcpy(out, d, sizeof(d));
}

static inline int is_zero(const u64 a[4]) { return (a[0] | a[1] | a[2] | a[3]) == 0; }

static void mpow(u64 out[4], const u64 a[4], const u64 e[4]) {
  u64 acc[4];
  memcpy(acc, R_ONE, sizeof(acc));
  for (int w = 3; w >= 0; --w) {
    for (int bit = 63; bit >= 0; --bit) {
      mmul(acc, acc, acc);
      if ((e[w] >> bit) & 1) mmul(acc, acc, a);
    }
  }
  memcpy(out, acc, sizeof(acc));
}

static void minv(u64 out[4], const u64 a[4]) {
  /* Fermat: a^(r-2); 0 maps to 0 */
  u64 e[4] = {R_MOD[0] - 2, R_MOD[1], R_MOD[2], R_MOD[3]};
  mpow(out, a, e);
}

void or_fr_mul(const u64 a[4], const u64 b[4], u64 out[4]) { mmul(out, a, b); }
void or_fr_add(const u64 a[4], const u64 b[4], u64 out[4]) { madd(out, a, b); }
void or_fr_sub(const u64 a[4], const u64 b[4], u64 out[4]) { msub(out, a, b); }
void or_fr_neg(const u64 a[4], u64 out[4]) {
  static const u64 z[4] = {0, 0, 0, 0};
  msub(out, z, a);
}
void or_fr_pow(const u64 a[4], const u64 e[4], u64 out[4]) { mpow(out, a, e); }
void or_fr_inv(const u64 a[4], u64 out[4]) { minv(out, a); }
void or_fr_to_mont(const u64 a[4], u64 out[4]) { mmul(out, a, R_RR); }
void or_fr_from_mont(const u64 a[4], u64 out[4]) {
  static const u64 one_raw[4] = {1, 0, 0, 0};
  mmul(out, a, one_raw);
}
void or_fr_one(u64 out[4]) { memcpy(out, R_ONE, 4 * sizeof(u64)); }

/* The reference's domain generator: group_gen = 7 and
 * forward_roots_of_unity[k] = 7^((r-1)/2^k)
 * (PLONK/utils/zkp/cuda/zksnark_ntt/parameters/bls12_381.h:8-83). */
void or_root_of_unity(int lg, int inverse, u64 out[4]) {
  u64 e[4] = {R_MOD[0] - 1, R_MOD[1], R_MOD[2], R_MOD[3]};
  for (int s = 0; s < lg; ++s) { /* e >>= 1 (r-1 has 32 trailing zeros) */
    e[0] = (e[0] >> 1) | (e[1] << 63);
    e[1] = (e[1] >> 1) | (e[2] << 63);
    e[2] = (e[2] >> 1) | (e[3] << 63);
    e[3] >>= 1;
  }
  u64 seven[4] = {7, 0, 0, 0}, g[4];
  or_fr_to_mont(seven, g);
  mpow(out, g, e);
  if (inverse) minv(out, out);
}

/* ---------------- seeded random canonical elements ---------------- */
static inline u64 mix64(u64 z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

void or_random_fr(u64 *out, u64 n, u64 seed, u64 first_index) {
#pragma omp parallel for schedule(static)
  for (long long li = 0; li < (long long)n; ++li) {
    u64 idx = first_index + (u64)li;
    u64 v[4];
    int ok = 0;
    for (u64 t = 0; t < 64 && !ok; ++t) {
      for (u64 j = 0; j < 4; ++j) {
        u64 ctr = (idx << 8) | (t << 2) | j;
        v[j] = mix64(seed + (ctr + 1) * 0x9E3779B97F4A7C15ULL);
      }
      v[3] &= 0x7fffffffffffffffULL;
      ok = !geq_r(v);
    }
    if (!ok) sub_r(v); /* v < 2^255 < 2r */
    memcpy(out + 4 * li, v, sizeof(v));
  }
}

/* ---------------- NTT ---------------- */
static inline u64 bitrev(u64 x, int bits) {
  u64 r = 0;
  for (int i = 0; i < bits; ++i) {
    r = (r << 1) | (x & 1);
    x >>= 1;
  }
  return r;
}

static int pick_threads(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

/* Natural-order in, natural-order out ("NN") transform
 * X_k = sum_j x_j w^(jk), w = omega_{2^lg_n} (inverse: w^-1 and a final
 * scaling by N^-1).  This is the function the reference's Ntt::forward /
 * Intt::forward compute (PLONK/utils/zkp/cuda/zksnark_ntt/ntt_kernel/
 * ntt.cuh:113-170 with the N^-1 fold at ct_mixed_radix_wide.cuh:173-176);
 * it is restated here as an iterative radix-2 decimation-in-time transform
 * after a bit-reversal permutation. */
void or_ntt(u64 *data, int lg_n, int inverse, int nthreads) {
  const u64 n = 1ULL << lg_n;
  const int nt = pick_threads(nthreads);
  if (lg_n == 0) return;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long long i = 0; i < (long long)n; ++i) {
    u64 j = bitrev((u64)i, lg_n);
    if ((u64)i < j) {
      u64 tmp[4];
      memcpy(tmp, data + 4 * i, 32);
      memcpy(data + 4 * i, data + 4 * j, 32);
      memcpy(data + 4 * j, tmp, 32);
    }
  }
  u64 *tw = (u64 *)malloc((n / 2) * 32);
  for (int s = 1; s <= lg_n; ++s) {
    const u64 half = 1ULL << (s - 1);
    u64 w[4];
    or_root_of_unity(s, inverse, w);
    /* twiddle table w^j, j < half (sequential chain, chunked for threads) */
    memcpy(tw, R_ONE, 32);
    for (u64 j = 1; j < half; ++j) mmul(tw + 4 * j, tw + 4 * (j - 1), w);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long long b = 0; b < (long long)(n / 2); ++b) {
      u64 j = (u64)b & (half - 1);
      u64 base = ((u64)b >> (s - 1)) << s;
      u64 *x0 = data + 4 * (base + j);
      u64 *x1 = data + 4 * (base + j + half);
      u64 t[4];
      mmul(t, x1, tw + 4 * j);
      msub(x1, x0, t);
      madd(x0, x0, t);
    }
  }
  free(tw);
  if (inverse) {
    u64 ninv[4], nn[4] = {n, 0, 0, 0};
    or_fr_to_mont(nn, nn);
    minv(ninv, nn);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long long i = 0; i < (long long)n; ++i) mmul(data + 4 * i, data + 4 * i, ninv);
  }
}

/* out[i] = in[i] * h^i for i < n, chunked so that threads start from h^start */
static void scale_by_powers(const u64 *in, u64 *out, u64 n, const u64 h[4], int nt) {
#pragma omp parallel num_threads(nt)
  {
    int tid = 0, T = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    T = omp_get_num_threads();
#endif
    u64 lo = n * (u64)tid / (u64)T, hi = n * (u64)(tid + 1) / (u64)T;
    u64 e[4] = {lo, 0, 0, 0}, p[4];
    mpow(p, h, e);
    for (u64 i = lo; i < hi; ++i) {
      mmul(out + 4 * i, in + 4 * i, p);
      mmul(p, p, h);
    }
  }
}

/* Reference coset LDE (lde.cu:1267-1365): the input is N coefficients a_i;
 * lde_spread_powers_kernel (lde.cu:623-648) scales the coefficient at
 * bit-reversed compact position c by 7^bitrev_L(c) = 7^(i*2^lambda) and
 * zero-spreads by 2^lambda, then an L = lg_n+lambda point NN transform
 * follows.  Output: p(h * omega_{2^L}^k), h = 7^(2^lambda), k < 2^L. */
void or_lde_coeffs(const u64 *coeffs, int lg_n, int lambda, u64 *out, int nthreads) {
  const int nt = pick_threads(nthreads);
  const int L = lg_n + lambda;
  const u64 n = 1ULL << lg_n, m = 1ULL << L;
  u64 seven[4] = {7, 0, 0, 0}, g[4], h[4];
  or_fr_to_mont(seven, g);
  u64 e[4] = {1ULL << lambda, 0, 0, 0};
  mpow(h, g, e);
  scale_by_powers(coeffs, out, n, h, nt);
  memset(out + 4 * n, 0, (m - n) * 32);
  or_ntt(out, L, 0, nt);
}

/* LDE from evaluations on the size-N subgroup, coset shift g = 7:
 * INTT_N, multiply coefficient i by 7^i, zero-pad to 2^L, NTT_{2^L}.
 * Output: p(7 * omega_{2^L}^k). */
void or_lde_evals(const u64 *evals, int lg_n, int lambda, u64 *out, int nthreads) {
  const int nt = pick_threads(nthreads);
  const int L = lg_n + lambda;
  const u64 n = 1ULL << lg_n, m = 1ULL << L;
  memcpy(out, evals, n * 32);
  or_ntt(out, lg_n, 1, nt);
  u64 seven[4] = {7, 0, 0, 0}, g[4];
  or_fr_to_mont(seven, g);
  scale_by_powers(out, out, n, g, nt);
  memset(out + 4 * n, 0, (m - n) * 32);
  or_ntt(out, L, 0, nt);
}

/* The reference's naive_lde (lde.cu:1367-1490, spread at :479-491): the input
 * is placed at natural positions i << lambda with no coset factor and an
 * L-point NN transform is applied. */
void or_lde_spread(const u64 *in, int lg_n, int lambda, u64 *out, int nthreads) {
  const int nt = pick_threads(nthreads);
  const int L = lg_n + lambda;
  const u64 n = 1ULL << lg_n, m = 1ULL << L;
  memset(out, 0, m * 32);
  for (u64 i = 0; i < n; ++i) memcpy(out + 4 * (i << lambda), in + 4 * i, 32);
  or_ntt(out, L, 0, nt);
}

/* ---------------- grand product ---------------- */
/* accumulate_mul_poly (PLONK/utils/mont/cuda/mont_arithmetic.cu:334-361,
 * kernels :181-201): exclusive prefix product written over the input,
 * out[0] = 1, out[i] = prod_{j<i} in[j]. */
void or_gp_prefix(u64 *inout, u64 n) {
  u64 acc[4];
  memcpy(acc, R_ONE, 32);
  for (u64 i = 0; i < n; ++i) {
    u64 v[4];
    memcpy(v, inout + 4 * i, 32);
    memcpy(inout + 4 * i, acc, 32);
    mmul(acc, acc, v);
  }
}

/* Montgomery's simultaneous inversion over a chunk; zero maps to zero. */
static void batch_inv(u64 *v, u64 n) {
  if (n == 0) return;
  u64 *pre = (u64 *)malloc(n * 32);
  u64 acc[4];
  memcpy(acc, R_ONE, 32);
  for (u64 i = 0; i < n; ++i) {
    memcpy(pre + 4 * i, acc, 32);
    if (!is_zero(v + 4 * i)) mmul(acc, acc, v + 4 * i);
  }
  u64 inv[4];
  minv(inv, acc);
  for (u64 i = n; i-- > 0;) {
    if (is_zero(v + 4 * i)) continue;
    u64 t[4];
    mmul(t, inv, pre + 4 * i);
    mmul(inv, inv, v + 4 * i);
    memcpy(v + 4 * i, t, 32);
  }
  free(pre);
}

/* PLONK copy-constraint grand product (the ratio form the reference's
 * permutation-constraint kernel uses, PLONK/utils/zkp/cuda/
 * zksnark_compute_permutation_constraint.cu:13-34):
 *   ratio_i = prod_j (w_j[i] + beta*k_j*omega^i + gamma)
 *           / prod_j (w_j[i] + beta*sigma_j[i] + gamma)
 *   z = exclusive prefix product of ratio (z_0 = 1), as accumulate_mul_poly. */
void or_gp_perm(const u64 *const w[3], const u64 *const sigma[3], const u64 beta[4],
                const u64 gamma[4], const u64 k[3][4], int lg_n, u64 *z, int nthreads) {
  const int nt = pick_threads(nthreads);
  const u64 n = 1ULL << lg_n;
  u64 omega[4];
  or_root_of_unity(lg_n, 0, omega);
  u64 *den = (u64 *)malloc(n * 32);
  u64 bk[3][4];
  for (int j = 0; j < 3; ++j) mmul(bk[j], beta, k[j]);
#pragma omp parallel num_threads(nt)
  {
    int tid = 0, T = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    T = omp_get_num_threads();
#endif
    u64 lo = n * (u64)tid / (u64)T, hi = n * (u64)(tid + 1) / (u64)T;
    u64 e[4] = {lo, 0, 0, 0}, wp[4];
    mpow(wp, omega, e);
    for (u64 i = lo; i < hi; ++i) {
      u64 num[4], d[4];
      memcpy(num, R_ONE, 32);
      memcpy(d, R_ONE, 32);
      for (int j = 0; j < 3; ++j) {
        u64 t[4], s[4];
        mmul(t, bk[j], wp);
        madd(t, t, w[j] + 4 * i);
        madd(t, t, gamma);
        mmul(num, num, t);
        mmul(s, beta, sigma[j] + 4 * i);
        madd(s, s, w[j] + 4 * i);
        madd(s, s, gamma);
        mmul(d, d, s);
      }
      memcpy(z + 4 * i, num, 32);
      memcpy(den + 4 * i, d, 32);
      mmul(wp, wp, omega);
    }
    batch_inv(den + 4 * lo, hi - lo);
    for (u64 i = lo; i < hi; ++i) mmul(z + 4 * i, z + 4 * i, den + 4 * i);
  }
  free(den);
  or_gp_prefix(z, n);
}

/* ---------------- evaluation ---------------- */
/* evaluate (PLONK/utils/function.cu:170-181 -> mont_arithmetic.cu:104-163):
 * y = sum_i poly[i] * x^i; an empty polynomial evaluates to 0.  Field
 * addition is exact, so the reference's summation order does not matter. */
void or_eval(const u64 *poly, u64 n, const u64 x[4], u64 y[4], int nthreads) {
  const int nt = pick_threads(nthreads);
  u64 total[4] = {0, 0, 0, 0};
  if (n == 0) {
    memcpy(y, total, 32);
    return;
  }
  int T = nt;
  if ((u64)T > n) T = (int)n;
  u64 *part = (u64 *)calloc((size_t)T, 32);
#pragma omp parallel for schedule(static, 1) num_threads(T)
  for (int t = 0; t < T; ++t) {
    u64 lo = n * (u64)t / (u64)T, hi = n * (u64)(t + 1) / (u64)T;
    u64 acc[4] = {0, 0, 0, 0};
    for (u64 i = hi; i-- > lo;) { /* Horner over the chunk */
      mmul(acc, acc, x);
      madd(acc, acc, poly + 4 * i);
    }
    u64 e[4] = {lo, 0, 0, 0}, p[4];
    mpow(p, x, e);
    mmul(part + 4 * t, acc, p);
  }
  for (int t = 0; t < T; ++t) madd(total, total, part + 4 * t);
  free(part);
  memcpy(y, total, 32);
}

/* ---------------- division by (X + c) ---------------- */
/* poly_div_poly (PLONK/utils/function.cu:183 -> mont_arithmetic.cu:305-331,
 * 531-542): S_i = sum_{j>=i} p_j (-c)^(j-i); the buffer becomes
 * q_i = S_{i+1} for i < n-1 and q_{n-1} = 0: the quotient of p by (X + c). */
void or_div_xplusc(u64 *inout, u64 n, const u64 c[4]) {
  if (n == 0) return;
  u64 s[4] = {0, 0, 0, 0};
  for (u64 i = n; i-- > 0;) {
    u64 p[4], t[4];
    memcpy(p, inout + 4 * i, 32);
    memcpy(inout + 4 * i, s, 32); /* q_i = S_{i+1} */
    mmul(t, s, c);
    msub(s, p, t); /* S_i = p_i - c * S_{i+1} */
  }
}

/* ---------------- the reference's CPU baselines ---------------- */
/* naive_gp (miss_ops.cu:34-47): out[i] = prod_{j<=i} in[j] for i < n-1,
 * out[n-1] = 0 (the output buffer starts zeroed). */
void or_naive_gp(const u64 *in, u64 n, u64 *out) {
  memset(out, 0, n * 32);
  if (n == 0) return;
  u64 state[4];
  memcpy(state, R_ONE, 32);
  memcpy(out, state, 32);
  for (u64 i = 0; i + 1 < n; ++i) {
    mmul(state, state, in + 4 * i);
    memcpy(out + 4 * i, state, 32);
  }
}

/* naive_div (miss_ops.cu:49-87): schoolbook long division by [c, 1] = X + c,
 * quotient of length n-1.  Returns -1 where the reference's
 * zero-leading-coefficient loop (:82-84) would run below index 0. */
int or_naive_div(const u64 *in, u64 n, const u64 c[4], u64 *quotient) {
  if (n < 2) return 0;
  u64 *rem = (u64 *)malloc(n * 32);
  memcpy(rem, in, n * 32);
  memset(quotient, 0, (n - 1) * 32);
  u64 len = n;
  int status = 0;
  while (len >= 2) {
    u64 q[4], t[4];
    memcpy(q, rem + 4 * (len - 1), 32); /* leading divisor coefficient is 1 */
    u64 deg = len - 2;
    memcpy(quotient + 4 * deg, q, 32);
    mmul(t, q, c);
    msub(rem + 4 * deg, rem + 4 * deg, t);
    msub(rem + 4 * (deg + 1), rem + 4 * (deg + 1), q);
    while (len > 0 && is_zero(rem + 4 * (len - 1))) len--;
    if (len == 0) {
      status = -1;
      break;
    }
  }
  free(rem);
  return status;
}

int64_t or_first_diff(const u64 *a, const u64 *b, u64 n) {
  for (u64 i = 0; i < n; ++i)
    if (memcmp(a + 4 * i, b + 4 * i, 32) != 0) return (int64_t)i;
  return -1;
}

/* ------------------------------------------------ quotient constraints ---
 * Element-wise PLONK quotient terms over the extended domain.  Vectors hold
 * n elements, scalars one.  Field arithmetic is exact, so the terms may be
 * grouped and ordered freely; each function follows the formula of the
 * reference kernel it names. */
typedef struct {
  u64 v[4];
} fe;

static inline fe fe_ld(const u64 *p) {
  fe r;
  memcpy(r.v, p, 32);
  return r;
}
static inline fe fm(fe a, fe b) {
  fe r;
  mmul(r.v, a.v, b.v);
  return r;
}
static inline fe fa(fe a, fe b) {
  fe r;
  madd(r.v, a.v, b.v);
  return r;
}
static inline fe fs(fe a, fe b) {
  fe r;
  msub(r.v, a.v, b.v);
  return r;
}
static inline fe fpow_small(fe a, int64_t e) {
  fe acc = fe_ld(R_ONE);
  for (int bit = 62; bit >= 0; --bit) {
    acc = fm(acc, acc);
    if ((e >> bit) & 1) acc = fm(acc, a);
  }
  return acc;
}

/* zksnark_compute_permutation_constraint.cu:5-16:
 * (x b + w_l + g)(x b k1 + w_r + g)(x b k2 + w_o + g)(x b k3 + w_4 + g) z alpha */
void or_quotient_identity(const u64 *x, const u64 *const w[4], const u64 *z, const u64 alpha[4],
                          const u64 beta[4], const u64 gamma[4], const u64 *const k[3], u64 *result,
                          u64 n) {
  const fe al = fe_ld(alpha), be = fe_ld(beta), ga = fe_ld(gamma);
  for (u64 i = 0; i < n; ++i) {
    const fe xb = fm(fe_ld(x + 4 * i), be);
    fe acc = fa(fa(xb, fe_ld(w[0] + 4 * i)), ga);
    for (int j = 1; j < 4; ++j)
      acc = fm(acc, fa(fa(fm(xb, fe_ld(k[j - 1])), fe_ld(w[j] + 4 * i)), ga));
    acc = fm(fm(acc, fe_ld(z + 4 * i)), al);
    memcpy(result + 4 * i, acc.v, 32);
  }
}

/* :18-34: result += mod - (s_l b + w_l + g)(s_r b + w_r + g)(s_o b + w_o + g)(s_4 b + w_4 + g) z' alpha */
void or_quotient_copy(const u64 *const sigma[4], const u64 *mod, const u64 *const w[4],
                      const u64 *z_next, const u64 alpha[4], const u64 beta[4], const u64 gamma[4],
                      u64 *result, u64 n) {
  const fe al = fe_ld(alpha), be = fe_ld(beta), ga = fe_ld(gamma);
  for (u64 i = 0; i < n; ++i) {
    fe acc = fe_ld(R_ONE);
    for (int j = 0; j < 4; ++j)
      acc = fm(acc, fa(fa(fm(fe_ld(sigma[j] + 4 * i), be), fe_ld(w[j] + 4 * i)), ga));
    acc = fm(fm(acc, fe_ld(z_next + 4 * i)), al);
    const fe r = fs(fa(fe_ld(result + 4 * i), fe_ld(mod + 4 * i)), acc);
    memcpy(result + 4 * i, r.v, 32);
  }
}

/* :36-45: result += (z - one) l1 */
void or_quotient_term_one(const u64 *z, const u64 *l1, const u64 one[4], u64 *result, u64 n) {
  const fe o = fe_ld(one);
  for (u64 i = 0; i < n; ++i) {
    const fe r = fa(fe_ld(result + 4 * i), fm(fs(fe_ld(z + 4 * i), o), fe_ld(l1 + 4 * i)));
    memcpy(result + 4 * i, r.v, 32);
  }
}

/* zksnark_comute_gate_constraint.cu:6-30 (allmerge_kernel), the sum of six
 * gate terms.  v[] holds the 22 vectors and s[] the 24 scalars in the order of
 * the kernel's arguments (PP_GATE_V_* / PP_GATE_S_* in include/pp_ops.h).
 * The reference writes d - (d - d_next) for d_next and forms its range/logic
 * "delta" as x (x three)((x one)(x two)) = x^4 * three * one * two. */
void or_gate_constraint(const u64 *const v[22], const u64 *const s[24], int64_t sbox_alpha,
                        u64 *out, u64 n) {
  fe S[24];
  for (int j = 0; j < 24; ++j) S[j] = fe_ld(s[j]);
  const fe four = S[0], one = S[1], two = S[2], three = S[3], kr = S[4], ksr = S[5], kcr = S[6],
           rch = S[7], pd = S[8], nine = S[9], kcl = S[10], e18 = S[11], e81 = S[12], e83 = S[13],
           kql = S[14], lch = S[15], pa = S[16], kfb = S[17], ksfb = S[18], kcfb = S[19],
           fbch = S[20], kvb = S[21], ksvb = S[22], vbch = S[23];
  const fe k312 = fm(fm(three, one), two);
  for (u64 i = 0; i < n; ++i) {
    fe V[22];
    for (int j = 0; j < 22; ++j) V[j] = fe_ld(v[j] + 4 * i);
    const fe a = V[0], b = V[1], c = V[2], d = V[3], an = V[4], bn = V[5], dn = V[6], qm = V[7],
             ql = V[8], qr = V[9], qo = V[10], q4 = V[11], qc = V[12], qhl = V[13], qhr = V[14],
             qh4 = V[15], qar = V[16], rng = V[17], lgc = V[18], fga = V[19], vga = V[20],
             pi = V[21];
#define DELTA(x) fm(fm(fm((x), (x)), fm((x), (x))), k312)
    const fe a4 = fm(a, four), b4 = fm(b, four), c4 = fm(c, four), d4 = fm(d, four);
    /* range */
    const fe rg = fm(fm(fa(fa(fa(fm(DELTA(fs(a4, dn)), kcr), fm(DELTA(fs(a, b4)), ksr)),
                              DELTA(fs(c, d4))),
                           fm(DELTA(fs(b, c4)), kr)),
                        rch),
                     rng);
    /* logic */
    const fe da = fs(a4, an), db = fs(b4, bn), w = fa(da, db), e = fs(dn, d4);
    const fe da2 = fm(da, da);
    const fe inner = fs(fm(w, e81), fa(fm(c, fm(fs(c4, fm(w, e18)), e81)), fm(fa(da2, da2), e18)));
    const fe A = fs(fm(fa(e, w), three), fm(fm(c, fm(inner, e83)), two));
    const fe B = fm(qc, fs(fm(e, nine), fm(w, three)));
    const fe lg = fm(fm(fa(fa(fa(fa(fm(fa(A, B), kql), fm(fs(c, fm(da, db)), kcl)), DELTA(e)),
                              DELTA(da)),
                           DELTA(db)),
                        lch),
                     lgc);
#undef DELTA
    /* arithmetic */
    fe ar = fa(fm(fpow_small(d, sbox_alpha), qh4), fm(fpow_small(b, sbox_alpha), qhr));
    ar = fa(ar, fm(fpow_small(a, sbox_alpha), qhl));
    ar = fa(fa(fa(ar, fm(d, q4)), fm(c, qo)), fm(b, qr));
    ar = fa(fa(fa(ar, fm(fm(a, b), qm)), fm(a, ql)), qc);
    ar = fm(ar, qar);
    /* fixed-base group addition */
    const fe abc = fm(fm(a, b), c);
    const fe qr2 = fm(fm(qr, fm(dn, dn)), fm(one, one));
    const fe f1 = fm(fs(c, fm(qc, dn)), kfb);
    const fe f2 = fm(fs(fs(bn, fm(fm(abc, bn), pd)), fs(fm(b, qr2), fm(a, fm(fm(ql, dn), pa)))), kcfb);
    const fe f3 = fm(fm(fm(dn, dn), dn), fm(one, one));
    const fe f4 = fm(fs(fa(an, fm(fm(abc, an), pd)), fa(fm(b, fm(ql, dn)), fm(a, qr2))), ksfb);
    const fe fb = fm(fm(fa(fa(fa(f1, f2), f3), f4), fbch), fga);
    /* variable-base group addition */
    const fe bc = fm(b, c);
    const fe v1 = fm(fs(fs(fm(b, d), fm(fm(a, c), pa)), fs(bn, fm(bc, fm(dn, fm(bn, pd))))), ksvb);
    const fe v2 = fa(fs(dn, fm(a, d)), fm(fs(fa(dn, bc), fa(an, fm(bc, fm(dn, fm(an, pd))))), kvb));
    const fe vb = fm(fm(fa(v1, v2), vbch), vga);
    const fe r = fa(fa(fa(fa(fa(fb, lg), rg), ar), pi), vb);
    memcpy(out + 4 * i, r.v, 32);
  }
}
