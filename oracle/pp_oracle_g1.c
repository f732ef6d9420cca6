/* pp_oracle_g1.c -- CPU restatement of BLS12-381 G1 multi-scalar
 * multiplication (test infrastructure only: the tests and the benchmark's CPU
 * leg use it as the checker; the product never links it).
 *
 * Follows the reference's MSM contract (PLONK/utils/function.cu:395-411
 * multi_scalar_mult -> zkp/cuda/zksnark_msm.cu:48-88 msm_zkp_cuda with
 * mont = false): points are affine (x, y) over Fq in Montgomery form with
 * R = 2^384 (6 little-endian 64-bit limbs each, 96 bytes; all-zero is the
 * point at infinity), scalars are 4 little-endian 64-bit limbs read as plain
 * integers, and the result is sum_i scalars[i] * points[i].
 * Constants: q and R^2 mod q as in PLONK/utils/mont/cuda/ff/bls12-381.hpp
 * (BLS12_381_P, BLS12_381_RR); the curve is y^2 = x^3 + 4.
 *
 * Method: Jacobian coordinates, left-to-right double-and-add per point and
 * a sum over points (threads take disjoint point ranges), then one
 * conversion to affine.  Deliberately simple and independent of the GPU's
 * Pippenger. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#include "pp_oracle.h"

typedef unsigned __int128 u128;
typedef uint64_t u64;

static const u64 Q[6] = {0xb9feffffffffaaabULL, 0x1eabfffeb153ffffULL, 0x6730d2a0f6b0f624ULL,
                         0x64774b84f38512bfULL, 0x4b1ba7b6434bacd7ULL, 0x1a0111ea397fe69aULL};
static const u64 QINV = 0x89f3fffcfffcfffdULL; /* -q^-1 mod 2^64 */
static const u64 ONE[6] = {0x760900000002fffdULL, 0xebf4000bc40c0002ULL, 0x5f48985753c758baULL,
                           0x77ce585370525745ULL, 0x5c071a97a256ec6dULL, 0x15f65ec3fa80e493ULL};

typedef struct {
  u64 v[6];
} fq;
typedef struct {
  fq x, y, z; /* Jacobian: (X / Z^2, Y / Z^3); Z = 0 is infinity */
} g1j;

static int geq_q(const u64 a[6]) {
  for (int i = 5; i >= 0; --i)
    if (a[i] != Q[i]) return a[i] > Q[i];
  return 1;
}
static void sub_q(u64 a[6]) {
  u64 br = 0;
  for (int i = 0; i < 6; ++i) {
    u128 d = (u128)a[i] - Q[i] - br;
    a[i] = (u64)d;
    br = (u64)(d >> 64) & 1;
  }
}
static fq fadd(fq a, fq b) {
  fq r;
  u64 c = 0;
  for (int i = 0; i < 6; ++i) {
    u128 s = (u128)a.v[i] + b.v[i] + c;
    r.v[i] = (u64)s;
    c = (u64)(s >> 64);
  }
  if (geq_q(r.v)) sub_q(r.v); /* a + b < 2q < 2^384 */
  return r;
}
static fq fsub(fq a, fq b) {
  fq r;
  u64 br = 0;
  for (int i = 0; i < 6; ++i) {
    u128 d = (u128)a.v[i] - b.v[i] - br;
    r.v[i] = (u64)d;
    br = (u64)(d >> 64) & 1;
  }
  if (br) {
    u64 c = 0;
    for (int i = 0; i < 6; ++i) {
      u128 s = (u128)r.v[i] + Q[i] + c;
      r.v[i] = (u64)s;
      c = (u64)(s >> 64);
    }
  }
  return r;
}
/* Montgomery product a b R^-1 mod q (CIOS, 64-bit words) */
static fq fmul(fq a, fq b) {
  u64 t[8] = {0};
  for (int i = 0; i < 6; ++i) {
    u64 c = 0;
    for (int j = 0; j < 6; ++j) {
      u128 uv = (u128)a.v[j] * b.v[i] + t[j] + c;
      t[j] = (u64)uv;
      c = (u64)(uv >> 64);
    }
    u128 uv = (u128)t[6] + c;
    t[6] = (u64)uv;
    t[7] = (u64)(uv >> 64);
    const u64 m = t[0] * QINV;
    uv = (u128)m * Q[0] + t[0];
    c = (u64)(uv >> 64);
    for (int j = 1; j < 6; ++j) {
      uv = (u128)m * Q[j] + t[j] + c;
      t[j - 1] = (u64)uv;
      c = (u64)(uv >> 64);
    }
    uv = (u128)t[6] + c;
    t[5] = (u64)uv;
    t[6] = t[7] + (u64)(uv >> 64);
  }
  fq r;
  memcpy(r.v, t, 48);
  if (t[6] || geq_q(r.v)) sub_q(r.v);
  return r;
}
static int fzero(fq a) { return (a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5]) == 0; }
static int feq(fq a, fq b) { return memcmp(a.v, b.v, 48) == 0; }
static fq fone(void) {
  fq r;
  memcpy(r.v, ONE, 48);
  return r;
}
/* a^(q-2) */
static fq finv(fq a) {
  u64 e[6];
  memcpy(e, Q, 48);
  e[0] -= 2;
  fq r = fone();
  for (int w = 5; w >= 0; --w)
    for (int b = 63; b >= 0; --b) {
      r = fmul(r, r);
      if ((e[w] >> b) & 1) r = fmul(r, a);
    }
  return r;
}

static g1j j_inf(void) {
  g1j p;
  memset(&p, 0, sizeof p);
  p.y = fone();
  return p;
}
static int j_is_inf(const g1j *p) { return fzero(p->z); }

/* dbl-2009-l (a = 0) */
static g1j j_dbl(const g1j *p) {
  if (j_is_inf(p) || fzero(p->y)) return j_inf();
  fq A = fmul(p->x, p->x), B = fmul(p->y, p->y), C = fmul(B, B);
  fq t = fadd(p->x, B);
  fq D = fsub(fsub(fmul(t, t), A), C);
  D = fadd(D, D);
  fq E = fadd(fadd(A, A), A), F = fmul(E, E);
  g1j r;
  r.x = fsub(F, fadd(D, D));
  fq C8 = fadd(C, C);
  C8 = fadd(C8, C8);
  C8 = fadd(C8, C8);
  r.y = fsub(fmul(E, fsub(D, r.x)), C8);
  fq yz = fmul(p->y, p->z);
  r.z = fadd(yz, yz);
  return r;
}

/* add-2007-bl, with the doubling and inverse cases */
static g1j j_add(const g1j *p, const g1j *q) {
  if (j_is_inf(p)) return *q;
  if (j_is_inf(q)) return *p;
  fq Z1Z1 = fmul(p->z, p->z), Z2Z2 = fmul(q->z, q->z);
  fq U1 = fmul(p->x, Z2Z2), U2 = fmul(q->x, Z1Z1);
  fq S1 = fmul(fmul(p->y, q->z), Z2Z2), S2 = fmul(fmul(q->y, p->z), Z1Z1);
  if (feq(U1, U2)) {
    if (feq(S1, S2)) return j_dbl(p);
    return j_inf();
  }
  fq H = fsub(U2, U1);
  fq I = fadd(H, H);
  I = fmul(I, I);
  fq J = fmul(H, I);
  fq r = fsub(S2, S1);
  r = fadd(r, r);
  fq V = fmul(U1, I);
  g1j o;
  o.x = fsub(fsub(fmul(r, r), J), fadd(V, V));
  fq s1j = fmul(S1, J);
  o.y = fsub(fmul(r, fsub(V, o.x)), fadd(s1j, s1j));
  fq zs = fadd(p->z, q->z);
  o.z = fmul(fsub(fsub(fmul(zs, zs), Z1Z1), Z2Z2), H);
  return o;
}

static g1j j_from_affine(const u64 a[12]) {
  g1j p;
  memcpy(p.x.v, a, 48);
  memcpy(p.y.v, a + 6, 48);
  if (fzero(p.x) && fzero(p.y)) return j_inf();
  p.z = fone();
  return p;
}
static void j_to_affine(const g1j *p, u64 out[12]) {
  if (j_is_inf(p)) {
    memset(out, 0, 96);
    return;
  }
  fq zi = finv(p->z), zi2 = fmul(zi, zi);
  fq x = fmul(p->x, zi2), y = fmul(p->y, fmul(zi2, zi));
  memcpy(out, x.v, 48);
  memcpy(out + 6, y.v, 48);
}

static g1j j_mul(const g1j *p, const u64 s[4]) {
  g1j r = j_inf();
  for (int w = 3; w >= 0; --w)
    for (int b = 63; b >= 0; --b) {
      r = j_dbl(&r);
      if ((s[w] >> b) & 1) r = j_add(&r, p);
    }
  return r;
}

void or_g1_msm(const uint64_t *points, const uint64_t *scalars, uint64_t n, uint64_t out[12],
               int nthreads) {
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  g1j *part = (g1j *)malloc(sizeof(g1j) * (size_t)nt);
  for (int t = 0; t < nt; ++t) part[t] = j_inf();
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    g1j acc = j_inf();
#pragma omp for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const g1j p = j_from_affine(points + 12 * i);
      const g1j sp = j_mul(&p, scalars + 4 * i);
      acc = j_add(&acc, &sp);
    }
    part[t] = acc;
  }
  g1j sum = j_inf();
  for (int t = 0; t < nt; ++t) sum = j_add(&sum, &part[t]);
  free(part);
  j_to_affine(&sum, out);
}

void or_g1_mul_gen(const uint64_t *scalars, uint64_t n, uint64_t *out, int nthreads) {
  static const u64 G[12] = {0x5cb38790fd530c16ULL, 0x7817fc679976fff5ULL, 0x154f95c7143ba1c1ULL,
                            0xf0ae6acdf3d0e747ULL, 0xedce6ecc21dbf440ULL, 0x120177419e0bfb75ULL,
                            0xbaac93d50ce72271ULL, 0x8c22631a7918fd8eULL, 0xdd595f13570725ceULL,
                            0x51ac582950405194ULL, 0x0e1c8c3fad0059c0ULL, 0x0bbc3efc5008a26aULL};
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  const g1j g = j_from_affine(G);
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const g1j p = j_mul(&g, scalars + 4 * i);
    j_to_affine(&p, out + 12 * i);
  }
}

void or_g1_add(const uint64_t a[12], const uint64_t b[12], uint64_t out[12]) {
  const g1j p = j_from_affine(a), q = j_from_affine(b);
  const g1j r = j_add(&p, &q);
  j_to_affine(&r, out);
}
