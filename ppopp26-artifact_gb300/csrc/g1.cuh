// g1.cuh -- BLS12-381 G1 (y^2 = x^3 + 4 over Fq) in XYZZ coordinates for
// the multi-scalar multiplication.
//
// A point (X, Y, ZZ, ZZZ) stands for the affine (X / ZZ, Y / ZZZ), with
// ZZ^3 = ZZZ^2; ZZ = 0 is the point at infinity.  Additions use the
// "add-2008-s" / "madd-2008-s" and doublings the "dbl-2008-s-1" formulas of
// the Explicit-Formulas Database (a = 0), with the equal-x cases handled
// explicitly.  Affine points are the reference's layout: x then y, all zero
// for infinity (PLONK/utils/zkp/cuda/zksnark_msm.cu:15-45, affine_t).
#pragma once
#include "fq.cuh"

namespace pp {

struct g1a {
  fq x, y;
};
struct g1x {
  fq x, y, zz, zzz;
};

// The group's standard generator, affine, Montgomery form (32-bit limbs, least
// significant first): the point blst calls BLS12_381_G1, which the MSM tests
// compare it with.
PP_HD g1a g1_generator() {
  return g1a{{{0xfd530c16u, 0x5cb38790u, 0x9976fff5u, 0x7817fc67u, 0x143ba1c1u, 0x154f95c7u,
                0xf3d0e747u, 0xf0ae6acdu, 0x21dbf440u, 0xedce6eccu, 0x9e0bfb75u, 0x12017741u}},
             {{0x0ce72271u, 0xbaac93d5u, 0x7918fd8eu, 0x8c22631au, 0x570725ceu, 0xdd595f13u,
                0x50405194u, 0x51ac5829u, 0xad0059c0u, 0x0e1c8c3fu, 0x5008a26au, 0x0bbc3efcu}}};
}

PP_HD g1x g1x_inf() {
  g1x p;
  p.x = fq_one();
  p.y = fq_one();
  p.zz = fq_zero();
  p.zzz = fq_zero();
  return p;
}
PP_HD bool g1x_is_inf(const g1x &p) { return fq_is_zero(p.zz); }
PP_HD bool g1a_is_inf(const g1a &p) { return fq_is_zero(p.x) && fq_is_zero(p.y); }

PP_HD g1a g1a_neg(const g1a &p) {
  g1a r = p;
  if (!g1a_is_inf(p)) r.y = fq_neg(p.y);
  return r;
}

PP_HD g1x g1x_from_affine(const g1a &p) {
  if (g1a_is_inf(p)) return g1x_inf();
  g1x r;
  r.x = p.x;
  r.y = p.y;
  r.zz = fq_one();
  r.zzz = fq_one();
  return r;
}

// 2P
PP_HD g1x g1x_dbl(const g1x &p) {
  if (g1x_is_inf(p) || fq_is_zero(p.y)) return g1x_inf();
  const fq u = fq_dbl(p.y);
  const fq v = fq_sqr(u);
  const fq w = fq_mul(u, v);
  const fq s = fq_mul(p.x, v);
  const fq x2 = fq_sqr(p.x);
  const fq m = fq_add(fq_dbl(x2), x2);
  g1x r;
  r.x = fq_sub(fq_sqr(m), fq_dbl(s));
  r.y = fq_sub(fq_mul(m, fq_sub(s, r.x)), fq_mul(w, p.y));
  r.zz = fq_mul(v, p.zz);
  r.zzz = fq_mul(w, p.zzz);
  return r;
}

// 2P for an affine P (ZZ = ZZZ = 1)
PP_HD g1x g1x_dbl_affine(const g1a &p) {
  if (g1a_is_inf(p) || fq_is_zero(p.y)) return g1x_inf();
  const fq u = fq_dbl(p.y);
  const fq v = fq_sqr(u);
  const fq w = fq_mul(u, v);
  const fq s = fq_mul(p.x, v);
  const fq x2 = fq_sqr(p.x);
  const fq m = fq_add(fq_dbl(x2), x2);
  g1x r;
  r.x = fq_sub(fq_sqr(m), fq_dbl(s));
  r.y = fq_sub(fq_mul(m, fq_sub(s, r.x)), fq_mul(w, p.y));
  r.zz = v;
  r.zzz = w;
  return r;
}

// P + Q, Q affine
PP_HD g1x g1x_add_affine(const g1x &p, const g1a &q) {
  if (g1a_is_inf(q)) return p;
  if (g1x_is_inf(p)) return g1x_from_affine(q);
  const fq u2 = fq_mul(q.x, p.zz);
  const fq s2 = fq_mul(q.y, p.zzz);
  const fq P = fq_sub(u2, p.x);
  const fq R = fq_sub(s2, p.y);
  if (fq_is_zero(P)) return fq_is_zero(R) ? g1x_dbl_affine(q) : g1x_inf();
  const fq pp = fq_sqr(P);
  const fq ppp = fq_mul(P, pp);
  const fq Q = fq_mul(p.x, pp);
  g1x r;
  r.x = fq_sub(fq_sub(fq_sqr(R), ppp), fq_dbl(Q));
  r.y = fq_sub(fq_mul(R, fq_sub(Q, r.x)), fq_mul(p.y, ppp));
  r.zz = fq_mul(p.zz, pp);
  r.zzz = fq_mul(p.zzz, ppp);
  return r;
}

// P + Q
PP_HD g1x g1x_add(const g1x &p, const g1x &q) {
  if (g1x_is_inf(q)) return p;
  if (g1x_is_inf(p)) return q;
  const fq u1 = fq_mul(p.x, q.zz);
  const fq u2 = fq_mul(q.x, p.zz);
  const fq s1 = fq_mul(p.y, q.zzz);
  const fq s2 = fq_mul(q.y, p.zzz);
  const fq P = fq_sub(u2, u1);
  const fq R = fq_sub(s2, s1);
  if (fq_is_zero(P)) return fq_is_zero(R) ? g1x_dbl(p) : g1x_inf();
  const fq pp = fq_sqr(P);
  const fq ppp = fq_mul(P, pp);
  const fq Q = fq_mul(u1, pp);
  g1x r;
  r.x = fq_sub(fq_sub(fq_sqr(R), ppp), fq_dbl(Q));
  r.y = fq_sub(fq_mul(R, fq_sub(Q, r.x)), fq_mul(s1, ppp));
  r.zz = fq_mul(fq_mul(p.zz, q.zz), pp);
  r.zzz = fq_mul(fq_mul(p.zzz, q.zzz), ppp);
  return r;
}

// 2^k P
PP_HD g1x g1x_dbl_n(g1x p, uint32_t k) {
  for (uint32_t i = 0; i < k; ++i) p = g1x_dbl(p);
  return p;
}

// affine (x, y) = (X / ZZ, Y / ZZZ) with one inversion; infinity -> all zero
PP_HD g1a g1x_to_affine(const g1x &p) {
  g1a r;
  if (g1x_is_inf(p)) {
    r.x = fq_zero();
    r.y = fq_zero();
    return r;
  }
  const fq t = fq_inv_fast(fq_mul(p.zz, p.zzz));  // 1 / (ZZ ZZZ)
  r.x = fq_mul(p.x, fq_mul(t, p.zzz));        // X / ZZ
  r.y = fq_mul(p.y, fq_mul(t, p.zz));         // Y / ZZZ
  return r;
}

}  // namespace pp
