// modinv.cuh -- modular inverse by Bernstein-Yang divsteps ("Fast
// constant-time gcd computation and modular inversion", D. J. Bernstein and
// B.-Y. Yang, TCHES 2019), in the variable-time form: runs of zero low bits
// of g are skipped at once, and the loop ends as soon as g is 0.  Variable
// time is fine here (public prover data).
//
// divstep(delta, f, g), f odd:
//   delta > 0 and g odd:  (1 - delta, g, (g - f) / 2)
//   g odd:                (1 + delta, f, (g + f) / 2)
//   g even:               (1 + delta, f, g / 2)
// Starting from (1, M, x) it reaches g = 0 with f = +-gcd(M, x) = +-1 within
// floor((49 * 256 + 57) / 17) = 741 steps for 256-bit inputs, and within
// 1101 for 381-bit ones.
//
// B divsteps depend only on the low B + 2 bits of f and g, so they run on
// one machine word each and record a 2x2 integer matrix T with
// 2^B [f', g'] = T [f, g]; |u| + |v| <= 2^B and |q| + |r| <= 2^B.  T is then
// applied to the full f, g (the division by 2^B is exact) and to the pair
// d, e with f = d x, g = e x (mod M), where the division by 2^B is done mod
// M by first adding the multiple of M that clears the low B bits.
//
// Numbers are NL limbs of B bits, least significant first; limbs below the
// top one are in [0, 2^B) and the top limb carries the sign.  Two widths:
// B = 30 on 32-bit words with 64-bit sums (the GPU form: every limb product
// is one 32 x 32 -> 64-bit multiply-add) and B = 62 on 64-bit words with
// 128-bit sums (a 64-bit host CPU's form).  Measured on a GB300 (ns per
// Fr inversion, 9728 warps):
//                         30-bit   62-bit   binary GCD
//   warp-uniform            21.5     30.5       37.6
//   one per lane             1.0      1.6        4.6
//   one thread (latency)   34.8 us  41.8 us    54.0 us
#pragma once
#include <cstdint>

namespace pp {

template <typename L>
struct LimbTraits;
template <>
struct LimbTraits<int32_t> {
  using U = uint32_t;
  using A = int64_t;  // sums of limb products
  static constexpr int B = 30;
};
template <>
struct LimbTraits<int64_t> {
  using U = uint64_t;
  using A = __int128;
  static constexpr int B = 62;
};

template <typename L, int NL>
struct SLimbs {
  L l[NL];
};

// modulus in B-bit limbs and M^-1 mod 2^B
template <typename L, int NL>
struct ModulusB {
  L m[NL];
  typename LimbTraits<L>::U inv;
};

PP_HD int ctz_word(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}
PP_HD int ctz_word(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __ffsll((long long)x) - 1;
#else
  return __builtin_ctzll(x);
#endif
}

// ---- B divsteps on the low words.  Returns the updated delta; T in u..r.
template <typename L>
PP_HD int divsteps_word(int delta, typename LimbTraits<L>::U f0, typename LimbTraits<L>::U g0,
                        L &u_out, L &v_out, L &q_out, L &r_out) {
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
  L u = 1, v = 0, q = 0, r = 1;
  int i = 0;
  while (i < B) {
    if (!(g0 & 1)) {
      // a run of zero bits: g / 2^z and the f row times 2^z
      int z = g0 ? ctz_word(g0) : B;
      if (z > B - i) z = B - i;
      g0 >>= z;
      u = (L)((U)u << z);
      v = (L)((U)v << z);
      delta += z;
      i += z;
      continue;
    }
    if (delta > 0) {
      const U nf = g0;
      g0 = (g0 - f0) >> 1;
      f0 = nf;
      const L nu = (L)(2 * q), nv = (L)(2 * r);
      q -= u;
      r -= v;
      u = nu;
      v = nv;
      delta = 1 - delta;
    } else {
      g0 = (g0 + f0) >> 1;
      q += u;
      r += v;
      u = (L)(2 * u);
      v = (L)(2 * v);
      delta += 1;
    }
    ++i;
  }
  u_out = u;
  v_out = v;
  q_out = q;
  r_out = r;
  return delta;
}

// [f, g] = T [f, g] / 2^B (exact)
template <typename L, int NL>
PP_HD void apply_fg(SLimbs<L, NL> &f, SLimbs<L, NL> &g, L u, L v, L q, L r) {
  using A = typename LimbTraits<L>::A;
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
  constexpr U MASK = ((U)1 << B) - 1;
  A cf = (A)u * f.l[0] + (A)v * g.l[0];
  A cg = (A)q * f.l[0] + (A)r * g.l[0];
  cf >>= B;
  cg >>= B;
#pragma unroll
  for (int i = 1; i < NL; ++i) {
    cf += (A)u * f.l[i] + (A)v * g.l[i];
    cg += (A)q * f.l[i] + (A)r * g.l[i];
    f.l[i - 1] = (L)((U)cf & MASK);
    g.l[i - 1] = (L)((U)cg & MASK);
    cf >>= B;
    cg >>= B;
  }
  f.l[NL - 1] = (L)cf;
  g.l[NL - 1] = (L)cg;
}

// x in (-M, 2M) -> [0, M)
template <typename L, int NL>
PP_HD void normalize_mod(SLimbs<L, NL> &x, const ModulusB<L, NL> &M) {
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
  constexpr U MASK = ((U)1 << B) - 1;
  int sgn = x.l[NL - 1] < 0 ? -1 : 0;
  if (!sgn) {
    // x >= M ?
    bool ge = true;
    for (int i = NL - 1; i >= 0; --i)
      if (x.l[i] != M.m[i]) {
        ge = x.l[i] > M.m[i];
        break;
      }
    if (ge) sgn = 1;
  }
  if (!sgn) return;
  L c = 0;
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    c += x.l[i] + (sgn < 0 ? M.m[i] : -M.m[i]);
    if (i < NL - 1) {
      x.l[i] = (L)((U)c & MASK);
      c >>= B;
    } else {
      x.l[i] = c;
    }
  }
}

// [d, e] = T [d, e] / 2^B mod M, d and e in [0, M)
template <typename L, int NL>
PP_HD void apply_de(SLimbs<L, NL> &d, SLimbs<L, NL> &e, L u, L v, L q, L r,
                    const ModulusB<L, NL> &M) {
  using A = typename LimbTraits<L>::A;
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
  constexpr U MASK = ((U)1 << B) - 1;
  A cd = (A)u * d.l[0] + (A)v * e.l[0];
  A ce = (A)q * d.l[0] + (A)r * e.l[0];
  // the multiples of M that clear the low B bits
  const U md = (U)(0 - (U)cd * M.inv) & MASK;
  const U me = (U)(0 - (U)ce * M.inv) & MASK;
  cd += (A)md * M.m[0];
  ce += (A)me * M.m[0];
  cd >>= B;
  ce >>= B;
#pragma unroll
  for (int i = 1; i < NL; ++i) {
    cd += (A)u * d.l[i] + (A)v * e.l[i] + (A)md * M.m[i];
    ce += (A)q * d.l[i] + (A)r * e.l[i] + (A)me * M.m[i];
    d.l[i - 1] = (L)((U)cd & MASK);
    e.l[i - 1] = (L)((U)ce & MASK);
    cd >>= B;
    ce >>= B;
  }
  d.l[NL - 1] = (L)cd;
  e.l[NL - 1] = (L)ce;
  normalize_mod(d, M);
  normalize_mod(e, M);
}

template <typename L, int NL>
PP_HD bool is_zero_limbs(const SLimbs<L, NL> &x) {
  L o = 0;
#pragma unroll
  for (int i = 0; i < NL; ++i) o |= x.l[i];
  return o == 0;
}

// x^-1 mod M for 0 <= x < M, M an odd prime; 0 -> 0.  max_batches bounds the
// loop: it must cover the divstep bound of the modulus's size (741 for
// 256-bit inputs, 1101 for 381-bit ones) in batches of B.  An input that does
// not finish within them (not below M) gives 0.
template <typename L, int NL>
PP_HD SLimbs<L, NL> modinv_divsteps(const SLimbs<L, NL> &x, const ModulusB<L, NL> &M,
                                    int max_batches) {
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
  SLimbs<L, NL> f, g, d, e;
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    f.l[i] = M.m[i];
    g.l[i] = x.l[i];
    d.l[i] = 0;
    e.l[i] = 0;
  }
  e.l[0] = 1;
  if (is_zero_limbs(g)) return d;
  int delta = 1;
  bool done = false;
  for (int b = 0; b < max_batches && !done; ++b) {
    L u, v, q, r;
    const U f0 = (U)f.l[0] | ((U)f.l[1] << B);
    const U g0 = (U)g.l[0] | ((U)g.l[1] << B);
    delta = divsteps_word<L>(delta, f0, g0, u, v, q, r);
    apply_fg(f, g, u, v, q, r);
    apply_de(d, e, u, v, q, r, M);
    done = is_zero_limbs(g);
  }
  if (!done) {
#pragma unroll
    for (int i = 0; i < NL; ++i) d.l[i] = 0;
    return d;
  }
  // f = +-1: x^-1 = +-d
  if (f.l[NL - 1] < 0 && !is_zero_limbs(d)) {
    constexpr U MASK = ((U)1 << B) - 1;
    L c = 0;
#pragma unroll
    for (int i = 0; i < NL; ++i) {
      c += M.m[i] - d.l[i];
      if (i < NL - 1) {
        d.l[i] = (L)((U)c & MASK);
        c >>= B;
      } else {
        d.l[i] = c;
      }
    }
  }
  return d;
}

// 32-bit words <-> B-bit limbs (non-negative values)
template <typename L, int NW, int NL>
PP_HD SLimbs<L, NL> words_to_limbs(const uint32_t w[NW]) {
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
  constexpr int UB = 8 * (int)sizeof(U);
  SLimbs<L, NL> x;
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    U acc = 0;
    const int bit = B * i;
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // a limb of at most 62 bits spans at most 3 words
      const int wi = bit / 32 + k;
      if (wi < NW) {
        const int sh = wi * 32 - bit;  // word wi's position within the limb
        const U wv = w[wi];
        if (sh >= 0) {
          if (sh < UB) acc |= wv << sh;
        } else {
          acc |= wv >> (-sh);
        }
      }
    }
    x.l[i] = (L)(acc & (((U)1 << B) - 1));
  }
  return x;
}

template <typename L, int NW, int NL>
PP_HD void limbs_to_words(const SLimbs<L, NL> &x, uint32_t w[NW]) {
  using U = typename LimbTraits<L>::U;
  constexpr int B = LimbTraits<L>::B;
#pragma unroll
  for (int k = 0; k < NW; ++k) {
    const int bit = 32 * k;
    const int li = bit / B, sh = bit % B;
    uint64_t v = (uint64_t)((U)x.l[li] >> sh);
    // bits of the next limb(s) above position B - sh
    if (li + 1 < NL && B - sh < 32) v |= (uint64_t)(U)x.l[li + 1] << (B - sh);
    if (li + 2 < NL && 2 * B - sh < 32) v |= (uint64_t)(U)x.l[li + 2] << (2 * B - sh);
    w[k] = (uint32_t)v;
  }
}

}  // namespace pp
