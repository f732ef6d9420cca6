// ntt.cu -- in-HBM multi-pass NTT over Fr for sm_103a.
//
// Structure (GB300-first, not the reference's 3-kernel CT layout):
//  * A transform of 2^L points is split into P passes of 2^k_p-point
//    sub-transforms (k_p <= 11), the four-step / Stockham factorisation
//    N = R_1 * R_2 * ... * R_P.  Pass p runs, for every prefix of already
//    transformed digits and every column c < S_p = R_{p+1}..R_P, an R_p-point
//    DFT over the elements at stride S_p, multiplies output k by the layer
//    twiddle w_{R_p S_p}^(c k) and stores it in place; the last pass writes
//    the digit-reversed (natural) output order directly, so no bit-reversal
//    kernel and no uncoalesced swap pass is needed.
//  * A thread block owns a tile of R_p x T_p elements (R_p * T_p <= 2048,
//    64 KiB of shared memory, XOR-swizzled 16-byte units); T_p adjacent
//    columns give >= 128-byte contiguous row segments for coalesced HBM
//    access.  Inside the tile each column's DFT runs as radix-8 rounds held in
//    registers (8 elements per thread), with a final radix-4/2 round.
//  * Every Montgomery multiply is on the integer pipe; the transform is
//    compute-bound (~11 multiplies per element at 2^24 against 3 HBM passes),
//    so the inter-pass twiddles are read from HBM tables (one load instead of
//    a multiply), and inverse transforms fold 2^-L into the first layer table.
//
// Reference behaviour restated: natural order in and out, w_N =
// forward_roots_of_unity[lg N] = 7^((r-1)/N) (PLONK/utils/zkp/cuda/
// zksnark_ntt/parameters/bls12_381.h:29-83), inverse scaled by N^-1
// (ct_mixed_radix_wide.cuh:173-176).
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "ntt.cuh"

namespace pp {

// ------------------------------------------------------------------ host math
static fr host_pow_limbs(const fr &a, const uint32_t e[8]) {
  fr acc = fr_one();
  bool started = false;
  for (int w = 7; w >= 0; --w)
    for (int b = 31; b >= 0; --b) {
      if (started) acc = fr_sqr(acc);
      if ((e[w] >> b) & 1) {
        acc = started ? fr_mul(acc, a) : a;
        started = true;
      }
    }
  return acc;
}

fr host_mont_small(uint64_t x) {
  fr t = fr_zero();
  t.v[0] = (uint32_t)x;
  t.v[1] = (uint32_t)(x >> 32);
  return fr_mul(t, fr_rr());
}
fr host_pow(const fr &a, uint64_t e) { return fr_pow_u64(a, e); }
fr host_inv(const fr &a) { return fr_inv(a); }

fr host_root_of_unity(int lg, bool inverse) {
  static std::once_flag once;
  static fr fwd[33], inv[33];
  std::call_once(once, [] {
    // (r - 1) >> 32, 32-bit limbs
    const uint32_t e[8] = {0xffffffffu, PP_R2, PP_R3, PP_R4, PP_R5, PP_R6, PP_R7, 0u};
    fwd[32] = host_pow_limbs(host_mont_small(7), e);
    for (int k = 31; k >= 0; --k) fwd[k] = fr_sqr(fwd[k + 1]);
    for (int k = 0; k <= 32; ++k) inv[k] = fr_inv(fwd[k]);
  });
  return inverse ? inv[lg] : fwd[lg];
}

// ------------------------------------------------------------- device code
__device__ __forceinline__ uint32_t swz(uint32_t u) {
  const uint32_t x = u >> 3;
  return u ^ ((x ^ (x >> 3) ^ (x >> 6) ^ (x >> 9)) & 7u);
}

struct SmemTile {
  uint4 *s;
  uint32_t lgT;
  __device__ __forceinline__ fr get(uint32_t row, uint32_t col) const {
    const uint32_t u = ((row << lgT) + col) << 1;
    const uint4 a = s[swz(u)], b = s[swz(u + 1)];
    return fr{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
  }
  __device__ __forceinline__ void put(uint32_t row, uint32_t col, const fr &v) const {
    const uint32_t u = ((row << lgT) + col) << 1;
    s[swz(u)] = make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
    s[swz(u + 1)] = make_uint4(v.v[4], v.v[5], v.v[6], v.v[7]);
  }
};

// Inside a transform values are kept below 2r (fr_*_lazy); the last round of
// the last pass makes them canonical before they leave the kernel.
__device__ __forceinline__ void bfly(fr &a, fr &b) {
  const fr t = a;
  a = fr_add_lazy(t, b);
  b = fr_sub_lazy(t, b);
}

// 8-point DFT, decimation in frequency; afterwards x[i] = X[bitrev3(i)]
__device__ __forceinline__ void dft8(fr x[8], const fr &w1, const fr &w2, const fr &w3) {
  bfly(x[0], x[4]);
  bfly(x[1], x[5]);
  bfly(x[2], x[6]);
  bfly(x[3], x[7]);
  x[5] = fr_mul_twiddle(x[5], w1);
  x[6] = fr_mul_twiddle(x[6], w2);
  x[7] = fr_mul_twiddle(x[7], w3);
  bfly(x[0], x[2]);
  bfly(x[1], x[3]);
  bfly(x[4], x[6]);
  bfly(x[5], x[7]);
  x[3] = fr_mul_twiddle(x[3], w2);
  x[7] = fr_mul_twiddle(x[7], w2);
  bfly(x[0], x[1]);
  bfly(x[2], x[3]);
  bfly(x[4], x[5]);
  bfly(x[6], x[7]);
}

__device__ __forceinline__ uint32_t digit_reverse(uint32_t o, uint32_t lgR) {
  uint32_t rem = lgR, p = 0, t = o;
  while (rem > 0) {
    const uint32_t lgr = rem >= 3 ? 3 : rem;
    const uint32_t k = t & ((1u << lgr) - 1);
    t >>= lgr;
    rem -= lgr;
    p += k << rem;
  }
  return p;
}

// w_{R S}^(o c) from the split tables (both canonical, so the product is)
__device__ __forceinline__ fr split_layer_twiddle(const PassArgs &a, uint32_t o, uint64_t c) {
  const uint64_t e = (uint64_t)o * c;
  return fr_mul(ldg_fr(a.tw_hi + (e >> a.tw_lgh)), ldg_fr(a.tw_lo + (e & ((1ull << a.tw_lgh) - 1))));
}

// One tile of one pass.  The block may be wider than the tile needs (batched
// launches use 256 threads for every job); surplus threads only join the
// barriers.
template <bool HOSTIO>
__device__ __forceinline__ void ntt_tile(const PassArgs &a, const uint64_t tileid, uint4 *sm) {
  // HOSTIO = false compiles out the host-endpoint paths (unit_in, unit_out);
  // every pass is still correct without them, with element-wise accesses
  const bool unit_in = HOSTIO && a.unit_in, unit_out = HOSTIO && a.unit_out;
  const SmemTile tile{sm, a.lgT};
  const uint32_t R = 1u << a.lgR, T = 1u << a.lgT, E = R << a.lgT;
  const uint32_t nthr = E >> 3;
  const uint32_t tid = threadIdx.x;
  const bool active = tid < nthr;

  uint64_t base = 0, col0 = 0, in_base = 0, out_base = 0;
  uint32_t lgS1 = 0;
  if (!a.last) {
    const uint32_t lgtpq = a.lgS - a.lgT;
    const uint64_t q = tileid >> lgtpq, ct = tileid & ((1ull << lgtpq) - 1);
    col0 = ct << a.lgT;
    base = (q << (a.lgR + a.lgS)) + col0;
  } else if (a.P > 1) {
    const uint32_t lgR1 = a.lgRp[0];
    lgS1 = a.lgN - lgR1;
    const uint32_t lgkb = lgR1 - a.lgT;
    const uint64_t kb = tileid & ((1ull << lgkb) - 1), rest = tileid >> lgkb;
    uint64_t rin = 0, r = rest;
    uint32_t acc = lgR1;
    for (uint32_t j = 1; j + 1 < a.P; ++j) {
      const uint32_t bits = a.lgRp[j];
      acc += bits;
      rin += (r & ((1ull << bits) - 1)) << (a.lgN - acc);
      r >>= bits;
    }
    in_base = ((kb << a.lgT) << lgS1) + rin;
    out_base = (kb << a.lgT) + (rest << lgR1);
  }

  // ---- load the tile (coalesced) into shared memory.  A host-memory input
  // without a multiply on the way in moves 16-byte halves, so one warp
  // instruction reads whole 128-byte lines; a thread's 16 loads issue in two
  // groups of eight before their shared-memory stores, so it waits on host
  // memory twice per tile instead of sixteen times.
  auto tile_src = [&](uint32_t e, uint32_t &n, uint32_t &col) -> uint64_t {
    if (!a.last) {
      n = e >> a.lgT;
      col = e & (T - 1);
      return base + ((uint64_t)n << a.lgS) + col;
    }
    if (a.P == 1) {
      n = e;
      col = 0;
      return n;
    }
    n = e & (R - 1);
    col = e >> a.lgR;
    return in_base + ((uint64_t)col << lgS1) + n;
  };
  if (unit_in && !(a.first && a.in_kind == NTT_IN_DIAG)) {
    const uint4 zero4 = make_uint4(0, 0, 0, 0);
    if (active) {
#pragma unroll
      for (uint32_t k0 = 0; k0 < 16; k0 += 8) {
        uint4 v[8];
        uint32_t dst[8];
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) {
          const uint32_t u = tid + (k0 + i) * nthr;
          const uint32_t e = u >> 1, h = u & 1;
          uint32_t n, col;
          const uint64_t g = tile_src(e, n, col);
          dst[i] = swz((((n << a.lgT) + col) << 1) + h);
          v[i] = zero4;
          if (!a.first) {
            v[i] = __ldcs(reinterpret_cast<const uint4 *>(a.in + g) + h);
          } else if (a.in_kind == NTT_IN_SPREAD) {
            if ((g & ((1ull << a.spread) - 1)) == 0)
              v[i] = __ldcs(reinterpret_cast<const uint4 *>(a.in + (g >> a.spread)) + h);
          } else if (g < a.n_valid) {
            v[i] = __ldcs(reinterpret_cast<const uint4 *>(a.in + g) + h);
          }
        }
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) tile.s[dst[i]] = v[i];
      }
    }
  } else {
    for (uint32_t e = tid; active && e < E; e += nthr) {
      uint32_t n, col;
      uint64_t g;
      if (!a.last) {
        n = e >> a.lgT;
        col = e & (T - 1);
        g = base + ((uint64_t)n << a.lgS) + col;
      } else if (a.P == 1) {
        n = e;
        col = 0;
        g = n;
      } else {
        n = e & (R - 1);
        col = e >> a.lgR;
        g = in_base + ((uint64_t)col << lgS1) + n;
      }
      fr v;
      if (a.first) {
        if (a.in_kind == NTT_IN_SPREAD) {
          v = (g & ((1ull << a.spread) - 1)) == 0 ? ldcs_fr(a.in + (g >> a.spread)) : fr_zero();
        } else if (g < a.n_valid) {
          v = ldcs_fr(a.in + g);
          if (a.in_kind == NTT_IN_DIAG) {
            const fr d = a.diag_hi ? fr_mul(ldg_fr(a.diag + (g & ((1ull << a.diag_lgh) - 1))),
                                            ldg_fr(a.diag_hi + (g >> a.diag_lgh)))
                                   : ldcs_fr(a.diag + g);
            v = fr_mul_twiddle(v, d);
          }
        } else {
          v = fr_zero();
        }
      } else {
        v = ldcs_fr(a.in + g);
      }
      tile.put(n, col, v);
    }
  }
  __syncthreads();

  // ---- column DFTs: radix-8 rounds, final radix-4/2 round
  {
    const uint32_t lgcpt = a.lgR - 3;
    const uint32_t col = tid >> lgcpt, d = tid & ((1u << lgcpt) - 1);
    uint32_t lgP = 0, rem = a.lgR;
    while (rem > 0) {
      const uint32_t lgr = rem >= 3 ? 3 : rem;
      const uint32_t lgSj = rem - lgr;
      if (!active) {
        // surplus thread of a wider block: barriers only
      } else if (lgr == 3) {
        const uint32_t c = d & ((1u << lgSj) - 1), prefix = d >> lgSj;
        const uint32_t pb = (prefix << (lgSj + 3)) + c;
        fr x[8];
        const fr w1 = ldg_fr(a.tw_inner + (R >> 3));
        const fr w2 = ldg_fr(a.tw_inner + (R >> 2));
        const fr w3 = ldg_fr(a.tw_inner + 3 * (R >> 3));
        if (lgP == 0 && a.zero_lg >= 3) {
          // first round over zero padding: only x[0] can be non-zero, and the
          // 8-point DFT of (x0, 0, ..., 0) is x0 in every output
          x[0] = tile.get(pb, col);
#pragma unroll
          for (int i = 1; i < 8; ++i) x[i] = x[0];
        } else if (lgP == 0 && a.zero_lg == 2) {
          // only x[0], x[1] can be non-zero: X[k] = x0 + x1 w^k, w^4 = -1,
          // stored bit-reversed like dft8 (x[i] = X[bitrev3(i)])
          const fr x0 = tile.get(pb, col), x1 = tile.get(pb + (1u << lgSj), col);
          const fr t1 = fr_mul_twiddle(x1, w1), t2 = fr_mul_twiddle(x1, w2), t3 = fr_mul_twiddle(x1, w3);
          x[0] = fr_add_lazy(x0, x1);
          x[1] = fr_sub_lazy(x0, x1);
          x[2] = fr_add_lazy(x0, t2);
          x[3] = fr_sub_lazy(x0, t2);
          x[4] = fr_add_lazy(x0, t1);
          x[5] = fr_sub_lazy(x0, t1);
          x[6] = fr_add_lazy(x0, t3);
          x[7] = fr_sub_lazy(x0, t3);
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) x[i] = tile.get(pb + ((uint32_t)i << lgSj), col);
          dft8(x, w1, w2, w3);
        }
        // x[i] holds output k = bitrev3(i)
        if (lgSj > 0) {
#pragma unroll
          for (int i = 1; i < 8; ++i) {
            const uint32_t k = ((i & 1) << 2) | (i & 2) | ((i >> 2) & 1);
            x[i] = fr_mul_twiddle(x[i], ldg_fr(a.tw_inner + ((c * k) << lgP)));
          }
        } else if (a.last && unit_out) {
          // the 16-byte store path copies tile words: canonical here
#pragma unroll
          for (int i = 0; i < 8; ++i) x[i] = fr_canon(x[i]);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint32_t k = ((i & 1) << 2) | (i & 2) | ((i >> 2) & 1);
          tile.put(pb + (k << lgSj), col, x[i]);
        }
      } else {
        // last round (S = 1): this thread owns positions 8d .. 8d+7
        fr x[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = tile.get((d << 3) + i, col);
        if (lgr == 2) {
          const fr w4 = ldg_fr(a.tw_inner + (R >> 2));
#pragma unroll
          for (int h = 0; h < 8; h += 4) {
            bfly(x[h + 0], x[h + 2]);
            bfly(x[h + 1], x[h + 3]);
            x[h + 3] = fr_mul_twiddle(x[h + 3], w4);
            bfly(x[h + 0], x[h + 1]);
            bfly(x[h + 2], x[h + 3]);
            const fr t = x[h + 1];  // bit-reversed -> natural
            x[h + 1] = x[h + 2];
            x[h + 2] = t;
          }
        } else {
#pragma unroll
          for (int h = 0; h < 8; h += 2) bfly(x[h], x[h + 1]);
        }
        if (a.last && unit_out) {
#pragma unroll
          for (int i = 0; i < 8; ++i) x[i] = fr_canon(x[i]);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) tile.put((d << 3) + i, col, x[i]);
      }
      __syncthreads();
      lgP += lgr;
      rem -= lgr;
    }
  }

  // ---- store (coalesced), with the layer twiddle or the final scale.  A
  // host-memory output without a scale moves 16-byte halves, so one warp
  // instruction writes whole 128-byte lines (partial lines cost C2C bandwidth).
  if (a.last && unit_out && !a.has_post_scale) {
    for (uint32_t u = tid; active && u < 2 * E; u += nthr) {
      const uint32_t e = u >> 1, h = u & 1;
      uint32_t o, col;
      if (a.P == 1) {
        o = e;
        col = 0;
      } else {
        o = e >> a.lgT;
        col = e & (T - 1);
      }
      const uint4 v = tile.s[swz((((digit_reverse(o, a.lgR) << a.lgT) + col) << 1) + h)];
      const uint64_t g =
          a.P == 1 ? (uint64_t)o : out_base + col + ((uint64_t)o << (a.lgN - a.lgR));
      reinterpret_cast<uint4 *>(a.out + g)[h] = v;
    }
    return;
  }
  if (!a.last && unit_out) {
    // host output of an intermediate pass: the layer twiddles go into the
    // tile first, then whole 128-byte lines leave it
    if (a.tw_layer || a.tw_lo) {
      for (uint32_t e = tid; active && e < E; e += nthr) {
        const uint32_t o = e >> a.lgT, col = e & (T - 1), r = digit_reverse(o, a.lgR);
        const fr w = a.tw_layer ? ldcs_fr(a.tw_layer + ((uint64_t)o << a.lgS) + col0 + col)
                                : split_layer_twiddle(a, o, col0 + col);
        tile.put(r, col, fr_mul_twiddle(tile.get(r, col), w));
      }
      __syncthreads();
    }
    for (uint32_t u = tid; active && u < 2 * E; u += nthr) {
      const uint32_t e = u >> 1, h = u & 1;
      const uint32_t o = e >> a.lgT, col = e & (T - 1);
      const uint4 v = tile.s[swz((((digit_reverse(o, a.lgR) << a.lgT) + col) << 1) + h)];
      reinterpret_cast<uint4 *>(a.out + base + ((uint64_t)o << a.lgS) + col)[h] = v;
    }
    return;
  }
  for (uint32_t e = tid; active && e < E; e += nthr) {
    uint32_t o, col;
    if (a.P == 1) {
      o = e;
      col = 0;
    } else {
      o = e >> a.lgT;
      col = e & (T - 1);
    }
    fr v = tile.get(digit_reverse(o, a.lgR), col);
    if (!a.last) {
      if (a.tw_layer) v = fr_mul_twiddle(v, ldcs_fr(a.tw_layer + ((uint64_t)o << a.lgS) + col0 + col));
      else if (a.tw_lo) v = fr_mul_twiddle(v, split_layer_twiddle(a, o, col0 + col));
      st_fr(a.out + base + ((uint64_t)o << a.lgS) + col, v);
    } else {
      v = fr_canon(v);  // one element at a time here, not 8 live in the last round
      if (a.has_post_scale) v = fr_mul(v, a.post_scale);
      const uint64_t g =
          a.P == 1 ? (uint64_t)o : out_base + col + ((uint64_t)o << (a.lgN - a.lgR));
      st_fr(a.out + g, v);
    }
  }
}

#ifndef PP_NTT_MINB
#define PP_NTT_MINB 2  // blocks per SM the pass kernels are compiled for
#endif
template <bool HOSTIO>
__global__ void __launch_bounds__(256, PP_NTT_MINB) k_ntt_pass(const PassArgs a) {
  extern __shared__ uint4 sm[];
  ntt_tile<HOSTIO>(a, blockIdx.x, sm);
}

// One batch level: the tiles of every job pass at this level are numbered
// consecutively (tile_start = prefix sums over the jobs), one block per tile
// as in k_ntt_pass; a block finds its job by a binary search over the starts.
__global__ void __launch_bounds__(256, PP_NTT_MINB) k_ntt_batch_level(const __grid_constant__ LevelParams p) {
  extern __shared__ uint4 sm[];
  const uint64_t t = blockIdx.x;
  uint32_t lo = 0, hi = p.count;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (p.tile_start[mid] <= t) lo = mid;
    else hi = mid;
  }
  ntt_tile<false>(p.args[lo], t - p.tile_start[lo], sm);  // device endpoints
}

// Transforms of 2^3 .. 2^11 points (single-pass plans) in one block: the
// input goes to shared memory in bit-reversed order, then radix-2
// decimation-in-time layers with w_N^(j N / 2m) from the plan's inner table
// leave the natural-order result.  Transforms this small are bound by
// latency, not by the multiply pipe.  The tiled pass kernel runs its unrolled
// radix-8 rounds once over a large code body and waits on instruction fetch
// (ncu at 2^11: no_instruction stalls 4.3 warps per issue; 46 us per call);
// this kernel's rolled loops keep its code small.  The input is read in full
// before anything is written, so in == out is allowed.
__global__ void __launch_bounds__(512) k_ntt_small(const PassArgs a) {
  extern __shared__ uint4 sm[];
  fr *x = reinterpret_cast<fr *>(sm);
  const uint32_t lg = a.lgN, N = 1u << lg, half = N >> 1;
#pragma unroll 1
  for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
    fr v;
    if (a.in_kind == NTT_IN_SPREAD) {
      v = (i & ((1u << a.spread) - 1)) == 0 ? ldcs_fr(a.in + (i >> a.spread)) : fr_zero();
    } else if (i < a.n_valid) {
      v = ldcs_fr(a.in + i);
      if (a.in_kind == NTT_IN_DIAG) v = fr_mul(v, ldcs_fr(a.diag + i));
    } else {
      v = fr_zero();
    }
    st_fr(x + (__brev(i) >> (32 - lg)), v);
  }
  __syncthreads();
#pragma unroll 1
  for (uint32_t s = 0; s < lg; ++s) {
#pragma unroll 1
    for (uint32_t b = threadIdx.x; b < half; b += blockDim.x) {
      const uint32_t j = b & ((1u << s) - 1);
      const uint32_t p = ((b >> s) << (s + 1)) + j, q = p + (1u << s);
      const fr t = fr_mul(ld_fr(x + q), ldg_fr(a.tw_inner + (j << (lg - 1 - s))));
      const fr u = ld_fr(x + p);
      st_fr(x + p, fr_add(u, t));
      st_fr(x + q, fr_sub(u, t));
    }
    __syncthreads();
  }
#pragma unroll 1
  for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
    fr v = ld_fr(x + i);
    if (a.has_post_scale) v = fr_mul(v, a.post_scale);
    st_fr(a.out + i, v);
  }
}

// One tile of a latency-form pass (2^9 .. 2^17 points, one column per tile):
// the tile geometry, inputs and outputs of ntt_tile, with each column's DFT
// as rolled radix-2 decimation-in-time layers over its bit-reversed copy in
// shared memory (so the result is in natural order), canonical throughout.
__global__ void __launch_bounds__(256) k_ntt_small_pass(const PassArgs a) {
  extern __shared__ uint4 sm[];
  fr *x = reinterpret_cast<fr *>(sm);  // column col at x[col R ..]
  const uint32_t lgR = a.lgR, R = 1u << lgR, T = 1u << a.lgT, E = R << a.lgT;
  const uint64_t tileid = blockIdx.x;
  uint64_t base = 0, col0 = 0, in_base = 0, out_base = 0;
  uint32_t lgS1 = 0;
  if (!a.last) {
    const uint32_t lgtpq = a.lgS - a.lgT;
    const uint64_t q = tileid >> lgtpq, ct = tileid & ((1ull << lgtpq) - 1);
    col0 = ct << a.lgT;
    base = (q << (a.lgR + a.lgS)) + col0;
  } else {
    const uint32_t lgR1 = a.lgRp[0];
    lgS1 = a.lgN - lgR1;
    const uint32_t lgkb = lgR1 - a.lgT;
    const uint64_t kb = tileid & ((1ull << lgkb) - 1), rest = tileid >> lgkb;
    uint64_t rin = 0, r = rest;
    uint32_t acc = lgR1;
    for (uint32_t j = 1; j + 1 < a.P; ++j) {
      const uint32_t bits = a.lgRp[j];
      acc += bits;
      rin += (r & ((1ull << bits) - 1)) << (a.lgN - acc);
      r >>= bits;
    }
    in_base = ((kb << a.lgT) << lgS1) + rin;
    out_base = (kb << a.lgT) + (rest << lgR1);
  }
#pragma unroll 1
  for (uint32_t e = threadIdx.x; e < E; e += blockDim.x) {
    uint32_t n, col;
    uint64_t g;
    if (!a.last) {
      n = e >> a.lgT;
      col = e & (T - 1);
      g = base + ((uint64_t)n << a.lgS) + col;
    } else {
      n = e & (R - 1);
      col = e >> a.lgR;
      g = in_base + ((uint64_t)col << lgS1) + n;
    }
    fr v;
    if (!a.first) {
      v = ldcs_fr(a.in + g);
    } else if (a.in_kind == NTT_IN_SPREAD) {
      v = (g & ((1ull << a.spread) - 1)) == 0 ? ldcs_fr(a.in + (g >> a.spread)) : fr_zero();
    } else if (g < a.n_valid) {
      v = ldcs_fr(a.in + g);
      if (a.in_kind == NTT_IN_DIAG) v = fr_mul(v, ldcs_fr(a.diag + g));
    } else {
      v = fr_zero();
    }
    st_fr(x + (col << lgR) + (__brev(n) >> (32 - lgR)), v);
  }
  __syncthreads();
  const uint32_t half = E >> 1, hmask = (R >> 1) - 1;
#pragma unroll 1
  for (uint32_t s = 0; s < lgR; ++s) {
#pragma unroll 1
    for (uint32_t b = threadIdx.x; b < half; b += blockDim.x) {
      fr *xc = x + ((b >> (lgR - 1)) << lgR);
      const uint32_t bb = b & hmask, j = bb & ((1u << s) - 1);
      const uint32_t p = ((bb >> s) << (s + 1)) + j, q = p + (1u << s);
      const fr t = fr_mul(ld_fr(xc + q), ldg_fr(a.tw_inner + (j << (lgR - 1 - s))));
      const fr u = ld_fr(xc + p);
      st_fr(xc + p, fr_add(u, t));
      st_fr(xc + q, fr_sub(u, t));
    }
    __syncthreads();
  }
#pragma unroll 1
  for (uint32_t e = threadIdx.x; e < E; e += blockDim.x) {
    const uint32_t o = e >> a.lgT, col = e & (T - 1);
    fr v = ld_fr(x + (col << lgR) + o);
    if (!a.last) {
      if (a.tw_layer) v = fr_mul(v, ldcs_fr(a.tw_layer + ((uint64_t)o << a.lgS) + col0 + col));
      st_fr(a.out + base + ((uint64_t)o << a.lgS) + col, v);
    } else {
      if (a.has_post_scale) v = fr_mul(v, a.post_scale);
      st_fr(a.out + out_base + col + ((uint64_t)o << (a.lgN - a.lgR)), v);
    }
  }
}

// transforms of 1, 2 or 4 points (one thread, direct evaluation)
__global__ void k_ntt_tiny(const fr *in, fr *out, uint32_t lgN, fr w, fr scale, int has_scale,
                           uint32_t in_kind, const fr *diag, uint64_t n_valid, uint32_t spread) {
  const uint32_t n = 1u << lgN;
  fr x[4], y[4];
  for (uint32_t i = 0; i < n; ++i) {
    if (in_kind == NTT_IN_SPREAD)
      x[i] = (i & ((1u << spread) - 1)) == 0 ? in[i >> spread] : fr_zero();
    else if (i < n_valid)
      x[i] = in_kind == NTT_IN_DIAG ? fr_mul(in[i], diag[i]) : in[i];
    else
      x[i] = fr_zero();
  }
  for (uint32_t k = 0; k < n; ++k) {
    fr acc = fr_zero(), wk = fr_one(), wkj = fr_one();
    for (uint32_t t = 0; t < k; ++t) wk = fr_mul(wk, w);
    for (uint32_t j = 0; j < n; ++j) {
      acc = fr_add(acc, fr_mul(x[j], wkj));
      wkj = fr_mul(wkj, wk);
    }
    y[k] = has_scale ? fr_mul(acc, scale) : acc;
  }
  for (uint32_t k = 0; k < n; ++k) out[k] = y[k];
}

// out[i] = base^e(i) via three 10-bit windows; e(i) = i (kind 0) or
// (i >> lgS) * (i & (2^lgS - 1)) (kind 1, layer tables); optional scale.
__global__ void k_pow_table(fr *out, uint64_t count, const fr *__restrict__ win, uint32_t kind,
                            uint32_t lgS, fr scale, int has_scale) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t e = kind == 0 ? i : (i >> lgS) * (i & ((1ull << lgS) - 1));
    fr v = ldg_fr(win + (e & 1023));
    if ((e >> 10) & 1023) v = fr_mul(v, ldg_fr(win + 1024 + ((e >> 10) & 1023)));
    if ((e >> 20) & 1023) v = fr_mul(v, ldg_fr(win + 2048 + ((e >> 20) & 1023)));
    if (has_scale) v = fr_mul(v, scale);
    st_fr(out + i, v);
  }
}

// ------------------------------------------------------------ host side
namespace {

std::mutex g_mu;

struct InnerKey {
  int dev;
  uint32_t lgR;
  bool inv;
  bool operator<(const InnerKey &o) const {
    return std::tie(dev, lgR, inv) < std::tie(o.dev, o.lgR, o.inv);
  }
};

struct Plan {
  uint32_t lgN = 0;
  bool inverse = false;
  uint32_t P = 0;
  uint32_t lgR[4] = {0, 0, 0, 0};
  uint32_t lgT[4] = {0, 0, 0, 0};
  const fr *tw_inner[4] = {nullptr, nullptr, nullptr, nullptr};
  fr *tw_layer[4] = {nullptr, nullptr, nullptr, nullptr};
  // host-pass plans: split layer tables instead of tw_layer
  fr *tw_lo[4] = {nullptr, nullptr, nullptr, nullptr};
  fr *tw_hi[4] = {nullptr, nullptr, nullptr, nullptr};
  uint32_t tw_lgh[4] = {0, 0, 0, 0};
  fr post_scale;
  bool has_post_scale = false;
};

void free_plan_tables(Plan *p) {
  for (int j = 0; j < 4; ++j) {
    cudaFree(p->tw_layer[j]);
    cudaFree(p->tw_lo[j]);
    cudaFree(p->tw_hi[j]);
  }
}

struct PlanKey {
  int dev;
  uint32_t lgN;
  bool inv;
  bool small;  // the latency form for single calls of 2^9 .. 2^17 points
  bool split;  // split layer tables (host-pass transforms)
  bool operator<(const PlanKey &o) const {
    return std::tie(dev, lgN, inv, small, split) < std::tie(o.dev, o.lgN, o.inv, o.small, o.split);
  }
};

struct PowKey {
  int dev;
  uint32_t lg;
  uint32_t h[8];
  bool operator<(const PowKey &o) const {
    if (dev != o.dev) return dev < o.dev;
    if (lg != o.lg) return lg < o.lg;
    return std::memcmp(h, o.h, sizeof(h)) < 0;
  }
};

std::map<InnerKey, fr *> g_inner;
std::map<PlanKey, Plan *> g_plans;
std::map<PowKey, fr *> g_pows;
std::map<uint32_t, std::vector<uint32_t>> g_split_override;

std::vector<uint32_t> default_split(uint32_t lgN) {
  std::vector<uint32_t> b;
  if (lgN <= 11) {
    b.push_back(lgN);
    return b;
  }
  const uint32_t P = (lgN + 8) / 9;
  for (uint32_t p = 0; p < P; ++p) b.push_back(lgN / P + (p < lgN % P ? 1 : 0));
  return b;
}

int build_windows(const fr &base, fr **d_win) {
  std::vector<fr> w(3072);
  fr step = base;
  for (int k = 0; k < 3; ++k) {
    w[1024 * k] = fr_one();
    for (int j = 1; j < 1024; ++j) w[1024 * k + j] = fr_mul(w[1024 * k + j - 1], step);
    fr s = step;
    for (int t = 0; t < 10; ++t) s = fr_sqr(s);  // step^(2^10)
    step = s;
  }
  PP_COUNT_ALLOC(3072 * sizeof(fr));
  PP_CUDA_TRY(cudaMalloc(d_win, 3072 * sizeof(fr)));
  PP_CUDA_TRY(cudaMemcpy(*d_win, w.data(), 3072 * sizeof(fr), cudaMemcpyHostToDevice));
  return PP_OK;
}

// builds base^e(i) for i < count on the device (synchronous: setup only)
int build_table(fr **out, uint64_t count, const fr &base, uint32_t kind, uint32_t lgS,
                const fr *scale) {
  fr *win = nullptr;
  int st = build_windows(base, &win);
  if (st) return st;
  PP_COUNT_ALLOC(count * sizeof(fr));
  cudaError_t e = cudaMalloc(out, count * sizeof(fr));
  if (e != cudaSuccess) {
    cudaFree(win);
    set_error("table allocation of %llu elements failed: %s", (unsigned long long)count,
              cudaGetErrorString(e));
    return PP_E_NOMEM;
  }
  const int threads = 256;
  const uint64_t blocks64 = (count + threads - 1) / threads;
  const int blocks = (int)(blocks64 < 152 * 64 ? blocks64 : 152 * 64);
  k_pow_table<<<blocks, threads>>>(*out, count, win, kind, lgS, scale ? *scale : fr_one(),
                                   scale ? 1 : 0);
  PP_COUNT_LAUNCH();
  e = cudaDeviceSynchronize();
  cudaFree(win);
  if (e != cudaSuccess) {
    set_error("table kernel failed: %s", cudaGetErrorString(e));
    return PP_E_CUDA;
  }
  return PP_OK;
}

int get_inner(int dev, uint32_t lgR, bool inv, const fr **out) {
  InnerKey k{dev, lgR, inv};
  auto it = g_inner.find(k);
  if (it != g_inner.end()) {
    *out = it->second;
    return PP_OK;
  }
  fr *t = nullptr;
  int st = build_table(&t, 1ull << lgR, host_root_of_unity((int)lgR, inv), 0, 0, nullptr);
  if (st) return st;
  g_inner[k] = t;
  *out = t;
  return PP_OK;
}

// small: two passes of about lgN / 2 bits with one column per tile, so that
// each pass of a 2^9 .. 2^17-point transform spreads over 16 .. 512 blocks
// (the throughput plan's 2048-element tiles give 1 .. 64)
// split: layer twiddles as two tables of about 2^(lgRS / 2) entries each
// (w^i and w^(i 2^h)) instead of one of 2^lgRS, for transforms whose data
// never sits in device memory
int get_plan(int dev, uint32_t lgN, bool inv, Plan **out, bool small = false, bool split = false) {
  PlanKey key{dev, lgN, inv, small, split};
  auto it = g_plans.find(key);
  if (it != g_plans.end()) {
    *out = it->second;
    return PP_OK;
  }
  auto ov = g_split_override.find(lgN);
  std::vector<uint32_t> bits = ov != g_split_override.end() ? ov->second : default_split(lgN);
  if (small) bits = {lgN - lgN / 2, lgN / 2};
  Plan *p = new Plan();
  p->lgN = lgN;
  p->inverse = inv;
  p->P = (uint32_t)bits.size();
  const fr ninv = host_inv(host_mont_small(1ull << lgN));
  uint32_t acc = 0;
  for (uint32_t j = 0; j < p->P; ++j) {
    p->lgR[j] = bits[j];
    acc += bits[j];
    const uint32_t lgS = lgN - acc;
    if (p->P == 1 || small) {
      p->lgT[j] = 0;
    } else if (j + 1 < p->P) {
      const uint32_t want = 11 - bits[j];
      p->lgT[j] = want < lgS ? want : lgS;
    } else {
      const uint32_t want = 11 - bits[j];
      p->lgT[j] = want < bits[0] ? want : bits[0];
    }
    int st = get_inner(dev, bits[j], inv, &p->tw_inner[j]);
    if (st) {
      free_plan_tables(p);
      delete p;
      return st;
    }
    if (j + 1 < p->P) {
      // w_{R S}^(c k) with R S = 2^(lgN - (acc - bits[j]))
      const uint32_t lgRS = lgN - (acc - bits[j]);
      const bool fold = inv && j == 0;  // 2^-lgN folded into the first layer
      const fr w = host_root_of_unity((int)lgRS, inv);
      if (!split) {
        st = build_table(&p->tw_layer[j], 1ull << lgRS, w, 1, lgS, fold ? &ninv : nullptr);
      } else {
        const uint32_t h = (lgRS + 1) / 2;
        p->tw_lgh[j] = h;
        st = build_table(&p->tw_lo[j], 1ull << h, w, 0, 0, fold ? &ninv : nullptr);
        if (!st) st = build_table(&p->tw_hi[j], 1ull << (lgRS - h), host_pow(w, 1ull << h), 0, 0, nullptr);
      }
      if (st) {
        free_plan_tables(p);
        delete p;
        return st;
      }
    }
  }
  if (inv && p->P == 1) {
    p->post_scale = ninv;
    p->has_post_scale = true;
  }
  g_plans[key] = p;
  *out = p;
  return PP_OK;
}

bool g_attr_set[64] = {false};

}  // namespace

int ntt_prepare(uint32_t lg_m, bool inverse) {
  if (lg_m > PP_MAX_LG_N) return PP_E_UNSUPPORTED;
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  if (lg_m <= 2) return PP_OK;
  Plan *p = nullptr;
  int st = get_plan(dev, lg_m, inverse, &p);
  if (!st && ntt_small_form(lg_m)) st = get_plan(dev, lg_m, inverse, &p, true);
  return st;
}

int ntt_set_split(uint32_t lg_m, const uint32_t *bits) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!bits) {
    g_split_override.erase(lg_m);
  } else {
    std::vector<uint32_t> b;
    uint32_t sum = 0;
    for (int i = 0; i < 4 && bits[i]; ++i) {
      if (bits[i] < 3 || bits[i] > 11) return PP_E_INVAL;
      b.push_back(bits[i]);
      sum += bits[i];
    }
    if (sum != lg_m || b.empty() || (b.size() > 1 && lg_m <= 3)) return PP_E_INVAL;
    g_split_override[lg_m] = b;
  }
  // drop cached plans of this size so the next call rebuilds them
  for (auto it = g_plans.begin(); it != g_plans.end();) {
    if (it->first.lgN == lg_m) {
      free_plan_tables(it->second);
      delete it->second;
      it = g_plans.erase(it);
    } else {
      ++it;
    }
  }
  return PP_OK;
}

void ntt_get_split(uint32_t lg_m, uint32_t *bits, uint32_t *npass) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto ov = g_split_override.find(lg_m);
  std::vector<uint32_t> b = ov != g_split_override.end() ? ov->second : default_split(lg_m);
  *npass = (uint32_t)b.size();
  for (size_t i = 0; i < b.size() && i < 4; ++i) bits[i] = b[i];
}

const fr *pow_table(const fr &h, uint32_t lg_n, int *status) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *status = PP_E_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  PowKey k{dev, lg_n, {}};
  std::memcpy(k.h, h.v, sizeof(k.h));
  auto it = g_pows.find(k);
  if (it != g_pows.end()) {
    *status = PP_OK;
    return it->second;
  }
  fr *t = nullptr;
  *status = build_table(&t, 1ull << lg_n, h, 0, 0, nullptr);
  if (*status) return nullptr;
  g_pows[k] = t;
  return t;
}

void ntt_release_tables() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto &kv : g_inner) cudaFree(kv.second);
  for (auto &kv : g_plans) {
    free_plan_tables(kv.second);
    delete kv.second;
  }
  for (auto &kv : g_pows) cudaFree(kv.second);
  g_inner.clear();
  g_plans.clear();
  g_pows.clear();
}

namespace {
int describe_passes(const fr *d_in, fr *d_out, fr *work, uint32_t lg_m, bool inverse,
                    const NttInputDesc &in, std::vector<PassArgs> &passes,
                    std::vector<uint64_t> &tiles, bool small, bool split);
}  // namespace

int ntt_describe(const fr *d_in, fr *d_out, fr *work, uint32_t lg_m, bool inverse,
                 const NttInputDesc &in, std::vector<PassArgs> &passes,
                 std::vector<uint64_t> &tiles, bool small) {
  return describe_passes(d_in, d_out, work, lg_m, inverse, in, passes, tiles, small, false);
}

namespace {
int describe_passes(const fr *d_in, fr *d_out, fr *work, uint32_t lg_m, bool inverse,
                    const NttInputDesc &in, std::vector<PassArgs> &passes,
                    std::vector<uint64_t> &tiles, bool small, bool split) {
  if (lg_m > PP_MAX_LG_N || lg_m < 3) {
    set_error("batched transform of 2^%u points: supported sizes are 2^3 .. 2^%d", lg_m, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  const uint64_t N = 1ull << lg_m;
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  Plan *plan = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    int st = get_plan(dev, lg_m, inverse, &plan, small, split);
    if (st) return st;
    if (dev < 64 && !g_attr_set[dev]) {
      PP_CUDA_TRY(cudaFuncSetAttribute(k_ntt_pass<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       2048 * (int)sizeof(fr)));
      PP_CUDA_TRY(cudaFuncSetAttribute(k_ntt_pass<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       2048 * (int)sizeof(fr)));
      PP_CUDA_TRY(cudaFuncSetAttribute(k_ntt_batch_level,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       2048 * (int)sizeof(fr)));
      PP_CUDA_TRY(cudaFuncSetAttribute(k_ntt_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       2048 * (int)sizeof(fr)));
      g_attr_set[dev] = true;
    }
  }
  if (plan->P > 1 && !work) {
    set_error("transform of 2^%u points needs a workspace", lg_m);
    return PP_E_INVAL;
  }
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.lgN = lg_m;
  a.P = plan->P;
  for (uint32_t j = 0; j < plan->P; ++j) a.lgRp[j] = plan->lgR[j];
  a.diag = in.diag;
  a.diag_hi = in.diag_hi;
  a.diag_lgh = in.diag_lgh;
  a.n_valid = in.n_valid ? in.n_valid : N;
  a.in_kind = (uint32_t)in.kind;
  a.spread = in.spread;
  uint32_t acc = 0;
  for (uint32_t j = 0; j < plan->P; ++j) {
    acc += plan->lgR[j];
    a.lgR = plan->lgR[j];
    a.lgT = plan->lgT[j];
    a.lgS = lg_m - acc;
    a.first = j == 0;
    a.last = j + 1 == plan->P;
    a.unit_in = a.first && in.in_host;
    // zero-padded input (n_valid = N / 2^z): pass 1's rows >= R >> z are zero
    a.zero_lg = 0;
    if (a.first && !a.last && in.kind != NTT_IN_SPREAD && in.n_valid && in.n_valid < N &&
        (in.n_valid & (in.n_valid - 1)) == 0) {
      uint32_t z = 0;
      while ((in.n_valid << z) < N) ++z;
      a.zero_lg = z;
    }
    a.unit_out = a.last && in.out_host;
    a.in = j == 0 ? d_in : work;
    a.out = a.last ? d_out : work;
    a.tw_inner = plan->tw_inner[j];
    a.tw_layer = plan->tw_layer[j];
    a.tw_lo = plan->tw_lo[j];
    a.tw_hi = plan->tw_hi[j];
    a.tw_lgh = plan->tw_lgh[j];
    a.has_post_scale = a.last && plan->has_post_scale;
    a.post_scale = plan->post_scale;
    passes.push_back(a);
    tiles.push_back(N >> (a.lgR + a.lgT));
  }
  return PP_OK;
}
}  // namespace

int ntt_launch_level(const LevelParams &params, cudaStream_t stream) {
  if (!params.total_tiles) return PP_OK;
  if (params.total_tiles > 0x7fffffffull) {
    set_error("batch level of %llu tiles exceeds one launch", (unsigned long long)params.total_tiles);
    return PP_E_UNSUPPORTED;
  }
  k_ntt_batch_level<<<(unsigned)params.total_tiles, 256, 2048 * sizeof(fr), stream>>>(params);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

int ntt_run(const fr *d_in, fr *d_out, uint32_t lg_m, bool inverse, const NttInputDesc &in,
            cudaStream_t stream) {
  if (lg_m > PP_MAX_LG_N) {
    set_error("transform of 2^%u points exceeds the supported 2^%d", lg_m, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  const uint64_t N = 1ull << lg_m;
  const uint64_t n_valid = in.n_valid ? in.n_valid : N;
  if (lg_m <= 2) {
    const fr w = host_root_of_unity((int)lg_m, inverse);
    const fr s = host_inv(host_mont_small(N));
    k_ntt_tiny<<<1, 1, 0, stream>>>(d_in, d_out, lg_m, w, s, inverse ? 1 : 0, in.kind, in.diag,
                                    n_valid, in.spread);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    return PP_OK;
  }
  const bool small = ntt_small_form(lg_m);
  uint32_t bits[4], np = 2;
  if (!small) ntt_get_split(lg_m, bits, &np);
  fr *work = nullptr;
  if (np > 1) {
    int st = PP_OK;
    work = static_cast<fr *>(workspace_get(N * sizeof(fr), stream, 0, &st));
    if (st) return st;
  }
  std::vector<PassArgs> passes;
  std::vector<uint64_t> tiles;
  int st = ntt_describe(d_in, d_out, work, lg_m, inverse, in, passes, tiles, small);
  if (st) return st;
  if (small) {
    for (size_t j = 0; j < passes.size(); ++j) {
      const uint32_t E = 1u << (passes[j].lgR + passes[j].lgT);
      const uint32_t threads = E / 2 < 32 ? 32 : (E / 2 > 256 ? 256 : E / 2);
      k_ntt_small_pass<<<(unsigned)tiles[j], threads, E * sizeof(fr), stream>>>(passes[j]);
      PP_COUNT_LAUNCH();
      PP_LAUNCH_CHECK();
    }
    return PP_OK;
  }
  if (passes.size() == 1 && lg_m <= 11) {
    const uint32_t threads = (uint32_t)(N / 2 < 32 ? 32 : (N / 2 > 512 ? 512 : N / 2));
    k_ntt_small<<<1, threads, N * sizeof(fr), stream>>>(passes[0]);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    return PP_OK;
  }
  for (size_t j = 0; j < passes.size(); ++j) {
    const uint32_t E = 1u << (passes[j].lgR + passes[j].lgT);
    if (passes[j].unit_in || passes[j].unit_out)
      k_ntt_pass<true><<<(unsigned)tiles[j], E / 8, E * sizeof(fr), stream>>>(passes[j]);
    else
      k_ntt_pass<false><<<(unsigned)tiles[j], E / 8, E * sizeof(fr), stream>>>(passes[j]);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
  }
  return PP_OK;
}

int ntt_host_plan_passes(uint32_t lg_m, uint32_t *passes) {
  if (lg_m <= 11) {
    *passes = 1;
    return PP_OK;
  }
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  Plan *plan = nullptr;
  const int st = get_plan(dev, lg_m, false, &plan, false, true);
  if (st) return st;
  *passes = plan->P;
  return PP_OK;
}

int ntt_run_host_passes(const fr *h_in, fr *h_out, fr *h_scratch, uint32_t lg_m, bool inverse,
                        cudaStream_t stream) {
  return ntt_run_host_passes(h_in, h_out, h_scratch, lg_m, inverse, NttInputDesc(), stream);
}

int ntt_run_host_passes(const fr *h_in, fr *h_out, fr *h_scratch, uint32_t lg_m, bool inverse,
                        const NttInputDesc &desc, cudaStream_t stream) {
  NttInputDesc in = desc;
  in.in_host = in.out_host = true;
  if (lg_m <= 11) {
    // one pass (or the tiny kernel): host in, host out, no intermediate; a
    // diagonal here is a full table (at most 2^11 entries)
    if (in.diag_hi) {
      set_error("transform of 2^%u points: split diagonal tables are for more than 2^11 points", lg_m);
      return PP_E_INVAL;
    }
    return ntt_run(h_in, h_out, lg_m, inverse, in, stream);
  }
  if (lg_m > PP_MAX_LG_N) {
    set_error("transform of 2^%u points exceeds the supported 2^%d", lg_m, PP_MAX_LG_N);
    return PP_E_UNSUPPORTED;
  }
  if (in.kind == NTT_IN_DIAG && !in.diag_hi) {
    set_error("transform of 2^%u points over host memory: the diagonal must be split", lg_m);
    return PP_E_INVAL;
  }
  std::vector<PassArgs> passes;
  std::vector<uint64_t> tiles;
  int st = describe_passes(h_in, h_out, h_scratch, lg_m, inverse, in, passes, tiles, false, true);
  if (st) return st;
  // pass j reads X_j and writes X_(j+1): X_0 = h_in, X_P = h_out, and the
  // intermediates alternate so that X_(P-1) = h_scratch
  const size_t P = passes.size();
  std::vector<fr *> X(P + 1);
  X[0] = const_cast<fr *>(h_in);
  X[P] = h_out;
  for (size_t j = P - 1; j >= 1; --j) X[j] = ((P - 1 - j) & 1) ? h_out : h_scratch;
  for (size_t j = 0; j < P; ++j) {
    PassArgs &a = passes[j];
    a.in = X[j];
    a.out = X[j + 1];
    a.unit_in = 1;
    a.unit_out = 1;
    const uint32_t E = 1u << (a.lgR + a.lgT);
    k_ntt_pass<true><<<(unsigned)tiles[j], E / 8, E * sizeof(fr), stream>>>(a);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
  }
  return PP_OK;
}

}  // namespace pp
