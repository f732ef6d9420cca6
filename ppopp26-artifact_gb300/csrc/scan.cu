// scan.cu -- grand product (exclusive prefix product), evaluation and division
// by (X + c) as blocked scans.
//
// The reference runs these as lg N Hillis-Steele launches over the whole
// vector (mont_arithmetic.cu:165-212, :305-361): O(N log N) multiplies and
// HBM traffic, plus a <<<1,1>>> squaring launch per step for division.  Here
// each is two launches with O(N) multiplies and two passes over HBM:
//  1. every thread folds a contiguous chunk of K elements into one summary
//     (a product for the grand product; an affine map S_start = a + b*S_end for
//     the backward recurrence S_i = p_i + m*S_{i+1} behind both evaluation,
//     m = x, and division, m = -c); a block-wide work-efficient scan over the
//     256 thread summaries in shared memory gives every thread its in-block
//     carry and the block its summary (evaluation needs only the summary);
//  2. every block folds the summaries of the blocks before it (grand product)
//     or after it (division) and each thread replays its chunk with the exact
//     carry; evaluation composes all block maps in one block.
// Field arithmetic is exact, so the grouping does not change any result.
#include <cuda.h>

#include "common.cuh"
#include "ntt.cuh"
#include "scan.cuh"

#include <mutex>

namespace pp {

// Blocks per SM each operator's geometry aims for (scan_geom): longer chunks
// cut the summaries to scan, more blocks hide more latency.  Swept over 1, 2,
// 4, 8 and 16 on GB300 at 2^20 / 2^22 elements: grand product 2 (80.0 us
// against 86.5 for 4; 4 is 3 % faster at 2^22), division 2 (94.5 / 222
// against 128 / 252), permutation product 8 (574 / 2125 against 592 / 2180;
// its local pass runs 2 blocks per SM, so it needs more of them to hide
// latency).  Evaluation has its own geometry (k_eval_tree).
constexpr uint32_t kGpBlocksPerSm = 2, kDivBlocksPerSm = 2,
                   kPermBlocksPerSm = 8;
// The grand product's chains grow with n while its block trees do not: at
// 2^22 3 blocks per SM beat 2 (0.210 against 0.220 ms), at 2^24 4 beat 2 and 3
// (0.712 against 0.764 / 0.730 ms); at 2^20 2 stays best (4: 0.081 against
// 0.075 ms).  The division's replay was best at 2 for all three sizes.
inline uint32_t gp_blocks_per_sm(uint64_t n) {
  return n <= (1ull << 21) ? kGpBlocksPerSm : n <= (1ull << 23) ? 3 : 4;
}

// ---------------------------------------------------------------- helpers
// Block scans are work-efficient (Blelloch, "Prefix sums and their
// applications", 1990): an up-sweep and a down-sweep over a balanced tree,
// 2(n-1) combines for n = blockDim.x (a power of two) instead of the n log n
// of a Hillis-Steele or warp-shuffle scan -- each combine here is one or two
// field multiplies.  All blocks of these launches are resident at once, so
// the scans' multiply count, not their depth, is what they cost: warp-shuffle
// scans (9 dependent steps instead of 16) made the 2^20 grand product,
// evaluation and division 13-36 % slower on GB300.

// prod p[i], lo <= i < hi (hi > lo), in ascending order
__device__ __forceinline__ fr chunk_product(const fr *p, uint64_t lo, uint64_t hi) {
  fr acc = ld_fr(p + lo);
  for (uint64_t i = lo + 1; i < hi; ++i) acc = fr_mul(acc, ld_fr(p + i));
  return acc;
}

// sum_{lo <= i < hi} p[i] x^(i - lo) (hi > lo) from pw[k] = x^k, k <= 16, in
// shared memory: groups of 16 coefficients are dot products with one
// reduction each (fr_mac17 / fr_redc17), joined by Horner steps with x^16
__device__ __forceinline__ fr chunk_dot(const fr *p, uint64_t lo, uint64_t hi, const fr *pw) {
  const uint64_t ng = (hi - lo + 15) >> 4;
  fr L = fr_zero();
#pragma unroll 1
  for (uint64_t g = ng; g-- > 0;) {
    const uint64_t b = lo + (g << 4);
    const uint32_t cnt = (uint32_t)(hi - b < 16 ? hi - b : 16);
    uint32_t acc[17];
#pragma unroll
    for (int k = 0; k < 17; ++k) acc[k] = 0;
    // each coefficient is loaded one term ahead of its multiply
    fr cur = ld_fr(p + b);
#pragma unroll 1
    for (uint32_t i = 0; i < cnt; ++i) {
      const fr nxt = i + 1 < cnt ? ld_fr(p + b + i + 1) : cur;
      fr_mac17(acc, cur, pw[i]);
      cur = nxt;
    }
    const fr S = fr_redc17(acc);
    L = g + 1 == ng ? S : fr_add(fr_mul(L, pw[16]), S);
  }
  return L;
}

// pw[k] = x^k, k <= 16, by the 32 lanes of one warp: four doubling steps
// (lanes 2^j < k <= 2^(j+1) take x^(k - 2^j) x^(2^j)); lanes 0..16 store
__device__ __forceinline__ void warp_power_table17(const fr &x, fr *pw) {
  const uint32_t lane = threadIdx.x & 31;
  fr v = lane == 0 ? fr_one() : x;
#pragma unroll 1
  for (uint32_t h = 1; h <= 8; h <<= 1) {
    fr lowv, hv;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      lowv.v[w] = __shfl_sync(0xffffffffu, v.v[w], (int)(lane >= h ? lane - h : 0));
      hv.v[w] = __shfl_sync(0xffffffffu, v.v[w], (int)h);
    }
    if (lane > h && lane <= 2 * h) v = fr_mul(lowv, hv);
  }
  if (lane <= 16) pw[lane] = v;
}

// inclusive prefix product over a block of 256 threads (commutative);
// afterwards s[t] holds thread t's inclusive product, which is also returned.
// A work-efficient up-sweep over the lowest three tree levels leaves the
// products of the 32 runs of 8; one warp scans those with shuffles (5 steps),
// and a three-level down-sweep hands the run prefixes back down.  12
// dependent multiplies against 17 for the full up- and down-sweep: the block
// scan is latency-bound (few threads multiply at each level).
__device__ __forceinline__ fr shfl_up_fr(const fr &v, int o);

__device__ fr block_prefix_product(fr v, fr *s) {
  const int t = threadIdx.x;
  constexpr int n = kScanThreads;
  static_assert(kScanThreads == 256, "32 runs of 8");
  s[t] = v;
  __syncthreads();
  for (int d = 1; d < 8; d <<= 1) {
    const int idx = (t + 1) * 2 * d - 1;
    if (idx < n) s[idx] = fr_mul(s[idx - d], s[idx]);
    __syncthreads();
  }
  if (t < 32) {
    fr inc = s[8 * t + 7];
    for (int o = 1; o < 32; o <<= 1) {
      const fr u = shfl_up_fr(inc, o);
      if (t >= o) inc = fr_mul(u, inc);
    }
    const fr ex = shfl_up_fr(inc, 1);
    s[8 * t + 7] = t ? ex : fr_one();
  }
  __syncthreads();
  for (int d = 4; d >= 1; d >>= 1) {
    const int idx = (t + 1) * 2 * d - 1;
    if (idx < n) {
      const fr left = s[idx - d];
      s[idx - d] = s[idx];
      s[idx] = fr_mul(s[idx], left);
    }
    __syncthreads();
  }
  const fr incl = fr_mul(s[t], v);
  __syncthreads();
  s[t] = incl;
  __syncthreads();
  return incl;
}

// Warp-shuffle (Kogge-Stone) forms: each warp scans its 32 values in 5
// steps, then warp 0 scans the warp totals -- 9 dependent multiplies and 3
// barriers against 16 of each, for about 2.5 times the multiplies.  They win
// where latency, not multiply throughput, bounds the block: the permutation
// product's local pass (2 blocks per SM) and its single-block carry pass
// (2^20: 0.607 -> 0.588 ms).  Afterwards s[t] holds thread t's inclusive
// prefix (or suffix) product, which is also returned.
__device__ __forceinline__ fr shfl_up_fr(const fr &v, int o) {
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = __shfl_up_sync(0xffffffffu, v.v[i], o);
  return r;
}
__device__ __forceinline__ fr shfl_down_fr(const fr &v, int o) {
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = __shfl_down_sync(0xffffffffu, v.v[i], o);
  return r;
}

__device__ fr warp_block_prefix_product(fr v, fr *s) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const fr u = shfl_up_fr(v, o);
    if (lane >= o) v = fr_mul(u, v);
  }
  if (lane == 31) s[w] = v;  // warp totals
  __syncthreads();
  if (w == 0) {
    fr x = lane < nw ? s[lane] : fr_one();
    for (int o = 1; o < nw; o <<= 1) {
      const fr u = shfl_up_fr(x, o);
      if (lane >= o) x = fr_mul(u, x);
    }
    if (lane < nw) s[lane] = x;  // warps 0 .. lane
  }
  __syncthreads();
  if (w > 0) v = fr_mul(s[w - 1], v);
  __syncthreads();
  s[t] = v;
  __syncthreads();
  return v;
}

__device__ fr warp_block_suffix_product(fr v, fr *s) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const fr u = shfl_down_fr(v, o);
    if (lane + o < 32) v = fr_mul(v, u);
  }
  if (lane == 0) s[w] = v;  // warp totals
  __syncthreads();
  if (w == 0) {
    fr x = lane < nw ? s[lane] : fr_one();
    for (int o = 1; o < nw; o <<= 1) {
      const fr u = shfl_down_fr(x, o);
      if (lane + o < nw) x = fr_mul(x, u);
    }
    if (lane < nw) s[lane] = x;  // warps lane .. nw-1
  }
  __syncthreads();
  if (w + 1 < nw) v = fr_mul(v, s[w + 1]);
  __syncthreads();
  s[t] = v;
  __syncthreads();
  return v;
}

// Suffix composition of affine maps f_t(x) = a_t + b_t x over the block.
// Afterwards (a, b) = F_t = f_t o f_{t+1} o ... o f_{n-1} and, when `all`,
// (sa[t], sb[t]) = F_t for every t; without `all` only F_0 is produced (in
// thread 0's (a, b) and sa[0], sb[0]).  Scanned in reversed order u = n-1-t,
// where the running composition is G_u = g_u o G_{u-1}.
// NAMED: the block also has a helper warp past the first 256 threads that
// does not take part, so the scan synchronises its 256 threads on a named
// barrier instead of __syncthreads.
template <bool NAMED>
__device__ __forceinline__ void scan_sync() {
  if (NAMED) asm volatile("bar.sync 1, 256;" ::: "memory");
  else __syncthreads();
}

template <bool NAMED = false>
__device__ void block_affine_suffix(fr &a, fr &b, fr *sa, fr *sb, bool all = true) {
  const int t = threadIdx.x, n = NAMED ? kScanThreads : blockDim.x;
  const int u = n - 1 - t;
  sa[u] = a;
  sb[u] = b;
  scan_sync<NAMED>();
  // The full scan of 256 maps takes the hybrid form of block_prefix_product:
  // three up-sweep levels, one warp scanning the 32 run maps, three
  // down-sweep levels.
  const bool hybrid = all && n == 256;
  // combine(left = earlier in u, right = later in u) = right o left
  for (int d = 1; d < (hybrid ? 8 : n); d <<= 1) {
    const int idx = (t + 1) * 2 * d - 1;
    if (idx < n) {
      const fr la = sa[idx - d], lb = sb[idx - d], ra = sa[idx], rb = sb[idx];
      sa[idx] = fr_add(ra, fr_mul(rb, la));
      sb[idx] = fr_mul(rb, lb);
    }
    scan_sync<NAMED>();
  }
  if (!all) {
    // sa[n-1], sb[n-1] = G_{n-1} = F_0
    if (t == 0) {
      a = sa[n - 1];
      b = sb[n - 1];
      sa[0] = a;
      sb[0] = b;
    }
    scan_sync<NAMED>();
    return;
  }
  if (hybrid) {
    if (t < 32) {
      // exclusive scan of the run maps at u = 8k + 7, in u order
      fr xa = sa[8 * t + 7], xb = sb[8 * t + 7];
      for (int o = 1; o < 32; o <<= 1) {
        const fr ua = shfl_up_fr(xa, o), ub = shfl_up_fr(xb, o);
        if (t >= o) {
          xa = fr_add(xa, fr_mul(xb, ua));
          xb = fr_mul(xb, ub);
        }
      }
      const fr ea = shfl_up_fr(xa, 1), eb = shfl_up_fr(xb, 1);
      sa[8 * t + 7] = t ? ea : fr_zero();
      sb[8 * t + 7] = t ? eb : fr_one();
    }
  } else if (t == 0) {
    sa[n - 1] = fr_zero();
    sb[n - 1] = fr_one();
  }
  scan_sync<NAMED>();
  for (int d = hybrid ? 4 : n >> 1; d >= 1; d >>= 1) {
    const int idx = (t + 1) * 2 * d - 1;
    if (idx < n) {
      const fr la = sa[idx - d], lb = sb[idx - d], pa = sa[idx], pb = sb[idx];
      sa[idx - d] = pa;
      sb[idx - d] = pb;
      sa[idx] = fr_add(la, fr_mul(lb, pa));  // left o P
      sb[idx] = fr_mul(lb, pb);
    }
    scan_sync<NAMED>();
  }
  // exclusive E_u in (sa[u], sb[u]); inclusive G_u = g_u o E_u = F_t
  const fr ea = sa[u], eb = sb[u];
  const fr ia = fr_add(a, fr_mul(b, ea)), ib = fr_mul(b, eb);
  scan_sync<NAMED>();
  sa[t] = ia;
  sb[t] = ib;
  a = ia;
  b = ib;
  scan_sync<NAMED>();
}

// ------------------------------------------------------------ grand product
__device__ __forceinline__ void gp_local_body(const fr *__restrict__ in, const ScanGeom &g,
                                              fr *__restrict__ thread_excl,
                                              fr *__restrict__ block_total, uint32_t blk, fr *s) {
  const uint64_t gt = blk * (uint64_t)kScanThreads + threadIdx.x;
  const uint64_t lo = gt * g.k, hi = lo + g.k < g.n ? lo + g.k : g.n;
  const fr p = lo < hi ? chunk_product(in, lo, hi) : fr_one();
  const fr incl = block_prefix_product(p, s);
  // exclusive = inclusive of the previous thread
  const fr excl = threadIdx.x ? s[threadIdx.x - 1] : fr_one();
  if (gt < g.threads) st_fr(thread_excl + gt, excl);
  if (threadIdx.x == blockDim.x - 1) st_fr(block_total + blk, incl);
}

__global__ void __launch_bounds__(kScanThreads) k_gp_local(const fr *__restrict__ in, ScanGeom g,
                                                            fr *__restrict__ thread_excl,
                                                            fr *__restrict__ block_total) {
  __shared__ fr s[kScanThreads];
  gp_local_body(in, g, thread_excl, block_total, blockIdx.x, s);
}

// out_excl[i] = prod_{j<i} in[j] and/or out_incl[i] = prod_{j<=i} in[j]; either
// output may be null or alias `in` (each element is read before it is written)
__device__ __forceinline__ void gp_apply_body(const fr *in, fr *out_excl, fr *out_incl,
                                              const ScanGeom &g, const fr *__restrict__ thread_excl,
                                              const fr *__restrict__ block_total, uint32_t blk,
                                              fr *s) {
  // product of the totals of all earlier blocks
  fr p = fr_one();
  for (uint32_t b = threadIdx.x; b < blk; b += blockDim.x) p = fr_mul(p, ld_fr(block_total + b));
  s[threadIdx.x] = p;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] = fr_mul(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  const fr block_prefix = s[0];
  const uint64_t gt = blk * (uint64_t)kScanThreads + threadIdx.x;
  if (gt >= g.threads) return;
  fr run = fr_mul(block_prefix, ld_fr(thread_excl + gt));
  const uint64_t lo = gt * g.k, hi = lo + g.k < g.n ? lo + g.k : g.n;
  for (uint64_t i = lo; i < hi; ++i) {
    const fr v = ld_fr(in + i);
    if (out_excl) st_fr(out_excl + i, run);
    run = fr_mul(run, v);
    if (out_incl) st_fr(out_incl + i, run);
  }
}

__global__ void __launch_bounds__(kScanThreads) k_gp_apply(const fr *in, fr *out_excl, fr *out_incl,
                                                            ScanGeom g,
                                                            const fr *__restrict__ thread_excl,
                                                            const fr *__restrict__ block_total) {
  __shared__ fr s[kScanThreads];
  gp_apply_body(in, out_excl, out_incl, g, thread_excl, block_total, blockIdx.x, s);
}

// Batched grand products: the blocks of all jobs are numbered consecutively
// (block_start = prefix sums); each block finds its job and runs the body.
__device__ __forceinline__ uint32_t find_job(const uint32_t *__restrict__ start, uint32_t count,
                                             uint32_t b) {
  uint32_t lo = 0, hi = count;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kScanThreads) k_gp_local_batch(const GpBatchJob *__restrict__ jobs,
                                                                  const uint32_t *__restrict__ start,
                                                                  uint32_t count) {
  __shared__ fr s[kScanThreads];
  const uint32_t j = find_job(start, count, blockIdx.x);
  const GpBatchJob jb = jobs[j];
  gp_local_body(jb.in, jb.g, jb.thread_excl, jb.block_total, blockIdx.x - start[j], s);
}

__global__ void __launch_bounds__(kScanThreads) k_gp_apply_batch(const GpBatchJob *__restrict__ jobs,
                                                                  const uint32_t *__restrict__ start,
                                                                  uint32_t count) {
  __shared__ fr s[kScanThreads];
  const uint32_t j = find_job(start, count, blockIdx.x);
  const GpBatchJob jb = jobs[j];
  gp_apply_body(jb.in, jb.out, nullptr, jb.g, jb.thread_excl, jb.block_total, blockIdx.x - start[j],
                s);
}

int gp_batch_launch(const GpBatchJob *d_jobs, const uint32_t *d_block_start, uint32_t count,
                    uint32_t total_blocks, cudaStream_t stream) {
  if (!total_blocks) return PP_OK;
  k_gp_local_batch<<<total_blocks, kScanThreads, 0, stream>>>(d_jobs, d_block_start, count);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_gp_apply_batch<<<total_blocks, kScanThreads, 0, stream>>>(d_jobs, d_block_start, count);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

struct PermArgs {
  const fr *w[3];
  const fr *sigma[3];
  const fr *params;     // beta, gamma, k1, k2, k3
  const fr *omega_pow;  // w^i, i < n
  fr *z;                // output; holds the numerators until the last pass
  fr *den;              // scratch: denominators
};

// Copy-constraint grand product z_i = prod_{j<i} num_j / den_j, computed as
//   z_i = (prod_{j<i} num_j) * (prod_{j>=i} den_j) / (prod_j den_j):
// a prefix product of the numerators and a suffix product of the
// denominators, both blocked scans, and one field inversion for the whole
// vector instead of one per block.  A zero denominator makes its ratio 0
// (num := 0, den := 1), the field-inverse-of-zero-is-zero convention.
//
// Pass 1: numerators and denominators; each thread's chunk products; their
// in-block exclusive prefix (numerators) and exclusive suffix (denominators);
// the block totals.
__global__ void __launch_bounds__(kScanThreads, 2)
    k_perm_local(const PermArgs a, ScanGeom g, fr *__restrict__ thread_num,
                 fr *__restrict__ thread_den, fr *__restrict__ block_num,
                 fr *__restrict__ block_den) {
  __shared__ fr s1[kScanThreads], s2[kScanThreads];
  const fr beta = ld_fr(a.params), gamma = ld_fr(a.params + 1);
  const fr bk0 = fr_mul(beta, ld_fr(a.params + 2));
  const fr bk1 = fr_mul(beta, ld_fr(a.params + 3));
  const fr bk2 = fr_mul(beta, ld_fr(a.params + 4));
  const uint64_t gt = blockIdx.x * (uint64_t)kScanThreads + threadIdx.x;
  const uint64_t lo = gt * g.k < g.n ? gt * g.k : g.n;
  const uint64_t hi = lo + g.k < g.n ? lo + g.k : g.n;
  fr N = fr_one(), D = fr_one();
  for (uint64_t i = lo; i < hi; ++i) {
    const fr wi = ld_fr(a.omega_pow + i);
    const fr x0 = ld_fr(a.w[0] + i), x1 = ld_fr(a.w[1] + i), x2 = ld_fr(a.w[2] + i);
    fr num = fr_add(fr_add(x0, fr_mul(bk0, wi)), gamma);
    num = fr_mul(num, fr_add(fr_add(x1, fr_mul(bk1, wi)), gamma));
    num = fr_mul(num, fr_add(fr_add(x2, fr_mul(bk2, wi)), gamma));
    fr den = fr_add(fr_add(x0, fr_mul(beta, ld_fr(a.sigma[0] + i))), gamma);
    den = fr_mul(den, fr_add(fr_add(x1, fr_mul(beta, ld_fr(a.sigma[1] + i))), gamma));
    den = fr_mul(den, fr_add(fr_add(x2, fr_mul(beta, ld_fr(a.sigma[2] + i))), gamma));
    if (fr_is_zero(den)) {
      num = fr_zero();
      den = fr_one();
    }
    st_fr(a.z + i, num);
    st_fr(a.den + i, den);
    N = fr_mul(N, num);
    D = fr_mul(D, den);
  }
  const fr incl_n = warp_block_prefix_product(N, s1);  // s1[t] = N_0 .. N_t
  const fr incl_d = warp_block_suffix_product(D, s2);  // s2[t] = D_t .. D_last
  if (gt < g.threads) {
    st_fr(thread_num + gt, threadIdx.x ? s1[threadIdx.x - 1] : fr_one());
    st_fr(thread_den + gt, threadIdx.x + 1 < blockDim.x ? s2[threadIdx.x + 1] : fr_one());
  }
  if (threadIdx.x == blockDim.x - 1) st_fr(block_num + blockIdx.x, incl_n);
  if (threadIdx.x == 0) st_fr(block_den + blockIdx.x, incl_d);
}

// Pass 2, one block: in place, block_num[b] := the product of the numerator
// totals of the blocks before b, block_den[b] := the product of the
// denominator totals of the blocks after b, divided by all denominators.
__global__ void __launch_bounds__(kScanThreads) k_perm_carry(fr *block_num, fr *block_den,
                                                              uint32_t nb) {
  __shared__ fr s1[kScanThreads], s2[kScanThreads];
  __shared__ fr s_inv;
  const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = threadIdx.x * per < nb ? threadIdx.x * per : nb;
  const uint32_t hi = lo + per < nb ? lo + per : nb;
  fr N = fr_one(), D = fr_one();
  for (uint32_t b = lo; b < hi; ++b) {
    N = fr_mul(N, ld_fr(block_num + b));
    D = fr_mul(D, ld_fr(block_den + b));
  }
  warp_block_prefix_product(N, s1);
  warp_block_suffix_product(D, s2);  // s2[0]: every denominator (none is zero)
  if (threadIdx.x == 0) s_inv = fr_inv_fast(s2[0]);
  __syncthreads();
  fr run_n = threadIdx.x ? s1[threadIdx.x - 1] : fr_one();
  fr run_d = fr_mul(s_inv, threadIdx.x + 1 < blockDim.x ? s2[threadIdx.x + 1] : fr_one());
  for (uint32_t b = lo; b < hi; ++b) {
    const fr v = ld_fr(block_num + b);
    st_fr(block_num + b, run_n);
    run_n = fr_mul(run_n, v);
  }
  for (uint32_t b = hi; b > lo; --b) {
    const fr v = ld_fr(block_den + b - 1);
    st_fr(block_den + b - 1, run_d);
    run_d = fr_mul(run_d, v);
  }
}

// Pass 3: z_i = (numerators before i) * (denominators from i on) / (all):
// forward over the chunk for the first factor (kept in z), backward for the
// second.
__global__ void __launch_bounds__(kScanThreads)
    k_perm_apply(const PermArgs a, ScanGeom g, const fr *__restrict__ thread_num,
                 const fr *__restrict__ thread_den, const fr *__restrict__ block_num,
                 const fr *__restrict__ block_den) {
  const uint64_t gt = blockIdx.x * (uint64_t)kScanThreads + threadIdx.x;
  if (gt >= g.threads) return;
  const uint64_t lo = gt * g.k, hi = lo + g.k < g.n ? lo + g.k : g.n;
  fr run = fr_mul(ld_fr(block_num + blockIdx.x), ld_fr(thread_num + gt));
  for (uint64_t i = lo; i < hi; ++i) {
    const fr v = ld_fr(a.z + i);
    st_fr(a.z + i, run);
    run = fr_mul(run, v);
  }
  run = fr_mul(ld_fr(block_den + blockIdx.x), ld_fr(thread_den + gt));
  for (uint64_t i = hi; i > lo; --i) {
    run = fr_mul(run, ld_fr(a.den + i - 1));
    st_fr(a.z + i - 1, fr_mul(ld_fr(a.z + i - 1), run));
  }
}

// --------------------------------------------- backward affine recurrence
// S_i = p_i + m * S_{i+1}: a thread's chunk [lo, hi) is the map
// S_lo = L + m^(hi-lo) * S_hi with L its Horner value.  m^K for the full
// chunk length K is shared by the block: only a shorter (last) chunk computes
// its own power.

// per-thread exclusive suffix map (optional) and per-block map.  Launched
// with kScanThreads + 32 threads: the extra warp computes m^K while the
// others evaluate their chunks (chunk_dot, after the first warp's table of
// m^0 .. m^16), which do not need it.
__global__ void __launch_bounds__(kScanThreads + 32) k_affine_local(const fr *__restrict__ p, ScanGeom g,
                                                                     const fr *__restrict__ m_ptr,
                                                                     int negate_m, fr *thread_a,
                                                                     fr *thread_b, fr *block_a,
                                                                     fr *block_b) {
  __shared__ fr sa[kScanThreads], sb[kScanThreads];
  __shared__ fr s_mk;
  __shared__ fr s_pw[17];  // m^k, k <= 16, for the chunks' dot products
  fr m = ld_fr(m_ptr);
  if (negate_m) m = fr_neg(m);
  if (threadIdx.x >= kScanThreads) {
    if (threadIdx.x == kScanThreads) s_mk = fr_pow_u64(m, g.k);
    __syncthreads();
    return;  // the scan below synchronises the other 256 threads by name
  }
  if (threadIdx.x < 32) warp_power_table17(m, s_pw);
  asm volatile("bar.sync 1, 256;" ::: "memory");
  const uint64_t gt = blockIdx.x * (uint64_t)kScanThreads + threadIdx.x;
  const uint64_t lo = gt * g.k < g.n ? gt * g.k : g.n;
  const uint64_t hi = lo + g.k < g.n ? lo + g.k : g.n;
  const fr L = hi > lo ? chunk_dot(p, lo, hi, s_pw) : fr_zero();
  __syncthreads();  // m^K ready
  fr a = L, b = hi - lo == g.k ? s_mk : hi > lo ? fr_pow_u64(m, hi - lo) : fr_one();
  block_affine_suffix<true>(a, b, sa, sb, thread_a != nullptr);
  if (thread_a && gt < g.threads) {
    const bool last = threadIdx.x == kScanThreads - 1;
    st_fr(thread_a + gt, last ? fr_zero() : sa[threadIdx.x + 1]);
    st_fr(thread_b + gt, last ? fr_one() : sb[threadIdx.x + 1]);
  }
  if (threadIdx.x == 0) {
    st_fr(block_a + blockIdx.x, a);
    st_fr(block_b + blockIdx.x, b);
  }
}

// ordered composition of the block maps [first, count) (from one block of
// threads); returns the composed map's a (the value applied to S = 0) and b.
__device__ void compose_blocks(const fr *block_a, const fr *block_b, uint32_t first,
                               uint32_t count, fr &A, fr &B, fr *sa, fr *sb) {
  const uint32_t span = count > first ? count - first : 0;
  const uint32_t per = (span + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = first + threadIdx.x * per;
  const uint32_t hi = lo + per < count ? lo + per : count;
  // sequential composition over [lo, hi): f_lo o ... o f_{hi-1}
  fr a = fr_zero(), b = fr_one();
  for (uint32_t i = hi; i > lo; --i) {  // prepend f_{i-1}
    const fr ai = ld_fr(block_a + i - 1), bi = ld_fr(block_b + i - 1);
    a = fr_add(ai, fr_mul(bi, a));
    b = fr_mul(bi, b);
  }
  block_affine_suffix(a, b, sa, sb, false);
  A = sa[0];
  B = sb[0];
}

__global__ void __launch_bounds__(kScanThreads) k_div_apply(fr *inout, ScanGeom g,
                                                             const fr *__restrict__ m_ptr,
                                                             const fr *__restrict__ thread_a,
                                                             const fr *__restrict__ thread_b,
                                                             const fr *__restrict__ block_a,
                                                             const fr *__restrict__ block_b) {
  __shared__ fr sa[kScanThreads], sb[kScanThreads];
  const fr m = fr_neg(ld_fr(m_ptr));
  fr A, B;
  compose_blocks(block_a, block_b, blockIdx.x + 1, g.blocks, A, B, sa, sb);
  const fr s_end_block = A;  // S at the end of this block (S_n = 0)
  const uint64_t gt = blockIdx.x * (uint64_t)kScanThreads + threadIdx.x;
  if (gt >= g.threads) return;
  fr s = fr_add(ld_fr(thread_a + gt), fr_mul(ld_fr(thread_b + gt), s_end_block));
  const uint64_t lo = gt * g.k, hi = lo + g.k < g.n ? lo + g.k : g.n;
  for (uint64_t i = hi; i > lo; --i) {
    const fr pi = ld_fr(inout + i - 1);
    st_fr(inout + i - 1, s);  // q_{i-1} = S_i
    s = fr_add(pi, fr_mul(m, s));
  }
}

__global__ void __launch_bounds__(kScanThreads) k_eval_final(const fr *__restrict__ block_a,
                                                              const fr *__restrict__ block_b,
                                                              uint32_t count, fr *y) {
  __shared__ fr sa[kScanThreads], sb[kScanThreads];
  fr A, B;
  compose_blocks(block_a, block_b, 0, count, A, B, sa, sb);
  if (threadIdx.x == 0) st_fr(y, A);
}

// ------------------------------------------------------------ evaluation
// y = sum_i p_i x^i in one launch.
//  * Thread t of block b takes the K contiguous coefficients from (256 b + t) K
//    and evaluates them: L = sum_{i<K} p_{(256 b + t) K + i} x^i, as dot
//    products of groups of 16 coefficients with x^0 .. x^15 (one reduction per
//    group, chunk_dot) joined by Horner steps with x^16.  The first Horner warp
//    builds x^0 .. x^16 first.  K is chosen as for the other scans (scan_geom;
//    blocks per SM below).
//  * Its term is L x^(K t) x^(256 K b).  Thread weights come from two 16-entry
//    tables, x^(K a) and x^(16 K a) for a < 16 (x^(K t) = one product of an
//    entry of each); the block's weight x^(256 K b) is one power.  Two helper
//    warps compute the tables and that power while the other eight run their
//    Horner chains.
//  * Weighted terms are summed with field additions (warp shuffles, then the
//    warps' sums); the block stores its sum times its weight, and the block
//    that finishes last (a ticket counter) adds the block sums into y.
// After the chains, a thread does two multiplies; every other step is an
// addition.  A binary fold of the same terms (L_u + x^(K s) L_(u+s)) needs
// eight dependent multiplies per block and as many more in the last block.
// The sum's grouping does not change the value: field addition is exact.
// Blocks per SM: 1 up to 2^21 coefficients, 2 above.  At 2^20 the helpers'
// powers (a chain of about 25 dependent multiplies, slowed by the Horner warps
// that share their SM) end after the chains, so fewer Horner warps per SM
// finish the block sooner (41.8 against 46.1 us); at 2^22 the chains are the
// longer part and two blocks per SM are as fast (106 against 108 us).
constexpr uint32_t kEvalBlocksPerSmSmall = 1, kEvalBlocksPerSm = 2;
constexpr uint64_t kEvalSmallMax = 1ull << 21;
constexpr uint32_t kEvalHelperWarps = 2;
// Horner threads per block (with the two helper warps on top).  128 per block
// (fewer Horner warps beside the helpers, twice the coefficients per thread)
// was slower: 37.9 against 35.5 us at 2^20, 85.2 against 82.8 us at 2^22.
constexpr uint32_t kEvalHorner = 256;

__device__ __forceinline__ fr ldcg_fr(const fr *p) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  uint4 a = __ldcg(q), b = __ldcg(q + 1);
  return fr{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
}

__device__ __forceinline__ fr shfl_xor_fr(const fr &v, int o) {
  fr r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = __shfl_xor_sync(0xffffffffu, v.v[i], o);
  return r;
}

// sum over the 32 lanes of a warp (every lane gets it)
__device__ __forceinline__ fr warp_sum_fr(fr v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fr_add(v, shfl_xor_fr(v, o));
  return v;
}

template <uint32_t HT>
__global__ void __launch_bounds__(HT + 32 * kEvalHelperWarps)
    k_eval_tree(const fr *__restrict__ p, ScanGeom g, const fr *__restrict__ xp,
                fr *__restrict__ block_val, uint32_t *__restrict__ ticket, fr *__restrict__ y) {
  static_assert(HT % 32 == 0 && HT <= 256, "Horner threads: whole warps, at most 256");
  constexpr uint32_t kHelpers = 32 * kEvalHelperWarps, kWarps = HT / 32;
  __shared__ fr tab[32];  // tab[a] = x^(K a), tab[16 + a] = x^(16 K a), a < 16
  __shared__ fr s_wb;     // x^(HT K b)
  __shared__ fr s_pw[17]; // x^k, k <= 16, for the Horner threads' dot products
  __shared__ fr s_warp[kWarps];
  __shared__ uint32_t s_last;
  // warps 0 and 1 are the helpers
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t t = threadIdx.x - kHelpers, warp = t >> 5;  // Horner thread and warp
  const fr x = ld_fr(xp);
  fr L = fr_zero();
  if (threadIdx.x < 32) {
    // the tables: lane a < 16 raises x^K to a, lane 16 + a raises x^(16 K) to a
    const fr v = fr_pow_u64(x, g.k);
    fr u = v;
#pragma unroll 1
    for (int i = 0; i < 4; ++i) u = fr_sqr(u);
    tab[lane] = fr_pow_u64(lane < 16 ? v : u, lane & 15);
  } else if (threadIdx.x < kHelpers) {
    // the block's weight: (x^(HT K))^b
    fr v = fr_pow_u64(x, g.k);
#pragma unroll 1
    for (uint32_t i = 1; i < HT; i <<= 1) v = fr_sqr(v);
    v = fr_pow_u64(v, blockIdx.x);
    if (lane == 0) s_wb = v;
  } else {
    // the first Horner warp builds x^0 .. x^16; the Horner threads wait for
    // it on a named barrier (the helper warps do not)
    if (warp == 0) warp_power_table17(x, s_pw);
    asm volatile("bar.sync 1, %0;" ::"n"(HT) : "memory");
    const uint64_t lo = ((uint64_t)blockIdx.x * HT + t) * g.k;
    if (lo < g.n) L = chunk_dot(p, lo, lo + g.k < g.n ? lo + g.k : g.n, s_pw);
  }
  __syncthreads();  // the tables, the block weight and the chunk values are ready
  if (threadIdx.x >= kHelpers) {
    const fr w = fr_mul(tab[t & 15], tab[16 + (t >> 4)]);  // x^(K t)
    const fr sum = warp_sum_fr(fr_mul(L, w));
    if (lane == 0) s_warp[warp] = sum;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    fr v = warp_sum_fr(lane < kWarps ? s_warp[lane] : fr_zero());
    if (lane == 0) {
      st_fr(block_val + blockIdx.x, fr_mul(v, s_wb));
      __threadfence();
      s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!s_last) return;
  // the last block: y = the sum of the gridDim.x weighted block sums
  __threadfence();
  if (threadIdx.x >= kHelpers) {
    fr acc = fr_zero();
    for (uint32_t b = t; b < gridDim.x; b += HT) acc = fr_add(acc, ldcg_fr(block_val + b));
    acc = warp_sum_fr(acc);
    if (lane == 0) s_warp[warp] = acc;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const fr v = warp_sum_fr(lane < kWarps ? s_warp[lane] : fr_zero());
    if (lane == 0) {
      st_fr(y, v);
      *ticket = 0;
    }
  }
}

__global__ void k_zero1(fr *y) { st_fr(y, fr_zero()); }

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace pp

using pp::fr;

extern "C" int pp_gp_scan(const void *d_in, void *d_excl, void *d_incl, uint64_t n, void *stream) {
  if (n == 0) return PP_OK;
  if (!d_in || !pp::aligned16(d_in) || (d_excl && !pp::aligned16(d_excl)) ||
      (d_incl && !pp::aligned16(d_incl)) || (!d_excl && !d_incl)) {
    pp::set_error("pp_gp_scan: need a 16-byte aligned input and at least one aligned output");
    return PP_E_INVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const pp::ScanGeom g = pp::scan_geom(n, pp::gp_blocks_per_sm(n));
  int st = PP_OK;
  fr *ws = static_cast<fr *>(
      pp::workspace_get((g.threads + g.blocks) * sizeof(fr), s, 1, &st));
  if (st) return st;
  fr *thread_excl = ws, *block_total = ws + g.threads;
  pp::k_gp_local<<<g.blocks, pp::kScanThreads, 0, s>>>(static_cast<const fr *>(d_in), g, thread_excl,
                                                       block_total);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_gp_apply<<<g.blocks, pp::kScanThreads, 0, s>>>(
      static_cast<const fr *>(d_in), static_cast<fr *>(d_excl), static_cast<fr *>(d_incl), g,
      thread_excl, block_total);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_gp_prefix(void *d_inout, uint64_t n, void *stream) {
  if (n && (!d_inout || !pp::aligned16(d_inout))) {
    pp::set_error("pp_gp_prefix: buffer must be a 16-byte aligned device pointer");
    return PP_E_INVAL;
  }
  return pp_gp_scan(d_inout, d_inout, nullptr, n, stream);
}

extern "C" int pp_div_xplusc(void *d_inout, uint64_t n, const void *d_c, void *stream) {
  if (n == 0) return PP_OK;
  if (!d_inout || !d_c || !pp::aligned16(d_inout) || !pp::aligned16(d_c)) {
    pp::set_error("pp_div_xplusc: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const pp::ScanGeom g = pp::scan_geom(n, pp::kDivBlocksPerSm);
  int st = PP_OK;
  fr *ws = static_cast<fr *>(
      pp::workspace_get((2 * g.threads + 2 * g.blocks) * sizeof(fr), s, 1, &st));
  if (st) return st;
  fr *ta = ws, *tb = ws + g.threads, *ba = ws + 2 * g.threads, *bb = ba + g.blocks;
  const fr *c = static_cast<const fr *>(d_c);
  pp::k_affine_local<<<g.blocks, pp::kScanThreads + 32, 0, s>>>(static_cast<const fr *>(d_inout), g, c,
                                                           1, ta, tb, ba, bb);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_div_apply<<<g.blocks, pp::kScanThreads, 0, s>>>(static_cast<fr *>(d_inout), g, c, ta, tb,
                                                        ba, bb);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_eval(const void *d_poly, uint64_t n, const void *d_x, void *d_y, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!d_y || !pp::aligned16(d_y) || (n && (!d_poly || !d_x || !pp::aligned16(d_poly) ||
                                            !pp::aligned16(d_x)))) {
    pp::set_error("pp_eval: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  if (n == 0) {
    pp::k_zero1<<<1, 1, 0, s>>>(static_cast<fr *>(d_y));
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    return PP_OK;
  }
  // scan_geom's rule with kEvalHorner threads per block
  constexpr uint32_t HT = pp::kEvalHorner;
  const uint32_t bps = n <= pp::kEvalSmallMax ? pp::kEvalBlocksPerSmSmall : pp::kEvalBlocksPerSm;
  pp::ScanGeom g;
  g.n = n;
  const uint64_t target = (uint64_t)pp::device_sm_count() * bps * HT;
  g.k = (n + target - 1) / target;
  if (g.k < 4) g.k = 4;
  g.threads = (n + g.k - 1) / g.k;
  g.blocks = (uint32_t)((g.threads + HT - 1) / HT);
  const uint32_t nb = g.blocks;
  int st = PP_OK;
  // block sums, then the ticket counter in its own 32-byte slot
  char *ws = static_cast<char *>(pp::workspace_get((nb + 1) * sizeof(fr), s, 1, &st));
  if (st) return st;
  fr *block_val = reinterpret_cast<fr *>(ws);
  uint32_t *ticket = reinterpret_cast<uint32_t *>(ws + nb * sizeof(fr));
  PP_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(uint32_t), s));
  pp::k_eval_tree<HT><<<nb, HT + 32 * pp::kEvalHelperWarps, 0, s>>>(
      static_cast<const fr *>(d_poly), g, static_cast<const fr *>(d_x), block_val, ticket,
      static_cast<fr *>(d_y));
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

extern "C" int pp_gp_perm(const void *const *d_w, const void *const *d_sigma, const void *d_params,
                          void *d_z, uint32_t lg_n, void *stream) {
  if (!d_w || !d_sigma || !d_params || !d_z || !pp::aligned16(d_params) || !pp::aligned16(d_z)) {
    pp::set_error("pp_gp_perm: null or misaligned pointer");
    return PP_E_INVAL;
  }
  for (int j = 0; j < 3; ++j) {
    if (!d_w[j] || !d_sigma[j] || !pp::aligned16(d_w[j]) || !pp::aligned16(d_sigma[j])) {
      pp::set_error("pp_gp_perm: null or misaligned wire/sigma pointer %d", j);
      return PP_E_INVAL;
    }
  }
  if (lg_n > PP_MAX_LG_N) {
    pp::set_error("pp_gp_perm: lg_n = %u too large", lg_n);
    return PP_E_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t n = 1ull << lg_n;
  const pp::ScanGeom g = pp::scan_geom(n, pp::kPermBlocksPerSm);
  int st = PP_OK;
  const fr *omega_pow = pp::pow_table(pp::host_root_of_unity((int)lg_n, false), lg_n, &st);
  if (st) return st;
  fr *ws = static_cast<fr *>(
      pp::workspace_get((n + 2 * g.threads + 2 * g.blocks) * sizeof(fr), s, 1, &st));
  if (st) return st;
  pp::PermArgs a;
  for (int j = 0; j < 3; ++j) {
    a.w[j] = static_cast<const fr *>(d_w[j]);
    a.sigma[j] = static_cast<const fr *>(d_sigma[j]);
  }
  a.params = static_cast<const fr *>(d_params);
  a.omega_pow = omega_pow;
  a.z = static_cast<fr *>(d_z);
  a.den = ws;
  fr *thread_num = ws + n, *thread_den = thread_num + g.threads;
  fr *block_num = thread_den + g.threads, *block_den = block_num + g.blocks;
  pp::k_perm_local<<<g.blocks, pp::kScanThreads, 0, s>>>(a, g, thread_num, thread_den, block_num,
                                                         block_den);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_perm_carry<<<1, pp::kScanThreads, 0, s>>>(block_num, block_den, g.blocks);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_perm_apply<<<g.blocks, pp::kScanThreads, 0, s>>>(a, g, thread_num, thread_den, block_num,
                                                         block_den);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

// ---------------------------------------------------------------------------
// Evaluation that allocates nothing.
//
// pp_eval takes its block summaries from a per-stream workspace that is
// created with cudaMalloc on first use.  Some callers cannot allow that: a
// serving process that has handed all free device memory to its own pool
// (a fresh cudaMalloc would fail or fragment it), or a latency-critical loop
// where cudaMalloc / cudaFree may synchronise the whole device and stall the
// work of other streams.  For them pp_eval_noalloc keeps its scratch in a
// file-scope device array that exists, for every device that loads this
// library, from module load until process exit:
//   2 * 1024 block summaries of 32 bytes = 64 KiB per device.
// With 16 elements per thread and 256 threads per block that bounds the
// polynomial at 1024 * 256 * 16 = 2^22 coefficients; longer ones are refused
// with PP_E_UNSUPPORTED before any device work.
// ---------------------------------------------------------------------------
namespace pp {

constexpr uint32_t kEvalNoAllocMaxBlocks = 1024;
constexpr uint64_t kEvalNoAllocChunk = 16;
static_assert((uint64_t)kEvalNoAllocMaxBlocks * kScanThreads * kEvalNoAllocChunk == PP_EVAL_NOALLOC_MAX_N,
              "header limit and scratch geometry disagree");

// [0, 1024): affine-map offsets a_b of the blocks, [1024, 2048): factors b_b
static __device__ __align__(256) fr g_eval_noalloc_scratch[2 * kEvalNoAllocMaxBlocks];

// Device address of g_eval_noalloc_scratch per device, with the id of the CUDA
// context it was looked up in.  A device reset (cudaDeviceReset) destroys the
// primary context and the module with it; the next context loads the module
// again, possibly elsewhere, under a new context id.  So the cached address is
// used only while the calling thread's current context has the stored id, and
// looked up again otherwise.
struct NoAllocAddr {
  unsigned long long ctx_id = 0;
  fr *addr = nullptr;
};
static std::mutex g_eval_noalloc_mu;
static NoAllocAddr g_eval_noalloc_addr[64];

// Id of the calling thread's current CUDA context (cuCtxGetCurrent + cuCtxGetId,
// reached through the runtime's driver entry points so that the library does
// not link the driver library), or 0 when there is none or it cannot be read.
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
      get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

}  // namespace pp

extern "C" int pp_eval_noalloc(const void *d_poly, uint64_t n, const void *d_x, void *d_y,
                               void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!d_y || !pp::aligned16(d_y) || (n && (!d_poly || !d_x || !pp::aligned16(d_poly) ||
                                            !pp::aligned16(d_x)))) {
    pp::set_error("pp_eval_noalloc: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  if (n > PP_EVAL_NOALLOC_MAX_N) {
    pp::set_error("pp_eval_noalloc: %llu coefficients exceed the 2^22 its static scratch covers; "
                  "use pp_eval",
                  (unsigned long long)n);
    return PP_E_UNSUPPORTED;
  }
  if (n == 0) {
    pp::k_zero1<<<1, 1, 0, s>>>(static_cast<fr *>(d_y));
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    return PP_OK;
  }
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    pp::set_error("pp_eval_noalloc: device index %d out of range", dev);
    return PP_E_INVAL;
  }
  fr *scratch = nullptr;
  {
    // set-up on the first call on this device (that device is current), and
    // again after its context changed: the host-side name of the array is not
    // a device address; ask the runtime
    std::lock_guard<std::mutex> lk(pp::g_eval_noalloc_mu);
    pp::NoAllocAddr &slot = pp::g_eval_noalloc_addr[dev];
    const unsigned long long ctx_id = pp::current_context_id();
    if (!slot.addr || ctx_id == 0 || slot.ctx_id != ctx_id) {
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, pp::g_eval_noalloc_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        pp::set_error("pp_eval_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return PP_E_CUDA;
      }
      slot.addr = static_cast<fr *>(p);
      // the look-up makes the device's primary context current if none was
      slot.ctx_id = ctx_id ? ctx_id : pp::current_context_id();
    }
    scratch = slot.addr;
  }
  pp::ScanGeom g;
  g.n = n;
  g.k = pp::kEvalNoAllocChunk;
  g.threads = (n + g.k - 1) / g.k;
  g.blocks = (uint32_t)((g.threads + pp::kScanThreads - 1) / pp::kScanThreads);
  // every block summary read by k_eval_final is written by k_affine_local in
  // the same call, so nothing in the array has to be cleared first
  fr *ba = scratch, *bb = scratch + pp::kEvalNoAllocMaxBlocks;
  pp::k_affine_local<<<g.blocks, pp::kScanThreads + 32, 0, s>>>(
      static_cast<const fr *>(d_poly), g, static_cast<const fr *>(d_x), 0, nullptr, nullptr, ba, bb);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  pp::k_eval_final<<<1, pp::kScanThreads, 0, s>>>(ba, bb, g.blocks, static_cast<fr *>(d_y));
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}
