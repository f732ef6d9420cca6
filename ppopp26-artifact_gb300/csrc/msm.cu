// msm.cu -- BLS12-381 G1 multi-scalar multiplication sum_i s_i P_i on the
// GPU (Pippenger's bucket method with signed digits).
//
// Replaces multi_scalar_mult (PLONK/utils/function.cu:395-411) ->
// cuda::msm_zkp_cuda (PLONK/utils/zkp/cuda/zksnark_msm.cu:48-88, sppark's
// Pippenger with mont = false) + cpu::msm_collect_cpu (zkp/cpu/
// msmcollect.cpp): same inputs (affine points over Fq in Montgomery form,
// scalars as plain 256-bit integers), one Jacobian point out, with the final
// aggregation on the GPU instead of the host.
//
// Pipeline (all on one stream, workspace slot 3):
//   1. digits    one thread per scalar: c-bit windows recoded to signed
//                digits in [-2^(c-1), 2^(c-1)], bucket |d| - 1 per window
//                (W = floor(256 / c) + 1 windows, so any 256-bit scalar is
//                exact); bucket sizes counted with warp-aggregated atomics
//   2. scan      exclusive prefix sum of the W * 2^(c-1) bucket sizes (tiled)
//   3. scatter   (point index, sign) into each bucket's slice: a counting sort
//   4. buckets   bucket sums in groups of at most K points per thread, then
//                levels of groups of K partial sums for buckets that had more
//                (a bucket can hold up to all n points: equal scalars, or the
//                few-bit top window), so no thread sums more than K values
//   5. segments  one thread per run of G buckets: running sums T = sum
//                (j + 1) B and R = sum B over its run
//   6. windows   sum T + G sum_s s R_s with sum_s s R_s = sum_k 2^k Q_k, Q_k
//                the R_s whose index has bit k set: plain sums in chunks, a
//                block tree per sum, then one warp per window for the Horner
//                chain over k
//   7. final     one warp: Horner over the windows (c doublings each, the
//                independent multiplies of each step on different lanes), one
//                inversion to affine
// Every step is integer-multiply bound (an Fq multiply is ~300 32-bit wide
// products) except the sort, which is a few bytes per point and window.
#include <atomic>
#include <cstring>

#include "common.cuh"
#include "g1.cuh"

namespace pp {
namespace {

constexpr uint32_t kNone = 0xffffffffu;

struct MsmPlan {
  uint32_t c;      // window bits
  uint32_t W;      // windows: W c >= 257, so the top window's carry has a home
  uint32_t B;      // buckets per bucket set, 2^(c-1)
  uint32_t G;      // buckets per aggregation segment
  uint32_t S;      // segments per bucket set, B / G
  uint32_t lgG;    // log2 G
  uint32_t lgS;    // log2 S
  uint32_t nsets;  // bucket sets: W (one per window), or 1 with window tables
};

// Buckets per segment: the longest run (fewer, cheaper window sums) that still
// gives 2^15 segment threads.  On GB300 this beat fixed 4, 8 and 16 (2^16
// points: 16 -> 4.65 ms, 4 -> 3.92 ms; 2^22: 4 -> 53.2 ms, 16 -> 51.3 ms).
constexpr uint32_t kSegmentMax = 16, kSegmentMin = 4, kSegmentThreads = 1u << 15;

// the rest of a plan once c and the number of bucket sets are fixed
MsmPlan msm_plan_for(uint32_t c, uint32_t nsets) {
  MsmPlan p{};
  p.c = c;
  p.W = 256 / c + 1;
  p.B = 1u << (c - 1);
  p.nsets = nsets;
  p.G = kSegmentMax;  // B >= 32 (c >= 6)
  while (p.G > kSegmentMin && (uint64_t)p.nsets * p.B / p.G < kSegmentThreads) p.G >>= 1;
  p.S = p.B / p.G;
  while ((1u << p.lgG) < p.G) ++p.lgG;
  while ((1u << p.lgS) < p.S) ++p.lgS;
  return p;
}

// per-size window bits set by pp_msm_g1_set_window_bits (index: ceil(lg n))
std::atomic<uint32_t> g_window_bits[33];

uint32_t ceil_lg(uint64_t n) {
  uint32_t lg = 0;
  while (lg < 32 && (1ull << lg) < n) ++lg;
  return lg;
}

// Window bits.  Scalars below r < 2^255 leave the top window few digit
// values unless c is 13, 16 or 20 (the top window then spans 232, 29678 or
// 29678 values): with other c about n entries share a handful of buckets, or
// one carry window, and those buckets need extra levels of serial group sums.
// Swept on GB300 (2^12..2^24 points, c = 10..20), these won: 13 up to 2^19
// points (2^14: 2.86 ms against 3.45 for the cost model's 11), 16 up to 2^23
// (2^22: 41.2 against 47.2 for 18), 18 beyond (2^24: 149.8 against 158.6 for
// 20).  Below 2^10 points the cost model decides.
//
// The model minimises W (10 n + 14 2^c) Fq multiplies: the bucket sums (one
// mixed add per point and window) against the aggregation (two adds per
// bucket).
MsmPlan msm_plan(uint64_t n) {
  const uint32_t lg = ceil_lg(n);
  const uint32_t forced = g_window_bits[lg].load(std::memory_order_relaxed);
  if (forced) return msm_plan_for(forced, 256 / forced + 1);
  if (lg >= 10) {
    const uint32_t c = lg <= 19 ? 13 : lg <= 23 ? 16 : 18;
    return msm_plan_for(c, 256 / c + 1);
  }
  uint32_t best_c = 0;
  double best = 0;
  for (uint32_t c = 6; c <= 20; ++c) {
    const double W = 256 / c + 1;
    const double cost = W * (10.0 * (double)n + 14.0 * (double)(1u << c));
    if (best_c == 0 || cost < best) {
      best = cost;
      best_c = c;
    }
  }
  return msm_plan_for(best_c, 256 / best_c + 1);
}

__device__ __forceinline__ g1a ld_g1a(const g1a *p) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  g1a r;
  uint32_t *w = reinterpret_cast<uint32_t *>(&r);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const uint4 u = __ldg(q + k);
    w[4 * k] = u.x;
    w[4 * k + 1] = u.y;
    w[4 * k + 2] = u.z;
    w[4 * k + 3] = u.w;
  }
  return r;
}

// bits [off, off + c) of a 256-bit scalar (8 little-endian words), c <= 20
__device__ __forceinline__ uint32_t window_bits(const uint32_t s[8], uint32_t off, uint32_t c) {
  const uint32_t w = off >> 5, sh = off & 31;
  if (w >= 8) return 0;
  uint64_t x = s[w];
  if (w + 1 < 8) x |= (uint64_t)s[w + 1] << 32;
  return (uint32_t)(x >> sh) & ((1u << c) - 1);
}

// atomicAdd(base + key, 1) for every active lane, one atomic per distinct key
// in the warp; returns the old value plus the lane's rank among equal keys
__device__ __forceinline__ uint32_t warp_increment(uint32_t *base, uint32_t key) {
  const uint32_t mask = __activemask();
  const uint32_t same = __match_any_sync(mask, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(same) - 1;
  uint32_t old = 0;
  if (lane == leader) old = atomicAdd(base + key, (uint32_t)__popc(same));
  old = __shfl_sync(same, old, leader);
  return old + __popc(same & ((1u << lane) - 1));
}

__global__ void k_msm_digits(const uint32_t *__restrict__ scalars, uint64_t n, MsmPlan p,
                             uint32_t *__restrict__ digits, uint32_t *__restrict__ counts) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s[8];
    const uint4 a = __ldg(reinterpret_cast<const uint4 *>(scalars) + 2 * i);
    const uint4 b = __ldg(reinterpret_cast<const uint4 *>(scalars) + 2 * i + 1);
    s[0] = a.x, s[1] = a.y, s[2] = a.z, s[3] = a.w, s[4] = b.x, s[5] = b.y, s[6] = b.z, s[7] = b.w;
    uint32_t carry = 0;
    for (uint32_t w = 0; w < p.W; ++w) {
      const uint32_t raw = window_bits(s, w * p.c, p.c) + carry;
      uint32_t mag, sign;
      if (raw > p.B) {  // d = raw - 2^c < 0
        mag = (1u << p.c) - raw;
        sign = 1;
        carry = 1;
      } else {
        mag = raw;
        sign = 0;
        carry = 0;
      }
      uint32_t e = kNone;
      if (mag) {
        const uint32_t bucket = mag - 1;
        e = (bucket << 1) | sign;
        warp_increment(counts, (p.nsets > 1 ? w * p.B : 0) + bucket);
      }
      digits[(uint64_t)w * n + i] = e;
    }
  }
}

// Exclusive prefix sum of len counts into out (len + 1 entries: the last is
// the total) and, when cursor is not null, a copy of it.  Three launches over
// tiles of 4096 entries: tile sums, a scan of the tile sums, tile scans.
constexpr int kScanThreads = 256, kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_sum[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kScanThreads / 32 ? warp_sum[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += y;
    }
    if (lane < kScanThreads / 32) warp_sum[lane] = w;
  }
  __syncthreads();
  const uint32_t before = (warp ? warp_sum[warp - 1] : 0) + x - v;
  *total = warp_sum[kScanThreads / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kScanThreads)
    k_scan_tiles(const uint32_t *__restrict__ in, uint64_t len, uint32_t *__restrict__ tile_sum) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint32_t v = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
    if (i < len) v += in[i];
  }
  uint32_t total;
  block_excl_scan(v, &total);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// exclusive scan of the tile sums in place, total at [ntiles]
__global__ void __launch_bounds__(kScanThreads) k_scan_top(uint32_t *tile_sum, uint32_t ntiles) {
  const uint32_t per = (ntiles + kScanThreads - 1) / kScanThreads;
  const uint32_t lo = threadIdx.x * per, hi = lo + per < ntiles ? lo + per : ntiles;
  uint32_t v = 0;
  for (uint32_t k = lo; k < hi; ++k) v += tile_sum[k];
  uint32_t total;
  uint32_t run = block_excl_scan(v, &total);
  for (uint32_t k = lo; k < hi; ++k) {
    const uint32_t t = tile_sum[k];
    tile_sum[k] = run;
    run += t;
  }
  if (threadIdx.x == 0) tile_sum[ntiles] = total;
}

__global__ void __launch_bounds__(kScanThreads)
    k_scan_down(const uint32_t *__restrict__ in, uint64_t len, const uint32_t *__restrict__ tile_off,
                uint32_t ntiles, uint32_t *__restrict__ out, uint32_t *__restrict__ cursor) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems], sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < len ? in[base + k] : 0;
    sum += v[k];
  }
  uint32_t total;
  uint32_t run = tile_off[blockIdx.x] + block_excl_scan(sum, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < len) {
      out[base + k] = run;
      if (cursor) cursor[base + k] = run;
    }
    run += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[len] = tile_off[ntiles];
}

int scan_u32(const uint32_t *in, uint64_t len, uint32_t *out, uint32_t *cursor, uint32_t *tiles,
             cudaStream_t s) {
  const uint32_t ntiles = (uint32_t)((len + kScanTile - 1) / kScanTile);
  k_scan_tiles<<<ntiles, kScanThreads, 0, s>>>(in, len, tiles);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_scan_top<<<1, kScanThreads, 0, s>>>(tiles, ntiles);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_scan_down<<<ntiles, kScanThreads, 0, s>>>(in, len, tiles, ntiles, out, cursor);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

// With one bucket set per window an entry names its point i; with window
// tables (one bucket set) it names the table entry w n + i = 2^(c w) P_i.
__global__ void k_msm_scatter(const uint32_t *__restrict__ digits, uint64_t n, MsmPlan p,
                              uint32_t *__restrict__ cursor, uint32_t *__restrict__ list) {
  const uint64_t total = (uint64_t)p.W * n;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t e = digits[t];
    if (e == kNone) continue;
    const uint64_t w = t / n, i = t - w * n;
    const bool per_window = p.nsets > 1;
    const uint32_t pos = warp_increment(cursor, (per_window ? (uint32_t)(w * p.B) : 0u) + (e >> 1));
    list[pos] = (uint32_t)(per_window ? i : t) | ((e & 1u) << 31);
  }
}

constexpr int kPointThreads = 128;
constexpr uint32_t kGroup = 16;  // values summed by one thread (16 beat 32 and 64 on GB300)

// Per bucket at one level: m values to sum.  groups = ceil(m / K) threads; a
// bucket with m <= K is finished by its one group, otherwise its groups leave
// ceil(m / K) partial sums for the next level (next = that count, else 0).
__global__ void k_msm_groups(const uint32_t *__restrict__ m, uint64_t nb,
                             uint32_t *__restrict__ groups, uint32_t *__restrict__ next) {
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb;
       b += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = m[b];
    const uint32_t g = (v + kGroup - 1) / kGroup;
    groups[b] = g;
    next[b] = v > kGroup ? g : 0;
  }
}

// the bucket whose group range [goff[b], goff[b+1]) holds group t
__device__ __forceinline__ uint32_t bucket_of(const uint32_t *goff, uint32_t nb, uint32_t t) {
  uint32_t lo = 0, hi = nb;  // goff[lo] <= t < goff[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (goff[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// One level of bucket sums.  Level 0 (list != null) adds signed affine points
// named by the sorted list; later levels add XYZZ partial sums.  Group t of
// bucket b sums values [off[b] + j K, ...) of that bucket (j = t - goff[b]);
// a finished bucket is written to buckets[b], else to part_out[noff[b] + j].
__global__ void __launch_bounds__(kPointThreads, 3)
    k_msm_level(const g1a *__restrict__ points, const uint32_t *__restrict__ list,
                const g1x *__restrict__ part_in, const uint32_t *__restrict__ m,
                const uint32_t *__restrict__ off, const uint32_t *__restrict__ goff,
                const uint32_t *__restrict__ noff, uint32_t nb, g1x *__restrict__ part_out,
                g1x *__restrict__ buckets) {
  const uint32_t total = goff[nb];
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const uint32_t b = bucket_of(goff, nb, t);
    const uint32_t j = t - goff[b];
    const uint32_t cnt = m[b];
    const uint32_t lo = off[b] + j * kGroup;
    const uint32_t hi = lo + kGroup < off[b] + cnt ? lo + kGroup : off[b] + cnt;
    g1x acc = g1x_inf();
    if (list) {
      for (uint32_t k = lo; k < hi; ++k) {
        const uint32_t e = list[k];
        g1a pt = ld_g1a(points + (e & 0x7fffffffu));
        if (e >> 31) pt = g1a_neg(pt);
        acc = g1x_add_affine(acc, pt);
      }
    } else {
      for (uint32_t k = lo; k < hi; ++k) acc = g1x_add(acc, part_in[k]);
    }
    if (cnt <= kGroup) buckets[b] = acc;
    else part_out[noff[b] + j] = acc;
  }
}

// Segment s of window w holds buckets b = s G + j, j < G.  Its thread leaves
// R_s = sum_j B_b and T_s = sum_j (j + 1) B_b (running sums from the top), so
// that the window sum sum_b (b + 1) B_b = sum_s T_s + G sum_s s R_s.
__global__ void __launch_bounds__(kPointThreads)
    k_msm_segments(const g1x *__restrict__ buckets, MsmPlan p, g1x *__restrict__ seg_t,
                   g1x *__restrict__ seg_r) {
  const uint64_t total = (uint64_t)p.nsets * p.S;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const g1x *row = buckets + t * p.G;  // segments are consecutive in each window
    g1x run = g1x_inf(), sum = g1x_inf();
    for (int j = (int)p.G - 1; j >= 0; --j) {
      run = g1x_add(run, row[j]);
      sum = g1x_add(sum, run);
    }
    seg_t[t] = sum;
    seg_r[t] = run;
  }
}

// Window sums from the segments: sum_b (b + 1) B_b = sum_s T_s + G sum_s s R_s,
// and sum_s s R_s = sum_k 2^k Q_k, where Q_k adds the R_s of the segments whose
// index s has bit k set.  So a window needs 1 + lg S plain sums (sum j = 0 is
// sum_s T_s, sum j = 1 + k is Q_k) and one short Horner chain; no sum weights
// a point by more than one doubling at a time.
//
// Each sum is cut into chunks of kChunk terms; one thread adds one chunk.
// Window w's chunks are part[w ncw + u]: u < nc0 for sum 0, then nc1 chunks
// for each Q_k in order of k.
constexpr uint32_t kChunk = 16;

struct ChunkCounts {
  uint32_t nc0, nc1, ncw;
};

__host__ __device__ __forceinline__ ChunkCounts chunk_counts(const MsmPlan &p) {
  ChunkCounts c;
  c.nc0 = (p.S + kChunk - 1) / kChunk;
  c.nc1 = (p.S / 2 + kChunk - 1) / kChunk;
  c.ncw = c.nc0 + p.lgS * c.nc1;
  return c;
}

__global__ void __launch_bounds__(kPointThreads)
    k_msm_bitsums(const g1x *__restrict__ seg_t, const g1x *__restrict__ seg_r, MsmPlan p,
                  g1x *__restrict__ part) {
  const ChunkCounts cc = chunk_counts(p);
  const uint64_t total = (uint64_t)p.nsets * cc.ncw;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t w = (uint32_t)(t / cc.ncw), u = (uint32_t)(t - (uint64_t)w * cc.ncw);
    g1x acc = g1x_inf();
    if (u < cc.nc0) {
      const g1x *row = seg_t + (uint64_t)w * p.S;
      const uint32_t lo = u * kChunk, hi = lo + kChunk < p.S ? lo + kChunk : p.S;
      for (uint32_t i = lo; i < hi; ++i) acc = g1x_add(acc, row[i]);
    } else {
      const uint32_t k = (u - cc.nc0) / cc.nc1, ch = (u - cc.nc0) - k * cc.nc1;
      const g1x *row = seg_r + (uint64_t)w * p.S;
      const uint32_t half = p.S >> 1;
      const uint32_t lo = ch * kChunk, hi = lo + kChunk < half ? lo + kChunk : half;
      for (uint32_t i = lo; i < hi; ++i) {
        // the i-th segment index with bit k set
        const uint32_t s = ((i >> k) << (k + 1)) | (1u << k) | (i & ((1u << k) - 1));
        acc = g1x_add(acc, row[s]);
      }
    }
    part[t] = acc;
  }
}

// One block per (window, sum): the sum's chunks, then a tree in shared memory.
// sums[w (1 + lg S) + j].
constexpr int kReduceThreads = 128;

__global__ void __launch_bounds__(kReduceThreads)
    k_msm_bitreduce(const g1x *__restrict__ part, MsmPlan p, g1x *__restrict__ sums) {
  __shared__ g1x red[kReduceThreads];
  const ChunkCounts cc = chunk_counts(p);
  const uint32_t L = 1 + p.lgS;
  const uint32_t w = blockIdx.x / L, j = blockIdx.x - w * L;
  const uint64_t first = (uint64_t)w * cc.ncw + (j == 0 ? 0 : cc.nc0 + (j - 1) * cc.nc1);
  const uint32_t cnt = j == 0 ? cc.nc0 : cc.nc1;
  g1x acc = g1x_inf();
  for (uint32_t i = threadIdx.x; i < cnt; i += kReduceThreads) acc = g1x_add(acc, part[first + i]);
  red[threadIdx.x] = acc;
  __syncthreads();
  for (uint32_t h = kReduceThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] = g1x_add(red[threadIdx.x], red[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = red[0];
}

// ---- final Horner chain in one warp.  Every lane holds the same point; the
// independent multiplies of a doubling (3 dependent levels instead of 9
// multiplies) or of an addition (4 levels instead of 14) run on different
// lanes and are exchanged by shuffles.
__device__ __forceinline__ fq shfl_fq(const fq &a, int src) {
  fq r;
#pragma unroll
  for (int i = 0; i < 12; ++i) r.v[i] = __shfl_sync(0xffffffffu, a.v[i], src);
  return r;
}

__device__ g1x dbl_warp(const g1x &p) {
  if (g1x_is_inf(p) || fq_is_zero(p.y)) return g1x_inf();
  const int lane = threadIdx.x & 31;
  const fq u = fq_dbl(p.y);
  // v = u^2 (lane 0), x2 = x^2 (lane 1): squares on every lane
  fq a = lane == 0 ? u : p.x;
  fq r = fq_sqr(a);
  const fq v = shfl_fq(r, 0), x2 = shfl_fq(r, 1);
  const fq m = fq_add(fq_dbl(x2), x2);
  // w = u v (0), s = x v (1), m^2 (2), zz' = v zz (3)
  a = lane == 0 ? u : lane == 1 ? p.x : lane == 2 ? m : v;
  fq b = lane == 0 ? v : lane == 1 ? v : lane == 2 ? m : p.zz;
  r = fq_mul(a, b);
  const fq w = shfl_fq(r, 0), s = shfl_fq(r, 1), m2 = shfl_fq(r, 2), zz = shfl_fq(r, 3);
  g1x o;
  o.x = fq_sub(m2, fq_dbl(s));
  // zzz' = w zzz (0), m (s - x') (1), w y (2)
  a = lane == 1 ? m : w;
  b = lane == 0 ? p.zzz : lane == 1 ? fq_sub(s, o.x) : p.y;
  r = fq_mul(a, b);
  o.zzz = shfl_fq(r, 0);
  o.y = fq_sub(shfl_fq(r, 1), shfl_fq(r, 2));
  o.zz = zz;
  return o;
}

__device__ g1x add_warp(const g1x &p, const g1x &q) {
  if (g1x_is_inf(q)) return p;
  if (g1x_is_inf(p)) return q;
  const int lane = threadIdx.x & 31;
  // u1 = X1 ZZ2, u2 = X2 ZZ1, s1 = Y1 ZZZ2, s2 = Y2 ZZZ1, ZZ1 ZZ2, ZZZ1 ZZZ2
  fq a = lane == 0 ? p.x : lane == 1 ? q.x : lane == 2 ? p.y : lane == 3 ? q.y
         : lane == 4 ? p.zz : p.zzz;
  fq b = lane == 0 ? q.zz : lane == 1 ? p.zz : lane == 2 ? q.zzz : lane == 3 ? p.zzz
         : lane == 4 ? q.zz : q.zzz;
  fq r = fq_mul(a, b);
  const fq u1 = shfl_fq(r, 0), u2 = shfl_fq(r, 1), s1 = shfl_fq(r, 2), s2 = shfl_fq(r, 3);
  const fq zz12 = shfl_fq(r, 4), zzz12 = shfl_fq(r, 5);
  const fq P = fq_sub(u2, u1), R = fq_sub(s2, s1);
  if (fq_is_zero(P)) return fq_is_zero(R) ? dbl_warp(p) : g1x_inf();
  // P^2 (0), R^2 (1)
  a = lane == 0 ? P : R;
  r = fq_sqr(a);
  const fq pp = shfl_fq(r, 0), rr = shfl_fq(r, 1);
  // P pp (0), u1 pp (1), zz12 pp (2)
  a = lane == 0 ? P : lane == 1 ? u1 : zz12;
  r = fq_mul(a, pp);
  const fq ppp = shfl_fq(r, 0), Q = shfl_fq(r, 1);
  g1x o;
  o.zz = shfl_fq(r, 2);
  o.x = fq_sub(fq_sub(rr, ppp), fq_dbl(Q));
  // R (Q - x') (0), s1 ppp (1), zzz12 ppp (2)
  a = lane == 0 ? R : lane == 1 ? s1 : zzz12;
  b = lane == 0 ? fq_sub(Q, o.x) : ppp;
  r = fq_mul(a, b);
  o.y = fq_sub(shfl_fq(r, 0), shfl_fq(r, 1));
  o.zzz = shfl_fq(r, 2);
  return o;
}

// One warp per window: win[w] = sum_s T_s + G sum_k 2^k Q_k (Horner over k)
__global__ void __launch_bounds__(32) k_msm_wincombine(const g1x *__restrict__ sums, MsmPlan p,
                                                       g1x *__restrict__ win) {
  const uint32_t w = blockIdx.x;
  const g1x *q = sums + (uint64_t)w * (1 + p.lgS);  // q[0] = sum T, q[1 + k] = Q_k
  g1x acc = p.lgS ? q[p.lgS] : g1x_inf();
  for (int k = (int)p.lgS - 2; k >= 0; --k) acc = add_warp(dbl_warp(acc), q[1 + k]);
  for (uint32_t i = 0; i < p.lgG; ++i) acc = dbl_warp(acc);
  acc = add_warp(acc, q[0]);
  if (threadIdx.x == 0) win[w] = acc;
}

// Horner over the windows (one warp), then affine; out = Jacobian (x, y, 1),
// or all zero for the point at infinity
__global__ void __launch_bounds__(32) k_msm_final(const g1x *__restrict__ win, MsmPlan p,
                                                  fq *__restrict__ out) {
  g1x acc = win[p.nsets - 1];
  for (int w = (int)p.nsets - 2; w >= 0; --w) {
    for (uint32_t k = 0; k < p.c; ++k) acc = dbl_warp(acc);
    acc = add_warp(acc, win[w]);
  }
  if (threadIdx.x != 0) return;
  const g1a a = g1x_to_affine(acc);
  const bool inf = g1x_is_inf(acc);
  out[0] = a.x;
  out[1] = a.y;
  out[2] = inf ? fq_zero() : fq_one();
}

struct MsmLayout {
  size_t digits, counts, offsets, cursor, list, groups, goff, next[2], noff[2], part[2], buckets,
      seg_t, seg_r, chunks, sums, win, tiles, total;
  uint64_t part_cap;  // partial sums one level can leave
  uint32_t levels;    // group levels: K^levels >= the largest bucket
};

MsmLayout msm_layout(uint64_t n, const MsmPlan &p) {
  MsmLayout L{};
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const uint64_t nb = (uint64_t)p.nsets * p.B;
  const uint64_t entries = (uint64_t)p.W * n;
  // a bucket of m > K values leaves ceil(m / K) <= 2 m / K partial sums
  L.part_cap = 2 * entries / kGroup + 1;
  // a bucket holds at most one entry per point and window: n with a bucket
  // set per window, W n when all windows share one
  const uint64_t largest = p.nsets > 1 ? n : entries;
  L.levels = 1;
  for (uint64_t span = kGroup; span < largest; span *= kGroup) ++L.levels;
  size_t o = 0;
  L.digits = o, o += up(entries * 4);
  L.counts = o, o += up(nb * 4);
  L.offsets = o, o += up((nb + 1) * 4);
  L.cursor = o, o += up(nb * 4);
  L.list = o, o += up(entries * 4);
  L.groups = o, o += up(nb * 4);
  L.goff = o, o += up((nb + 1) * 4);
  for (int k = 0; k < 2; ++k) {
    L.next[k] = o, o += up(nb * 4);
    L.noff[k] = o, o += up((nb + 1) * 4);
  }
  L.part[0] = o, o += up(L.part_cap * sizeof(g1x));
  L.part[1] = o, o += up(L.part_cap * sizeof(g1x));
  L.buckets = o, o += up(nb * sizeof(g1x));
  L.seg_t = o, o += up((size_t)p.nsets * p.S * sizeof(g1x));
  L.seg_r = o, o += up((size_t)p.nsets * p.S * sizeof(g1x));
  L.chunks = o, o += up((size_t)p.nsets * chunk_counts(p).ncw * sizeof(g1x));
  L.sums = o, o += up((size_t)p.nsets * (1 + p.lgS) * sizeof(g1x));
  L.win = o, o += up((size_t)p.nsets * sizeof(g1x));
  L.tiles = o, o += up(((nb + kScanTile - 1) / kScanTile + 1) * 4);
  L.total = o;
  return L;
}

// one thread per unit of work (loops stride only past 2^31 - 1 blocks): 2^20
// points took 13.77 ms, against 14.09 ms with grids capped at 8-16 blocks
// per SM
unsigned grid_for(uint64_t work, int threads) {
  const uint64_t want = (work + threads - 1) / threads;
  const uint64_t cap = 0x7fffffffull;
  return (unsigned)(want < cap ? (want ? want : 1) : cap);
}

// ---- window tables of a fixed point set: table[w n + i] = 2^(c w) P_i in
// affine form.  Window w + 1 comes from window w by c doublings in XYZZ and a
// batched conversion back to affine: Montgomery's simultaneous inversion over
// runs of kTableRun points, one field inversion per run.
constexpr uint32_t kTableRun = 32;

__global__ void __launch_bounds__(kPointThreads)
    k_msm_table_double(const g1a *__restrict__ prev, uint64_t n, uint32_t c, g1x *__restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    g1x q = g1x_dbl_affine(ld_g1a(prev + i));
    for (uint32_t k = 1; k < c; ++k) q = g1x_dbl(q);
    out[i] = q;
  }
}

// x = X / ZZ, y = Y / ZZZ with 1 / (ZZ ZZZ) from the run's one inversion; the
// forward pass parks the running products in out[].x, the backward pass reads
// each one before it overwrites it.  Infinity (ZZ = 0) becomes all zero.
__global__ void __launch_bounds__(kPointThreads)
    k_msm_table_affine(const g1x *__restrict__ q, uint64_t n, g1a *__restrict__ out) {
  const uint64_t runs = (n + kTableRun - 1) / kTableRun;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < runs;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = r * kTableRun, hi = lo + kTableRun < n ? lo + kTableRun : n;
    fq acc = fq_one();
    for (uint64_t j = lo; j < hi; ++j) {
      const g1x p = q[j];
      if (!g1x_is_inf(p)) acc = fq_mul(acc, fq_mul(p.zz, p.zzz));
      out[j].x = acc;
    }
    fq inv = fq_inv_fast(acc);  // acc is a product of non-zero values
    for (uint64_t j = hi; j > lo; --j) {
      const g1x p = q[j - 1];
      g1a a;
      if (g1x_is_inf(p)) {
        a.x = fq_zero();
        a.y = fq_zero();
      } else {
        const fq before = j - 1 > lo ? out[j - 2].x : fq_one();
        const fq inv_d = fq_mul(inv, before);  // 1 / (ZZ ZZZ) of this point
        inv = fq_mul(inv, fq_mul(p.zz, p.zzz));
        a.x = fq_mul(p.x, fq_mul(inv_d, p.zzz));
        a.y = fq_mul(p.y, fq_mul(inv_d, p.zz));
      }
      out[j - 1] = a;
    }
  }
}

// Window bits for a fixed point set, from the same kind of sweep (c = 12..20,
// 2^14..2^24 points on GB300) and the same top-window effect: 13 up to 2^14
// points, 16 up to 2^21 (2^20: 10.72 ms against 10.98 for 17 and 11.83 for
// 15), 20 beyond (2^22: 33.8 against 35.8 for 19).  One bucket set serves all
// windows, so a large c costs little aggregation.
uint32_t fixed_window_bits(uint64_t n) {
  const uint32_t lg = ceil_lg(n);
  return lg <= 14 ? 13 : lg <= 21 ? 16 : 20;
}

// The pipeline behind both entry points.  points holds n affine points (one
// bucket set per window) or the W n window-table entries (one bucket set);
// scalars n plain 256-bit integers; out receives (x, y, 1), or zeros.
int msm_run(const g1a *points, const uint32_t *scalars, uint64_t n, const MsmPlan &p, fq *out,
            cudaStream_t s) {
  const MsmLayout L = msm_layout(n, p);
  int st = PP_OK;
  char *ws = static_cast<char *>(workspace_get(L.total, s, 3, &st));
  if (st) return st;
  auto u32 = [&](size_t off) { return reinterpret_cast<uint32_t *>(ws + off); };
  auto pts = [&](size_t off) { return reinterpret_cast<g1x *>(ws + off); };
  uint32_t *digits = u32(L.digits), *counts = u32(L.counts), *offsets = u32(L.offsets);
  uint32_t *cursor = u32(L.cursor), *list = u32(L.list), *groups = u32(L.groups);
  uint32_t *goff = u32(L.goff), *tiles = u32(L.tiles);
  g1x *buckets = pts(L.buckets), *seg_t = pts(L.seg_t), *seg_r = pts(L.seg_r), *win = pts(L.win);
  g1x *chunks = pts(L.chunks), *sums = pts(L.sums);
  const uint64_t nb = (uint64_t)p.nsets * p.B;

  // 1-3: signed digits, bucket sizes, counting sort of (point, sign) by bucket
  PP_CUDA_TRY(cudaMemsetAsync(counts, 0, nb * 4, s));
  k_msm_digits<<<grid_for(n, 256), 256, 0, s>>>(scalars, n, p, digits, counts);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  if ((st = scan_u32(counts, nb, offsets, cursor, tiles, s))) return st;
  k_msm_scatter<<<grid_for((uint64_t)p.W * n, 256), 256, 0, s>>>(digits, n, p, cursor, list);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();

  // 4: bucket sums, at most K values per thread, over L.levels levels
  PP_CUDA_TRY(cudaMemsetAsync(buckets, 0, nb * sizeof(g1x), s));  // all zero = infinity
  const uint32_t *m = counts, *off = offsets;
  const g1x *part_in = nullptr;
  for (uint32_t lv = 0; lv < L.levels; ++lv) {
    uint32_t *next = u32(L.next[lv & 1]), *noff = u32(L.noff[lv & 1]);
    g1x *part_out = pts(L.part[lv & 1]);
    k_msm_groups<<<grid_for(nb, 256), 256, 0, s>>>(m, nb, groups, next);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    if ((st = scan_u32(groups, nb, goff, nullptr, tiles, s))) return st;
    if ((st = scan_u32(next, nb, noff, nullptr, tiles, s))) return st;
    k_msm_level<<<grid_for((uint64_t)p.W * n / 4 + nb, kPointThreads), kPointThreads, 0, s>>>(
        points, lv == 0 ? list : nullptr, part_in, m, off, goff, noff,
        (uint32_t)nb, part_out, buckets);
    PP_COUNT_LAUNCH();
    PP_LAUNCH_CHECK();
    m = next;
    off = noff;
    part_in = part_out;
  }

  // 5-7: weighted bucket sums per bucket set, sets combined, affine result
  k_msm_segments<<<grid_for((uint64_t)p.nsets * p.S, kPointThreads), kPointThreads, 0, s>>>(
      buckets, p, seg_t, seg_r);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_msm_bitsums<<<grid_for((uint64_t)p.nsets * chunk_counts(p).ncw, kPointThreads), kPointThreads,
                  0, s>>>(seg_t, seg_r, p, chunks);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_msm_bitreduce<<<p.nsets * (1 + p.lgS), kReduceThreads, 0, s>>>(chunks, p, sums);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_msm_wincombine<<<p.nsets, 32, 0, s>>>(sums, p, win);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  k_msm_final<<<1, 32, 0, s>>>(win, p, out);
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}

}  // namespace
}  // namespace pp

extern "C" int pp_msm_g1(const void *d_points, const void *d_scalars, uint64_t n, void *d_out,
                         void *stream) {
  using namespace pp;
  auto aligned16 = [](const void *q) { return q && (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
  if (!aligned16(d_out) || (n && (!aligned16(d_points) || !aligned16(d_scalars)))) {
    set_error("pp_msm_g1: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  if (n >= (1ull << 31)) {
    set_error("pp_msm_g1: n = %llu points; at most 2^31 - 1", (unsigned long long)n);
    return PP_E_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    PP_CUDA_TRY(cudaMemsetAsync(d_out, 0, 3 * sizeof(fq), s));
    return PP_OK;
  }
  const MsmPlan p = msm_plan(n);
  if ((uint64_t)p.W * n >= (1ull << 32)) {
    set_error("pp_msm_g1: n = %llu points is too many for 32-bit bucket offsets",
              (unsigned long long)n);
    return PP_E_UNSUPPORTED;
  }
  return msm_run(static_cast<const g1a *>(d_points), static_cast<const uint32_t *>(d_scalars), n, p,
                 static_cast<fq *>(d_out), s);
}

extern "C" int pp_msm_g1_window_bits(uint64_t n) { return (int)pp::msm_plan(n).c; }

extern "C" int pp_msm_g1_set_window_bits(uint32_t lg_n, uint32_t window_bits) {
  if (lg_n > 32 || (window_bits && (window_bits < 6 || window_bits > 20))) {
    pp::set_error("pp_msm_g1_set_window_bits: lg_n <= 32 and window_bits 0 or 6..20");
    return PP_E_INVAL;
  }
  pp::g_window_bits[lg_n].store(window_bits, std::memory_order_relaxed);
  return PP_OK;
}

// ---- fixed-base form: the window tables of one point set stay in HBM ----
struct pp_msm_bases {
  int device;
  uint64_t n;
  uint32_t c;
  pp::g1a *table;  // W n affine points, table[w n + i] = 2^(c w) P_i
};

extern "C" int pp_msm_g1_bases_create(const void *d_points, uint64_t n, uint32_t window_bits,
                                      pp_msm_bases **bases, void *stream) {
  using namespace pp;
  if (!bases) {
    set_error("pp_msm_g1_bases_create: null handle pointer");
    return PP_E_INVAL;
  }
  *bases = nullptr;
  if (!d_points || (reinterpret_cast<uintptr_t>(d_points) & 15)) {
    set_error("pp_msm_g1_bases_create: points must be a 16-byte aligned device pointer");
    return PP_E_INVAL;
  }
  if (n == 0 || (window_bits && (window_bits < 6 || window_bits > 20))) {
    set_error("pp_msm_g1_bases_create: need n >= 1 and window_bits 0 (automatic) or 6..20");
    return PP_E_INVAL;
  }
  const uint32_t c = window_bits ? window_bits : fixed_window_bits(n);
  const uint64_t W = 256 / c + 1;
  if (W * n >= (1ull << 31)) {
    set_error("pp_msm_g1_bases_create: %llu windows x %llu points exceed 2^31 table entries",
              (unsigned long long)W, (unsigned long long)n);
    return PP_E_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  g1a *table = nullptr;
  PP_COUNT_ALLOC(W * n * sizeof(g1a));
  if (cudaMalloc(&table, W * n * sizeof(g1a)) != cudaSuccess) {
    cudaGetLastError();
    set_error("pp_msm_g1_bases_create: cannot allocate %llu bytes of window tables",
              (unsigned long long)(W * n * sizeof(g1a)));
    return PP_E_NOMEM;
  }
  g1x *tmp = nullptr;
  PP_COUNT_ALLOC(n * sizeof(g1x));
  if (cudaMallocAsync(&tmp, n * sizeof(g1x), s) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(table);
    set_error("pp_msm_g1_bases_create: cannot allocate %llu bytes of scratch",
              (unsigned long long)(n * sizeof(g1x)));
    return PP_E_NOMEM;
  }
  int st = PP_OK;
  if (cudaMemcpyAsync(table, d_points, n * sizeof(g1a), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
    st = PP_E_CUDA;
    set_error("pp_msm_g1_bases_create: copying the points failed: %s",
              cudaGetErrorString(cudaGetLastError()));
  }
  for (uint64_t w = 1; st == PP_OK && w < W; ++w) {
    k_msm_table_double<<<grid_for(n, kPointThreads), kPointThreads, 0, s>>>(table + (w - 1) * n,
                                                                               n, c, tmp);
    PP_COUNT_LAUNCH();
    k_msm_table_affine<<<grid_for((n + kTableRun - 1) / kTableRun, kPointThreads), kPointThreads,
                         0, s>>>(tmp, n, table + w * n);
    PP_COUNT_LAUNCH();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      st = PP_E_CUDA;
      set_error("pp_msm_g1_bases_create: kernel launch failed: %s", cudaGetErrorString(e));
    }
  }
  cudaFreeAsync(tmp, s);
  if (st) {
    cudaFree(table);
    return st;
  }
  *bases = new pp_msm_bases{dev, n, c, table};
  return PP_OK;
}

extern "C" int pp_msm_g1_bases_destroy(pp_msm_bases *bases) {
  if (!bases) return PP_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(bases->device);
  const cudaError_t e = cudaFree(bases->table);
  cudaSetDevice(cur);
  delete bases;
  if (e != cudaSuccess) {
    pp::set_error("pp_msm_g1_bases_destroy: cudaFree failed: %s", cudaGetErrorString(e));
    return PP_E_CUDA;
  }
  return PP_OK;
}

extern "C" int pp_msm_g1_bases_info(const pp_msm_bases *bases, uint64_t *n, uint32_t *window_bits,
                                    uint64_t *table_bytes) {
  if (!bases) {
    pp::set_error("pp_msm_g1_bases_info: null handle");
    return PP_E_INVAL;
  }
  const uint64_t W = 256 / bases->c + 1;
  if (n) *n = bases->n;
  if (window_bits) *window_bits = bases->c;
  if (table_bytes) *table_bytes = W * bases->n * sizeof(pp::g1a);
  return PP_OK;
}

extern "C" int pp_msm_g1_fixed(const pp_msm_bases *bases, const void *d_scalars, void *d_out,
                               void *stream) {
  using namespace pp;
  auto aligned16 = [](const void *q) { return q && (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
  if (!bases || !aligned16(d_scalars) || !aligned16(d_out)) {
    set_error("pp_msm_g1_fixed: need a handle and 16-byte aligned device buffers");
    return PP_E_INVAL;
  }
  int dev = 0;
  PP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != bases->device) {
    set_error("pp_msm_g1_fixed: the tables live on device %d, the current device is %d",
              bases->device, dev);
    return PP_E_INVAL;
  }
  return msm_run(bases->table, static_cast<const uint32_t *>(d_scalars), bases->n,
                 msm_plan_for(bases->c, 1), static_cast<fq *>(d_out), (cudaStream_t)stream);
}

// ---- s_i G for the generator: test and benchmark points, commitments to
// known constants.  One thread per scalar, double-and-add from bit 255.
namespace pp {
namespace {

__global__ void __launch_bounds__(kPointThreads)
    k_g1_mul_gen(const uint32_t *__restrict__ scalars, uint64_t n, g1a *__restrict__ out) {
  const g1a G = g1_generator();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) s[k] = scalars[8 * i + k];
    g1x acc = g1x_inf();
    for (int b = 255; b >= 0; --b) {
      acc = g1x_dbl(acc);
      if ((s[b >> 5] >> (b & 31)) & 1u) acc = g1x_add_affine(acc, G);
    }
    out[i] = g1x_to_affine(acc);
  }
}

}  // namespace
}  // namespace pp

extern "C" int pp_g1_mul_gen(const void *d_scalars, uint64_t n, void *d_out, void *stream) {
  using namespace pp;
  auto aligned16 = [](const void *q) { return q && (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
  if (n == 0) return PP_OK;
  if (!aligned16(d_scalars) || !aligned16(d_out)) {
    set_error("pp_g1_mul_gen: buffers must be 16-byte aligned device pointers");
    return PP_E_INVAL;
  }
  k_g1_mul_gen<<<grid_for(n, kPointThreads), kPointThreads, 0, (cudaStream_t)stream>>>(
      static_cast<const uint32_t *>(d_scalars), n, static_cast<g1a *>(d_out));
  PP_COUNT_LAUNCH();
  PP_LAUNCH_CHECK();
  return PP_OK;
}
