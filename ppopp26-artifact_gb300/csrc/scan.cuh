// scan.cuh -- blocked-scan geometry shared by the single-call and batched
// grand-product / evaluation / division kernels (internal interface).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fr.cuh"

namespace pp {

constexpr int kScanThreads = 256;

// n elements, k per thread, ceil(n / k) threads in blocks of kScanThreads
struct ScanGeom {
  uint64_t n;
  uint64_t k;
  uint64_t threads;
  uint32_t blocks;
};

int device_sm_count();

// about blocks_per_sm blocks of 256 threads per SM, at least 4 elements per
// thread (fewer blocks: longer chunks, fewer summaries to scan)
inline ScanGeom scan_geom(uint64_t n, uint32_t blocks_per_sm = 4) {
  ScanGeom g;
  g.n = n;
  const uint64_t target_threads = (uint64_t)device_sm_count() * blocks_per_sm * kScanThreads;
  uint64_t k = (n + target_threads - 1) / target_threads;
  if (k < 4) k = 4;
  g.k = k;
  g.threads = (n + k - 1) / k;
  g.blocks = (uint32_t)((g.threads + kScanThreads - 1) / kScanThreads);
  return g;
}

// one grand product of a batch: exclusive prefix product in -> out (may alias)
struct GpBatchJob {
  const fr *in;
  fr *out;
  ScanGeom g;
  fr *thread_excl;  // g.threads elements
  fr *block_total;  // g.blocks elements
};

// two launches over the blocks of all jobs (d_block_start: count prefix sums)
int gp_batch_launch(const GpBatchJob *d_jobs, const uint32_t *d_block_start, uint32_t count,
                    uint32_t total_blocks, cudaStream_t stream);

}  // namespace pp
