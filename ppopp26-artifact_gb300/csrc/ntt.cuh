// ntt.cuh -- in-HBM multi-pass NTT engine (internal interface).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "fr.cuh"

namespace pp {

// Everything one launch of the pass kernel needs for one pass of one transform.
struct PassArgs {
  const fr *in;
  fr *out;
  const fr *tw_inner;  // w_R^e, e < R
  const fr *tw_layer;  // w_{R S}^(c k) at [k][c], or null
  // split layer twiddles (when tw_layer is null): w_{R S}^e =
  // tw_hi[e >> tw_lgh] * tw_lo[e mod 2^tw_lgh], e = c k, or null
  const fr *tw_lo, *tw_hi;
  const fr *diag;      // first pass, NTT_IN_DIAG
  // split diagonal (when non-null): diag factor of element g is
  // diag[g mod 2^diag_lgh] * diag_hi[g >> diag_lgh]
  const fr *diag_hi;
  fr post_scale;
  uint64_t n_valid;
  uint32_t lgR, lgT, lgS, lgN;
  uint32_t first, last, has_post_scale, in_kind, spread;
  uint32_t unit_in, unit_out;  // move 16-byte halves (host-memory input / output)
  uint32_t zero_lg;  // first pass: rows >= R >> zero_lg of every tile are zero (padding)
  uint32_t tw_lgh;   // split layer twiddles: bits of the low table
  uint32_t diag_lgh; // split diagonal: bits of the low table
  uint32_t P;
  uint32_t lgRp[4];
};

// Host-side field helpers (exact, via the host emulation of fr.cuh).
fr host_root_of_unity(int lg, bool inverse);  // 7^((r-1)/2^lg) (or its inverse)
fr host_mont_small(uint64_t x);               // Montgomery form of a small integer
fr host_pow(const fr &a, uint64_t e);
fr host_inv(const fr &a);

// Input side of a forward/inverse transform of 2^lg_m points:
//   NTT_IN_PLAIN : in[i] for i < n_valid, 0 above (zero padding)
//   NTT_IN_DIAG  : in[i] * diag[i] for i < n_valid, 0 above
//   NTT_IN_SPREAD: in[i >> spread] where i is a multiple of 2^spread, else 0
enum NttInput { NTT_IN_PLAIN = 0, NTT_IN_DIAG = 1, NTT_IN_SPREAD = 2 };

struct NttInputDesc {
  int kind = NTT_IN_PLAIN;
  const fr *diag = nullptr;
  // NTT_IN_DIAG with split tables: diag holds h^j (j < 2^diag_lgh) and
  // diag_hi holds h^(j 2^diag_lgh), so the factor h^g costs one more multiply
  // and O(2^(lg / 2)) table entries instead of 2^lg
  const fr *diag_hi = nullptr;
  uint32_t diag_lgh = 0;
  uint64_t n_valid = 0;  // 0 = all 2^lg_m
  uint32_t spread = 0;
  // the input / output is page-locked host memory: the first pass reads and
  // the last pass writes in 16-byte halves, so every warp access covers whole
  // 128-byte lines of the NVLink-C2C traffic
  bool in_host = false;
  bool out_host = false;
};

// The transform of 2^lg_m points with every pass reading and writing
// page-locked host memory (h_in -> h_out, intermediates in h_scratch, all
// three distinct) and the layer twiddles taken from split tables, so device
// memory holds only tables of O(2^(lg_m / 2)) elements whatever lg_m is.
int ntt_run_host_passes(const fr *h_in, fr *h_out, fr *h_scratch, uint32_t lg_m, bool inverse,
                        cudaStream_t stream);
// The same with an input side (NTT_IN_PLAIN with n_valid, NTT_IN_DIAG with
// split tables (diag_hi) above 2^11 points, NTT_IN_SPREAD); the host flags of
// `in` are ignored (both ends are host memory).
int ntt_run_host_passes(const fr *h_in, fr *h_out, fr *h_scratch, uint32_t lg_m, bool inverse,
                        const NttInputDesc &in, cudaStream_t stream);

// Passes of the plan ntt_run_host_passes uses for 2^lg_m points (1 up to 2^11).
int ntt_host_plan_passes(uint32_t lg_m, uint32_t *passes);

// Runs the transform of 2^lg_m points: d_in -> d_out (may alias), on stream.
// Returns a PP_* status.  Tables are built and cached on first use per device.
int ntt_run(const fr *d_in, fr *d_out, uint32_t lg_m, bool inverse, const NttInputDesc &in,
            cudaStream_t stream);

// Per-pass descriptors (and tile counts) of one transform whose passes use
// `work` (2^lg_m elements) between them; for batch plans.  lg_m >= 3.
// small = the latency form of single calls (ntt_small_form); batch plans use
// the throughput form.
int ntt_describe(const fr *d_in, fr *d_out, fr *work, uint32_t lg_m, bool inverse,
                 const NttInputDesc &in, std::vector<PassArgs> &passes,
                 std::vector<uint64_t> &tiles, bool small = false);

// Single calls of 2^9 .. 2^17 points run the latency form: two passes with
// one column per tile (k_ntt_small_pass).  Those sizes are bound by latency
// (a few microseconds of work), and the throughput plan's 2048-element tiles
// would leave most SMs idle.
inline bool ntt_small_form(uint32_t lg_m) { return lg_m >= 9 && lg_m <= 17; }
// One launch over the tiles of up to kLevelJobs job passes, one block per
// tile.  The arguments travel as the kernel's parameters (20.5 KB; CUDA
// allows 32 KB): the tile code then reads them as constant operands, as
// k_ntt_pass does.  Two earlier forms were slower: arguments in device memory
// loaded into registers (tiles 15 % slower than separate pass launches), and
// a persistent grid striding over the tiles (a 96-polynomial batch took
// 28.8 ms against 25.6 ms for one block per tile).
constexpr uint32_t kLevelJobs = 128;
struct LevelParams {
  uint64_t tile_start[kLevelJobs];  // job j's tiles are tile_start[j] .. tile_start[j+1]-1
  PassArgs args[kLevelJobs];
  uint64_t total_tiles;
  uint32_t count;
};
int ntt_launch_level(const LevelParams &params, cudaStream_t stream);

// Builds (or fetches) the cached tables for a transform size (for graph capture
// the tables must exist before capture starts).
int ntt_prepare(uint32_t lg_m, bool inverse);

// h^i for i < n as a cached device table (coset diagonals)
const fr *pow_table(const fr &h, uint32_t lg_n, int *status);

// radix plan override for the autotuner: bits per pass (0-terminated); pass
// nullptr to restore the default split.
int ntt_set_split(uint32_t lg_m, const uint32_t *bits);
void ntt_get_split(uint32_t lg_m, uint32_t *bits, uint32_t *npass);

void ntt_release_tables();

}  // namespace pp
