/*
 * pp_ops.h -- C ABI of the GB300 Fr prover-operator library (libppfr.so).
 *
 * Every entry point takes plain pointers and sizes.  Field elements are
 * BLS12-381 scalar-field values, 32 bytes each: 4 little-endian uint64 limbs,
 * Montgomery form with R = 2^256, canonical (< r) -- the reference's in-memory
 * format (PLONK/utils/mont/cuda/ff/bls12-381.hpp:7-45; raw files read by
 * miss_ops.cu:8-24).  "d_" pointers are device pointers of the current CUDA
 * device; "stream" is a cudaStream_t (NULL = legacy default stream).  All
 * calls are stream-ordered and asynchronous unless stated otherwise; the
 * caller owns all buffers.  The library owns only cached constant tables and
 * per-stream workspace, created on first use and kept until pp_release().
 *
 * Every call returns PP_OK (0) or an error status; it never exits or traps.
 * pp_last_error() gives a message for the calling thread's last failure.
 */
#ifndef PP_OPS_H
#define PP_OPS_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PP_OK 0
#define PP_E_INVAL 1       /* bad argument (size, alignment, null pointer) */
#define PP_E_NOMEM 2       /* device allocation failed or over the memory budget */
#define PP_E_CUDA 3        /* CUDA runtime error */
#define PP_E_TIMEOUT 4     /* a bounded device-side wait ran out */
#define PP_E_UNSUPPORTED 5 /* size outside what this build supports */
#define PP_E_CANCELLED 6   /* serving: request cancelled */
#define PP_E_BUSY 7        /* serving: admission refused (queue or budget full) */

#define PP_MAX_LG_N 30 /* largest transform handled: 2^30 elements */

const char *pp_status_string(int status);
const char *pp_last_error(void);
/* library version string and build architecture ("sm_103a") */
const char *pp_version(void);

/* ---------------------------------------------------------------- NTT ---
 * Natural-order in, natural-order out transform of 2^lg_n elements,
 * X_k = sum_j x_j w^(jk) with w = 7^((r-1)/2^lg_n); inverse = 1 uses w^-1 and
 * scales by 2^-lg_n.  d_in == d_out is allowed (in place).
 * Replaces Ntt::forward / Intt::forward (PLONK/utils/function.cu:280, :330 ->
 * PLONK/utils/zkp/cuda/zksnark_ntt.cu:342-393), the transform the reference's
 * segmented our_ntt (ntt.cu:979-1037) and four-step standard4_ntt
 * (ntt.cu:1039-1138) reproduce bit for bit.  0 <= lg_n <= PP_MAX_LG_N. */
int pp_ntt(const void *d_in, void *d_out, uint32_t lg_n, int inverse, void *stream);

/* Builds (synchronously) the cached twiddle tables of a transform size so
 * that later pp_ntt calls of that size only launch the pass kernels (e.g.
 * before CUDA-graph capture).  The reference builds its table blob in the
 * Ntt constructor (function.cu:278 -> zksnark_ntt.cu:17-39). */
int pp_ntt_prepare(uint32_t lg_n, int inverse);

/* Radix split of a transform size: bits = 0-terminated pass sizes (log2,
 * each 3..11, at most 4, summing to lg_n); NULL restores the default.  The
 * reference fixes its split per kernel (ntt.cuh:113-170; the segmented
 * drivers take lg_i/lg_k arguments, ntt.cu:979); here it is a tunable. */
int pp_ntt_set_split(uint32_t lg_n, const uint32_t *bits);
int pp_ntt_get_split(uint32_t lg_n, uint32_t *bits4);
/* Times every balanced ordered split of 2^lg_n on the current GPU (CUDA
 * events, reps calls each), keeps the fastest and returns it (and its time).
 * Allocates and synchronises: a set-up step, not for hot paths. */
int pp_ntt_autotune(uint32_t lg_n, int reps, uint32_t *best_bits4, float *best_ms);
/* Persist / restore the chosen splits as JSON keyed by GPU name
 * ({"gpu": ..., "ntt": {"<lg>": [k1, ...]}}); load ignores another GPU's file. */
int pp_tune_save(const char *path);
int pp_tune_load(const char *path);

/* Measured integer-pipe rates of the current GPU, the denominators of the
 * integer roofline: out[0] mad.lo.u32, out[1] mad.hi.u32, out[2] mad.wide.u32
 * (64-bit addend) lane operations per second, each from a full-occupancy loop
 * of independent chains; out[3] standalone Montgomery multiplies per second.
 * No counterpart in the reference.  About 40 ms of GPU time. */
int pp_measure_int_rates(double out[4]);

/* The same rates and two more: out[4] mul.wide.u32 (no addend) lane
 * operations per second, out[5] mul.wide.u32 followed by a dependent add.u64
 * (the addend on the ALU instead), per second.  n is 4 .. 6; out[i] for
 * i < n is written.  No counterpart in the reference. */
int pp_measure_int_rates_ex(double *out, int n);

/* ---------------------------------------------------------------- LDE ---
 * Low-degree extension onto 2^(lg_n+lambda) points, natural order out.
 *  mode 0 (PP_LDE_COEFFS): d_in holds 2^lg_n coefficients a_i; output is
 *    p(h * w_L^k) with h = 7^(2^lambda), w_L the 2^(lg_n+lambda)-th root:
 *    the function the reference's our_lde computes (lde.cu:1267-1365 with
 *    lde_spread_powers_kernel lde.cu:623-648).
 *  mode 1 (PP_LDE_EVALS): d_in holds evaluations on the size-2^lg_n subgroup;
 *    INTT, multiply coefficient i by 7^i, zero-pad, NTT: p(7 * w_L^k).
 *  mode 2 (PP_LDE_SPREAD): the reference's naive_lde baseline (lde.cu:1367,
 *    spread at :479-491): inputs placed at i << lambda, no coset factor.
 *    That transform equals NTT_N(a)[k mod N]; it is computed as one
 *    2^lg_n-point transform and 2^lambda - 1 copies.
 * d_out must not overlap d_in.  lambda <= 8. */
#define PP_LDE_COEFFS 0
#define PP_LDE_EVALS 1
#define PP_LDE_SPREAD 2
int pp_lde(const void *d_in, void *d_out, uint32_t lg_n, uint32_t lambda, uint32_t mode,
           void *stream);

/* ------------------------------------------------- host-resident forms ---
 * The same transforms with input and output in page-locked host memory
 * (cudaHostAlloc / cudaMallocHost / cudaHostRegister).  The first pass reads
 * the input from host memory and the last pass writes the output there
 * (NVLink-C2C on Grace hosts); the intermediate passes use an HBM workspace.
 * Asynchronous on the stream: synchronise it before reading h_out.  A buffer
 * that is not page-locked host memory is refused with PP_E_INVAL before any
 * kernel is launched.  h_in == h_out is allowed for pp_ntt_host.
 * Replaces the reference's host-resident drivers our_ntt (ntt.cu:979-1037,
 * in place on a pinned host buffer, with run_first_ntt_pass :801 and
 * run_second_ntt_pass_async_scatter :861 staging chunks through the device
 * and permuting on the CPU) and our_lde (lde.cu:1267-1365, host input
 * lde.cu:1033 run_first_lde_pass, host output). */
int pp_ntt_host(const void *h_in, void *h_out, uint32_t lg_n, int inverse, void *stream);
int pp_lde_host(const void *h_in, void *h_out, uint32_t lg_n, uint32_t lambda, uint32_t mode,
                void *stream);

/* Out-of-core transform: input, output and one intermediate buffer (all
 * 32 * 2^lg_n bytes, page-locked host memory, three distinct buffers) stay in
 * host memory.  Every pass reads its tiles from host memory and writes them
 * back (NVLink-C2C on Grace hosts), whole 128-byte lines per warp access; the
 * inter-pass twiddles come from two tables of about 2^(lg_n / 2) elements
 * (w^i and w^(i 2^h), one extra multiply per element and pass), so device
 * memory holds only those tables and the in-pass twiddles: under 5 MiB at
 * 2^30 points.  The result equals pp_ntt bit for bit.  h_scratch is
 * overwritten.  Asynchronous on the stream.  Replaces the reference's
 * segmented out-of-core pipeline our_ntt (ntt.cu:979-1037), which streams
 * chunks of 2^(lg_i + lg_k) elements through device buffers
 * (run_first_ntt_pass :801, run_second_ntt_pass_async_scatter :861) and
 * gathers and scatters them on the CPU; here the permutation is the tiles'
 * own index arithmetic on the GPU. */
int pp_ntt_out_of_core(const void *h_in, void *h_out, void *h_scratch, uint32_t lg_n, int inverse,
                       void *stream);

/* The LDE of pp_lde (same modes and results, bit for bit) with page-locked
 * host input (2^lg_n elements), output and scratch (2^(lg_n + lambda) each),
 * three distinct buffers: every pass reads and writes host memory, and the
 * coset factors come from split tables of about 2^(lg_n / 2) entries, so
 * device memory does not grow with the polynomial.  PP_LDE_EVALS also uses
 * the output or the scratch buffer for the INTT's coefficients.  h_scratch
 * is overwritten.  Asynchronous on the stream.  Replaces the reference's
 * segmented out-of-core LDE (lde.cu:1033-1265: run_first_lde_pass :1033,
 * run_lde_stage_pass :1137, under our_lde :1267). */
int pp_lde_out_of_core(const void *h_in, void *h_out, void *h_scratch, uint32_t lg_n,
                       uint32_t lambda, uint32_t mode, void *stream);

/* count transforms of page-locked host polynomials of 2^lg_n elements:
 * h_out[j] = NTT (or INTT) of h_in[j].  h_in[j] == h_out[j] is allowed; an
 * output must not overlap another polynomial's input.  Each polynomial is
 * copied to HBM, transformed and copied back, and the copies of neighbouring
 * polynomials overlap the transforms (two internal copy streams, three
 * rotating device buffers of 32 * 2^lg_n bytes held as workspace of the
 * stream).  Asynchronous on the stream: synchronise it before reading
 * h_out.  Buffers that are not page-locked are refused with PP_E_INVAL
 * before any copy is queued; count = 0 does nothing.  The reference's
 * our_ntt (ntt.cu:979-1037) transforms one host polynomial per call and
 * leaves overlap across polynomials to the caller; this is that loop with
 * the overlap built in. */
int pp_ntt_host_many(const void *const *h_in, void *const *h_out, uint32_t count, uint32_t lg_n,
                     int inverse, void *stream);

/* ------------------------------------------------------- grand product ---
 * Exclusive prefix product in place: out[0] = 1, out[i] = prod_{j<i} in[j].
 * Replaces accumulate_mul_poly (PLONK/utils/function.cu:256 ->
 * PLONK/utils/mont/cuda/mont_arithmetic.cu:334-361, :544-550). n >= 1. */
int pp_gp_prefix(void *d_inout, uint64_t n, void *stream);

/* Both scans of the same input: d_excl[i] = prod_{j<i} in[j] and
 * d_incl[i] = prod_{j<=i} in[j] (either may be NULL or equal d_in).  The
 * reference's accumulate_mul_poly_(product, output) leaves exactly these in
 * (product, output) (mont_arithmetic.cu:334-361, :552-556). */
int pp_gp_scan(const void *d_in, void *d_excl, void *d_incl, uint64_t n, void *stream);

/* PLONK copy-constraint grand product over 2^lg_n rows:
 *   ratio_i = prod_j (w_j[i] + beta*k_j*w^i + gamma) / prod_j (w_j[i] + beta*sigma_j[i] + gamma)
 *   z = exclusive prefix product of ratio (z_0 = 1)
 * d_w / d_sigma: 3 device pointers each; d_params: device array of 5 elements
 * (beta, gamma, k1, k2, k3).  A zero denominator contributes a factor 0.
 * The reference's permutation-constraint kernel uses this ratio form
 * (PLONK/utils/zkp/cuda/zksnark_compute_permutation_constraint.cu:13-34) and
 * passes its product to accumulate_mul_poly. */
int pp_gp_perm(const void *const *d_w, const void *const *d_sigma, const void *d_params, void *d_z,
               uint32_t lg_n, void *stream);

/* ------------------------------------------------- element-wise Fr ops ---
 * Vectors of n field elements (Montgomery form).  The output may be the
 * same buffer as an input (the reference's in-place "_" forms).
 * Replace add_mod / sub_mod / mul_mod / div_mod and their _ and _scalar
 * forms, neg_mod, inv_mod, exp_mod, gen_sequence and repeat_to_poly
 * (PLONK/utils/function.cu:23-170 -> PLONK/utils/mont/cuda/
 * mont_arithmetic.cu:6-52, :414-520).
 *
 * pp_fr_binary: c[i] = a[i] op b[i], or a[i] op b[0] when b_is_scalar (b must
 * then not overlap c).  Division by 0 gives 0, as the reference's
 * reciprocal (ff/mont_t.cuh:1117) does.  pp_fr_unary: c[i] = -a[i] or
 * 1 / a[i] (0 for 0).  pp_fr_pow: c[i] = a[i]^exponent for any exponent,
 * 0 and 1 included (the reference's exp_mod traps for exponents below 2).
 * pp_fr_powers: out[i] = x^i (gen_sequence).  pp_fr_fill: out[i] = x
 * (repeat_to_poly).  x is one element that must not lie inside the output. */
#define PP_FR_ADD 0
#define PP_FR_SUB 1
#define PP_FR_MUL 2
#define PP_FR_DIV 3
int pp_fr_binary(uint32_t op, const void *d_a, const void *d_b, void *d_c, uint64_t n,
                 int b_is_scalar, void *stream);
#define PP_FR_NEG 0
#define PP_FR_INV 1
int pp_fr_unary(uint32_t op, const void *d_a, void *d_c, uint64_t n, void *stream);
int pp_fr_pow(const void *d_a, void *d_c, uint64_t n, uint64_t exponent, void *stream);
int pp_fr_powers(const void *d_x, void *d_out, uint64_t n, void *stream);
int pp_fr_fill(const void *d_x, void *d_out, uint64_t n, void *stream);

/* --------------------------------------------------------- evaluation ---
 * d_y[0] = sum_i poly[i] * x^i (x = d_x[0]); n == 0 gives 0.
 * Replaces evaluate (PLONK/utils/function.cu:170-181 ->
 * mont_arithmetic.cu:104-163, :507-529). */
int pp_eval(const void *d_poly, uint64_t n, const void *d_x, void *d_y, void *stream);

/* pp_eval for callers that must not allocate device memory during the call:
 * processes whose device memory is all reserved by their own pool, and
 * latency-critical loops that cannot absorb the device-wide synchronisation
 * cudaMalloc/cudaFree may cause.  No reference counterpart: the reference's
 * evaluate allocates a power table and partial sums on every call.
 * Its scratch is a static 64 KiB device array (present on every device that
 * loads the library, until exit), so n <= PP_EVAL_NOALLOC_MAX_N (2^22);
 * larger n returns PP_E_UNSUPPORTED.  The first call on a device looks the
 * array's address up (cudaGetSymbolAddress, no allocation); make that first
 * call before any stream capture.  All calls share the one array: calls that
 * overlap on the GPU (e.g. on two streams) race and must be ordered by the
 * caller.  Same result as pp_eval, bit for bit. */
#define PP_EVAL_NOALLOC_MAX_N (1ull << 22)
int pp_eval_noalloc(const void *d_poly, uint64_t n, const void *d_x, void *d_y, void *stream);

/* ----------------------------------------------------------- division ---
 * In place: the buffer p (n coefficients) becomes q with q_i = S_{i+1},
 * S_i = sum_{j>=i} p_j (-c)^(j-i), q_{n-1} = 0 -- the quotient of p by (X + c)
 * (equivalently of (p(X) - p(z)) by (X - z), z = -c).
 * Replaces poly_div_poly (PLONK/utils/function.cu:183 ->
 * mont_arithmetic.cu:305-331, :531-542).  n >= 1. */
int pp_div_xplusc(void *d_inout, uint64_t n, const void *d_c, void *stream);

/* -------------------------------------------------------------- batch ---
 * Many polynomials of uneven power-of-two sizes in one plan: every transform
 * job is split into its passes, and each pass level of the whole batch is one
 * launch (per 128 jobs) over the tiles of all jobs at that level; grand products
 * run as two launches over all of them.  A plan owns its workspaces and
 * descriptors (allocated by pp_batch_create), so pp_batch_run allocates
 * nothing; pp_batch_capture records the run as a CUDA graph that later
 * pp_batch_run calls replay.  Buffers are fixed at creation.  The reference
 * has no batched form: each of its operators is one call per polynomial. */
#define PP_JOB_NTT 0        /* d_out = NTT(d_in), 2^lg_n points */
#define PP_JOB_INTT 1       /* d_out = INTT(d_in) */
#define PP_JOB_LDE_COEFFS 2 /* as pp_lde mode 0, 2^(lg_n+lambda) outputs */
#define PP_JOB_LDE_EVALS 3  /* as pp_lde mode 1 */
#define PP_JOB_LDE_SPREAD 4 /* as pp_lde mode 2 */
#define PP_JOB_GP 5         /* d_out = exclusive prefix product of d_in (may alias) */
typedef struct pp_job {
  const void *d_in;
  void *d_out;
  uint32_t lg_n;
  uint32_t kind;
  uint32_t lambda; /* LDE jobs only */
  uint32_t reserved;
} pp_job;
int pp_batch_create(const pp_job *jobs, uint32_t count, void **plan);
int pp_batch_run(void *plan, void *stream);
int pp_batch_capture(void *plan);
/* launches per run, tiles of all transform levels, number of levels */
int pp_batch_info(void *plan, uint32_t *launches, uint64_t *tiles, uint32_t *levels);
int pp_batch_destroy(void *plan);

/* ------------------------------------------------------------ serving ---
 * Continuous-batching request loop for prover-round bundles.  A bundle on
 * 2^lg_n-coefficient polynomials is: 3 coset LDEs (mode 0) of the wires w_j,
 * the copy-constraint grand product z of (w, sigma), the quotient of a
 * polynomial by (X + c), and 6 evaluations (w_1..3, sigma_1..3 at z_1..6).
 * Inputs are 7 * 2^lg_n elements (w1..3, sigma1..3, the polynomial to divide)
 * and 12 parameters (beta, gamma, k1..3, c, z1..6), copied from pinned host
 * memory or generated on the device from `seed` when the pointers are NULL.
 * A scheduler thread admits queued bundles whenever one of `slots` streams is
 * free and the bundle's memory fits in `budget_bytes`; admitted bundles run
 * concurrently.  Tables and workspaces for lg in [min_lg, max_lg] are built
 * at creation and stay resident; results stay on the device until
 * pp_server_release.  All waits are bounded.  No reference counterpart: the
 * reference runs one operator call at a time on the default stream. */
typedef struct pp_server_config {
  uint64_t budget_bytes; /* device memory for bundle buffers (admission limit) */
  uint32_t slots;        /* concurrent bundles (one stream each), 1..64 */
  uint32_t min_lg, max_lg;
  uint32_t lambda;       /* LDE blowup of every bundle */
  uint32_t max_queue;    /* 0 = unbounded; else pp_server_submit returns PP_E_BUSY when full */
  /* 0 = no limit; else a bundle is admitted only while the estimated work of
   * the running bundles plus its own stays at or below this many Montgomery
   * multiplies (pp_bundle_work), or when nothing runs: large bundles then run
   * nearly alone and small ones fill in beside them */
  uint64_t max_inflight_mm;
} pp_server_config;
typedef struct pp_bundle {
  uint32_t lg_n;
  uint32_t lambda;
  uint64_t seed;
  const void *h_inputs; /* pinned host, 7 * 2^lg_n elements, or NULL */
  const void *h_params; /* pinned host, 12 elements, or NULL */
} pp_bundle;
typedef struct pp_bundle_result {
  uint64_t ticket;
  int status;
  double latency_ms; /* submit -> completion seen by the scheduler */
  double queue_ms;   /* submit -> admission */
  void *d_lde[3];    /* 2^(lg_n+lambda) each */
  void *d_z;         /* 2^lg_n */
  void *d_quotient;  /* 2^lg_n (top entry 0) */
  void *d_evals;     /* 6 */
  void *d_w[3], *d_sigma[3], *d_params;
} pp_bundle_result;
typedef struct pp_server_stats {
  uint64_t completed, queued, budget_used, budget_peak, admitted_while_busy, max_concurrent;
  double p50_ms, p99_ms, bundles_per_s;
} pp_server_stats;
/* the algorithmic Montgomery multiplies of one bundle (the admission estimate):
 * 3 LDEs of 2^lg_n coefficients onto 2^(lg_n+lambda) points, the grand
 * product (16 per element), the division and 6 evaluations (1 per element each) */
uint64_t pp_bundle_work(uint32_t lg_n, uint32_t lambda);
int pp_server_create(const pp_server_config *cfg, void **server);
int pp_server_submit(void *server, const pp_bundle *bundle, uint64_t *ticket);
int pp_server_wait(void *server, uint64_t ticket, int timeout_ms, pp_bundle_result *result);
int pp_server_release(void *server, uint64_t ticket);
int pp_server_cancel(void *server, uint64_t ticket);
int pp_server_get_stats(void *server, pp_server_stats *stats);
int pp_server_reset_stats(void *server);
int pp_server_destroy(void *server);

/* ---------------------------------------------- quotient constraints ---
 * Element-wise PLONK quotient terms over n points of the extended domain (the
 * LDE outputs).  Vectors hold n elements; scalars are device pointers to one
 * element, as the reference passes one-element SyncedMemory buffers.  n = 0
 * is a no-op.  result may alias none of the inputs except where noted. */
typedef struct {
  const void *x;        /* domain points */
  const void *w[4];     /* w_l, w_r, w_o, w_4 */
  const void *z;        /* permutation polynomial */
  const void *z_next;   /* its shift */
  const void *sigma[4]; /* left, right, out, fourth sigma */
  const void *mod;      /* vector added by the copy term */
  const void *l1;       /* first Lagrange polynomial */
  const void *alpha, *beta, *gamma, *k[3], *one; /* scalars */
} pp_perm_quotient_args;

/* result[i] = (x b + w_l + g)(x b k1 + w_r + g)(x b k2 + w_o + g)(x b k3 + w_4 + g) z alpha
 * (b = beta, g = gamma).  Uses x, w, z, alpha, beta, gamma, k.  Replaces
 * compute_quotient_identity_range_check_i
 * (PLONK/utils/zkp/cuda/zksnark_compute_permutation_constraint.cu:5-16, :49-78). */
int pp_quotient_identity(const pp_perm_quotient_args *a, void *d_result, uint64_t n, void *stream);
/* result[i] += mod[i] - (s_l b + w_l + g)(s_r b + w_r + g)(s_o b + w_o + g)(s_4 b + w_4 + g) z_next alpha
 * Uses sigma, mod, w, z_next, alpha, beta, gamma.  Replaces
 * compute_quotient_copy_range_check_i (:18-36, :80-111). */
int pp_quotient_copy(const pp_perm_quotient_args *a, void *d_result, uint64_t n, void *stream);
/* result[i] += (z[i] - one) l1[i].  Uses z, l1, one.  Replaces
 * compute_quotient_term_check_one_i (:38-47, :113-124). */
int pp_quotient_term_one(const pp_perm_quotient_args *a, void *d_result, uint64_t n, void *stream);
/* The three above in one pass: result = identity + mod - copy + (z - one) l1,
 * the value the reference's three launches leave in result.  result is
 * written only (its old contents are not read). */
int pp_quotient_permutation(const pp_perm_quotient_args *a, void *d_result, uint64_t n,
                            void *stream);

/* Gate constraint: the sum of the arithmetic, range, logic, fixed-base and
 * variable-base group-addition gate terms and the public-input vector.
 * Replaces compute_gate_constraint_allmerge_cuda / allmerge_kernel
 * (PLONK/utils/zkp/cuda/zksnark_comute_gate_constraint.cu:5-27, :30-111).
 * v[] and s[] follow the reference's argument order (PP_GATE_V_*, PP_GATE_S_*).
 * sbox_alpha is the power x^sbox_alpha of the arithmetic gate; the
 * reference's mont_t power traps for exponents below 2 (mont_t.cuh:446-449),
 * here those are refused with PP_E_INVAL, as are exponents >= 2^31. */
#define PP_GATE_NV 22
#define PP_GATE_NS 24
enum {
  PP_GATE_V_A, PP_GATE_V_B, PP_GATE_V_C, PP_GATE_V_D, PP_GATE_V_A_NEXT, PP_GATE_V_B_NEXT,
  PP_GATE_V_D_NEXT, PP_GATE_V_Q_M, PP_GATE_V_Q_L, PP_GATE_V_Q_R, PP_GATE_V_Q_O, PP_GATE_V_Q_4,
  PP_GATE_V_Q_C, PP_GATE_V_Q_HL, PP_GATE_V_Q_HR, PP_GATE_V_Q_H4, PP_GATE_V_Q_ARITH,
  PP_GATE_V_RANGE, PP_GATE_V_LOGIC, PP_GATE_V_FIXED_GROUP_ADD, PP_GATE_V_VARIABLE_GROUP_ADD,
  PP_GATE_V_PI
};
enum {
  PP_GATE_S_FOUR, PP_GATE_S_ONE, PP_GATE_S_TWO, PP_GATE_S_THREE, PP_GATE_S_KAPPA_RANGE,
  PP_GATE_S_KAPPA_SQ_RANGE, PP_GATE_S_KAPPA_CU_RANGE, PP_GATE_S_RANGE_CHALLENGE, PP_GATE_S_P_D,
  PP_GATE_S_NINE, PP_GATE_S_KAPPA_CU_LOGIC, PP_GATE_S_EIGHTEEN, PP_GATE_S_EIGHTYONE,
  PP_GATE_S_EIGHTYTHREE, PP_GATE_S_KAPPA_QU_LOGIC, PP_GATE_S_LOGIC_CHALLENGE, PP_GATE_S_P_A,
  PP_GATE_S_KAPPA_FB, PP_GATE_S_KAPPA_SQ_FB, PP_GATE_S_KAPPA_CU_FB, PP_GATE_S_FB_CHALLENGE,
  PP_GATE_S_KAPPA_VB, PP_GATE_S_KAPPA_SQ_VB, PP_GATE_S_VB_CHALLENGE
};
typedef struct {
  const void *v[PP_GATE_NV]; /* n-element vectors */
  const void *s[PP_GATE_NS]; /* one-element scalars */
  int64_t sbox_alpha;
} pp_gate_args;
int pp_gate_constraint(const pp_gate_args *a, void *d_out, uint64_t n, void *stream);

/* ------------------------------------------- G1 multi-scalar multiply ---
 * d_out = sum_i s_i P_i over BLS12-381 G1 (y^2 = x^3 + 4 over Fq).
 *  d_points: n affine points (x, y), each coordinate 6 little-endian 64-bit
 *    limbs in Montgomery form (R = 2^384, canonical), 96 bytes per point; an
 *    all-zero point is infinity and contributes nothing.
 *  d_scalars: n scalars of 4 little-endian 64-bit limbs, read as plain
 *    integers (no Montgomery decoding), as the reference's MSM does.
 *  d_out: one Jacobian point (X, Y, Z), 144 bytes, normalised to Z = 1
 *    (Montgomery form) -- the affine result -- or all zero for infinity.
 * Replaces multi_scalar_mult (PLONK/utils/function.cu:395-411) ->
 * cuda::msm_zkp_cuda (PLONK/utils/zkp/cuda/zksnark_msm.cu:48-88) and
 * cpu::msm_collect_cpu (PLONK/utils/zkp/cpu/msmcollect.cpp:5-41); the final
 * window aggregation runs on the GPU.  n < 2^31.  Uses a per-stream device
 * workspace of at most 56 W n + 360 W 2^(c-1) bytes (c = window bits, W =
 * 256 / c + 1 windows; pp_msm_g1_window_bits gives c): 1.1 GB for 2^20
 * points, 4.0 GB for 2^22. */
int pp_msm_g1(const void *d_points, const void *d_scalars, uint64_t n, void *d_out, void *stream);
int pp_msm_g1_window_bits(uint64_t n);
/* Tuning: the window bits pp_msm_g1 uses for n with ceil(lg n) = lg_n
 * (0 restores the built-in choice; otherwise 6..20).  Process-wide; the
 * result does not depend on it. */
int pp_msm_g1_set_window_bits(uint32_t lg_n, uint32_t window_bits);

/* Fixed-base form of pp_msm_g1, for a point set that many MSMs share (a
 * prover's commitment key).  No reference counterpart: an addition beside
 * multi_scalar_mult (PLONK/utils/function.cu:395-411) whose results are the
 * same bit for bit, for any points and scalars.
 *
 * pp_msm_g1_bases_create builds, in HBM, the window tables 2^(c w) P_i
 * (affine, w < W = 256 / c + 1) of n points: W n 96-byte entries, e.g.
 * 1.7 GB for 2^20 points at c = 16, 5.2 GB for 2^22 at c = 20.  window_bits
 * 0 picks c for n; 6..20 sets it.  It reads d_points on `stream` (keep them valid until that work is
 * done) and allocates with cudaMalloc; W n must stay below 2^31.
 * pp_msm_g1_fixed then computes sum_i s_i P_i for n scalars like pp_msm_g1:
 * every window's digits go to one shared set of 2^(c-1) buckets, so the
 * window sums run once and there is no Horner chain over the windows.  Call
 * it with the device of the tables current.  pp_msm_g1_bases_destroy frees
 * the tables (a null handle is fine). */
typedef struct pp_msm_bases pp_msm_bases;
int pp_msm_g1_bases_create(const void *d_points, uint64_t n, uint32_t window_bits,
                           pp_msm_bases **bases, void *stream);
int pp_msm_g1_bases_destroy(pp_msm_bases *bases);
int pp_msm_g1_bases_info(const pp_msm_bases *bases, uint64_t *n, uint32_t *window_bits,
                         uint64_t *table_bytes);
int pp_msm_g1_fixed(const pp_msm_bases *bases, const void *d_scalars, void *d_out, void *stream);

/* s_i G for the G1 generator G and n plain 256-bit scalars (32 bytes each,
 * the MSM's scalar format) -> n affine points (96 bytes each, all zero for
 * infinity), one thread per scalar.  For test and benchmark points and
 * commitments to known constants; the reference builds such points on the
 * host with blst.  Buffers 16-byte aligned. */
int pp_g1_mul_gen(const void *d_scalars, uint64_t n, void *d_out, void *stream);

/* -------------------------------------------------------- data formats ---
 * The reference's element files are raw 32-byte little-endian Montgomery
 * elements (read_file miss_ops.cu:8-24, read_file_exact lde.cu:222-231);
 * host/io.h reads and writes them.  These convert on the device:
 *   pp_to_mont: a -> a R mod r (any 256-bit a; canonical output).  Replaces
 *     to_mont (PLONK/utils/function.cu:5-12 -> mont_arithmetic.cu:57-63,
 *     :222-229, :372-389; mont_t::to, mont_t.cuh:473).
 *   pp_to_base: a -> a R^-1 mod r, back to plain integers.  Replaces to_base
 *     (function.cu:14-21 -> mont_arithmetic.cu:65-71, :231-238, :391-411;
 *     mont_t::from, mont_t.cuh:503).
 * d_in == d_out is allowed.  n = 0 is a no-op. */
int pp_to_mont(const void *d_in, void *d_out, uint64_t n, void *stream);
int pp_to_base(const void *d_in, void *d_out, uint64_t n, void *stream);
/* *d_count = number of elements of d_in that are >= r (not canonical), e.g.
 * to validate a raw file before it enters the operators.  d_count is a device
 * pointer; the count is written asynchronously on the stream. */
int pp_count_noncanonical(const void *d_in, uint64_t n, uint64_t *d_count, void *stream);

/* ----------------------------------------------------------- utilities --- */
/* n seeded uniformly random canonical elements: element (first_index + i)
 * limb j is the SplitMix64 output at counter ((first_index+i) << 8 | t << 2 | j)
 * of the stream seeded with seed, bit 255 cleared, rejection-sampled < r
 * (attempt t), stored as the Montgomery representation. */
int pp_random_fr(void *d_out, uint64_t n, uint64_t seed, uint64_t first_index, void *stream);

/* synchronous device -> host copy (for callers without their own CUDA binding) */
int pp_copy_to_host(void *h_dst, const void *d_src, uint64_t bytes);

/* number of kernel launches this library has issued from the calling process */
uint64_t pp_launch_count(void);

/* number of device allocations (cudaMalloc, cudaMallocAsync,
 * cudaMallocFromPoolAsync) this library has requested in the calling process;
 * a diagnostic with no counterpart in the reference, which lets a caller check
 * that a call allocated nothing */
uint64_t pp_device_alloc_count(void);
/* bytes of those allocations (requested sizes, freed or not) */
uint64_t pp_device_alloc_bytes(void);

/* drop cached tables and workspaces of the current device (synchronises it) */
int pp_release(void);

#ifdef __cplusplus
}
#endif
#endif
