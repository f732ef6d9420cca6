// function.h -- the reference's operator entry points for the Fr prover path,
// with the same names, argument meaning and buffer conventions, forwarding to
// the C ABI of libppfr.so (include/pp_ops.h).
//
//   reference                                   here
//   PLONK/utils/function.cuh:67  accumulate_mul_poly(product, stream)
//   PLONK/utils/function.cuh:52  evaluate(poly, x)
//   PLONK/utils/function.cuh:54  poly_div_poly(divid, c)
//   PLONK/utils/function.cuh:81  class Ntt  (forward, forward_)
//   PLONK/utils/function.cuh:102 class Intt (forward, forward_, _forward_)
//   ntt.cu:979                   our_ntt(input, lg_N, lg_i, lg_j, lg_k, ...)
//   ntt.cu:1039                  standard4_ntt(input, lg_N, lg_i, lg_j, lg_k, ...)
//   lde.cu:1267                  our_lde(input, lg_N, lambda, lg_k, ...)
//   lde.cu:1367                  naive_lde(input, lg_N, lambda, lg_k, ...)
//
// The reference's segmented drivers (our_ntt, our_lde, standard4_ntt,
// naive_lde) stream host-resident data through the GPU in chunks and permute
// on the CPU.  On GB300 the whole problem fits in HBM and the GPU reaches
// page-locked host memory directly: our_ntt and our_lde run pp_ntt_host /
// pp_lde_host, whose first pass reads the host input and whose last pass
// writes the host output, with only the middle passes in HBM.  A pageable
// caller buffer (our_lde's input), standard4_ntt and naive_lde take the
// staged form instead: one copy in, the in-HBM transform, one copy out.  The
// segmentation and CPU-thread arguments are accepted for source compatibility
// and do not change the result (which the reference's own --check-* modes
// require to equal Ntt::forward bit for bit).
#pragma once
#include <cstdint>

#include "fr_cpu.h"  // cpu::BLS12_381_Fr_G1, the reference's host field element
#include "syncedmem.h"

SyncedMemory accumulate_mul_poly(SyncedMemory product, cudaStream_t stream = (cudaStream_t)0);
void accumulate_mul_poly_(SyncedMemory product, SyncedMemory output,
                          cudaStream_t stream = (cudaStream_t)0);
SyncedMemory evaluate(SyncedMemory poly, SyncedMemory x);
SyncedMemory poly_div_poly(SyncedMemory divid, SyncedMemory c);

// ---- element-wise field operators and buffer helpers
// (PLONK/utils/function.cuh:12-71, zk_function.cu:3), in field_ops.cpp.  The
// arithmetic runs on the GPU whatever the head of the inputs (the reference
// has CPU twins for some of them; the values are the same).  The inverse of
// 0 is 0.  exp_mod takes any exponent >= 0 (the reference traps below 2) and
// throws for a negative one.
SyncedMemory neg_mod(SyncedMemory input);
SyncedMemory inv_mod(SyncedMemory input);
SyncedMemory add_mod(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
void add_mod_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory sub_mod(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
void sub_mod_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory mul_mod(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
void mul_mod_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory div_mod(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
void div_mod_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory exp_mod(SyncedMemory input, int exp);
SyncedMemory add_mod_scalar(SyncedMemory input1, SyncedMemory input2,
                            cudaStream_t stream = (cudaStream_t)0);
void add_mod_scalar_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory sub_mod_scalar(SyncedMemory input1, SyncedMemory input2,
                            cudaStream_t stream = (cudaStream_t)0);
void sub_mod_scalar_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory mul_mod_scalar(SyncedMemory input1, SyncedMemory input2,
                            cudaStream_t stream = (cudaStream_t)0);
void mul_mod_scalar_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory div_mod_scalar(SyncedMemory input1, SyncedMemory input2,
                            cudaStream_t stream = (cudaStream_t)0);
void div_mod_scalar_(SyncedMemory input1, SyncedMemory input2, cudaStream_t stream = (cudaStream_t)0);
// [1, x, x^2, ..., x^(N-1)]
SyncedMemory gen_sequence(uint64_t N, SyncedMemory x, cudaStream_t stream = (cudaStream_t)0);
void gen_sequence_(uint64_t N, SyncedMemory x, SyncedMemory y, cudaStream_t stream = (cudaStream_t)0);
// N copies of x[0]
SyncedMemory repeat_to_poly(SyncedMemory x, uint64_t N, cudaStream_t stream = (cudaStream_t)0);
void repeat_to_poly_(SyncedMemory x, SyncedMemory y, uint64_t N, cudaStream_t stream = (cudaStream_t)0);
// x followed by zeros up to N elements (x must not be longer)
SyncedMemory pad_poly(SyncedMemory x, uint64_t N, cudaStream_t stream = (cudaStream_t)0);
void pad_poly_(SyncedMemory x, SyncedMemory out, uint64_t N, cudaStream_t stream = (cudaStream_t)0);
SyncedMemory repeat_zero(uint64_t N);  // N zero elements in host memory
SyncedMemory cat(SyncedMemory a, SyncedMemory b);
SyncedMemory slice(SyncedMemory a, uint64_t len, bool forward);  // first / last len elements
// pad_len elements; element i holds the 64-bit word i of input as (w, 0, 0, 0)
SyncedMemory make_tensor(SyncedMemory input, uint64_t pad_len);
// a > b as integers of little-endian 64-bit words (host data)
bool gt_zkp(SyncedMemory a, SyncedMemory b);

class Ntt {
 public:
  // The reference's twiddle blob; the transform tables here are cached by
  // libppfr.so per device and size, so this handle stays empty.
  SyncedMemory Params;
  // domain_size: log2 of the largest transform this object will run
  explicit Ntt(int domain_size, cudaStream_t stream = (cudaStream_t)0);
  SyncedMemory forward(SyncedMemory input, cudaStream_t stream = (cudaStream_t)0);
  void forward_(SyncedMemory input, SyncedMemory output, cudaStream_t stream = (cudaStream_t)0);
  int max_lg() const { return max_lg_; }

 protected:
  int max_lg_;
  bool inverse_ = false;
};

class Intt : public Ntt {
 public:
  explicit Intt(int domain_size, cudaStream_t stream = (cudaStream_t)0);
  void _forward_(SyncedMemory input, cudaStream_t stream = (cudaStream_t)0);  // in place
};

struct StageIndexMap;  // host permutation maps of the segmented passes; unused here

void our_ntt(SyncedMemory input, int lg_N, int lg_i, int lg_j, int lg_k, int step1_thread,
             int step2_thread, Ntt ntt, const StageIndexMap *second_stage_map = nullptr);
void standard4_ntt(SyncedMemory input, int lg_N, int lg_i, int lg_j, int lg_k,
                   int transpose_threads, Ntt ntt);
// returns milliseconds like the reference; the extension of 2^lg_N
// coefficients onto 2^(lg_N+lambda) points (shift 7^(2^lambda)) is kept in
// last_lde_output() until the next call
float our_lde(cpu::BLS12_381_Fr_G1 *input, int lg_N, int lambda, int lg_k, int step1_thread,
              int step2_thread, Ntt &ntt);
// the reference's baseline: spread at i << lambda, no coset factor
float naive_lde(cpu::BLS12_381_Fr_G1 *input, int lg_N, int lambda, int lg_k, int pad_threads,
                int transpose_threads, Ntt &ntt);
SyncedMemory last_lde_output();

// PLONK/utils/function.cuh:144: sum_i scalars[i] * points[i] over G1.  points
// holds affine (x, y) Fq pairs (96 bytes each, Montgomery form), scalars plain
// 256-bit integers (32 bytes each); the first min(#points, #scalars) pairs are
// used.  Returns a 144-byte Jacobian point (x, y, 1), all zero for infinity.
SyncedMemory multi_scalar_mult(SyncedMemory points, SyncedMemory scalars,
                               cudaStream_t stream = (cudaStream_t)0);
