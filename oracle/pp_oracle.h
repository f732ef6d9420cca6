/*
 * pp_oracle.h -- CPU oracle for the Fr prover-operator path (TEST INFRASTRUCTURE).
 *
 * This header and pp_oracle.c are the checker, not the product.  Only tests,
 * the smoke check and the CPU-baseline leg of the benchmark may load them.
 *
 * Elements are BLS12-381 scalar-field (Fr) values stored as 4 little-endian
 * uint64 limbs in Montgomery form with R = 2^256, exactly like the
 * reference's cpu::BLS12_381_Fr_G1 (PLONK/utils/mont/cpu/ff/bls12-381.hpp:6-32)
 * and cuda::BLS12_381_Fr_G1 (PLONK/utils/mont/cuda/ff/bls12-381.hpp:7-45).
 * Every value handed in must be canonical (< r); every value returned is.
 */
#ifndef PP_ORACLE_H
#define PP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* scalar field arithmetic (Montgomery form in, Montgomery form out) */
void or_fr_mul(const uint64_t a[4], const uint64_t b[4], uint64_t out[4]);
void or_fr_add(const uint64_t a[4], const uint64_t b[4], uint64_t out[4]);
void or_fr_sub(const uint64_t a[4], const uint64_t b[4], uint64_t out[4]);
void or_fr_neg(const uint64_t a[4], uint64_t out[4]);
void or_fr_pow(const uint64_t a[4], const uint64_t e[4], uint64_t out[4]);
void or_fr_inv(const uint64_t a[4], uint64_t out[4]); /* 0 -> 0 */
void or_fr_to_mont(const uint64_t a[4], uint64_t out[4]);
void or_fr_from_mont(const uint64_t a[4], uint64_t out[4]);
void or_fr_one(uint64_t out[4]);
/* omega_{2^lg} = 7^((r-1)/2^lg) (inverse=1: its inverse), Montgomery form */
void or_root_of_unity(int lg, int inverse, uint64_t out[4]);

/* seeded canonical random Fr: element i, limb j is a SplitMix64 output of a
 * counter derived from (seed, i, attempt, j); bit 255 cleared, rejection
 * sampled below r, stored as the Montgomery representation. */
void or_random_fr(uint64_t *out, uint64_t n, uint64_t seed, uint64_t first_index);

/* operators; nthreads <= 0 means "all OpenMP threads" */
void or_ntt(uint64_t *data, int lg_n, int inverse, int nthreads);
void or_lde_coeffs(const uint64_t *coeffs, int lg_n, int lambda, uint64_t *out, int nthreads);
void or_lde_evals(const uint64_t *evals, int lg_n, int lambda, uint64_t *out, int nthreads);
void or_lde_spread(const uint64_t *evals, int lg_n, int lambda, uint64_t *out, int nthreads);
void or_gp_prefix(uint64_t *inout, uint64_t n);
void or_gp_perm(const uint64_t *const w[3], const uint64_t *const sigma[3],
                const uint64_t beta[4], const uint64_t gamma[4], const uint64_t k[3][4],
                int lg_n, uint64_t *z, int nthreads);
void or_eval(const uint64_t *poly, uint64_t n, const uint64_t x[4], uint64_t y[4], int nthreads);
void or_div_xplusc(uint64_t *inout, uint64_t n, const uint64_t c[4]);

/* restatements of the reference's single-thread CPU baselines
 * (miss_ops.cu:34-47 and :49-87) */
void or_naive_gp(const uint64_t *in, uint64_t n, uint64_t *out);
int or_naive_div(const uint64_t *in, uint64_t n, const uint64_t c[4], uint64_t *quotient);

/* PLONK quotient constraints (element-wise over the extended domain):
 * zksnark_compute_permutation_constraint.cu:5-47 and
 * zksnark_comute_gate_constraint.cu:6-30.  Scalars are one element. */
void or_quotient_identity(const uint64_t *x, const uint64_t *const w[4], const uint64_t *z,
                          const uint64_t alpha[4], const uint64_t beta[4], const uint64_t gamma[4],
                          const uint64_t *const k[3], uint64_t *result, uint64_t n);
void or_quotient_copy(const uint64_t *const sigma[4], const uint64_t *mod, const uint64_t *const w[4],
                      const uint64_t *z_next, const uint64_t alpha[4], const uint64_t beta[4],
                      const uint64_t gamma[4], uint64_t *result, uint64_t n);
void or_quotient_term_one(const uint64_t *z, const uint64_t *l1, const uint64_t one[4],
                          uint64_t *result, uint64_t n);
void or_gate_constraint(const uint64_t *const v[22], const uint64_t *const s[24], int64_t sbox_alpha,
                        uint64_t *out, uint64_t n);

/* BLS12-381 G1 (pp_oracle_g1.c).  Affine points are 12 uint64 (x, y in
 * Montgomery form over Fq, R = 2^384; all zero = infinity); scalars 4 uint64
 * read as plain integers.  or_g1_msm: sum_i s_i P_i (PLONK/utils/function.cu:
 * 395-411 multi_scalar_mult); or_g1_mul_gen: s_i G for the standard
 * generator; or_g1_add: a + b.  nthreads <= 0 uses all. */
void or_g1_msm(const uint64_t *points, const uint64_t *scalars, uint64_t n, uint64_t out[12],
               int nthreads);
void or_g1_mul_gen(const uint64_t *scalars, uint64_t n, uint64_t *out, int nthreads);
void or_g1_add(const uint64_t a[12], const uint64_t b[12], uint64_t out[12]);

/* bit-exact byte comparison helper: index of first differing element or -1 */
int64_t or_first_diff(const uint64_t *a, const uint64_t *b, uint64_t n);

#ifdef __cplusplus
}
#endif
#endif
