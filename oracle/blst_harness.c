/* blst_harness.c -- C entry points over the reference's vendored blst
 * (PLONK/blst, compiled unmodified from src/server.c and src/assembly.S by
 * the Makefile's `ref` target) for the G1 multi-scalar multiplication golden
 * vectors.  Test infrastructure only.
 *
 * Layouts are the reference's: an affine G1 point is (x, y), each 6
 * little-endian 64-bit limbs in Montgomery form (R = 2^384), 96 bytes; the
 * all-zero point is infinity.  A scalar is 4 little-endian 64-bit limbs read
 * as a plain integer, as the reference's MSM passes mont = false to its
 * Pippenger (PLONK/utils/zkp/cuda/zksnark_msm.cu:35-45). */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef uint8_t byte;
typedef uint64_t limb_t;
typedef struct { limb_t x[6], y[6], z[6]; } POINTonE1;
typedef struct { limb_t x[6], y[6]; } POINTonE1_affine;

/* blst exports used here (src/e1.c, src/multi_scalar.c) */
const POINTonE1 *blst_p1_generator(void);
void blst_p1_mult(POINTonE1 *out, const POINTonE1 *a, const byte *scalar, size_t nbits);
void blst_p1_to_affine(POINTonE1_affine *out, const POINTonE1 *a);
void blst_p1_from_affine(POINTonE1 *out, const POINTonE1_affine *a);
void blst_p1_add_or_double(POINTonE1 *out, const POINTonE1 *a, const POINTonE1 *b);
size_t blst_p1s_mult_pippenger_scratch_sizeof(size_t npoints);
void blst_p1s_mult_pippenger(POINTonE1 *ret, const POINTonE1_affine *const points[], size_t npoints,
                             const byte *const scalars[], size_t nbits, limb_t *scratch);

static void scalar_bytes(const uint64_t s[4], byte out[32]) {
  for (int i = 0; i < 32; ++i) out[i] = (byte)(s[i / 8] >> (8 * (i % 8)));
}

void refg1_generator(uint64_t out[12]) {
  POINTonE1_affine a;
  blst_p1_to_affine(&a, blst_p1_generator());
  memcpy(out, &a, 96);
}

/* k * G for n scalars, affine */
void refg1_mul_gen(const uint64_t *scalars, size_t n, uint64_t *out) {
  for (size_t i = 0; i < n; ++i) {
    byte k[32];
    POINTonE1 p;
    POINTonE1_affine a;
    scalar_bytes(scalars + 4 * i, k);
    blst_p1_mult(&p, blst_p1_generator(), k, 256);
    blst_p1_to_affine(&a, &p);
    memcpy(out + 12 * i, &a, 96);
  }
}

/* a + b (affine in, affine out) */
void refg1_add(const uint64_t a[12], const uint64_t b[12], uint64_t out[12]) {
  POINTonE1 pa, pb, r;
  POINTonE1_affine o;
  blst_p1_from_affine(&pa, (const POINTonE1_affine *)a);
  blst_p1_from_affine(&pb, (const POINTonE1_affine *)b);
  blst_p1_add_or_double(&r, &pa, &pb);
  blst_p1_to_affine(&o, &r);
  memcpy(out, &o, 96);
}

/* sum_i scalars[i] * points[i] with blst's own Pippenger, nbits = 255 */
int refg1_msm(const uint64_t *points, const uint64_t *scalars, size_t n, uint64_t out[12]) {
  if (n == 0) {
    memset(out, 0, 96);
    return 0;
  }
  const POINTonE1_affine **pp = malloc(n * sizeof(*pp));
  const byte **sp = malloc(n * sizeof(*sp));
  byte *sb = malloc(n * 32);
  limb_t *scratch = malloc(blst_p1s_mult_pippenger_scratch_sizeof(n) + 64);
  if (!pp || !sp || !sb || !scratch) return -1;
  for (size_t i = 0; i < n; ++i) {
    pp[i] = (const POINTonE1_affine *)(points + 12 * i);
    scalar_bytes(scalars + 4 * i, sb + 32 * i);
    sp[i] = sb + 32 * i;
  }
  POINTonE1 r;
  POINTonE1_affine o;
  blst_p1s_mult_pippenger(&r, pp, n, sp, 255, scratch);
  blst_p1_to_affine(&o, &r);
  memcpy(out, &o, 96);
  free(pp);
  free(sp);
  free(sb);
  free(scratch);
  return 0;
}
