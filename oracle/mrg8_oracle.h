/*
 * mrg8_oracle.h -- CPU restatement of the MRG8 generator.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this code, and only as
 * the oracle for comparisons or as the timed CPU baseline.  The product (mrg8_gb300/) never
 * calls it; the product path fails loudly when its CUDA library is missing.
 *
 * Each function restates the algorithm of the reference file:line it cites
 * (kenmiura/mrg8).  Parity of this restatement is pinned against the
 * reference itself compiled from its own sources (oracle/Makefile ->
 * oracle/_ref/) and against the golden vectors in tests/golden/.
 */
#ifndef MRG8_ORACLE_H
#define MRG8_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_P 2147483647u /* 2^31 - 1 */
#define ORC_NTAB 247      /* A^(2^j), j = 0..246 */

/* Output kinds of the generic generator below. */
enum {
    ORC_U32 = 0,           /* randint: S in [1, p]                         */
    ORC_F64_ORIGINAL = 1,  /* (double)S * (1/p), range (0, 1]              */
    ORC_F64_SHIFTED = 2,   /* (double)(S-1) * (1/p), range [0, 1)          */
    ORC_F32_ORIGINAL = 3,  /* (float) of ORC_F64_ORIGINAL                  */
    ORC_F32_SHIFTED = 4    /* (float) of ORC_F64_SHIFTED                   */
};

/* The eight recurrence coefficients a_1..a_8 (original/mrg8.cpp:16-18). */
extern const uint32_t orc_coeff[8];

/* mcg64ni seeding (original/mrg8.cpp:180-194); seed 0 means 97531. */
void orc_seed(uint32_t seed, uint32_t st[8]);

/* bigDotProd (original/mrg8.cpp:72-82): sum x[i]*y[i] mod p, representative
 * in [1, p] for a non-zero sum, 0 for an all-zero sum. */
uint32_t orc_dot(const uint32_t x[8], const uint32_t y[8]);

/* randint (original/mrg8.cpp:197-222): n steps, state updated in place. */
void orc_randint(uint32_t st[8], uint32_t *out, uint64_t n);

/* rand (original/mrg8.cpp:231-239 for ORIGINAL, knl/mrg8.h:353-362 for
 * SHIFTED).  scaling: 0 = ORIGINAL, 1 = SHIFTED. */
void orc_rand_f64(uint32_t st[8], double *out, uint64_t n, int scaling);
void orc_rand_f32(uint32_t st[8], float *out, uint64_t n, int scaling);

/* Scalar conversions used above (exposed for the conversion tests). */
double orc_u31_to_f64(uint32_t s, int scaling);
float orc_u31_to_f32(uint32_t s, int scaling);

/* mrg8dnz2 (cuda/mrg8.cpp:290-339, ORIGINAL; knl/mrg8.h:387-436, SHIFTED):
 * the same stream through a 1024-deep buffer. */
void orc_mrg8dnz2(uint32_t st[8], double *out, uint64_t n, int scaling);

/* Jump table A^(2^j) mod p, j = 0..246, column-major per matrix:
 * (A^(2^j))(r,c) = tab[j*64 + r + 8*c]  (format of original/mrg8.cpp:85-102,
 * jump_matrix.txt).  Entries are canonical residues in [0, p-1]. */
void orc_jump_table(uint32_t *tab /* ORC_NTAB*64 */);

/* Parse a jump_matrix.txt text file into tab (returns 0 on success). */
int orc_read_jump_matrix(const char *path, uint32_t *tab);

/* jump_calc (original/mrg8.cpp:145-176): J = prod of A^(2^nb) over set bits,
 * row-major J[r*8+c]. */
void orc_jump_calc(const uint32_t *tab, const short bits[200], uint32_t J[64]);

/* jump_ahead (original/mrg8.cpp:104-129): state <- J * state, in place. */
void orc_jump_ahead_bits(uint32_t st[8], const uint32_t *tab, const short bits[200]);
void orc_jump_ahead(uint32_t st[8], const uint32_t *tab, uint64_t k);

/* jump_ahead with out-parameter by per-bit matrix-vector products
 * (knl/mrg8.h:212-238); st is left unchanged. */
void orc_jump_ahead_matvec(const uint32_t st[8], const uint32_t *tab, uint64_t k,
                           uint32_t new_state[8]);

/* Generic generator: n outputs of the given kind, state advanced in place.
 * nthreads > 1 splits the range into per-thread blocks that start by
 * jump-ahead (knl/mrg8.h:445-470, knl/mrg8_vec.h:500-525); every thread then
 * runs the A^8 block recurrence of knl/mrg8_vec.h:416-450 (8 outputs per
 * 8x8 matrix-vector product).  Results equal the sequential stream. */
void orc_generate(uint32_t st[8], const uint32_t *tab, void *out, uint64_t n,
                  int kind, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
