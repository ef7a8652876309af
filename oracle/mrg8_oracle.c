/*
 * mrg8_oracle.c -- CPU restatement of the MRG8 generator (kenmiura/mrg8).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA path and the timed CPU
 * baseline.  The product never links or calls this file.  See mrg8_oracle.h
 * for the reference file:line each function restates.
 */
#include "mrg8_oracle.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MASK 2147483647ull

/* original/mrg8.cpp:16-18 (constructor initialiser list COEFF0..COEFF7). */
const uint32_t orc_coeff[8] = {1089656042u, 1906537547u, 1764115693u, 1304127872u,
                               189748160u,  1984088114u, 626062218u,  1927846343u};

/* original/mrg8.cpp:180-194 -- multiplicative congruential seeding. */
void orc_seed(uint32_t seed, uint32_t st[8]) {
    uint64_t x = seed == 0 ? 97531u : seed;
    for (int k = 0; k < 8; ++k) {
        x = 6364136223846793005ull * x;
        st[k] = (uint32_t)((x >> 32) >> 1);
    }
}

/* original/mrg8.cpp:72-82 -- two 4-term 64-bit sums, three Mersenne folds. */
uint32_t orc_dot(const uint32_t x[8], const uint32_t y[8]) {
    uint64_t s1 = 0, s2 = 0, s;
    for (int q = 0; q < 4; ++q) {
        s1 += (uint64_t)x[q] * y[q];
        s2 += (uint64_t)x[4 + q] * y[4 + q];
    }
    s = (s1 & MASK) + (s1 >> 31) + (s2 & MASK) + (s2 >> 31);
    s = (s & MASK) + (s >> 31);
    return (uint32_t)((s & MASK) + (s >> 31));
}

/* original/mrg8.cpp:197-222 -- one step of the recurrence per output. */
void orc_randint(uint32_t st[8], uint32_t *out, uint64_t n) {
    for (uint64_t k = 0; k < n; ++k) {
        uint32_t z = orc_dot(orc_coeff, st);
        memmove(st + 1, st, 7 * sizeof(uint32_t));
        st[0] = z;
        out[k] = z;
    }
}

/* original/mrg8.cpp:231-237 (ORIGINAL: S * (1/MASK)) and knl/mrg8.h:356-359
 * (SHIFTED: (S - 1) * (1/MASK)).  rnorm is the double nearest 1/(2^31-1). */
double orc_u31_to_f64(uint32_t s, int scaling) {
    const double rnorm = 1.0 / (double)MASK;
    return scaling ? (double)(uint32_t)(s - 1u) * rnorm : (double)s * rnorm;
}

/* No fp32 path exists in the reference; fp32 is defined as the
 * round-to-nearest cast of the fp64 value above. */
float orc_u31_to_f32(uint32_t s, int scaling) { return (float)orc_u31_to_f64(s, scaling); }

void orc_rand_f64(uint32_t st[8], double *out, uint64_t n, int scaling) {
    for (uint64_t k = 0; k < n; ++k) {
        uint32_t z;
        orc_randint(st, &z, 1);
        out[k] = orc_u31_to_f64(z, scaling);
    }
}

void orc_rand_f32(uint32_t st[8], float *out, uint64_t n, int scaling) {
    for (uint64_t k = 0; k < n; ++k) {
        uint32_t z;
        orc_randint(st, &z, 1);
        out[k] = orc_u31_to_f32(z, scaling);
    }
}

/* cuda/mrg8.cpp:290-339 and knl/mrg8.h:387-436: a 1024+8 word buffer in
 * which x[k+1..k+8] are the eight previous values of x[k]. */
void orc_mrg8dnz2(uint32_t st[8], double *out, uint64_t n, int scaling) {
    enum { KMAX = 1024 };
    uint32_t x[KMAX + 8];
    uint64_t nn = n % KMAX;
    for (int k = 0; k < 8; ++k) x[KMAX + k] = st[k];
    for (uint64_t j = 0; j < n - nn; j += KMAX) {
        for (int k = KMAX - 1; k >= 0; --k) {
            x[k] = orc_dot(orc_coeff, x + k + 1);
            out[j + KMAX - 1 - k] = orc_u31_to_f64(x[k], scaling);
        }
        for (int k = 0; k < 8; ++k) x[KMAX + k] = x[k];
    }
    for (int k = 0; k < 8; ++k) st[k] = x[KMAX + k];
    if (nn > 0) orc_rand_f64(st, out + (n - nn), nn, scaling);
}

/* ---------------------------------------------------------------- jumps */

/* Row-major 8x8 product C = X * Y mod p with canonical entries [0, p-1]. */
static void matmul_mod(const uint32_t X[64], const uint32_t Y[64], uint32_t C[64]) {
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) {
            uint64_t acc = 0;
            for (int q = 0; q < 8; ++q) acc += ((uint64_t)X[r * 8 + q] * Y[q * 8 + c]) % MASK;
            C[r * 8 + c] = (uint32_t)(acc % MASK);
        }
}

/* The table of original/mrg8.cpp:85-102, generated instead of read: A is the
 * companion matrix of the recurrence (row 0 = coefficients, sub-diagonal of
 * ones), and A^(2^(j+1)) = (A^(2^j))^2. */
void orc_jump_table(uint32_t *tab) {
    uint32_t M[64], T[64];
    memset(M, 0, sizeof(M));
    for (int c = 0; c < 8; ++c) M[c] = orc_coeff[c];
    for (int r = 1; r < 8; ++r) M[r * 8 + r - 1] = 1;
    for (int j = 0; j < ORC_NTAB; ++j) {
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) tab[j * 64 + r + 8 * c] = M[r * 8 + c];
        matmul_mod(M, M, T);
        memcpy(M, T, sizeof(M));
    }
}

int orc_read_jump_matrix(const char *path, uint32_t *tab) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    for (int k = 0; k < ORC_NTAB * 64; ++k) {
        unsigned long v;
        if (fscanf(f, "%lu", &v) != 1) {
            fclose(f);
            return -2;
        }
        tab[k] = (uint32_t)v;
    }
    fclose(f);
    return 0;
}

/* original/mrg8.cpp:145-176. */
void orc_jump_calc(const uint32_t *tab, const short bits[200], uint32_t J[64]) {
    uint32_t tmp[64], v1[8], v2[8];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) J[r * 8 + c] = (r == c);
    for (int nb = 0; nb < 200; ++nb) {
        if (!bits[nb]) continue;
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) {
                for (int q = 0; q < 8; ++q) {
                    v1[q] = J[r * 8 + q];
                    v2[q] = tab[64 * nb + q + 8 * c];
                }
                tmp[r * 8 + c] = orc_dot(v1, v2);
            }
        memcpy(J, tmp, sizeof(tmp));
    }
}

/* original/mrg8.cpp:104-122. */
void orc_jump_ahead_bits(uint32_t st[8], const uint32_t *tab, const short bits[200]) {
    uint32_t J[64], ns[8];
    orc_jump_calc(tab, bits, J);
    for (int r = 0; r < 8; ++r) ns[r] = orc_dot(J + r * 8, st);
    memcpy(st, ns, sizeof(ns));
}

/* original/mrg8.cpp:125-141 (dec2bin keeps the 64 low bits). */
void orc_jump_ahead(uint32_t st[8], const uint32_t *tab, uint64_t k) {
    short bits[200];
    memset(bits, 0, sizeof(bits));
    for (int nb = 0; nb < 64; ++nb) bits[nb] = (short)((k >> nb) & 1u);
    orc_jump_ahead_bits(st, tab, bits);
}

/* knl/mrg8.h:212-238. */
void orc_jump_ahead_matvec(const uint32_t st[8], const uint32_t *tab, uint64_t k,
                           uint32_t new_state[8]) {
    uint32_t cur[8], nxt[8], row[8];
    memcpy(cur, st, sizeof(cur));
    for (int nb = 0; nb < 64; ++nb) {
        if (!((k >> nb) & 1u)) continue;
        for (int i = 0; i < 8; ++i) {
            for (int q = 0; q < 8; ++q) row[q] = tab[64 * nb + i + 8 * q];
            nxt[i] = orc_dot(row, cur);
        }
        memcpy(cur, nxt, sizeof(cur));
    }
    memcpy(new_state, cur, sizeof(cur));
}

/* ----------------------------------------------- block-split generation */

static void store_kind(void *out, uint64_t i, uint32_t s, int kind) {
    switch (kind) {
    case ORC_U32: ((uint32_t *)out)[i] = s; break;
    case ORC_F64_ORIGINAL: ((double *)out)[i] = orc_u31_to_f64(s, 0); break;
    case ORC_F64_SHIFTED: ((double *)out)[i] = orc_u31_to_f64(s, 1); break;
    case ORC_F32_ORIGINAL: ((float *)out)[i] = orc_u31_to_f32(s, 0); break;
    default: ((float *)out)[i] = orc_u31_to_f32(s, 1); break;
    }
}

/* One block: A^8 outer-product steps (knl/mrg8_vec.h:416-450, the non-AVX
 * path; folded to completion as in bigDotProd), then single steps for the
 * ragged end.  st is advanced in place. */
static void gen_block(uint32_t st[8], const uint32_t *tab, void *out, uint64_t base,
                      uint64_t n, int kind) {
    /* A8T[j*8 + k] = A^8(7-k, j): output k of a block is row 7-k of A^8. */
    uint32_t A8T[64];
    for (int j = 0; j < 8; ++j)
        for (int k = 0; k < 8; ++k) A8T[j * 8 + k] = tab[3 * 64 + (7 - k) + 8 * j];
    uint64_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t s1[8], s2[8];
        uint32_t z[8];
        for (int k = 0; k < 8; ++k) s1[k] = s2[k] = 0;
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 8; ++k) {
                s1[k] += (uint64_t)A8T[j * 8 + k] * st[j];
                s2[k] += (uint64_t)A8T[(j + 4) * 8 + k] * st[j + 4];
            }
        for (int k = 0; k < 8; ++k) {
            uint64_t s = (s1[k] & MASK) + (s1[k] >> 31) + (s2[k] & MASK) + (s2[k] >> 31);
            s = (s & MASK) + (s >> 31);
            z[k] = (uint32_t)((s & MASK) + (s >> 31));
        }
        for (int k = 0; k < 8; ++k) {
            store_kind(out, base + i + k, z[k], kind);
            st[7 - k] = z[k];
        }
    }
    for (; i < n; ++i) {
        uint32_t z;
        orc_randint(st, &z, 1);
        store_kind(out, base + i, z, kind);
    }
}

typedef struct {
    const uint32_t *st0;
    const uint32_t *tab;
    void *out;
    uint64_t start, n;
    int kind;
    uint32_t end_state[8];
} blk_t;

static void *blk_run(void *arg) {
    blk_t *b = (blk_t *)arg;
    uint32_t st[8];
    if (b->start) {
        orc_jump_ahead_matvec(b->st0, b->tab, b->start, st);
    } else {
        memcpy(st, b->st0, sizeof(st));
    }
    gen_block(st, b->tab, b->out, b->start, b->n, b->kind);
    memcpy(b->end_state, st, sizeof(st));
    return NULL;
}

void orc_generate(uint32_t st[8], const uint32_t *tab, void *out, uint64_t n, int kind,
                  int nthreads) {
    if (n == 0) return;
    if (nthreads < 1) nthreads = 1;
    /* Sequential semantics for short runs (the final state keeps any raw
     * words that have not been shifted out yet). */
    if (n < 8 || nthreads == 1) {
        if (n < 8) {
            for (uint64_t i = 0; i < n; ++i) {
                uint32_t z;
                orc_randint(st, &z, 1);
                store_kind(out, i, z, kind);
            }
        } else {
            gen_block(st, tab, out, 0, n, kind);
        }
        return;
    }
    /* knl/mrg8_vec.h:506-512: each block a multiple of 8, the last takes
     * the remainder and supplies the next state. */
    uint64_t each = (n / (uint64_t)nthreads) / 8 * 8;
    if (each == 0) nthreads = 1, each = 0;
    blk_t *blk = (blk_t *)calloc((size_t)nthreads, sizeof(blk_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        blk[t].st0 = st;
        blk[t].tab = tab;
        blk[t].out = out;
        blk[t].start = each * (uint64_t)t;
        blk[t].n = (t == nthreads - 1) ? n - each * (uint64_t)t : each;
        blk[t].kind = kind;
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, blk_run, &blk[t]);
    blk_run(&blk[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    memcpy(st, blk[nthreads - 1].end_state, 8 * sizeof(uint32_t));
    free(blk);
    free(th);
}
