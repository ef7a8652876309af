/*
 * ref_driver.cpp -- C entry points around the reference's own MRG8 classes.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the reference sources where they lie (kenmiura/mrg8 original/mrg8.cpp,
 * cuda/mrg8.cpp, knl/mrg8.h), once per flavour, into oracle/_ref/.  Tests use
 * the result to pin the CPU restatement in mrg8_oracle.c and to regenerate
 * tests/golden/.  Nothing here is part of the product.
 *
 * Flavours (one per shared object, because each defines class mrg8):
 *   REF_ORIGINAL  original/mrg8.{h,cpp}   jump_ahead mutates the state
 *   REF_CUDAHOST  cuda/mrg8.{h,cpp}       jump_ahead(k, new_state), mrg8dnz2
 *   REF_KNL       knl/mrg8.h              SHIFTED array rand, rand_tp
 */
#include <stdint.h>
#include <unistd.h>
#include <limits.h>

#if defined(REF_ORIGINAL) || defined(REF_CUDAHOST)
#include "mrg8.h"
#elif defined(REF_KNL)
#include "mrg8.h"
#include <omp.h>
#else
#error "define REF_ORIGINAL, REF_CUDAHOST or REF_KNL"
#endif

#define API extern "C" __attribute__((visibility("default")))

static mrg8 *g_gen = nullptr;

/* The reference constructor reads ./jump_matrix.txt and exits when it is
 * missing, so construct it with the reference directory as the CWD. */
API int ref_init(const char *refdir) {
    if (g_gen) return 0;
    char old[PATH_MAX];
    if (!getcwd(old, sizeof(old))) return -1;
    if (chdir(refdir) != 0) return -2;
    g_gen = new mrg8(13579u);
    if (chdir(old) != 0) return -3;
    return 0;
}

API void ref_seed(uint32_t seed, uint32_t st[8]) {
    g_gen->seed_init(seed);
    g_gen->get_state(st);
}

API void ref_randint(const uint32_t st[8], uint32_t *out, int n, uint32_t end[8]) {
    g_gen->set_state(st);
    g_gen->randint(out, n);
    g_gen->get_state(end);
}

API void ref_rand(const uint32_t st[8], double *out, int n, uint32_t end[8]) {
    g_gen->set_state(st);
    g_gen->rand(out, n);
    g_gen->get_state(end);
}

API uint32_t ref_randint1(const uint32_t st[8], uint32_t end[8]) {
    g_gen->set_state(st);
    uint32_t r = g_gen->randint();
    g_gen->get_state(end);
    return r;
}

API double ref_rand1(const uint32_t st[8], uint32_t end[8]) {
    g_gen->set_state(st);
    double r = g_gen->rand();
    g_gen->get_state(end);
    return r;
}

#if defined(REF_ORIGINAL)
API void ref_jump(const uint32_t st[8], uint64_t k, uint32_t out[8]) {
    g_gen->set_state(st);
    g_gen->jump_ahead(k);
    g_gen->get_state(out);
}
API void ref_jump_bits(const uint32_t st[8], const short bits[200], uint32_t out[8]) {
    g_gen->set_state(st);
    g_gen->jump_ahead(bits);
    g_gen->get_state(out);
}
#else
API void ref_jump(const uint32_t st[8], uint64_t k, uint32_t out[8]) {
    g_gen->set_state(st);
    g_gen->jump_ahead(k, out);
}
API void ref_jump_bits(const uint32_t st[8], const short bits[200], uint32_t out[8]) {
    g_gen->set_state(st);
    g_gen->jump_ahead(bits, out);
}
API void ref_mrg8dnz2(const uint32_t st[8], double *out, int n, uint32_t end[8]) {
    g_gen->set_state(st);
    g_gen->mrg8dnz2(out, n);
    g_gen->get_state(end);
}
#endif

#if defined(REF_KNL)
API void ref_rand_tp(const uint32_t st[8], double *out, int n, int nthreads, uint32_t end[8]) {
    omp_set_num_threads(nthreads);
    g_gen->set_state(st);
    g_gen->rand_tp(out, n);
    g_gen->get_state(end);
}
#endif
