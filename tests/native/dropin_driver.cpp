// dropin_driver.cpp -- reference-style caller of the drop-in classes.
//
// Written the way the reference's drivers use mrg8 / mrg8_cuda
// (cuda/tests/test_mrg8_outer.cu:35-61): construct with a seed, seed_init,
// generate, read the state.  Built by tests/test_dropin.py against
// include/mrg8_cuda.hpp and libmrg8g.so; prints values for the test to check.
//   dropin_driver host   seeding and jumps only (no GPU needed)
//   dropin_driver gpu    device and host generation through the classes
//   dropin_driver dnz2   mrg8dnz2 in both scalings, consecutive calls on one
//                        object: a digest of each call's values (sum over i
//                        of word_i * (2 i + 1), mod 2^64)
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "mrg8_cuda.hpp"

static void print_state(const char* tag, const mrg8& m) {
    uint32_t st[8];
    m.get_state(st);
    std::printf("%s", tag);
    for (int i = 0; i < 8; ++i) std::printf(" %u", st[i]);
    std::printf("\n");
}

static uint64_t digest(const double* v, int n) {
    uint64_t h = 0;
    for (int i = 0; i < n; ++i) {
        uint64_t w;
        std::memcpy(&w, v + i, 8);
        h += w * (2ull * (uint64_t)i + 1ull);
    }
    return h;
}

int main(int argc, char** argv) {
    const uint32_t iseed = 13579;
    if (argc > 1 && !std::strcmp(argv[1], "dnz2")) {
        const int ns[] = {1, 1023, 1024, 1025, 3000, 1000000};
        for (int scaling : {MRG8G_ORIGINAL, MRG8G_SHIFTED}) {
            mrg8 m(iseed);
            for (int n : ns) {
                std::vector<double> v(n);
                if (scaling == MRG8G_ORIGINAL) m.mrg8dnz2(v.data(), n);
                else m.mrg8dnz2(v.data(), n, MRG8G_SHIFTED);
                std::printf("dnz2_%d_%d %llu %.17g\n", scaling, n, (unsigned long long)digest(v.data(), n), v[n - 1]);
            }
            print_state(scaling == MRG8G_ORIGINAL ? "dnz2_state_0" : "dnz2_state_1", m);
        }
        return 0;
    }
    if (argc > 1 && !std::strcmp(argv[1], "host")) {
        mrg8 m(iseed);
        print_state("seeded", m);
        uint32_t js[8];
        m.jump_ahead((uint64_t)1000, js);
        std::printf("jump1000");
        for (int i = 0; i < 8; ++i) std::printf(" %u", js[i]);
        std::printf("\n");
        m.jump_ahead((uint64_t)1000);
        print_state("after_jump", m);
        short bits[200] = {0};
        bits[199] = 1;
        m.jump_ahead(bits);
        print_state("after_jump2^199", m);
        return 0;
    }
    const int N = 1 << 20;
    double* d_ran = nullptr;
    if (cudaMalloc((void**)&d_ran, sizeof(double) * N) != cudaSuccess) return 3;
    mrg8_cuda m(iseed);
    m.seed_init(iseed);
    m.mrg8_outer_32(d_ran, N, 64, 65536);  // SHIFTED, as cuda/mrg8_cuda.cu
    std::vector<double> ran(N);
    cudaMemcpy(ran.data(), d_ran, sizeof(double) * N, cudaMemcpyDeviceToHost);
    m.state_cpy_DtH();
    print_state("after_outer", m);
    std::printf("outer_first %.17g %.17g last %.17g\n", ran[0], ran[1], ran[N - 1]);
    m.seed_init(iseed);
    m.mrg8_inner(d_ran, N, 1024);
    std::vector<double> ran2(N);
    cudaMemcpy(ran2.data(), d_ran, sizeof(double) * N, cudaMemcpyDeviceToHost);
    std::printf("inner_equals_outer %d\n", (int)(ran == ran2));
    mrg8 h(iseed);  // host buffers, ORIGINAL scaling as original/mrg8.cpp
    std::vector<double> f(1000);
    h.rand(f.data(), 1000);
    std::printf("rand_first %.17g last %.17g\n", f[0], f[999]);
    std::vector<uint32_t> r(10);
    h.randint(r.data(), 10);
    std::printf("randint");
    for (uint32_t v : r) std::printf(" %u", v);
    std::printf("\n");
    std::printf("scalar %u %.17g %.17g\n", h.randint(), h.rand(), h());
    print_state("final", h);
    cudaFree(d_ran);
    return 0;
}
