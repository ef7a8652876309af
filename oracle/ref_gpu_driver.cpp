/*
 * ref_gpu_driver.cpp -- runs the reference's own GPU kernel, rng_outer_32 of
 * cuda/mrg8_cuda.cu:282-399, from the cubin that `make refcubin` compiles out
 * of the reference sources (oracle/_ref/mrg8_ref_cuda.cubin), so that it can
 * be checked against the oracle and timed on the same GPU as ours.
 * TEST INFRASTRUCTURE ONLY: nothing in mrg8_gb300/ uses it.
 *
 * The host side is this file's own: it loads the cubin with the CUDA driver
 * API and prepares the kernel's inputs in the layouts the reference's host
 * class builds (cuda/mrg8_cuda.cu:44-70, 81-128, 178-198):
 *   - d_JUMP_MATRIX: the 247 matrices A^(2^i) with both indices reversed,
 *     row-major: R[i][7-r][7-c] = A^(2^i)[r][c];
 *   - d_JUMP_MATRIX_8s_32: A^8, A^16, A^24 = A^16 A^8 (bigDotProd entries),
 *     A^32 of R stacked as a 32 x 8 array with row stride 1, column stride 32;
 *   - d_state: the state with its word order reversed;
 * and launches it as mrg8_cuda::mrg8_outer_32(d_ran, n, BS, TNUM) does
 * (cuda/mrg8_cuda.cu:414-425): TNUM / BS blocks of BS threads,
 * each_itr = n / (TNUM / 32).
 *
 *   ref_gpu_driver <cubin> check <n> <seed> <TNUM> <BS> <out.bin> [inner]
 *       one launch; writes the n fp64 outputs and then the 8-word next state
 *       (newest first) to out.bin
 *   ref_gpu_driver <cubin> time <n> <seed> <TNUM> <BS> <reps> [inner]
 *       prints "TNUM BS n ms_per_launch Gsamples/s" (kernel time only, CUDA
 *       events around the launches)
 * With "inner" the kernel is rng_inner (cuda/mrg8_cuda.cu:201-280), launched
 * as mrg8_cuda::mrg8_inner does (cuda/mrg8_cuda.cu:402-412): TNUM / 64 blocks
 * of 64 threads, each_itr = n / (TNUM / 64); BS is ignored.
 */
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mrg8_oracle.h"

#define CK(x)                                                                          \
    do {                                                                               \
        CUresult r_ = (x);                                                             \
        if (r_ != CUDA_SUCCESS) {                                                      \
            const char* s_ = nullptr;                                                  \
            cuGetErrorString(r_, &s_);                                                 \
            std::fprintf(stderr, "%s:%d: %s: %s\n", __FILE__, __LINE__, #x, s_ ? s_ : "?"); \
            std::exit(2);                                                              \
        }                                                                              \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 8) {
        std::fprintf(stderr, "usage: %s <cubin> check|time <n> <seed> <TNUM> <BS> <out|reps>\n", argv[0]);
        return 1;
    }
    const std::string mode = argv[2];
    const bool inner = argc > 8 && std::string(argv[8]) == "inner";
    const int n = std::atoi(argv[3]);
    const uint32_t seed = (uint32_t)std::strtoul(argv[4], nullptr, 10);
    const int TNUM = std::atoi(argv[5]), BS = std::atoi(argv[6]);
    if (n <= 0 || TNUM < 64 || BS < 32 || BS > 1024 || BS > TNUM || TNUM % BS || BS % 32) {
        std::fprintf(stderr, "bad arguments\n");
        return 1;
    }

    // Tables in the reference kernel's layouts (see the file comment).
    std::vector<uint32_t> tab(ORC_NTAB * 64), R(ORC_NTAB * 64), s32(8 * 8 * 4);
    orc_jump_table(tab.data());  // column-major: tab[i*64 + r + 8*c] = A^(2^i)[r][c]
    for (int i = 0; i < ORC_NTAB; ++i)
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) R[i * 64 + (7 - r) * 8 + (7 - c)] = tab[i * 64 + r + 8 * c];
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) {
            s32[i + 32 * j] = R[3 * 64 + i * 8 + j];       // A^8
            s32[8 + i + 32 * j] = R[4 * 64 + i * 8 + j];   // A^16
            s32[24 + i + 32 * j] = R[5 * 64 + i * 8 + j];  // A^32
        }
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) s32[16 + i + 32 * j] = orc_dot(&R[4 * 64 + i * 8], &s32[j * 32]);  // A^24
    uint32_t st[8], rst[8];
    orc_seed(seed, st);
    for (int i = 0; i < 8; ++i) rst[i] = st[7 - i];

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CUmodule mod;
    CK(cuModuleLoad(&mod, argv[1]));
    unsigned int nf = 0;
    CK(cuModuleGetFunctionCount(&nf, mod));
    std::vector<CUfunction> fs(nf);
    CK(cuModuleEnumerateFunctions(fs.data(), nf, mod));
    CUfunction fn = nullptr;
    for (CUfunction f : fs) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, f));
        if (name && std::strstr(name, inner ? "rng_inner" : "rng_outer_32")) fn = f;
    }
    if (!fn) {
        std::fprintf(stderr, "%s not found in %s\n", inner ? "rng_inner" : "rng_outer_32", argv[1]);
        return 3;
    }

    CUdeviceptr d_ran, d_jm, d_s32, d_state, d_next;
    CK(cuMemAlloc(&d_ran, (size_t)n * sizeof(double)));
    CK(cuMemAlloc(&d_jm, R.size() * 4));
    CK(cuMemAlloc(&d_s32, s32.size() * 4));
    CK(cuMemAlloc(&d_state, 32));
    CK(cuMemAlloc(&d_next, 32));
    CK(cuMemcpyHtoD(d_jm, R.data(), R.size() * 4));
    CK(cuMemcpyHtoD(d_s32, s32.data(), s32.size() * 4));
    CK(cuMemcpyHtoD(d_state, rst, 32));

    const int pnum = inner ? TNUM / 64 : TNUM / 32;
    int each_itr = n / pnum;
    const unsigned grid = inner ? (unsigned)pnum : (unsigned)(pnum / (BS / 32));
    const unsigned block = inner ? 64u : (unsigned)BS;
    uint64_t MASK = 2147483647ull;
    double rnorm = 1.0 / 2147483647.0;
    int nn = n;
    void* args_outer[] = {&d_ran, &d_jm, &d_s32, &d_state, &d_next, &nn, &MASK, &rnorm, &each_itr};
    void* args_inner[] = {&d_ran, &d_jm, &d_state, &d_next, &nn, &MASK, &rnorm, &each_itr};
    void** args = inner ? args_inner : args_outer;
    auto launch = [&] { CK(cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr)); };

    if (mode == "check") {
        launch();
        CK(cuCtxSynchronize());
        std::vector<double> out(n);
        uint32_t next[8], nst[8];
        CK(cuMemcpyDtoH(out.data(), d_ran, (size_t)n * sizeof(double)));
        CK(cuMemcpyDtoH(next, d_next, 32));
        for (int i = 0; i < 8; ++i) nst[i] = next[7 - i];
        FILE* f = std::fopen(argv[7], "wb");
        if (!f) return 4;
        std::fwrite(out.data(), sizeof(double), out.size(), f);
        std::fwrite(nst, 4, 8, f);
        std::fclose(f);
    } else {
        const int reps = std::atoi(argv[7]);
        for (int w = 0; w < 3; ++w) launch();
        CUevent e0, e1;
        CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
        CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
        CK(cuEventRecord(e0, nullptr));
        for (int r = 0; r < reps; ++r) launch();
        CK(cuEventRecord(e1, nullptr));
        CK(cuEventSynchronize(e1));
        float ms = 0;
        CK(cuEventElapsedTime(&ms, e0, e1));
        ms /= reps;
        std::printf("%d %d %d %.4f %.3f\n", TNUM, BS, n, ms, n / (ms * 1e-3) / 1e9);
    }
    cuMemFree(d_ran);
    cuMemFree(d_jm);
    cuMemFree(d_s32);
    cuMemFree(d_state);
    cuMemFree(d_next);
    cuModuleUnload(mod);
    cuDevicePrimaryCtxRelease(dev);
    return 0;
}
