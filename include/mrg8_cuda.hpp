// mrg8_cuda.hpp -- drop-in C++ classes `mrg8` and `mrg8_cuda` over the C ABI
// of mrg8g.h (libmrg8g.so).
//
// Replaces the reference headers original/mrg8.h, cuda/mrg8.h and
// cuda/mrg8_cuda.h: same class names, member names, argument meaning and
// state conventions, so code written against the reference (for example its
// benchmark drivers cuda/tests/test_mrg8_outer.cu) compiles against this
// header and links with -lmrg8g.  Differences, all deliberate:
//   - every value is generated by the GB300 kernels, host-buffer calls
//     included (rand(double*, n) copies the GPU result back);
//   - the state is always current: get_state() after a device call returns
//     the advanced state, set_state() governs later device calls, and
//     state_cpy_DtH() has nothing to copy;
//   - jump tables are generated on the host; jump_matrix.txt is not read;
//   - failures throw std::runtime_error with mrg8g_last_error() (the
//     reference does not check errors);
//   - the destructor releases the handle (the reference leaks).
#pragma once

#include <cstdint>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>

#include "mrg8g.h"

namespace mrg8g_detail {
inline void check(int rc) {
    if (rc != MRG8G_SUCCESS) throw std::runtime_error(std::string("mrg8g: ") + mrg8g_last_error());
}
}  // namespace mrg8g_detail

// original/mrg8.h:21-56, cuda/mrg8.h:23-79.
class mrg8 {
public:
    const uint32_t MAX_RND;

    mrg8() : mrg8(0u) {}
    explicit mrg8(const uint32_t seed_val) : MAX_RND(2147483646u), g_(nullptr) {
        mrg8g_detail::check(mrg8g_create(seed_val, &g_));
    }
    mrg8(const mrg8&) = delete;
    mrg8& operator=(const mrg8&) = delete;
    virtual ~mrg8() { mrg8g_destroy(g_); }

    // original/mrg8.cpp:31-34
    void seed_init(const uint32_t seed_val) { mrg8g_detail::check(mrg8g_seed_init(g_, seed_val)); }
    // original/mrg8.cpp:36-39
    void get_state(uint32_t st[8]) const { mrg8g_detail::check(mrg8g_get_state(g_, st)); }
    // original/mrg8.cpp:56-59
    void set_state(const uint32_t st[8]) { mrg8g_detail::check(mrg8g_set_state(g_, st)); }

    // original/mrg8.cpp:197-222: n values in [1, 2^31-1] into host memory.
    void randint(uint32_t* iran, int n) { host(iran, n, MRG8G_U32); }
    uint32_t randint() {
        uint32_t r;
        randint(&r, 1);
        return r;
    }
    // original/mrg8.cpp:231-239: ORIGINAL scaling, (0, 1].
    void rand(double* fran, int n) { host(fran, n, MRG8G_F64_ORIGINAL); }
    double rand() {
        double r;
        rand(&r, 1);
        return r;
    }
    double operator()() { return rand(); }
    // cuda/mrg8.cpp:290-339: the same values as rand(), ORIGINAL scaling
    // (S * rnorm, in (0, 1]), which is what the mrg8 / mrg8_cuda classes of
    // the reference's cuda/ and original/ trees return.  The reference's KNL
    // class (knl/mrg8.h:387-436) returns SHIFTED values ((S - 1) * rnorm, in
    // [0, 1)) from the same signature; a caller ported from there passes
    // MRG8G_SHIFTED to the overload below.
    void mrg8dnz2(double* ran, int n) { rand(ran, n); }
    void mrg8dnz2(double* ran, int n, int scaling) {
        if (scaling != MRG8G_ORIGINAL && scaling != MRG8G_SHIFTED)
            throw std::invalid_argument("mrg8dnz2: scaling must be MRG8G_ORIGINAL or MRG8G_SHIFTED");
        host(ran, n, scaling == MRG8G_SHIFTED ? MRG8G_F64_SHIFTED : MRG8G_F64_ORIGINAL);
    }

    // original/mrg8.cpp:104-129: jumps that advance this stream.
    void jump_ahead(const short jump_val_bin[200]) { mrg8g_detail::check(mrg8g_jump_ahead_bits(g_, jump_val_bin)); }
    void jump_ahead(const uint64_t jump_val) { mrg8g_detail::check(mrg8g_jump_ahead(g_, jump_val)); }
    // cuda/mrg8.cpp:127-150, knl/mrg8.h:194-238: jumped state into new_state.
    void jump_ahead(const short jump_val_bin[200], uint32_t* new_state) const {
        mrg8g_detail::check(mrg8g_jump_state_bits(g_, jump_val_bin, new_state));
    }
    void jump_ahead(const uint64_t jump_val, uint32_t* new_state) const {
        mrg8g_detail::check(mrg8g_jump_state(g_, jump_val, new_state));
    }

    // original/mrg8.cpp:41-54
    void print_state() const {
        uint32_t st[8];
        get_state(st);
        std::cout << "(S[n-1], S[n-2], ..., S[n-8])= (";
        for (int i = 0; i < 7; ++i) std::cout << std::setw(10) << st[i] << ", ";
        std::cout << st[7] << ")" << std::endl;
    }
    void print_matrix(const uint32_t jm[8][8]) const {
        for (int i = 0; i < 8; ++i) {
            for (int j = 0; j < 8; ++j) std::cout << std::setw(10) << jm[i][j] << " ";
            std::cout << std::endl;
        }
    }

    // Handle of the C ABI (for mixing with the batch and serving entry points).
    mrg8g_generator* handle() const { return g_; }

protected:
    mrg8g_generator* g_;

    void host(void* out, int n, int kind) {
        if (n < 0) throw std::invalid_argument("mrg8: negative count");
        mrg8g_detail::check(mrg8g_generate_host(g_, out, (uint64_t)n, kind));
    }
};

// cuda/mrg8_cuda.h:20-45.
class mrg8_cuda : public mrg8 {
public:
    mrg8_cuda() : mrg8() {}
    explicit mrg8_cuda(const uint32_t seed_val) : mrg8(seed_val) {}

    // cuda/mrg8_cuda.cu:66-70
    void seed_init(const uint32_t seed_val) { mrg8::seed_init(seed_val); }

    // cuda/mrg8_cuda.cu:402-412: SHIFTED fp64, [0, 1), into device memory.
    void mrg8_inner(double* d_ran, const int n, const int TNUM) {
        launch_check(32, TNUM);
        device_f64(d_ran, n);
    }
    // cuda/mrg8_cuda.cu:414-436.  BS / TNUM shaped the reference's launch;
    // they are validated and otherwise do not change the (identical) values.
    void mrg8_outer_32(double* d_ran, const int n) { device_f64(d_ran, n); }
    void mrg8_outer_32(double* d_ran, const int n, const int TNUM) {
        launch_check(32, TNUM);
        device_f64(d_ran, n);
    }
    void mrg8_outer_32(double* d_ran, const int n, const int BS, const int TNUM) {
        launch_check(BS, TNUM);
        device_f64(d_ran, n);
    }

    // cuda/mrg8_cuda.cu:72-79: the host state is always current here.
    void state_cpy_DtH() {}

private:
    static void launch_check(int BS, int TNUM) {
        if (BS < 32 || BS > 1024 || BS % 32 || TNUM < 32)
            throw std::invalid_argument("mrg8_cuda: BS must be a multiple of 32 in [32,1024] and TNUM >= 32");
    }
    // Like the reference, returns when the values are in d_ran (the
    // reference synchronises the device after its launch).
    void device_f64(double* d_ran, int n) {
        if (n < 0) throw std::invalid_argument("mrg8_cuda: negative count");
        mrg8g_detail::check(mrg8g_rand(g_, d_ran, (uint64_t)n, MRG8G_SHIFTED, nullptr));
        mrg8g_detail::check(mrg8g_stream_sync(nullptr));
    }
};
