// mrg8g_tables.cpp -- host generation of the jump tables, window tables and
// decimated-recurrence coefficients (see mrg8g_tables.h).
#include "mrg8g_tables.h"

#include <cstring>
#include <mutex>
#include <stdexcept>

#include "mrg8g_arith.cuh"

namespace mrg8g {

// original/mrg8.cpp:16-18.
static const uint32_t kCoef[8] = {1089656042u, 1906537547u, 1764115693u, 1304127872u,
                                  189748160u,  1984088114u, 626062218u,  1927846343u};

static uint32_t mulmod(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) % kP); }
static uint32_t addmod(uint32_t a, uint32_t b) {
    uint32_t s = a + b;  // both < 2^31
    return s >= kP ? s - kP : s;
}
static uint32_t submod(uint32_t a, uint32_t b) { return a >= b ? a - b : a + kP - b; }
static uint32_t powmod(uint32_t a, uint64_t e) {
    uint64_t r = 1, x = a % kP;
    while (e) {
        if (e & 1) r = r * x % kP;
        x = x * x % kP;
        e >>= 1;
    }
    return (uint32_t)r;
}
static uint32_t invmod(uint32_t a) { return powmod(a, kP - 2); }  // p prime

void matmul_mod(const uint32_t* X, const uint32_t* Y, uint32_t* C) {
    uint32_t T[64];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) {
            uint64_t acc = 0;
            for (int q = 0; q < 8; ++q) acc += ((uint64_t)X[r * 8 + q] * Y[q * 8 + c]) % kP;
            T[r * 8 + c] = (uint32_t)(acc % kP);
        }
    std::memcpy(C, T, sizeof(T));
}

static void matvec_mod(const uint32_t* M, const uint32_t* v, uint32_t* out) {
    uint32_t t[8];
    for (int r = 0; r < 8; ++r) {
        uint64_t acc = 0;
        for (int q = 0; q < 8; ++q) acc += ((uint64_t)M[r * 8 + q] * v[q]) % kP;
        t[r] = (uint32_t)(acc % kP);
    }
    std::memcpy(out, t, sizeof(t));
}

// Solve C beta = rhs (mod p) for an invertible 8x8 C (Gauss-Jordan).
static bool solve8(uint32_t C[8][9], uint32_t beta[8]) {
    for (int col = 0; col < 8; ++col) {
        int piv = -1;
        for (int r = col; r < 8; ++r)
            if (C[r][col]) { piv = r; break; }
        if (piv < 0) return false;
        if (piv != col)
            for (int c = 0; c < 9; ++c) std::swap(C[piv][c], C[col][c]);
        const uint32_t inv = invmod(C[col][col]);
        for (int c = 0; c < 9; ++c) C[col][c] = mulmod(C[col][c], inv);
        for (int r = 0; r < 8; ++r) {
            if (r == col || !C[r][col]) continue;
            const uint32_t f = C[r][col];
            for (int c = 0; c < 9; ++c) C[r][c] = submod(C[r][c], mulmod(f, C[col][c]));
        }
    }
    for (int r = 0; r < 8; ++r) beta[r] = C[r][8];
    return true;
}

// beta_k with M^8 v = sum_k beta_k M^(8-k) v for every v (characteristic
// polynomial of M, which is irreducible for powers of A, so any non-zero v is
// cyclic).  Solved on v = e_0 and checked on a second vector.
static void charpoly_coeffs(const uint32_t* M, uint32_t beta[8]) {
    uint32_t pw[9][8];
    std::memset(pw, 0, sizeof(pw));
    pw[0][0] = 1;
    for (int i = 1; i <= 8; ++i) matvec_mod(M, pw[i - 1], pw[i]);
    uint32_t C[8][9];
    for (int r = 0; r < 8; ++r) {
        for (int k = 1; k <= 8; ++k) C[r][k - 1] = pw[8 - k][r];
        C[r][8] = pw[8][r];
    }
    if (!solve8(C, beta)) throw std::runtime_error("mrg8g: singular Krylov matrix");
    uint32_t q[9][8];
    for (int r = 0; r < 8; ++r) q[0][r] = (uint32_t)(r * 7919 + 13);
    for (int i = 1; i <= 8; ++i) matvec_mod(M, q[i - 1], q[i]);
    for (int r = 0; r < 8; ++r) {
        uint32_t acc = 0;
        for (int k = 1; k <= 8; ++k) acc = addmod(acc, mulmod(beta[k - 1], q[8 - k][r]));
        if (acc != q[8][r]) throw std::runtime_error("mrg8g: characteristic polynomial check failed");
    }
}

// K1 == sum_k c_k - 1 (mod p) for lags x = S - 1, K1 == 0 (mod p) for lags
// s = S mod p (mod_lags).
static LeapCoef make_leap(const uint32_t beta[8], bool mod_lags) {
    LeapCoef lc;
    int64_t csum = 0;
    unsigned __int128 negsum = 0, possum = 0;
    for (int k = 0; k < 8; ++k) {
        const int64_t c = beta[k] <= (kP - 1) / 2 ? (int64_t)beta[k] : (int64_t)beta[k] - (int64_t)kP;
        lc.c[k] = (int32_t)c;
        csum += c;
        if (c < 0) negsum += (unsigned __int128)(-c);
        else possum += (unsigned __int128)c;
    }
    // K1 == cmod (mod p), the smallest such value >= negsum (p - 1), so that
    // K1 + sum c_k x_k (x_k in [0, p-1]) stays in [0, 2^64 - 1).
    const uint64_t cmod = mod_lags ? 0 : (uint64_t)(((csum - 1) % (int64_t)kP + (int64_t)kP) % (int64_t)kP);
    const unsigned __int128 base = negsum * (kP - 1);
    const uint64_t bmod = (uint64_t)(base % kP);
    const unsigned __int128 K1 = base + (cmod + kP - bmod) % kP;
    const unsigned __int128 top = K1 + possum * (kP - 1);
    if (top >= ~(unsigned __int128)0 >> 64) throw std::runtime_error("mrg8g: accumulator range exceeds 64 bits");
    lc.K1 = (uint64_t)K1;
    return lc;
}

static void build(HostTables& t) {
    uint32_t M[64];
    std::memset(M, 0, sizeof(M));
    for (int c = 0; c < 8; ++c) M[c] = kCoef[c];
    for (int r = 1; r < 8; ++r) M[r * 8 + r - 1] = 1;
    for (int i = 0; i < kNumJump; ++i) {
        std::memcpy(t.jump[i], M, sizeof(M));
        matmul_mod(M, M, M);
    }
    for (int w = 0; w < kJumpBytes; ++w) {
        std::memcpy(t.jwin[w * 255], t.jump[8 * w], sizeof(M));  // A^(256^w)
        for (int j = 2; j <= 255; ++j) matmul_mod(t.jwin[w * 255 + j - 2], t.jump[8 * w], t.jwin[w * 255 + j - 1]);
    }
    // Row vectors u_m = e_0^T A^m, m = 1..1024.
    static uint32_t u[8 * 128 + 1][8];
    for (int c = 0; c < 8; ++c) u[1][c] = kCoef[c];
    for (int m = 2; m <= 8 * 128; ++m)
        for (int c = 0; c < 8; ++c)  // (u A)[c] = u[0] a_c + u[c+1]
            u[m][c] = addmod(mulmod(u[m - 1][0], kCoef[c]), c < 7 ? u[m - 1][c + 1] : 0u);
    for (int li = 0; li < kNumLayouts; ++li) {
        const int d = layout_stride(li);
        uint32_t* w = t.win + win_offset(li);
        for (int o = 0; o < d; ++o)
            for (int j = 0; j < 8; ++j)
                for (int c = 0; c < 8; ++c) w[(o * 8 + j) * 8 + c] = u[o + 1 + d * j][c];
        std::memcpy(t.dstep[li][0], t.jump[5 + li], sizeof(M));  // A^d = A^(2^(5+li))
        for (int j = 2; j <= 7; ++j) matmul_mod(t.dstep[li][j - 2], t.jump[5 + li], t.dstep[li][j - 1]);
        uint32_t beta[8];
        charpoly_coeffs(t.jump[5 + li], beta);
        t.leap[li] = make_leap(beta, false);
        t.leap_mod[li] = make_leap(beta, true);
    }
}

const HostTables& host_tables() {
    static HostTables t;  // static storage: built once, no heap
    static std::once_flag once;
    std::call_once(once, [] { build(t); });
    return t;
}

void mcg64ni(uint32_t seed, uint32_t st[8]) {
    uint64_t x = seed == 0 ? 97531u : seed;
    for (int k = 0; k < 8; ++k) {
        x = 6364136223846793005ull * x;
        st[k] = (uint32_t)((x >> 32) >> 1);
    }
}

static void matvec_ref(const uint32_t* Mrow, const uint32_t* v, uint32_t* out) {
    uint32_t t[8];
    for (int r = 0; r < 8; ++r) t[r] = dot8_ref(Mrow + r * 8, v);
    std::memcpy(out, t, sizeof(t));
}

void jump_matvec(const uint32_t st[8], uint64_t k, uint32_t out[8]) {
    const HostTables& t = host_tables();
    uint32_t cur[8];
    std::memcpy(cur, st, sizeof(cur));
    for (int i = 0; i < 64; ++i)
        if ((k >> i) & 1u) matvec_ref(t.jump[i], cur, cur);
    std::memcpy(out, cur, sizeof(cur));
}

void jump_matvec_bits(const uint32_t st[8], const short bits[200], uint32_t out[8]) {
    const HostTables& t = host_tables();
    uint32_t cur[8];
    std::memcpy(cur, st, sizeof(cur));
    for (int i = 0; i < 200; ++i)
        if (bits[i]) matvec_ref(t.jump[i], cur, cur);
    std::memcpy(out, cur, sizeof(cur));
}

void jump_exact_bits(const uint32_t st[8], const short bits[200], uint32_t out[8]) {
    const HostTables& t = host_tables();
    uint32_t J[64], T[64], col[8];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) J[r * 8 + c] = (r == c);
    for (int nb = 0; nb < 200; ++nb) {
        if (!bits[nb]) continue;
        for (int c = 0; c < 8; ++c) {
            for (int q = 0; q < 8; ++q) col[q] = t.jump[nb][q * 8 + c];
            for (int r = 0; r < 8; ++r) T[r * 8 + c] = dot8_ref(J + r * 8, col);
        }
        std::memcpy(J, T, sizeof(T));
    }
    matvec_ref(J, st, out);
}

void step_host(uint32_t st[8], uint64_t n, uint32_t* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t z = dot8_ref(kCoef, st);
        std::memmove(st + 1, st, 7 * sizeof(uint32_t));
        st[0] = z;
        if (out) out[i] = z;
    }
}

}  // namespace mrg8g
