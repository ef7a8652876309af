// check_kernel_math.cpp -- CPU check of the arithmetic the kernels run.
//
// Built by tests/test_kernel_math.py with g++ against the library's host
// sources (mrg8g_tables.cpp and the shared header mrg8g_arith.cuh).
//
//   check_kernel_math conv
//       every v in [1, 2^31-1]: integer fp64/fp32 words == RN(double(v) *
//       (1.0/(2^31-1))) and (float) of it; plus the SHIFTED zero.  Also the
//       fp32 word of the kernels' FP32-pipe form (f32_bits_fp in
//       mrg8g_device.cuh), through an exact integer emulation of its two
//       roundings (round-toward-zero fma, round-to-nearest add); and the
//       fp64 ORIGINAL form that takes s = S mod p (f64_bits_orig).
//   check_kernel_math leap <stream.bin> <s0..s7>
//       stream.bin holds the oracle's outputs S[0..N) from state s; checks
//       the window tables (S[B + o + d j] = row . s_B at B = 0), the kernels'
//       window setup (row j = 0 against the states A^(d j) s_B formed from
//       the dstep table with the warp's folded arithmetic), and runs every
//       layout's decimated recurrence with the kernels' step (mad_wide_s32 +
//       reduce_acc, and reduce_acc_alu of the 4-byte kernels) over the whole
//       stream; writes the row-major jump table to
//       stdout as raw u32 for the Python side to compare.
//   check_kernel_math jwin <s0..s7> <k...>
//       the device jump (warp_jump in mrg8g_device.cuh) emulated lane by lane
//       on the byte-window table: for each offset k, prints A^k s as
//       canonical residues, after checking it against jump_matvec (one
//       product per set bit of k) and every window matrix against
//       A^(j 256^w) formed from the A^(2^i) table.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mrg8g_arith.cuh"
#include "mrg8g_tables.h"

using namespace mrg8g;

static int bitlen(uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; }

// Float bits of f32_bits_fp(v): fh = vh 2^-15 and fl = vl 2^-31 are exact;
// c = RZ(fh 2^-31 + fl) and f = RN(fh + c) are emulated on integers in
// units of 2^-46 (both operands are exact multiples of it).
static uint32_t f32_fp_core(uint32_t v) {
    const uint64_t vh = v >> 16, vl = v & 0xFFFFu;
    uint64_t c = (vl << 15) + vh;  // (vl + vh 2^-15) 2^-31 in units of 2^-46
    int nb = bitlen(c);
    if (nb > 24) c &= ~((1ull << (nb - 24)) - 1);  // round toward zero to 24 bits
    uint64_t s = (vh << 31) + c;                   // fh + c in units of 2^-46
    nb = bitlen(s);
    if (nb > 24) {  // round to nearest even to 24 bits
        const int sh = nb - 24;
        uint64_t q = s >> sh;
        const uint64_t rem = s & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1))) ++q;
        s = q << sh;
    }
    const float f = (float)((double)s * 0x1p-46);  // exact: at most 24 significant bits
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}
static uint32_t f32_fp_emulated(uint32_t v) { return v == 0x7FFFFFBFu ? 0x3F800000u : f32_fp_core(v); }

static int conv() {
    const double rnorm = 1.0 / 2147483647.0;
    unsigned long bad = 0;
    for (uint64_t v = 1; v <= 2147483647ull; ++v) {
        const double d = (double)(uint32_t)v * rnorm;
        uint64_t db;
        std::memcpy(&db, &d, 8);
        const float f = (float)d;
        uint32_t fb;
        std::memcpy(&fb, &f, 4);
        if (db != f64_bits_to_p((uint32_t)v) || fb != f32_bits_of((uint32_t)v) || fb != f32_fp_emulated((uint32_t)v)) {
            if (bad++ < 8) std::fprintf(stderr, "mismatch at v=%lu\n", (unsigned long)v);
        }
        // SHIFTED converts x = S - 1 = v; ORIGINAL converts v = x + 1.
        if (v < 2147483647ull && (f64_bits((uint32_t)v, true) != db || f32_bits((uint32_t)v, true) != fb))
            bad++;
        if (f64_bits((uint32_t)v - 1, false) != db || f32_bits((uint32_t)v - 1, false) != fb) bad++;
        // The fp64 ORIGINAL kernels convert s = S mod p (S = p -> s = 0).
        const uint32_t s = (uint32_t)(v % 2147483647ull);
        if (f64_bits_orig(s) != db) {
            if (bad++ < 8) std::fprintf(stderr, "ORIGINAL lag-form mismatch at v=%lu\n", (unsigned long)v);
        }
    }
    if (f64_bits(0, true) != 0 || f32_bits(0, true) != 0 || f32_fp_emulated(0) != 0) bad++;
    std::printf("conv bad=%lu\n", bad);
    return bad ? 1 : 0;
}

static int leap(const char* path, const uint32_t s0[8]) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return 2;
    std::vector<uint32_t> S;
    uint32_t buf[4096];
    size_t got;
    while ((got = std::fread(buf, 4, 4096, f)) > 0) S.insert(S.end(), buf, buf + got);
    std::fclose(f);
    const HostTables& t = host_tables();
    unsigned long bad = 0, checked = 0;
    for (int li = 0; li < kNumLayouts; ++li) {
        const int d = layout_stride(li);
        const uint32_t* w = t.win + win_offset(li);
        const LeapCoef& lc = t.leap[li];
        if (S.size() < (size_t)d * 16) return 3;
        const size_t rows = S.size() / d;
        // The kernels' lane_window: the states at B + d j from the dstep
        // table with the warp's folded arithmetic, then row j = 0 of the
        // window table against each.
        uint32_t st[8][8];
        std::memcpy(st[0], s0, sizeof(st[0]));
        for (int j = 1; j < 8; ++j)
            for (int r = 0; r < 8; ++r) {
                uint64_t fsum = 0;
                for (int l4 = 0; l4 < 4; ++l4) {
                    const uint32_t* M = t.dstep[li][j - 1];
                    const uint64_t part = (uint64_t)M[r * 8 + 2 * l4] * s0[2 * l4] + (uint64_t)M[r * 8 + 2 * l4 + 1] * s0[2 * l4 + 1];
                    fsum += (part & kP) + (part >> 31);
                }
                st[j][r] = mod_p64(fsum);
            }
        for (int o = 0; o < d; ++o) {
            uint32_t x[8];
            for (int j = 0; j < 8; ++j) {
                const uint32_t v = dot8_ref(w + (o * 8 + j) * 8, s0);
                const uint32_t Sv = v ? v : kP;
                if (Sv != S[o + (size_t)d * j]) bad++;
                x[j] = Sv - 1u;
                const uint32_t vd = dot8_ref(w + o * 64, st[j]);
                if ((vd ? vd : kP) - 1u != x[j]) {
                    if (bad++ < 8) std::fprintf(stderr, "window mismatch d=%d o=%d j=%d\n", d, o, j);
                }
            }
            uint32_t sm[8];  // the same substream with lags S mod p (fp64 ORIGINAL kernels)
            for (int j = 0; j < 8; ++j) sm[j] = lag_mod(x[j] + 1u);
            const LeapCoef& lm = t.leap_mod[li];
            for (size_t j = 8; j < rows; ++j) {
                uint64_t acc = lc.K1, accm = lm.K1;
                for (int k = 1; k <= 8; ++k) {
                    acc = mad_wide_s32(lc.c[k - 1], x[(j - k) & 7], acc);
                    accm = mad_wide_s32(lm.c[k - 1], sm[(j - k) & 7], accm);
                }
                const uint32_t xn = reduce_acc(acc);
                if (reduce_acc_alu(acc) != xn) bad++;
                x[j & 7] = xn;
                sm[j & 7] = reduce_acc(accm);
                if (xn + 1u != S[o + (size_t)d * j] || sm[j & 7] != S[o + (size_t)d * j] % kP) {
                    if (bad++ < 8) std::fprintf(stderr, "leap mismatch d=%d o=%d j=%zu\n", d, o, j);
                }
                checked++;
            }
        }
    }
    std::fwrite(t.jump, 4, sizeof(t.jump) / 4, stdout);
    std::fprintf(stderr, "leap checked=%lu bad=%lu\n", checked, bad);
    return bad ? 1 : 0;
}

// warp_jump of mrg8g_device.cuh, one lane at a time: lane l holds row l/4,
// columns 2(l%4) and 2(l%4)+1; the four lanes of a row add their folded
// partial sums (the two xor-shuffles) and reduce with mod_p64.
static void warp_jump_emulated(const HostTables& t, uint32_t s[8], uint64_t k) {
    if (k == 0) return;
    uint32_t v[8];
    std::memcpy(v, s, sizeof(v));
    for (int w = 0; w < kJumpBytes; ++w) {
        const uint32_t j = (uint32_t)(k >> (8 * w)) & 255u;
        if (!j) continue;
        const uint32_t* M = t.jwin[w * 255 + j - 1];
        uint32_t nv[8];
        for (int r = 0; r < 8; ++r) {
            uint64_t f = 0;
            for (int l4 = 0; l4 < 4; ++l4) {
                const uint64_t part = (uint64_t)M[r * 8 + 2 * l4] * v[2 * l4] + (uint64_t)M[r * 8 + 2 * l4 + 1] * v[2 * l4 + 1];
                f += (part & kP) + (part >> 31);
            }
            nv[r] = mod_p64(f);
        }
        std::memcpy(v, nv, sizeof(v));
    }
    std::memcpy(s, v, sizeof(v));
}

static int jwin(const uint32_t s0[8], int nk, char** ks) {
    const HostTables& t = host_tables();
    unsigned long bad = 0;
    for (int w = 0; w < kJumpBytes; ++w) {  // A^(j 256^w) = A^((j-1) 256^w) A^(256^w), independently
        uint32_t P[64];
        std::memcpy(P, t.jump[8 * w], sizeof(P));
        for (int j = 1; j <= 255; ++j) {
            if (std::memcmp(P, t.jwin[w * 255 + j - 1], sizeof(P))) bad++;
            // P <- P * A^(256^w) by bits: A^(256^w) = prod of its own square chain
            uint32_t Q[64];
            matmul_mod(t.jump[8 * w], P, Q);
            std::memcpy(P, Q, sizeof(P));
        }
    }
    for (int i = 0; i < nk; ++i) {
        const uint64_t k = std::strtoull(ks[i], nullptr, 10);
        uint32_t a[8], b[8];
        std::memcpy(a, s0, sizeof(a));
        warp_jump_emulated(t, a, k);
        jump_matvec(s0, k, b);
        for (int q = 0; q < 8; ++q) {
            if (k && a[q] >= kP) bad++;
            if (a[q] % kP != b[q] % kP) bad++;
        }
        std::printf("%llu", (unsigned long long)k);
        for (int q = 0; q < 8; ++q) std::printf(" %u", a[q]);
        std::printf("\n");
    }
    std::printf("bad=%lu\n", bad);
    return bad ? 1 : 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && !std::strcmp(argv[1], "conv")) return conv();
    if (argc >= 10 && !std::strcmp(argv[1], "jwin")) {
        uint32_t s[8];
        for (int q = 0; q < 8; ++q) s[q] = (uint32_t)std::strtoul(argv[2 + q], nullptr, 10);
        return jwin(s, argc - 10, argv + 10);
    }
    if (argc >= 11 && !std::strcmp(argv[1], "leap")) {
        uint32_t s[8];
        for (int q = 0; q < 8; ++q) s[q] = (uint32_t)std::strtoul(argv[3 + q], nullptr, 10);
        return leap(argv[2], s);
    }
    std::fprintf(stderr, "usage: check_kernel_math conv | leap <stream.bin> s0..s7 | jwin s0..s7 k...\n");
    return 2;
}
