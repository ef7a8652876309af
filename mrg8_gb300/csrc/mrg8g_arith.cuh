// mrg8g_arith.cuh -- exact modular arithmetic and integer-only uniform
// conversion shared by the host runtime and the sm_103a kernels.
//
// Uniform conversion.  The reference forms fp64 uniforms as
//   ORIGINAL: RN(double(S) * rnorm)      (original/mrg8.cpp:231-237)
//   SHIFTED : RN(double(S - 1) * rnorm)  (cuda/mrg8_cuda.cu:251-252,363)
// with rnorm = RN(1/(2^31-1)).  Since 1/(2^31-1) = 2^-31 (1 + 2^-31 + 2^-62
// + ...), rnorm = 2^-31 + 2^-62 exactly, so for a 31-bit integer v the exact
// product is (v * 2^31 + v) * 2^-62: a 62-bit integer whose two copies of v
// do not overlap.  The functions below round that integer to 53 bits
// (round-to-nearest-even) and assemble the IEEE-754 word directly, which is
// bit-identical to the multiply but runs on the integer pipes: GB300's FP64
// rate is far too low to convert at HBM speed.  fp32 is (float) of the fp64
// value, i.e. a second round-to-nearest-even from 53 to 24 bits (the two
// roundings are not always equal to one rounding of the exact product, e.g.
// v = 0x7FFFFFBF, so both are done).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MRG8G_HD __host__ __device__ __forceinline__
#else
#define MRG8G_HD inline
#endif

namespace mrg8g {

constexpr uint32_t kP = 2147483647u;  // 2^31 - 1

MRG8G_HD uint32_t clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__clz((int)v);
#else
    return v ? (uint32_t)__builtin_clz(v) : 32u;
#endif
}

// 32 x 32 -> 64-bit unsigned multiply-add (one IMAD.WIDE.U32 on the device).
MRG8G_HD uint64_t mad_wide_u32(uint32_t a, uint32_t b, uint64_t c) {
#if defined(__CUDA_ARCH__)
    uint64_t d;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
#else
    return (uint64_t)a * b + c;
#endif
}

// Normalised 53-bit significand m (2^52 <= m <= 2^53) and the biased exponent
// minus one, for RN(v * rnorm), 1 <= v <= 2^31 - 1.  With xn = v << lz
// (leading one at bit 31) the exact product scaled to [2^52, 2^53) is
// xn (2^31 + 1) / 2^10, so one multiply-add forms it together with the
// round-to-nearest-even bias 0x1FF + (bit 10 of xn), and m is that sum >> 10.
struct Sig53 {
    uint64_t m;
    uint32_t em1;  // biased exponent - 1 (the implicit bit of m adds one)
};

MRG8G_HD Sig53 sig53(uint32_t v) {
    const uint32_t lz = clz32(v);                // 1..31
    const uint32_t xn = v << lz;                 // leading one at bit 31
    const uint32_t lsb = (xn >> 10) & 1u;        // the bit rounded to
    Sig53 r;
    r.m = mad_wide_u32(xn, 0x80000001u, 0x1FFu + lsb) >> 10;
    r.em1 = 1022u - lz;                          // value in [2^-lz, 2^(1-lz))
    return r;
}

// IEEE-754 bits of RN(v * rnorm) for 1 <= v <= 2^31 - 1.
MRG8G_HD uint64_t f64_bits_pos(uint32_t v) {
    const Sig53 s = sig53(v);
    return ((uint64_t)s.em1 << 52) + s.m;  // m == 2^53 carries into the exponent
}

// IEEE-754 bits of (float)RN(v * rnorm) for 1 <= v <= 2^31 - 1.
MRG8G_HD uint32_t f32_bits_pos(uint32_t v) {
    const Sig53 s = sig53(v);
    const uint32_t lsb = (uint32_t)(s.m >> 29) & 1u;
    const uint32_t m24 = (uint32_t)((s.m + 0x0FFFFFFFull + lsb) >> 29);  // 2^23..2^24
    return ((s.em1 - 896u) << 23) + m24;
}

// x is the stream value minus one, 0 <= x <= p - 1 (S = x + 1 in [1, p]).
MRG8G_HD uint64_t f64_bits(uint32_t x, bool shifted) {
    if (shifted) return x ? f64_bits_pos(x) : 0ull;
    return f64_bits_pos(x + 1u);
}

MRG8G_HD uint32_t f32_bits(uint32_t x, bool shifted) {
    if (shifted) return x ? f32_bits_pos(x) : 0u;
    return f32_bits_pos(x + 1u);
}

// ------------------------------------------------------------ modular math

// bigDotProd of original/mrg8.cpp:72-82: representative in [1, p] for a
// non-zero sum, 0 for an all-zero sum.  Operands must be < 2^31.
MRG8G_HD uint32_t dot8_ref(const uint32_t* x, const uint32_t* y) {
    uint64_t s1 = 0, s2 = 0;
    for (int q = 0; q < 4; ++q) {
        s1 += (uint64_t)x[q] * y[q];
        s2 += (uint64_t)x[4 + q] * y[4 + q];
    }
    const uint64_t M = kP;
    uint64_t s = (s1 & M) + (s1 >> 31) + (s2 & M) + (s2 >> 31);
    s = (s & M) + (s >> 31);
    return (uint32_t)((s & M) + (s >> 31));
}

// Canonical residue in [0, p-1] of a value below 2^64.
MRG8G_HD uint32_t mod_p64(uint64_t v) {
    uint64_t s = (v & kP) + (v >> 31);   // < 2^34
    s = (s & kP) + (s >> 31);            // < 2^31 + 8
    uint32_t r = (uint32_t)s;
    return r >= kP ? r - kP : r;
}

// One decimated-recurrence step: acc = K + sum_k c_k x_{j-k} in [1, 2^64)
// (signed 32x32 -> 64-bit multiply-adds, wrapping mod 2^64), then a Mersenne
// reduction to x_j = S_j - 1 in [0, p-1]:
//   acc = H 2^32 + L == 2H + L (mod p);  s = L + 2H < 3 * 2^32;
//   t = (s & p) + (s >> 31) in [1, p + 5];  x = t - 1, minus p when >= p.
MRG8G_HD uint64_t mad_wide_s32(int32_t a, uint32_t b, uint64_t c) {
#if defined(__CUDA_ARCH__)
    uint64_t d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
#else
    return c + (uint64_t)((int64_t)a * (int64_t)(int32_t)b);
#endif
}

MRG8G_HD uint32_t reduce_acc(uint64_t acc) {
    const uint32_t L = (uint32_t)acc, H = (uint32_t)(acc >> 32);
    const uint64_t s = (uint64_t)L + ((uint64_t)H << 1);
    const uint32_t t = ((uint32_t)s & kP) + (uint32_t)(s >> 31);
    const uint32_t x = t - 1u;
    const uint32_t y = x - kP;
    return x < y ? x : y;
}

// Residue in [0, p-1] -> stream representative in [1, p].
MRG8G_HD uint32_t rep1p(uint32_t r) { return r ? r : kP; }

}  // namespace mrg8g
