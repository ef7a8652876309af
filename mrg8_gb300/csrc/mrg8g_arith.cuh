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

// Left shift that yields 0 for a shift count of 32 (PTX shl clamps).
MRG8G_HD uint32_t shl_clamp(uint32_t a, uint32_t s) {
#if defined(__CUDA_ARCH__)
    uint32_t d;
    asm("shl.b32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(s));
    return d;
#else
    return s >= 32 ? 0u : a << s;
#endif
}

// IEEE-754 bits of RN(v * rnorm), rnorm = 2^-31 + 2^-62 = RN(1/(2^31-1)).
// The exact product is (v 2^31 + v) 2^-62.  With lz = clz(v) and
// xm = (v << lz) >> 1 (leading one at bit 30), the 53-bit significand is
// M = xm 2^22 + RNE(xm / 2^9), RNE(xm / 2^9) = (xm + 0xFF + bit 9 of xm) >> 9
// (no overflow: xm < 2^31), and the biased exponent is 1023 - lz, entering
// the high word as (1022 - lz) 2^20 plus M's leading one at bit 52.  The low
// word (xm << 22) + RNE(...) carries into the high word only at v = p, whose
// value rounds up to 1.0.  v = 0 gives xm = 0 and min(high word, xm) = 0
// (xm >= 2^30 exceeds every high word otherwise).  Shifts and adds only: no
// multiply, which would occupy the FMA-heavy pipe that the recurrence's
// multiply-adds already saturate.
//
// For 0 <= v <= p - 1 (SHIFTED: v = S - 1).
MRG8G_HD uint64_t f64_bits_below_p(uint32_t v) {
    const uint32_t lz = clz32(v);
    const uint32_t xm = shl_clamp(v, lz) >> 1;
    const uint32_t t = (xm + 0xFFu + ((xm >> 9) & 1u)) >> 9;
    const uint32_t lo = (xm << 22) + t;
    uint32_t hi = (xm >> 10) - (lz << 20) + (1022u << 20);
    hi = hi < xm ? hi : xm;
    return ((uint64_t)hi << 32) | lo;
}

// For 0 <= v <= p (ORIGINAL: v = S), with the low word's carry.
MRG8G_HD uint64_t f64_bits_to_p(uint32_t v) {
    const uint32_t lz = clz32(v);
    const uint32_t xm = shl_clamp(v, lz) >> 1;
    const uint32_t t = (xm + 0xFFu + ((xm >> 9) & 1u)) >> 9;
    const uint32_t lo = (xm << 22) + t;
    uint32_t hi = (xm >> 10) - (lz << 20) + (1022u << 20) + (lo < t ? 1u : 0u);
    hi = hi < xm ? hi : xm;
    return ((uint64_t)hi << 32) | lo;
}

// IEEE-754 bits of (float)RN(v * rnorm) for 0 <= v <= 2^31 - 1.  A single
// round-to-nearest-even of the exact product to 24 bits is
// ((xn >> 1) + 0x40) >> 7 with xn = v << lz (xn is even and the halfway case
// cannot occur); it equals the double rounding through fp64 for every v
// except v = 0x7FFFFFBF, where the fp64 value lands on a halfway point and
// rounds up once more.  v = 0 gives +0 through min(., xn).
MRG8G_HD uint32_t f32_bits_of(uint32_t v) {
    const uint32_t lz = clz32(v);
    const uint32_t xn = shl_clamp(v, lz);
    const uint32_t m24 = ((xn >> 1) + 0x40u) >> 7;
    uint32_t bits = ((126u - lz) << 23) + m24 + (v == 0x7FFFFFBFu ? 1u : 0u);
    return bits < xn ? bits : xn;
}

// ORIGINAL from s = S mod p in [0, p-1] (the lag form of the fp64 ORIGINAL
// kernels): for s >= 1 the word of f64_bits_below_p (no carry below p), and
// s = 0 (S = p) gives 1.0, whose low word the same assembly already yields.
MRG8G_HD uint64_t f64_bits_orig(uint32_t s) {
    const uint32_t lz = clz32(s);
    const uint32_t xm = shl_clamp(s, lz) >> 1;
    const uint32_t t = (xm + 0xFFu + ((xm >> 9) & 1u)) >> 9;
    const uint32_t lo = (xm << 22) + t;
    const uint32_t hi = (xm >> 10) - (lz << 20) + (1022u << 20);
    return ((uint64_t)(s ? hi : 0x3FF00000u) << 32) | lo;
}

// x is the stream value minus one, 0 <= x <= p - 1 (S = x + 1 in [1, p]).
MRG8G_HD uint64_t f64_bits(uint32_t x, bool shifted) { return shifted ? f64_bits_below_p(x) : f64_bits_to_p(x + 1u); }
MRG8G_HD uint32_t f32_bits(uint32_t x, bool shifted) { return f32_bits_of(shifted ? x : x + 1u); }


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

// One decimated-recurrence step.  The multiply-adds form
// a = K1 + sum_k c_k x_{j-k} in [0, 2^64 - 1) with a == S_j - 1 (mod p)
// (signed 32x32 -> 64-bit products, wrapping mod 2^64; K1 is chosen on the
// host).  The reduction to x_j = S_j - 1 in [0, p-1]:
//   a = H 2^32 + L == 2H + L (mod p);  s = 2H + L < 3 * 2^32  (one mad.wide);
//   y = (s mod 2^31) + (s >> 31) = s_lo - (s >> 31) p  in [0, p + 5];
//   x = y, or y - p when y >= p.
//
// The multiply-add is plain 64-bit C++ on both sides: nvcc schedules it
// better than an inline mad.wide.s32 (fewer companion ALU instructions per
// product on sm_103a).
MRG8G_HD uint64_t mad_wide_s32(int32_t a, uint32_t b, uint64_t c) {
    return c + (uint64_t)((int64_t)a * (int64_t)(int32_t)b);
}

MRG8G_HD uint32_t reduce_acc(uint64_t a) {
    const uint64_t s = mad_wide_u32((uint32_t)(a >> 32), 2u, (uint32_t)a);
    const uint32_t q = (uint32_t)(s >> 31);
    const uint32_t y = (uint32_t)s - q * kP;
    const uint32_t z = y - kP;
    return y < z ? y : z;
}

// The same value as reduce_acc with its tail on the integer ALU:
// y = (s mod 2^31) + (s >> 31) by a funnel shift, a mask and an add instead
// of s_lo - q p (a 32-bit multiply, which shares the FMA-heavy pipe with the
// recurrence's wide multiply-adds).  The kernels whose outputs are 4 bytes
// are bound by that pipe and use this form (u32 1003 -> 1045 Goutputs/s at
// 2^30); the fp64 kernels measured slightly faster with reduce_acc.
MRG8G_HD uint32_t reduce_acc_alu(uint64_t a) {
    const uint64_t s = mad_wide_u32((uint32_t)(a >> 32), 2u, (uint32_t)a);
#if defined(__CUDA_ARCH__)
    uint32_t r;
    asm("{ .reg .u32 l, h, q, y, z;\n\t"
        "mov.b64 {l, h}, %1;\n\t"
        "shf.l.clamp.b32 q, l, h, 1;\n\t"
        "and.b32 y, l, 0x7FFFFFFF;\n\t"
        "add.u32 y, y, q;\n\t"
        "sub.u32 z, y, 0x7FFFFFFF;\n\t"
        "min.u32 %0, y, z; }"
        : "=r"(r)
        : "l"(s));
    return r;
#else
    const uint32_t y = ((uint32_t)s & kP) + (uint32_t)(s >> 31);
    const uint32_t z = y - kP;
    return y < z ? y : z;
#endif
}

// Residue in [0, p-1] -> stream representative in [1, p].
MRG8G_HD uint32_t rep1p(uint32_t r) { return r ? r : kP; }

// Lag forms of the kernels' recurrences, from a dot8_ref result S in [0, p]
// (0 only for an all-zero sum, i.e. residue 0): x = S - 1 in [0, p-1], or
// s = S mod p in [0, p-1] for the fp64 ORIGINAL outputs (whose conversion
// then needs no + 1).
MRG8G_HD uint32_t lag_minus1(uint32_t S) { return (S ? S : kP) - 1u; }
MRG8G_HD uint32_t lag_mod(uint32_t S) {
    const uint32_t z = S - kP;
    return S < z ? S : z;
}

}  // namespace mrg8g
