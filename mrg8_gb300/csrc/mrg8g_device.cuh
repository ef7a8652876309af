// mrg8g_device.cuh -- sm_103a device building blocks of the MRG8 kernels.
//
// Every kernel translation unit includes this header once; it gets its own
// copy of the device tables (module globals, uploaded per device by
// MRG8G_DEFINE_TABLE_UPLOAD) so no kernel ever needs a cudaMalloc.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mrg8g_arith.cuh"
#include "mrg8g_tables.h"

namespace mrg8g {

constexpr unsigned kFull = 0xFFFFFFFFu;
// Shared-memory words per warp for lane_window of layout V (the eight
// states, then the window values of the lane's V substreams; lane_window_rows
// uses the values' part only).
MRG8G_HDC constexpr int window_scratch(int V) { return 64 + 8 * V * 32; }

// Output kinds; the numbering is part of the C ABI (include/mrg8g.h).
enum Kind : int { kU32 = 0, kF64Orig = 1, kF64Shift = 2, kF32Orig = 3, kF32Shift = 4 };

template <int KIND> struct OutOf;
template <> struct OutOf<kU32> { using T = uint32_t; };
template <> struct OutOf<kF64Orig> { using T = uint64_t; };
template <> struct OutOf<kF64Shift> { using T = uint64_t; };
template <> struct OutOf<kF32Orig> { using T = uint32_t; };
template <> struct OutOf<kF32Shift> { using T = uint32_t; };

// IEEE-754 bits of (float)RN(v * rnorm) for 0 <= v <= 2^31 - 1, the value
// f32_bits_of (mrg8g_arith.cuh) assembles with integer operations, computed
// here on the FP32 pipes, which the integer recurrence leaves idle.
//
// With v = vh 2^16 + vl (vh < 2^15, vl < 2^16) and e = v * 2^-31 < 1, the
// exact product is (v + e) 2^-31.  Rounding the 31-bit v + e to 24 bits
// differs from rounding v itself only where v sits exactly on a rounding
// boundary (e > 0 then rounds up) or where the preceding fp64 rounding of e
// reaches 1 (v > 2^31 - 2^8, of which only v = 0x7FFFFFBF changes the
// result).  So any e' in (0, 1) for v >= 2^24, and any e' below half an ulp
// of v for v < 2^24, gives the same float as RN(v + e') 2^-31, except at
// 0x7FFFFFBF, whose result is 1.0.  Here
//   fh = vh 2^-15 and fl = vl 2^-31, both exact (bit-pattern magic with an
//        exact FP32 subtraction),
//   c  = RZ(fh 2^-31 + fl) = RZ((vl + vh 2^-15) 2^-31): e' = vh 2^-15 less
//        the truncation, in (0, 1) for v >= 2^24 and below half an ulp of v
//        otherwise,
//   f  = RN(fh + c) = RN(v + e') 2^-31, one rounding of an exact sum.
// v = 0 gives +0.  Checked on every v in [0, 2^31 - 1] against the GPU's own
// (float)((double)v * rnorm) (the exhaustive conversion test) and against an
// exact integer emulation of both roundings on the host.  On the u32-bound
// recurrence this conversion costs far less than the integer one: fp32 at
// 2^30 went from 834 to 883 Goutputs/s.
__device__ __forceinline__ uint32_t f32_bits_fp(uint32_t v) {
    const float fh = __fsub_rn(__int_as_float(__byte_perm(v, 0x43800000u, 0x7632)), 256.0f);
    const float fl = __fsub_rn(__int_as_float((v & 0xFFFFu) | 0x3B800000u), 0x1p-8f);
    const float c = __fmaf_rz(fh, 0x1p-31f, fl);
    const float f = __fadd_rn(fh, c);
    return v == 0x7FFFFFBFu ? 0x3F800000u : __float_as_uint(f);
}

// fp64 ORIGINAL keeps its lags as S mod p, the other kinds as S - 1
// (lag_mod / lag_minus1 of mrg8g_arith.cuh, LeapCoef of mrg8g_tables.h):
// its conversion then needs neither the + 1 nor the carry into the high word
// (fp64 ORIGINAL at 2^30: 713 -> 747 Goutputs/s).  fp32 ORIGINAL measured
// slightly slower in that form (834 -> 828, a comparison s - 1 >= 0x7FFFFFBE
// selecting 1.0 in place of the + 1) and keeps S - 1.
template <int KIND>
constexpr bool kLagMod = KIND == kF64Orig;

template <int KIND>
__device__ __forceinline__ uint32_t lag_of(uint32_t S) {
    if constexpr (kLagMod<KIND>) return lag_mod(S);
    else return lag_minus1(S);
}

// Output word for a lag of the kind's form (S mod p for fp64 ORIGINAL, else
// S - 1).
template <int KIND>
__device__ __forceinline__ typename OutOf<KIND>::T convert(uint32_t lag) {
    if constexpr (KIND == kU32) return lag + 1u;
    else if constexpr (KIND == kF64Orig) return f64_bits_orig(lag);
    else if constexpr (KIND == kF64Shift) return f64_bits(lag, true);
    else if constexpr (KIND == kF32Orig) return f32_bits_fp(lag + 1u);
    else return f32_bits_fp(lag);
}

}  // namespace mrg8g

// Per-translation-unit device tables and their uploader.
#define MRG8G_DEFINE_TABLE_UPLOAD(fn_name)                                                      \
    static __device__ __align__(16) uint32_t g_jwin[::mrg8g::kJumpWinMats * 64];                \
    static __device__ __align__(16) uint32_t g_win[::mrg8g::kWinWords];                         \
    static __device__ __align__(16) uint32_t g_dstep[::mrg8g::kNumLayouts * 7 * 64];            \
    cudaError_t fn_name() {                                                                    \
        const ::mrg8g::HostTables& t = ::mrg8g::host_tables();                                 \
        cudaError_t e = cudaMemcpyToSymbol(g_jwin, t.jwin, sizeof(g_jwin));                    \
        if (e != cudaSuccess) return e;                                                        \
        e = cudaMemcpyToSymbol(g_dstep, t.dstep, sizeof(g_dstep));                             \
        if (e != cudaSuccess) return e;                                                        \
        return cudaMemcpyToSymbol(g_win, t.win, sizeof(g_win));                                \
    }

namespace mrg8g {

// Lane-uniform 8-word state s (canonical or raw words < 2^31) -> A^k s, as
// canonical residues in [0, p-1] (k = 0 leaves s as it is), computed by the
// whole warp from the byte-window table `jwin` (kJumpWinMats matrices
// A^(j 256^w)): one matrix-vector product per non-zero byte of k, at most
// eight.  The eight matrices' entries are all requested before the first
// product, so the jump waits for one table round trip rather than one per
// step.  Lane l owns row l/4 and columns 2(l%4), 2(l%4)+1 of each matrix (one
// 8-byte load); partial sums meet by two xor-shuffles and the new vector is
// re-broadcast.  Must be called by all 32 lanes with the same s and k.
__device__ __forceinline__ void warp_jump(const uint32_t* __restrict__ jwin, uint32_t s[8], uint64_t k) {
    if (k == 0) return;
    const int lane = threadIdx.x & 31;
    const int c0 = (lane & 3) << 1;
    uint2 m[kJumpBytes];
#pragma unroll
    for (int w = 0; w < kJumpBytes; ++w) {
        const uint32_t j = (uint32_t)(k >> (8 * w)) & 255u;
        m[w] = j ? __ldg(reinterpret_cast<const uint2*>(jwin + (w * 255 + j - 1) * 64) + lane) : make_uint2(0u, 0u);
    }
    uint32_t a0 = c0 == 0 ? s[0] : c0 == 2 ? s[2] : c0 == 4 ? s[4] : s[6];
    uint32_t a1 = c0 == 0 ? s[1] : c0 == 2 ? s[3] : c0 == 4 ? s[5] : s[7];
    uint32_t val = 0;
#pragma unroll
    for (int w = 0; w < kJumpBytes; ++w) {
        if (((k >> (8 * w)) & 255u) == 0) continue;  // lane-uniform
        const uint64_t part = (uint64_t)m[w].x * a0 + (uint64_t)m[w].y * a1;  // < 2^63
        uint64_t f = (part & kP) + (part >> 31);                              // < 2^33
        f += __shfl_xor_sync(kFull, f, 1);
        f += __shfl_xor_sync(kFull, f, 2);                                    // < 2^35
        val = mod_p64(f);
        a0 = __shfl_sync(kFull, val, c0 << 2);
        a1 = __shfl_sync(kFull, val, (c0 << 2) + 4);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) s[q] = __shfl_sync(kFull, val, q << 2);
}

// Offset within a warp row (32 V outputs) of lane `lane`'s substream v, for
// outputs of ELEM bytes.  A lane owns V consecutive outputs, except 8-byte
// outputs with V = 4: there lane l owns the pairs at 2 l and 64 + 2 l, so that
// each 16-byte store instruction of the warp covers 512 contiguous bytes.
template <int V, int ELEM>
MRG8G_HDC uint32_t sub_offset(uint32_t lane, uint32_t v) {
    return (ELEM == 8 && V == 4) ? 64u * (v >> 1) + 2u * lane + (v & 1u) : (uint32_t)V * lane + v;
}

// Initial window of a lane for layout V: x[v][j] = the lag (S - 1, or S mod p
// when LAG_MOD) of S[B + o + d j] with
// o = sub_offset(lane, v) and d = 32 V, for j = 0..7, from the state s taken
// at stream position B (canonical or raw words < 2^31).  Since
// S[B + o + d j] = e_0^T A^(o + 1) s_(B + d j) with s_(B + d j) = A^(d j) s,
// the warp forms the seven states s_(B + d j), j = 1..7 (one warp-cooperative
// product each, all seven at once, from the `dstep` table) and each lane takes
// the dot products of its V rows e_0^T A^(o + 1) (row j = 0 of the window
// table) with the eight states.  The matrices' parts and the first two rows
// of every lane are requested together, before the first product, so the
// setup waits for one table round trip after the jump (rows 2 and 3 of V = 4
// are requested after the products, to keep the register peak below the main
// loop's).  The states and the finished values pass through the warp's
// `scratch` (window_scratch(V) words: 64 for the states, then the values
// laid out [slot][lane]).
template <int V, int ELEM, bool LAG_MOD>
__device__ __forceinline__ void lane_window(const uint32_t* __restrict__ win, const uint32_t* __restrict__ dstep,
                                            const uint32_t s[8], int lane, uint32_t* scratch, uint32_t (&x)[V][8]) {
    constexpr int li = layout_index(V);
    constexpr int VE = V < 2 ? V : 2;  // rows requested with the matrices
    const uint4* rows = reinterpret_cast<const uint4*>(win + win_offset(li));
    uint4 r[V][2];
#pragma unroll
    for (int v = 0; v < VE; ++v) {
        r[v][0] = __ldg(rows + sub_offset<V, ELEM>(lane, v) * 16);
        r[v][1] = __ldg(rows + sub_offset<V, ELEM>(lane, v) * 16 + 1);
    }
    uint2 m[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) m[j] = __ldg(reinterpret_cast<const uint2*>(dstep + (li * 7 + j) * 64) + lane);
    const int c0 = (lane & 3) << 1;
    const uint32_t a0 = c0 == 0 ? s[0] : c0 == 2 ? s[2] : c0 == 4 ? s[4] : s[6];
    const uint32_t a1 = c0 == 0 ? s[1] : c0 == 2 ? s[3] : c0 == 4 ? s[5] : s[7];
    if (lane == 0) {
        reinterpret_cast<uint4*>(scratch)[0] = make_uint4(s[0], s[1], s[2], s[3]);
        reinterpret_cast<uint4*>(scratch)[1] = make_uint4(s[4], s[5], s[6], s[7]);
    }
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        const uint64_t part = (uint64_t)m[j].x * a0 + (uint64_t)m[j].y * a1;  // < 2^63
        uint64_t f = (part & kP) + (part >> 31);                              // < 2^33
        f += __shfl_xor_sync(kFull, f, 1);
        f += __shfl_xor_sync(kFull, f, 2);                                    // < 2^35
        if ((lane & 3) == 0) scratch[(j + 1) * 8 + (lane >> 2)] = mod_p64(f);
    }
#pragma unroll
    for (int v = VE; v < V; ++v) {
        r[v][0] = __ldg(rows + sub_offset<V, ELEM>(lane, v) * 16);
        r[v][1] = __ldg(rows + sub_offset<V, ELEM>(lane, v) * 16 + 1);
    }
    __syncwarp();
    uint32_t* const xs = scratch + 64;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint4 h0 = reinterpret_cast<const uint4*>(scratch + j * 8)[0];
        const uint4 h1 = reinterpret_cast<const uint4*>(scratch + j * 8)[1];
        const uint32_t st[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const uint32_t rv[8] = {r[v][0].x, r[v][0].y, r[v][0].z, r[v][0].w,
                                    r[v][1].x, r[v][1].y, r[v][1].z, r[v][1].w};
            const uint32_t S = dot8_ref(rv, st);  // [1, p], or 0 for residue 0
            xs[(v * 8 + j) * 32 + lane] = LAG_MOD ? lag_mod(S) : lag_minus1(S);
        }
    }
    __syncwarp();
#pragma unroll
    for (int v = 0; v < V; ++v)
#pragma unroll
        for (int j = 0; j < 8; ++j) x[v][j] = xs[(v * 8 + j) * 32 + lane];
    __syncwarp();  // the scratch words are free again
}

// The same window from 8 V rows of the window table per lane (row
// e_0^T A^(o + 1 + d j) against s itself), four rows at a time, through the
// warp's scratch ([slot][lane], 8 V * 32 words).  Four table round trips
// instead of one, but fewer instructions and a lower register peak: the
// batch kernel uses it for launches with more tiles than warps, where the
// setup's latency hides behind other warps' work and the main loop's speed
// counts (10,000 uneven instances: 888 against 876 Goutputs/s).  `scratch`
// holds at least 8 V * 32 words.
template <int V, int ELEM, bool LAG_MOD>
__device__ __forceinline__ void lane_window_rows(const uint32_t* __restrict__ win, const uint32_t s[8], int lane,
                                                 uint32_t* scratch, uint32_t (&x)[V][8]) {
    const uint32_t* w = win + win_offset(layout_index(V));
#pragma unroll 1
    for (int i0 = 0; i0 < 8 * V; i0 += 4) {
        uint4 r[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = i0 + q, v = i >> 3, j = i & 7;
            const uint4* row = reinterpret_cast<const uint4*>(w + (sub_offset<V, ELEM>(lane, v) * 8 + j) * 8);
            r[2 * q] = __ldg(row);
            r[2 * q + 1] = __ldg(row + 1);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 r0 = r[2 * q], r1 = r[2 * q + 1];
            const uint32_t rv[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            const uint32_t S = dot8_ref(rv, s);  // [1, p], or 0 for residue 0
            scratch[(i0 + q) * 32 + lane] = LAG_MOD ? lag_mod(S) : lag_minus1(S);
        }
    }
#pragma unroll
    for (int v = 0; v < V; ++v)
#pragma unroll
        for (int j = 0; j < 8; ++j) x[v][j] = scratch[(v * 8 + j) * 32 + lane];  // the lane's own words
}

}  // namespace mrg8g
