// mrg8g_gen.cuh -- the warp-level generation routine shared by the bulk
// kernel (mrg8g_plain.cu) and the batch kernel (mrg8g_batch.cu).
//
// A warp that holds the stream state s at output position B (lane-uniform)
// writes the `len` outputs B .. B+len-1 to out[0 .. len): lane l owns the V
// interleaved decimated substreams at positions B + V l + v + 32 V j, whose
// first eight values come from the window tables and whose later values come
// from the order-8 decimated recurrence (8 multiply-adds per output, no
// communication), and row j of the warp is one contiguous 32 V-element run
// written with 16-byte vector stores.
#pragma once
#include "mrg8g_device.cuh"

namespace mrg8g {

// One row of every substream of the lane.  The oldest lag is accumulated
// first so that only the last multiply-add waits for the previous row.
// ALU_TAIL selects reduce_acc_alu (4-byte outputs) over reduce_acc.
template <int V, bool ALU_TAIL>
__device__ __forceinline__ void leap_row(uint32_t (&x)[V][8], int u, const LeapCoef& lc) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
        uint64_t acc = lc.K1;
#pragma unroll
        for (int k = 8; k >= 1; --k) acc = mad_wide_s32(lc.c[k - 1], x[v][(u - k) & 7], acc);
        x[v][u] = ALU_TAIL ? reduce_acc_alu(acc) : reduce_acc(acc);
    }
}

// Store slot u of every substream of the lane at p, the lane's first output
// of the row (the others follow sub_offset).
template <int V, int KIND>
__device__ __forceinline__ void store_vec(typename OutOf<KIND>::T* p, const uint32_t (&x)[V][8], int u) {
    using T = typename OutOf<KIND>::T;
    if constexpr (sizeof(T) == 8) {
        if constexpr (V == 1) {
            p[0] = convert<KIND>(x[0][u]);
        } else {
            // pairs at p + 64 h / 2 (sub_offset: each store covers 512 contiguous bytes)
#pragma unroll
            for (int h = 0; h < V; h += 2)
                *reinterpret_cast<ulonglong2*>(p + 32 * h) =
                    make_ulonglong2(convert<KIND>(x[h][u]), convert<KIND>(x[h + 1][u]));
        }
    } else {
        if constexpr (V == 1) {
            p[0] = convert<KIND>(x[0][u]);
        } else if constexpr (V == 2) {
            *reinterpret_cast<uint2*>(p) = make_uint2(convert<KIND>(x[0][u]), convert<KIND>(x[1][u]));
        } else {
            *reinterpret_cast<uint4*>(p) = make_uint4(convert<KIND>(x[0][u]), convert<KIND>(x[1][u]),
                                                      convert<KIND>(x[2][u]), convert<KIND>(x[3][u]));
        }
    }
}

// Row `row` of the run, checked element by element against its length.
template <int V, int KIND>
__device__ __forceinline__ void store_checked(typename OutOf<KIND>::T* p, const uint32_t (&x)[V][8], int u,
                                              uint64_t row, uint64_t full, uint64_t len, uint32_t lane) {
    using T = typename OutOf<KIND>::T;
    constexpr uint32_t D = 32 * V;
    if (row < full) {
        store_vec<V, KIND>(p + row * D, x, u);
    } else {
        const uint32_t base = sub_offset<V, sizeof(T)>(lane, 0);
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const uint32_t o = sub_offset<V, sizeof(T)>(lane, v);
            if (row * D + o < len) p[row * D + (o - base)] = convert<KIND>(x[v][u]);
        }
    }
}

// The run of `len` outputs from state s (see the file comment).  `out` must
// be 16-byte aligned when V > 1; `scratch` is the warp's window_scratch(V)
// words of shared memory (16-byte aligned).  quick_setup (lane-uniform) picks
// the window setup of one table round trip (lane_window) over the row-table
// form (lane_window_rows).
template <int V, int KIND>
__device__ __forceinline__ void warp_generate(const uint32_t* __restrict__ win, const uint32_t* __restrict__ dstep,
                                              const uint32_t s[8], typename OutOf<KIND>::T* out, uint64_t len,
                                              const LeapCoef& lc, uint32_t* scratch, bool quick_setup = true) {
    using T = typename OutOf<KIND>::T;
    constexpr uint32_t D = 32 * V;
    constexpr bool kAluTail = sizeof(T) == 4;
    const int lane = threadIdx.x & 31;
    uint32_t x[V][8];
    if (quick_setup) lane_window<V, sizeof(T), kLagMod<KIND>>(win, dstep, s, lane, scratch, x);
    else lane_window_rows<V, sizeof(T), kLagMod<KIND>>(win, s, lane, scratch, x);

    const uint64_t rows = (len + D - 1) / D, full = len / D;
    T* const p = out + sub_offset<V, sizeof(T)>((uint32_t)lane, 0);

#pragma unroll
    for (int u = 0; u < 8; ++u)
        if ((uint64_t)u < rows) store_checked<V, KIND>(p, x, u, (uint64_t)u, full, len, (uint32_t)lane);

    uint64_t m = 8;
    for (; m + 8 <= full; m += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            leap_row<V, kAluTail>(x, u, lc);
            store_vec<V, KIND>(p + (m + u) * D, x, u);
        }
    }
    if (m < rows) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            leap_row<V, kAluTail>(x, u, lc);
            if (m + u < rows) store_checked<V, KIND>(p, x, u, m + u, full, len, (uint32_t)lane);
        }
    }
}

// `count` (< V in practice) outputs from state s, one lane, sequentially;
// the state is advanced.  Used for unaligned heads.
template <int KIND>
__device__ __forceinline__ void lane_sequential(const uint32_t* __restrict__ coef, uint32_t st[8],
                                                typename OutOf<KIND>::T* out, uint64_t count) {
    for (uint64_t i = 0; i < count; ++i) {
        const uint32_t S = dot8_ref(coef, st);
#pragma unroll
        for (int q = 7; q > 0; --q) st[q] = st[q - 1];
        st[0] = S;
        out[i] = convert<KIND>(lag_of<KIND>(S));
    }
}

}  // namespace mrg8g
