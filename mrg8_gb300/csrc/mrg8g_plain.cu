// mrg8g_plain.cu -- the single-stream bulk generator for sm_103a and its
// small companions (device jump of many offsets, integer -> uniform
// conversion).
//
// Replaces rng_outer_32 / rng_inner of cuda/mrg8_cuda.cu:201-399.  Layout of
// the work: the call's n outputs (stream positions 0..n-1 after the handle's
// current state) are cut into one contiguous tile per warp.  A warp jumps its
// state to the tile start with the resident byte-window jump table, then lane l owns V
// interleaved decimated substreams (positions B + V l + v + 32 V j); each is
// an order-8 recurrence of its own (coefficients of the characteristic
// polynomial of A^(32V)), so a lane needs 8 multiply-adds per output, no
// shuffles and no shared memory after its setup, and every row j of the warp is one
// contiguous 32 V-element run written with 16-byte vector stores.
#include "mrg8g_device.cuh"
#include "mrg8g_gen.cuh"
#include "mrg8g_internal.h"

namespace mrg8g {

MRG8G_DEFINE_TABLE_UPLOAD(upload_tables_plain)

// Resident blocks the register allocation must allow: eight for 4-byte
// outputs with four substreams per lane (64 registers); nine for fp64
// ORIGINAL with two (56 registers instead of 64: 718 against 710
// Goutputs/s); else no bound (fp64 SHIFTED measured 791 Goutputs/s
// unbounded, 56 registers, and 772 when held to 48 for ten blocks per SM).
template <int V, int KIND>
constexpr int plain_min_blocks() {
    return (V == 4 && sizeof(typename OutOf<KIND>::T) == 4) ? 8 : (V == 2 && KIND == kF64Orig) ? 9 : 1;
}

template <int V, int KIND>
__global__ void __launch_bounds__(kPlainThreads, plain_min_blocks<V, KIND>())
    k_plain(const __grid_constant__ PlainArgs a) {
    using T = typename OutOf<KIND>::T;
    __shared__ __align__(16) uint32_t scratch[kPlainThreads / 32][window_scratch(V)];
    T* const out = static_cast<T*>(a.out);
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;

    // Unaligned head: the first `head` (< V) outputs, one lane, sequential.
    if (warp == 0 && lane == 0 && a.head) {
        uint32_t st[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) st[q] = a.st[q];
        lane_sequential<KIND>(g_jwin, st, out, a.head);  // row 0 of A = coefficients
    }

    const uint64_t B = a.head + warp * a.tile;
    if (B >= a.n) return;
    uint32_t s[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) s[q] = a.st[q];
    warp_jump(g_jwin, s, B);
    warp_generate<V, KIND>(g_win, g_dstep, s, out + B, min(a.tile, a.n - B), a.lc, scratch[threadIdx.x >> 5]);
}

// Uniforms from raw stream integers S in [1, p] (grid-stride).
template <int KIND>
__global__ void k_convert(const uint32_t* __restrict__ in, typename OutOf<KIND>::T* __restrict__ out,
                          uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = convert<KIND>(lag_of<KIND>(in[i]));
}

// states[8 i .. 8 i + 7] = A^offsets[i] st, one warp per offset.  Offsets
// below 8 step sequentially (raw words shift through unchanged, as in the
// reference); larger ones jump and come back as representatives in [1, p].
__global__ void __launch_bounds__(kPlainThreads)
    k_jump_states(const __grid_constant__ JumpArgs a) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < a.count; w += nwarps) {
        const uint64_t k = a.offsets[w];
        uint32_t s[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] = a.st[q];
        if (k < 8) {
            if (lane == 0) {
                for (uint64_t i = 0; i < k; ++i) {
                    const uint32_t S = dot8_ref(g_jwin, s);  // row 0 of A
#pragma unroll
                    for (int q = 7; q > 0; --q) s[q] = s[q - 1];
                    s[0] = S;
                }
            }
        } else {
            warp_jump(g_jwin, s, k);
#pragma unroll
            for (int q = 0; q < 8; ++q) s[q] = rep1p(s[q]);
        }
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < 8; ++q) a.states[w * 8 + q] = s[q];
        }
    }
}

// ------------------------------------------------------------- launchers

template <int V, int KIND>
static cudaError_t launch_plain_t(const PlainArgs& a, int blocks, cudaStream_t st) {
    k_plain<V, KIND><<<blocks, kPlainThreads, 0, st>>>(a);
    return cudaGetLastError();
}

template <int V, int KIND>
static int occupancy_t() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_plain<V, KIND>, kPlainThreads, 0) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}

#define MRG8G_KIND_SWITCH(V, FN, ...)                       \
    switch (kind) {                                         \
    case kU32: return FN<V, kU32>(__VA_ARGS__);             \
    case kF64Orig: return FN<V, kF64Orig>(__VA_ARGS__);     \
    case kF64Shift: return FN<V, kF64Shift>(__VA_ARGS__);   \
    case kF32Orig: return FN<V, kF32Orig>(__VA_ARGS__);     \
    default: return FN<V, kF32Shift>(__VA_ARGS__);          \
    }

cudaError_t launch_plain(int kind, int V, const PlainArgs& a, int blocks, cudaStream_t st) {
    if (V == 1) { MRG8G_KIND_SWITCH(1, launch_plain_t, a, blocks, st) }
    if (V == 2) { MRG8G_KIND_SWITCH(2, launch_plain_t, a, blocks, st) }
    MRG8G_KIND_SWITCH(4, launch_plain_t, a, blocks, st)
}

int plain_blocks_per_sm(int kind, int V) {
    if (V == 1) { MRG8G_KIND_SWITCH(1, occupancy_t) }
    if (V == 2) { MRG8G_KIND_SWITCH(2, occupancy_t) }
    MRG8G_KIND_SWITCH(4, occupancy_t)
}

cudaError_t launch_convert(int kind, const uint32_t* in, void* out, uint64_t n, int blocks, cudaStream_t st) {
    switch (kind) {
    case kF64Orig: k_convert<kF64Orig><<<blocks, 256, 0, st>>>(in, (uint64_t*)out, n); break;
    case kF64Shift: k_convert<kF64Shift><<<blocks, 256, 0, st>>>(in, (uint64_t*)out, n); break;
    case kF32Orig: k_convert<kF32Orig><<<blocks, 256, 0, st>>>(in, (uint32_t*)out, n); break;
    case kF32Shift: k_convert<kF32Shift><<<blocks, 256, 0, st>>>(in, (uint32_t*)out, n); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_jump_states(const JumpArgs& a, int blocks, cudaStream_t st) {
    k_jump_states<<<blocks, kPlainThreads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace mrg8g
