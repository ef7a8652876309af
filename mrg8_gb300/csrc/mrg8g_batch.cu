// mrg8g_batch.cu -- one persistent launch generating many independent
// generator instances (each with its own state, offset, length, output
// buffer and output kind).
//
// The host cuts every instance into tiles (a short unaligned head tile plus
// body tiles of a tuned number of rows), longest instances first.  Resident
// warps pull tile indices from a device counter; each tile jumps the
// instance's state to the tile's first output with the resident A^(2^i)
// table and runs the same warp routine as the bulk kernel (mrg8g_gen.cuh), so
// every instance's values equal its own sequential stream.  This replaces
// one mrg8_cuda::mrg8_outer_32 launch per instance (cuda/mrg8_cuda.cu:414-436).
#include "mrg8g_device.cuh"
#include "mrg8g_gen.cuh"
#include "mrg8g_internal.h"
#include "mrg8g_runtime.h"

namespace mrg8g {

MRG8G_DEFINE_TABLE_UPLOAD(upload_tables_batch)

template <int KIND>
__device__ __forceinline__ void run_tile(const BatchInst& in, const BatchTile& t, const uint32_t s[8],
                                         const BatchArgs& a, uint32_t* scratch) {
    using T = typename OutOf<KIND>::T;
    T* out = static_cast<T*>(in.out) + t.start;
    constexpr int V = sizeof(T) == 8 ? 2 : 4;
    warp_generate<V, KIND>(g_win, s, out, t.len_flags, a.leap[layout_index(V)], scratch);
}

template <int KIND>
__device__ __forceinline__ void run_head(const BatchInst& in, const BatchTile& t, uint32_t s[8]) {
    using T = typename OutOf<KIND>::T;
    lane_sequential<KIND>(g_jump, s, static_cast<T*>(in.out) + t.start, t.len_flags & ~kTileHead);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_batch(const __grid_constant__ BatchArgs a) {
    __shared__ uint32_t scratch[THREADS / 32][8 * 4 * 32];
    const int lane = threadIdx.x & 31;
    uint32_t* sc = scratch[threadIdx.x >> 5];
    for (;;) {
        uint32_t ti = 0;
        if (lane == 0) ti = atomicAdd(a.counter, 1u);
        ti = __shfl_sync(kFull, ti, 0);
        if (ti >= a.ntiles) break;
        const BatchTile t = a.tiles[ti];
        const BatchInst in = a.insts[t.inst];
        const uint32_t* src = in.slot1 ? a.states + 8ull * (in.slot1 - 1) : in.st;
        uint32_t s[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] = src[q];
        warp_jump(g_jump, s, in.offset + t.start);
        if (t.len_flags & kTileHead) {
            if (lane == 0) {
                switch (in.kind) {
                case kU32: run_head<kU32>(in, t, s); break;
                case kF64Orig: run_head<kF64Orig>(in, t, s); break;
                case kF64Shift: run_head<kF64Shift>(in, t, s); break;
                case kF32Orig: run_head<kF32Orig>(in, t, s); break;
                default: run_head<kF32Shift>(in, t, s); break;
                }
            }
            continue;
        }
        switch (in.kind) {
        case kU32: run_tile<kU32>(in, t, s, a, sc); break;
        case kF64Orig: run_tile<kF64Orig>(in, t, s, a, sc); break;
        case kF64Shift: run_tile<kF64Shift>(in, t, s, a, sc); break;
        case kF32Orig: run_tile<kF32Orig>(in, t, s, a, sc); break;
        default: run_tile<kF32Shift>(in, t, s, a, sc); break;
        }
    }
}

cudaError_t launch_batch(const BatchArgs& a, int threads, int blocks, cudaStream_t st) {
    if (threads == 256) k_batch<256><<<blocks, 256, 0, st>>>(a);
    else k_batch<128><<<blocks, 128, 0, st>>>(a);
    return cudaGetLastError();
}

int batch_blocks_per_sm(int threads) {
    int nb = 0;
    cudaError_t e = threads == 256
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<256>, 256, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<128>, 128, 0);
    if (e != cudaSuccess || nb <= 0) return 1;
    return nb;
}

}  // namespace mrg8g
