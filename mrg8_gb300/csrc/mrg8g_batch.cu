// mrg8g_batch.cu -- one persistent launch generating many independent
// generator instances (each with its own state, offset, length, output
// buffer and output kind).
//
// The host cuts every instance into tiles (a short unaligned head tile plus
// body tiles of a tuned number of rows), longest instances first.  Resident
// warps pull tile indices from a device counter (or, in a launch with no more
// tiles than warps, take the tile of their own index); each tile jumps the instance's
// state to the tile's first output with the resident byte-window jump table
// and runs the same warp routine as the bulk kernel (mrg8g_gen.cuh), so every
// instance's values equal its own sequential stream.  This replaces one
// mrg8_cuda::mrg8_outer_32 launch per instance (cuda/mrg8_cuda.cu:414-436).
#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/mrg8g.h"
#include "mrg8g_device.cuh"
#include "mrg8g_gen.cuh"
#include "mrg8g_internal.h"
#include "mrg8g_runtime.h"

namespace mrg8g {

MRG8G_DEFINE_TABLE_UPLOAD(upload_tables_batch)

// Tiles shorter than this many outputs (256 rows) form their windows in one
// table round trip even in a launch with more tiles than warps: there the
// setup is a large part of the tile (65,536 tiles of 4,096 outputs: 818
// against 754 Goutputs/s), while long tiles run about 1 % faster with the
// row-table setup.
constexpr uint32_t kQuickSetupElems = 256u * 32u * kBatchLayoutV;

template <int KIND, bool QUICK>
__device__ __forceinline__ void run_tile(const BatchInst& in, const BatchTile& t, const uint32_t s[8],
                                         const BatchArgs& a, uint32_t* scratch) {
    using T = typename OutOf<KIND>::T;
    T* out = static_cast<T*>(in.out) + t.start;
    warp_generate<kBatchLayoutV, KIND>(g_win, g_dstep, s, out, t.len_flags, a.leap[kLagMod<KIND> ? 1 : 0], scratch,
                                       QUICK || t.len_flags < kQuickSetupElems);
}

template <int KIND>
__device__ __forceinline__ void run_head(const BatchInst& in, const BatchTile& t, uint32_t s[8],
                                         const uint32_t* jump) {
    using T = typename OutOf<KIND>::T;
    lane_sequential<KIND>(jump, s, static_cast<T*>(in.out) + t.start, t.len_flags & ~kTileHead);
}

// Instance owning tile ti of a device-tiled launch: the largest i with
// tile_base[i] <= ti, found by a 32-way search (one load per lane per level,
// one level for up to 32 instances).  Called by all 32 lanes with the same ti.
__device__ __forceinline__ uint32_t tile_owner(const uint32_t* __restrict__ base, uint32_t ninst, uint32_t ti) {
    const int lane = threadIdx.x & 31;
    uint32_t lo = 0, hi = ninst;  // base[lo] <= ti < base[hi]
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t c = lo + (uint32_t)lane * step;
        const unsigned m = __ballot_sync(kFull, c < hi && base[c] <= ti);
        lo += (uint32_t)(31 - __clz((int)m)) * step;
        hi = min(hi, lo + step);
    }
    return lo;
}


__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// QUICK: a launch with no more tiles than warps (launch_batch decides), whose
// time is its latency: each warp takes the tile of its own index in the grid
// (no wait on the counter) and forms its window in one table round trip.
// Otherwise warps pull tiles from the counter, and long tiles use the
// row-table window, the faster form when the setup's latency hides behind
// other warps' work (10,000 uneven instances: 888 Goutputs/s against 876
// with the QUICK forms).
template <int THREADS, bool QUICK>
__global__ void __launch_bounds__(THREADS, THREADS == 128 ? 9 : 4) k_batch(const __grid_constant__ BatchArgs a) {
    if (a.times && blockIdx.x == 0 && threadIdx.x == 0) a.times[0] = global_ns();
    __shared__ __align__(16) uint32_t scratch[THREADS / 32][window_scratch(kBatchLayoutV)];
    const int lane = threadIdx.x & 31;
    uint32_t* sc = scratch[threadIdx.x >> 5];
    for (int round = 0;; ++round) {
        uint32_t ti;
        if constexpr (QUICK) {
            if (round) break;
            ti = blockIdx.x * (THREADS / 32) + (threadIdx.x >> 5);
        } else {
            uint32_t q = 0;
            if (lane == 0) q = atomicAdd(a.counter, 1u);
            ti = __shfl_sync(kFull, q, 0);
        }
        if (ti >= a.ntiles) break;
        BatchTile t;
        BatchInst in;
        if (a.tiles) {
            t = a.tiles[ti];
            in = a.insts[t.inst];
        } else {
            const uint32_t i = tile_owner(a.tile_base, a.ninst, ti);
            in = a.insts[i];
            t = derive_tile(ti - a.tile_base[i], in, i, a.tile_elems);
        }
        const uint32_t* src = in.slot1 ? a.states + 8ull * (in.slot1 - 1) : in.st;
        uint32_t s[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] = src[q];
        warp_jump(g_jwin, s, in.offset + t.start);
        if (t.len_flags & kTileHead) {
            if (lane == 0) {
                switch (in.kind) {
                case kU32: run_head<kU32>(in, t, s, g_jwin); break;
                case kF64Orig: run_head<kF64Orig>(in, t, s, g_jwin); break;
                case kF64Shift: run_head<kF64Shift>(in, t, s, g_jwin); break;
                case kF32Orig: run_head<kF32Orig>(in, t, s, g_jwin); break;
                default: run_head<kF32Shift>(in, t, s, g_jwin); break;
                }
            }
            continue;
        }
        switch (in.kind) {
        case kU32: run_tile<kU32, QUICK>(in, t, s, a, sc); break;
        case kF64Orig: run_tile<kF64Orig, QUICK>(in, t, s, a, sc); break;
        case kF64Shift: run_tile<kF64Shift, QUICK>(in, t, s, a, sc); break;
        case kF32Orig: run_tile<kF32Orig, QUICK>(in, t, s, a, sc); break;
        default: run_tile<kF32Shift, QUICK>(in, t, s, a, sc); break;
        }
    }
    // Self-resetting queue: once every block has left the loop, no warp
    // reads the counter again in this launch.
    // Every thread's outputs are made visible device-wide before its block
    // counts itself finished, so that when the last block stamps the end of
    // the launch into host memory, the host may take the outputs as complete.
    if (a.done_blocks) {
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0 && atomicAdd(a.done_blocks, 1u) == gridDim.x - 1) {
            *a.counter = 0;
            *a.done_blocks = 0;
            if (a.times) {
                __threadfence();
                a.times[1] = global_ns();
                __threadfence_system();
            }
        }
    }
}

cudaError_t launch_batch(const BatchArgs& a, int threads, int blocks, cudaStream_t st) {
    const bool quick = (uint64_t)a.ntiles <= (uint64_t)blocks * (uint64_t)(threads / 32);
    if (threads == 256) {
        if (quick) k_batch<256, true><<<blocks, 256, 0, st>>>(a);
        else k_batch<256, false><<<blocks, 256, 0, st>>>(a);
    } else {
        if (quick) k_batch<128, true><<<blocks, 128, 0, st>>>(a);
        else k_batch<128, false><<<blocks, 128, 0, st>>>(a);
    }
    return cudaGetLastError();
}

int batch_blocks_per_sm(int threads) {
    int nb = 0;
    cudaError_t e = threads == 256
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<256, false>, 256, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<128, false>, 128, 0);
    if (e != cudaSuccess || nb <= 0) return 1;
    return nb;
}

}  // namespace mrg8g

// ---------------------------------------------------------------------------
// Allocation-free batch entry point (mrg8g_batch_generate_noalloc).
//
// Some callers of this library may not allocate device memory themselves:
// plugins whose host application (or a framework's caching allocator) owns
// all of the GPU's memory, and latency-critical loops that cannot afford the
// device-wide synchronisation and unpredictable cost of cudaMalloc/cudaFree.
// For them the batch path runs from a fixed scratch area that lives in this
// module as a file-scope device array: the counter of the work queue, the
// instance descriptors and the tiles.  Every GPU that loads the library holds
// this array (about 1.3 MB) until the process exits.
//
// Layout: [0, 256) work counter | instances (64 B each) | tiles (16 B each).
namespace mrg8g {
namespace {

constexpr size_t kNoAllocInstOff = 256;
constexpr size_t kNoAllocTileOff = kNoAllocInstOff + (size_t)MRG8G_NOALLOC_MAX_INSTANCES * sizeof(BatchInst);
constexpr size_t kNoAllocBytes = kNoAllocTileOff + (size_t)MRG8G_NOALLOC_MAX_TILES * sizeof(BatchTile);
static_assert(sizeof(BatchInst) == 64 && sizeof(BatchTile) == 16, "descriptor layout");
constexpr int kNoAllocTileRows = 512;
constexpr int kMaxDevices = 64;

}  // namespace
}  // namespace mrg8g

static __device__ __align__(256) unsigned char g_noalloc_scratch[mrg8g::kNoAllocBytes];

namespace mrg8g {
namespace {

// Host staging laid out like the device array (one copy per call).
alignas(256) unsigned char g_noalloc_host[kNoAllocBytes];
std::mutex g_noalloc_mu;
void* g_noalloc_dev[kMaxDevices];

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the host-side name is only a stand-in, never a device address).
int noalloc_scratch(int dev, void** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(MRG8G_ERR_INVALID_ARGUMENT, "device %d out of range", dev);
    if (!g_noalloc_dev[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_dev[dev] = p;
    }
    *out = g_noalloc_dev[dev];
    return MRG8G_SUCCESS;
}

// Tiles written straight into the staging area (no heap), cut as every plan
// cuts them (mrg8g_tiles.h); the largest-first order of make_tiles by an
// in-place sort.
int noalloc_tiles(const BatchInst* insts, uint32_t count, BatchTile* tiles, uint32_t* ntiles) {
    uint32_t k = 0;
    const uint64_t T = (uint64_t)kNoAllocTileRows * 32 * (uint64_t)kBatchLayoutV;
    for (uint32_t i = 0; i < count; ++i) {
        const uint64_t m = instance_tiles(insts[i], T);
        if ((uint64_t)k + m > MRG8G_NOALLOC_MAX_TILES)
            return fail(MRG8G_ERR_BUDGET, "batch needs more than %d tiles (the no-alloc limit)", MRG8G_NOALLOC_MAX_TILES);
        for (uint64_t li = 0; li < m; ++li) tiles[k++] = derive_tile((uint32_t)li, insts[i], i, (uint32_t)T);
    }
    std::sort(tiles, tiles + k, [&](const BatchTile& x, const BatchTile& y) {
        const uint64_t bx = (uint64_t)(x.len_flags & ~kTileHead) * kind_elem_bytes(insts[x.inst].kind);
        const uint64_t by = (uint64_t)(y.len_flags & ~kTileHead) * kind_elem_bytes(insts[y.inst].kind);
        return bx != by ? bx > by : (x.inst != y.inst ? x.inst < y.inst : x.start < y.start);
    });
    *ntiles = k;
    return MRG8G_SUCCESS;
}

}  // namespace
}  // namespace mrg8g

extern "C" int mrg8g_batch_generate_noalloc(const mrg8g_instance* inst, uint64_t count, void* stream) {
    using namespace mrg8g;
    if (count && !inst) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null instance array");
    if (count > MRG8G_NOALLOC_MAX_INSTANCES)
        return fail(MRG8G_ERR_BUDGET, "%llu instances exceed the no-alloc limit of %d", (unsigned long long)count,
                    MRG8G_NOALLOC_MAX_INSTANCES);
    // A stream that is capturing would record the descriptor copy below as a
    // graph node reading g_noalloc_host at replay time, after later calls have
    // rewritten it; such calls are refused before anything is enqueued.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t qe = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
    if (qe != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(qe, "cudaStreamIsCapturing");
    }
    if (cap != cudaStreamCaptureStatusNone)
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "the no-alloc batch cannot be enqueued on a stream that is capturing");
    int dev = 0;
    int rc = ensure_device(&dev, nullptr);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    void* scratch = nullptr;
    if ((rc = noalloc_scratch(dev, &scratch))) return rc;
    BatchInst* h_insts = reinterpret_cast<BatchInst*>(g_noalloc_host + kNoAllocInstOff);
    BatchTile* h_tiles = reinterpret_cast<BatchTile*>(g_noalloc_host + kNoAllocTileOff);
    for (uint64_t i = 0; i < count; ++i) {
        const mrg8g_instance& s = inst[i];
        if (!kind_valid(s.kind))
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "instance %llu: unknown kind %d", (unsigned long long)i, s.kind);
        if ((rc = validate_state(s.state))) return rc;
        const int elem = kind_elem_bytes(s.kind);
        if (s.n && (!s.out || (uintptr_t)s.out % elem))
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "instance %llu: null or misaligned output", (unsigned long long)i);
        if (s.n > (1ull << 62) || s.offset > ~0ull - s.n)
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "instance %llu: offset + n overflows", (unsigned long long)i);
        BatchInst& d = h_insts[i];
        std::memcpy(d.st, s.state, sizeof(d.st));
        d.offset = s.offset;
        d.n = s.n;
        d.out = s.out;
        d.kind = s.kind;
        d.slot1 = 0;
    }
    uint32_t ntiles = 0;
    if ((rc = noalloc_tiles(h_insts, (uint32_t)count, h_tiles, &ntiles))) return rc;
    if (ntiles == 0) return MRG8G_SUCCESS;
    // The work counter must start at zero; the array keeps the last call's
    // contents, so the copy below rewrites it together with the descriptors.
    std::memset(g_noalloc_host, 0, kNoAllocInstOff);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* d = static_cast<unsigned char*>(scratch);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d, g_noalloc_host, kNoAllocInstOff + count * sizeof(BatchInst), cudaMemcpyHostToDevice,
                             st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + kNoAllocTileOff, g_noalloc_host + kNoAllocTileOff, ntiles * sizeof(BatchTile),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(e, "copy of the no-alloc descriptors");
    BatchArgs a;
    a.insts = reinterpret_cast<const BatchInst*>(d + kNoAllocInstOff);
    a.tiles = reinterpret_cast<const BatchTile*>(d + kNoAllocTileOff);
    a.ntiles = ntiles;
    a.counter = reinterpret_cast<uint32_t*>(d);
    a.done_blocks = nullptr;
    a.tile_base = nullptr;
    a.ninst = count;
    a.tile_elems = 0;
    a.states = nullptr;
    a.times = nullptr;
    set_batch_leaps(a);
    const int sms = device_sms();
    const uint64_t want = (ntiles + 3) / 4;
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * batch_blocks_per_sm(128), want));
    if ((e = launch_batch(a, 128, blocks, st)) != cudaSuccess) return cuda_fail(e, "launching the no-alloc batch");
    return MRG8G_SUCCESS;
}
