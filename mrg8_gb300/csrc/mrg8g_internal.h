// mrg8g_internal.h -- launch interfaces between the C ABI and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mrg8g_tables.h"

namespace mrg8g {

constexpr int kPlainThreads = 128;  // 4 warps per block

// One bulk call: n outputs starting at the stream position of `st`.
struct PlainArgs {
    uint32_t st[8];   // state at stream position 0 of the call (raw words)
    uint64_t n;       // outputs
    uint64_t head;    // outputs [0, head) written by one lane (alignment)
    uint64_t tile;    // outputs per warp, a multiple of 32 V
    void* out;        // device pointer to output element 0
    LeapCoef lc;      // decimated recurrence of the layout
};

struct JumpArgs {
    uint32_t st[8];
    const uint64_t* offsets;
    uint32_t* states;
    uint64_t count;
};

// ---- batches of independent instances

// Device copy of one instance (mrg8g_instance of the C ABI).  slot1 = 0: the
// state is st; slot1 = k + 1: the state is row k of the device-resident
// generator table (serving), st unused.
struct BatchInst {
    uint32_t st[8];
    uint64_t offset;
    uint64_t n;
    void* out;
    int32_t kind;
    uint32_t slot1;
};

// One unit of work: outputs [start, start + len) of instance `inst`.  Bit 31
// of len_flags marks an unaligned head (fewer outputs than one vector),
// written sequentially by one lane.
constexpr uint32_t kTileHead = 0x80000000u;
struct BatchTile {
    uint64_t start;
    uint32_t inst;
    uint32_t len_flags;
};

// Tiles are either listed by the host (`tiles`) or, when `tiles` is null,
// derived on the device: instance i owns tiles [tile_base[i], tile_base[i+1])
// of the launch, its head (outputs before the first 16-byte boundary of its
// buffer, if any) and then body tiles of `tile_elems` outputs.
struct BatchArgs {
    const BatchInst* insts;
    const BatchTile* tiles;
    const uint32_t* tile_base;  // ninst + 1 prefix counts, used when tiles is null
    uint32_t ninst;
    uint32_t tile_elems;        // body tile length (a multiple of 32 * kBatchLayoutV)
    uint32_t ntiles;
    uint32_t* counter;        // work-queue position, zero before each launch
    uint32_t* done_blocks;    // null, or blocks finished: the last block then
                              // zeroes *counter and *done_blocks for the next launch
    const uint32_t* states;   // generator table (8 words per slot) or null
    unsigned long long* times;  // null, or [start, end] of the launch in
                                // %globaltimer ns (block 0's start, the last
                                // block's end), written for the serving stats
    LeapCoef leap[2];  // the batch layout's recurrence: [0] lags S - 1, [1] lags S mod p
};

cudaError_t upload_tables_plain();
cudaError_t launch_batch(const BatchArgs& a, int threads, int blocks, cudaStream_t st);
int batch_blocks_per_sm(int threads);
cudaError_t launch_plain(int kind, int V, const PlainArgs& a, int blocks, cudaStream_t st);
int plain_blocks_per_sm(int kind, int V);
cudaError_t launch_convert(int kind, const uint32_t* in, void* out, uint64_t n, int blocks, cudaStream_t st);
cudaError_t launch_jump_states(const JumpArgs& a, int blocks, cudaStream_t st);

}  // namespace mrg8g
