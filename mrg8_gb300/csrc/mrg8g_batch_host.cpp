// mrg8g_batch_host.cpp -- batches of independent generator instances: the
// plan (tiles, device descriptors, work-queue counter), its CUDA-graph
// launch and its autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <exception>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mrg8g.h"
#include "mrg8g_internal.h"
#include "mrg8g_runtime.h"
#include "mrg8g_tables.h"

using namespace mrg8g;


struct mrg8g_batch {
    int dev = -1;
    std::vector<BatchInst> insts;
    std::vector<BatchTile> tiles;
    uint64_t outputs = 0, bytes = 0;
    mrg8g_batch_config cfg{};
    int blocks = 0;
    BatchInst* d_insts = nullptr;
    BatchTile* d_tiles = nullptr;
    uint32_t* d_counter = nullptr;
    size_t d_tiles_cap = 0;
    uint32_t* d_base = nullptr;    // tile prefix counts (derived tiling)
    bool d_insts_sorted = false;   // d_insts holds the longest-first order
    bool planned = false;
    uint64_t ntiles = 0;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    // Recorded after every launch outside a stream capture: a re-plan waits
    // for it before it rewrites the descriptors or drops the graph, which a
    // launch on the caller's (possibly non-blocking) stream may still read.
    cudaEvent_t last = nullptr;
};

namespace {

constexpr int kDefaultTileRows = 512;
// Host-listed tiles are 16 bytes each on the host and the device; above this
// many a plan must use the derived tiling (O(instances) descriptors).
constexpr uint64_t kMaxListedTiles = 1ull << 26;

void release_graph(mrg8g_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

int normalise(mrg8g_batch_config& c) {
    if (c.tile_rows == 0) c.tile_rows = kDefaultTileRows;
    if (c.threads == 0) c.threads = 128;
    if (c.tile_rows < 8 || c.tile_rows > (1 << 20) || (c.tile_rows & 7))
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "tile_rows must be a multiple of 8 in [8, 2^20]");
    if (c.threads != 128 && c.threads != 256) return fail(MRG8G_ERR_INVALID_ARGUMENT, "threads must be 128 or 256");
    if (c.blocks_per_sm < 0) return fail(MRG8G_ERR_INVALID_ARGUMENT, "negative blocks_per_sm");
    if (c.use_graph < 0 || c.use_graph > 1) return fail(MRG8G_ERR_INVALID_ARGUMENT, "use_graph must be 0 or 1");
    if (c.tiling < 0 || c.tiling > 1) return fail(MRG8G_ERR_INVALID_ARGUMENT, "tiling must be 0 or 1");
    return MRG8G_SUCCESS;
}

int upload_insts(mrg8g_batch* b, const BatchInst* src, bool sorted) {
    cudaError_t e;
    if (!b->insts.empty() &&
        (e = copy_to_device(b->d_insts, src, b->insts.size() * sizeof(BatchInst))) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(instances)");
    b->d_insts_sorted = sorted;
    return MRG8G_SUCCESS;
}

// Derived tiling: instances longest first in d_insts, prefix counts in d_base.
int plan_derived(mrg8g_batch* b) {
    const uint32_t count = (uint32_t)b->insts.size();
    std::vector<BatchInst> sorted(b->insts);
    sort_largest_first(sorted.data(), count);
    std::vector<uint32_t> base(count + 1);
    const uint64_t total = tile_prefix(sorted.data(), count, (uint64_t)b->cfg.tile_rows * 32 * kBatchLayoutV, base.data());
    if (total > 0xFFFFFFFFull) return fail(MRG8G_ERR_INVALID_ARGUMENT, "more than 2^32-1 tiles; raise tile_rows");
    cudaError_t e;
    if (!b->d_base && (e = cudaMalloc(&b->d_base, base.size() * sizeof(uint32_t))) != cudaSuccess)
        return cuda_fail(e, "cudaMalloc(tile counts)");
    if ((e = copy_to_device(b->d_base, base.data(), base.size() * sizeof(uint32_t))) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(tile counts)");
    int rc = upload_insts(b, sorted.data(), true);
    if (rc) return rc;
    b->tiles.clear();
    b->ntiles = total;
    return MRG8G_SUCCESS;
}

void build_tiles(mrg8g_batch* b) {
    make_tiles(b->insts.data(), (uint32_t)b->insts.size(), (uint64_t)b->cfg.tile_rows * 32 * kBatchLayoutV, b->tiles);
}

int upload_tiles(mrg8g_batch* b) {
    cudaError_t e;
    const size_t need = std::max<size_t>(b->tiles.size(), 1) * sizeof(BatchTile);
    if (need > b->d_tiles_cap) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->d_tiles = nullptr;
        if ((e = cudaMalloc(&b->d_tiles, need)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(tiles)");
        b->d_tiles_cap = need;
    }
    if (!b->tiles.empty() &&
        (e = copy_to_device(b->d_tiles, b->tiles.data(), b->tiles.size() * sizeof(BatchTile))) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(tiles)");
    return MRG8G_SUCCESS;
}

// Validates c completely before changing the plan: a configuration that is
// refused leaves the previous plan and configuration in place.
int apply_config(mrg8g_batch* b, const mrg8g_batch_config& c) {
    mrg8g_batch_config n = c;
    int rc = normalise(n);
    if (rc) return rc;
    if (b->last) {
        const cudaError_t e = cudaEventSynchronize(b->last);
        if (e != cudaSuccess) return cuda_fail(e, "waiting for the plan's last launch");
    }
    const bool retile = n.tile_rows != b->cfg.tile_rows || n.tiling != b->cfg.tiling || !b->planned;
    if (retile) {
        const uint64_t total =
            count_tiles(b->insts.data(), (uint32_t)b->insts.size(), (uint64_t)n.tile_rows * 32 * kBatchLayoutV);
        if (total > 0xFFFFFFFFull)
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "%llu tiles: more than 2^32-1; raise tile_rows",
                        (unsigned long long)total);
        if (!n.tiling && total > kMaxListedTiles)
            return fail(MRG8G_ERR_INVALID_ARGUMENT,
                        "%llu tiles exceed the %llu of a host-listed plan; use tiling = 1 or more tile_rows",
                        (unsigned long long)total, (unsigned long long)kMaxListedTiles);
    }
    b->cfg = n;
    if (retile) {
        b->planned = false;
        if (n.tiling) {
            if ((rc = plan_derived(b))) return rc;
        } else {
            build_tiles(b);
            if ((rc = upload_tiles(b))) return rc;
            if (b->d_insts_sorted && (rc = upload_insts(b, b->insts.data(), false))) return rc;
            if (b->tiles.size() > 0xFFFFFFFFull)
                return fail(MRG8G_ERR_INVALID_ARGUMENT, "more than 2^32-1 tiles; raise tile_rows");
            b->ntiles = b->tiles.size();
        }
        b->planned = true;
    }
    const int sms = device_sms();
    if (!sms) return MRG8G_ERR_CUDA;
    int bps = batch_blocks_per_sm(n.threads);
    if (n.blocks_per_sm > 0 && n.blocks_per_sm < bps) bps = n.blocks_per_sm;
    const uint64_t wpb = (uint64_t)n.threads / 32;
    const uint64_t want = (b->ntiles + wpb - 1) / wpb;
    b->blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * bps, want));
    release_graph(b);
    return MRG8G_SUCCESS;
}

BatchArgs args_of(const mrg8g_batch* b) {
    BatchArgs a;
    a.insts = b->d_insts;
    a.tiles = b->cfg.tiling ? nullptr : b->d_tiles;
    a.ntiles = (uint32_t)b->ntiles;
    a.counter = b->d_counter;
    a.done_blocks = nullptr;
    a.tile_base = b->cfg.tiling ? b->d_base : nullptr;
    a.ninst = (uint32_t)b->insts.size();
    a.tile_elems = (uint32_t)((uint64_t)b->cfg.tile_rows * 32 * kBatchLayoutV);
    a.states = nullptr;
    a.times = nullptr;
    set_batch_leaps(a);
    return a;
}

// Counter reset + persistent kernel, on stream s.
int enqueue(mrg8g_batch* b, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(counter)");
    e = launch_batch(args_of(b), b->cfg.threads, b->blocks, s);
    if (e != cudaSuccess) return cuda_fail(e, "launching the batch kernel");
    return MRG8G_SUCCESS;
}

int build_graph(mrg8g_batch* b) {
    cudaError_t e;
    if (!b->cap && (e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamCreate(capture)");
    if ((e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamBeginCapture");
    int rc = enqueue(b, b->cap);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->cap, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return MRG8G_SUCCESS;
}

void destroy_plan(mrg8g_batch* b) {
    if (b->last) cudaEventSynchronize(b->last), cudaEventDestroy(b->last);
    release_graph(b);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->d_insts) cudaFree(b->d_insts);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->d_counter) cudaFree(b->d_counter);
    if (b->d_base) cudaFree(b->d_base);
    delete b;
}

}  // namespace

// Host allocation failures inside the planners come back as status codes
// (no exception crosses the C ABI).
template <class F>
static int guarded(F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(MRG8G_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(MRG8G_ERR_INVALID_STATE, "%s", e.what());
    }
}

static int batch_create(const mrg8g_instance* inst, uint64_t count, const mrg8g_batch_config* cfg,
                        mrg8g_batch** out) {
    if (!out) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (count && !inst) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null instance array");
    if (count > 0xFFFFFFFFull) return fail(MRG8G_ERR_INVALID_ARGUMENT, "at most 2^32-1 instances");
    int dev = 0;
    int rc = ensure_device(&dev, nullptr);
    if (rc) return rc;
    mrg8g_batch* b = new (std::nothrow) mrg8g_batch;
    if (!b) return fail(MRG8G_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->dev = dev;
    b->insts.resize(count);
    for (uint64_t i = 0; i < count; ++i) {
        const mrg8g_instance& s = inst[i];
        if (!kind_valid(s.kind)) {
            delete b;
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "instance %llu: unknown kind %d", (unsigned long long)i, s.kind);
        }
        if ((rc = validate_state(s.state))) {
            delete b;
            return rc;
        }
        const int elem = kind_elem_bytes(s.kind);
        if (s.n && (!s.out || (uintptr_t)s.out % elem)) {
            delete b;
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "instance %llu: null or misaligned output",
                        (unsigned long long)i);
        }
        if (s.n > (1ull << 62) || s.offset > ~0ull - s.n) {
            delete b;
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "instance %llu: offset + n overflows", (unsigned long long)i);
        }
        BatchInst& d = b->insts[i];
        std::memcpy(d.st, s.state, sizeof(d.st));
        d.offset = s.offset;
        d.n = s.n;
        d.out = s.out;
        d.kind = s.kind;
        d.slot1 = 0;
        b->outputs += s.n;
        b->bytes += s.n * elem;
    }
    cudaError_t e;
    if ((e = cudaMalloc(&b->d_insts, std::max<size_t>(count, 1) * sizeof(BatchInst))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_counter, sizeof(uint32_t))) != cudaSuccess) {
        destroy_plan(b);
        return cuda_fail(e, "cudaMalloc(batch)");
    }
    if (count && (e = copy_to_device(b->d_insts, b->insts.data(), count * sizeof(BatchInst))) != cudaSuccess) {
        destroy_plan(b);
        return cuda_fail(e, "cudaMemcpy(instances)");
    }
    mrg8g_batch_config c{};
    if (cfg) c = *cfg;
    else c.use_graph = 1;
    if ((rc = apply_config(b, c))) {
        destroy_plan(b);
        return rc;
    }
    *out = b;
    return MRG8G_SUCCESS;
}


static int batch_autotune(mrg8g_batch* b, void* stream, mrg8g_batch_config* chosen) {
    if (!b) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null batch");
    if (!b->ntiles) {
        if (chosen) *chosen = b->cfg;
        return MRG8G_SUCCESS;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess)
        return cuda_fail(e, "cudaEventCreate");
    const int use_graph = b->cfg.use_graph;
    const int rows[] = {128, 256, 512, 1024, 2048};
    const int threads[] = {128, 256};
    float best_ms = 1e30f;
    mrg8g_batch_config best = b->cfg;
    int rc = MRG8G_SUCCESS;
    for (int r : rows) {
        for (int t : threads) {
          for (int tiling = 0; tiling < 2; ++tiling) {
            mrg8g_batch_config c{r, t, 0, use_graph, tiling};
            if ((rc = apply_config(b, c))) {
                if (rc == MRG8G_ERR_INVALID_ARGUMENT) {  // too many tiles for this shape
                    rc = MRG8G_SUCCESS;
                    continue;
                }
                break;
            }
            if ((rc = mrg8g_batch_launch(b, s))) break;  // warm-up (and graph build)
            cudaEventRecord(e0, s);
            for (int k = 0; k < 3 && !rc; ++k) rc = mrg8g_batch_launch(b, s);
            cudaEventRecord(e1, s);
            if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
                rc = cuda_fail(e, "cudaEventSynchronize");
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) best_ms = ms, best = c;
          }
          if (rc) break;
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = apply_config(b, best))) return rc;
    if (chosen) *chosen = best;
    return MRG8G_SUCCESS;
}


extern "C" {

int mrg8g_batch_create(const mrg8g_instance* inst, uint64_t count, const mrg8g_batch_config* cfg,
                       mrg8g_batch** out) {
    return guarded([&] { return batch_create(inst, count, cfg, out); });
}

int mrg8g_batch_launch(mrg8g_batch* b, void* stream) {
    if (!b) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null batch");
    if (!b->planned) return fail(MRG8G_ERR_INVALID_STATE, "the batch has no valid plan (a re-plan failed)");
    if (!b->ntiles) return MRG8G_SUCCESS;
    cudaStream_t s = (cudaStream_t)stream;
    int rc;
    if (!b->cfg.use_graph) {
        if ((rc = enqueue(b, s))) return rc;
    } else {
        if (!b->exec && (rc = build_graph(b))) return rc;
        cudaError_t e = cudaGraphLaunch(b->exec, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cs);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone) return MRG8G_SUCCESS;  // captured: no real record to wait for
    if (!b->last && (e = cudaEventCreateWithFlags(&b->last, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(e, "cudaEventCreate");
    if ((e = cudaEventRecord(b->last, s)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    return MRG8G_SUCCESS;
}

int mrg8g_batch_get_config(const mrg8g_batch* b, mrg8g_batch_config* cfg) {
    if (!b || !cfg) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    *cfg = b->cfg;
    return MRG8G_SUCCESS;
}

int mrg8g_batch_set_config(mrg8g_batch* b, const mrg8g_batch_config* cfg) {
    if (!b || !cfg) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    return guarded([&] { return apply_config(b, *cfg); });
}

int mrg8g_batch_stats(const mrg8g_batch* b, uint64_t* tiles, uint64_t* outputs, uint64_t* bytes) {
    if (!b) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null batch");
    if (tiles) *tiles = b->ntiles;
    if (outputs) *outputs = b->outputs;
    if (bytes) *bytes = b->bytes;
    return MRG8G_SUCCESS;
}

int mrg8g_batch_autotune(mrg8g_batch* b, void* stream, mrg8g_batch_config* chosen) {
    return guarded([&] { return batch_autotune(b, stream, chosen); });
}

int mrg8g_generate_each(const mrg8g_instance* inst, uint64_t count, void* stream) {
    if (count && !inst) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null instance array");
    for (uint64_t i = 0; i < count; ++i) {
        int rc = mrg8g_generate_from_state(inst[i].state, inst[i].offset, inst[i].out, inst[i].n, inst[i].kind, stream);
        if (rc) return rc;
    }
    return MRG8G_SUCCESS;
}

int mrg8g_batch_destroy(mrg8g_batch* b) {
    if (!b) return MRG8G_SUCCESS;
    destroy_plan(b);
    return MRG8G_SUCCESS;
}

}  // extern "C"
