// mrg8g_capi.cpp -- the C ABI of include/mrg8g.h: generator handles, host
// state bookkeeping, launch planning and the host-buffer pipeline.
#include "../../include/mrg8g.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mrg8g_arith.cuh"
#include "mrg8g_internal.h"
#include "mrg8g_runtime.h"
#include "mrg8g_tables.h"

using namespace mrg8g;

struct mrg8g_generator {
    uint32_t st[8];
    // Device staging of the host-buffer path (allocated on first use).
    int stage_dev = -1;
    void* stage[2] = {nullptr, nullptr};
    cudaStream_t sstream[2] = {nullptr, nullptr};
};

// ------------------------------------------------------------ error state

static thread_local std::string t_err;

namespace mrg8g {

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MRG8G_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// ------------------------------------------------------- per-device setup

struct DeviceInfo {
    bool ready = false;
    int sms = 0;
    int bps[5][3] = {};  // blocks per SM of the plain kernel, per kind and layout
};

static std::mutex g_mu;
static std::vector<DeviceInfo> g_dev;

int ensure_device(int* dev_out, const DeviceInfo** info) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_dev.size() <= dev) g_dev.resize(dev + 1);
    DeviceInfo& d = g_dev[dev];
    if (!d.ready) {
        e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
        e = upload_tables_plain();
        if (e != cudaSuccess) return cuda_fail(e, "uploading the jump tables");
        e = upload_tables_batch();
        if (e != cudaSuccess) return cuda_fail(e, "uploading the jump tables (batch)");
        // The uploads come from pageable memory on the legacy default stream:
        // wait until they have landed, since kernels on non-blocking streams
        // are not ordered after them.
        e = cudaStreamSynchronize(0);
        if (e != cudaSuccess) return cuda_fail(e, "uploading the jump tables (wait)");
        for (int k = 0; k < 5; ++k)
            for (int li = 0; li < kNumLayouts; ++li) d.bps[k][li] = plain_blocks_per_sm(k, 1 << li);
        d.ready = true;
    }
    if (dev_out) *dev_out = dev;
    if (info) *info = &d;
    return MRG8G_SUCCESS;
}

int device_sms() {
    const DeviceInfo* d = nullptr;
    if (ensure_device(nullptr, &d) != MRG8G_SUCCESS) return 0;
    return d->sms;
}

int kind_elem_bytes(int kind) { return (kind == MRG8G_F64_ORIGINAL || kind == MRG8G_F64_SHIFTED) ? 8 : 4; }

bool kind_valid(int kind) { return kind >= MRG8G_U32 && kind <= MRG8G_F32_SHIFTED; }

// Substreams per lane: one 16-byte vector of outputs per row.
// Substreams per lane: two for 8-byte outputs (776 Gsamples/s fp64 SHIFTED at
// 2^30, against 756 with four), four for 4-byte outputs (fp32 834 vs 829,
// u32 1003 vs 993).
int default_layout_V(int kind) { return kind_elem_bytes(kind) == 8 ? 2 : 4; }

// Process-wide launch-shape overrides (mrg8g_tune_plain).
static std::atomic<int> g_tune_V[5];
static std::atomic<int> g_tune_bps[5];

int validate_state(const uint32_t st[8]) {
    bool any = false;
    for (int q = 0; q < 8; ++q) {
        if (st[q] >= 0x80000000u)
            return fail(MRG8G_ERR_INVALID_STATE, "state word %d = %u is not below 2^31", q, st[q]);
        any |= st[q] != 0;
    }
    if (!any) return fail(MRG8G_ERR_INVALID_STATE, "the all-zero state does not generate a stream");
    return MRG8G_SUCCESS;
}

// State after n outputs, exactly as the reference's sequential loop leaves it
// (original/mrg8.cpp:209-219): short runs step on the host so untouched raw
// words shift through unchanged; longer runs jump (all eight words are then
// outputs, whose representatives the jump reproduces).
void advance_state(uint32_t st[8], uint64_t n) {
    if (n == 0) return;
    if (n < 8) {
        step_host(st, n, nullptr);
        return;
    }
    jump_matvec(st, n, st);
}

// Launch the plain kernel for n outputs of `kind` from state st into d_out.
int launch_plain_call(const uint32_t st[8], void* d_out, uint64_t n, int kind, cudaStream_t s, int V) {
    if (n == 0) return MRG8G_SUCCESS;
    const DeviceInfo* dev = nullptr;
    int rc = ensure_device(nullptr, &dev);
    if (rc) return rc;
    const int elem = kind_elem_bytes(kind);
    const uintptr_t addr = (uintptr_t)d_out;
    if (!d_out) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null output pointer");
    if (addr % elem) return fail(MRG8G_ERR_INVALID_ARGUMENT, "output pointer not aligned to %d bytes", elem);
    if (V <= 0) V = g_tune_V[kind].load(std::memory_order_relaxed);
    if (V <= 0) V = default_layout_V(kind);
    const int li = layout_index(V);
    int bps = g_tune_bps[kind].load(std::memory_order_relaxed);
    if (bps <= 0 || bps > dev->bps[kind][li]) bps = dev->bps[kind][li];
    const uint64_t D = 32ull * V;
    uint64_t head = ((16 - addr % 16) % 16) / elem;
    if (head > n) head = n;
    const uint64_t body = n - head;
    const uint64_t max_warps = (uint64_t)dev->sms * bps * (kPlainThreads / 32);
    uint64_t tile = (body + max_warps - 1) / max_warps;
    tile = (tile + D - 1) / D * D;
    tile = std::max<uint64_t>(tile, std::max<uint64_t>(D * 32, 4096));  // >= 4096 outputs and 32 rows per warp
    uint64_t warps = body ? (body + tile - 1) / tile : 1;
    const uint64_t blocks = (warps + kPlainThreads / 32 - 1) / (kPlainThreads / 32);
    if (blocks > (uint64_t)INT32_MAX)
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "bulk launch of %llu blocks exceeds the grid limit",
                    (unsigned long long)blocks);

    PlainArgs a;
    std::memcpy(a.st, st, sizeof(a.st));
    a.n = n;
    a.head = head;
    a.tile = tile;
    a.out = d_out;
    a.lc = kind == MRG8G_F64_ORIGINAL ? host_tables().leap_mod[li] : host_tables().leap[li];  // kLagMod
    cudaError_t e = launch_plain(kind, V, a, (int)blocks, s);
    if (e != cudaSuccess) return cuda_fail(e, "launching the bulk kernel");
    return MRG8G_SUCCESS;
}

}  // namespace mrg8g

// -------------------------------------------------------------------- ABI

#define CHECK_G(g) \
    if (!(g)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null generator handle")

extern "C" {

int mrg8g_version(void) { return MRG8G_VERSION; }

const char* mrg8g_last_error(void) { return t_err.c_str(); }

int mrg8g_create(uint32_t seed, mrg8g_generator** out) {
    if (!out) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null output handle pointer");
    host_tables();
    mrg8g_generator* g = new (std::nothrow) mrg8g_generator;
    if (!g) return fail(MRG8G_ERR_OUT_OF_MEMORY, "host allocation failed");
    mcg64ni(seed, g->st);
    *out = g;
    return MRG8G_SUCCESS;
}

int mrg8g_destroy(mrg8g_generator* g) {
    if (!g) return MRG8G_SUCCESS;
    if (g->stage_dev >= 0) {
        int cur = 0;
        cudaGetDevice(&cur);
        cudaSetDevice(g->stage_dev);
        for (int i = 0; i < 2; ++i) {
            if (g->sstream[i]) cudaStreamSynchronize(g->sstream[i]), cudaStreamDestroy(g->sstream[i]);
            if (g->stage[i]) cudaFree(g->stage[i]);
        }
        cudaSetDevice(cur);
    }
    delete g;
    return MRG8G_SUCCESS;
}

int mrg8g_seed_init(mrg8g_generator* g, uint32_t seed) {
    CHECK_G(g);
    mcg64ni(seed, g->st);
    return MRG8G_SUCCESS;
}

int mrg8g_get_state(const mrg8g_generator* g, uint32_t st[8]) {
    CHECK_G(g);
    if (!st) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null state pointer");
    std::memcpy(st, g->st, sizeof(g->st));
    return MRG8G_SUCCESS;
}

int mrg8g_set_state(mrg8g_generator* g, const uint32_t st[8]) {
    CHECK_G(g);
    if (!st) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null state pointer");
    int rc = validate_state(st);
    if (rc) return rc;
    std::memcpy(g->st, st, sizeof(g->st));
    return MRG8G_SUCCESS;
}

static bool has_zero_word(const uint32_t st[8]) {
    for (int q = 0; q < 8; ++q)
        if (st[q] == 0) return true;
    return false;
}

// original/mrg8.cpp:104-176 semantics.  Without zero words the per-bit
// matrix-vector form gives the same words as forming J first (every sum is
// positive, so both return the [1, p] representative); with zero words the
// exact matrix-product algorithm is used so such words survive as in the
// reference.
static void jump_bits_ref(const uint32_t st[8], const short bits[200], uint32_t out[8]) {
    if (has_zero_word(st)) jump_exact_bits(st, bits, out);
    else jump_matvec_bits(st, bits, out);
}

static void bits_of(uint64_t k, short bits[200]) {
    std::memset(bits, 0, 200 * sizeof(short));
    for (int i = 0; i < 64; ++i) bits[i] = (short)((k >> i) & 1u);
}

int mrg8g_jump_ahead(mrg8g_generator* g, uint64_t k) {
    CHECK_G(g);
    short bits[200];
    bits_of(k, bits);
    jump_bits_ref(g->st, bits, g->st);
    return MRG8G_SUCCESS;
}

int mrg8g_jump_ahead_bits(mrg8g_generator* g, const short bits[200]) {
    CHECK_G(g);
    if (!bits) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null bit array");
    jump_bits_ref(g->st, bits, g->st);
    return MRG8G_SUCCESS;
}

int mrg8g_jump_state(const mrg8g_generator* g, uint64_t k, uint32_t new_state[8]) {
    CHECK_G(g);
    if (!new_state) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null state pointer");
    short bits[200];
    bits_of(k, bits);
    jump_bits_ref(g->st, bits, new_state);
    return MRG8G_SUCCESS;
}

int mrg8g_jump_state_bits(const mrg8g_generator* g, const short bits[200], uint32_t new_state[8]) {
    CHECK_G(g);
    if (!new_state || !bits) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    jump_bits_ref(g->st, bits, new_state);
    return MRG8G_SUCCESS;
}

int mrg8g_generate(mrg8g_generator* g, void* d_out, uint64_t n, int kind, void* stream) {
    CHECK_G(g);
    if (!kind_valid(kind)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown output kind %d", kind);
    if (n > (1ull << 62)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "n = %llu is too large", (unsigned long long)n);
    int rc = launch_plain_call(g->st, d_out, n, kind, (cudaStream_t)stream, 0);
    if (rc) return rc;
    advance_state(g->st, n);
    return MRG8G_SUCCESS;
}

int mrg8g_randint(mrg8g_generator* g, uint32_t* d_out, uint64_t n, void* stream) {
    return mrg8g_generate(g, d_out, n, MRG8G_U32, stream);
}

int mrg8g_rand(mrg8g_generator* g, double* d_out, uint64_t n, int scaling, void* stream) {
    if (scaling != MRG8G_ORIGINAL && scaling != MRG8G_SHIFTED)
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown scaling %d", scaling);
    return mrg8g_generate(g, d_out, n, scaling ? MRG8G_F64_SHIFTED : MRG8G_F64_ORIGINAL, stream);
}

int mrg8g_rand_f32(mrg8g_generator* g, float* d_out, uint64_t n, int scaling, void* stream) {
    if (scaling != MRG8G_ORIGINAL && scaling != MRG8G_SHIFTED)
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown scaling %d", scaling);
    return mrg8g_generate(g, d_out, n, scaling ? MRG8G_F32_SHIFTED : MRG8G_F32_ORIGINAL, stream);
}

static const size_t kStageBytes = 64ull << 20;

int mrg8g_generate_host(mrg8g_generator* g, void* h_out, uint64_t n, int kind) {
    CHECK_G(g);
    if (!kind_valid(kind)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown output kind %d", kind);
    if (n == 0) return MRG8G_SUCCESS;
    if (!h_out) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null output pointer");
    int dev = 0;
    int rc = ensure_device(&dev, nullptr);
    if (rc) return rc;
    cudaError_t e;
    if (g->stage_dev != dev) {
        if (g->stage_dev >= 0) return fail(MRG8G_ERR_INVALID_ARGUMENT, "handle staging belongs to device %d", g->stage_dev);
        for (int i = 0; i < 2; ++i) {
            if ((e = cudaMalloc(&g->stage[i], kStageBytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(staging)");
            if ((e = cudaStreamCreateWithFlags(&g->sstream[i], cudaStreamNonBlocking)) != cudaSuccess)
                return cuda_fail(e, "cudaStreamCreate");
        }
        g->stage_dev = dev;
    }
    const int elem = kind_elem_bytes(kind);
    const uint64_t chunk = kStageBytes / elem;
    uint32_t st[8];
    std::memcpy(st, g->st, sizeof(st));
    char* dst = static_cast<char*>(h_out);
    uint64_t off = 0;
    for (int i = 0; off < n; ++i) {
        const uint64_t c = std::min(chunk, n - off);
        cudaStream_t s = g->sstream[i & 1];
        rc = launch_plain_call(st, g->stage[i & 1], c, kind, s, 0);
        if (rc) return rc;
        advance_state(st, c);
        e = cudaMemcpyAsync(dst + off * elem, g->stage[i & 1], c * elem, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(D2H)");
        off += c;
    }
    for (int i = 0; i < 2; ++i)
        if ((e = cudaStreamSynchronize(g->sstream[i])) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    std::memcpy(g->st, st, sizeof(st));
    return MRG8G_SUCCESS;
}

int mrg8g_generate_from_state(const uint32_t st[8], uint64_t offset, void* d_out, uint64_t n, int kind,
                              void* stream) {
    if (!st) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null state pointer");
    if (!kind_valid(kind)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown output kind %d", kind);
    int rc = validate_state(st);
    if (rc) return rc;
    uint32_t s[8];
    std::memcpy(s, st, sizeof(s));
    advance_state(s, offset);
    return launch_plain_call(s, d_out, n, kind, (cudaStream_t)stream, 0);
}

int mrg8g_seed_state(uint32_t seed, uint32_t st[8]) {
    if (!st) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null state pointer");
    mcg64ni(seed, st);
    return MRG8G_SUCCESS;
}

int mrg8g_stream_sync(void* stream) {
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return MRG8G_SUCCESS;
}

int mrg8g_tune_plain(int kind, int V, int blocks_per_sm) {
    if (!kind_valid(kind)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown output kind %d", kind);
    if (V != 0 && V != 1 && V != 2 && V != 4) return fail(MRG8G_ERR_INVALID_ARGUMENT, "V must be 0, 1, 2 or 4");
    if (blocks_per_sm < 0) return fail(MRG8G_ERR_INVALID_ARGUMENT, "negative blocks per SM");
    g_tune_V[kind].store(V);
    g_tune_bps[kind].store(blocks_per_sm);
    return MRG8G_SUCCESS;
}

int mrg8g_get_plain_tuning(int kind, int* V, int* blocks_per_sm) {
    if (!kind_valid(kind) || !V || !blocks_per_sm) return fail(MRG8G_ERR_INVALID_ARGUMENT, "bad argument");
    *V = g_tune_V[kind].load();
    *blocks_per_sm = g_tune_bps[kind].load();
    return MRG8G_SUCCESS;
}

int mrg8g_write_jump_matrix(const char* path) {
    if (!path) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null path");
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(MRG8G_ERR_INVALID_ARGUMENT, "cannot open %s for writing", path);
    const HostTables& t = host_tables();
    for (int j = 0; j < kNumJump; ++j) {
        for (int c = 0; c < 8; ++c)
            for (int r = 0; r < 8; ++r) std::fprintf(f, "%12u", t.jump[j][r * 8 + c]);
        std::fprintf(f, "\n");
    }
    const bool ok = std::fclose(f) == 0;
    return ok ? MRG8G_SUCCESS : fail(MRG8G_ERR_INVALID_ARGUMENT, "error writing %s", path);
}

int mrg8g_verify_jump_matrix(const char* path, uint64_t* mismatches) {
    if (!path) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null path");
    FILE* f = std::fopen(path, "r");
    if (!f) return fail(MRG8G_ERR_INVALID_ARGUMENT, "cannot open %s", path);
    const HostTables& t = host_tables();
    uint64_t bad = 0;
    for (int k = 0; k < kNumJump * 64; ++k) {
        unsigned long v;
        if (std::fscanf(f, "%lu", &v) != 1) {
            std::fclose(f);
            return fail(MRG8G_ERR_INVALID_ARGUMENT, "%s: %d numbers, expected %d", path, k, kNumJump * 64);
        }
        const int j = k / 64, r = k % 8, c = (k % 64) / 8;  // column-major per matrix
        bad += v != t.jump[j][r * 8 + c];
    }
    std::fclose(f);
    if (mismatches) *mismatches = bad;
    if (bad) return fail(MRG8G_ERR_INVALID_STATE, "%s differs from A^(2^j) in %llu entries", path, (unsigned long long)bad);
    return MRG8G_SUCCESS;
}

int mrg8g_convert(const uint32_t* d_in, void* d_out, uint64_t n, int kind, void* stream) {
    if (kind == MRG8G_U32 || !kind_valid(kind))
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "convert needs a floating-point kind, got %d", kind);
    if (n == 0) return MRG8G_SUCCESS;
    if (!d_in || !d_out) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    const int sms = device_sms();
    if (!sms) return MRG8G_ERR_CUDA;
    const uint64_t want = (n + 255) / 256;
    const int blocks = (int)std::min<uint64_t>(want, (uint64_t)sms * 8);
    cudaError_t e = launch_convert(kind, d_in, d_out, n, blocks, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "launching the conversion kernel");
    return MRG8G_SUCCESS;
}

int mrg8g_jump_states(const uint32_t st[8], const uint64_t* d_offsets, uint32_t* d_states, uint64_t count,
                      void* stream) {
    if (!st) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null state pointer");
    int rc = validate_state(st);
    if (rc) return rc;
    if (count == 0) return MRG8G_SUCCESS;
    if (!d_offsets || !d_states) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    const int sms = device_sms();
    if (!sms) return MRG8G_ERR_CUDA;
    JumpArgs a;
    std::memcpy(a.st, st, sizeof(a.st));
    a.offsets = d_offsets;
    a.states = d_states;
    a.count = count;
    const uint64_t want = (count + 3) / 4;
    const int blocks = (int)std::min<uint64_t>(want, (uint64_t)sms * 16);
    cudaError_t e = launch_jump_states(a, blocks, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "launching the jump kernel");
    return MRG8G_SUCCESS;
}

}  // extern "C"
