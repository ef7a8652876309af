// mrg8g_serve.cpp -- serving: continuous batching of draw requests.
//
// A scheduler thread admits requests first-in first-out against a device
// output arena (the admission budget), packs the admitted ones into a batch
// (the batch kernel of mrg8g_batch.cu, deriving its tiles on the device from
// the requests' tile counts) and launches it on one of
// several streams, so that requests arriving while others are on the GPU are
// admitted as soon as a stream slot and arena space are free and their work
// overlaps on the device.  Generator states live in a device table; a draw
// from a registered generator continues its stream (the host keeps only the
// position).  A launch is complete when its kernel's end stamp reaches mapped
// host memory (the last block writes it after every block fenced its
// outputs); its completion event is queried too, every sixteenth check and
// for launches without a kernel, so that errors surface.  While launches are
// in flight the scheduler polls (and yields between polls); it blocks on a
// condition variable only when nothing is in flight.  The arena places blocks
// first-fit (mrg8g_arena.h), so space released in any order is reused.
// Nothing on the device waits: the kernels are the batch kernel and every
// host wait is bounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <exception>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <memory>
#include <string>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/mrg8g.h"
#include "mrg8g_internal.h"
#include "mrg8g_runtime.h"
#include "mrg8g_arena.h"
#include "mrg8g_tables.h"

using namespace mrg8g;

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    mrg8g_request r;
    uint32_t state[8];  // stateless requests
    uint64_t offset;    // jump distance from the (embedded or table) state
    uint64_t bytes = 0, arena_off = 0, arena_seq = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int status = MRG8G_SUCCESS;
    bool done = false;
};

struct Slot {
    int idx = 0;
    cudaStream_t stream = nullptr;
    char* d_stage = nullptr;        // instances, then tile prefix counts (one copy per launch)
    char* h_stage = nullptr;        // pinned staging of the same layout
    uint32_t* d_counter = nullptr;  // work-queue counter, finished-block counter
    cudaEvent_t done_ev = nullptr;  // recorded after the batch
    // [start, end] of the slot's kernel in %globaltimer ns, written by the
    // kernel into mapped pinned host memory (no API call on the launch path).
    volatile unsigned long long* h_times = nullptr;
    unsigned long long* d_times = nullptr;
    bool has_kernel = false;  // the launch has a kernel, which stamps its end
    uint32_t polls = 0;       // completion checks since the launch
    std::vector<uint64_t> tickets;
    bool busy = false;
    mrg8g_server* server = nullptr;
};

}  // namespace

struct mrg8g_server {
    mrg8g_server_config cfg{};
    int dev = 0, sms = 0, bps = 1;
    void* arena_base = nullptr;
    uint32_t* d_states = nullptr;
    std::vector<uint64_t> gen_pos;
    std::vector<std::array<uint32_t, 8>> gen_state;
    std::unique_ptr<mrg8g::Arena> arena;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::atomic<uint64_t> wake_seq{0};  // bumped by submissions and releases
    std::atomic<bool> stop{false};
    std::deque<uint64_t> pending;  // admission order
    std::deque<uint64_t> completed;
    std::unordered_map<uint64_t, Req> reqs;
    uint64_t next_ticket = 1;
    int error = MRG8G_SUCCESS;
    std::string error_msg;
    std::thread thread;

    // statistics
    uint64_t submitted = 0, finished = 0, launches = 0, launched_requests = 0, samples = 0, peak_bytes = 0;
    uint64_t max_inflight = 0, overlapped = 0;
    uint64_t kernel_ns = 0, kernel_timed = 0;  // device time of stamped launches
    // Kernel intervals of the most recent finished launches (%globaltimer
    // ns), to find launches that ran on the device at the same time.
    struct Interval {
        unsigned long long t0, t1;
        bool counted;
    };
    static constexpr int kRecent = 64;
    Interval recent[kRecent] = {};
    int nrecent = 0, next_recent = 0;
};

namespace {

// Fewest rows per tile of a serving launch.  Below about this many rows the
// per-tile jump of the state costs more than generating the tile.
constexpr uint64_t kMinServeTileRows = 16;

// Resident warps of one batch launch.
uint64_t launch_warps(const mrg8g_server* sv) { return (uint64_t)sv->sms * sv->bps * (sv->cfg.threads / 32); }

// Descriptors of the tickets admitted to slot `sl` (lock held): the
// instances, largest first, and the prefix counts of their tiles, which the
// batch kernel turns into tiles itself.  Rows per tile: as many as spread
// the launch's rows over the resident warps, between kMinServeTileRows and
// the configured maximum, so that a request that would not fill the GPU with
// full tiles still runs on many warps at once.
void describe_slot(mrg8g_server* sv, Slot& sl, std::vector<BatchInst>& insts, std::vector<uint32_t>& base,
                   uint32_t* tile_elems) {
    const uint32_t count = (uint32_t)sl.tickets.size();
    insts.resize(count);
    constexpr uint64_t D = 32 * kBatchLayoutV;
    uint64_t rows = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const Req& q = sv->reqs[sl.tickets[i]];
        BatchInst& d = insts[i];
        std::memcpy(d.st, q.state, sizeof(d.st));
        d.offset = q.offset;
        d.n = q.r.n;
        d.out = static_cast<char*>(sv->arena_base) + q.arena_off;
        d.kind = q.r.kind;
        d.slot1 = q.r.generator == MRG8G_NO_GENERATOR ? 0u : q.r.generator + 1u;
        rows += (d.n + D - 1) / D;
    }
    sort_largest_first(insts.data(), count);
    const uint64_t warps = launch_warps(sv);
    uint64_t tr = ((rows + warps - 1) / warps + 7) / 8 * 8;
    tr = std::min<uint64_t>(std::max<uint64_t>(tr, kMinServeTileRows), (uint64_t)sv->cfg.tile_rows);
    *tile_elems = (uint32_t)(tr * D);
    base.resize(count + 1);
    tile_prefix(insts.data(), count, tr * D, base.data());  // < 2^32 (checked at creation)
}

// Enqueue slot `sl`'s batch on its stream (lock not held; the slot is owned
// by the scheduler thread while busy).
int enqueue_slot(mrg8g_server* sv, Slot& sl, const std::vector<BatchInst>& insts, const std::vector<uint32_t>& base,
                 uint32_t tile_elems) {
    const size_t count = insts.size();
    const uint32_t ntiles = base[count];
    const size_t ib = count * sizeof(BatchInst), bb = (count + 1) * sizeof(uint32_t);
    std::memcpy(sl.h_stage, insts.data(), ib);
    std::memcpy(sl.h_stage + ib, base.data(), bb);
    cudaError_t e;
    sl.h_times[0] = 0;
    sl.h_times[1] = 0;
    sl.has_kernel = ntiles != 0;
    sl.polls = 0;
    if (ntiles) {
        if ((e = cudaMemcpyAsync(sl.d_stage, sl.h_stage, ib + bb, cudaMemcpyHostToDevice, sl.stream)) != cudaSuccess)
            return cuda_fail(e, "serving: copy of the batch descriptors");
        BatchArgs a;
        a.insts = reinterpret_cast<const BatchInst*>(sl.d_stage);
        a.tiles = nullptr;
        a.tile_base = reinterpret_cast<const uint32_t*>(sl.d_stage + ib);
        a.ninst = (uint32_t)count;
        a.tile_elems = tile_elems;
        a.ntiles = ntiles;
        a.counter = sl.d_counter;
        a.done_blocks = sl.d_counter + 1;  // the kernel leaves both at zero
        a.states = sv->d_states;
        a.times = sl.d_times;
        set_batch_leaps(a);
        const uint64_t wpb = (uint64_t)sv->cfg.threads / 32;
        const uint64_t want = (ntiles + wpb - 1) / wpb;
        const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sv->sms * sv->bps, want));
        if ((e = launch_batch(a, sv->cfg.threads, blocks, sl.stream)) != cudaSuccess)
            return cuda_fail(e, "serving: batch launch");
    }
    if ((e = cudaEventRecord(sl.done_ev, sl.stream)) != cudaSuccess)
        return cuda_fail(e, "serving: completion event");
    return MRG8G_SUCCESS;
}

// Kernel interval of a finished launch against the recent ones (lock held;
// the launch's end stamp or completion event has been seen, so the kernel's
// stamps are in host memory).  A launch that overlaps an earlier one counts both, once
// each.  Launches without a kernel (no tiles) have no stamps.
void note_interval(mrg8g_server* sv, Slot& sl) {
    const unsigned long long a = sl.h_times[0], b = sl.h_times[1];
    if (a == 0 || b < a) return;
    sv->kernel_ns += b - a;
    sv->kernel_timed++;
    mrg8g_server::Interval cur{a, b, false};
    for (int i = 0; i < sv->nrecent; ++i) {
        mrg8g_server::Interval& o = sv->recent[i];
        if (cur.t0 < o.t1 && o.t0 < cur.t1) {
            if (!o.counted) o.counted = true, sv->overlapped++;
            if (!cur.counted) cur.counted = true, sv->overlapped++;
        }
    }
    sv->recent[sv->next_recent] = cur;
    sv->next_recent = (sv->next_recent + 1) % mrg8g_server::kRecent;
    sv->nrecent = std::min(sv->nrecent + 1, (int)mrg8g_server::kRecent);
}

// Requests of a finished slot complete at time t with status rc (lock held).
void finish_slot(mrg8g_server* sv, Slot& sl, double t, int rc) {
    if (rc == MRG8G_SUCCESS) note_interval(sv, sl);
    for (uint64_t tk : sl.tickets) {
        Req& q = sv->reqs[tk];
        q.t_done = t;
        q.status = rc;
        q.done = true;
        sv->completed.push_back(tk);
        sv->finished++;
        if (rc == MRG8G_SUCCESS) sv->samples += q.r.n;
    }
    sl.tickets.clear();
    sl.busy = false;
}

// The scheduler spins (yielding) while launches are in flight and for
// cfg.spin_us after the last activity, so that requests arriving at a steady
// rate find it awake; after that it sleeps on cv_sched.

void scheduler_loop(mrg8g_server* sv);

// The scheduler thread: its loop, with a host allocation failure turned into
// a failed server (later submissions are refused; waiters time out) instead of
// an exception that would end the process.
void scheduler(mrg8g_server* sv) {
    try {
        scheduler_loop(sv);
    } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->error = MRG8G_ERR_OUT_OF_MEMORY;
        sv->error_msg = std::string("scheduler: ") + e.what();
        sv->cv_done.notify_all();
    }
}

void scheduler_loop(mrg8g_server* sv) {
    cudaSetDevice(sv->dev);
    std::vector<BatchInst> insts;
    std::vector<uint32_t> base;
    uint32_t tile_elems = 0;
    struct Done {
        int idx;
        double t;
        cudaError_t e;
    };
    std::vector<Done> done;
    uint64_t seen = ~0ull;
    double active = now_s();
    const double spin_idle = sv->cfg.spin_us < 0 ? 0.0 : sv->cfg.spin_us * 1e-6;
    bool inflight = false;
    while (!sv->stop.load(std::memory_order_acquire)) {
        // In-flight launches, polled without the lock (the scheduler thread
        // owns the slots while they are busy).
        // A launch is complete when its kernel's end stamp reaches host
        // memory (the kernel makes all its outputs visible first), which the
        // host sees sooner than the completion event; the event is still
        // queried every few checks, and for launches without a kernel, so
        // that an execution error is reported.
        done.clear();
        for (Slot& sl : sv->slots) {
            if (!sl.busy) continue;
            if (sl.has_kernel && sl.h_times[1] != 0) {
                done.push_back({sl.idx, now_s(), cudaSuccess});
                continue;
            }
            if (sl.has_kernel && (++sl.polls & 15u) != 0) continue;
            const cudaError_t q = cudaEventQuery(sl.done_ev);
            if (q != cudaErrorNotReady) done.push_back({sl.idx, now_s(), q});
        }
        const uint64_t ws = sv->wake_seq.load(std::memory_order_acquire);
        if (done.empty() && ws == seen) {  // nothing new
            if (inflight || now_s() - active < spin_idle) {
                std::this_thread::yield();
                continue;
            }
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv_sched.wait_for(lk, std::chrono::microseconds(500), [&] {
                return sv->stop.load(std::memory_order_relaxed) || sv->wake_seq.load(std::memory_order_relaxed) != seen;
            });
            continue;
        }
        seen = ws;
        active = now_s();
        std::unique_lock<std::mutex> lk(sv->mu);
        for (const Done& d : done) {
            int rc = MRG8G_SUCCESS;
            if (d.e != cudaSuccess) {
                rc = cuda_fail(d.e, "serving: batch execution");
                sv->error = rc;
                sv->error_msg = mrg8g_last_error();
            }
            finish_slot(sv, sv->slots[d.idx], d.t, rc);
        }
        if (!done.empty()) sv->cv_done.notify_all();
        // Admission into free slots, first in first out.
        for (Slot& sl : sv->slots) {
            if (sl.busy || sv->pending.empty() || sv->error) continue;
            const double t = now_s();
            while (!sv->pending.empty() && sl.tickets.size() < sv->cfg.max_batch) {
                Req& q = sv->reqs[sv->pending.front()];
                if (!sv->arena->alloc(q.bytes, &q.arena_off, &q.arena_seq)) break;  // head of line waits for space
                q.t_admit = t;
                sl.tickets.push_back(sv->pending.front());
                sv->pending.pop_front();
            }
            if (sl.tickets.empty()) break;
            sv->peak_bytes = std::max(sv->peak_bytes, sv->arena->used());
            describe_slot(sv, sl, insts, base, &tile_elems);
            sl.busy = true;
            sv->launches++;
            sv->launched_requests += sl.tickets.size();
            uint64_t busy = 0;
            for (const Slot& o : sv->slots) busy += o.busy ? 1 : 0;
            sv->max_inflight = std::max(sv->max_inflight, busy);
            lk.unlock();
            const int rc = enqueue_slot(sv, sl, insts, base, tile_elems);
            std::string msg = rc ? mrg8g_last_error() : "";
            lk.lock();
            if (rc) {
                sv->error = rc;
                sv->error_msg = msg;
                finish_slot(sv, sl, now_s(), rc);
                sv->cv_done.notify_all();
            }
        }
        inflight = false;
        for (const Slot& sl : sv->slots) inflight |= sl.busy;
    }
}

void destroy_server(mrg8g_server* sv) {
    if (sv->thread.joinable()) {
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->stop.store(true, std::memory_order_release);
            sv->cv_sched.notify_all();
        }
        sv->thread.join();
    }
    for (Slot& sl : sv->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream), cudaStreamDestroy(sl.stream);
        if (sl.d_stage) cudaFree(sl.d_stage);
        if (sl.d_counter) cudaFree(sl.d_counter);
        if (sl.h_stage) cudaFreeHost(sl.h_stage);
        if (sl.done_ev) cudaEventDestroy(sl.done_ev);
        if (sl.h_times) cudaFreeHost((void*)sl.h_times);
    }
    if (sv->arena_base) cudaFree(sv->arena_base);
    if (sv->d_states) cudaFree(sv->d_states);
    delete sv;
}

}  // namespace

extern "C" {

int mrg8g_server_create(const mrg8g_server_config* cfg, mrg8g_server** out) {
    if (!out) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    mrg8g_server_config c{};
    if (cfg) c = *cfg;
    if (!c.budget_bytes) c.budget_bytes = 16ull << 30;
    if (!c.max_batch) c.max_batch = 1024;
    if (!c.inflight) c.inflight = 3;
    if (!c.max_generators) c.max_generators = 65536;
    if (!c.tile_rows) c.tile_rows = 256;
    if (!c.threads) c.threads = 128;
    if (!c.spin_us) c.spin_us = 2000;
    if (c.tile_rows < 8 || (c.tile_rows & 7) || c.tile_rows > (1 << 16) || (c.threads != 128 && c.threads != 256) ||
        c.inflight > 16)
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "bad server configuration");
    int dev = 0;
    int rc = ensure_device(&dev, nullptr);
    if (rc) return rc;
    mrg8g_server* sv = new (std::nothrow) mrg8g_server;
    if (!sv) return fail(MRG8G_ERR_OUT_OF_MEMORY, "host allocation failed");
    sv->cfg = c;
    sv->dev = dev;
    sv->sms = device_sms();
    sv->bps = batch_blocks_per_sm(c.threads);
    sv->arena.reset(new mrg8g::Arena(c.budget_bytes));
    sv->gen_pos.reserve(1024);
    cudaError_t e;
    if ((e = cudaMalloc(&sv->arena_base, c.budget_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&sv->d_states, (size_t)c.max_generators * 8 * sizeof(uint32_t))) != cudaSuccess) {
        destroy_server(sv);
        return cuda_fail(e, "serving: arena allocation");
    }
    // A launch's tile count (at most 2 per request plus its bytes / 4 KiB,
    // 4 KiB being the shortest body tile) must fit the kernel's 32-bit queue.
    if (c.budget_bytes / 4096 + 2ull * c.max_batch >= 0xFFFFFFFFull) {
        destroy_server(sv);
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "budget or max_batch too large");
    }
    sv->slots.resize(c.inflight);
    for (uint32_t i = 0; i < c.inflight; ++i) {
        Slot& sl = sv->slots[i];
        sl.idx = (int)i;
        sl.server = sv;
        const size_t stage = c.max_batch * sizeof(BatchInst) + ((size_t)c.max_batch + 1) * sizeof(uint32_t);
        if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaMalloc(&sl.d_stage, stage)) != cudaSuccess ||
            (e = cudaMalloc(&sl.d_counter, 2 * sizeof(uint32_t))) != cudaSuccess ||
            (e = cudaMemsetAsync(sl.d_counter, 0, 2 * sizeof(uint32_t), sl.stream)) != cudaSuccess ||
            (e = cudaHostAlloc(&sl.h_stage, stage, cudaHostAllocDefault)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&sl.done_ev, cudaEventDisableTiming)) != cudaSuccess) {
            destroy_server(sv);
            return cuda_fail(e, "serving: slot allocation");
        }
        void* ht = nullptr;
        if ((e = cudaHostAlloc(&ht, 2 * sizeof(unsigned long long), cudaHostAllocMapped)) != cudaSuccess) {
            destroy_server(sv);
            return cuda_fail(e, "serving: slot allocation");
        }
        sl.h_times = static_cast<volatile unsigned long long*>(ht);
        sl.h_times[0] = sl.h_times[1] = 0;
        if ((e = cudaHostGetDevicePointer((void**)&sl.d_times, ht, 0)) != cudaSuccess) {
            destroy_server(sv);
            return cuda_fail(e, "serving: mapped timing words");
        }
    }
    try {
        sv->thread = std::thread(scheduler, sv);
    } catch (...) {
        destroy_server(sv);
        return fail(MRG8G_ERR_OUT_OF_MEMORY, "cannot start the scheduler thread");
    }
    *out = sv;
    return MRG8G_SUCCESS;
}

int mrg8g_server_add_generator(mrg8g_server* sv, const uint32_t state[8], uint32_t* slot) {
    if (!sv || !state || !slot) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    int rc = validate_state(state);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->gen_pos.size() >= sv->cfg.max_generators) return fail(MRG8G_ERR_BUDGET, "generator table is full");
    const uint32_t k = (uint32_t)sv->gen_pos.size();
    cudaError_t e = copy_to_device(sv->d_states + 8ull * k, state, 8 * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(e, "serving: generator upload");
    std::array<uint32_t, 8> st;
    std::memcpy(st.data(), state, sizeof(uint32_t) * 8);
    sv->gen_state.push_back(st);
    sv->gen_pos.push_back(0);
    *slot = k;
    return MRG8G_SUCCESS;
}

int mrg8g_server_generator_state(mrg8g_server* sv, uint32_t slot, uint32_t state[8]) {
    if (!sv || !state) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    uint32_t base[8];
    uint64_t pos;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (slot >= sv->gen_pos.size()) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown generator %u", slot);
        std::memcpy(base, sv->gen_state[slot].data(), sizeof(base));
        pos = sv->gen_pos[slot];
    }
    std::memcpy(state, base, sizeof(base));
    advance_state(state, pos);
    return MRG8G_SUCCESS;
}

int mrg8g_server_submit(mrg8g_server* sv, const mrg8g_request* r, uint64_t* ticket) {
    if (!sv || !r || !ticket) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    if (!kind_valid(r->kind)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown kind %d", r->kind);
    const uint64_t bytes = r->n * (uint64_t)kind_elem_bytes(r->kind);
    if (r->n > (1ull << 40) || bytes > sv->cfg.budget_bytes)
        return fail(MRG8G_ERR_BUDGET, "request of %llu bytes exceeds the budget", (unsigned long long)bytes);
    Req q;
    q.r = *r;
    q.bytes = bytes;
    q.t_submit = now_s();
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->error) return fail(sv->error, "server failed: %s", sv->error_msg.c_str());
    if (r->generator == MRG8G_NO_GENERATOR) {
        mcg64ni(r->seed, q.state);
        q.offset = r->offset;
        if (r->offset > ~0ull - r->n) return fail(MRG8G_ERR_INVALID_ARGUMENT, "offset + n overflows");
    } else {
        if (r->generator >= sv->gen_pos.size()) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown generator");
        std::memset(q.state, 0, sizeof(q.state));
        q.offset = sv->gen_pos[r->generator];
        sv->gen_pos[r->generator] += r->n;
    }
    const uint64_t tk = sv->next_ticket++;
    try {
        sv->reqs.emplace(tk, q);
        sv->pending.push_back(tk);
    } catch (const std::bad_alloc&) {
        sv->reqs.erase(tk);
        if (r->generator != MRG8G_NO_GENERATOR) sv->gen_pos[r->generator] -= r->n;
        return fail(MRG8G_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    sv->submitted++;
    sv->wake_seq.fetch_add(1, std::memory_order_release);
    sv->cv_sched.notify_one();
    *ticket = tk;
    return MRG8G_SUCCESS;
}

int mrg8g_server_poll(mrg8g_server* sv, mrg8g_completion* out, uint32_t max, uint32_t* count, uint32_t timeout_us) {
    if (!sv || !count || (max && !out)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    std::unique_lock<std::mutex> lk(sv->mu);
    if (sv->completed.empty() && timeout_us)
        sv->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !sv->completed.empty(); });
    uint32_t k = 0;
    while (k < max && !sv->completed.empty()) {
        const uint64_t tk = sv->completed.front();
        sv->completed.pop_front();
        const Req& q = sv->reqs[tk];
        mrg8g_completion& c = out[k++];
        c.ticket = tk;
        c.tag = q.r.tag;
        c.out = static_cast<char*>(sv->arena_base) + q.arena_off;
        c.n = q.r.n;
        c.kind = q.r.kind;
        c.status = q.status;
        c.t_submit = q.t_submit;
        c.t_admit = q.t_admit;
        c.t_done = q.t_done;
    }
    *count = k;
    return MRG8G_SUCCESS;
}

int mrg8g_server_read(mrg8g_server* sv, uint64_t ticket, void* host, uint64_t bytes) {
    if (!sv || (bytes && !host)) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    const void* src = nullptr;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->reqs.find(ticket);
        if (it == sv->reqs.end()) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown ticket %llu", (unsigned long long)ticket);
        const Req& q = it->second;
        if (!q.done) return fail(MRG8G_ERR_NOT_READY, "ticket %llu is not complete", (unsigned long long)ticket);
        if (q.status) return fail(q.status, "ticket %llu failed", (unsigned long long)ticket);
        if (bytes > q.bytes) return fail(MRG8G_ERR_INVALID_ARGUMENT, "read past the result");
        src = static_cast<const char*>(sv->arena_base) + q.arena_off;
    }
    // A plain blocking copy: the request is done, i.e. the scheduler has seen
    // its launch complete (the kernel's end stamp, written after every block
    // fenced its outputs, or the launch's completion event), so its outputs are
    // complete in device memory and no ordering with the launch's
    // (non-blocking) stream is needed.  The region stays the request's until
    // mrg8g_server_release.
    cudaError_t e = cudaMemcpy(host, src, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "serving: result read");
    return MRG8G_SUCCESS;
}

int mrg8g_server_release(mrg8g_server* sv, uint64_t ticket) {
    if (!sv) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return fail(MRG8G_ERR_INVALID_ARGUMENT, "unknown ticket %llu", (unsigned long long)ticket);
    if (!it->second.done) return fail(MRG8G_ERR_NOT_READY, "ticket %llu is not complete", (unsigned long long)ticket);
    if (it->second.t_admit > 0) sv->arena->release(it->second.arena_seq);
    sv->reqs.erase(it);
    sv->wake_seq.fetch_add(1, std::memory_order_release);
    sv->cv_sched.notify_one();
    return MRG8G_SUCCESS;
}

int mrg8g_server_get_stats(mrg8g_server* sv, mrg8g_server_stats* st) {
    if (!sv || !st) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    std::lock_guard<std::mutex> lk(sv->mu);
    st->submitted = sv->submitted;
    st->completed = sv->finished;
    st->pending = sv->pending.size();
    st->launches = sv->launches;
    st->launched_requests = sv->launched_requests;
    st->samples = sv->samples;
    st->bytes_in_use = sv->arena->used();
    st->peak_bytes = sv->peak_bytes;
    st->error = sv->error;
    st->reserved = 0;
    st->max_inflight = sv->max_inflight;
    st->overlapped_launches = sv->overlapped;
    st->mean_batch = sv->launches ? (double)sv->launched_requests / (double)sv->launches : 0.0;
    st->kernel_ns = sv->kernel_ns;
    st->kernel_launches = sv->kernel_timed;
    return MRG8G_SUCCESS;
}

int mrg8g_server_destroy(mrg8g_server* sv) {
    if (!sv) return MRG8G_SUCCESS;
    destroy_server(sv);
    return MRG8G_SUCCESS;
}

// Open-loop Poisson load: arrivals at `rate` per second for `duration_s`,
// lengths log-uniform in [n_min, n_max], offsets uniform in [0, offset_max),
// kinds uniform over kinds_mask, seeds random; every completion is held for
// hold_us and then released.  Latency = completion time - submit time.
int mrg8g_server_loadtest(mrg8g_server* sv, const mrg8g_loadtest_config* cfg, mrg8g_loadtest_result* res) {
    if (!sv || !cfg || !res) return fail(MRG8G_ERR_INVALID_ARGUMENT, "null pointer");
    if (cfg->rate <= 0 || cfg->duration_s <= 0 || cfg->n_min == 0 || cfg->n_max < cfg->n_min || !(cfg->kinds_mask & 31))
        return fail(MRG8G_ERR_INVALID_ARGUMENT, "bad load-test configuration");
    std::mt19937_64 rng(cfg->rng_seed);
    std::exponential_distribution<double> gap(cfg->rate);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    std::vector<int> kinds;
    for (int k = 0; k < 5; ++k)
        if (cfg->kinds_mask & (1u << k)) kinds.push_back(k);
    mrg8g_server_stats st0;
    mrg8g_server_get_stats(sv, &st0);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->max_inflight = 0;  // high-water marks of this run
        sv->peak_bytes = sv->arena->used();
    }
    std::atomic<bool> done_submitting{false};
    std::atomic<uint64_t> submitted{0};
    std::vector<double> lat;
    lat.reserve((size_t)(cfg->rate * cfg->duration_s * 1.2) + 16);
    uint64_t samples = 0, bytes = 0;
    double t_first = 0, t_last = 0;
    int consumer_rc = MRG8G_SUCCESS;
    std::thread consumer([&] {
        std::vector<mrg8g_completion> buf(256);
        std::deque<std::pair<double, uint64_t>> held;
        uint64_t seen = 0;
        while (true) {
            uint32_t n = 0;
            int rc = mrg8g_server_poll(sv, buf.data(), (uint32_t)buf.size(), &n, 200);
            if (rc) {
                consumer_rc = rc;
                break;
            }
            const double t = now_s();
            for (uint32_t i = 0; i < n; ++i) {
                const mrg8g_completion& c = buf[i];
                if (c.status) consumer_rc = c.status;
                lat.push_back(c.t_done - c.t_submit);
                samples += c.n;
                bytes += c.n * kind_elem_bytes(c.kind);
                t_last = std::max(t_last, c.t_done);
                held.push_back({t + cfg->hold_us * 1e-6, c.ticket});
            }
            seen += n;
            while (!held.empty() && held.front().first <= now_s()) {
                mrg8g_server_release(sv, held.front().second);
                held.pop_front();
            }
            if (done_submitting.load() && seen >= submitted.load()) {
                for (auto& h : held) mrg8g_server_release(sv, h.second);
                break;
            }
        }
    });
    const double t0 = now_s();
    t_first = t0;
    double t_next = t0;
    uint64_t late = 0, count = 0;
    const double lmin = std::log((double)cfg->n_min), lmax = std::log((double)cfg->n_max + 1.0);
    int rc = MRG8G_SUCCESS;
    while (true) {
        t_next += gap(rng);
        if (t_next - t0 > cfg->duration_s) break;
        mrg8g_request r{};
        r.generator = MRG8G_NO_GENERATOR;
        r.seed = (uint32_t)rng();
        r.offset = cfg->offset_max ? rng() % cfg->offset_max : 0;
        r.n = std::min<uint64_t>(cfg->n_max, (uint64_t)std::exp(lmin + (lmax - lmin) * u01(rng)));
        r.kind = kinds[rng() % kinds.size()];
        r.tag = count;
        double t;
        while ((t = now_s()) < t_next) {
        }
        if (t - t_next > 100e-6) late++;
        uint64_t tk;
        rc = mrg8g_server_submit(sv, &r, &tk);
        if (rc) break;
        submitted.fetch_add(1);
        count++;
    }
    done_submitting.store(true);
    consumer.join();
    if (rc) return rc;
    if (consumer_rc) return consumer_rc;
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) { return lat.empty() ? 0.0 : lat[std::min(lat.size() - 1, (size_t)(p * (lat.size() - 1) + 0.5))]; };
    mrg8g_server_stats st;
    mrg8g_server_get_stats(sv, &st);
    res->requests = lat.size();
    res->samples = samples;
    res->bytes = bytes;
    res->wall_s = t_last - t_first;
    res->gsamples_per_s = res->wall_s > 0 ? samples / res->wall_s / 1e9 : 0;
    double sum = 0;
    for (double v : lat) sum += v;
    res->mean_us = lat.empty() ? 0 : sum / lat.size() * 1e6;
    res->p50_us = pct(0.50) * 1e6;
    res->p90_us = pct(0.90) * 1e6;
    res->p99_us = pct(0.99) * 1e6;
    res->max_us = lat.empty() ? 0 : lat.back() * 1e6;
    res->launches = st.launches - st0.launches;
    res->mean_batch = res->launches ? (double)(st.launched_requests - st0.launched_requests) / res->launches : 0;
    res->max_inflight = st.max_inflight;
    res->overlapped_launches = st.overlapped_launches - st0.overlapped_launches;
    const uint64_t kl = st.kernel_launches - st0.kernel_launches;
    res->mean_kernel_us = kl ? (double)(st.kernel_ns - st0.kernel_ns) / (double)kl * 1e-3 : 0.0;
    res->peak_bytes = st.peak_bytes;
    res->late_submits = late;
    return MRG8G_SUCCESS;
}

}  // extern "C"
