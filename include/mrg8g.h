/*
 * mrg8g.h -- C ABI of the GB300-native MRG8 generator (libmrg8g.so).
 *
 * MRG8 is L'Ecuyer's order-8 multiple recursive generator modulo 2^31-1:
 *     S[n] = sum_{k=1..8} a_k S[n-k]  mod (2^31 - 1),
 * with the state (S[n-1], ..., S[n-8]) kept newest first.  Every stream
 * output is the representative in [1, 2^31-1] (0 is represented by 2^31-1),
 * and every output of this library is bit-identical to the reference's
 * sequential stream (kenmiura/mrg8 original/mrg8.cpp) for the same state.
 *
 * The reference interface is the C++ class pair mrg8 / mrg8_cuda
 * (original/mrg8.h:21-56, cuda/mrg8.h:23-79, cuda/mrg8_cuda.h:20-45).  Each
 * entry point below names the member it replaces.  include/mrg8_cuda.hpp
 * re-creates those classes on top of this ABI.
 *
 * Conventions
 *  - Every function returns MRG8G_SUCCESS (0) or a negative error code;
 *    mrg8g_last_error() describes the last failure of the calling thread.
 *  - Device pointers are plain CUDA device addresses on the current device;
 *    `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Generation calls are stream-ordered and asynchronous; the handle's state
 *    advances on the host immediately, so the next call may be issued at once.
 *  - A handle is not thread-safe (neither is the reference); distinct handles
 *    may be used from distinct threads.
 *  - Output buffers must be aligned to their element size.
 */
#ifndef MRG8G_H
#define MRG8G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MRG8G_VERSION 1

#if defined(__GNUC__)
#define MRG8G_API __attribute__((visibility("default")))
#else
#define MRG8G_API
#endif

/* Return codes. */
#define MRG8G_SUCCESS 0
#define MRG8G_ERR_INVALID_ARGUMENT (-1)
#define MRG8G_ERR_INVALID_STATE (-2) /* state word >= 2^31, or all-zero state */
#define MRG8G_ERR_CUDA (-3)
#define MRG8G_ERR_OUT_OF_MEMORY (-4)
#define MRG8G_ERR_TIMEOUT (-5)
#define MRG8G_ERR_BUDGET (-6)
#define MRG8G_ERR_NOT_READY (-7)

/* Uniform scalings.  The reference uses both:
 *   ORIGINAL  u = S * rnorm          in (0, 1]  original/mrg8.cpp:231-237
 *   SHIFTED   u = (S - 1) * rnorm    in [0, 1)  cuda/mrg8_cuda.cu:251-252,363,
 *                                               knl/mrg8.h:353-362
 * with rnorm = 1.0 / (2^31 - 1) in double.  fp32 outputs are (float) of the
 * fp64 value (no fp32 path exists in the reference). */
#define MRG8G_ORIGINAL 0
#define MRG8G_SHIFTED 1

/* Output kinds for the generic entry points. */
#define MRG8G_U32 0          /* S in [1, 2^31-1]              */
#define MRG8G_F64_ORIGINAL 1
#define MRG8G_F64_SHIFTED 2
#define MRG8G_F32_ORIGINAL 3
#define MRG8G_F32_SHIFTED 4

typedef struct mrg8g_generator mrg8g_generator;

/* ---- lifetime, seeding and state ------------------------------------- */

/* Replaces mrg8::mrg8(seed) (original/mrg8.cpp:23-28) and
 * mrg8_cuda::mrg8_cuda(seed) (cuda/mrg8_cuda.cu:44-63).  Seeds with mcg64ni
 * (original/mrg8.cpp:180-194; seed 0 means 97531).  The jump tables are
 * generated on the host, not read from jump_matrix.txt. */
MRG8G_API int mrg8g_create(uint32_t seed, mrg8g_generator **out);

/* No reference counterpart (the reference classes have no destructor and
 * leak their device memory, cuda/mrg8_cuda.h:20-45). */
MRG8G_API int mrg8g_destroy(mrg8g_generator *g);

/* Replaces mrg8::seed_init (original/mrg8.cpp:31-34) and
 * mrg8_cuda::seed_init (cuda/mrg8_cuda.cu:66-70). */
MRG8G_API int mrg8g_seed_init(mrg8g_generator *g, uint32_t seed);

/* Replaces mrg8::get_state (original/mrg8.cpp:36-39) and, because the state
 * is always current here, mrg8_cuda::state_cpy_DtH (cuda/mrg8_cuda.cu:72-79).
 * st[0] = S[n-1] ... st[7] = S[n-8]. */
MRG8G_API int mrg8g_get_state(const mrg8g_generator *g, uint32_t st[8]);

/* Replaces mrg8::set_state (original/mrg8.cpp:56-59).  Unlike the reference
 * CUDA class the new state also governs later device calls.  Words must be
 * below 2^31 and not all zero (MRG8G_ERR_INVALID_STATE otherwise; the
 * reference overflows or emits a constant stream on such input). */
MRG8G_API int mrg8g_set_state(mrg8g_generator *g, const uint32_t st[8]);

/* ---- jump-ahead ------------------------------------------------------- */

/* Replaces mrg8::jump_ahead(uint64_t) (original/mrg8.cpp:125-129): the
 * handle's state advances by k outputs. */
MRG8G_API int mrg8g_jump_ahead(mrg8g_generator *g, uint64_t k);

/* Replaces mrg8::jump_ahead(const short[200]) (original/mrg8.cpp:104-122):
 * bits[i] != 0 sets bit i of a 200-bit jump distance (bits[0] = LSB). */
MRG8G_API int mrg8g_jump_ahead_bits(mrg8g_generator *g, const short bits[200]);

/* Replaces mrg8::jump_ahead(uint64_t, uint32_t*) (cuda/mrg8.cpp:145-150,
 * knl/mrg8.h:212-238): writes the state k outputs ahead, handle unchanged. */
MRG8G_API int mrg8g_jump_state(const mrg8g_generator *g, uint64_t k, uint32_t new_state[8]);

/* Replaces mrg8::jump_ahead(const short[200], uint32_t*) (cuda/mrg8.cpp:127-141). */
MRG8G_API int mrg8g_jump_state_bits(const mrg8g_generator *g, const short bits[200], uint32_t new_state[8]);

/* ---- bulk generation into device memory ------------------------------- */

/* Replaces mrg8::randint(uint32_t*, int) (original/mrg8.cpp:197-222) for a
 * device buffer: the next n stream values S in [1, 2^31-1]. */
MRG8G_API int mrg8g_randint(mrg8g_generator *g, uint32_t *d_out, uint64_t n, void *stream);

/* Replaces mrg8::rand(double*, int) (original/mrg8.cpp:231-239, ORIGINAL)
 * and mrg8_cuda::mrg8_outer_32 / mrg8_inner (cuda/mrg8_cuda.cu:402-436,
 * SHIFTED) for a device buffer: the next n uniforms in fp64. */
MRG8G_API int mrg8g_rand(mrg8g_generator *g, double *d_out, uint64_t n, int scaling, void *stream);

/* fp32 uniforms: (float) of the fp64 value of mrg8g_rand. */
MRG8G_API int mrg8g_rand_f32(mrg8g_generator *g, float *d_out, uint64_t n, int scaling, void *stream);

/* Generic form of the three above (kind = MRG8G_U32 ... MRG8G_F32_SHIFTED). */
MRG8G_API int mrg8g_generate(mrg8g_generator *g, void *d_out, uint64_t n, int kind, void *stream);

/* ---- bulk generation into host memory --------------------------------- */

/* The reference's host calls (mrg8::randint / rand / mrg8dnz2, e.g.
 * original/mrg8.cpp:197-239, cuda/mrg8.cpp:290-339) for a host buffer: the
 * values are generated on the GPU in chunks through a per-handle device
 * staging area and copied back; returns when h_out is complete.  Pinned
 * host memory gives the full copy bandwidth. */
MRG8G_API int mrg8g_generate_host(mrg8g_generator *g, void *h_out, uint64_t n, int kind);

/* One instance through the bulk kernel without a handle: the n outputs of
 * `kind` that follow the first `offset` outputs after state st.  This is the
 * per-instance path (one launch per generator) that the batch entry points
 * replace. */
MRG8G_API int mrg8g_generate_from_state(const uint32_t st[8], uint64_t offset, void *d_out, uint64_t n,
                                        int kind, void *stream);

/* ---- batches of independent instances ---------------------------------- */

/* One generator instance of a batch: the n outputs of `kind` that follow the
 * first `offset` outputs after `state` go to the device buffer `out`.  A
 * batch replaces one mrg8_cuda object and one mrg8_outer_32 launch per
 * instance (cuda/mrg8_cuda.cu:414-436); every instance's values equal its own
 * sequential stream. */
typedef struct mrg8g_instance {
    uint32_t state[8]; /* as get_state (mrg8g_seed_state for a seed)      */
    uint64_t offset;   /* outputs skipped before the first one written     */
    uint64_t n;        /* outputs                                          */
    void *out;         /* device pointer aligned to the element size       */
    int32_t kind;      /* MRG8G_U32 ... MRG8G_F32_SHIFTED                   */
    int32_t reserved;  /* 0                                                */
} mrg8g_instance;

/* Launch shape of a batch; zero fields take the defaults. */
typedef struct mrg8g_batch_config {
    int32_t tile_rows;     /* warp rows per tile, multiple of 8 (512)        */
    int32_t threads;       /* threads per block, 128 or 256 (128)            */
    int32_t blocks_per_sm; /* resident blocks per SM cap (0 = occupancy max) */
    int32_t use_graph;     /* 1: launch through a captured CUDA graph        */
    int32_t tiling;        /* 0: the host lists every tile, longest first;
                              1: the kernel derives the tiles from per-instance
                              tile counts (instances longest first): host work
                              and descriptor bytes O(instances), not O(tiles) */
} mrg8g_batch_config;

typedef struct mrg8g_batch mrg8g_batch;

/* Plan a batch: validates the instances, cuts them into tiles (longest
 * first) and uploads the descriptors.  cfg may be NULL (defaults, graph on).
 * No reference counterpart (the reference has one object per stream). */
MRG8G_API int mrg8g_batch_create(const mrg8g_instance *inst, uint64_t count, const mrg8g_batch_config *cfg,
                                 mrg8g_batch **out);

/* Enqueue the whole batch on `stream`: one persistent kernel (plus the reset
 * of its work counter), through the plan's CUDA graph when use_graph = 1.
 * Launches of one plan must not overlap each other on the device. */
MRG8G_API int mrg8g_batch_launch(mrg8g_batch *b, void *stream);

/* The per-instance path the batch replaces: one bulk-kernel launch per
 * instance (as one mrg8_cuda::mrg8_outer_32 call per object,
 * cuda/mrg8_cuda.cu:414-436), all on `stream`.  Same values as a batch. */
MRG8G_API int mrg8g_generate_each(const mrg8g_instance *inst, uint64_t count, void *stream);

/* Largest batch accepted by mrg8g_batch_generate_noalloc. */
#define MRG8G_NOALLOC_MAX_INSTANCES 4096
/* Body tiles hold 32,768 outputs (512 warp rows of 64); an instance whose
 * output does not start on a 16-byte boundary takes one extra head tile. */
#define MRG8G_NOALLOC_MAX_TILES 65536

/* Allocation-free form of a batch.  No reference counterpart: the reference
 * has no batches, and this entry point exists for callers that may not
 * allocate device memory themselves -- code whose host application or
 * framework allocator owns all of the GPU's memory, and latency-critical loops
 * that cannot take cudaMalloc/cudaFree's device-wide synchronisation.  It
 * generates the same values as mrg8g_batch_create + mrg8g_batch_launch but
 * calls no cudaMalloc, cudaFree or other allocating routine: the work queue,
 * instance descriptors and tiles live in a fixed scratch array inside the
 * library (about 1.3 MB, held on every GPU that loads the library until the
 * process exits).  The caller still passes the instance array (host memory)
 * and the output buffers.  Limits: at most MRG8G_NOALLOC_MAX_INSTANCES
 * instances and MRG8G_NOALLOC_MAX_TILES tiles per call (MRG8G_ERR_BUDGET
 * beyond).  The first call on a device looks up the scratch array's device
 * address (and uploads the jump tables if nothing else did), so make that
 * first call before any stream capture.  The descriptors are copied from a
 * host staging area inside the library that every call rewrites, so a call
 * on a stream that is capturing is refused (MRG8G_ERR_INVALID_ARGUMENT,
 * nothing enqueued).  All calls share the one array: two calls whose work
 * overlaps on the GPU (different streams without ordering) race; calls on the
 * same stream are ordered. */
MRG8G_API int mrg8g_batch_generate_noalloc(const mrg8g_instance *inst, uint64_t count, void *stream);

/* Time the candidate shapes on this batch (tile rows 128..2048 x 128 or 256
 * threads x both tilings; synchronises `stream`), keep the fastest and report
 * it in *chosen (may be NULL). */
MRG8G_API int mrg8g_batch_autotune(mrg8g_batch *b, void *stream, mrg8g_batch_config *chosen);

MRG8G_API int mrg8g_batch_get_config(const mrg8g_batch *b, mrg8g_batch_config *cfg);
/* Change the launch shape.  A new tiling rewrites the plan's device
 * descriptors, so this first waits for the plan's last launch (on whatever
 * stream it went); a launch made while its stream was capturing is not
 * tracked: do not change the plan while a graph that holds it may run. */
MRG8G_API int mrg8g_batch_set_config(mrg8g_batch *b, const mrg8g_batch_config *cfg);
MRG8G_API int mrg8g_batch_stats(const mrg8g_batch *b, uint64_t *tiles, uint64_t *outputs, uint64_t *bytes);
MRG8G_API int mrg8g_batch_destroy(mrg8g_batch *b);

/* ---- serving: continuous batching of draw requests ---------------------- */

/* A server keeps generator states resident on the device and serves draw
 * requests: a scheduler thread admits them first-in first-out against a
 * device output arena (the admission budget), packs whatever is admitted into
 * one batch launch (the batch kernel above) on one of `inflight` streams, and
 * keeps admitting and launching while earlier batches run, so requests that
 * arrive while others are on the GPU are admitted as slots and memory free up
 * and their work overlaps on the device.  Each result equals the request's own
 * stream segment whatever else is in flight.  No reference counterpart. */
typedef struct mrg8g_server_config {
    uint64_t budget_bytes;   /* output arena = admission budget (0: 16 GiB)  */
    uint32_t max_batch;      /* requests per launch at most (0: 1024)        */
    uint32_t inflight;       /* launches in flight, one stream each (0: 3)   */
    uint32_t max_generators; /* device-resident generator slots (0: 65536)   */
    int32_t tile_rows;       /* batch-kernel tile rows at most (0: 256); a
                                launch too small to fill the GPU with such
                                tiles uses shorter ones (16 rows at least)  */
    int32_t threads;         /* batch-kernel block size, 128 or 256 (0: 128) */
    int32_t spin_us;         /* the scheduler thread stays awake (one busy
                                host core) this long after its last
                                activity: 0 = 2000 us, < 0 = sleep as soon as
                                nothing is in flight (lower CPU use, higher
                                latency for the next request)               */
} mrg8g_server_config;

#define MRG8G_NO_GENERATOR 0xFFFFFFFFu

typedef struct mrg8g_request {
    uint32_t generator; /* slot of a registered generator (its draws continue
                           its stream), or MRG8G_NO_GENERATOR              */
    uint32_t seed;      /* without a generator: the stream seeded by `seed` */
    uint64_t offset;    /* ... starting `offset` outputs in                 */
    uint64_t n;         /* outputs                                          */
    int32_t kind;       /* MRG8G_U32 ... MRG8G_F32_SHIFTED                   */
    int32_t reserved;   /* 0                                                */
    uint64_t tag;       /* returned with the completion                     */
} mrg8g_request;

typedef struct mrg8g_completion {
    uint64_t ticket;
    uint64_t tag;
    void *out;          /* device pointer to the n outputs, valid until
                           mrg8g_server_release(ticket)                     */
    uint64_t n;
    int32_t kind;
    int32_t status;     /* MRG8G_SUCCESS or the error that failed the batch */
    double t_submit, t_admit, t_done; /* host steady clock, seconds         */
} mrg8g_completion;

typedef struct mrg8g_server_stats {
    uint64_t submitted, completed, pending, launches, launched_requests, samples;
    uint64_t bytes_in_use, peak_bytes;
    int32_t error, reserved;
    /* Most launches in flight at once (enqueued, completion not yet seen). */
    uint64_t max_inflight;
    /* Launches whose kernel ran on the device at the same time as another
     * launch's kernel (intervals from the device's global timer, stamped by
     * the kernel's first and last blocks). */
    uint64_t overlapped_launches;
    double mean_batch; /* launched_requests / launches */
    /* Device time of the launches with a kernel, first block's start to last
     * block's end (global timer), summed, and how many launches it covers. */
    uint64_t kernel_ns, kernel_launches;
} mrg8g_server_stats;

typedef struct mrg8g_server mrg8g_server;

MRG8G_API int mrg8g_server_create(const mrg8g_server_config *cfg, mrg8g_server **out);
/* Register a generator (its state goes to the device table); *slot names it. */
MRG8G_API int mrg8g_server_add_generator(mrg8g_server *s, const uint32_t state[8], uint32_t *slot);
/* The generator's state after every draw submitted so far. */
MRG8G_API int mrg8g_server_generator_state(mrg8g_server *s, uint32_t slot, uint32_t state[8]);
/* Queue a request (thread-safe, returns at once); MRG8G_ERR_BUDGET if it can
 * never fit the arena. */
MRG8G_API int mrg8g_server_submit(mrg8g_server *s, const mrg8g_request *req, uint64_t *ticket);
/* Up to `max` completed requests, waiting at most timeout_us for the first. */
MRG8G_API int mrg8g_server_poll(mrg8g_server *s, mrg8g_completion *out, uint32_t max, uint32_t *count,
                                uint32_t timeout_us);
/* Copy a completed request's outputs to host memory (bytes <= n * element
 * size; synchronous). */
MRG8G_API int mrg8g_server_read(mrg8g_server *s, uint64_t ticket, void *host, uint64_t bytes);
/* Give a completed request's output region back to the arena. */
MRG8G_API int mrg8g_server_release(mrg8g_server *s, uint64_t ticket);
MRG8G_API int mrg8g_server_get_stats(mrg8g_server *s, mrg8g_server_stats *st);
/* Stops the scheduler after the work in flight and frees everything. */
MRG8G_API int mrg8g_server_destroy(mrg8g_server *s);

/* Open-loop load test: Poisson arrivals at `rate` per second for
 * `duration_s`; lengths log-uniform in [n_min, n_max]; offsets uniform in
 * [0, offset_max); kinds uniform over the set bits of kinds_mask (bit k =
 * kind k); random seeds; each result held hold_us, then released. */
typedef struct mrg8g_loadtest_config {
    double rate, duration_s, hold_us;
    uint64_t n_min, n_max, offset_max, rng_seed;
    uint32_t kinds_mask, reserved;
} mrg8g_loadtest_config;

typedef struct mrg8g_loadtest_result {
    uint64_t requests, samples, bytes, launches, peak_bytes, late_submits;
    double wall_s, gsamples_per_s, mean_us, p50_us, p90_us, p99_us, max_us, mean_batch;
    /* over this run: most launches in flight at once, launches that
     * overlapped another on the device (peak_bytes is this run's too) */
    uint64_t max_inflight, overlapped_launches;
    /* mean device time of this run's launches (kernel_ns / kernel_launches) */
    double mean_kernel_us;
} mrg8g_loadtest_result;

MRG8G_API int mrg8g_server_loadtest(mrg8g_server *s, const mrg8g_loadtest_config *cfg, mrg8g_loadtest_result *res);

/* ---- utilities ---------------------------------------------------------- */

/* st = the state seeded from `seed` by mcg64ni (original/mrg8.cpp:180-194). */
MRG8G_API int mrg8g_seed_state(uint32_t seed, uint32_t st[8]);

/* Wait for the work queued on `stream` (NULL = legacy default stream).  The
 * synchronous drop-in methods use it: the reference synchronises the device
 * after each launch (cuda/mrg8_cuda.cu:409,423). */
MRG8G_API int mrg8g_stream_sync(void *stream);

/* Launch shape of the bulk kernel for one output kind, process-wide (set by
 * the autotuner): V = substreams per lane (1, 2 or 4; 0 = default for the
 * kind) and blocks_per_sm = resident blocks per SM (0 = occupancy maximum). */
MRG8G_API int mrg8g_tune_plain(int kind, int V, int blocks_per_sm);
MRG8G_API int mrg8g_get_plain_tuning(int kind, int *V, int *blocks_per_sm);

/* Uniforms from raw stream values: d_out[i] = scaling of d_in[i], where
 * d_in[i] must lie in [1, 2^31-1]; kind = MRG8G_F64_* or MRG8G_F32_*.
 * The conversion of rng_outer_32's epilogue (cuda/mrg8_cuda.cu:363). */
MRG8G_API int mrg8g_convert(const uint32_t *d_in, void *d_out, uint64_t n, int kind, void *stream);

/* Device batch of jumps: d_states[8 i .. 8 i + 7] = state st advanced by
 * d_offsets[i] outputs (the per-warp jump prologue of
 * cuda/mrg8_cuda.cu:313-337, generalised to 64-bit offsets). */
MRG8G_API int mrg8g_jump_states(const uint32_t st[8], const uint64_t *d_offsets, uint32_t *d_states,
                      uint64_t count, void *stream);

/* The jump table in the reference's file format (jump_matrix.txt, read by
 * original/mrg8.cpp:85-102): A^(2^j), j = 0..246, one matrix per line,
 * column-major ((r,c) at index r + 8c).  mrg8g_write_jump_matrix writes the
 * table this library generates; mrg8g_verify_jump_matrix parses a file and
 * compares it entry by entry (MRG8G_ERR_INVALID_STATE and *mismatches > 0 if
 * it differs; mismatches may be NULL). */
MRG8G_API int mrg8g_write_jump_matrix(const char *path);
MRG8G_API int mrg8g_verify_jump_matrix(const char *path, uint64_t *mismatches);

/* Description of the last error on the calling thread ("" if none). */
MRG8G_API const char *mrg8g_last_error(void);

/* MRG8G_VERSION of the loaded library. */
MRG8G_API int mrg8g_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MRG8G_H */
