// mrg8g_runtime.h -- host runtime helpers shared by the C ABI translation
// units (errors, per-device setup, launch planning, state bookkeeping).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <vector>

#include "mrg8g_internal.h"

namespace mrg8g {

struct DeviceInfo;

// Record an error for mrg8g_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// Make the current device ready (tables uploaded, limits queried).
int ensure_device(int* dev_out, const DeviceInfo** info);
int device_sms();

int kind_elem_bytes(int kind);
bool kind_valid(int kind);
int default_layout_V(int kind);
// Lane layout of the batch kernel for every kind: two substreams per lane
// keeps its register count (one kernel holds the code of all five kinds) low
// enough for eight resident blocks of 128 threads per SM.
constexpr int kBatchLayoutV = 2;

// BatchArgs::leap for the batch layout (both lag forms).
inline void set_batch_leaps(BatchArgs& a) {
    a.leap[0] = host_tables().leap[layout_index(kBatchLayoutV)];
    a.leap[1] = host_tables().leap_mod[layout_index(kBatchLayoutV)];
}
// Host -> device copy from pageable memory that has reached the device when
// it returns.  A plain cudaMemcpy from pageable memory may return once the
// data is staged, before the copy lands, and nothing orders that copy (on the
// legacy default stream) before work on a non-blocking stream, such as the
// serving slots or a caller's stream.
inline cudaError_t copy_to_device(void* dst, const void* src, size_t bytes) {
    cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    return e != cudaSuccess ? e : cudaStreamSynchronize(0);
}

int validate_state(const uint32_t st[8]);
void advance_state(uint32_t st[8], uint64_t n);
int launch_plain_call(const uint32_t st[8], void* d_out, uint64_t n, int kind, cudaStream_t s, int V);

cudaError_t upload_tables_batch();

}  // namespace mrg8g

// Tiles of a batch: make_tiles, sort_largest_first, count_tiles, tile_prefix.
#include "mrg8g_tiles.h"
