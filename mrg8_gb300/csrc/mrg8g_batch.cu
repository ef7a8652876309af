// mrg8g_batch.cu -- batched generation of many independent instances.
#include "mrg8g_device.cuh"
#include "mrg8g_internal.h"
#include "mrg8g_runtime.h"

namespace mrg8g {

MRG8G_DEFINE_TABLE_UPLOAD(upload_tables_batch)

}  // namespace mrg8g
