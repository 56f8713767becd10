// Persistent multi-capture gather kernels for __nv_bfloat16 storage.
#include "batch_launch.cuh"

namespace fbp {
FBP_INSTANTIATE_BATCH(__nv_bfloat16)
}  // namespace fbp
