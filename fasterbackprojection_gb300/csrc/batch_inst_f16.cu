// Persistent multi-capture gather kernels for __half storage.
#include "batch_launch.cuh"

namespace fbp {
FBP_INSTANTIATE_BATCH(__half)
}  // namespace fbp
