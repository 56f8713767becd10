// Persistent multi-capture gather kernels for float storage.
#include "batch_launch.cuh"

namespace fbp {
FBP_INSTANTIATE_BATCH(float)
}  // namespace fbp
