// Batched 2D CPML step, float, orders 1-2.
#include "batch2d_kernel.cuh"

namespace sssi {
SSSI_BATCH2D_INSTANCE(float, 1)
SSSI_BATCH2D_INSTANCE(float, 2)
}  // namespace sssi
