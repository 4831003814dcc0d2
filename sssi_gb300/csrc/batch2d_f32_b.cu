// Batched 2D CPML step, float, orders 3-4.
#include "batch2d_kernel.cuh"

namespace sssi {
SSSI_BATCH2D_INSTANCE(float, 3)
SSSI_BATCH2D_INSTANCE(float, 4)
}  // namespace sssi
