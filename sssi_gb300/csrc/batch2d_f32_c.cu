// Batched 2D CPML step, float, orders 5-6.
#include "batch2d_kernel.cuh"

namespace sssi {
SSSI_BATCH2D_INSTANCE(float, 5)
SSSI_BATCH2D_INSTANCE(float, 6)
}  // namespace sssi
