// Batched 2D CPML step, float, orders 7-8.
#include "batch2d_kernel.cuh"

namespace sssi {
SSSI_BATCH2D_INSTANCE(float, 7)
SSSI_BATCH2D_INSTANCE(float, 8)
}  // namespace sssi
