// Batched 2D CPML step, double, orders 1-4.
#include "batch2d_kernel.cuh"

namespace sssi {
SSSI_BATCH2D_INSTANCE(double, 1)
SSSI_BATCH2D_INSTANCE(double, 2)
SSSI_BATCH2D_INSTANCE(double, 3)
SSSI_BATCH2D_INSTANCE(double, 4)
}  // namespace sssi
