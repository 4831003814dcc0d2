// Batched 2D CPML step, double, orders 5-8.
#include "batch2d_kernel.cuh"

namespace sssi {
SSSI_BATCH2D_INSTANCE(double, 5)
SSSI_BATCH2D_INSTANCE(double, 6)
SSSI_BATCH2D_INSTANCE(double, 7)
SSSI_BATCH2D_INSTANCE(double, 8)
}  // namespace sssi
