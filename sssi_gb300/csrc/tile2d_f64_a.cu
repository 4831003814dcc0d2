// Tiled 2D CPML step, double, orders 1-4.
#include "tile2d_kernel.cuh"

namespace sssi {
SSSI_TILE2D_INSTANCE(double, 1)
SSSI_TILE2D_INSTANCE(double, 2)
SSSI_TILE2D_INSTANCE(double, 3)
SSSI_TILE2D_INSTANCE(double, 4)
}  // namespace sssi
