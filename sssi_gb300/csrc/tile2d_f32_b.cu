// Tiled 2D CPML step, float, orders 5-8.
#include "tile2d_kernel.cuh"

namespace sssi {
SSSI_TILE2D_INSTANCE(float, 5)
SSSI_TILE2D_INSTANCE(float, 6)
SSSI_TILE2D_INSTANCE(float, 7)
SSSI_TILE2D_INSTANCE(float, 8)
}  // namespace sssi
