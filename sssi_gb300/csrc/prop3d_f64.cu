// 3D CPML step, FP64, orders 1-8.
#include "prop3d_kernel.cuh"

namespace sssi {
SSSI_PROP3D_INSTANCE(double, 1)
SSSI_PROP3D_INSTANCE(double, 2)
SSSI_PROP3D_INSTANCE(double, 3)
SSSI_PROP3D_INSTANCE(double, 4)
SSSI_PROP3D_INSTANCE(double, 5)
SSSI_PROP3D_INSTANCE(double, 6)
SSSI_PROP3D_INSTANCE(double, 7)
SSSI_PROP3D_INSTANCE(double, 8)
}  // namespace sssi
