// 3D CPML step, FP32 (compensated memory variables), orders 1-8.
#include "prop3d_kernel.cuh"

namespace sssi {
SSSI_PROP3D_INSTANCE(float, 1)
SSSI_PROP3D_INSTANCE(float, 2)
SSSI_PROP3D_INSTANCE(float, 3)
SSSI_PROP3D_INSTANCE(float, 4)
SSSI_PROP3D_INSTANCE(float, 5)
SSSI_PROP3D_INSTANCE(float, 6)
SSSI_PROP3D_INSTANCE(float, 7)
SSSI_PROP3D_INSTANCE(float, 8)
}  // namespace sssi
