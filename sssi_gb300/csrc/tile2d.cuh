// Tile geometry and numerics shared by the tiled 2D CPML kernels (FP32 and
// fused FP64) for sm_103a; the kernel itself is batch2d_kernel.cuh.
//
// One persistent launch advances the grid by one time step.  Each CTA walks a
// strided list of TZ x TX tiles.  For every tile a single thread issues three
// TMA box copies into shared memory -- the current field with its halo (the
// P box: rows z0-HZ .. z0+TZ+HZ, columns x0-l .. x0+TX+l), the previous field
// and (v dt)^2 (TZ x TX each) -- double-buffered, so the copies of tile k+1
// overlap the arithmetic of tile k.  Each thread owns a block of 4 rows x RX
// columns and reads shared memory in 16-byte vectors: the z stencil of a
// column comes from one register window, the x stencil from RX + 2l column
// vectors streamed through registers.
//
// Interior tiles use the composed second-derivative stencil
//     Lz P(i) = a_0 P(i) + sum_{m=1..l} a_m (P(i+m) + P(i-m)),
// which is the staggered pair D-(D+ P) of the reference multiplied out (exact
// in real arithmetic wherever the CPML memory variables are zero).  Tiles whose
// stencil reaches a damped band use the two-stage form with the memory
// variables: A = D+P + phi, phi = b phi + (b-1) D+P, and D-A + psi.  In FP32
// the memory variables are carried as compensated (hi, lo) pairs; in FP64 as
// doubles.
#pragma once

#include "cpml2d.cuh"
#include <type_traits>

#include "tma.cuh"

namespace sssi {

template <typename T>
struct TileShape;
// TZ x TX cells per tile; each thread owns 4 rows x RX columns; kMinBlocks
// CTAs per SM is the register budget the compiler is held to.
template <>
struct TileShape<float> {
    static constexpr int TZ = 64, TX = 32, RX = 2;
    static constexpr int kThreads = (TZ / 4) * (TX / RX), kMinBlocks = 2;
};
template <>
struct TileShape<double> {
    static constexpr int TZ = 32, TX = 32, RX = 2;
    static constexpr int kThreads = (TZ / 4) * (TX / RX), kMinBlocks = 2;
};

// Tile shapes of the batched step: shape 0 is TileShape<T>; FP32 also has
// shape 1, 32 x 32 tiles with four blocks per SM, and shape 2, 128 x 16 tiles
// (a z-block twice as deep as shape 0's, half as wide).  The batch's tuner
// times the shapes on the first steps of a large schedule and keeps the
// fastest: the z-block depth (32, 64 or 128 rows) and the width that goes
// with it.
template <typename T, int V>
struct BatchShape;
template <typename T>
struct BatchShape<T, 0> : TileShape<T> {
    static constexpr int kIndex = 0;
};
template <>
struct BatchShape<float, 1> {
    static constexpr int TZ = 32, TX = 32, RX = 2;
    static constexpr int kThreads = (TZ / 4) * (TX / RX), kMinBlocks = 4;
    static constexpr int kIndex = 1;
};
template <>
struct BatchShape<float, 2> {
    static constexpr int TZ = 128, TX = 16, RX = 2;
    static constexpr int kThreads = (TZ / 4) * (TX / RX), kMinBlocks = 2;
    static constexpr int kIndex = 2;
};
constexpr int kMaxBatchShapes = 3;
template <typename T>
constexpr int kBatchShapes = std::is_same<T, float>::value ? 3 : 1;

template <typename T>
struct MemVar;
template <>
struct MemVar<double> {
    using type = double;
};
template <>
struct MemVar<float> {
    using type = float2;  // compensated sum hi + lo
};

// Rows of halo above and below a tile in the P box: l rounded up to 4 so that
// every row window starts on a 16-byte boundary.
__host__ __device__ constexpr int tile_halo_rows(int N) { return ((2 * N - 1) + 3) / 4 * 4; }

}  // namespace sssi
