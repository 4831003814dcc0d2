// 2D acoustic propagation with the sponge absorbing boundary: forward
// modelling, reverse propagation and the RTM shot of
//   src/fwdTimeSpongeFor2dAw.m:36-101, src/rvsTimeSpongeFor2dAw.m:36-103,
//   applications/rtm_2d_acoustic/mainRtmTimeSpongeFor2dAw.m:160-161,247-268,310.
//
// The reference (MATLAB) advances a zero-bordered field with the second-order
// five-point update
//     fdm3 = b .* fdm2 - fdm1 + ax .* (right + left) + az .* (down + up) - vdtSq .* source
// (b = 2 - 2ax - 2az, ax = (v dt/dx)^2, az = (v dt/dz)^2, vdtSq = (v dt)^2),
// rotates (fdm1 <- fdm2, fdm2 <- fdm3) and then multiplies BOTH the new past
// and the new present by the sponge factors of the left / right columns
// (rows above the bottom band) and of the bottom rows (every column):
//     boundary(k) = exp(-(alpha (nB - k + 1))^2)^10,  alpha = 0.015.
// The past of the next step is therefore s .* (present of this step), which
// this kernel forms at the cell itself when it reads its previous value: one
// pair of field buffers, each step reading the present and overwriting the
// previous present of its own cell with s .* fdm3.  No cell is read by a
// neighbour after it is overwritten (neighbours read only the present).
//
// GB300 layout and launch: each field is (ldp rows) x (nx + 2 columns) with a
// zero border (row -1 and row nz, columns -1 and nx), every column's interior
// starting on a 32-element boundary; the coefficient arrays share the layout.
// A warp takes 32 rows (coalesced along z) and marches along x over a run
// of columns, so that each value of the present is fetched once; warps take
// tiles z-fastest from a persistent grid.  One step
// is one launch; runs of kSpGraphSteps steps replay a CUDA graph that reads the
// step number and the chunked hooks (sources, snapshots) from device memory.
//
// Arithmetic: SSSI_MODE_FP64_STRICT rounds every operation as the MATLAB
// expression is written (left to right, no fused multiply-add); SSSI_MODE_FP64
// fuses b*present - past, ax*(.) and az*(.) into multiply-adds; SSSI_MODE_FP32
// keeps the field in FP32 and derives ax, az, b from (v dt)^2 in the kernel
// (16 bytes of HBM traffic per cell and step).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "api_util.cuh"
#include "sssi_internal.h"

namespace sssi {
namespace {

using namespace api;

constexpr int kSpRows = 32;              // a warp's rows (one per lane)
constexpr int kSpThreads = 256;          // 8 warps, each an independent worker
constexpr int kSpOrgRow = 32;             // interior row 0 within a column (row -1 is zero padding)
constexpr int kSpGraphSteps = 32;
constexpr double kSpongeAlpha = 0.015;    // src/fwdTimeSpongeFor2dAw.m:45

// Per-chunk hooks, read from device memory by every launch (a captured graph
// keeps its launch parameters; these change between chunks).
template <typename T>
struct SpongeHooks {
    const T* src_dense;  // nz x nx slices (pitch nz), slice of step t at src_dense + (t - dense_t0) * nz * nx
    T* snap;             // the same layout for snapshots
    const T* fsnap;      // forward snapshots for imaging (t - fsnap_t0)
    int dense_t0, snap_t0, fsnap_t0, pad;
};

template <typename T>
struct SpongeParams {
    T* field[2];                // ping-pong fields (interior origin applied)
    const T* cb;                // FP64 modes: b, ax, az, (v dt)^2 (interior origin applied)
    const T* cax;
    const T* caz;
    const T* cvdt2;             // all modes: (v dt)^2
    const T* bnd;               // sponge factors, nB entries
    const SpongeHooks<T>* hooks;
    const int* step_base;       // device step counter (graph replays); the step is *step_base + step_offset
    int step_offset;
    int nz, nx, nB, nt;
    int64_t ldp;
    int ntz, ntiles;
    int march;                  // columns a warp marches over (a multiple of kSpAhead)
    int reverse;                // time runs nt-1 .. 0 and row 0 takes src_row
    T kx, kz, kxz2;             // FP32: 1/dx^2, 1/dz^2 (ax = vdt2 kx, az = vdt2 kz), 2 (kx + kz)
    // point sources (forward): cell (src_iz[k], src_ix[k]) adds wavelets[k * nt + t]
    int nsrc;
    const int* src_iz;
    const int* src_ix;
    const T* wavelets;
    const T* src_row;           // reverse: data, nx x nt (row 0 source of step t at src_row + t * nx)
    T* rec;                     // data, nx x nt: row 0 of the new present
    double* im;                 // imaging sums (FP64 fused RTM): M and S2, nz x nx (pitch nz)
    double* is2;
};

// The sponge factors of cell (i, j) applied to x in the order of the
// reference's loop (src/fwdTimeSpongeFor2dAw.m:80-90): for ixb = 2..nB+1 the
// left column ixb, the right column nx-nB+ixb, the bottom row nz-nB+ixb.  A
// cell is hit by the bottom rows alone or by the side columns of its row;
// both side columns hit it only when nx < 2 nB (the right one first unless
// nx == nB).
// The grid's sizes and the profile come by value (a reference to the
// __grid_constant__ parameter block would be read through generic loads,
// repeated after every store).
struct SpongeGeom {
    int nz, nx, nB;
};

template <typename T, int kMode>
__device__ __forceinline__ T sponge(T x, int i, int j, SpongeGeom g, const T* __restrict__ bnd) {
    const int nB = g.nB;
    if (i >= g.nz - nB) return kMode == SSSI_MODE_FP32 ? x * bnd[g.nz - 1 - i] : __dmul_rn(bnd[g.nz - 1 - i], x);
    const bool left = j < nB, right = j >= g.nx - nB;
    if (!(left | right)) return x;
    auto mul = [](T a, T b) -> T {
        if constexpr (kMode == SSSI_MODE_FP32)
            return a * b;
        else
            return __dmul_rn(a, b);
    };
    if (left && right) {
        const T bl = bnd[j], br = bnd[g.nx - 1 - j];
        return g.nx > nB ? mul(bl, mul(br, x)) : mul(br, mul(bl, x));
    }
    return mul(bnd[left ? j : g.nx - 1 - j], x);
}

// Loads issued ahead per thread in the FP32 step: the columns a warp fetches
// before it computes them (memory-level parallelism of the HBM-bound stream).
template <typename T>
constexpr int kSpAhead = 4;

// The update of one cell from its five present values, its own previous
// present po (not yet damped) and its coefficients; kGeneral adds the sponge
// factors and the injected value src (has_src), which interior tiles without
// sources skip.
template <typename T>
struct SpongeK {
    T kx, kz, kxz2;  // FP32 mode: ax = vdt2 kx, az = vdt2 kz, b = 2 - vdt2 kxz2
};

template <typename T, int kMode, bool kGeneral>
__device__ __forceinline__ T sponge_cell(SpongeGeom g, const T* __restrict__ bnd, SpongeK<T> k, int i, int j, T c,
                                         T up, T dn, T lf, T rt, T po, T vdt2, T cb, T cx, T cz, bool has_src,
                                         T src) {
    const T past = kGeneral ? sponge<T, kMode>(po, i, j, g, bnd) : po;
    T r;
    if constexpr (kMode == SSSI_MODE_FP64_STRICT) {
        r = __dsub_rn(__dmul_rn(cb, c), past);
        r = __dadd_rn(r, __dmul_rn(cx, __dadd_rn(rt, lf)));
        r = __dadd_rn(r, __dmul_rn(cz, __dadd_rn(dn, up)));
        if (kGeneral && has_src) r = __dsub_rn(r, __dmul_rn(vdt2, src));
    } else if constexpr (kMode == SSSI_MODE_FP64) {
        r = fma(cb, c, -past);
        r = fma(cx, rt + lf, r);
        r = fma(cz, dn + up, r);
        if (kGeneral && has_src) r = fma(-vdt2, src, r);
    } else {
        const T ax = vdt2 * k.kx, az = vdt2 * k.kz;
        const T b = fmaf(-vdt2, k.kxz2, T(2));  // 2 - 2 ax - 2 az
        r = fmaf(b, c, -past);
        r = fmaf(ax, rt + lf, r);
        r = fmaf(az, dn + up, r);
        if (kGeneral && has_src) r = fmaf(-vdt2, src, r);
    }
    return kGeneral ? sponge<T, kMode>(r, i, j, g, bnd) : r;
}

// The FP32 step.  A warp owns 64 rows, two consecutive ones per lane (one
// 8-byte access), and marches along x over p.march columns, keeping left /
// centre / right of the present in registers (each value of the present is
// fetched once by its owner); the neighbours across lanes come from shuffles,
// the tile's edge rows from two predicated loads, and the update of a lane's
// two cells is one packed two-lane sequence.  Lanes below the grid fetch zero
// padding and store nothing.  A tile clear of the sponge bands, row 0 and every
// source (the common case) takes the lean update; the others go cell by cell.
constexpr int kSpMarchRows = 64;

template <typename T, int kMode>
__global__ void __launch_bounds__(kSpThreads, 3) sponge2d_march_kernel(const __grid_constant__ SpongeParams<T> p) {
    static_assert(kMode == SSSI_MODE_FP32 && std::is_same<T, float>::value, "the marching step is the FP32 form");
    constexpr int U = kSpAhead<T>;
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int step = *reinterpret_cast<volatile const int*>(p.step_base) + p.step_offset;
    const int t = p.reverse ? p.nt - 1 - step : step;
    const float* __restrict__ cur = p.field[step & 1];
    float* __restrict__ nxt = p.field[(step & 1) ^ 1];
    const SpongeHooks<float> h = *p.hooks;
    const int64_t n = (int64_t)p.nz * p.nx;
    const float* src_dense = h.src_dense ? h.src_dense + (int64_t)(t - h.dense_t0) * n : nullptr;
    float* snap = h.snap ? h.snap + (int64_t)(t - h.snap_t0) * n : nullptr;
    const int lane = threadIdx.x & 31;
    const int64_t ldp = p.ldp;
    const int nwarps = gridDim.x * (kSpThreads / 32);
    const SpongeGeom g{p.nz, p.nx, p.nB};
    const SpongeK<float> kk{p.kx, p.kz, p.kxz2};
    const float* __restrict__ bnd = p.bnd;
    const float2 kx2 = make_float2(p.kx, p.kx), kz2 = make_float2(p.kz, p.kz), kxz2 = make_float2(p.kxz2, p.kxz2);
    const float2 two = make_float2(2.0f, 2.0f);
    for (int tile = blockIdx.x * (kSpThreads / 32) + (threadIdx.x >> 5); tile < p.ntiles; tile += nwarps) {
        const int tz = tile % p.ntz, tx = tile / p.ntz;
        const int i0 = tz * kSpMarchRows, i = i0 + 2 * lane, j0 = tx * p.march;
        const int jend = min(j0 + p.march, p.nx);
        const bool ok0 = i < p.nz, ok1 = i + 1 < p.nz;
        // warp-uniform: does the tile touch a sponge band, row 0 or a point source?
        bool general = i0 + kSpMarchRows > p.nz - p.nB || j0 < p.nB || jend > p.nx - p.nB || src_dense ||
                       ((p.src_row || p.rec) && i0 == 0) || snap;
        for (int k = 0; k < p.nsrc; ++k) {
            const int si = p.src_iz[k], sj = p.src_ix[k];
            general |= si >= i0 && si < i0 + kSpMarchRows && sj >= j0 && sj < jend;
        }
        const int64_t q0 = i + (int64_t)j0 * ldp;
        const float* pc = cur + q0;  // (i, j) of the column being computed
        float* pn = nxt + q0;
        const float* pv = p.cvdt2 + q0;
        float2 lf = __ldg(reinterpret_cast<const float2*>(pc - ldp));
        float2 c = __ldg(reinterpret_cast<const float2*>(pc));
        for (int jb = j0; jb < jend; jb += U) {
            float2 rt[U], po[U], vd[U];
            float eg[U];
            const bool whole = jb + U <= jend;  // warp-uniform; a partial group only at the grid's last column
#pragma unroll
            for (int u = 0; u < U; ++u) {
                // past the end: a repeat of the last column, unused
                const int64_t o = whole ? (int64_t)u * ldp : (int64_t)min(u, jend - 1 - jb) * ldp;
                rt[u] = __ldg(reinterpret_cast<const float2*>(pc + o + ldp));
                po[u] = *reinterpret_cast<const float2*>(pn + o);
                vd[u] = __ldg(reinterpret_cast<const float2*>(pv + o));
                eg[u] = lane == 0 ? __ldg(pc + o - 1) : (lane == 31 ? __ldg(pc + o + 2) : 0.0f);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = jb + u;
                if (j >= jend) break;  // warp-uniform
                const float up_s = __shfl_up_sync(0xffffffffu, c.y, 1), dn_s = __shfl_down_sync(0xffffffffu, c.x, 1);
                const float up0 = lane == 0 ? eg[u] : up_s;   // row i - 1
                const float dn1 = lane == 31 ? eg[u] : dn_s;  // row i + 2
                const int64_t o = (int64_t)u * ldp;
                float2 out;
                if (!general) {
                    const float2 v = vd[u];
                    const float2 ax = __fmul2_rn(v, kx2), az = __fmul2_rn(v, kz2);
                    const float2 b = __ffma2_rn(make_float2(-v.x, -v.y), kxz2, two);  // 2 - 2 ax - 2 az
                    float2 r = __ffma2_rn(b, c, make_float2(-po[u].x, -po[u].y));
                    r = __ffma2_rn(ax, __fadd2_rn(rt[u], lf), r);
                    r = __ffma2_rn(az, __fadd2_rn(make_float2(c.y, dn1), make_float2(up0, c.x)), r);
                    out = r;
                } else {
                    // the general update of each of the lane's two cells
                    float res[2] = {0.0f, 0.0f};
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int ii = i + e;
                        if (ii >= p.nz) continue;
                        const float cc = e ? c.y : c.x, up = e ? c.x : up0, dn = e ? dn1 : c.y;
                        const float lfe = e ? lf.y : lf.x, rte = e ? rt[u].y : rt[u].x;
                        const float poe = e ? po[u].y : po[u].x, vde = e ? vd[u].y : vd[u].x;
                        float src = 0.0f;
                        bool has_src = false;
                        if (src_dense) {
                            src = src_dense[ii + (int64_t)j * p.nz];
                            has_src = true;
                        }
                        if (p.src_row && ii == 0) {
                            src = p.src_row[j + (int64_t)t * p.nx];
                            has_src = true;
                        }
                        for (int k = 0; k < p.nsrc; ++k)
                            if (p.src_iz[k] == ii && p.src_ix[k] == j) {
                                const float wv = p.wavelets[(int64_t)k * p.nt + t];
                                src = has_src ? src + wv : wv;
                                has_src = true;
                            }
                        res[e] = sponge_cell<float, kMode, true>(g, bnd, kk, ii, j, cc, up, dn, lfe, rte, poe, vde,
                                                                 0.0f, 0.0f, 0.0f, has_src, src);
                        if (p.rec && ii == 0) p.rec[j + (int64_t)t * p.nx] = res[e];
                        if (snap) snap[ii + (int64_t)j * p.nz] = res[e];
                    }
                    out = make_float2(res[0], res[1]);
                }
                if (ok1)
                    *reinterpret_cast<float2*>(pn + o) = out;
                else if (ok0)
                    pn[o] = out.x;
                lf = c;
                c = rt[u];
            }
            const int64_t adv = (int64_t)U * ldp;
            pc += adv;
            pn += adv;
            pv += adv;
        }
    }
}

// The FP64 step: FP64 is bound by its pipe (about 5 to 8 FP64 operations a
// cell), so every thread takes one cell of a 32-row x 8-column block tile
// (one warp per column) and the SM holds as many warps as it can; the x
// neighbours of a tile's inner columns come from L1.
constexpr int kSpCellCols = kSpThreads / 32;

template <typename T, int kMode>
__global__ void __launch_bounds__(kSpThreads) sponge2d_cell_kernel(const __grid_constant__ SpongeParams<T> p) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int step = *reinterpret_cast<volatile const int*>(p.step_base) + p.step_offset;
    const int t = p.reverse ? p.nt - 1 - step : step;
    const T* __restrict__ cur = p.field[step & 1];
    T* __restrict__ nxt = p.field[(step & 1) ^ 1];
    const SpongeHooks<T> h = *p.hooks;
    const int64_t n = (int64_t)p.nz * p.nx;
    const T* src_dense = h.src_dense ? h.src_dense + (int64_t)(t - h.dense_t0) * n : nullptr;
    T* snap = h.snap ? h.snap + (int64_t)(t - h.snap_t0) * n : nullptr;
    const T* fsnap = h.fsnap ? h.fsnap + (int64_t)(t - h.fsnap_t0) * n : nullptr;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t ldp = p.ldp;
    const SpongeGeom g{p.nz, p.nx, p.nB};
    const SpongeK<T> kk{p.kx, p.kz, p.kxz2};
    const T* __restrict__ bnd = p.bnd;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int tz = tile % p.ntz, tx = tile / p.ntz;
        const int i0 = tz * kSpRows, j0 = tx * kSpCellCols;
        const int i = i0 + lane, j = j0 + w;
        // block-uniform: does the tile touch a sponge band, row 0 or a point source?
        bool general = i0 + kSpRows > p.nz - p.nB || j0 < p.nB || j0 + kSpCellCols > p.nx - p.nB || src_dense ||
                       i0 == 0;
        for (int k = 0; k < p.nsrc; ++k) {
            const int si = p.src_iz[k], sj = p.src_ix[k];
            general |= si >= i0 && si < i0 + kSpRows && sj >= j0 && sj < j0 + kSpCellCols;
        }
        if (i >= p.nz || j >= p.nx) continue;
        const int64_t q = i + (int64_t)j * ldp;
        const T c = __ldg(cur + q), up = __ldg(cur + q - 1), dn = __ldg(cur + q + 1);
        const T lf = __ldg(cur + q - ldp), rt = __ldg(cur + q + ldp);
        const T po = nxt[q], vdt2 = __ldg(p.cvdt2 + q);
        const T cb = __ldg(p.cb + q), cx = __ldg(p.cax + q), cz = __ldg(p.caz + q);
        T out;
        if (!general) {
            out = sponge_cell<T, kMode, false>(g, bnd, kk, i, j, c, up, dn, lf, rt, po, vdt2, cb, cx, cz, false, T(0));
        } else {
            T src = T(0);
            bool has_src = false;
            if (src_dense) {
                src = src_dense[i + (int64_t)j * p.nz];
                has_src = true;
            }
            if (p.src_row && i == 0) {
                src = p.src_row[j + (int64_t)t * p.nx];
                has_src = true;
            }
            for (int k = 0; k < p.nsrc; ++k)
                if (p.src_iz[k] == i && p.src_ix[k] == j) {
                    const T wv = p.wavelets[(int64_t)k * p.nt + t];
                    src = has_src ? src + wv : wv;
                    has_src = true;
                }
            out = sponge_cell<T, kMode, true>(g, bnd, kk, i, j, c, up, dn, lf, rt, po, vdt2, cb, cx, cz, has_src, src);
            if (p.rec && i == 0) p.rec[j + (int64_t)t * p.nx] = out;
        }
        nxt[q] = out;
        if (snap || fsnap) {
            const int64_t qd = i + (int64_t)j * p.nz;
            if (snap) snap[qd] = out;
            if constexpr (kMode == SSSI_MODE_FP64) {
                if (fsnap) {
                    const double f = fsnap[qd];
                    p.im[qd] = fma(f, (double)out, p.im[qd]);
                    p.is2[qd] = fma(f, f, p.is2[qd]);
                }
            }
        }
    }
}

template <typename T, int kMode>
void launch_sponge_step(const SpongeParams<T>& p, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSpThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if constexpr (kMode == SSSI_MODE_FP32)
        SSSI_CHECK_CUDA(cudaLaunchKernelEx(&cfg, sponge2d_march_kernel<T, kMode>, p));
    else
        SSSI_CHECK_CUDA(cudaLaunchKernelEx(&cfg, sponge2d_cell_kernel<T, kMode>, p));
    count_launch();
}

// The sponge profile boundary(1..nB) of src/fwdTimeSpongeFor2dAw.m:43-46,
// evaluated as written: (exp(-(alpha (nB - iz))^2))^10 for iz = 0..nB-1.
std::vector<double> sponge_profile(int nB) {
    std::vector<double> b((size_t)nB);
    for (int iz = 0; iz < nB; ++iz) {
        const double a = kSpongeAlpha * (double)(nB - iz);
        b[(size_t)iz] = std::pow(std::exp(-(a * a)), 10.0);
    }
    return b;
}

// ax = (v dt/dx)^2, az = (v dt/dz)^2, vdtSq = (v dt)^2 and b = 2 - 2ax - 2az
// rounded as the MATLAB expressions are written (explicit round-to-nearest
// operations: nothing is fused), into the padded layout (interior origin
// applied to the outputs; b, ax, az only in the FP64 modes).
template <typename T>
__global__ void sponge_coef_kernel(const double* v, int nz, int nx, int64_t ldp, double dz, double dx, double dt,
                                   T* vdt2, T* b, T* ax, T* az) {
    const int64_t n = (int64_t)nz * nx;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q % nz, j = q / nz, o = i + j * ldp;
        const double vdt = __dmul_rn(v[q], dt);
        const double tx = __ddiv_rn(vdt, dx), tz = __ddiv_rn(vdt, dz);
        const double cx = __dmul_rn(tx, tx), cz = __dmul_rn(tz, tz);
        vdt2[o] = (T)__dmul_rn(vdt, vdt);
        if (b) {
            ax[o] = (T)cx;
            az[o] = (T)cz;
            b[o] = (T)__dsub_rn(__dsub_rn(2.0, __dmul_rn(2.0, cx)), __dmul_rn(2.0, cz));
        }
    }
}

// One propagation (forward or reverse) of one shot: fields, coefficients,
// hooks and the step loop (graphs of kSpGraphSteps steps).
template <typename T>
class Sponge2d {
  public:
    // v: the velocity model in device memory (nz x nx doubles)
    Sponge2d(const double* v, int64_t nz, int64_t nx, int nB, double dz, double dx, double dt, int mode, int64_t nt,
             bool reverse, cudaStream_t s)
        : nz_((int)nz), nx_((int)nx), mode_(mode), s_(s) {
        // rows: kSpOrgRow above the interior, then the interior rounded up to whole
        // 32-row tiles plus one more row of zeros (row nz and the lanes below the grid)
        // interior rows rounded up to whole tiles (64 rows in FP32, 32 in FP64),
        // plus one more tile row of zeros (row nz and the lanes below the grid)
        const int trows = mode == SSSI_MODE_FP32 ? kSpMarchRows : kSpRows;
        ldp_ = (int64_t)kSpOrgRow + (nz + trows - 1) / trows * trows + trows;
        const int64_t cols = nx + 2;
        const size_t cells = (size_t)(ldp_ * cols);
        org_ = kSpOrgRow + ldp_;  // interior (0, 0): row kSpOrgRow of column 1
        for (auto& f : F_) {
            f.allocate(cells * sizeof(T));
            f.zero(s);
        }
        // coefficients as the reference forms them (src/fwdTimeSpongeFor2dAw.m:51-55),
        // on the device from v (device memory, nz x nx); the padding stays zero
        const bool fp64 = mode != SSSI_MODE_FP32;
        auto make = [&](DeviceBuffer& d) {
            d.allocate(cells * sizeof(T));
            d.zero(s);
            return d.template as<T>() + org_;
        };
        T* dv2 = make(vdt2_);
        T *db = nullptr, *dax = nullptr, *daz = nullptr;
        if (fp64) {
            db = make(b_);
            dax = make(ax_);
            daz = make(az_);
        }
        sponge_coef_kernel<T><<<152 * 4, 256, 0, s>>>(v, (int)nz, (int)nx, ldp_, dz, dx, dt, dv2, db, dax, daz);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        const std::vector<double> prof = sponge_profile(nB);
        std::vector<T> hp(prof.begin(), prof.end());
        bnd_.allocate(std::max<size_t>(hp.size(), 1) * sizeof(T));
        if (!hp.empty())
            SSSI_CHECK_CUDA(cudaMemcpyAsync(bnd_.get(), hp.data(), hp.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        hooks_dev_.allocate(sizeof(SpongeHooks<T>));
        ctr_.allocate(sizeof(int));
        ctr_.zero(s);

        p_ = SpongeParams<T>{};
        p_.field[0] = F_[0].template as<T>() + org_;
        p_.field[1] = F_[1].template as<T>() + org_;
        p_.cvdt2 = vdt2_.template as<T>() + org_;
        if (fp64) {
            p_.cb = b_.template as<T>() + org_;
            p_.cax = ax_.template as<T>() + org_;
            p_.caz = az_.template as<T>() + org_;
        }
        p_.bnd = bnd_.template as<T>();
        p_.hooks = hooks_dev_.template as<SpongeHooks<T>>();
        p_.step_base = ctr_.template as<int>();
        p_.nz = nz_;
        p_.nx = nx_;
        p_.nB = nB;
        p_.nt = (int)nt;
        p_.ldp = ldp_;
        p_.ntz = mode == SSSI_MODE_FP32 ? (nz_ + kSpMarchRows - 1) / kSpMarchRows : (nz_ + kSpRows - 1) / kSpRows;
        p_.reverse = reverse ? 1 : 0;
        p_.kx = (T)(1.0 / (dx * dx));
        p_.kz = (T)(1.0 / (dz * dz));
        p_.kxz2 = (T)(2.0 * (1.0 / (dx * dx) + 1.0 / (dz * dz)));
        int dev = 0, sms = 0;
        SSSI_CHECK_CUDA(cudaGetDevice(&dev));
        SSSI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int per_sm = 0;
        if (mode == SSSI_MODE_FP32) {
            SSSI_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, (const void*)sponge2d_march_kernel<float, SSSI_MODE_FP32>, kSpThreads, 0));
            per_sm = std::max(per_sm, 1);
            // each warp takes every nwarps-th tile, so the step lasts ceil(tiles / warps)
            // tiles of (march + 1) column loads (the +1: the column left of a tile):
            // the march with the smallest such cost, the longer one on a tie
            const int64_t warps = (int64_t)sms * per_sm * (kSpThreads / 32);
            int march = 4;
            int64_t best = -1;
            for (int m = 64; m >= 4; m /= 2) {
                const int64_t tiles = (int64_t)p_.ntz * ((nx_ + m - 1) / m);
                const int64_t cost = (tiles + warps - 1) / warps * (m + 1);
                if (best < 0 || cost < best) {
                    best = cost;
                    march = m;
                }
            }
            p_.march = march;
            p_.ntiles = p_.ntz * ((nx_ + march - 1) / march);
            grid_ = (int)std::max<int64_t>(1, std::min<int64_t>((p_.ntiles + kSpThreads / 32 - 1) / (kSpThreads / 32),
                                                                 (int64_t)sms * per_sm));
        } else {
            // FP64: block tiles of 32 x 8 cells over a persistent grid
            SSSI_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, (const void*)sponge2d_cell_kernel<double, SSSI_MODE_FP64_STRICT>, kSpThreads, 0));
            per_sm = std::max(per_sm, 1);
            p_.march = kSpCellCols;
            p_.ntiles = p_.ntz * ((nx_ + kSpCellCols - 1) / kSpCellCols);
            grid_ = std::max(1, std::min(p_.ntiles, sms * per_sm));
        }
        set_hooks(SpongeHooks<T>{});
    }
    ~Sponge2d() {
        if (graph_) cudaGraphExecDestroy(graph_);
    }
    SpongeParams<T>& params() { return p_; }
    void set_hooks(const SpongeHooks<T>& h) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(hooks_dev_.get(), &h, sizeof(h), cudaMemcpyHostToDevice, s_));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s_));  // the host copy may go out of scope
    }
    // The present field after `done` steps (interior origin, pitch ldp).
    const T* present(int done) const { return p_.field[done & 1]; }
    int64_t ldp() const { return ldp_; }
    // Steps step_ .. step_ + nsteps - 1 (params() must not change while a graph is live).
    void run(int nsteps) {
        int q = 0;
        if (nsteps >= kSpGraphSteps) {
            int* base = ctr_.template as<int>();
            if (!graph_) {
                std::lock_guard<std::mutex> lock(capture_mutex());
                cudaStream_t cs = capture_stream();
                cudaGraph_t g = nullptr;
                SSSI_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                try {
                    for (int k = 0; k < kSpGraphSteps; ++k) launch(k, cs);
                    launch_add_int(base, kSpGraphSteps, cs);
                } catch (...) {
                    cudaStreamEndCapture(cs, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                count_launch(-kSpGraphSteps);  // recorded, not run
                cudaError_t e = cudaStreamEndCapture(cs, &g);
                if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
                if (g) cudaGraphDestroy(g);
                if (e != cudaSuccess) graph_ = nullptr;
                SSSI_CHECK_CUDA(e);
            }
            launch_store_int(base, step_, s_);
            count_launch();
            for (; q + kSpGraphSteps <= nsteps; q += kSpGraphSteps) {
                SSSI_CHECK_CUDA(cudaGraphLaunch(graph_, s_));
                count_launch(kSpGraphSteps + 1);
            }
        }
        if (q < nsteps) {
            launch_store_int(ctr_.template as<int>(), step_ + q, s_);
            count_launch();
            for (int k = 0; q + k < nsteps; ++k) launch(k, s_);
        }
        step_ += nsteps;
    }

  private:
    void launch(int offset, cudaStream_t s) {
        SpongeParams<T> p = p_;
        p.step_offset = offset;
        if constexpr (std::is_same<T, float>::value) {
            launch_sponge_step<T, SSSI_MODE_FP32>(p, grid_, s);
        } else {
            if (mode_ == SSSI_MODE_FP64_STRICT)
                launch_sponge_step<T, SSSI_MODE_FP64_STRICT>(p, grid_, s);
            else
                launch_sponge_step<T, SSSI_MODE_FP64>(p, grid_, s);
        }
    }
    int nz_, nx_, mode_;
    cudaStream_t s_;
    int64_t ldp_ = 0, org_ = 0;
    DeviceBuffer F_[2], b_, ax_, az_, vdt2_, bnd_, hooks_dev_, ctr_;
    SpongeParams<T> p_{};
    int grid_ = 1, step_ = 0;
    cudaGraphExec_t graph_ = nullptr;
};

void check_sponge(int64_t nz, int64_t nx, int64_t nt, int nB, double dz, double dx, double dt, int mode) {
    SSSI_REQUIRE(nz > 0 && nx > 0 && nt >= 0, SSSI_ERR_ARG, "bad sizes nz=%lld nx=%lld nt=%lld", (long long)nz,
                 (long long)nx, (long long)nt);
    SSSI_REQUIRE(nz < (1 << 30) && nx < (1 << 30) && nt < (1 << 30) && nz * nx < (int64_t(1) << 40), SSSI_ERR_ARG,
                 "grid too large");
    SSSI_REQUIRE(nB >= 0 && nB <= nz && nB <= nx, SSSI_ERR_ARG,
                 "nBoundary must be in 0..min(nz, nx) (got %d): the sponge rows and columns lie inside the grid", nB);
    SSSI_REQUIRE(dz > 0 && dx > 0 && dt > 0, SSSI_ERR_ARG, "dz, dx, dt must be positive");
    SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64 || mode == SSSI_MODE_FP32, SSSI_ERR_ARG,
                 "unknown mode %d", mode);
}

// Forward modelling (dense source and/or point sources).  data: nx x nt (row 0
// of every step), snapshot: nz x nx x nt; either may be NULL.
template <typename T>
void sponge_fwd(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt, int nB, double dz,
                double dx, double dt, int mode, int nsrc, const int64_t* src_iz, const int64_t* src_ix,
                const double* wavelets, double* data, double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    DeviceView dv(v, (size_t)n, true, s);
    Sponge2d<T> P(dv.ptr, nz, nx, nB, dz, dx, dt, mode, nt, false, s);
    Staged<T> rec(data, (size_t)(nx * nt), false, s);
    Staged<T> wav(wavelets, (size_t)(nsrc * nt), true, s);
    DeviceBuffer d_iz, d_ix;
    if (nsrc > 0) {
        std::vector<int> hz((size_t)nsrc), hx((size_t)nsrc);
        for (int k = 0; k < nsrc; ++k) {
            SSSI_REQUIRE(src_iz[k] >= 0 && src_iz[k] < nz && src_ix[k] >= 0 && src_ix[k] < nx, SSSI_ERR_ARG,
                         "point source %d at (%lld, %lld) lies outside the %lld x %lld grid", k, (long long)src_iz[k],
                         (long long)src_ix[k], (long long)nz, (long long)nx);
            hz[(size_t)k] = (int)src_iz[k];
            hx[(size_t)k] = (int)src_ix[k];
        }
        d_iz.allocate(sizeof(int) * nsrc);
        d_ix.allocate(sizeof(int) * nsrc);
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_iz.get(), hz.data(), sizeof(int) * nsrc, cudaMemcpyHostToDevice, s));
        SSSI_CHECK_CUDA(cudaMemcpyAsync(d_ix.get(), hx.data(), sizeof(int) * nsrc, cudaMemcpyHostToDevice, s));
        P.params().nsrc = nsrc;
        P.params().src_iz = d_iz.template as<int>();
        P.params().src_ix = d_ix.template as<int>();
        P.params().wavelets = wav.ptr;
    }
    P.params().rec = rec.ptr;
    const int64_t K = (source || snapshot) ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> src(const_cast<double*>(source), n, K), snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t0 = 0; t0 < nt; t0 += K) {
        const int64_t kk = std::min(K, nt - t0);
        src.load(t0, kk, s);
        SpongeHooks<T> h{};
        h.src_dense = source ? src.slice(t0, t0) : nullptr;
        h.dense_t0 = (int)t0;
        h.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        h.snap_t0 = (int)t0;
        P.set_hooks(h);
        P.run((int)kk);
        snap.store(t0, kk, s);
    }
    timing_end(s);
    rec.download(data, s);
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// Copies the interior of a padded field into a dense nz x nx array of doubles.
template <typename T>
__global__ void sponge_interior_kernel(const T* f, int64_t ldp, int nz, int nx, double* out) {
    const int64_t n = (int64_t)nz * nx;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q % nz, j = q / nz;
        out[q] = (double)f[i + j * ldp];
    }
}

// Reverse propagation of data (nx x nt) injected on row 0, t = nt-1 .. 0.
// model: nz x nx, the present field after the last step (t = 0); the
// reference's rvsTimeSpongeFor2dAw.m never assigns its `model` output.
template <typename T>
void sponge_rvs(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt, int nB, double dz,
                double dx, double dt, int mode, double* model, double* snapshot) {
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    DeviceView dv(v, (size_t)n, true, s);
    Sponge2d<T> P(dv.ptr, nz, nx, nB, dz, dx, dt, mode, nt, true, s);
    Staged<T> rows(data, (size_t)(nx * nt), true, s);
    P.params().src_row = data ? rows.ptr : nullptr;
    const int64_t K = snapshot ? chunk_steps(nt, n) : std::max<int64_t>(nt, 1);
    SliceStream<T> snap(snapshot, n, K);
    timing_begin(s);
    for (int64_t t_hi = nt; t_hi > 0; t_hi -= K) {
        const int64_t t0 = std::max<int64_t>(0, t_hi - K);
        SpongeHooks<T> h{};
        h.snap = snapshot ? snap.slice(t0, t0) : nullptr;
        h.snap_t0 = (int)t0;
        P.set_hooks(h);
        P.run((int)(t_hi - t0));
        snap.store(t0, t_hi - t0, s);
    }
    timing_end(s);
    if (model) {
        DeviceView out(model, (size_t)n, false, s);
        sponge_interior_kernel<T><<<152 * 4, 256, 0, s>>>(P.present((int)nt), P.ldp(), (int)nz, (int)nx, out.ptr);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        out.download(model, (size_t)n, s);
    }
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// One RTM shot (FP64 modes): forward in v (dataTrue) and vs (dataSmooth, the
// forward snapshots), reverse of dataTrue - dataSmooth in v, and
//     image = M ./ s2,  M = sum_t f_t .* r_t,  s2 = epsilon + sum_t f_t.^2
// (mainRtmTimeSpongeFor2dAw.m:247-268,310).  Strict: every snapshot kept in FP64
// and the sums formed in the reference's order (t ascending) after the
// reverse pass; fused: the sums accumulate inside the reverse step.
void sponge_rtm(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int nB, double dz, double dx,
                double dt, const double* wavelet, int64_t siz, int64_t six, double eps, int mode, double* image,
                double* data_true, double* data_smooth) {
    SSSI_REQUIRE(siz >= 0 && siz < nz && six >= 0 && six < nx, SSSI_ERR_ARG, "source (%lld, %lld) outside the grid",
                 (long long)siz, (long long)six);
    cudaStream_t s = current_stream();
    const int64_t n = nz * nx;
    DeviceView dv(v, (size_t)n, true, s), dvs(vs, (size_t)n, true, s);
    Staged<double> wav(wavelet, (size_t)nt, true, s);
    DeviceBuffer d_src(2 * sizeof(int));
    const int hsrc[2] = {(int)siz, (int)six};
    SSSI_CHECK_CUDA(cudaMemcpyAsync(d_src.get(), hsrc, sizeof(hsrc), cudaMemcpyHostToDevice, s));
    DeviceBuffer rec_true((size_t)(nx * std::max<int64_t>(nt, 1)) * sizeof(double)),
        rec_smooth((size_t)(nx * std::max<int64_t>(nt, 1)) * sizeof(double));
    DeviceBuffer fsnap((size_t)(n * std::max<int64_t>(nt, 1)) * sizeof(double));
    const bool strict = mode == SSSI_MODE_FP64_STRICT;
    timing_begin(s);
    for (int pass = 0; pass < 2; ++pass) {
        Sponge2d<double> P(pass == 0 ? dv.ptr : dvs.ptr, nz, nx, nB, dz, dx, dt, mode, nt, false, s);
        SpongeParams<double>& p = P.params();
        p.nsrc = 1;
        p.src_iz = d_src.as<int>();
        p.src_ix = d_src.as<int>() + 1;
        p.wavelets = wav.ptr;
        p.rec = (pass == 0 ? rec_true : rec_smooth).as<double>();
        SpongeHooks<double> h{};
        if (pass == 1) h.snap = fsnap.as<double>();
        P.set_hooks(h);
        P.run((int)nt);
    }
    timing_mark(s);
    DeviceBuffer delta((size_t)(nx * std::max<int64_t>(nt, 1)) * sizeof(double));
    diff_kernel<double><<<152 * 4, 256, 0, s>>>(rec_true.as<double>(), rec_smooth.as<double>(), delta.as<double>(),
                                               nx * nt);
    count_launch();
    SSSI_CHECK_CUDA(cudaGetLastError());
    DeviceView img(image, (size_t)n, false, s);
    {
        Sponge2d<double> R(dv.ptr, nz, nx, nB, dz, dx, dt, mode, nt, true, s);
        R.params().src_row = delta.as<double>();
        DeviceBuffer rsnap, msum, ssum;
        SpongeHooks<double> h{};
        if (strict) {
            rsnap.allocate((size_t)(n * std::max<int64_t>(nt, 1)) * sizeof(double));
            h.snap = rsnap.as<double>();
        } else {
            msum.allocate((size_t)n * sizeof(double));
            ssum.allocate((size_t)n * sizeof(double));
            msum.zero(s);
            ssum.zero(s);
            h.fsnap = fsnap.as<double>();
            R.params().im = msum.as<double>();
            R.params().is2 = ssum.as<double>();
        }
        R.set_hooks(h);
        R.run((int)nt);
        if (strict) {
            image_ascending_kernel<<<152 * 4, 256, 0, s>>>(fsnap.as<double>(), rsnap.as<double>(), n, nt, eps, img.ptr);
        } else {
            image_finish_kernel<<<152 * 4, 256, 0, s>>>(msum.as<double>(), ssum.as<double>(), n, 1.0, eps, img.ptr);
        }
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
    }
    timing_end(s);
    img.download(image, (size_t)n, s);
    if (data_true)
        SSSI_CHECK_CUDA(cudaMemcpyAsync(data_true, rec_true.get(), sizeof(double) * nx * nt, cudaMemcpyDefault, s));
    if (data_smooth)
        SSSI_CHECK_CUDA(
            cudaMemcpyAsync(data_smooth, rec_smooth.get(), sizeof(double) * nx * nt, cudaMemcpyDefault, s));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" {

int sssi_fwdTimeSpongeFor2dAw(const double* v, const double* source, int64_t nz, int64_t nx, int64_t nt,
                              int nBoundary, double dz, double dx, double dt, double* data, double* snapshot,
                              int mode) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && source, SSSI_ERR_ARG, "v and source are required");
        ensure_device();
        if (nt == 0) return;
        if (mode == SSSI_MODE_FP32)
            sponge_fwd<float>(v, source, nz, nx, nt, nBoundary, dz, dx, dt, mode, 0, nullptr, nullptr, nullptr, data,
                              snapshot);
        else
            sponge_fwd<double>(v, source, nz, nx, nt, nBoundary, dz, dx, dt, mode, 0, nullptr, nullptr, nullptr, data,
                               snapshot);
    });
}

int sssi_fwdTimeSpongeFor2dAwPoint(const double* v, int64_t nz, int64_t nx, int64_t nt, int nBoundary, double dz,
                                   double dx, double dt, int nsrc, const int64_t* src_iz, const int64_t* src_ix,
                                   const double* wavelets, double* data, double* snapshot, int mode) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v, SSSI_ERR_ARG, "v is required");
        SSSI_REQUIRE(nsrc >= 0 && nsrc <= 64, SSSI_ERR_ARG, "nsrc must be in 0..64 (got %d)", nsrc);
        SSSI_REQUIRE(nsrc == 0 || (src_iz && src_ix && wavelets), SSSI_ERR_ARG, "point sources need positions and wavelets");
        ensure_device();
        if (nt == 0) return;
        if (mode == SSSI_MODE_FP32)
            sponge_fwd<float>(v, nullptr, nz, nx, nt, nBoundary, dz, dx, dt, mode, nsrc, src_iz, src_ix, wavelets,
                              data, snapshot);
        else
            sponge_fwd<double>(v, nullptr, nz, nx, nt, nBoundary, dz, dx, dt, mode, nsrc, src_iz, src_ix, wavelets,
                               data, snapshot);
    });
}

int sssi_rvsTimeSpongeFor2dAw(const double* v, const double* data, int64_t nz, int64_t nx, int64_t nt,
                              int nBoundary, double dz, double dx, double dt, double* model, double* snapshot,
                              int mode) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && data, SSSI_ERR_ARG, "v and data are required");
        ensure_device();
        if (nt == 0) {
            if (model) {
                cudaStream_t s = current_stream();
                DeviceView out(model, (size_t)(nz * nx), false, s);
                fill(out.ptr, nz * nx, 0.0, s);
                out.download(model, (size_t)(nz * nx), s);
                SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
            }
            return;
        }
        if (mode == SSSI_MODE_FP32)
            sponge_rvs<float>(v, data, nz, nx, nt, nBoundary, dz, dx, dt, mode, model, snapshot);
        else
            sponge_rvs<double>(v, data, nz, nx, nt, nBoundary, dz, dx, dt, mode, model, snapshot);
    });
}

int sssi_rtmTimeSpongeFor2dAw(const double* v, const double* vs, int64_t nz, int64_t nx, int64_t nt, int nBoundary,
                              double dz, double dx, double dt, const double* wavelet, int64_t src_iz, int64_t src_ix,
                              double epsilon, int mode, double* image, double* data_true, double* data_smooth) {
    return guarded([&] {
        check_sponge(nz, nx, nt, nBoundary, dz, dx, dt, mode);
        SSSI_REQUIRE(v && vs && wavelet && image, SSSI_ERR_ARG, "v, vs, wavelet and image are required");
        SSSI_REQUIRE(nt >= 1, SSSI_ERR_ARG, "nt must be at least 1");
        SSSI_REQUIRE(mode != SSSI_MODE_FP32, SSSI_ERR_ARG,
                     "the sponge RTM shot runs in FP64 (SSSI_MODE_FP64 or SSSI_MODE_FP64_STRICT)");
        ensure_device();
        sponge_rtm(v, vs, nz, nx, nt, nBoundary, dz, dx, dt, wavelet, src_iz, src_ix, epsilon, mode, image, data_true,
                   data_smooth);
    });
}

}  // extern "C"
