"""3D elastic SPML propagation on the GPU (src/fwdTimeSpmlFor3dEw.m) against the
restatement pinned to the reference's compiled diffOperator_mex: strict FP64
bit-identical, fused FP64 within 1e-12 and FP32 within 1e-4 relative L2."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = __import__("pathlib").Path(__file__).resolve().parents[1]
NAMES = ("Vzp", "Vxp", "Vyp", "Vzs", "Vxs", "Vys")


def _case(golden, k):
    g = golden("elastic3d.npz")
    nz, nx, ny, nt, N, nB = (int(x) for x in g[f"c{k}_params"])
    dz, dx, dy, dt = (float(x) for x in g["spacing"])
    srcs = (g[f"c{k}_src_x"], g[f"c{k}_src_y"], g[f"c{k}_src_z"])
    return g, nt, N, nB, dz, dx, dy, dt, g[f"c{k}_vp"], g[f"c{k}_vs"], srcs


@pytest.mark.parametrize("k", range(3))
def test_elastic3d_strict_bit_identical(gpu, golden, k):
    g, nt, N, nB, dz, dx, dy, dt, vp, vs, srcs = _case(golden, k)
    snaps = gpu.fwdTimeSpmlFor3dEw(vp, vs, *srcs, N, nB, dz, dx, dy, dt, mode="fp64-strict")
    for name, a in zip(NAMES, snaps):
        assert np.array_equal(a[:, :, :, nt // 2], g[f"c{k}_{name}_mid"]), name
        assert np.array_equal(a[:, :, :, -1], g[f"c{k}_{name}_last"]), name


@pytest.mark.parametrize("k", range(3))
def test_elastic3d_fused_and_fp32(gpu, golden, oracle_mod, k):
    g, nt, N, nB, dz, dx, dy, dt, vp, vs, srcs = _case(golden, k)
    s64 = gpu.fwdTimeSpmlFor3dEw(vp, vs, *srcs, N, nB, dz, dx, dy, dt, mode="fp64")
    s32 = gpu.fwdTimeSpmlFor3dEw(vp, vs, *srcs, N, nB, dz, dx, dy, dt, mode="fp32")
    for name, a, b in zip(NAMES, s64, s32):
        ref = g[f"c{k}_{name}_last"]
        assert oracle_mod.rel_l2(a[:, :, :, -1], ref) <= 1e-12, name
        assert oracle_mod.rel_l2(b[:, :, :, -1], ref) <= 1e-4, name


def test_elastic3d_point_sources_larger_grid(gpu, oracle_mod):
    """Point sources (components x and z, two on one cell) equal the dense
    sources, on a grid with more tiles than resident blocks, for longer than
    one graph of steps; strict FP64 equals the restatement."""
    rng = np.random.default_rng(41)
    nz, nx, ny, nt, N, nB = 40, 48, 36, 20, 2, 6
    vp = rng.uniform(2000.0, 4000.0, (nz, nx, ny))
    vs = vp / np.sqrt(3.0)
    w = rng.standard_normal((3, nt))
    iz, ix, iy, comp = [0, 10, 10], [24, 7, 7], [18, 30, 30], [0, 2, 2]
    srcs = [np.zeros((nz, nx, ny, nt), order="F") for _ in range(3)]
    for k in range(3):
        srcs[comp[k]][iz[k], ix[k], iy[k], :] += w[k]
    dense = gpu.fwdTimeSpmlFor3dEw(vp, vs, *srcs, N, nB, 10.0, 10.0, 10.0, 5e-4, mode="fp64-strict")
    point = gpu.fwdTimeSpmlFor3dEwPoint(vp, vs, nt, iz, ix, iy, comp, w, N, nB, 10.0, 10.0, 10.0, 5e-4,
                                        mode="fp64-strict")
    for a, b in zip(dense, point):
        assert np.array_equal(a, b)
    ref = oracle_mod.fwd_elastic3d_np(vp, vs, *srcs, N, nB, 10.0, 10.0, 10.0, 5e-4)
    for name, a, r in zip(NAMES, dense, ref):
        assert np.array_equal(a, r), name


def test_elastic3d_mex_gateway(gpu, golden, oracle_mod):
    O = oracle_mod
    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeSpmlFor3dEw_mex.so")
    g, nt, N, nB, dz, dx, dy, dt, vp, vs, srcs = _case(golden, 0)
    old = os.environ.get("SSSI_MEX_MODE")
    try:
        os.environ["SSSI_MEX_MODE"] = "strict"
        outs = O.shim_call(gw, 6, vp, vs, *srcs, float(N), float(nB), dz, dx, dy, dt)
        for name, a in zip(NAMES, outs):
            assert np.array_equal(a[:, :, :, -1], g[f"c0_{name}_last"]), name
    finally:
        if old is None:
            os.environ.pop("SSSI_MEX_MODE", None)
        else:
            os.environ["SSSI_MEX_MODE"] = old
