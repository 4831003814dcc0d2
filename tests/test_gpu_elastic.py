"""2D elastic SPML propagation on the GPU (src/fwdTimeSpmlFor2dEw.m) against
the restatement pinned to the reference's compiled diffOperator_mex: strict
FP64 bit-identical, fused FP64 within 1e-12 and FP32 within 1e-4 relative L2."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import dense_source

pytestmark = pytest.mark.gpu

ROOT = __import__("pathlib").Path(__file__).resolve().parents[1]
NAMES = ("Vzp", "Vxp", "Vzs", "Vxs")


def _case(golden, k):
    g = golden("elastic2d.npz")
    nz, nx, nt, N, nB = (int(x) for x in g[f"c{k}_params"])
    dz, dx, dt = (float(x) for x in g["dzdxdt"])
    src = dense_source(nz, nx, nt, g[f"c{k}_trace"], g[f"c{k}_imp"], g[f"c{k}_amp"])
    return g, nz, nx, nt, N, nB, dz, dx, dt, g[f"c{k}_vp"], g[f"c{k}_vs"], src


@pytest.mark.parametrize("k", range(4))
def test_elastic_strict_bit_identical(gpu, golden, k):
    g, nz, nx, nt, N, nB, dz, dx, dt, vp, vs, src = _case(golden, k)
    snaps = gpu.fwdTimeSpmlFor2dEw(vp, vs, src, N, nB, dz, dx, dt, mode="fp64-strict")
    for name, a in zip(NAMES, snaps):
        assert np.array_equal(a[:, :, nt // 2], g[f"c{k}_{name}_mid"]), name
        assert np.array_equal(a[:, :, -1], g[f"c{k}_{name}_last"]), name


@pytest.mark.parametrize("k", range(4))
def test_elastic_fused_and_fp32(gpu, golden, oracle_mod, k):
    g, nz, nx, nt, N, nB, dz, dx, dt, vp, vs, src = _case(golden, k)
    s64 = gpu.fwdTimeSpmlFor2dEw(vp, vs, src, N, nB, dz, dx, dt, mode="fp64")
    s32 = gpu.fwdTimeSpmlFor2dEw(vp, vs, src, N, nB, dz, dx, dt, mode="fp32")
    for name, a, b in zip(NAMES, s64, s32):
        for when, sl in (("mid", nt // 2), ("last", -1)):
            ref = g[f"c{k}_{name}_{when}"]
            assert oracle_mod.rel_l2(a[:, :, sl], ref) <= 1e-12, (name, when)
            assert oracle_mod.rel_l2(b[:, :, sl], ref) <= 1e-4, (name, when)


def test_elastic_point_sources_and_longer_run(gpu, oracle_mod):
    """Point sources equal the dense source (two on one cell add up); a grid with
    more tiles than resident blocks and runs long enough for graph replays."""
    rng = np.random.default_rng(31)
    nz, nx, nt, N, nB = 150, 420, 70, 3, 20
    vp = rng.uniform(2000.0, 4000.0, (nz, nx))
    vs = vp / np.sqrt(3.0)
    w = rng.standard_normal((3, nt))
    iz, ix = [0, 40, 40], [200, 13, 13]
    src = np.zeros((nz, nx, nt), order="F")
    for k in range(3):
        src[iz[k], ix[k], :] += w[k]
    dense = gpu.fwdTimeSpmlFor2dEw(vp, vs, src, N, nB, 10.0, 10.0, 5e-4, mode="fp64-strict")
    point = gpu.fwdTimeSpmlFor2dEwPoint(vp, vs, nt, iz, ix, w, N, nB, 10.0, 10.0, 5e-4, mode="fp64-strict")
    for a, b in zip(dense, point):
        assert np.array_equal(a, b)
    ref = oracle_mod.fwd_elastic2d_np(vp, vs, src, N, nB, 10.0, 10.0, 5e-4)
    for name, a, r in zip(NAMES, dense, ref):
        assert np.array_equal(a, r), name


def test_elastic_selected_snapshots_and_zero_steps(gpu, golden):
    g, nz, nx, nt, N, nB, dz, dx, dt, vp, vs, src = _case(golden, 0)
    out = gpu.fwdTimeSpmlFor2dEw(vp, vs, src, N, nB, dz, dx, dt, mode="fp64-strict",
                                 want_snapshot=(False, True, False, False))
    assert out[0] is None and out[2] is None and out[3] is None
    assert np.array_equal(out[1][:, :, -1], g["c0_Vxp_last"])
    z = gpu.fwdTimeSpmlFor2dEw(vp, vs, np.zeros((nz, nx, 0)), N, nB, dz, dx, dt)
    assert z[0].shape == (nz, nx, 0)


def test_elastic_mex_gateway(gpu, golden, oracle_mod):
    O = oracle_mod
    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeSpmlFor2dEw_mex.so")
    g, nz, nx, nt, N, nB, dz, dx, dt, vp, vs, src = _case(golden, 2)
    old = os.environ.get("SSSI_MEX_MODE")
    try:
        os.environ["SSSI_MEX_MODE"] = "strict"
        outs = O.shim_call(gw, 4, vp, vs, src, float(N), float(nB), dz, dx, dt)
        for name, a in zip(NAMES, outs):
            assert np.array_equal(a[:, :, -1], g[f"c2_{name}_last"]), name
        os.environ.pop("SSSI_MEX_MODE")
        (vzp,) = O.shim_call(gw, 1, vp, vs, src, float(N), float(nB), dz, dx, dt)
        assert O.rel_l2(vzp[:, :, -1], g["c2_Vzp_last"]) <= 1e-12
    finally:
        if old is None:
            os.environ.pop("SSSI_MEX_MODE", None)
        else:
            os.environ["SSSI_MEX_MODE"] = old
