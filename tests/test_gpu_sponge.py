"""Sponge-ABC propagation on the GPU (src/fwdTimeSpongeFor2dAw.m,
src/rvsTimeSpongeFor2dAw.m, mainRtmTimeSpongeFor2dAw.m) against the two CPU
restatements: strict FP64 bit-identical, fused FP64 within 1e-12 and FP32
within 1e-4 relative L2."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import dense_source

pytestmark = pytest.mark.gpu

ROOT = __import__("pathlib").Path(__file__).resolve().parents[1]


def _case(golden, k):
    g = golden("sponge2d.npz")
    nz, nx, nt, nB = (int(x) for x in g[f"c{k}_params"])
    dz, dx, dt = (float(x) for x in g["dzdxdt"])
    src = dense_source(nz, nx, nt, g[f"c{k}_trace"], g[f"c{k}_imp"], g[f"c{k}_amp"])
    return g, nz, nx, nt, nB, dz, dx, dt, g[f"c{k}_v"], src


@pytest.mark.parametrize("k", range(4))
def test_sponge_strict_bit_identical(gpu, golden, k):
    """Forward and reverse, strict FP64: every value equals the restatements'
    (side bands overlapping, nx == nB, no sponge included)."""
    g, nz, nx, nt, nB, dz, dx, dt, v, src = _case(golden, k)
    data, snap = gpu.fwdTimeSpongeFor2dAw(v, src, nB, dz, dx, dt, mode="fp64-strict")
    assert np.array_equal(data, g[f"c{k}_data"])
    assert np.array_equal(snap[:, :, nt // 2], g[f"c{k}_snap_mid"])
    assert np.array_equal(snap[:, :, -1], g[f"c{k}_snap_last"])
    model, rsnap = gpu.rvsTimeSpongeFor2dAw(v, data, nB, dz, dx, dt, mode="fp64-strict")
    assert np.array_equal(model, g[f"c{k}_model"])
    assert np.array_equal(rsnap[:, :, 0], g[f"c{k}_rsnap_first"])
    assert np.array_equal(rsnap[:, :, nt // 2], g[f"c{k}_rsnap_mid"])


@pytest.mark.parametrize("k", range(4))
def test_sponge_fused_and_fp32(gpu, golden, oracle_mod, k):
    g, nz, nx, nt, nB, dz, dx, dt, v, src = _case(golden, k)
    ref_d = g[f"c{k}_data"]
    d64, s64 = gpu.fwdTimeSpongeFor2dAw(v, src, nB, dz, dx, dt, mode="fp64")
    assert oracle_mod.rel_l2(d64, ref_d) <= 1e-12
    assert oracle_mod.rel_l2(s64[:, :, -1], g[f"c{k}_snap_last"]) <= 1e-12
    m64, _ = gpu.rvsTimeSpongeFor2dAw(v, ref_d, nB, dz, dx, dt, mode="fp64")
    assert oracle_mod.rel_l2(m64, g[f"c{k}_model"]) <= 1e-12
    d32, s32 = gpu.fwdTimeSpongeFor2dAw(v, src, nB, dz, dx, dt, mode="fp32")
    assert oracle_mod.rel_l2(d32, ref_d) <= 1e-4
    assert oracle_mod.rel_l2(s32[:, :, -1], g[f"c{k}_snap_last"]) <= 1e-4
    m32, _ = gpu.rvsTimeSpongeFor2dAw(v, ref_d, nB, dz, dx, dt, mode="fp32")
    assert oracle_mod.rel_l2(m32, g[f"c{k}_model"]) <= 1e-4


def test_sponge_point_sources_equal_dense(gpu):
    rng = np.random.default_rng(12)
    nz, nx, nt, nB = 37, 45, 70, 9
    v = rng.uniform(1500.0, 4000.0, (nz, nx))
    w = rng.standard_normal((3, nt))
    iz, ix = [0, 9, 9], [20, 3, 3]  # two on one cell: they add up
    src = np.zeros((nz, nx, nt), order="F")
    for k in range(3):
        src[iz[k], ix[k], :] += w[k]
    d1, s1 = gpu.fwdTimeSpongeFor2dAw(v, src, nB, 10.0, 10.0, 1e-3, mode="fp64-strict")
    d2, s2 = gpu.fwdTimeSpongeFor2dAwPoint(v, nt, iz, ix, w, nB, 10.0, 10.0, 1e-3, mode="fp64-strict",
                                           want_snapshot=True)
    assert np.array_equal(d1, d2) and np.array_equal(s1, s2)


def test_sponge_large_grid_chunks_and_graphs(gpu, co):
    """A grid with more tiles than resident blocks (the persistent loop), a
    dense source and snapshots streamed in more than one chunk, and runs long
    enough for graph replays: strict FP64 still equals the C restatement."""
    rng = np.random.default_rng(21)
    nz, nx, nt, nB = 650, 1300, 70, 20
    v = rng.uniform(1500.0, 4000.0, (nz, nx))
    src = np.zeros((nz, nx, nt), order="F")
    src[1, 640, :] = np.sin(np.arange(nt) * 0.3)
    src[300, 20, 5:9] = 1.0
    data, snap = gpu.fwdTimeSpongeFor2dAw(v, src, nB, 10.0, 10.0, 1e-3, mode="fp64-strict")
    dc, sc, _ = co.sponge2d(v, nt, nB, 10.0, 10.0, 1e-3, source=src)
    assert np.array_equal(data, dc)
    assert np.array_equal(snap, sc)
    model, rsnap = gpu.rvsTimeSpongeFor2dAw(v, dc, nB, 10.0, 10.0, 1e-3, mode="fp64-strict")
    _, rc, mc = co.sponge2d(v, nt, nB, 10.0, 10.0, 1e-3, rdata=dc)
    assert np.array_equal(model, mc) and np.array_equal(rsnap, rc)


def test_sponge_rtm(gpu, golden, oracle_mod):
    g = golden("sponge2d.npz")
    nz, nx, nt, nB = (int(x) for x in g["rtm_params"])
    img, dtr, dsm = gpu.rtmTimeSpongeFor2dAw(g["rtm_v"], g["rtm_vs"], g["rtm_trace"], 0, int(g["rtm_src_ix"]), nB,
                                             10.0, 10.0, 1e-3, epsilon=1e-3, mode="fp64-strict", want_data=True)
    assert np.array_equal(dtr, g["rtm_data_true"]) and np.array_equal(dsm, g["rtm_data_smooth"])
    assert np.array_equal(img, g["rtm_image"])
    img64 = gpu.rtmTimeSpongeFor2dAw(g["rtm_v"], g["rtm_vs"], g["rtm_trace"], 0, int(g["rtm_src_ix"]), nB, 10.0,
                                     10.0, 1e-3, epsilon=1e-3, mode="fp64")
    assert oracle_mod.rel_l2(img64, g["rtm_image"]) <= 1e-12
    with pytest.raises(gpu.SSSIError, match="FP64"):
        gpu.rtmTimeSpongeFor2dAw(g["rtm_v"], g["rtm_vs"], g["rtm_trace"], 0, 5, nB, 10.0, 10.0, 1e-3, mode="fp32")


def test_sponge_device_tensors(gpu, golden):
    """Inputs and outputs as CUDA tensors (column-major): the same bits."""
    import torch

    g, nz, nx, nt, nB, dz, dx, dt, v, src = _case(golden, 0)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().T

    data, snap = gpu.fwdTimeSpongeFor2dAw(dev(v), dev(src), nB, dz, dx, dt, mode="fp64-strict")
    assert data.is_cuda
    assert np.array_equal(data.cpu().numpy(), g["c0_data"])
    assert np.array_equal(snap[:, :, -1].cpu().numpy(), g["c0_snap_last"])


def test_sponge_zero_steps(gpu):
    v = np.full((12, 14), 2000.0)
    data, snap = gpu.fwdTimeSpongeFor2dAw(v, np.zeros((12, 14, 0)), 3, 10.0, 10.0, 1e-3)
    assert data.shape == (14, 0) and snap.shape == (12, 14, 0)
    model, _ = gpu.rvsTimeSpongeFor2dAw(v, np.zeros((14, 0)), 3, 10.0, 10.0, 1e-3)
    assert model.shape == (12, 14) and not model.any()


def test_sponge_mex_gateways(gpu, golden, oracle_mod):
    """Both gateways through the test shim: strict (SSSI_MEX_MODE=strict)
    bit-identical, the default (fused FP64) within 1e-12."""
    O = oracle_mod
    fgw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeSpongeFor2dAw_mex.so")
    rgw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_rvsTimeSpongeFor2dAw_mex.so")
    g, nz, nx, nt, nB, dz, dx, dt, v, src = _case(golden, 1)
    old = os.environ.get("SSSI_MEX_MODE")
    try:
        os.environ["SSSI_MEX_MODE"] = "strict"
        data, snap = O.shim_call(fgw, 2, v, src, float(nB), dz, dx, dt)
        assert np.array_equal(data, g["c1_data"]) and np.array_equal(snap[:, :, -1], g["c1_snap_last"])
        model, rsnap = O.shim_call(rgw, 2, v, data, float(nB), dz, dx, dt)
        assert np.array_equal(model, g["c1_model"]) and np.array_equal(rsnap[:, :, 0], g["c1_rsnap_first"])
        os.environ.pop("SSSI_MEX_MODE")
        (d64,) = O.shim_call(fgw, 1, v, src, float(nB), dz, dx, dt)
        assert O.rel_l2(d64, g["c1_data"]) <= 1e-12
    finally:
        if old is None:
            os.environ.pop("SSSI_MEX_MODE", None)
        else:
            os.environ["SSSI_MEX_MODE"] = old
