"""The 3D propagator (fwdTimeCpmlFor3dAw) against the FP64 oracle: the golden
fixture, ragged grids (partial tiles in z and x, several y chunks, every band
combination), point sources against the dense source volume, a run long
enough for the wavefront to reach the damped bands, argument errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_FP32 = 1e-4


def test_fwd3d_golden(gpu, golden, oracle_mod):
    S = gpu
    g = golden("fwd3d.npz")
    nz, nx, ny, nt, N, nB = (int(x) for x in g["params"])
    src = np.zeros((nz, nx, ny, nt), order="F")
    src[1, nx // 2, ny // 2, :] = g["trace"]
    for mode, tol in (("fp64-strict", TOL_FP64), ("fp64", TOL_FP64), ("fp32", TOL_FP32)):
        d, s = S.fwdTimeCpmlFor3dAw(g["v"], src, N, nB, 10.0, 10.0, 10.0, 1e-3, mode=mode)
        assert oracle_mod.rel_l2(d, g["data"]) <= tol, mode
        assert oracle_mod.rel_l2(s[:, :, :, -1], g["snap_last"]) <= tol, mode
        assert oracle_mod.rel_l2(s[:, :, :, nt // 2], g["snap_mid"]) <= tol, mode


SHAPES = [  # nz, nx, ny, N, nB
    (37, 29, 41, 4, 5),
    (16, 16, 16, 1, 0),
    (70, 45, 33, 8, 6),
    (33, 70, 50, 2, 8),
    (20, 66, 70, 3, 4),
    (45, 34, 36, 5, 3),
]


@pytest.mark.parametrize("shape", SHAPES)
def test_fwd3d_vs_oracle(gpu, co, oracle_mod, shape):
    S = gpu
    nz, nx, ny, N, nB = shape
    nt = 24
    rng = np.random.default_rng(nz * 31 + nx * 7 + ny + N)
    v = rng.uniform(1500, 4000, (nz, nx, ny))
    tr = oracle_mod.ricker(40.0, nt, 5e-4)
    pos = (min(3, nz - 1), nx // 3, ny // 2)
    src = np.zeros((nz, nx, ny, nt), order="F")
    src[pos[0], pos[1], pos[2], :] = tr
    src[nz - 1, nx - 1, ny - 1, :] = 0.5 * tr  # a source in the far corner (inside every band)
    d_ref, s_ref = co.fwd3d(v, src, N, nB, 10.0, 12.0, 11.0, 5e-4)
    d, s = S.fwdTimeCpmlFor3dAw(v, src, N, nB, 10.0, 12.0, 11.0, 5e-4, mode="fp64")
    assert oracle_mod.rel_l2(d, d_ref) <= TOL_FP64
    assert oracle_mod.rel_l2(s, s_ref) <= TOL_FP64
    d32, s32 = S.fwdTimeCpmlFor3dAw(v, src, N, nB, 10.0, 12.0, 11.0, 5e-4, mode="fp32")
    assert oracle_mod.rel_l2(d32, d_ref) <= TOL_FP32
    assert oracle_mod.rel_l2(s32, s_ref) <= TOL_FP32


def test_fwd3d_point_equals_dense(gpu, oracle_mod):
    S = gpu
    nz, nx, ny, nt, N, nB = 30, 35, 40, 20, 4, 5
    rng = np.random.default_rng(4)
    v = rng.uniform(1800, 3500, (nz, nx, ny))
    w = rng.standard_normal((2, nt))
    iz, ix, iy = [0, 17], [3, 20], [39, 9]
    src = np.zeros((nz, nx, ny, nt), order="F")
    for k in range(2):
        src[iz[k], ix[k], iy[k], :] += w[k]
    for mode, tol in (("fp64", TOL_FP64), ("fp32", 1e-6)):
        a, _ = S.fwdTimeCpmlFor3dAw(v, src, N, nB, 10.0, 10.0, 10.0, 1e-3, mode=mode, want_snapshot=False)
        b, _ = S.fwdTimeCpmlFor3dAwPoint(v, nt, iz, ix, iy, w, N, nB, 10.0, 10.0, 10.0, 1e-3, mode=mode)
        assert oracle_mod.rel_l2(b, a) <= tol, mode


def test_fwd3d_long_run_reaches_bands(gpu, co, oracle_mod):
    """Long enough for the wavefront to cross the damped bands on every side."""
    S = gpu
    nz, nx, ny, nt, N, nB = 48, 52, 56, 260, 4, 10
    rng = np.random.default_rng(12)
    v = np.full((nz, nx, ny), 2000.0)
    v[20:] = 2600.0
    v += rng.uniform(-30, 30, v.shape)
    tr = oracle_mod.ricker(25.0, nt, 1e-3)
    pos = (2, nx // 2, ny // 2)
    d_ref, _ = co.fwd3d(v, None, N, nB, 10.0, 10.0, 10.0, 1e-3, point=(tr, *pos), want_snapshot=False)
    for mode, tol in (("fp64", TOL_FP64), ("fp32", TOL_FP32)):
        d, _ = S.fwdTimeCpmlFor3dAwPoint(v, nt, [pos[0]], [pos[1]], [pos[2]], tr[None, :], N, nB, 10.0, 10.0, 10.0,
                                         1e-3, mode=mode)
        err = oracle_mod.rel_l2(d, d_ref)
        assert err <= tol, (mode, err)
        # 260 steps: the schedule tuner timed its four candidates and kept the fastest
        sched, ms = S.debug_schedule3d()
        assert 0 <= sched < 4 and all(t > 0 for t in ms) and ms[sched] == min(ms), (mode, sched, ms)


def test_fwd3d_errors(gpu):
    S = gpu
    v = np.full((8, 8, 8), 2000.0)
    src = np.zeros((8, 8, 8, 4), order="F")
    with pytest.raises(S.SSSIError):
        S.fwdTimeCpmlFor3dAw(v, src, 9, 2, 10.0, 10.0, 10.0, 1e-3, mode="fp64")  # order out of range
    with pytest.raises(S.SSSIError):
        S.fwdTimeCpmlFor3dAw(v, src, 2, 5, 10.0, 10.0, 10.0, 1e-3, mode="fp64")  # 2 nB > nx
    with pytest.raises(S.SSSIError):
        S.fwdTimeCpmlFor3dAwPoint(v, 4, [9], [0], [0], np.zeros((1, 4)), 2, 1, 10.0, 10.0, 10.0, 1e-3)


def test_fwd3d_mex_gateway(gpu, golden, oracle_mod):
    """fwdTimeCpmlFor3dAw_mex (built on the test shim) on the golden case: the
    MATLAB call [data, snapshot] = fwdTimeCpmlFor3dAw(v, source, N, nB, dz, dx, dy, dt)."""
    import subprocess
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    subprocess.run(["make", "-s", "-C", str(root / "oracle"), "mexgw"], check=True)
    gw = oracle_mod.load_shim_library(root / "oracle" / "_build" / "mexgw_fwdTimeCpmlFor3dAw_mex.so")
    g = golden("fwd3d.npz")
    nz, nx, ny, nt, N, nB = (int(x) for x in g["params"])
    src = np.zeros((nz, nx, ny, nt), order="F")
    src[1, nx // 2, ny // 2, :] = g["trace"]
    data, snap = oracle_mod.shim_call(gw, 2, g["v"], src, N, nB, 10.0, 10.0, 10.0, 1e-3)
    assert data.shape == (nx, ny, nt) and snap.shape == (nz, nx, ny, nt)
    assert oracle_mod.rel_l2(data, g["data"]) <= TOL_FP64
    assert oracle_mod.rel_l2(snap[:, :, :, -1], g["snap_last"]) <= TOL_FP64
