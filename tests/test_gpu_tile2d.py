"""The tiled 2D kernel (fused FP64 and FP32 modes) against the FP64 oracle on
ragged grids: partial tiles in z and x, tiles that straddle the CPML bands,
every order from 1 to 8, dense, surface-row and point sources."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_FP32 = 1e-4

SHAPES = [(37, 53, 4, 8), (130, 97, 3, 10), (257, 300, 4, 20), (16, 16, 1, 0), (70, 45, 6, 5), (33, 140, 8, 4),
          (64, 32, 4, 0), (65, 33, 2, 2), (129, 65, 5, 12), (200, 70, 7, 9)]


@pytest.mark.parametrize("shape", SHAPES)
def test_tiled_fp64_and_fp32_vs_oracle(gpu, co, oracle_mod, shape):
    S = gpu
    nz, nx, N, nB = shape
    nt = 30
    rng = np.random.default_rng(nz * 7 + nx * 13 + N)
    v = rng.uniform(1500, 4000, (nz, nx))
    src = np.asfortranarray(rng.standard_normal((nz, nx, nt)))
    dt = 4e-4
    d_ref, s_ref = co.fwd2d(v, src, N, nB, 10.0, 12.0, dt)
    d, s = S.fwdTimeCpmlFor2dAw(v, src, N, nB, 10.0, 12.0, dt, mode="fp64")
    assert oracle_mod.rel_l2(d, d_ref) <= TOL_FP64
    assert oracle_mod.rel_l2(s, s_ref) <= TOL_FP64
    m_ref, r_ref = co.rvs2d(v, d_ref, N, nB, 10.0, 12.0, dt)
    m, r = S.rvsTimeCpmlFor2dAw(v, d_ref, N, nB, 10.0, 12.0, dt, mode="fp64")
    assert oracle_mod.rel_l2(m, m_ref) <= TOL_FP64
    assert oracle_mod.rel_l2(r, r_ref) <= TOL_FP64
    d32, s32 = S.fwdTimeCpmlFor2dAw(v, src, N, nB, 10.0, 12.0, dt, mode="fp32")
    assert oracle_mod.rel_l2(d32, d_ref) <= TOL_FP32
    assert oracle_mod.rel_l2(s32, s_ref) <= TOL_FP32
    m32, r32 = S.rvsTimeCpmlFor2dAw(v, d_ref, N, nB, 10.0, 12.0, dt, mode="fp32")
    assert oracle_mod.rel_l2(r32, r_ref) <= TOL_FP32


def test_tiled_long_run_pml_absorbs(gpu, co, oracle_mod):
    """A Ricker shot long enough for the wavefront to cross the CPML bands."""
    S = gpu
    nz, nx, nt, N, nB = 160, 220, 900, 4, 20
    rng = np.random.default_rng(77)
    v = np.full((nz, nx), 2000.0)
    v[60:, :] = 2800.0
    v[110:, :] = 3500.0
    v += rng.uniform(-20, 20, (nz, nx))
    tr = oracle_mod.ricker(20.0, nt, 1e-3)
    d_ref, _ = co.fwd2d(v, None, N, nB, 10.0, 10.0, 1e-3, point=(tr, 2, 110), want_snapshot=False)
    for mode, tol in (("fp64", TOL_FP64), ("fp32", TOL_FP32)):
        d, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, [2], [110], tr[None, :], N, nB, 10.0, 10.0, 1e-3, mode=mode)
        err = oracle_mod.rel_l2(d, d_ref)
        assert err <= tol, (mode, err)


def test_tiled_multiple_point_sources(gpu, co, oracle_mod):
    S = gpu
    nz, nx, nt, N, nB = 90, 150, 80, 4, 10
    rng = np.random.default_rng(8)
    v = rng.uniform(1800, 3500, (nz, nx))
    iz = [0, 5, 40, 89]
    ix = [3, 149, 75, 20]
    w = rng.standard_normal((4, nt))
    src = np.zeros((nz, nx, nt), order="F")
    for k in range(4):
        src[iz[k], ix[k], :] += w[k]
    d_ref, _ = co.fwd2d(v, src, N, nB, 10.0, 10.0, 1e-3, want_snapshot=False)
    d, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, N, nB, 10.0, 10.0, 1e-3, mode="fp64")
    assert oracle_mod.rel_l2(d, d_ref) <= TOL_FP64


def test_tile_shapes_give_identical_results(gpu):
    """Every tile shape of the batched FP32 step -- 64 x 32, 32 x 32 and the deep
    128 x 16 z-blocks the tuner also considers -- computes each cell by the same
    formula: forward modelling (the variant without rare outputs), a run with
    snapshots (rare outputs), and an RTM shot are bit-identical across shapes."""
    rng = np.random.default_rng(17)
    nz, nx, nt, N, nB = 301, 413, 120, 4, 20
    v = rng.uniform(1500.0, 4000.0, (nz, nx))
    w = np.sin(np.arange(nt) * 0.3)[None, :]
    src = np.zeros((nz, nx, 40), order="F")
    src[3, 200, :] = np.cos(np.arange(40) * 0.2)
    outs = []
    try:
        for shape in (0, 1, 2):
            gpu.debug_tile_shape(shape)
            d, _ = gpu.fwdTimeCpmlFor2dAwPoint(v, nt, [2], [nx // 2], w, N, nB, 10.0, 10.0, 8e-4, mode="fp32")
            d2, s2 = gpu.fwdTimeCpmlFor2dAw(v, src, N, nB, 10.0, 10.0, 8e-4, mode="fp32")
            img = gpu.rtmTimeCpmlFor2dAw(v, v * 0.98, w[0, :80], 0, nx // 2, N, nB, 10.0, 10.0, 8e-4, mode="fp32",
                                         snap_stride=1)
            outs.append((d, d2, s2, img))
    finally:
        gpu.debug_tile_shape(-1)
    for k in (1, 2):
        for a, b in zip(outs[0], outs[k]):
            assert np.array_equal(a, b), k


def test_tuner_times_every_shape(gpu):
    """A batch large enough to tune times all three tile shapes (the tuner's
    z-block depth choice) and keeps the fastest; the plan reports both."""
    rng = np.random.default_rng(23)
    nt = 400
    models = [rng.uniform(1500.0, 4000.0, (700, 1300)) for _ in range(6)]  # ready before the first submit
    w = np.sin(np.arange(nt) * 0.2)[None, :]
    with gpu.Plan(4, 10.0, 10.0, mode="fp32") as plan:
        tickets = [plan.submit_fwd2d(v, nt, [2], [650], w, 20, 8e-4) for v in models]
        for t in tickets:
            plan.wait(t)
        st = plan.stats()
    assert st["batch_steps"] < 6 * nt  # the shots ran together
    ms = st["batch2d_tune_ms"]
    assert all(x > 0 for x in ms), ms
    assert st["batch2d_tile_shape"] == int(np.argmin(ms))
