"""The FP32 precision form of the RTM shot against FP64, at the 1e-4 relative
L2 bound on the image and on both seismograms and their difference.

The hard case is a model whose thick uniform top layer makes the direct wave
dominate both seismograms equally: dataTrue - dataSmooth (the reverse
source, mainRtmTimeCpmlFor2dAw.m:252) is then a small difference of two large
traces.  The FP32 form advances the migration-model field and the residual
(true-model field minus migration-model field) as one residual pair, so the
difference keeps FP32 accuracy relative to itself."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-4


def _ext(v, nB):
    w = np.concatenate([np.repeat(v[:, :1], nB, 1), v, np.repeat(v[:, -1:], nB, 1)], axis=1)
    return np.asfortranarray(np.concatenate([w, np.repeat(w[-1:, :], nB, 0)], axis=0))


def uniform_top_models(nz0, nx0, top, vels, nB=20, seed=3):
    """A layered model with a uniform top layer `top` cells thick (velocity
    vels[0]), flat interfaces below at seeded depths, and its Gaussian-smoothed
    copy (sigma 15 cells, edges replicated) as migration model; both padded
    like extBoundary (no top layer)."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    depths = [top] + sorted(rng.choice(np.arange(top + 20, nz0 - 10), len(vels) - 2, replace=False).tolist())
    v = np.full((nz0, nx0), float(vels[0]))
    for d, c in zip(depths, vels[1:]):
        v[d:, :] = c
    vs = gaussian_filter(v, sigma=15, mode="nearest")
    return _ext(v, nB), _ext(vs, nB)


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("stride", [1, 4])
def test_rtm_fp32_uniform_top_layer_vs_oracle(gpu, co, oracle_mod, stride):
    S = gpu
    V, VS = uniform_top_models(180, 260, 110, [1800.0, 2600.0, 3300.0])
    nz, nx = V.shape
    nt, dt, eps = 1600, 8e-4, 1e-3
    w = oracle_mod.ricker(15.0, nt, dt)
    six = nx // 2
    img_ref, dtr_ref, dsm_ref = co.rtm2d(V, VS, w, 0, six, 4, 20, 10.0, 10.0, dt, eps)
    resid_ref = dtr_ref - dsm_ref
    # the residual is a small part of the data here: that is what makes the case hard
    assert np.linalg.norm(resid_ref) < 0.05 * np.linalg.norm(dtr_ref)
    img, dtr, dsm = S.rtmTimeCpmlFor2dAw(V, VS, w, 0, six, 4, 20, 10.0, 10.0, dt, epsilon=eps, mode="fp32",
                                         snap_stride=stride, want_data=True)
    assert _rel(dtr - dsm, resid_ref) <= TOL_FP32
    assert _rel(dtr, dtr_ref) <= TOL_FP32
    assert _rel(dsm, dsm_ref) <= TOL_FP32
    assert _rel(img, img_ref) <= TOL_FP32, _rel(img, img_ref)


@pytest.mark.slow
def test_rtm_fp32_full_size(gpu):
    """The benchmark's RTM shot at full size (620 x 1240 padded, nt = 4000,
    FP16 snapshots every 4th step) against the FP64 drop-in on the GPU."""
    from bench import EPS, STRIDE, workload

    S = gpu
    V, VS, w, siz, six, nz, nx = workload()
    ref = S.rtmTimeCpmlFor2dAw(V, VS, w, siz, six, 4, 20, 10.0, 10.0, 8e-4, epsilon=EPS, mode="fp64",
                               want_data=True)
    got = S.rtmTimeCpmlFor2dAw(V, VS, w, siz, six, 4, 20, 10.0, 10.0, 8e-4, epsilon=EPS, mode="fp32",
                               snap_stride=STRIDE, want_data=True)
    assert _rel(got[1] - got[2], ref[1] - ref[2]) <= TOL_FP32
    assert _rel(got[1], ref[1]) <= TOL_FP32
    assert _rel(got[2], ref[2]) <= TOL_FP32
    assert _rel(got[0], ref[0]) <= TOL_FP32


def test_plan_rtm_uniform_top_mix(gpu, oracle_mod):
    """FP32 plan: two uniform-top-layer RTM shots of different sizes mixed with
    forward shots, the forward field stored and imaged every step.  Each image
    equals its single-shot result exactly and is within 1e-4 of FP64."""
    S = gpu
    shots = []
    # records long enough to hold each model's first reflection (two-way time of
    # the top layer at 1700 m/s: about 1180 and 1030 steps)
    for k, (nz0, nx0, top, nt) in enumerate([(140, 220, 80, 1800), (120, 300, 70, 1500)]):
        V, VS = uniform_top_models(nz0, nx0, top, [1700.0, 2500.0, 3100.0], seed=10 + k)
        w = oracle_mod.ricker(15.0, nt, 8e-4)
        shots.append((V, VS, w, V.shape[1] // 2 + 7 * k))
    with S.Plan(4, 10.0, 10.0, mode="fp32", steps_per_round=48) as plan:
        tf = plan.submit_fwd2d(shots[0][0], 900, [2], [40], oracle_mod.ricker(20.0, 900, 8e-4)[None, :], 20, 8e-4)
        ts = [plan.submit_rtm2d(V, VS, w, 0, ix, 20, 8e-4, epsilon=1e-3, snap_stride=1, want_data=True)
              for (V, VS, w, ix) in shots]
        tg = plan.submit_fwd2d(shots[1][0], 900, [0], [100], oracle_mod.ricker(20.0, 900, 8e-4)[None, :], 20, 8e-4)
        outs = [plan.wait(t) for t in ts]
        plan.wait(tf)
        plan.wait(tg)
    for (V, VS, w, ix), o in zip(shots, outs):
        img, dtr, _ = S.rtmTimeCpmlFor2dAw(V, VS, w, 0, ix, 4, 20, 10.0, 10.0, 8e-4, epsilon=1e-3, mode="fp32",
                                           snap_stride=1, want_data=True)
        assert np.array_equal(o["image"], img)
        assert np.array_equal(o["data"], dtr)
        ref = S.rtmTimeCpmlFor2dAw(V, VS, w, 0, ix, 4, 20, 10.0, 10.0, 8e-4, epsilon=1e-3, mode="fp64")
        assert _rel(o["image"], ref) <= TOL_FP32, _rel(o["image"], ref)
