"""Plans (sssi_plan_*): shots of different grids, lengths and kinds resident
together on the GPU give exactly what the single-shot entry points give; a
small memory budget serialises admission without changing results; argument
errors are refused at submit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(rng, nz, nx, ny=None):
    shape = (nz, nx) if ny is None else (nz, nx, ny)
    v = rng.uniform(1600, 3800, shape)
    return np.asfortranarray(v)


def _fwd_cases(oracle_mod):
    rng = np.random.default_rng(11)
    cases = []
    for (nz, nx, nt, nB, iz, ix) in [(70, 130, 90, 8, 2, 60), (45, 64, 40, 5, 0, 3), (130, 97, 120, 10, 30, 90),
                                     (64, 32, 17, 4, 63, 31)]:
        v = _model(rng, nz, nx)
        w = oracle_mod.ricker(30.0, nt, 1e-3)[None, :]
        cases.append((v, nt, [iz], [ix], w, nB))
    return cases


@pytest.mark.parametrize("mode", ["fp32", "fp64"])
def test_plan_fwd2d_equals_single_shot(gpu, oracle_mod, mode):
    S = gpu
    cases = _fwd_cases(oracle_mod)
    with S.Plan(4, 10.0, 10.0, mode=mode) as plan:
        tickets = [plan.submit_fwd2d(v, nt, iz, ix, w, nB, 1e-3) for (v, nt, iz, ix, w, nB) in cases]
        outs = [plan.wait(t)["data"] for t in tickets]
        st = plan.stats()
    assert st["done"] == len(cases) and st["failed"] == 0 and st["running"] == 0
    for (v, nt, iz, ix, w, nB), got in zip(cases, outs):
        ref, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, nB, 10.0, 10.0, 1e-3, mode=mode)
        assert np.array_equal(got, ref), (mode, v.shape, np.abs(got - ref).max())


def test_plan_fwd2d_matches_oracle(gpu, co, oracle_mod):
    S = gpu
    (v, nt, iz, ix, w, nB) = _fwd_cases(oracle_mod)[0]
    with S.Plan(4, 10.0, 10.0, mode="fp64") as plan:
        got = plan.wait(plan.submit_fwd2d(v, nt, iz, ix, w, nB, 1e-3))["data"]
    ref, _ = co.fwd2d(v, None, 4, nB, 10.0, 10.0, 1e-3, point=(w[0], iz[0], ix[0]), want_snapshot=False)
    assert oracle_mod.rel_l2(got, ref) <= 1e-12


@pytest.mark.parametrize("mode,stride", [("fp32", 4), ("fp64", 1)])
def test_plan_rtm2d_equals_single_shot(gpu, oracle_mod, mode, stride):
    S = gpu
    rng = np.random.default_rng(5)
    shots = []
    for (nz, nx, nt) in [(60, 90, 80), (48, 70, 61)]:
        v = _model(rng, nz, nx)
        vs = np.asfortranarray(0.5 * (v + v.mean()))
        w = oracle_mod.ricker(25.0, nt, 1e-3)
        shots.append((v, vs, w, nx // 2))
    with S.Plan(4, 10.0, 10.0, mode=mode) as plan:
        ts = [plan.submit_rtm2d(v, vs, w, 0, ix, 6, 1e-3, epsilon=1e-3, snap_stride=stride, want_data=True)
              for (v, vs, w, ix) in shots]
        # a forward shot in the same batch
        tf = plan.submit_fwd2d(shots[0][0], 50, [3], [10], oracle_mod.ricker(30.0, 50, 1e-3)[None, :], 6, 1e-3)
        outs = [plan.wait(t) for t in ts]
        plan.wait(tf)
    for (v, vs, w, ix), o in zip(shots, outs):
        img, dtrue, _ = S.rtmTimeCpmlFor2dAw(v, vs, w, 0, ix, 4, 6, 10.0, 10.0, 1e-3, epsilon=1e-3, mode=mode,
                                              snap_stride=stride, want_data=True)
        assert np.array_equal(o["image"], img), (mode, np.abs(o["image"] - img).max())
        assert np.array_equal(o["data"], dtrue)


def test_plan_fwd3d_equals_single_shot(gpu, oracle_mod):
    S = gpu
    rng = np.random.default_rng(9)
    v = _model(rng, 40, 36, 34)
    nt = 30
    w = oracle_mod.ricker(30.0, nt, 1e-3)[None, :]
    with S.Plan(4, 10.0, 10.0, 10.0, mode="fp32") as plan:
        t3 = plan.submit_fwd3d(v, nt, [1], [18], [17], w, 5, 1e-3)
        t2 = plan.submit_fwd2d(v[:, :, 0], 40, [0], [5], oracle_mod.ricker(30.0, 40, 1e-3)[None, :], 5, 1e-3)
        d3 = plan.wait(t3)["data"]
        plan.wait(t2)
    ref, _ = S.fwdTimeCpmlFor3dAwPoint(v, nt, [1], [18], [17], w, 4, 5, 10.0, 10.0, 10.0, 1e-3, mode="fp32")
    assert np.array_equal(d3, ref)


def test_plan_small_budget_serialises(gpu, oracle_mod):
    """A budget below one shot's footprint admits one shot at a time."""
    S = gpu
    cases = _fwd_cases(oracle_mod)[:3]
    with S.Plan(4, 10.0, 10.0, mode="fp32", device_bytes=1, steps_per_round=16) as plan:
        ts = [plan.submit_fwd2d(v, nt, iz, ix, w, nB, 1e-3) for (v, nt, iz, ix, w, nB) in cases]
        outs = [plan.wait(t)["data"] for t in ts]
        infos = [t.info for t in ts]
    # admitted one after another: each starts after the previous one is done
    for a, b in zip(infos, infos[1:]):
        assert b["start_s"] >= a["done_s"] - 1e-9
    for (v, nt, iz, ix, w, nB), got in zip(cases, outs):
        ref, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, nB, 10.0, 10.0, 1e-3, mode="fp32")
        assert np.array_equal(got, ref)


def test_plan_errors(gpu):
    S = gpu
    v = np.full((20, 30), 2000.0)
    with S.Plan(4, 10.0, 10.0, mode="fp32") as plan:
        with pytest.raises(S.SSSIError):
            plan.submit_fwd2d(v, 10, [25], [3], np.zeros((1, 10)), 3, 1e-3)  # source outside the grid
        with pytest.raises(S.SSSIError):
            plan.submit_fwd2d(v, 10, [0], [3], np.zeros((1, 10)), 20, 1e-3)  # 2 nB > nx
        t = plan.submit_fwd2d(v, 0, [0], [3], np.zeros((1, 0)), 3, 1e-3)  # nothing to do: completes
        plan.wait(t)
        assert plan.poll(t)["state"] == "done"


def test_plan_join_mid_flight(gpu, oracle_mod):
    """Continuous batching: shot B is submitted while shot A is running and has
    advanced; B joins the running batch and both give their single-shot results
    exactly."""
    import time

    S = gpu
    rng = np.random.default_rng(21)
    va, vb = _model(rng, 120, 200), _model(rng, 90, 160)
    wa = oracle_mod.ricker(25.0, 3000, 1e-3)[None, :]
    wb = oracle_mod.ricker(25.0, 600, 1e-3)[None, :]
    with S.Plan(4, 10.0, 10.0, mode="fp32", steps_per_round=16) as plan:
        ta = plan.submit_fwd2d(va, 3000, [3], [100], wa, 10, 1e-3)
        for _ in range(4000):
            if plan.poll(ta)["state"] == "running" and plan.stats()["batch_steps"] >= 64:
                break
            time.sleep(0.001)
        steps_before = plan.stats()["batch_steps"]
        assert plan.poll(ta)["state"] == "running" and steps_before >= 64
        tb = plan.submit_fwd2d(vb, 600, [0], [40], wb, 10, 1e-3)
        db = plan.wait(tb)["data"]
        da = plan.wait(ta)["data"]
    ia, ib = ta.info, tb.info
    assert ia["start_s"] < ib["start_s"] < ia["done_s"]  # B ran while A was running
    ra, _ = S.fwdTimeCpmlFor2dAwPoint(va, 3000, [3], [100], wa, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    rb, _ = S.fwdTimeCpmlFor2dAwPoint(vb, 600, [0], [40], wb, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    assert np.array_equal(da, ra) and np.array_equal(db, rb)


@pytest.mark.parametrize("mode", ["fp32", "fp64"])
def test_plan_stack(gpu, oracle_mod, mode):
    """Device-resident stacking (Stacked = Stacked + M ./ s2 of the reference's
    shot loop): three RTM shots on windows of one model add their images to one
    stack; the stack equals the sum of the shots' own images placed at their
    windows."""
    S = gpu
    rng = np.random.default_rng(4)
    nz, nx = 70, 200
    v = _model(rng, nz, nx)
    vs = np.asfortranarray(0.5 * (v + v.mean()))
    nt = 120
    w = oracle_mod.ricker(25.0, nt, 1e-3)
    windows = [(0, 0, 100), (0, 50, 120), (10, 120, 80)]  # (z0, x0, width)
    expect = np.zeros((nz, nx), order="F")
    with S.Plan(4, 10.0, 10.0, mode=mode) as plan:
        sid = plan.stack(nz, nx)
        ts = []
        for (z0, x0, width) in windows:
            vv = np.asfortranarray(v[z0:, x0:x0 + width])
            vvs = np.asfortranarray(vs[z0:, x0:x0 + width])
            ts.append(plan.submit_rtm2d(vv, vvs, w, 0, width // 2, 6, 1e-3, epsilon=1e-3, snap_stride=1,
                                        stack=sid, stack_z0=z0, stack_x0=x0))
            img = S.rtmTimeCpmlFor2dAw(vv, vvs, w, 0, width // 2, 4, 6, 10.0, 10.0, 1e-3, epsilon=1e-3, mode=mode,
                                       snap_stride=1)
            expect[z0:, x0:x0 + width] += img
        out = plan.stack_get(sid, np.zeros((nz, nx), order="F"))
        for t, (z0, x0, width) in zip(ts, windows):  # each shot also returned its own image
            assert plan.wait(t)["image"].shape == (nz - z0, width)
    assert oracle_mod.rel_l2(out, expect) <= 1e-14


def test_stack_to_mat_file(gpu, tmp_path):
    """The device-resident stacked image of a plan goes to a MAT-file straight
    from device memory (StackedRTM, mainRtmTimeCpmlFor2dAw.m:348-351) and reads
    back equal, on the host and into a device tensor."""
    import torch
    import scipy.io as sio

    nz, nx, nt = 60, 90, 200
    rng = np.random.default_rng(3)
    v = np.full((nz, nx), 2000.0)
    v[30:, :] = 2600.0
    vs = v.copy()
    w = np.sin(np.arange(nt) * 0.2) * np.exp(-((np.arange(nt) - 30) / 10.0) ** 2)
    with gpu.Plan(4, 10.0, 10.0, mode="fp64") as plan:
        st = plan.stack(nz, nx)
        t = plan.submit_rtm2d(v + rng.uniform(-5, 5, v.shape), vs, w, 0, nx // 2, 8, 1e-3, stack=st)
        plan.wait(t)
        dev = torch.zeros((nx, nz), dtype=torch.float64, device="cuda").T
        plan.stack_get(st, dev)
    path = tmp_path / "StackedRTM.mat"
    gpu.mat_write(path, {"StackedRTM": dev})
    host = sio.loadmat(path)["StackedRTM"]
    assert np.array_equal(host, dev.cpu().numpy()) and np.abs(host).max() > 0
    back = torch.zeros((nx, nz), dtype=torch.float64, device="cuda").T
    gpu.mat_read(path, "StackedRTM", out=back)
    assert torch.equal(back, dev)
