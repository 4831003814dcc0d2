"""Failure handling on the GPU without faulting it.

- A time step beyond the stability limit makes the wavefield blow up: the
  call returns SSSI_ERR_UNSTABLE, and in a plan only that shot fails.
- A bounded wait that runs out: a test knob makes the first block of one
  batched step withhold one tile's copies, so that tile's barrier wait gives
  up after a short limit; the call reports SSSI_ERR_INTERNAL and the device
  stays usable (the next call gives the same result as before).
- Cancellation of queued and running plan shots.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_INTERNAL, ERR_UNSTABLE, ERR_CANCELLED = 6, 4, 7


def _shot(oracle_mod, nz=90, nx=140, nt=300, seed=1):
    rng = np.random.default_rng(seed)
    v = np.asfortranarray(rng.uniform(1800.0, 3200.0, (nz, nx)))
    w = oracle_mod.ricker(25.0, nt, 1e-3)[None, :]
    return v, nt, [2], [nx // 2], w


@pytest.mark.parametrize("mode", ["fp32", "fp64"])
def test_blowup_is_reported(gpu, oracle_mod, mode):
    S = gpu
    v, nt, iz, ix, w = _shot(oracle_mod)
    # dt five times the stability limit of this grid: the field grows without bound
    with pytest.raises(S.SSSIError) as e:
        S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, 10, 10.0, 10.0, 5e-3, mode=mode)
    assert e.value.code == ERR_UNSTABLE and "non-finite" in str(e.value)
    # a stable call afterwards is fine
    d, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, 10, 10.0, 10.0, 1e-3, mode=mode)
    assert np.isfinite(d).all()


def test_blowup_fails_only_its_plan_shot(gpu, oracle_mod):
    S = gpu
    v, nt, iz, ix, w = _shot(oracle_mod)
    with S.Plan(4, 10.0, 10.0, mode="fp32", steps_per_round=32) as plan:
        good = plan.submit_fwd2d(v, nt, iz, ix, w, 10, 1e-3)
        bad = plan.submit_fwd2d(v, nt, iz, ix, w, 10, 5e-3)
        good2 = plan.submit_fwd2d(v, nt, [5], [20], w, 10, 1e-3)
        with pytest.raises(S.SSSIError) as e:
            plan.wait(bad)
        assert e.value.code == ERR_UNSTABLE
        d1 = plan.wait(good)["data"]
        d2 = plan.wait(good2)["data"]
        st = plan.stats()
    assert st["failed"] == 1 and st["done"] == 2
    ref1, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    ref2, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, [5], [20], w, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    assert np.array_equal(d1, ref1) and np.array_equal(d2, ref2)


def test_bounded_wait_runs_out_and_device_recovers(gpu, oracle_mod):
    S = gpu
    v, nt, iz, ix, w = _shot(oracle_mod, nt=120)
    ref, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    try:
        S.debug_withhold_copy(7, 4096)
        with pytest.raises(S.SSSIError) as e:
            S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
        assert e.value.code == ERR_INTERNAL and "wait limit" in str(e.value)
        # in a plan: the shots of that step fail, the plan carries on with later shots
        with S.Plan(4, 10.0, 10.0, mode="fp32", steps_per_round=16) as plan:
            t1 = plan.submit_fwd2d(v, nt, iz, ix, w, 10, 1e-3)
            with pytest.raises(S.SSSIError) as e:
                plan.wait(t1)
            assert e.value.code == ERR_INTERNAL
            S.debug_withhold_copy(-1)
            t2 = plan.submit_fwd2d(v, nt, iz, ix, w, 10, 1e-3)
            assert np.array_equal(plan.wait(t2)["data"], ref)
    finally:
        S.debug_withhold_copy(-1)
    d, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, iz, ix, w, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    assert np.array_equal(d, ref)


def test_cancel_queued_and_running(gpu, oracle_mod):
    S = gpu
    v, _, iz, ix, _ = _shot(oracle_mod, nz=200, nx=300)
    nlong = 200000  # about a second of steps: long enough to be cancelled while it runs
    long_w = oracle_mod.ricker(20.0, nlong, 1e-3)[None, :]
    short_w = oracle_mod.ricker(20.0, 200, 1e-3)[None, :]
    # a budget of one shot: the second waits in the queue behind the first
    with S.Plan(4, 10.0, 10.0, mode="fp32", device_bytes=1, steps_per_round=16) as plan:
        running = plan.submit_fwd2d(v, nlong, iz, ix, long_w, 10, 1e-3)
        queued = plan.submit_fwd2d(v, nlong, iz, ix, long_w, 10, 1e-3)
        after = plan.submit_fwd2d(v, 200, iz, ix, short_w, 10, 1e-3)
        import time
        for _ in range(2000):  # until the first shot has been admitted and stepped
            if plan.poll(running)["state"] == "running":
                break
            time.sleep(0.005)
        plan.cancel(queued)
        assert plan.poll(queued)["state"] == "failed" and plan.poll(queued)["status"] == ERR_CANCELLED
        plan.cancel(running)
        with pytest.raises(S.SSSIError) as e:
            plan.wait(running)
        assert e.value.code == ERR_CANCELLED
        d = plan.wait(after)["data"]
        st = plan.stats()
    assert st["failed"] == 2 and st["done"] == 1
    ref, _ = S.fwdTimeCpmlFor2dAwPoint(v, 200, iz, ix, short_w, 4, 10, 10.0, 10.0, 1e-3, mode="fp32")
    assert np.array_equal(d, ref)
