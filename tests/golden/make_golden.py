"""Generates the committed golden vectors in tests/golden/ from the reference's
own C gateways (src/fd_cmex/*_mex.c compiled unmodified against the project's
mex.h shim by ``make -C oracle ref``).  Run where the reference tree exists:

    python tests/golden/make_golden.py

Outputs (all float64, MATLAB index order):
  dcoef.npz     dCoef(N,'s') for N = 1..8 (reference dCoef through the shim's mldivide)
  damppml.npz   reference dampPml on a 30 x 40 model, nB = 5, both bands
  fwd2d_rvs2d.npz  15 cases (37 x 53, nt = 48, N = 1..5, nB in {0, 3, 8}):
                inputs, reference data, two forward snapshots, reverse model
                and two reverse snapshots
  rtm2d.npz     one reference RTM shot (40 x 60, nt = 120): dataTrue, dataSmooth,
                and image = M./s2 with the sums in ascending time order
  fwd3d.npz     3D forward (24 x 20 x 18, nt = 32, N = 3, nB = 4) from the C
                restatement (the reference has no C for 3D; its MATLAB file is
                restated and cross-checked against the numpy restatement here,
                which is run a second time with the reference's own compiled
                diffOperator_mex for every derivative: the routine the MATLAB
                file's diffOperator calls resolve to)
  diffop.npz    the reference's diffOperator_mex on seeded 2D (37 x 53) and 3D
                (16 x 13 x 11) arrays, orders 1..5, every dimension, plus the
                gateway's dim rule (a 2D array takes dim 3 as 2, a 3D one dim 7 as 3)

  sponge2d.npz  sponge-ABC forward and reverse (src/fwdTimeSpongeFor2dAw.m,
                src/rvsTimeSpongeFor2dAw.m; MATLAB only in the reference) on
                four grids (side bands overlapping when nx < 2 nB, nx == nB,
                no sponge) and one sponge RTM shot, from the numpy restatement,
                which must agree bit for bit with the C restatement first.
                These two restatements are the only pin of that part: no
                compiled reference exists for it.

  elastic2d.npz 2D elastic SPML propagation (src/fwdTimeSpmlFor2dEw.m; MATLAB only in
                the reference) on four grids (nDiffOrder 1..4, no sponge, side
                bands meeting at nx = 2 nB): the numpy restatement, run twice --
                with its own diffOperator and with the reference's compiled
                diffOperator_mex for every derivative (the routine the file's
                diffOperator calls resolve to) -- which must agree bit for bit.

  elastic3d.npz 3D elastic SPML propagation (src/fwdTimeSpmlFor3dEw.m, MATLAB only) on
                three grids (nDiffOrder 1..3, with and without the sponge), made
                and pinned the same way.

``python tests/golden/make_golden.py diffop`` writes diffop.npz alone; ``elastic``
elastic2d.npz and elastic3d.npz (it needs the reference tree); ``sponge``
writes sponge2d.npz alone (it needs only the two restatements, not the
reference tree).
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
CASES_2D = [(37, 53, 48, N, nB) for N in (1, 2, 3, 4, 5) for nB in (0, 3, 8)]


def source_2d(rng, nz, nx, nt):
    """Ricker at (2, nx//2) plus 12 random impulses (iz, ix, it, amplitude)."""
    trace = O.ricker(25.0, nt, 1e-3)
    imp = np.stack([rng.integers(0, nz, 12), rng.integers(0, nx, 12), rng.integers(0, nt, 12)], axis=1)
    amp = rng.standard_normal(12)
    return trace, imp.astype(np.int64), amp


def dense_source(nz, nx, nt, trace, imp, amp):
    src = np.zeros((nz, nx, nt), order="F")
    src[2, nx // 2, :] = trace
    for (iz, ix, it), a in zip(imp, amp):
        src[iz, ix, it] += a
    return src


def main() -> None:
    O.build(reference=True)
    fwd = O.RefMex("fwdTimeCpmlFor2dAw_mex")
    rvs = O.RefMex("rvsTimeCpmlFor2dAw_mex")
    co = O.COracle()

    np.savez_compressed(OUT / "dcoef.npz", **{f"N{N}": fwd.dcoef(N) for N in range(1, 9)})

    # reference dampPml(pu, pv, m, n, L) on both band shapes
    lib = fwd.lib
    lib.dampPml.restype = ctypes.POINTER(ctypes.c_double)
    lib.dampPml.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_double]
    rng = np.random.default_rng(7)
    v = rng.uniform(1500.0, 4000.0, (30, 40))
    nB, dx = 5, 10.0
    u_left = np.asfortranarray(np.tile((nB - np.arange(nB)) * dx, (30, 1)))
    v_left = np.asfortranarray(v[:, :nB])
    p = lib.dampPml(u_left.ctypes.data, v_left.ctypes.data, 30, nB, nB * dx)
    d_left = np.ctypeslib.as_array(p, shape=(nB * 30,)).copy().reshape((30, nB), order="F")
    u_bot = np.asfortranarray(np.tile(((np.arange(nB) + 1) * dx)[:, None], (1, 40)))
    v_bot = np.asfortranarray(v[30 - nB:, :])
    p = lib.dampPml(u_bot.ctypes.data, v_bot.ctypes.data, nB, 40, nB * dx)
    d_bot = np.ctypeslib.as_array(p, shape=(nB * 40,)).copy().reshape((nB, 40), order="F")
    np.savez_compressed(OUT / "damppml.npz", v=v, nB=nB, dx=dx, u_left=u_left, d_left=d_left, u_bot=u_bot,
                        d_bot=d_bot)

    rec = {}
    for k, (nz, nx, nt, N, nB) in enumerate(CASES_2D):
        rng = np.random.default_rng(1000 + k)
        v = rng.uniform(1500.0, 4000.0, (nz, nx))
        trace, imp, amp = source_2d(rng, nz, nx, nt)
        src = dense_source(nz, nx, nt, trace, imp, amp)
        data, snap = fwd.call(2, v, src, N, nB, 10.0, 10.0, 1e-3)
        model, rsnap = rvs.call(2, v, data, N, nB, 10.0, 10.0, 1e-3)
        # the restatement must agree bit for bit before anything is stored
        d2, s2 = co.fwd2d(v, src, N, nB, 10.0, 10.0, 1e-3)
        m2, r2 = co.rvs2d(v, data, N, nB, 10.0, 10.0, 1e-3)
        assert np.array_equal(d2, data) and np.array_equal(s2, snap)
        assert np.array_equal(m2, model) and np.array_equal(r2, rsnap)
        pre = f"c{k}_"
        rec.update({pre + "params": np.array([nz, nx, nt, N, nB]), pre + "v": v, pre + "trace": trace,
                    pre + "imp": imp, pre + "amp": amp, pre + "data": data,
                    pre + "snap_mid": snap[:, :, nt // 2], pre + "snap_last": snap[:, :, -1], pre + "model": model,
                    pre + "rsnap_first": rsnap[:, :, 0], pre + "rsnap_mid": rsnap[:, :, nt // 2]})
    rec["ncases"] = np.array(len(CASES_2D))
    np.savez_compressed(OUT / "fwd2d_rvs2d.npz", **rec)

    # one RTM shot of the reference application, at small size
    nz, nx, nt, N, nB = 40, 60, 120, 4, 8
    rng = np.random.default_rng(2024)
    v = np.full((nz, nx), 2000.0)
    v[18:, :] = 2600.0
    v[30:, :] = 3300.0
    v += rng.uniform(-50, 50, (nz, nx))
    vs = v.copy()
    for _ in range(4):  # a light smoothing; the exact filter does not matter to parity
        vs[1:-1, 1:-1] = 0.2 * (vs[1:-1, 1:-1] + vs[:-2, 1:-1] + vs[2:, 1:-1] + vs[1:-1, :-2] + vs[1:-1, 2:])
    trace = O.ricker(30.0, nt, 1e-3)
    src = np.zeros((nz, nx, nt), order="F")
    src[0, nx // 2, :] = trace
    d_true, _ = fwd.call(2, v, src, N, nB, 10.0, 10.0, 1e-3)
    d_smooth, f_snap = fwd.call(2, vs, src, N, nB, 10.0, 10.0, 1e-3)
    _, r_snap = rvs.call(2, v, d_true - d_smooth, N, nB, 10.0, 10.0, 1e-3)
    image = O.image_np(f_snap, r_snap, 1e-3)
    img_c, dt_c, ds_c = co.rtm2d(v, vs, trace, 0, nx // 2, N, nB, 10.0, 10.0, 1e-3, 1e-3)
    assert np.array_equal(img_c, image) and np.array_equal(dt_c, d_true) and np.array_equal(ds_c, d_smooth)
    np.savez_compressed(OUT / "rtm2d.npz", params=np.array([nz, nx, nt, N, nB]), v=v, vs=vs, trace=trace,
                        src_ix=nx // 2, epsilon=1e-3, data_true=d_true, data_smooth=d_smooth, image=image)

    # 3D forward from the C restatement, cross-checked with the numpy restatement
    nz, nx, ny, nt, N, nB = 24, 20, 18, 32, 3, 4
    rng = np.random.default_rng(33)
    v = rng.uniform(1500.0, 4000.0, (nz, nx, ny))
    trace = O.ricker(30.0, nt, 1e-3)
    src = np.zeros((nz, nx, ny, nt), order="F")
    src[1, nx // 2, ny // 2, :] = trace
    d3, s3 = co.fwd3d(v, src, N, nB, 10.0, 10.0, 10.0, 1e-3)
    d3n, s3n = O.fwd3d_np(v, src, N, nB, 10.0, 10.0, 10.0, 1e-3)
    assert np.array_equal(d3, d3n) and np.array_equal(s3, s3n)
    # and with the reference's own compiled diffOperator_mex for every derivative
    d3r, s3r = O.fwd3d_np(v, src, N, nB, 10.0, 10.0, 10.0, 1e-3, diff=O.reference_diff(O.RefMex("diffOperator_mex")))
    assert np.array_equal(d3, d3r) and np.array_equal(s3, s3r)
    np.savez_compressed(OUT / "fwd3d.npz", params=np.array([nz, nx, ny, nt, N, nB]), v=v, trace=trace, data=d3,
                        snap_last=s3[:, :, :, -1], snap_mid=s3[:, :, :, nt // 2])
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


def make_diffop() -> None:
    O.build(reference=True)
    ref = O.RefMex("diffOperator_mex")
    co = O.COracle()
    rng = np.random.default_rng(77)
    rec = {}
    n = 0
    for shape in [(37, 53), (16, 13, 11)]:
        x = rng.standard_normal(shape)
        rec[f"x{len(shape)}"] = x
        for order in (1, 2, 3, 4, 5):
            c = co.dcoef(order)
            rec[f"c{order}"] = c
            dims = list(range(1, len(shape) + 1)) + [len(shape) == 2 and 3 or 7]  # and one out-of-range dim
            for dim in dims:
                eff = dim if dim <= len(shape) else len(shape)
                if shape[eff - 1] < 2 * order - 1:
                    continue
                out = ref.call(1, x, c, 10.0, dim)[0]
                assert np.array_equal(out, co.diff_operator(x, c, 10.0, eff))
                rec[f"d{len(shape)}_o{order}_dim{dim}"] = out
                n += 1
    np.savez_compressed(OUT / "diffop.npz", **rec)
    print("diffop.npz", n, "cases")


ELASTIC_CASES = [(30, 44, 40, 3, 8), (27, 33, 30, 2, 0), (25, 40, 35, 4, 10), (33, 34, 30, 1, 17)]


def make_elastic() -> None:
    O.build(reference=True)
    refdiff = O.reference_diff(O.RefMex("diffOperator_mex"))
    rec = {}
    for k, (nz, nx, nt, N, nB) in enumerate(ELASTIC_CASES):
        rng = np.random.default_rng(5000 + k)
        vp = rng.uniform(2000.0, 4000.0, (nz, nx))
        vs = vp / np.sqrt(3.0) * rng.uniform(0.95, 1.05, (nz, nx))
        trace, imp, amp = source_2d(rng, nz, nx, nt)
        src = dense_source(nz, nx, nt, trace, imp, amp)
        dz, dx, dt = 10.0, 12.0, 5e-4
        snaps = O.fwd_elastic2d_np(vp, vs, src, N, nB, dz, dx, dt)
        snaps_ref = O.fwd_elastic2d_np(vp, vs, src, N, nB, dz, dx, dt, diff=refdiff)
        assert all(np.array_equal(a, b) for a, b in zip(snaps, snaps_ref))
        pre = f"c{k}_"
        rec.update({pre + "params": np.array([nz, nx, nt, N, nB]), pre + "vp": vp, pre + "vs": vs,
                    pre + "trace": trace, pre + "imp": imp, pre + "amp": amp})
        for name, a in zip(("Vzp", "Vxp", "Vzs", "Vxs"), snaps):
            rec[pre + name + "_mid"] = a[:, :, nt // 2]
            rec[pre + name + "_last"] = a[:, :, -1]
    rec["ncases"] = np.array(len(ELASTIC_CASES))
    rec["dzdxdt"] = np.array([10.0, 12.0, 5e-4])
    np.savez_compressed(OUT / "elastic2d.npz", **rec)
    print("elastic2d.npz", (OUT / "elastic2d.npz").stat().st_size)


ELASTIC3D_CASES = [(14, 16, 18, 12, 3, 4), (12, 10, 10, 10, 2, 0), (10, 12, 12, 8, 1, 5)]


def make_elastic3d() -> None:
    O.build(reference=True)
    refdiff = O.reference_diff(O.RefMex("diffOperator_mex"))
    rec = {}
    for k, (nz, nx, ny, nt, N, nB) in enumerate(ELASTIC3D_CASES):
        rng = np.random.default_rng(6000 + k)
        vp = rng.uniform(2000.0, 4000.0, (nz, nx, ny))
        vs = vp / np.sqrt(3.0) * rng.uniform(0.95, 1.05, (nz, nx, ny))
        tr = O.ricker(30.0, nt, 5e-4)
        srcs = [np.zeros((nz, nx, ny, nt), order="F") for _ in range(3)]
        for c, s_ in enumerate(srcs):
            s_[0, nx // 2, ny // 2, :] = tr * (1.0, 0.5, -0.25)[c]
            for _ in range(4):
                s_[rng.integers(nz), rng.integers(nx), rng.integers(ny), rng.integers(nt)] += rng.standard_normal()
        dz, dx, dy, dt = 10.0, 11.0, 12.0, 5e-4
        snaps = O.fwd_elastic3d_np(vp, vs, *srcs, N, nB, dz, dx, dy, dt)
        snaps_ref = O.fwd_elastic3d_np(vp, vs, *srcs, N, nB, dz, dx, dy, dt, diff=refdiff)
        assert all(np.array_equal(a, b) for a, b in zip(snaps, snaps_ref))
        pre = f"c{k}_"
        rec.update({pre + "params": np.array([nz, nx, ny, nt, N, nB]), pre + "vp": vp, pre + "vs": vs,
                    pre + "src_x": srcs[0], pre + "src_y": srcs[1], pre + "src_z": srcs[2]})
        for name, a in zip(("Vzp", "Vxp", "Vyp", "Vzs", "Vxs", "Vys"), snaps):
            rec[pre + name + "_mid"] = a[:, :, :, nt // 2]
            rec[pre + name + "_last"] = a[:, :, :, -1]
    rec["ncases"] = np.array(len(ELASTIC3D_CASES))
    rec["spacing"] = np.array([10.0, 11.0, 12.0, 5e-4])
    np.savez_compressed(OUT / "elastic3d.npz", **rec)
    print("elastic3d.npz", (OUT / "elastic3d.npz").stat().st_size)


SPONGE_CASES = [(33, 47, 60, 6), (40, 30, 50, 18), (25, 20, 40, 20), (30, 41, 50, 0)]


def make_sponge() -> None:
    O.build(reference=False)
    co = O.COracle()
    rec = {}
    for k, (nz, nx, nt, nB) in enumerate(SPONGE_CASES):
        rng = np.random.default_rng(3000 + k)
        v = rng.uniform(1500.0, 4000.0, (nz, nx))
        trace, imp, amp = source_2d(rng, nz, nx, nt)
        src = dense_source(nz, nx, nt, trace, imp, amp)
        dz, dx, dt = 10.0, 12.0, 1e-3
        data, snap = O.fwd_sponge_np(v, src, nB, dz, dx, dt)
        model, rsnap = O.rvs_sponge_np(v, data, nB, dz, dx, dt)
        dc, sc, _ = co.sponge2d(v, nt, nB, dz, dx, dt, source=src)
        _, rc, mc = co.sponge2d(v, nt, nB, dz, dx, dt, rdata=data)
        assert np.array_equal(dc, data) and np.array_equal(sc, snap)
        assert np.array_equal(mc, model) and np.array_equal(rc, rsnap)
        pre = f"c{k}_"
        rec.update({pre + "params": np.array([nz, nx, nt, nB]), pre + "v": v, pre + "trace": trace,
                    pre + "imp": imp, pre + "amp": amp, pre + "data": data, pre + "snap_mid": snap[:, :, nt // 2],
                    pre + "snap_last": snap[:, :, -1], pre + "model": model, pre + "rsnap_first": rsnap[:, :, 0],
                    pre + "rsnap_mid": rsnap[:, :, nt // 2]})
    rec["ncases"] = np.array(len(SPONGE_CASES))
    rec["dzdxdt"] = np.array([10.0, 12.0, 1e-3])
    # one sponge RTM shot
    nz, nx, nt, nB = 40, 60, 150, 10
    rng = np.random.default_rng(4040)
    v = np.full((nz, nx), 2000.0)
    v[18:, :] = 2600.0
    v[30:, :] = 3300.0
    v += rng.uniform(-50, 50, (nz, nx))
    vs = v.copy()
    for _ in range(4):
        vs[1:-1, 1:-1] = 0.2 * (vs[1:-1, 1:-1] + vs[:-2, 1:-1] + vs[2:, 1:-1] + vs[1:-1, :-2] + vs[1:-1, 2:])
    trace = O.ricker(30.0, nt, 1e-3)
    image, d_true, d_smooth = O.rtm_sponge_np(v, vs, trace, 0, nx // 2, nB, 10.0, 10.0, 1e-3, 1e-3)
    dct, _, _ = co.sponge2d(v, nt, nB, 10.0, 10.0, 1e-3, point=([0], [nx // 2], trace[None, :]), want_snapshot=False)
    dcs, fcs, _ = co.sponge2d(vs, nt, nB, 10.0, 10.0, 1e-3, point=([0], [nx // 2], trace[None, :]))
    _, rcs, _ = co.sponge2d(v, nt, nB, 10.0, 10.0, 1e-3, rdata=dct - dcs)
    assert np.array_equal(dct, d_true) and np.array_equal(dcs, d_smooth)
    assert np.array_equal(O.image_np(fcs, rcs, 1e-3), image)
    rec.update({"rtm_params": np.array([nz, nx, nt, nB]), "rtm_v": v, "rtm_vs": vs, "rtm_trace": trace,
                "rtm_src_ix": np.array(nx // 2), "rtm_image": image, "rtm_data_true": d_true,
                "rtm_data_smooth": d_smooth})
    np.savez_compressed(OUT / "sponge2d.npz", **rec)
    print("sponge2d.npz", (OUT / "sponge2d.npz").stat().st_size)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "diffop":
        make_diffop()
    elif len(sys.argv) > 1 and sys.argv[1] == "sponge":
        make_sponge()
    elif len(sys.argv) > 1 and sys.argv[1] == "elastic":
        make_elastic()
        make_elastic3d()
    else:
        main()
        make_diffop()
        make_sponge()
        make_elastic()
        make_elastic3d()
