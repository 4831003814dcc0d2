"""Pins the CPU oracle: the C restatement (oracle/sssi_oracle.c) and the numpy
restatement agree bit for bit with each other, with the committed golden
vectors made from the reference's own C gateways, and -- where the reference
tree exists -- with those gateways themselves."""
from fractions import Fraction

import numpy as np
import pytest

from tests.golden.make_golden import dense_source


def exact_staggered(N):
    """dCoef(N,'s') in exact rationals (Gaussian elimination over Q)."""
    A = [[Fraction((2 * j + 1) ** (2 * i + 1)) for j in range(N)] for i in range(N)]
    b = [Fraction(1)] + [Fraction(0)] * (N - 1)
    for k in range(N):
        p = max(range(k, N), key=lambda r: abs(A[r][k]))
        A[k], A[p] = A[p], A[k]
        b[k], b[p] = b[p], b[k]
        for r in range(k + 1, N):
            f = A[r][k] / A[k][k]
            for c in range(k, N):
                A[r][c] -= f * A[k][c]
            b[r] -= f * b[k]
    x = [Fraction(0)] * N
    for k in range(N - 1, -1, -1):
        x[k] = (b[k] - sum(A[k][c] * x[c] for c in range(k + 1, N))) / A[k][k]
    return x


def test_dcoef_kat(co, oracle_mod, golden):
    g = golden("dcoef.npz")
    # 8th-order (N=4) coefficients 1225/1024, -245/3072, 49/5120, -5/7168
    assert [Fraction(x).limit_denominator(10000) for x in co.dcoef(4)] == [
        Fraction(1225, 1024), Fraction(-245, 3072), Fraction(49, 5120), Fraction(-5, 7168)]
    for N in range(1, 9):
        c = co.dcoef(N)
        assert np.array_equal(c, g[f"N{N}"]), N
        assert np.array_equal(oracle_mod.dcoef(N), c), N
        exact = [float(x) for x in exact_staggered(N)]
        ulps = np.abs(c - np.array(exact)) / np.spacing(np.abs(np.array(exact)))
        # the system is Vandermonde-like: LU rounding grows with N exactly as
        # it does for the reference's mldivide (N=4: 2 ulp, N=5: 40 ulp, ...)
        bound = {1: 0, 2: 0, 3: 0, 4: 4, 5: 64, 6: 4096, 7: 2e5, 8: 1e7}[N]
        assert ulps.max() <= bound, (N, ulps)


def test_damppml_kat(co, oracle_mod, golden):
    g = golden("damppml.npz")
    nB, dx = int(g["nB"]), float(g["dx"])
    v = g["v"]
    assert np.array_equal(oracle_mod.damp_pml_c(g["u_left"], v[:, :nB], nB * dx), g["d_left"])
    assert np.array_equal(oracle_mod.damp_pml_c(g["u_bot"], v[30 - nB:, :], nB * dx), g["d_bot"])
    # the full 2D profile of the C restatement uses the same numbers
    xb, zb = co.damping_2d(v, nB, dx, dx, 1e-3)
    import math

    assert np.array_equal(xb[:, :nB], np.vectorize(math.exp)(-g["d_left"] * 1e-3))
    assert np.array_equal(zb[30 - nB:, :], np.vectorize(math.exp)(-g["d_bot"] * 1e-3))
    assert np.all(zb[:30 - nB, :] == 1.0)  # no top layer


def _case(g, k):
    nz, nx, nt, N, nB = (int(x) for x in g[f"c{k}_params"])
    v = g[f"c{k}_v"]
    src = dense_source(nz, nx, nt, g[f"c{k}_trace"], g[f"c{k}_imp"], g[f"c{k}_amp"])
    return nz, nx, nt, N, nB, v, src


@pytest.mark.parametrize("k", range(15))
def test_fwd_rvs_2d_golden(co, golden, k):
    g = golden("fwd2d_rvs2d.npz")
    nz, nx, nt, N, nB, v, src = _case(g, k)
    data, snap = co.fwd2d(v, src, N, nB, 10.0, 10.0, 1e-3)
    assert np.array_equal(data, g[f"c{k}_data"])
    assert np.array_equal(snap[:, :, nt // 2], g[f"c{k}_snap_mid"])
    assert np.array_equal(snap[:, :, -1], g[f"c{k}_snap_last"])
    model, rsnap = co.rvs2d(v, g[f"c{k}_data"], N, nB, 10.0, 10.0, 1e-3)
    assert np.array_equal(model, g[f"c{k}_model"])
    assert np.array_equal(rsnap[:, :, 0], g[f"c{k}_rsnap_first"])
    assert np.array_equal(rsnap[:, :, nt // 2], g[f"c{k}_rsnap_mid"])


@pytest.mark.parametrize("k", [0, 4, 10, 14])
def test_numpy_restatement_matches_c(co, oracle_mod, golden, k):
    g = golden("fwd2d_rvs2d.npz")
    nz, nx, nt, N, nB, v, src = _case(g, k)
    d_np, s_np = oracle_mod.fwd2d_np(v, src, N, nB, 10.0, 10.0, 1e-3)
    assert np.array_equal(d_np, g[f"c{k}_data"])
    assert np.array_equal(s_np[:, :, -1], g[f"c{k}_snap_last"])
    m_np, r_np = oracle_mod.rvs2d_np(v, g[f"c{k}_data"], N, nB, 10.0, 10.0, 1e-3)
    assert np.array_equal(m_np, g[f"c{k}_model"])


def test_rtm_golden(co, golden, oracle_mod):
    g = golden("rtm2d.npz")
    nz, nx, nt, N, nB = (int(x) for x in g["params"])
    img, d_true, d_smooth = co.rtm2d(g["v"], g["vs"], g["trace"], 0, int(g["src_ix"]), N, nB, 10.0, 10.0, 1e-3,
                                     float(g["epsilon"]))
    assert np.array_equal(d_true, g["data_true"])
    assert np.array_equal(d_smooth, g["data_smooth"])
    assert np.array_equal(img, g["image"])
    assert np.abs(img).max() > 0


def test_fwd3d_golden(co, golden, oracle_mod):
    g = golden("fwd3d.npz")
    nz, nx, ny, nt, N, nB = (int(x) for x in g["params"])
    src = np.zeros((nz, nx, ny, nt), order="F")
    src[1, nx // 2, ny // 2, :] = g["trace"]
    d, s = co.fwd3d(g["v"], src, N, nB, 10.0, 10.0, 10.0, 1e-3)
    assert np.array_equal(d, g["data"])
    assert np.array_equal(s[:, :, :, -1], g["snap_last"])
    # the point-source form is the same computation
    d2, _ = co.fwd3d(g["v"], None, N, nB, 10.0, 10.0, 10.0, 1e-3, point=(g["trace"], 1, nx // 2, ny // 2),
                     want_snapshot=False)
    assert np.array_equal(d2, g["data"])


def test_point_source_equals_dense(co, oracle_mod):
    rng = np.random.default_rng(3)
    nz, nx, nt = 30, 41, 30
    v = rng.uniform(1500, 4000, (nz, nx))
    tr = oracle_mod.ricker(25.0, nt, 1e-3)
    src = np.zeros((nz, nx, nt), order="F")
    src[4, 9, :] = tr
    a, _ = co.fwd2d(v, src, 3, 5, 10.0, 10.0, 1e-3, want_snapshot=False)
    b, _ = co.fwd2d(v, None, 3, 5, 10.0, 10.0, 1e-3, point=(tr, 4, 9), want_snapshot=False)
    assert np.array_equal(a, b)


def test_reference_gateways_live(co, oracle_mod):
    """Against the reference C itself (only where the reference tree was built)."""
    if not oracle_mod.available_reference():
        pytest.skip("reference gateways not built here (no reference tree)")
    fwd = oracle_mod.RefMex("fwdTimeCpmlFor2dAw_mex")
    rvs = oracle_mod.RefMex("rvsTimeCpmlFor2dAw_mex")
    rng = np.random.default_rng(11)
    for (nz, nx, nt, N, nB) in [(29, 31, 20, 4, 6), (17, 22, 15, 2, 0), (33, 19, 18, 3, 9)]:
        v = rng.uniform(1500, 4000, (nz, nx))
        src = rng.standard_normal((nz, nx, nt))
        d_ref, s_ref = fwd.call(2, v, src, N, nB, 10.0, 12.5, 8e-4)
        d, s = co.fwd2d(v, src, N, nB, 10.0, 12.5, 8e-4)
        assert np.array_equal(d, d_ref) and np.array_equal(s, s_ref)
        m_ref, r_ref = rvs.call(2, v, d_ref, N, nB, 10.0, 12.5, 8e-4)
        m, r = co.rvs2d(v, d_ref, N, nB, 10.0, 12.5, 8e-4)
        assert np.array_equal(m, m_ref) and np.array_equal(r, r_ref)
    with pytest.raises(oracle_mod.MexError, match="All 7 input arguments"):
        fwd.call(2, v, src)


def test_image_accumulation_order(co, oracle_mod):
    rng = np.random.default_rng(4)
    f = rng.standard_normal((7, 9, 13))
    r = rng.standard_normal((7, 9, 13))
    m, s2 = co.image(f, r, 1e-3)
    assert np.array_equal(m / s2, oracle_mod.image_np(f, r, 1e-3))


def test_ext_boundary_and_ricker(oracle_mod):
    V = np.arange(12.0).reshape(3, 4)
    W = oracle_mod.ext_boundary(V, 2, 2)
    assert W.shape == (5, 8)
    assert np.array_equal(W[:3, 2:6], V)
    assert np.all(W[3:, :] == W[2, :])  # bottom repeats the last row
    assert np.all(W[:3, 0] == V[:, 0]) and np.all(W[:3, -1] == V[:, -1])
    V3 = np.arange(24.0).reshape(2, 3, 4)
    W3 = oracle_mod.ext_boundary(V3, 1, 3)
    assert W3.shape == (3, 5, 6)
    w = oracle_mod.ricker(20.0, 200, 1e-3)
    assert np.argmax(w) == 50 and abs(w[50] - 1.0) < 1e-12


def test_diff_operator_restatement_matches_golden(co, golden):
    """The C restatement of diffOperator_mex reproduces the reference gateway's
    outputs (golden vectors made from it), including the gateway's dim rule."""
    g = golden("diffop.npz")
    n = 0
    for key in g.files:
        if not key.startswith("d"):
            continue
        nd, order, dim = key[1], int(key.split("_o")[1].split("_")[0]), int(key.split("dim")[1])
        x = g[f"x{nd}"]
        eff = dim if dim <= int(nd) else int(nd)
        assert np.array_equal(co.diff_operator(x, g[f"c{order}"], 10.0, eff), g[key]), key
        n += 1
    assert n >= 30


def test_diff_operator_reference_live(co, oracle_mod):
    if not (oracle_mod.REF_DIR / "diffOperator_mex.so").exists():
        pytest.skip("reference gateways not built here (no reference tree)")
    ref = oracle_mod.RefMex("diffOperator_mex")
    rng = np.random.default_rng(8)
    for shape in [(41, 29), (9, 23, 12)]:
        x = rng.standard_normal(shape)
        for order in (2, 4):
            for dim in range(1, len(shape) + 1):
                c = co.dcoef(order)
                assert np.array_equal(ref.call(1, x, c, 7.5, dim)[0], co.diff_operator(x, c, 7.5, dim))


def test_fwd3d_restatement_with_reference_derivatives(oracle_mod, golden):
    """The 3D MATLAB file (src/fwdTimeCpmlFor3dAw.m) has no C in the reference, but
    its derivatives are the reference's C: on the MATLAB path diffOperator is
    src/fd_cmex/diffOperator.m, i.e. diffOperator_mex.c.  The numpy restatement
    run with that compiled gateway for every derivative reproduces the 3D golden
    vectors (from the C restatement) bit for bit, so only the file's
    elementwise statements remain restated."""
    if not (oracle_mod.REF_DIR / "diffOperator_mex.so").exists():
        pytest.skip("reference gateways not built here (no reference tree)")
    g = golden("fwd3d.npz")
    nz, nx, ny, nt, N, nB = (int(x) for x in g["params"])
    src = np.zeros((nz, nx, ny, nt), order="F")
    src[1, nx // 2, ny // 2, :] = g["trace"]
    diff = oracle_mod.reference_diff(oracle_mod.RefMex("diffOperator_mex"))
    d, s = oracle_mod.fwd3d_np(g["v"], src, N, nB, 10.0, 10.0, 10.0, 1e-3, diff=diff)
    assert np.array_equal(d, g["data"])
    assert np.array_equal(s[:, :, :, -1], g["snap_last"])


@pytest.mark.parametrize("k", range(4))
def test_sponge_restatements_match_golden(co, oracle_mod, golden, k):
    """The two sponge restatements (numpy and C; the reference's sponge
    propagators are MATLAB only, so these are its only pin) reproduce the
    committed vectors bit for bit, including the overlapping side bands
    (nx < 2 nB), nx == nB and the case without a sponge."""
    g = golden("sponge2d.npz")
    nz, nx, nt, nB = (int(x) for x in g[f"c{k}_params"])
    dz, dx, dt = (float(x) for x in g["dzdxdt"])
    v = g[f"c{k}_v"]
    src = dense_source(nz, nx, nt, g[f"c{k}_trace"], g[f"c{k}_imp"], g[f"c{k}_amp"])
    data, snap = oracle_mod.fwd_sponge_np(v, src, nB, dz, dx, dt)
    assert np.array_equal(data, g[f"c{k}_data"])
    assert np.array_equal(snap[:, :, nt // 2], g[f"c{k}_snap_mid"])
    assert np.array_equal(snap[:, :, -1], g[f"c{k}_snap_last"])
    dc, sc, _ = co.sponge2d(v, nt, nB, dz, dx, dt, source=src)
    assert np.array_equal(dc, data) and np.array_equal(sc, snap)
    _, rs, model = co.sponge2d(v, nt, nB, dz, dx, dt, rdata=data)
    assert np.array_equal(model, g[f"c{k}_model"])
    assert np.array_equal(rs[:, :, 0], g[f"c{k}_rsnap_first"])
    assert np.array_equal(rs[:, :, nt // 2], g[f"c{k}_rsnap_mid"])


def test_sponge_rtm_golden(co, oracle_mod, golden):
    g = golden("sponge2d.npz")
    nz, nx, nt, nB = (int(x) for x in g["rtm_params"])
    image, d_true, d_smooth = oracle_mod.rtm_sponge_np(g["rtm_v"], g["rtm_vs"], g["rtm_trace"], 0,
                                                       int(g["rtm_src_ix"]), nB, 10.0, 10.0, 1e-3, 1e-3)
    assert np.array_equal(image, g["rtm_image"])
    assert np.array_equal(d_true, g["rtm_data_true"]) and np.array_equal(d_smooth, g["rtm_data_smooth"])


def test_sponge_point_source_equals_dense(co, oracle_mod):
    """Point sources are the dense source with zeros elsewhere (the term
    vdtSq .* 0 subtracts nothing); two sources on one cell add up."""
    rng = np.random.default_rng(9)
    nz, nx, nt, nB = 21, 26, 30, 5
    v = rng.uniform(1500.0, 4000.0, (nz, nx))
    w = rng.standard_normal((3, nt))
    iz, ix = [2, 7, 7], [5, 11, 11]
    src = np.zeros((nz, nx, nt), order="F")
    for k in range(3):
        src[iz[k], ix[k], :] += w[k]
    d1, s1 = oracle_mod.fwd_sponge_np(v, src, nB, 10.0, 10.0, 1e-3)
    d2, s2 = oracle_mod.fwd_sponge_point_np(v, nt, iz, ix, w, nB, 10.0, 10.0, 1e-3)
    d3, s3, _ = co.sponge2d(v, nt, nB, 10.0, 10.0, 1e-3, point=(iz, ix, w))
    assert np.array_equal(d1, d2) and np.array_equal(s1, s2)
    assert np.array_equal(d2, d3) and np.array_equal(s2, s3)


def test_sponge_profile_values(oracle_mod):
    """boundary(k) = exp(-(0.015 (nB - k + 1))^2)^10: strongest at the outer
    cell, rising towards 1 inside."""
    b = oracle_mod.sponge_profile(20)
    assert b.shape == (20,)
    assert np.all(np.diff(b) > 0) and b[-1] < 1.0
    assert abs(b[0] - np.exp(-(0.3 ** 2)) ** 10) < 1e-15


def _elastic_case(golden, k):
    g = golden("elastic2d.npz")
    nz, nx, nt, N, nB = (int(x) for x in g[f"c{k}_params"])
    dz, dx, dt = (float(x) for x in g["dzdxdt"])
    src = dense_source(nz, nx, nt, g[f"c{k}_trace"], g[f"c{k}_imp"], g[f"c{k}_amp"])
    return g, nz, nx, nt, N, nB, dz, dx, dt, g[f"c{k}_vp"], g[f"c{k}_vs"], src


@pytest.mark.parametrize("k", range(4))
def test_elastic_restatement_matches_golden(oracle_mod, golden, k):
    """The numpy restatement of src/fwdTimeSpmlFor2dEw.m reproduces the committed
    vectors (made with the reference's compiled diffOperator_mex for every
    derivative) bit for bit."""
    g, nz, nx, nt, N, nB, dz, dx, dt, vp, vs, src = _elastic_case(golden, k)
    snaps = oracle_mod.fwd_elastic2d_np(vp, vs, src, N, nB, dz, dx, dt)
    for name, a in zip(("Vzp", "Vxp", "Vzs", "Vxs"), snaps):
        assert np.array_equal(a[:, :, nt // 2], g[f"c{k}_{name}_mid"]), name
        assert np.array_equal(a[:, :, -1], g[f"c{k}_{name}_last"]), name


def test_elastic_restatement_with_reference_derivatives(oracle_mod, golden):
    """Live, where the reference tree exists: the restatement run with the
    reference's own diffOperator_mex equals the one with its own derivative."""
    if not oracle_mod.available_reference():
        pytest.skip("reference gateways not built (SSSI_REFERENCE_SRC unset)")
    g, nz, nx, nt, N, nB, dz, dx, dt, vp, vs, src = _elastic_case(golden, 0)
    diff = oracle_mod.reference_diff(oracle_mod.RefMex("diffOperator_mex"))
    a = oracle_mod.fwd_elastic2d_np(vp, vs, src, N, nB, dz, dx, dt)
    b = oracle_mod.fwd_elastic2d_np(vp, vs, src, N, nB, dz, dx, dt, diff=diff)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def _elastic3d_case(golden, k):
    g = golden("elastic3d.npz")
    nz, nx, ny, nt, N, nB = (int(x) for x in g[f"c{k}_params"])
    dz, dx, dy, dt = (float(x) for x in g["spacing"])
    return g, nz, nx, ny, nt, N, nB, dz, dx, dy, dt


@pytest.mark.parametrize("k", range(3))
def test_elastic3d_restatement_matches_golden(oracle_mod, golden, k):
    """The numpy restatement of src/fwdTimeSpmlFor3dEw.m reproduces the
    committed vectors (made with the reference's compiled diffOperator_mex for
    every derivative) bit for bit."""
    g, nz, nx, ny, nt, N, nB, dz, dx, dy, dt = _elastic3d_case(golden, k)
    snaps = oracle_mod.fwd_elastic3d_np(g[f"c{k}_vp"], g[f"c{k}_vs"], g[f"c{k}_src_x"], g[f"c{k}_src_y"],
                                        g[f"c{k}_src_z"], N, nB, dz, dx, dy, dt)
    for name, a in zip(("Vzp", "Vxp", "Vyp", "Vzs", "Vxs", "Vys"), snaps):
        assert np.array_equal(a[:, :, :, nt // 2], g[f"c{k}_{name}_mid"]), name
        assert np.array_equal(a[:, :, :, -1], g[f"c{k}_{name}_last"]), name
