"""diffOperator (src/fd_cmex/diffOperator_mex.c:29-213) on the GPU, through the
C ABI and the MEX gateway: strict FP64 bit-identical to the reference's golden
outputs and to the oracle, fused FP64 within 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _cases(g):
    for key in g.files:
        if key.startswith("d"):
            nd = int(key[1])
            order = int(key.split("_o")[1].split("_")[0])
            dim = int(key.split("dim")[1])
            yield key, g[f"x{nd}"], g[f"c{order}"], dim if dim <= nd else nd


def test_diff_operator_golden(gpu, golden, oracle_mod):
    S = gpu
    g = golden("diffop.npz")
    for key, x, c, dim in _cases(g):
        assert np.array_equal(S.diffOperator(x, c, 10.0, dim, mode="fp64-strict"), g[key]), key
        assert oracle_mod.rel_l2(S.diffOperator(x, c, 10.0, dim), g[key]) <= TOL_FP64, key


@pytest.mark.parametrize("shape", [(300, 257), (64, 70, 90), (5, 200, 33), (130, 1, 40)])
def test_diff_operator_vs_oracle(gpu, co, shape):
    S = gpu
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    for order in (1, 3, 4, 8):
        c = co.dcoef(order)
        for dim in range(1, len(shape) + 1):
            if shape[dim - 1] < 2 * order - 1:
                continue
            ref = co.diff_operator(x, c, 12.5, dim)
            assert np.array_equal(S.diffOperator(x, c, 12.5, dim, mode="fp64-strict"), ref), (order, dim)
            got = S.diffOperator(x, c, 12.5, dim)
            if ref.size and np.abs(ref).max() > 0:
                assert float(np.linalg.norm(got - ref) / np.linalg.norm(ref)) <= TOL_FP64


def test_diff_operator_device_and_empty(gpu, co):
    import torch

    S = gpu
    rng = np.random.default_rng(2)
    x = rng.standard_normal((40, 30, 20))
    c = co.dcoef(4)
    xd = torch.from_numpy(np.ascontiguousarray(x.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    out = S.diffOperator(xd, c, 10.0, 3, mode="fp64-strict")
    assert out.is_cuda and tuple(out.shape) == (40, 30, 13)
    assert np.array_equal(out.cpu().numpy(), co.diff_operator(x, c, 10.0, 3))
    assert S.diffOperator(x[:, :7, :], c, 10.0, 2).shape == (40, 0, 20)  # the stencil exactly fills the dimension


def test_diff_operator_mex_gateway(gpu, golden, oracle_mod, monkeypatch):
    """diffData = diffOperator_mex(data, c, d, dim) through the shim, default and strict."""
    import subprocess
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    subprocess.run(["make", "-s", "-C", str(root / "oracle"), "mexgw"], check=True)
    gw = oracle_mod.load_shim_library(root / "oracle" / "_build" / "mexgw_diffOperator_mex.so")
    g = golden("diffop.npz")
    for mode in (None, "strict"):
        if mode:
            monkeypatch.setenv("SSSI_MEX_MODE", mode)
        else:
            monkeypatch.delenv("SSSI_MEX_MODE", raising=False)
        for key in g.files:
            if not key.startswith("d"):
                continue
            nd = int(key[1])
            order = int(key.split("_o")[1].split("_")[0])
            dim = int(key.split("dim")[1])  # the gateway applies the reference's dim rule itself
            (out,) = oracle_mod.shim_call(gw, 1, g[f"x{nd}"], g[f"c{order}"], 10.0, dim)
            if mode == "strict":
                assert np.array_equal(out, g[key]), key
            else:
                assert oracle_mod.rel_l2(out, g[key]) <= TOL_FP64, key
        # dim defaults to 1
        (out,) = oracle_mod.shim_call(gw, 1, g["x2"], g["c4"], 10.0)
        assert out.shape == g["d2_o4_dim1"].shape
