"""The C ABI without a GPU: the library loads, exports every symbol the header
declares, computes the host-side building blocks exactly like the oracle, and
turns bad arguments (and a missing GPU) into status codes, not crashes."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "sssi_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sssi_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from sssi_gb300 import _native
    from sssi_gb300.build import LIB, build_library

    if not LIB.exists():
        build_library()
    return _native.lib()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from sssi_gb300._native import SIGNATURES

    missing = [s for s in declared_symbols() if s not in SIGNATURES]
    assert not missing, missing


def test_dcoef_matches_oracle(lib, co):
    import sssi_gb300 as S

    for N in range(1, 9):
        assert np.array_equal(S.dCoef(N), co.dcoef(N)), N
    from sssi_gb300._native import SSSIError

    with pytest.raises(SSSIError, match="order"):
        S.dCoef(9)


def test_damppml_matches_reference_golden(lib, golden):
    import sssi_gb300 as S

    g = golden("damppml.npz")
    nB, dx = int(g["nB"]), float(g["dx"])
    assert np.array_equal(S.dampPml(g["u_left"], g["v"][:, :nB], nB * dx), g["d_left"])
    assert np.array_equal(S.dampPml(g["u_bot"], g["v"][30 - nB:, :], nB * dx), g["d_bot"])


def test_bad_arguments_are_status_codes(lib):
    v = np.full((20, 30), 2000.0, order="F")
    src = np.zeros((20, 30, 5), order="F")
    out = np.zeros((30, 5), order="F")
    p = lambda a: a.ctypes.data  # noqa: E731
    # nDiffOrder out of range
    rc = lib.sssi_fwdTimeCpmlFor2dAw(p(v), p(src), 20, 30, 5, 0, 3, 10.0, 10.0, 1e-3, p(out), None, 0)
    assert rc == 1 and b"nDiffOrder" in lib.sssi_last_error()
    # negative spacing
    rc = lib.sssi_rvsTimeCpmlFor2dAw(p(v), p(out), 20, 30, 5, 4, 3, -10.0, 10.0, 1e-3, None, None, 0)
    assert rc == 1
    # unknown mode
    rc = lib.sssi_fwdTimeCpmlFor2dAw(p(v), p(src), 20, 30, 5, 4, 3, 10.0, 10.0, 1e-3, p(out), None, 9)
    assert rc == 1 and b"mode" in lib.sssi_last_error()
    # a source outside the model
    img = np.zeros((20, 30), order="F")
    w = np.zeros(5)
    rc = lib.sssi_rtmTimeCpmlFor2dAw(p(v), p(v), 20, 30, 5, 4, 3, 10.0, 10.0, 1e-3, p(w), 25, 3, 1e-3, 2, 4,
                                     p(img), None, None)
    assert rc == 1 and b"outside" in lib.sssi_last_error()


def test_no_gpu_is_a_status_code(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    v = np.full((20, 30), 2000.0, order="F")
    src = np.zeros((20, 30, 5), order="F")
    out = np.zeros((30, 5), order="F")
    rc = lib.sssi_fwdTimeCpmlFor2dAw(v.ctypes.data, src.ctypes.data, 20, 30, 5, 4, 3, 10.0, 10.0, 1e-3,
                                     out.ctypes.data, None, 0)
    assert rc == 2, lib.sssi_last_error()


def test_mex_gateways_export_mexfunction():
    """This project's gateways, built on the test shim, export the MEX entry point."""
    import subprocess

    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "mexgw"], check=True)
    for name in ("fwdTimeCpmlFor2dAw_mex", "rvsTimeCpmlFor2dAw_mex", "fwdTimeCpmlFor3dAw_mex",
                 "fwdTimeSpongeFor2dAw_mex", "rvsTimeSpongeFor2dAw_mex", "fwdTimeSpmlFor2dEw_mex",
                 "fwdTimeSpmlFor3dEw_mex"):
        gw = ctypes.CDLL(str(ROOT / "oracle" / "_build" / f"mexgw_{name}.so"), mode=ctypes.RTLD_LOCAL)
        assert hasattr(gw, "mexFunction")


def test_mex_gateway_error_message():
    """Too few arguments: the reference's message, raised through mexErrMsgTxt."""
    from oracle import oracle as O

    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeCpmlFor2dAw_mex.so")
    with pytest.raises(O.MexError, match="All 7 input arguments shall be provided!"):
        O.shim_call(gw, 2, np.ones((3, 3)), np.zeros((3, 3, 2)))


def test_mex_gateway_3d_error_message():
    """The 3D gateway: too few arguments is refused before any GPU work."""
    from oracle import oracle as O

    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeCpmlFor3dAw_mex.so")
    with pytest.raises(O.MexError, match="All 8 input arguments shall be provided!"):
        O.shim_call(gw, 2, np.ones((3, 3, 3)), np.zeros((3, 3, 3, 2)), 2, 1, 10.0, 10.0, 10.0)


def test_no_alloc_rejects_sizes_out_of_range(lib):
    """The no-allocation entry point bounds nz, nx and nt before any size
    arithmetic (a huge nx must not wrap into a small layout), without a GPU."""
    big = (1 << 61) + 1000
    for nz, nx, nt in ((40, big, 3), (big, 40, 3), (40, 40, 1 << 40), (1 << 29, 1 << 29, 1 << 20)):
        rc = lib.sssi_fwdTimeCpmlFor2dAwNoAlloc(None, None, nz, nx, nt, 4, 5, 10.0, 10.0, 1e-3, None, None, 1)
        assert rc == 1, (nz, nx, nt)
        assert b"out of range" in lib.sssi_last_error()


def test_diff_operator_gateway_error_message():
    """diffOperator_mex with too few arguments: the reference's message."""
    from oracle import oracle as O

    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_diffOperator_mex.so")
    with pytest.raises(O.MexError, match="Input data, finite difference coefficients and distance per sample"):
        O.shim_call(gw, 1, np.ones((5, 5)), np.ones(2))


def test_diff_operator_bad_arguments(lib):
    x = np.ones((10, 10), order="F")
    dims = np.array([10, 10], dtype=np.int64)
    c = np.array([1.0, 0.1])
    out = np.zeros((7, 10), order="F")
    p = lambda a: a.ctypes.data  # noqa: E731
    assert lib.sssi_diffOperator(p(x), 4, p(dims), p(c), 2, 1.0, 1, p(out), 1) == 1  # ndims
    assert lib.sssi_diffOperator(p(x), 2, p(dims), p(c), 2, 1.0, 3, p(out), 1) == 1  # dim
    assert lib.sssi_diffOperator(p(x), 2, p(dims), p(c), 2, 0.0, 1, p(out), 1) == 1  # distance
    assert lib.sssi_diffOperator(p(x), 2, p(dims), p(c), 2, 1.0, 1, p(out), 2) == 1  # mode
    assert b"mode" in lib.sssi_last_error()


def test_sponge_bad_arguments(lib):
    v = np.full((20, 30), 2000.0, order="F")
    src = np.zeros((20, 30, 5), order="F")
    out = np.zeros((30, 5), order="F")
    p = lambda a: a.ctypes.data  # noqa: E731
    # the sponge must lie inside the grid
    rc = lib.sssi_fwdTimeSpongeFor2dAw(p(v), p(src), 20, 30, 5, 21, 10.0, 10.0, 1e-3, p(out), None, 1)
    assert rc == 1 and b"nBoundary" in lib.sssi_last_error()
    rc = lib.sssi_rvsTimeSpongeFor2dAw(p(v), p(out), 20, 30, 5, 3, 10.0, 0.0, 1e-3, None, None, 1)
    assert rc == 1
    rc = lib.sssi_fwdTimeSpongeFor2dAw(p(v), p(src), 20, 30, 5, 3, 10.0, 10.0, 1e-3, p(out), None, 7)
    assert rc == 1 and b"mode" in lib.sssi_last_error()
    img = np.zeros((20, 30), order="F")
    w = np.zeros(5)
    rc = lib.sssi_rtmTimeSpongeFor2dAw(p(v), p(v), 20, 30, 5, 3, 10.0, 10.0, 1e-3, p(w), 2, 3, 1e-3, 2, p(img),
                                       None, None)
    assert rc == 1 and b"FP64" in lib.sssi_last_error()  # the sponge RTM shot is FP64 only
    iz = np.array([25], dtype=np.int64)
    ix = np.array([3], dtype=np.int64)
    rc = lib.sssi_fwdTimeSpongeFor2dAwPoint(p(v), 20, 30, 5, 3, 10.0, 10.0, 1e-3, 65, p(iz), p(ix), p(w), p(out),
                                            None, 1)
    assert rc == 1 and b"nsrc" in lib.sssi_last_error()


def test_sponge_gateway_error_messages():
    from oracle import oracle as O

    for name in ("fwdTimeSpongeFor2dAw_mex", "rvsTimeSpongeFor2dAw_mex"):
        gw = O.load_shim_library(ROOT / "oracle" / "_build" / f"mexgw_{name}.so")
        with pytest.raises(O.MexError, match="All 6 input arguments shall be provided!"):
            O.shim_call(gw, 2, np.ones((3, 3)), np.zeros((3, 3, 2)))


def test_elastic_bad_arguments(lib):
    v = np.full((20, 30), 2000.0, order="F")
    src = np.zeros((20, 30, 5), order="F")
    p = lambda a: a.ctypes.data  # noqa: E731
    # side bands may not overlap (the reference concatenates [left, zeros(nx - 2nB), right])
    rc = lib.sssi_fwdTimeSpmlFor2dEw(p(v), p(v), p(src), 20, 30, 5, 3, 16, 10.0, 10.0, 1e-3, None, None, None, None, 1)
    assert rc == 1 and b"nBoundary" in lib.sssi_last_error()
    rc = lib.sssi_fwdTimeSpmlFor2dEw(p(v), p(v), p(src), 20, 30, 5, 9, 3, 10.0, 10.0, 1e-3, None, None, None, None, 1)
    assert rc == 1 and b"nDiffOrder" in lib.sssi_last_error()
    rc = lib.sssi_fwdTimeSpmlFor2dEw(p(v), p(v), p(src), 20, 30, 5, 3, 3, 10.0, 10.0, 1e-3, None, None, None, None, 5)
    assert rc == 1 and b"mode" in lib.sssi_last_error()


def test_elastic_gateway_error_message():
    from oracle import oracle as O

    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeSpmlFor2dEw_mex.so")
    with pytest.raises(O.MexError, match="All 8 input arguments shall be provided!"):
        O.shim_call(gw, 4, np.ones((3, 3)), np.ones((3, 3)), np.zeros((3, 3, 2)))


def test_elastic3d_bad_arguments_and_gateway_message(lib):
    from oracle import oracle as O

    v = np.full((10, 12, 14), 2000.0, order="F")
    p = lambda a: a.ctypes.data  # noqa: E731
    rc = lib.sssi_fwdTimeSpmlFor3dEw(p(v), p(v), None, None, None, 10, 12, 14, 5, 3, 7, 10.0, 10.0, 10.0, 1e-3,
                                     None, None, None, None, None, None, 1)
    assert rc == 1 and b"nBoundary" in lib.sssi_last_error()  # 2 nB > nx
    gw = O.load_shim_library(ROOT / "oracle" / "_build" / "mexgw_fwdTimeSpmlFor3dEw_mex.so")
    with pytest.raises(O.MexError, match="All 11 input arguments shall be provided!"):
        O.shim_call(gw, 6, v, v)


def test_debug_entries_check_arguments(lib):
    """The test entries of the strict division and the 3D schedule tuner reject
    bad arguments before touching a GPU; with no 3D propagation tuned yet the
    schedule query reports -1 (this process has run none)."""
    fast = np.zeros(4)
    ieee = np.zeros(4)
    a = np.ones(4)
    assert lib.sssi_debug_divide(a.ctypes.data, -1, 10.0, fast.ctypes.data, ieee.ctypes.data) == 1
    assert lib.sssi_debug_divide(None, 4, 10.0, fast.ctypes.data, ieee.ctypes.data) == 1
    assert b"NULL" in lib.sssi_last_error()
    assert lib.sssi_debug_divide(None, 0, 10.0, None, None) == 0  # nothing to divide
    assert lib.sssi_debug_schedule3d(None, None) == 1
    import ctypes

    sched = ctypes.c_int(7)
    ms = (ctypes.c_float * 4)()
    assert lib.sssi_debug_schedule3d(ctypes.byref(sched), ms) == 0
    assert sched.value == -1 and list(ms) == [0.0] * 4
