"""MAT-file persistence (the applications' save/load of seismograms, snapshots
and images, mainRtmTimeCpmlFor2dAw.m:170-183,250-266,348-351): the library's
Level-5 writer and reader against scipy.io, host arrays (no GPU needed)."""
import numpy as np
import pytest

sio = pytest.importorskip("scipy.io")


@pytest.fixture(scope="module")
def S():
    import sssi_gb300

    return sssi_gb300


def test_write_then_scipy_reads(S, tmp_path):
    rng = np.random.default_rng(1)
    arrays = {"dataTrue": rng.standard_normal((37, 53)), "snapshotSmooth": rng.standard_normal((9, 11, 7)),
              "four": rng.standard_normal((3, 4, 5, 2)), "StackedRTM": np.asfortranarray(rng.standard_normal((20, 30)))}
    path = tmp_path / "a.mat"
    S.mat_write(path, arrays)
    m = sio.loadmat(path)
    for k, a in arrays.items():
        assert m[k].shape == a.shape and np.array_equal(m[k], a), k


def test_scipy_writes_then_read(S, tmp_path):
    rng = np.random.default_rng(2)
    a = rng.standard_normal((41, 17))
    path = tmp_path / "b.mat"
    # uncompressed Level 5, as save(..., '-v6') writes; small integer arrays land in narrow types
    sio.savemat(path, {"dataSmooth": a, "small": np.array([[3.0]]), "ints": np.arange(6, dtype=np.int16).reshape(2, 3),
                       "cube": rng.standard_normal((4, 5, 6))}, do_compression=False)
    assert np.array_equal(S.mat_read(path, "dataSmooth"), a)
    assert S.mat_read(path, "small").tolist() == [[3.0]]
    assert np.array_equal(S.mat_read(path, "ints"), np.arange(6).reshape(2, 3))
    out = np.zeros((4, 5, 6), order="F")
    S.mat_read(path, "cube", out=out)
    assert np.array_equal(out, sio.loadmat(path)["cube"])


def test_round_trip_and_empty(S, tmp_path):
    path = tmp_path / "c.mat"
    S.mat_write(path, {"e": np.zeros((0, 5)), "v": np.arange(7.0)})
    assert S.mat_read(path, "e").shape == (0, 5)
    assert S.mat_read(path, "v").shape == (7, 1)  # MATLAB arrays have two dimensions at least


def test_errors(S, tmp_path):
    path = tmp_path / "d.mat"
    sio.savemat(path, {"x": np.ones((3, 3))}, do_compression=True)
    with pytest.raises(S.SSSIError, match="compressed"):
        S.mat_read(path, "x")
    S.mat_write(path, {"x": np.ones((3, 3))})
    with pytest.raises(S.SSSIError, match="no variable named y"):
        S.mat_read(path, "y")
    with pytest.raises(S.SSSIError, match="capacity"):
        S.mat_read(path, "x", out=np.zeros(4))
    with pytest.raises(S.SSSIError, match="name"):
        S.mat_write(path, {"n" * 64: np.ones(2)})


def test_size_limit_checked_before_any_access(S, tmp_path):
    """A variable above the format's 4 GiB element limit is refused from its
    shape alone (the data pointer is never read)."""
    import ctypes

    lib = S._native.lib()
    dims = np.array([70000, 70000], dtype=np.int64)
    names = (ctypes.c_char_p * 1)(b"big")
    arrs = (ctypes.c_void_p * 1)(1)  # never dereferenced
    nd = (ctypes.c_int * 1)(2)
    dp = (ctypes.c_void_p * 1)(dims.ctypes.data)
    rc = lib.sssi_mat_write(str(tmp_path / "e.mat").encode(), 1, ctypes.addressof(names), ctypes.addressof(arrs),
                            ctypes.addressof(nd), ctypes.addressof(dp))
    assert rc == 1 and b"4 GiB" in lib.sssi_last_error()
