"""sssi_fwdTimeCpmlFor2dAwNoAlloc, the forward-modelling entry point that
allocates nothing, for callers that cannot allocate while they run (a service
whose GPU memory belongs to its own pool, a loop that cannot afford the
synchronisation of cudaMalloc/cudaFree).  It keeps its working state in a
fixed array inside the library; these tests check, through the C ABI, that two
calls in a row give the same result as the allocating entry point
sssi_fwdTimeCpmlFor2dAw (bit for bit in the strict FP64 mode, which also
reproduces the golden vectors of the reference C), and that grids too large
for the array and host pointers are refused.  The file name makes pytest
collect it last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _dev(a):
    import torch

    a = np.asarray(a)
    rev = tuple(reversed(range(a.ndim)))
    return torch.from_numpy(np.ascontiguousarray(a.transpose(rev))).cuda().permute(*rev)


def _zeros(shape):
    import torch

    return torch.zeros(tuple(reversed(shape)), dtype=torch.float64, device="cuda").permute(
        *reversed(range(len(shape))))


def _rel(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("shape", [(130, 170, 60, 4, 12), (37, 53, 40, 3, 5)])
def test_no_alloc_matches_allocating_entry_point(gpu, mode, shape):
    import torch

    from sssi_gb300._native import lib

    L = lib()
    nz, nx, nt, N, nB = shape
    rng = np.random.default_rng(nz + nx + mode)
    v = _dev(rng.uniform(1500.0, 4000.0, (nz, nx)))
    src = _dev(rng.standard_normal((nz, nx, nt)))
    args = (nz, nx, nt, N, nB, 10.0, 10.0, 5e-4)

    d_ref, s_ref = _zeros((nx, nt)), _zeros((nz, nx, nt))
    rc = L.sssi_fwdTimeCpmlFor2dAw(v.data_ptr(), src.data_ptr(), *args, d_ref.data_ptr(), s_ref.data_ptr(), mode)
    assert rc == 0, L.sssi_last_error()
    torch.cuda.synchronize()

    for call in range(2):  # two calls in a row: the second starts from the first's leftovers
        d, s = _zeros((nx, nt)), _zeros((nz, nx, nt))
        rc = L.sssi_fwdTimeCpmlFor2dAwNoAlloc(v.data_ptr(), src.data_ptr(), *args, d.data_ptr(), s.data_ptr(),
                                              mode)
        assert rc == 0, L.sssi_last_error()
        torch.cuda.synchronize()
        if mode == 0:  # strict FP64: the same bits as the allocating entry point
            assert torch.equal(d, d_ref) and torch.equal(s, s_ref), call
        assert _rel(d, d_ref) <= TOL_FP64, call
        assert _rel(s, s_ref) <= TOL_FP64, call
        assert float(d.abs().max()) > 0


@pytest.mark.parametrize("k", [0, 7, 14])
def test_no_alloc_strict_reproduces_golden(gpu, golden, k):
    """Strict FP64 through the fixed array reproduces the reference C's outputs."""
    import torch

    from sssi_gb300._native import lib
    from tests.golden.make_golden import dense_source

    L = lib()
    g = golden("fwd2d_rvs2d.npz")
    nz, nx, nt, N, nB = (int(x) for x in g[f"c{k}_params"])
    v = _dev(g[f"c{k}_v"])
    src = _dev(dense_source(nz, nx, nt, g[f"c{k}_trace"], g[f"c{k}_imp"], g[f"c{k}_amp"]))
    for call in range(2):
        d, s = _zeros((nx, nt)), _zeros((nz, nx, nt))
        rc = L.sssi_fwdTimeCpmlFor2dAwNoAlloc(v.data_ptr(), src.data_ptr(), nz, nx, nt, N, nB, 10.0, 10.0, 1e-3,
                                              d.data_ptr(), s.data_ptr(), 0)
        assert rc == 0, L.sssi_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), g[f"c{k}_data"]), call
        assert np.array_equal(s[:, :, nt // 2].cpu().numpy(), g[f"c{k}_snap_mid"]), call
        assert np.array_equal(s[:, :, -1].cpu().numpy(), g[f"c{k}_snap_last"]), call


def test_no_alloc_refuses_oversize_grid(gpu):
    from sssi_gb300._native import lib

    L = lib()
    nz, nx = 2000, 3000
    v = _dev(np.full((nz, nx), 2000.0))
    d = _zeros((nx, 2))
    rc = L.sssi_fwdTimeCpmlFor2dAwNoAlloc(v.data_ptr(), None, nz, nx, 2, 4, 20, 10.0, 10.0, 1e-3, d.data_ptr(),
                                          None, 1)
    assert rc == 1
    msg = L.sssi_last_error().decode()
    assert "fixed" in msg and "bytes" in msg


def test_no_alloc_refuses_host_memory(gpu):
    from sssi_gb300._native import lib

    L = lib()
    v = np.full((40, 50), 2000.0, order="F")
    d = np.zeros((50, 3), order="F")
    rc = L.sssi_fwdTimeCpmlFor2dAwNoAlloc(v.ctypes.data, None, 40, 50, 3, 4, 5, 10.0, 10.0, 1e-3, d.ctypes.data,
                                          None, 1)
    assert rc == 1 and b"device memory" in L.sssi_last_error()
    assert ctypes.c_int(rc).value == 1
