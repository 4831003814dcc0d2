"""CPU oracle for SSSI's acoustic CPML finite-difference hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg import this module, and only as the checker;
the product (``sssi_gb300``) never imports it.

Three layers, each pinned against the next:

* :class:`RefMex` -- the reference's own C gateways
  (``src/fd_cmex/fwdTimeCpmlFor2dAw_mex.c``, ``rvsTimeCpmlFor2dAw_mex.c``)
  compiled unmodified against the project's ``mex.h`` shim into
  ``oracle/_ref/`` (``make -C oracle ref``).  Available only where the
  reference tree exists; it pins the two restatements below and generates the
  committed golden vectors in ``tests/golden/``.
* :class:`COracle` -- ``oracle/sssi_oracle.c``, a C99 restatement of the same
  algorithm (2D forward/reverse, 3D forward, imaging), bit-identical to
  :class:`RefMex` on every case the tests run.  It is the checker on machines
  without the reference tree and the CPU baseline timed by ``bench.py``.
* the numpy functions below -- a vectorised restatement of the MATLAB twins
  (``src/fd_matlab/fwdTimeCpmlFor2dAw.m:88-119``,
  ``src/fd_matlab/rvsTimeCpmlFor2dAw.m:82-127``, ``src/fwdTimeCpmlFor3dAw.m:110-147``)
  with the same operation order, used for small cases and for the 3D path,
  which has no C in the reference.

Array conventions follow MATLAB: a model ``v`` is indexed ``v[z, x]`` (or
``v[z, x, y]``), sources ``source[z, x, t]``, data ``data[x, t]``, snapshots
``snapshot[z, x, t]``; all are handed to C as column-major (Fortran) memory.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
REF_DIR = ORACLE_DIR / "_ref"
# The reference's src/fd_cmex directory, where its tree exists (the environment
# variable SSSI_REFERENCE_SRC); without it the reference gateways are not built
# and the tests that need them skip.
_REF_ENV = os.environ.get("SSSI_REFERENCE_SRC", "")
REFERENCE_SRC = Path(_REF_ENV) if _REF_ENV else None

_i64 = ctypes.c_int64
# glibc's log/exp, as the C gateways use (numpy's vectorised loops may round differently)
_LOGR = math.log(1e-6)
_exp = np.vectorize(math.exp, otypes=[float])
_dp = ctypes.POINTER(ctypes.c_double)


def build(reference: bool | None = None) -> None:
    """Compile the C restatement (always) and the reference gateways (when the
    reference tree is present, or when ``reference`` is True)."""
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "all"], check=True)
    if reference is None:
        reference = REFERENCE_SRC is not None and (REFERENCE_SRC / "fwdTimeCpmlFor2dAw_mex.c").exists()
    if reference:
        if REFERENCE_SRC is None:
            raise RuntimeError("set SSSI_REFERENCE_SRC to the reference's src/fd_cmex directory")
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "ref", f"REF_SRC={REFERENCE_SRC}"], check=True)


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _f64(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


# --------------------------------------------------------------------------
# C restatement
# --------------------------------------------------------------------------
class COracle:
    """ctypes view of ``oracle/_build/liboracle.so`` (build it with :func:`build`)."""

    def __init__(self, path: Path | None = None):
        path = Path(path or BUILD_DIR / "liboracle.so")
        if not path.exists():
            build(reference=False)
        self.lib = ctypes.CDLL(str(path))
        L = self.lib
        L.orc_dcoef.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
        L.orc_damp_pml.argtypes = [_dp, _dp, _i64, ctypes.c_double, _dp]
        L.orc_damping_2d.argtypes = [_dp, _i64, _i64, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, _dp, _dp]
        L.orc_damping_3d.argtypes = [_dp, _i64, _i64, _i64, ctypes.c_int, ctypes.c_double, _dp, _dp, _dp]
        L.orc_fwd2d.argtypes = [_dp, _dp, _dp, _i64, _i64, _i64, _i64, _i64, ctypes.c_int, ctypes.c_int,
                                ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _dp]
        L.orc_rvs2d.argtypes = [_dp, _dp, _i64, _i64, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp, _dp]
        L.orc_fwd3d.argtypes = [_dp, _dp, _dp, _i64, _i64, _i64, _i64, _i64, _i64, _i64, ctypes.c_int,
                                ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                _dp, _dp]
        L.orc_image_accum.argtypes = [_dp, _dp, _i64, _dp, _dp]
        L.orc_image_stack.argtypes = [_dp, _dp, _i64, _dp]
        L.orc_diff_operator.argtypes = [_dp, _i64, _i64, _i64, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp]
        L.orc_sponge2d.argtypes = [_dp, _i64, _i64, _i64, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, _dp, ctypes.c_int, ctypes.POINTER(_i64), ctypes.POINTER(_i64), _dp,
                                   _dp, _dp, _dp, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_num_threads.argtypes = [ctypes.c_int]

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_num_threads(int(n))

    def threads(self) -> int:
        return int(self.lib.orc_num_threads())

    def diff_operator(self, data, c, d, dim=1) -> np.ndarray:
        """diffOperator (src/fd_cmex/diffOperator_mex.c:29-213) of a 2D or 3D array."""
        data = _f64(data)
        c = np.ascontiguousarray(np.atleast_1d(np.asarray(c, dtype=np.float64)).ravel())
        shape = list(data.shape) + [1] * (3 - data.ndim)
        oshape = list(data.shape)
        oshape[dim - 1] -= 2 * len(c) - 1
        out = np.zeros(oshape, order="F")
        self.lib.orc_diff_operator(_ptr(data), shape[0], shape[1], shape[2], _ptr(c), len(c), float(d), int(dim),
                                   _ptr(out))
        return out

    def sponge2d(self, v, nt, nB, dz, dx, dt, *, source=None, point=None, rdata=None, want_snapshot=True):
        """Sponge propagation (src/fwdTimeSpongeFor2dAw.m, src/rvsTimeSpongeFor2dAw.m):
        ``source`` dense (nz, nx, nt), or ``point=(iz, ix, wavelets)``, or ``rdata``
        (nx, nt) for the reverse pass.  Returns (data, snapshot, last)."""
        v = _f64(v)
        nz, nx = v.shape
        src = _f64(source) if source is not None else None
        iz = ix = w = None
        nsrc = 0
        if point is not None:
            iz = np.ascontiguousarray(np.atleast_1d(point[0]), dtype=np.int64)
            ix = np.ascontiguousarray(np.atleast_1d(point[1]), dtype=np.int64)
            w = np.ascontiguousarray(np.atleast_2d(np.asarray(point[2], dtype=np.float64)))
            nsrc = len(iz)
        rd = _f64(rdata) if rdata is not None else None
        data = np.zeros((nx, nt), order="F")
        snap = np.zeros((nz, nx, nt), order="F") if want_snapshot else None
        last = np.zeros((nz, nx), order="F")
        ip = (lambda a: a.ctypes.data_as(ctypes.POINTER(_i64)) if a is not None else None)
        rc = self.lib.orc_sponge2d(_ptr(v), nz, nx, int(nt), int(nB), float(dz), float(dx), float(dt), _ptr(src),
                                   nsrc, ip(iz), ip(ix), _ptr(w), _ptr(rd), _ptr(data), _ptr(snap), _ptr(last))
        if rc:
            raise MemoryError("orc_sponge2d: allocation failed")
        return data, snap, last

    def dcoef(self, order: int) -> np.ndarray:
        c = np.zeros(order)
        if self.lib.orc_dcoef(order, 1, _ptr(c)):
            raise ValueError("order out of range")
        return c

    def damping_2d(self, v, nB, dz, dx, dt):
        v = _f64(v)
        nz, nx = v.shape
        xb = np.zeros((nz, nx), order="F")
        zb = np.zeros((nz, nx), order="F")
        self.lib.orc_damping_2d(_ptr(v), nz, nx, nB, dz, dx, dt, _ptr(xb), _ptr(zb))
        return xb, zb

    def damping_3d(self, v, nB, dt):
        v = _f64(v)
        nz, nx, ny = v.shape
        out = [np.zeros((nz, nx, ny), order="F") for _ in range(3)]
        self.lib.orc_damping_3d(_ptr(v), nz, nx, ny, nB, dt, *[_ptr(a) for a in out])
        return tuple(out)

    def fwd2d(self, v, source, N, nB, dz, dx, dt, *, nt=None, point=None, want_snapshot=True):
        """Forward modelling.  ``source`` dense (nz, nx, nt), or None with
        ``point=(trace, iz, ix)`` for a single point source."""
        v = _f64(v)
        nz, nx = v.shape
        if source is not None:
            source = _f64(source)
            nt = source.shape[2]
            trace, iz, ix = None, 0, 0
        else:
            trace, iz, ix = point
            trace = np.ascontiguousarray(trace, dtype=np.float64)
            nt = nt or trace.shape[0]
        data = np.zeros((nx, nt), order="F")
        snap = np.zeros((nz, nx, nt), order="F") if want_snapshot else None
        rc = self.lib.orc_fwd2d(_ptr(v), _ptr(source), _ptr(trace), iz, ix, nz, nx, nt, N, nB, dz, dx, dt,
                                _ptr(data), _ptr(snap))
        if rc:
            raise ValueError("orc_fwd2d failed")
        return data, snap

    def rvs2d(self, v, data, N, nB, dz, dx, dt, *, want_snapshot=True, fwd_snapshot=None):
        v = _f64(v)
        data = _f64(data)
        nz, nx = v.shape
        nt = data.shape[1]
        l = 2 * N - 1
        model = np.zeros((nz + 2 * l, nx + 2 * l), order="F")
        snap = np.zeros((nz, nx, nt), order="F") if want_snapshot else None
        m = s2 = None
        if fwd_snapshot is not None:
            fwd_snapshot = _f64(fwd_snapshot)
            m = np.zeros((nz, nx), order="F")
            s2 = np.zeros((nz, nx), order="F")
        rc = self.lib.orc_rvs2d(_ptr(v), _ptr(data), nz, nx, nt, N, nB, dz, dx, dt, _ptr(model), _ptr(snap),
                                _ptr(fwd_snapshot), _ptr(m), _ptr(s2))
        if rc:
            raise ValueError("orc_rvs2d failed")
        if fwd_snapshot is not None:
            return model, snap, m, s2
        return model, snap

    def fwd3d(self, v, source, N, nB, dz, dx, dy, dt, *, nt=None, point=None, want_snapshot=True):
        v = _f64(v)
        nz, nx, ny = v.shape
        if source is not None:
            source = _f64(source)
            nt = source.shape[3]
            trace, iz, ix, iy = None, 0, 0, 0
        else:
            trace, iz, ix, iy = point
            trace = np.ascontiguousarray(trace, dtype=np.float64)
            nt = nt or trace.shape[0]
        data = np.zeros((nx, ny, nt), order="F")
        snap = np.zeros((nz, nx, ny, nt), order="F") if want_snapshot else None
        rc = self.lib.orc_fwd3d(_ptr(v), _ptr(source), _ptr(trace), iz, ix, iy, nz, nx, ny, nt, N, nB, dz, dx, dy,
                                dt, _ptr(data), _ptr(snap))
        if rc:
            raise ValueError("orc_fwd3d failed")
        return data, snap

    def image(self, fwd_snap, rvs_snap, epsilon):
        """M./s2 with the sums taken in ascending time order
        (mainRtmTimeCpmlFor2dAw.m:268-275)."""
        f = _f64(fwd_snap)
        r = _f64(rvs_snap)
        nz, nx, nt = f.shape
        m = np.zeros((nz, nx), order="F")
        s2 = np.full((nz, nx), float(epsilon), order="F")
        for t in range(nt):
            ft = np.asfortranarray(f[:, :, t])
            rt = np.asfortranarray(r[:, :, t])
            self.lib.orc_image_accum(_ptr(ft), _ptr(rt), nz * nx, _ptr(m), _ptr(s2))
        return m, s2

    def rtm2d(self, v, vs, trace, src_iz, src_ix, N, nB, dz, dx, dt, epsilon):
        """One reference RTM shot (mainRtmTimeCpmlFor2dAw.m:156-166,252-275,315):
        data in V and VS, reverse propagation of their difference in V, zero-lag
        imaging against the VS forward snapshots.  Returns (image, dataTrue,
        dataSmooth) with image = M ./ s2 (one shot's contribution to Stacked)."""
        d_true, _ = self.fwd2d(v, None, N, nB, dz, dx, dt, point=(trace, src_iz, src_ix), want_snapshot=False)
        d_smooth, f_snap = self.fwd2d(vs, None, N, nB, dz, dx, dt, point=(trace, src_iz, src_ix))
        delta = d_true - d_smooth
        _, r_snap = self.rvs2d(v, delta, N, nB, dz, dx, dt)
        m, s2 = self.image(f_snap, r_snap, epsilon)
        stacked = np.zeros_like(m, order="F")
        self.lib.orc_image_stack(_ptr(m), _ptr(s2), m.size, _ptr(stacked))
        return stacked, d_true, d_smooth


# --------------------------------------------------------------------------
# reference gateways on the shim
# --------------------------------------------------------------------------
class RefMex:
    """One reference MEX gateway compiled from the reference tree on the shim.

    ``name`` is the gateway file stem, e.g. ``fwdTimeCpmlFor2dAw_mex``;
    ``variant`` is "" (parity build), "_o3" (reference flags) or "openmp".
    """

    def __init__(self, name: str, variant: str = ""):
        if variant == "openmp":
            stem = name.replace("_mex", "_openmp_mex")
        else:
            stem = name + variant
        path = REF_DIR / f"{stem}.so"
        if not path.exists():
            raise FileNotFoundError(f"{path} (build with `make -C oracle ref` where the reference tree exists)")
        self.lib = load_shim_library(path)

    def call(self, nlhs: int, *args):
        return shim_call(self.lib, nlhs, *args)

    def dcoef(self, order: int) -> np.ndarray:
        self.lib.dCoef.restype = _dp
        self.lib.dCoef.argtypes = [ctypes.c_int, ctypes.c_char_p]
        p = self.lib.dCoef(order, b"s")
        return np.array([p[i] for i in range(order)])


def available_reference() -> bool:
    return (REF_DIR / "fwdTimeCpmlFor2dAw_mex.so").exists()


def load_shim_library(path) -> ctypes.CDLL:
    """Load a gateway library linked with the shim and declare the harness."""
    lib = ctypes.CDLL(str(path), mode=ctypes.RTLD_LOCAL)
    vp = ctypes.c_void_p
    lib.shim_array_new.restype = vp
    lib.shim_array_new.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
    lib.shim_array_borrow.restype = vp
    lib.shim_array_borrow.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), _dp]
    lib.shim_array_free.argtypes = [vp]
    lib.shim_array_data.restype = _dp
    lib.shim_array_data.argtypes = [vp]
    lib.shim_array_ndim.restype = ctypes.c_int
    lib.shim_array_ndim.argtypes = [vp]
    lib.shim_array_dim.restype = ctypes.c_longlong
    lib.shim_array_dim.argtypes = [vp, ctypes.c_int]
    lib.shim_last_error.restype = ctypes.c_char_p
    lib.shim_call.restype = ctypes.c_int
    lib.shim_call.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(vp)]
    return lib


class MexError(RuntimeError):
    pass


def shim_call(lib, nlhs: int, *args):
    """Call ``mexFunction`` of ``lib`` with numpy arguments (scalars become 1x1).
    Returns a tuple of nlhs Fortran-ordered arrays; raises MexError with the
    gateway's message when it calls mexErrMsgTxt."""
    keep = []
    prhs = (ctypes.c_void_p * max(len(args), 1))()
    for k, a in enumerate(args):
        arr = _f64(np.atleast_1d(a) if np.ndim(a) == 0 else a)
        keep.append(arr)
        dims = (ctypes.c_longlong * max(arr.ndim, 2))(*(list(arr.shape) + [1] * (2 - arr.ndim)))
        prhs[k] = lib.shim_array_borrow(max(arr.ndim, 2), dims, _ptr(arr))
    plhs = (ctypes.c_void_p * max(nlhs, 2))()
    try:
        rc = lib.shim_call(nlhs, plhs, len(args), prhs)
        if rc:
            raise MexError(lib.shim_last_error().decode())
        outs = []
        for k in range(max(nlhs, 1)):
            a = plhs[k]
            if not a:
                outs.append(None)
                continue
            nd = lib.shim_array_ndim(a)
            shape = tuple(lib.shim_array_dim(a, i) for i in range(nd))
            n = int(np.prod(shape))
            out = np.empty(shape, order="F")
            if n:
                ctypes.memmove(out.ctypes.data, lib.shim_array_data(a), n * 8)
            outs.append(out)
        return tuple(outs)
    finally:
        for k in range(len(args)):
            lib.shim_array_free(prhs[k])
        for k in range(max(nlhs, 2)):
            if plhs[k]:
                lib.shim_array_free(plhs[k])


# --------------------------------------------------------------------------
# numpy restatement (MATLAB twins)
# --------------------------------------------------------------------------
def dcoef(order: int) -> np.ndarray:
    """dCoef(order, 's') by LU with partial pivoting (src/dCoef.m:35-48)."""
    n = order
    A = np.array([[float((2 * j + 1) ** (2 * i + 1)) for j in range(n)] for i in range(n)])
    x = np.zeros(n)
    x[0] = 1.0
    piv = list(range(n))
    for k in range(n):
        p = k + int(np.argmax(np.abs(A[k:, k])))
        piv[k] = p
        if p != k:
            A[[k, p], :] = A[[p, k], :]
        if A[k, k] != 0.0:
            r = 1.0 / A[k, k]
            A[k + 1:, k] *= r
        for j in range(k + 1, n):
            t = -A[k, j]
            A[k + 1:, j] += A[k + 1:, k] * t
    for k in range(n):
        if piv[k] != k:
            x[k], x[piv[k]] = x[piv[k]], x[k]
    for k in range(n):
        if x[k] != 0.0:
            x[k + 1:] -= x[k] * A[k + 1:, k]
    for k in range(n - 1, -1, -1):
        if x[k] != 0.0:
            x[k] /= A[k, k]
            x[:k] -= x[k] * A[:k, k]
    return x


def damp_pml_c(u, v, L):
    """finiteDifference.c:253-280 operation order."""
    d0 = -(3.0 * v) / (2 * L) * _LOGR
    return d0 * (u / L) * (u / L)


def damp_pml_m(u, v, L):
    """src/dampPml.m:16-18 operation order."""
    d0 = -(3 * v) / (2 * L) * _LOGR
    q = u / L
    return d0 * (q * q)


def ext_boundary(V, nB: int, dim: int = 2) -> np.ndarray:
    """Pad left/right (and front/rear in 3D) by edge replication and the bottom
    by repeating the last row; no top padding (src/extBoundary.m:22-39)."""
    V = np.asarray(V, dtype=np.float64)
    if dim == 2:
        W = np.concatenate([np.repeat(V[:, :1], nB, 1), V, np.repeat(V[:, -1:], nB, 1)], axis=1)
        return np.concatenate([W, np.repeat(W[-1:, :], nB, 0)], axis=0)
    W = np.concatenate([np.repeat(V[:, :1, :], nB, 1), V, np.repeat(V[:, -1:, :], nB, 1)], axis=1)
    W = np.concatenate([np.repeat(W[:, :, :1], nB, 2), W, np.repeat(W[:, :, -1:], nB, 2)], axis=2)
    return np.concatenate([W, np.repeat(W[-1:, :, :], nB, 0)], axis=0)


def ricker(f: float, n: int, dt: float, t0: float | None = None) -> np.ndarray:
    """Causal Ricker wavelet peaking at t0 = 1/f (src/ricker.m:61-71)."""
    t0 = 1.0 / f if t0 is None else t0
    t = np.arange(n) * dt
    tau = t - t0
    return (1 - 2 * tau * tau * f ** 2 * np.pi ** 2) * np.exp(-(tau ** 2) * np.pi ** 2 * f ** 2)


def _diff(data: np.ndarray, c: np.ndarray, d: float, axis: int) -> np.ndarray:
    """diffOperator.m: out = sum_ii c(ii)*(data(idx1)-data(idx2))/d, shrinking
    ``axis`` by 2N-1 (src/fd_matlab/diffOperator.m:29-66)."""
    order = len(c)
    k = 2 * order - 1
    n = data.shape[axis]
    m = n - k
    out = np.zeros(data.shape[:axis] + (m,) + data.shape[axis + 1:])
    base = np.arange(order, order + m)
    for ii in range(order):
        a = np.take(data, base + ii, axis=axis)
        b = np.take(data, base - ii - 1, axis=axis)
        out = out + c[ii] * (a - b) / d
    return out


def fwd2d_np(v, source, N, nB, dz, dx, dt):
    """fwdTimeCpmlFor2dAw with the C gateway's damping order; returns (data, snapshot)."""
    return _run2d(v, source, None, N, nB, dz, dx, dt)


def rvs2d_np(v, data, N, nB, dz, dx, dt):
    """rvsTimeCpmlFor2dAw; returns (model, snapshot)."""
    return _run2d(v, None, data, N, nB, dz, dx, dt)


def _run2d(v, source, rdata, N, nB, dz, dx, dt):
    v = np.asarray(v, dtype=np.float64)
    nz, nx = v.shape
    nt = source.shape[2] if source is not None else rdata.shape[1]
    c = dcoef(N)
    k = 2 * N - 1
    xd = np.zeros((nz, nx))
    zd = np.zeros((nz, nx))
    if nB:
        xd[:, :nB] = damp_pml_c(np.tile(np.arange(nB, 0, -1) * dx, (nz, 1)), v[:, :nB], nB * dx)
        xd[:, nx - nB:] = damp_pml_c(np.tile(np.arange(1, nB + 1) * dx, (nz, 1)), v[:, nx - nB:], nB * dx)
        zd[nz - nB:, :] = damp_pml_c(np.tile((np.arange(1, nB + 1) * dz)[:, None], (1, nx)), v[nz - nB:, :],
                                     nB * dz)
    xb = _exp(-xd * dt)
    zb = _exp(-zd * dt)
    fdm = np.zeros((3, nz + 2 * k, nx + 2 * k))
    zPhi = np.zeros((nz + 2 * k, nx))
    xPhi = np.zeros((nz, nx + 2 * k))
    zA = np.zeros((nz + 2 * k, nx))
    xA = np.zeros((nz, nx + 2 * k))
    zPsi = np.zeros((nz + k, nx))
    xPsi = np.zeros((nz, nx + k))
    zP = np.zeros((nz + k, nx))
    xP = np.zeros((nz, nx + k))
    vdtSq = (v * dt) * (v * dt)
    izi = slice(k, nz + k)
    ixi = slice(k, nx + k)
    izl = np.arange(N - 1, nz + 2 * k - N)
    ixl = np.arange(N - 1, nx + 2 * k - N)
    data = np.zeros((nx, nt))
    snapshot = np.zeros((nz, nx, nt))
    steps = range(nt) if source is not None else range(nt - 1, -1, -1)
    for it in steps:
        if source is not None:
            src = source[:, :, it]
        else:
            src = np.zeros((nz, nx))
            src[0, :] = rdata[:, it]
        cur = fdm[1]
        zPhi[izi, :] = zb * zPhi[izi, :] + (zb - 1) * _diff(cur[izl + 1][:, ixi], c, dz, 0)
        xPhi[:, ixi] = xb * xPhi[:, ixi] + (xb - 1) * _diff(cur[izi][:, ixl + 1], c, dx, 1)
        zA[izl, :] = _diff(cur[:, ixi], c, dz, 0) + zPhi[izl, :]
        xA[:, ixl] = _diff(cur[izi, :], c, dx, 1) + xPhi[:, ixl]
        dzA = _diff(zA[izl, :], c, dz, 0)
        dxA = _diff(xA[:, ixl], c, dx, 1)
        zPsi[izi, :] = zb * zPsi[izi, :] + (zb - 1) * dzA
        xPsi[:, ixi] = xb * xPsi[:, ixi] + (xb - 1) * dxA
        zP[izi, :] = dzA + zPsi[izi, :]
        xP[:, ixi] = dxA + xPsi[:, ixi]
        fdm[2][izi, ixi] = vdtSq * (zP[izi, :] + xP[:, ixi] + src) + 2 * fdm[1][izi, ixi] - fdm[0][izi, ixi]
        fdm[0] = fdm[1].copy()
        fdm[1] = fdm[2].copy()
        data[:, it] = fdm[1][k, ixi]
        snapshot[:, :, it] = fdm[1][izi, ixi]
    if source is not None:
        return data, snapshot
    return fdm[0].copy(), snapshot


def reference_diff(gateway: "RefMex"):
    """A derivative function with _diff's signature that calls the reference's
    own diffOperator_mex (compiled on the shim): the routine the MATLAB path
    resolves diffOperator to (src/fd_cmex/diffOperator.m shadows
    src/fd_matlab/diffOperator.m), so the 3D MATLAB file's derivatives come from
    the reference's C."""
    def diff(data, c, d, axis):
        data = np.asfortranarray(data)
        return gateway.call(1, data, np.asarray(c, dtype=np.float64), float(d), axis + 1)[0].reshape(
            data.shape[:axis] + (data.shape[axis] - (2 * len(c) - 1),) + data.shape[axis + 1:], order="F")
    return diff


def fwd3d_np(v, source, N, nB, dz, dx, dy, dt, diff=None):
    """fwdTimeCpmlFor3dAw.m restated (src/fwdTimeCpmlFor3dAw.m:37-147).  ``diff``
    replaces the derivative routine (default: the restatement _diff; with
    reference_diff, the reference's compiled diffOperator_mex)."""
    _diff = diff or globals()["_diff"]
    v = np.asarray(v, dtype=np.float64)
    nz, nx, ny = v.shape
    nt = source.shape[3]
    c = dcoef(N)
    k = 2 * N - 1
    xd = np.zeros((nz, nx, ny))
    yd = np.zeros((nz, nx, ny))
    zd = np.zeros((nz, nx, ny))
    if nB:
        L = float(nB)
        xl = damp_pml_m(np.tile(np.arange(nB, 0, -1, dtype=float), (nz, 1)), v[:, :nB, 0], L)
        xr = damp_pml_m(np.tile(np.arange(1, nB + 1, dtype=float), (nz, 1)), v[:, nx - nB:, 0], L)
        xd[:, :nB, :] = xl[:, :, None]
        xd[:, nx - nB:, :] = xr[:, :, None]
        yf = damp_pml_m(np.tile(np.arange(nB, 0, -1, dtype=float), (nx, 1)), v[0, :, :nB], L)
        yr = damp_pml_m(np.tile(np.arange(1, nB + 1, dtype=float), (nx, 1)), v[0, :, ny - nB:], L)
        yd[:, :, :nB] = yf[None, :, :]
        yd[:, :, ny - nB:] = yr[None, :, :]
        zdn = damp_pml_m(np.tile(np.arange(1, nB + 1, dtype=float)[:, None], (1, nx)), v[nz - nB:, :, 0], L)
        zd[nz - nB:, :, :] = zdn[:, :, None]
    xb = _exp(-xd * dt)
    yb = _exp(-yd * dt)
    zb = _exp(-zd * dt)
    fdm = np.zeros((3, nz + 2 * k, nx + 2 * k, ny + 2 * k))
    zPhi = np.zeros((nz + 2 * k, nx, ny))
    xPhi = np.zeros((nz, nx + 2 * k, ny))
    yPhi = np.zeros((nz, nx, ny + 2 * k))
    zA = np.zeros((nz + 2 * k, nx, ny))
    xA = np.zeros((nz, nx + 2 * k, ny))
    yA = np.zeros((nz, nx, ny + 2 * k))
    zPsi = np.zeros((nz + k, nx, ny))
    xPsi = np.zeros((nz, nx + k, ny))
    yPsi = np.zeros((nz, nx, ny + k))
    zP = np.zeros((nz + k, nx, ny))
    xP = np.zeros((nz, nx + k, ny))
    yP = np.zeros((nz, nx, ny + k))
    vdtSq = (v * dt) * (v * dt)
    izi, ixi, iyi = slice(k, nz + k), slice(k, nx + k), slice(k, ny + k)
    izl = np.arange(N - 1, nz + 2 * k - N)
    ixl = np.arange(N - 1, nx + 2 * k - N)
    iyl = np.arange(N - 1, ny + 2 * k - N)
    data = np.zeros((nx, ny, nt))
    snapshot = np.zeros((nz, nx, ny, nt))
    for it in range(nt):
        cur = fdm[1]
        zPhi[izi] = zb * zPhi[izi] + (zb - 1) * _diff(cur[izl + 1][:, ixi][:, :, iyi], c, dz, 0)
        xPhi[:, ixi] = xb * xPhi[:, ixi] + (xb - 1) * _diff(cur[izi][:, ixl + 1][:, :, iyi], c, dx, 1)
        yPhi[:, :, iyi] = yb * yPhi[:, :, iyi] + (yb - 1) * _diff(cur[izi][:, ixi][:, :, iyl + 1], c, dy, 2)
        zA[izl] = _diff(cur[:, ixi, iyi], c, dz, 0) + zPhi[izl]
        xA[:, ixl] = _diff(cur[izi][:, :, iyi], c, dx, 1) + xPhi[:, ixl]
        yA[:, :, iyl] = _diff(cur[izi, ixi, :], c, dy, 2) + yPhi[:, :, iyl]
        dzA = _diff(zA[izl], c, dz, 0)
        dxA = _diff(xA[:, ixl], c, dx, 1)
        dyA = _diff(yA[:, :, iyl], c, dy, 2)
        zPsi[izi] = zb * zPsi[izi] + (zb - 1) * dzA
        xPsi[:, ixi] = xb * xPsi[:, ixi] + (xb - 1) * dxA
        yPsi[:, :, iyi] = yb * yPsi[:, :, iyi] + (yb - 1) * dyA
        zP[izi] = dzA + zPsi[izi]
        xP[:, ixi] = dxA + xPsi[:, ixi]
        yP[:, :, iyi] = dyA + yPsi[:, :, iyi]
        fdm[2][izi, ixi, iyi] = vdtSq * (zP[izi] + xP[:, ixi] + yP[:, :, iyi] + source[:, :, :, it]) \
            + 2 * fdm[1][izi, ixi, iyi] - fdm[0][izi, ixi, iyi]
        fdm[0] = fdm[1].copy()
        fdm[1] = fdm[2].copy()
        data[:, :, it] = fdm[1][k, ixi, iyi]
        snapshot[:, :, :, it] = fdm[1][izi, ixi, iyi]
    return data, snapshot


def image_np(fwd_snap, rvs_snap, epsilon):
    """M = sum_t f.*r, s2 = epsilon + sum_t f.^2 in ascending t; returns M./s2."""
    m = np.zeros(fwd_snap.shape[:2])
    s2 = np.full(fwd_snap.shape[:2], float(epsilon))
    for t in range(fwd_snap.shape[2]):
        m = fwd_snap[:, :, t] * rvs_snap[:, :, t] + m
        s2 = fwd_snap[:, :, t] ** 2 + s2
    return m / s2


# ---------------------------------------------------------------- elastic SPML
def fwd_elastic2d_np(vp, vs, source, N, nB, dz, dx, dt, diff=None):
    """src/fwdTimeSpmlFor2dEw.m:38-103 restated statement by statement (three
    time levels per field, as the file keeps them).  ``diff`` replaces the
    derivative routine (default: the restatement _diff; with reference_diff,
    the reference's compiled diffOperator_mex, which the file's diffOperator
    calls resolve to).  Returns (snapshotVzp, snapshotVxp, snapshotVzs,
    snapshotVxs), each nz x nx x nt."""
    D = diff or _diff
    vp = np.asarray(vp, dtype=np.float64)
    vs = np.asarray(vs, dtype=np.float64)
    source = np.asarray(source, dtype=np.float64)
    nz, nx, nt = source.shape
    c = dcoef(N)
    iz = slice(N, nz + N)
    ix = slice(N, nx + N)
    xDamp = np.zeros((nz, nx))
    zDamp = np.zeros((nz, nx))
    if nB:
        L = float(nB)
        ixb = np.arange(1, nB + 1, dtype=float)
        xDamp[:, :nB] = damp_pml_m(np.tile(ixb[::-1], (nz, 1)), vp[:, :nB], L)
        xDamp[:, nx - nB:] = damp_pml_m(np.tile(ixb, (nz, 1)), vp[:, nx - nB:], L)
        zDamp[nz - nB:, :] = damp_pml_m(np.tile(ixb[:, None], (1, nx)), vp[nz - nB:, :], L)
    shape = (3, nz + 2 * N, nx + 2 * N)
    A_z, A_x, A, B_z, B_x, B = (np.zeros(shape) for _ in range(6))
    Vxp, Vxs, Vx, Vzp, Vzs, Vz = (np.zeros(shape) for _ in range(6))
    vpSq = np.pad(vp * vp, N, mode="edge")
    vsSq = np.pad(vs * vs, N, mode="edge")
    out = [np.zeros((nz, nx, nt)) for _ in range(4)]
    zi = np.arange(N, nz + N)[:, None]
    xi = np.arange(N, nx + N)[None, :]
    for it in range(nt):
        A_x[1][iz, ix] = (1 - 0.5 * xDamp * dt) / (1 + 0.5 * xDamp * dt) * A_x[0][iz, ix] \
            + dt / (1 + 0.5 * xDamp * dt) * D(Vx[1][iz, :-1], c, dx, 1)
        A_z[1][iz, ix] = (1 - 0.5 * zDamp * dt) / (1 + 0.5 * zDamp * dt) * A_z[0][iz, ix] \
            + dt / (1 + 0.5 * zDamp * dt) * D(Vz[1][:-1, ix], c, dz, 0)
        A[1][iz, ix] = A_x[1][iz, ix] + A_z[1][iz, ix]
        B_z[1][iz, ix] = (1 - 0.5 * zDamp * dt) / (1 + 0.5 * zDamp * dt) * B_z[0][iz, ix] \
            + dt / (1 + 0.5 * zDamp * dt) * D(Vx[1][1:, ix], c, dz, 0)
        B_x[1][iz, ix] = (1 - 0.5 * xDamp * dt) / (1 + 0.5 * xDamp * dt) * B_x[0][iz, ix] \
            - dt / (1 + 0.5 * xDamp * dt) * D(Vz[1][iz, 1:], c, dx, 1)
        B[1][iz, ix] = B_z[1][iz, ix] + B_x[1][iz, ix]
        Vzp[2][iz, ix] = (1 - 0.5 * zDamp * dt) / (1 + 0.5 * zDamp * dt) * Vzp[1][iz, ix] \
            + 0.25 * (vpSq[zi, xi] + vpSq[zi + 1, xi] + vpSq[zi + 1, xi - 1] + vpSq[zi, xi - 1]) * dt \
            / (1 + 0.5 * zDamp * dt) * D(A[1][1:, ix], c, dz, 0) \
            + dt / (1 + 0.5 * zDamp * dt) * source[:, :, it]
        Vxp[2][iz, ix] = (1 - 0.5 * xDamp * dt) / (1 + 0.5 * xDamp * dt) * Vxp[1][iz, ix] \
            + vpSq[iz, ix] * dt / (1 + 0.5 * xDamp * dt) * D(A[1][iz, 1:], c, dx, 1) \
            + dt / (1 + 0.5 * xDamp * dt) * source[:, :, it]
        Vzs[2][iz, ix] = (1 - 0.5 * xDamp * dt) / (1 + 0.5 * xDamp * dt) * Vzs[1][iz, ix] \
            - vsSq[iz, ix] * dt / (1 + 0.5 * xDamp * dt) * D(B[1][iz, :-1], c, dx, 1)
        Vxs[2][iz, ix] = (1 - 0.5 * zDamp * dt) / (1 + 0.5 * zDamp * dt) * Vxs[1][iz, ix] \
            + 0.25 * (vsSq[zi, xi] + vsSq[zi, xi + 1] + vsSq[zi - 1, xi + 1] + vsSq[zi - 1, xi]) * dt \
            / (1 + 0.5 * zDamp * dt) * D(B[1][:-1, ix], c, dz, 0)
        Vx[2][iz, ix] = Vxp[2][iz, ix] + Vxs[2][iz, ix]
        Vz[2][iz, ix] = Vzp[2][iz, ix] + Vzs[2][iz, ix]
        for f in (A_z, A_x, A, B_z, B_x, B, Vxp, Vzp, Vxs, Vzs, Vx, Vz):
            f[0] = f[1].copy()
            f[1] = f[2].copy()
        out[1][:, :, it] = Vxp[1][iz, ix]
        out[0][:, :, it] = Vzp[1][iz, ix]
        out[3][:, :, it] = Vxs[1][iz, ix]
        out[2][:, :, it] = Vzs[1][iz, ix]
    return tuple(out)


def fwd_elastic3d_np(vp, vs, source_x, source_y, source_z, N, nB, dz, dx, dy, dt, diff=None):
    """src/fwdTimeSpmlFor3dEw.m:40-236 restated statement by statement (three
    time levels per field).  Damping as the file takes it: x and z profiles from
    the y = 1 slice of vp, y profiles from its top row, each replicated along
    the missing axis.  ``diff`` as in fwd_elastic2d_np.  Returns the six
    snapshots (Vzp, Vxp, Vyp, Vzs, Vxs, Vys), each nz x nx x ny x nt."""
    D = diff or _diff
    vp = np.asarray(vp, dtype=np.float64)
    vs = np.asarray(vs, dtype=np.float64)
    sx_, sy_, sz_ = (np.asarray(a, dtype=np.float64) for a in (source_x, source_y, source_z))
    nz, nx, ny, nt = sx_.shape
    c = dcoef(N)
    xDamp = np.zeros((nz, nx, ny))
    yDamp = np.zeros((nz, nx, ny))
    zDamp = np.zeros((nz, nx, ny))
    if nB:
        L = float(nB)
        b = np.arange(1, nB + 1, dtype=float)
        xDamp[:, :nB, :] = damp_pml_m(np.tile(b[::-1], (nz, 1)), vp[:, :nB, 0], L)[:, :, None]
        xDamp[:, nx - nB:, :] = damp_pml_m(np.tile(b, (nz, 1)), vp[:, nx - nB:, 0], L)[:, :, None]
        yDamp[:, :, :nB] = damp_pml_m(np.tile(b[::-1][None, :], (nx, 1)), vp[0, :, :nB], L)[None, :, :]
        yDamp[:, :, ny - nB:] = damp_pml_m(np.tile(b[None, :], (nx, 1)), vp[0, :, ny - nB:], L)[None, :, :]
        zDamp[nz - nB:, :, :] = damp_pml_m(np.tile(b[:, None], (1, nx)), vp[nz - nB:, :, 0], L)[:, :, None]
    shape = (3, nz + 2 * N, nx + 2 * N, ny + 2 * N)
    names = ("A_x", "A_y", "A_z", "A", "B1_y", "B1_z", "B1", "B2_z", "B2_x", "B2", "B3_x", "B3_y", "B3",
             "Vxp", "Vxs_y", "Vxs_z", "Vxs", "Vx", "Vyp", "Vys_x", "Vys_z", "Vys", "Vy",
             "Vzp", "Vzs_x", "Vzs_y", "Vzs", "Vz")
    F = {k: np.zeros(shape) for k in names}
    vpSq = np.pad(vp * vp, N, mode="edge")
    vsSq = np.pad(vs * vs, N, mode="edge")
    I = (slice(N, nz + N), slice(N, nx + N), slice(N, ny + N))

    def sh(a, oz, ox, oy):  # a(iz + oz, ix + ox, iy + oy)
        return a[N + oz:nz + N + oz, N + ox:nx + N + ox, N + oy:ny + N + oy]

    def r_(d):
        return (1 - 0.5 * d * dt) / (1 + 0.5 * d * dt)

    def s_(d):
        return dt / (1 + 0.5 * d * dt)

    def cur(k):
        return F[k][1]

    out = [np.zeros((nz, nx, ny, nt)) for _ in range(6)]
    for it in range(nt):
        Vx, Vy, Vz = cur("Vx"), cur("Vy"), cur("Vz")
        F["A_x"][1][I] = r_(xDamp) * F["A_x"][0][I] + s_(xDamp) * D(Vx[N:nz + N, :-1, N:ny + N], c, dx, 1)
        F["A_y"][1][I] = r_(yDamp) * F["A_y"][0][I] + s_(yDamp) * D(Vy[N:nz + N, N:nx + N, :-1], c, dy, 2)
        F["A_z"][1][I] = r_(zDamp) * F["A_z"][0][I] + s_(zDamp) * D(Vz[:-1, N:nx + N, N:ny + N], c, dz, 0)
        F["A"][1][I] = F["A_x"][1][I] + F["A_y"][1][I] + F["A_z"][1][I]
        F["B1_y"][1][I] = r_(yDamp) * F["B1_y"][0][I] + s_(yDamp) * D(Vz[N:nz + N, N:nx + N, 1:], c, dy, 2)
        F["B1_z"][1][I] = r_(zDamp) * F["B1_z"][0][I] - s_(zDamp) * D(Vy[1:, N:nx + N, N:ny + N], c, dz, 0)
        F["B1"][1][I] = F["B1_y"][1][I] + F["B1_z"][1][I]
        F["B2_z"][1][I] = r_(zDamp) * F["B2_z"][0][I] + s_(zDamp) * D(Vx[1:, N:nx + N, N:ny + N], c, dz, 0)
        F["B2_x"][1][I] = r_(xDamp) * F["B2_x"][0][I] - s_(xDamp) * D(Vz[N:nz + N, 1:, N:ny + N], c, dx, 1)
        F["B2"][1][I] = F["B2_z"][1][I] + F["B2_x"][1][I]
        F["B3_x"][1][I] = r_(xDamp) * F["B3_x"][0][I] + s_(xDamp) * D(Vy[N:nz + N, 1:, N:ny + N], c, dx, 1)
        F["B3_y"][1][I] = r_(yDamp) * F["B3_y"][0][I] - s_(yDamp) * D(Vx[N:nz + N, N:nx + N, 1:], c, dy, 2)
        F["B3"][1][I] = F["B3_x"][1][I] + F["B3_y"][1][I]
        A, B1, B2, B3 = cur("A"), cur("B1"), cur("B2"), cur("B3")
        avg_zy = lambda q: sh(q, 0, 0, 0) + sh(q, -1, 0, 0) + sh(q, -1, 0, -1) + sh(q, 0, 0, -1)  # noqa: E731
        avg_zx = lambda q: sh(q, 0, 0, 0) + sh(q, 0, -1, 0) + sh(q, -1, -1, 0) + sh(q, -1, 0, 0)  # noqa: E731
        avg_xy = lambda q: sh(q, 0, 0, 0) + sh(q, 0, -1, 0) + sh(q, 0, -1, -1) + sh(q, 0, 0, -1)  # noqa: E731
        F["Vxp"][2][I] = r_(xDamp) * F["Vxp"][1][I] + 0.25 * avg_zy(vpSq) * dt / (1 + 0.5 * xDamp * dt) \
            * D(A[N:nz + N, 1:, N:ny + N], c, dx, 1) + s_(xDamp) * sx_[:, :, :, it]
        F["Vyp"][2][I] = r_(yDamp) * F["Vyp"][1][I] + 0.25 * avg_zx(vpSq) * dt / (1 + 0.5 * yDamp * dt) \
            * D(A[N:nz + N, N:nx + N, 1:], c, dy, 2) + s_(yDamp) * sy_[:, :, :, it]
        F["Vzp"][2][I] = r_(zDamp) * F["Vzp"][1][I] + 0.25 * avg_xy(vpSq) * dt / (1 + 0.5 * zDamp * dt) \
            * D(A[1:, N:nx + N, N:ny + N], c, dz, 0) + s_(zDamp) * sz_[:, :, :, it]
        F["Vxs_y"][2][I] = r_(yDamp) * F["Vxs_y"][1][I] - 0.25 * avg_zy(vsSq) * dt / (1 + 0.5 * yDamp * dt) \
            * D(B3[N:nz + N, N:nx + N, :-1], c, dy, 2)
        F["Vxs_z"][2][I] = r_(zDamp) * F["Vxs_z"][1][I] + 0.25 * avg_zy(vsSq) * dt / (1 + 0.5 * zDamp * dt) \
            * D(B2[:-1, N:nx + N, N:ny + N], c, dz, 0)
        F["Vxs"][2][I] = F["Vxs_y"][2][I] + F["Vxs_z"][2][I]
        F["Vys_x"][2][I] = r_(xDamp) * F["Vys_x"][1][I] + 0.25 * avg_zx(vsSq) * dt / (1 + 0.5 * xDamp * dt) \
            * D(B3[N:nz + N, :-1, N:ny + N], c, dx, 1)
        F["Vys_z"][2][I] = r_(zDamp) * F["Vys_z"][1][I] - 0.25 * avg_zx(vsSq) * dt / (1 + 0.5 * zDamp * dt) \
            * D(B1[:-1, N:nx + N, N:ny + N], c, dz, 0)
        F["Vys"][2][I] = F["Vys_x"][2][I] + F["Vys_z"][2][I]
        F["Vzs_x"][2][I] = r_(xDamp) * F["Vzs_x"][1][I] - 0.25 * avg_xy(vsSq) * dt / (1 + 0.5 * xDamp * dt) \
            * D(B2[N:nz + N, :-1, N:ny + N], c, dx, 1)
        F["Vzs_y"][2][I] = r_(yDamp) * F["Vzs_y"][1][I] + 0.25 * avg_xy(vsSq) * dt / (1 + 0.5 * yDamp * dt) \
            * D(B1[N:nz + N, N:nx + N, :-1], c, dy, 2)
        F["Vzs"][2][I] = F["Vzs_x"][2][I] + F["Vzs_y"][2][I]
        F["Vx"][2][I] = F["Vxp"][2][I] + F["Vxs"][2][I]
        F["Vy"][2][I] = F["Vyp"][2][I] + F["Vys"][2][I]
        F["Vz"][2][I] = F["Vzp"][2][I] + F["Vzs"][2][I]
        for k in names:
            F[k][0] = F[k][1].copy()
            F[k][1] = F[k][2].copy()
        for o, k in zip(out, ("Vzp", "Vxp", "Vyp", "Vzs", "Vxs", "Vys")):
            o[:, :, :, it] = F[k][1][I]
    return tuple(out)


# ---------------------------------------------------------------- sponge ABC
# Restatement of src/fwdTimeSpongeFor2dAw.m:36-101 and
# src/rvsTimeSpongeFor2dAw.m:36-103 (MATLAB only in the reference: parity of
# this part is unpinned -- no compiled reference exists to check it against).
SPONGE_ALPHA = 0.015  # src/fwdTimeSpongeFor2dAw.m:45


def sponge_profile(nB: int) -> np.ndarray:
    """boundary = (exp(-((alpha*(nB-iz)).^2))).^10 for iz = 0..nB-1
    (src/fwdTimeSpongeFor2dAw.m:43-47), with glibc's exp and pow."""
    out = np.zeros(nB)
    for iz in range(nB):
        a = SPONGE_ALPHA * float(nB - iz)
        out[iz] = math.pow(math.exp(-(a * a)), 10.0)
    return out


def _sponge_run(v, src_slice, nt, nB, dz, dx, dt, reverse=False):
    """The time loop of the two sponge propagators.  src_slice(it) returns the
    nz x nx source of step it (or None); returns (data nx x nt, snapshot
    nz x nx x nt, final present nz x nx)."""
    v = np.asarray(v, dtype=np.float64)
    nz, nx = v.shape
    boundary = sponge_profile(nB)
    t = v * dt / dx
    ax = t * t
    t = v * dt / dz
    az = t * t
    t = v * dt
    vdtSq = t * t
    b = 2 - 2 * ax - 2 * az
    fdm = [np.zeros((nz + 2, nx + 2)) for _ in range(3)]
    data = np.zeros((nx, nt))
    snapshot = np.zeros((nz, nx, nt))
    izb = slice(1, nz - nB + 1)  # rows (1:nz-nB)+1 of the padded field, 0-based
    steps = range(nt - 1, -1, -1) if reverse else range(nt)
    for it in steps:
        P = fdm[1]
        new = b * P[1:-1, 1:-1] - fdm[0][1:-1, 1:-1] + ax * (P[1:-1, 2:] + P[1:-1, :-2]) \
            + az * (P[2:, 1:-1] + P[:-2, 1:-1])
        s = src_slice(it)
        if s is not None:
            new = new - vdtSq * s
        fdm[2][1:-1, 1:-1] = new
        fdm[0] = fdm[1].copy()
        fdm[1] = fdm[2].copy()
        for ixb in range(2, nB + 2):  # 1-based padded column ixb
            c = ixb - 1
            for f in (fdm[0], fdm[1]):
                f[izb, c] = boundary[ixb - 2] * f[izb, c]
            ixb2 = nx - nB + ixb
            c2 = ixb2 - 1
            for f in (fdm[0], fdm[1]):
                f[izb, c2] = boundary[nx - ixb2 + 1] * f[izb, c2]
            izb2 = nz - nB + ixb
            r2 = izb2 - 1
            for f in (fdm[0], fdm[1]):
                f[r2, :] = boundary[nz - izb2 + 1] * f[r2, :]
        data[:, it] = fdm[1][1, 1:-1]
        snapshot[:, :, it] = fdm[1][1:-1, 1:-1]
    return data, snapshot, fdm[1][1:-1, 1:-1].copy()


def fwd_sponge_np(v, source, nB, dz, dx, dt):
    """[data, snapshot] = fwdTimeSpongeFor2dAw(v, source, nBoundary, dz, dx, dt)."""
    source = np.asarray(source, dtype=np.float64)
    data, snap, _ = _sponge_run(v, lambda it: source[:, :, it], source.shape[2], nB, dz, dx, dt)
    return data, snap


def fwd_sponge_point_np(v, nt, src_iz, src_ix, wavelets, nB, dz, dx, dt):
    """The same with point sources (sources on one cell add up, in order)."""
    v = np.asarray(v, dtype=np.float64)
    w = np.atleast_2d(np.asarray(wavelets, dtype=np.float64))
    iz, ix = np.atleast_1d(src_iz), np.atleast_1d(src_ix)

    def slice_at(it):
        s = np.zeros(v.shape)
        seen = set()
        for k in range(len(iz)):
            key = (int(iz[k]), int(ix[k]))
            s[key] = s[key] + w[k, it] if key in seen else w[k, it]
            seen.add(key)
        return s
    data, snap, _ = _sponge_run(v, slice_at, nt, nB, dz, dx, dt)
    return data, snap


def rvs_sponge_np(v, data, nB, dz, dx, dt):
    """[model, snapshot] = rvsTimeSpongeFor2dAw(v, data, nBoundary, dz, dx, dt);
    model is the field after the last step (the reference never assigns it)."""
    v = np.asarray(v, dtype=np.float64)
    data = np.asarray(data, dtype=np.float64)

    def slice_at(it):
        s = np.zeros(v.shape)
        s[0, :] = data[:, it]
        return s
    _, snap, model = _sponge_run(v, slice_at, data.shape[1], nB, dz, dx, dt, reverse=True)
    return model, snap


def rtm_sponge_np(v, vs, wavelet, src_iz, src_ix, nB, dz, dx, dt, epsilon):
    """One shot of mainRtmTimeSpongeFor2dAw.m:160-161,247-268,310: returns
    (M./s2, dataTrue, dataSmooth)."""
    w = np.asarray(wavelet, dtype=np.float64).ravel()
    nt = len(w)
    d_true, _ = fwd_sponge_point_np(v, nt, [src_iz], [src_ix], w[None, :], nB, dz, dx, dt)
    d_smooth, f_snap = fwd_sponge_point_np(vs, nt, [src_iz], [src_ix], w[None, :], nB, dz, dx, dt)
    _, r_snap = rvs_sponge_np(v, d_true - d_smooth, nB, dz, dx, dt)
    return image_np(f_snap, r_snap, epsilon), d_true, d_smooth


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = float(np.linalg.norm(b.ravel()))
    num = float(np.linalg.norm((a - b).ravel()))
    return num / den if den else num
