"""MATLAB-shaped entry points of the SSSI acoustic CPML core on the GPU.

The functions mirror the MATLAB wrappers the application scripts call
(``src/fd_cmex/fwdTimeCpmlFor2dAw.m:37``, ``src/fd_cmex/rvsTimeCpmlFor2dAw.m:31``,
``src/fwdTimeCpmlFor3dAw.m:1``): same names, same positional arguments, same
array shapes, MATLAB (column-major) index order ``v[z, x]``,
``source[z, x, t]``, ``data[x, t]``, ``snapshot[z, x, t]``.  Inputs may be
numpy arrays (host) or CUDA torch tensors (device; they must be Fortran
ordered, i.e. ``t.T.contiguous().T`` / created via ``permute``); outputs come
back as the same kind.

``mode`` selects the arithmetic (``"fp64"``, the default as in the MEX
gateways: folded coefficients and fused multiply-adds, within 1e-12 relative
L2 of the reference; ``"fp64-strict"``: the reference's rounding sequence,
bit-identical to the reference C; ``"fp32"``: FP32 wavefield with
compensated FP32 CPML memory variables).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import check, lib

MODES = {"fp64-strict": 0, "fp64": 1, "fp32": 2}


def _mode(mode) -> int:
    if isinstance(mode, int):
        return mode
    try:
        return MODES[mode]
    except KeyError:
        raise ValueError(f"unknown mode {mode!r}; expected one of {sorted(MODES)}") from None


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _in(a, name: str):
    """(address, keepalive, shape) of an input array as column-major float64."""
    if a is None:
        return None, None, None
    if _is_torch(a):
        import torch

        if a.dtype != torch.float64:
            raise TypeError(f"{name}: expected a float64 tensor")
        if a.dim() >= 2 and not a.is_contiguous() and not a.T.is_contiguous():
            raise ValueError(f"{name}: tensor must be column-major (Fortran ordered)")
        if a.dim() >= 2 and a.is_contiguous() and not a.T.is_contiguous():
            raise ValueError(f"{name}: tensor must be column-major (Fortran ordered)")
        return a.data_ptr(), a, tuple(a.shape)
    arr = np.asfortranarray(np.asarray(a, dtype=np.float64))
    return arr.ctypes.data, arr, arr.shape


def _out_like(ref, shape):
    """A zeroed column-major float64 output on the same side (host/device) as ``ref``."""
    if ref is not None and _is_torch(ref):
        import torch

        t = torch.zeros(tuple(reversed(shape)), dtype=torch.float64, device=ref.device)
        return t.permute(*reversed(range(len(shape)))), t
    arr = np.zeros(shape, order="F")
    return arr, arr


def _addr(a):
    if a is None:
        return None
    if _is_torch(a):
        return a.data_ptr()
    return a.ctypes.data


def dCoef(order: int) -> np.ndarray:
    """Staggered-grid coefficients c_1..c_N (src/dCoef.m, finiteDifference.c:24-82)."""
    c = np.zeros(order)
    check(lib().sssi_dCoef(int(order), c.ctypes.data))
    return c


def dampPml(u, v, L: float) -> np.ndarray:
    """d = -(3v)/(2L) ln(1e-6) (u/L)^2 elementwise (finiteDifference.c:253-280)."""
    u = np.asfortranarray(np.asarray(u, dtype=np.float64))
    v = np.asfortranarray(np.asarray(v, dtype=np.float64))
    if u.shape != v.shape:
        raise ValueError("u and v must have the same shape")
    d = np.zeros(u.shape, order="F")
    check(lib().sssi_dampPml(u.ctypes.data, v.ctypes.data, u.size, float(L), d.ctypes.data))
    return d


def diffOperator(data, c, d, dim=1, *, mode="fp64"):
    """diffData = diffOperator(data, c, d, dim) (src/fd_cmex/diffOperator.m): staggered
    first derivative of a 2D or 3D array along dimension ``dim`` (1-based), whose
    length shrinks by 2 numel(c) - 1."""
    pd, kd, shape = _in(data, "data")
    if len(shape) not in (2, 3):
        raise ValueError("data must be 2D or 3D")
    cc = np.ascontiguousarray(np.atleast_1d(np.asarray(c, dtype=np.float64)).ravel())
    order = len(cc)
    oshape = list(shape)
    oshape[int(dim) - 1] -= 2 * order - 1
    if oshape[int(dim) - 1] < 0:
        raise ValueError("the stencil is longer than the dimension")
    out, _ = _out_like(data, tuple(oshape))
    dims = np.asarray(shape, dtype=np.int64)
    check(lib().sssi_diffOperator(pd, len(shape), dims.ctypes.data, cc.ctypes.data, order, float(d), int(dim),
                                  _addr(out), _mode(mode)))
    return out


def fwdTimeCpmlFor2dAw(v, source, nDiffOrder, nBoundary, dz, dx, dt, *, mode="fp64", want_snapshot=True):
    """[data, snapshot] = fwdTimeCpmlFor2dAw(v, source, nDiffOrder, nBoundary, dz, dx, dt)."""
    pv, kv, vshape = _in(v, "v")
    ps, ks, sshape = _in(source, "source")
    if vshape is None or len(vshape) != 2:
        raise ValueError("v must be nz x nx")
    nz, nx = vshape
    if sshape is None or len(sshape) != 3 or sshape[:2] != (nz, nx):
        raise ValueError("source must be nz x nx x nt with the grid of v")
    nt = sshape[2]
    data, dkeep = _out_like(v, (nx, nt))
    snap, skeep = _out_like(v, (nz, nx, nt)) if want_snapshot else (None, None)
    check(lib().sssi_fwdTimeCpmlFor2dAw(pv, ps, nz, nx, nt, int(nDiffOrder), int(nBoundary), float(dz), float(dx),
                                        float(dt), _addr(data), _addr(snap), _mode(mode)))
    return data, snap


def fwdTimeCpmlFor2dAwPoint(v, nt, src_iz, src_ix, wavelets, nDiffOrder, nBoundary, dz, dx, dt, *,
                            mode="fp64", want_snapshot=False):
    """Forward modelling with point sources: source s at interior (src_iz[s], src_ix[s])
    with amplitude wavelets[s, t].  Returns (data, snapshot or None)."""
    pv, kv, vshape = _in(v, "v")
    nz, nx = vshape
    iz = np.ascontiguousarray(np.atleast_1d(src_iz), dtype=np.int64)
    ix = np.ascontiguousarray(np.atleast_1d(src_ix), dtype=np.int64)
    w = np.ascontiguousarray(np.atleast_2d(np.asarray(wavelets, dtype=np.float64)))
    if w.shape != (len(iz), nt) or len(ix) != len(iz):
        raise ValueError("wavelets must be nsrc x nt and src_iz/src_ix of length nsrc")
    data, _ = _out_like(v, (nx, nt))
    snap, _ = _out_like(v, (nz, nx, nt)) if want_snapshot else (None, None)
    check(lib().sssi_fwdTimeCpmlFor2dAwPoint(pv, nz, nx, int(nt), int(nDiffOrder), int(nBoundary), float(dz),
                                             float(dx), float(dt), len(iz), iz.ctypes.data, ix.ctypes.data,
                                             w.ctypes.data, _addr(data), _addr(snap), _mode(mode)))
    return data, snap


def rvsTimeCpmlFor2dAw(v, data, nDiffOrder, nBoundary, dz, dx, dt, *, mode="fp64", want_snapshot=True):
    """[model, snapshot] = rvsTimeCpmlFor2dAw(v, data, nDiffOrder, nBoundary, dz, dx, dt)."""
    pv, kv, vshape = _in(v, "v")
    pd, kd, dshape = _in(data, "data")
    if vshape is None or len(vshape) != 2:
        raise ValueError("v must be nz x nx")
    nz, nx = vshape
    if dshape is None or len(dshape) != 2 or dshape[0] != nx:
        raise ValueError("data must be nx x nt")
    nt = dshape[1]
    l = 2 * int(nDiffOrder) - 1
    model, _ = _out_like(v, (nz + 2 * l, nx + 2 * l))
    snap, _ = _out_like(v, (nz, nx, nt)) if want_snapshot else (None, None)
    check(lib().sssi_rvsTimeCpmlFor2dAw(pv, pd, nz, nx, nt, int(nDiffOrder), int(nBoundary), float(dz), float(dx),
                                        float(dt), _addr(model), _addr(snap), _mode(mode)))
    return model, snap


def fwdTimeCpmlFor3dAw(v, source, nDiffOrder, nBoundary, dz, dx, dy, dt, *, mode="fp64",
                       want_snapshot=True):
    """[data, snapshot] = fwdTimeCpmlFor3dAw(v, source, nDiffOrder, nBoundary, dz, dx, dy, dt)."""
    pv, kv, vshape = _in(v, "v")
    ps, ks, sshape = _in(source, "source")
    if vshape is None or len(vshape) != 3:
        raise ValueError("v must be nz x nx x ny")
    nz, nx, ny = vshape
    if sshape is None or len(sshape) != 4 or sshape[:3] != (nz, nx, ny):
        raise ValueError("source must be nz x nx x ny x nt with the grid of v")
    nt = sshape[3]
    data, _ = _out_like(v, (nx, ny, nt))
    snap, _ = _out_like(v, (nz, nx, ny, nt)) if want_snapshot else (None, None)
    check(lib().sssi_fwdTimeCpmlFor3dAw(pv, ps, nz, nx, ny, nt, int(nDiffOrder), int(nBoundary), float(dz), float(dx),
                                        float(dy), float(dt), _addr(data), _addr(snap), _mode(mode)))
    return data, snap


def fwdTimeCpmlFor3dAwPoint(v, nt, src_iz, src_ix, src_iy, wavelets, nDiffOrder, nBoundary, dz, dx, dy, dt, *,
                            mode="fp64", want_snapshot=False):
    """3D forward modelling with point sources: source s at interior
    (src_iz[s], src_ix[s], src_iy[s]) with amplitude wavelets[s, t].  Returns
    (data nx x ny x nt, snapshot or None)."""
    pv, kv, vshape = _in(v, "v")
    if vshape is None or len(vshape) != 3:
        raise ValueError("v must be nz x nx x ny")
    nz, nx, ny = vshape
    iz = np.ascontiguousarray(np.atleast_1d(src_iz), dtype=np.int64)
    ix = np.ascontiguousarray(np.atleast_1d(src_ix), dtype=np.int64)
    iy = np.ascontiguousarray(np.atleast_1d(src_iy), dtype=np.int64)
    w = np.ascontiguousarray(np.atleast_2d(np.asarray(wavelets, dtype=np.float64)))
    if w.shape != (len(iz), nt) or len(ix) != len(iz) or len(iy) != len(iz):
        raise ValueError("wavelets must be nsrc x nt and src_iz/src_ix/src_iy of length nsrc")
    data, _ = _out_like(v, (nx, ny, nt))
    snap, _ = _out_like(v, (nz, nx, ny, nt)) if want_snapshot else (None, None)
    check(lib().sssi_fwdTimeCpmlFor3dAwPoint(pv, nz, nx, ny, int(nt), int(nDiffOrder), int(nBoundary), float(dz),
                                             float(dx), float(dy), float(dt), len(iz), iz.ctypes.data, ix.ctypes.data,
                                             iy.ctypes.data, w.ctypes.data, _addr(data), _addr(snap), _mode(mode)))
    return data, snap


def rtmTimeCpmlFor2dAw(v, vs, wavelet, src_iz, src_ix, nDiffOrder, nBoundary, dz, dx, dt, *, epsilon=1e-3,
                       mode="fp64", snap_stride=4, want_data=False):
    """One RTM shot: image = M./s2 of mainRtmTimeCpmlFor2dAw.m:268-275,315 for a
    point source at interior (src_iz, src_ix).  Returns image, or (image,
    dataTrue, dataSmooth) with ``want_data``."""
    pv, kv, vshape = _in(v, "v")
    pvs, kvs, vsshape = _in(vs, "vs")
    pw, kw, wshape = _in(wavelet, "wavelet")
    if vshape != vsshape or len(vshape) != 2:
        raise ValueError("v and vs must be nz x nx of the same size")
    nz, nx = vshape
    nt = wshape[0]
    image, _ = _out_like(v, (nz, nx))
    dt_, _ = _out_like(v, (nx, nt)) if want_data else (None, None)
    ds_, _ = _out_like(v, (nx, nt)) if want_data else (None, None)
    check(lib().sssi_rtmTimeCpmlFor2dAw(pv, pvs, nz, nx, nt, int(nDiffOrder), int(nBoundary), float(dz), float(dx),
                                        float(dt), pw, int(src_iz), int(src_ix), float(epsilon), _mode(mode),
                                        int(snap_stride), _addr(image), _addr(dt_), _addr(ds_)))
    if want_data:
        return image, dt_, ds_
    return image


def fwdTimeSpongeFor2dAw(v, source, nBoundary, dz, dx, dt, *, mode="fp64", want_snapshot=True):
    """[data, snapshot] = fwdTimeSpongeFor2dAw(v, source, nBoundary, dz, dx, dt)
    (src/fwdTimeSpongeFor2dAw.m): second-order five-point propagation with the
    sponge absorbing boundary."""
    pv, kv, vshape = _in(v, "v")
    ps, ks, sshape = _in(source, "source")
    if vshape is None or len(vshape) != 2:
        raise ValueError("v must be nz x nx")
    nz, nx = vshape
    if sshape is None or len(sshape) != 3 or sshape[:2] != (nz, nx):
        raise ValueError("source must be nz x nx x nt with the grid of v")
    nt = sshape[2]
    data, _ = _out_like(v, (nx, nt))
    snap, _ = _out_like(v, (nz, nx, nt)) if want_snapshot else (None, None)
    check(lib().sssi_fwdTimeSpongeFor2dAw(pv, ps, nz, nx, nt, int(nBoundary), float(dz), float(dx), float(dt),
                                          _addr(data), _addr(snap), _mode(mode)))
    return data, snap


def fwdTimeSpongeFor2dAwPoint(v, nt, src_iz, src_ix, wavelets, nBoundary, dz, dx, dt, *, mode="fp64",
                              want_snapshot=False):
    """Sponge forward modelling with point sources: source s at interior
    (src_iz[s], src_ix[s]) with amplitude wavelets[s, t].  Returns (data,
    snapshot or None)."""
    pv, kv, vshape = _in(v, "v")
    if vshape is None or len(vshape) != 2:
        raise ValueError("v must be nz x nx")
    nz, nx = vshape
    iz = np.ascontiguousarray(np.atleast_1d(src_iz), dtype=np.int64)
    ix = np.ascontiguousarray(np.atleast_1d(src_ix), dtype=np.int64)
    w = np.ascontiguousarray(np.atleast_2d(np.asarray(wavelets, dtype=np.float64)))
    if w.shape != (len(iz), nt) or len(ix) != len(iz):
        raise ValueError("wavelets must be nsrc x nt and src_iz/src_ix of length nsrc")
    data, _ = _out_like(v, (nx, nt))
    snap, _ = _out_like(v, (nz, nx, nt)) if want_snapshot else (None, None)
    check(lib().sssi_fwdTimeSpongeFor2dAwPoint(pv, nz, nx, int(nt), int(nBoundary), float(dz), float(dx), float(dt),
                                               len(iz), iz.ctypes.data, ix.ctypes.data, w.ctypes.data, _addr(data),
                                               _addr(snap), _mode(mode)))
    return data, snap


def rvsTimeSpongeFor2dAw(v, data, nBoundary, dz, dx, dt, *, mode="fp64", want_snapshot=True):
    """[model, snapshot] = rvsTimeSpongeFor2dAw(v, data, nBoundary, dz, dx, dt)
    (src/rvsTimeSpongeFor2dAw.m).  ``model`` (nz x nx) is the field after the
    last step; the reference declares that output without assigning it."""
    pv, kv, vshape = _in(v, "v")
    pd, kd, dshape = _in(data, "data")
    if vshape is None or len(vshape) != 2:
        raise ValueError("v must be nz x nx")
    nz, nx = vshape
    if dshape is None or len(dshape) != 2 or dshape[0] != nx:
        raise ValueError("data must be nx x nt")
    nt = dshape[1]
    model, _ = _out_like(v, (nz, nx))
    snap, _ = _out_like(v, (nz, nx, nt)) if want_snapshot else (None, None)
    check(lib().sssi_rvsTimeSpongeFor2dAw(pv, pd, nz, nx, nt, int(nBoundary), float(dz), float(dx), float(dt),
                                          _addr(model), _addr(snap), _mode(mode)))
    return model, snap


def rtmTimeSpongeFor2dAw(v, vs, wavelet, src_iz, src_ix, nBoundary, dz, dx, dt, *, epsilon=1e-3, mode="fp64",
                         want_data=False):
    """One sponge RTM shot: image = M./s2 of mainRtmTimeSpongeFor2dAw.m:247-268,310
    for a point source at interior (src_iz, src_ix).  FP64 modes only.
    Returns image, or (image, dataTrue, dataSmooth) with ``want_data``."""
    pv, kv, vshape = _in(v, "v")
    pvs, kvs, vsshape = _in(vs, "vs")
    pw, kw, wshape = _in(wavelet, "wavelet")
    if vshape != vsshape or len(vshape) != 2:
        raise ValueError("v and vs must be nz x nx of the same size")
    nz, nx = vshape
    nt = wshape[0]
    image, _ = _out_like(v, (nz, nx))
    dt_, _ = _out_like(v, (nx, nt)) if want_data else (None, None)
    ds_, _ = _out_like(v, (nx, nt)) if want_data else (None, None)
    check(lib().sssi_rtmTimeSpongeFor2dAw(pv, pvs, nz, nx, nt, int(nBoundary), float(dz), float(dx), float(dt), pw,
                                          int(src_iz), int(src_ix), float(epsilon), _mode(mode), _addr(image),
                                          _addr(dt_), _addr(ds_)))
    if want_data:
        return image, dt_, ds_
    return image


def fwdTimeSpmlFor2dEw(vp, vs, source, nDiffOrder, nBoundary, dz, dx, dt, *, mode="fp64", want_snapshot=True):
    """[snapshotVzp, snapshotVxp, snapshotVzs, snapshotVxs] =
    fwdTimeSpmlFor2dEw(vp, vs, source, nDiffOrder, nBoundary, dz, dx, dt)
    (src/fwdTimeSpmlFor2dEw.m): 2D elastic propagation with the simplified PML.
    ``want_snapshot`` may be a sequence of four booleans (which snapshots to return;
    the others come back as None)."""
    pp, kp, pshape = _in(vp, "vp")
    ps_, ks_, sshape_ = _in(vs, "vs")
    pr, kr, rshape = _in(source, "source")
    if pshape is None or len(pshape) != 2 or sshape_ != pshape:
        raise ValueError("vp and vs must be nz x nx of the same size")
    nz, nx = pshape
    if rshape is None or len(rshape) != 3 or rshape[:2] != (nz, nx):
        raise ValueError("source must be nz x nx x nt with the grid of vp")
    nt = rshape[2]
    want = [bool(want_snapshot)] * 4 if isinstance(want_snapshot, bool) else [bool(w) for w in want_snapshot]
    outs = [(_out_like(vp, (nz, nx, nt))[0] if w else None) for w in want]
    check(lib().sssi_fwdTimeSpmlFor2dEw(pp, ps_, pr, nz, nx, nt, int(nDiffOrder), int(nBoundary), float(dz),
                                        float(dx), float(dt), *[_addr(o) for o in outs], _mode(mode)))
    return tuple(outs)


def fwdTimeSpmlFor2dEwPoint(vp, vs, nt, src_iz, src_ix, wavelets, nDiffOrder, nBoundary, dz, dx, dt, *,
                            mode="fp64", want_snapshot=True):
    """The elastic propagation with point sources: source s at interior
    (src_iz[s], src_ix[s]) with amplitude wavelets[s, t].  Returns the four
    snapshots (Vzp, Vxp, Vzs, Vxs)."""
    pp, kp, pshape = _in(vp, "vp")
    ps_, ks_, sshape_ = _in(vs, "vs")
    if pshape is None or len(pshape) != 2 or sshape_ != pshape:
        raise ValueError("vp and vs must be nz x nx of the same size")
    nz, nx = pshape
    iz = np.ascontiguousarray(np.atleast_1d(src_iz), dtype=np.int64)
    ix = np.ascontiguousarray(np.atleast_1d(src_ix), dtype=np.int64)
    w = np.ascontiguousarray(np.atleast_2d(np.asarray(wavelets, dtype=np.float64)))
    if w.shape != (len(iz), nt) or len(ix) != len(iz):
        raise ValueError("wavelets must be nsrc x nt and src_iz/src_ix of length nsrc")
    want = [bool(want_snapshot)] * 4 if isinstance(want_snapshot, bool) else [bool(x) for x in want_snapshot]
    outs = [(_out_like(vp, (nz, nx, nt))[0] if x else None) for x in want]
    check(lib().sssi_fwdTimeSpmlFor2dEwPoint(pp, ps_, nz, nx, int(nt), int(nDiffOrder), int(nBoundary), float(dz),
                                             float(dx), float(dt), len(iz), iz.ctypes.data, ix.ctypes.data,
                                             w.ctypes.data, *[_addr(o) for o in outs], _mode(mode)))
    return tuple(outs)


def fwdTimeSpmlFor3dEw(vp, vs, source_x, source_y, source_z, nDiffOrder, nBoundary, dz, dx, dy, dt, *,
                       mode="fp64", want_snapshot=True):
    """[snapshotVzp, snapshotVxp, snapshotVyp, snapshotVzs, snapshotVxs, snapshotVys] =
    fwdTimeSpmlFor3dEw(vp, vs, source_x, source_y, source_z, nDiffOrder, nBoundary, dz, dx, dy, dt)
    (src/fwdTimeSpmlFor3dEw.m).  Any source may be None (no source);
    ``want_snapshot`` may be a sequence of six booleans."""
    pp, kp, pshape = _in(vp, "vp")
    ps_, ks_, sshape_ = _in(vs, "vs")
    if pshape is None or len(pshape) != 3 or sshape_ != pshape:
        raise ValueError("vp and vs must be nz x nx x ny of the same size")
    nz, nx, ny = pshape
    srcs, keep, nt = [], [], None
    for name, a in (("source_x", source_x), ("source_y", source_y), ("source_z", source_z)):
        pa, ka, shp = _in(a, name)
        if shp is not None:
            if len(shp) != 4 or shp[:3] != (nz, nx, ny) or (nt is not None and shp[3] != nt):
                raise ValueError(f"{name} must be nz x nx x ny x nt with the grid of vp")
            nt = shp[3]
        srcs.append(pa)
        keep.append(ka)
    if nt is None:
        raise ValueError("at least one source is needed (it sets nt)")
    want = [bool(want_snapshot)] * 6 if isinstance(want_snapshot, bool) else [bool(w) for w in want_snapshot]
    outs = [(_out_like(vp, (nz, nx, ny, nt))[0] if w else None) for w in want]
    check(lib().sssi_fwdTimeSpmlFor3dEw(pp, ps_, *srcs, nz, nx, ny, nt, int(nDiffOrder), int(nBoundary), float(dz),
                                        float(dx), float(dy), float(dt), *[_addr(o) for o in outs], _mode(mode)))
    return tuple(outs)


def fwdTimeSpmlFor3dEwPoint(vp, vs, nt, src_iz, src_ix, src_iy, src_component, wavelets, nDiffOrder, nBoundary,
                            dz, dx, dy, dt, *, mode="fp64", want_snapshot=True):
    """3D elastic propagation with point sources: source s at interior
    (src_iz[s], src_ix[s], src_iy[s]) into component src_component[s] (0 x, 1 y,
    2 z) with amplitude wavelets[s, t].  Returns the six snapshots."""
    pp, kp, pshape = _in(vp, "vp")
    ps_, ks_, sshape_ = _in(vs, "vs")
    if pshape is None or len(pshape) != 3 or sshape_ != pshape:
        raise ValueError("vp and vs must be nz x nx x ny of the same size")
    nz, nx, ny = pshape
    iz = np.ascontiguousarray(np.atleast_1d(src_iz), dtype=np.int64)
    ix = np.ascontiguousarray(np.atleast_1d(src_ix), dtype=np.int64)
    iy = np.ascontiguousarray(np.atleast_1d(src_iy), dtype=np.int64)
    cp = np.ascontiguousarray(np.atleast_1d(src_component), dtype=np.int32)
    w = np.ascontiguousarray(np.atleast_2d(np.asarray(wavelets, dtype=np.float64)))
    if w.shape != (len(iz), nt) or not (len(ix) == len(iy) == len(cp) == len(iz)):
        raise ValueError("wavelets must be nsrc x nt and the positions and components of length nsrc")
    want = [bool(want_snapshot)] * 6 if isinstance(want_snapshot, bool) else [bool(x) for x in want_snapshot]
    outs = [(_out_like(vp, (nz, nx, ny, nt))[0] if x else None) for x in want]
    check(lib().sssi_fwdTimeSpmlFor3dEwPoint(pp, ps_, nz, nx, ny, int(nt), int(nDiffOrder), int(nBoundary), float(dz),
                                             float(dx), float(dy), float(dt), len(iz), iz.ctypes.data, ix.ctypes.data,
                                             iy.ctypes.data, cp.ctypes.data, w.ctypes.data,
                                             *[_addr(o) for o in outs], _mode(mode)))
    return tuple(outs)


def mat_write(path, variables):
    """save(path, names..., '-v6'): writes a dict {name: array} (numpy arrays or
    CUDA tensors, column-major doubles) to a Level-5 MAT-file that MATLAB's load
    and scipy.io.loadmat read.  Device arrays are streamed without a full host
    copy."""
    names = list(variables)
    keep, ptrs, nds, dimarrs = [], [], [], []
    for name in names:
        p, k, shape = _in(variables[name], name)
        keep.append(k)
        ptrs.append(p or 0)
        nds.append(max(len(shape), 1))
        dimarrs.append(np.asarray(shape if len(shape) else (1,), dtype=np.int64))
    n = len(names)
    cnames = (ctypes.c_char_p * max(n, 1))(*[x.encode() for x in names])
    carrs = (ctypes.c_void_p * max(n, 1))(*ptrs)
    cnd = (ctypes.c_int * max(n, 1))(*nds)
    cdims = (ctypes.c_void_p * max(n, 1))(*[d.ctypes.data for d in dimarrs])
    check(lib().sssi_mat_write(str(path).encode(), n, ctypes.addressof(cnames), ctypes.addressof(carrs),
                               ctypes.addressof(cnd), ctypes.addressof(cdims)))


def mat_read(path, name, *, out=None):
    """load(path, name) for one real numeric variable of a Level-5 MAT-file:
    returns a column-major float64 numpy array, or fills ``out`` (a numpy array
    or CUDA tensor of the same number of elements, column-major) and returns it."""
    nd = ctypes.c_int(0)
    dims = np.zeros(8, dtype=np.int64)
    check(lib().sssi_mat_read(str(path).encode(), name.encode(), None, 0, ctypes.addressof(nd), dims.ctypes.data))
    shape = tuple(int(x) for x in dims[:nd.value])
    if out is None:
        out = np.zeros(shape, order="F")
    capacity = int(out.numel()) if _is_torch(out) else int(np.asarray(out).size)
    if not _is_torch(out) and out.ndim > 1 and not out.flags.f_contiguous:
        raise ValueError("out must be column-major (Fortran ordered)")
    check(lib().sssi_mat_read(str(path).encode(), name.encode(), _addr(out), capacity, ctypes.addressof(nd),
                              dims.ctypes.data))
    return out


def set_stream(stream) -> None:
    """Make the library launch on ``stream`` (a torch.cuda.Stream, a raw handle, or None)."""
    handle = getattr(stream, "cuda_stream", stream) or 0
    check(lib().sssi_set_stream(ctypes.c_void_p(handle)))


def enable_timing(on: bool = True) -> None:
    """Record CUDA events at phase boundaries of each propagation call."""
    check(lib().sssi_enable_timing(1 if on else 0))


def last_timing():
    """[(device ms, kernels launched)] per phase of the last timed call."""
    ms = np.zeros(16)
    nl = np.zeros(16, dtype=np.int64)
    n = ctypes.c_int(0)
    check(lib().sssi_last_timing(ms.ctypes.data, nl.ctypes.data, 16, ctypes.addressof(n)))
    return [(float(ms[k]), int(nl[k])) for k in range(min(n.value, 16))]


def measure_fp64_rate() -> float:
    """FP64 fused multiply-adds per second of the current GPU (measurement helper)."""
    r = ctypes.c_double(0.0)
    check(lib().sssi_measure_fp64_rate(ctypes.addressof(r)))
    return r.value


def debug_withhold_copy(step: int, wait_limit: int = 0) -> None:
    """Test knob: at batch step ``step`` of later calls and plans, the first
    block of the batched 2D step withholds one tile's copies, so its bounded
    wait runs out (after ``wait_limit`` polls) and the call fails cleanly;
    ``step < 0`` turns it off."""
    check(lib().sssi_debug_withhold_copy(int(step), int(wait_limit)))


def debug_tile_shape(shape: int) -> None:
    """Test knob: batches built from now on use tile shape ``shape`` (0: 64 x 32,
    1: 32 x 32, 2: 128 x 16 cells) instead of the tuner's choice; -1 restores
    the tuner.  Results do not depend on the shape."""
    check(lib().sssi_debug_tile_shape(int(shape)))


def debug_schedule3d() -> tuple[int, list[float]]:
    """The 3D schedule tuner's last choice (-1 before any) and its four timed
    runs in ms (0: even chunks, about three items per resident block; 1, 2, 3:
    cost-cut chunks, about three, two or four)."""
    sched = ctypes.c_int(-1)
    ms = (ctypes.c_float * 4)()
    check(lib().sssi_debug_schedule3d(ctypes.byref(sched), ms))
    return sched.value, [float(x) for x in ms]


def debug_divide(a, d: float):
    """Test entry: the strict forms' division of each element of ``a`` by ``d``
    and the IEEE division, as two float64 arrays (equal bit for bit)."""
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    fast = np.empty_like(a)
    ieee = np.empty_like(a)
    check(lib().sssi_debug_divide(a.ctypes.data, a.size, float(d), fast.ctypes.data, ieee.ctypes.data))
    return fast, ieee


def release_cache() -> None:
    check(lib().sssi_release_cache())


def launch_count() -> int:
    return _native.launch_count()


# ---------------------------------------------------------------- plans (batched / served shots)
SHOT_FWD2D, SHOT_RTM2D, SHOT_FWD3D = 0, 1, 2
SHOT_STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}


class Ticket:
    """A submitted shot: ``id`` for the C ABI, ``outputs`` filled when it completes."""

    def __init__(self, plan, tid, outputs, keep):
        self.plan = plan
        self.id = tid
        self.outputs = outputs
        self._keep = keep  # inputs and outputs must stay alive until the shot completes


class Plan:
    """Many shots resident on one GPU (``sssi_plan_*``): 2D forward-modelling and
    RTM shots of any grid size advance together in the batched step kernel,
    3D shots alongside; shots are admitted first come first served while their
    device memory fits ``device_bytes`` and leave as they finish.

    Results equal the single-shot functions of the same mode."""

    def __init__(self, nDiffOrder, dz, dx, dy=None, *, mode="fp32", device_bytes=0, steps_per_round=0):
        from ._native import PlanConfig

        cfg = PlanConfig(_mode(mode), int(nDiffOrder), float(dz), float(dx), float(dy if dy is not None else dx),
                         int(device_bytes), int(steps_per_round))
        h = ctypes.c_void_p()
        check(lib().sssi_plan_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            check(lib().sssi_plan_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _submit(self, desc, outputs, keep):
        from ._native import c_i64

        t = c_i64()
        check(lib().sssi_shot_submit(self._h, ctypes.byref(desc), ctypes.byref(t)))
        return Ticket(self, int(t.value), outputs, keep)

    def submit_fwd2d(self, v, nt, src_iz, src_ix, wavelets, nBoundary, dt, *, data=None):
        """Forward modelling with point sources; outputs: data (nx x nt), into
        ``data`` when given (a column-major float64 array, host or device)."""
        from ._native import ShotDesc

        pv, kv, vshape = _in(v, "v")
        nz, nx = vshape
        iz, ix, w = _points(src_iz, src_ix, None, wavelets, nt)
        data, kd = _out_like(v, (nx, nt)) if data is None else (data, None)
        d = ShotDesc(kind=SHOT_FWD2D, v=pv, nz=nz, nx=nx, ny=1, nt=int(nt), nBoundary=int(nBoundary), dt=float(dt),
                     nsrc=len(iz), src_iz=iz.ctypes.data, src_ix=ix.ctypes.data, wavelets=w.ctypes.data,
                     data=_addr(data))
        return self._submit(d, {"data": data}, (kv, kd, iz, ix, w, v))

    def submit_rtm2d(self, v, vs, wavelet, src_iz, src_ix, nBoundary, dt, *, epsilon=1e-3, snap_stride=4,
                     want_data=False, image=None, stack=0, stack_z0=0, stack_x0=0, want_image=True):
        """One RTM shot (as :func:`rtmTimeCpmlFor2dAw`); outputs: image (nz x nx)
        unless ``want_image`` is False, and dataTrue (nx x nt) with ``want_data``.
        With ``stack`` (from :meth:`stack`) the image is also added to that
        stack at (``stack_z0``, ``stack_x0``) on the device."""
        from ._native import ShotDesc

        pv, kv, vshape = _in(v, "v")
        pvs, kvs, _ = _in(vs, "vs")
        nz, nx = vshape
        nt = len(np.asarray(wavelet)) if not _is_torch(wavelet) else wavelet.shape[0]
        iz, ix, w = _points([src_iz], [src_ix], None, np.asarray(wavelet, dtype=np.float64)[None, :], nt)
        if image is None and want_image:
            image, ki = _out_like(v, (nz, nx))
        else:
            ki = None
        data, kd = _out_like(v, (nx, nt)) if want_data else (None, None)
        d = ShotDesc(kind=SHOT_RTM2D, v=pv, vs=pvs, nz=nz, nx=nx, ny=1, nt=int(nt), nBoundary=int(nBoundary),
                     dt=float(dt), nsrc=1, src_iz=iz.ctypes.data, src_ix=ix.ctypes.data, wavelets=w.ctypes.data,
                     epsilon=float(epsilon), snap_stride=int(snap_stride), data=_addr(data), image=_addr(image),
                     stack=int(stack), stack_z0=int(stack_z0), stack_x0=int(stack_x0))
        return self._submit(d, {"image": image, "data": data}, (kv, kvs, ki, kd, iz, ix, w, v, vs))

    def submit_fwd3d(self, v, nt, src_iz, src_ix, src_iy, wavelets, nBoundary, dt, *, data=None):
        """3D forward modelling with point sources; outputs: data (nx x ny x nt)."""
        from ._native import ShotDesc

        pv, kv, vshape = _in(v, "v")
        nz, nx, ny = vshape
        iz, ix, w = _points(src_iz, src_ix, None, wavelets, nt)
        iy = np.ascontiguousarray(np.atleast_1d(src_iy), dtype=np.int64)
        data, kd = _out_like(v, (nx, ny, nt)) if data is None else (data, None)
        d = ShotDesc(kind=SHOT_FWD3D, v=pv, nz=nz, nx=nx, ny=ny, nt=int(nt), nBoundary=int(nBoundary), dt=float(dt),
                     nsrc=len(iz), src_iz=iz.ctypes.data, src_ix=ix.ctypes.data, src_iy=iy.ctypes.data,
                     wavelets=w.ctypes.data, data=_addr(data))
        return self._submit(d, {"data": data}, (kv, kd, iz, ix, iy, w, v))

    @staticmethod
    def _info(info):
        return {"state": SHOT_STATES.get(info.state, info.state), "status": info.status,
                "submit_s": info.submit_s, "start_s": info.start_s, "done_s": info.done_s,
                "cell_updates": int(info.cell_updates)}

    def poll(self, ticket):
        from ._native import ShotInfo

        info = ShotInfo()
        check(lib().sssi_poll(self._h, ticket.id, ctypes.byref(info)))
        return self._info(info)

    def stack(self, nz, nx):
        """A zeroed nz x nx image on the device that RTM shots add to (returns its id)."""
        from ._native import c_i64

        sid = c_i64()
        check(lib().sssi_plan_stack_create(self._h, int(nz), int(nx), ctypes.byref(sid)))
        return int(sid.value)

    def stack_get(self, stack, out):
        """Waits for the shots submitted to ``stack`` and copies the stacked image
        into ``out`` (its nz x nx shape, float64 column-major, host or device)."""
        check(lib().sssi_plan_stack_get(self._h, int(stack), _addr(out)))
        return out

    def cancel(self, ticket):
        """Cancels a queued or running shot (it ends failed, status SSSI_ERR_CANCELLED)."""
        check(lib().sssi_cancel(self._h, ticket.id))

    def wait(self, ticket):
        """Blocks until the shot completes; returns its outputs (raises on failure)."""
        from ._native import ShotInfo

        info = ShotInfo()
        check(lib().sssi_wait(self._h, ticket.id, ctypes.byref(info)))
        ticket.info = self._info(info)
        return ticket.outputs

    def stats(self):
        from ._native import PlanStats

        st = PlanStats()
        check(lib().sssi_plan_stats_get(self._h, ctypes.byref(st)))
        out = {k: getattr(st, k) for k, _ in PlanStats._fields_}
        out["batch2d_tune_ms"] = list(out["batch2d_tune_ms"])
        return out


def _points(src_iz, src_ix, src_iy, wavelets, nt):
    iz = np.ascontiguousarray(np.atleast_1d(src_iz), dtype=np.int64)
    ix = np.ascontiguousarray(np.atleast_1d(src_ix), dtype=np.int64)
    w = np.ascontiguousarray(np.atleast_2d(np.asarray(wavelets, dtype=np.float64)))
    if w.shape != (len(iz), nt) or len(ix) != len(iz):
        raise ValueError("wavelets must be nsrc x nt and the source index arrays of length nsrc")
    return iz, ix, w
