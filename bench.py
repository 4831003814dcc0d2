#!/usr/bin/env python3
"""Benchmark of the SSSI acoustic CPML hot path on GB300.

Workload (one "step" = one reverse-time-migration shot): 2D single-shot RTM
on a 600 x 1200 physical grid (620 x 1240 after extBoundary with a 20-cell
CPML on the bottom/left/right, no top layer), dx = dz = 10 m, dt = 0.8 ms,
nt = 4000, 8th-order staggered space (nDiffOrder = 4), 15 Hz Ricker source at
the surface centre, seeded 6-layer velocity model (1500-4000 m/s increasing
with depth) and its Gaussian-smoothed copy (sigma = 15 cells) as migration
model.  One shot = forward modelling in both models + reverse propagation of
dataTrue - dataSmooth + zero-lag imaging: 3 * 620 * 1240 * 4000 = 9.23e9
cell-updates.

Headline arm (default): the FP64 drop-in (fused FP64, within 1e-12 relative
L2 of the reference C), the same arithmetic width as the reference's CPU
code.  ``value`` times the shot with every input already in HBM; ``e2e``
calls the same C ABI entry point (sssi_rtmTimeCpmlFor2dAw) with host buffers
(models and wavelet copied in, image copied out inside the timed region).
The FP64 stencil is bound by the FP64 pipe on GB300, so its roofline is FP64
operations per second against the FP64 FMA rate measured in the same run.

Beside it, in the same JSON line: ``fp32`` (the precision form: FP32
wavefield, compensated FP32 memory variables and imaging sums, FP16 forward
snapshots every 4th step; with its HBM roofline and its error against
FP64), ``c1`` (plain 2D forward modelling of 220 x 340 x 2000 through the
MEX-shaped dense API with host buffers), ``fwd3d``, ``batch2d`` and
``serve``.

``--impl reference`` times the CPU implementation of the same shot (the C
restatement of the reference's algorithm, OpenMP over every host core) on a
bounded number of time steps and reports the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-updates/s (2D RTM shot, 620x1240 padded, nt=4000)"
UNIT = "Gcell-updates/s"

# ---------------------------------------------------------------- workload
NZ0, NX0, NB, N_ORDER = 600, 1200, 20, 4
NT, DT, DX, DZ, FREQ, EPS = 4000, 8e-4, 10.0, 10.0, 15.0, 1e-3
STRIDE = 4


def ext_boundary(V, nB):
    W = np.concatenate([np.repeat(V[:, :1], nB, 1), V, np.repeat(V[:, -1:], nB, 1)], axis=1)
    return np.concatenate([W, np.repeat(W[-1:, :], nB, 0)], axis=0)


def ext_boundary_3d(V, nB):
    """The 3D padding: edge values replicated nB times on both x sides, both y
    sides and below (no layer on top)."""
    return np.asfortranarray(np.pad(V, ((0, nB), (nB, nB), (nB, nB)), mode="edge"))


def model_3d_c4(nb=16):
    """The 3D workload's model: the seeded dipping-layer model on a 256^3
    physical grid, padded with the damping bands to 272 x 288 x 288."""
    return ext_boundary_3d(dipping_model_3d(256), nb)


def ricker(f, n, dt):
    t = np.arange(n) * dt
    tau = t - 1.0 / f
    return (1 - 2 * tau * tau * f ** 2 * np.pi ** 2) * np.exp(-(tau ** 2) * np.pi ** 2 * f ** 2)


def make_models(seed=20240601):
    """Seeded 6-layer model (flat interfaces at sorted random depths, velocities
    sorted uniform in [1500, 4000]) and its Gaussian-smoothed copy."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    depths = np.sort(rng.choice(np.arange(40, NZ0 - 20), 5, replace=False))
    vel = np.sort(rng.uniform(1500.0, 4000.0, 6))
    v = np.empty((NZ0, NX0))
    edges = [0, *depths, NZ0]
    for k in range(6):
        v[edges[k]:edges[k + 1], :] = vel[k]
    vs = gaussian_filter(v, sigma=15, mode="nearest")
    V = np.asfortranarray(ext_boundary(v, NB))
    VS = np.asfortranarray(ext_boundary(vs, NB))
    return V, VS


def workload():
    V, VS = make_models()
    nz, nx = V.shape
    w = ricker(FREQ, NT, DT)
    return V, VS, w, 0, NB + NX0 // 2, nz, nx


def cell_updates(nz, nx, nt):
    return 3 * nz * nx * nt


# dram__bytes_read.sum + dram__bytes_write.sum of one forward step of the FP32
# RTM shot (the residual pair on 620 x 1240), from `ncu --set full --clock-control
# none -k regex:batch2d -s 40 -c 2 python bench.py --case rtm-short`
FWD_STEP_DRAM_BYTES = 35_389_440
# the same for one FP64 forward step of the RTM shot (fused FP64), from
# `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
# --clock-control none -k regex:batch2d -s 40 -c 2 python bench.py --case rtm-short-fp64`
# (42,652,672 B read, 10,240 B written: the step's writes stay in L2)
FWD64_STEP_DRAM_BYTES = 42_662_912
# the same for one 3D step of the 272 x 288 x 288 grid with 16-cell bands, from
# `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
# --clock-control none -k regex:prop3d_kernel -s 2 -c 1 python bench.py --case step3d-fp32`
STEP3D_DRAM_BYTES = 394_253_824 + 118_571_008
# the same for one batched step of the 64-shot workload while all 64 shots are
# active (the 301st launch), from `ncu --metrics dram__bytes_read.sum,
# dram__bytes_write.sum,gpu__time_duration.sum -k regex:batch2d -s 300 -c 2
# python bench.py --case batch64`
BATCH_STEP_DRAM_BYTES = 1_209_339_392 + 373_152_000


# FP64 instructions per cell of one step in the composed-stencil form of the
# fused FP64 kernel: z sum 1 mul + 7 (add + fma), x sum 15 fma, update
# lz + lx, 2P - Pold, (v dt)^2 * lap + ... (3): the least any cell needs
# (cells next to a damped band take the two-stage form and more).
FP64_OPS_PER_CELL = 33


def step_bytes_per_cell_fp64(nz, nx, nb):
    """Algorithmic HBM bytes of one FP64 step per cell: 32 B for P(t), P(t-1),
    (v dt)^2 read and P(t+1) written, plus 48 B per damped cell and axis
    (phi and psi read and written, b and b-1 read)."""
    return 32 + 48 * (nb / nz + 2 * nb / nx)


def pair_bytes_per_cell(nz, nx, nb, stride):
    """Algorithmic HBM bytes per cell of one step of the FP32 RTM forward pair:
    P as hi + lo (current and previous read, new written: 24 B), the residual
    D (12 B), (v dt)^2 and its difference (8 B); every `stride` steps the FP16
    snapshot (2 B), its error feedback (4 B read and written) and the FP32
    illumination sum (8 B read and written); per damped cell and axis the
    compensated memory variables of both fields (64 B) and b, b-1, b_Q-b_P (12 B)."""
    return 44 + (2 + 8 + 16) / stride + 76 * (nb / nz + 2 * nb / nx)


def step_bytes_per_cell(nz, nx, nb):
    """Algorithmic HBM bytes of one FP32 step per cell: P(t), P(t-1), (v dt)^2
    read and P(t+1) written (16 B), plus, per damped cell and axis, the
    compensated memory variables phi (read, write) and psi (read, write) at
    8 B each and the coefficients b, b-1 at 4 B each (40 B)."""
    return 16 + 40 * (nb / nz + 2 * nb / nx)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.rows = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=5)
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 7 for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch

    import sssi_gb300 as S

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    S.set_stream(stream)

    V, VS, w, siz, six, nz, nx = workload()

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().T

    dV, dVS, dw = dev(V), dev(VS), torch.from_numpy(w).cuda()
    dimg = dev(np.zeros((nz, nx)))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def shot(mode, stride, vv, vvs, ww, img):
        return S.api.lib().sssi_rtmTimeCpmlFor2dAw(
            S.api._addr(vv), S.api._addr(vvs), nz, nx, NT, N_ORDER, NB, DZ, DX, DT, S.api._addr(ww), siz, six, EPS,
            S.api._mode(mode), stride, S.api._addr(img), None, None)

    def timed_shots(mode, stride, steps, warmup, host=False):
        if host:
            hV = torch.from_numpy(np.ascontiguousarray(V.T)).pin_memory().T
            hVS = torch.from_numpy(np.ascontiguousarray(VS.T)).pin_memory().T
            hw = torch.from_numpy(w).pin_memory()
            himg = torch.zeros((nx, nz), dtype=torch.float64).pin_memory().T
            operands = (hV, hVS, hw, himg)
        else:
            operands = (dV, dVS, dw, dimg)
        for _ in range(warmup):
            S.api.check(shot(mode, stride, *operands))
        total = 0.0
        phases = []
        launches0 = S.launch_count()
        for _ in range(steps):
            flush.zero_()
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            S.api.check(shot(mode, stride, *operands))
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
            phases.append(S.last_timing())
        launches = S.launch_count() - launches0
        ms = total / steps
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms, phases, launches // max(steps, 1)

    S.enable_timing(True)
    # headline: the FP64 drop-in, timed with the clocks sampled
    clocks = ClockSampler()
    clocks.start()
    ms64, ph64, launches64 = timed_shots("fp64", 1, args.steps, args.warmup)
    clk = clocks.stop()
    ms64_e2e, _, _ = timed_shots("fp64", 1, max(2, args.steps // 2), 1, host=True)
    # the precision form beside it
    ms32, ph32, launches32 = timed_shots("fp32", STRIDE, args.steps, args.warmup)
    ms32_e2e, _, _ = timed_shots("fp32", STRIDE, max(2, args.steps // 2), 1, host=True)
    fma_rate = S.measure_fp64_rate()

    accuracy = rtm_accuracy(S, dV, dVS, dw, siz, six, nz, nx) if (rank == 0 and not args.no_accuracy) else None

    cells = cell_updates(nz, nx, NT)
    value = world * cells / (ms64 * 1e-3) / 1e9
    e2e = world * cells / (ms64_e2e * 1e-3) / 1e9
    value32 = world * cells / (ms32 * 1e-3) / 1e9
    e2e32 = world * cells / (ms32_e2e * 1e-3) / 1e9
    h2d = int(2 * nz * nx * 8 + NT * 8)
    d2h = int(nz * nx * 8)
    peak, peak_kind = peaks()

    # roofline of the dominant kernel, the fused FP64 step, timed over the
    # forward phase (CUDA events on the launching stream): one forward step
    # advances the shots in v and in vs and stores the vs field (FP64 snapshot)
    fwd64_ms = float(np.mean([p[0][0] for p in ph64]))
    step64_ms = fwd64_ms / NT
    ops64 = 2 * nz * nx * FP64_OPS_PER_CELL
    achieved64 = ops64 / (step64_ms * 1e-3) / 1e9
    bytes64 = nz * nx * (2 * step_bytes_per_cell_fp64(nz, nx, NB) + 8)
    hbm64 = bytes64 / (step64_ms * 1e-3) / 1e9

    # the same for the FP32 step (HBM-bound)
    fwd_ms = float(np.mean([p[0][0] for p in ph32]))
    per_launch_ms = fwd_ms / NT
    # a forward launch advances the residual pair (the field in vs and the
    # residual of the field in v)
    bytes_cell = pair_bytes_per_cell(nz, nx, NB, STRIDE)
    alg_bytes = nz * nx * bytes_cell
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms64, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded layered model, Ricker source)",
        "config": {"workload": "rtm2d-single-shot", "nz": nz, "nx": nx, "nt": NT, "nDiffOrder": N_ORDER,
                   "nBoundary": NB, "dt": DT, "dx": DX, "arithmetic": "fused FP64 (<= 1e-12 of the reference)",
                   "snapshot": "fp64 every step", "cell_updates_per_step": cells,
                   "l2": "flushed (512 MB write) before every timed step",
                   "parallelism": "replicas" if world > 1 else "single-gpu"},
        "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(ms64_e2e, 3), "api": "sssi_rtmTimeCpmlFor2dAw (host buffers)"},
        "roofline": {"bound": "fp64", "achieved": round(achieved64, 1), "peak": round(fma_rate / 1e9, 1),
                     "unit": "Gop/s", "frac": round(achieved64 * 1e9 / fma_rate, 4), "traffic": FWD64_STEP_DRAM_BYTES,
                     "traffic_note": "dram read+write of one FP64 forward step from an ncu capture of the same grid "
                                     "(caches flushed per pass); its algorithmic bytes are " + str(int(bytes64)),
                     "peak_kind": "measured in this run: FP64 fused multiply-adds per second "
                                  "(sssi_measure_fp64_rate, 8 independent chains per thread)",
                     "ops_per_cell": FP64_OPS_PER_CELL, "alg_ops_per_launch": int(ops64),
                     "kernel": "batch2d step (fused fp64, forward phase)", "launch_ms": round(step64_ms, 5),
                     "tflops": round(achieved64 * 1e9 * (57.0 / 33.0) / 1e12, 3),
                     "hbm": {"achieved": round(hbm64, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(hbm64 / peak, 4), "peak_kind": peak_kind,
                             "bytes_per_cell": round(step_bytes_per_cell_fp64(nz, nx, NB), 2)}},
        "gpu_launches": int(launches64),
        "clocks": clk,
        "phases_ms": {"forward": round(fwd64_ms, 2),
                      "reverse+imaging": round(float(np.mean([p[1][0] for p in ph64])), 2),
                      "finish": round(float(np.mean([p[2][0] for p in ph64])), 3)},
        "fp32": {"value": round(value32, 3), "unit": UNIT, "ms_per_step": round(ms32, 3), "dtype": "fp32",
                 "form": f"FP32 wavefield, compensated FP32 memory variables and imaging sums, FP16 forward "
                         f"snapshots every {STRIDE} steps",
                 "speedup_vs_fp64": round(value32 / value, 2), "gpu_launches": int(launches32),
                 "e2e": {"value": round(e2e32, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h, "ms_per_step": round(ms32_e2e, 3),
                         "api": "sssi_rtmTimeCpmlFor2dAw (host buffers)"},
                 "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                              "frac": round(achieved / peak, 4), "traffic": FWD_STEP_DRAM_BYTES,
                              "traffic_note": "dram read+write of one forward pair step from an ncu capture of the "
                                              "same grid (caches flushed per pass); the timed steps run from L2",
                              "alg_bytes_per_launch": int(alg_bytes), "peak_kind": peak_kind,
                              "kernel": "batch2d step (fp32 residual pair, forward phase)",
                              "bytes_per_cell": round(bytes_cell, 2),
                              "launch_ms": round(per_launch_ms, 5)},
                 "phases_ms": {"forward": round(fwd_ms, 2),
                               "reverse+imaging": round(float(np.mean([p[1][0] for p in ph32])), 2),
                               "finish": round(float(np.mean([p[2][0] for p in ph32])), 3)}},
    }
    if accuracy is not None:
        line["fp32"]["accuracy"] = accuracy
    if rank == 0 and not args.no_c1:
        line["c1"] = bench_c1(S, args)
    if rank == 0 and not args.no_3d:
        line["fwd3d"] = bench_3d(S, args)
    if rank == 0 and not args.no_diffop:
        line["diff_operator"] = bench_diffop(S, args, fma_rate)
    if rank == 0 and not args.no_sponge:
        line["sponge"] = bench_sponge(S, args, fma_rate)
    if rank == 0 and not args.no_elastic:
        line["elastic2d"] = bench_elastic(S, args, fma_rate)
    if rank == 0 and not args.no_batch:
        line["batch2d"] = bench_batch(S, args)
    if rank == 0 and not args.no_serve:
        line["serve"] = bench_serve(S, args)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def c1_model(seed=20240515):
    """The plain forward-modelling workload: a seeded 4-layer model on a 200 x
    300 physical grid (flat interfaces at sorted random depths, velocities
    sorted uniform in [1500, 4000] m/s), padded by extBoundary with 20 cells
    to 220 x 340."""
    rng = np.random.default_rng(seed)
    nz0, nx0 = 200, 300
    depths = np.sort(rng.choice(np.arange(20, nz0 - 10), 3, replace=False))
    vel = np.sort(rng.uniform(1500.0, 4000.0, 4))
    v = np.empty((nz0, nx0))
    edges = [0, *depths, nz0]
    for k in range(4):
        v[edges[k]:edges[k + 1], :] = vel[k]
    return np.asfortranarray(ext_boundary(v, 20))


def bench_c1(S, args):
    """Plain 2D forward modelling as the MATLAB application calls the MEX
    (mainWaveTimeCpmlFor2dAw.m:131): 220 x 340 padded model, nt = 2000, dt =
    1 ms, N = 4, nB = 20, dense nz x nx x nt source holding a 20 Hz Ricker at
    physical (2, 150), data and the full snapshot returned.  Timed through
    sssi_fwdTimeCpmlFor2dAw with pinned host buffers (1.2 GB of source in, 1.2
    GB of snapshot out per call, inside the timed region) and with device
    buffers; fused FP64 (the default of the MEX gateways) and strict FP64."""
    import torch

    v = c1_model()
    nz, nx = v.shape
    nt, dt = 2000, 1e-3
    w = ricker(20.0, nt, dt)
    src_h = torch.zeros((nt, nx, nz), dtype=torch.float64).pin_memory()
    src_h[:, 170, 2] = torch.from_numpy(w)
    src_h = src_h.permute(2, 1, 0)
    snap_h = torch.empty((nt, nx, nz), dtype=torch.float64).pin_memory().permute(2, 1, 0)
    data_h = torch.empty((nt, nx), dtype=torch.float64).pin_memory().T
    v_h = torch.from_numpy(np.ascontiguousarray(v.T)).pin_memory().T
    src_d, snap_d = src_h.cuda(), torch.empty_like(src_h, device="cuda")
    data_d, v_d = torch.empty_like(data_h, device="cuda"), v_h.cuda()

    def call(mode, vv, src, data, snap):
        S.api.check(S.api.lib().sssi_fwdTimeCpmlFor2dAw(
            S.api._addr(vv), S.api._addr(src), nz, nx, nt, N_ORDER, 20, 10.0, 10.0, dt, S.api._addr(data),
            S.api._addr(snap), S.api._mode(mode)))

    def timed(mode, host, reps):
        ops = (v_h, src_h, data_h, snap_h) if host else (v_d, src_d, data_d, snap_d)
        call(mode, *ops)
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            call(mode, *ops)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts)), S.last_timing()

    cells = nz * nx * nt
    out = {"metric": "Gcell-updates/s (2D forward modelling 220x340, nt=2000, dense source and snapshot)",
           "unit": UNIT, "cell_updates": cells, "dtype": "f64",
           "h2d_bytes_per_call": int(8 * (nz * nx + nz * nx * nt)), "d2h_bytes_per_call": int(8 * (nx * nt + nz * nx * nt)),
           "config": {"workload": "fwd2d-dense-c1", "grid": [nz, nx], "nt": nt, "dt": dt, "nDiffOrder": N_ORDER,
                      "nBoundary": 20, "model": "seeded 4-layer model, 1500-4000 m/s",
                      "source": "20 Hz Ricker at physical (2, 150), dense nz x nx x nt"}}
    data = {}
    for mode in ("fp64", "fp64-strict"):
        ms_h, ph_h = timed(mode, True, 3)
        ms_d, ph_d = timed(mode, False, 3)
        data[mode] = data_d.clone()
        out[mode] = {"e2e": round(cells / (ms_h * 1e-3) / 1e9, 3), "ms_e2e": round(ms_h, 2),
                     "value": round(cells / (ms_d * 1e-3) / 1e9, 3), "ms_device": round(ms_d, 2),
                     "propagation_ms_host_call": round(ph_h[0][0], 2) if ph_h else None}
    a, b = data["fp64"], data["fp64-strict"]
    out["fp64_vs_strict_data_rel_l2"] = float(torch.linalg.norm((a - b).flatten()) / torch.linalg.norm(b.flatten()))
    return out


def rtm_accuracy(S, dV, dVS, dw, siz, six, nz, nx):
    """FP32 (FP16 snapshots every STRIDE steps) against the FP64 drop-in on the
    full shot: relative L2 of the image and of both seismograms."""
    import torch

    res = {}
    for mode, stride in (("fp64", 1), ("fp32", STRIDE)):
        img = torch.zeros((nx, nz), dtype=torch.float64, device="cuda").T
        dtrue = torch.zeros((NT, nx), dtype=torch.float64, device="cuda").T
        dsm = torch.zeros((NT, nx), dtype=torch.float64, device="cuda").T
        S.api.check(S.api.lib().sssi_rtmTimeCpmlFor2dAw(
            S.api._addr(dV), S.api._addr(dVS), nz, nx, NT, N_ORDER, NB, DZ, DX, DT, S.api._addr(dw), siz, six, EPS,
            S.api._mode(mode), stride, S.api._addr(img), S.api._addr(dtrue), S.api._addr(dsm)))
        res[mode] = (img, dtrue, dsm)
    torch.cuda.synchronize()

    def rel(a, b):
        return float(torch.linalg.norm((a - b).flatten()) / torch.linalg.norm(b.flatten()))

    return {"image_rel_l2": rel(res["fp32"][0], res["fp64"][0]),
            "seismogram_rel_l2": rel(res["fp32"][1], res["fp64"][1]),
            "seismogram_smooth_rel_l2": rel(res["fp32"][2], res["fp64"][2]),
            "against": "fp64 drop-in on the same shot (the fp64 path matches the reference C-MEX to <= 1e-12)",
            "bound": 1e-4}


def dipping_model_3d(n, seed=20240617):
    """Seeded 5-layer model with dipping planar interfaces (dip <= 15 degrees in
    x and y), velocities sorted uniform in [1500, 4500] m/s."""
    rng = np.random.default_rng(seed)
    vel = np.sort(rng.uniform(1500.0, 4500.0, 5))
    depth = np.sort(rng.uniform(0.15, 0.9, 4)) * n
    dips = np.tan(np.radians(rng.uniform(-15.0, 15.0, (4, 2))))
    z = np.arange(n)[:, None, None]
    x = np.arange(n)[None, :, None] - n / 2
    y = np.arange(n)[None, None, :] - n / 2
    v = np.full((n, n, n), vel[0])
    for k in range(4):
        v = np.where(z >= depth[k] + dips[k, 0] * x + dips[k, 1] * y, vel[k + 1], v)
    return np.asfortranarray(v)


def bench_3d(S, args):
    """3D forward modelling: a 256^3 physical grid padded with 16-cell CPML
    bands to 272 x 288 x 288, nt = 2000, N = 4, point source at the surface
    centre; FP32 timed, receivers (every 2 cells) compared with the FP64 path."""
    import torch

    nt, nb, dt3 = args.nt3d, 16, 8e-4
    v = model_3d_c4(nb)
    nz, nx, ny = v.shape
    dv = torch.from_numpy(np.ascontiguousarray(v.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    w = np.ascontiguousarray(ricker(20.0, nt, dt3)[None, :])
    iz = np.array([0], dtype=np.int64)
    ix = np.array([nx // 2], dtype=np.int64)
    iy = np.array([ny // 2], dtype=np.int64)

    def run(mode, data):
        S.api.check(S.api.lib().sssi_fwdTimeCpmlFor3dAwPoint(
            S.api._addr(dv), nz, nx, ny, nt, N_ORDER, nb, 10.0, 10.0, 10.0, dt3, 1, iz.ctypes.data, ix.ctypes.data,
            iy.ctypes.data, w.ctypes.data, S.api._addr(data), None, S.api._mode(mode)))

    d32 = torch.zeros((nt, ny, nx), dtype=torch.float64, device="cuda").permute(2, 1, 0)
    run("fp32", d32)  # warm-up
    times = []
    for _ in range(max(1, args.steps3d)):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run("fp32", d32)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    sched, sched_ms = S.debug_schedule3d()
    d64 = torch.zeros((nt, ny, nx), dtype=torch.float64, device="cuda").permute(2, 1, 0)
    t0 = time.perf_counter()
    run("fp64", d64)
    torch.cuda.synchronize()
    ms64 = (time.perf_counter() - t0) * 1e3
    a, b = d32[::2, ::2, :], d64[::2, ::2, :]
    err = float(torch.linalg.norm((a - b).flatten()) / torch.linalg.norm(b.flatten()))
    cells = nz * nx * ny * nt
    # algorithmic bytes of one step: 16 B per cell, plus per damped cell and axis
    # phi (read, write) and psi (read, write), 16 B (the band coefficients vary in
    # two dimensions only and stay cached)
    alg3 = 16.0 * nz * nx * ny + 16.0 * nb * (nx * ny + 2 * nz * ny + 2 * nz * nx)
    return {"metric": "Gcell-updates/s (3D forward shot, 256^3 + 16-cell bands = 272x288x288, nt=%d)" % nt,
            "value": round(cells / (ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_shot": round(ms, 2),
            "us_per_step": round(ms * 1e3 / nt, 2), "dtype": "fp32", "shots": len(times),
            "achieved_gbs_alg": round(alg3 / (ms * 1e-3 / nt) / 1e9, 1),
            "roofline": {"bound": "hbm", "achieved": round(alg3 / (ms * 1e-3 / nt) / 1e9, 1), "peak": peaks()[0],
                         "unit": "GB/s", "frac": round(alg3 / (ms * 1e-3 / nt) / 1e9 / peaks()[0], 4),
                         "peak_kind": peaks()[1], "alg_bytes_per_step": int(alg3),
                         "traffic": STEP3D_DRAM_BYTES,
                         "traffic_note": "dram read+write of one step from an ncu capture of the same grid (cold)"},
            "fp64": {"value": round(cells / (ms64 * 1e-3) / 1e9, 3), "ms_per_shot": round(ms64, 1)},
            "receivers_rel_l2_vs_fp64": err, "receivers": "surface grid every 2 cells (144 x 144)",
            "schedule": sched, "schedule_tune_ms": [round(t, 3) for t in sched_ms],
            "schedule_candidates": "0: even chunks along y, ~3 items per resident block; 1/2/3: cost-cut chunks, ~3/2/4",
            "config": {"workload": "fwd3d-point-source", "grid": [nz, nx, ny], "physical": [256, 256, 256],
                       "nt": nt, "nDiffOrder": N_ORDER, "nBoundary": nb,
                       "dt": dt3, "dx": 10.0, "model": "seeded 5-layer dipping-interface model, 1500-4500 m/s",
                       "source": "20 Hz Ricker at the surface centre"}}


def bench_diffop(S, args, fma_rate):
    """The stand-alone staggered derivative (diffOperator) of a 272 x 288 x 288
    array (the 3D workload's grid, 180 MB, larger than L2) along each dimension,
    8th order (4 coefficients), device arrays.  Fused FP64 does 8 FP64
    instructions per output (4 subtractions, 4 multiply-adds): bound by the FP64
    pipe (fraction of the FP64 FMA rate measured in the run); the byte view is 8 B
    read and 8 B written per output (the stencil's other reads hit L1/L2)."""
    import torch

    shape = (272, 288, 288)
    x = torch.randn(tuple(reversed(shape)), dtype=torch.float64, device="cuda").permute(2, 1, 0)
    c = S.dCoef(4)
    peak, peak_kind = peaks()
    out = {"metric": "GB/s (staggered derivative of a 272x288x288 FP64 array, 4 coefficients)",
           "config": {"workload": "diffOperator-3d", "shape": list(shape), "order": 4}}
    for mode in ("fp64", "fp64-strict"):
        for dim in (1, 2, 3):
            S.diffOperator(x, c, 10.0, dim, mode=mode)  # warm-up
            ts = []
            for _ in range(5):
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                S.diffOperator(x, c, 10.0, dim, mode=mode)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = float(np.median(ts))
            nout = np.prod(shape) * (shape[dim - 1] - 7) / shape[dim - 1]
            gbs = 16.0 * nout / (ms * 1e-3) / 1e9
            gops = 8.0 * nout / (ms * 1e-3) / 1e9
            out[f"{mode}_dim{dim}"] = {"ms": round(ms, 3), "gbs": round(gbs, 1), "frac_hbm": round(gbs / peak, 4),
                                       "fp64_gops": round(gops, 1), "frac_fp64": round(gops * 1e9 / fma_rate, 4)}
    out["roofline"] = {"bound": "fp64", "peak": round(fma_rate / 1e9, 1), "unit": "Gop/s",
                       "ops_per_output": 8, "achieved": out["fp64_dim1"]["fp64_gops"],
                       "frac": out["fp64_dim1"]["frac_fp64"]}
    out["hbm_peak"] = peak
    out["hbm_peak_kind"] = peak_kind
    out["timing"] = "CUDA events around the C-ABI call, inputs and outputs on the device (includes the output allocation)"
    return out


def bench_sponge(S, args, fma_rate):
    """One sponge-ABC RTM shot (applications/rtm_2d_acoustic/mainRtmTimeSpongeFor2dAw.m:
    forward in V and VS, reverse of dataTrue - dataSmooth, zero-lag imaging) on
    the RTM workload's 620 x 1240 model, dt from that file's rule
    0.75 min(dz / v / sqrt(2)), nt = 4000, through sssi_rtmTimeSpongeFor2dAw
    with host buffers (e2e).  Fused FP64 is the line's value; strict FP64
    (the MATLAB rounding sequence) beside it, and FP32 forward modelling of the
    same shot with its seismogram error against FP64.  The fused step does 5
    FP64 operations a cell (2 additions, 3 multiply-adds), the reverse step 2
    more for the imaging sums: bound by the FP64 pipe."""
    from oracle import oracle as O

    V, VS, _, siz, six, nz, nx = workload()
    nt = 4000
    dt = 0.75 * float(np.min(DZ / V / np.sqrt(2.0)))
    w = ricker(20.0, nt, dt)
    cells = 3.0 * nz * nx * nt
    out = {"metric": "Gcell-updates/s (sponge-ABC RTM shot, 620x1240, nt=4000, 3 propagations)",
           "config": {"workload": "rtm-sponge", "nz": nz, "nx": nx, "nt": nt, "dt": dt, "nBoundary": NB,
                      "source": "20 Hz Ricker at row 0", "epsilon": 1e-3}}
    # warm-up (short), then one shot per mode
    S.rtmTimeSpongeFor2dAw(V, VS, w[:64], siz, six, NB, DZ, DX, dt, epsilon=1e-3, mode="fp64")
    imgs = {}
    for mode in ("fp64", "fp64-strict"):
        S.enable_timing(True)
        t0 = time.perf_counter()
        img, d_true, d_smooth = S.rtmTimeSpongeFor2dAw(V, VS, w, siz, six, NB, DZ, DX, dt, epsilon=1e-3, mode=mode,
                                                       want_data=True)
        wall = time.perf_counter() - t0
        ph = S.last_timing()
        S.enable_timing(False)
        dev_ms = sum(p[0] for p in ph)
        imgs[mode] = img
        out[mode] = {"value": round(cells / wall / 1e9, 3), "unit": UNIT, "wall_ms": round(wall * 1e3, 2),
                     "device_ms": round(dev_ms, 2), "device_value": round(cells / (dev_ms * 1e-3) / 1e9, 3),
                     "launches": int(sum(p[1] for p in ph))}
    ops = nz * nx * nt * (5.0 + 5.0 + 7.0)
    dev_s = out["fp64"]["device_ms"] * 1e-3
    bytes_cell = (56.0 + 64.0 + 96.0) / 3.0  # fwd V; fwd VS + snapshot write; rvs + snapshot read + sums
    peak, peak_kind = peaks()
    out["value"] = out["fp64"]["value"]
    out["unit"] = UNIT
    out["e2e"] = {"value": out["fp64"]["value"], "unit": UNIT, "h2d_bytes_per_step": int(2 * nz * nx * 8 + nt * 8),
                  "d2h_bytes_per_step": int(nz * nx * 8 + 2 * nx * nt * 8),
                  "api": "sssi_rtmTimeSpongeFor2dAw (host buffers)"}
    out["roofline"] = {"bound": "fp64", "achieved": round(ops / dev_s / 1e9, 1), "peak": round(fma_rate / 1e9, 1),
                       "unit": "Gop/s", "frac": round(ops / dev_s / fma_rate, 4),
                       "ops_per_cell": round((5.0 + 5.0 + 7.0) / 3.0, 3),
                       "peak_kind": "measured in this run: FP64 fused multiply-adds per second",
                       "kernel": "sponge2d cell step (fused fp64), all three propagations",
                       "hbm": {"achieved": round(cells * bytes_cell / dev_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                               "frac": round(cells * bytes_cell / dev_s / 1e9 / peak, 4), "peak_kind": peak_kind,
                               "bytes_per_cell": round(bytes_cell, 2)}}
    out["accuracy"] = {"image_rel_l2_fused_vs_strict": O.rel_l2(imgs["fp64"], imgs["fp64-strict"])}
    # FP32 forward modelling of the same shot against FP64
    d64, _ = S.fwdTimeSpongeFor2dAwPoint(V, nt, [siz], [six], w[None, :], NB, DZ, DX, dt, mode="fp64")
    t0 = time.perf_counter()
    d32, _ = S.fwdTimeSpongeFor2dAwPoint(V, nt, [siz], [six], w[None, :], NB, DZ, DX, dt, mode="fp32")
    wall32 = time.perf_counter() - t0
    out["fp32_forward"] = {"value": round(nz * nx * nt / wall32 / 1e9, 3), "unit": UNIT,
                           "seismogram_rel_l2_vs_fp64": O.rel_l2(d32, d64), "bound": 1e-4}
    # parity at a bounded nt: strict GPU image equal to the C restatement's
    if not args.no_cpu:
        ntc = min(args.cpu_nt, nt)
        co = O.COracle()
        img_g = S.rtmTimeSpongeFor2dAw(V, VS, w[:ntc], siz, six, NB, DZ, DX, dt, epsilon=1e-3, mode="fp64-strict")
        t0 = time.perf_counter()
        dct, _, _ = co.sponge2d(V, ntc, NB, DZ, DX, dt, point=([siz], [six], w[None, :ntc]), want_snapshot=False)
        dcs, fcs, _ = co.sponge2d(VS, ntc, NB, DZ, DX, dt, point=([siz], [six], w[None, :ntc]))
        _, rcs, _ = co.sponge2d(V, ntc, NB, DZ, DX, dt, rdata=dct - dcs)
        img_c = O.image_np(fcs, rcs, 1e-3)
        cpu_s = time.perf_counter() - t0
        out["accuracy"]["strict_equals_c_restatement"] = bool(np.array_equal(img_g, img_c))
        out["accuracy"]["checked_nt"] = ntc
        out["cpu_baseline"] = {"value": round(3.0 * nz * nx * ntc / cpu_s / 1e9, 4), "unit": UNIT,
                               "cores": co.threads(), "kind": "port",
                               "sample": f"the same shot for nt={ntc}: the C restatement of the MATLAB sponge "
                                         "propagators (OpenMP) plus numpy imaging"}
    return out


def bench_elastic(S, args, fma_rate):
    """2D elastic SPML forward modelling (src/fwdTimeSpmlFor2dEw.m, the work of
    applications/wave_2d_elastic/mainWaveTimeSpmlFor2dEw.m:102) on the RTM
    workload's 620 x 1240 model as vp, vs = vp / sqrt(3) (a Poisson solid; the
    application's own models are .mat files that are not available here),
    nDiffOrder 3, nBoundary 20, dt = 0.5 min(dx, dz) / vpmax / sqrt(2) (the
    application's rule), 20 Hz Ricker at row 0, nt = 2000, through
    sssi_fwdTimeSpmlFor2dEwPoint.  The application keeps all four snapshot
    volumes (4 x 620 x 1240 x 2000 doubles = 49 GB); the timed runs keep none
    (the step's work is the same; the snapshots would add their device-to-host
    copies), and the FP32 error is measured on the Vzp snapshots of a shorter
    run.  Fused FP64: 62 FP64 operations an interior cell-step (8 staggered
    derivatives of 3 terms, the split updates; the velocity coefficients are
    formed once per run): bound by the FP64 pipe."""
    from oracle import oracle as O

    V, _, _, _, _, nz, nx = workload()
    vs = V / np.sqrt(3.0)
    N, nt = 3, 2000
    dt = 0.5 * min(DX, DZ) / float(V.max()) / np.sqrt(2.0)
    w = ricker(20.0, nt, dt)[None, :]
    six = NB + 49
    cells = float(nz * nx * nt)
    out = {"metric": "Gcell-updates/s (2D elastic SPML forward, 620x1240, nt=2000)",
           "config": {"workload": "elastic-2d", "nz": nz, "nx": nx, "nt": nt, "nDiffOrder": N, "nBoundary": NB,
                      "dt": dt, "vs": "vp / sqrt(3)", "snapshots": "none kept in the timed runs"}}
    S.fwdTimeSpmlFor2dEwPoint(V, vs, 32, [0], [six], w[:, :32], N, NB, DZ, DX, dt, mode="fp64", want_snapshot=False)
    for mode in ("fp64", "fp64-strict", "fp32"):
        S.enable_timing(True)
        t0 = time.perf_counter()
        S.fwdTimeSpmlFor2dEwPoint(V, vs, nt, [0], [six], w, N, NB, DZ, DX, dt, mode=mode, want_snapshot=False)
        wall = time.perf_counter() - t0
        ph = S.last_timing()
        S.enable_timing(False)
        dev_ms = sum(p[0] for p in ph)
        out[mode] = {"value": round(cells / wall / 1e9, 3), "wall_ms": round(wall * 1e3, 1),
                     "device_ms": round(dev_ms, 1), "device_value": round(cells / (dev_ms * 1e-3) / 1e9, 3)}
    # FP32 against FP64 on the first 300 steps, the whole Vzp snapshot volume
    nta = 300
    a64 = S.fwdTimeSpmlFor2dEwPoint(V, vs, nta, [0], [six], w[:, :nta], N, NB, DZ, DX, dt, mode="fp64",
                                    want_snapshot=(True, False, False, False))[0]
    a32 = S.fwdTimeSpmlFor2dEwPoint(V, vs, nta, [0], [six], w[:, :nta], N, NB, DZ, DX, dt, mode="fp32",
                                    want_snapshot=(True, False, False, False))[0]
    out["value"] = out["fp64"]["value"]
    out["unit"] = UNIT
    # FP64 operations of an interior cell-step at nDiffOrder N: 4 staggered derivatives
    # per phase (N subtractions and N multiply-adds each), the potentials' updates and
    # sums (7), the velocities' updates and sums (7); band cells add the damping
    # products, which the count leaves out
    ops_cell = 16 * N + 14
    ops = float(ops_cell) * cells
    dev_s = out["fp64"]["device_ms"] * 1e-3
    out["roofline"] = {"bound": "fp64", "achieved": round(ops / dev_s / 1e9, 1), "peak": round(fma_rate / 1e9, 1),
                       "unit": "Gop/s", "frac": round(ops / dev_s / fma_rate, 4), "ops_per_cell": ops_cell,
                       "peak_kind": "measured in this run: FP64 fused multiply-adds per second",
                       "kernel": "elastic2d phase 1 + phase 2 (fused fp64)"}
    out["accuracy"] = {"vzp_snapshot_rel_l2_fp32_vs_fp64": O.rel_l2(a32, a64), "bound": 1e-4,
                       "sample": f"the Vzp snapshots of the first {nta} steps"}
    # 3D (src/fwdTimeSpmlFor3dEw.m, the work of applications/wave_3d_elastic/
    # mainWaveTimeSpmlFor3dEw.m): a 148^3 grid with 10-cell bands, nDiffOrder 3, dt by the
    # application's rule 0.5 min(d) / vpmax / sqrt(3), a z-force at the top centre
    n3, nt3, nb3 = 148, 200, 10
    rng = np.random.default_rng(20240801)
    vp3 = np.sort(rng.uniform(2000.0, 4000.0, n3))[:, None, None] * np.ones((n3, n3, n3))
    vs3 = vp3 / np.sqrt(3.0)
    dt3 = 0.5 * 10.0 / float(vp3.max()) / np.sqrt(3.0)
    w3 = ricker(20.0, nt3, dt3)[None, :]
    S.fwdTimeSpmlFor3dEwPoint(vp3, vs3, 16, [0], [n3 // 2], [n3 // 2], [2], w3[:, :16], 3, nb3, 10.0, 10.0, 10.0,
                              dt3, mode="fp64", want_snapshot=False)
    out["3d"] = {"config": {"workload": "elastic-3d", "n": n3, "nt": nt3, "nBoundary": nb3, "nDiffOrder": 3,
                            "dt": dt3, "model": "layered vp sorted uniform(2000, 4000), vs = vp / sqrt(3)",
                            "snapshots": "none kept"}}
    for mode in ("fp64", "fp64-strict", "fp32"):
        S.enable_timing(True)
        S.fwdTimeSpmlFor3dEwPoint(vp3, vs3, nt3, [0], [n3 // 2], [n3 // 2], [2], w3, 3, nb3, 10.0, 10.0, 10.0, dt3,
                                  mode=mode, want_snapshot=False)
        ph = S.last_timing()
        S.enable_timing(False)
        dev_ms = sum(p[0] for p in ph)
        out["3d"][mode] = {"device_ms": round(dev_ms, 1),
                           "device_value": round(n3 ** 3 * nt3 / (dev_ms * 1e-3) / 1e9, 3)}
    if not args.no_cpu:
        ntc = 10
        src = np.zeros((nz, nx, ntc), order="F")
        src[0, six, :] = w[0, :ntc]
        t0 = time.perf_counter()
        O.fwd_elastic2d_np(V, vs, src, N, NB, DZ, DX, dt)
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(nz * nx * ntc / cpu_s / 1e9, 4), "unit": UNIT, "cores": 1,
                               "kind": "port", "sample": f"the same model for nt={ntc}: the numpy restatement of "
                                                         "the MATLAB file (vectorised statements, one core)"}
    return out


# ---------------------------------------------------------------- batched and served shots (plan API)
def model_2d_anomalies(nz, nx, seed):
    """Seeded 6-layer model (flat interfaces, velocities sorted uniform) with 3
    Gaussian anomalies of +-15 %, clipped to [1500, 4500] m/s."""
    rng = np.random.default_rng(seed)
    depths = np.sort(rng.choice(np.arange(30, nz - 20), 5, replace=False))
    vel = np.sort(rng.uniform(1500.0, 4200.0, 6))
    v = np.empty((nz, nx))
    edges = [0, *depths, nz]
    for k in range(6):
        v[edges[k]:edges[k + 1], :] = vel[k]
    z = np.arange(nz)[:, None]
    x = np.arange(nx)[None, :]
    for _ in range(3):
        cz, cx = rng.uniform(0.2, 0.8) * nz, rng.uniform(0.1, 0.9) * nx
        r = rng.uniform(0.05, 0.12) * min(nz, nx)
        v = v * (1 + rng.choice([-0.15, 0.15]) * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * r * r)))
    return np.clip(v, 1500.0, 4500.0)


def batch_shots(seed=20240702):
    """64 shots on an 800 x 2400 model: sources every 35 cells at the surface,
    each shot on an aperture window of w ~ U[600, 2400] columns around its
    source (clipped to the model), nt ~ U[2000, 4000]."""
    nz0, nx0 = 800, 2400
    v = model_2d_anomalies(nz0, nx0, seed)
    rng = np.random.default_rng(seed + 1)
    shots = []
    for k in range(64):
        xs = 20 + 35 * k
        w = int(rng.integers(600, 2401))
        a = max(0, xs - w // 2)
        b = min(nx0, a + w)
        a = max(0, b - w)
        nt = int(rng.integers(2000, 4001))
        shots.append((np.asfortranarray(ext_boundary(v[:, a:b], NB)), nt, 0, xs - a + NB))
    return shots


def bench_batch(S, args):
    """The 64 shots submitted at once to a plan (FP32), timed end to end with
    host models in and host seismograms out; beside it the same shots' rate
    through the single-shot entry point, and the FP32 error against FP64."""
    dt = 8e-4
    shots = batch_shots()
    waves = [ricker(20.0, nt, dt)[None, :] for (_, nt, _, _) in shots]
    cells = float(sum(V.shape[0] * V.shape[1] * nt for (V, nt, _, _) in shots))
    with S.Plan(N_ORDER, DZ, DX, mode="fp32") as plan:
        V, nt, iz, ix = shots[0]
        plan.wait(plan.submit_fwd2d(V, 200, [iz], [ix], waves[0][:, :200], NB, dt))  # warm-up
        # the batch twice: the first pass fills the device-memory pool (a serving
        # plan runs warm); the second is the measurement
        walls = []
        for rep in range(2):
            st0 = plan.stats()
            t0 = time.perf_counter()
            tickets = [plan.submit_fwd2d(V, nt, [iz], [ix], w, NB, dt) for (V, nt, iz, ix), w in zip(shots, waves)]
            outs = [plan.wait(t)["data"] for t in tickets]
            walls.append(time.perf_counter() - t0)
            st1 = plan.stats()
        el = walls[-1]
        st = {k: (st1[k] - st0[k]) if isinstance(st1[k], float) or k == "batch_steps" else st1[k] for k in st1}
    # the same kind of shots one call at a time
    sample = list(range(0, 64, 8))
    t0 = time.perf_counter()
    for k in sample:
        V, nt, iz, ix = shots[k]
        S.fwdTimeCpmlFor2dAwPoint(V, nt, [iz], [ix], waves[k], N_ORDER, NB, DZ, DX, dt, mode="fp32")
    el1 = time.perf_counter() - t0
    cells1 = float(sum(shots[k][0].shape[0] * shots[k][0].shape[1] * shots[k][1] for k in sample))
    errs = []
    for k in sample[:2]:
        V, nt, iz, ix = shots[k]
        ref, _ = S.fwdTimeCpmlFor2dAwPoint(V, nt, [iz], [ix], waves[k], N_ORDER, NB, DZ, DX, dt, mode="fp64")
        errs.append(float(np.linalg.norm(outs[k] - ref) / np.linalg.norm(ref)))
    value = cells / el / 1e9
    single = cells1 / el1 / 1e9
    # the batched step kernel alone: device time of the plan's 2D rounds
    alg_bytes = sum(V.shape[0] * V.shape[1] * nt * step_bytes_per_cell(V.shape[0], V.shape[1], NB)
                    for (V, nt, _, _) in shots)
    peak, peak_kind = peaks()
    kern_s = st["batch2d_gpu_s"]
    kernel = {"value": round(st["batch2d_cell_updates"] / kern_s / 1e9, 2), "unit": UNIT,
              "device_s": round(kern_s, 4),
              "roofline": {"bound": "hbm", "achieved": round(alg_bytes / kern_s / 1e9, 1), "peak": peak,
                           "unit": "GB/s", "frac": round(alg_bytes / kern_s / 1e9 / peak, 4), "peak_kind": peak_kind,
                           "bytes_per_cell": round(alg_bytes / cells, 2),
                           "traffic": BATCH_STEP_DRAM_BYTES,
                           "traffic_note": "dram read+write of one step with all 64 shots active (ncu, cold); "
                                           "its algorithmic bytes are " + str(int(sum(
                                               V.shape[0] * V.shape[1] * step_bytes_per_cell(V.shape[0], V.shape[1], NB)
                                               for (V, _, _, _) in shots)))},
              "timing": "CUDA events around each round of batched steps inside the plan (whole batch, all rounds)",
              "tile_shape": ["64x32", "32x32", "128x16"][int(st["batch2d_tile_shape"])],
              "tuner_ms": {"64x32": round(st["batch2d_tune_ms"][0], 3), "32x32": round(st["batch2d_tune_ms"][1], 3),
                           "128x16": round(st["batch2d_tune_ms"][2], 3),
                           "note": "the tuner's trial steps with each tile shape (z-block depth 64, 32, 128 rows)"}}
    return {"metric": "Gcell-updates/s (64-shot batched forward modelling, 800x2400 model)",
            "value": round(value, 2), "unit": UNIT, "wall_s": round(el, 3), "first_pass_wall_s": round(walls[0], 3),
            "shots_per_s": round(64 / el, 2),
            "cell_updates": cells, "dtype": "fp32", "batch_steps": int(st["batch_steps"]),
            "plan_host_s": {k: round(st[k], 3) for k in ("admit_s", "round_s", "gpu_wait_s", "deliver_s")},
            "step_kernel": kernel,
            "single_shot_value": round(single, 2), "speedup_vs_single_shot": round(value / single, 2),
            "single_shot_sample": "8 of the 64 shots, one sssi_fwdTimeCpmlFor2dAwPoint call each",
            "data_rel_l2_vs_fp64_max": max(errs), "error_sample": "2 shots against the fp64 path",
            "e2e": "host models in, host seismograms (double) out, inside the timed region",
            "config": {"workload": "batched-fwd2d", "model": "800x2400, 6 layers + 3 Gaussian anomalies (+-15%)",
                       "shots": 64, "aperture": "U[600, 2400] columns", "nt": "U[2000, 4000]", "dt": dt,
                       "nDiffOrder": N_ORDER, "nBoundary": NB, "source": "20 Hz Ricker, every 35 cells"}}


def bench_serve(S, args):
    """A seeded Poisson stream of requests served by one FP32 plan: 2D forward
    modelling (200x300 .. 1000x3000), 2D RTM with FP16 snapshots (400x800 ..
    800x2400), 3D forward modelling (128^3 .. 256^3), nt in [1000, 4000]."""
    import torch
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(20240801)
    n_req, rate = args.serve_requests, args.serve_rate
    big2d = model_2d_anomalies(1000, 3000, 7)
    smooth2d = gaussian_filter(big2d, sigma=15, mode="nearest")
    big3d = dipping_model_3d(256, seed=99)
    reqs = []
    t = 0.0
    for k in range(n_req):
        t += rng.exponential(1.0 / rate)
        kind = rng.choice(["fwd2d", "rtm2d", "fwd3d"], p=[0.45, 0.35, 0.20])
        nt = int(rng.integers(1000, 4001))
        if kind == "fwd2d":
            nz, nx = int(rng.integers(200, 1001)), int(rng.integers(300, 3001))
        elif kind == "rtm2d":
            nz, nx = int(rng.integers(400, 801)), int(rng.integers(800, 2401))
        else:
            nz = nx = int(rng.integers(128, 257))
        z0 = int(rng.integers(0, (1000 if kind != "fwd3d" else 256) - nz + 1))
        x0 = int(rng.integers(0, (3000 if kind != "fwd3d" else 256) - nx + 1))
        reqs.append((t, kind, nz, nx, nt, z0, x0))
    # outputs: a pinned sink per kind (requests overwrite it in turn), own arrays for the checked
    # sample: a seeded stratified sample of every kind (RTM images weigh most: their reverse
    # source is a difference of two seismograms)
    per_kind = {"fwd2d": args.serve_check_fwd, "rtm2d": args.serve_check_rtm, "fwd3d": args.serve_check_3d}
    check = set()
    for kind, m in per_kind.items():
        idx = [k for k, r in enumerate(reqs) if r[1] == kind]
        check.update(int(k) for k in rng.choice(idx, min(m, len(idx)), replace=False))

    def sink(n):
        return torch.empty(n, dtype=torch.float64).pin_memory().numpy()

    sinks = {"fwd2d": sink(3000 * 4000), "rtm2d": sink(800 * 2400), "fwd3d": sink(256 * 256 * 4000)}

    def view(kind, shape, own):
        n = int(np.prod(shape))
        return np.zeros(shape, order="F") if own else sinks[kind][:n].reshape(shape, order="F")

    tickets, inputs = [], {}
    dt = 8e-4
    S.release_cache()  # the headline's cached FP64 buffers go back before the plan takes its budget
    with S.Plan(N_ORDER, DZ, DX, DX, mode="fp32", device_bytes=int(args.serve_budget_gb * (1 << 30))) as plan:
        plan.wait(plan.submit_fwd2d(np.asfortranarray(big2d[:200, :300]), 100, [0], [150],
                                    ricker(20.0, 100, dt)[None, :], NB, dt))  # warm-up
        def submit(k, kind, nz, nx, nt, z0, x0, own):
            w = ricker(20.0 if kind != "rtm2d" else 15.0, nt, dt)
            vs = None
            if kind == "fwd2d":
                v = np.asfortranarray(big2d[z0:z0 + nz, x0:x0 + nx])
                tk = plan.submit_fwd2d(v, nt, [0], [nx // 2], w[None, :], NB, dt, data=view(kind, (nx, nt), own))
            elif kind == "rtm2d":
                v = np.asfortranarray(big2d[z0:z0 + nz, x0:x0 + nx])
                vs = np.asfortranarray(smooth2d[z0:z0 + nz, x0:x0 + nx])
                tk = plan.submit_rtm2d(v, vs, w, 0, nx // 2, NB, dt, epsilon=EPS, snap_stride=args.serve_stride,
                                       image=view(kind, (nz, nx), own))
            else:
                v = np.asfortranarray(big3d[z0:z0 + nz, x0:x0 + nx, :nx])
                tk = plan.submit_fwd3d(v, nt, [0], [nx // 2], [nx // 2], w[None, :], 16, dt,
                                       data=view(kind, (nx, nx, nt), own))
            if own:
                inputs[k] = (kind, v, vs, w, nt)
            return tk

        t_start = time.perf_counter()
        for k, (ta, kind, nz, nx, nt, z0, x0) in enumerate(reqs):
            delay = ta - (time.perf_counter() - t_start)
            if delay > 0:
                time.sleep(delay)
            tickets.append(submit(k, kind, nz, nx, nt, z0, x0, k in check))
        for tk in tickets:
            plan.wait(tk)
        st = plan.stats()
        # capacity: the first requests of the stream submitted all at once (the plan saturated)
        sat = []
        if args.serve_saturate > 0:
            t0s = time.perf_counter()
            sat = [submit(k, *reqs[k][1:], False) for k in range(min(args.serve_saturate, n_req))]
            for tk in sat:
                plan.wait(tk)
            sat_wall = time.perf_counter() - t0s
    saturated = None
    if sat:
        sinfo = [tk.info for tk in sat]
        sat_span = max(i["done_s"] for i in sinfo) - min(i["submit_s"] for i in sinfo)
        saturated = {"shots": len(sat), "shots_per_s": round(len(sat) / sat_span, 3), "span_s": round(sat_span, 2),
                     "wall_s": round(sat_wall, 2),
                     "gcell_updates_per_s": round(sum(i["cell_updates"] for i in sinfo) / sat_span / 1e9, 2),
                     "note": "the first requests of the same stream submitted at once: the plan's capacity"}
    infos = [tk.info for tk in tickets]
    lat = np.array([i["done_s"] - i["submit_s"] for i in infos])
    span = max(i["done_s"] for i in infos) - min(i["submit_s"] for i in infos)
    cells = float(sum(i["cell_updates"] for i in infos))
    errs = {}
    for k, (kind, v, vs, w, nt) in sorted(inputs.items()):
        if kind == "fwd2d":
            ref, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, [0], [v.shape[1] // 2], w[None, :], N_ORDER, NB, DZ, DX, dt,
                                               mode="fp64")
            got = tickets[k].outputs["data"]
        elif kind == "rtm2d":
            ref = S.rtmTimeCpmlFor2dAw(v, vs, w, 0, v.shape[1] // 2, N_ORDER, NB, DZ, DX, dt, epsilon=EPS,
                                       mode="fp64")
            got = tickets[k].outputs["image"]
        else:
            n = v.shape[1]
            ref, _ = S.fwdTimeCpmlFor3dAwPoint(v, nt, [0], [n // 2], [n // 2], w[None, :], N_ORDER, 16, DZ, DX, DX,
                                               dt, mode="fp64")
            got = tickets[k].outputs["data"]
        errs[f"{k}:{kind}"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    kinds = [r[1] for r in reqs]
    return {"metric": "served shots/s (Poisson stream of %d mixed requests)" % n_req,
            "value": round(n_req / span, 3), "unit": "shots/s", "p50_latency_s": round(float(np.percentile(lat, 50)), 3),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 3), "mean_latency_s": round(float(lat.mean()), 3),
            "gcell_updates_per_s": round(cells / span / 1e9, 2), "span_s": round(span, 2),
            "offered_rate_per_s": rate, "requests": {k: kinds.count(k) for k in ("fwd2d", "rtm2d", "fwd3d")},
            "saturated": saturated,
            "rel_l2_vs_fp64": errs, "rel_l2_vs_fp64_max": max(errs.values()) if errs else None,
            "rel_l2_vs_fp64_max_by_kind": {kd: max([e for k, e in errs.items() if k.endswith(kd)], default=None)
                                           for kd in ("fwd2d", "rtm2d", "fwd3d")},
            "checked": {kd: sum(1 for k in errs if k.endswith(kd)) for kd in ("fwd2d", "rtm2d", "fwd3d")},
            "admission_budget_bytes": int(st["device_bytes_budget"]), "failed": int(st["failed"]), "dtype": "fp32",
            "plan_host_s": {k: round(st[k], 3) for k in ("admit_s", "round_s", "gpu_wait_s", "deliver_s")},
            "config": {"workload": "serve-mixed", "fwd2d": "200x300 .. 1000x3000", "rtm2d": "400x800 .. 800x2400, "
                       f"16-bit snapshots every {args.serve_stride} steps", "fwd3d": "128^3 .. 256^3, nB 16", "nt": "U[1000, 4000]",
                       "dt": dt, "arrivals": "Poisson, seeded", "models": "cut from a seeded layered+anomaly 2D "
                       "model (1000x3000) and a seeded dipping-layer 3D model (256^3)"}}


# ---------------------------------------------------------------- CPU arm
def cpu_rtm_rate(nt_sample, threads=None):
    """Gcell-updates/s of the CPU RTM shot (C restatement, OpenMP) on nt_sample steps."""
    from oracle import oracle as O

    co = O.COracle()
    if threads:
        co.set_threads(threads)
    V, VS, w, siz, six, nz, nx = workload()
    t0 = time.perf_counter()
    co.rtm2d(V, VS, w[:nt_sample], siz, six, N_ORDER, NB, DZ, DX, DT, EPS)
    el = time.perf_counter() - t0
    return cell_updates(nz, nx, nt_sample) / el / 1e9, co.threads(), el


def cpu_baseline(args):
    from oracle import oracle as O

    O.build(reference=False)
    rate, cores, el = cpu_rtm_rate(args.cpu_nt)
    return {"value": round(rate, 4), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one RTM shot on the same 620x1240 grid for nt={args.cpu_nt} of 4000 steps "
                      f"({el:.1f} s); C restatement of the reference algorithm, OpenMP"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    O.build(reference=False)
    for _ in range(args.warmup):
        cpu_rtm_rate(max(2, args.cpu_nt // 10))
    rates, times = [], []
    for _ in range(args.steps):
        r, cores, el = cpu_rtm_rate(args.cpu_nt)
        rates.append(r)
        times.append(el)
    value = float(np.mean(rates))
    nz, nx = NZ0 + NB, NX0 + 2 * NB
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * float(np.mean(times)), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded layered model, Ricker source)", "impl": "reference",
            "config": {"workload": "rtm2d-single-shot", "nz": nz, "nx": nx, "nt": NT,
                       "sample_nt": args.cpu_nt, "nDiffOrder": N_ORDER, "nBoundary": NB},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"each step: one RTM shot on the 620x1240 grid for nt={args.cpu_nt} "
                                       "(rate extrapolates linearly in nt)"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- profiling cases
CASES = {
    # name: (nz, nx, nt, mode) -- a grid larger than L2 so DRAM counters mean something
    "step2d-fp32-large": (4096, 4096, 6, "fp32"),
    "step2d-fp64-large": (4096, 4096, 4, "fp64"),
    "step2d-strict-large": (4096, 4096, 3, "fp64-strict"),
    "step2d-strict-c2": (620, 1240, 6, "fp64-strict"),  # the RTM workload's grid, strict FP64
    "step3d-fp32": (272, 288, 6, "fp32"),  # the 3D workload's grid (256^3 + 16-cell CPML)
    "step3d-fp32-nb0": (272, 288, 6, "fp32"),  # the same grid without damped bands
}


def run_case(name):
    """Runs one small fixed workload (for ncu captures); prints a short status line."""
    import torch

    import sssi_gb300 as S

    torch.cuda.set_device(0)
    if name == "batch64":
        # the 64-shot batch submitted once to an FP32 plan (launch 301 is a step
        # with all 64 shots active), in the 32 x 32 tiles the tuner keeps in the
        # timed run (under a profiler its trial timings would not be meaningful)
        dt = 8e-4
        shots = batch_shots()
        S.debug_tile_shape(1)
        with S.Plan(N_ORDER, DZ, DX, mode="fp32") as plan:
            tickets = [plan.submit_fwd2d(V, nt, [iz], [ix], ricker(20.0, nt, dt)[None, :], NB, dt)
                       for (V, nt, iz, ix) in shots]
            outs = [plan.wait(t)["data"] for t in tickets]
        print(f"case {name}: 64 shots ok, data max {max(float(np.abs(o).max()) for o in outs):.3e}")
        return
    if name.startswith("elastic-620x1240"):
        # 24 steps of 2D elastic forward modelling on the RTM workload's model (no snapshots)
        mode = name.rsplit("-", 1)[1]
        V, _, _, _, _, nz, nx = workload()
        dt = 0.5 * min(DX, DZ) / float(V.max()) / np.sqrt(2.0)
        w = ricker(20.0, 24, dt)[None, :]
        S.fwdTimeSpmlFor2dEwPoint(V, V / np.sqrt(3.0), 24, [0], [NB + 49], w, 3, NB, DZ, DX, dt, mode=mode,
                                  want_snapshot=False)
        torch.cuda.synchronize()
        print(f"case {name}: ok")
        return
    if name.startswith("sponge-2000x4000"):
        # 24 steps of sponge forward modelling (one point source, 20-cell sponge)
        mode = name.rsplit("-", 1)[1]
        rng = np.random.default_rng(1)
        nz, nx, nt = 2000, 4000, 24
        v = rng.uniform(1500.0, 4000.0, (nz, nx))
        w = np.sin(np.arange(nt) * 0.05)[None, :]
        d, _ = S.fwdTimeSpongeFor2dAwPoint(v, nt, [1], [nx // 2], w, 20, 10.0, 10.0, 8e-4, mode=mode)
        torch.cuda.synchronize()
        print(f"case {name}: ok, data max {np.abs(d).max():.3e}")
        return
    if name in ("rtm-short", "rtm-short-fp64"):
        V, VS, w, siz, six, nz, nx = workload()
        fp64 = name.endswith("fp64")
        img = S.rtmTimeCpmlFor2dAw(V, VS, w[:64], siz, six, N_ORDER, NB, DZ, DX, DT, epsilon=EPS,
                                   mode="fp64" if fp64 else "fp32", snap_stride=1 if fp64 else STRIDE)
        print(f"case {name}: image max {np.abs(img).max():.3e}")
        return
    nz, nx, nt, mode = CASES[name]
    if name.startswith("step3d"):
        nb = 0 if name.endswith("nb0") else 16
        v = model_3d_c4(16)  # the 3D workload's 272 x 288 x 288 grid
        n3 = v.shape
        d, _ = S.fwdTimeCpmlFor3dAwPoint(v, nt, [0], [n3[1] // 2], [n3[2] // 2], ricker(20.0, nt, 8e-4)[None, :],
                                         N_ORDER, nb, 10.0, 10.0, 10.0, 8e-4, mode=mode)
        torch.cuda.synchronize()
        print(f"case {name}: {n3} nt={nt} {mode} ok, data max {np.abs(d).max():.3e}")
        return
    rng = np.random.default_rng(1)
    v = rng.uniform(1500.0, 4000.0, (nz, nx))
    d, _ = S.fwdTimeCpmlFor2dAwPoint(v, nt, [2], [nx // 2], ricker(FREQ, nt, DT)[None, :], N_ORDER, NB, DZ, DX, DT,
                                     mode=mode)
    torch.cuda.synchronize()
    print(f"case {name}: {nz}x{nx} nt={nt} {mode} ok, data max {np.abs(d).max():.3e}")


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--case", choices=sorted(CASES) + ["rtm-short", "rtm-short-fp64", "batch64",
                                                       "sponge-2000x4000-fp64", "sponge-2000x4000-fp32",
                                                       "elastic-620x1240-fp64", "elastic-620x1240-fp32"],
                    help="run one small fixed workload for a profiler capture and exit")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-nt", type=int, default=200, help="time steps of the bounded CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the fp32-vs-fp64 error report")
    ap.add_argument("--no-3d", action="store_true", help="skip the 3D forward-modelling line")
    ap.add_argument("--no-c1", action="store_true", help="skip the plain forward-modelling (dense API) line")
    ap.add_argument("--no-diffop", action="store_true", help="skip the stand-alone derivative line")
    ap.add_argument("--no-sponge", action="store_true", help="skip the sponge-ABC RTM line")
    ap.add_argument("--no-elastic", action="store_true", help="skip the elastic forward-modelling line")
    ap.add_argument("--nt3d", type=int, default=2000)
    ap.add_argument("--steps3d", type=int, default=2)
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-shot batched line")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-stream line")
    ap.add_argument("--serve-requests", type=int, default=500)
    ap.add_argument("--serve-rate", type=float, default=10.0, help="mean arrivals per second")
    ap.add_argument("--serve-stride", type=int, default=1,
                    help="served RTM requests: forward field stored (16-bit) and imaged every this many steps")
    ap.add_argument("--serve-budget-gb", type=float, default=160.0, help="device memory the serving plan may hold")
    ap.add_argument("--serve-saturate", type=int, default=120,
                    help="requests submitted at once after the stream, to measure the plan's capacity")
    ap.add_argument("--serve-check-rtm", type=int, default=16, help="served RTM requests checked against FP64")
    ap.add_argument("--serve-check-fwd", type=int, default=6, help="served 2D forward requests checked")
    ap.add_argument("--serve-check-3d", type=int, default=3, help="served 3D requests checked")
    args = ap.parse_args()
    if args.warmup < 3:
        print("note: fewer than 3 warm-up steps requested", file=sys.stderr)
    if args.case:
        run_case(args.case)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
