"""Benchmark: ms per Q_r field at 1 % RMS error on the 128^3 correlated-k
channel (synthetic k(band, g, T, x_H2O) table of 64 bands x 16 g x 50 T x 8 x,
8 band groups), plus rays/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--method net|cv|plain] [--workload ck128|grey64|batched|particles]

A step is one full solve of one Q_r field with the inputs resident in HBM,
timed with CUDA events on the solver's stream: for the default network
control variate, the network's features, forward pass and ray allocation,
then the sampling-table upload, the control-variate preparation, the march,
the finalize kernel (Q and sigma = sqrt(var), rounded to float on the
device) and the copy of the float Q and sigma into pinned host memory.  The
network is the committed one for the grid (dnsmc_gb300/nets/ck128_g8.cvnet) or,
when absent, trained before the timed region on 16 snapshots the Monte Carlo
itself produces.  The ray budget (mean rays per cell and group) is the
smallest one whose estimated RMS error sqrt(mean var(Q)) / rms(Q) is <= 1 %
(pilot solve, 1/N scaling, refined once, then checked on the timed solves).
The profile control variate (beta = (1, -1), uniform rays) is timed once at
its own 1 % budget and plain MC is extrapolated from a pilot, for the
comparison block.  Inputs (16.8 MB) fit in L2, so L2 is flushed (a 256 MB
device write) before every timed step.  `e2e` repeats the step through the
public API from host arrays: dnsmc_set_fields (host->device, packing and
the field checks on the device) + network + solve +
dnsmc_get_results_float (the float results into the caller's arrays), wall
clock.  `gpu_launches` counts this library's kernels in the timed region
(dnsmc_get_launch_count).

`validation` states the timed field's error against the oracle's FP64
solution (64 x the timed rays, its own control variate and exact means, on
2048 cells) and against a GPU solution of the whole field at 1024 rays per
cell and group.  `roofline` is the march's instruction-issue bound:
warp instructions per SM cycle from the per-lane-step counts of the
committed ncu capture (profiles/march_pair_kernel_ck128_counters.md) and
the lane-steps and march time of this run, beside its gather rate and DRAM
traffic.  `c0` is the grey 64^3 channel (plain MC at 1 %, the reference's
grey-band representation beside the CPU reference on the same tables, and
the isothermal slab against its analytic E2 solution); `c2` the batched
workload (16 snapshots of 96^3 in one graph-replayed launch, rays from the
local optical thickness, autotuned launch shape: ms per field at 1 %).

With --gpus N (torchrun), every rank solves its own snapshots (seed = rank):
cells are independent, no collective is needed; the whole-job value is the
max-over-ranks time divided by the fields all ranks produced (weak scaling).

--impl reference times the reference's estimator as restated in the oracle
(one thread per cell, code/mc_gpu.cu:44-438; the reference's CUDA file does
not build with CUDA 13) on all host cores, FP32 like the reference build, on
a bounded sample of cells, and extrapolates ms per field at 1 % RMS.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per Q_r field at 1% RMS error: plain vs NN-control-variate MC; rays/s"
N_CELL = 128
GROUPS = 8
BYTES_PER_STEP = 32  # T 4 + x_H2O 4 + k bilinear 4x4 + Ib linear 2x4
TARGET_ERR = 0.01
# RQMC replicates per (cell, band group); sigma from their means.  2 longer
# Sobol' nets beat 4 or 8 shorter ones at the same rays (222 / 256 / 274 ms
# per field at 1 %), and the field error estimated from them matched the
# error measured against an independent 1024-ray solution (0.956 vs 0.960 %)
REPLICATES = 2


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu_index=0):
        self.samples = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) > 8 for i in range(4) if s[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_inputs(seed):
    from dnsmc_gb300 import synth
    d = synth.ck_channel(N_CELL, seed)
    return d["T"], d["x"], d["T_wall"]


def make_solver(table, T_wall, seed, threads=0, cv=1):
    import dnsmc_gb300 as D
    cfg = D.default_config(model=D.MODEL_TABLE, imax=N_CELL, jmax=N_CELL, kmax=N_CELL, Lx=2.0, Ly=2 * math.pi,
                           Lz=math.pi, stretched_x=0, T_west=T_wall, T_east=T_wall, n_groups=GROUPS, seed=seed,
                           block_threads=threads or 128, sampler=D.SAMPLER_RQMC, local_sampling=1, nvar=REPLICATES,
                           control_variate=cv)
    s = D.Solver(cfg)
    s.set_table(table["k"], table["wvc"], table["T0"], table["dT"], dnu=table["dnu"], wq=table["wq"],
                X0=table["X0"], dX=table["dX"])
    return s


def rms_error(Q, S):
    Q = np.asarray(Q, np.float64)
    S = np.asarray(S, np.float64)
    return float(math.sqrt(float((S ** 2).mean())) / math.sqrt(float((Q ** 2).mean())))


def _result_f32():
    from dnsmc_gb300 import _lib
    return _lib.RESULT_F32


def _launches():
    from dnsmc_gb300 import _lib
    return _lib.launch_count()


def plain_extrapolated(table, T, x, T_wall, seed, pilot=128):
    """Plain MC (no control variate) at 1 % RMS: ray budget from a pilot solve,
    time = measured solve time per ray x that budget (solve time is linear in
    rays; reported as extrapolated)."""
    s = make_solver(table, T_wall, seed, cv=0)
    s.set_fields(T, x)
    r, e = ray_budget(s, pilot)
    s.set_rays(pilot)
    s.solve(timeout_s=600)
    a, b = s.timing()
    s.close()
    return dict(rays_per_cell_per_group=r, rms_error_at_pilot=e, pilot_rays=pilot, pilot_solve_ms=a,
                ms_at_1pct_extrapolated=a * r / pilot)


def ray_budget(s, pilot=256):
    """Rays per cell per band group for 1 % RMS: pilot solve, 1/N scaling
    (conservative for RQMC, whose error falls at least as fast)."""
    s.set_rays(pilot)
    Q, S = s.solve(timeout_s=600)
    e = rms_error(Q, S)
    r = int(math.ceil(pilot * (e / TARGET_ERR) ** 2))
    r = max(REPLICATES, min(1 << 17, -(-r // REPLICATES) * REPLICATES))
    return r, e


def flush_l2(buf):
    if buf is not None:
        buf.fill_(1.0)
        import torch
        torch.cuda.synchronize()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl != "reference" else "gloo")
        pg = dist
    return world, rank, local, pg


def barrier_max(pg, value):
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def _ref_sample(Tf, n, cells, kw, budget_s):
    """Time the oracle's reference estimator on `cells` with photmax grown
    until one run takes about budget_s / 4; returns (result, seconds, photmax)."""
    from oracle import oracle as O
    photmax = 64
    while True:
        t0 = time.perf_counter()
        r = O.ref_mc(Tf.ravel(), cells, photmax=photmax, **kw)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or photmax >= 1 << 16:
            return r, dt, photmax
        photmax = int(photmax * max(2.0, min(8.0, budget_s / 4 / max(dt, 1e-3))))


def _ref_field_ms(r, dt, photmax, nvar, ncell_field, sample_cells):
    """ms per field at 1 % RMS from a timed sample: per-ray variance of each
    sampled cell, rays per cell for 1 % of the sample's RMS Q, time per ray."""
    rays = sample_cells * nvar * photmax
    rays_s = rays / dt
    var_ray = r["se"] ** 2 * (nvar * photmax)
    qrms = math.sqrt(float((r["Q"] ** 2).mean()))
    n_needed = float(var_ray.mean()) / (TARGET_ERR * qrms) ** 2
    return n_needed * ncell_field / rays_s * 1e3, rays_s, n_needed


def cpu_reference(table, T, x, T_wall, rays_per_cell, sample_cells=96, budget_s=20.0):
    """Reference estimator (oracle port, FP32 as the reference build) on all
    host cores over a sample of cells; returns rays/s and ms per field at 1 %."""
    from oracle import oracle as O
    n = N_CELL
    xbar = float(x.mean())
    # x-uniform slice of the table in the reference layout (the reference has
    # no x_H2O axis): k(band, T, g) at xbar, CDFs and Planck mean from it
    tables = O.ref_tables_x_slice(table, xbar)
    Tf = np.zeros((n + 2, n + 2, n + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    rng = np.random.default_rng(0)
    cells = np.stack([rng.integers(1, n + 1, sample_cells) for _ in range(3)], 1)
    cores = os.cpu_count() or 1
    kw = dict(imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi, T_west=T_wall, T_east=T_wall, model=0,
              tables=tables, nvar=2, grid_num=1, stretched=0, use_double=0, seed=5, threads=cores)
    r, dt, photmax = _ref_sample(Tf, n, cells, kw, budget_s)
    ms_field, rays_s, n_needed = _ref_field_ms(r, dt, photmax, 2, n ** 3, sample_cells)
    return dict(rays_s=rays_s, steps_s=float(r["steps"].sum()) / dt, ms_field=ms_field, rays_per_cell_1pct=n_needed,
                cores=cores, sample=f"{sample_cells} random cells x {2 * photmax} rays of the 128^3 field (x-uniform "
                                     f"table slice at mean x_H2O), {dt:.1f} s, FP32 oracle port")


# ---- the grey 64^3 channel (the reference's grey path) -------------------------
C0_N = 64


def c0_inputs():
    from dnsmc_gb300 import synth
    return synth.grey_channel(C0_N, 0)


def cpu_reference_c0(T, T_wall, sample_cells=96, budget_s=12.0):
    """The reference estimator on the grey channel as the reference runs it:
    its grey tables (code/grey_tables.cpp:19-109: 1000 equal bands to 15000
    1/cm, kappa in every band, T grid from 0.9 x 500 K to 1.1 Tmax), band
    drawn from the emission CDF at Tmax, FP32 like the reference build, all
    host cores, a sample of cells; ms per field at 1 % RMS extrapolated."""
    n = C0_N
    Tf = np.zeros((n + 2, n + 2, n + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    rng = np.random.default_rng(0)
    cells = np.stack([rng.integers(1, n + 1, sample_cells) for _ in range(3)], 1)
    cores = os.cpu_count() or 1
    kw = dict(imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi, T_west=T_wall, T_east=T_wall, model=1,
              kappa=1.0, nvar=2, grid_num=1, stretched=0, use_double=0, seed=5, threads=cores)
    r, dt, photmax = _ref_sample(Tf, n, cells, kw, budget_s)
    ms_field, rays_s, n_needed = _ref_field_ms(r, dt, photmax, 2, n ** 3, sample_cells)
    return dict(value=ms_field, unit="ms", cores=cores, kind="port", rays_per_s=rays_s,
                rays_per_cell_1pct=n_needed,
                sample=f"{sample_cells} random cells x {2 * photmax} rays of the grey 64^3 channel, {dt:.1f} s, "
                       "FP32 oracle port of the reference estimator with its grey-band tables")


def c0_solver(seed, bands=False):
    import dnsmc_gb300 as D
    cfg = D.default_config(model=D.MODEL_GREY_BANDS if bands else D.MODEL_GREY, imax=C0_N, jmax=C0_N, kmax=C0_N,
                           Lx=2.0, Ly=2 * math.pi, Lz=math.pi, stretched_x=0, T_west=300.0, T_east=300.0, kappa=1.0,
                           seed=seed, sampler=D.SAMPLER_RQMC, nvar=REPLICATES)
    s = D.Solver(cfg)
    if bands:
        s.use_grey_band_tables(1000, 55, 15000.0, 500.0)
    s.set_result_type(D.RESULT_F32)
    return s


def c0_timed(s, rays, steps, warmup, flushbuf):
    """Device time (CUDA events on the solver's stream) of `steps` solves."""
    import torch
    s.set_rays(rays)
    for _ in range(max(3, warmup)):
        s.solve(timeout_s=300)
    stream = torch.cuda.ExternalStream(s.stream())
    ms, errs, rays_tot, steps_tot = [], [], 0.0, 0.0
    for _ in range(steps):
        flush_l2(flushbuf)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.solve_async()
        e1.record(stream)
        s.wait(300)
        e1.synchronize()
        Q, S = s.results_float()
        ms.append(e0.elapsed_time(e1))
        errs.append(rms_error(Q.astype(np.float64), S.astype(np.float64)))
        c = s.counters()
        rays_tot += c.rays
        steps_tot += c.steps
    t = float(np.sum(ms)) / 1e3
    return dict(ms=float(np.mean(ms)), rms_error=float(np.mean(errs)), rays_per_s=rays_tot / t,
                ray_steps_per_s=steps_tot / t, Q=Q, S=S)


def c0_budget(s, pilot=256):
    """Rays per cell for 1 % RMS: pilot at the config's 256 rays per cell,
    1/N scaling, refined once."""
    s.set_rays(pilot)
    Q, S = s.solve(timeout_s=300)
    e = rms_error(Q.astype(np.float64), S.astype(np.float64))
    r = max(2 * REPLICATES, -(-int(math.ceil(pilot * (e / TARGET_ERR) ** 2)) // REPLICATES) * REPLICATES)
    s.set_rays(r)
    Q, S = s.solve(timeout_s=300)
    e1 = rms_error(Q.astype(np.float64), S.astype(np.float64))
    if e1 > 0.98 * TARGET_ERR:
        r = -(-int(math.ceil(r * (e1 / (0.98 * TARGET_ERR)) ** 2)) // REPLICATES) * REPLICATES
    return r, e


def dropin_e2e(T, rays, steps, warmup):
    """The grey-band channel through the reference's own call surface: the
    drop-in pair mc_gpu_ / get_results_ on host arrays in the Fortran
    layout (ghost layer, code/param.h:110-111), float results; wall clock
    of one call pair per field."""
    import ctypes
    import dnsmc_gb300 as D
    from dnsmc_gb300 import _lib
    lib = _lib.load()
    n = C0_N
    cfg = D.default_config(model=D.MODEL_GREY_BANDS, imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                           stretched_x=0, T_west=300.0, T_east=300.0, kappa=1.0, seed=104, sampler=D.SAMPLER_RQMC,
                           nvar=REPLICATES, photmax=max(1, rays // REPLICATES), p_row=1)
    _lib.check(lib.dnsmc_dropin_configure(ctypes.byref(cfg), None))
    Tf = np.zeros((n + 2, n + 2, n + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    res = np.zeros_like(Tf)
    sig = np.zeros_like(Tf)
    fp = lambda a: a.ctypes.data_as(_lib.c_float_p)
    ystart = ctypes.c_int(1)
    for _ in range(max(3, warmup)):
        lib.mc_gpu_(fp(Tf), ctypes.byref(ystart))
        lib.get_results_(fp(res), fp(sig))
    ms = []
    for _ in range(steps):
        t0 = time.perf_counter()
        lib.mc_gpu_(fp(Tf), ctypes.byref(ystart))
        lib.get_results_(fp(res), fp(sig))
        ms.append((time.perf_counter() - t0) * 1e3)
    lib.dnsmc_dropin_release()
    Q, S = res[1:-1, 1:-1, 1:-1].astype(np.float64), sig[1:-1, 1:-1, 1:-1].astype(np.float64)
    return {"ms": float(np.mean(ms)), "rays_per_cell": 2 * (rays // 2), "rms_error": rms_error(Q, S),
            "calls": "mc_gpu_(T, ystart) + get_results_(res, var) per field, host float arrays "
                     f"({n + 2}^3 with the ghost layer), wall clock",
            "h2d_bytes_per_step": int(Tf.nbytes), "d2h_bytes_per_step": int(2 * n ** 3 * 4)}


def run_c0(steps, warmup, flushbuf, with_cpu=True):
    """The grey 64^3 channel: T = 300 + 700 (1 - y^2) K + 5 % Fourier
    fluctuation, kappa = 1 per half-height, black walls at 300 K, plain MC
    (RQMC rays, no control variate) at its 1 % RMS budget and at the
    config's 256 rays per cell; the same channel with the reference's grey
    band tables (its representation of a grey gas) beside the CPU reference
    estimator on those tables; and the isothermal slab (T = 1000 K, kappa =
    1, tau_L = 2, walls 0 K and 300 K) against its analytic E2 solution."""
    from oracle import oracle as O
    g = c0_inputs()
    out = {"workload": "grey channel 64^3 (x,z periodic 2pi x pi, y walls black 300 K), T 300 + 700 (1 - y^2) K "
                       "+ 5% Fourier, kappa = 1 per half-height, plain MC (RQMC rays, 2 replicates), FP32 march, "
                       "FP64 tallies", "n": C0_N}
    s = c0_solver(101)
    s.set_fields(g["T"])
    r, e_pilot = c0_budget(s)
    t = c0_timed(s, r, steps, warmup, flushbuf)
    t256 = c0_timed(s, 256, max(1, steps // 4), 1, flushbuf)
    s.close()
    out["gpu_grey"] = {"rays_per_cell": r, "ms_at_1pct": t["ms"], "rms_error": t["rms_error"],
                       "rms_error_pilot_256": e_pilot, "rays_per_s": t["rays_per_s"],
                       "ray_steps_per_s": t["ray_steps_per_s"],
                       "at_256_rays": {"ms": t256["ms"], "rms_error": t256["rms_error"]}}
    # the reference's representation: 1000 grey bands, band drawn at Tmax
    sb = c0_solver(102, bands=True)
    sb.set_fields(g["T"])
    rb, _ = c0_budget(sb)
    tb = c0_timed(sb, rb, max(1, steps // 2), warmup, flushbuf)
    sb.close()
    out["gpu_grey_bands"] = {"rays_per_cell": rb, "ms_at_1pct": tb["ms"], "rms_error": tb["rms_error"],
                             "rays_per_s": tb["rays_per_s"],
                             "tables": "the reference's grey tables (code/grey_tables.cpp:19-109), as the CPU arm"}
    # the same through the reference's call surface, end to end from host arrays
    out["gpu_grey_bands"]["dropin_e2e"] = dropin_e2e(g["T"], rb, max(1, steps), warmup)
    # isothermal slab against E2
    import dnsmc_gb300 as D
    sl = D.Solver(D.default_config(model=D.MODEL_GREY, imax=C0_N, jmax=C0_N, kmax=C0_N, Lx=2.0, Ly=2 * math.pi,
                                   Lz=math.pi, stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=103,
                                   sampler=D.SAMPLER_RQMC, nvar=REPLICATES))
    sl.set_fields(np.full((C0_N, C0_N, C0_N), 1000.0, np.float32))
    sl.set_rays(256)
    Qs, Ss = sl.solve(timeout_s=300)
    sl.close()
    yc = (np.arange(C0_N) + 0.5) * 2.0 / C0_N
    exact = O.slab_divq(yc, 2.0, 1.0, 1000.0, 0.0, 300.0)[None, None, None, :]
    erms = math.sqrt(float((exact ** 2).mean()))
    out["slab_e2"] = {"case": "isothermal slab T 1000 K, kappa 1, tau_L 2, walls 0 K and 300 K, 64^3, 256 rays",
                      "rms_error_vs_analytic": math.sqrt(float(((Qs - exact) ** 2).mean())) / erms,
                      "rms_error_estimated": math.sqrt(float((Ss ** 2).mean())) / erms,
                      "oracle": "analytic E2 solution of the isothermal grey slab"}
    if with_cpu:
        try:
            cpu = cpu_reference_c0(g["T"], g["T_wall"])
            out["cpu_baseline"] = cpu
            out["same_config"] = True
            out["speedup_vs_cpu_same_tables"] = cpu["value"] / tb["ms"]
        except Exception as ex:  # the baseline must not take the GPU number down
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {ex}"}
    return out


def run_reference(args):
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return 0
    if args.workload == "grey64":
        g = c0_inputs()
        vals = [cpu_reference_c0(g["T"], g["T_wall"], budget_s=max(4.0, 40.0 / (args.warmup + args.steps)))
                for _ in range(args.warmup + args.steps)][args.warmup:]
        v = float(np.mean([c["value"] for c in vals]))
        out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": "grey channel 64^3, the reference's grey-band tables, extrapolated from a "
                                      "sample", "parallelism": "host threads"},
               "cpu_baseline": dict(vals[-1], value=v), "rays_per_s": vals[-1]["rays_per_s"],
               "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return 0
    from dnsmc_gb300 import synth
    T, x, Tw = make_inputs(0)
    table = synth.ck_table()
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        info = cpu_reference(table, T, x, Tw, None, budget_s=max(4.0, 60.0 / (args.warmup + args.steps)))
        if i >= args.warmup:
            vals.append(info["ms_field"])
    v = float(np.mean(vals))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "ck channel 128^3, 64 bands x 16 g x 50 T x 8 x_H2O, extrapolated from a sample",
                      "parallelism": "host threads"},
           "cpu_baseline": {"value": v, "unit": "ms", "cores": info["cores"], "kind": "port", "sample": info["sample"]},
           "rays_per_s": info["rays_s"],
           "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.workload == "ck128":
        # the grey 64^3 channel on the reference's own grey tables: the
        # configuration the reference covers completely
        g = c0_inputs()
        c0 = cpu_reference_c0(g["T"], g["T_wall"])
        out["c0"] = {"workload": "grey channel 64^3, the reference's grey-band tables", "ms_at_1pct": c0["value"],
                     "cpu_baseline": c0}
    print(json.dumps(out), flush=True)
    return 0


def get_network(table, log):
    """The control-variate network: the committed one for this grid if present,
    else trained here (untimed) on 16 snapshots the Monte Carlo produces."""
    from dnsmc_gb300 import CvNet, cvtrain
    path = os.path.join(ROOT, "dnsmc_gb300", "nets", f"ck{N_CELL}_g{GROUPS}.cvnet")
    if os.path.exists(path):
        try:
            return CvNet.load(path), {"source": os.path.relpath(path, ROOT)}
        except Exception as ex:  # a file of another network layout: train instead
            log(f"network file not usable ({ex}); training")
    net, info = cvtrain.train(table, N_CELL, range(1000, 1016), rays=64, epochs=3, j_slab=min(32, N_CELL), log=log,
                              groups=GROUPS)
    info = {k: v for k, v in info.items() if k != "loss"}
    info["source"] = "trained in this run before the timed region (16 snapshots, seeds 1000-1015)"
    return net, info


class Arm:
    """One estimator: plain MC, the profile control variate (beta = (1, -1),
    uniform rays) or the network control variate (coefficients and rays per
    (band group, packet) from the network, re-evaluated every step)."""

    def __init__(self, method, table, T, x, Tw, seed, threads, net=None):
        self.method, self.net = method, net
        self.s = make_solver(table, Tw, seed=seed, threads=threads, cv=0 if method == "plain" else 1)
        # Q and sigma rounded to float on the device: 8 bytes per cell reach
        # the host, like the reference's real(4) result arrays
        self.s.set_result_type(_result_f32())
        self.s.set_fields(T, x)
        self.rays = 0

    def enqueue(self):
        if self.method == "net":
            self.net.apply(self.s, beta=True, rays=True, mean_rays=self.rays, min_rays=2 * REPLICATES,
                           max_rays=4096)
        else:
            self.s.set_rays(self.rays)
        self.s.solve_async()

    def solve(self, rays=None):
        if rays is not None:
            self.rays = rays
        self.enqueue()
        self.s.wait(600)
        return self.results()

    def results(self, out=None):
        Q, S = self.s.results_float(out)
        return Q, S

    def budget(self, pilot=64, rays=0):
        """Rays per cell per group (uniform, or the mean of the network's
        allocation) for 1 % RMS: pilot solve, 1/N scaling, refined once."""
        if rays:
            self.rays = -(-rays // REPLICATES) * REPLICATES
            return None
        Q, S = self.solve(pilot)
        e = rms_error(Q, S)
        r = int(math.ceil(pilot * (e / TARGET_ERR) ** 2))
        r = max(2 * REPLICATES, min(1 << 17, -(-r // REPLICATES) * REPLICATES))
        Q, S = self.solve(r)
        e1 = rms_error(Q, S)
        if e1 > 0.98 * TARGET_ERR:
            r = -(-int(math.ceil(r * (e1 / (0.98 * TARGET_ERR)) ** 2)) // REPLICATES) * REPLICATES
        self.rays = r
        return e

    def timed(self, steps, warmup, flushbuf):
        import torch
        stream = torch.cuda.ExternalStream(self.s.stream())
        for _ in range(max(3, warmup)):
            self.solve()
        out = dict(ms=[], march_ms=[], steps=0.0, warp_steps=0.0, rays=0.0, errs=[], launches=0)
        torch.cuda.synchronize()
        for _ in range(steps):
            flush_l2(flushbuf)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            n0 = _launches()
            e0.record(stream)
            self.enqueue()
            e1.record(stream)
            self.s.wait(600)
            e1.synchronize()
            out["launches"] += _launches() - n0  # this library's kernels in the timed region
            Q, S = self.results()
            out["ms"].append(e0.elapsed_time(e1))
            out["march_ms"].append(self.s.timing()[1])
            c = self.s.counters()
            out["steps"] += c.steps
            out["rays"] += c.rays
            out["warp_steps"] += float(self.s.item_steps().sum())
            out["errs"].append(rms_error(Q, S))
        out["Q"], out["S"] = Q, S
        ta, tb = self.s.packet_shape()
        out["packet_cells"] = ta * tb  # cells of a packet: one warp marches them together
        return out

    def e2e(self, T, x, steps):
        """Wall clock of steps through the public API from host arrays; the
        results land in persistent arrays, as in a DNS that keeps its Q_r
        field from step to step."""
        ms = []
        Q, S = self.results()  # the persistent result arrays (touched once)
        for _ in range(steps):
            t0 = time.perf_counter()
            self.s.set_fields(T, x)
            self.enqueue()
            self.results(out=(Q, S))
            ms.append((time.perf_counter() - t0) * 1e3)
        return ms, Q, S

    def close(self):
        self.s.close()


def run_batched(args, flushbuf_mb=256):
    """The batched workload as the bench's JSON line (--workload batched)."""
    print(json.dumps(batched_block(args, flushbuf_mb)), flush=True)
    return 0


def batched_block(args, flushbuf_mb=256):
    """16 snapshots of 96^3 (seeds 0-15) in one solve: one persistent march
    launch over all snapshots, replayed from a CUDA graph, rays per packet
    proportional to local optical thickness (64-4096), launch shape and
    band-group size from the autotuner, the profile control variate."""
    import torch
    from dnsmc_gb300 import autotune, cvtrain, synth
    n, nsnap = 96, 16
    table = synth.ck_table()
    ds = [synth.ck_channel(n, q) for q in range(nsnap)]
    T = np.stack([d["T"] for d in ds])
    x = np.stack([d["x"] for d in ds])
    Tw = ds[0]["T_wall"]

    def make(bt, ta, ng):
        return cvtrain.ck_solver(table, n, Tw, seed=77, groups=ng, threads=bt, tile_a=ta, cv=True)

    # piloted at the ray floor: RQMC errors fall faster than 1/sqrt(rays), so
    # a pilot far below the target's ray count misjudges it, and at the floor
    # a decomposition whose packets would all sit there is measured as such
    tune = autotune.autotune(make, lambda sv: sv.set_fields(T, x), f"ck {nsnap}x{n}^3 cv", nbands=64,
                             rays=args.ray_floor, repeats=1, log=log, target_error=TARGET_ERR,
                             floor=args.ray_floor, error_fn=rms_error)
    cfg = tune["config"]
    s = make(cfg["block_threads"], cfg["tile_a"], cfg["n_groups"])
    s.set_graph(True)
    s.set_fields(T, x)
    floor = args.ray_floor
    per_tau = 400.0
    e = None
    for _ in range(4):  # rays_per_tau for 1 % RMS (the clamps make the error non-linear in it)
        s.set_rays_adaptive(per_tau, floor, 4096)
        Q, S = s.solve(timeout_s=900)
        e = rms_error(Q, S)
        if 0.9 * TARGET_ERR <= e <= 0.99 * TARGET_ERR:
            break
        per_tau *= (e / (0.97 * TARGET_ERR)) ** 2
    s.set_rays_adaptive(per_tau, floor, 4096)
    rp = s.rays_per_item()
    # the allocation: packets per ray-count bin (powers of two from the floor)
    edges = [floor]
    while edges[-1] < 4096:
        edges.append(edges[-1] * 2)
    counts, _ = np.histogram(rp, bins=edges + [1 << 30])
    hist = {f"{a}-{b - 1}" if b < (1 << 30) else f">={a}": int(c) for a, b, c in zip(edges, edges[1:] + [1 << 30],
                                                                                     counts)}
    stream = torch.cuda.ExternalStream(s.stream())
    flushbuf = torch.empty(flushbuf_mb * 256 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(max(3, args.warmup)):
        s.solve(timeout_s=900)
    ms, errs, steps, rays_tot, march = [], [], 0.0, 0.0, []
    launches = 0
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flushbuf)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            n0 = _launches()
            e0.record(stream)
            s.solve_async()
            e1.record(stream)
            s.wait(900)
            e1.synchronize()
            launches += _launches() - n0
            Q, S = s.results()
            ms.append(e0.elapsed_time(e1))
            march.append(s.timing()[1])
            c = s.counters()
            steps += c.steps
            rays_tot += c.rays
            errs.append(rms_error(Q, S))
    t = float(np.sum(ms))
    ms_field = t / (args.steps * nsnap)
    clocks = clk.summary()
    # the replayed graph's time brackets the whole sequence, so this
    # per-step issue rate is a lower bound for the march itself
    roof = issue_roofline(steps / args.steps, float(np.mean(march)), clocks)
    roof["note"] = ("instructions per lane-step of the 128^3 network-control-variate capture (the same march "
                    "kernel); time = the replayed graph")
    cap, glaunches = s.graph_info()
    out = {
        "metric": METRIC, "value": ms_field, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t / args.steps, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched: {nsnap} ck channel snapshots of {n}^3 (seeds 0-15) in one graph-replayed "
                               f"persistent launch, rays per packet ~ local optical thickness clamped to {floor}-4096, "
                               "profile control variate, RQMC rays",
                   "snapshots": nsnap, "n": n, "rays_per_tau": per_tau, "rays_floor": floor,
                   "rays_mean": float(rp.mean()), "rays_min": int(rp.min()), "rays_max": int(rp.max()),
                   "rays_histogram_packets": hist, "rays_at_floor": float((rp == floor).mean()), "autotuned": cfg,
                   "autotune_cached": tune["cached"], "target_rms_error": TARGET_ERR,
                   "rms_error_timed": float(np.mean(errs)), "graph_captures": cap, "graph_launches": glaunches,
                   "l2": "flushed before every timed step (256 MB device write)", "parallelism": "cells x1"},
        "autotune": tune["results"],
        "rays_per_s": rays_tot / (t / 1e3), "ray_steps_per_s": steps / (t / 1e3), "march_ms": float(np.mean(march)),
        "roofline": roof,
        "cpu_baseline": None,
        "e2e": None,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    s.close()
    return out


def run_c4(args):
    """Gas + scattering particles, 192^3: the correlated-k channel gas, particle
    volume fraction 1e-5 (1 + 0.5 f), smooth per-band particle optics (64 bands,
    albedo 0.3-0.9), Henyey-Greenstein g = 0.6, grey walls eps = 0.8; the
    profile control variate timed at its 1 % budget, plain MC extrapolated."""
    import torch
    from dnsmc_gb300 import cvtrain, synth
    n = args.n if args.n != 128 else 192
    table = synth.ck_table()
    d = synth.ck_channel(n, 0)
    fv = synth.particle_fraction(n, 0)
    pt = synth.particle_table(64)

    def solver(cv, seed):
        import dnsmc_gb300 as D
        cfg = D.default_config(model=D.MODEL_TABLE, imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                               stretched_x=0, T_west=d["T_wall"], T_east=d["T_wall"], eps_west=0.8, eps_east=0.8,
                               n_groups=GROUPS, seed=seed, block_threads=128, sampler=D.SAMPLER_RQMC,
                               local_sampling=1, nvar=REPLICATES, control_variate=cv)
        s = D.Solver(cfg)
        s.set_table(table["k"], table["wvc"], table["T0"], table["dT"], dnu=table["dnu"], wq=table["wq"],
                    X0=table["X0"], dX=table["dX"])
        s.set_fields(d["T"], d["x"])
        s.set_particles(pt["absorption"], pt["scattering"], pt["g"])
        s.set_particle_field(fv)
        return s

    s = solver(1, 41)
    if args.rays:  # fixed rays (profiling cases): no 1 % budget
        r, e = args.rays, None
        s.set_rays(r)
    else:
        r, e = ray_budget(s, 32)
        s.set_rays(r)
        Q, S = s.solve(timeout_s=1800)
        e1 = rms_error(Q, S)
        if e1 > 0.98 * TARGET_ERR:
            r = -(-int(math.ceil(r * (e1 / (0.98 * TARGET_ERR)) ** 2)) // REPLICATES) * REPLICATES
            s.set_rays(r)
    for _ in range(max(3, args.warmup)):
        s.solve(timeout_s=1800)
    stream = torch.cuda.ExternalStream(s.stream())
    flushbuf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ms, march, errs, steps, rays_tot = [], [], [], 0.0, 0.0
    launches = 0
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush_l2(flushbuf)
            e0 = torch.cuda.Event(enable_timing=True)
            e1_ = torch.cuda.Event(enable_timing=True)
            n0 = _launches()
            e0.record(stream)
            s.solve_async()
            e1_.record(stream)
            s.wait(1800)
            e1_.synchronize()
            launches += _launches() - n0
            Q, S = s.results()
            ms.append(e0.elapsed_time(e1_))
            march.append(s.timing()[1])
            c = s.counters()
            steps += c.steps
            rays_tot += c.rays
            errs.append(rms_error(Q, S))
    s.close()
    p = solver(0, 43)
    rp, ep = ray_budget(p, 32)
    p.set_rays(32)
    p.solve(timeout_s=1800)
    pilot_ms = p.timing()[0]
    p.close()
    value = float(np.mean(ms))
    clocks = clk.summary()
    roof = issue_roofline(steps / args.steps, float(np.mean(march)), clocks, bytes_per_step=36)
    # the general-medium march has its own instruction mix: no per-step
    # counters of it here, only its gather rate (36 B per step)
    for k_ in ("achieved", "frac", "traffic", "hbm_gbs", "hbm_frac", "l2_bytes", "l2_gbs", "source"):
        roof[k_] = None
    roof["note"] = "36 B per ray-voxel step (T, x_H2O, fv, bilinear k, linear Ib); issue-bound like the gas march"
    out = {
        "metric": METRIC, "value": value, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"gas + scattering particles {n}^3: ck channel gas, fv = 1e-5 (1 + 0.5 f), 64-band "
                               "particle optics (albedo 0.3-0.9), Henyey-Greenstein g = 0.6, grey walls eps = 0.8, "
                               "profile control variate, RQMC rays",
                   "n": n, "rays_per_cell_per_group": r, "target_rms_error": TARGET_ERR,
                   "rms_error_pilot": e, "rms_error_timed": float(np.mean(errs)),
                   "l2": "flushed before every timed step (256 MB device write)", "parallelism": "cells x1"},
        "comparison": {"plain_mc": {"rays_per_cell_per_group": rp, "rms_error_at_pilot": ep, "pilot_rays": 32,
                                    "pilot_solve_ms": pilot_ms, "ms_at_1pct_extrapolated": pilot_ms * rp / 32}},
        "rays_per_s": rays_tot / (np.sum(ms) / 1e3), "ray_steps_per_s": steps / (np.sum(ms) / 1e3),
        "march_ms": float(np.mean(march)),
        "roofline": roof,
        "cpu_baseline": None, "e2e": None, "gpu_launches": launches, "clocks": clocks,
    }
    print(json.dumps(out), flush=True)
    return 0


# Per lane-step figures of the two-cell march at the bench configuration
# (128^3 correlated-k channel, network control variate, 1 % budget), from
# the committed ncu capture: warp instructions issued, L2 bytes, DRAM bytes.
MARCH_PROFILE = os.path.join(ROOT, "profiles", "march_pair_kernel_ck128_counters.md")
ISSUE_PEAK = 4.0  # warp instructions per SM cycle: four schedulers, one issue each


def march_counters():
    """The `bench-constants:` line of the march profile, as floats, or None."""
    try:
        with open(MARCH_PROFILE) as fh:
            for line in fh:
                if line.startswith("bench-constants:"):
                    return {k: float(v) for k, v in (kv.split("=") for kv in line.split(":", 1)[1].split())}
    except (OSError, ValueError):
        pass
    return None


def issue_roofline(lane_steps, march_ms, clocks, bytes_per_step=BYTES_PER_STEP):
    """The march's bound: instruction issue.  achieved = warp instructions
    per SM cycle = (instructions per lane-step from the ncu capture x the
    lane-steps this launch counted) / (march time x median SM clock sampled
    during the timed region x SMs); peak = 4.  Beside it the algorithmic
    gather rate and the DRAM traffic (ncu per lane-step x lane-steps) against
    the measured HBM copy bandwidth."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    hbm, hbm_kind = peaks()
    c = march_counters()
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    sec = march_ms / 1e3
    out = {"bound": "issue", "achieved": None, "peak": ISSUE_PEAK, "unit": "warp instructions per SM cycle",
           "frac": None, "traffic": None, "peak_kind": "architectural (4 schedulers x 1 issue per cycle)",
           "gather_bytes": bytes_per_step * lane_steps, "gather_gbs": bytes_per_step * lane_steps / sec / 1e9,
           "lane_steps": lane_steps, "sms": sms, "sm_mhz": mhz}
    if c and mhz:
        inst = c["warp_inst_per_lane_step"] * lane_steps
        out["achieved"] = inst / (sec * mhz * 1e6 * sms)
        out["frac"] = out["achieved"] / ISSUE_PEAK
        out["traffic"] = c["dram_bytes_per_lane_step"] * lane_steps
        out["hbm_gbs"] = out["traffic"] / sec / 1e9
        out["hbm_frac"] = out["hbm_gbs"] / hbm
        out["hbm_peak_gbs"], out["hbm_peak_kind"] = hbm, hbm_kind
        out["l2_bytes"] = c["l2_bytes_per_lane_step"] * lane_steps
        out["l2_gbs"] = out["l2_bytes"] / sec / 1e9
        out["source"] = os.path.relpath(MARCH_PROFILE, ROOT)
    return out


def fp64_validation(table, T, x, Tw, Q, S, rays_timed, threads=0):
    """The timed field's error against the oracle's FP64 solution: the
    packet scheme in float64 with its own layer-mean control variate and
    exact means (oracle.fp64_cv_solution), 64 x the timed mean rays per cell
    and group in 8 RQMC replicates, independent seed, on every 4th
    wall-normal layer of the 8 x 8 column j, k < 8 (32 packets, 2048 cells).
    The error is sqrt(mean (Q - Q*)^2 - mean var(Q*)) / rms(Q*), the
    oracle's own variance removed in quadrature."""
    import dnsmc_gb300 as D
    from oracle import oracle as O
    n = N_CELL
    rays = 64 * int(rays_timed)
    rays = -(-rays // 8) * 8
    cfg = D.default_config(model=D.MODEL_TABLE, imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                           stretched_x=0, T_west=Tw, T_east=Tw, n_groups=GROUPS, seed=9001,
                           sampler=D.SAMPLER_RQMC, local_sampling=1, nvar=8, control_variate=0)
    m = D.Solver(cfg)  # host-only mirror: geometry, packets and sampling tables, no GPU work
    m.set_table(table["k"], table["wvc"], table["T0"], table["dT"], dnu=table["dnu"], wq=table["wq"],
                X0=table["X0"], dX=table["dX"])
    m.set_region(0, n, 0, 8, 0, 8)
    m.prepare_sampling(float(max(T.max(), Tw)), float(x.mean()))
    m.set_rays(8)
    t0 = time.perf_counter()
    Qo, Vo = O.fp64_cv_solution(m, table["dnu"], table["wq"], T[None], x[None], rays=rays, nbatch=8, seed=9001,
                                threads=threads or (os.cpu_count() or 1), layer_step=4)
    dt = time.perf_counter() - t0
    m.close()
    Qo, Vo = Qo[0][..., ::4], Vo[0][..., ::4]
    Qg = np.asarray(Q[0], np.float64)[:8, :8, ::4]
    Sg = np.asarray(S[0], np.float64)[:8, :8, ::4]
    qrms = math.sqrt(float((Qo ** 2).mean()))
    d2 = float(((Qg - Qo) ** 2).mean())
    return {"reference": "FP64 oracle: float64 packet scheme with its own layer-mean control variate and exact "
                         f"means, {rays} RQMC rays per cell and group (64 x the timed mean), 8 replicates, "
                         "independent seed",
            "cells": int(Qo.size), "sample": "every 4th wall-normal layer of the 8 x 8 column j, k < 8",
            "reference_rms_error": math.sqrt(float(Vo.mean())) / qrms,
            "rms_error_vs_fp64": math.sqrt(max(0.0, d2 - float(Vo.mean()))) / qrms,
            "rms_error_vs_fp64_raw": math.sqrt(d2) / qrms,
            "rms_error_estimated": math.sqrt(float((Sg ** 2).mean())) / qrms,
            "cpu_seconds": dt}


def run_grey64(args):
    """The grey 64^3 channel as the headline workload: ms per field at 1 %
    RMS of plain MC, with the CPU reference on the same channel and tables."""
    import torch
    flushbuf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    n0 = _launches()
    with ClockSampler(0) as clk:
        c0 = run_c0(args.steps, args.warmup, flushbuf, with_cpu=not args.no_cpu)
    g = c0["gpu_grey"]
    out = {"metric": METRIC, "value": g["ms_at_1pct"], "unit": "ms", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": g["ms_at_1pct"], "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": c0["workload"], "rays_per_cell": g["rays_per_cell"], "target_rms_error": TARGET_ERR,
                      "l2": "flushed before every timed step (256 MB device write)", "parallelism": "cells x1"},
           "rays_per_s": g["rays_per_s"], "c0": c0, "cpu_baseline": c0.get("cpu_baseline"), "e2e": None,
           "gpu_launches": _launches() - n0, "clocks": clk.summary()}
    print(json.dumps(out), flush=True)
    return 0


def main():
    global N_CELL, GROUPS, REPLICATES
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--n", type=int, default=128, help="cells per axis (profiling cases)")
    ap.add_argument("--rays", type=int, default=0, help="fixed rays per cell per group (skips the 1%% budget)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--method", default="net", choices=["net", "cv", "plain"],
                    help="timed estimator: network control variate (default), profile control variate, plain MC")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the profile-CV and extrapolated plain-MC comparison arms")
    ap.add_argument("--workload", default="ck128", choices=["ck128", "grey64", "batched", "particles"],
                    help="ck128: the 128^3 correlated-k channel (default); grey64: the grey 64^3 channel and "
                         "the isothermal slab; batched: 16 snapshots of 96^3; particles: gas + scattering "
                         "particles with grey walls, 192^3")
    ap.add_argument("--no-c0", action="store_true", help="skip the grey 64^3 block of the default workload")
    ap.add_argument("--no-c2", action="store_true", help="skip the batched 16 x 96^3 block of the default workload")
    ap.add_argument("--ray-floor", type=int, default=64,
                    help="batched workload: smallest rays per packet of the optical-thickness allocation (64 as "
                         "the configuration names; lower floors let the allocation vary)")
    ap.add_argument("--groups", type=int, default=GROUPS, help="band groups (stratification) of the solves")
    ap.add_argument("--no-validate", action="store_true",
                    help="skip the check of the timed field against an independent high-ray solution")
    ap.add_argument("--replicates", type=int, default=REPLICATES, help="RQMC replicates per (cell, band group)")
    args = ap.parse_args()
    N_CELL = args.n
    GROUPS = args.groups
    REPLICATES = args.replicates
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in ("batched", "particles", "grey64"):
        import torch
        torch.cuda.set_device(0)
        if args.workload == "grey64":
            return run_grey64(args)
        return run_batched(args) if args.workload == "batched" else run_c4(args)

    world, rank, local, pg = dist_setup(args)
    import torch
    torch.cuda.set_device(local)
    from dnsmc_gb300 import synth
    table = synth.ck_table()
    T, x, Tw = make_inputs(rank)
    net, net_info = (None, None)
    if args.method == "net":
        net, net_info = get_network(table, log)
    arm = Arm(args.method, table, T, x, Tw, 1000 + rank, args.threads, net)
    e_pilot = arm.budget(64, args.rays)
    arm.rays = int(barrier_max(pg, arm.rays))
    flushbuf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    # ---- device-resident timed region --------------------------------------
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        r = arm.timed(args.steps, args.warmup, flushbuf)
    torch.cuda.synchronize()
    t_rank = float(np.sum(r["ms"]))
    t_max = barrier_max(pg, t_rank)
    fields = args.steps * world
    ms_field = t_max / fields
    rays_s = r["rays"] * world / (t_max / 1e3)
    march_avg = float(np.mean(r["march_ms"]))
    steps_per_launch = r["steps"] / args.steps
    clocks = clk.summary()
    roof = issue_roofline(steps_per_launch, march_avg, clocks)
    # ---- end to end through the public API from host arrays ------------------
    e2e_ms, Qh, Sh = ([], r["Q"], r["S"]) if args.no_e2e else arm.e2e(T, x, args.steps)
    e2e_rank = float(np.sum(e2e_ms)) if e2e_ms else 0.0
    e2e_max = barrier_max(pg, e2e_rank) / fields if e2e_ms else None
    h2d = T.nbytes + x.nbytes
    d2h = Qh.nbytes + Sh.nbytes
    alloc = None
    if args.method == "net":
        rp = arm.s.rays_per_item()
        alloc = {"mean": float(rp.mean()), "min": int(rp.min()), "max": int(rp.max()),
                 "per_group_mean": [float(v) for v in rp.mean(1)]}
    arm.close()
    if rank != 0:
        if pg is not None:
            pg.destroy_process_group()
        return 0
    # ---- the timed field's actual error against independent solutions --------
    validation = None
    if not args.no_validate:
        validation = fp64_validation(table, T, x, Tw, r["Q"], r["S"], arm.rays)
        # and against a GPU solution of the whole field at many more rays
        v = Arm("cv", table, T, x, Tw, 5000 + rank, args.threads)
        Qref, Sref = v.solve(-(-1024 // REPLICATES) * REPLICATES)
        v.close()
        qrms = math.sqrt(float((np.asarray(Qref, np.float64) ** 2).mean()))
        d2 = float(((np.asarray(r["Q"], np.float64) - Qref) ** 2).mean()) - float(
            (np.asarray(Sref, np.float64) ** 2).mean())
        validation["whole_field_gpu"] = {
            "reference": "profile control variate on the GPU, 1024 rays per cell and group, independent seed",
            "reference_rms_error": rms_error(Qref, Sref),
            "rms_error_vs_reference": math.sqrt(max(0.0, d2)) / qrms,
            "rms_error_estimated": rms_error(r["Q"], r["S"])}
    c0 = None
    if not args.no_c0 and world == 1:
        c0 = run_c0(max(3, args.steps // 2), args.warmup, flushbuf, with_cpu=not args.no_cpu)
    c2 = None
    if not args.no_c2 and world == 1:
        b = batched_block(args)
        c2 = {k: b[k] for k in ("value", "unit", "steps", "warmup", "ms_per_step", "march_ms", "rays_per_s",
                                "gpu_launches", "clocks")}
        c2["config"] = {k: v for k, v in b["config"].items() if k != "l2"}
        c2["roofline"] = {k: b["roofline"].get(k) for k in ("bound", "achieved", "peak", "frac", "unit")}
    compare = {}
    if not args.no_compare and not args.rays:
        if args.method != "cv":
            c = Arm("cv", table, T, x, Tw, 3000 + rank, args.threads)
            c.budget(64)
            rc = c.timed(1, 1, flushbuf)
            compare["cv_profile"] = {"rays_per_cell_per_group": c.rays, "ms_at_1pct": float(rc["ms"][0]),
                                     "rms_error": rc["errs"][0]}
            c.close()
        if args.method != "plain":
            compare["plain_mc"] = plain_extrapolated(table, T, x, Tw, seed=2000 + rank)
    cpu = None
    if not args.no_cpu:
        try:
            info = cpu_reference(table, T, x, Tw, arm.rays)
            cpu = {"value": info["ms_field"], "unit": "ms", "cores": info["cores"], "kind": "port",
                   "sample": info["sample"], "rays_per_s": info["rays_s"]}
        except Exception as ex:  # the baseline must not take the GPU number down
            cpu = {"value": None, "unit": "ms", "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {ex}"}
    desc = {"plain": "plain MC",
            "cv": "control variate: the same ray through the plane-averaged profile, exact 1-D mean added back "
                  "(beta = (1, -1), uniform rays)",
            "net": "network control variate: the same ray through the plane-averaged profile, exact 1-D mean added "
                   "back, coefficients (beta_a, beta_b) per cell and band group and rays per (band group, packet) "
                   "from the BF16 MLP evaluated every step"}[args.method]
    out = {
        "metric": METRIC, "value": ms_field, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_field, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ck channel 128^3 (x,z periodic 2pi x pi, y walls black 400 K), T 400-1800 K + 5% "
                               "Fourier, x_H2O 0.1+0.05f, k table 64 bands x 16 g x 50 T x 8 x, 8 band groups, "
                               + desc + f", RQMC rays ({REPLICATES} shifted Sobol' replicates), spectral sampling at "
                                        "the packet temperature",
                   "method": args.method, "n": N_CELL,
                   "rays_per_cell_per_group": arm.rays, "rays_per_cell": arm.rays * GROUPS,
                   "target_rms_error": TARGET_ERR, "rms_error_pilot": e_pilot,
                   "rms_error_timed": float(np.mean(r["errs"])),
                   "l2": "flushed before every timed step (256 MB device write)", "parallelism": f"cells x{world}",
                   "network": net_info, "ray_allocation": alloc},
        "comparison": compare,
        "validation": validation,
        "rays_per_s": rays_s, "ray_steps_per_s": r["steps"] * world / (t_max / 1e3),
        "march_ms": march_avg, "step_ms": float(np.mean(r["ms"])), "march_lane_steps": steps_per_launch,
        "lane_efficiency": r["steps"] / (r["packet_cells"] * r["warp_steps"]) if r["warp_steps"] else None,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_max, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "timing": "wall clock around set_fields + (network) + solve + get_results_float (Q and sigma "
                          "rounded to float on the device)"},
        "gpu_launches": int(r["launches"]),
        "clocks": clocks,
        "c0": c0,
        "c2": c2,
    }
    print(json.dumps(out), flush=True)
    if net is not None:
        net.close()
    if pg is not None:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
