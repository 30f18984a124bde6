"""Benchmark: split-field FDTD on the curvilinear strip-waveguide bend.

Workload (the configuration the headline metric is quoted on): a silicon strip
90-degree bend (R = 2 um, core 0.45 x 0.22 um, eps 12.11 in 2.085) in
orthogonal curvilinear coordinates, 256 x 192 x 160 cells with nonuniform
metric factors (15-25 nm), 12-cell split PML on all faces; a batch of 8
excitations (2 ports x 4 guided modes, TE0/TM0/TE1/TM1 sheets); Gaussian pulse
source; FP64-accumulated running DFT at 21 wavelengths (1.50-1.60 um) on both
port planes.  Seeded synthetic structure (no dataset).

One bench "step" = one Yee step (the reference main_calc) of every excitation
of the batch.  Reported:
  value      FP32 batched Gcell-updates/s, device-resident, K timed steps
  e2e        the same metric through the C ABI from host buffers: plan creation
             (host precompute + uploads), incident sheets, schedule, a full
             8000-step run and the DFT read-back, per simulated step
  fp64       the plain FP64 (bit-identical to the reference) kernel: Gcell/s
  s_cols     S-matrix columns per second of full 8000-step runs, FP32 batched
             and FP64 plain, and the max relative S-parameter error FP32 vs FP64
  roofline   achieved HBM GB/s of the dominant kernel (the fused FP32 step, or
             the sweeps) from algorithmic bytes / CUDA-event launch time, against
             MEASURED_PEAKS.json: per cell-update the 6 field components read and
             written, the 6 per-cell coefficients and the aux slots of split cells
             (87.6 B on this workload); beside it the compulsory traffic of the
             batch, which reads the coefficient stream once for all excitations
  cpu_baseline  the CPU oracle (a restatement of the reference main_calc) on a
             bounded sample of the same workload on this host's cores

`--impl reference` times the reference CPU implementation instead (the
oracle; all host cores as independent processes, one excitation each).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s & S-cols/s: batched FP32 vs plain FP64 on 1 GB300 at stated error"
LAMS = list(np.linspace(1.50, 1.60, 21))
FULL_STEPS = 8000
BATCH = 8
N_MODES = 4
WORKLOAD = ("bend 256x192x160 curvilinear (R=2um, Si strip in SiO2), 12-cell split PML on 6 faces, "
            "batch 8 = 2 ports x 4 port eigenmodes (GPU mode solver), Gaussian pulse, "
            "FP64 DFT at 21 wavelengths on 2 port planes")


# DRAM traffic per update launch on the bench workload (dram__bytes_read.sum +
# dram__bytes_write.sum from one ncu capture of the full-size workload, a
# one-pass metric set; the summaries are kept with the other ncu summaries),
# keyed by (kernel, tile_y, z_chunk) of the launch configuration
TRAFFIC_PER_LAUNCH = {
    (2, 1, 0): 1.95e9 + 0.977e9,              # k_sweep32v, H or E sweep
    (6, 5, 32): 2.594e9 + 2.008e9,            # k_row32, one fused step
    (6, 5, 24): 2.619e9 + 2.007e9,
    (6, 5, 20): 2.617e9 + 2.007e9,
    (6, 4, 32): 2.582e9 + 2.008e9,
    (6, 5, 0): 2.567e9 + 2.010e9,             # k_row32, persistent CTAs
    (6, 2, 0): 2.766e9 + 2.016e9,
}


def launches_per_step(tuning, L2):
    """Update-kernel launches of one step: one fused launch (kernel 6), or an
    H and an E sweep per z-chunk (kernels 0, 2; z_chunk 0 = one chunk)."""
    if tuning[0] == 6:
        return 1
    zc = tuning[2]
    return 2 * (1 if zc <= 0 or zc >= L2 else math.ceil(L2 / zc))


def algorithmic_bytes_per_step(n3, n_split, batch, s_f=4, coef_bytes=24):
    """Algorithmic bytes of one step, per cell-update: every field component
    read and written (12*s_f), the per-cell coefficients (6 on a metric mesh,
    coef_bytes), the aux slot of a split cell read and written (12*s_f, for the
    N_split/N share of cells); sigma tables and DFT samples excluded.  Times N
    cells and the batch's excitations."""
    return batch * (n3 * (12 * s_f + coef_bytes) + n_split * 12 * s_f)


def compulsory_bytes_per_step(n3, n_split, batch, s_f=4, coef_bytes=24):
    """The same with the coefficient stream read once per step for the whole
    batch (the excitations of a plan share it): the least traffic a step of
    the batch can move."""
    return n3 * (12 * s_f * batch + coef_bytes) + n_split * 12 * s_f * batch


class Clocks:
    """nvidia-smi sampling in the background during the timed regions."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def make_workload(shape=(256, 192, 160), solve_modes=True):
    """The bend, its precompute and its port modes: the first N_MODES
    eigenmodes of the port layer from the GPU mode solver (forward sheets
    for the bottom-port excitations, backward ones for the top port, and the
    dual columns S is projected on).  solve_modes=False gives Gaussian
    stand-in sheets instead (used where only the step time matters)."""
    from smatranem_gb300 import workloads as W
    bend = W.bend_structure(shape=shape)
    pr = W.prepare(bend.s, dt_factor=1.0 / 0.99)
    if solve_modes:
        ms = W.port_modes(bend, N_MODES)
        k = ms.n_found
        modes = {"fwd": [ms.incident(m) for m in range(1, k + 1)],
                 "bwd": [ms.incident(-m) for m in range(1, k + 1)],
                 "cols": np.array([ms.dual(m) for m in range(1, k + 1)] + [ms.dual(-m) for m in range(1, k + 1)]),
                 "theta": ms.theta[:k].real.tolist(), "solver": ms.info}
    else:
        sheets = W.mode_profiles(bend, n_modes=N_MODES)
        modes = {"fwd": sheets, "bwd": sheets, "cols": mode_columns(sheets), "theta": None, "solver": None}
    return bend, pr, modes


def excitations(bend, modes):
    """(port plane, inci_mode sign, Hinc, Einc) for 2 ports x 4 modes: forward
    modes launched at the bottom port, backward ones at the top port (the
    reference picks the backward Xi column for a negative inci_mode,
    set_incident :497-499)."""
    out = []
    for plane, sign, key in ((bend.iI, 1, "fwd"), (bend.iT - 2, -1, "bwd")):
        for Hinc, Einc in modes[key]:
            out.append((plane, sign, Hinc, Einc))
    return out


def make_plan(bend, pr, modes, precision, batch, nsteps, stream=None, tuning="auto"):
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    s = bend.s
    p = F.Plan.create(s.L, s.iBc, (bend.iB, bend.iT, bend.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi,
                      pr.sigma, precision=precision, batch=batch, stream=stream)
    if tuning == "auto":
        p.autotune(4)
    elif tuning is not None:
        p.set_tuning(*tuning)
    ex = excitations(bend, modes)
    for b in range(batch):
        plane, sign, Hinc, Einc = ex[b % len(ex)]
        p.set_incident(b, Hinc, Einc)
        p.set_source_plane(b, plane, sign)
    src, ph = W.pulse_schedule(nsteps, pr.dt, lams_um=LAMS)
    p.set_schedule(src, planes=(bend.iB, bend.iT), phase=ph)
    return p


def mode_columns(modes):
    """Overlap columns (4*npix rows: Hx, Hy, -Ey, Ex) of stand-in mode sheets."""
    cols = []
    for Hinc, Einc in modes:
        cols.append(np.concatenate([Hinc[0::2], Hinc[1::2], -Einc[1::2], Einc[0::2]]))
    return np.array(cols)


S_FLOOR = 1e-3


def s_parameter_errors(S32, S64, floor=S_FLOOR):
    """Per excitation, over all its S parameters (2 port planes x 21
    wavelengths x 8 mode columns): the largest |S32 - S64| / max(|S64|,
    floor * m) with m the excitation's largest |S64| (relative error, entries
    under the floor judged against floor * m), the largest relative error of
    the entries at or above the floor, and the largest |S32 - S64| / m."""
    floored, rel_above, abs_over = [], [], []
    below = 0
    for a, r in zip(S32, S64):
        m = float(np.abs(r).max())
        d = np.abs(a - r)
        big = np.abs(r) >= floor * m
        floored.append(float(np.max(d / np.maximum(np.abs(r), floor * m))))
        rel_above.append(float(np.max(d[big] / np.abs(r)[big])))
        abs_over.append(float(d.max() / m))
        below += int((~big).sum())
    return {"per_excitation_max_rel": floored, "max_rel": max(floored),
            "per_excitation_max_rel_above_floor": rel_above,
            "per_excitation_max_abs_over_max": abs_over, "max_abs_over_max": max(abs_over),
            "floor": f"{floor:g} x the excitation's largest |S|", "entries_below_floor": below,
            "entries": int(sum(r.size for r in S64)),
            "over": "every excitation: 2 port planes x 21 wavelengths x 8 mode columns (4 port modes, forward and "
                    "backward dual columns); FP64 side: the plain FP64 plan (bit-identical to the reference loop) "
                    "on the same batch"}


def dft_fields(p, b):
    """The running DFT of excitation b: [wavelength][port plane][Hx, Hy, Ex, Ey][pixel]."""
    nf, nq = p.dft_count()
    return np.array([[p.get_dft(b, fi, q) for q in range(nq)] for fi in range(nf)])


def s_parameters(p, bend, modes, b):
    """Mode overlaps on the GPU (FP64): [port plane][lambda][mode column]."""
    return np.stack([p.overlap(b, q, modes["cols"]) for q in range(2)])


# ---------------------------------------------------------------------------
# CPU baseline (oracle) -- bounded samples
# ---------------------------------------------------------------------------

def _cpu_worker(shape, warmup, nsteps, kind, idx, barrier, queue):
    """One process: `warmup` untimed then `nsteps` timed main_calc steps of the
    full bend, one excitation, on the CPU oracle.  Loads only the oracle's
    libraries: the structure is numpy (workloads' generators), the
    precompute is the oracle port's (oracle.prepare), the sheet is a Gaussian
    stand-in (the update rate does not depend on the sheet)."""
    try:
        import oracle
        from smatranem_gb300 import workloads as W
        bend = W.bend_structure(shape=shape)
        s = bend.s
        pr = oracle.prepare(s.L, s.mu, s.epsi, s.omega, s.min_dt, dt_factor=1.0 / 0.99)
        bend.s = s = dataclasses.replace(s, mu=None, epsi=None)  # the media are no longer needed
        o = oracle.Oracle(kind)
        n3 = s.L[0] * s.L[1] * s.L[2]
        pl = s.L[0] * s.L[1]
        H = np.zeros(3 * (n3 + pr["lnotn"] + 1))
        E = np.zeros_like(H)
        Hinc, Einc = W.mode_profiles(bend, n_modes=N_MODES)[idx % N_MODES]
        rng = np.random.default_rng(idx)
        H[:3 * n3] = rng.standard_normal(3 * n3) * 1e-3
        mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
        args = (s.L, pr["Ah"], pr["Bh"], pr["Ae"], pr["Be"], s.iBc, H, E, (bend.iB, bend.iT, bend.iI, 1), Hinc, Einc,
                pr["n2pi"], (1, 1, 3))
        o.time_loop(*args, 0, warmup, *mons, pr["cont"], pr["addr"])
        barrier.wait(timeout=1800)
        t0 = time.perf_counter()
        o.time_loop(*args, warmup, warmup + nsteps, *mons, pr["cont"], pr["addr"])
        queue.put((idx, time.perf_counter() - t0, n3, pr["lnotn"], None))
    except Exception as e:  # reported by the parent
        barrier.abort()
        queue.put((idx, None, None, None, repr(e)))


def cpu_rate(nproc, shape, warmup, nsteps, kind):
    """nproc independent oracle processes (spawned, no CUDA in any of them),
    their timed regions started together behind a barrier.  Returns
    (cell-updates/s over all processes, the slowest process's timed seconds,
    cells, split cells)."""
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nproc)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_cpu_worker, args=(shape, warmup, nsteps, kind, i, barrier, queue))
             for i in range(nproc)]
    for pr in procs:
        pr.start()
    res = []
    try:
        while len(res) < nproc:
            try:
                res.append(queue.get(timeout=5))
            except Exception:
                dead = [pr.exitcode for pr in procs if pr.exitcode not in (None, 0)]
                if dead:
                    raise RuntimeError(f"CPU oracle worker died (exit {dead[0]})")
    finally:
        for pr in procs:
            pr.join(timeout=60)
            if pr.is_alive():
                pr.kill()
    bad = [r[4] for r in res if r[4]]
    if bad:
        raise RuntimeError("CPU oracle worker failed: " + bad[0])
    tmax = max(r[1] for r in res)
    n3, lnotn = res[0][2], res[0][3]
    return nproc * n3 * nsteps / tmax, tmax, n3, lnotn


def oracle_kind():
    import oracle
    oracle.build()
    if oracle.reference_available():
        try:
            oracle.Oracle("reference")
            return "reference"
        except OSError:
            pass
    return "port"


# ---------------------------------------------------------------------------
# runs
# ---------------------------------------------------------------------------

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    return ws, rank, local


def dist_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def bench_config(n3, n_split, batch, ws):
    """The `config` of the contract line (the same for both arms)."""
    return {"workload": WORKLOAD, "cells": n3, "split_cells": n_split, "batch": batch,
            "l2": "inputs larger than L2 (fields of %d excitations: %.1f GB)" % (batch, batch * 4 * 3 * n3 * 4 / 1e9),
            "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU"}


def run_reference(args):
    """The reference arm: the reference's CPU implementation of the step (the
    oracle: the reference compiled from its own source where it was built
    here, else the restatement) on every host core, as independent
    single-threaded processes (the reference has no threads; S columns are
    independent), each stepping one excitation of the full bend: --warmup
    untimed steps, then exactly --steps timed steps, started together.  No
    process loads the CUDA library."""
    ws, rank, local = dist_setup()
    if rank != 0:
        return
    kind = oracle_kind()
    nproc = os.cpu_count() or 1
    shape = (256, 192, 160)
    t_all = time.perf_counter()
    rate, tmax, n3, lnotn = cpu_rate(nproc, shape, args.warmup, args.steps, kind)
    g = rate / 1e9
    sample = (f"{nproc} independent single-threaded processes, one excitation of the full bend each (Gaussian "
              f"stand-in sheet), {args.warmup} untimed + {args.steps} timed main_calc steps each, timed regions "
              f"started together; slowest process {tmax:.2f} s")
    line = {"impl": "reference", "metric": METRIC, "value": g, "unit": "Gcell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tmax / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(n3, lnotn, args.batch, args.gpus),
            "cpu_baseline": {"value": g, "unit": "Gcell-updates/s", "cores": nproc, "kind": kind,
                             "sample": sample},
            "e2e": {"value": g, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0, "wall_s": time.perf_counter() - t_all}
    print(json.dumps(line))


def run_ours(args):
    ws, rank, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    from smatranem_gb300 import fdtd as F
    clocks = Clocks(local)
    bend, pr, modes = make_workload()
    n3 = bend.s.n3
    n_split = pr.lnotn
    batch = args.batch
    stream = torch.cuda.Stream()
    # ---- FP32 batched, device resident: the headline value --------------
    tun = tuple(int(x) for x in args.tuning.split(",")) if args.tuning else "auto"
    p32 = make_plan(bend, pr, modes, F.FP32, batch, FULL_STEPS, stream=stream.cuda_stream, tuning=tun)
    p32.run(0, args.warmup)
    dist_barrier(ws)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    p32.run(args.warmup, args.warmup + args.steps, sync=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_ms = dist_max(ev0.elapsed_time(ev1), ws)
    dist_barrier(ws)
    value = ws * batch * n3 * args.steps / (t_ms * 1e-3) / 1e9
    ms_step = t_ms / args.steps
    # per-kernel launch times for the roofline (same stream, CUDA events)
    kt = p32.time_kernels(args.warmup + args.steps, 64)
    tuning = p32.get_tuning()
    per_step = launches_per_step(tuning, bend.s.L[2])
    bytes_step = algorithmic_bytes_per_step(n3, n_split, batch)
    comp_step = compulsory_bytes_per_step(n3, n_split, batch)
    step_kernel_ms = kt[0] + kt[1]  # the update kernels of one step (DFT flush apart)
    launch_ms = step_kernel_ms / per_step
    achieved = bytes_step / (step_kernel_ms * 1e-3) / 1e9
    achieved_comp = comp_step / (step_kernel_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    launches = per_step * args.steps + 2 * math.ceil(args.steps / 32) + 1
    # ---- full runs: S-matrix columns/s and the FP32-vs-FP64 errors --------
    full = args.full_steps
    p32b = make_plan(bend, pr, modes, F.FP32, batch, full, stream=stream.cuda_stream, tuning=tuning)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p32b.run(0, full)
    t_full32 = time.perf_counter() - t0
    S32 = [s_parameters(p32b, bend, modes, b) for b in range(batch)]
    D32 = [dft_fields(p32b, b) for b in range(batch)]
    finite32 = p32b.check_finite()[0]
    p32b.close()
    p32.close()
    # the plain FP64 kernel (bit-identical to the reference loop) on the same
    # batch of excitations: its S-cols/s and the FP64 side of every error
    p64 = make_plan(bend, pr, modes, F.FP64, batch, full, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0.record(stream)
    p64.run(0, full, sync=False)
    ev1.record(stream)
    p64.sync()
    t_full64 = time.perf_counter() - t0
    t64_ms = ev0.elapsed_time(ev1)
    fp64_rate = batch * n3 * full / (t64_ms * 1e-3) / 1e9
    S64 = [s_parameters(p64, bend, modes, b) for b in range(batch)]
    d_l2, d_max = [], []
    for b in range(batch):
        D64 = dft_fields(p64, b)
        dd = (D32[b] - D64).reshape(D64.shape[0], D64.shape[1], -1)
        dr = D64.reshape(dd.shape)
        d_l2.append(float(np.max(np.linalg.norm(dd, axis=2) / np.linalg.norm(dr, axis=2))))
        d_max.append(float(np.max(np.abs(dd).max(axis=2) / np.abs(dr).max(axis=2))))
    p64.close()
    del D32
    clocks.stop()
    s_err = s_parameter_errors(S32, S64)
    # ---- e2e through the C ABI from host buffers --------------------------
    # plan creation from host arrays (precompute, uploads), the tuning (the
    # autotuner's cached pick for this grid, batch and GPU), sheets, schedule,
    # the full run and every excitation's S parameters read back
    t0 = time.perf_counter()
    pe = make_plan(bend, pr, modes, F.FP32, batch, full, tuning="auto")
    pe.run(0, full)
    Se = [s_parameters(pe, bend, modes, b) for b in range(batch)]
    h2d, d2h = pe.copy_bytes()
    pe.close()
    t_e2e = time.perf_counter() - t0
    e2e = ws * batch * n3 * full / t_e2e / 1e9
    del Se
    # ---- CPU baseline (bounded sample, oracle) -----------------------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        kind = oracle_kind()
        rate, tmax, _, _ = cpu_rate(1, (256, 192, 160), 1, args.cpu_steps, kind)
        cpu = {"value": rate / 1e9, "unit": "Gcell-updates/s", "cores": 1, "kind": kind,
               "sample": f"{args.cpu_steps} main_calc steps of the full bend after 1 untimed, one excitation, "
                         f"{tmax:.1f} s on 1 core"}
    # ---- the other workloads, bounded: one summary each ---------------------
    extras = {}
    if rank == 0 and args.extras:
        t_start = time.perf_counter()
        todo = [x for x in args.extras.split(",") if x]
        # (key, estimated seconds, call)
        runs = {"cube": ("config_cube_96_fp64", 20, lambda: config_cube(4000, args.warmup)),
                "adjoint": ("config_adjoint_160x160x120", 70, lambda: config_adjoint(6000, args.extra_fd_cells)),
                "group": ("config_group_bend8_slabs16", 120,
                          lambda: config_group(args.warmup, 40, 0, 300, bend_workload=(bend, pr, modes))),
                "large": ("config_large_640x640x512", 150, lambda: config_large(args.warmup, 20, 300)),
                "scalc": ("config_scalc_grating32x32", 40, lambda: config_scalc(32, 32, 10, 2, "both", True))}
        for name in todo:
            key, est, fn = runs[name]
            left = args.extras_budget - (time.perf_counter() - t_start)
            if left < est:
                extras[key] = {"skipped": f"time budget: {left:.0f} s left of --extras-budget {args.extras_budget} s, "
                                          f"about {est} s needed"}
                continue
            t0 = time.perf_counter()
            extras[key] = dict(fn(), wall_s=time.perf_counter() - t0)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(n3, n_split, batch, ws),
        "e2e": {"value": e2e, "unit": "Gcell-updates/s", "h2d_bytes_per_step": h2d / full,
                "d2h_bytes_per_step": d2h / full,
                "what": f"through the C ABI from host arrays: plan creation (precompute + uploads), the autotuner's "
                        f"cached tuning, sheets, schedule, {full} steps, S of all {batch} excitations read back; "
                        f"{t_e2e:.2f} s; copies counted by the library (smat_fdtd_copy_bytes)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": TRAFFIC_PER_LAUNCH.get(tuple(tuning[:3])) if batch == BATCH else None,
                     "traffic_per": "launch (ncu, dram read + write)",
                     "kernel": {2: "k_sweep32v (H, E; float4)" + (f", z-chunks of {tuning[2]} planes"
                                                                   if 0 < tuning[2] < bend.s.L[2] else ""),
                                6: f"k_row32 (one fused H+E launch per step: z-march of {tuning[1]} whole x rows"
                                   f" per CTA, float4 quads)",
                                0: "k_sweep32 (H, E)"}[tuning[0]],
                     "tuning": {"kernel": tuning[0], "tile_y": tuning[1], "z_chunk": tuning[2],
                                "ctas_per_sm": tuning[3], "slots": tuning[4]},
                     "bytes_per_launch": bytes_step / per_step,
                     "bytes_per_cell_update": bytes_step / (n3 * batch),
                     "compulsory": {"bytes_per_launch": comp_step / per_step, "achieved": achieved_comp,
                                    "frac": achieved_comp / peak,
                                    "what": "coefficient stream read once per step for all excitations"},
                     "ms_per_launch": launch_ms,
                     "launches_per_step": per_step, "ms_per_step_kernels": step_kernel_ms,
                     "ms_dft_flush_per_step": kt[2]},
        "fp64_plain": {"value": fp64_rate, "unit": "Gcell-updates/s", "steps": full, "batch": batch,
                       "s_cols_per_s": batch / t_full64, "full_run_s": t_full64},
        "fp32_batched": {"s_cols_per_s": batch / t_full32, "full_run_s": t_full32, "full_steps": full,
                         "finite": finite32},
        "s_cols_speedup_fp32_vs_fp64": (batch / t_full32) / (batch / t_full64),
        "s_param_rel_err_fp32_vs_fp64": s_err,
        "dft_field_rel_err_fp32_vs_fp64": {
            "per_excitation_max_rel_l2": d_l2, "max_rel_l2": max(d_l2),
            "per_excitation_max_abs_over_max": d_max, "max_abs_over_max": max(d_max),
            "over": "per excitation: Hx, Hy, Ex, Ey on both port planes, relative L2 (and largest deviation over "
                    "the slice's largest value) of each (wavelength, plane) slice, the worst of the 21 x 2 slices; "
                    "FP64 side: the plain FP64 plan (bit-identical to the reference loop) on the same batch"},
        "port_modes": {"theta": modes["theta"], "solver": modes["solver"]},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    line.update(extras)
    print(json.dumps(line))


def run_profile(args):
    """A small case for ncu: the bend cross-section with fewer z-layers (inputs
    still larger than L2), `--warmup` + `--steps` steps of the chosen precision."""
    import torch
    from smatranem_gb300 import fdtd as F
    shape = tuple(int(x) for x in args.shape.split(","))
    bend, pr, modes = make_workload(shape)
    prec = F.FP32 if args.profile == "fp32" else F.FP64
    tuning = tuple(int(x) for x in args.tuning.split(",")) if args.tuning else "auto"
    p = make_plan(bend, pr, modes, prec, args.batch if prec == F.FP32 else 1, args.warmup + args.steps,
                  tuning=tuning)
    p.run(0, args.warmup)
    p.run(args.warmup, args.warmup + args.steps)
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "shape": shape, "batch": p.batch, "steps": args.steps,
                      "tuning": p.get_tuning(), "device_bytes": p.device_bytes}))
    p.close()


# ---------------------------------------------------------------------------
# the other configurations, one JSON summary line each (not the contract line)
# ---------------------------------------------------------------------------

def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def config_adjoint(nsteps=6000, fd_cells=32, K=64):
    """Adjoint gradient workload: 160x160x120 cells, a 60x60x20 design region of
    seeded eps_r in [2.085, 12.11] between two strip-waveguide ports, objective
    |overlap of the output-port DFT at 1.55 um with TE0|^2, FP32 with a
    checkpoint every K steps, through the torch.autograd wrapper.  Checked
    against central differences (delta eps_r = 1e-3) of the FP64 forward --
    bit-identical to the reference loop -- on fd_cells seeded cells, and against
    the FP64 adjoint over the whole design box."""
    import torch
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    from smatranem_gb300.autograd import PortOverlap, objective_and_grad
    d = W.design_structure(shape=(160, 160, 120), design=(60, 60, 20), pml=12, seed=0)
    pr = W.prepare(d.s, dt_factor=1.0 / 0.99)
    src, ph = W.pulse_schedule(nsteps, pr.dt, lams_um=[1.55])
    mode = W.mode_profiles(d, n_modes=1)[0]
    kw = dict(nsteps=nsteps, K=K, mode=mode, src=src, phase=ph)
    objective_and_grad(d, d.eps, precision=F.FP32, **dict(kw, nsteps=min(nsteps, 2 * K)))  # warm-up, tuning
    eps_t = torch.tensor(d.eps, dtype=torch.float64, requires_grad=True)

    def fp32():
        J = PortOverlap.apply(eps_t, d, dict(kw, precision=F.FP32))
        J.backward()
        return float(J.detach()), eps_t.grad.numpy().copy()
    (J32, g32), t32 = _timed(fp32)
    (J64, g64), t64 = _timed(lambda: objective_and_grad(d, d.eps, precision=F.FP64, **kw))
    rng = np.random.default_rng(7)
    flat = rng.choice(d.eps.size, size=fd_cells, replace=False)
    cells = [np.unravel_index(i, d.eps.shape) for i in flat]

    def objective(eps):
        s = d.with_eps(eps)
        prx = W.prepare(s, dt_factor=1.0 / 0.99)
        p = F.Plan.create(s.L, s.iBc, (d.iB, d.iT, d.iI, 1), prx.invtau_R, prx.invtau_I, prx.mu, prx.epsi,
                          prx.sigma, precision=F.FP64, batch=1)
        with p:
            p.set_incident(0, *mode)
            p.set_schedule(src, planes=(d.iB, d.iT), phase=ph)
            p.run(0, nsteps)
            return abs(W.overlap(p.get_dft(0, 0, 1), *mode)) ** 2

    t0 = time.perf_counter()
    fd = []
    for c in cells:
        e = d.eps.copy()
        e[c] += 1e-3
        jp = objective(e)
        e[c] -= 2e-3
        fd.append((jp - objective(e)) / 2e-3)
    t_fd = time.perf_counter() - t0
    fd = np.array(fd)
    a32 = np.array([g32[c] for c in cells])
    a64 = np.array([g64[c] for c in cells])
    fs = float(np.max(np.abs(fd))) if len(cells) else float("nan")
    cells_total = d.s.n3 * nsteps
    nan = float("nan")
    return {
        "config": "design 160x160x120, 60x60x20 design cells (eps_r ~ U[2.085, 12.11], seed 0), 12-cell split PML "
                  "on 6 faces, TE0 output-port overlap at 1.55 um, Gaussian pulse, FP32, checkpoints every "
                  f"{K} steps, through the torch.autograd wrapper",
        "steps": nsteps, "checkpoint_every": K, "J_fp32": J32, "J_fp64": J64,
        "gradient_fp32_s": t32, "gradient_fp64_s": t64,
        "gradient_fp32_gcell_per_s": 3 * cells_total / t32 / 1e9,
        "gcell_what": "forward + recompute + adjoint cell-updates (3 x cells x steps) per second",
        "design_cells": int(d.eps.size), "fd_cells": int(fd_cells), "fd_s": t_fd,
        "err_fp32_adjoint_vs_fd": float(np.max(np.abs(a32 - fd)) / fs) if len(cells) else nan,
        "err_fp64_adjoint_vs_fd": float(np.max(np.abs(a64 - fd)) / fs) if len(cells) else nan,
        "err_fp32_vs_fp64_adjoint_whole_box": float(np.max(np.abs(g32 - g64)) / np.max(np.abs(g64))),
        "errors_are": "max |g - g_fd| / max |g_fd| over the FD cells (central differences, delta eps_r = 1e-3, of "
                      "the FP64 forward); whole box: max |g32 - g64| / max |g64|",
    }


def run_adjoint(args):
    print(json.dumps(dict({"mode": "adjoint"}, **config_adjoint(args.adj_steps, args.fd_cells))))


def _slab_plan(sl, prec, nsteps, lams=LAMS):
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    prs = W.prepare(sl.s, dt_factor=1.0 / 0.99)
    p = F.Plan.create(sl.s.L, sl.s.iBc, (sl.iB, sl.iT, sl.iI, 1), prs.invtau_R, prs.invtau_I, prs.mu,
                      prs.epsi, prs.sigma, precision=prec, batch=1)
    p.set_incident(0, *W.mode_profiles(sl, n_modes=1)[0])
    src, ph = W.pulse_schedule(nsteps, prs.dt, lams_um=lams)
    p.set_schedule(src, planes=(sl.iB, sl.iT), phase=ph)
    return p, prs


def _rel_l2_slices(a, b):
    """Largest relative L2 error over the (wavelength, plane) slices of DFT
    arrays [nfreq][nplanes][4][pl]."""
    d = (a - b).reshape(a.shape[0], a.shape[1], -1)
    r = b.reshape(d.shape)
    return float(np.max(np.linalg.norm(d, axis=2) / np.linalg.norm(r, axis=2)))


def config_group(warmup=5, steps=40, seed=0, acc_steps=300, bend_workload=None, autotune=False):
    """Batched S-matrix workload: the bend with its 8 excitations plus 16 slabs
    of uneven size (128^3 .. 256x256x192, 1-6 random cuboid inclusions each,
    one excitation each), FP32, 21-wavelength FP64 DFT on 2 planes each, all
    advanced by one group: by default in one persistent fused launch per step
    for every member (form 3; autotune=True lets the group autotuner choose
    among its forms).  Roofline on the group's compulsory bytes (every
    member's fields and aux slots read and written, its coefficient stream
    read once).  Accuracy: a fresh one-launch group run for acc_steps steps of
    the pulse against the FP64 plan of every member (the bend: all 8
    excitations, DFT and S)."""
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    bend, pr, modes = bend_workload or make_workload()
    nsteps = warmup + steps
    shapes = W.slab_shapes(16, seed=seed)
    slabs = [W.slab_structure(shp, seed=100 + i) for i, shp in enumerate(shapes)]

    def members(n):
        ps = [make_plan(bend, pr, modes, F.FP32, BATCH, n, tuning=None)]
        splits = [pr.lnotn]
        for sl in slabs:
            p, prs = _slab_plan(sl, F.FP32, n)
            ps.append(p)
            splits.append(prs.lnotn)
        return ps, splits
    plans, splits = members(nsteps)
    cells = bend.s.n3 * BATCH + sum(sl.s.n3 for sl in slabs)
    comp = compulsory_bytes_per_step(bend.s.n3, pr.lnotn, BATCH) + sum(
        compulsory_bytes_per_step(sl.s.n3, sp, 1) for sl, sp in zip(slabs, splits[1:]))
    g = F.Group(plans)
    if autotune:
        (gmode, by), _ = g.autotune(4)
    else:
        gmode, by = 3, 1
        g.set_tuning(gmode, by)
    g.run(0, warmup)
    _, t = _timed(lambda: g.run(warmup, nsteps))
    device_gb = sum(p.device_bytes for p in plans) / 1e9
    g.close()
    for p in plans:
        p.close()
    peak, peak_kind = measured_peak()
    achieved = comp * steps / t / 1e9
    # accuracy: a fresh group of every member, FP32 against each member's FP64 plan
    plans, _ = members(acc_steps)
    g = F.Group(plans)
    g.set_tuning(gmode, by)
    g.run(0, acc_steps)
    g.close()
    d32 = [[dft_fields(plans[0], b) for b in range(BATCH)]] + [[dft_fields(p, 0)] for p in plans[1:]]
    s32 = [s_parameters(plans[0], bend, modes, b) for b in range(BATCH)]
    for p in plans:
        p.close()
    p64 = make_plan(bend, pr, modes, F.FP64, BATCH, acc_steps, tuning=None)
    p64.run(0, acc_steps)
    bend_err = [_rel_l2_slices(d32[0][b], dft_fields(p64, b)) for b in range(BATCH)]
    s64 = [s_parameters(p64, bend, modes, b) for b in range(BATCH)]
    p64.close()
    slab_err = []
    for sl, d in zip(slabs, d32[1:]):
        p, _ = _slab_plan(sl, F.FP64, acc_steps)
        p.run(0, acc_steps)
        slab_err.append(_rel_l2_slices(d[0], dft_fields(p, 0)))
        p.close()
    serr = s_parameter_errors(s32, s64)
    return {
        "config": "bend 256x192x160 x 8 excitations + 16 slabs 128^3..256x256x192 (1-6 seeded inclusions), FP32, "
                  "21-wavelength FP64 DFT on 2 planes each",
        "structures": 17, "cell_excitations": cells, "steps": steps,
        "form": ["one grouped launch per sweep", "members' own sweep launches in one graph",
                 "members' own autotuned launch forms in one graph",
                 "one persistent fused launch per step for every member"][gmode] + (
                     ", CTAs of 384 threads" if gmode == 3 and by == 1 else
                     ", CTAs of 192 threads" if gmode == 3 else ""),
        "gcell_per_s": cells * steps / t / 1e9, "ms_per_step": 1e3 * t / steps, "device_gb": device_gb,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "bytes_per_step": comp,
                     "what": "the group's compulsory bytes (fields and aux slots of every excitation read and "
                             "written, each member's coefficient stream once) per step / step time"},
        "fp32_vs_fp64": {"steps": acc_steps,
                         "bend_dft_max_rel_l2_per_excitation": bend_err,
                         "slab_dft_max_rel_l2": slab_err,
                         "bend_s_max_rel_per_excitation": serr["per_excitation_max_rel"],
                         "bend_s_max_abs_over_max_per_excitation": serr["per_excitation_max_abs_over_max"],
                         "s_floor": serr["floor"],
                         "over": "fresh group (same form) vs every member's FP64 plan: DFT relative L2 of the worst "
                                 "(wavelength, plane) slice; bend S over 2 planes x 21 wavelengths x 8 mode columns"},
    }


def run_group(args):
    print(json.dumps(dict({"mode": "group"}, **config_group(args.warmup, args.steps, args.group_seed,
                                                             autotune=args.group_form != 3))))


def _cube_cpu_worker(args):
    """One process: `nsteps` oracle main_calc steps of the 96^3 cube (precompute
    by the oracle port; no CUDA library in this process)."""
    nsteps, kind = args
    import oracle
    from smatranem_gb300 import workloads as W
    c = W.cube_structure()
    s = c.s
    pr = oracle.prepare(s.L, s.mu, s.epsi, s.omega, s.min_dt, dt_factor=1.0 / 0.99)
    o = oracle.Oracle(kind)
    Ah, Bh, Ae, Be = pr["Ah"], pr["Bh"], pr["Ae"], pr["Be"]
    cells = np.flatnonzero(s.pec)
    for k in range(3):  # the PEC plate
        Ae[3 * cells + k] = 0.0
        Be[3 * cells + k] = 0.0
    n3, pl = s.n3, s.L[0] * s.L[1]
    H = np.zeros(3 * (n3 + pr["lnotn"] + 1))
    E = np.zeros_like(H)
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    t0 = time.perf_counter()
    o.time_loop(s.L, Ah, Bh, Ae, Be, s.iBc, H, E, (c.iM, c.iM, c.iI, 1), *W.point_source(c), pr["n2pi"],
                (1, 1, 3), 0, nsteps, *mons, pr["cont"], pr["addr"])
    return time.perf_counter() - t0, n3 * nsteps


def config_cube(nsteps=4000, warmup=5, cpu_steps=0):
    """The plain FP64 benchmark case: 96^3 cells in vacuum, a centred 30^3
    block of eps 12.11, a 40x40 one-cell PEC plate 15 cells below it, 10-cell
    split PML on all faces (grading 3, R = 1e-6), an x point source driven by a
    Gaussian-modulated sine (1.55 um, 20 % bandwidth), nsteps steps at Courant
    0.99/sqrt(3), running DFT at 11 wavelengths on one plane.  FP64 (bit-
    identical to the reference loop) and FP32 (autotuned) on the GPU, timed
    with CUDA events over the steps after warmup; roofline of the FP64 step on
    145.4 B per cell-update (fields and aux slots read and written, a material
    index per cell); the CPU oracle on cpu_steps steps (0: none)."""
    import torch
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    c = W.cube_structure()
    pr = W.prepare(c.s, dt_factor=1.0 / 0.99)
    lams = [float(x) for x in np.linspace(1.55 * 0.9, 1.55 * 1.1, 11)]
    src, ph = W.pulse_schedule(nsteps, pr.dt, lam0_um=1.55, bandwidth=0.2, lams_um=lams)
    Hinc, Einc = W.point_source(c)
    res, dft = {}, {}
    n3, ns = c.s.n3, pr.lnotn
    peak, peak_kind = measured_peak()
    st = torch.cuda.Stream()
    for prec, name in ((F.FP64, "fp64"), (F.FP32, "fp32")):
        p = F.Plan.create(c.s.L, c.s.iBc, (c.iM, c.iM, c.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi,
                          pr.sigma, precision=prec, batch=1, pec=c.s.pec, stream=st.cuda_stream)
        tuning = list(p.autotune(4)[0]) if prec == F.FP32 else None
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src, planes=(c.iM,), phase=ph)
        p.run(0, warmup)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(st)
        p.run(warmup, nsteps, sync=False)
        ev1.record(st)
        torch.cuda.synchronize()
        t = ev0.elapsed_time(ev1) * 1e-3
        dft[name] = np.array([p.get_dft(0, fi, 0) for fi in range(len(lams))])
        res[name] = {"gcell_per_s": n3 * (nsteps - warmup) / t / 1e9, "ms_per_step": 1e3 * t / (nsteps - warmup),
                     "tuning": tuning}
        if prec == F.FP64:
            bpc = (n3 * (12 * 8 + 1) + ns * 12 * 8) / n3
            ach = bpc * n3 * (nsteps - warmup) / t / 1e9
            res[name]["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                                     "frac": ach / peak, "peak_kind": peak_kind, "bytes_per_cell_update": bpc,
                                     "note": "the FP64 state and coefficients (about 0.2 GB) stay largely in "
                                             "the 126 MB L2 between steps"}
        p.close()
    rel = np.abs(dft["fp32"] - dft["fp64"]).reshape(len(lams), -1)
    err = float(np.max(np.linalg.norm(rel, axis=1) / np.linalg.norm(dft["fp64"].reshape(len(lams), -1), axis=1)))
    cpu = None
    if cpu_steps > 0:
        kind = oracle_kind()
        ctx = mp.get_context("spawn")
        with ctx.Pool(1) as pool:
            t_cpu, cells = pool.map(_cube_cpu_worker, [(cpu_steps, kind)])[0]
        cpu = {"value": cells / t_cpu / 1e9, "unit": "Gcell-updates/s", "cores": 1, "kind": kind,
               "sample": f"{cpu_steps} main_calc steps of the 96^3 cube, {t_cpu:.1f} s on 1 core"}
    return {
        "config": "96^3 vacuum, 30^3 block eps 12.11, 40x40 PEC plate 15 cells below, 10-cell split PML on 6 faces "
                  "(R = 1e-6, grading 3), x point source, Gaussian-modulated sine 1.55 um / 20 %, Courant "
                  "0.99/sqrt(3), DFT at 11 wavelengths on one plane",
        "cells": n3, "split_cells": ns, "pec_cells": int(c.s.pec.sum()), "steps": nsteps,
        "fp64": res["fp64"], "fp32": res["fp32"],
        "dft_rel_l2_fp32_vs_fp64": err,
        "dft_err_over": "per wavelength, relative L2 over the plane's Hx, Hy, Ex, Ey; the worst of 11",
        "fp64_bit_identical_to_reference": "tests/test_gpu_cube.py",
        "cpu_baseline": cpu,
    }


def run_cube(args):
    print(json.dumps(dict({"mode": "cube"}, **config_cube(args.cube_steps, args.warmup,
                                                           0 if args.no_cpu else args.cpu_steps))))


def config_large(warmup=5, steps=20, check_steps=600):
    """Large-domain throughput: 640x640x512 cells (~210M) in FP32, split PML,
    gently curved substrate (radius 50 um), PEC patch-array grating, DFT at 5
    wavelengths on 2 planes; the autotuner's launch form timed over `steps`
    steps; roofline on the algorithmic bytes (fields and aux slots read and
    written, 6 coefficients per cell); fresh FP32 and FP64 plans after
    check_steps pulse steps compared (0: no check)."""
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    t0 = time.perf_counter()
    st = W.large_structure()
    pr = W.prepare(st.s, dt_factor=1.0 / 0.99)
    nsteps = warmup + steps
    lams = list(np.linspace(1.50, 1.60, 5))
    sheets = W.mode_profiles(st, n_modes=1)[0]

    def plan(prec, n):
        q = F.Plan.create(st.s.L, st.s.iBc, (st.iB, st.iT, st.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi,
                          pr.sigma, precision=prec, batch=1, pec=st.s.pec)
        q.set_incident(0, *sheets)
        src, ph = W.pulse_schedule(n, pr.dt, lams_um=lams)
        q.set_schedule(src, planes=(st.iB, st.iT), phase=ph)
        return q

    p = plan(F.FP32, nsteps)
    t_setup = time.perf_counter() - t0
    best, _ = p.autotune(2)
    p.run(0, warmup)
    _, t = _timed(lambda: p.run(warmup, nsteps))
    ok, mx = p.check_finite()
    dev_gb = p.device_bytes / 1e9
    p.close()
    n3, ns = st.s.n3, pr.lnotn
    peak, peak_kind = measured_peak()
    bstep = algorithmic_bytes_per_step(n3, ns, 1)
    achieved = bstep * steps / t / 1e9
    check = None
    if check_steps > 0:
        n = check_steps
        d = {}
        for prec in (F.FP32, F.FP64):
            q = plan(prec, n)
            if prec == F.FP32:
                q.set_tuning(*best)
            q.run(0, n)
            d[prec] = dft_fields(q, 0)
            q.close()
        dd = (d[F.FP32] - d[F.FP64]).reshape(len(lams), 2, -1)
        rr = d[F.FP64].reshape(dd.shape)
        nd, nr = np.linalg.norm(dd, axis=2), np.linalg.norm(rr, axis=2)
        live = nr > 1e-9 * nr.max()  # a plane the pulse has not reached yet holds no field
        check = {"steps": n, "dft_max_rel_l2": float(np.max(nd[live] / nr[live])),
                 "slices": int(live.sum()), "of": int(live.size),
                 "over": "Hx, Hy, Ex, Ey on both planes x 5 wavelengths, per (wavelength, plane) slice holding "
                         "field"}
    return {
        "config": "640x640x512 FP32, 12-cell split PML, curved substrate R=50um, PEC patch array (16x16 patches, "
                  "period 40, 20x20x2 cells) over an eps 2.085 slab, DFT at 5 wavelengths (1.50-1.60 um) on 2 planes",
        "cells": n3, "split_cells": ns, "steps": steps, "tuning": list(best),
        "gcell_per_s": n3 * steps / t / 1e9, "ms_per_step": 1e3 * t / steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "bytes_per_cell_update": bstep / n3},
        "device_gb": dev_gb, "setup_s": t_setup, "finite": ok, "fp32_vs_fp64": check,
    }


def run_large(args):
    print(json.dumps(dict({"mode": "large"}, **config_large(args.warmup, args.steps, args.large_check_steps))))


def run_modes(args):
    """Port-mode solver (f)-3: the N_MODES propagating modes of the bend's
    256 x 192 port layer (n = 98,304 unknowns) on the GPU, timed over
    --steps solves after --warmup; the CPU side is the dense reference
    algorithm (oracle restatement of Mcalc's calc_Xi) on the largest
    cross-section it handles in seconds, scaled to the full size by n^3."""
    import torch
    from smatranem_gb300 import modes as M
    from smatranem_gb300 import workloads as W
    bend = W.bend_structure(shape=(256, 192, 64))
    L0, L1 = 256, 192
    for _ in range(max(1, args.warmup)):
        M.solve(bend.port_med, bend.s.omega, L0, L1, (0, 0), N_MODES)
    torch.cuda.synchronize()
    times, infos = [], []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        ms = M.solve(bend.port_med, bend.s.omega, L0, L1, (0, 0), N_MODES)
        times.append(time.perf_counter() - t0)
        infos.append(ms.info)
    cpu = None
    if not args.no_cpu:
        from oracle import mode_oracle as MO
        c0, c1 = 40, 30   # the same graded mesh around the core, cropped
        sub = W.bend_structure(shape=(c0, c1, 64), core_cell0=c0 // 2)
        V, _ = MO.set_V(sub.port_med, sub.s.omega)
        maa, mbb = MO.set_M((0, 0), c0, c1, V)
        A = (mbb @ maa).real
        t0 = time.perf_counter()
        MO.eigen(A, real=True)  # Mcalc's dominant step: dense dgeev of mbb*maa (Mcalc.c:884)
        t_cpu = time.perf_counter() - t0
        scale = (L0 * L1 / (c0 * c1)) ** 3
        cpu = {"value": t_cpu * scale, "unit": "s per solve (dense eigen solve, extrapolated as n^3)",
               "cores": os.cpu_count(), "kind": "port",
               "sample": f"dgeev of the {2 * c0 * c1}x{2 * c0 * c1} mbb*maa of a {c0}x{c1} crop of the same mesh: "
                         f"{t_cpu:.2f} s, x (n ratio)^3 = {scale:.3g}; the full {2 * L0 * L1}^2 matrix alone "
                         f"would take {(2 * L0 * L1) ** 2 * 8 / 1e9:.0f} GB"}
    print(json.dumps({
        "mode": "modes", "config": f"bend port layer {L0}x{L1} (graded 15-25 nm mesh), BoundC 0, {N_MODES} modes",
        "ms_per_solve": 1e3 * float(np.median(times)), "solves": len(times),
        "theta": ms.theta[:ms.n_found].real.tolist(), "info": infos[-1],
        "cpu_baseline": cpu}))


def config_scalc(L0=32, L1=32, nl=10, steps=2, dense="both", cpu=True):
    """Layer-transfer S matrix (Scalc, (f)-4) on the GPU: a periodic grating
    between uniform ports, L0 x L1 cells, nl layers (default 32x32, 10 layers:
    dense matrices of order NA = 2*L0*L1 = 2048, all propagating modes of the
    ports in S), both directions.  CPU side: the same dense steps (zgesv of
    B2^T with NA + N_real right-hand sides, the projection zgemm) through
    LAPACK / BLAS on the host cores, one of each timed at full size and
    multiplied by their counts."""
    import torch
    from smatranem_gb300 import scalc as SC
    from smatranem_gb300 import workloads as W
    om = 0.405
    t0 = time.perf_counter()
    theta, Xi, nr = W.plane_wave_basis(L0, L1, omega=om)
    meds = W.grating_layers(L0, L1, nl, seed=7)
    t_setup = time.perf_counter() - t0
    NA = 2 * L0 * L1
    res = {}
    modes = [(1, "tensor_cores"), (0, "fp64_kernel")]
    if dense != "both":
        modes = [m for m in modes if m[1].startswith(dense[:2])]
    for mode, name in modes:
        SC.dense_mode(mode)
        SC.smatrix(meds[:2], om, L0, L1, (1, 1), Xi, nr, Xi, nr)  # warm-up (allocations, module load)
        torch.cuda.synchronize()
        times = []
        for _ in range(max(1, steps)):
            t0 = time.perf_counter()
            S, info = SC.smatrix(meds, om, L0, L1, (1, 1), Xi, nr, Xi, nr)
            times.append(time.perf_counter() - t0)
        res[name] = (float(min(times)), S, info, len(times))
    SC.dense_mode(1)
    best, S, info, nruns = res["tensor_cores"] if "tensor_cores" in res else res["fp64_kernel"]
    best64, S64, info64, _ = res["fp64_kernel"] if "fp64_kernel" in res else (None, None, None, None)
    solves = info["solves"]
    # complex LU of order NA (8/3 NA^3 real flops), the solve with NA + N_real
    # right-hand sides (8 NA^2 per column), the elimination's zgemm, and the
    # two projections on the dual modes ((2NA)^2 x (NA + N_real))
    flops = solves * (8.0 / 3.0 * NA ** 3 + 8.0 * NA ** 2 * (NA + nr) + 8.0 * (NA + nr) * nr * NA) \
        + 2 * 8.0 * (2 * NA) ** 2 * (NA + nr)
    cpu_line = None
    if cpu:
        import scipy.linalg as sl
        rng = np.random.default_rng(0)
        A = rng.standard_normal((NA, NA)) + 1j * rng.standard_normal((NA, NA))
        B = rng.standard_normal((NA, NA + nr)) + 1j * rng.standard_normal((NA, NA + nr))
        t0 = time.perf_counter()
        sl.solve(A, B, check_finite=False)
        t_solve = time.perf_counter() - t0
        P = rng.standard_normal((2 * NA, 2 * NA)) + 1j * rng.standard_normal((2 * NA, 2 * NA))
        F = rng.standard_normal((2 * NA, NA + nr)) + 1j * rng.standard_normal((2 * NA, NA + nr))
        t0 = time.perf_counter()
        P.conj().T @ F
        t_mm = time.perf_counter() - t0
        est = solves * t_solve + 2 * t_mm
        cpu_line = {"value": est, "unit": "s per S matrix (LAPACK zgesv x solves + 2 projection zgemm)",
                    "cores": os.cpu_count(), "kind": "port",
                    "sample": f"one zgesv of order {NA} with {NA + nr} right-hand sides: {t_solve:.2f} s (x {solves}); "
                              f"one {2 * NA}^2 x {NA + nr} zgemm: {t_mm:.2f} s (x 2); threads of the host BLAS"}
    return {
        "config": f"periodic grating {L0}x{L1}, {nl} layers, uniform ports eps 2.085, "
                  f"NA = {NA}, N_real = {nr} per port, both directions",
        "s_per_smatrix": best, "runs": nruns, "solves": solves,
        "fp64_tflops": flops / best / 1e12,
        "products": "FP64-accurate complex products on the tensor cores (7 bf16 slices per operand, Ozaki scheme, "
                    "tcgen05.mma); LU panels and triangle blocks in FP64",
        "fp64_kernel": None if best64 is None else {"s_per_smatrix": best64, "fp64_tflops": flops / best64 / 1e12,
                                                    "speedup_tensor_cores": best64 / best},
        "s_max_abs_diff_vs_fp64_kernel": None if S64 is None else float(np.abs(S - S64).max()),
        "unitarity": info["unitarity"], "unitarity_fp64_kernel": None if info64 is None else info64["unitarity"],
        "transpose": info["transpose"], "setup_s": t_setup, "cpu_baseline": cpu_line}


def run_scalc(args):
    """--mode scalc: config_scalc's line; --shape L0,L1,nlayers (default 32,32,10)."""
    parts = [int(x) for x in args.shape.split(",")] if args.shape != "256,192,48" else [32, 32, 10]
    print(json.dumps(dict({"mode": "scalc"}, **config_scalc(parts[0], parts[1], parts[2], args.steps, args.dense,
                                                              not args.no_cpu))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", default="main", choices=["main", "adjoint", "group", "large", "modes", "scalc",
                                                       "cube"],
                    help="main: the contract line; the others: the adjoint, batched-structures and large-domain "
                         "workloads (one summary line each)")
    ap.add_argument("--adj-steps", type=int, default=6000)
    ap.add_argument("--cube-steps", type=int, default=4000)
    ap.add_argument("--fd-cells", type=int, default=32)
    ap.add_argument("--group-seed", type=int, default=0)
    ap.add_argument("--large-check-steps", type=int, default=600,
                    help="--mode large: steps of the FP32-vs-FP64 DFT check (0: none)")
    ap.add_argument("--group-form", type=int, default=-1, choices=[-1, 3],
                    help="--mode group: -1 = the group autotuner's pick, 3 = the one-launch form directly")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--full-steps", type=int, default=FULL_STEPS)
    ap.add_argument("--cpu-steps", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--dense", default="both", choices=["both", "tensor_cores", "fp64_kernel"],
                    help="--mode scalc: the dense products timed (tensor cores, the FP64 kernel, or both)")
    ap.add_argument("--extras", default="cube,adjoint,group,large,scalc",
                    help="main mode: the other workloads summarised in the contract line (comma list of cube, "
                         "adjoint, group, large, scalc; empty: none)")
    ap.add_argument("--extras-budget", type=float, default=420.0,
                    help="seconds the extras may take together; one that would not fit is reported as skipped")
    ap.add_argument("--extra-fd-cells", type=int, default=4,
                    help="finite-difference cells of the adjoint summary in the main mode (--mode adjoint: --fd-cells)")
    ap.add_argument("--profile", choices=["fp32", "fp64"], help="small case for ncu captures")
    ap.add_argument("--shape", default="256,192,48")
    ap.add_argument("--tuning", default="", help="kernel,tile_y,z_chunk,ctas_per_sm,slots (default: autotuned)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile:
        run_profile(args)
    elif args.mode != "main":
        {"adjoint": run_adjoint, "group": run_group, "large": run_large, "modes": run_modes,
         "scalc": run_scalc, "cube": run_cube}[args.mode](args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
