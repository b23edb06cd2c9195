#!/usr/bin/env python3
"""Throughput of the ATSAT dynamical core on GB300, in cell-steps per second.

One step is one iteration of the dycore part of cSaturnModel::Run on the reference's default grid
41x181x361 (planet/cSaturnModel.cpp:864-1111): on even iterations computeMixtureDensity and the
red-black pressure call (PressureSolver<cSaturnModel>::run), then RungeKuttaSat (four RHSSat stages
and the RK4 update), the boundary conditions and restoreVar -- all resident on the device
(atsat_dyn_iterate). Cells per step = im * jm * km.

  value   device-resident throughput, the state already in HBM (2.6 GB, far larger than L2, so no
          L2 flush is needed between iterations)
  e2e     the same metric through the C ABI with HOST buffers, as a drop-in driver calls it: every
          step uploads the step's inputs from pinned host memory, runs the pressure call (even
          steps) and the RK4 step, and downloads what the host reads back
  roofline  the fused RK stage kernel (the dominant kernel): algorithmic bytes per launch over its
          mean launch time from CUDA events in the timed region, against the measured HBM copy peak
  cpu_baseline  this repository's C restatement of the reference's OpenMP path, timed on the host
          cores on a bounded sample of the same workload (rank 0, N = 1)

--impl reference times the reference's CPU path (the C restatement with all host threads; the
reference's own build cannot travel to this machine) on the same workload and metric.
Multi-GPU runs are independent replicas (one per rank, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s, 1 GB300: mixed-prec vs FP64 GPU at ≤1e-6 rel err; %HBM peak"
UNIT = "Mcell-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", default="41,181,361")
    ap.add_argument("--e2e-steps", type=int, default=10, help="timed host-fed steps (0 skips the e2e loops)")
    ap.add_argument("--e2e-rows-steps", type=int, default=8,
                    help="steps of the e2e loop over ragged pageable rows (0 skips it)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--copy-engines", action="store_true",
                    help="move host bindings with the copy engines even where the SMs can address host memory")
    ap.add_argument("--stage-variant", default="auto",
                    choices=["auto", "direct", "tiled", "split", "split3", "split13", "split_tiled", "tiled2",
                             "march"],
                    help="mixed precision: the RK stage kernel (auto: the autotuner's choice)")
    ap.add_argument("--march-levels", type=int, default=0,
                    help="with --stage-variant march: radial levels per block (0: the library's default)")
    ap.add_argument("--poisson", action="store_true",
                    help="the standalone pressure-equation solves instead of the dycore iteration")
    ap.add_argument("--sor-sweeps", type=int, default=4000)
    ap.add_argument("--glue", action="store_true",
                    help="time the driver's glue (p_dyn filter, species floor, turbulence closure) per call and per iteration")
    ap.add_argument("--press-variants", action="store_true",
                    help="time one pressure call with and without PRESS_LINE / PRESS_BAROTROPIC")
    ap.add_argument("--ensemble", action="store_true",
                    help="the 32-member mixed-size ensemble: concurrent graph replays vs one after another")
    ap.add_argument("--cpu-table", action="store_true",
                    help="the CPU restatement's throughput per benchmark configuration, build and thread count")
    ap.add_argument("--precision", default="mixed,fp64",
                    help="comma list; the first is the headline value, the others are reported beside it")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    a.shape = tuple(int(x) for x in a.shape.split(","))
    a.precisions = [p.strip() for p in a.precision.split(",") if p.strip()]
    assert all(p in ("mixed", "fp64") for p in a.precisions), a.precisions
    return a


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        if vis:
            ids = vis.split(",")
            os.environ["CUDA_VISIBLE_DEVICES"] = ids[local % len(ids)]
        else:
            os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as td
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        td.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as td
        td.barrier()


def reduce_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as td
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons, kept for the timed region: the sampler starts
    ahead of it (nvidia-smi takes a moment to start) and samples every 50 ms with a timestamp; the samples
    between mark_start() and mark_stop() are the ones reported."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()

    @staticmethod
    def _when(stamp):
        import datetime
        try:
            return datetime.datetime.strptime(stamp.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10 or (vis.isdigit() and f[1] != vis):
                continue
            rows.append((self._when(f[0]), f))
        inside = [f for w, f in rows if w is not None and self.t0 is not None and self.t1 is not None
                  and self.t0 <= w <= self.t1]
        window = "timed region"
        if not inside:                    # no timestamped sample inside: every sample of the run
            inside = [f for _, f in rows]
            window = "whole measurement (none inside the timed region)"
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for f in inside:
            try:
                sm.append(float(f[2]))
                smax.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[6:10]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "window": window}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_launch(kernel: str):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def interior_rk(g):
    return (g.im - 2) * (g.jm - 4) * (g.km - 1)


# Bytes moved per interior-RK cell by the four stage launches of one RK4 step, as laid out here.
# FP64: stage 0 reads Y_s, y_n and the 21 auxiliary inputs (3 stencil, 18 point) and writes acc and Y_1;
# stages 1-2 also read acc; stage 3 writes y_{n+1}, rhs_u/v/w and aux_u/v/w instead of acc and Y.
RK_BYTES_FP64 = 8 * ((17 + 17 + 21 + 34) + 2 * (17 + 21 + 17 + 17 + 34) + (17 + 21 + 17 + 17 + 23))
# mixed: every stage reads the FP32 copy of y_n of all 17 fields and w's low word (72 B), the 9 frozen
# FP32 momentum terms (36 B) and the 17 point inputs read at the default knobs in FP32 (68 B); stages
# 1-3 read the FP32 stage increment (68 B); stages 0-2 write the next increment (68 B) and the running
# tke/dis sums (8 B, read back by stages 1-3); stage 3 reads dl_1 and dl_2 of the 15 unclamped fields
# (120 B) and y_n in FP64 (136 B) and writes y_{n+1} in FP64 (136 B) and FP32 (68 B + 4 B for w's low
# word), rhs_u/v/w and aux_u/v/w (48 B).
_MIX_IN = 72 + 36 + 68
RK_BYTES_MIXED = ((_MIX_IN + 68 + 8) + 2 * (_MIX_IN + 68 + 68 + 16)
                  + (_MIX_IN + 68 + 8 + 120 + 136 + 136 + 72 + 48))
RK_BYTES = {"fp64": RK_BYTES_FP64, "mixed": RK_BYTES_MIXED}
KERNEL_NAME = {"fp64": "rk_stage_fp64_kernel (fused RHSSat + RK4 stage, FP64)",
               "mixed": "rk_stage_mixed_kernel (fused RHSSat + RK4 stage, FP32 stencils / FP64 state)",
               "mixed_tiled": "rk_tile_kernel (TMA-tiled fused RHSSat + RK4 stage, FP32 stencils / FP64 state)",
               "mixed_split": "rk_mom_kernel + rk_tracer_kernel<1> (split RHSSat + RK4 stage, FP32 stencils / FP64 state)",
               "mixed_split3": "rk_mom_kernel + rk_tracer_kernel<3> (split RHSSat + RK4 stage, FP32 stencils / FP64 state)",
               "mixed_split13": "rk_mom_kernel + rk_tracer_kernel<13> (split RHSSat + RK4 stage, FP32 stencils / FP64 state)",
               "mixed_split_tiled": "rk_mom_kernel + rk_tracer_tile_kernel (split RHSSat + RK4 stage, TMA-tiled tracers; "
                                    "final stage + final_combine_kernel)",
               "mixed_tiled2": "rk_mom_tile_kernel + rk_tracer_tile_kernel (split RHSSat + RK4 stage, all inputs "
                               "TMA-streamed; final stage + final_combine_kernel)",
               "mixed_march": "rk_mom_march_kernel + rk_tracer_tile_kernel (split RHSSat + RK4 stage: the momentum "
                              "part as a radial march, one TMA plane per stencil array and level; final stage + "
                              "final_combine_kernel)"}


def cpu_baseline(g, P, seed, target_s=3.0):
    """The C restatement of the reference's OpenMP path on this host, all cores, bounded sample."""
    from atsat_gb300 import synth
    from oracle import oracle
    st = synth.saturn_state(g, P, seed=seed)
    oracle.lib()
    t0 = time.perf_counter()
    n = 0
    while n < 2 or (time.perf_counter() - t0 < target_s and n < 8):
        oracle.steps(st, P, 1, iter0=1 + n)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": n * g.cells / dt / 1e6, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"{n} dycore iterations at {g.im}x{g.jm}x{g.km} (pressure on the even ones), "
                      f"{dt:.2f} s wall on {os.cpu_count()} OpenMP threads"}


def cpu_baseline_child(shape, threads=None, build=""):
    """The same bounded sample in a child process: on one OpenMP thread (OpenMP fixes its thread count when
    the library loads), or with the restatement's fast build (-O3, multiply-add contraction allowed; a timed
    baseline only, never the parity oracle)."""
    code = ("import json, os, sys; sys.path.insert(0, %r); import bench; from atsat_gb300 import abi, synth; "
            "g = synth.make_grid(*%r); r = bench.cpu_baseline(g, abi.default_params(), seed=0, target_s=2.0); "
            "n = int(os.environ.get('OMP_NUM_THREADS') or os.cpu_count()); r['cores'] = n; "
            "r['sample'] = r['sample'].replace('%%d OpenMP threads' %% os.cpu_count(), '%%d OpenMP thread%%s' "
            "%% (n, '' if n == 1 else 's')); print(json.dumps(r))") % (ROOT, tuple(shape))
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    if build:
        env["ATSAT_ORACLE_BUILD"] = build
    try:
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
        r = json.loads(out.stdout.strip().splitlines()[-1])
    except (subprocess.SubprocessError, ValueError, IndexError, OSError):
        return None
    if build == "fast":
        r["build"] = "gcc -O3 -fopenmp -ffp-contract=fast (no -march/-mcpu: the same flags on x86-64 and Arm)"
    return r


def cpu_baseline_one_thread(shape):
    return cpu_baseline_child(shape, threads=1)


def run_reference(a, rank, world):
    if rank != 0:
        return None
    from atsat_gb300 import abi, synth
    from oracle import oracle
    g = synth.make_grid(*a.shape)
    P = abi.default_params()
    st = synth.saturn_state(g, P, seed=0)
    oracle.lib()
    for it in range(1, a.warmup + 1):
        oracle.steps(st, P, 1, iter0=it)
    t0 = time.perf_counter()
    oracle.steps(st, P, a.steps, iter0=a.warmup + 1)
    dt = time.perf_counter() - t0
    v = a.steps * g.cells / dt / 1e6
    return {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt * 1e3 / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(g, "fp64"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{a.steps} full dycore iterations after {a.warmup} warm-up"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def config(g, precision):
    return {"workload": f"ATSAT dycore iteration (RK4 step + red-black pressure call on even steps + "
                        f"boundary conditions + restoreVar) at {g.im}x{g.jm}x{g.km}",
            "grid": f"{g.im}x{g.jm}x{g.km}", "cells_per_step": g.cells, "interior_rk_cells": interior_rk(g),
            "precision": precision, "press_sweeps": 1, "l2": "state of 2.6 GB resident, larger than L2: no flush",
            "parallelism": "replicas"}


def omp_threads():
    """Threads the library's OpenMP host loops use (OMP_NUM_THREADS, else every core)."""
    v = os.environ.get("OMP_NUM_THREADS", "")
    return int(v) if v.isdigit() and int(v) > 0 else os.cpu_count()


def measure(a, rank, world, g, P, st, pinned, precision):
    """Resident throughput, e2e throughput and the stage kernel's roofline of one precision."""
    import numpy as np
    from atsat_gb300 import abi, dyn, fields as F
    d = dyn.Dycore(g, dict(P, precision=1 if precision == "mixed" else 0))
    if a.copy_engines and d.host_direct():
        d.set_host_direct(False)
    for fid in range(F.NFIELDS):
        pinned[fid].array[...] = 0.0 if st.arrays.get(fid) is None else st.arrays[fid]
        d.bind(fid, pinned[fid].array)
    d.upload(list(range(F.NFIELDS)))
    d.set_tables(st.cell_vbar0, st.cell_ubar0, st.p_baro)

    # ---- device-resident throughput ----
    clocks = Clocks()
    clocks.start()                        # ahead of the timed region: nvidia-smi needs a moment to start
    d.iterate(1, a.warmup)
    tune = None
    if precision == "mixed" and a.stage_variant == "auto":
        chosen, tms = d.autotune(reps=5)
        tune = {"stage_variant": dyn.Dycore.STAGE_NAMES[chosen], "march_levels": d.march_levels(),
                "autotune_ms_per_stage": {n: (t if t > 0 else None) for n, t in zip(dyn.Dycore.STAGE_NAMES, tms)}}
    elif precision == "mixed":
        d.set_stage_variant(dyn.Dycore.STAGE_NAMES.index(a.stage_variant))
        if a.stage_variant == "march" and a.march_levels > 0:
            d.set_march_levels(a.march_levels)
        tune = {"stage_variant": a.stage_variant, "march_levels": d.march_levels()}
    it0 = a.warmup + 1
    d.iterate(it0, 2)                     # untimed: a capture starts from two settled resident iterations
    it0 += 2
    # the headline timed region: the resident loop replayed as a CUDA graph of two iterations (the public
    # atsat_dyn_graph_capture / atsat_dyn_graph_launch path; replays are bit-identical to plain iterations,
    # the pressure call on the even one), plus one plain iteration when the step count is odd
    d.graph_capture(it0, 2)
    d.graph_launch(1)                     # untimed: the first replay uploads the graph
    d.sync()
    it0 += 2
    l0 = d.launches()
    barrier(world)
    clocks.mark_start()
    d.timer_start()
    d.graph_launch(a.steps // 2)
    if a.steps % 2:
        d.iterate(it0 + a.steps - 1, 1)
    ms = d.timer_stop()
    clocks.mark_stop()
    barrier(world)
    clk = clocks.stop()
    launches = d.launches() - l0
    ms = reduce_max(world, ms)
    value = world * a.steps * g.cells / (ms / 1e3) / 1e6
    it0 += a.steps
    # the roofline's kernel timed live: the same iterations launched one by one, with two event records
    # around every RK stage launch group (events cannot time single kernels inside a graph replay)
    d.profile_classes([abi.K_RK_STAGE])
    d.profile_reset()
    d.timer_start()
    d.iterate(it0, a.steps)
    ms_plain = reduce_max(world, d.timer_stop())
    n_rk, ms_rk = d.profile_read(abi.K_RK_STAGE)
    d.profile(False)
    it0 += a.steps
    # per-class breakdown: an even number of further iterations with every class profiled
    nb = max(2, min(a.steps, 20) // 2 * 2)
    d.profile(True)
    d.profile_reset()
    d.iterate(it0, nb)
    kern = {abi.K_NAMES[c]: dict(zip(("launches", "ms"), d.profile_read(c))) for c in range(len(abi.K_NAMES))}
    kern["iterations"] = nb
    d.profile(False)

    # ---- end to end through the C ABI with host buffers ----
    ins = F.STEP_INPUTS
    outs = F.STEP_OUTPUTS

    def xfer_path(d):
        return ("one kernel per upload / download reading and writing host memory in place over NVLink-C2C"
                if d.host_direct() else "copy engines through staging buffers")

    def e2e_step(it):
        """One drop-in step: upload the inputs, pressure call on even steps, RK4, download; bytes moved.
        The calls are queued in the handle's asynchronous mode; sync() ends the step with the outputs in the
        host arrays."""
        up, down = len(ins) * g.cells * 8, len(outs) * g.cells * 8
        d.upload(ins)
        if it % 2 == 0:
            d.computeMixtureDensity()
            d.PressureSolver_run(stats=False)
            d.download([F.P_DYN])
            down += g.cells * 8
        d.RungeKuttaSat()
        d.download(outs)
        d.sync()
        return up, down

    it = it0 + nb
    e2e = None
    d.set_async(True)
    if a.e2e_steps > 0:
        e2e_step(it)             # untimed: the first host-fed step leaves the resident (aliased) state
        it += 1
        h2d = d2h = 0
        barrier(world)
        t0 = time.perf_counter()
        for s in range(a.e2e_steps):
            up, down = e2e_step(it)
            h2d += up
            d2h += down
            it += 1
        e2e_s = reduce_max(world, time.perf_counter() - t0)
        e2e = {"value": world * a.e2e_steps * g.cells / e2e_s / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": h2d // a.e2e_steps, "d2h_bytes_per_step": d2h // a.e2e_steps,
               "steps": a.e2e_steps, "ms_per_step": e2e_s * 1e3 / a.e2e_steps,
               "binding": "contiguous pinned arrays (bind_host_array)", "path": xfer_path(d),
               "calls": "asynchronous mode, one atsat_dyn_sync per step"}

    # the same loop over the reference's own storage: one pageable row of km doubles per (i, j), as
    # lib/Array.cpp allocates it, bound through bind_host_rows (packed on the host into pinned staging)
    if e2e is not None and a.e2e_rows_steps > 0:
        keep = {}
        for fid in sorted(set(ins) | set(outs) | {F.P_DYN}):
            base = np.array(pinned[fid].array, copy=True)
            rows = [base[i, j] for i in range(g.im) for j in range(g.jm)]
            keep[fid] = base
            d.bind_rows(fid, rows)
        for _ in range(2):       # untimed: first device touches of the freshly allocated pageable rows
            e2e_step(it)
            it += 1
        barrier(world)
        t0 = time.perf_counter()
        for s in range(a.e2e_rows_steps):
            e2e_step(it)
            it += 1
        rows_s = reduce_max(world, time.perf_counter() - t0)
        e2e["rows"] = {"value": world * a.e2e_rows_steps * g.cells / rows_s / 1e6, "unit": UNIT,
                       "steps": a.e2e_rows_steps, "ms_per_step": rows_s * 1e3 / a.e2e_rows_steps,
                       "binding": "ragged pageable rows (bind_host_rows)", "path": xfer_path(d),
                       "host_threads": omp_threads()}
        del keep
    d.set_async(False)

    peak, peak_kind = peaks()
    bytes_per_launch = RK_BYTES[precision] / 4 * interior_rk(g)
    avg_ms = ms_rk / max(n_rk, 1)
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
    kname = KERNEL_NAME.get("mixed_" + tune["stage_variant"], KERNEL_NAME[precision]) if tune else KERNEL_NAME[precision]
    roof = {"kernel": kname, "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": traffic_per_launch("rk_stage_" + precision + ("_" + tune["stage_variant"] if tune else "")),
            "algorithmic_bytes_per_launch": bytes_per_launch,
            "launches": n_rk, "mean_launch_ms": avg_ms,
            "timed_region": f"{a.steps} iterations launched one by one after the graph-timed region "
                            f"({ms_plain / a.steps:.4f} ms per iteration there)"}
    if precision == "fp64":
        roof["note"] = "bound by GB300's FP64 pipe (2 DFMA per SM per cycle), not by HBM"
        # the FP64 roofline that binds: FP64 instructions per interior cell and stage counted by ncu
        # (profiles/rk_stage_fp64_21x91x181.md) over the same CUDA-event stage time, against 2 per SM per cycle
        sm_hz = (clk.get("sm_mhz") or 2070.0) * 1e6
        per_cell = 590.0
        ach = per_cell * interior_rk(g) / (avg_ms / 1e3)
        peak64 = 2.0 * 152 * sm_hz
        roof["fp64_pipe"] = {"instructions_per_cell": per_cell, "achieved_per_s": ach, "peak_per_s": peak64,
                             "frac": ach / peak64, "source": "ncu count, profiles/rk_stage_fp64_21x91x181.md"}
    d.close()
    # the pressure call on every iteration, beside the reference's even-iteration schedule
    pe = None
    if a.steps > 0:
        d = dyn.Dycore(g, dict(P, precision=1 if precision == "mixed" else 0, press_every_step=1))
        d.load_state(st.copy())
        if tune:
            d.set_stage_variant(dyn.Dycore.STAGE_NAMES.index(tune["stage_variant"]))
            if tune.get("march_levels"):
                d.set_march_levels(tune["march_levels"])
        d.iterate(1, a.warmup)
        n_pe = max(2, min(a.steps, 100) // 2 * 2)
        barrier(world)
        d.timer_start()
        d.iterate(a.warmup + 1, n_pe)
        ms_pe = reduce_max(world, d.timer_stop())
        d.close()
        pe = {"value": world * n_pe * g.cells / (ms_pe / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms_pe / n_pe,
              "steps": n_pe}
    return {"value": value, "ms_per_step": ms / a.steps, "e2e": e2e, "roofline": roof, "gpu_launches": launches,
            "timed_loop": "the resident loop as replays of a captured two-iteration CUDA graph "
                          "(atsat_dyn_graph_capture / atsat_dyn_graph_launch)",
            "clocks": clk, "kernels_ms": kern, "tune": tune, "pressure_every_step": pe}


def run_ours(a, rank, world):
    from atsat_gb300 import abi, dyn, fields as F, synth
    g = synth.make_grid(*a.shape)
    P = abi.default_params()
    cpu = cpu1 = cpu_fast = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        cpu = cpu_baseline(g, P, seed=0)          # before the first CUDA call
        cpu1 = cpu_baseline_one_thread(a.shape)
        cpu_fast = cpu_baseline_child(a.shape, build="fast")
    st = synth.saturn_state(g, P, seed=rank)
    pinned = {fid: dyn.PinnedArray(g.shape) for fid in range(F.NFIELDS)}
    res = {p: measure(a, rank, world, g, P, st, pinned, p) for p in a.precisions}
    for pa in pinned.values():
        pa.free()
    if rank != 0:
        return None
    head = a.precisions[0]
    r = res[head]
    out = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64" if head == "mixed" else "f64", "data": "synthetic",
           "config": dict(config(g, head), **(r["tune"] or {})), "e2e": r["e2e"], "roofline": r["roofline"],
           "gpu_launches": r["gpu_launches"], "clocks": r["clocks"], "kernels_ms": r["kernels_ms"],
           "pressure_every_step": r["pressure_every_step"], "timed_loop": r["timed_loop"]}
    for p in a.precisions[1:]:
        out[p] = {k: res[p][k] for k in ("value", "ms_per_step", "e2e", "roofline", "gpu_launches", "clocks",
                                         "pressure_every_step")}
        out["mixed_over_" + p] = r["value"] / res[p]["value"]
    if cpu:
        out["cpu_baseline"] = cpu
    if cpu1:
        out["cpu_baseline_one_thread"] = cpu1
    if cpu_fast:
        out["cpu_baseline_o3"] = cpu_fast
    return out


def run_poisson(a, rank, world):
    """Standalone red-black Poisson configuration: the pressure equation on the default grid with the
    reference's boundary planes, source N(0,1) (fixed seed) smoothed by a 3-point box filter in theta and
    phi and made compatible with the singular operator. Methods: FP64 SOR (the reference's sweep, omega 1),
    FP32 SOR, FP32 SOR sweeps inside FP64 defect correction, and the spectral direct solves (FP64 = the
    reference solution, FP32, FP32 inside FP64 defect correction to 1e-10)."""
    if rank != 0:
        return None
    import numpy as np
    from atsat_gb300 import abi, dyn, synth
    g = synth.make_grid(*a.shape)
    P = abi.default_params()
    src = synth.poisson_source(g, seed=7)
    runs = [("direct64", {}), ("direct32", {}), ("refine_direct", {"tol": 1e-10, "max_iter": 30}),
            ("sor64", {"tol": 1e-10, "max_iter": a.sor_sweeps, "omega": 1.0}),
            ("sor32", {"tol": 1e-10, "max_iter": a.sor_sweeps, "omega": 1.0}),
            ("refine_sor", {"tol": 1e-10, "max_iter": 20, "inner": a.sor_sweeps // 20, "omega": 1.0})]
    out = {}
    with dyn.Dycore(g, P) as d:
        t0 = time.perf_counter()
        f = d.poisson_project(src)
        setup_s = time.perf_counter() - t0
        d.poisson_solve("direct64", f)                       # warm-up
        ref, _ = d.poisson_solve("direct64", f)
        scale = float(np.max(np.abs(ref)))
        for name, kw in runs:
            p, st = d.poisson_solve(name, f, **kw)
            st["max_rel_error_vs_fp64_direct"] = float(np.max(np.abs(p - ref))) / scale
            out[name] = st
    best = out["refine_direct"]
    return {"metric": "standalone Poisson solve, 1 GB300: iterations, time and error vs the FP64 solution",
            "value": best["ms"], "unit": "ms (FP32 direct inner solves + FP64 defect correction to 1e-10)",
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": f"pressure equation on {g.im}x{g.jm}x{g.km}, interior "
                                   f"{g.interior_p} cells, source N(0,1) seed 7, 3-point box filter in theta and phi",
                       "setup_s": setup_s},
            "methods": out}


def run_press_variants(a, rank, world):
    """One pressure call (PressureSolver<cSaturnModel>::run with prepareProjectionBoundaries) at the
    workload grid in its four forms: the default pointwise red-black sweep, + PRESS_LINE (a radial
    Thomas solve per column, held interior mean), + PRESS_BAROTROPIC (DFT in phi and a theta tridiagonal
    per mode), and both. FP64 on the device (CUDA events around K calls after W warm-up calls) beside the
    oracle's FP64 OpenMP restatement of the same call on the host cores (one call)."""
    if rank != 0:
        return None
    from atsat_gb300 import abi, dyn, fields as F, synth
    from oracle import oracle
    g = synth.make_grid(*a.shape)
    out = {}
    for name, over in (("default", {}), ("line", {"press_line": 1}), ("barotropic", {"press_baro": 1}),
                       ("line+barotropic", {"press_line": 1, "press_baro": 1})):
        P = abi.default_params(**over)
        st = synth.saturn_state(g, P, seed=11, exercise=True)
        t0 = time.perf_counter()
        oracle.pressure(st.copy(), P)
        cpu_s = time.perf_counter() - t0
        with dyn.Dycore(g, P) as d:
            d.load_state(st)
            for _ in range(a.warmup):
                d.PressureSolver_run()
            d.profile(True)
            d.profile_reset()
            d.timer_start()
            for _ in range(a.steps):
                d.PressureSolver_run()
            ms = d.timer_stop() / a.steps
            kern = {abi.K_NAMES[c]: d.profile_read(c)[1] / a.steps for c in range(len(abi.K_NAMES))
                    if d.profile_read(c)[0] > 0}
            d.profile(False)
        out[name] = {"ms_per_call": ms, "kernel_ms_per_call": kern, "cpu_oracle_s_per_call": cpu_s,
                     "cpu_cores": os.cpu_count()}
    return {"metric": "pressure call (PressureSolver::run) device time, 1 GB300, FP64, per variant",
            "value": out["line+barotropic"]["ms_per_call"], "unit": "ms per call (PRESS_LINE + PRESS_BAROTROPIC)",
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic", "steps": a.steps, "warmup": a.warmup,
            "config": {"workload": f"pressure call on {g.im}x{g.jm}x{g.km}, interior {g.interior_p} cells, "
                                   "seeded synthetic state with stale tendencies (exercise)"},
            "variants": out}


def run_glue(a, rank, world):
    """The driver's glue around the dycore at the workload grid: one call each of the p_dyn filter
    (damp_wiggles), the species floor (clampNegativeSpecies) and the turbulence closure (Turbulence::run),
    device time from CUDA events around K calls after W warm-up calls, beside the oracle's OpenMP
    restatement of one call on the host cores; and whole iterations of the resident loop with the glue
    (params.driver_glue = 1) against the plain dycore loop, mixed and FP64."""
    if rank != 0:
        return None
    from atsat_gb300 import abi, dyn, synth
    from oracle import oracle
    g = synth.make_grid(*a.shape)
    P = abi.default_params()
    st = synth.saturn_state(g, P, seed=13, exercise=True)
    calls = {}
    for name, fn, ofn in (("damp_pdyn", "damp_pdyn", oracle.damp_pdyn),
                          ("clampNegativeSpecies", "clampNegativeSpecies", oracle.clamp_negative_species),
                          ("TurbulenceSat_run", "TurbulenceSat_run", oracle.turbulence)):
        t0 = time.perf_counter()
        ofn(st.copy(), P)
        cpu_s = time.perf_counter() - t0
        with dyn.Dycore(g, P) as d:
            d.load_state(st)
            for _ in range(a.warmup):
                getattr(d, fn)()
            d.timer_start()
            for _ in range(a.steps):
                getattr(d, fn)()
            ms = d.timer_stop() / a.steps
        calls[name] = {"device_ms_per_call": ms, "cpu_oracle_s_per_call": cpu_s, "cpu_cores": os.cpu_count()}
    loops = {}
    for prec in ("mixed", "fp64"):
        for glue in (0, 1):
            with dyn.Dycore(g, dict(P, precision=1 if prec == "mixed" else 0, driver_glue=glue)) as d:
                d.load_state(st)
                if prec == "mixed":
                    d.set_stage_variant(dyn.Dycore.STAGE_NAMES.index("tiled2"))
                d.iterate(1, a.warmup)
                d.timer_start()
                d.iterate(a.warmup + 1, a.steps)
                ms = d.timer_stop() / a.steps
            loops[f"{prec}{'_glue' if glue else ''}"] = {"ms_per_iteration": ms,
                                                          "Mcell_steps_per_s": g.cells / (ms / 1e3) / 1e6}
    return {"metric": "driver glue around the dycore, 1 GB300, FP64 device time per call and per iteration",
            "value": loops["mixed_glue"]["Mcell_steps_per_s"], "unit": UNIT + " (mixed, iteration with the glue)",
            "higher_is_better": True, "n_gpus": 1, "data": "synthetic", "steps": a.steps, "warmup": a.warmup,
            "config": {"workload": f"{g.im}x{g.jm}x{g.km}, seeded synthetic state with every input exercised"},
            "calls": calls, "iterations": loops}


def run_ensemble(a, rank, world):
    """32 independent members, 16 at 21x91x181, 12 at 41x181x361 and 4 at 61x271x541, each from the seeded
    generator with its own seed and noise amplitude U[0.5, 2], mixed precision, stage kernels autotuned per
    shape. Ten iterations per member (a) one member after another with plain resident iterations, (b) one
    after another as replays of each member's captured two-iteration CUDA graph, (c) all members' graphs
    replayed concurrently, one stream per member. Device time from CUDA events."""
    if rank != 0:
        return None
    from atsat_gb300 import abi, dyn, synth
    shapes = [(21, 91, 181)] * 16 + [(41, 181, 361)] * 12 + [(61, 271, 541)] * 4
    scale = 0.5 + 1.5 * synth.uniform(2024, 77, len(shapes))
    P = dict(abi.default_params(), precision=1)
    members, cells, tuned = [], 0, {}
    t0 = time.perf_counter()
    for m, shp in enumerate(shapes):
        g = synth.make_grid(*shp)
        st = synth.saturn_state(g, P, seed=1000 + m, noise_scale=float(scale[m]))
        d = dyn.Dycore(g, P)
        d.load_state(st)
        if shp not in tuned:
            tuned[shp] = (d.autotune(reps=3)[0], d.march_levels())
        else:
            d.set_stage_variant(tuned[shp][0])
            d.set_march_levels(tuned[shp][1])
        d.iterate(1, 2)
        members.append(d)
        cells += g.cells
    setup_s = time.perf_counter() - t0
    steps = 10
    seq_plain = 0.0
    per_shape = {}
    for d, shp in zip(members, shapes):
        d.timer_start()
        d.iterate(3, steps)
        ms = d.timer_stop()
        seq_plain += ms
        e = per_shape.setdefault(f"{shp[0]}x{shp[1]}x{shp[2]}", {"members": 0, "ms": 0.0, "cells": 0})
        e["members"] += 1
        e["ms"] += ms
        e["cells"] += shp[0] * shp[1] * shp[2]
    for e in per_shape.values():
        e["ms_per_member_iteration"] = e["ms"] / e["members"] / steps
        e["Mcell_steps_per_s"] = e["cells"] * steps / (e["ms"] / 1e3) / 1e6
    # the bound on batching: the members of the shapes whose kernels fill the GPU gain nothing from running
    # beside others; at best every member runs at the best per-cell rate any shape reaches alone
    best = max(e["Mcell_steps_per_s"] for e in per_shape.values())
    t_best = cells * steps / (best * 1e6) * 1e3
    for d in members:
        d.graph_capture(3 + steps, 2)
    seq_graph = dyn.ensemble_run(members, reps=steps // 2, concurrent=False)
    conc = dyn.ensemble_run(members, reps=steps // 2, concurrent=True)
    launches = sum(d.launches() for d in members)
    for d in members:
        d.close()
    mcs = lambda ms: cells * steps / (ms / 1e3) / 1e6
    return {"metric": "ensemble aggregate Mcell-steps/s, 1 GB300, 32 mixed-size members, mixed precision",
            "value": mcs(conc), "unit": "Mcell-steps/s", "higher_is_better": True, "n_gpus": 1, "steps": steps,
            "data": "synthetic", "dtype": "f32+f64",
            "config": {"workload": "16 x 21x91x181 + 12 x 41x181x361 + 4 x 61x271x541 members, 10 iterations each",
                       "cells": cells, "stage_variant_per_shape": {f"{s[0]}x{s[1]}x{s[2]}":
                                                                   f"{dyn.Dycore.STAGE_NAMES[v[0]]} (march depth {v[1]})"
                                                                   for s, v in tuned.items()},
                       "setup_s": setup_s},
            "per_shape_sequential": per_shape,
            "bound": {"ms_if_every_member_ran_at_the_best_shape_rate": t_best,
                      "max_batched_over_sequential": seq_plain / t_best},
            "modes": {"sequential_plain": {"ms": seq_plain, "value": mcs(seq_plain)},
                      "sequential_graphs": {"ms": seq_graph, "value": mcs(seq_graph)},
                      "concurrent_graphs": {"ms": conc, "value": mcs(conc)}},
            "batched_over_sequential": seq_plain / conc}


# one child process of the CPU table: the restatement's dycore iterations per grid, timed after one
# untimed iteration; prints one JSON object {grid: {"iterations", "s", "Mcell_steps_per_s"}}
_CPU_CHILD = r"""
import json, sys, time
sys.path.insert(0, %(root)r)
from atsat_gb300 import abi, synth
from oracle import oracle
P = abi.default_params()
out = {}
for shape, n in %(work)r:
    g = synth.make_grid(*shape)
    st = synth.saturn_state(g, P, seed=0)
    oracle.steps(st, P, 1, iter0=1)
    t0 = time.perf_counter()
    oracle.steps(st, P, n, iter0=2)
    dt = time.perf_counter() - t0
    out["%%dx%%dx%%d" %% shape] = {"iterations": n, "s": dt, "Mcell_steps_per_s": n * g.cells / dt / 1e6}
    del st
print(json.dumps(out))
"""


def run_cpu_table(a, rank, world):
    """The CPU restatement of the reference's OpenMP path per benchmark grid: the parity build (-O2, no
    contraction) and the fast build (-O3, contraction allowed), on all host cores and on one; each a
    bounded sample of dycore iterations (pressure call on the even ones) after one untimed iteration."""
    if rank != 0:
        return None
    small = [((41, 181, 361), 2), ((21, 91, 181), 4), ((61, 271, 541), 1)]
    runs = {"o2_all": ("", None, small + [((81, 361, 721), 1)]), "fast_all": ("fast", None, small),
            "o2_one": ("", "1", [((41, 181, 361), 1), ((21, 91, 181), 2)]),
            "fast_one": ("fast", "1", [((41, 181, 361), 1), ((21, 91, 181), 2)])}
    out = {}
    for name, (build, threads, work) in runs.items():
        env = dict(os.environ, ATSAT_ORACLE_BUILD=build)
        if threads:
            env["OMP_NUM_THREADS"] = threads
        else:
            env.pop("OMP_NUM_THREADS", None)
        code = _CPU_CHILD % {"root": ROOT, "work": work}
        t0 = time.perf_counter()
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=1800)
        try:
            out[name] = json.loads(r.stdout.strip().splitlines()[-1])
        except (ValueError, IndexError):
            out[name] = {"error": (r.stderr or r.stdout)[-400:]}
        out[name]["wall_s"] = time.perf_counter() - t0
    return {"metric": "CPU restatement of the dycore iteration, Mcell-steps/s per grid, build and threads",
            "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "runs": out,
            "builds": {"o2": "gcc -O2 -fopenmp -ffp-contract=off (the parity oracle)",
                       "fast": "gcc -O3 -fopenmp -ffp-contract=fast (timed baseline only)"}}


def main():
    a = parse()
    rank, world, _ = dist()
    if a.cpu_table:
        res = run_cpu_table(a, rank, world)
    elif a.ensemble:
        res = run_ensemble(a, rank, world)
    elif a.poisson:
        res = run_poisson(a, rank, world)
    elif a.press_variants:
        res = run_press_variants(a, rank, world)
    elif a.glue:
        res = run_glue(a, rank, world)
    else:
        res = run_reference(a, rank, world) if a.impl == "reference" else run_ours(a, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
