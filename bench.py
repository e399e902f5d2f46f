#!/usr/bin/env python
"""Benchmark: minidisk Godunov update, cell-updates/s on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload minidisk-4096|minidisk-256] [--precision mixed|fp64]

Default workload (the large-minidisk configuration): [-8,8]^2 on 4096^2 cells
(64x64 blocks of 64^2), mass ratio 0.5, eccentricity 0.1, Mach 20, viscosity
5e-4, softening/sink radius 0.05, sink rate 10, buffer rate 100 / scale 0.2,
PLM theta 1.5, RK2, CFL 0.3 with the fastest-wavespeed reduction, seeded +-1%
density perturbation; FP32 fluxes/sources with FP64 state accumulation. A step
is one RK2 step of the whole mesh; inputs are synthetic (seeded), resident in
HBM; the 403 MB FP64 state exceeds the 129 MB L2, so no flush is needed.

One JSON line on rank 0. `value` is device-timed cell-updates/s over all ranks;
`e2e` is the same metric through the reference-facing host-buffer call
(mara_minidisk_advance_host: H2D state, step, D2H state, every step); the
roofline line is for the dominant stage kernel, timed with CUDA events on the
stream it runs on. With --gpus N under torchrun each rank advances its own
independent replica (replicas only; no data-path collective).

--impl reference times the reference's CPU scheme (the oracle restatement of
problems/minidisk_scheme.cpp, run per block on all host threads as the
reference's thread-pool executor does) on a bounded window of the same mesh.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # the large minidisk: [-8,8]^2 on 4096^2 cells, q = 0.5, e = 0.1, Mach 20, nu = 5e-4
    "minidisk-4096": dict(block_size=64, depth=6, omega_frame=1.0, mach_number=20.0, nu=5e-4, domain_radius=8.0,
                          softening_length=0.05, eccentricity=0.1, mass_ratio=0.5, sink_radius=0.05, sink_rate=10.0,
                          buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=1.5),
    # the reference-sized minidisk: [-4,4]^2 on 256^2 cells (4x4 blocks of 64^2), equal-mass circular binary
    "minidisk-256": dict(block_size=64, depth=2, omega_frame=1.0, mach_number=10.0, nu=1e-3, domain_radius=4.0,
                         softening_length=0.05, eccentricity=0.0, mass_ratio=1.0, sink_radius=0.05, sink_rate=10.0,
                         buffer_rate=100.0, buffer_scale=0.2, cfl=0.3, plm_theta=1.5),
    # the ensemble: 64 seeded members (mesh 128^2..1024^2, q, e, Mach, nu drawn per member) on this
    # base physics; the entry itself (a 256^2 member) is what the CPU reference arm times
    "minidisk-ensemble-64": dict(block_size=64, depth=2, omega_frame=1.0, mach_number=10.0, nu=1e-3,
                                 domain_radius=4.0, softening_length=0.05, eccentricity=0.0, mass_ratio=1.0,
                                 sink_radius=0.05, sink_rate=10.0, buffer_rate=100.0, buffer_scale=0.2, cfl=0.3,
                                 plm_theta=1.5),
}
ENSEMBLE_MEMBERS = 64
# Algorithmic HBM bytes per cell for each stage kernel (FP64 state = 24 B/cell,
# FP32 increment = 12 B/cell):
#   mixed stage 1: read u0 (24) + write d1 (12)                  = 36
#   mixed stage 2: read u0 (24) + read d1 (12) + write u (24)    = 60
#   fp64 stage 1 : read u0 (24) + write u1 (24)                  = 48
#   fp64 stage 2 : read u1 (24) + read u0 (24) + write u (24)    = 72
GRAPH_STEPS = 10
STAGE_BYTES = {("mixed", 1): 36, ("mixed", 2): 60, ("fp64", 1): 48, ("fp64", 2): 72}
L2_BYTES = 129 * 2**20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["mhd-128", "srhd-c2p", "srhd-tube", "sedov-tracks"], default="minidisk-4096")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--cpu-sample-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--launch", default=None,
                    help="ensemble launch shape blocks_per_sm,chunks_per_warp,cols_per_lane,register_variant "
                         "(default: tuned)")
    ap.add_argument("--no-looped", action="store_true", help="ensemble: skip the looped single-mesh comparison")
    ap.add_argument("--no-diagnostics-timing", action="store_true",
                    help="minidisk: skip timing the step with the fused time-series sums")
    ap.add_argument("--no-fp64-variant", action="store_true",
                    help="minidisk: skip timing the plain FP64 GPU path on the same mesh")
    ap.add_argument("--no-workloads", action="store_true",
                    help="default run: skip the compact lines of the other workloads (MHD, SRHD, tube, ensemble, "
                         "sedov) in the headline line")
    ap.add_argument("--accuracy-steps", type=int, default=2000,
                    help="mixed vs FP64 error check: RK2 steps of both paths from one state (0 = skip); the "
                         "4096^2 configuration's own 2000 by default")
    ap.add_argument("--accuracy-control", action="store_true",
                    help="minidisk: with the error check, a third run, FP64 from the same state with each value "
                         "moved by one unit of 2^-24 (one FP32 rounding), compared with the FP64 run the same way "
                         "(about 90 s more at 4096^2)")
    return ap.parse_args()


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


_FP64_RATE = None


def fp64_peak() -> float:
    """Thread-level DFMA/s of this GPU, measured live (mara_measure_fp64_rate)."""
    global _FP64_RATE
    if _FP64_RATE is None:
        import torch

        from mara3p_gb300._capi import check, lib
        r = ctypes.c_double()
        check(lib.mara_measure_fp64_rate(ctypes.byref(r), torch.cuda.current_stream().cuda_stream), "fp64 rate")
        _FP64_RATE = r.value
    return _FP64_RATE


def host_link(host_buf, h2d_bytes: int, d2h_bytes: int, ms_per_call: float, stage_ms) -> dict:
    """The host link's rates (mara_measure_host_link, on the call's own pinned
    output buffer and a device buffer of its size) and the floor they put
    under one host-buffer call: the input read over the link by a kernel,
    then stage 1 (which needs the CFL maximum over the whole input), then
    stage 2 writing the output over the link (its compute hidden under the
    writes). No schedule with the reference's CFL time step does better."""
    import torch

    from mara3p_gb300._capi import check, lib
    dev = torch.empty(host_buf.numel() * host_buf.element_size(), dtype=torch.uint8, device="cuda")
    g = (ctypes.c_double * 5)()
    check(lib.mara_measure_host_link(host_buf.data_ptr(), dev.data_ptr(), dev.numel(), g,
                                     torch.cuda.current_stream().cuda_stream), "host link")
    del dev
    names = ["h2d_copy_engine_gbs", "d2h_copy_engine_gbs", "kernel_read_gbs", "kernel_write_gbs",
             "read_and_write_together_gbs"]
    out = {k: round(v, 1) for k, v in zip(names, g)}
    floor = (h2d_bytes / (g[2] * 1e9) + d2h_bytes / (g[3] * 1e9)) * 1e3 + stage_ms[0]
    out.update({"floor_ms_per_call": floor, "frac_of_floor": floor / ms_per_call,
                "floor": "input read by a kernel at kernel_read_gbs + stage 1 + output written at kernel_write_gbs"})
    return out


def fp64_pipe_fraction(key: str, units: float, ms: float):
    """The FP64-pipe roofline of an FP64-bound kernel: its FP64 thread
    instructions per unit (an ncu count in profiles/fp64_ops.json) x units
    per CUDA-event millisecond, against the live-measured DFMA rate."""
    f = ROOT / "profiles" / "fp64_ops.json"
    if not f.exists():
        return None
    rec = json.loads(f.read_text()).get(key)
    if rec is None:
        return None
    peak = fp64_peak()
    achieved = rec["fp64_inst_per_unit"] * units / (ms * 1e-3)
    return {"bound": "fp64", "achieved": achieved / 1e9, "peak": peak / 1e9,
            "unit": "G FP64 thread-instructions/s", "frac": achieved / peak,
            "fp64_inst_per_unit": rec["fp64_inst_per_unit"], "kernels": rec.get("kernels"),
            "peak_source": "measured live: mara_measure_fp64_rate (DFMA chains on every SM)",
            "counts_source": "profiles/fp64_ops.json (ncu sm__inst_executed_pipe_fp64 x 32 per unit)"}


def fp64_roofline(key: str, units: float, ms: float, hbm: dict) -> dict:
    """The roofline of an FP64-bound workload: the FP64 pipe where its counts
    are known (the HBM figures kept beside it), else the HBM line."""
    fp = fp64_pipe_fraction(key, units, ms)
    if fp is None:
        return hbm
    fp["hbm"] = {k: hbm[k] for k in ("achieved", "peak", "unit", "frac")}
    fp["kernel"] = hbm.get("kernel")
    fp["traffic"] = hbm.get("traffic")
    return fp


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# Replicas only: under torchrun every rank advances its own seeded mesh (seed
# base + rank) with no data exchange; the process group serves the barriers
# around the timed region and the maximum of the ranks' times, and rank 0
# prints the one line, whose value counts the units of all ranks.
def init_replicas(world: int) -> None:
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def emit(line: dict, rank: int) -> bool:
    """Print the JSON line on rank 0 only; returns whether it printed."""
    if rank != 0:
        return False
    print(json.dumps(line), flush=True)
    return True


def finish_replicas(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.device)], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if self.proc is None:
            return None
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for name, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class CpuBaseline:
    """Oracle restatement of the reference scheme on all host threads, on a
    bounded window of blocks of the same mesh: one RK2 step = two substeps,
    one task per block per substep (the reference's compute_threaded shape)."""

    def __init__(self, sd_kw: dict, seconds: float):
        from oracle.oracle import MinidiskParams, dptr, load_oracle
        self.o, self.dptr = load_oracle(), dptr
        self.p = MinidiskParams(**sd_kw)
        p = self.p
        self.N = p.block_size << p.depth
        self.nb = 1 << p.depth
        self.threads = os.cpu_count() or 1
        self.u = np.zeros(3 * self.N * self.N)
        self.o.oracle_minidisk_initial_conserved(ctypes.byref(p), ctypes.c_uint64(1), ctypes.c_double(0.01),
                                                 dptr(self.u))
        self.out = np.zeros_like(self.u)
        self.t = 1.0
        self.dt = self.o.oracle_minidisk_dt_formula(ctypes.byref(p), ctypes.c_double(1.0))
        probe = min(max(self.threads, 16), self.nb * self.nb)
        per_block = self.step(probe) / probe
        self.count = int(min(self.nb * self.nb, max(self.threads, seconds / max(per_block, 1e-9))))

    def step(self, count=None) -> float:
        count = self.count if count is None else count
        o, p, d = self.o, self.p, self.dptr
        t0 = time.perf_counter()
        o.oracle_minidisk_substep_blocks(ctypes.byref(p), d(self.u), d(self.out), ctypes.c_double(self.t),
                                         ctypes.c_double(self.dt), self.threads, 0, count)
        o.oracle_minidisk_substep_blocks(ctypes.byref(p), d(self.out), d(self.u), ctypes.c_double(self.t + self.dt),
                                         ctypes.c_double(self.dt), self.threads, 0, count)
        return time.perf_counter() - t0

    def measure(self) -> dict:
        elapsed = self.step()
        cells = self.count * self.p.block_size ** 2
        return {"value": cells / elapsed, "unit": "cell-updates/s", "cores": self.threads, "kind": "port",
                "sample": f"one RK2 step on {self.count} of {self.nb * self.nb} blocks ({cells} cells) of the "
                          f"{self.N}^2 mesh, {elapsed:.1f} s, {self.threads} threads, one task per block per substep"}


def cpu_baseline(sd_kw: dict, seconds: float) -> dict:
    return CpuBaseline(sd_kw, seconds).measure()


def minidisk_config(workload: str, world: int) -> dict:
    """The `config` of a minidisk workload's line, the same in both arms."""
    kw = WORKLOADS[workload]
    N = kw["block_size"] << kw["depth"]
    nb = 1 << kw["depth"]
    return {"workload": workload, "cells": N * N,
            "mesh": f"{N}^2 ({nb}x{nb} blocks of {kw['block_size']}^2)",
            "scheme": f"PLM(theta={kw['plm_theta']})+HLLE+viscosity+gravity/sink/buffer sources, RK2, "
                      f"CFL {kw['cfl']} wavespeed reduction",
            "physics": {k: kw[k] for k in ("domain_radius", "mass_ratio", "eccentricity", "mach_number", "nu",
                                           "softening_length", "sink_radius", "sink_rate", "buffer_rate",
                                           "buffer_scale")},
            "parallelism": f"replicas x{world}",
            "l2": f"no flush: FP64 state {3 * N * N * 8 / 1e6:.0f} MB > L2 {L2_BYTES / 1e6:.0f} MB"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    sd_kw = WORKLOADS[args.workload]
    cb = CpuBaseline(sd_kw, seconds=min(args.cpu_sample_seconds, 3.0))
    vals = []
    for i in range(args.warmup + args.steps):
        r = cb.measure()
        if i >= args.warmup:
            vals.append(r["value"])
    value = float(np.mean(vals))
    N = sd_kw["block_size"] << sd_kw["depth"]
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * N * N / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": minidisk_config(args.workload, args.gpus),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": r["cores"], "kind": r["kind"],
                         "sample": r["sample"]},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def mixed_accuracy(md, sd, u0, steps: int, control: bool = False) -> dict:
    """Mixed vs FP64 relative L1 after `steps` RK2 steps from one state, each
    path with its own CFL dt (an FP64 evaluation in both), also at half the
    horizon; globally and over the interior, the mesh less a frame of 0.5
    along the box edges. The frame holds the periodic seams where the buffer
    ring r ~ domain_radius meets the box edge: the tangential velocity jumps
    by about 2 Omega R across them, and that shear layer amplifies any
    difference between two runs (FP64 runs from states 1e-12 apart included)."""
    import torch
    N = sd.cells_per_side
    x = (torch.arange(N, device="cuda", dtype=torch.float64) + 0.5) * (2 * sd.domain_radius / N) - sd.domain_radius
    inner = x.abs() < sd.domain_radius - 0.5
    mask = (inner[:, None] & inner[None, :]).to(torch.float64)
    runs = {p: md.Run(sd, u0.clone(), rk_order=2, precision=p, dt_mode=md.DT_CFL) for p in (md.FP64, md.MIXED)}
    if control:
        # the control: FP64 from the state with every value moved by a relative
        # 2^-24 of seeded sign, once, at the start (the mixed path rounds to
        # FP32 in every flux of every step, a larger perturbation)
        g = torch.Generator(device="cuda")
        g.manual_seed(12345)
        sign = torch.randint(0, 2, u0.shape, generator=g, device="cuda").to(torch.float64) * 2 - 1
        runs["control"] = md.Run(sd, u0 * (1 + sign * 2.0 ** -24), rk_order=2, precision=md.FP64,
                                 dt_mode=md.DT_CFL)
    out = {"dt": "CFL 0.3, FP64 in each path",
           "interior": "|x|, |y| < domain_radius - 0.5 (the periodic seams excluded)"}
    done = 0
    for target in sorted({steps // 2, steps}):
        for r in runs.values():
            r.advance(target - done)
        done = target
        torch.cuda.synchronize()
        a, b = runs[md.MIXED].u, runs[md.FP64].u
        rel = [float((a[k] - b[k]).abs().sum() / b[k].abs().sum()) for k in range(3)]
        reli = [float(((a[k] - b[k]).abs() * mask).sum() / (b[k].abs() * mask).sum()) for k in range(3)]
        out[str(target)] = {"rel_l1_vs_fp64": {"density": rel[0], "momentum_x": rel[1], "momentum_y": rel[2]},
                            "interior_rel_l1_vs_fp64": {"density": reli[0], "momentum_x": reli[1],
                                                        "momentum_y": reli[2]},
                            "time": runs[md.MIXED].time, "time_fp64": runs[md.FP64].time}
        if control:
            c = runs["control"].u
            out[str(target)]["control_fp64_perturbed_2e-24"] = {
                "rel_l1_vs_fp64": {"density": float((c[0] - b[0]).abs().sum() / b[0].abs().sum())},
                "interior_rel_l1_vs_fp64": {"density": float(((c[0] - b[0]).abs() * mask).sum()
                                                             / (b[0].abs() * mask).sum())},
                "time": runs["control"].time}
    out["steps"] = steps
    out["rel_l1_vs_fp64"] = out[str(steps)]["rel_l1_vs_fp64"]
    out["finite"] = bool(torch.isfinite(runs[md.MIXED].u).all().item() and torch.isfinite(runs[md.FP64].u).all().item())
    del runs
    return out


def run_ours(args):
    import torch

    import mara3p_gb300.minidisk as md
    from mara3p_gb300._capi import check, lib

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    init_replicas(world)
    sd = md.SolverData(**WORKLOADS[args.workload])
    N = sd.cells_per_side
    cells = N * N
    prec = md.MIXED if args.precision == "mixed" else md.FP64
    u0 = md.initial_conserved(sd, seed=1 + rank, amplitude=0.01)
    run = md.Run(sd, u0.clone(), rk_order=2, precision=prec, dt_mode=md.DT_CFL)
    stream = torch.cuda.current_stream()

    # steps replay from a captured CUDA graph of GRAPH_STEPS steps (the
    # reference driver's fold batch); preparing it is part of the warm-up
    run.use_graph(GRAPH_STEPS)
    run.advance(max(args.warmup - GRAPH_STEPS, 0))
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as sampler:
        torch.cuda.synchronize()
        e0.record(stream)
        run.advance(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    value = cells * args.steps * world / (ms * 1e-3)
    # per replay of GRAPH_STEPS steps, and per direct call of the remainder:
    # clock begin + per step (stage 1, stage 2, clock)
    full, rest = divmod(args.steps, GRAPH_STEPS)
    gpu_launches = full * (1 + 3 * GRAPH_STEPS) + (1 + 3 * rest if rest else 0)

    # Per-stage kernel durations (dominant kernel for the roofline): the same
    # stage kernels, launched one by one through mara_minidisk_stage on the
    # same stream with CUDA events around each launch.
    c = sd.to_c()
    ws = run.workspace
    clock = run.clock.data_ptr()
    d1 = ws.data_ptr() + 3 * cells * 8
    alt = ws.data_ptr()
    kind1, kind2 = (1, 2) if prec == md.MIXED else (0, 0)
    reps = max(3, min(args.steps, 10))
    t1, t2 = [], []
    for _ in range(reps):
        a, b, d = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        a.record(stream)
        if prec == md.MIXED:
            check(lib.mara_minidisk_stage(ctypes.byref(c), kind1, run.u.data_ptr(), None, None, None, d1, clock, 0, 0,
                                          stream.cuda_stream))
            b.record(stream)
            check(lib.mara_minidisk_stage(ctypes.byref(c), kind2, run.u.data_ptr(), d1, None, alt, None, clock, 1, 1,
                                          stream.cuda_stream))
        else:
            check(lib.mara_minidisk_stage(ctypes.byref(c), 0, run.u.data_ptr(), None, None, alt, None, clock, 0, 0,
                                          stream.cuda_stream))
            b.record(stream)
            check(lib.mara_minidisk_stage(ctypes.byref(c), 0, alt, None, run.u.data_ptr(), run.u.data_ptr(), None,
                                          clock, 1, 1, stream.cuda_stream))
        d.record(stream)
        torch.cuda.synchronize()
        t1.append(a.elapsed_time(b))
        t2.append(b.elapsed_time(d))
    pname = args.precision
    s1, s2 = float(np.median(t1)), float(np.median(t2))
    dominant = 2 if s2 >= s1 else 1
    dom_ms = s2 if dominant == 2 else s1
    dom_bytes = STAGE_BYTES[(pname, dominant)] * cells
    peak, peak_kind = measured_peaks()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic, traffic_source = None, None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        tk = json.loads(tfile.read_text()).get(f"{args.workload}/{pname}/stage{dominant}")
        if tk is not None:
            traffic = float(tk["bytes_per_cell"]) * cells
            traffic_source = tk["source"] + " x cells, from profiles/traffic.json (not measured in this run)"
    step_bytes = (STAGE_BYTES[(pname, 1)] + STAGE_BYTES[(pname, 2)]) * cells
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic,
                "kernel": f"sweep_kernel (stage {dominant})" if prec == md.MIXED else f"stage_kernel<double, 0> (stage {dominant})",
                "kernel_ms": dom_ms, "algorithmic_bytes": dom_bytes, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic_source": traffic_source,
                "stage_ms": [s1, s2],
                "step_frac": step_bytes / (ms / args.steps * 1e-3) / 1e9 / peak}

    # e2e: the reference-facing host-buffer call, H2D + step + D2H every step.
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty((3, N, N), dtype=torch.float64, pin_memory=True)
        host_out = torch.empty((3, N, N), dtype=torch.float64, pin_memory=True)
        host_in.copy_(run.u.cpu())
        hws = torch.empty(lib.mara_minidisk_host_workspace_bytes(ctypes.byref(c), 2, prec), dtype=torch.uint8,
                          device="cuda")
        tout = ctypes.c_double()
        e2e_steps = max(2, min(args.steps, 10))

        def host_step():
            check(lib.mara_minidisk_advance_host(ctypes.byref(c), host_in.data_ptr(), host_out.data_ptr(), 1.0, 1, 2,
                                                 prec, md.DT_CFL, ctypes.byref(tout), hws.data_ptr(),
                                                 stream.cuda_stream))
        host_step()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            host_step()
        el = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": cells * e2e_steps * world / el, "unit": "cell-updates/s",
               "h2d_bytes_per_step": 3 * cells * 8, "d2h_bytes_per_step": 3 * cells * 8,
               "call": "mara_minidisk_advance_host (pinned host state in/out, 1 RK2 step per call)",
               "ms_per_call": el / e2e_steps * 1e3}
        e2e["link"] = host_link(host_out, e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"],
                                e2e["ms_per_call"], [s1, s2])

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(WORKLOADS[args.workload], args.cpu_sample_seconds)

    # Mixed-precision error: both paths advanced from the same state, each
    # with its own CFL time step (an FP64 evaluation in both: the mixed path's
    # reduction names the fastest cell and the clock evaluates it in FP64),
    # relative L1 per component after S steps. (The reference's fixed-formula
    # dt lets this configuration develop negative densities after ~600 steps
    # in both precisions, so the CFL dt is used.)
    # the time series (forces, torques, work, accretion and buffer rates)
    # fused into the stage kernels: the same step with the sums on
    diag_line = None
    if prec == md.MIXED and not args.no_diagnostics_timing:
        drun = md.Run(sd, u0.clone(), rk_order=2, precision=prec, dt_mode=md.DT_CFL, diagnostics=True)
        drun.use_graph(GRAPH_STEPS)
        torch.cuda.synchronize()
        d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d0.record(stream)
        drun.advance(args.steps)
        d1.record(stream)
        torch.cuda.synchronize()
        dms = d0.elapsed_time(d1) / args.steps
        diag_line = {"ms_per_step": dms, "cell_updates_per_s": cells / (dms * 1e-3),
                     "overhead": dms / (ms / args.steps) - 1.0,
                     "what": "Run(diagnostics=True): 13 rate sums fused into both stage kernels, integrated by "
                             "the clock kernel"}
        del drun
    # the plain FP64 GPU path on the same mesh and state: the metric's comparator
    variants = None
    if prec == md.MIXED and not args.no_fp64_variant:
        frun = md.Run(sd, u0.clone(), rk_order=2, precision=md.FP64, dt_mode=md.DT_CFL)
        frun.advance(1)
        torch.cuda.synchronize()
        k = max(2, min(args.steps, 5))
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        frun.advance(k)
        f1.record(stream)
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1) / k
        fval = cells * world / (fms * 1e-3)
        fbytes = (STAGE_BYTES[("fp64", 1)] + STAGE_BYTES[("fp64", 2)]) * cells
        variants = {"fp64": {"value": fval, "unit": "cell-updates/s", "ms_per_step": fms, "steps": k,
                             "mixed_over_fp64": value / fval,
                             "hbm_frac": fbytes / (fms * 1e-3) / 1e9 / measured_peaks()[0],
                             "kernel": "stage_kernel<double, 0> (16x32 tiles, TMA halo copy), same RK2 + CFL step"}}
        fp64_pipe = fp64_pipe_fraction("minidisk-4096/fp64", cells, fms)
        if fp64_pipe is not None:
            variants["fp64"]["fp64_pipe"] = fp64_pipe
        del frun
    accuracy = None
    if prec == md.MIXED and args.accuracy_steps > 0:
        accuracy = mixed_accuracy(md, sd, u0, args.accuracy_steps, args.accuracy_control)

    if rank == 0:
        line = {
            "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 compute, f64 state" if prec == md.MIXED else "f64", "data": "synthetic",
            "config": minidisk_config(args.workload, world),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
            "clocks": sampler.summary(), "accuracy": accuracy, "diagnostics": diag_line, "variants": variants,
        }
        return line
    return None


def _line(args, world, value, unit, ms_per_step, dtype, config, roofline, extra=None):
    line = {"metric": unit, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic", "config": config, "roofline": roofline}
    line.update(extra or {})
    return line


def host_loop(pairs_in, step, pairs_out, steps):
    """End-to-end time per step through a public call: each step copies the
    inputs from pinned host buffers to the device (pairs_in: (host, device)),
    runs `step`, and copies the results back (pairs_out: (device, host)).
    Returns (seconds per step, H2D bytes, D2H bytes per step)."""
    import torch
    for h, d in pairs_in:
        d.copy_(h, non_blocking=True)
    step()
    for d, h in pairs_out:
        h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for h, d in pairs_in:
            d.copy_(h, non_blocking=True)
        step()
        for d, h in pairs_out:
            h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    el = (time.perf_counter() - t0) / steps
    return (el, sum(h.numel() * h.element_size() for h, _ in pairs_in),
            sum(h.numel() * h.element_size() for _, h in pairs_out))


def pinned_like(t):
    import torch
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h


def run_mhd(args):
    """128^3 constrained-transport MHD (examples/mhd3d.cpp RK2), seeded
    velocity and vector-potential modes (k <= 4, rms v 0.5, beta 10)."""
    import torch

    import mara3p_gb300.mhd as mh
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    N = 128
    cfg = mh.MhdConfig(N=N)
    prec = mh.MIXED if args.precision == "mixed" else mh.FP64
    s = mh.initial_state(cfg, seed=1 + rank, modes=24)
    run = mh.Run(s, precision=prec)
    run.advance(args.warmup)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as sampler:
        e0.record(stream)
        run.advance(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = N ** 3
    value = cells * args.steps * world / (ms * 1e-3)
    peak, kind = measured_peaks()
    # per step: clock begin, per stage (prim, dt, fused stage | 3 faces + 2 updates), clock end
    fused = prec == mh.MIXED and N % 32 == 0
    # 8 FP64 values per cell (5 conserved + 3 face B), read and written per stage, RK2 = 320 B per cell-update
    achieved = 320.0 * cells / (ms / args.steps * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
            "kernel": ("whole RK2 step (prim, fused faces + EMFs + updates per stage)" if fused
                       else "whole RK2 step (prim, 3 x face, 2 x update per stage)"), "peak_source": f"{kind} hbm_gbs"}
    c = run.clock.read()
    accuracy = None
    if prec == mh.MIXED and args.accuracy_steps > 0:
        k = min(args.accuracy_steps, 50)
        out = {}
        for p in (mh.FP64, mh.MIXED):
            r = mh.Run(mh.initial_state(cfg, seed=1 + rank, modes=24), precision=p)
            r.advance(k)
            torch.cuda.synchronize()
            out[p] = (r.state, r.clock.read()["time"], r.max_div_b())
        (sf, tf, _), (sm, tm, dbm) = out[mh.FP64], out[mh.MIXED]
        rel = {name: float((a - b).abs().sum() / b.abs().sum())
               for name, a, b in (("density", sm.uc[0], sf.uc[0]), ("energy", sm.uc[4], sf.uc[4]),
                                  ("bx_faces", sm.bf[0], sf.bf[0]))}
        accuracy = {"steps": k, "rel_l1_vs_fp64": rel, "time_mixed": tm, "time_fp64": tf,
                    "dt": "CFL in each path (times differ by the FP32 wavespeed)", "max_div_b_mixed": dbm}
    e2e = None
    if not args.no_e2e:
        st = run.state
        dev = [st.uc] + list(st.bf)
        hosts = [pinned_like(t) for t in dev]
        el, bi, bo = host_loop(list(zip(hosts, dev)), lambda: run.advance(1), list(zip(dev, hosts)),
                               max(2, min(args.steps, 10)))
        e2e = {"value": cells * world / el, "unit": "cell-updates/s", "h2d_bytes_per_step": bi,
               "d2h_bytes_per_step": bo, "call": "mhd.Run.advance (mara_mhd_advance), state and face fields "
                                                 "copied in and out through pinned host buffers every step"}
    line = _line(args, world, value, "cell-updates/s", ms / args.steps,
                 "f32 compute, f64 state" if prec == mh.MIXED else "f64",
                 {"workload": "mhd-128", "cells": cells, "scheme": "PLM(1.5)+HLLE+CT, RK2, CFL 0.3",
                  "precision": args.precision, "l2": "state 126 MB + intermediates > L2, no flush"}, roof,
                 {"max_div_b": run.max_div_b(), "failures": c["failures"], "time": c["time"],
                  "clocks": sampler.summary(), "gpu_launches": (8 if fused else 16) * args.steps,
                  "accuracy": accuracy, "e2e": e2e})
    return line if rank == 0 else None


def run_srhd(args):
    """2^24 seeded SRHD zones (rho 1e-4..1, p 1e-6..10, W 1..50, isotropic):
    conserved -> primitive recovery, default guess vs the trained MLP guess."""
    import torch

    import mara3p_gb300.srhd as sr
    from mara3p_gb300._capi import lib
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    n = 1 << 24
    cons = torch.empty((5, n), dtype=torch.float64, device="cuda")
    prim0 = torch.empty_like(cons)
    from mara3p_gb300._capi import check as check_
    check_(lib.mara_srhd_seeded_zones(1 + rank, n, 1e-4, 1.0, 1e-6, 10.0, 50.0, 4.0 / 3.0, prim0.data_ptr(),
                                      cons.data_ptr(), torch.cuda.current_stream().cuda_stream), "seeded zones")
    # train the guess on pairs from the library's own FP64 recovery of other zones
    tcons = torch.empty((5, 1 << 18), dtype=torch.float64, device="cuda")
    tprim = torch.empty_like(tcons)
    check_(lib.mara_srhd_seeded_zones(1000 + rank, 1 << 18, 1e-4, 1.0, 1e-6, 10.0, 50.0, 4.0 / 3.0, tprim.data_ptr(),
                                      tcons.data_ptr(), torch.cuda.current_stream().cuda_stream), "seeded zones")
    rec = sr.recover_primitive(tcons)
    net = sr.PressureGuess()
    net.prepare(tcons, rec.prim, seed=1)
    net.train(steps=2000, batch=8192, lr=2e-3, seed=1)
    torch.cuda.synchronize()
    results = {}
    for name, kw in {"default": {}, "mlp": dict(mlp=net, refine32=2)}.items():
        for _ in range(args.warmup):
            sr.recover_primitive(cons, **kw)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            r = sr.recover_primitive(cons, **kw)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        results[name] = {"ms": ms, "zones_per_s": n / (ms * 1e-3), "mean_newton_iterations": r.iterations.float().mean().item(),
                         "max_newton_iterations": int(r.iterations.max().item()), "failures": int((r.status != 0).sum().item())}
    peak, kind = measured_peaks()
    best = results["mlp"]
    achieved = 80.0 * n / (best["ms"] * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
            "kernel": "c2p_mlp_kernel (FP64-Newton bound; 80 B/zone algorithmic)", "peak_source": f"{kind} hbm_gbs"}
    roof = fp64_roofline("srhd-c2p/mlp", n, best["ms"], roof)
    fd = fp64_pipe_fraction("srhd-c2p/default", n, results["default"]["ms"])
    if fd is not None:
        results["default"]["fp64_pipe_frac"] = fd["frac"]
    e2e = None
    if not args.no_e2e:
        # the host-buffer call: conserved in from and primitives out to pinned
        # host memory, pipelined through the GPU in eight chunks
        hc = pinned_like(cons)
        hr = sr.HostRecovery(mlp=net, refine32=2, chunks=8)
        hp = hr.recover(hc)
        bi = hc.numel() * 8
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        k = max(2, min(args.steps, 10))
        for _ in range(k):
            hp = hr.recover(hc)
        el = (time.perf_counter() - t0) / k
        e2e = {"value": n * world / el, "unit": "zones/s", "h2d_bytes_per_step": bi,
               "d2h_bytes_per_step": hp.numel() * 8,
               "call": "srhd.HostRecovery.recover (mara_srhd_recover_primitive_host) with the learned guess: "
                       "conserved in and primitives out through pinned host buffers, eight chunks on three streams"}
    line = _line(args, world, best["zones_per_s"] * world, "zones/s", best["ms"], "f64 (bf16 guess)",
                 {"workload": "srhd-c2p-2^24", "zones": n, "gamma": 4.0 / 3.0}, roof, {"variants": results, "e2e": e2e})
    return line if rank == 0 else None


def run_ensemble(args):
    """The ensemble: 64 independent minidisk members (mesh from 128^2 to
    1024^2, mass ratio, eccentricity, Mach number and viscosity drawn per
    member by seed), mixed precision, RK2, CFL. One step = one RK2 step of
    every member: one persistent sweep launch per stage and one clock launch,
    replayed from a CUDA graph, launch shape picked by the tuner. Compared with
    looping the single-mesh advance over the members."""
    import dataclasses

    import torch

    import mara3p_gb300.ensemble as en
    import mara3p_gb300.minidisk as md

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    init_replicas(world)
    members = en.seeded_members(5 + rank, ENSEMBLE_MEMBERS, md.SolverData(**WORKLOADS[args.workload]))
    cells = sum(sd.cells_per_side ** 2 for sd in members)
    u0 = [md.initial_conserved(sd, seed=100 + m, amplitude=0.01) for m, sd in enumerate(members)]
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    e = en.Ensemble(members, [u.clone() for u in u0], precision=md.MIXED, dt_mode=md.DT_CFL,
                    autotune=0 if args.launch else 1)
    if args.launch:
        b, c, k, v = (int(x) for x in args.launch.split(","))
        e.set_config(blocks_per_sm=b, chunks_per_warp=c, cols_per_lane=k, register_variant=v)
    tune_s = time.perf_counter() - t0

    def timed(fn, steps):
        fn(args.warmup)
        torch.cuda.synchronize()
        barrier(world)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn(steps)
        b.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(a.elapsed_time(b), world)

    with ClockSampler(local) as sampler:
        ms = timed(e.advance, args.steps)
    value = cells * args.steps * world / (ms * 1e-3)
    gpu_launches = 1 + 3 * args.steps + (args.steps % 2)   # clock begin, per step 2 sweeps + clock, copy-back

    # the same members advanced one at a time through the single-mesh call
    looped_line = None
    if not args.no_looped:
        runs = [md.Run(sd, u.clone(), rk_order=2, precision=md.MIXED, dt_mode=md.DT_CFL) for sd, u in zip(members, u0)]

        def looped(k):
            for r in runs:
                r.advance(k)
        ms_loop = timed(looped, args.steps)
        looped_line = {"value": cells * args.steps * world / (ms_loop * 1e-3), "ms_per_step": ms_loop / args.steps,
                       "gpu_launches": len(members) * (1 + 3 * args.steps)}
        del runs

    s1, s2 = e.stage_times(5)
    peak, kind = measured_peaks()
    dom_ms = max(s1, s2)
    dominant = 2 if s2 >= s1 else 1
    dom_bytes = STAGE_BYTES[("mixed", dominant)] * cells
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    step_bytes = (STAGE_BYTES[("mixed", 1)] + STAGE_BYTES[("mixed", 2)]) * cells
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        tk = json.loads(tfile.read_text()).get(f"{args.workload}/mixed/stage{dominant}")
        if tk is not None:
            traffic = float(tk["bytes_per_cell"]) * cells
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": f"ensemble_sweep_kernel (stage {dominant})", "kernel_ms": dom_ms,
            "algorithmic_bytes": dom_bytes, "peak_source": f"{kind} hbm_gbs", "stage_ms": [s1, s2],
            "step_frac": step_bytes / (ms / args.steps * 1e-3) / 1e9 / peak}

    e2e = None
    if not args.no_e2e:
        # every member's input and output as views of one pinned allocation
        # per direction (with 64 separately pinned tensors this line varied by
        # 1.7x from run to run)
        sizes = [u.numel() for u in e.states]
        pin_in = torch.empty(sum(sizes), dtype=torch.float64).pin_memory()
        pin_out = torch.empty(sum(sizes), dtype=torch.float64).pin_memory()
        offs = np.concatenate([[0], np.cumsum(sizes)])
        hosts = [pin_in[offs[m]:offs[m + 1]].view(u.shape) for m, u in enumerate(e.states)]
        outs = [pin_out[offs[m]:offs[m + 1]].view(u.shape) for m, u in enumerate(e.states)]
        for h, u in zip(hosts, e.states):
            h.copy_(u)

        def host_step():
            for h, u in zip(hosts, e.states):
                u.copy_(h, non_blocking=True)
            e.advance(1)
            for o, u in zip(outs, e.states):
                o.copy_(u, non_blocking=True)
            torch.cuda.synchronize()
        host_step()
        k = max(2, min(args.steps, 10))
        t1 = time.perf_counter()
        for _ in range(k):
            host_step()
        el = time.perf_counter() - t1
        nbytes = 3 * cells * 8
        e2e = {"value": cells * k * world / el, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes,
               "call": "Ensemble.advance(1) with every member's state copied from and to pinned host memory"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(dataclasses.asdict(members[0]) | {"depth": 2, "block_size": 64},
                           args.cpu_sample_seconds)
    sizes = sorted(sd.cells_per_side for sd in members)
    line = _line(args, world, value, "cell-updates/s", ms / args.steps, "f32 compute, f64 state",
                 {"workload": args.workload, "members": len(members), "cells": cells,
                  "meshes": {str(n): sizes.count(n) for n in sorted(set(sizes))},
                  "scheme": "PLM(theta=1.5)+HLLE+viscosity+gravity/sink/buffer sources, RK2, CFL 0.3 per member",
                  "launch": e.config, "tune_seconds": tune_s, "parallelism": f"replicas x{world}",
                  "l2": f"no flush: FP64 states {3 * cells * 8 / 1e6:.0f} MB > L2 {L2_BYTES / 1e6:.0f} MB"},
                 roof, {"looped_single_mesh": looped_line,
                        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
                        "clocks": sampler.summary()})
    e.close()
    return line if rank == 0 else None


def run_tube(args):
    """1024^2 relativistic shock tube (rho 10 / p 13.33 left, rho 1 / p 1e-6
    right, interface at 30 degrees), PLM + HLLE, RK2, recovery seeded by the
    trained MLP guess (FP64 Newton polish)."""
    import torch

    import mara3p_gb300.srhd as sr
    from mara3p_gb300._capi import check as check_, lib
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    N = 1024
    prec = 1 if args.precision == "mixed" else 0
    tcons = torch.empty((5, 1 << 18), dtype=torch.float64, device="cuda")
    tprim = torch.empty_like(tcons)
    check_(lib.mara_srhd_seeded_zones(1000 + rank, 1 << 18, 1e-4, 1.0, 1e-6, 10.0, 50.0, 4.0 / 3.0, tprim.data_ptr(),
                                      tcons.data_ptr(), torch.cuda.current_stream().cuda_stream), "seeded zones")
    net = sr.PressureGuess()
    net.prepare(tcons, sr.recover_primitive(tcons).prim, seed=1)
    net.train(steps=2000, batch=8192, lr=2e-3, seed=1)
    results = {}
    for name, kw in {"default": dict(guess=sr.GUESS_ZERO), "mlp": dict(guess=sr.GUESS_MLP, mlp=net, refine32=2),
                     "warm": dict(guess=sr.GUESS_PREVIOUS)}.items():
        tube = sr.ShockTube(N=N)
        tube.advance(args.warmup, precision=prec, **kw)
        torch.cuda.synchronize()
        n0 = tube.clock_state()["newton"]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        tube.advance(args.steps, precision=prec, **kw)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        c = tube.clock_state()
        results[name] = {"ms_per_step": ms, "cell_updates_per_s": N * N / (ms * 1e-3),
                         "mean_newton_per_recovery": (c["newton"] - n0) / (2.0 * N * N * args.steps),
                         "failures": c["failures"]}
    peak, kind = measured_peaks()
    best = results["mlp"]
    achieved = 160.0 * N * N / (best["ms_per_step"] * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "whole RK2 step (FP64 Newton recovery bound)", "peak_source": f"{kind} hbm_gbs"}
    roof = fp64_roofline(f"srhd-tube/{args.precision}/mlp", N * N, best["ms_per_step"], roof)
    e2e = None
    if not args.no_e2e:
        tube = sr.ShockTube(N=N)
        kw = dict(guess=sr.GUESS_MLP, mlp=net, refine32=2)
        hu = pinned_like(tube.u)
        el, bi, bo = host_loop([(hu, tube.u)], lambda: tube.advance(1, precision=prec, **kw), [(tube.u, hu)],
                               max(2, min(args.steps, 10)))
        e2e = {"value": N * N * world / el, "unit": "cell-updates/s", "h2d_bytes_per_step": bi,
               "d2h_bytes_per_step": bo, "call": "srhd.ShockTube.advance with the learned guess, state copied in "
                                                 "and out through pinned host buffers every step"}
    line = _line(args, world, best["cell_updates_per_s"] * world, "cell-updates/s", best["ms_per_step"],
                 "f32 compute, f64 state" if prec else "f64",
                 {"workload": "srhd-tube-1024", "cells": N * N, "scheme": "PLM(1.5)+HLLE, RK2, CFL 0.3",
                  "precision": args.precision}, roof, {"variants": results, "e2e": e2e})
    return line if rank == 0 else None


def run_sedov(args):
    """Spherical-track SRHD (the sedov2d scheme): 1024 radial tracks over
    [0, pi], each from generate_radial_track(1, 1.8, aspect 2) as
    problems/sedov2d.cpp lays them out (its default is 128 tracks; 1024 gives
    522,919 cells), a seeded wind with a hot core, forward Euler (the
    driver's default rk = 1), dt = 0.5 * min spacing. One step is the
    driver's (problems/sedov2d.cpp:700-712): recovery, radial and transverse
    HLLC fluxes, update and face motion of every cell, then sedov::remesh of
    every track (max aspect 2, min 0.5, inner radius 1)."""
    import torch

    import mara3p_gb300.sedov as sv
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    T = 1024
    ncells, theta, radii, u = sv.seeded_tracks(T, seed=3 + rank)
    tracks = sv.Tracks(ncells, theta, radii, u)
    C, F = tracks.cells, tracks.cells + T
    rk = 1
    wind = lambda r: [r ** -2, 0.4, 0.0, 0.0, 1e-3 * r ** -2]   # noqa: E731
    gin = np.tile(wind(1.0), (rk, T, 1))
    gout = np.tile(wind(1.8), (rk, T, 1))
    dt = 0.5 * tracks.min_spacing()

    def step():
        tracks.advance(dt, gin, gout, rk_order=rk)
        tracks.remesh(2.0, 0.5, 1.0)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    C, F = tracks.cells, tracks.cells + T
    stream = torch.cuda.current_stream()
    # each step reads the new cell count back and allocates the remeshed
    # arrays on the host's side, so one slow host call (an allocator miss)
    # stalls the GPU inside the timed region: the line reports the median of
    # the per-step CUDA-event times (and the mean beside it)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    cells_done = 0
    with ClockSampler(local) as sampler:
        ev[0].record(stream)
        for s_ in range(args.steps):
            cells_done += tracks.cells
            step()
            ev[s_ + 1].record(stream)
        torch.cuda.synchronize()
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    ms = float(np.median(per_step))
    mean_ms = float(np.mean(per_step))
    value = cells_done / args.steps / (ms * 1e-3) * world
    # algorithmic bytes per cell and stage: conserved in and out (2 x 40 B),
    # face radii in and out (2 x 8 B per face)
    peak, kind = measured_peaks()
    Cm = cells_done / args.steps
    achieved = (80.0 * Cm + 16.0 * (Cm + T)) * rk / (ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "whole step (prim, grad, radial, polar, update kernels, then remesh; bound by FP64 recovery and "
                                       "HLLC arithmetic, not by HBM)", "peak_source": f"{kind} hbm_gbs"}
    roof = fp64_roofline("sedov-tracks", Cm, ms, roof)
    extra = {"gpu_launches": (1 + 5 * rk + 3) * args.steps, "clocks": sampler.summary(), "failures": tracks.failure_count(),
             "timing": f"median of {args.steps} per-step CUDA-event times (mean {mean_ms:.3f} ms)"}
    if not args.no_e2e:
        # through the public calls with host buffers: the tracks' state to the
        # GPU, one driver step, the (remeshed) state back, every step
        cap = tracks.cells + (args.steps + 1) * T
        hu = torch.empty(5 * cap, dtype=torch.float64).pin_memory()
        hr = torch.empty(cap + T, dtype=torch.float64).pin_memory()
        n0 = tracks.cells
        hu[: 5 * n0].copy_(tracks.u.reshape(-1).cpu())
        hr[: n0 + T].copy_(tracks.radii.cpu())
        torch.cuda.synchronize()
        h2d = d2h = e2e_cells = 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            n = tracks.cells
            e2e_cells += n
            tracks.u.reshape(-1).copy_(hu[: 5 * n], non_blocking=True)
            tracks.radii.copy_(hr[: n + T], non_blocking=True)
            step()
            m = tracks.cells
            hu[: 5 * m].copy_(tracks.u.reshape(-1), non_blocking=True)
            hr[: m + T].copy_(tracks.radii, non_blocking=True)
            h2d += 48 * n + 8 * T
            d2h += 48 * m + 8 * T
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
        extra["e2e"] = {"value": e2e_cells / args.steps / e2e_s * world, "unit": "cell-updates/s",
                        "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps}
    if rank == 0 and not args.no_cpu_baseline:
        from oracle.oracle import dptr, load_oracle
        o = load_oracle()
        ru, rr = tracks.u.cpu().numpy().T.copy().ravel(), tracks.radii.cpu().numpy().copy()
        th = np.ascontiguousarray(theta.ravel())
        nc = np.ascontiguousarray(tracks.ncells, dtype=np.int64)
        Cb = tracks.cells
        g_in, g_out = np.ascontiguousarray(gin.ravel()), np.ascontiguousarray(gout.ravel())
        o.oracle_sedov_remesh.restype = ctypes.c_int64
        t0 = time.perf_counter()
        o.oracle_sedov_advance_rk(ctypes.c_int32(T), nc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), dptr(th),
                                  dptr(rr), dptr(ru), dptr(g_in), dptr(g_out), ctypes.c_double(dt), ctypes.c_int32(rk),
                                  ctypes.c_int32(1))
        # sedov::remesh track by track, each in a buffer with room for a split
        c0 = 0
        for j in range(T):
            n = int(nc[j])
            rj = np.zeros(n + 2)
            rj[: n + 1] = rr[c0 + j: c0 + j + n + 1]
            uj = np.zeros(5 * (n + 1))
            uj[: 5 * n] = ru[5 * c0: 5 * (c0 + n)]
            o.oracle_sedov_remesh(ctypes.c_int64(n), ctypes.c_double(th[2 * j]), ctypes.c_double(th[2 * j + 1]),
                                  dptr(rj), dptr(uj), ctypes.c_double(2.0), ctypes.c_double(0.5), ctypes.c_double(1.0))
            c0 += n
        el = time.perf_counter() - t0
        extra["cpu_baseline"] = {"value": Cb / el, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                                 "sample": f"one driver step (forward Euler, then remesh of every track) of all {T} "
                                           f"tracks ({Cb} cells), {el:.2f} s, one thread (the reference's sedov:: "
                                           "functions restated)"}
    line = _line(args, world, value, "cell-updates/s", ms, "f64",
                 {"workload": "sedov-tracks-1024", "tracks": T, "cells": C, "rk": rk,
                  "scheme": "PLM(1) + HLLC across contacts, moving radial faces, theta PLM + HLLC on transverse "
                            "faces, spherical sources",
                  "inputs": f"state resident, {(96.0 * C) / 2**20:.0f} MiB read and written per step (below L2, "
                            "no flush: the step is arithmetic-bound)"},
                 roof, extra)
    return line if rank == 0 else None


RUNNERS = {"mhd-128": "run_mhd", "srhd-c2p": "run_srhd", "srhd-tube": "run_tube",
           "minidisk-ensemble-64": "run_ensemble", "sedov-tracks": "run_sedov"}


def compact(line: dict) -> dict:
    """The figures of a workload's line that the headline line carries."""
    keep = ("metric", "value", "unit", "ms_per_step", "dtype", "config", "variants", "accuracy", "max_div_b",
            "failures", "looped_single_mesh", "gpu_launches", "cpu_baseline", "timing")
    out = {k: line[k] for k in keep if line.get(k) is not None}
    if line.get("e2e"):
        out["e2e"] = {k: line["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")}
    roof = line.get("roofline") or {}
    out["roofline"] = {k: roof[k] for k in ("bound", "achieved", "peak", "unit", "frac", "kernel") if k in roof}
    return out


def other_workloads(args) -> dict:
    """Short runs of the other workloads (mixed precision, their own default
    sizes; at most 20 timed steps, one call), each timed as its own --workload run times it, for the headline
    line: the 256^2 minidisk, MHD 128^3, the 2^24-zone SRHD recovery, the
    1024^2 shock tube, the 64-member ensemble and the 1024-track sedov step."""
    import argparse as ap_
    import gc

    import torch
    out = {}
    runners = {"minidisk-256": "run_ours", **RUNNERS}

    def release():
        # device and pinned host memory the earlier runs cached: a later
        # run's pinned buffers otherwise come from whatever is left, and the
        # ensemble's host-buffer line measured 0.8 to 3.3 G cell-updates/s
        # depending on what ran before it
        gc.collect()
        torch.cuda.empty_cache()
        if hasattr(torch._C, "_host_emptyCache"):
            torch._C._host_emptyCache()

    release()
    for name, fn in runners.items():
        sub = ap_.Namespace(**vars(args))
        sub.workload = name
        sub.precision = "mixed"
        sub.steps = min(args.steps, 20)
        sub.warmup = max(args.warmup, 3)
        sub.no_cpu_baseline = name != "sedov-tracks"
        sub.no_looped = False
        sub.launch = None
        sub.accuracy_steps = 100 if name == "minidisk-256" else 50   # the reference-sized disk runs 100 steps
        sub.no_diagnostics_timing = True
        t0 = time.perf_counter()
        line = globals()[fn](sub)
        torch.cuda.synchronize()
        release()
        if line is not None:
            out[name] = compact(line)
            out[name]["wall_s"] = time.perf_counter() - t0
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, _ = dist_info()
    if args.workload in RUNNERS:
        line = globals()[RUNNERS[args.workload]](args)
        if args.workload == "minidisk-ensemble-64":
            finish_replicas(world)
    else:
        line = run_ours(args)
        if (line is not None and args.workload == "minidisk-4096" and world == 1 and not args.no_workloads
                and args.precision == "mixed"):
            line["workloads"] = other_workloads(args)
        finish_replicas(world)
    if line is not None:
        emit(line, rank)


if __name__ == "__main__":
    main()
