"""Benchmark of the MOL right-hand side (PeleC getMOLSrcTerm path) on GB300.

    python bench.py [--gpus N --steps K --warmup W] [--impl gb300|reference]
                    [--workload c4|c2|c1] [--precision fp64] [--no-level] [--no-adjoint]
                    [--no-trajectory] [--no-cpu-baseline] [--no-c2]

One step = one full-level RHS evaluation of the workload (default C4: one
256^3 box of the 9-species premixed flame, FP64).  The value is cell-RHS
evaluations per second over the K timed steps (device-resident inputs, CUDA
events on the launch stream, barrier + synchronize on both sides, max over
ranks).  ``e2e`` repeats the measurement through the public API with the
state copied from pinned host memory and the RHS copied back every step
(double-buffered: the copies of neighbouring steps overlap the kernels).
The mixed-precision form runs on the same box beside it, with its error
against the FP64 result per component.  Under torchrun each rank evaluates
its own box (weak scaling, no data-path collective).  ``c2`` repeats the
FP64 and mixed measurements on the 128^3 box; ``level_c3`` adds the
batched-level measurement (400 uneven boxes: per-box launches vs one batched
launch vs the autotuned tile shape vs a CUDA-graph replay, FP64 and mixed);
both run outside the headline's timed region.  ``--impl reference`` times
the CPU restatement of the reference path (the oracle, pinned bit for bit to
the reference's own code) on the host cores with all threads, each step one
RHS of the same full box.
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

METRIC = "MOL RHS cell-evals/s, 1 GB300: FP64 vs mixed at stated error; adjoint/fwd time"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c4", choices=["c4", "c2", "c1"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64_rcp"],
                    help="FP64 form of the headline: fp64 (every quotient correctly rounded, the oracle's "
                         "arithmetic) or fp64_rcp (quotients by a shared divisor as products with its "
                         "reciprocal); the other form is measured beside it")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-level", action="store_true", help="skip the 400-box batched-level measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint and trajectory-gradient measurement")
    ap.add_argument("--no-trajectory", action="store_true", help="skip the trajectory-gradient measurement only")
    ap.add_argument("--no-c2", action="store_true", help="skip the 128^3 sub-line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(name: str, seed: int = 1):
    from pelec_gb300 import problems

    if name == "c1":
        mech, st = problems.tgv(64, seed=0)
        desc = "C1: Taylor-Green vortex 64^3 periodic, 1 species, GammaLaw, constant transport"
    else:
        n = 256 if name == "c4" else 128
        mech, st, _ = problems.flame((n, n, n), seed=seed)
        desc = ("%s: premixed H2/air flame %d^3, dx=1e-3 cm, 9 species (synthetic NASA-7/transport table), "
                "ideal-mixture EOS, mixture-averaged transport, periodic x/y, foextrap z" % (name.upper(), n))
    return mech, st, desc


def alg_bytes(st) -> int:
    """Algorithmic bytes of one RHS: the stencil footprint (+-2) read once and
    the RHS written once, FP64: 8 NVAR [(nx+4)(ny+4)(nz+4) + nx ny nz]."""
    nx, ny, nz = st.shape
    nvar = st.S.shape[0]
    return 8 * nvar * ((nx + 4) * (ny + 4) * (nz + 4) + nx * ny * nz)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not mhz:
            return None
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(mhz)}


def cpu_baseline(st, cfg, reps: int = 2) -> dict:
    """The oracle (CPU restatement, pinned bit for bit to the reference's own
    code) on the full box of the workload, all threads."""
    from oracle import pyoracle

    threads = pyoracle.max_threads()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        pyoracle.mol_rhs_sub(cfg, st.S, st.begin, st.lo, st.hi, st.dx, nthreads=threads)
        times.append(time.perf_counter() - t0)
    nx, ny, nz = st.shape
    return {"value": st.ncells / statistics.median(times), "unit": "cell-evals/s", "cores": threads, "kind": "port",
            "sample": f"the full {nx}x{ny}x{nz} box of the workload, median of {reps}, OpenMP {threads} threads",
            "best_s": min(times), "median_s": statistics.median(times)}


# Sources that define the FP64 cell and flux kernels whose traffic and
# instruction counts a profile describes, and the unit that compiles them; a
# profile records their hash (with the compile flags of that unit), and a
# figure whose hash no longer matches is reported as stale (null), not used.
PROFILED_SOURCES = ("pelec_gb300/csrc/pc_kernels.cuh", "pelec_gb300/csrc/pc_device.cuh", "pelec_gb300/csrc/pc_exp.h",
                    "pelec_gb300/csrc/pc_exp_tables.h")
PROFILED_UNIT = "pc_mol.cu"


def kernel_source_hash() -> str:
    import hashlib

    from pelec_gb300 import build

    h = hashlib.sha256()
    for f in PROFILED_SOURCES:
        h.update(f.encode())
        h.update(open(os.path.join(ROOT, f), "rb").read())
    flags = [fl for src, fl in build.LIBS["libpelec_mol.so"] if src == PROFILED_UNIT][0]
    h.update(repr((build.ARCH, build.COMMON, PROFILED_UNIT, flags)).encode())
    return h.hexdigest()[:16]


def profile_figures(workload_name: str, form: str, st) -> dict:
    """Per-RHS figures of the committed ncu summary for this FP64 form:
    profiles/dram_traffic_<workload>_<form>.txt when the workload itself was
    captured, else the 128^3 (C2) capture scaled to this box by its count of
    grow(valid, 2) cells, the cells whose records the passes write and read.
    Returns {} when there is none, and the figures with stale=True when the
    kernel sources changed after the capture."""
    out = {}
    for name in (workload_name, "c2"):
        path = os.path.join(ROOT, "profiles", f"dram_traffic_{name}_{form}.txt")
        if os.path.exists(path):
            break
    else:
        return out
    meta = {}
    for ln in open(path):
        if ":" in ln and not ln.startswith("#"):
            k, v = (x.strip() for x in ln.split(":", 1))
            try:
                out[k] = float(v)
            except ValueError:
                meta[k] = v
    nx, ny, nz = st.shape
    cells2 = (nx + 4) * (ny + 4) * (nz + 4)
    scale = cells2 / out.get("captured_grow2_cells", cells2)
    for k in ("dram_bytes_per_rhs", "fp64_flops_per_rhs", "fp64_instructions_per_rhs"):
        if k in out:
            out[k] *= scale
    out["source"] = os.path.relpath(path, ROOT) + ("" if scale == 1 else ", scaled by grow(valid,2) cells x%.4f" % scale)
    out["stale"] = meta.get("source_sha256") != kernel_source_hash()
    return out


def fp_peaks() -> dict:
    """FP64 / FP32 FMA rates measured live (pelec_gb300/_lib/libpc_peaks.so)."""
    import ctypes

    path = os.path.join(ROOT, "pelec_gb300", "_lib", "libpc_peaks.so")
    try:
        lib = ctypes.CDLL(path)
        out = (ctypes.c_double * 2)()
        if lib.pc_measure_fp_rates(out) != 0:
            return {}
        return {"fp64_fma_tflops": out[0], "fp32_fma_tflops": out[1], "source": "pc_peaks.cu, measured in this run"}
    except OSError:
        return {}


def launches_per_rhs(form: str) -> int:
    """Kernel launches of one RHS: the cell and flux passes, and for the
    exact FP64 form each pass's exact twin (which returns at once unless a
    lane of the fast pass needs an IEEE division)."""
    return 4 if form == "fp64" else 2


def fp64_roofline(prof: dict, ms_rhs: float, peaks: dict) -> dict:
    """The roofline that binds: executed FP64 work of one RHS (ncu counters of
    the committed profile, profile_figures) over the two passes' time, against
    the FP64 FMA rate measured in this run."""
    flops, inst = prof.get("fp64_flops_per_rhs"), prof.get("fp64_instructions_per_rhs")
    peak = peaks.get("fp64_fma_tflops")
    if not flops or not peak or prof.get("stale"):
        return {"frac": None, "note": "no current FP64 counts for these kernel sources" if flops else "no profile"}
    achieved = flops / (ms_rhs * 1e-3) / 1e12
    # one FP64 instruction (DFMA, DADD or DMUL) per lane and issue: 2 flops at FMA peak
    issue = inst / (ms_rhs * 1e-3) / (peak * 1e12 / 2.0)
    return {"unit": "TFLOP/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "issue_frac": issue, "flops_per_rhs": flops, "instructions_per_rhs": inst,
            "peak_source": "FP64 FMA loop measured in this run (pc_peaks.cu)",
            "counts_source": "ncu DFMA/DADD/DMUL thread-instruction counters of one RHS (a DFMA counts 2 flops), "
                             + prof.get("source", "")}


def algorithmic_flops(workload_name: str) -> dict:
    """Exact algorithmic FP64 work of one RHS of the workload (flops and
    transcendentals), counted by running the reference's own hot-path code and
    the oracle's EOS and transport with a counting scalar type
    (oracle/count_flops.py -> profiles/algorithmic_flops.txt); {} if absent."""
    path = os.path.join(ROOT, "profiles", "algorithmic_flops.txt")
    out = {}
    if not os.path.exists(path):
        return out
    for ln in open(path):
        if ln.startswith(workload_name + "_") and ":" in ln:
            k, v = (x.strip() for x in ln.split(":", 1))
            out[k[len(workload_name) + 1:]] = float(v)
    return out


def fp64_algorithmic(workload_name: str, ms_rhs: float, peaks: dict) -> dict:
    """The algorithm's FP64 flops of one RHS over the RHS time against the
    FP64 FMA rate measured in this run (the executed counts of fp64_roofline
    also hold the extra instructions of divisions, square roots and
    exponentials)."""
    a = algorithmic_flops(workload_name)
    peak = peaks.get("fp64_fma_tflops")
    if not a or not peak:
        return {"frac": None, "note": "no algorithmic count for this workload"}
    achieved = a["flops_per_rhs"] / (ms_rhs * 1e-3) / 1e12
    return {"unit": "TFLOP/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "flops_per_rhs": a["flops_per_rhs"], "flops_per_cell": a["flops_per_cell"],
            "transcendentals_per_cell": a["transcendentals_per_cell"],
            "counts_source": "profiles/algorithmic_flops.txt (oracle/count_flops.py: the reference's hot-path code "
                             "and the oracle's EOS/transport run with a counting double; add+mul+div+sqrt+2 fma)"}


def fp32_algorithmic(workload_name: str, ms_rhs: float, peaks: dict) -> dict:
    """The same algorithmic flop count over a mixed-precision RHS time,
    against the FP32 FMA rate measured in this run: where the mixed forms
    stand on the FP32 roof.  They execute more FP32 instructions than the
    count (double-float arithmetic takes several per operation; the FP64
    Newton solve and divergence of PC_PRECISION_MIXED_FP64 are on the FP64
    pipe), and their passes are bound by issue and latency, not by the FP32
    pipe (profiles/flux_kernel_mixed_c2.md, cell_kernel_mixed_c2.md)."""
    a = algorithmic_flops(workload_name)
    peak = peaks.get("fp32_fma_tflops")
    if not a or not peak:
        return {"frac": None, "note": "no algorithmic count for this workload"}
    achieved = a["flops_per_rhs"] / (ms_rhs * 1e-3) / 1e12
    return {"unit": "TFLOP/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "flops_per_rhs": a["flops_per_rhs"], "peak_source": "FP32 FMA loop measured in this run (pc_peaks.cu)",
            "counts_source": "profiles/algorithmic_flops.txt"}


def launch_name(t: int) -> str:
    """'8x8x4', or '8x8x4/persistent', for flux-pass launch configuration t."""
    from pelec_gb300 import abi, mol

    name = "x".join(map(str, mol.MOLOperator.tile_shape(t)[:3]))
    return name + "/persistent" if t >= abi.PC_LAUNCH_PERSISTENT else name


def bench_level(args, rank: int, local: int, maxover, barrier) -> dict:
    """C3: 400 uneven boxes (edges from {8,16,24,32,48,64} per axis, seeded),
    9 species.  Times one RHS of the whole level per step as (a) one launch per
    box and pass, (b) one batched launch per pass at the default tile shape,
    (c) batched at the autotuned shape, (d) a CUDA-graph replay of (c), for
    FP64 and for mixed precision; plus the oracle on a sample of the boxes."""
    import numpy as np
    import torch

    from pelec_gb300 import mol, problems

    mech, boxes = problems.level_boxes(400, seed=3 + 1000 * rank)
    cells = sum(b.ncells for b in boxes)
    S = mol.MultiFab([(b.lo, b.hi) for b in boxes], boxes[0].S.shape[0], boxes[0].ng,
                     fabs=[torch.from_numpy(b.S).cuda() for b in boxes])
    R = mol.MultiFab(S.boxes, S.ncomp, 0)
    dx = boxes[0].dx
    stream = torch.cuda.current_stream()
    steps = max(1, min(args.steps, 10))

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        barrier()
        return maxover(e0.elapsed_time(e1) / 1e3) / steps

    out = {"workload": "C3: %d boxes, edges per axis from {8,16,24,32,48,64} (seeded), %d cells, 9-species flame "
                       "at per-box seeded offsets" % (len(boxes), cells),
           "cells": cells, "steps": steps, "unit": "cell-evals/s"}
    ref = None
    for prec, name in ((abi_precision(0), "fp64"), (abi_precision(1), "mixed")):
        op = mol.MOLOperator(problems.make_config(mech, precision=prec))
        res = {}
        t_per_box = timed(lambda: op.rhs_level(S, R, dx, per_box=True))
        op.set_tile(0)
        t_default = timed(lambda: op.rhs_level(S, R, dx))
        op.set_tile(-1)
        best, ms = op.autotune(S, R, dx, reps=3)
        t_tuned = timed(lambda: op.rhs_level(S, R, dx))
        torch.cuda.synchronize()
        r = [t.cpu().numpy() for t in R.fabs]
        g = op.graph(S, R, dx)
        t_graph = timed(g.launch)
        g.close()
        nl = launches_per_rhs(name)
        res["per_box"] = {"value": cells / t_per_box, "ms_per_step": 1e3 * t_per_box,
                          "gpu_launches_per_step": nl * len(boxes)}
        res["batched_default_tile"] = {"value": cells / t_default, "ms_per_step": 1e3 * t_default,
                                       "tile": mol.MOLOperator.tile_shape(0), "gpu_launches_per_step": nl}
        res["batched_autotuned"] = {"value": cells / t_tuned, "ms_per_step": 1e3 * t_tuned,
                                    "launch": launch_name(best), "gpu_launches_per_step": nl,
                                    "autotune_ms_per_launch": {launch_name(t): v for t, v in enumerate(ms)}}
        res["graph"] = {"value": cells / t_graph, "ms_per_step": 1e3 * t_graph, "gpu_launches_per_step": nl,
                        "note": "one cudaGraphLaunch of the autotuned batched RHS"}
        res["speedup_graph_vs_per_box"] = t_per_box / t_graph
        if prec == 0:
            ref = r
        else:
            num = np.zeros(S.ncomp)
            den = np.zeros(S.ncomp)
            for a, b in zip(r, ref):
                num += ((a - b) ** 2).sum(axis=(1, 2, 3))
                den += (b ** 2).sum(axis=(1, 2, 3))
            l2 = np.sqrt(num / np.maximum(den, 1e-300))
            res["rel_l2_vs_fp64"] = {"max": float(l2.max()), "per_component": [float(v) for v in l2]}
        out[name] = res
        op.close()
    out["mixed_speedup_vs_fp64_graph"] = out["fp64"]["graph"]["ms_per_step"] / out["mixed"]["graph"]["ms_per_step"]
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import pyoracle

        cfg = problems.make_config(mech)
        sample = boxes[:40]
        ncs = sum(b.ncells for b in sample)
        t0 = time.perf_counter()
        pyoracle.mol_rhs(cfg, sample, nthreads=pyoracle.max_threads())
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": ncs / dt, "unit": "cell-evals/s", "cores": pyoracle.max_threads(),
                               "kind": "port", "sample": f"first 40 of the 400 boxes ({ncs} cells), one pass"}
    del S, R
    torch.cuda.empty_cache()
    return out


def bench_sub_box(args, name: str, rank: int, maxover, barrier, nspec: int = 9) -> dict:
    """FP64 and mixed RHS of another single-box workload (device-resident,
    autotuned launch), with the mixed form's error against the FP64 result.
    nspec = 21: the same flame with the synthetic 21-species mechanism."""
    import numpy as np
    import torch

    from pelec_gb300 import abi, mechanism, mol, problems

    if nspec == 21:
        n = 128 if name == "c2" else 256
        mech, st, _ = problems.flame((n, n, n), seed=1 + rank, mech=mechanism.drm_synthetic())
        desc = (f"{name.upper()} geometry ({n}^3 flame) with 21 species (synthetic table in DRM19 species order): "
                "the kernels instantiated for NUM_SPECIES = 21")
    else:
        mech, st, desc = workload(name, seed=1 + rank)
    S = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], st.ng, fabs=[torch.from_numpy(st.S).cuda()])
    R = mol.MultiFab(S.boxes, S.ncomp, 0)
    stream = torch.cuda.current_stream()
    out = {"workload": desc, "cells": st.ncells, "steps": args.steps, "unit": "cell-evals/s"}
    res = {}
    for prec, form in ((abi.PC_PRECISION_FP64, "fp64"), (abi.PC_PRECISION_MIXED, "mixed"),
                       (abi.PC_PRECISION_MIXED_FP64, "mixed_fp64_split")):
        op = mol.MOLOperator(problems.make_config(mech, time_passes=1, precision=prec))
        best, tune_ms = op.autotune(S, R, st.dx, reps=3)
        for _ in range(max(3, args.warmup)):
            op.rhs_level(S, R, st.dx)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            op.rhs_level(S, R, st.dx)
        e1.record(stream)
        barrier()
        t = maxover(e0.elapsed_time(e1) / 1e3) / args.steps
        op.rhs_level(S, R, st.dx)
        torch.cuda.synchronize()
        res[form] = R.fabs[0].cpu().numpy()
        out[form] = {"value": st.ncells / t, "ms_per_step": 1e3 * t, "flux_launch": launch_name(best),
                     "autotune_ms_per_launch": {launch_name(q): v for q, v in enumerate(tune_ms)},
                     "gpu_launches_per_step": launches_per_rhs(form)}
        op.close()
    b = res["fp64"]
    for form in ("mixed", "mixed_fp64_split"):
        a = res[form]
        l2 = [float(np.sqrt(((a[n] - b[n]) ** 2).sum() / max((b[n] ** 2).sum(), 1e-300))) for n in range(b.shape[0])]
        out[form]["rel_l2_vs_fp64"] = {"max": max(l2), "per_component": l2}
        out[form]["speedup_vs_fp64"] = out["fp64"]["ms_per_step"] / out[form]["ms_per_step"]
    del S, R
    torch.cuda.empty_cache()
    return out


def bench_step_graph(args, rank: int, maxover, barrier) -> dict:
    """One SSP-RK2 step of a 64^3 flame box (periodic x/y, outflow z, FP64):
    the host-driven sequence of nine library calls (advance.ssprk2_step)
    against one CUDA-graph replay per step (advance.Stepper), K steps each,
    CUDA events on the launch stream (host gaps between launches included)."""
    import numpy as np
    import torch

    from pelec_gb300 import abi, advance, mol, problems

    mech, st, _ = problems.flame((64, 64, 64), seed=5 + rank)
    geom = abi.geometry(st.lo, st.hi, (0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW))
    op = mol.MOLOperator(problems.make_config(mech))
    mk = lambda: mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], st.ng, fabs=[torch.from_numpy(st.S.copy()).cuda()])
    S_old, S_new, R = mk(), mk(), mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    op.fill_ghosts(S_old, geom)
    dt = op.est_dt(S_old, st.dx, 0.3)
    stepper = advance.Stepper(op, mk(), mk(), mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0), geom, st.dx)
    stream = torch.cuda.current_stream()
    steps = max(5, args.steps)

    def host_step():
        nonlocal S_old, S_new
        advance.ssprk2_step(op, S_old, S_new, R, geom, st.dx, dt)
        S_old, S_new = S_new, S_old

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        barrier()
        return maxover(e0.elapsed_time(e1)) / steps

    t_host = timed(host_step)
    t_graph = timed(lambda: stepper.step(dt))
    torch.cuda.synchronize()
    same = bool(np.isfinite(stepper.state.fabs[0].cpu().numpy()).all())
    stepper.close()
    op.close()
    return {"workload": "one SSP-RK2 step (2 fills, 2 RHS, 3 LinComb, 2 computeTemp) of a 64^3 flame box, "
                        "9 species, FP64, periodic x/y, outflow z", "steps": steps,
            "host_driven_ms_per_step": t_host, "graph_ms_per_step": t_graph, "speedup": t_host / t_graph,
            "finite": same, "cells": st.ncells,
            "graph": "pc_mol_step_graph: both directions of the state pair captured once, dt written to a device "
                     "scalar before each replay"}


def bench_adjoint_rhs(args, st, mech, S, maxover, barrier) -> dict:
    """Adjoint (VJP) and tangent (JVP) of one RHS on the headline box, timed
    like the RHS itself: ms per call with CUDA events, and the ratio to the
    forward RHS (the metric's adjoint/forward time)."""
    import numpy as np
    import torch

    from pelec_gb300 import mol, problems

    op = mol.MOLOperator(problems.make_config(mech))
    R = mol.MultiFab(S.boxes, S.ncomp, 0)
    Rb = mol.MultiFab(S.boxes, S.ncomp, 0,
                      fabs=[torch.from_numpy(np.random.default_rng(5).normal(size=R.fabs[0].shape)).cuda()])
    Ub = mol.MultiFab(S.boxes, S.ncomp, 2)
    Sd = mol.MultiFab(S.boxes, S.ncomp, 2)
    Sd.fabs[0].copy_(S.fabs[0][:, 2:-2, 2:-2, 2:-2] * 1e-3)
    Rd = mol.MultiFab(S.boxes, S.ncomp, 0)
    stream = torch.cuda.current_stream()
    steps = max(3, min(args.steps, 10))

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        barrier()
        return maxover(e0.elapsed_time(e1)) / steps

    t_rhs = timed(lambda: op.rhs_level(S, R, st.dx))
    t_vjp = timed(lambda: op.rhs_vjp(S, Rb, Ub, st.dx))
    t_jvp = timed(lambda: op.rhs_jvp(S, Sd, R, Rd, st.dx))
    op.close()
    return {"workload": "the headline box", "ms_rhs": t_rhs, "ms_vjp": t_vjp, "ms_jvp": t_jvp,
            "vjp_over_rhs": t_vjp / t_rhs, "jvp_over_rhs": t_jvp / t_rhs, "steps": steps,
            "vjp": "hand-written reverse mode: record pass + face adjoint + cell adjoint (IFT for the T solve)",
            "jvp": "forward passes instantiated with dual numbers"}


def bench_trajectory(args, rank: int) -> dict:
    """C5: 64^3 flame, 9 species, FP64; J = sum(T dV) after 50 SSP-RK2 steps
    at CFL 0.3 (time steps frozen, those of the oracle's base trajectory);
    gradient by the checkpointed adjoint (every 5 steps).  Times the forward
    trajectory (one step-graph replay per step) and the gradient, records the
    device memory, and checks the gradient against (a) central differences of
    the ORACLE's CPU trajectory on 20 seeded state directions, h = 1e-6
    relative, and Richardson differences in the first three wrinkle
    amplitudes (tests/golden/c5_fd.npz, made by tests/golden/make_c5_fd.py),
    and (b) the forward-mode tangent of the GPU trajectory along the same
    directions."""
    import dataclasses
    import time

    import numpy as np
    import torch

    from pelec_gb300 import abi, mol, problems, trajectory

    path = os.path.join(ROOT, "tests", "golden", "c5_fd.npz")
    fx = np.load(path)
    nsteps, every = int(fx["nsteps"]), 5
    shape = tuple(int(v) for v in fx["shape"])
    out = {"workload": "C5: 64^3 premixed flame, 9 species, FP64, 50 SSP-RK2 steps at CFL 0.3, "
                       "J = sum(T dV) at step 50, checkpoint every 5", "nsteps": nsteps, "every": every,
           "fd_reference": "central differences of the oracle's CPU trajectory (pinned bit for bit to the "
                           "reference's own hot-path code), tests/golden/c5_fd.npz"}

    def direction(st, s):
        v = torch.from_numpy(s[:, None, None, None] * st.S).cuda()
        for ax in (1, 2, 3):
            v.narrow(ax, 0, 4).zero_()
            v.narrow(ax, v.shape[ax] - 4, 4).zero_()
        return v

    def case(tag, w_noise, ntan, with_params):
        mech, st, fp = problems.flame(shape, seed=int(fx["seed"]), w_noise=w_noise)
        op = mol.MOLOperator(problems.make_config(mech))
        S0 = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 4, fabs=[torch.from_numpy(st.S).cuda()])
        geom = abi.geometry(st.lo, st.hi, (0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW))
        tr = trajectory.Trajectory(op, S0, geom, st.dx)
        dts = [float(v) for v in fx[f"{tag}_dts"]]
        tr.run(S0, dts, every)  # warm-up (graphs, layouts, uploads)
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base_alloc = torch.cuda.memory_allocated()  # tensors of the rest of the bench still alive
        fwd = []
        for _ in range(3):
            t0 = time.perf_counter()
            final, _ = tr.run(S0, dts, every)
            J = tr.objective(final)
            fwd.append(time.perf_counter() - t0)
            del final
        t_fwd = min(fwd)
        t0 = time.perf_counter()
        J2, L = tr.gradient(S0, dts, every)
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        free1, total = torch.cuda.mem_get_info()
        res = {"J": J, "J_oracle": float(fx[f"{tag}_J0"]), "forward_s": t_fwd, "forward_s_runs": fwd,
               "gradient_s": t_grad, "adjoint_sweep_s": t_grad - t_fwd, "gradient_over_forward": t_grad / t_fwd,
               "adjoint_sweep_over_forward": (t_grad - t_fwd) / t_fwd,
               "peak_torch_bytes": int(torch.cuda.max_memory_allocated() - base_alloc),
               "device_bytes_in_use_after_gradient": int(total - free1), "dt_first_last": [dts[0], dts[-1]]}
        h = float(fx["h_state"])
        fd_err, tan_err, t_tan = [], [], []
        for d, s in enumerate(fx[f"{tag}_scales"]):
            v = direction(st, s)
            ad = float((L.fabs[0] * v).sum())
            fd = (float(fx[f"{tag}_Jp"][d]) - float(fx[f"{tag}_Jm"][d])) / (2 * h)
            fd_err.append(abs(fd - ad) / abs(ad))
            if d < ntan:
                t0 = time.perf_counter()
                _, tan = tr.tangent(S0, dts, mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[v]))
                t_tan.append(time.perf_counter() - t0)
                tan_err.append(abs(tan - ad) / abs(ad))
        res["fd_state_directions"] = {"n": len(fd_err), "h": h, "max_rel_err": max(fd_err),
                                      "median_rel_err": float(np.median(fd_err)), "rel_err": fd_err,
                                      "direction": "each conserved component scaled by a seeded N(0,1) factor"}
        res["tangent_state_directions"] = {"n": len(tan_err), "max_rel_err": max(tan_err),
                                           "tangent_s": float(np.median(t_tan)),
                                           "note": "forward mode through the whole trajectory (dual-number RHS)"}
        if with_params:
            lam = L.fabs[0].cpu().numpy()
            ha = float(fx["h_amp"])
            perr = []
            for m in range(3):
                def U0(amps):
                    return problems.flame(shape, seed=int(fx["seed"]), w_noise=w_noise,
                                          params=dataclasses.replace(fp, amps=amps))[1].S
                hg = 1e-3 * max(fp.amps[m], 1e-6)
                e = hg * (np.arange(len(fp.amps)) == m)
                dU = (U0(fp.amps + e) - U0(fp.amps - e)) / (2 * hg)
                ad = float((lam * dU).sum())
                _, tan = tr.tangent(S0, dts, mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[torch.from_numpy(dU).cuda()]))
                dJ1, dJ2 = (float(x) for x in fx["config_dJamp"][m])
                fd, fd2 = dJ1 / (2 * ha), dJ2 / (4 * ha)
                perr.append({"mode": m, "amplitude_cm": float(fp.amps[m]), "h_cm": ha, "adjoint": ad, "tangent": tan,
                             "fd_central": fd, "rel_err_fd": abs(fd - ad) / abs(ad),
                             "rel_err_fd_twice_the_step": abs(fd2 - ad) / abs(ad),
                             "rel_err_tangent": abs(tan - ad) / abs(ad)})
            res["wrinkle_amplitudes"] = perr
        op.close()
        del S0, L
        torch.cuda.empty_cache()
        return res

    out["config_state"] = case("config", 0.0, 20, True)
    out["config_state"]["note"] = ("p and w uniform up to rounding: the limiter's acoustic slopes and the slopes of w "
                                   "are evaluated at rounding-size arguments, so a finite step crosses its switches; "
                                   "the tangent follows the adjoint's branches")
    out["w_noise_state"] = case("wnoise", 1.0, 5, False)
    out["w_noise_state"]["note"] = "same state with seeded N(0, 1 cm/s) noise on w, as on u and v"
    return out


FORM_NOTE = {
    "fp64": "every operation FP64, every quotient correctly rounded: the oracle's arithmetic bit for bit",
    "fp64_rcp": "every operation FP64; quotients by a divisor shared by several numerators taken as products "
                "with its correctly rounded reciprocal (within one ulp of the correctly rounded quotient)",
}


def abi_precision(mixed: int) -> int:
    from pelec_gb300 import abi

    return abi.PC_PRECISION_MIXED if mixed else abi.PC_PRECISION_FP64


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import build as ob

    ob.build()
    from pelec_gb300 import problems

    mech, st, desc = workload(args.workload)
    cfg = problems.make_config(mech)
    for _ in range(args.warmup):
        cpu_baseline(st, cfg, reps=1)
    vals, meds = [], []
    t0 = time.perf_counter()
    res = None
    for _ in range(args.steps):
        res = cpu_baseline(st, cfg, reps=1)
        vals.append(res["value"])
        meds.append(res["median_s"])
    elapsed = time.perf_counter() - t0
    value = statistics.median(vals)
    cb = {"value": value, "unit": "cell-evals/s", "cores": res["cores"], "kind": "port",
          "sample": res["sample"].replace("median of 1", f"median of {args.steps} steps")}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "boxes_per_gpu": 1, "cells_per_gpu": st.ncells, "nspec": mech.nspec,
                       "precision": "fp64", "implementation":
                       "CPU restatement of getMOLSrcTerm (oracle/), pinned bit for bit to the reference's own "
                       "hot-path code compiled from its sources (oracle/ref_build.py); the reference's full build "
                       "(AMReX, PelePhysics, SUNDIALS) cannot be compiled here"},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "cell-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        pg = dist

    from pelec_gb300 import build as cb

    cb.build()
    from pelec_gb300 import mol, problems

    from pelec_gb300 import abi

    mech, st, desc = workload(args.workload, seed=1 + rank)
    forms = {"fp64": abi.PC_PRECISION_FP64, "fp64_rcp": abi.PC_PRECISION_FP64_RCP}
    other = "fp64" if args.precision == "fp64_rcp" else "fp64_rcp"
    cfg = problems.make_config(mech, time_passes=1, precision=forms[args.precision])
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import build as ob

        ob.build()
        cpu = cpu_baseline(st, problems.make_config(mech))

    op = mol.MOLOperator(cfg)
    S_h = torch.from_numpy(np.ascontiguousarray(st.S)).pin_memory()
    S = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], st.ng, fabs=[S_h.cuda()])
    R = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    R_h = torch.empty(R.fabs[0].shape, dtype=torch.float64).pin_memory()
    stream = torch.cuda.current_stream()
    cells = st.ncells

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    def maxover(x: float) -> float:
        if pg is None:
            return x
        t = torch.tensor([x], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        return float(t.item())

    def timed_steps(o, with_clocks=False):
        """K device-resident steps; returns (seconds, clock record)."""
        for _ in range(max(3, args.warmup)):
            o.rhs_level(S, R, st.dx)
        clocks = ClockSampler(local) if with_clocks else None
        if clocks:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            o.rhs_level(S, R, st.dx)
        e1.record(stream)
        barrier()
        clk = clocks.stop() if clocks else None
        return maxover(e0.elapsed_time(e1) / 1e3), clk

    def pass_times(o):
        tc, tf = [], []
        for _ in range(args.steps):
            o.rhs_level(S, R, st.dx)
            a, b = o.pass_times()
            tc.append(a)
            tf.append(b)
        return statistics.mean(tc), statistics.mean(tf)

    # Launch configuration of the flux pass: the autotuner's choice for this
    # BoxArray (setup, outside the timed region, as a user would run it).
    best, tune_ms = op.autotune(S, R, st.dx, reps=3)
    t_dev, clk = timed_steps(op, with_clocks=True)
    ms_cell, ms_flux = pass_times(op)
    status = op.status()
    # The headline RHS and the scale of the flux differences it is made of
    # (max over faces of |F_n| / V per component): the measure of round-off.
    Fx = op.rhs_level_fluxes(S, R, st.dx)[0]
    torch.cuda.synchronize()
    r64 = R.fabs[0].cpu().numpy()
    flux_scale = np.max([f.abs().amax(dim=(1, 2, 3)).cpu().numpy() for f in Fx], axis=0) / float(np.prod(st.dx))
    del Fx
    # End to end through the public API: every step copies its state from
    # pinned host memory, evaluates the RHS and copies the RHS back.  Two
    # device buffer pairs and separate upload/download streams let step k+1's
    # upload and step k's download run under step k's kernels.
    S2 = mol.MultiFab(S.boxes, S.ncomp, S.ngrow)
    R2 = mol.MultiFab(R.boxes, R.ncomp, 0)
    R_h2 = torch.empty_like(R_h).pin_memory()
    Sb, Rb_, Rh = [S, S2], [R, R2], [R_h, R_h2]
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    loaded = [torch.cuda.Event(), torch.cuda.Event()]
    computed = [torch.cuda.Event(), torch.cuda.Event()]
    freed = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_steps(n):
        for k in range(n):
            b = k % 2
            with torch.cuda.stream(up):
                if k >= 2:
                    up.wait_event(computed[b])  # the previous user of buffer b has read its state
                Sb[b].fabs[0].copy_(S_h, non_blocking=True)
                loaded[b].record(up)
            stream.wait_event(loaded[b])
            if k >= 2:
                stream.wait_event(freed[b])  # its previous RHS has been downloaded
            op.rhs_level(Sb[b], Rb_[b], st.dx, stream=stream)
            computed[b].record(stream)
            with torch.cuda.stream(down):
                down.wait_event(computed[b])
                Rh[b].copy_(Rb_[b].fabs[0], non_blocking=True)
                freed[b].record(down)

    e2e_steps(2)  # warm-up of the second buffer pair (layout, box table)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    up.wait_event(e0)
    e2e_steps(args.steps)
    stream.wait_stream(up)
    stream.wait_stream(down)
    e1.record(stream)
    barrier()
    t_e2e = maxover(e0.elapsed_time(e1) / 1e3)
    del S2, R2

    # the other FP64 form on the same state, error against the headline form
    opo = mol.MOLOperator(problems.make_config(mech, time_passes=1, precision=forms[other]))
    best_o, tune_ms_o = opo.autotune(S, R, st.dx, reps=3)
    t_oth, _ = timed_steps(opo)
    ms_cell_o, ms_flux_o = pass_times(opo)
    opo.rhs_level(S, R, st.dx)
    torch.cuda.synchronize()
    r_oth = R.fabs[0].cpu().numpy()
    mx_o = [float(np.abs(r_oth[n] - r64[n]).max() / max(np.abs(r64[n]).max(), 1e-300)) for n in range(r64.shape[0])]
    fs_o = [float(np.abs(r_oth[n] - r64[n]).max() / max(flux_scale[n], 1e-300)) for n in range(r64.shape[0])]
    opo.close()

    # mixed precision on the same state, error against the FP64 result
    opm = mol.MOLOperator(problems.make_config(mech, time_passes=1, precision=1))
    best_m, tune_ms_m = opm.autotune(S, R, st.dx, reps=3)
    t_mix, _ = timed_steps(opm)
    ms_cell_m, ms_flux_m = pass_times(opm)
    opm.rhs_level(S, R, st.dx)
    torch.cuda.synchronize()
    r32 = R.fabs[0].cpu().numpy()
    l2 = [float(np.sqrt(((r32[n] - r64[n]) ** 2).sum() / max((r64[n] ** 2).sum(), 1e-300))) for n in range(r64.shape[0])]
    mx = [float(np.abs(r32[n] - r64[n]).max() / max(np.abs(r64[n]).max(), 1e-300)) for n in range(r64.shape[0])]
    fs_m = [float(np.abs(r32[n] - r64[n]).max() / max(flux_scale[n], 1e-300)) for n in range(r64.shape[0])]

    opm.close()

    # the same with the Newton solve, cell mass fractions and divergence in FP64
    ops = mol.MOLOperator(problems.make_config(mech, time_passes=1, precision=abi.PC_PRECISION_MIXED_FP64))
    best_s, tune_ms_s = ops.autotune(S, R, st.dx, reps=3)
    t_mix_s, _ = timed_steps(ops)
    ms_cell_s, ms_flux_s = pass_times(ops)
    ops.rhs_level(S, R, st.dx)
    torch.cuda.synchronize()
    r32s = R.fabs[0].cpu().numpy()
    l2_s = [float(np.sqrt(((r32s[n] - r64[n]) ** 2).sum() / max((r64[n] ** 2).sum(), 1e-300)))
            for n in range(r64.shape[0])]
    mx_s = [float(np.abs(r32s[n] - r64[n]).max() / max(np.abs(r64[n]).max(), 1e-300)) for n in range(r64.shape[0])]
    ops.close()
    sub = sub21 = None
    if args.workload != "c2" and not args.no_c2:
        sub = bench_sub_box(args, "c2", rank, maxover, barrier)
    if not args.no_c2:
        sub21 = bench_sub_box(args, "c2", rank, maxover, barrier, nspec=21)
    stepg = None if args.no_level else bench_step_graph(args, rank, maxover, barrier)
    level = None if args.no_level else bench_level(args, rank, local, maxover, barrier)
    adj = None if args.no_adjoint else bench_adjoint_rhs(args, st, mech, S, maxover, barrier)
    traj = None if (args.no_adjoint or args.no_trajectory or rank != 0) else bench_trajectory(args, rank)

    if rank != 0:
        if pg is not None:
            pg.destroy_process_group()
        return 0
    value = world * cells * args.steps / t_dev
    ms_rhs = ms_cell + ms_flux
    ab = alg_bytes(st)
    import json as _json

    peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    # the measured copy bandwidth of the GB300s, else the stated
    # fallback (6.8 TB/s, one earlier GB300 measurement), labelled as such
    hbm_peak = peaks.get("hbm_gbs")
    hbm_source = "MEASURED_PEAKS.json hbm_gbs (of measured)"
    if not hbm_peak:
        hbm_peak = 6800.0
        hbm_source = "fallback 6.8 TB/s, MEASURED_PEAKS.json absent (of fallback)"
    achieved = ab / (ms_rhs * 1e-3) / 1e9
    prof = profile_figures(args.workload, args.precision, st)
    traffic = None if prof.get("stale", True) else prof.get("dram_bytes_per_rhs")
    peaks_fp = fp_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": "cell-evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "boxes_per_gpu": 1, "cells_per_gpu": cells, "nspec": mech.nspec,
                   "precision": args.precision, "precision_note": FORM_NOTE[args.precision],
                   "l2": "inputs larger than L2 (state %.0f MB, scratch records %.0f MB)" % (
                       st.S.nbytes / 1e6, cells * (13 + 4 * mech.nspec) * 8 * 1.1 / 1e6),
                   "flux_launch": launch_name(best),
                   "autotune_ms_per_launch": {launch_name(t): v for t, v in enumerate(tune_ms)}},
        "e2e": {"value": world * cells * args.steps / t_e2e, "unit": "cell-evals/s",
                "h2d_bytes_per_step": int(S_h.numel() * 8), "d2h_bytes_per_step": int(R_h.numel() * 8)},
        "gpu_launches": launches_per_rhs(args.precision) * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "traffic_source": (prof.get("source", "no profile") +
                                        ("; STALE: the kernel sources changed after the capture"
                                         if prof.get("stale") else "; kernel-source hash matches")),
                     "kernel": "cell_kernel + flux_kernel (one RHS)",
                     "alg_bytes_per_rhs": ab, "peak_source": hbm_source,
                     "binding_resource": "FP64 pipe",
                     "fp64": fp64_roofline(prof, ms_rhs, peaks_fp),
                     "fp64_algorithmic": fp64_algorithmic(args.workload, ms_rhs, peaks_fp),
                     "fp64_pipe_active_pct": {"flux_kernel": prof.get("fp64_pipe_active_pct_flux_kernel"),
                                              "cell_kernel": prof.get("fp64_pipe_active_pct_cell_kernel"),
                                              "source": "ncu, " + prof.get("source", "no profile")},
                     "fp_peaks": peaks_fp},
        "passes_ms": {"cell_kernel": ms_cell, "flux_kernel": ms_flux},
        other: {"value": world * cells * args.steps / t_oth, "unit": "cell-evals/s",
                "ms_per_step": 1e3 * t_oth / args.steps, "passes_ms": {"cell_kernel": ms_cell_o, "flux_kernel": ms_flux_o},
                "flux_launch": launch_name(best_o),
                "autotune_ms_per_launch": {launch_name(t): v for t, v in enumerate(tune_ms_o)},
                "rel_max_vs_headline": {"max": max(mx_o), "per_component": mx_o},
                "flux_scaled_max_vs_headline": {"max": max(fs_o), "per_component": fs_o,
                                                "scale": "max over faces of |F_n| / V per component"},
                "precision_note": FORM_NOTE[other]},
        "mixed": {"value": world * cells * args.steps / t_mix, "unit": "cell-evals/s",
                  "ms_per_step": 1e3 * t_mix / args.steps, "speedup_vs_fp64": t_dev / t_mix,
                  "passes_ms": {"cell_kernel": ms_cell_m, "flux_kernel": ms_flux_m},
                  "flux_launch": launch_name(best_m),
                  "autotune_ms_per_launch": {launch_name(t): v for t, v in enumerate(tune_ms_m)},
                  "rel_l2_vs_fp64": {"max": max(l2), "per_component": l2},
                  "rel_max_vs_fp64": {"max": max(mx), "per_component": mx},
                  "flux_scaled_max_vs_fp64": {"max": max(fs_m), "per_component": fs_m},
                  "fp32_algorithmic": fp32_algorithmic(args.workload, 1e3 * t_mix / args.steps, peaks_fp),
                  "precision": "PC_PRECISION_MIXED: FP32 reconstruction/Riemann/diffusion; Newton, cell mass "
                               "fractions, Godunov energy and divergence in double-float (~48 bits, FP32 pipe)"},
        "mixed_fp64_split": {"value": world * cells * args.steps / t_mix_s, "unit": "cell-evals/s",
                             "ms_per_step": 1e3 * t_mix_s / args.steps, "speedup_vs_fp64": t_dev / t_mix_s,
                             "passes_ms": {"cell_kernel": ms_cell_s, "flux_kernel": ms_flux_s},
                             "flux_launch": launch_name(best_s),
                             "autotune_ms_per_launch": {launch_name(t): v for t, v in enumerate(tune_ms_s)},
                             "rel_l2_vs_fp64": {"max": max(l2_s), "per_component": l2_s},
                             "rel_max_vs_fp64": {"max": max(mx_s), "per_component": mx_s},
                             "fp32_algorithmic": fp32_algorithmic(args.workload, 1e3 * t_mix_s / args.steps,
                                                                  peaks_fp),
                             "precision": "PC_PRECISION_MIXED_FP64: as mixed, with the Newton solve, the cell mass "
                                          "fractions and the divergence accumulation in FP64"},
        "gpu_launches_mixed": launches_per_rhs("mixed") * args.steps,
        "status": {"cells": status.cells, "newton_nonconverged": status.newton_nonconverged,
                   "nonpositive_state": status.nonpositive_state, "nonfinite_output": status.nonfinite_output,
                   "exact_recomputes": status.exact_recomputes},
        "clocks": clk,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if sub is not None:
        line["c2"] = sub
    if sub21 is not None:
        line["c2_21_species"] = sub21
    if stepg is not None:
        line["step_graph"] = stepg
    if level is not None:
        line["level_c3"] = level
    if adj is not None:
        line["adjoint"] = adj
    if traj is not None:
        line["trajectory_c5"] = traj
    print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
