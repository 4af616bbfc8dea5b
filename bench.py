#!/usr/bin/env python3
"""miniAMR hot path on GB300: cell-variable updates/s and HBM roofline.

Workload (the precision variant of the uniform 4096-block mesh): 8x8x8
initial blocks of 16^3 cells uniformly refined once -> 4096 blocks, 40
variables, 27-point stencil, 4 stages per timestep, checksum every 5th
stage (the reference's default cadence), initial values from the
reference's init().  One step = one timestep (4 stages of comm + stencil
over every block and variable, checksums on stage 0).

Headline `value`: the batched FP32 path (one fused ghost+stencil+checksum
launch per stage, CUDA graph) with the pool resident in HBM (3.4 GB of
interior FP32 cells -- far larger than L2, so no flush is needed).  `e2e`:
the same run through the C ABI from pinned host buffers -- the initial
blocks uploaded, refined on the device, stepped, checksums read back every
step.  Also reported (`paths`): the plain FP64 path (bit-exact with the
reference), the batched FP64 path and the plain FP32 path, each timed with
CUDA events over the same timesteps; and (`fp32_checksum_error`) the max /
RMS relative error of every FP32 checksum against the plain FP64 path's
checksums of the same stages (that path is bit-exact with the reference's
code on this mesh: tests/test_gpu_benchmark_mesh.py).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores (the CPU
oracle: FP64, OpenMP over blocks, all host threads) on the same workload:
W untimed and K timed timesteps of the 4096-block mesh.  The oracle is a
restatement of the reference's code, not the reference binary (which is
not built where this runs); on the same host and case it runs about 1.4x
faster than the reference binary (single thread, 64 blocks of 16^3, 40
variables, 27-point), so ratios against it are conservative.
Under torchrun each rank runs an independent replica ("replicas only":
the hot path has no exchange between GPUs on one logical rank).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = ("cell-var updates/s + %HBM roofline: FP32-batched vs FP64 GPU at "
          "1e-6 rel chksum")
UNIT = "cell-var updates/s"
INIT = (8, 8, 8)
N = 16
V = 40
STENCIL = 27
SPT = 4
FREQ = 5
N0 = INIT[0] * INIT[1] * INIT[2]
N_BLOCKS = N0 * 8
CAP = N0 + N_BLOCKS + 8
UPD_PER_STAGE = N_BLOCKS * N ** 3 * V
# one-thread CPU baseline sample: the same blocks, variables and stencil on
# a 2x2x2-initial mesh refined once (64 blocks)
SAMPLE_INIT = (2, 2, 2)
WORKLOAD = {
    "workload": "uniform mesh 4096 blocks of 16^3 (8x8x8 initial, uniform "
                "refine 1), 40 vars, 27-point, 4 stages/ts, checksum every "
                "5th stage",
    "blocks": N_BLOCKS, "cells_per_block": N ** 3, "num_vars": V,
    "stencil": STENCIL, "stages_per_ts": SPT, "checksum_freq": FREQ,
    "path": "batched FP32 (fused ghost+stencil+checksum, CUDA graph)",
    "l2": "inputs larger than L2 (3.4 GB FP32 interiors per pool)",
}


def updates(steps):
    return steps * SPT * UPD_PER_STAGE


def build_mesh(lib, dtype, init=INIT, cap=CAP, ctx=None, host=None,
               stencil=STENCIL):
    from miniamr_gb300 import mesh as meshmod
    from miniamr_gb300.abi import Config
    n0 = init[0] * init[1] * init[2]
    cfg = Config.make(N, N, N, V, cap, stencil=stencil, dtype=dtype)
    if ctx is None:
        ctx = lib.context(cfg)
    if host is None:
        host = lib.initial_values(cfg, n0)
    m = meshmod.initial_mesh(*init, 1, cap)
    ctx.upload(np.arange(n0), host)
    ctx.split(m.split_all())
    ctx.set_mesh(m.blocks())
    return ctx, m


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a run."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.p:
            time.sleep(0.15)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out, _ = self.p.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        p = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM traffic of the stage kernel from the committed ncu
    summary (profiles/batched_stage_fp32_27pt_4096blk.json): read, write
    and total bytes scaled to one 40-variable launch, if present."""
    p = os.path.join(REPO, "profiles", "batched_stage_fp32_27pt_4096blk.json")
    try:
        d = json.load(open(p))
    except (OSError, ValueError):
        return None
    keys = ("dram_bytes_per_launch", "dram_read_bytes_per_launch",
            "dram_write_bytes_per_launch", "captured_vars", "scale",
            "write_below_stored")
    return {k: d[k] for k in keys if k in d}


def fp64_pipe_rate(lib):
    """FP64 add instructions per second the device sustains (the bound of
    the bit-exact FP64 paths): mamr_probe_fp64_rate, best of three."""
    try:
        return max(lib.probe_fp64_rate() for _ in range(3))
    except (AttributeError, RuntimeError):
        return None


def oracle_rate(steps, threads=None, stages=SPT, warm=1, init=INIT):
    """The reference algorithm on the host cores: CPU oracle, FP64, OpenMP
    over blocks, on the uniform mesh of init^3 initial blocks refined once
    (the benchmark mesh by default): `warm` untimed timesteps, then `steps`
    timed timesteps of `stages` stages; returns (updates/s, threads,
    seconds)."""
    from miniamr_gb300 import build
    from miniamr_gb300.abi import FP64, Library
    threads = threads or os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    lib = Library(build.build_oracle())
    n0 = init[0] * init[1] * init[2]
    ctx, _ = build_mesh(lib, FP64, init=init, cap=n0 * 9 + 8)
    if warm:
        ctx.run_timesteps(warm, stages, FREQ)
    t0 = time.perf_counter()
    ctx.run_timesteps(steps, stages, FREQ, first_stage=warm * stages)
    dt = time.perf_counter() - t0
    ctx.close()
    return steps * stages * n0 * 8 * N ** 3 * V / dt, threads, dt


def amr_sphere(lib, dtype, flags=0):
    """The AMR run with one moving sphere (4^3 blocks of 16^3, 40 vars,
    27-point, 4 levels, refine every 5 steps, 100 timesteps; up to 7429
    blocks) replayed from the reference's recorded mesh sequence, each
    stretch of stages between refinements as one run: through the plain
    path (flags 0: the drop-in's call sequence of comm, stencil and
    check_sum, queued without host syncs) or the batched path (one fused
    launch per stage, edge and corner ghosts from their recipes, a CUDA
    graph captured per stretch).  FP64: every checksum compared bit for bit
    with the reference's; FP32 pool: max and RMS relative error of every
    checksum against the reference's FP64 checksums.  For the batched path
    a first replay lets the tuner time its launch shapes."""
    import torch
    from miniamr_gb300.abi import FP64
    from miniamr_gb300.trace import read_trace, replay_batched
    path = os.path.join(REPO, "tests", "golden", "config2.trace.xz")
    if not os.path.exists(path):
        return None
    recs = read_trace(path)
    if flags:
        _, ctx, _ = replay_batched(lib, recs, flags, dtype=dtype)
        ctx.close()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sums, ctx, timings = replay_batched(lib, recs, flags, dtype=dtype)
    torch.cuda.synchronize()
    total = time.perf_counter() - t0
    ctx.close()
    cells = N ** 3
    stages = sum(n for n, _, _ in timings)
    upd = sum(n * nb * cells * V for n, _, nb in timings)
    run_s = sum(t for _, t, _ in timings)
    out = {"stages": stages, "runs": len(timings),
           "mean_blocks": upd / (stages * cells * V),
           "max_blocks": max(nb for _, _, nb in timings),
           "updates_per_s": upd / run_s, "run_seconds": run_s,
           "replay_seconds_incl_refinement_and_host": total,
           "checksums": len(sums)}
    if dtype == FP64:
        out["checksums_bit_exact"] = all(
            np.float64(a).tobytes() == np.float64(b).tobytes()
            for _, a, b in sums)
    else:
        rel = np.array([abs(a - b) / abs(b) for _, a, b in sums if b != 0.0])
        out["checksum_rel_error_vs_reference_fp64"] = {
            "max": float(rel.max()), "rms": float(np.sqrt(np.mean(rel ** 2)))}
    return out


def one_thread_oracle_rate():
    """The CPU oracle on one host thread (a fresh process, so that OpenMP
    starts with one thread): one timestep of the 64-block sample."""
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__),
                        "--oracle-rate-steps", "1"], env=env,
                       capture_output=True, text=True)
    try:
        return json.loads(r.stdout.strip().splitlines()[-1])
    except (ValueError, IndexError):
        return None


def uniform_stencil0(lib):
    """The variable-work stencils (--stencil 0) on the uniform 4096-block
    mesh, 40 FP64 vars: one cycle of six stages (stencil_0, _x, _y, _z,
    _7, _27, each followed by stencil_check; variable 0 takes the 7-point
    stencil), checksums every 5th stage, through the plain path; beside it
    the CPU oracle (OpenMP) on the 512-block sample of the same setup."""
    import torch
    from miniamr_gb300 import build
    from miniamr_gb300.abi import FP64, Library
    out = {}
    for name, L, init, cap in (
            ("gpu", lib, INIT, CAP),
            ("cpu_oracle", Library(build.build_oracle()), (4, 4, 4),
             4 * 4 * 4 * 9 + 8)):
        ctx, _ = build_mesh(L, FP64, init=init, cap=cap, stencil=0)
        ctx.set_work_params(*L.work_coefficients(V))
        ctx.run_timesteps(1, 6, 5)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.run_timesteps(1, 6, 5, first_stage=6)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        ctx.close()
        n = init[0] * init[1] * init[2] * 8
        out[name] = 6 * n * N ** 3 * V / dt
    out["cpu_threads"] = os.cpu_count()
    out["speedup"] = out["gpu"] / out["cpu_oracle"]
    out["workload"] = ("4096 blocks of 16^3 (CPU: 512), 40 FP64 vars, "
                       "--stencil 0, six stages")
    return out


def uniform_fp64_7pt(lib, steps):
    """The uniform 4096-block mesh with 40 FP64 variables and the 7-point
    stencil, 4 stages per timestep: the batched path (fused ghost+stencil,
    CUDA graph, autotuned launch shape) over `steps` timesteps against one
    stencil launch per (block, variable) after the per-call exchange, one
    stage (updates/s, CUDA events on the library's stream)."""
    from miniamr_gb300.abi import FP64, RUN_BATCHED, RUN_GRAPH, RUN_PER_BLOCK
    ctx, _ = build_mesh(lib, FP64, stencil=7)
    ctx.run_timesteps(1, SPT, FREQ, flags=RUN_BATCHED | RUN_GRAPH)
    ms = timed(ctx, lambda: ctx.run_timesteps(steps, SPT, FREQ,
                                              first_stage=SPT,
                                              flags=RUN_BATCHED | RUN_GRAPH))
    batched = updates(steps) / (ms / 1e3)
    shape = ctx.tuning()
    ms1 = timed(ctx, lambda: ctx.run_timesteps(1, 1, 0, flags=RUN_PER_BLOCK))
    per_block = UPD_PER_STAGE / (ms1 / 1e3)
    ctx.close()
    return {"workload": "4096 blocks of 16^3, 40 FP64 vars, 7-point, 4 "
                        "stages/ts", "batched_graph": batched,
            "batched_timesteps": steps, "launch_shape": shape,
            "one_launch_per_block_var": per_block,
            "speedup": batched / per_block}


def timed(ctx, fn):
    """Milliseconds of fn() on the context's stream (CUDA events, the
    device synchronised on both sides)."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def stress_multilevel(lib, dtype):
    """The multi-level stress run (4^3 blocks of 8^3, 5 levels, four moving
    objects, refine every 2 steps, 7-point, 20 timesteps x 2 stages; about
    22k blocks, 35,884 at most) replayed from the reference's recorded mesh
    sequence with 40 variables: each stretch of stages between refinements
    is one batched run under a freshly captured CUDA graph.  Rate = updates
    over the run calls' wall time (descriptor build and graph capture
    included; the device finishes the preceding refinement before each
    run's clock starts); refinement data movement and mesh set-up are
    timed separately."""
    import torch
    from miniamr_gb300.abi import RUN_BATCHED, RUN_GRAPH
    from miniamr_gb300.trace import read_trace, replay_batched
    path = os.path.join(REPO, "tests", "golden", "config5.trace.xz")
    if not os.path.exists(path):
        return None
    recs = read_trace(path)
    # first pass: the autotuner times its candidates for each work size
    _, ctx, _ = replay_batched(lib, recs, RUN_BATCHED | RUN_GRAPH,
                               dtype=dtype, num_vars=V)
    ctx.close()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, ctx, timings = replay_batched(lib, recs, RUN_BATCHED | RUN_GRAPH,
                                     dtype=dtype, num_vars=V)
    torch.cuda.synchronize()
    total = time.perf_counter() - t0
    ctx.close()
    # a third pass with every split and consolidation call synchronised on
    # both sides: the refinement data movement on its own
    refine = {"split": [0.0, 0], "consolidate": [0.0, 0]}
    orig = lib.context

    def timed(cfg):
        c = orig(cfg)
        for name in refine:
            f = getattr(c, name)

            def wrapped(jobs, f=f, name=name):
                c.sync()
                t = time.perf_counter()
                f(jobs)
                c.sync()
                refine[name][0] += time.perf_counter() - t
                refine[name][1] += len(jobs)
            setattr(c, name, wrapped)
        return c
    lib.context = timed
    try:
        _, ctx, _ = replay_batched(lib, recs, RUN_BATCHED | RUN_GRAPH,
                                   dtype=dtype, num_vars=V)
    finally:
        lib.context = orig
    stages = sum(n for n, _, _ in timings)
    run_s = sum(t for _, t, _ in timings)
    cells = 8 ** 3
    upd = sum(n * nb * cells * V for n, _, nb in timings)
    ctx.close()
    return {"stages": stages, "runs": len(timings),
            "mean_blocks": upd / (stages * cells * V),
            "max_blocks": max(nb for _, _, nb in timings),
            "updates_per_s": upd / run_s, "run_seconds": run_s,
            "replay_seconds_incl_refinement_and_host": total,
            "refinement_data_movement": {
                name: {"jobs": n, "ms": t * 1e3,
                       "ms_per_job": t * 1e3 / max(n, 1)}
                for name, (t, n) in refine.items()}}


def _reflog_sums(name):
    """Every checksum of a committed reference log, in call order."""
    import lzma
    import struct
    path = os.path.join(REPO, "tests", "golden", name + ".reflog.xz")
    if not os.path.exists(path):
        return None
    ref = []
    with lzma.open(path, "rt") as f:
        for ln in f:
            p = ln.split()
            if p[0] == "cs":
                ref.append(struct.unpack(
                    "<d", int(p[3], 16).to_bytes(8, "little"))[0])
    return np.array(ref)


def _reflog_meshes(name):
    import lzma
    path = os.path.join(REPO, "tests", "golden", name + ".reflog.xz")
    if not os.path.exists(path):
        return None
    with lzma.open(path, "rt") as f:
        return [(int(p[1]), int(p[2]), p[3]) for p in
                (ln.split() for ln in f) if p[0] == "mesh"]


def stress_driver(lib, dtype, case="config5_300", fp64_sums=None):
    """The multi-level stress run at its full length through the AMR driver
    (mamr_amr_run): 4^3 blocks of 8^3, 40 variables, 7-point, 5 levels,
    four moving objects, refine every 2 steps, 300 timesteps x 2 stages,
    checksum every stage -- 151 refinements, each up to five marking steps
    on the device, the library's split/consolidation bookkeeping, the cell
    movement on the device and a new mesh; every stretch of stages one
    batched run under a freshly captured CUDA graph.  case "config5_300":
    the objects of the recorded stress run (13k-24k blocks); case
    "config5_named_mesh": the objects at the sizes the benchmark's
    description names (spheres of radius 0.1, a cylinder of radius 0.05, a
    box of side 0.2; 30k-53k blocks), run at 8^3 cells and 40 variables.
    A 10-timestep run first lets the tuner time its launch shapes.  Rates:
    updates over the stretches' wall time (each stretch synchronised) and
    over the whole call (initial values, upload and refinement included);
    the refinement time split into its parts (the marking and bookkeeping
    run ahead on the driver's planning thread, overlapping the stages; the
    stage side waits for them, moves the cells and sets each mesh).
    Checksums against the
    reference's own log of the run (FP64 bit for bit, FP32 max and RMS
    relative error) or, for the named objects, the FP32 checksums against
    fp64_sums (this path's FP64 run) and the meshes against the reference's
    log of the meshes.  Returns (summary, checksums)."""
    from miniamr_gb300 import run as runmod
    meta = json.load(open(os.path.join(REPO, "tests", "golden",
                                       "cases.json")))
    if case not in meta:
        return None, None
    spec = runmod.parse(meta[case]["args"])
    spec.opts.update(nx=8, ny=8, nz=8, num_vars=V)
    spec.fp32 = dtype != 0
    cfg = spec.config()
    warm = spec.params()
    warm.num_tsteps = 10
    with lib.context(cfg) as ctx:
        ctx.amr_run(warm, spec.objects)
    with lib.context(cfg) as ctx:
        sums, st, ev = ctx.amr_run(spec.params(), spec.objects,
                                   events=case != "config5_300")
    out = {"timesteps": spec.opts["num_tsteps"],
           "refinements": st["refinements"],
           "marking_steps": st["marking_steps"],
           "max_blocks": st["max_active"], "final_blocks": st["final_active"],
           "updates": st["updates"],
           "updates_per_s": st["updates"] / st["stage_seconds"],
           "updates_per_s_whole_run": st["updates"] / st["total_seconds"],
           "stage_seconds": st["stage_seconds"],
           "refine_seconds": st["refine_seconds"],
           # the planning thread's work (overlapping the stages) and the
           # stage side's part of each refinement
           "planning_thread_seconds": {
               k: st[k + "_seconds"] for k in ("mark", "bookkeeping")},
           "refine_parts_seconds": {
               k: st[k + "_seconds"] for k in ("wait", "data", "mesh")},
           "total_seconds": st["total_seconds"], "checksums": sums.size,
           "timing": "host wall clock around each synchronised call"}
    ref = _reflog_sums(case) if case == "config5_300" else None
    got = sums.reshape(-1)
    if ref is not None and got.size == ref.size:
        if dtype == 0:
            out["checksums_bit_exact_vs_reference"] = bool(
                np.array_equal(got.view(np.uint64), ref.view(np.uint64)))
        else:
            rel = np.abs(got - ref) / np.abs(ref)
            out["checksum_rel_error_vs_reference_fp64"] = {
                "max": float(rel.max()),
                "rms": float(np.sqrt(np.mean(rel ** 2)))}
    elif ref is not None:
        out["checksum_count_mismatch"] = [int(got.size), int(ref.size)]
    if fp64_sums is not None and fp64_sums.size == got.size:
        rel = np.abs(got - fp64_sums.reshape(-1)) / np.abs(
            fp64_sums.reshape(-1))
        out["checksum_rel_error_vs_fp64_run"] = {
            "max": float(rel.max()), "rms": float(np.sqrt(np.mean(rel ** 2)))}
    meshes = _reflog_meshes(case) if case != "config5_300" else None
    if meshes is not None:
        from miniamr_gb300 import build
        from miniamr_gb300.abi import Library
        import ctypes as C
        ol = Library(build.ORACLE_LIB if os.path.exists(build.ORACLE_LIB)
                     else build.build_oracle())
        f = ol.lib.mamr_oracle_mesh_hash
        f.restype = C.c_uint64
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
        mine = []
        for e in ev:
            if e[0] == "mesh":
                b, num, cen = (np.ascontiguousarray(e[2]),
                               np.ascontiguousarray(e[3]),
                               np.ascontiguousarray(e[4]))
                mine.append((e[1], len(b), "%016x" % f(
                    b.ctypes.data, num.ctypes.data, cen.ctypes.data,
                    len(b))))
        out["meshes_equal_reference"] = mine == meshes
    return out, sums


def refine_marking(lib):
    """Refinement marking (mamr_mark_refine: reset_all, check_objects and
    refine_level of one rank) on the recorded steps of the multi-level
    stress run (config5.mark.xz: about 20k blocks of five levels, four
    moving objects).  Time per call -- block and parent lists to the device,
    the object tests and the rule passes, flags back -- after two warm-up
    calls, best of three, against the CPU oracle on one thread; both checked
    against the reference's own flags."""
    from miniamr_gb300 import build
    from miniamr_gb300.abi import Config, Library
    from miniamr_gb300.trace import read_marks
    path = os.path.join(REPO, "tests", "golden", "config5.mark.xz")
    if not os.path.exists(path):
        return None
    steps = read_marks(path)
    cap = max(int(st.blocks["slot"].max()) for st in steps) + 1
    out = {"steps": len(steps), "blocks": [len(st.blocks) for st in steps],
           "objects": len(steps[0].objects)}
    for name, L in (("gpu", lib), ("cpu_oracle_1_thread",
                                   Library(build.build_oracle()))):
        ms, same = [], True
        with L.context(Config.make(*steps[0].block_size, 1, cap)) as ctx:
            for st in steps:
                ts = []
                for _ in range(5):
                    t0 = time.perf_counter()
                    br, pr = ctx.mark_refine(st.params, st.objects,
                                             st.blocks, st.parents)
                    ts.append(time.perf_counter() - t0)
                act = st.parents["active"] == 1
                same &= bool(np.array_equal(br, st.block_refine) and
                             np.array_equal(pr[act], st.parent_refine[act]))
                ms.append(min(ts[2:]) * 1e3)
        out[name + "_ms"] = ms
        out[name + "_flags_equal_reference"] = same
    out["speedup"] = sum(out["cpu_oracle_1_thread_ms"]) / sum(out["gpu_ms"])
    return out


def profile_case(name):
    """Small batched runs for ncu captures, launched stage by stage (no
    graph), with the stage kernel's launch shape forced to candidate
    MAMR_PROFILE_SHAPE (default 0, the one the tuner keeps for the
    benchmark workload) so that launch indices are stable.
      fp32_27, fp32_7, fp64_27, fp64_7: 4096 blocks of 16^3, 4 vars (268 MB
        of FP32 interior cells per pool, twice the L2; MAMR_PROFILE_VARS
        sets another count), two timesteps of four stages (checksums on
        each timestep's first stage, as in the benchmark);
      stress_fp32, stress_fp64: the recorded multi-level stress run (8^3
        blocks, ~22k of them, 4 vars -- MAMR_PROFILE_VARS sets another
        count -- 7-point), replayed batched: 40 stages, one run per stretch
        between refinements, with its splits and consolidations;
      amr27_fp32, amr27_fp64: the AMR sphere run (16^3 blocks, up to 7429,
        4 levels, 27-point, 40 vars unless MAMR_PROFILE_VARS says
        otherwise), replayed batched in the same way: 100 stages in 20
        runs;
      plain_fp32_27, plain_fp64_27: the benchmark mesh (4096 blocks of
        16^3, 40 vars) through the plain path, the driver's call sequence:
        two timesteps of four stages."""
    global V, UPD_PER_STAGE
    import torch
    from miniamr_gb300 import build, load
    from miniamr_gb300.abi import FP32, FP64, RUN_BATCHED
    global STENCIL
    dtype = FP32 if "fp32" in name else FP64
    shape = int(os.environ.get("MAMR_PROFILE_SHAPE", "0"))
    build.build_library()
    lib = load()
    if name.startswith("stress") or name.startswith("amr27"):
        from miniamr_gb300.trace import read_trace, replay_batched
        recs = read_trace(os.path.join(
            REPO, "tests", "golden",
            "config5.trace.xz" if name.startswith("stress")
            else "config2.trace.xz"))
        orig = lib.context

        def forced(cfg):
            c = orig(cfg)
            c.set_tuning(shape)
            return c
        lib.context = forced
        nv = os.environ.get("MAMR_PROFILE_VARS")
        _, ctx, timings = replay_batched(lib, recs, RUN_BATCHED, dtype=dtype,
                                         num_vars=int(nv) if nv else None)
        torch.cuda.synchronize()
        ctx.close()
        print(f"profile case {name}: {sum(n for n, _, _ in timings)} "
              f"batched stages in {len(timings)} runs")
        return 0
    if name.startswith("plain"):
        from miniamr_gb300.abi import RUN_PLAIN
        STENCIL = 27 if name.endswith("27") else 7
        ctx, _ = build_mesh(lib, dtype)
        ctx.run_timesteps(1, SPT, FREQ, flags=RUN_PLAIN)
        ctx.run_timesteps(1, SPT, FREQ, first_stage=SPT, flags=RUN_PLAIN)
        torch.cuda.synchronize()
        ctx.close()
        print(f"profile case {name}: {2 * SPT} plain stages, {V} vars")
        return 0
    STENCIL = 27 if name.endswith("27") else 7
    V = int(os.environ.get("MAMR_PROFILE_VARS", "4"))
    UPD_PER_STAGE = N_BLOCKS * N ** 3 * V
    ctx, _ = build_mesh(lib, dtype)
    ctx.set_tuning(shape)
    # the benchmark's cadence: 4 stages per timestep, checksum on stage 0
    ctx.run_timesteps(1, SPT, FREQ, flags=RUN_BATCHED)
    ctx.run_timesteps(1, SPT, FREQ, first_stage=SPT, flags=RUN_BATCHED)
    torch.cuda.synchronize()
    ctx.close()
    print(f"profile case {name}: {2 * SPT} batched stages, {V} vars")
    return 0


def max_over_ranks(x, dist=None, device="cpu"):
    """The slowest rank's value (the job's time); x itself on one rank."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    return world, rank, local, pg


def reference_arm(args, world, rank, pg):
    """The reference algorithm on the host cores on the benchmark workload
    itself: W untimed, then K timed timesteps of the 4096-block mesh (FP64,
    all host threads).  Rank 0 only."""
    if rank != 0:
        return 0
    steps = max(1, args.steps)
    rate, threads, dt = oracle_rate(steps, warm=max(0, args.warmup))
    line = {
        "metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": dt / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: the reference's init() values (rand(), seed 1), "
                "uniform mesh",
        "config": dict(WORKLOAD),
        "cpu_baseline": {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the whole workload: 4096 blocks of 16^3 (8x8x8 "
                      f"initial, refine 1), 40 vars, 27-point, FP64, {steps} "
                      "timesteps of 4 stages; CPU oracle (restatement of "
                      "ref/stencil.c, ref/comm.c, ref/check_sum.c), OpenMP "
                      "over blocks; 1.4x the reference binary's rate on "
                      "one thread of the same host"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--oracle-rate-steps", type=int, default=0,
                    help=argparse.SUPPRESS)
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the FP64 7-point and multi-level stress "
                         "measurements")
    ap.add_argument("--fp64-steps", type=int, default=None,
                    help="timesteps of the FP64 comparison runs")
    ap.add_argument("--profile-case", default=None,
                    choices=["fp32_27", "fp32_7", "fp64_27", "fp64_7",
                             "stress_fp32", "stress_fp64", "amr27_fp32",
                             "amr27_fp64", "plain_fp32_27", "plain_fp64_27"],
                    help="a small case for ncu (see profile_case)")
    args = ap.parse_args()
    if args.oracle_rate_steps:
        rate, threads, dt = oracle_rate(
            args.oracle_rate_steps, int(os.environ.get("OMP_NUM_THREADS",
                                                       "1")),
            warm=0, init=SAMPLE_INIT)
        print(json.dumps({"value": rate, "unit": UNIT, "cores": threads,
                          "seconds": dt}))
        return 0
    if args.profile_case:
        return profile_case(args.profile_case)
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        return reference_arm(args, world, rank, pg)

    import torch
    from miniamr_gb300 import build, load
    from miniamr_gb300.abi import (FP32, FP64, RUN_BATCHED, RUN_GRAPH,
                                   RUN_PER_BLOCK, RUN_PLAIN)

    torch.cuda.set_device(local)
    build.build_library()
    lib = load()
    K, W = args.steps, max(3, args.warmup)
    flags = RUN_BATCHED | RUN_GRAPH

    # ---- headline: FP32 batched, pool resident -----------------------
    ctx, _ = build_mesh(lib, FP32)
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.run_timesteps(W, SPT, FREQ, flags=flags)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        sums32 = ctx.run_timesteps(K, SPT, FREQ, first_stage=W * SPT,
                                   flags=flags)
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = ctx.launch_count() - l0
    shape = ctx.tuning()
    ms_head = max_over_ranks(ev0.elapsed_time(ev1), pg, "cuda")
    value = updates(K) * world / (ms_head / 1e3)
    n_stage_launches = K * SPT
    per_launch_s = ms_head / 1e3 / n_stage_launches
    alg_bytes = UPD_PER_STAGE * 2 * 4
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / per_launch_s / 1e9
    traffic = ncu_traffic() or {}
    ctx.close()

    # ---- e2e through the C ABI from pinned host buffers -----------------
    from miniamr_gb300.abi import Config
    cfg = Config.make(N, N, N, V, CAP, stencil=STENCIL, dtype=FP32)
    pinned = torch.empty((N0, V, N + 2, N + 2, N + 2), dtype=torch.float64,
                         pin_memory=True)
    host = pinned.numpy()
    host[...] = lib.initial_values(cfg, N0)
    ctx = lib.context(cfg)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    build_mesh(lib, FP32, ctx=ctx, host=host)
    e2e_sums = ctx.run_timesteps(K, SPT, FREQ, flags=flags)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, pg, "cuda")
    ctx.close()
    h2d = host.nbytes
    d2h = e2e_sums.nbytes

    # ---- FP64 paths and the FP32 checksum error ------------------------
    # the same W + K timesteps on FP64 pools, the K timed with CUDA events:
    # plain (the driver's call sequence; bit-exact with the reference) and
    # batched + graph; and the plain path on an FP32 pool
    K64 = max(10, K)
    ctx64p, _ = build_mesh(lib, FP64)
    ctx64p.run_timesteps(W, SPT, FREQ, flags=RUN_PLAIN)
    box = {}
    ms = timed(ctx64p, lambda: box.setdefault("s", ctx64p.run_timesteps(
        K64, SPT, FREQ, first_stage=W * SPT, flags=RUN_PLAIN)))
    s64_plain = box["s"]
    fp64_plain = updates(K64) / (ms / 1e3)
    # the naive port: one stencil launch per (block, variable), one stage
    ms = timed(ctx64p, lambda: ctx64p.run_timesteps(
        1, 1, 0, flags=RUN_PLAIN | RUN_PER_BLOCK))
    fp64_per_block = UPD_PER_STAGE / (ms / 1e3)
    ctx64p.close()
    ctx64, _ = build_mesh(lib, FP64)
    ctx64.run_timesteps(W, SPT, FREQ, flags=flags)
    ms = timed(ctx64, lambda: box.setdefault("b", ctx64.run_timesteps(
        K64, SPT, FREQ, first_stage=W * SPT, flags=flags)))
    fp64_batched = updates(K64) / (ms / 1e3)
    fp64_batched_same = bool(np.array_equal(
        box["b"].view(np.uint64), s64_plain.view(np.uint64)))
    ctx64.close()
    ctx32p, _ = build_mesh(lib, FP32)
    ctx32p.run_timesteps(W, SPT, FREQ, flags=RUN_PLAIN)
    ms = timed(ctx32p, lambda: ctx32p.run_timesteps(
        K64, SPT, FREQ, first_stage=W * SPT, flags=RUN_PLAIN))
    fp32_plain = updates(K64) / (ms / 1e3)
    ctx32p.close()
    ref = s64_plain[:len(sums32)]
    got = sums32[:len(ref)]
    rel = np.abs(got - ref) / np.abs(ref)
    err = {"checksums": int(rel.size), "max_rel": float(rel.max()),
           "rms_rel": float(np.sqrt(np.mean(rel ** 2))),
           "fp64_reference": "plain FP64 path over the same stages (bit-"
                             "exact with the reference's code and the FP64 "
                             "oracle on this mesh)"}
    fp64_rate = fp64_pipe_rate(lib)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": ms_head / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: the reference's init() values "
                                "(rand(), seed 1), uniform mesh",
        "config": dict(WORKLOAD, launch_shape=shape),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "frac_of_nominal_8000": achieved / 8000.0,
                     "traffic": traffic.get("dram_bytes_per_launch"),
                     "traffic_detail": traffic or None,
                     "peak_source": peak_kind,
                     "kernel": "pencil_stage_kernel<float,27>",
                     "alg_bytes_per_launch": alg_bytes},
        "e2e": {"value": updates(K) * world / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "seconds": e2e_s},
        "gpu_launches": launches,
    }
    if not args.no_configs:
        line["configs"] = {
            "uniform_fp64_7pt": uniform_fp64_7pt(lib, max(20, K)),
            "amr_sphere_27pt_plain_fp64": amr_sphere(lib, FP64),
            "amr_sphere_27pt_plain_fp32": amr_sphere(lib, FP32),
            "amr_sphere_27pt_batched_fp64": amr_sphere(lib, FP64, flags),
            "amr_sphere_27pt_batched_fp32": amr_sphere(lib, FP32, flags),
            "uniform_stencil0_fp64": uniform_stencil0(lib),
            "stress_multilevel_7pt_fp32": stress_multilevel(lib, FP32),
            "stress_multilevel_7pt_fp64": stress_multilevel(lib, FP64),
            "stress_300ts_amr_driver_fp32": stress_driver(lib, FP32)[0],
            "stress_300ts_amr_driver_fp64": stress_driver(lib, FP64)[0],
            "stress_named_objects_300ts_amr_driver_fp32": stress_driver(
                lib, FP32, "config5_named_mesh")[0],
            "refine_marking_stress": refine_marking(lib),
        }
    # the figures the targets rest on last, where a truncated tail of the
    # output still shows them
    line["paths"] = {
        "timesteps": K64, "timing": "CUDA events on the library's stream",
        "fp32_batched": value / world, "fp64_batched": fp64_batched,
        "fp64_plain": fp64_plain, "fp32_plain": fp32_plain,
        "fp64_batched_sums_equal_plain": fp64_batched_same,
        "fp64_one_launch_per_block_var": fp64_per_block,
        "fp32_batched_over_fp64_plain": value / world / fp64_plain,
        "fp64_pipe_instr_per_s": fp64_rate}
    line["fp32_checksum_error"] = err
    line["clocks"] = clk.summary()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        one = one_thread_oracle_rate()
        rate, threads, dt = oracle_rate(1)
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the whole workload for one timestep (4096 blocks of "
                      "16^3, 40 vars, 27-point, FP64, 4 stages) after one "
                      "untimed; CPU oracle with OpenMP over blocks "
                      f"({dt:.1f} s)"}
        if one:
            one["sample"] = ("64 blocks of 16^3 (2x2x2 initial, refine 1), "
                             "one timestep")
            line["cpu_baseline"]["single_thread"] = one
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
