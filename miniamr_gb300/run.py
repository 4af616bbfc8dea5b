"""The reference's command line over the GB300 library: a whole miniAMR run.

    python -m miniamr_gb300.run --init_x 4 --init_y 4 --init_z 4 --nx 8 ...

takes the reference executable's options (ref/main.c:56-178; defaults
ref/param.h) and runs them through mamr_amr_run() on the GPU: init(), the
initial refine(0), then every timestep's stages, move() and refine()
(ref/driver.c:36-140), one rank.  It checks each checksum stage's
per-variable sums the way the reference does (ref/driver.c:93-101: relative
change against the previous checksum above 10^-error_tol; only variable 0
for --stencil 0) and reports the first stage that fails; the reference
stops there, this runs to the end and exits 1.

Options of the reference that only matter on more than one rank (--npx/y/z
above 1, --lb_opt, --inbalance, --blocking_send, --change_dir,
--group_blocks, --break_ties, --limit_move, --send_faces, --rcb, --reorder)
are accepted and have no effect on one rank; --comm_vars only groups the
exchanges of the variables, which does not change any value on one rank.
Options this library does not run are refused: --morton, --hilbert and
--trunc_hilbert (lb_method > 0 reorders the initial blocks and the
children), --time (time-based stepping) and --plot_freq > 0.

Three options are this library's own: --fp32 (cells in FP32,
MAMR_FP32), --plain (the per-call path instead of the batched one) and
--tuning K (the batched path's launch-shape candidate K, mamr_set_tuning,
instead of the tuner's choice).
"""
from __future__ import annotations

import sys
from dataclasses import dataclass

import numpy as np

from .abi import (AMR_OBJECT_DTYPE, FP32, FP64, RUN_BATCHED, RUN_GRAPH,
                  RUN_PLAIN, AmrParams, Config)

# ref/param.h
DEFAULTS = dict(max_blocks=500, num_refine=5, uniform_refine=0, nx=10,
                ny=10, nz=10, num_vars=40, comm_vars=0, init_x=1, init_y=1,
                init_z=1, npx=1, npy=1, npz=1, refine_freq=5, error_tol=8,
                num_tsteps=20, stages_per_ts=20, checksum_freq=5, stencil=7,
                report_perf=12, plot_freq=0, block_change=0, code=0,
                permute=0, refine_ghost=0, report_diffusion=0, lb_method=0)

_INT_OPTS = {
    "--max_blocks": "max_blocks", "--num_refine": "num_refine",
    "--block_change": "block_change", "--uniform_refine": "uniform_refine",
    "--nx": "nx", "--ny": "ny", "--nz": "nz", "--num_vars": "num_vars",
    "--comm_vars": "comm_vars", "--init_x": "init_x", "--init_y": "init_y",
    "--init_z": "init_z", "--npx": "npx", "--npy": "npy", "--npz": "npz",
    "--refine_freq": "refine_freq", "--error_tol": "error_tol",
    "--num_tsteps": "num_tsteps", "--stages_per_ts": "stages_per_ts",
    "--checksum_freq": "checksum_freq", "--stencil": "stencil",
    "--report_perf": "report_perf", "--plot_freq": "plot_freq",
    "--code": "code",
}
# one-rank no-ops that take a value / take none
_IGNORED_VALUE = {"--reorder", "--inbalance", "--lb_opt", "--limit_move"}
_IGNORED_FLAG = {"--blocking_send", "--change_dir", "--group_blocks",
                 "--break_ties", "--send_faces", "--rcb"}


@dataclass
class RunSpec:
    """A parsed command line."""

    opts: dict
    objects: np.ndarray
    fp32: bool = False
    plain: bool = False
    tuning: int = -1

    @property
    def tol(self) -> float:
        return 10.0 ** (-self.opts["error_tol"])

    def config(self) -> Config:
        o = self.opts
        return Config.make(o["nx"], o["ny"], o["nz"], o["num_vars"],
                           o["max_blocks"], stencil=o["stencil"],
                           dtype=FP32 if self.fp32 else FP64,
                           permute=o["permute"], code=o["code"])

    def run_flags(self) -> int:
        """The batched path with a graph per stretch where it runs this
        configuration (stencil 7/27, code 0, no permuted 27-point); the
        per-call path otherwise or with --plain."""
        o = self.opts
        if (self.plain or o["stencil"] == 0 or o["code"] != 0
                or (o["permute"] and o["stencil"] == 27)):
            return RUN_PLAIN
        return RUN_BATCHED | RUN_GRAPH

    def params(self, run_flags: int | None = None) -> AmrParams:
        o = self.opts
        return AmrParams.make(
            init=(o["init_x"], o["init_y"], o["init_z"]),
            num_refine=o["num_refine"], block_change=o["block_change"],
            refine_freq=o["refine_freq"], uniform_refine=o["uniform_refine"],
            refine_ghost=o["refine_ghost"], num_tsteps=o["num_tsteps"],
            stages_per_ts=o["stages_per_ts"],
            checksum_freq=o["checksum_freq"],
            run_flags=self.run_flags() if run_flags is None else run_flags)


def parse(argv) -> RunSpec:
    """The reference's option parsing and check_input() (ref/main.c:56-191,
    :655-760) for one rank.  Raises ValueError where the reference prints
    an error and aborts, and for the options this library does not run."""
    o = dict(DEFAULTS)
    objs, n_objects = [], None
    fp32 = plain = False
    tuning = -1
    argv = list(argv)
    i = 0

    def take(k):
        if i + k >= len(argv):
            raise ValueError(f"{argv[i]}: missing value")
        return argv[i + 1:i + 1 + k]

    while i < len(argv):
        a = argv[i]
        if a in _INT_OPTS:
            o[_INT_OPTS[a]] = int(take(1)[0])
            i += 2
        elif a == "--num_objects":
            n_objects = int(take(1)[0])
            i += 2
        elif a == "--object":
            if n_objects is None or len(objs) >= n_objects:
                raise ValueError("object number greater than num_objects")
            v = take(14)
            objs.append((int(v[0]), int(v[1]),
                         [float(x) for x in v[2:5]],
                         [float(x) for x in v[5:8]],
                         [float(x) for x in v[8:11]],
                         [float(x) for x in v[11:14]]))
            i += 15
        elif a == "--permute":
            o["permute"] = 1
            i += 1
        elif a == "--refine_ghost":
            o["refine_ghost"] = 1
            i += 1
        elif a == "--report_diffusion":
            o["report_diffusion"] = 1
            i += 1
        elif a in ("--morton", "--hilbert", "--trunc_hilbert"):
            raise ValueError(f"{a}: only --rcb (lb_method 0) is supported")
        elif a == "--time":
            raise ValueError("--time: time-based stepping is not supported")
        elif a in _IGNORED_VALUE:
            take(1)
            i += 2
        elif a in _IGNORED_FLAG:
            i += 1
        elif a == "--fp32":
            fp32 = True
            i += 1
        elif a == "--plain":
            plain = True
            i += 1
        elif a == "--tuning":
            tuning = int(take(1)[0])
            if tuning < 0:
                raise ValueError("--tuning: a candidate index >= 0")
            i += 2
        else:
            raise ValueError(f"Unknown input parameter {a}")
    if (n_objects or 0) != len(objs):
        raise ValueError("number of objects less than specified")
    if min(o["init_x"], o["init_y"], o["init_z"]) < 1:
        raise ValueError("initial blocks on processor must be positive")
    if o["max_blocks"] < o["init_x"] * o["init_y"] * o["init_z"]:
        raise ValueError("max_blocks not enough for initial blocks")
    for d in ("nx", "ny", "nz"):
        if o[d] < 1 or o[d] % 2:
            raise ValueError(f"block size {d} must be even and positive")
    if o["num_refine"] < 0 or o["block_change"] < 0 or o["num_vars"] < 1:
        raise ValueError("num_refine, block_change >= 0 and num_vars >= 1 "
                         "required")
    if o["npx"] * o["npy"] * o["npz"] != 1:
        raise ValueError("one rank: npx * npy * npz must be 1")
    if o["stencil"] not in (0, 7, 27):
        raise ValueError("illegal value for stencil")
    if o["stencil"] == 0 and o["num_vars"] < 8:
        raise ValueError("if stencil is 0, num_vars must be more than 8")
    if not 0 <= o["code"] <= 2:
        raise ValueError("code must be 0, 1, or 2")
    if o["plot_freq"]:
        raise ValueError("--plot_freq: plot files are not written")
    if o["refine_freq"] < 1 and o["num_refine"] and not o["uniform_refine"]:
        raise ValueError("refine_freq must be positive")
    if o["error_tol"] < 0:
        raise ValueError("error_tol must be >= 0")
    if o["block_change"] == 0:
        o["block_change"] = o["num_refine"]
    objects = np.zeros(len(objs), dtype=AMR_OBJECT_DTYPE)
    for q, (t, b, c, m, s, inc) in enumerate(objs):
        objects[q] = (t, b, c, m, s, inc)
    return RunSpec(o, objects, fp32=fp32, plain=plain, tuning=tuning)


def check_tolerance(spec: RunSpec, sums: np.ndarray):
    """The reference's check of each checksum stage against the previous
    one (ref/driver.c:93-101): returns (stage, var) of the first variable
    whose relative change exceeds the tolerance, or None.  sums[0] holds
    the initial checksums."""
    o = spec.opts
    prev = sums[0].copy()
    for st in range(1, len(sums)):
        for v in range(sums.shape[1]):
            s = sums[st, v]
            if o["stencil"] or v == 0:
                if abs(s - prev[v]) / prev[v] > spec.tol:
                    return st, v
            prev[v] = s
    return None


def main(argv=None) -> int:
    from . import load
    spec = parse(sys.argv[1:] if argv is None else argv)
    lib = load()
    cfg = spec.config()
    with lib.context(cfg) as ctx:
        if spec.tuning >= 0:
            ctx.set_tuning(spec.tuning)
        sums, st, _ = ctx.amr_run(spec.params(), spec.objects)
        tun = ctx.tuning()
    o = spec.opts
    print(f"miniAMR on one GB300: {o['nx']}x{o['ny']}x{o['nz']} cells, "
          f"{o['num_vars']} variables, stencil {o['stencil']}, "
          f"{'FP32' if spec.fp32 else 'FP64'} cells, "
          f"{'plain' if spec.run_flags() == RUN_PLAIN else 'batched'} path")
    print(f"blocks: max {st['max_active']} final {st['final_active']}, "
          f"{st['refinements']} refinements")
    bad = check_tolerance(spec, sums)
    if bad is not None:
        stage, v = bad
        print(f"checksum stage {stage} variable {v}: difference too large "
              f"(tolerance {spec.tol:g})")
    print(f"final checksums: {' '.join(f'{x:.15e}' for x in sums[-1][:4])}"
          + (" ..." if sums.shape[1] > 4 else ""))
    rate = st["updates"] / st["stage_seconds"] if st["stage_seconds"] else 0
    print(f"time: total {st['total_seconds']:.3f} s, stages "
          f"{st['stage_seconds']:.3f} s ({rate:.3e} cell-var updates/s), "
          f"refinement {st['refine_seconds']:.3f} s")
    if tun["choice"] >= 0:
        print(f"launch shape: candidate {tun['choice']} of "
              f"{tun['candidates']} ({tun['threads']} threads, "
              f"{tun['vars_per_cta']} variables per CTA, "
              f"{tun['rows_per_thread']} rows, "
              f"{tun['planes_per_thread']} planes per thread, "
              f"{tun['ctas']} CTAs)")
    return 1 if bad is not None else 0


if __name__ == "__main__":
    sys.exit(main())
