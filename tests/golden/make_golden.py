"""Generates the golden fixtures in tests/golden/ from the miniAMR reference.

Needs the reference sources -- the directory MAMR_REFERENCE_SRC names, or
the ref/ directory of a miniAMR checkout named "reference" beside this
repository -- and runs only where they exist; the fixtures it writes are
committed so that the tests need no reference at run time.

For every case in CASES it
  1. runs the unmodified reference (oracle/_ref/miniamr_ref) with its
     check_sum/refine hooks, producing <name>.reflog.xz: every checksum the
     reference computed (exact bits) with a hash of every cell of that
     variable, and a hash of the mesh after each refine(); for the cases in
     MARK also <name>.mark.xz: the inputs and the reference's flags of each
     refinement step's marking (oracle/ref_hooks.c, split_blocks hook);
  2. runs the reference's driver over the drop-in translation units and the
     CPU oracle (oracle/_ref/miniamr_hybrid_trace), which must produce the
     identical log, and records every mamr_* call it made as
     <name>.trace.xz (not for the cases in REFLOG_ONLY).
cases.json lists each case's command line.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import lzma
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(REPO, "oracle", "_ref", "miniamr_ref")
HYB_BIN = os.path.join(REPO, "oracle", "_ref", "miniamr_hybrid_trace")

SPHERE = ["--num_objects", "1", "--object", "2", "1", "0.25", "0.25", "0.25",
          "0.03", "0.03", "0.03", "0.15", "0.15", "0.15", "0", "0", "0"]


def small(stencil, extra=()):
    return (["--init_x", "2", "--init_y", "2", "--init_z", "2", "--nx", "8",
             "--ny", "8", "--nz", "8", "--num_vars", "4", "--stencil",
             str(stencil), "--num_refine", "3", "--refine_freq", "2",
             "--num_tsteps", "16", "--stages_per_ts", "2", "--checksum_freq",
             "1", "--error_tol", "0", "--max_blocks", "4000"] + SPHERE +
            list(extra))


CASES = {
    # the reference's own CPU case: 2^3 blocks of 8^3, 40 vars, 7-point,
    # no refinement, 20 timesteps x 1 stage, checksum every stage
    "config1": ["--init_x", "2", "--init_y", "2", "--init_z", "2", "--nx",
                "8", "--ny", "8", "--nz", "8", "--num_vars", "40",
                "--stencil", "7", "--num_refine", "0", "--num_tsteps", "20",
                "--stages_per_ts", "1", "--checksum_freq", "1"],
    # moving sphere, refine + coarsen every 2 timesteps, up to 3 levels
    "amr27": small(27),
    "amr7": small(7),
    "amr27_permute": small(27, ["--permute"]) [:],
    # uniform refinement, non-cubic blocks, 27-point
    "uniform27": ["--init_x", "2", "--init_y", "1", "--init_z", "3", "--nx",
                  "4", "--ny", "6", "--nz", "8", "--num_vars", "3",
                  "--stencil", "27", "--num_refine", "2", "--uniform_refine",
                  "1", "--num_tsteps", "5", "--stages_per_ts", "2",
                  "--checksum_freq", "1", "--error_tol", "0", "--max_blocks",
                  "4000"],
    # the AMR configuration at full size: 4^3 blocks of 16^3, 40 vars,
    # 27-point, up to 4 levels around a surface sphere (r 0.15) moving at
    # 0.01/step and bouncing inside the cube, refine every 5 steps, 100
    # steps; the 27-point stencil does not conserve the sum under
    # refinement, so the run needs --error_tol 0.  Cell hashes every 10th
    # checksum stage.
    "config2": ["--init_x", "4", "--init_y", "4", "--init_z", "4", "--nx",
                "16", "--ny", "16", "--nz", "16", "--num_vars", "40",
                "--stencil", "27", "--num_refine", "4", "--refine_freq", "5",
                "--num_tsteps", "100", "--stages_per_ts", "1",
                "--checksum_freq", "1", "--error_tol", "0", "--max_blocks",
                "8000", "--num_objects", "1", "--object", "2", "1", "0.25",
                "0.25", "0.25", "0.01", "0.01", "0.01", "0.15", "0.15", "0.15",
                "0", "0", "0"],
    # the multi-level stress mesh, shortened: 4^3 blocks of 8^3, 5 levels,
    # four moving objects (surface sphere r 0.06, solid sphere r 0.05,
    # surface cylinder r 0.03, surface box of half-side 0.06; sizes tuned on
    # the reference so the mesh holds ~21k-24k blocks), 7-point, refine every
    # 2 steps, 20 steps x 2 stages, 4 variables (the block sequence does not
    # depend on the variable count).  Cell hashes every 8th checksum stage.
    "config5": ["--init_x", "4", "--init_y", "4", "--init_z", "4", "--nx",
                "8", "--ny", "8", "--nz", "8", "--num_vars", "4",
                "--stencil", "7", "--num_refine", "5", "--refine_freq", "2",
                "--num_tsteps", "20", "--stages_per_ts", "2",
                "--checksum_freq", "1", "--max_blocks", "40000",
                "--num_objects", "4",
                "--object", "2", "1", "0.3", "0.3", "0.3", "0.01", "0.007",
                "0.005", "0.06", "0.06", "0.06", "0", "0", "0",
                "--object", "3", "1", "0.7", "0.6", "0.4", "-0.008", "0.006",
                "0.01", "0.05", "0.05", "0.05", "0", "0", "0",
                "--object", "20", "1", "0.5", "0.5", "0.7", "0.006", "-0.01",
                "0.004", "0.12", "0.03", "0.03", "0", "0", "0",
                "--object", "0", "1", "0.3", "0.7", "0.7", "0.007", "-0.005",
                "-0.009", "0.06", "0.06", "0.06", "0", "0", "0"],
    # whole-ghost exchanges (--code 1 and 2; identical on one rank: the two
    # differ only in how ranks pack messages): level jumps fill the edge
    # ghosts too, so the 27-point stencil reads no stale values
    "code1_amr27": small(27, ["--code", "1"]),
    "code2_amr7": small(7, ["--code", "2"]),
    # the variable-work stencils (--stencil 0): 8 variables (mat = 2), six
    # stages per timestep so that every kernel (calc_stage % 6) runs on
    # every variable class, refinement and coarsening around a moving
    # sphere, checksums every stage
    "stencil0": ["--init_x", "2", "--init_y", "2", "--init_z", "2", "--nx",
                 "8", "--ny", "8", "--nz", "8", "--num_vars", "8",
                 "--stencil", "0", "--num_refine", "3", "--refine_freq",
                 "2", "--num_tsteps", "8", "--stages_per_ts", "6",
                 "--checksum_freq", "1", "--error_tol", "0",
                 "--max_blocks", "4000"] + SPHERE,
    # refinement marking across object types: surface and solid boxes,
    # the x half-spheroids (surface and solid, both halves), surface and
    # solid cylinders along x, a sphere whose negative x size (it grows)
    # keeps it disabled for the first steps, and two solid spheres that
    # leave the domain with bounce 2 and bounce 0 (neither reflects: the
    # reference's bounce-2 branch cannot run); 4^3 blocks, 1 variable
    "mark_shapes": ["--init_x", "2", "--init_y", "2", "--init_z", "2",
                    "--nx", "4", "--ny", "4", "--nz", "4", "--num_vars", "1",
                    "--stencil", "7", "--num_refine", "3", "--refine_freq",
                    "1", "--num_tsteps", "10", "--stages_per_ts", "1",
                    "--checksum_freq", "1", "--error_tol", "0",
                    "--max_blocks", "20000", "--num_objects", "11",
                    "--object", "0", "1", "0.3", "0.3", "0.3", "0.01",
                    "0.02", "0.015", "0.12", "0.08", "0.1", "0", "0", "0",
                    "--object", "1", "1", "0.7", "0.25", "0.6", "-0.02",
                    "0.01", "0.0", "0.05", "0.07", "0.04", "0", "0", "0",
                    "--object", "4", "1", "0.5", "0.7", "0.3", "0.0",
                    "-0.01", "0.01", "0.15", "0.15", "0.15", "0", "0", "0",
                    "--object", "5", "1", "0.25", "0.75", "0.75", "0.01",
                    "0.0", "-0.01", "0.1", "0.08", "0.06", "0", "0", "0",
                    "--object", "6", "1", "0.75", "0.5", "0.8", "-0.01",
                    "0.01", "0.0", "0.1", "0.1", "0.1", "0", "0", "0",
                    "--object", "7", "1", "0.6", "0.6", "0.5", "0.0", "0.0",
                    "0.02", "0.07", "0.09", "0.08", "0", "0", "0",
                    "--object", "20", "1", "0.5", "0.3", "0.7", "0.0",
                    "0.01", "-0.01", "0.3", "0.05", "0.06", "0", "0", "0",
                    "--object", "21", "1", "0.4", "0.85", "0.2", "0.01",
                    "0.0", "0.0", "0.2", "0.04", "0.04", "0", "0", "0",
                    "--object", "2", "1", "0.2", "0.5", "0.5", "0.0", "0.0",
                    "0.0", "-0.05", "0.1", "0.1", "0.02", "0.0", "0.0",
                    "--object", "3", "2", "0.93", "0.4", "0.6", "0.02",
                    "0.0", "0.0", "0.05", "0.05", "0.05", "0", "0", "0",
                    "--object", "3", "0", "0.06", "0.6", "0.4", "-0.02",
                    "0.0", "0.0", "0.05", "0.05", "0.05", "0", "0", "0"],
    # the y and z half-spheroids and the y/z cylinders, with --refine_ghost
    # (the extent with ghosts, and the parent's extent before coarsening)
    "mark_shapes_ghost": ["--init_x", "2", "--init_y", "2", "--init_z",
                          "2", "--nx", "4", "--ny", "4", "--nz", "4",
                          "--num_vars", "1", "--stencil", "7",
                          "--num_refine", "3", "--refine_freq", "1",
                          "--num_tsteps", "10", "--stages_per_ts", "1",
                          "--checksum_freq", "1", "--error_tol", "0",
                          "--max_blocks", "20000", "--refine_ghost",
                          "--num_objects", "12"] + sum(
        (["--object", str(t), "1"] + [str(x) for x in v] + ["0", "0", "0"]
         for t, v in [
             (8, (0.3, 0.3, 0.3, 0.01, 0.0, 0.01, 0.12, 0.12, 0.12)),
             (9, (0.7, 0.3, 0.3, 0.0, 0.01, 0.01, 0.08, 0.1, 0.08)),
             (10, (0.3, 0.7, 0.3, 0.01, -0.01, 0.0, 0.1, 0.1, 0.1)),
             (11, (0.7, 0.7, 0.3, -0.01, 0.0, 0.01, 0.09, 0.09, 0.09)),
             (12, (0.3, 0.3, 0.7, 0.0, 0.01, -0.01, 0.11, 0.11, 0.11)),
             (13, (0.7, 0.3, 0.7, 0.01, 0.01, 0.0, 0.08, 0.08, 0.08)),
             (14, (0.3, 0.7, 0.7, -0.01, 0.0, 0.0, 0.1, 0.12, 0.1)),
             (15, (0.7, 0.7, 0.7, 0.0, -0.01, -0.01, 0.09, 0.09, 0.09)),
             (22, (0.5, 0.5, 0.2, 0.01, 0.0, 0.0, 0.05, 0.3, 0.05)),
             (23, (0.2, 0.5, 0.8, 0.0, 0.0, 0.01, 0.04, 0.25, 0.04)),
             (24, (0.8, 0.2, 0.5, 0.0, 0.01, 0.0, 0.05, 0.05, 0.3)),
             (25, (0.15, 0.85, 0.5, 0.01, -0.01, 0.0, 0.04, 0.04, 0.2)),
         ]), []),
    # two objects, volume + surface refinement, 7-point, 4 levels, default
    # checksum cadence (every 5th stage of 3)
    # the benchmark mesh at an eighth of its size: 4^3 blocks of 16^3
    # uniformly refined once (512 blocks on one level), 40 variables, 4
    # stages per timestep, 2 timesteps, a checksum and the cell hashes at
    # every stage; 27-point (the benchmark's stencil) and its 7-point twin
    "uniform16_27": ["--init_x", "4", "--init_y", "4", "--init_z", "4",
                     "--nx", "16", "--ny", "16", "--nz", "16", "--num_vars",
                     "40", "--stencil", "27", "--num_refine", "1",
                     "--uniform_refine", "1", "--num_tsteps", "2",
                     "--stages_per_ts", "4", "--checksum_freq", "1",
                     "--error_tol", "0", "--max_blocks", "600"],
    "uniform16_7": ["--init_x", "4", "--init_y", "4", "--init_z", "4",
                    "--nx", "16", "--ny", "16", "--nz", "16", "--num_vars",
                    "40", "--stencil", "7", "--num_refine", "1",
                    "--uniform_refine", "1", "--num_tsteps", "2",
                    "--stages_per_ts", "4", "--checksum_freq", "1",
                    "--error_tol", "0", "--max_blocks", "600"],
    # large blocks: 32^3 cells (a block-variable with ghosts is 308 KB in
    # FP64, more than one CTA's shared memory), 27-point, refinement and
    # coarsening around a moving sphere
    "big32_amr27": ["--init_x", "1", "--init_y", "1", "--init_z", "2",
                    "--nx", "32", "--ny", "32", "--nz", "32", "--num_vars",
                    "2", "--stencil", "27", "--num_refine", "2",
                    "--refine_freq", "2", "--num_tsteps", "6",
                    "--stages_per_ts", "2", "--checksum_freq", "1",
                    "--error_tol", "0", "--max_blocks", "400"] + SPHERE,
    "amr7_objects": ["--init_x", "2", "--init_y", "2", "--init_z", "2",
                     "--nx", "6", "--ny", "6", "--nz", "6", "--num_vars", "3",
                     "--stencil", "7", "--num_refine", "4", "--refine_freq",
                     "1", "--num_tsteps", "12", "--stages_per_ts", "3",
                     "--max_blocks", "20000",
                     "--num_objects", "2",
                     "--object", "3", "1", "0.3", "0.6", "0.5", "0.04",
                     "-0.03", "0.0", "0.12", "0.12", "0.12", "0", "0", "0",
                     "--object", "2", "1", "0.7", "0.3", "0.4", "-0.03",
                     "0.04", "0.02", "0.1", "0.1", "0.1", "0", "0", "0"],
}


# config 5 at its full size: 40 variables, 300 timesteps.  Only the
# reference's log is kept (checksums, mesh hashes); the AMR driver's GPU
# test replays the run from the command line alone.
CASES["config5_300"] = list(CASES["config5"])
CASES["config5_300"][CASES["config5_300"].index("--num_vars") + 1] = "40"
CASES["config5_300"][CASES["config5_300"].index("--num_tsteps") + 1] = "300"
# config 5 with the objects at the sizes the benchmark's description
# names (spheres of radius 0.1, a cylinder of radius 0.05, a box of side
# 0.2; about 30k-53k blocks), for its meshes only: 2^3-cell blocks and one
# variable, since without --refine_ghost the marking does not depend on the
# cell count.
_c5 = CASES["config5"]
CASES["config5_named_mesh"] = _c5[:_c5.index("--num_objects")] + [
    "--num_objects", "4",
    "--object", "2", "1", "0.3", "0.3", "0.3", "0.01", "0.007", "0.005",
    "0.1", "0.1", "0.1", "0", "0", "0",
    "--object", "3", "1", "0.7", "0.6", "0.4", "-0.008", "0.006", "0.01",
    "0.1", "0.1", "0.1", "0", "0", "0",
    "--object", "20", "1", "0.5", "0.5", "0.7", "0.006", "-0.01", "0.004",
    "0.12", "0.05", "0.05", "0", "0", "0",
    "--object", "0", "1", "0.3", "0.7", "0.7", "0.007", "-0.005", "-0.009",
    "0.1", "0.1", "0.1", "0", "0", "0", "--error_tol", "0"]
for _k, _v in (("--nx", "2"), ("--ny", "2"), ("--nz", "2"),
               ("--num_vars", "1"), ("--num_tsteps", "300"),
               ("--max_blocks", "80000")):
    CASES["config5_named_mesh"][CASES["config5_named_mesh"].index(_k) + 1] = _v
REFLOG_ONLY = {"config5_300", "config5_named_mesh"}

HASH_STRIDE = {"config2": 10, "config5": 8, "config5_300": 100,
               "config5_named_mesh": 1000}
# cases whose marking is dumped: (every n-th refinement step, at most m)
MARK = {"amr7": (1, 1000), "amr7_objects": (1, 1000), "uniform27": (1, 1000),
        "mark_shapes": (1, 1000), "mark_shapes_ghost": (1, 1000),
        "config2": (8, 2), "config5": (6, 2)}


def run_case(name, args):
    with tempfile.TemporaryDirectory() as td:
        rlog = os.path.join(td, "r.log")
        hlog = os.path.join(td, "h.log")
        trc = os.path.join(td, "t.trc")
        base_env = dict(os.environ,
                        MAMR_REF_HASH_STRIDE=str(HASH_STRIDE.get(name, 1)))
        mlog = os.path.join(td, "m.mark")
        env = dict(base_env, MAMR_REF_LOG=rlog)
        if name in MARK:
            env.update(MAMR_MARK_DUMP=mlog,
                       MAMR_MARK_DUMP_EVERY=str(MARK[name][0]),
                       MAMR_MARK_DUMP_MAX=str(MARK[name][1]))
        r = subprocess.run([REF_BIN] + args, cwd=td, env=env,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name}: reference failed\n{r.stdout[-2000:]}")
        if name in MARK:
            with lzma.open(os.path.join(HERE, name + ".mark.xz"), "wb",
                           preset=9) as f:
                f.write(open(mlog, "rb").read())
        summary = [l for l in r.stdout.splitlines() if l.startswith("Summary")]
        if name in REFLOG_ONLY:
            with lzma.open(os.path.join(HERE, name + ".reflog.xz"), "wb",
                           preset=9) as f:
                f.write(open(rlog, "rb").read())
            return summary[-1] if summary else ""
        env = dict(base_env, MAMR_REF_LOG=hlog, MAMR_TRACE=trc)
        h = subprocess.run([HYB_BIN] + args, cwd=td, env=env,
                           capture_output=True, text=True)
        if h.returncode != 0:
            raise RuntimeError(f"{name}: hybrid failed\n{h.stdout[-2000:]}")
        ref_log = open(rlog, "rb").read()
        if open(hlog, "rb").read() != ref_log:
            raise RuntimeError(f"{name}: drop-in hybrid differs from the "
                               "reference")
        with lzma.open(os.path.join(HERE, name + ".reflog.xz"), "wb",
                       preset=9) as f:
            f.write(ref_log)
        with lzma.open(os.path.join(HERE, name + ".trace.xz"), "wb",
                       preset=9) as f:
            f.write(open(trc, "rb").read())
        return summary[-1] if summary else ""


def main(argv):
    if not os.path.exists(REF_BIN) or not os.path.exists(HYB_BIN):
        sys.path.insert(0, REPO)
        from miniamr_gb300 import build
        if not build.build_reference_binaries():
            sys.exit("make_golden.py: no reference sources (set "
                     "MAMR_REFERENCE_SRC to miniAMR's ref/ directory)")
    names = argv or list(CASES)
    meta_path = os.path.join(HERE, "cases.json")
    meta = json.load(open(meta_path)) if os.path.exists(meta_path) else {}
    for n in names:
        s = run_case(n, CASES[n])
        meta[n] = {"args": CASES[n], "reference_summary": s}
        print(n, s)
    json.dump(meta, open(meta_path, "w"), indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:])
