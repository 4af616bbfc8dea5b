"""The AMR driver (mamr_amr_run: refinement bookkeeping, marking, stage
loop) over the CPU oracle against the reference's recorded runs.

For every recorded case the driver runs the case's command line and must
reproduce, exactly:
* every mesh the reference's refine() left -- the reference-side hook's
  FNV hash of (number, slot, level, nei_level, all four nei entries,
  centre) per block in sorted order, stale entries of reused slots
  included, and the block count;
* every split and consolidation job list (parent/child/target slots in
  the reference's order) the drop-in build recorded;
* every checksum of the reference, bit for bit (the oracle's stages are
  the reference's arithmetic).
The two large cases (config 2 and config 5) run with 2^3-cell blocks and
one variable: without --refine_ghost the marking does not depend on the
cell count, so their meshes and job lists are the reference's at full size;
their checksums are the GPU tests' business.
"""
import numpy as np
import pytest

from golden_util import (HEAVY, cases, check_jobs, check_meshes, reflog,
                         run_case, traced_cases)
from miniamr_gb300 import run as runmod
from miniamr_gb300.abi import RUN_PLAIN, AmrParams, MamrError


LIGHT = [n for n in traced_cases() if n not in HEAVY]


@pytest.mark.parametrize("name", LIGHT)
def test_driver_reproduces_reference_run(oracle_lib, name):
    args = cases()[name]["args"]
    spec, sums, st, ev = run_case(oracle_lib, args, RUN_PLAIN)
    check_meshes(oracle_lib, name, ev)
    check_jobs(name, ev)
    ref, _, _ = reflog(name)
    V = spec.opts["num_vars"]
    assert sums.size == len(ref)
    flat = sums.reshape(-1)
    for q, (var, val) in enumerate(ref):
        assert var == q % V
        assert flat[q].tobytes() == np.float64(val).tobytes(), \
            f"checksum {q} (var {var}): {flat[q]!r} != {val!r}"
    assert st["final_active"] == (ev[-1][2].shape[0]
                                  if any(e[0] == "mesh" for e in ev)
                                  else spec.opts["init_x"] *
                                  spec.opts["init_y"] * spec.opts["init_z"])


@pytest.mark.parametrize("name", [n for n in traced_cases() if n in HEAVY])
def test_driver_meshes_of_large_runs(oracle_lib, name):
    _, _, st, ev = run_case(oracle_lib, cases()[name]["args"], RUN_PLAIN,
                            shrink=True)
    check_meshes(oracle_lib, name, ev)
    check_jobs(name, ev)


def test_parse_defaults_and_refusals():
    spec = runmod.parse([])
    o = spec.opts
    assert (o["nx"], o["num_vars"], o["num_refine"], o["max_blocks"]) == \
        (10, 40, 5, 500)
    assert o["block_change"] == o["num_refine"]
    assert spec.tol == 1e-8
    for bad in (["--hilbert"], ["--time", "1.0"], ["--nx", "3"],
                ["--npx", "2"], ["--stencil", "9"], ["--bogus"],
                ["--num_objects", "1"], ["--plot_freq", "2"],
                ["--tuning", "-1"], ["--tuning"]):
        with pytest.raises(ValueError):
            runmod.parse(bad)
    # one-rank no-ops are accepted
    runmod.parse(["--lb_opt", "2", "--send_faces", "--rcb", "--reorder",
                  "1", "--comm_vars", "5"])
    assert spec.tuning == -1
    assert runmod.parse(["--tuning", "3", "--fp32"]).tuning == 3


def test_driver_errors(oracle_lib):
    spec = runmod.parse(["--init_x", "2", "--nx", "4", "--ny", "4", "--nz",
                         "4", "--num_vars", "2", "--max_blocks", "9",
                         "--num_refine", "2", "--uniform_refine", "1",
                         "--num_tsteps", "1", "--stages_per_ts", "1"])
    with oracle_lib.context(spec.config()) as ctx:
        # 2 blocks refine into 16: more than 9 slots
        with pytest.raises(MamrError, match="max_blocks"):
            ctx.amr_run(spec.params(RUN_PLAIN))
        p = spec.params(RUN_PLAIN)
        p.reserved[3] = 1
        with pytest.raises(MamrError, match="reserved"):
            ctx.amr_run(p)
        p = AmrParams.make(init=(0, 1, 1))
        with pytest.raises(MamrError, match="bad parameters"):
            ctx.amr_run(p)


def test_check_tolerance():
    spec = runmod.parse(["--num_vars", "2", "--error_tol", "2"])
    sums = np.array([[1.0, 2.0], [1.005, 2.0], [1.005, 2.1]])
    assert runmod.check_tolerance(spec, sums) == (2, 1)
    spec0 = runmod.parse(["--num_vars", "8", "--stencil", "0",
                          "--error_tol", "2"])
    s8 = np.ones((2, 8))
    s8[1, 3] = 5.0      # only variable 0 is checked for stencil 0
    assert runmod.check_tolerance(spec0, s8) is None
