"""The AMR driver on the GPU: whole runs from the reference's command line
(mamr_amr_run -- marking on the device, the library's own split and
consolidation bookkeeping, cell movement on the device, each stretch of
stages one batched graph-captured call) against the reference's recorded
runs.

* every recorded case, FP64, on the batched path where it runs the case and
  on the per-call path: every checksum bit-identical to the reference's,
  every mesh (block count and the reference-side hash of numbers, slots,
  neighbour tables and centres) and every job list equal;
* config 2 (the AMR sphere run, 16^3 blocks, 27-point, 100 timesteps) and
  config 5 (four moving objects, 8^3 blocks, up to ~23k blocks on six
  levels, 20 timesteps) at full size, the same checks;
* config 5 at its full 40 variables and 300 timesteps (151 refinements):
  FP64 checksums bit-identical to the reference's own log, meshes equal,
  and FP32 cells within 1e-6 relative of them at every checksum;
* config 5 with its objects at the sizes the benchmark's description names
  (30k-53k blocks), 300 timesteps on 2^3-cell blocks: every mesh and
  checksum the reference's.
"""
import os

import numpy as np
import pytest

from golden_util import (GOLDEN, HEAVY, cases, check_jobs, check_meshes,
                         reflog, run_case)
from miniamr_gb300.abi import RUN_PLAIN

pytestmark = pytest.mark.gpu

ALL = sorted(n for n in cases() if n != "config5_300")


def _equal_sums(name, spec, sums):
    ref, _, _ = reflog(name)
    V = spec.opts["num_vars"]
    assert sums.size == len(ref), (sums.size, len(ref))
    got = sums.reshape(-1)
    want = np.array([v for _, v in ref])
    bad = np.nonzero(got.view(np.uint64) != want.view(np.uint64))[0]
    assert bad.size == 0, \
        f"{bad.size} checksums differ, first {bad[0]} (var {bad[0] % V})"


@pytest.mark.parametrize("path", ["auto", "plain"])
@pytest.mark.parametrize("name", ALL)
def test_driver_run_equals_reference(gpu_lib, oracle_lib, name, path):
    args = cases()[name]["args"]
    if path == "plain" and name in HEAVY:
        pytest.skip("the large runs take the batched path only")
    spec, sums, st, ev = run_case(gpu_lib, args,
                                  RUN_PLAIN if path == "plain" else None)
    _equal_sums(name, spec, sums)
    check_meshes(oracle_lib, name, ev)
    check_jobs(name, ev)


@pytest.mark.skipif(not os.path.exists(
    os.path.join(GOLDEN, "config5_300.reflog.xz")),
    reason="no 300-timestep config 5 log")
def test_config5_300_timesteps(gpu_lib, oracle_lib):
    args = cases()["config5_300"]["args"]
    spec, sums, st, ev = run_case(gpu_lib, args)
    _equal_sums("config5_300", spec, sums)
    check_meshes(oracle_lib, "config5_300", ev)
    assert st["refinements"] == 151
    _, s32, _, _ = run_case(gpu_lib, args, fp32=True)
    rel = np.abs(s32 - sums) / np.abs(sums)
    assert rel.max() <= 1e-6, rel.max()


def test_command_line(gpu_lib, capsys):
    """python -m miniamr_gb300.run with a recorded case's own options:
    exits 0 (every checksum within the case's tolerance) and prints the
    reference's final checksums."""
    from miniamr_gb300 import run as runmod
    args = cases()["amr7"]["args"]
    assert runmod.main(args) == 0
    out = capsys.readouterr().out
    ref, _, _ = reflog("amr7")
    V = int(args[args.index("--num_vars") + 1])
    assert f"{ref[-V][1]:.15e}" in out
    assert runmod.main(args + ["--fp32"]) == 0
