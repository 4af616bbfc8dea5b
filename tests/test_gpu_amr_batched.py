"""The batched path on the reference's own multi-level meshes.

Each recorded run is replayed with every stretch of stages between two
refinements executed as one batched, graph-captured call (the graph is
re-captured after each refinement), and every checksum must equal the
reference's bit for bit in FP64 -- the face exchange across level jumps
(coarse/4 and 4-cell sums) gathered inside the fused kernel, and for the
27-point runs (amr27; config2, the AMR sphere run at full size) the edge
and corner ghosts from their recipes, stale cells included."""
import os

import numpy as np
import pytest

from golden_util import GOLDEN, trace_path
from miniamr_gb300.abi import FP32, FP64, RUN_BATCHED, RUN_GRAPH
from miniamr_gb300.trace import read_trace, replay_batched

pytestmark = pytest.mark.gpu

RUNS = [n for n in ("amr7", "amr7_objects", "config5", "amr27", "config2")
        if os.path.exists(os.path.join(GOLDEN, n + ".trace.xz"))]


@pytest.mark.parametrize("name", RUNS)
def test_batched_replay_fp64_equals_reference(gpu_lib, name):
    recs = read_trace(trace_path(name))
    sums, ctx, _ = replay_batched(gpu_lib, recs, RUN_BATCHED | RUN_GRAPH,
                                  dtype=FP64)
    ctx.close()
    assert len(sums) > 0
    bad = [(v, got, rec) for v, got, rec in sums if got != rec]
    assert not bad, bad[:3]


@pytest.mark.parametrize("name", RUNS)
def test_batched_replay_fp32_within_1e6(gpu_lib, name):
    recs = read_trace(trace_path(name))
    sums, ctx, _ = replay_batched(gpu_lib, recs, RUN_BATCHED | RUN_GRAPH,
                                  dtype=FP32)
    ctx.close()
    rel = np.array([abs(got - rec) / abs(rec) for _, got, rec in sums
                    if rec != 0.0])
    assert rel.max() <= 1e-6, rel.max()
