"""The benchmark mesh pinned to the reference and to the oracle.

* uniform16_27 / uniform16_7: the benchmark's single-level mesh of 16^3
  blocks at an eighth of its size (4^3 initial blocks uniformly refined
  once: 512 blocks), 40 variables, 4 stages per timestep, 2 timesteps, the
  reference's checksums and cell hashes at every stage.  Replayed through
  the batched path (the pencil kernel) under every launch shape the tuner
  can pick: every FP64 checksum and the final cells, ghosts included,
  bit-identical to the reference's.
* the full benchmark mesh -- 8^3 initial blocks uniformly refined once
  (4096 blocks of 16^3), 40 variables, 27-point -- for one timestep of
  four stages (checksums on stages 0 and 2), batched + graph and plain, in
  FP64 and FP32: every checksum and every cell bit-identical to the oracle
  (the FP32 oracle rounds every operation to float in the same order).
"""
import numpy as np
import pytest

from golden_util import reflog, trace_path
from miniamr_gb300 import mesh as meshmod
from miniamr_gb300.abi import (FP32, FP64, RUN_BATCHED, RUN_GRAPH, RUN_PLAIN,
                               Config)
from miniamr_gb300.trace import (OP_SET_MESH, cell_hashes, read_trace,
                                 replay_batched)

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def _forced(lib, choice):
    """lib.context that forces launch-shape candidate `choice`."""
    orig = lib.context

    def make(cfg):
        c = orig(cfg)
        c.set_tuning(choice)
        return c
    return orig, make


@pytest.mark.parametrize("name", ["uniform16_27", "uniform16_7"])
def test_benchmark_mesh_every_shape_equals_reference(gpu_lib, name):
    sums_ref, hashes_ref, _ = reflog(name)
    recs = read_trace(trace_path(name))
    last_mesh = [r for r in recs if r.op == OP_SET_MESH][-1]
    blocks, numbers = last_mesh.args
    V = next(r.args[0].num_vars for r in recs if r.op == 1)
    choice, n_cands = 0, 1
    while choice < n_cands:
        orig, make = _forced(gpu_lib, choice)
        gpu_lib.context = make
        try:
            sums, ctx, _ = replay_batched(gpu_lib, recs,
                                          RUN_BATCHED | RUN_GRAPH, dtype=FP64)
        finally:
            gpu_lib.context = orig
        tun = ctx.tuning()
        assert tun["choice"] == choice
        n_cands = tun["candidates"]
        assert len(sums) == len(sums_ref)
        bad = [(v, got, rec) for v, got, rec in sums if got != rec]
        assert not bad, (choice, bad[:3])
        cells = ctx.download(blocks["slot"])
        assert cell_hashes(cells, numbers) == hashes_ref[-V:], \
            f"final cells differ from the reference (shape {choice})"
        ctx.close()
        choice += 1
    assert n_cands >= 3


def _benchmark_mesh(lib, dtype):
    init = (8, 8, 8)
    n0 = init[0] * init[1] * init[2]
    cap = n0 * 9 + 8
    cfg = Config.make(16, 16, 16, 40, cap, stencil=27, dtype=dtype)
    m = meshmod.initial_mesh(*init, 1, cap)
    ctx = lib.context(cfg)
    ctx.upload(np.arange(n0), lib.initial_values(cfg, n0))
    ctx.split(m.split_all())
    ctx.set_mesh(m.blocks())
    return ctx, m


@pytest.fixture(scope="module", params=[FP64, FP32], ids=["fp64", "fp32"])
def oracle_benchmark_run(request, oracle_lib):
    """The oracle's timestep of the full benchmark mesh (kept for the
    module: its pool is 8.6 GB of host memory)."""
    ctx, m = _benchmark_mesh(oracle_lib, request.param)
    sums = ctx.run_timesteps(1, 4, 2)
    yield request.param, ctx, m, sums
    ctx.close()


@pytest.mark.parametrize("flags", [RUN_BATCHED | RUN_GRAPH, RUN_PLAIN],
                         ids=["batched_graph", "plain"])
def test_full_benchmark_mesh_equals_oracle(gpu_lib, oracle_benchmark_run,
                                           flags):
    dtype, octx, m, osums = oracle_benchmark_run
    gctx, _ = _benchmark_mesh(gpu_lib, dtype)
    gsums = gctx.run_timesteps(1, 4, 2, flags=flags)
    assert gsums.shape == (2, 40)
    assert np.array_equal(bits(gsums), bits(osums))
    slots = m.sorted_slots()
    for part in np.array_split(slots, 16):
        assert np.array_equal(bits(gctx.download(part)),
                              bits(octx.download(part))), \
            f"cells differ in slots {part[0]}..{part[-1]}"
    gctx.close()
