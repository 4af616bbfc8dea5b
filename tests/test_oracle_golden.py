"""The CPU oracle against the reference's golden vectors (no GPU).

The fixtures come from the reference itself (tests/golden/make_golden.py):
every checksum it computed, bit for bit, and a hash of every cell at each
checksum.  These tests pin the oracle -- the checker the GPU library is
compared with -- to the reference, and pin the host-side mesh builder and
initial values used by the benchmark to the reference's init()/refine().
"""
import numpy as np
import pytest

from golden_util import (HEAVY, arg, cases, hashed_stages, reflog,
                         trace_path, traced_cases)
from miniamr_gb300 import mesh as meshmod
from miniamr_gb300.abi import FP64, Config
from miniamr_gb300.trace import read_trace, replay

CASES = [c for c in traced_cases() if c not in HEAVY]


@pytest.mark.parametrize("name", CASES)
def test_trace_replay_matches_reference(oracle_lib, name):
    sums, hashes, _ = reflog(name)
    recs = read_trace(trace_path(name))
    V = next(r.args[0].num_vars for r in recs if r.op == 1)
    want = hashed_stages(hashes, V)
    res = replay(oracle_lib, recs, hash_stages=want)
    assert len(res.checksums) == len(sums)
    for (var, got, rec), (rvar, rval) in zip(res.checksums, sums):
        assert var == rvar
        assert got == rec == rval          # bit-exact
    assert len(res.hashes) == len(want)
    for st, hs in res.hashes:
        assert hs == hashes[st * V:(st + 1) * V], f"stage {st}"


def _driver_checksums(ctx, V, num_ts, spt, freq):
    """ref/driver.c:73-108 through the ABI, one call at a time."""
    out = []
    stage_g = 0
    for _ in range(num_ts):
        for st in range(spt):
            ctx.comm(0, V, stage_g)
            for v in range(V):
                ctx.stencil_driver(v, stage_g)
                if freq and st % freq == 0:
                    out.append((v, ctx.check_sum(v)))
            stage_g += 1
    return out


def test_config1_from_mesh_builder(oracle_lib):
    """config 1 built by the host mesh builder (no trace): the initial
    lattice and init() values reproduce every reference checksum."""
    a = cases()["config1"]["args"]
    sums, hashes, _ = reflog("config1")
    V = int(arg(a, "--num_vars"))
    m = meshmod.initial_mesh(2, 2, 2, 0, 8)
    cfg = Config.make(8, 8, 8, V, 8, stencil=7, dtype=FP64)
    with oracle_lib.context(cfg) as ctx:
        ctx.upload(np.arange(8), oracle_lib.initial_values(cfg, 8))
        ctx.set_mesh(m.blocks())
        got = [(v, ctx.check_sum(v)) for v in range(V)]
        got += _driver_checksums(ctx, V, 20, 1, 1)
    assert got == sums


def test_uniform27_from_mesh_builder(oracle_lib):
    """uniform refinement (refine(0), two passes) by the host mesh builder:
    slots, numbering, split data and sorted order reproduce the reference's
    checksums exactly."""
    sums, _, _ = reflog("uniform27")
    V, nx, ny, nz = 3, 4, 6, 8
    m = meshmod.initial_mesh(2, 1, 3, 2, 4000)
    cfg = Config.make(nx, ny, nz, V, 4000, stencil=27, dtype=FP64)
    with oracle_lib.context(cfg) as ctx:
        ctx.upload(np.arange(6), oracle_lib.initial_values(cfg, 6))
        ctx.set_mesh(m.blocks())
        got = [(v, ctx.check_sum(v)) for v in range(V)]
        for _ in range(2):
            ctx.split(m.split_all())
        ctx.set_mesh(m.blocks())
        got += _driver_checksums(ctx, V, 5, 2, 1)
    assert got == sums


def test_initial_values_match_reference_init(oracle_lib):
    """mamr_initial_values == the reference's init() (its first checksums
    are those of the initial blocks)."""
    sums, _, _ = reflog("config1")
    cfg = Config.make(8, 8, 8, 40, 8)
    vals = oracle_lib.initial_values(cfg, 8)
    for v in range(40):
        s = 0.0
        for b in range(7, -1, -1):      # sorted order: number descending
            bs = 0.0
            for x in vals[b, v, 1:9, 1:9, 1:9].reshape(-1):
                bs += float(x)
            s += bs
        assert s == sums[v][1]
