"""The batched path (one fused ghost+stencil+checksum launch per stage,
ping-pong pools, optional CUDA graph) against the plain per-call path:
every cell and every checksum bit-identical."""
import numpy as np
import pytest

from golden_util import trace_path
from miniamr_gb300 import mesh as meshmod
from miniamr_gb300.abi import (FP32, FP64, RUN_BATCHED, RUN_GRAPH,
                               RUN_NO_GHOSTS, RUN_PER_BLOCK, Config,
                               MamrError)
from miniamr_gb300.trace import read_trace, replay

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


UNIFORM = [
    ((2, 2, 2), (8, 8, 8), 3, 7, 1),
    ((2, 2, 2), (8, 8, 8), 3, 27, 1),
    ((2, 1, 2), (16, 16, 16), 2, 7, 1),
    ((1, 2, 2), (16, 16, 16), 2, 27, 1),
    ((3, 1, 2), (4, 6, 8), 2, 27, 1),
    ((2, 2, 1), (6, 6, 6), 2, 7, 0),
]


@pytest.mark.parametrize("flags", [RUN_BATCHED, RUN_BATCHED | RUN_GRAPH,
                                   RUN_PER_BLOCK])
@pytest.mark.parametrize("dtype", [FP64, FP32])
@pytest.mark.parametrize("case", UNIFORM)
def test_batched_equals_plain_uniform(gpu_lib, case, dtype, flags):
    (ix, iy, iz), (nx, ny, nz), V, st, passes = case
    n0 = ix * iy * iz
    cap = n0 * (1 + 8 ** passes) + 8
    cfg = Config.make(nx, ny, nz, V, cap, stencil=st, dtype=dtype)
    init = gpu_lib.initial_values(cfg, n0)
    outs = []
    for fl in (0, flags):
        m = meshmod.initial_mesh(ix, iy, iz, passes, cap)
        with gpu_lib.context(cfg) as ctx:
            ctx.upload(np.arange(n0), init)
            for _ in range(passes):
                ctx.split(m.split_all())
            ctx.set_mesh(m.blocks())
            s1 = ctx.run_timesteps(2, 3, 2, flags=fl)
            s2 = ctx.run_timesteps(1, 3, 1, first_stage=6, flags=fl)
            outs.append((s1, s2, ctx.download(np.arange(cap))))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(bits(a), bits(b))


def _multilevel_prefix(recs, n_meshes=2):
    """The records of a run up to its n-th multi-level mesh (a state on
    several levels without replaying the whole run)."""
    from miniamr_gb300.trace import OP_SET_MESH
    seen = 0
    for q, r in enumerate(recs):
        if r.op == OP_SET_MESH and len(set(r.args[0]["level"].tolist())) > 1:
            seen += 1
            if seen == n_meshes:
                return recs[:q + 1]
    return recs


@pytest.mark.parametrize("name", ["amr7", "amr7_objects", "amr27",
                                  "config2"])
@pytest.mark.parametrize("dtype", [FP64, FP32])
def test_batched_equals_plain_multilevel(gpu_lib, name, dtype):
    """The reference's own multi-level meshes (states reached by replaying
    its recorded runs), every cell and checksum against the plain path, by
    every launch-shape candidate: face ghosts across level jumps (coarse/4
    and 4-cell sums) gathered inside the fused kernel (amr7's 8^3 blocks
    include the warp-per-block kernel's); for the 27-point stencil also the
    edge and corner ghosts -- chains of face exchanges, level-jump
    transforms and cells no exchange writes -- from their recipes."""
    recs = read_trace(trace_path(name))
    if name == "config2":          # 16^3 blocks: the state after its 2nd
        recs = _multilevel_prefix(recs)   # multi-level mesh
    res = replay(gpu_lib, recs, dtype=dtype)
    assert len(np.unique(res.mesh["level"])) > 1
    ctx = res.ctx
    cap = ctx.cfg.max_blocks
    every = np.arange(cap)
    state = ctx.download(every)

    def run(flags, choice=None):
        ctx.upload(every, state)
        ctx.set_tuning(-1 if choice is None else choice)
        s = ctx.run_timesteps(2, 2, 1, flags=flags)
        return s, ctx.download(every), ctx.tuning()

    ref = run(0)
    n = run(RUN_BATCHED)[2]["candidates"]
    kernels = set()
    for k in range(n):
        got = run(RUN_BATCHED | RUN_GRAPH, k)
        assert got[2]["choice"] == k
        kernels.add(got[2]["planes_per_thread"] == 0)
        for a, b in zip(ref[:2], got[:2]):
            assert np.array_equal(bits(a), bits(b)), (k, got[2])
    if name == "amr7":
        assert kernels == {True, False}
    if name in ("amr7", "amr27", "config2"):
        # the double-buffered tile kernel is among the shapes tried
        assert n >= 3
    ctx.close()


SHAPE_CASES = [
    ((2, 1, 2), (16, 16, 16), 3, 27, 1),   # pencil kernel
    ((1, 2, 2), (16, 16, 16), 2, 7, 1),
    ((2, 2, 2), (8, 8, 8), 5, 7, 1),       # generic kernel, 5 vars: the
    ((3, 1, 2), (4, 6, 8), 5, 27, 1),      # 4-per-CTA shape has a part group
]


@pytest.mark.parametrize("dtype", [FP64, FP32])
@pytest.mark.parametrize("case", SHAPE_CASES)
def test_every_launch_shape_equals_plain(gpu_lib, case, dtype):
    """Each launch-shape candidate of the autotuner, forced in turn, gives
    the plain path's cells and checksums bit for bit; the automatic choice
    is one of them."""
    (ix, iy, iz), (nx, ny, nz), V, st, passes = case
    n0 = ix * iy * iz
    cap = n0 * (1 + 8 ** passes) + 8
    cfg = Config.make(nx, ny, nz, V, cap, stencil=st, dtype=dtype)
    init = gpu_lib.initial_values(cfg, n0)

    def run(flags, choice=None):
        m = meshmod.initial_mesh(ix, iy, iz, passes, cap)
        with gpu_lib.context(cfg) as ctx:
            if choice is not None:
                ctx.set_tuning(choice)
            ctx.upload(np.arange(n0), init)
            for _ in range(passes):
                ctx.split(m.split_all())
            ctx.set_mesh(m.blocks())
            s = ctx.run_timesteps(2, 2, 1, flags=flags)
            return s, ctx.download(np.arange(cap)), ctx.tuning()

    ref = run(0)
    auto = run(RUN_BATCHED)
    n = auto[2]["candidates"]
    assert n >= 2 and 0 <= auto[2]["choice"] < n
    for k in range(n):
        got = run(RUN_BATCHED | RUN_GRAPH, k)
        assert got[2]["choice"] == k
        for a, b in zip(ref[:2], got[:2]):
            assert np.array_equal(bits(a), bits(b)), (k, got[2])


@pytest.mark.parametrize("stencil", [7, 27])
@pytest.mark.parametrize("dtype", [FP64, FP32])
def test_pencil_division_fixup(gpu_lib, dtype, stencil):
    """Sums outside the window where the three-step quotient is exact
    (-0, zero, subnormal, huge) on the 16^3 pencil path: the kernel's
    fix-up pass stores the IEEE quotient and moves the FP32 checksum term,
    so every cell and every checksum equals the plain path's."""
    rng = np.random.default_rng(11)
    ix, iy, iz, V = 2, 1, 3, 3
    n0 = ix * iy * iz
    cfg = Config.make(16, 16, 16, V, n0 + 8, stencil=stencil, dtype=dtype)
    mant = rng.uniform(-2, 2, size=(n0, V, 16, 16, 16))
    lo, hi = (-1070, 1015) if dtype == FP64 else (-149, 8)
    expo = rng.integers(lo, hi, size=mant.shape)
    vals = np.zeros((n0, V, 18, 18, 18))
    inner = vals[:, :, 1:17, 1:17, 1:17]
    inner[...] = np.ldexp(mant, expo) / (64.0 if dtype == FP64 else 1.0)
    inner[0, 0] = -0.0                      # sums of -0: the quotient is -0
    inner[1, 1] = np.ldexp(mant[1, 1], lo + 8)   # subnormal sums
    inner[2, 2, :8] = 0.0
    outs = []
    for fl in (0, RUN_BATCHED | RUN_GRAPH):
        m = meshmod.initial_mesh(ix, iy, iz, 0, n0 + 8)
        with gpu_lib.context(cfg) as ctx:
            ctx.upload(np.arange(n0), vals)
            ctx.set_mesh(m.blocks())
            s = ctx.run_timesteps(2, 2, 1, flags=fl)
            outs.append((s, ctx.download(np.arange(n0))))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(bits(a), bits(b))
    assert np.signbit(outs[1][1][0, 0, 8, 8, 8])


def test_batched_27_permute_is_refused(gpu_lib):
    """With --permute the exchange phases run in a stage-dependent order,
    and 27-point edge and corner ghosts then carry neighbours' ghost values
    from the previous stage: the batched path refuses it (the plain path
    runs it, tests/test_gpu_parity.py) and the context keeps working."""
    recs = read_trace(trace_path("amr27_permute"))
    res = replay(gpu_lib, recs)
    with pytest.raises(MamrError) as e:
        res.ctx.run_timesteps(1, 1, 1, flags=RUN_BATCHED)
    assert e.value.status == -5 and "permute" in str(e.value)
    res.ctx.run_timesteps(1, 1, 1)
    res.ctx.close()


@pytest.mark.parametrize("dtype", [FP64, FP32])
def test_no_ghosts_runs_then_a_full_run(gpu_lib, dtype):
    """A batched 7-point run with MAMR_RUN_NO_GHOSTS (its last stage writes
    no ghost layer back), then a run without the flag: every cell of the
    pool -- ghosts included -- and every checksum as the plain path's, on
    the reference's own multi-level mesh (the AMR driver's GPU tests cover
    the flag with splits and consolidations between the runs).  The flag
    is refused without the batched path and with the 27-point stencil."""
    recs = _multilevel_prefix(read_trace(trace_path("amr7")))
    res = replay(gpu_lib, recs, dtype=dtype)
    ctx = res.ctx
    cap = ctx.cfg.max_blocks
    every = np.arange(cap)
    state = ctx.download(every)
    outs = []
    for first in (0, RUN_BATCHED | RUN_GRAPH | RUN_NO_GHOSTS):
        ctx.upload(every, state)
        s1 = ctx.run_timesteps(1, 3, 1, flags=first)
        s2 = ctx.run_timesteps(1, 2, 1, first_stage=3,
                               flags=RUN_BATCHED if first else 0)
        outs.append((s1, s2, ctx.download(every)))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(bits(a), bits(b))
    with pytest.raises(MamrError, match="NO_GHOSTS"):
        ctx.run_timesteps(1, 1, 1, flags=RUN_NO_GHOSTS)
    ctx.close()
    cfg = Config.make(8, 8, 8, 2, 16, stencil=27, dtype=dtype)
    with gpu_lib.context(cfg) as c27:
        with pytest.raises(MamrError, match="NO_GHOSTS"):
            c27.run_timesteps(1, 1, 1, flags=RUN_BATCHED | RUN_NO_GHOSTS)
