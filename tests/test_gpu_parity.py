"""GPU library parity: bit-exact against the reference's golden vectors and
the CPU oracle, through the C ABI."""
import numpy as np
import pytest

from golden_util import (cases, hashed_stages, reflog, trace_path,
                         traced_cases)
from miniamr_gb300 import mesh as meshmod
from miniamr_gb300.abi import FP32, FP64, MamrError, Config
from miniamr_gb300.trace import read_trace, replay

pytestmark = pytest.mark.gpu
CASES = traced_cases()
# the variable-work stencils (--stencil 0) run on FP64 pools only
FP32_CASES = [c for c in CASES if "--stencil" not in cases()[c]["args"] or
              cases()[c]["args"][cases()[c]["args"].index("--stencil") + 1]
              != "0"]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", CASES)
def test_trace_fp64_bit_exact_vs_reference(gpu_lib, name):
    """The reference's own call sequence replayed on the GPU: every
    checksum bit-identical to the reference's, and every cell (ghosts
    included) at the first, middle and last checksum stage."""
    sums, hashes, _ = reflog(name)
    recs = read_trace(trace_path(name))
    V = next(r.args[0].num_vars for r in recs if r.op == 1)
    want = hashed_stages(hashes, V)
    res = replay(gpu_lib, recs, hash_stages=want)
    got = [(v, s) for v, s, _ in res.checksums]
    assert got == sums
    assert len(res.hashes) == len(want)
    for st, hs in res.hashes:
        assert hs == hashes[st * V:(st + 1) * V], f"cells differ, stage {st}"
    res.ctx.close()


@pytest.mark.parametrize("name", FP32_CASES)
def test_trace_fp32_vs_oracle_and_reference(gpu_lib, oracle_lib, name):
    """FP32 pools: bit-identical to the FP32 oracle (same operation order,
    correctly rounded FP32 division, exact fixed-point checksum) and within
    1e-6 relative of the reference's FP64 checksums."""
    sums, _, _ = reflog(name)
    recs = read_trace(trace_path(name))
    g = replay(gpu_lib, recs, dtype=FP32)
    o = replay(oracle_lib, recs, dtype=FP32)
    assert [s for _, s, _ in g.checksums] == [s for _, s, _ in o.checksums]
    slots = g.mesh["slot"]
    assert np.array_equal(bits(g.ctx.download(slots)),
                          bits(o.ctx.download(slots)))
    rel = [abs(s - r) / abs(r) for (_, s, _), (_, r) in zip(g.checksums, sums)
           if r != 0.0]
    assert max(rel) <= 1e-6, max(rel)
    g.ctx.close()
    o.ctx.close()


UNIFORM = [
    # (lattice, block, vars, stencil, refine passes, permute)
    ((2, 2, 2), (8, 8, 8), 4, 7, 0, 0),
    ((2, 2, 2), (8, 8, 8), 4, 27, 1, 0),
    ((3, 1, 2), (4, 6, 8), 3, 27, 1, 1),
    ((2, 2, 1), (16, 16, 16), 2, 7, 1, 1),
    ((1, 2, 2), (16, 16, 16), 2, 27, 1, 0),
]


@pytest.mark.parametrize("dtype", [FP64, FP32])
@pytest.mark.parametrize("case", UNIFORM)
def test_uniform_run_vs_oracle(gpu_lib, oracle_lib, case, dtype):
    (ix, iy, iz), (nx, ny, nz), V, st, passes, perm = case
    n0 = ix * iy * iz
    cap = n0 * (1 + 8 ** passes) + 8
    cfg = Config.make(nx, ny, nz, V, cap, stencil=st, dtype=dtype,
                      permute=perm)
    init = gpu_lib.initial_values(cfg, n0)
    outs = []
    for lib in (gpu_lib, oracle_lib):
        m = meshmod.initial_mesh(ix, iy, iz, passes, cap)
        ctx = lib.context(cfg)
        ctx.upload(np.arange(n0), init)
        for _ in range(passes):
            ctx.split(m.split_all())
        ctx.set_mesh(m.blocks())
        sums = ctx.run_timesteps(3, 2, 1)
        outs.append((sums, ctx.download(m.sorted_slots())))
        ctx.close()
    assert np.array_equal(bits(outs[0][0]), bits(outs[1][0]))
    assert np.array_equal(bits(outs[0][1]), bits(outs[1][1]))


def test_division_edge_values(gpu_lib, oracle_lib):
    """Stencil averages over cells spanning the whole FP64 range (tiny,
    huge, negative, zero) -- both division paths -- match the oracle's IEEE
    division bit for bit."""
    rng = np.random.default_rng(7)
    for st in (7, 27):
        cfg = Config.make(8, 8, 8, 2, 8, stencil=st, dtype=FP64)
        vals = np.zeros((8, 2, 10, 10, 10))
        mant = rng.uniform(-2, 2, size=(8, 2, 8, 8, 8))
        expo = rng.integers(-1070, 1015, size=(8, 2, 8, 8, 8))
        vals[:, :, 1:9, 1:9, 1:9] = np.ldexp(mant, expo) / 64.0
        vals[0, 0, 1:9, 1:9, 1:9] = np.ldexp(mant[0, 0], -930)
        m = meshmod.initial_mesh(2, 2, 2, 0, 8)
        outs = []
        for lib in (gpu_lib, oracle_lib):
            with lib.context(cfg) as ctx:
                ctx.upload(np.arange(8), vals)
                ctx.set_mesh(m.blocks())
                for s in range(2):
                    ctx.comm(0, 2, s)
                    ctx.stencil_driver(0, s)
                    ctx.stencil_driver(1, s)
                outs.append(ctx.download(np.arange(8)))
        assert np.array_equal(bits(outs[0]), bits(outs[1]))


def test_errors_are_reported_and_context_survives(gpu_lib):
    cfg = Config.make(8, 8, 8, 2, 16, stencil=7, dtype=FP32)
    m = meshmod.initial_mesh(2, 2, 2, 0, 16)
    with gpu_lib.context(cfg) as ctx:
        with pytest.raises(MamrError) as e:
            ctx.upload([99], np.zeros((1, 2, 10, 10, 10)))
        assert e.value.status == -1
        bad = m.blocks()
        bad["nei_level"][0, 1] = 5
        with pytest.raises(MamrError) as e:
            ctx.set_mesh(bad)
        assert e.value.status == -4
        ctx.set_mesh(m.blocks())
        v = np.zeros((8, 2, 10, 10, 10))
        v[3, 1, 4, 4, 4] = 5000.0      # outside the fixed-point window:
        ctx.upload(np.arange(8), v)    # the compensated FP64 sum instead
        assert ctx.check_sum(1) == 5000.0
        assert ctx.check_sum(0) == 0.0
        with pytest.raises(MamrError):
            ctx.comm(1, 5, 0)
        assert ctx.check_sum(1) == 5000.0   # context still usable


def test_long_mesh_refusals_keep_the_last_mesh(gpu_lib):
    """Mistakes planted in a 4913-block mesh (long enough that the library
    checks it on several threads) are refused with the status and message
    of the first mistake in list order; the context keeps the last mesh it
    took: a batched run after the refusals equals one without them."""
    from miniamr_gb300.abi import RUN_BATCHED
    cap = 5000
    cfg = Config.make(8, 8, 8, 1, cap, stencil=7, dtype=FP32)
    good = meshmod.initial_mesh(17, 17, 17, 0, cap).blocks()
    n, s = len(good), good["slot"]
    assert n >= 4096 and s.max() < cap - 1
    q = int(np.flatnonzero(good["nei_level"][:, 1] == 0)[n // 3])
    plants = []
    b = good.copy(); b["slot"][n - 1] = s[5]
    plants.append((b, -1, f"slot {s[5]} listed twice"))
    b = good.copy(); b["slot"][n // 2] = cap
    plants.append((b, -1, f"block {n // 2}: slot {cap} out of range"))
    b = good.copy(); b["nei_level"][n - 3, 2] = 3
    plants.append((b, -4, f"misconnected block (slot {s[n - 3]} face 2)"))
    b = good.copy(); b["nei"][q, 1, 0, 0] = -7
    plants.append((b, -4, f"misconnected block (slot {s[q]} face 1 nei -7)"))
    b = good.copy(); b["nei"][q, 1, 0, 0] = cap - 1
    plants.append((b, -4, f"neighbour slot {cap - 1} not active"))
    b = good.copy(); b["nei_level"][10, 0] = 4; b["slot"][n - 1] = s[0]
    plants.append((b, -4, f"misconnected block (slot {s[10]} face 0)"))
    rng = np.random.default_rng(11)
    vals = rng.uniform(-1, 1, size=(n, 1, 10, 10, 10))
    outs = []
    for refuse in (True, False):
        with gpu_lib.context(cfg) as ctx:
            ctx.upload(np.arange(n), vals)
            ctx.set_mesh(good)
            if refuse:
                for blk, status, msg in plants:
                    with pytest.raises(MamrError) as e:
                        ctx.set_mesh(blk)
                    assert e.value.status == status
                    assert str(e.value).endswith(msg), (str(e.value), msg)
            ctx.run_timesteps(2, 2, 1, flags=RUN_BATCHED)
            outs.append(ctx.download(np.arange(n)))
    assert np.array_equal(bits(outs[0]), bits(outs[1]))


def test_batched_refuses_a_coarse_face_that_omits_the_block(gpu_lib):
    """The batched descriptors of a multi-level mesh are built on the
    device; a fine block whose coarser neighbour does not list it on the
    shared face (which mamr_set_mesh does not check) is refused with the
    host builder's message, and the context keeps working."""
    from miniamr_gb300.abi import RUN_BATCHED
    from miniamr_gb300.trace import OP_CREATE, OP_SET_MESH
    recs = read_trace(trace_path("amr7"))
    cfg = Config.from_buffer_copy(bytes(
        next(r for r in recs if r.op == OP_CREATE).args[0]))
    good = next(r.args[0] for r in recs if r.op == OP_SET_MESH
                and len(set(r.args[0]["level"].tolist())) > 1)
    bad = good.copy()
    pos = {int(s): q for q, s in enumerate(bad["slot"])}
    done = False
    for q in range(len(bad)):
        for l in range(6):
            if bad["nei_level"][q, l] != bad["level"][q] - 1:
                continue
            pm = pos[int(bad["nei"][q, l, 0, 0])]
            face = bad["nei"][pm, l ^ 1]
            hit = np.argwhere(face == bad["slot"][q])
            if len(hit):
                iq, jq = hit[0]
                face[iq, jq] = face[1 - iq, jq]   # another fine neighbour
                done = True
                break
        if done:
            break
    assert done
    with gpu_lib.context(cfg) as ctx:
        ctx.set_mesh(bad)
        with pytest.raises(MamrError) as e:
            ctx.run_timesteps(1, 1, 0, flags=RUN_BATCHED)
        assert e.value.status == -4 and "child face" in str(e.value)
        ctx.set_mesh(good)
        ctx.run_timesteps(1, 1, 0, flags=RUN_BATCHED)


def test_division_selftest(gpu_lib):
    """The kernels' x/7 and x/27 equal IEEE division: FP32 on every float
    in [1, 2) (which decides its whole fast-path window) and on hashed
    floats of every class, FP64 on 2^26 hashed doubles of every class."""
    import ctypes as C
    f = gpu_lib.lib.mamr_selftest_division
    f.argtypes = [C.c_int64, C.POINTER(C.c_int64)]
    f.restype = C.c_int
    out = (C.c_int64 * 4)()
    assert f(1 << 26, out) == 0
    assert list(out) == [0, 0, 0, 0]


def test_stencil0_fp32_and_batched_are_refused(gpu_lib):
    """--stencil 0 runs on FP64 pools through the plain path only."""
    with pytest.raises(MamrError) as e:
        gpu_lib.context(Config.make(8, 8, 8, 8, 16, stencil=0, dtype=FP32))
    assert e.value.status == -5
    from miniamr_gb300.abi import RUN_BATCHED
    cfg = Config.make(8, 8, 8, 8, 16, stencil=0)
    with gpu_lib.context(cfg) as ctx:
        m = meshmod.initial_mesh(2, 1, 1, 0, 16)
        ctx.upload(np.arange(2), gpu_lib.initial_values(cfg, 2))
        ctx.set_mesh(m.blocks())
        ctx.set_work_params(*gpu_lib.work_coefficients(8))
        with pytest.raises(MamrError) as e:
            ctx.run_timesteps(1, 1, 1, flags=RUN_BATCHED)
        assert e.value.status == -5
        ctx.run_timesteps(1, 6, 1)           # the plain path runs


def test_code12_batched_is_refused(gpu_lib):
    """--code 1/2 exchanges whole ghost planes; the batched path gathers
    code-0 ghosts and refuses them (the plain path runs them)."""
    from miniamr_gb300.abi import RUN_BATCHED
    cfg = Config.make(8, 8, 8, 2, 16, stencil=27, code=1)
    with gpu_lib.context(cfg) as ctx:
        m = meshmod.initial_mesh(2, 1, 1, 0, 16)
        ctx.upload(np.arange(2), gpu_lib.initial_values(cfg, 2))
        ctx.set_mesh(m.blocks())
        with pytest.raises(MamrError) as e:
            ctx.run_timesteps(1, 1, 1, flags=RUN_BATCHED)
        assert e.value.status == -5
        ctx.run_timesteps(1, 2, 1)


@pytest.mark.parametrize("nxyz", [(8, 8, 8), (16, 16, 16), (4, 6, 8)])
def test_fp32_split_consolidate_edge_values(gpu_lib, oracle_lib, nxyz):
    """FP32 split and consolidation on values of every kind: children whose
    exponents span a few binades (the exact-sum path of the consolidation)
    or many (the compensated FP64 sum), +-0, float subnormals, huge
    magnitudes, mixed signs; split of the result back into children.  Every
    cell equals the oracle's bit for bit."""
    from miniamr_gb300.abi import CONSOLIDATE_DTYPE, SPLIT_DTYPE
    nx, ny, nz = nxyz
    V = 3
    rng = np.random.default_rng(11)
    shape = (8, V, nx + 2, ny + 2, nz + 2)
    # variable 0: exponents within a few binades (the exact-sum path);
    # variable 1: the same with zeros; variable 2: every kind mixed
    kind = rng.integers(0, 6, size=shape)
    kind[:, 0] = 0
    kind[:, 1] = np.where(kind[:, 1] % 2 == 0, 0, 3)
    mant = rng.uniform(1.0, 2.0, size=shape) * rng.choice([-1.0, 1.0],
                                                           size=shape)
    expo = np.where(kind == 0, rng.integers(-3, 3, size=shape),
           np.where(kind == 1, rng.integers(-40, 40, size=shape),
           np.where(kind == 2, rng.integers(-120, -100, size=shape),
                    rng.integers(-8, 8, size=shape))))
    vals = np.ldexp(mant, expo)
    vals[kind == 3] = 0.0
    vals[kind == 4] *= np.float32(2.0 ** 90)          # huge
    sub = rng.random(size=shape) < 0.03
    sub[:, :2] = False
    vals[sub] = rng.integers(1, 1 << 20, size=int(sub.sum())) * 2.0 ** -149
    negz = rng.random(size=shape) < 0.02
    negz[:, 0] = False
    vals[negz] = -0.0
    vals = vals.astype(np.float32).astype(np.float64)   # exact floats
    cfg = Config.make(nx, ny, nz, V, 24, stencil=7, dtype=FP32)
    cons = np.zeros(1, dtype=CONSOLIDATE_DTYPE)
    cons["child"][0] = np.arange(8)
    cons["target"][0] = 8
    split = np.zeros(1, dtype=SPLIT_DTYPE)
    split["parent"][0] = 8
    split["child"][0] = np.arange(12, 20)
    outs = []
    for lib in (gpu_lib, oracle_lib):
        with lib.context(cfg) as ctx:
            ctx.upload(np.arange(8), vals)
            ctx.consolidate(cons)
            ctx.split(split)
            outs.append(ctx.download(np.arange(24)))
    assert np.array_equal(bits(outs[0]), bits(outs[1]))


@pytest.mark.parametrize("dtype", [FP64, FP32])
def test_checksums_follow_every_change(gpu_lib, oracle_lib, dtype):
    """mamr_check_sum after each kind of change to the pool or the mesh --
    upload, another mesh, comm, one stencil, split, consolidation, a run --
    equals the oracle's after the same calls (the FP64 path sums every
    variable on the first call after a change and reuses the sums until
    the next one).  Split and consolidation write a slot the current mesh
    already lists, so only their own call changes what the sums see."""
    from miniamr_gb300.abi import CONSOLIDATE_DTYPE, SPLIT_DTYPE
    V = 3
    cfg = Config.make(8, 8, 8, V, 40, stencil=7, dtype=dtype)
    init = gpu_lib.initial_values(cfg, 8)
    mb = meshmod.initial_mesh(2, 2, 2, 0, 40).blocks()

    def relabel(old, new):
        out = mb.copy()
        out["slot"][out["slot"] == old] = new
        out["nei"][out["nei"] == old] = new
        return out
    rng = np.random.default_rng(3)
    other = rng.uniform(0, 1, size=(1, V, 10, 10, 10))
    split = np.zeros(1, dtype=SPLIT_DTYPE)
    split["parent"][0] = 9
    split["child"][0] = np.arange(10, 18)
    cons = np.zeros(1, dtype=CONSOLIDATE_DTYPE)
    cons["child"][0] = np.arange(10, 18)
    cons["target"][0] = 20
    outs = []
    for lib in (gpu_lib, oracle_lib):
        got = []
        with lib.context(cfg) as ctx:
            def sums():
                got.append([ctx.check_sum(v) for v in range(V)])
                got.append([ctx.check_sum(v) for v in reversed(range(V))])
            ctx.upload(np.arange(8), init)
            ctx.set_mesh(mb)
            sums()
            ctx.upload([3], other)
            sums()
            ctx.set_mesh(relabel(0, 10))
            sums()
            ctx.set_mesh(mb)
            sums()
            ctx.comm(0, V, 0)
            sums()
            ctx.stencil_driver(1, 0)
            sums()
            ctx.upload([9], other)
            ctx.set_mesh(relabel(0, 10))
            sums()
            ctx.split(split)
            sums()
            ctx.set_mesh(relabel(0, 20))
            sums()
            ctx.consolidate(cons)
            sums()
            ctx.run_timesteps(1, 2, 1)
            sums()
        outs.append(np.array(got))
    assert np.array_equal(bits(outs[0]), bits(outs[1]))
    # the sums do move: not all rows alike
    assert len({tuple(r) for r in outs[0].tolist()}) > 5


def _window_values(n, nxyz, V):
    """Cells in and out of the FP32 checksum's fixed-point window (v == 0
    or 2^-52 <= |v| < 2^10): variable 0 entirely inside, variable 1 with
    one cell too large for the accumulator, variable 2 with a block of
    cells too small to register, variable 3 with an infinite cell."""
    rng = np.random.default_rng(3)
    X = nxyz + 2
    v = np.zeros((n, V, X, X, X))
    v[:, :, 1:-1, 1:-1, 1:-1] = rng.uniform(0, 1, (n, V) + (nxyz,) * 3)
    v[3, 1, 4, 4, 4] = 5000.0
    v[5, 2, 1:-1, 1:-1, 1:-1] = 1e-20
    v[6, 3, 2, 3, 4] = np.inf
    return v


@pytest.mark.parametrize("flags", [0, 1 | 2], ids=["plain", "batched_graph"])
@pytest.mark.parametrize("stencil", [7, 27])
@pytest.mark.parametrize("nxyz", [8, 16])
def test_fp32_checksum_window_fallback(gpu_lib, oracle_lib, nxyz, stencil,
                                       flags):
    """FP32 checksums of variables with a cell outside the fixed-point
    window take the reference's order in compensated FP64 instead of
    failing: single check_sum calls and the checksums of plain and batched
    runs (fused into the pencil, warp-per-block and generic stage kernels)
    equal the oracle's bit for bit, and variables inside the window keep
    the exact fixed-point sum."""
    V, cap = 4, 80
    cfg = Config.make(nxyz, nxyz, nxyz, V, cap, stencil=stencil, dtype=FP32)
    init = _window_values(8, nxyz, V)
    out = []
    for lib in (gpu_lib, oracle_lib):
        m = meshmod.initial_mesh(2, 2, 2, 1, cap)
        with lib.context(cfg) as ctx:
            ctx.upload(np.arange(8), init)
            ctx.split(m.split_all())
            ctx.set_mesh(m.blocks())
            single = [ctx.check_sum(v) for v in range(V)]
            sums = ctx.run_timesteps(2, 2, 1, flags=flags)
            out.append((np.array(single), sums,
                        ctx.download(m.sorted_slots())))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(bits(a), bits(b))
    single, sums, _ = out[0]
    assert np.isfinite(single[:3]).all() and np.isinf(single[3])
    assert np.isfinite(sums[:, :3]).all()
