"""Access to the committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py from the reference itself)."""
import ctypes as C
import json
import lzma
import os

import numpy as np

from miniamr_gb300 import run as runmod
from miniamr_gb300.abi import BLOCK_DTYPE
from miniamr_gb300.trace import OP_CONSOLIDATE, OP_SPLIT, read_trace

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return json.load(open(os.path.join(GOLDEN, "cases.json")))


def traced_cases():
    """Cases with a recorded drop-in trace (all but the log-only ones)."""
    return sorted(n for n in cases() if os.path.exists(trace_path(n)))


def reflog(name):
    """(checksums, cell_hashes, meshes) from the reference's hook log:
    checksums[i] = (var, value) of the i-th check_sum call, cell_hashes[i]
    the hash of that variable's cells, meshes = [(ts, n_active, hash)]."""
    sums, hashes, meshes = [], [], []
    with lzma.open(os.path.join(GOLDEN, name + ".reflog.xz"), "rt") as f:
        for line in f:
            p = line.split()
            if p[0] == "cs":
                v = int(p[3], 16)
                sums.append((int(p[2]),
                             __import__("struct").unpack(
                                 "<d", v.to_bytes(8, "little"))[0]))
                hashes.append(int(p[4], 16))
            elif p[0] == "mesh":
                meshes.append((int(p[1]), int(p[2]), p[3]))
    return sums, hashes, meshes


def trace_path(name):
    return os.path.join(GOLDEN, name + ".trace.xz")


def arg(args, flag, default=None):
    return args[args.index(flag) + 1] if flag in args else default


# Cases too large to replay through the CPU oracle inside the CPU suite;
# they are pinned by make_golden.py (hybrid == reference) and replayed on
# the GPU.
HEAVY = {"config2", "config5", "config5_300", "config5_named_mesh"}


def hashed_stages(hashes, V):
    """Checksum stages whose cell hashes the log carries (0 = not taken);
    returns first, middle and last of them."""
    st = [s for s in range(len(hashes) // V) if hashes[s * V] != 0]
    return {st[0], st[len(st) // 2], st[-1]} if st else set()


def mark_cases():
    """Cases with a marking fixture (<name>.mark.xz)."""
    return sorted(f[:-len(".mark.xz")] for f in os.listdir(GOLDEN)
                  if f.endswith(".mark.xz"))


def mark_path(name):
    return os.path.join(GOLDEN, name + ".mark.xz")


def mesh_hash(lib, blocks, numbers, cen) -> int:
    """The reference-side hook's hash of a mesh (oracle/ref_hooks.c), taken
    by the oracle library's helper."""
    f = lib.lib.mamr_oracle_mesh_hash
    f.restype = C.c_uint64
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    blocks = np.ascontiguousarray(blocks, dtype=BLOCK_DTYPE)
    numbers = np.ascontiguousarray(numbers, dtype=np.int64)
    cen = np.ascontiguousarray(cen, dtype=np.int32)
    return int(f(blocks.ctypes.data, numbers.ctypes.data, cen.ctypes.data,
                 len(blocks)))


def run_case(lib, args, run_flags=None, shrink=False, fp32=False):
    """Runs a recorded case's command line through mamr_amr_run on `lib`:
    (RunSpec, checksums, stats, events).  shrink: 2^3-cell blocks and one
    variable (the meshes stay the reference's where --refine_ghost is
    off)."""
    spec = runmod.parse(args)
    spec.fp32 = fp32
    if shrink:
        assert not spec.opts["refine_ghost"]
        spec.opts.update(nx=2, ny=2, nz=2, num_vars=1)
    cfg = spec.config()
    with lib.context(cfg) as ctx:
        sums, st, ev = ctx.amr_run(spec.params(run_flags), spec.objects,
                                   events=True)
    return spec, sums, st, ev


def check_meshes(lib, name, ev):
    """Every mesh event equals the reference's mesh after that refine():
    block count and hash.  lib: the oracle library (for the hash)."""
    _, _, meshes_ref = reflog(name)
    got = [(ts, len(b), f"{mesh_hash(lib, b, num, cen):016x}")
           for kind, ts, *rest in ev if kind == "mesh"
           for b, num, cen in [rest]]
    assert len(got) == len(meshes_ref)
    for g, r in zip(got, meshes_ref):
        assert g == r, f"mesh after refine({r[0]}) differs"


def check_jobs(name, ev):
    """The split/consolidate job lists equal those the drop-in build
    recorded, in order (for the cases with a recorded trace)."""
    if not os.path.exists(trace_path(name)):
        return
    recs = [r for r in read_trace(trace_path(name))
            if r.op in (OP_SPLIT, OP_CONSOLIDATE)]
    got = [e for e in ev if e[0] in ("split", "consolidate")]
    assert len(got) == len(recs)
    for e, r in zip(got, recs):
        assert e[0] == ("split" if r.op == OP_SPLIT else "consolidate")
        assert np.array_equal(e[2], r.args[0])
