"""Recorded miniAMR runs at the mamr_* boundary, and their replay.

A trace is the exact sequence of ABI calls the reference's own driver,
init and refine code made through the drop-in translation units
(miniamr_gb300/dropin/), recorded on a machine that has the reference
sources (format in oracle/trace_hooks.c).  Replaying it through any
implementation of the ABI repeats that run call for call -- mesh changes,
split/consolidate jobs, comm/stencil/check_sum -- and the recorded
check_sum results are the reference's own checksums.

Initial cell data is not stored: the replay regenerates it with
mamr_initial_values() (the reference's init() values) and checks it against
the recorded hash.
"""
from __future__ import annotations

import gzip
import lzma
import struct
from dataclasses import dataclass

import numpy as np

from .abi import (BLOCK_DTYPE, CONSOLIDATE_DTYPE, SPLIT_DTYPE, Config,
                  Context, Library)

OP_CREATE, OP_UPLOAD, OP_SET_MESH, OP_COMM, OP_STENCIL, OP_CHECK_SUM, \
    OP_SPLIT, OP_CONSOLIDATE, OP_WORK_PARAMS = range(1, 10)


@dataclass
class Record:
    op: int
    args: tuple


def _open(path: str) -> bytes:
    if path.endswith(".xz"):
        return lzma.open(path, "rb").read()
    if path.endswith(".gz"):
        return gzip.open(path, "rb").read()
    with open(path, "rb") as f:
        return f.read()


def read_trace(path: str) -> list[Record]:
    data = _open(path)
    if data[:8] != b"MAMRTRC1":
        raise ValueError(f"{path}: not a mamr trace")
    pos, out = 8, []
    while pos < len(data):
        op, n = struct.unpack_from("<ii", data, pos)
        pos += 8
        p = data[pos:pos + n]
        pos += n
        if op == OP_CREATE:
            cfg = Config.from_buffer_copy(p)
            out.append(Record(op, (cfg,)))
        elif op == OP_UPLOAD:
            (m,) = struct.unpack_from("<i", p, 0)
            slots = np.frombuffer(p, "<i4", m, 4).copy()
            (h,) = struct.unpack_from("<Q", p, 4 + 4 * m)
            out.append(Record(op, (slots, h)))
        elif op == OP_SET_MESH:
            (m,) = struct.unpack_from("<i", p, 0)
            blocks = np.frombuffer(p, BLOCK_DTYPE, m, 4).copy()
            numbers = np.frombuffer(p, "<i8", m,
                                    4 + BLOCK_DTYPE.itemsize * m).copy()
            out.append(Record(op, (blocks, numbers)))
        elif op == OP_COMM:
            out.append(Record(op, struct.unpack_from("<iii", p, 0)))
        elif op == OP_STENCIL:
            out.append(Record(op, struct.unpack_from("<ii", p, 0)))
        elif op == OP_CHECK_SUM:
            var, _, s = struct.unpack_from("<iid", p, 0)
            out.append(Record(op, (var, s)))
        elif op == OP_SPLIT:
            (m,) = struct.unpack_from("<i", p, 0)
            out.append(Record(op, (np.frombuffer(p, SPLIT_DTYPE, m, 4).copy(),)))
        elif op == OP_CONSOLIDATE:
            (m,) = struct.unpack_from("<i", p, 0)
            out.append(Record(op, (np.frombuffer(p, CONSOLIDATE_DTYPE, m,
                                                 4).copy(),)))
        elif op == OP_WORK_PARAMS:
            (m,) = struct.unpack_from("<i", p, 0)
            (a1,) = struct.unpack_from("<d", p, 8)
            a0 = np.frombuffer(p, "<f8", m, 16).copy()
            out.append(Record(op, (a1, a0)))
        else:
            raise ValueError(f"{path}: unknown op {op}")
    return out


def upload_hash(a: np.ndarray) -> int:
    """Hash of an upload buffer (oracle/trace_hooks.c): the sum over 64-bit
    words q of bits[q] * (mix64(q) | 1), mod 2^64."""
    bits = np.ascontiguousarray(a, dtype=np.float64).reshape(-1).view(
        np.uint64)
    with np.errstate(over="ignore"):
        w = _mix64(np.arange(bits.size, dtype=np.uint64)) | np.uint64(1)
        return int((bits * w).sum(dtype=np.uint64))


def _mix64(z: np.ndarray) -> np.ndarray:
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def cell_hashes(cells: np.ndarray, numbers: np.ndarray) -> list[int]:
    """Per-variable cell hashes of an active mesh (the var_cell_hash of
    oracle/ref_hooks.c).  cells: [n_blocks in sorted order][V][X][Y][Z]
    doubles; numbers: the blocks' numbers in the same order."""
    n, V = cells.shape[:2]
    per = int(np.prod(cells.shape[2:]))
    with np.errstate(over="ignore"):
        pos = np.arange(n, dtype=np.uint64) << np.uint64(32)
        wn = _mix64(pos | np.uint64(0xFFFFFFFF)) | np.uint64(1)
        base = (numbers.astype(np.int64).view(np.uint64) * wn).sum(
            dtype=np.uint64)
        w = _mix64(pos[:, None] | np.arange(per, dtype=np.uint64)[None, :]) \
            | np.uint64(1)
        out = []
        for v in range(V):
            bits = np.ascontiguousarray(cells[:, v]).reshape(n, per).view(
                np.uint64)
            out.append(int((base + (bits * w).sum(dtype=np.uint64))
                           & np.uint64(0xFFFFFFFFFFFFFFFF)))
    return out


@dataclass
class ReplayResult:
    checksums: list          # (var, replayed value, recorded value)
    hashes: list             # (stage index, [per-var cell hashes])
    ctx: Context
    mesh: np.ndarray
    numbers: np.ndarray


def replay(lib: Library, records: list[Record], dtype: int | None = None,
           hash_stages: set | None = None, max_blocks: int | None = None):
    """Replays a trace through ``lib``.

    dtype overrides the recorded pool precision.  hash_stages: indices of
    checksum stages (counting groups of check_sum calls that end with the
    last variable) after which the per-variable cell hashes are taken."""
    ctx = None
    mesh = numbers = None
    sums, hashes = [], []
    stage_idx = 0
    cfg = None
    for r in records:
        if r.op == OP_CREATE:
            cfg = Config.from_buffer_copy(bytes(r.args[0]))
            if dtype is not None:
                cfg.dtype = dtype
            if max_blocks is not None:
                cfg.max_blocks = max_blocks
            ctx = lib.context(cfg)
        elif r.op == OP_UPLOAD:
            slots, h = r.args
            n0 = int(slots.max()) + 1
            data = lib.initial_values(cfg, n0)[slots]
            if upload_hash(data) != h:
                raise AssertionError("regenerated initial values differ "
                                     "from the recorded upload")
            ctx.upload(slots, data)
        elif r.op == OP_SET_MESH:
            mesh, numbers = r.args
            ctx.set_mesh(mesh)
        elif r.op == OP_COMM:
            ctx.comm(*r.args)
        elif r.op == OP_STENCIL:
            ctx.stencil_driver(*r.args)
        elif r.op == OP_CHECK_SUM:
            var, rec = r.args
            sums.append((var, ctx.check_sum(var), rec))
            if var == cfg.num_vars - 1:
                if hash_stages is not None and stage_idx in hash_stages:
                    cells = ctx.download(mesh["slot"])
                    hashes.append((stage_idx, cell_hashes(cells, numbers)))
                stage_idx += 1
        elif r.op == OP_SPLIT:
            ctx.split(r.args[0])
        elif r.op == OP_CONSOLIDATE:
            ctx.consolidate(r.args[0])
        elif r.op == OP_WORK_PARAMS:
            ctx.set_work_params(*r.args)
    return ReplayResult(sums, hashes, ctx, mesh, numbers)


def replay_batched(lib: Library, records: list[Record], flags: int,
                   dtype: int | None = None, num_vars: int | None = None):
    """Replays a trace with every run of consecutive stages between mesh
    changes executed as one mamr_run_timesteps call (flags: RUN_BATCHED,
    RUN_GRAPH ...), one timestep of one stage per recorded stage.  Returns
    (checksums [(var, replayed, recorded)], ReplayResult-like context),
    plus per-call timings [(stages, seconds, active blocks)] for throughput
    figures.

    Checksum cadence must be uniform inside a run: stages are grouped by
    whether they computed checksums.  num_vars overrides the recorded
    variable count (the mesh sequence does not depend on it; the initial
    values are then regenerated for the new count without the upload hash
    check, and recorded checksums are not comparable)."""
    import time
    ctx = None
    cfg = None
    sums = []
    timings = []
    pending = []          # [(stage, with_checksums, recorded sums)]

    def flush():
        i = 0
        while i < len(pending):
            j = i
            while (j + 1 < len(pending) and pending[j + 1][1] == pending[i][1]
                   and pending[j + 1][0] == pending[j][0] + 1):
                j += 1
            n = j - i + 1
            cs = pending[i][1]
            # the refinement before this run (split, consolidate, mesh
            # upload) is asynchronous: finish it outside the run's time
            ctx.sync()
            t0 = time.perf_counter()
            got = ctx.run_timesteps(n, 1, 1 if cs else 0, pending[i][0],
                                    flags=flags)
            timings.append((n, time.perf_counter() - t0, n_active))
            if cs:
                for q in range(n):
                    for var, rec in pending[i + q][2]:
                        if var < cfg.num_vars:
                            sums.append((var, float(got[q][var]), rec))
            i = j + 1
        pending.clear()

    stage = None
    n_active = 0
    for r in records:
        if r.op == OP_CREATE:
            cfg = Config.from_buffer_copy(bytes(r.args[0]))
            if dtype is not None:
                cfg.dtype = dtype
            rec_vars = cfg.num_vars
            if num_vars is not None:
                cfg.num_vars = num_vars
            ctx = lib.context(cfg)
        elif r.op == OP_UPLOAD:
            slots, h = r.args
            data = lib.initial_values(cfg, int(slots.max()) + 1)[slots]
            if cfg.num_vars == rec_vars and upload_hash(data) != h:
                raise AssertionError("regenerated initial values differ")
            ctx.upload(slots, data)
        elif r.op in (OP_SET_MESH, OP_SPLIT, OP_CONSOLIDATE):
            flush()
            if r.op == OP_SET_MESH:
                ctx.set_mesh(r.args[0])
                n_active = len(r.args[0])
            elif r.op == OP_SPLIT:
                ctx.split(r.args[0])
            else:
                ctx.consolidate(r.args[0])
        elif r.op == OP_WORK_PARAMS:
            ctx.set_work_params(*r.args)
        elif r.op == OP_COMM:
            if r.args[0] != 0 or r.args[1] != rec_vars:
                raise ValueError("batched replay needs comm over all vars")
            stage = [r.args[2], False, []]
            pending.append(stage)
        elif r.op == OP_CHECK_SUM:
            if stage is None:
                # init()'s checksums, before any stage
                if r.args[0] < cfg.num_vars:
                    sums.append((r.args[0], ctx.check_sum(r.args[0]),
                                 r.args[1]))
            else:
                stage[1] = True
                stage[2].append(r.args)
    flush()
    return sums, ctx, timings


@dataclass
class MarkStep:
    """One refinement step's marking as the reference computed it: the
    inputs of mamr_mark_refine and the reference's flags (oracle/ref_hooks.c
    writes them at each split_blocks() call)."""
    call: int
    block_size: tuple
    params: object
    objects: np.ndarray
    blocks: np.ndarray
    parents: np.ndarray
    block_refine: np.ndarray
    parent_refine: np.ndarray


def read_marks(path: str) -> list[MarkStep]:
    """Parses a marking dump (format in oracle/ref_hooks.c)."""
    from .abi import (MARK_BLOCK_DTYPE, MARK_PARENT_DTYPE, OBJECT_DTYPE,
                      MarkParams)
    lines = _open(path).decode().splitlines()
    steps, i = [], 0
    while i < len(lines):
        h = lines[i].split()
        if h[0] != "step":
            raise ValueError(f"{path}: line {i + 1}: expected a step")
        call, nb, npar, nref, ghost, uni, m0, m1, m2, bx, by, bz, nobj = \
            map(int, h[1:])
        i += 1
        objs = np.zeros(nobj, dtype=OBJECT_DTYPE)
        for o in range(nobj):
            f = lines[i + o].split()
            objs[o]["type"] = int(f[1])
            v = np.array([int(x, 16) for x in f[2:8]], dtype=np.uint64)
            d = v.view(np.float64)
            objs[o]["cen"] = d[:3]
            objs[o]["size"] = d[3:]
        i += nobj
        b = np.array([list(map(int, lines[i + k].split()[1:]))
                      for k in range(nb)], dtype=np.int32).reshape(nb, 19)
        i += nb
        p = np.array([list(map(int, lines[i + k].split()[1:]))
                      for k in range(npar)], dtype=np.int32).reshape(npar, 11)
        i += npar
        blocks = np.zeros(nb, dtype=MARK_BLOCK_DTYPE)
        blocks["slot"], blocks["level"], blocks["parent"] = b[:, 0], b[:, 1], \
            b[:, 2]
        blocks["cen"], blocks["nei_level"], blocks["nei"] = b[:, 3:6], \
            b[:, 6:12], b[:, 12:18]
        parents = np.zeros(npar, dtype=MARK_PARENT_DTYPE)
        parents["active"], parents["child"] = p[:, 1], p[:, 2:10]
        steps.append(MarkStep(
            call, (bx, by, bz),
            MarkParams.make(nref, (m0, m1, m2), ghost, uni), objs, blocks,
            parents, b[:, 18].copy(), p[:, 10].copy()))
    return steps
