"""ctypes binding of the mamr_* C ABI declared in include/miniamr_gb300.h.

The same ABI is exported by the GB300 library (the product) and by the CPU
oracle used in tests; :class:`Library` binds either one, given its path.
Array arguments are numpy arrays with the record dtypes below, which match
the C structs field for field (all int32, no padding).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

FP64 = 0
FP32 = 1

RUN_PLAIN = 0
RUN_BATCHED = 1
RUN_GRAPH = 2
RUN_PER_BLOCK = 4
RUN_NO_GHOSTS = 8

STATUS = {
    0: "MAMR_OK",
    -1: "MAMR_EINVAL",
    -2: "MAMR_ENOMEM",
    -3: "MAMR_ECUDA",
    -4: "MAMR_EMESH",
    -5: "MAMR_EUNSUP",
    -6: "MAMR_EDEVICE",
}

# struct mamr_block
BLOCK_DTYPE = np.dtype([
    ("slot", "<i4"),
    ("level", "<i4"),
    ("nei_level", "<i4", (6,)),
    ("nei", "<i4", (6, 2, 2)),
])
# struct mamr_split_job
SPLIT_DTYPE = np.dtype([("parent", "<i4"), ("child", "<i4", (8,))])
# struct mamr_consolidate_job
CONSOLIDATE_DTYPE = np.dtype([("child", "<i4", (8,)), ("target", "<i4")])
# struct mamr_object
OBJECT_DTYPE = np.dtype([("type", "<i4"), ("reserved", "<i4"),
                         ("cen", "<f8", (3,)), ("size", "<f8", (3,))])
# struct mamr_mark_block
MARK_BLOCK_DTYPE = np.dtype([
    ("slot", "<i4"), ("level", "<i4"), ("parent", "<i4"),
    ("cen", "<i4", (3,)), ("nei_level", "<i4", (6,)), ("nei", "<i4", (6,)),
])
# struct mamr_mark_parent
MARK_PARENT_DTYPE = np.dtype([("active", "<i4"), ("child", "<i4", (8,))])


class MarkParams(C.Structure):
    """struct mamr_mark_params."""

    _fields_ = [
        ("num_refine", C.c_int32), ("refine_ghost", C.c_int32),
        ("uniform_refine", C.c_int32), ("mesh_size", C.c_int32 * 3),
        ("max_passes", C.c_int32), ("reserved", C.c_int32 * 9),
    ]

    @classmethod
    def make(cls, num_refine, mesh_size, refine_ghost=0,
             uniform_refine=0) -> "MarkParams":
        return cls(num_refine, refine_ghost, uniform_refine,
                   (C.c_int32 * 3)(*mesh_size))


class AmrParams(C.Structure):
    """struct mamr_amr_params: the command-line parameters of a whole run
    (mamr_amr_run)."""

    _fields_ = [
        ("init_x", C.c_int32), ("init_y", C.c_int32), ("init_z", C.c_int32),
        ("num_refine", C.c_int32), ("block_change", C.c_int32),
        ("refine_freq", C.c_int32), ("uniform_refine", C.c_int32),
        ("refine_ghost", C.c_int32), ("num_tsteps", C.c_int32),
        ("stages_per_ts", C.c_int32), ("checksum_freq", C.c_int32),
        ("run_flags", C.c_int32), ("reserved", C.c_int32 * 8),
    ]

    @classmethod
    def make(cls, init=(1, 1, 1), num_refine=5, block_change=0,
             refine_freq=5, uniform_refine=0, refine_ghost=0, num_tsteps=20,
             stages_per_ts=20, checksum_freq=5, run_flags=0) -> "AmrParams":
        """Defaults are the reference's (ref/param.h)."""
        return cls(init[0], init[1], init[2], num_refine, block_change,
                   refine_freq, uniform_refine, refine_ghost, num_tsteps,
                   stages_per_ts, checksum_freq, run_flags)


# struct mamr_amr_object: one --object (type, bounce, cen, move, size, inc)
AMR_OBJECT_DTYPE = np.dtype([
    ("type", "<i4"), ("bounce", "<i4"), ("cen", "<f8", (3,)),
    ("move", "<f8", (3,)), ("size", "<f8", (3,)), ("inc", "<f8", (3,)),
])


class AmrStats(C.Structure):
    """struct mamr_amr_stats."""

    _fields_ = [
        ("stage_seconds", C.c_double), ("refine_seconds", C.c_double),
        ("total_seconds", C.c_double), ("mark_seconds", C.c_double),
        ("bookkeeping_seconds", C.c_double), ("data_seconds", C.c_double),
        ("mesh_seconds", C.c_double), ("wait_seconds", C.c_double),
        ("updates", C.c_int64),
        ("refinements", C.c_int32), ("marking_steps", C.c_int32),
        ("max_active", C.c_int32), ("final_active", C.c_int32),
        ("stretches", C.c_int32), ("plain_stretches", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


AMR_EVENT = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                        C.c_int32, C.c_void_p, C.c_void_p)
EVENT_SPLIT, EVENT_CONSOLIDATE, EVENT_MESH = 1, 2, 3


class MamrError(RuntimeError):
    """A mamr_* call returned a negative status."""

    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}: {message}")


class Config(C.Structure):
    """struct mamr_config."""

    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("num_vars", C.c_int32), ("max_blocks", C.c_int32),
        ("stencil", C.c_int32), ("code", C.c_int32), ("permute", C.c_int32),
        ("dtype", C.c_int32), ("reserved", C.c_int32 * 7),
    ]

    @classmethod
    def make(cls, nx, ny, nz, num_vars, max_blocks, stencil=7, dtype=FP64,
             permute=0, code=0) -> "Config":
        return cls(nx, ny, nz, num_vars, max_blocks, stencil, code, permute,
                   dtype)


_I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class Library:
    """One loaded implementation of the ABI (GPU library or oracle)."""

    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.path = path
        self.lib = C.CDLL(path)
        L = self.lib
        vp = C.c_void_p
        i32 = C.c_int32
        sig = {
            "mamr_create": [C.POINTER(Config), C.POINTER(vp)],
            "mamr_destroy": [vp],
            "mamr_stream": [vp, C.POINTER(vp)],
            "mamr_sync": [vp],
            "mamr_upload_blocks": [vp, vp, i32, vp],
            "mamr_download_blocks": [vp, vp, i32, vp],
            "mamr_set_mesh": [vp, vp, i32],
            "mamr_comm": [vp, i32, i32, i32],
            "mamr_stencil": [vp, i32, i32],
            "mamr_check_sum": [vp, i32, C.POINTER(C.c_double)],
            "mamr_split": [vp, vp, i32],
            "mamr_consolidate": [vp, vp, i32],
            "mamr_run_timesteps": [vp, i32, i32, i32, i32, i32, vp,
                                   C.POINTER(i32)],
            "mamr_launch_count": [vp, C.POINTER(C.c_int64)],
            "mamr_set_tuning": [vp, C.c_int32],
            "mamr_set_work_params": [vp, C.c_double, vp, C.c_int32],
            "mamr_get_tuning": [vp, C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
            "mamr_mark_refine": [vp, C.POINTER(MarkParams), vp, i32, vp,
                                 i32, vp, i32, vp, vp],
            "mamr_amr_run": [vp, C.POINTER(Config), C.POINTER(AmrParams),
                             vp, i32, vp, C.c_int64, C.POINTER(C.c_int64),
                             AMR_EVENT, vp, C.POINTER(AmrStats)],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.mamr_last_error.argtypes = []
        L.mamr_last_error.restype = C.c_char_p
        L.mamr_initial_values.argtypes = [C.POINTER(Config), i32, vp]
        L.mamr_initial_values.restype = C.c_int
        L.mamr_work_coefficients.argtypes = [i32, C.POINTER(C.c_double), vp]
        L.mamr_work_coefficients.restype = C.c_int

    def check(self, status: int, where: str) -> None:
        if status != 0:
            msg = self.lib.mamr_last_error() or b""
            raise MamrError(status, where, msg.decode(errors="replace"))

    def context(self, cfg: Config) -> "Context":
        return Context(self, cfg)

    def work_coefficients(self, num_vars: int):
        """(a1, a0[num_vars/4]) that init() draws for --stencil 0
        (mamr_work_coefficients)."""
        a1 = C.c_double()
        a0 = np.zeros(max(1, num_vars // 4))
        self.check(self.lib.mamr_work_coefficients(
            int(num_vars), C.byref(a1), _ptr(a0)), "mamr_work_coefficients")
        return a1.value, a0[:num_vars // 4]

    def probe_fp64_rate(self) -> float:
        """FP64 add instructions per second the device sustains
        (mamr_probe_fp64_rate; GPU library only)."""
        add, fma = C.c_double(), C.c_double()
        self.check(self.lib.mamr_probe_fp64_rate(C.byref(add), C.byref(fma)),
                   "mamr_probe_fp64_rate")
        return add.value

    def initial_values(self, cfg: Config, n_blocks: int) -> np.ndarray:
        """The reference's init() values for its first n_blocks blocks,
        [n][num_vars][nx+2][ny+2][nz+2] (mamr_initial_values)."""
        out = np.empty((n_blocks, cfg.num_vars, cfg.nx + 2, cfg.ny + 2,
                        cfg.nz + 2), dtype=np.float64)
        self.check(self.lib.mamr_initial_values(C.byref(cfg), n_blocks,
                                                _ptr(out)),
                   "mamr_initial_values")
        return out


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """A mamr_ctx: one cell pool plus its mesh, driven call by call.

    Method names follow the reference entry points each call replaces
    (comm, stencil_driver, check_sum, split_blocks, consolidate_blocks).
    """

    def __init__(self, lib: Library, cfg: Config):
        self.lib = lib
        self.cfg = cfg
        self.h = C.c_void_p()
        lib.check(lib.lib.mamr_create(C.byref(cfg), C.byref(self.h)),
                  "mamr_create")
        self.shape = (cfg.num_vars, cfg.nx + 2, cfg.ny + 2, cfg.nz + 2)

    def close(self) -> None:
        if self.h:
            self.lib.lib.mamr_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name, *args):
        self.lib.check(getattr(self.lib.lib, name)(self.h, *args), name)

    # ---- data ------------------------------------------------------------
    def upload(self, slots, data: np.ndarray) -> None:
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        data = np.ascontiguousarray(data, dtype=np.float64)
        if data.shape != (len(slots),) + self.shape:
            raise ValueError(f"data shape {data.shape} != "
                             f"{(len(slots),) + self.shape}")
        self._call("mamr_upload_blocks", _ptr(slots), len(slots), _ptr(data))

    def download(self, slots) -> np.ndarray:
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        out = np.empty((len(slots),) + self.shape, dtype=np.float64)
        self._call("mamr_download_blocks", _ptr(slots), len(slots), _ptr(out))
        return out

    def set_mesh(self, blocks: np.ndarray) -> None:
        blocks = np.ascontiguousarray(blocks, dtype=BLOCK_DTYPE)
        self._call("mamr_set_mesh", _ptr(blocks), len(blocks))

    # ---- hot path --------------------------------------------------------
    def comm(self, start: int, num_comm: int, stage: int) -> None:
        self._call("mamr_comm", start, num_comm, stage)

    def stencil_driver(self, var: int, calc_stage: int = 0) -> None:
        self._call("mamr_stencil", var, calc_stage)

    def check_sum(self, var: int) -> float:
        out = C.c_double()
        self._call("mamr_check_sum", var, C.byref(out))
        return out.value

    def split(self, jobs: np.ndarray) -> None:
        jobs = np.ascontiguousarray(jobs, dtype=SPLIT_DTYPE)
        self._call("mamr_split", _ptr(jobs), len(jobs))

    def consolidate(self, jobs: np.ndarray) -> None:
        jobs = np.ascontiguousarray(jobs, dtype=CONSOLIDATE_DTYPE)
        self._call("mamr_consolidate", _ptr(jobs), len(jobs))

    def set_work_params(self, a1: float, a0) -> None:
        """--stencil 0 coefficients a1 and a0[num_vars/4]
        (mamr_set_work_params)."""
        a0 = np.ascontiguousarray(a0, dtype=np.float64)
        self._call("mamr_set_work_params", float(a1), _ptr(a0), len(a0))

    def mark_refine(self, params: "MarkParams", objects, blocks, parents):
        """Refine flags of one refinement step (mamr_mark_refine): returns
        (flags of `blocks` in their order, flags of `parents`, -2 for the
        inactive entries)."""
        objects = np.ascontiguousarray(objects, dtype=OBJECT_DTYPE)
        blocks = np.ascontiguousarray(blocks, dtype=MARK_BLOCK_DTYPE)
        parents = np.ascontiguousarray(parents, dtype=MARK_PARENT_DTYPE)
        bref = np.zeros(max(len(blocks), 1), dtype=np.int32)
        pref = np.full(max(len(parents), 1), -2, dtype=np.int32)
        self._call("mamr_mark_refine", C.byref(params), _ptr(objects),
                   len(objects), _ptr(blocks), len(blocks), _ptr(parents),
                   len(parents), _ptr(bref), _ptr(pref))
        return bref[:len(blocks)], pref[:len(parents)]

    def run_timesteps(self, num_ts: int, stages_per_ts: int,
                      checksum_freq: int, first_stage: int = 0,
                      flags: int = RUN_PLAIN, want_sums: bool = True):
        per_ts = sum(1 for st in range(stages_per_ts)
                     if checksum_freq and st % checksum_freq == 0)
        n = per_ts * num_ts
        sums = np.zeros((max(n, 1), self.cfg.num_vars), dtype=np.float64)
        cnt = C.c_int32()
        self._call("mamr_run_timesteps", num_ts, stages_per_ts,
                   checksum_freq, first_stage, flags,
                   _ptr(sums) if want_sums else None, C.byref(cnt))
        return sums[:cnt.value]

    def amr_run(self, params: "AmrParams", objects=None, max_sums=None,
                events: bool = False):
        """A whole run (mamr_amr_run) on this context: returns (checksums
        [n][num_vars], the initial ones first; stats dict; the event list --
        ("split", ts, jobs), ("consolidate", ts, jobs), ("mesh", ts, blocks,
        numbers, centres) -- when `events`)."""
        if objects is None:
            objects = np.zeros(0, dtype=AMR_OBJECT_DTYPE)
        objects = np.ascontiguousarray(objects, dtype=AMR_OBJECT_DTYPE)
        V = self.cfg.num_vars
        if max_sums is None:
            spt, cf = params.stages_per_ts, params.checksum_freq
            per_ts = sum(1 for st in range(spt) if cf and st % cf == 0)
            max_sums = V * (1 + per_ts * max(1, params.num_tsteps))
        sums = np.zeros(max(max_sums, 1), dtype=np.float64)
        n = C.c_int64()
        stats = AmrStats()
        got = []

        def on_event(user, kind, ts, data, cnt, numbers, cen):
            if kind == EVENT_SPLIT:
                a = np.ctypeslib.as_array(
                    C.cast(data, C.POINTER(C.c_int32)), (cnt * 9,))
                got.append(("split", ts, a.view(SPLIT_DTYPE).copy()))
            elif kind == EVENT_CONSOLIDATE:
                a = np.ctypeslib.as_array(
                    C.cast(data, C.POINTER(C.c_int32)), (cnt * 9,))
                got.append(("consolidate", ts,
                            a.view(CONSOLIDATE_DTYPE).copy()))
            elif kind == EVENT_MESH:
                per = BLOCK_DTYPE.itemsize // 4
                a = np.ctypeslib.as_array(
                    C.cast(data, C.POINTER(C.c_int32)), (cnt * per,))
                num = np.ctypeslib.as_array(
                    C.cast(numbers, C.POINTER(C.c_int64)), (cnt,)).copy()
                c = np.ctypeslib.as_array(
                    C.cast(cen, C.POINTER(C.c_int32)), (cnt * 3,))
                got.append(("mesh", ts, a.view(BLOCK_DTYPE).copy(), num,
                            c.reshape(cnt, 3).copy()))

        cb = AMR_EVENT(on_event) if events else AMR_EVENT()
        self._call("mamr_amr_run", C.byref(self.cfg), C.byref(params),
                   _ptr(objects), len(objects), _ptr(sums), int(max_sums),
                   C.byref(n), cb, None, C.byref(stats))
        st = {f: getattr(stats, f) for f, _ in AmrStats._fields_
              if f != "reserved"}
        return sums[:n.value].reshape(-1, V), st, got

    def sync(self) -> None:
        self._call("mamr_sync")

    def stream(self) -> int:
        s = C.c_void_p()
        self._call("mamr_stream", C.byref(s))
        return s.value or 0

    def launch_count(self) -> int:
        n = C.c_int64()
        self._call("mamr_launch_count", C.byref(n))
        return n.value

    def set_tuning(self, choice: int = -1) -> None:
        """Force launch-shape candidate `choice` of the batched path
        (< 0: automatic)."""
        self._call("mamr_set_tuning", int(choice))

    def tuning(self) -> dict:
        """The last batched run's launch shape: candidate index, number of
        candidates, threads, variables per CTA, rows and planes per thread,
        CTAs."""
        ch, n = C.c_int32(), C.c_int32()
        sh = (C.c_int32 * 5)()
        self._call("mamr_get_tuning", C.byref(ch), C.byref(n), sh)
        return {"choice": ch.value, "candidates": n.value,
                "threads": sh[0], "vars_per_cta": sh[1],
                "rows_per_thread": sh[2], "planes_per_thread": sh[3],
                "ctas": sh[4]}
