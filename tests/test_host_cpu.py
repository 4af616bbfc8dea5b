"""Host-side checks that need no GPU: the GPU library loads and exports the
whole ABI, the replica reduction of the benchmark across ranks, argument
validation in the oracle, and the drop-in against the reference on a case
outside the committed fixtures (where the reference sources exist)."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "miniamr_gb300.h")


def header_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mamr_\w+)\s*\(",
                                 src, re.M)))


def test_gpu_library_exports_every_abi_function():
    from miniamr_gb300 import build
    lib = build.build_library()
    out = subprocess.run(["nm", "-D", "--defined-only", lib],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(mamr_\w+)$", out, re.M))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing
    import ctypes
    ctypes.CDLL(lib)                     # loads without a GPU


def test_oracle_exports_the_hot_path_abi(oracle_lib):
    for f in header_functions():
        if f in ("mamr_check_sum_fp64_noalloc", "mamr_selftest_division",
                 "mamr_probe_fp64_rate"):
            continue                     # device-only entry points
        assert hasattr(oracle_lib.lib, f), f


def test_oracle_rejects_bad_arguments(oracle_lib):
    from miniamr_gb300.abi import Config, MamrError
    with pytest.raises(MamrError) as e:
        oracle_lib.context(Config.make(7, 8, 8, 2, 4))     # odd block size
    assert e.value.status == -1
    with pytest.raises(MamrError) as e:                    # needs 8 vars
        oracle_lib.context(Config.make(8, 8, 8, 2, 4, stencil=0))
    assert e.value.status == -1
    with pytest.raises(MamrError) as e:                    # FP64 only
        oracle_lib.context(Config.make(8, 8, 8, 8, 4, stencil=0, dtype=1))
    assert e.value.status == -5
    with pytest.raises(MamrError) as e:
        oracle_lib.context(Config.make(8, 8, 8, 8, 4, stencil=5))
    assert e.value.status == -5
    with oracle_lib.context(Config.make(8, 8, 8, 2, 4)) as ctx:
        with pytest.raises(MamrError):
            ctx.check_sum(2)
        with pytest.raises(MamrError):
            ctx.upload([4], np.zeros((1, 2, 10, 10, 10)))
        ctx.set_mesh(np.zeros(0, dtype=__import__(
            "miniamr_gb300.abi", fromlist=["BLOCK_DTYPE"]).BLOCK_DTYPE))
        assert ctx.check_sum(0) == 0.0   # empty mesh


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                            rank=rank, world_size=world)
    q.put((rank, bench.max_over_ranks(10.0 + rank, dist)))
    dist.destroy_process_group()


def test_replica_time_is_max_over_ranks_gloo():
    """bench.py under torchrun: each rank times its own replica and the job
    time is the slowest rank's (world size 2, gloo on CPU)."""
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 11.0), (1, 11.0)]


def _reference_sources():
    from miniamr_gb300 import build
    return build.reference_sources()


@pytest.mark.skipif(_reference_sources() is None,
                    reason="reference sources absent")
def test_dropin_matches_reference_on_fresh_case(tmp_path):
    """The reference's driver over the drop-in units and the oracle equals
    the unmodified reference on a case the fixtures do not contain
    (cylinder object, 7-point, block_change 2, checksum every 2nd stage)."""
    from miniamr_gb300 import build
    assert build.build_reference_binaries()
    args = ["--init_x", "1", "--init_y", "2", "--init_z", "2", "--nx", "6",
            "--ny", "4", "--nz", "6", "--num_vars", "2", "--stencil", "7",
            "--num_refine", "3", "--block_change", "2", "--refine_freq", "1",
            "--num_tsteps", "6", "--stages_per_ts", "4", "--checksum_freq",
            "2", "--max_blocks", "6000", "--num_objects", "1", "--object",
            "20", "1", "0.5", "0.4", "0.5", "0.02", "0.03", "0.0", "0.15",
            "0.15", "0.6", "0", "0", "0"]
    logs = []
    for binary in ("miniamr_ref", "miniamr_hybrid_oracle"):
        log = tmp_path / (binary + ".log")
        r = subprocess.run([os.path.join(REPO, "oracle", "_ref", binary)] +
                           args, cwd=tmp_path, capture_output=True, text=True,
                           env=dict(os.environ, MAMR_REF_LOG=str(log)))
        assert r.returncode == 0, r.stdout[-500:]
        logs.append(log.read_text())
    assert len(logs[0]) > 0 and logs[0] == logs[1]
    assert "mesh" in logs[0]


def test_work_coefficients_match_reference_init(oracle_lib):
    """--stencil 0: a1 and a0[] as the reference's init() drew them
    (recorded by the hybrid run that pins the stencil-0 golden case)."""
    from golden_util import trace_path
    from miniamr_gb300.trace import OP_WORK_PARAMS, read_trace
    recs = read_trace(trace_path("stencil0"))
    a1, a0 = next(r.args for r in recs if r.op == OP_WORK_PARAMS)
    got1, got0 = oracle_lib.work_coefficients(8)
    assert got1 == a1 and np.array_equal(got0, a0)


def test_bench_reference_arm_json_line():
    """bench.py --impl reference: the CPU algorithm on the host cores prints
    one JSON line with the benchmark contract's keys, its own cpu_baseline
    and an e2e block without host-device bytes."""
    import json
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"),
                        "--impl", "reference", "--steps", "1", "--warmup",
                        "1"], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup",
                "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
                "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 1
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]


REF_BIN = os.path.join(REPO, "oracle", "_ref", "miniamr_ref")


@pytest.mark.skipif(not os.path.exists(REF_BIN),
                    reason="reference binary not built here")
def test_cpu_port_keeps_up_with_the_reference_binary(tmp_path):
    """The CPU baseline (bench.py's reference arm and cpu_baseline) times the
    oracle, a restatement of the reference's code; it must run at least at
    1/1.25 of the reference binary's own rate on this host, one thread,
    same case: 64 blocks of 16^3 (2x2x2 initial, uniform refine 1), 40
    variables, 27-point, 2 timesteps of 4 stages, checksum every 5th stage.
    Reference rate from its Summary line (calc + comm + red,
    ref/profile.c:1298); best of three runs each."""
    n_upd = 2 * 4 * 64 * 16 ** 3 * 40
    args = ["--init_x", "2", "--init_y", "2", "--init_z", "2", "--nx", "16",
            "--ny", "16", "--nz", "16", "--num_vars", "40", "--stencil", "27",
            "--num_refine", "1", "--uniform_refine", "1", "--num_tsteps", "2",
            "--stages_per_ts", "4", "--checksum_freq", "5", "--max_blocks",
            "100"]
    ref = []
    for _ in range(3):
        r = subprocess.run([REF_BIN] + args, cwd=tmp_path, capture_output=True,
                           text=True, check=True)
        f = [l.split() for l in r.stdout.splitlines()
             if l.startswith("Summary")][-1]
        t = float(f[f.index("calc") + 1]) + float(f[f.index("comm") + 1]) + \
            float(f[f.index("red") + 1])
        ref.append(n_upd / t)
    port = []
    env = dict(os.environ, OMP_NUM_THREADS="1")
    for _ in range(3):
        r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"),
                            "--oracle-rate-steps", "2"], env=env,
                           capture_output=True, text=True, check=True)
        port.append(__import__("json").loads(
            r.stdout.strip().splitlines()[-1])["value"])
    factor = max(ref) / max(port)
    print(f"reference {max(ref):.3e}, port {max(port):.3e} updates/s: the "
          f"port is {factor:.2f}x slower")
    assert factor <= 1.25, (ref, port)


@pytest.mark.skipif(_reference_sources() is None,
                    reason="reference sources absent")
def test_dropin_links_against_the_gpu_library(tmp_path):
    """The binding INTEGRATION.md gives: the reference's host files and the
    drop-in units linked against libminiamr_gb300.so (oracle/Makefile
    target gpu).  It links with every mamr_* symbol resolved from the GPU
    library, and runs the reference's driver up to the first device call:
    without a GPU that call fails and the drop-in stops in the reference's
    error style; with one, the run equals the reference's log."""
    import torch
    from miniamr_gb300 import build
    build.build_library()
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "gpu",
                    "REF=" + _reference_sources()], check=True)
    exe = os.path.join(REPO, "oracle", "_ref", "miniamr_gpu")
    need = subprocess.run(["readelf", "-d", exe], capture_output=True,
                          text=True, check=True).stdout
    assert "libminiamr_gb300.so" in need
    args = ["--init_x", "1", "--init_y", "1", "--init_z", "2", "--nx", "8",
            "--ny", "8", "--nz", "8", "--num_vars", "2", "--stencil", "27",
            "--num_tsteps", "2", "--checksum_freq", "1"]
    log = tmp_path / "gpu.log"
    r = subprocess.run([exe] + args, cwd=tmp_path, capture_output=True,
                       text=True, timeout=300,
                       env=dict(os.environ, MAMR_REF_LOG=str(log)))
    if not torch.cuda.is_available():
        assert "mamr_create" in r.stdout + r.stderr
        return
    assert r.returncode == 0, r.stdout[-1000:]
    ref = tmp_path / "ref.log"
    subprocess.run([os.path.join(REPO, "oracle", "_ref", "miniamr_ref")] +
                   args, cwd=tmp_path, check=True, capture_output=True,
                   env=dict(os.environ, MAMR_REF_LOG=str(ref)))
    assert log.read_text() == ref.read_text()


@pytest.mark.parametrize("init,passes,cap", [
    ((8, 8, 8), 1, 4624), ((2, 2, 2), 2, 600), ((3, 1, 2), 1, 60),
    ((1, 1, 1), 3, 600), ((4, 3, 2), 2, 1800)])
def test_uniform_split_closed_form_equals_the_slot_walk(monkeypatch, init,
                                                       passes, cap):
    """The uniform-mesh helper's closed form for the initial lattice's
    split gives the jobs, numbers, levels and meshes of the reference's
    slot walk (the helper's general path)."""
    from miniamr_gb300 import mesh as meshmod

    def run():
        m = meshmod.initial_mesh(*init, passes, cap)
        out = [m.split_all().tobytes() for _ in range(passes)]
        return out + [m.blocks().tobytes(), m.number.tobytes()]

    fast = run()
    monkeypatch.setattr(meshmod.UniformMesh, "_split_fresh_lattice",
                        lambda self: None)
    assert run() == fast


def test_no_ghosts_flag_is_accepted_by_the_oracle(oracle_lib):
    """MAMR_RUN_NO_GHOSTS is part of the ABI: the oracle (which always
    writes ghost layers back) accepts it and gives the same cells and
    checksums as without it."""
    from miniamr_gb300 import mesh as meshmod
    from miniamr_gb300.abi import RUN_BATCHED, RUN_NO_GHOSTS, Config
    cfg = Config.make(4, 4, 4, 2, 40, stencil=7)
    init = oracle_lib.initial_values(cfg, 4)
    outs = []
    for fl in (RUN_BATCHED, RUN_BATCHED | RUN_NO_GHOSTS):
        m = meshmod.initial_mesh(2, 2, 1, 1, 40)
        with oracle_lib.context(cfg) as ctx:
            ctx.upload(np.arange(4), init)
            ctx.split(m.split_all())
            ctx.set_mesh(m.blocks())
            s = ctx.run_timesteps(2, 2, 1, flags=fl)
            outs.append((s, ctx.download(np.arange(40))))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
