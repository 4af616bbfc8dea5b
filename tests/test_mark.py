"""Refinement marking (mamr_mark_refine: reset_all, check_objects /
uniform assignment and refine_level of one rank) against the reference's
own flags, recorded at every split_blocks() of its golden runs
(tests/golden/*.mark.xz, oracle/ref_hooks.c): the CPU oracle here, the GPU
library under -m gpu.  The cases cover every object type (boxes,
spheroids and their halves, cylinders along each axis, surface and solid),
--refine_ghost, the uniform assignment, a disabled (negative size) object,
and the reference's multi-object stress mesh."""
import numpy as np
import pytest

from golden_util import mark_cases, mark_path
from miniamr_gb300.abi import (MARK_BLOCK_DTYPE, MARK_PARENT_DTYPE,
                               OBJECT_DTYPE, Config, MamrError, MarkParams)
from miniamr_gb300.trace import read_marks


def check_case(lib, name):
    steps = read_marks(mark_path(name))
    assert steps
    cap = max(int(st.blocks["slot"].max()) for st in steps) + 1
    for st in steps:
        cfg = Config.make(*st.block_size, 1, cap)
        with lib.context(cfg) as ctx:
            br, pr = ctx.mark_refine(st.params, st.objects, st.blocks,
                                     st.parents)
        act = st.parents["active"] == 1
        assert np.array_equal(br, st.block_refine), (name, st.call)
        assert np.array_equal(pr[act], st.parent_refine[act]), (name, st.call)
    return len(steps)


@pytest.mark.parametrize("name", mark_cases())
def test_oracle_marking_equals_reference(oracle_lib, name):
    assert check_case(oracle_lib, name) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", mark_cases())
def test_gpu_marking_equals_reference(gpu_lib, name):
    assert check_case(gpu_lib, name) > 0


def bad_inputs():
    """(what, params, objects, blocks, parents) each of which the library
    must refuse with MAMR_EINVAL."""
    prm = MarkParams.make(2, (16, 16, 16))
    obj = np.zeros(1, dtype=OBJECT_DTYPE)
    obj["type"], obj["size"] = 2, 0.1
    blk = np.zeros(2, dtype=MARK_BLOCK_DTYPE)
    blk["slot"], blk["parent"], blk["nei_level"] = [0, 1], -1, -2
    blk["cen"] = [[4, 4, 4], [12, 4, 4]]
    par = np.zeros(1, dtype=MARK_PARENT_DTYPE)
    out = []
    b = blk.copy(); b["slot"] = [0, 0]
    out.append(("slot listed twice", prm, obj, b, par))
    b = blk.copy(); b["slot"][1] = 99
    out.append(("slot out of range", prm, obj, b, par))
    b = blk.copy(); b["parent"][0] = 5
    out.append(("parent out of range", prm, obj, b, par))
    b = blk.copy(); b["level"][0] = 3
    out.append(("level above num_refine", prm, obj, b, par))
    b = blk.copy(); b["nei_level"][0, 1] = 0; b["nei"][0, 1] = 7
    out.append(("neighbour not listed", prm, obj, b, par))
    p = par.copy(); p["active"] = 1; p["child"][0, 0] = -9
    out.append(("child parent out of range", prm, obj, blk, p))
    q = MarkParams.make(2, (16, 0, 16))
    out.append(("mesh size", q, obj, blk, par))
    q = MarkParams.make(2, (16, 16, 16)); q.reserved[3] = 1
    out.append(("reserved parameter", q, obj, blk, par))
    return out


def check_refusals(lib):
    cfg = Config.make(8, 8, 8, 1, 16)
    with lib.context(cfg) as ctx:
        for what, prm, obj, blk, par in bad_inputs():
            with pytest.raises(MamrError) as e:
                ctx.mark_refine(prm, obj, blk, par)
            assert e.value.status == -1, what
        # the context stays usable: two level-0 blocks, the object at the
        # first one's corner region refines it, the other stays
        prm, obj, blk, par = bad_inputs()[0][1:]
        blk = blk.copy(); blk["slot"] = [0, 1]
        obj = obj.copy(); obj["cen"] = [0.25, 0.25, 0.25]
        br, _ = ctx.mark_refine(prm, obj, blk, par)
        assert list(br) == [1, 0]


def test_oracle_refuses_bad_marking_input(oracle_lib):
    check_refusals(oracle_lib)


@pytest.mark.gpu
def test_gpu_refuses_bad_marking_input(gpu_lib):
    check_refusals(gpu_lib)


def check_pass_cap(lib):
    """The rule passes stop at params.max_passes: a cap below what a
    recorded step needs ends the call with MAMR_EDEVICE (the device loop's
    bound, not a hang), and the same context then gives the reference's
    flags without the cap."""
    from miniamr_gb300.abi import MamrError
    steps = read_marks(mark_path("amr7_objects"))
    st = steps[6]
    cfg = Config.make(*st.block_size, 1, int(st.blocks["slot"].max()) + 1)
    with lib.context(cfg) as ctx:
        st.params.max_passes = 1
        with pytest.raises(MamrError) as e:
            ctx.mark_refine(st.params, st.objects, st.blocks, st.parents)
        assert e.value.status == -6 and "settle" in str(e.value)
        st.params.max_passes = 0
        br, pr = ctx.mark_refine(st.params, st.objects, st.blocks,
                                 st.parents)
        act = st.parents["active"] == 1
        assert np.array_equal(br, st.block_refine)
        assert np.array_equal(pr[act], st.parent_refine[act])


def test_oracle_marking_pass_cap(oracle_lib):
    check_pass_cap(oracle_lib)


@pytest.mark.gpu
def test_gpu_marking_pass_cap(gpu_lib):
    check_pass_cap(gpu_lib)


def long_list_refusals(lib):
    """Mistakes planted in the stress mesh's longest block list (about 20k
    blocks, where the library checks the list on several threads): each is
    refused with MAMR_EINVAL and its message; with two mistakes the one the
    serial check meets first is named.  The context then gives the
    reference's flags for the untouched list."""
    steps = read_marks(mark_path("config5"))
    st = max(steps, key=lambda s: len(s.blocks))
    n = len(st.blocks)
    assert n >= 4096
    cap = int(st.blocks["slot"].max()) + 1
    plants = []
    b = st.blocks.copy(); b["slot"][n - 1] = b["slot"][3]
    plants.append(b)
    b = st.blocks.copy(); b["slot"][n // 2] = cap
    plants.append(b)
    b = st.blocks.copy(); b["level"][n - 2] = st.params.num_refine + 1
    b["slot"][n - 1] = b["slot"][0]
    plants.append(b)
    b = st.blocks.copy()
    i = int(np.flatnonzero(b["nei_level"][:, 0] == b["level"])[-1])
    b["nei"][i, 0] = -1
    plants.append(b)
    b = st.blocks.copy(); b["parent"][7] = len(st.parents)
    b["slot"][n - 1] = cap + 5
    plants.append(b)
    msgs = []
    cfg = Config.make(*st.block_size, 1, cap)
    with lib.context(cfg) as ctx:
        for blk in plants:
            with pytest.raises(MamrError) as e:
                ctx.mark_refine(st.params, st.objects, blk, st.parents)
            assert e.value.status == -1
            msgs.append(str(e.value).rsplit(": ", 1)[-1])
        br, pr = ctx.mark_refine(st.params, st.objects, st.blocks,
                                 st.parents)
    act = st.parents["active"] == 1
    assert np.array_equal(br, st.block_refine)
    assert np.array_equal(pr[act], st.parent_refine[act])
    assert "listed twice" in msgs[0] and "out of range" in msgs[1]
    assert "level or parent" in msgs[2] and "neighbour" in msgs[3]
    assert "level or parent" in msgs[4]
    return msgs


def test_oracle_refuses_long_bad_lists(oracle_lib):
    long_list_refusals(oracle_lib)


@pytest.mark.gpu
def test_gpu_refuses_long_bad_lists_like_oracle(gpu_lib, oracle_lib):
    assert long_list_refusals(gpu_lib) == long_list_refusals(oracle_lib)
