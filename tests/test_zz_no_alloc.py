"""The allocation-free FP64 checksum entry point, called through the C ABI.

Some callers cannot allocate device memory (all of it reserved up front by
another allocator, or a path that must not risk an allocation's device-wide
synchronisation); mamr_check_sum_fp64_noalloc serves them with a static
device scratch array.  It must give exactly what mamr_check_sum gives on
the same blocks, call after call, and refuse block counts beyond its
scratch.  This file is collected last so that a failure here comes after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from miniamr_gb300 import mesh as meshmod
from miniamr_gb300.abi import FP64, Config

pytestmark = pytest.mark.gpu

MAX_BLOCKS = 65536   # MAMR_STATIC_MAX_BLOCKS


def _bind(lib):
    f = lib.lib.mamr_check_sum_fp64_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(Config), C.c_void_p, C.c_int32,
                  C.c_int32, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_checksum_equals_check_sum(gpu_lib):
    import torch
    cap = 80
    cfg = Config.make(8, 8, 8, 3, cap, stencil=27, dtype=FP64)
    m = meshmod.initial_mesh(2, 2, 2, 1, cap)
    with gpu_lib.context(cfg) as ctx:
        ctx.upload(np.arange(8), gpu_lib.initial_values(cfg, 8))
        ctx.split(m.split_all())
        ctx.set_mesh(m.blocks())
        ctx.run_timesteps(1, 2, 1)
        slots = m.sorted_slots().astype(np.int32)
        # the caller's own device copy of the blocks, dense layout
        dev_blocks = torch.from_numpy(ctx.download(np.arange(cap))).cuda()
        dev_slots = torch.from_numpy(slots).cuda()
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        f = _bind(gpu_lib)
        stream = torch.cuda.current_stream().cuda_stream
        want = {var: ctx.check_sum(var) for var in (0, 2)}

        def call(var):
            rc = f(dev_blocks.data_ptr(), C.byref(cfg), dev_slots.data_ptr(),
                   len(slots), var, out.data_ptr(), stream)
            assert rc == 0, gpu_lib.lib.mamr_last_error()
            torch.cuda.synchronize()
            return out.item()
        # the first call on the device looks up the scratch's address
        call(0)
        free_before = torch.cuda.mem_get_info()[0]
        got = {var: call(var) for var in (0, 2)}   # two calls in a row
        assert torch.cuda.mem_get_info()[0] == free_before, \
            "the allocation-free checksum changed the free device memory"
        assert got == want                          # bit-exact
        rc = f(dev_blocks.data_ptr(), C.byref(cfg), dev_slots.data_ptr(),
               MAX_BLOCKS + 1, 0, out.data_ptr(), stream)
        assert rc == -1
        assert b"exceed" in gpu_lib.lib.mamr_last_error()
