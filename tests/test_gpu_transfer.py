"""Block uploads and downloads from pinned host memory, which the device
reads and writes in place (one kernel over the host link), against the
staged path that pageable buffers take: the same pool, bit for bit, for
FP64 and FP32 pools, with ghosts and in scattered slots."""
import numpy as np
import pytest

from miniamr_gb300.abi import FP32, FP64, Config, _ptr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [FP64, FP32])
def test_pinned_transfers_equal_staged(gpu_lib, dtype):
    import torch
    cfg = Config.make(8, 8, 8, 3, 40, stencil=7, dtype=dtype)
    rng = np.random.default_rng(5)
    slots = np.array([7, 0, 31, 12, 5], dtype=np.int32)
    shape = (len(slots), 3, 10, 10, 10)
    vals = rng.uniform(-4, 4, size=shape)
    pinned = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    pin = pinned.numpy()
    pin[...] = vals
    with gpu_lib.context(cfg) as a, gpu_lib.context(cfg) as b:
        a.upload(slots, vals)                  # pageable: staged
        b.upload(slots, pin)                   # pinned: read in place
        got_a, got_b = a.download(slots), b.download(slots)
        assert np.array_equal(got_a.view(np.uint64), got_b.view(np.uint64))
        # the download into pinned memory, written in place
        out = torch.zeros(shape, dtype=torch.float64, pin_memory=True)
        o = out.numpy()
        b._call("mamr_download_blocks", _ptr(slots), len(slots), _ptr(o))
        assert np.array_equal(o.view(np.uint64), got_a.view(np.uint64))
    if dtype == FP64:
        assert np.array_equal(got_a, vals)
    else:
        assert np.array_equal(got_a, vals.astype(np.float32).astype(np.float64))
