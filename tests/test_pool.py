"""The server's device-pool allocator, exercised on the host (no GPU)."""
import ctypes as C

import numpy as np

from gpucadforam_gb300 import _native as N


def run(size, ops):
    lib = N.load()
    op = np.array(ops, np.int64)
    res = np.zeros(len(ops), np.int64)
    ranges = lib.gcm_test_pool_script(size, op.ctypes.data, res.ctypes.data, len(ops))
    return res, ranges


def test_first_fit_alignment_and_exhaustion():
    res, ranges = run(4096, [100, 300, 256, 4096])
    assert list(res[:3]) == [0, 256, 768]  # 256-byte granules
    assert res[3] == -1  # does not fit any more
    assert ranges == 1


def test_release_coalesces_neighbours():
    # a, b, c; free b then a then c: one range again; then the whole pool fits
    res, ranges = run(1024, [256, 256, 256, -2, -1, -3, 1024])
    assert res[6] == 0
    assert ranges == 0


def test_fragmentation_and_reuse():
    res, ranges = run(1024, [256, 256, 256, 256, -2, -4, 512, 256])
    assert res[6] == -1  # two separate 256-byte holes cannot hold 512
    assert res[7] == 256  # first fit reuses the lower hole
    assert ranges == 1
