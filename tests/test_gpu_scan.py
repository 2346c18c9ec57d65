"""GPU: gcm_scan_exclusive_u32, the drop-in for the reference's thrust
exclusive scans of the vertex and occupancy arrays
(src/Isosurface.cu:425-431, thrust::exclusive_scan over uint).

Exclusive prefix sums of 32-bit values wrap modulo 2^32 exactly as a 32-bit
scan's do; the returned total is the full 64-bit sum.  Sizes cover empty,
single, ragged (not a multiple of 4, of a warp's 512-element segment or of the
4096-element tile) and multi-tile arrays; views one element off a 16-byte
boundary take the scalar load form.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    yield c
    c.close()


def _expect(vals):
    c = np.cumsum(vals.astype(np.uint64), dtype=np.uint64)
    excl = np.concatenate([[0], c[:-1]]).astype(np.uint64) if len(vals) else c
    return (excl & np.uint64(0xFFFFFFFF)).astype(np.uint32), int(c[-1]) if len(vals) else 0


@pytest.mark.parametrize("n", [1, 3, 4, 5, 127, 128, 511, 512, 513, 4095, 4096, 4097, 8191, 100_003, 1 << 20,
                               (1 << 22) + 7])
@pytest.mark.parametrize("offset", [0, 1])
def test_scan_matches_numpy(ctx, n, offset):
    rng = np.random.default_rng(n * 2 + offset)
    vals = rng.integers(0, 16, n, dtype=np.uint32)
    buf = torch.zeros(n + 8, dtype=torch.int32, device="cuda")
    buf[offset:offset + n] = torch.from_numpy(vals.view(np.int32)).cuda()
    got, total = ctx.scan(buf[offset:offset + n])
    want, want_total = _expect(vals)
    assert total == want_total
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("n", [4096 * 3 + 17, 1 << 18])
def test_scan_large_values_wrap_and_total(ctx, n):
    """Values near 2^32: outputs wrap modulo 2^32, the total does not."""
    rng = np.random.default_rng(7)
    vals = rng.integers(2**31, 2**32, n, dtype=np.uint64).astype(np.uint32)
    got, total = ctx.scan(torch.from_numpy(vals.view(np.int32)).cuda())
    want, want_total = _expect(vals)
    assert total == want_total and total > 2**40
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want)


def test_scan_full_size_window_counts(ctx):
    """A 50 M-element array (about 12 k tiles), all ones: out[i] = i."""
    n = 50_000_017
    got, total = ctx.scan(torch.ones(n, dtype=torch.int32, device="cuda"))
    assert total == n
    idx = torch.arange(n, dtype=torch.int64, device="cuda").to(torch.int32)
    assert torch.equal(got, idx)


def test_scan_empty(ctx):
    from gpucadforam_gb300 import _native as N

    import ctypes as C

    tot = C.c_uint64(123)
    assert ctx.lib.gcm_scan_exclusive_u32(ctx.h, None, None, 0, C.byref(tot), None) == N.GCM_OK
    assert tot.value == 0
