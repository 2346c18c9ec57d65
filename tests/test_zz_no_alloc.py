"""The allocation-free entry point gives the same mesh as the context-based one.

gcm_mesh_field_noalloc exists for callers that may not allocate device memory
(applications that own every allocation through their own arena, code running
while a stream is captured into a CUDA graph, loops that cannot take an
allocation's implicit synchronisation).  It keeps its look-back scratch in a
fixed array of the library's device image, so consecutive calls reuse the same
scratch: the test runs it twice in a row and checks both results against
gcm_mesh_field, bit for bit (the tolerance of every marching-cubes test here).

This file is collected last, so a stop at the first failure has run every other
test first; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_context_entry_point_on_two_calls():
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import Context, make_grid

    lib = N.load()
    n = 96
    host_field = O.lattice_field((n, n, n), 0, (1, 1, 1), np.array([24.0], np.float32),
                                 types=np.array([5], np.uint8))
    field = torch.from_numpy(host_field).cuda()
    h = np.float32(1.0 / (n - 1))
    iso = 0.1
    ctx = Context(0)
    ref_pos, ref_norm, ref = ctx.mesh_field(field, iso, (h, h, h), (0, 0, 0))
    cap = ref.total_verts
    assert cap > 0
    grid = make_grid(field.shape, (h, h, h), (0, 0, 0))
    for call in range(2):
        pos = torch.full((cap, 4), float("nan"), device="cuda")
        norm = torch.full((cap, 4), float("nan"), device="cuda")
        counts = torch.full((4,), -1, dtype=torch.int64, device="cuda")
        rc = lib.gcm_mesh_field_noalloc(_ptr(field), C.byref(grid), iso, _ptr(pos), _ptr(norm), cap, _ptr(counts),
                                        _stream())
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        c = counts.cpu().numpy().view(np.uint64)
        assert int(c[0]) == ref.active_voxels and int(c[1]) == ref.total_verts, (call, c)
        assert int(c[2]) & 0xFFFFFFFF == 0, (call, c)
        assert pos.cpu().numpy().tobytes() == ref_pos.cpu().numpy().tobytes(), f"call {call}: positions differ"
        assert norm.cpu().numpy().tobytes() == ref_norm.cpu().numpy().tobytes(), f"call {call}: normals differ"
    ctx.close()


def _tilted_plane(shape):
    """A plane tilted across every voxel plane of the grid: every tile has
    work and the look-back runs across the whole grid, with a mesh of modest
    size (one sheet)."""
    nz, ny, nx = shape
    z = torch.arange(nz, dtype=torch.float32, device="cuda").view(nz, 1, 1)
    y = torch.arange(ny, dtype=torch.float32, device="cuda").view(1, ny, 1)
    x = torch.arange(nx, dtype=torch.float32, device="cuda").view(1, 1, nx)
    return (z - 0.5 * nz - 0.25) + 0.3 * (x - 0.5 * nx) + 0.2 * (y - 0.5 * ny)


@pytest.mark.parametrize("shape", [(907, 907, 907), (16401, 1025, 9)], ids=["cube907", "thin9x1025x16401"])
def test_noalloc_grows_its_tiles_to_fit(shape):
    """Grids whose default tiles need more states than the fixed array holds:
    the entry point takes more voxel rows per tile (907^3, the largest cube
    that fits: 7 rows instead of 1; the thin grid: 147 instead of 128) and
    still gives gcm_mesh_field's mesh bit for bit, on two calls in a row."""
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import Context, make_grid

    lib = N.load()
    field = _tilted_plane(shape)
    ctx = Context(0)
    ref_pos, ref_norm, ref = ctx.mesh_field(field, 0.0)
    cap = ref.total_verts
    assert cap > 0
    grid = make_grid(field.shape)
    for call in range(2):
        pos = torch.full((cap, 4), float("nan"), device="cuda")
        norm = torch.full((cap, 4), float("nan"), device="cuda")
        counts = torch.full((4,), -1, dtype=torch.int64, device="cuda")
        rc = lib.gcm_mesh_field_noalloc(_ptr(field), C.byref(grid), 0.0, _ptr(pos), _ptr(norm), cap, _ptr(counts),
                                        _stream())
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        c = counts.cpu().numpy().view(np.uint64)
        assert int(c[0]) == ref.active_voxels and int(c[1]) == ref.total_verts, (call, c)
        assert int(c[2]) & 0xFFFFFFFF == 0, (call, c)
        assert torch.equal(pos.view(torch.int32), ref_pos.view(torch.int32)), f"call {call}: positions differ"
        assert torch.equal(norm.view(torch.int32), ref_norm.view(torch.int32)), f"call {call}: normals differ"
        del pos, norm
    ctx.close()


def test_noalloc_refuses_the_first_cube_beyond_its_scratch():
    """908^3 needs 137,864 tile states at the largest tiles that fit the
    shared-memory budget, more than the fixed array's 131,056: refused on the
    host, so the dummy pointers below are never launched on or read."""
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import make_grid

    lib = N.load()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    counts = torch.zeros(4, dtype=torch.int64, device="cuda")
    grid = make_grid((908, 908, 908))
    rc = lib.gcm_mesh_field_noalloc(_ptr(dummy), C.byref(grid), 0.0, _ptr(dummy), _ptr(dummy), 0, _ptr(counts),
                                    _stream())
    codes = {name: code for code, name in N.STATUS.items()}
    assert rc == codes["GCM_ERR_NOT_SUPPORTED"]


def test_noalloc_rejects_grids_beyond_its_fixed_scratch():
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import make_grid

    lib = N.load()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    counts = torch.zeros(4, dtype=torch.int64, device="cuda")
    # 16384 x 65536 x 65536 samples would need far more tile states than the
    # fixed array holds: refused on the host, nothing is launched or read.
    grid = make_grid((65536, 65536, 16384))
    rc = lib.gcm_mesh_field_noalloc(_ptr(dummy), C.byref(grid), 0.0, _ptr(dummy), _ptr(dummy), 0, _ptr(counts),
                                    _stream())
    codes = {name: code for code, name in N.STATUS.items()}
    assert rc == codes["GCM_ERR_NOT_SUPPORTED"]
