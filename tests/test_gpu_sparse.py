"""GPU: the sparse extraction path (window counts, scan, emission of the
windows that hold triangles) writes exactly the fused path's vertices, counts
and overflow behaviour, on sparse, dense and ragged fields, through
gcm_mesh_field, gcm_mesh_field_async and gcm_mesh_csg (which takes the sparse
path by default).  gcm_count_field (the window count kernel) agrees with both."""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctxs():
    from gpucadforam_gb300.mesher import Context

    fused, sparse = Context(0), Context(0)
    fused.set_mesh_path("fused")
    sparse.set_mesh_path("sparse")
    yield fused, sparse
    fused.close()
    sparse.close()


def _fields():
    rng = np.random.default_rng(0x5A)
    out = {"noise_33x17x9": rng.uniform(-1, 1, (9, 17, 33)).astype(np.float32),
           "noise_2x5x7": rng.uniform(-1, 1, (7, 5, 2)).astype(np.float32),
           "gyroid_65x64x63": O.lattice_field((65, 64, 63), 0, (1, 1, 1), np.array([14.0], np.float32)),
           "exact_iso_40": rng.choice(np.array([-1.0, 0.0, 1.0], np.float32), (40, 40, 40))}
    return out


@pytest.mark.parametrize("name", list(_fields()))
def test_sparse_equals_fused(ctxs, name):
    fused, sparse = ctxs
    f = torch.from_numpy(_fields()[name]).cuda()
    vs = (0.37, 1.3, 0.011)
    gc = (0.5, -2.25, 7.0)
    a = fused.mesh_field(f, 0.0, vs, gc)
    b = sparse.mesh_field(f, 0.0, vs, gc)
    assert a[2].total_verts == b[2].total_verts and a[2].active_voxels == b[2].active_voxels
    assert torch.equal(a[0].view(torch.int32), b[0].view(torch.int32))
    assert torch.equal(a[1].view(torch.int32), b[1].view(torch.int32))
    c = sparse.count_field(f, 0.0)
    assert (c.total_verts, c.active_voxels) == (a[2].total_verts, a[2].active_voxels)


def test_sparse_csg_scene(ctxs):
    """The C3 scene at 256^3 through gcm_mesh_csg: sparse by default, the same
    mesh as the fused path."""
    import bench
    from gpucadforam_gb300.mesher import Context, make_frame, primitives_to_device

    fused, _ = ctxs
    prims = bench.csg_scene(bench.SEED + 1)
    n = 256
    h = np.float32(1.0 / (n - 1))
    d_prims = primitives_to_device(prims)
    frame = make_frame((0, 0, 0), (h, h, h))
    field = fused.csg_field(d_prims, len(prims), frame, (n, n, n))
    ref = fused.mesh_field(field, 0.0, (h, h, h), (0, 0, 0))
    auto = Context(0)
    pos = torch.empty_like(ref[0])
    norm = torch.empty_like(ref[1])
    try:
        cnt = auto.mesh_csg(d_prims, len(prims), frame, (n, n, n), 0.0, (h, h, h), (0, 0, 0), pos=pos, norm=norm)
    finally:
        auto.close()
    assert cnt.total_verts == ref[2].total_verts and cnt.active_voxels == ref[2].active_voxels
    assert torch.equal(pos.view(torch.int32), ref[0].view(torch.int32))
    assert torch.equal(norm.view(torch.int32), ref[1].view(torch.int32))


@pytest.mark.parametrize("short", [1, 2, 3, 1000])
def test_sparse_overflow_like_fused(ctxs, short):
    """Too small an output: the same whole triangles are written, the rest left
    untouched, and the true counts come back with GCM_ERR_OUTPUT_OVERFLOW."""
    fused, sparse = ctxs
    f = torch.from_numpy(_fields()["gyroid_65x64x63"]).cuda()
    total = fused.count_field(f, 0.0).total_verts
    cap = total - short
    outs = []
    for c in (fused, sparse):
        pos = torch.full((cap, 4), -7.0, device="cuda")
        norm = torch.full((cap, 4), -7.0, device="cuda")
        cnt = c.mesh_field(f, 0.0, pos=pos, norm=norm, capacity=cap, allow_overflow=True)[2]
        outs.append((cnt, pos, norm))
    (ca, pa, na), (cb, pb, nb) = outs
    assert ca.total_verts == cb.total_verts == total and ca.status == cb.status != 0
    assert torch.equal(pa.view(torch.int32), pb.view(torch.int32))
    assert torch.equal(na.view(torch.int32), nb.view(torch.int32))


@pytest.mark.parametrize("seed,n_prims,shape,spacing,iso", [
    (31, 40, (70, 45, 97), 1.0 / 64, 0.0),      # ragged: partial tiles on every axis
    (32, 64, (64, 64, 64), -1.0 / 63, 0.0),     # mirrored frame
    (33, 24, (9, 130, 33), 1.0 / 100, 0.02),    # thin grid, an isovalue above 0
    (34, 48, (50, 40, 60), 1.0 / 55, -0.03),    # an isovalue below 0
])
def test_csg_tile_states_change_nothing(ctxs, seed, n_prims, shape, spacing, iso):
    """gcm_mesh_csg records per sample tile whether the folded field's
    enclosure lies wholly below or above iso, and its count pass skips tasks
    whose tiles all agree.  Every primitive kind, subtract and intersect runs,
    mirrored frames and isovalues off zero: the same mesh as the field meshed
    on the fused path, and gcm_mesh_csg_async the same as gcm_mesh_csg."""
    from gpucadforam_gb300.mesher import Context, make_frame, primitives_to_device
    from tests.test_gpu_csg_cull import _scene

    fused, _ = ctxs
    prims = _scene(seed, n_prims)
    for i in range(min(4, n_prims)):
        prims[i]["op"] = 2 if i % 2 else 1  # leading subtract and intersect runs
    nz, ny, nx = shape
    origin = (0.0, 0.0, 0.0) if spacing > 0 else tuple(float(v) for v in (nx, ny, nz))
    frame = make_frame(origin, (spacing,) * 3)
    d_prims = primitives_to_device(prims)
    vs = (abs(spacing),) * 3
    field = fused.csg_field(d_prims, len(prims), frame, shape)
    ref = fused.mesh_field(field, iso, vs, (0, 0, 0))
    auto = Context(0)
    try:
        pos = torch.empty((max(ref[2].total_verts, 1), 4), device="cuda")
        norm = torch.empty_like(pos)
        cnt = auto.mesh_csg(d_prims, len(prims), frame, shape, iso, vs, (0, 0, 0), pos=pos, norm=norm)
        assert cnt.total_verts == ref[2].total_verts and cnt.active_voxels == ref[2].active_voxels
        k = cnt.total_verts
        assert torch.equal(pos[:k].view(torch.int32), ref[0].view(torch.int32))
        assert torch.equal(norm[:k].view(torch.int32), ref[1].view(torch.int32))
        pos2 = torch.full_like(pos, -5.0)
        norm2 = torch.full_like(norm, -5.0)
        d_counts = torch.zeros(4, dtype=torch.int64, device="cuda")
        auto.mesh_csg_async(d_prims, len(prims), frame, shape, iso, pos2, norm2, d_counts, vs, (0, 0, 0))
        torch.cuda.synchronize()
        c = d_counts.cpu().numpy().view(np.uint64)
        assert int(c[1]) == k and int(c[0]) == cnt.active_voxels
        assert torch.equal(pos2[:k], pos[:k]) and torch.equal(norm2[:k], norm[:k])
    finally:
        auto.close()
