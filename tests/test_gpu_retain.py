"""GPU retained primitive editing (gcm_csg_retain, gcm_mesh_retained) against
the reference's own kernels (tests/golden/golden_retain.npz) and, on larger
and ragged grids, against the oracle; bit for bit."""
import numpy as np
import pytest
import torch

import oracle as O
from tests.helpers import golden
from tests.test_oracle_retain import OPS, case, n_cases, preview

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[(128, 1024), (256, 2048)], ids=["128x1024", "256x2048"])
def ctx(request):
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    c.set_launch_shape(*request.param)
    yield c
    c.close()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("i", range(n_cases()))
def test_retained_matches_reference(ctx, i):
    R = golden("golden_retain.npz")
    pre, n, iso, vs, gc, folds, pf, pop = case(i)
    acc = ctx.csg_accumulator(n[::-1])
    for op, f, band in folds:
        ctx.csg_retain(acc, dev(f), OPS[int(op)], iso, band=band)
    assert acc.cpu().numpy().tobytes() == R[pre + "acc"].tobytes()
    mode, lat, band = preview(i)
    if mode >= 2:
        pos, norm, cnt = ctx.mesh_lattice_preview(dev(lat), band, acc=acc if mode == 3 else None,
                                                  field=dev(pf) if mode == 2 else None, op=pop, iso=iso,
                                                  voxel_size=vs, grid_center=gc)
    else:
        pos, norm, cnt = ctx.mesh_retained(acc, None if pf is None else dev(pf), pop, iso, vs, gc)
    assert cnt.active_voxels == len(R[pre + "compacted"])
    assert pos.cpu().numpy().tobytes() == R[pre + "pos"].tobytes()
    assert norm.cpu().numpy().tobytes() == R[pre + "norm"].tobytes()


@pytest.mark.parametrize("shape", [(33, 29, 41), (7, 64, 5), (2, 3, 70), (96, 80, 72)])
@pytest.mark.parametrize("mode", ["region", "union", "subtract", "intersect"])
def test_retained_vs_oracle(ctx, shape, mode):
    rng = np.random.default_rng(sum(shape) + len(mode))
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float32), np.arange(ny, dtype=np.float32),
                          np.arange(nx, dtype=np.float32), indexing="ij")

    def sphere():
        c = rng.uniform(0, 1, 3) * np.array([nx, ny, nz])
        r = rng.uniform(0.2, 0.5) * min(nx, ny, nz) + 1.0
        return ((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 - np.float32(r * r)).astype(np.float32)

    folds = [("union", sphere()), ("union", sphere()), ("subtract", sphere()), ("intersect", sphere() - 400.0)]
    acc_o = O.csg_accumulator(shape)
    acc_g = ctx.csg_accumulator(shape)
    for op, f in folds:
        O.csg_retain(acc_o, f, op, 0.0)
        ctx.csg_retain(acc_g, dev(f), op, 0.0)
    assert acc_g.cpu().numpy().tobytes() == acc_o.tobytes()
    pf = None if mode == "region" else sphere()
    op = "union" if mode == "region" else mode
    vs, gc = (0.5, 0.25, 2.0), (1.0, 0.0, -3.0)
    opos, onorm, oact = O.mesh_retained(acc_o, pf, op, vs, gc, 0.0)
    cnt = ctx.count_retained(acc_g, None if pf is None else dev(pf), op, 0.0)
    pos, norm, c2 = ctx.mesh_retained(acc_g, None if pf is None else dev(pf), op, 0.0, vs, gc)
    assert cnt.total_verts == c2.total_verts == len(opos) and c2.active_voxels == oact
    assert pos.cpu().numpy().tobytes() == opos.tobytes()
    assert norm.cpu().numpy().tobytes() == onorm.tobytes()


def test_retained_rejects_misaligned_accumulator(ctx):
    from gpucadforam_gb300 import _native as N

    acc = ctx.csg_accumulator((8, 8, 8))
    flat = acc.view(-1)
    bad = flat[1:].view(torch.int32)
    import ctypes as C

    from gpucadforam_gb300.mesher import make_grid

    g = make_grid((8, 8, 8))
    c = N.GcmCounts()
    rc = ctx.lib.gcm_count_retained(ctx.h, C.c_void_p(bad.data_ptr()), None, 0, C.byref(g), 0.0, C.byref(c),
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.GCM_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("shape", [(33, 29, 41), (2, 3, 70), (96, 80, 72)])
@pytest.mark.parametrize("op", ["union", "subtract", "intersect"])
def test_band_folds_vs_oracle(ctx, shape, op):
    """Lattice-band folds (the reference's dynamic mode) on ragged grids: the
    accumulator and the region mesh equal the oracle's bit for bit."""
    rng = np.random.default_rng(sum(shape) + len(op) + 7)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    k = 2 * np.pi / rng.uniform(6, 14)
    gyr = (np.sin(k * x) * np.cos(k * y) + np.sin(k * y) * np.cos(k * z) + np.sin(k * z) * np.cos(k * x)).astype(np.float32)
    c = rng.uniform(0, 1, 3) * np.array([nx, ny, nz])
    r = 0.4 * min(nx, ny, nz) + 1.0
    sph = ((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 - r * r).astype(np.float32)
    folds = [("union", sph, None), (op, gyr, (-0.3, 0.35)), ("union", gyr + 0.5, (0.0, 0.4))]
    acc_o = O.csg_accumulator(shape)
    acc_g = ctx.csg_accumulator(shape)
    for fop, f, band in folds:
        O.csg_retain(acc_o, f, fop, 0.0, band=band)
        ctx.csg_retain(acc_g, dev(f), fop, 0.0, band=band)
    assert acc_g.cpu().numpy().tobytes() == acc_o.tobytes()
    opos, onorm, oact = O.mesh_retained(acc_o, None, "union", (1, 1, 1), (0, 0, 0))
    pos, norm, cnt = ctx.mesh_retained(acc_g, None, "union", 0.0)
    assert cnt.active_voxels == oact and cnt.total_verts == len(opos)
    assert pos.cpu().numpy().tobytes() == opos.tobytes() and norm.cpu().numpy().tobytes() == onorm.tobytes()


@pytest.mark.parametrize("shape", [(33, 29, 41), (2, 3, 70), (64, 48, 40)])
@pytest.mark.parametrize("op", ["union", "subtract", "intersect"])
@pytest.mark.parametrize("form", ["fixed", "dynamic"])
def test_lattice_preview_vs_oracle(ctx, shape, op, form):
    """The editor's lattice previews on ragged grids: counts, positions and
    normals equal the oracle's bit for bit."""
    rng = np.random.default_rng(sum(shape) + len(op) + len(form))
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    k = 2 * np.pi / rng.uniform(6, 14)
    lat = (np.sin(k * x) * np.cos(k * y) + np.sin(k * y) * np.cos(k * z) + np.sin(k * z) * np.cos(k * x)).astype(np.float32)
    c = rng.uniform(0, 1, 3) * np.array([nx, ny, nz])
    r = 0.4 * min(nx, ny, nz) + 1.0
    sph = ((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 - r * r).astype(np.float32)
    band = (-0.3, 0.35)
    vs, gc = (0.5, 1.0, 0.25), (1.0, 0.0, -2.0)
    if form == "fixed":
        opos, onorm, oact = O.mesh_lattice_preview(None, sph, lat, band, op, vs, gc)
        pos, norm, cnt = ctx.mesh_lattice_preview(dev(lat), band, field=dev(sph), op=op, voxel_size=vs,
                                                  grid_center=gc)
    else:
        acc_o = O.csg_accumulator(shape)
        acc_g = ctx.csg_accumulator(shape)
        for f, b in ((sph, None), (lat + 0.5, (0.0, 0.4))):
            O.csg_retain(acc_o, f, "union", 0.0, band=b)
            ctx.csg_retain(acc_g, dev(f), "union", 0.0, band=b)
        opos, onorm, oact = O.mesh_lattice_preview(acc_o, None, lat, band, op, vs, gc)
        pos, norm, cnt = ctx.mesh_lattice_preview(dev(lat), band, acc=acc_g, op=op, voxel_size=vs, grid_center=gc)
    assert cnt.active_voxels == oact and cnt.total_verts == len(opos)
    assert pos.cpu().numpy().tobytes() == opos.tobytes() and norm.cpu().numpy().tobytes() == onorm.tobytes()
