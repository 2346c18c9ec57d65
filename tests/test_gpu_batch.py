"""Batched extraction (config-C4 style) against one-at-a-time extraction.

Every instance's mesh in the batched output must be bit for bit the mesh
gcm_mesh_lattice makes for that instance alone; graph replay and autotuned
launch shapes must not change a bit either."""
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


def _plain(ctx, lat, shape):
    cnt = ctx.mesh_lattice(lat, shape, 0.0)  # count through the public call (no outputs)
    pos = torch.empty((max(cnt.total_verts, 1), 4), device="cuda")
    norm = torch.empty((max(cnt.total_verts, 1), 4), device="cuda")
    c2 = ctx.mesh_lattice(lat, shape, 0.0, pos=pos, norm=norm)
    assert c2.total_verts == cnt.total_verts
    return pos[: c2.total_verts], norm[: c2.total_verts], c2


@pytest.fixture(scope="module")
def batch(ctx):
    from gpucadforam_gb300.mesher import Batch, random_batch_lattices

    lats, shapes = random_batch_lattices(14, seed=0xD4A + 4, dims=(17, 72), blend_every=5)
    b = Batch(ctx, lats, shapes)
    yield b, lats, shapes
    b.close()


def test_batch_equals_one_at_a_time(ctx, batch):
    b, lats, shapes = batch
    verts, active, tot = b.count()
    pos, norm, offsets, counts = b.buffers(tot.total_verts)
    b.mesh_async(pos, norm, offsets, counts)
    torch.cuda.synchronize()
    off = offsets.cpu().numpy().view(np.uint64)
    c = counts.cpu().numpy().view(np.uint64)
    assert int(c[1]) == tot.total_verts and int(c[2]) & 0xFFFFFFFF == 0
    assert int(off[-1]) == tot.total_verts
    for i, (lat, shape) in enumerate(zip(lats, shapes)):
        ppos, pnorm, pc = _plain(ctx, lat, shape)
        a, e = int(off[i]), int(off[i + 1])
        assert e - a == pc.total_verts == verts[i], i
        assert active[i] == pc.active_voxels, i
        assert pos[a:e].cpu().numpy().tobytes() == ppos.cpu().numpy().tobytes(), f"instance {i} positions"
        assert norm[a:e].cpu().numpy().tobytes() == pnorm.cpu().numpy().tobytes(), f"instance {i} normals"


def test_graph_replay_is_identical(ctx, batch):
    b, _, _ = batch
    _, _, tot = b.count()
    pos, norm, offsets, counts = b.buffers(tot.total_verts)
    b.mesh_async(pos, norm, offsets, counts)
    torch.cuda.synchronize()
    ref = pos.clone(), norm.clone(), offsets.clone()
    for _ in range(3):
        pos.fill_(0)
        offsets.fill_(0)
        b.mesh_async(pos, norm, offsets, counts, graph=True)
        torch.cuda.synchronize()
        assert torch.equal(pos, ref[0]) and torch.equal(norm, ref[1]) and torch.equal(offsets, ref[2])


def test_tuner_keeps_results_and_reuses_its_cache(ctx, batch, tmp_path):
    b, _, _ = batch
    _, _, tot = b.count()
    pos, norm, offsets, counts = b.buffers(tot.total_verts)
    b.mesh_async(pos, norm, offsets, counts)
    torch.cuda.synchronize()
    ref = pos.clone()
    cache = str(tmp_path / "tune.txt")
    t, v = b.tune(pos, norm, cache)
    assert t in (128, 256) and v in (1024, 2048, 4096, 8192)
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and lines[0].startswith("gcm-tune-v1 ")
    assert b.tune(pos, norm, cache) == (t, v)
    assert len(open(cache).read().splitlines()) == 1  # second call read the cache
    b.mesh_async(pos, norm, offsets, counts)
    torch.cuda.synchronize()
    assert torch.equal(pos, ref)


@pytest.mark.parametrize("shape_", [(128, 1024), (256, 4096), (128, 8192), (256, 64)])
def test_single_grid_launch_shapes_are_identical(shape_):
    import oracle as O
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    f = torch.from_numpy(O.lattice_field((90, 70, 50), 0, (1, 1, 1), np.array([14.0], np.float32),
                                         types=np.array([1], np.uint8))).cuda()
    ref_pos, ref_norm, _ = c.mesh_field(f, 0.2)
    c.set_launch_shape(*shape_)
    pos, norm, _ = c.mesh_field(f, 0.2)
    assert torch.equal(pos, ref_pos) and torch.equal(norm, ref_norm)
    c.close()


def test_batch_with_wide_control_grid(ctx):
    """An instance whose control grid has more columns than a warp stages
    (40 > 32) goes through the second, unstaged batched field form; every
    instance still equals its one-at-a-time mesh."""
    from gpucadforam_gb300.mesher import Batch, Lattice, random_batch_lattices

    lats, shapes = random_batch_lattices(3, seed=0xD4A + 9, dims=(24, 64))
    rng = np.random.default_rng(5)
    cw = (40, 6, 5)
    nc = int(np.prod(cw))
    shape = (48, 40, 90)
    lats.insert(1, Lattice.from_numpy(0, cw, rng.uniform(12, 40, nc).astype(np.float32),
                                      rng.uniform(-np.pi / 4, np.pi / 4, 3 * nc).astype(np.float32),
                                      rng.uniform(-0.6, 0.6, nc).astype(np.float32),
                                      rng.choice(np.array([0, 1, 5], np.uint8), nc),
                                      origin=((shape[2] - 1) / 2, (shape[1] - 1) / 2, (shape[0] - 1) / 2)))
    shapes.insert(1, shape)
    b = Batch(ctx, lats, shapes)
    try:
        verts, active, tot = b.count()
        pos, norm, offsets, counts = b.buffers(tot.total_verts)
        b.mesh_async(pos, norm, offsets, counts)
        torch.cuda.synchronize()
        off = offsets.cpu().numpy().view(np.uint64)
        for i, (lat, shp) in enumerate(zip(lats, shapes)):
            ppos, pnorm, pc = _plain(ctx, lat, shp)
            a, e = int(off[i]), int(off[i + 1])
            assert e - a == pc.total_verts, i
            assert pos[a:e].cpu().numpy().tobytes() == ppos.cpu().numpy().tobytes(), i
            assert norm[a:e].cpu().numpy().tobytes() == pnorm.cpu().numpy().tobytes(), i
    finally:
        b.close()


@pytest.mark.parametrize("shape", [(36, 30, 75), (37, 29, 5), (13, 11, 33)])
@pytest.mark.parametrize("cw", [(1, 1, 1), (2, 2, 2), (3, 4, 2), (5, 2, 3), (7, 3, 2), (32, 3, 2), (31, 1, 4)])
def test_batch_staged_control_grid_edges(ctx, cw, shape):
    """The staged batched field form takes groups of 32 / cx sample rows (at
    most 8) per warp, one control column per lane, each cell's second column
    from the next lane, and runs a group's samples as one sequence.  A single
    column (its own), groups that leave lanes without a column (3, 5 and 7
    columns), 31 or 32 columns (a row per group), row counts that leave a
    partial last group, and rows shorter than a warp (5 and 33 samples, so one
    lane's samples span several rows) must give each instance its
    one-at-a-time mesh bit for bit."""
    from gpucadforam_gb300.mesher import Batch, Lattice, random_batch_lattices

    lats, shapes = random_batch_lattices(2, seed=0xD4A + 11, dims=(24, 56))
    rng = np.random.default_rng(sum(cw) + shape[2])
    nc = int(np.prod(cw))
    lats.insert(1, Lattice.from_numpy(0, cw, rng.uniform(12, 40, nc).astype(np.float32),
                                      rng.uniform(-np.pi / 4, np.pi / 4, 3 * nc).astype(np.float32),
                                      rng.uniform(-0.6, 0.6, nc).astype(np.float32),
                                      rng.choice(np.array([0, 1, 2, 3, 5], np.uint8), nc),
                                      origin=((shape[2] - 1) / 2, (shape[1] - 1) / 2, (shape[0] - 1) / 2)))
    shapes.insert(1, shape)
    b = Batch(ctx, lats, shapes)
    try:
        verts, active, tot = b.count()
        pos, norm, offsets, counts = b.buffers(tot.total_verts)
        b.mesh_async(pos, norm, offsets, counts)
        torch.cuda.synchronize()
        off = offsets.cpu().numpy().view(np.uint64)
        for i, (lat, shp) in enumerate(zip(lats, shapes)):
            ppos, pnorm, pc = _plain(ctx, lat, shp)
            a, e = int(off[i]), int(off[i + 1])
            assert e - a == pc.total_verts, i
            assert pos[a:e].cpu().numpy().tobytes() == ppos.cpu().numpy().tobytes(), i
            assert norm[a:e].cpu().numpy().tobytes() == pnorm.cpu().numpy().tobytes(), i
    finally:
        b.close()
