"""GPU: the CSG field kernel skips, per tile of samples, primitives whose value
enclosure shows they cannot change the running min/max.  The result must be
bit-identical to folding every primitive in order, for all primitive kinds,
rotations, operation runs, ragged grids and mirrored frames.

The fold is formed from single-primitive fields (a lone union primitive is
never skipped: its field is g itself) combined on the host with the same
min/max semantics, so the check needs no oracle and covers the rotated kinds
whose trig the oracle does not reproduce bit for bit.
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


def _scene(seed, n, kinds=range(8), size=(0.03, 0.2), ops=(0, 1, 2), run=4):
    rng = np.random.default_rng(seed)
    prims = []
    op = 0
    for i in range(n):
        if i % run == 0 and i:
            op = int(rng.choice(ops))
        kind = int(rng.choice(list(kinds)))
        c = rng.uniform(-0.1, 1.1, 3).astype(np.float32)
        lo, hi = size
        if kind == 0:
            p = [rng.uniform(lo, hi), rng.uniform(0.2, 0.6) * lo]
            v3 = (0.0, 0.0, 0.0)
        elif kind == 1:
            p = [rng.uniform(lo, hi), rng.uniform(0.2, 0.6) * lo, rng.uniform(lo, 2 * hi)]
            v3 = tuple(rng.normal(size=3))
        else:
            v3 = tuple(rng.uniform(-np.pi, np.pi, 3))
            if kind == 2:
                p = list(rng.uniform(lo, 2 * hi, 3))
            elif kind == 3:
                p = list(rng.uniform(2 * lo, 2 * hi, 3)) + [rng.uniform(0.2, 0.5) * lo]
            elif kind == 4:
                p = [rng.uniform(lo, hi), rng.uniform(0.2, 0.5) * lo]
            elif kind == 5:
                p = [rng.uniform(lo, hi), rng.uniform(lo, 2 * hi)]
            elif kind == 6:
                p = [rng.uniform(lo, hi) * 0.5, rng.uniform(lo, hi), rng.uniform(lo, 2 * hi)]
            else:
                p = [rng.uniform(lo, hi), rng.uniform(lo, hi) * 0.5, rng.uniform(lo, 2 * hi), rng.uniform(lo, hi),
                     rng.uniform(lo, hi) * 0.5]
        prims.append(dict(kind=kind, op=op, flag=int(rng.integers(0, 2)) if kind in (0, 1) else 0, center=c,
                          v3=v3, p=[float(x) for x in p]))
    return prims


def _fold(ctx, prims, frame, shape):
    from gpucadforam_gb300.mesher import primitives_to_device

    f = torch.full(shape, float("inf"), device="cuda")
    for q in prims:
        g = ctx.csg_field(primitives_to_device([dict(q, op=0)]), 1, frame, shape)
        if q["op"] == 1:
            f = torch.fmax(f, -g)
        elif q["op"] == 2:
            f = torch.fmax(f, g)
        else:
            f = torch.fmin(f, g)
    return f


def _same(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    assert np.array_equal(a, b, equal_nan=True)
    nz = a != 0
    assert a[nz].tobytes() == b[nz].tobytes()


@pytest.mark.parametrize("seed,n,shape,spacing", [
    (1, 40, (37, 45, 70), 1.0 / 64),
    (2, 64, (64, 64, 64), 1.0 / 63),
    (3, 24, (9, 130, 33), 1.0 / 100),
    (4, 48, (50, 40, 60), -1.0 / 55),  # mirrored frame: positions decrease with the index
])
def test_cull_equals_full_fold_all_kinds(ctx, seed, n, shape, spacing):
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    prims = _scene(seed, n)
    origin = (0.0, 0.0, 0.0) if spacing > 0 else tuple(float(s) for s in shape[::-1])
    frame = make_frame(origin, (spacing,) * 3)
    got = ctx.csg_field(primitives_to_device(prims), len(prims), frame, shape)
    _same(got, _fold(ctx, prims, frame, shape))


@pytest.mark.parametrize("seed,n,shape,spacing", [
    (21, 48, (40, 52, 36), 1.0 / 50),
    (22, 64, (64, 64, 64), -1.0 / 63),
])
def test_cull_equals_full_fold_reference_arith(seed, n, shape, spacing):
    """The same with GCM_PRIM_ARITH_REFERENCE (powf squares, per-sample cone
    bases): the enclosures still hold."""
    from gpucadforam_gb300.mesher import Context, make_frame, primitives_to_device

    c = Context(0)
    try:
        c.set_primitive_arith(True)
        prims = _scene(seed, n)
        origin = (0.0, 0.0, 0.0) if spacing > 0 else tuple(float(s) for s in shape[::-1])
        frame = make_frame(origin, (spacing,) * 3)
        got = c.csg_field(primitives_to_device(prims), len(prims), frame, shape)
        _same(got, _fold(c, prims, frame, shape))
    finally:
        c.close()


def test_cull_many_small_primitives(ctx):
    """256 small primitives (the most a scene may hold): most tiles keep only a few."""
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    prims = _scene(7, 256, size=(0.01, 0.05), ops=(0, 0, 0, 1), run=16)
    shape = (96, 96, 96)
    frame = make_frame((0.0, 0.0, 0.0), (1.0 / 95,) * 3)
    got = ctx.csg_field(primitives_to_device(prims), len(prims), frame, shape)
    _same(got, _fold(ctx, prims, frame, shape))


def test_cull_leading_subtract_and_intersect(ctx):
    """Runs that start the scene: subtract and intersect from +inf."""
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    prims = _scene(11, 30)
    for i in range(5):
        prims[i]["op"] = 1
    for i in range(5, 9):
        prims[i]["op"] = 2
    shape = (40, 48, 56)
    frame = make_frame((0.0, 0.0, 0.0), (1.0 / 47,) * 3)
    got = ctx.csg_field(primitives_to_device(prims), len(prims), frame, shape)
    _same(got, _fold(ctx, prims, frame, shape))


def test_cull_c3_scene_full_size(ctx):
    """The 384^3 scene of 64 spheres, capped cylinders and boxes, 8 subtracted."""
    import bench
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    prims = bench.csg_scene(bench.SEED + 1)
    n = 384
    h = np.float32(1.0 / (n - 1))
    frame = make_frame((0, 0, 0), (h, h, h))
    got = ctx.csg_field(primitives_to_device(prims), len(prims), frame, (n, n, n))
    _same(got, _fold(ctx, prims, frame, (n, n, n)))


def test_unbounded_primitives_are_kept(ctx):
    """Primitives whose enclosure is not finite (a centre at 1e30, a NaN
    radius, a cone of zero base radius) get (-inf, +inf) and are evaluated
    everywhere; as union members their NaN or infinite values leave the fold
    as the full evaluation leaves it."""
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    prims = _scene(21, 20, ops=(0, 1))
    extra = [dict(kind=0, op=0, center=np.array([1e30, 0.5, 0.5], np.float32), p=[0.1, 0.0]),
             dict(kind=0, op=0, center=np.array([0.5, 0.5, 0.5], np.float32), p=[float("nan"), 0.0]),
             dict(kind=5, op=0, center=np.array([0.4, 0.6, 0.5], np.float32), v3=(0.3, 0.2, 0.1), p=[0.0, 0.2])]
    prims = prims[:7] + extra + prims[7:]
    shape = (33, 40, 48)
    frame = make_frame((0.0, 0.0, 0.0), (1.0 / 39,) * 3)
    got = ctx.csg_field(primitives_to_device(prims), len(prims), frame, shape)
    _same(got, _fold(ctx, prims, frame, shape))


def test_primitive_count_limits(ctx):
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    import ctypes as C

    prims = _scene(3, 257)
    d = primitives_to_device(prims)
    out = torch.empty((4, 4, 4), device="cuda")
    frame = make_frame((0.0, 0.0, 0.0), (0.25,) * 3)
    rc = ctx.lib.gcm_field_csg(ctx.h, C.c_void_p(d.data_ptr()), 257, C.byref(frame), 4, 4, 4,
                               C.c_void_p(out.data_ptr()), None)
    assert rc == N.GCM_ERR_NOT_SUPPORTED
    rc = ctx.lib.gcm_field_csg(ctx.h, C.c_void_p(d.data_ptr()), 0, C.byref(frame), 4, 4, 4,
                               C.c_void_p(out.data_ptr()), None)
    assert rc == N.GCM_ERR_INVALID_ARGUMENT
    got = ctx.csg_field(d, 256, frame, (4, 4, 4))  # the largest scene
    _same(got, _fold(ctx, prims[:256], frame, (4, 4, 4)))
