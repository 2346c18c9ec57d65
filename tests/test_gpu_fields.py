"""GPU parity of the field kernels, through the C ABI.

Unit cells and primitives against the reference's own kernels (fixtures);
primitives bit for bit against the reference's own kernels; graded lattices bit
for bit against the oracle's restatement of the kernels' compensated float
arithmetic and within 1e-5 relative of the FP64 oracle; CSG scenes against the
FP32 and FP64 oracles.  Tolerances are written in each test.
"""
import numpy as np
import pytest
import torch

import oracle as O
from tests.helpers import assert_field_close, assert_rel_close, golden, n_cases

pytestmark = pytest.mark.gpu

FIELDS = golden("golden_fields.npz")


@pytest.fixture(scope="module")
def ctx():
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    yield c
    c.close()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "unit")))
def test_unit_cell_vs_reference(ctx, i):
    nx, ny, nz, t = (int(v) for v in FIELDS[f"in/unit{i}"])
    got = host(ctx.unit_cell(t, nx, ny, nz))
    # same CUDA trig library as the reference; differences come only from
    # expression contraction in the reference build
    assert_field_close(got, FIELDS[f"sm103a/unit{i}"], k_rel=2, k_scale=4)


@pytest.mark.parametrize("shape", [(300, 7, 9), (5, 40, 33), (257, 65, 3), (96, 130, 2)])
@pytest.mark.parametrize("t", range(6))
def test_unit_cell_layouts_vs_oracle(ctx, shape, t):
    """The unit-cell kernel forms its double coordinate factors once per
    column (per thread) and once per sample row (in shared memory), over
    column chunks of up to 256 and items of 64 rows: several chunks with a
    ragged last one (300, 257), rows narrower than a warp (5), row counts
    that leave a partial item, and planes of 2 and 3 samples must give the
    per-sample values.  The oracle computes every sample on its own with
    the host's trig, so the tolerance is the oracle's against the reference
    kernels plus the kernel's own."""
    nx, ny, nz = shape
    got = host(ctx.unit_cell(t, nx, ny, nz))
    assert_field_close(got, O.unit_cell(t, nx, ny, nz), k_rel=6, k_scale=12)


def _prim_case(i):
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    q = FIELDS[f"in/prim{i}"]
    nx, ny, nz = (int(v) for v in q[:3])
    prim = dict(kind=int(q[6]), flag=int(q[7]), center=q[8:11], v3=q[11:14], p=q[14:20], op=0)
    origin = [np.float32((n - 1) / 2.0) for n in (nx, ny, nz)]  # the reference's centred frame
    return primitives_to_device([prim]), make_frame(origin, q[3:6]), (nz, ny, nx), q


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "prim")))
def test_primitive_vs_reference(ctx, i):
    """Default arithmetic: the reference build's operation order and fused
    multiply-adds with correctly rounded squares (the reference's powf(v, 2)
    differs from them in the last bit for some floats): within 4 ulp of the
    value plus 3 ulp of the field's scale."""
    prims, frame, shape, q = _prim_case(i)
    got = host(ctx.csg_field(prims, 1, frame, shape))
    assert_field_close(got, FIELDS[f"sm103a/prim{i}"], k_rel=4, k_scale=3)
    if int(q[6]) in (0, 1) or not q[11:14].any():
        # no trig: the oracle restates the default arithmetic bit for bit
        ref32 = O.primitive(int(q[6]), shape[::-1], q[3:6], q[8:11], q[11:14], q[14:20], int(q[7]))
        assert got.tobytes() == ref32.tobytes()


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "prim")))
def test_primitive_reference_arith_bit_exact(i):
    """GCM_PRIM_ARITH_REFERENCE: the reference's own kernels' values, bit for bit."""
    from gpucadforam_gb300.mesher import Context

    prims, frame, shape, _ = _prim_case(i)
    c = Context(0)
    try:
        c.set_primitive_arith(True)
        got = host(c.csg_field(prims, 1, frame, shape))
    finally:
        c.close()
    assert got.tobytes() == FIELDS[f"sm103a/prim{i}"].tobytes()


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "norm")))
def test_normalise_band_vs_reference(ctx, i):
    P = FIELDS[f"in/norm{i}/params"]
    nx, ny, nz = (int(v) for v in P[:3])
    f = FIELDS[f"in/norm{i}/field"].reshape(nz, ny, nx)
    lab, nf, mm = ctx.normalise_band(dev(f), float(np.float32(P[3])), float(np.float32(P[4])))
    assert np.array_equal(np.array(mm, np.float32), FIELDS[f"sm103a/norm{i}/minmax"])
    assert np.array_equal(host(lab).reshape(-1), FIELDS[f"sm103a/norm{i}/label"])
    assert np.array_equal(host(nf).reshape(-1), FIELDS[f"sm103a/norm{i}/normf"])


def _graded(seed, C, mode):
    rng = np.random.default_rng(seed)
    n = C ** 3
    return dict(mode=mode, ctrl=(C, C, C), period=rng.uniform(16, 64, n).astype(np.float32),
                euler=rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32),
                thickness=rng.uniform(-0.6, 0.6, n).astype(np.float32),
                types=rng.choice(np.array([0, 1, 2, 3, 5], np.uint8), n))


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("shape", [(96, 96, 96), (40, 70, 33)])
def test_graded_lattice_vs_oracle(ctx, mode, shape):
    from gpucadforam_gb300.mesher import Lattice

    nz, ny, nx = shape
    L = _graded(7 + mode, 8, mode)
    origin = ((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2)
    lat = Lattice.from_numpy(L["mode"], L["ctrl"], L["period"], L["euler"], L["thickness"], L["types"], origin)
    got = host(ctx.lattice_field(lat, shape))
    ref32 = O.lattice_field((nx, ny, nz), mode, L["ctrl"], L["period"], L["euler"], L["thickness"], L["types"], origin)
    ref64 = O.lattice_field((nx, ny, nz), mode, L["ctrl"], L["period"], L["euler"], L["thickness"], L["types"], origin,
                            fp64=True)
    # the oracle restates the kernels' compensated float arithmetic step for step
    assert got.tobytes() == ref32.tobytes()
    # FP64 oracle: within 1e-5 relative, |f - f64| <= 1e-5 * max(1, |f64|)
    assert_rel_close(got, ref64, 1e-5)


@pytest.mark.parametrize("shape,ctrl", [
    ((20, 18, 40), (1, 1, 1)),        # one control point: a single lattice
    ((30, 26, 61), (3, 2, 5)),        # warp per row, few columns
    ((24, 20, 100), (24, 4, 4)),      # warp per row, widest in the default shared memory (24 columns)
    ((20, 16, 90), (25, 3, 3)),       # warp per row in opt-in shared memory
    ((12, 10, 120), (80, 2, 2)),      # warp per row at its widest (80 columns)
    ((10, 8, 140), (81, 2, 2)),       # CTA per row, records staged by the CTA
    ((10, 8, 300), (140, 2, 2)),      # CTA per row, records read from the setup buffer
])
def test_blend_lattice_kernel_forms_vs_oracle(ctx, shape, ctrl):
    """The blend grading runs as a warp per sample row (control grids up to 80
    columns, above 24 in opt-in shared memory) or a CTA per row (staged up to
    128 columns, else unstaged); every form equals the oracle bit for bit and
    the FP64 oracle within 1e-5."""
    from gpucadforam_gb300.mesher import Lattice

    nz, ny, nx = shape
    rng = np.random.default_rng(sum(shape) + sum(ctrl) + 1)
    n = ctrl[0] * ctrl[1] * ctrl[2]
    period = rng.uniform(16, 64, n).astype(np.float32)
    euler = rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32)
    thick = rng.uniform(-0.6, 0.6, n).astype(np.float32)
    types = rng.choice(np.array([0, 1, 2, 3, 5], np.uint8), n)
    origin = ((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2)
    lat = Lattice.from_numpy(1, ctrl, period, euler, thick, types, origin)
    got = host(ctx.lattice_field(lat, shape))
    ref32 = O.lattice_field((nx, ny, nz), 1, ctrl, period, euler, thick, types, origin)
    assert got.tobytes() == ref32.tobytes()
    ref64 = O.lattice_field((nx, ny, nz), 1, ctrl, period, euler, thick, types, origin, fp64=True)
    assert_rel_close(got, ref64, 1e-5)


@pytest.mark.parametrize("shape,ctrl", [
    ((200, 200, 64), (16, 16, 16)),   # 40,000 sample rows: 8 rows per warp
    ((150, 150, 64), (16, 16, 16)),   # 22,500 rows: 4 per warp
    ((110, 110, 70), (16, 16, 16)),   # 12,100 rows: 2 per warp; rows of 70 end on a single-sample step
    ((40, 40, 100), (16, 16, 16)),    # 1,600 rows: 1 per warp; a ragged second segment
    ((24, 20, 300), (64, 4, 4)),      # 64 control columns: one row's records per warp fit
    ((12, 10, 500), (200, 3, 3)),     # 200 control columns: one row per warp in opt-in shared memory
    ((6, 5, 700), (300, 2, 2)),       # 300 control columns: the unstaged kernel
])
def test_graded_lattice_kernel_forms_vs_oracle(ctx, shape, ctrl):
    """Each staged form of the PARAMS field kernel (rows per warp picked from
    the row count and the control-grid width) and the unstaged kernel agree
    with the FP32 oracle to the trig tolerance."""
    from gpucadforam_gb300.mesher import Lattice

    nz, ny, nx = shape
    rng = np.random.default_rng(sum(shape) + sum(ctrl))
    n = ctrl[0] * ctrl[1] * ctrl[2]
    period = rng.uniform(16, 64, n).astype(np.float32)
    euler = rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32)
    thick = rng.uniform(-0.6, 0.6, n).astype(np.float32)
    types = rng.choice(np.array([0, 1, 2, 3, 5], np.uint8), n)
    origin = ((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2)
    lat = Lattice.from_numpy(0, ctrl, period, euler, thick, types, origin)
    got = host(ctx.lattice_field(lat, shape))
    ref32 = O.lattice_field((nx, ny, nz), 0, ctrl, period, euler, thick, types, origin)
    assert got.tobytes() == ref32.tobytes()
    ref64 = O.lattice_field((nx, ny, nz), 0, ctrl, period, euler, thick, types, origin, fp64=True)
    assert_rel_close(got, ref64, 1e-5)


def test_c1_uniform_gyroid_fp64(ctx):
    from gpucadforam_gb300.mesher import Lattice

    lat = Lattice.from_numpy(0, (1, 1, 1), np.array([32.0], np.float32))
    got = host(ctx.lattice_field(lat, (128, 128, 128)))
    z, y, x = np.meshgrid(*(np.arange(128, dtype=np.float64),) * 3, indexing="ij")
    k = 2 * np.pi / 32
    ref = np.sin(k * x) * np.cos(k * y) + np.sin(k * y) * np.cos(k * z) + np.sin(k * z) * np.cos(k * x)
    # phases i/16 are exact in FP32, so only sinpi/cospi rounding remains
    assert np.abs(got - ref).max() < 1e-6


def _csg_scene(seed, n_prims=64, n_sub=8):
    rng = np.random.default_rng(seed)
    prims = []
    for i in range(n_prims):
        kind = int(rng.integers(0, 3))
        c = rng.uniform(0, 1, 3).astype(np.float32)
        op = 1 if i >= n_prims - n_sub else 0
        if kind == 0:
            prims.append(dict(kind=0, op=op, center=c, p=[rng.uniform(0.02, 0.15), 0.0]))
        elif kind == 1:
            r, hh = rng.uniform(0.02, 0.12, 2)
            prims.append(dict(kind=1, op=op, center=c, v3=(0.0, 0.0, 1.0), p=[r, 0.0, 2 * hh]))
        else:
            he = rng.uniform(0.02, 0.12, 3)
            prims.append(dict(kind=2, op=op, center=c, v3=(0.0, 0.0, 0.0), p=list(2 * he)))
    return prims


def test_csg_scene_vs_oracle(ctx):
    from gpucadforam_gb300.mesher import make_frame, primitives_to_device

    n = 96
    prims = _csg_scene(0xD4A + 3)
    h = np.float32(1.0 / (n - 1))
    got = host(ctx.csg_field(primitives_to_device(prims), len(prims), make_frame((0, 0, 0), (h, h, h)), (n, n, n)))
    ref32 = O.csg_field(prims, (n, n, n), (0, 0, 0), (h, h, h))
    # spheres, z-axis cylinders and unrotated boxes use no trig: the oracle
    # restates the default arithmetic operation for operation
    assert got.tobytes() == ref32.tobytes()
    ref64 = O.csg_field(prims, (n, n, n), (0, 0, 0), (h, h, h), fp64=True)
    assert np.abs(got - ref64).max() < 1e-5 * max(1.0, float(np.abs(ref64).max()))


def test_lattice_mesh_equals_oracle_mc_of_device_field(ctx):
    """End to end: the fused lattice mesher's output equals marching cubes (oracle)
    of the field the device evaluated; cube indices of that field differ from the
    FP64 field's only where |f - iso| < 1e-5 (the stated field tolerance)."""
    from gpucadforam_gb300.mesher import Lattice

    n = 80
    L = _graded(11, 8, 0)
    origin = ((n - 1) / 2,) * 3
    lat = Lattice.from_numpy(0, L["ctrl"], L["period"], L["euler"], L["thickness"], L["types"], origin)
    field = ctx.lattice_field(lat, (n, n, n))
    cap = ctx.count_field(field, 0.0).total_verts
    pos = torch.empty((cap, 4), device="cuda")
    norm = torch.empty((cap, 4), device="cuda")
    cnt = ctx.mesh_lattice(lat, (n, n, n), 0.0, pos=pos, norm=norm)
    f = host(field)
    opos, onorm, _ = O.mesh(f, (1, 1, 1), (0, 0, 0), 0.0)
    assert cnt.total_verts == len(opos)
    assert host(pos).tobytes() == opos.tobytes() and host(norm).tobytes() == onorm.tobytes()
    f64 = O.lattice_field((n, n, n), 0, L["ctrl"], L["period"], L["euler"], L["thickness"], L["types"], origin,
                          fp64=True)
    _, _, c32 = O.mc_classify(f, 0.0)
    _, _, c64 = O.mc_classify(f64.astype(np.float32), 0.0)
    diff = c32 != c64
    if diff.any():
        # every differing voxel has a corner within tolerance of the isovalue
        near = np.abs(f64) < 1e-5
        nv = np.zeros(c32.shape, bool)
        m = near
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    nv |= m[dz:dz + n - 1, dy:dy + n - 1, dx:dx + n - 1].reshape(-1)
        assert nv[diff].all()


def test_mesh_lattice_async_equals_sync(ctx):
    """gcm_mesh_lattice_async: same vertices and counts as gcm_mesh_lattice, the
    counts left on the device, for two calls in flight on one stream into
    different buffers (the second reuses the context's field buffer)."""
    from gpucadforam_gb300.mesher import Lattice

    shapes = [(72, 80, 64), (64, 64, 64)]
    lats = []
    for k, shape in enumerate(shapes):
        L = _graded(31 + k, 8, 0)
        origin = tuple((d - 1) / 2 for d in shape[::-1])
        lats.append(Lattice.from_numpy(0, L["ctrl"], L["period"], L["euler"], L["thickness"], L["types"], origin))
    ref = []
    for lat, shape in zip(lats, shapes):
        cap = ctx.count_field(ctx.lattice_field(lat, shape), 0.0).total_verts
        pos = torch.empty((cap, 4), device="cuda")
        norm = torch.empty((cap, 4), device="cuda")
        c = ctx.mesh_lattice(lat, shape, 0.0, pos=pos, norm=norm)
        ref.append((c, host(pos), host(norm)))
    outs = []
    for (c, p, _), lat, shape in zip(ref, lats, shapes):
        pos = torch.full((c.total_verts, 4), float("nan"), device="cuda")
        norm = torch.full((c.total_verts, 4), float("nan"), device="cuda")
        d_counts = torch.zeros(4, dtype=torch.int64, device="cuda")
        ctx.mesh_lattice_async(lat, shape, 0.0, pos, norm, d_counts)
        outs.append((pos, norm, d_counts))
    torch.cuda.synchronize()
    for (c, p, n), (pos, norm, d_counts) in zip(ref, outs):
        dc = host(d_counts)
        assert int(dc[0]) == c.active_voxels and int(dc[1]) == c.total_verts and int(dc[2]) == 0
        assert host(pos).tobytes() == p.tobytes() and host(norm).tobytes() == n.tobytes()


def test_lattice_grids_with_too_many_sample_rows_are_refused(ctx):
    """The lattice field kernels count sample rows (ny * nz) in 32 bits: a grid
    of 2^31 rows or more is refused before anything launches or allocates,
    by the single-grid call and by a batch."""
    import ctypes as C

    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import Batch, Lattice

    lat = Lattice.from_numpy(0, (1, 1, 1), np.array([16.0], np.float32))
    s = ctx.lattice_struct(lat)
    dummy = torch.empty(16, device="cuda")
    rc = ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), 2, 65536, 32768, C.c_void_p(dummy.data_ptr()), None)
    assert rc == N.GCM_ERR_NOT_SUPPORTED
    with pytest.raises(N.GcmError) as e:
        Batch(ctx, [lat, lat], [(16, 16, 16), (32768, 65536, 2)])
    assert e.value.code == N.GCM_ERR_NOT_SUPPORTED
    # a small grid on the same context still evaluates (12 samples into the 16-float buffer)
    rc = ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), 2, 2, 3, C.c_void_p(dummy.data_ptr()), None)
    assert rc == N.GCM_OK
