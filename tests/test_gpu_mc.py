"""GPU parity of the marching-cubes kernels, through the C ABI.

Bit-exact against the fixtures made by the reference's own kernels
(tests/golden/golden_mc.npz) and against the CPU oracle on larger grids; the
full-size cases check size-independent properties (count pass == emit pass,
repeat runs identical, overflow keeps the true counts).
"""
import numpy as np
import pytest
import torch

import oracle as O
from tests.helpers import band_case, golden, n_cases, plain_case

pytestmark = pytest.mark.gpu

MC = golden("golden_mc.npz")


@pytest.fixture(scope="module", params=[(256, 2048), (128, 1024), "sparse"], ids=["256x2048", "128x1024", "sparse"])
def ctx(request):
    """Every case runs through two launch shapes of the fused kernel and
    through the sparse (window) path."""
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    if request.param == "sparse":
        c.set_mesh_path("sparse")
    else:
        c.set_launch_shape(*request.param)
    yield c
    c.close()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("i", range(n_cases(MC, "plain")))
def test_fused_matches_reference(ctx, i):
    f, iso, vs, gc = plain_case(MC, i)
    pos, norm, cnt = ctx.mesh_field(dev(f), iso, tuple(vs), tuple(gc))
    ref_pos = MC[f"sm103a/plain{i}/pos"]
    assert cnt.total_verts == len(ref_pos)
    assert cnt.active_voxels == len(MC[f"sm103a/plain{i}/compacted"])
    assert host(pos).tobytes() == ref_pos.tobytes()
    assert host(norm).tobytes() == MC[f"sm103a/plain{i}/norm"].tobytes()


@pytest.mark.parametrize("i", range(n_cases(MC, "plain")))
def test_staged_matches_reference(ctx, i):
    f, iso, vs, gc = plain_case(MC, i)
    df = dev(f)
    verts, occ, cube = ctx.classify(df, iso)
    assert np.array_equal(host(verts).view(np.uint32), MC[f"sm103a/plain{i}/verts"])
    assert np.array_equal(host(occ).view(np.uint32), MC[f"sm103a/plain{i}/occ"])
    occ_scan, active = ctx.scan(occ)
    verts_scan, total = ctx.scan(verts)
    assert np.array_equal(host(occ_scan).view(np.uint32), MC[f"sm103a/plain{i}/occ_scan"])
    assert np.array_equal(host(verts_scan).view(np.uint32), MC[f"sm103a/plain{i}/verts_scan"])
    comp = ctx.compact(occ, occ_scan, active)
    assert np.array_equal(host(comp).view(np.uint32), MC[f"sm103a/plain{i}/compacted"])
    pos, norm = ctx.generate(df, iso, comp, verts_scan, total, tuple(vs), tuple(gc))
    assert host(pos).tobytes() == MC[f"sm103a/plain{i}/pos"].tobytes()
    assert host(norm).tobytes() == MC[f"sm103a/plain{i}/norm"].tobytes()


@pytest.mark.parametrize("i", range(n_cases(MC, "band")))
def test_band_matches_reference(ctx, i):
    lab, nf, iso, lo, hi, vs, gc = band_case(MC, i)
    pos, norm, cnt = ctx.mesh_band(dev(lab), dev(nf), iso, lo, hi, tuple(vs), tuple(gc))
    assert host(pos).tobytes() == MC[f"sm103a/band{i}/pos"].tobytes()
    assert host(norm).tobytes() == MC[f"sm103a/band{i}/norm"].tobytes()


def _gyroid_c1(n=128, period=32.0):
    """Uniform gyroid on the voxel index (k = 2 pi / period), as the oracle evaluates it."""
    return O.lattice_field((n, n, n), 0, (1, 1, 1), np.array([period], np.float32))


def test_c1_gyroid_128_bit_exact_vs_oracle(ctx):
    f = _gyroid_c1()
    h = np.float32(1.0 / 127.0)
    pos, norm, cnt = ctx.mesh_field(dev(f), 0.0, (h, h, h), (0, 0, 0))
    opos, onorm, oact = O.mesh(f, (h, h, h), (0, 0, 0), 0.0)
    assert cnt.total_verts == len(opos) and cnt.active_voxels == oact
    assert host(pos).tobytes() == opos.tobytes()
    assert host(norm).tobytes() == onorm.tobytes()


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 2, 5), (2, 17, 3), (9, 33, 70), (5, 300, 7), (40, 3, 600),
                                   (3, 2, 9000)])
def test_ragged_shapes_vs_oracle(ctx, shape):
    rng = np.random.default_rng(sum(shape))
    f = rng.standard_normal(shape).astype(np.float32)
    pos, norm, cnt = ctx.mesh_field(dev(f), 0.1, (0.5, 0.25, 2.0), (1.0, 0.0, -3.0))
    opos, onorm, oact = O.mesh(f, (0.5, 0.25, 2.0), (1.0, 0.0, -3.0), 0.1)
    assert cnt.total_verts == len(opos) and cnt.active_voxels == oact
    assert host(pos).tobytes() == opos.tobytes()
    assert host(norm).tobytes() == onorm.tobytes()


def test_misaligned_field_takes_scalar_path(ctx):
    f = _gyroid_c1(48, 12.0)
    flat = torch.empty(f.size + 1, dtype=torch.float32, device="cuda")
    flat[1:] = dev(f).reshape(-1)
    view = flat[1:].view(f.shape)  # 4-byte aligned, not 16-byte aligned
    assert view.data_ptr() % 16 != 0
    pos_a, norm_a, _ = ctx.mesh_field(dev(f), 0.2)
    pos_b, norm_b, _ = ctx.mesh_field(view, 0.2)
    assert host(pos_a).tobytes() == host(pos_b).tobytes()
    assert host(norm_a).tobytes() == host(norm_b).tobytes()


def test_no_surface(ctx):
    f = np.ones((20, 21, 22), np.float32)
    cnt = ctx.count_field(dev(f), 0.5)
    assert cnt.total_verts == 0 and cnt.active_voxels == 0
    pos, norm, cnt = ctx.mesh_field(dev(f), 0.5)
    assert cnt.total_verts == 0


def test_band_default_shape_equals_explicit(ctx):
    """A context whose launch shape was never set meshes band fields with its
    own default shape; the output equals that of the explicit shapes."""
    from gpucadforam_gb300.mesher import Context

    lab, nf, iso, lo, hi, vs, gc = band_case(MC, 0)
    ref = ctx.mesh_band(dev(lab), dev(nf), iso, lo, hi, tuple(vs), tuple(gc))
    fresh = Context(0)
    try:
        got = fresh.mesh_band(dev(lab), dev(nf), iso, lo, hi, tuple(vs), tuple(gc))
    finally:
        fresh.close()
    assert got[2].total_verts == ref[2].total_verts
    assert host(got[0]).tobytes() == host(ref[0]).tobytes() and host(got[1]).tobytes() == host(ref[1]).tobytes()


def test_iso_exactly_everywhere_is_outside(ctx):
    """f == iso at every sample: no corner is inside (f < iso), no triangles."""
    f = np.full((9, 10, 11), 0.25, np.float32)
    cnt = ctx.count_field(dev(f), 0.25)
    assert cnt.total_verts == 0 and cnt.active_voxels == 0


def test_nan_and_inf_samples_vs_oracle(ctx):
    """NaN samples are outside (f < iso is false); infinities are ordinary
    corners whose edges interpolate to an end point or to NaN.  Counts and
    cube indices are exact; positions and normals match bit for bit where
    they are numbers and are NaN in the same places (NaN payloads differ
    between the host's and the GPU's arithmetic)."""
    rng = np.random.default_rng(77)
    f = rng.standard_normal((23, 29, 37)).astype(np.float32)
    flat = f.reshape(-1)
    pick = rng.choice(flat.size, 400, replace=False)
    flat[pick[:150]] = np.nan
    flat[pick[150:280]] = np.inf
    flat[pick[280:]] = -np.inf
    pos, norm, cnt = ctx.mesh_field(dev(f), 0.0, (0.5, 1.0, 0.25), (0.0, 1.0, 0.0))
    opos, onorm, oact = O.mesh(f, (0.5, 1.0, 0.25), (0.0, 1.0, 0.0), 0.0)
    assert cnt.total_verts == len(opos) and cnt.active_voxels == oact
    _, _, cube = ctx.classify(dev(f), 0.0)
    _, _, ocube = O.mc_classify(f, 0.0)
    assert np.array_equal(host(cube).reshape(-1), ocube.reshape(-1))
    for got, ref in ((host(pos), opos), (host(norm), onorm)):
        gn, rn = np.isnan(got), np.isnan(ref)
        assert np.array_equal(gn, rn)
        assert got[~gn].tobytes() == ref[~rn].tobytes()
    assert np.isnan(host(pos)).any()  # the case does reach the NaN edges


def test_overflow_reports_true_counts(ctx):
    f = _gyroid_c1(64, 16.0)
    full_pos, full_norm, full = ctx.mesh_field(dev(f), 0.0)
    cap = (full.total_verts // 2) // 3 * 3 + 1
    pos = torch.full((cap, 4), -7.0, device="cuda")
    norm = torch.full((cap, 4), -7.0, device="cuda")
    p, n, cnt = ctx.mesh_field(dev(f), 0.0, pos=pos, norm=norm, capacity=cap, allow_overflow=True)
    assert cnt.status == 2 and cnt.total_verts == full.total_verts
    fits = (cap // 3) * 3
    assert host(pos[:fits]).tobytes() == host(full_pos[:fits]).tobytes()
    assert bool((pos[fits:] == -7.0).all())


def test_repeat_runs_identical_and_count_matches(ctx):
    f = O.lattice_field((96, 80, 72), 0, (1, 1, 1), np.array([10.0], np.float32), types=np.array([5], np.uint8))
    d = dev(f)
    a = ctx.mesh_field(d, 0.3)
    b = ctx.mesh_field(d, 0.3)
    c = ctx.count_field(d, 0.3)
    assert host(a[0]).tobytes() == host(b[0]).tobytes() and host(a[1]).tobytes() == host(b[1]).tobytes()
    assert c.total_verts == a[2].total_verts and c.active_voxels == a[2].active_voxels


def test_lookback_wait_runs_out_and_context_survives(ctx):
    import ctypes as C
    from gpucadforam_gb300 import _native as N

    ntiles, stall = 64, 20
    out = torch.zeros(ntiles, dtype=torch.int64, device="cuda")
    rc = ctx.lib.gcm_test_lookback_stall(ctx.h, ntiles, stall, 5_000_000, C.c_void_p(out.data_ptr()),
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.GCM_ERR_DEVICE_TIMEOUT
    pre = host(out).view(np.uint64)
    assert list(pre[:stall]) == list(range(stall))  # tiles before the stalled one are exact
    # the context and device still work
    f = _gyroid_c1(32, 8.0)
    pos, norm, cnt = ctx.mesh_field(dev(f), 0.0)
    opos, _, _ = O.mesh(f, (1, 1, 1), (0, 0, 0), 0.0)
    assert host(pos).tobytes() == opos.tobytes()
