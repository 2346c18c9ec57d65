"""GPU, through the C ABI: the SVL period-field generator (gcm_svl_period_field),
its min/max range map (gcm_normalise_range) and the lattice mask
(gcm_lattice_mask), bit for bit against the reference's own kernels
(tests/golden/golden_period_mask.npz), and against the oracle on larger and
ragged grids."""
import numpy as np
import pytest
import torch

import oracle as O
from tests.helpers import golden

pytestmark = pytest.mark.gpu

PM = golden("golden_period_mask.npz")


@pytest.fixture(scope="module")
def ctx():
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    yield c
    c.close()


def host(t):
    return t.detach().cpu().numpy()


def _period(i):
    P = PM[f"period{i}/params"]
    return tuple(int(v) for v in P[:3]), P[3:6], P[6:9], chr(int(P[9])), float(P[10]), float(P[11])


@pytest.mark.parametrize("i", range(4))
def test_period_field_and_range_vs_reference(ctx, i):
    """set_period_kernel then GPU_buffer_normalise_three in place, as
    src/main.cu:3929-3931 calls them: raw field, min/max and mapped field."""
    n, d, mean, axis, a1, b1 = _period(i)
    f = ctx.svl_period_field(n[::-1], d, mean, axis)
    assert host(f).tobytes() == PM[f"period{i}/raw"].tobytes()
    out, mm = ctx.normalise_range(f, a1, b1, out=f)
    assert host(out).tobytes() == PM[f"period{i}/mapped"].tobytes()
    assert np.array(mm, np.float32).tobytes() == PM[f"period{i}/minmax"].tobytes()


@pytest.mark.parametrize("i", range(6))
def test_lattice_mask_vs_reference(ctx, i):
    f = PM[f"mask{i}/flags"]
    n = len(PM[f"mask{i}/lat"])
    lat = torch.from_numpy(PM[f"mask{i}/lat"].copy()).cuda().view(1, 1, n)
    acc = torch.from_numpy(PM[f"mask{i}/acc"].copy()).cuda()
    prim = torch.from_numpy(PM[f"mask{i}/prim"].copy()).cuda()
    ctx.lattice_mask(lat, acc, prim, bool(f[0]), bool(f[1]))
    assert host(lat).tobytes() == PM[f"mask{i}/out"].tobytes()


@pytest.mark.parametrize("shape", [(37, 50, 61), (128, 96, 80)])
def test_period_and_mask_vs_oracle_ragged(ctx, shape):
    nz, ny, nx = shape
    mean = (nx / 2.0, ny / 2.0, nz / 2.0)
    f = ctx.svl_period_field(shape, (1.0, 1.0, 1.0), mean, "z")
    ref = O.svl_period_field((nx, ny, nz), (1.0, 1.0, 1.0), mean, "z")
    assert host(f).tobytes() == ref.tobytes()
    out, _ = ctx.normalise_range(f, nx // 10, nx // 4)
    oref, _ = O.normalise_range(ref, np.float32(nx // 10), np.float32(nx // 4))
    assert host(out).tobytes() == oref.tobytes()
    rng = np.random.default_rng(sum(shape))
    accn = np.zeros((nz * ny * nx, 4), np.float32)
    accn.view(np.int32)[:, 0] = rng.integers(-1, 2, nz * ny * nx)
    prim = rng.uniform(-1, 1, shape).astype(np.float32)
    for fixed, dynamic in ((1, 0), (0, 1)):
        lat = torch.from_numpy(host(out).copy()).cuda()
        ctx.lattice_mask(lat, torch.from_numpy(accn).cuda(), torch.from_numpy(prim).cuda(), fixed, dynamic)
        assert host(lat).tobytes() == O.lattice_mask(host(out), accn, prim, fixed, dynamic).tobytes()


def test_period_field_feeds_the_svl_solve(ctx):
    """The generated period field drives gcm_svl_lattice exactly as the same
    values made by the reference's kernels do (the spatial-lattice run needs
    no reference kernel)."""
    n, d, mean, axis, a1, b1 = _period(0)
    f = ctx.svl_period_field(n[::-1], d, mean, axis)
    ctx.normalise_range(f, a1, b1, out=f)
    ref = torch.from_numpy(PM["period0/mapped"].copy()).cuda().view_as(f)
    coef = ctx.svl_coefficients(0, 21, 2)
    a = ctx.svl_lattice(n, coef, kind="r", period_type=2, d_period=f, n_coeff=8)
    b = ctx.svl_lattice(n, coef, kind="r", period_type=2, d_period=ref, n_coeff=8)
    assert host(a[0]).tobytes() == host(b[0]).tobytes()
    assert list(a[1]) == list(b[1])
