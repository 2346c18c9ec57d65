"""The headline configuration at full size, against the oracles.

The 512^3 graded TPMS lattice that bench.py measures (16^3 control grid of
seeded uniform values, gyroid / Schwarz-P / diamond, period 16-64 voxels, Euler
angles in [-pi/4, pi/4], thickness in [-0.6, 0.6], phase origin at the grid
centre), evaluated and meshed on the GPU exactly as the bench step does:

* field: equal bit for bit to the oracle's restatement of the compensated
  arithmetic, and within 1e-5 relative (|f - f64| <= 1e-5 * max(1, |f64|)) of
  the FP64 oracle, on the corner, centre and top plane pairs (where the phase
  |X| is largest and smallest) and on random planes;
* classification: a sample is on a different side of the isovalue than the
  FP64 field only where |f64 - iso| < 1e-5;
* mesh: the vertices of each of those voxel planes, cut out of the full mesh
  by the per-plane vertex counts, equal marching cubes (oracle) of the device
  field's two planes bit for bit;
* counts: the fused pass, the count pass and the staged classify + scans agree,
  and every vertex lies inside the grid box.
"""
import numpy as np
import pytest
import torch

import oracle as O
from bench import N_CTRL, N_GRID, c2_controls

pytestmark = pytest.mark.gpu

N = N_GRID
ORIGIN = ((N - 1) / 2,) * 3
SLABS = (0, 255, N - 2)
REL = 1e-5


def host(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def headline():
    from gpucadforam_gb300.mesher import Context, Lattice

    ctx = Context(0)
    period, euler, thick, types = c2_controls()
    lat = Lattice.from_numpy(0, (N_CTRL,) * 3, period, euler, thick, types, ORIGIN)
    field = ctx.lattice_field(lat, (N, N, N))
    cnt = ctx.count_field(field, 0.0)
    pos = torch.empty((cnt.total_verts, 4), dtype=torch.float32, device="cuda")
    norm = torch.empty((cnt.total_verts, 4), dtype=torch.float32, device="cuda")
    mcnt = ctx.mesh_lattice(lat, (N, N, N), 0.0, pos=pos, norm=norm)
    verts, occ, _ = ctx.classify(field, 0.0)
    plane_verts = verts.view(N - 1, (N - 1) * (N - 1)).sum(1, dtype=torch.int64)
    start = host(torch.cumsum(plane_verts, 0) - plane_verts)
    yield dict(ctx=ctx, controls=(period, euler, thick, types), field=field, count=cnt, mesh_count=mcnt, pos=pos,
               norm=norm, verts=verts, occ=occ, start=start, plane_verts=host(plane_verts))
    ctx.close()


def _oracle_planes(h, z0, nplanes, fp64=False):
    period, euler, thick, types = h["controls"]
    return O.lattice_slab((N, N, N), z0, nplanes, 0, (N_CTRL,) * 3, period, euler, thick, types, ORIGIN,
                          fp64=fp64)


def _planes_to_check():
    rng = np.random.default_rng(20261204)
    return sorted(set(SLABS) | {int(z) for z in rng.integers(0, N - 1, 4)})


@pytest.mark.parametrize("z0", _planes_to_check())
def test_headline_field_vs_oracles(headline, z0):
    got = host(headline["field"][z0:z0 + 2])
    ref32 = _oracle_planes(headline, z0, 2)
    ref64 = _oracle_planes(headline, z0, 2, fp64=True)
    # the oracle restates the kernel's float operations one for one
    assert got.tobytes() == ref32.tobytes()
    err = np.abs(got.astype(np.float64) - ref64)
    rel = err / np.maximum(1.0, np.abs(ref64))
    assert rel.max() <= REL, f"worst relative error {rel.max():.3e}"
    # side of the isovalue (cube-index bits) differs only within 1e-5 of it
    flip = (got < 0.0) != (ref64 < 0.0)
    assert (np.abs(ref64[flip]) < REL).all()


@pytest.mark.parametrize("z0", SLABS)
def test_headline_mesh_planes_vs_oracle_mc(headline, z0):
    slab = host(headline["field"][z0:z0 + 2])
    # the slab's voxel plane is plane z0 of the full grid: grid centre -z0 along
    # z gives the same d = gridPos - gridcenter, so the same vertex arithmetic
    opos, onorm, _ = O.mesh(slab, (1, 1, 1), (0, 0, -z0), 0.0)
    a, n = int(headline["start"][z0]), int(headline["plane_verts"][z0])
    assert n == len(opos)
    assert host(headline["pos"][a:a + n]).tobytes() == opos.tobytes()
    assert host(headline["norm"][a:a + n]).tobytes() == onorm.tobytes()


def test_headline_counts_and_bounds(headline):
    ctx = headline["ctx"]
    cnt, mcnt = headline["count"], headline["mesh_count"]
    _, total = ctx.scan(headline["verts"])
    _, active = ctx.scan(headline["occ"])
    assert total == cnt.total_verts == mcnt.total_verts
    assert active == cnt.active_voxels == mcnt.active_voxels
    assert int(headline["plane_verts"].sum()) == total
    pos, norm = headline["pos"], headline["norm"]
    assert float(pos[:, :3].min()) >= 0.0 and float(pos[:, :3].max()) <= N - 1
    assert bool((pos[:, 3] == 1.0).all()) and bool((norm[:, 3] == 0.0).all())
