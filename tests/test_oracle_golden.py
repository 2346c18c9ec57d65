"""Pins the CPU oracle to outputs of the reference's own CUDA kernels.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py, which
runs the reference's kernels (compiled from its sources by oracle/ref/build_ref.py)
on a GB300.  Marching-cubes data is integer/byte work plus IEEE-rounded vertex
arithmetic and must match bit for bit; analytic fields go through sinf/cosf, whose
CUDA and glibc implementations differ by a few ulp, and are checked to the stated
tolerance.
"""
import numpy as np
import pytest

import oracle as O
from tests.helpers import assert_field_close, band_case, golden, n_cases, plain_case

MC = golden("golden_mc.npz")
FIELDS = golden("golden_fields.npz")


@pytest.mark.parametrize("i", range(n_cases(MC, "plain")))
def test_plain_classify_scan_compact(i):
    f, iso, vs, gc = plain_case(MC, i)
    verts, occ, _ = O.mc_classify(f, iso)
    assert np.array_equal(verts, MC[f"sm103a/plain{i}/verts"])
    assert np.array_equal(occ, MC[f"sm103a/plain{i}/occ"])
    occ_scan, _ = O.scan_exclusive(occ)
    verts_scan, _ = O.scan_exclusive(verts)
    assert np.array_equal(occ_scan, MC[f"sm103a/plain{i}/occ_scan"])
    assert np.array_equal(verts_scan, MC[f"sm103a/plain{i}/verts_scan"])
    assert np.array_equal(O.mc_compact(occ, occ_scan), MC[f"sm103a/plain{i}/compacted"])


@pytest.mark.parametrize("i", range(n_cases(MC, "plain")))
def test_plain_vertices_bit_exact(i):
    f, iso, vs, gc = plain_case(MC, i)
    pos, norm, _ = O.mesh(f, vs, gc, iso)
    assert pos.tobytes() == MC[f"sm103a/plain{i}/pos"].tobytes()
    assert norm.tobytes() == MC[f"sm103a/plain{i}/norm"].tobytes()


def test_contraction_pattern_is_unique():
    """Only the default pattern reproduces the reference's normals and positions."""
    f, iso, vs, gc = plain_case(MC, 1)
    verts, occ, _ = O.mc_classify(f, iso)
    occ_scan, _ = O.scan_exclusive(occ)
    verts_scan, total = O.scan_exclusive(verts)
    comp = O.mc_compact(occ, occ_scan)
    matches = []
    for a in range(64):
        if ((a >> 2) & 3) == 3 or ((a >> 4) & 3) == 3:
            continue
        pos, norm = O.mc_generate(f, vs, gc, iso, comp, verts_scan, total, arith=a)
        if pos.tobytes() == MC["sm103a/plain1/pos"].tobytes() and norm.tobytes() == MC["sm103a/plain1/norm"].tobytes():
            matches.append(a)
    assert matches == [O.default_arith()]


@pytest.mark.parametrize("i", range(n_cases(MC, "band")))
def test_band_bit_exact(i):
    lab, nf, iso, lo, hi, vs, gc = band_case(MC, i)
    verts, occ, _ = O.mc_classify(lab, iso)
    assert np.array_equal(verts, MC[f"sm103a/band{i}/verts"])
    pos, norm, _ = O.mesh_band(lab, nf, vs, gc, iso, lo, hi)
    assert pos.tobytes() == MC[f"sm103a/band{i}/pos"].tobytes()
    assert norm.tobytes() == MC[f"sm103a/band{i}/norm"].tobytes()
    # the two-field kernel the lattice path calls gives the same mesh
    assert MC[f"sm103a/band{i}/pos_new"].tobytes() == MC[f"sm103a/band{i}/pos"].tobytes()


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "unit")))
def test_unit_cell(i):
    nx, ny, nz, t = (int(v) for v in FIELDS[f"in/unit{i}"])
    assert_field_close(O.unit_cell(t, nx, ny, nz), FIELDS[f"sm103a/unit{i}"])


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "prim")))
def test_primitive(i):
    q = FIELDS[f"in/prim{i}"]
    n = tuple(int(v) for v in q[:3])
    got = O.primitive(int(q[6]), n, q[3:6], q[8:11], q[11:14], q[14:20], int(q[7]))
    # The cylinder's distance to its axis is |w1 x w2| / |w3| (src/Modelling.cu:
    # 276-281): its rounding scales with |w1||w2|, about the square of the grid
    # extent, so it gets a wider absolute term than the other primitives.
    k_scale = 32 if int(q[6]) == 1 else 8
    assert_field_close(got, FIELDS[f"sm103a/prim{i}"], k_scale=k_scale)


@pytest.mark.parametrize("i", range(n_cases(FIELDS, "norm")))
def test_normalise_band_bit_exact(i):
    P = FIELDS[f"in/norm{i}/params"]
    nx, ny, nz = (int(v) for v in P[:3])
    f = FIELDS[f"in/norm{i}/field"].reshape(nz, ny, nx)
    lab, nf, mm = O.normalise_band(f, float(np.float32(P[3])), float(np.float32(P[4])))
    assert np.array_equal(mm, FIELDS[f"sm103a/norm{i}/minmax"])
    assert np.array_equal(lab.reshape(-1), FIELDS[f"sm103a/norm{i}/label"])
    assert np.array_equal(nf.reshape(-1), FIELDS[f"sm103a/norm{i}/normf"])
