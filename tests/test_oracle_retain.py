"""The oracle's retained primitive editing against the reference's own kernels
(tests/golden/golden_retain.npz, made by tests/golden/make_golden_retain.py):
the accumulator after every fold sequence, and the region and live-model meshes,
bit for bit."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import golden

R = golden("golden_retain.npz")
NAMES = {"union": 0, "subtract": 1, "intersect": 2}
OPS = {v: k for k, v in NAMES.items()}


def n_cases():
    return len({k.split("/")[0] for k in R.files})


def case(i):
    pre = f"case{i}/"
    p = R[pre + "params"]
    n = tuple(int(v) for v in p[:3])
    iso, vs, gc, mode, pop = float(p[3]), tuple(p[4:7]), tuple(p[7:10]), int(p[10]), int(p[11])
    bands = R[pre + "fold_band"] if pre + "fold_band" in R.files else np.zeros((len(R[pre + "fold_ops"]), 3))
    # (op, field, band): band (iso1, iso2) for a lattice-band fold, else None
    folds = [(op, f, (float(b[1]), float(b[2])) if b[0] else None)
             for op, f, b in zip(R[pre + "fold_ops"], R[pre + "fold_fields"], bands)]
    pf = R[pre + "preview_field"] if pre + "preview_field" in R.files else None
    return pre, n, iso, vs, gc, folds, pf, OPS[pop]


def preview(i):
    """(mode, lattice, band): mode 0 region, 1 primitive preview, 2 lattice
    "fixed", 3 lattice "dynamic"; lattice and band for modes 2 and 3."""
    pre = f"case{i}/"
    mode = int(R[pre + "params"][10])
    if mode >= 2:
        return mode, R[pre + "lattice"], tuple(float(v) for v in R[pre + "lattice_band"])
    return mode, None, None


@pytest.mark.parametrize("i", range(n_cases()))
def test_accumulator_bit_exact(i):
    pre, n, iso, vs, gc, folds, pf, pop = case(i)
    acc = O.csg_accumulator(n[::-1])
    for op, f, band in folds:
        O.csg_retain(acc, f, OPS[int(op)], iso, band=band)
    assert acc.tobytes() == R[pre + "acc"].tobytes()


def test_fixtures_hold_band_folds_and_lattice_previews():
    assert any(b is not None for i in range(n_cases()) for _, _, b in case(i)[5])
    assert {preview(i)[0] for i in range(n_cases())} == {0, 1, 2, 3}


@pytest.mark.parametrize("i", range(n_cases()))
def test_mesh_bit_exact(i):
    pre, n, iso, vs, gc, folds, pf, pop = case(i)
    acc = R[pre + "acc"].copy()
    mode, lat, band = preview(i)
    if mode >= 2:
        pos, norm, active = O.mesh_lattice_preview(acc, pf if mode == 2 else None, lat, band, pop, vs, gc, iso)
    else:
        pos, norm, active = O.mesh_retained(acc, pf, pop, vs, gc, iso)
    assert active == len(R[pre + "compacted"])
    assert pos.tobytes() == R[pre + "pos"].tobytes()
    assert norm.tobytes() == R[pre + "norm"].tobytes()
