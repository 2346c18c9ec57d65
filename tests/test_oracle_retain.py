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
    folds = list(zip(R[pre + "fold_ops"], R[pre + "fold_fields"]))
    pf = R[pre + "preview_field"] if mode == 1 else None
    return pre, n, iso, vs, gc, folds, pf, OPS[pop]


@pytest.mark.parametrize("i", range(n_cases()))
def test_accumulator_bit_exact(i):
    pre, n, iso, vs, gc, folds, pf, pop = case(i)
    acc = O.csg_accumulator(n[::-1])
    for op, f in folds:
        O.csg_retain(acc, f, OPS[int(op)], iso)
    assert acc.tobytes() == R[pre + "acc"].tobytes()


@pytest.mark.parametrize("i", range(n_cases()))
def test_mesh_bit_exact(i):
    pre, n, iso, vs, gc, folds, pf, pop = case(i)
    acc = R[pre + "acc"].copy()
    pos, norm, active = O.mesh_retained(acc, pf, pop, vs, gc, iso)
    assert active == len(R[pre + "compacted"])
    assert pos.tobytes() == R[pre + "pos"].tobytes()
    assert norm.tobytes() == R[pre + "norm"].tobytes()
