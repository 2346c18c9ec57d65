"""CPU: the oracle's SVL period field, range map and lattice mask against the
reference's own kernels (tests/golden/golden_period_mask.npz, made by
tests/golden/make_golden_period_mask.py)."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import golden

PM = golden("golden_period_mask.npz")


def _period(i):
    P = PM[f"period{i}/params"]
    return tuple(int(v) for v in P[:3]), P[3:6], P[6:9], chr(int(P[9])), np.float32(P[10]), np.float32(P[11])


@pytest.mark.parametrize("i", range(4))
def test_period_field(i):
    n, d, mean, axis, a1, b1 = _period(i)
    got = O.svl_period_field(n, d, mean, axis).reshape(-1)
    ref = PM[f"period{i}/raw"]
    # correctly rounded squares where the reference calls powf(v, 2): at most
    # one ulp apart (none on these grids with power-of-two spacings)
    ulp = np.abs(got.view(np.int32).astype(np.int64) - ref.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1
    if all(float(v) in (0.5, 1.0) for v in d):
        assert got.tobytes() == ref.tobytes()


@pytest.mark.parametrize("i", range(4))
def test_range_map(i):
    _, _, _, _, a1, b1 = _period(i)
    out, mm = O.normalise_range(PM[f"period{i}/raw"], a1, b1)
    assert out.tobytes() == PM[f"period{i}/mapped"].tobytes()
    assert mm.tobytes() == PM[f"period{i}/minmax"].tobytes()


@pytest.mark.parametrize("i", range(6))
def test_lattice_mask(i):
    f = PM[f"mask{i}/flags"]
    out = O.lattice_mask(PM[f"mask{i}/lat"], PM[f"mask{i}/acc"], PM[f"mask{i}/prim"], f[0], f[1])
    assert out.tobytes() == PM[f"mask{i}/out"].tobytes()
