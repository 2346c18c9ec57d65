"""CPU checks of the graded-lattice arithmetic.

The oracle's float restatement of the kernels' compensated arithmetic stays
within 1e-5 relative (|f - f64| <= 1e-5 * max(1, |f64|)) of the FP64 oracle in
both grading modes, on plane pairs of 512^3 grids (corner, centre, top: the
largest and smallest phases) and on the headline configuration itself; the
angle table header is what its generator writes.
"""
import importlib.util
import os

import numpy as np
import pytest

import oracle as O
from bench import N_CTRL, c2_controls
from tests.helpers import assert_rel_close

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _controls(seed, C, types=(0, 1, 2, 3, 5)):
    rng = np.random.default_rng(seed)
    n = C ** 3
    return (rng.uniform(16, 64, n).astype(np.float32), rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32),
            rng.uniform(-0.6, 0.6, n).astype(np.float32), rng.choice(np.array(types, np.uint8), n))


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("n,C", [(512, 8), (512, 16), (300, 3), (96, 8)])
def test_compensated_field_vs_fp64(mode, n, C):
    P, E, T, Ty = _controls(5 + n + C, C)
    origin = ((n - 1) / 2,) * 3
    for z0 in (0, n // 2, n - 2):
        a = O.lattice_slab((n, n, n), z0, 2, mode, (C,) * 3, P, E, T, Ty, origin)
        b = O.lattice_slab((n, n, n), z0, 2, mode, (C,) * 3, P, E, T, Ty, origin, fp64=True)
        assert_rel_close(a, b, 1e-5)


def test_headline_field_vs_fp64():
    n = 512
    period, euler, thick, types = c2_controls()
    origin = ((n - 1) / 2,) * 3
    for z0 in (0, 255, 510):
        a = O.lattice_slab((n, n, n), z0, 2, 0, (N_CTRL,) * 3, period, euler, thick, types, origin)
        b = O.lattice_slab((n, n, n), z0, 2, 0, (N_CTRL,) * 3, period, euler, thick, types, origin, fp64=True)
        assert_rel_close(a, b, 1e-5)


def test_wide_angles_vs_fp64():
    """Angles beyond the table's [-3.156, 3.156] take the double reduction."""
    rng = np.random.default_rng(3)
    C, n = 4, 64
    nc = C ** 3
    P = rng.uniform(16, 64, nc).astype(np.float32)
    E = rng.uniform(-40.0, 40.0, 3 * nc).astype(np.float32)
    T = rng.uniform(-0.6, 0.6, nc).astype(np.float32)
    Ty = rng.choice(np.array([0, 1, 5], np.uint8), nc)
    for mode in (0, 1):
        a = O.lattice_field((n, n, n), mode, (C,) * 3, P, E, T, Ty, ((n - 1) / 2,) * 3)
        b = O.lattice_field((n, n, n), mode, (C,) * 3, P, E, T, Ty, ((n - 1) / 2,) * 3, fp64=True)
        assert_rel_close(a, b, 1e-5)


def test_angle_table_header_is_generated():
    path = os.path.join(REPO, "gpucadforam_gb300", "csrc", "make_angle_table.py")
    spec = importlib.util.spec_from_file_location("make_angle_table", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    with open(mod.HEADER) as f:
        assert f.read() == mod.render()
