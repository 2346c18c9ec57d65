"""The oracle's spatially variant lattice against the reference's own kernels
(tests/golden/golden_svl.npz, made by tests/golden/make_golden_svl.py).

Bit for bit: the conjugate-gradient solves given the reference's right-hand
sides (phases and step counts), and the right-hand sides themselves where no
trigonometric function enters (kind 'n').  Within tolerance: right-hand sides
of the rotated kinds (the host's atan2f/sinf/cosf against CUDA's, 1-2 ulp of
the angle amplified by the frequency, bounded by 2e-4 relative here) and the
lattice (the reference filters through the texture unit: 8 fractional weight
bits and its own arithmetic; bounded by 2e-6 absolute)."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import golden

G = golden("golden_svl.npz")
NCASE = len({k.split("/")[0] for k in G.files if k.startswith("case")})


def case(i):
    pre = f"case{i}/"
    p = G[pre + "params"]
    n = tuple(int(v) for v in p[:3])
    kind = chr(int(p[3]))
    prm = O.svl_params(n, kind, int(p[4]), float(p[5]), tuple(p[6:9]), lcon=float(p[9]), lcon_1=float(p[10]),
                       sinewave_z=bool(p[11]), n_coeff=int(p[12]))
    per = G[pre + "period_field"] if int(p[4]) == 2 else None
    return pre, prm, kind, per


def test_dft_symmetry_and_mean():
    u = O.unit_cell(0, 21, 21, 21).reshape(21, 21, 21)
    c = O.svl_dft(u, 2)
    w = 5
    for m in range(w ** 3):
        i, j, k = m % w - 2, (m // w) % w - 2, m // (w * w) - 2
        mc = (-i + 2) + w * ((-j + 2) + w * (-k + 2))
        assert abs(c[m, 0] - c[mc, 0]) < 1e-7 and abs(c[m, 1] + c[mc, 1]) < 1e-7
    assert abs(c[62, 0] - float(np.mean(u.astype(np.float64)))) < 1e-7 and abs(c[62, 1]) < 1e-7
    assert np.array_equal(c, G["coef"])


@pytest.mark.parametrize("i", range(NCASE))
def test_rhs(i):
    pre, p, kind, per = case(i)
    for m, ref in zip(G[pre + "keep"], G[pre + "rhs"]):
        got = O.svl_rhs(p, int(m), per)
        if kind == "n":
            assert got.tobytes() == ref.tobytes(), m
        else:
            assert np.allclose(got, ref, rtol=2e-4, atol=2e-4 * float(np.abs(ref).max())), m


@pytest.mark.parametrize("i", range(NCASE))
def test_cg_bit_exact_from_reference_rhs(i):
    pre, p, kind, per = case(i)
    for m, rhs, ref, it in zip(G[pre + "keep"], G[pre + "rhs"], G[pre + "phase"], G[pre + "iters"][G[pre + "keep"]]):
        x, got_it = O.svl_cg(p, rhs)
        assert got_it == it, m
        assert x.tobytes() == ref.tobytes(), m


@pytest.mark.parametrize("i", [k for k in range(NCASE) if chr(int(golden("golden_svl.npz")[f"case{k}/params"][3])) == "n"])
def test_lattice_within_texture_tolerance(i):
    pre, p, kind, per = case(i)
    svl, _, iters = O.svl_lattice(p, G["coef"], per)
    assert iters == list(G[pre + "iters"])
    assert float(np.abs(svl - G[pre + "svl"]).max()) < 2e-6
