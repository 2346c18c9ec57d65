"""GPU spatially variant lattice (gcm_svl_coefficients, gcm_svl_lattice)
against the reference's own kernels (tests/golden/golden_svl.npz) and the
oracle: right-hand sides, phases and step counts bit for bit (CUDA's trig on
both sides), the lattice within the texture-filtering tolerance of the
reference (2e-6 absolute) and within the host-trig tolerance of the oracle."""
import numpy as np
import pytest
import torch

import oracle as O
from tests.helpers import golden
from tests.test_oracle_svl import NCASE, case

pytestmark = pytest.mark.gpu

G = golden("golden_svl.npz")


@pytest.fixture(scope="module")
def ctx():
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    yield c
    c.close()


def run(ctx, p, coef, per):
    d_per = None if per is None else torch.from_numpy(per).cuda()
    return ctx.svl_lattice((p.nx, p.ny, p.nz), torch.from_numpy(np.ascontiguousarray(coef)).cuda(), chr(p.kind),
                           p.period_type, p.period, (p.period_x, p.period_y, p.period_z), d_per,
                           lcon=p.lcon, lcon_1=p.lcon_1, sinewave_z=bool(p.sinewave_z), n_coeff=p.n_coeff,
                           want_phase=True)


@pytest.mark.parametrize("i", range(NCASE))
def test_svl_matches_reference(ctx, i):
    pre, p, kind, per = case(i)
    svl, iters, phase = run(ctx, p, G["coef"], per)
    assert iters == list(G[pre + "iters"])
    ph = phase.cpu().numpy().reshape(p.n_coeff, -1)
    for m, ref in zip(G[pre + "keep"], G[pre + "phase"]):
        assert ph[m].tobytes() == ref.tobytes(), m
    assert float(np.abs(svl.cpu().numpy().reshape(-1) - G[pre + "svl"]).max()) < 2e-6


def test_coefficients_match_oracle_dft(ctx):
    got = ctx.svl_coefficients(0, 21, 2).cpu().numpy()
    assert np.abs(got - G["coef"]).max() < 2e-7


@pytest.mark.parametrize("shape", [(32, 24, 16), (20, 12, 9), (9, 7, 5)])  # the last: P not a multiple of 4
def test_svl_vs_oracle(ctx, shape):
    p = O.svl_params(shape, "n", 1, 8.0, (7.0, 9.5, 6.0), n_coeff=40)
    coef = G["coef"]
    osvl, oph, oit = O.svl_lattice(p, coef)
    svl, iters, phase = run(ctx, p, coef, None)
    assert iters == oit
    assert phase.cpu().numpy().reshape(p.n_coeff, -1).tobytes() == oph.tobytes()
    assert float(np.abs(svl.cpu().numpy().reshape(-1) - osvl).max()) < 2e-6


def test_svl_accumulates_into_the_given_lattice(ctx):
    pre, p, kind, per = case(0)
    base = torch.full((2 * p.nz, 2 * p.ny, 2 * p.nx), 0.5, device="cuda")
    svl, _, _ = ctx.svl_lattice((p.nx, p.ny, p.nz), torch.from_numpy(G["coef"]).cuda(), "n", p.period_type,
                                p.period, n_coeff=p.n_coeff, svl=base.clone())
    ref, _, _ = run(ctx, p, G["coef"], per)
    assert float((svl - ref - 0.5).abs().max()) < 1e-5
