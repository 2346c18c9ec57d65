"""Shared test helpers: fixture loading and tolerance checks."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def plain_case(d, i):
    """Inputs of golden plain-MC case i: (field[z,y,x], iso, vs, gc)."""
    P = d[f"in/plain{i}/params"]
    nx, ny, nz = (int(v) for v in P[:3])
    return d[f"in/plain{i}/field"].reshape(nz, ny, nx), float(np.float32(P[3])), P[4:7], P[7:10]


def band_case(d, i):
    P = d[f"in/band{i}/params"]
    nx, ny, nz = (int(v) for v in P[:3])
    iso, lo, hi = (float(np.float32(v)) for v in P[3:6])
    lab = d[f"in/band{i}/label"].reshape(nz, ny, nx)
    nf = d[f"in/band{i}/normf"].reshape(nz, ny, nx)
    return lab, nf, iso, lo, hi, P[6:9], P[9:12]


def n_cases(d, prefix):
    return len({k.split("/")[1] for k in d.files if k.startswith(f"in/{prefix}")})


def ulp32(x):
    x = np.abs(np.asarray(x, np.float32))
    return np.spacing(np.maximum(x, np.float32(np.finfo(np.float32).tiny)))


def assert_field_close(got, ref, k_rel=4, k_scale=8):
    """Field tolerance: |got - ref| <= k_rel ulp(|ref|) + k_scale ulp(max|ref|).

    The second term covers cancellation: a field that is a sum of O(S) terms
    carries O(ulp(S)) absolute rounding however small its value."""
    got = np.asarray(got, np.float32).reshape(-1)
    ref = np.asarray(ref, np.float32).reshape(-1)
    scale = np.float32(np.max(np.abs(ref))) if ref.size else np.float32(1)
    tol = k_rel * ulp32(ref) + k_scale * ulp32(scale)
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    bad = err > tol
    assert not bad.any(), (f"{bad.sum()} of {ref.size} values out of tolerance; worst err {err.max():.3e} "
                           f"at {int(err.argmax())} (ref {ref[err.argmax()]!r}, got {got[err.argmax()]!r})")


def assert_rel_close(got, ref64, rel):
    """|got - ref| <= rel * max(1, |ref|): relative to the value, with the
    field's unit scale as the floor (a field near its zero set has no
    meaningful relative error)."""
    got = np.asarray(got, np.float64).reshape(-1)
    ref64 = np.asarray(ref64, np.float64).reshape(-1)
    err = np.abs(got - ref64) / np.maximum(1.0, np.abs(ref64))
    assert err.max() <= rel, f"worst relative error {err.max():.3e} at {int(err.argmax())}"
