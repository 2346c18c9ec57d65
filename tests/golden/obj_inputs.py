"""Deterministic vertex buffers for the .obj writer fixtures and tests.

Marching-cubes meshes from golden_mc.npz plus adversarial buffers: positions
on a coarse lattice (many vertices weld together, many faces degenerate or
repeated), negative coordinates (truncation toward zero), coordinates near the
weld key limit, and an empty buffer.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _pos(xyz):
    n = xyz.shape[0]
    out = np.zeros((n, 4), np.float32)
    out[:, :3] = xyz
    out[:, 3] = 1.0
    return out


def cases():
    d = np.load(os.path.join(HERE, "golden_mc.npz"))
    out = []
    for k in sorted(k for k in d.files if k.startswith("sm103a/") and k.endswith("/pos")):
        out.append((k.split("/")[1], np.ascontiguousarray(d[k], np.float32)))
    rng = np.random.default_rng(0xD4A0B7)
    # coarse lattice + sub-quantum noise: heavy welding, degenerate faces
    xyz = rng.integers(-20, 21, (3 * 4000, 3)) * 0.05 + rng.uniform(0, 0.0009, (3 * 4000, 3))
    p = _pos(xyz.astype(np.float32))
    tri = p.reshape(-1, 3, 4)
    idx = rng.integers(0, tri.shape[0], 600)
    tri[rng.integers(0, tri.shape[0], 600)] = tri[idx]  # repeated identical faces
    out.append(("lattice_dups", np.ascontiguousarray(tri.reshape(-1, 4))))
    out.append(("negative", _pos(rng.uniform(-3, 3, (3 * 5000, 3)).astype(np.float32))))
    out.append(("near_limit", _pos(rng.uniform(-1048.0, 1048.0, (3 * 3000, 3)).astype(np.float32))))
    out.append(("empty", np.zeros((0, 4), np.float32)))
    return out
