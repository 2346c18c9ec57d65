"""Fixtures of the reference's retained primitive editing, from its own kernels.

Run on a machine with a GPU after ``oracle/ref/build_ref.py`` has produced the
reference fatbins in ``oracle/_ref/``:

    python tests/golden/make_golden_retain.py --out <dir>

Each case folds a seeded sequence of primitive fields into a zeroed
grid_points accumulator with the reference's classify_copy_Voxel
(src/MarchingCubes_kernel.cu:158-447) and meshes it with its classifyVoxel,
compactVoxels and generateTriangles_lattice_kernel (:869-1052, :1594-1608,
:1865-2200), in the region mode or with one more primitive field (job kind 10
of oracle/ref/ref_runner.cpp).  A fold is static (the field is the object) or
a lattice band (classify_copy_Voxel's dynamic mode: the open band
iso1 < field < iso2 is the object).  Meshes: the region (mode 0), the model
with one more primitive field (mode 1), and the lattice previews of
classifyVoxel / generateTriangles_lattice_kernel with `fixed` (mode 2: a
primitive field with the lattice band) or `dynamic` (mode 3: the model with
the lattice band) set.  Both reference build variants (sm103a SASS and
the Makefile's compute_89 PTX) must agree bit for bit; the sm103a outputs are
written to ``golden_retain.npz`` with the inputs.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

OPS = {"union": 0, "subtract": 1, "intersect": 2}


def _grid(n):
    nx, ny, nz = n
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float32), np.arange(ny, dtype=np.float32),
                          np.arange(nx, dtype=np.float32), indexing="ij")
    return x, y, z


def sphere(n, c, r):
    x, y, z = _grid(n)
    return ((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 - np.float32(r * r)).astype(np.float32)


def box(n, c, h):
    x, y, z = _grid(n)
    return np.maximum(np.maximum(np.abs(x - c[0]) - h[0], np.abs(y - c[1]) - h[1]),
                      np.abs(z - c[2]) - h[2]).astype(np.float32)


def gyroid(n, period):
    x, y, z = _grid(n)
    k = 2.0 * np.pi / period
    x, y, z = (k * x.astype(np.float64), k * y.astype(np.float64), k * z.astype(np.float64))
    return (np.sin(x) * np.cos(y) + np.sin(y) * np.cos(z) + np.sin(z) * np.cos(x)).astype(np.float32)


def cases():
    """(name, n, iso, vs, gc, folds [(op, field) or (op, field, (iso1, iso2))],
    mode, preview op, preview field)."""
    rng = np.random.default_rng(0xD4A7)
    out = []
    n = (20, 18, 16)
    a = sphere(n, (7.3, 8.1, 7.6), 4.7)
    b = box(n, (11.2, 9.4, 8.3), (3.6, 2.9, 4.1))
    c = sphere(n, (9.5, 6.2, 9.1), 3.1)
    d = sphere(n, (9.0, 9.0, 8.0), 7.9)
    e = sphere(n, (12.6, 11.3, 6.4), 3.3)
    folds = [("union", a), ("union", b), ("subtract", c)]
    out.append(("region", n, 0.0, (0.5, 0.5, 0.5), (0.0, 0.0, 0.0), folds + [("intersect", d)], 0, "union", None))
    for op in ("union", "subtract", "intersect"):
        out.append((f"preview_{op}", n, 0.0, (0.5, 0.5, 0.5), (0.0, 0.0, 0.0), folds, 1, op, e))
    # integer-valued fields: samples exactly at the isovalue, fractions of 0
    n = (14, 13, 12)
    s1 = sphere(n, (6, 6, 5), 4)
    s2 = sphere(n, (8, 7, 6), 3)
    s3 = box(n, (5, 5, 5), (3, 2, 4))
    out.append(("exact_region", n, 0.0, (1.0, 1.0, 1.0), (2.0, -1.5, 0.25),
                [("union", s1), ("union", s2), ("subtract", s3)], 0, "union", None))
    out.append(("exact_preview", n, 0.0, (0.37, 1.3, 0.011), (2.0, -1.5, 0.25), [("union", s1), ("union", s3)], 1,
                "subtract", s2))
    # random fields (every cube configuration), random ops
    n = (17, 15, 13)
    folds = [(["union", "subtract", "intersect"][int(rng.integers(0, 3))], rng.uniform(-1, 1, n[::-1]).astype(np.float32))
             for _ in range(5)]
    out.append(("random_region", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), folds, 0, "union", None))
    out.append(("random_preview", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), folds[:3], 1, "intersect",
                rng.uniform(-1, 1, n[::-1]).astype(np.float32)))
    # lattice-band folds (the dynamic mode)
    n = (24, 22, 20)
    g = gyroid(n, 10.0)
    a = sphere(n, (9.3, 10.1, 8.6), 6.2)
    c = sphere(n, (14.5, 9.2, 11.1), 4.1)
    b = box(n, (12.2, 11.4, 9.3), (5.6, 4.9, 6.1))
    e = sphere(n, (8.6, 12.3, 10.4), 4.3)
    out.append(("band_region", n, 0.0, (0.5, 0.5, 0.5), (0.0, 0.0, 0.0),
                [("union", a), ("union", g, (-0.35, 0.35)), ("subtract", c)], 0, "union", None))
    out.append(("band_diff_preview", n, 0.0, (0.5, 0.5, 0.5), (0.0, 0.0, 0.0),
                [("union", b), ("subtract", g, (-0.3, 0.3))], 1, "union", e))
    out.append(("band_intersect_region", n, 0.0, (1.0, 1.0, 1.0), (1.0, -2.0, 0.5),
                [("union", sphere(n, (12.0, 11.0, 10.0), 9.5)), ("intersect", g, (-0.5, 0.5))], 0, "union", None))
    # integer lattice values: samples exactly at the band edges, crossings onto them
    n = (14, 13, 12)
    x, y, z = _grid(n)
    gi = (np.mod(x + 2 * y + 3 * z, 5.0) - 2.0).astype(np.float32)
    out.append(("band_exact", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0),
                [("union", sphere(n, (6, 6, 5), 4)), ("union", gi, (-1.0, 1.0)), ("subtract", gi, (0.0, 2.0))], 0,
                "union", None))
    # random fields, static and band folds mixed
    n = (17, 15, 13)
    folds = []
    for k in range(6):
        op = ["union", "subtract", "intersect"][int(rng.integers(0, 3))]
        f = rng.uniform(-1, 1, n[::-1]).astype(np.float32)
        folds.append((op, f, (-0.25, 0.3)) if k % 2 else (op, f))
    out.append(("band_random_region", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), folds, 0, "union", None))
    out.append(("band_random_preview", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), folds[:4], 1, "subtract",
                rng.uniform(-1, 1, n[::-1]).astype(np.float32)))
    # lattice previews: mode 2 ("fixed": a primitive field with the lattice
    # band) and mode 3 ("dynamic": the accumulated model with the lattice band)
    n = (24, 22, 20)
    g = gyroid(n, 10.0)
    a = sphere(n, (9.3, 10.1, 8.6), 6.2)
    c = sphere(n, (14.5, 9.2, 11.1), 4.1)
    e = sphere(n, (11.6, 12.3, 10.4), 5.3)
    for op in ("union", "subtract", "intersect"):
        out.append((f"latfixed_{op}", n, 0.0, (0.5, 0.5, 0.5), (0.0, 0.0, 0.0), [("union", a)], 2, op, e, g,
                    (-0.35, 0.35)))
        out.append((f"latdyn_{op}", n, 0.0, (0.5, 0.5, 0.5), (1.0, 0.0, -0.5), [("union", a), ("subtract", c)], 3,
                    op, None, g, (-0.3, 0.3)))
    n = (14, 13, 12)
    x, y, z = _grid(n)
    gi = (np.mod(x + 2 * y + 3 * z, 5.0) - 2.0).astype(np.float32)
    s1 = sphere(n, (6, 6, 5), 4)
    out.append(("latfixed_exact", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), [("union", s1)], 2, "union",
                sphere(n, (7, 6, 6), 3), gi, (-1.0, 1.0)))
    out.append(("latdyn_exact", n, 0.0, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), [("union", s1), ("union", gi, (0.0, 2.0))],
                3, "subtract", None, gi, (-1.0, 1.0)))
    return out


def fold_band(fold):
    """(dynamic, iso1, iso2) of a fold tuple."""
    return (1, float(fold[2][0]), float(fold[2][1])) if len(fold) > 2 else (0, 0.0, 0.0)


def build_job():
    parts, meta = [], []
    for case in cases():
        name, n, iso, vs, gc, folds, mode, pop, pf = case[:9]
        lat, lband = (case[9], case[10]) if len(case) > 9 else (None, None)
        b = MG._p("I", 10) + MG._p("3I", *n) + MG._p("f", iso) + MG._p("3f", *vs) + MG._p("3f", *gc)
        b += MG._p("I", len(folds))
        for fold in folds:
            dyn, i1, i2 = fold_band(fold)
            b += MG._p("I", OPS[fold[0]]) + MG._p("I", dyn) + MG._p("2f", i1, i2) + fold[1].astype("<f4").tobytes()
        b += MG._p("2I", mode, OPS[pop])
        if mode >= 2:
            b += MG._p("2f", *lband)
        if mode in (1, 2):
            b += pf.astype("<f4").tobytes()
        if mode >= 2:
            b += lat.astype("<f4").tobytes()
        parts.append(b)
        meta.append(dict(name=name, n=n, iso=iso, vs=vs, gc=gc, folds=folds, mode=mode, pop=pop, pf=pf, lat=lat,
                         lband=lband))
    return MG._p("I", MG.MAGIC) + MG._p("I", len(parts)) + b"".join(parts), meta


def parse(blob, meta):
    B = MG.Buf(blob)
    res = []
    for c in meta:
        assert int(B.u32()) == 10
        P = c["n"][0] * c["n"][1] * c["n"][2]
        r = dict(meta=c, acc=B.arr(np.int32, 4 * P).reshape(*c["n"][::-1], 4))
        nvox, act, tot = int(B.u32()), int(B.u32()), int(B.u32())
        r.update(verts=B.u32(nvox), occ=B.u32(nvox), occ_scan=B.u32(nvox), verts_scan=B.u32(nvox),
                 compacted=B.u32(act))
        r["pos"] = B.f32(4 * tot).reshape(-1, 4)
        r["norm"] = B.f32(4 * tot).reshape(-1, 4)
        res.append(r)
    assert B.o == len(blob)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    exe = MG.build_runner()
    blob, meta = build_job()
    job = os.path.join(args.out, "job_retain.bin")
    with open(job, "wb") as f:
        f.write(blob)
    results = {}
    for var in ("sm103a", "ptx89"):
        out = os.path.join(args.out, f"out_retain_{var}.bin")
        subprocess.run([exe, MG.REF_DIR, var, MG.TABLES, job, out], check=True)
        with open(out, "rb") as f:
            results[var] = parse(f.read(), meta)
    bad = []
    for a, b in zip(results["sm103a"], results["ptx89"]):
        for k in ("acc", "verts", "occ", "compacted", "pos", "norm"):
            if a[k].tobytes() != b[k].tobytes():
                bad.append(f"{a['meta']['name']}: {k}")
    print("variant differences:", bad or "none")
    if bad:
        return 1
    d = {}
    for i, r in enumerate(results["sm103a"]):
        c = r["meta"]
        pre = f"case{i}/"
        d[pre + "params"] = np.array([*c["n"], c["iso"], *c["vs"], *c["gc"], c["mode"], OPS[c["pop"]]], np.float64)
        d[pre + "name"] = np.array(c["name"])
        d[pre + "fold_ops"] = np.array([OPS[fold[0]] for fold in c["folds"]], np.int32)
        d[pre + "fold_fields"] = np.stack([fold[1] for fold in c["folds"]])
        d[pre + "fold_band"] = np.array([fold_band(fold) for fold in c["folds"]], np.float32)
        if c["pf"] is not None:
            d[pre + "preview_field"] = c["pf"]
        if c["lat"] is not None:
            d[pre + "lattice"] = c["lat"]
            d[pre + "lattice_band"] = np.array(c["lband"], np.float32)
        for k in ("acc", "verts", "occ", "compacted", "pos", "norm"):
            d[pre + k] = r[k]
    np.savez_compressed(os.path.join(args.out, "golden_retain.npz"), **d)
    print("wrote", os.path.join(args.out, "golden_retain.npz"), len(results["sm103a"]), "cases")
    return 0


if __name__ == "__main__":
    sys.exit(main())
