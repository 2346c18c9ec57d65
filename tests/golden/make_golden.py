"""Generates the golden fixtures of this directory by running the reference's own
CUDA kernels on seeded inputs.

Run on a machine with a GPU, after ``oracle/ref/build_ref.py`` has produced the
reference fatbins in ``oracle/_ref/`` (that step needs the reference sources; this
one does not):

    python tests/golden/make_golden.py --out <dir>

It builds ``oracle/_ref/ref_runner`` from ``oracle/ref/ref_runner.cpp`` (this
project's driver-API program), runs every job once per reference build variant
(``sm103a``: compiled for the GB300; ``ptx89``: the reference Makefile's PTX-only
form, JIT-compiled by the driver), checks that both variants agree, and writes

Only the sm103a outputs are stored (keys ``sm103a/...``); the script refuses to
write fixtures if the two variants differ anywhere (``variant_report.txt``).

* ``golden_mc.npz``     - plain and band marching cubes: inputs, per-voxel counts,
  occupancy, both scans, compaction, vertex and normal buffers;
* ``golden_fields.npz`` - TPMS unit cells, primitive fields, band normalisation.

All inputs are deterministic (numpy default_rng with fixed seeds).
"""
from __future__ import annotations

import argparse
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_DIR = os.path.join(REPO, "oracle", "_ref")
TABLES = os.path.join(HERE, "ref_tables.bin")
MAGIC = 0x4A4D4347

# ---------------------------------------------------------------- inputs


def _gyroid(n, k, shift):
    z, y, x = np.meshgrid(*(np.arange(m, dtype=np.float64) for m in n[::-1]), indexing="ij")
    x, y, z = x + shift[0], y + shift[1], z + shift[2]
    g = np.sin(k * x) * np.cos(k * y) + np.sin(k * y) * np.cos(k * z) + np.sin(k * z) * np.cos(k * x)
    return g


def plain_cases():
    """Strictly positive fields (the reference generate kernel's own cube index
    additionally requires f > 0), isovalues inside their range."""
    rng = np.random.default_rng(0xD4A1)
    cases = []
    n = (12, 10, 9)
    cases.append(dict(name="random", n=n, iso=1.0, vs=(1.0, 1.0, 1.0), gc=(0.0, 0.0, 0.0),
                      field=rng.uniform(0.5, 1.5, n[::-1]).astype(np.float32)))
    n = (34, 30, 28)
    cases.append(dict(name="gyroid_h127", n=n, iso=2.0, vs=(1 / 127,) * 3, gc=(0.0, 0.0, 0.0),
                      field=(2.0 + _gyroid(n, 2 * np.pi / 12, (0.3, 0.1, 0.7))).astype(np.float32)))
    n = (16, 15, 14)
    levels = np.array([0.5, 0.75, 1.0, 1.25, 1.5], np.float32)
    f = levels[rng.integers(0, 5, n[::-1])]
    near = rng.random(n[::-1]) < 0.15
    f = np.where(near, np.nextafter(np.float32(1.0), np.float32(2.0 * rng.integers(0, 2, n[::-1]))), f)
    cases.append(dict(name="exact_iso", n=n, iso=1.0, vs=(0.5, 0.5, 0.5), gc=(3.0, 2.0, 1.0),
                      field=f.astype(np.float32)))
    n = (22, 21, 20)
    f = np.where(rng.random(n[::-1]) < 0.5, 0.6, 1.4) + rng.uniform(-0.3, 0.3, n[::-1])
    cases.append(dict(name="all_cases", n=n, iso=1.0, vs=(0.37, 1.3, 0.011), gc=(0.5, -2.25, 7.0),
                      field=f.astype(np.float32)))
    n = (40, 36, 44)
    cases.append(dict(name="gyroid_unit", n=n, iso=1.85, vs=(1.0, 1.0, 1.0), gc=(0.0, 0.0, 0.0),
                      field=(2.0 + _gyroid(n, 2 * np.pi / 32, (0.0, 0.0, 0.0))).astype(np.float32)))
    n = (30, 26, 22)
    cases.append(dict(name="gyroid_odd_vs", n=n, iso=2.1, vs=(0.0173, 0.0291, 0.2113), gc=(1.5, 0.25, 3.0),
                      field=(2.0 + _gyroid(n, 2 * np.pi / 9, (0.5, 0.25, 0.125))).astype(np.float32)))
    return cases


def band_cases():
    """Label + normalised field as GPU_buffer_normalise_four makes them
    (src/lattice_files/Gratings.cu:1089-1134), computed here in numpy."""
    cases = []
    for name, n, k, lo, hi, vs in (("band_gyroid", (32, 16, 24), 2 * np.pi / 10, 0.2, 0.3, (1.0, 1.0, 1.0)),
                                   ("band_wide", (24, 20, 18), 2 * np.pi / 7, 0.35, 0.65, (0.5, 0.5, 0.5))):
        g = _gyroid(n, k, (0.2, 0.4, 0.1)).astype(np.float32)
        a, b = min(np.float32(0), g.min()), max(np.float32(0), g.max())
        kf = ((g - a) / (b - a)).astype(np.float32)
        lab = ((kf >= np.float32(lo)) & (kf <= np.float32(hi))).astype(np.float32)
        edge = np.zeros(g.shape, bool)
        edge[0, :, :] = edge[-1, :, :] = edge[:, 0, :] = edge[:, -1, :] = edge[:, :, 0] = edge[:, :, -1] = True
        lab[edge] = 0
        kf[edge] = 0
        cases.append(dict(name=name, n=n, iso=0.25 if name == "band_gyroid" else 0.5, lo=lo, hi=hi, vs=vs,
                          gc=(0.0, 0.0, 0.0), label=lab, normf=kf))
    return cases


UNIT_SIZES = [(32, 16, 24), (48, 24, 16)]

# (kind, flag, center, v3, p)  - grid units of the primitive's own frame
PRIMS = [
    (0, 0, (0.3, -0.2, 0.1), (0, 0, 0), (3.1, 0.0)),
    (0, 1, (0.0, 0.4, -0.3), (0, 0, 0), (3.4, 1.2)),
    (1, 0, (0.2, 0.1, 0.0), (0.3, 0.2, 1.0), (2.2, 0.0, 4.5)),
    (1, 1, (0.0, 0.0, 0.3), (1.0, 0.0, 0.2), (2.6, 0.9, 3.0)),
    (2, 0, (0.1, -0.3, 0.2), (0.3, -0.2, 0.5), (4.0, 3.0, 2.5)),
    (3, 0, (0.0, 0.2, 0.0), (0.1, 0.4, -0.3), (5.0, 4.2, 3.3, 0.8)),
    (4, 0, (0.2, 0.0, -0.1), (0.5, 0.1, 0.0), (3.2, 1.1)),
    (5, 0, (0.0, -1.0, 0.2), (0.0, 0.0, 0.3), (2.4, 4.0)),
    (6, 0, (0.1, -1.2, 0.0), (0.2, 0.0, 0.1), (1.2, 2.8, 3.6)),
    (7, 0, (0.0, -1.0, 0.1), (0.0, 0.3, 0.0), (5.0, 2.0, 3.5, 4.4, 1.6)),
]
PRIM_GRIDS = [((24, 20, 16), (0.5, 0.5, 0.5)), ((17, 19, 21), (0.43, 0.37, 0.51))]

NORM_CASES = [("norm_gyroid", (32, 16, 24), 0.2, 0.3, 0.0), ("norm_positive", (16, 16, 8), 0.4, 0.6, 3.0)]


def _p(fmt, *v):
    return struct.pack("<" + fmt, *v)


def build_job():
    parts = []
    meta = []
    for c in plain_cases():
        parts.append(_p("I", 1) + _p("3I", *c["n"]) + _p("f", c["iso"]) + _p("3f", *c["vs"]) + _p("3f", *c["gc"])
                     + c["field"].astype("<f4").tobytes())
        meta.append(("plain", c))
    for c in band_cases():
        parts.append(_p("I", 2) + _p("3I", *c["n"]) + _p("3f", c["iso"], c["lo"], c["hi"]) + _p("3f", *c["vs"])
                     + _p("3f", *c["gc"]) + c["label"].astype("<f4").tobytes() + c["normf"].astype("<f4").tobytes())
        meta.append(("band", c))
    for n in UNIT_SIZES:
        for t in range(6):
            parts.append(_p("I", 3) + _p("4I", *n, t))
            meta.append(("unit", dict(n=n, type=t)))
    for gi, (n, d) in enumerate(PRIM_GRIDS):
        for pi, (kind, flag, center, v3, p) in enumerate(PRIMS):
            pp = list(p) + [0.0] * (6 - len(p))
            parts.append(_p("I", 4) + _p("I", kind) + _p("3i", *n) + _p("3f", *d) + _p("3f", *center)
                         + _p("3f", *v3) + _p("6f", *pp) + _p("I", flag))
            meta.append(("prim", dict(n=n, d=d, kind=kind, flag=flag, center=center, v3=v3, p=pp, grid=gi, idx=pi)))
    for name, n, lo, hi, off in NORM_CASES:
        g = (_gyroid(n, 2 * np.pi / 8, (0.1, 0.2, 0.3)) + off).astype(np.float32)
        parts.append(_p("I", 5) + _p("3i", *n) + _p("2f", lo, hi) + g.astype("<f4").tobytes())
        meta.append(("norm", dict(name=name, n=n, lo=lo, hi=hi, field=g)))
    blob = _p("I", MAGIC) + _p("I", len(parts)) + b"".join(parts)
    return blob, meta


# ---------------------------------------------------------------- outputs


class Buf:
    def __init__(self, b):
        self.b, self.o = b, 0

    def u32(self, n=None):
        return self.arr(np.uint32, n)

    def f32(self, n=None):
        return self.arr(np.float32, n)

    def arr(self, dt, n):
        k = 1 if n is None else n
        a = np.frombuffer(self.b, dtype=np.dtype(dt).newbyteorder("<"), count=k, offset=self.o).copy()
        self.o += a.nbytes
        return a[0] if n is None else a


def parse(out_bytes, meta):
    B = Buf(out_bytes)
    res = []
    for kind_name, c in meta:
        kind = int(B.u32())
        r = dict(meta=c, kind=kind_name)
        if kind in (1, 2):
            nvox, act, tot = int(B.u32()), int(B.u32()), int(B.u32())
            r.update(nvox=nvox, active=act, total=tot, verts=B.u32(nvox), occ=B.u32(nvox), occ_scan=B.u32(nvox),
                     verts_scan=B.u32(nvox), compacted=B.u32(act))
            r["pos"] = B.f32(4 * tot).reshape(-1, 4)
            r["norm"] = B.f32(4 * tot).reshape(-1, 4)
            if kind == 2:
                r["pos_new"] = B.f32(4 * tot).reshape(-1, 4)
                r["norm_new"] = B.f32(4 * tot).reshape(-1, 4)
        elif kind in (3, 4):
            n = c["n"]
            r["field"] = B.f32(n[0] * n[1] * n[2])
        elif kind == 5:
            n = c["n"]
            r["minmax"] = B.f32(2)
            r["label"] = B.f32(n[0] * n[1] * n[2])
            r["normf"] = B.f32(n[0] * n[1] * n[2])
        res.append(r)
    assert B.o == len(out_bytes), (B.o, len(out_bytes))
    return res


def build_runner():
    exe = os.path.join(REF_DIR, "ref_runner")
    src = os.path.join(REPO, "oracle", "ref", "ref_runner.cpp")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", src, "-I", os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64"),
           "-L", os.path.join(cuda, "lib64", "stubs"), "-lcuda", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def same(a, b):
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    exe = build_runner()
    blob, meta = build_job()
    job = os.path.join(args.out, "job.bin")
    with open(job, "wb") as f:
        f.write(blob)
    results = {}
    for var in ("sm103a", "ptx89"):
        out = os.path.join(args.out, f"out_{var}.bin")
        subprocess.run([exe, REF_DIR, var, TABLES, job, out], check=True)
        with open(out, "rb") as f:
            results[var] = parse(f.read(), meta)
    # Variant agreement report.
    report = []
    for i, (a, b) in enumerate(zip(results["sm103a"], results["ptx89"])):
        keys = [k for k in a if isinstance(a[k], np.ndarray)]
        diff = [k for k in keys if not same(a[k], b[k])]
        report.append(f"{i:3d} {a['kind']:6s} {a['meta'].get('name', '')!s:14s} differs: {diff}")
    with open(os.path.join(args.out, "variant_report.txt"), "w") as f:
        f.write("\n".join(report) + "\n")
    print("\n".join(report))
    # Only one copy is kept: both variants must agree bit for bit.
    mismatches = [line for line in report if not line.endswith("differs: []")]
    if mismatches:
        print("reference build variants disagree; fixtures not written", file=sys.stderr)
        return 1
    save({"sm103a": results["sm103a"]}, args.out)
    return 0


def save(results, out):
    mc, fields = {}, {}
    for var, res in results.items():
        pi = bi = ui = qi = ni = 0
        for r in res:
            c = r["meta"]
            if r["kind"] == "plain":
                pre = f"{var}/plain{pi}/"
                pi += 1
                if var == "sm103a":
                    mc[pre.replace(var, "in") + "field"] = c["field"]
                    mc[pre.replace(var, "in") + "params"] = np.array(
                        [*c["n"], c["iso"], *c["vs"], *c["gc"]], np.float64)
                for k in ("verts", "occ", "occ_scan", "verts_scan", "compacted", "pos", "norm"):
                    mc[pre + k] = r[k]
            elif r["kind"] == "band":
                pre = f"{var}/band{bi}/"
                bi += 1
                if var == "sm103a":
                    mc[pre.replace(var, "in") + "label"] = c["label"]
                    mc[pre.replace(var, "in") + "normf"] = c["normf"]
                    mc[pre.replace(var, "in") + "params"] = np.array(
                        [*c["n"], c["iso"], c["lo"], c["hi"], *c["vs"], *c["gc"]], np.float64)
                for k in ("verts", "occ", "occ_scan", "verts_scan", "compacted", "pos", "norm", "pos_new", "norm_new"):
                    mc[pre + k] = r[k]
            elif r["kind"] == "unit":
                fields[f"{var}/unit{ui}"] = r["field"]
                if var == "sm103a":
                    fields[f"in/unit{ui}"] = np.array([*c["n"], c["type"]], np.int64)
                ui += 1
            elif r["kind"] == "prim":
                fields[f"{var}/prim{qi}"] = r["field"]
                if var == "sm103a":
                    fields[f"in/prim{qi}"] = np.array([*c["n"], *c["d"], c["kind"], c["flag"], *c["center"],
                                                       *c["v3"], *c["p"]], np.float64)
                qi += 1
            elif r["kind"] == "norm":
                fields[f"{var}/norm{ni}/minmax"] = r["minmax"]
                fields[f"{var}/norm{ni}/label"] = r["label"]
                fields[f"{var}/norm{ni}/normf"] = r["normf"]
                if var == "sm103a":
                    fields[f"in/norm{ni}/field"] = c["field"]
                    fields[f"in/norm{ni}/params"] = np.array([*c["n"], c["lo"], c["hi"]], np.float64)
                ni += 1
    np.savez_compressed(os.path.join(out, "golden_mc.npz"), **mc)
    np.savez_compressed(os.path.join(out, "golden_fields.npz"), **fields)
    print("saved", out)


if __name__ == "__main__":
    sys.exit(main())
