"""Fixtures of the reference's spatially variant lattice, from its own kernels.

Run on a machine with a GPU after ``oracle/ref/build_ref.py`` has produced the
reference fatbins in ``oracle/_ref/``:

    python tests/golden/make_golden_svl.py --out <dir>

Each case runs job kind 8 of oracle/ref/ref_runner.cpp: for each of the first n
Fourier coefficients of a gyroid unit cell (coefficients from the oracle's DFT,
an input, since the reference takes them from cuFFT) the reference's
finding_phi_kernel, its GPUCG_lattice loop with its kernels, its texture
upsampling (grating_kernel) and accumulation (svl_kernel), on grids whose
sizes are multiples of those kernels' block shapes.  Both reference build
variants must agree bit for bit; ``golden_svl.npz`` keeps, per case, the inputs,
the right-hand sides and phases of a few coefficients, every solve's step count
and the accumulated lattice.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import make_golden as MG  # noqa: E402

KEEP = (0, 7, 31, 61)  # coefficients whose right-hand side and phase are stored


def coefficients():
    import oracle as O

    u = O.unit_cell(0, 21, 21, 21).reshape(21, 21, 21)
    return O.svl_dft(u, 2)


def cases():
    rng = np.random.default_rng(0xD4A8)
    out = [
        dict(name="plain_const", n=(16, 8, 8), kind="n", ptype=0, period=8.0, periods=(8.0, 8.0, 8.0), nc=62),
        dict(name="plain_axes", n=(8, 8, 16), kind="n", ptype=1, period=8.0, periods=(6.0, 9.0, 7.0), nc=62),
        dict(name="round", n=(16, 16, 8), kind="r", ptype=0, period=7.0, periods=(8.0, 8.0, 8.0), nc=32),
        dict(name="bend_field", n=(16, 8, 8), kind="b", ptype=2, period=8.0, periods=(8.0, 8.0, 8.0), nc=32),
        dict(name="sine_z", n=(16, 8, 8), kind="s", ptype=0, period=9.0, periods=(8.0, 8.0, 8.0), nc=32,
             lcon=0.3, lcon_1=0.05, sinez=1),
    ]
    for c in out:
        nx, ny, nz = c["n"]
        c["field"] = (rng.uniform(6.0, 12.0, nx * ny * nz).astype(np.float32) if c["ptype"] == 2
                      else np.zeros(nx * ny * nz, np.float32))
    return out


def build_job(coef):
    parts, meta = [], []
    for c in cases():
        nx, ny, nz = c["n"]
        b = MG._p("I", 8) + MG._p("3i", nx, ny, nz) + MG._p("3f", 1.0, 1.0, 1.0) + MG._p("I", ord(c["kind"]))
        b += MG._p("i", c["ptype"]) + MG._p("4f", c["period"], *c["periods"])
        b += MG._p("2f", c.get("lcon", 0.0), c.get("lcon_1", 0.0)) + MG._p("I", c.get("sinez", 0))
        b += MG._p("i", 2) + MG._p("2I", c["nc"], 500) + MG._p("f", 0.01)
        b += c["field"].astype("<f4").tobytes() + coef.astype("<f4").tobytes()
        parts.append(b)
        meta.append(c)
    return MG._p("I", MG.MAGIC) + MG._p("I", len(parts)) + b"".join(parts), meta


def parse(blob, meta):
    B = MG.Buf(blob)
    res = []
    for c in meta:
        assert int(B.u32()) == 8
        P = c["n"][0] * c["n"][1] * c["n"][2]
        rhs, phase, iters = [], [], []
        for _ in range(c["nc"]):
            rhs.append(B.f32(P))
            phase.append(B.f32(P))
            iters.append(int(B.u32()))
        r = dict(meta=c, rhs=np.stack(rhs), phase=np.stack(phase), iters=np.array(iters, np.int32),
                 svl=B.f32(8 * P))
        res.append(r)
    assert B.o == len(blob)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    exe = MG.build_runner()
    coef = coefficients()
    blob, meta = build_job(coef)
    job = os.path.join(args.out, "job_svl.bin")
    with open(job, "wb") as f:
        f.write(blob)
    results = {}
    for var in ("sm103a", "ptx89"):
        out = os.path.join(args.out, f"out_svl_{var}.bin")
        subprocess.run([exe, MG.REF_DIR, var, MG.TABLES, job, out], check=True)
        with open(out, "rb") as f:
            results[var] = parse(f.read(), meta)
    bad = [f"{a['meta']['name']}: {k}" for a, b in zip(results["sm103a"], results["ptx89"])
           for k in ("rhs", "phase", "iters", "svl") if a[k].tobytes() != b[k].tobytes()]
    print("variant differences:", bad or "none")
    if bad:
        return 1
    d = {"coef": coef}
    for i, r in enumerate(results["sm103a"]):
        c = r["meta"]
        pre = f"case{i}/"
        d[pre + "name"] = np.array(c["name"])
        d[pre + "params"] = np.array([*c["n"], ord(c["kind"]), c["ptype"], c["period"], *c["periods"],
                                      c.get("lcon", 0.0), c.get("lcon_1", 0.0), c.get("sinez", 0), c["nc"]],
                                     np.float64)
        d[pre + "period_field"] = c["field"]
        keep = [m for m in KEEP if m < c["nc"]]
        d[pre + "keep"] = np.array(keep, np.int32)
        d[pre + "rhs"] = r["rhs"][keep]
        d[pre + "phase"] = r["phase"][keep]
        d[pre + "iters"] = r["iters"]
        d[pre + "svl"] = r["svl"]
    np.savez_compressed(os.path.join(args.out, "golden_svl.npz"), **d)
    print("wrote", os.path.join(args.out, "golden_svl.npz"), len(meta), "cases")
    return 0


if __name__ == "__main__":
    sys.exit(main())
