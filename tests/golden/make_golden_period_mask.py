"""Fixtures of the reference's SVL period field and lattice mask, from its own kernels.

Run on a machine with a GPU after ``oracle/ref/build_ref.py`` has produced the
reference fatbins in ``oracle/_ref/``:

    python tests/golden/make_golden_period_mask.py --out <dir>

* job kind 11 of oracle/ref/ref_runner.cpp: Gratings::period_data
  (set_period_kernel) then GPU_buffer_normalise_three in place, as the round
  lattice of src/main.cu:3929-3931 calls them, on grids that fill whole
  1024-thread blocks (set_period_kernel synchronises inside its bounds test);
* job kind 12: Gratings::primitive_field (primitive_field_kernel) in its fixed,
  dynamic and combined forms, on accumulators with every sign and primitive
  fields with exact zeros and NaNs.

The two reference build forms (sm_103a and the PTX-only compute_89 form the
driver compiles) agree on the masks; on period fields with spacings other than
powers of two they can fuse differently, so ``golden_period_mask.npz`` keeps
the inputs and the sm_103a outputs and lists those cases in
``variant_differs``.
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


def period_cases():
    # (n, spacing, mean, axis, range_lo, range_span); the reference's round
    # lattice: mean N/2.0, range N/10 and N/4 in integer division
    return [
        dict(name="round_z16", n=(16, 16, 16), d=(1.0, 1.0, 1.0), mean=(8.0, 8.0, 8.0), axis="z", a1=1.0, b1=4.0),
        dict(name="round_y", n=(32, 16, 8), d=(0.5, 0.5, 0.5), mean=(16.0, 8.0, 4.0), axis="y", a1=3.0, b1=8.0),
        dict(name="plain_x", n=(16, 8, 8), d=(1.0, 1.0, 1.0), mean=(0.0, 0.0, 0.0), axis="x", a1=1.0, b1=4.0),
        dict(name="odd_spacing", n=(64, 32, 16), d=(0.37, 0.41, 0.5), mean=(32.0, 16.0, 8.0), axis="z", a1=6.0,
             b1=16.0),
    ]


def mask_cases():
    rng = np.random.default_rng(0xD4AC)
    out = []
    for i, (fixed, dynamic) in enumerate([(1, 0), (0, 1), (1, 1), (0, 0), (1, 0), (0, 1)]):
        n = int(rng.integers(3000, 9000))
        acc = np.zeros((n, 4), np.float32)
        val = rng.choice(np.array([-1, 0, 1, 5, -7], np.int32), n, p=[0.4, 0.2, 0.3, 0.05, 0.05])
        acc.view(np.int32)[:, 0] = val
        acc[:, 1:] = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
        prim = rng.uniform(-1, 1, n).astype(np.float32)
        prim[rng.random(n) < 0.05] = 0.0
        prim[rng.random(n) < 0.02] = -0.0
        prim[rng.random(n) < 0.02] = np.nan
        lat = rng.uniform(-2, 2, n).astype(np.float32)
        out.append(dict(name=f"mask{i}", fixed=fixed, dynamic=dynamic, acc=acc, prim=prim, lat=lat))
    return out


def build_job():
    parts = []
    for c in period_cases():
        b = MG._p("I", 11) + MG._p("3i", *c["n"]) + MG._p("3f", *c["d"]) + MG._p("3f", *c["mean"])
        b += MG._p("I", ord(c["axis"])) + MG._p("2f", c["a1"], c["b1"])
        parts.append(b)
    for c in mask_cases():
        n = len(c["lat"])
        b = MG._p("I", 12) + MG._p("3I", n, c["fixed"], c["dynamic"])
        b += c["acc"].tobytes() + c["prim"].astype("<f4").tobytes() + c["lat"].astype("<f4").tobytes()
        parts.append(b)
    return MG._p("I", MG.MAGIC) + MG._p("I", len(parts)) + b"".join(parts)


def parse(blob):
    B = MG.Buf(blob)
    res = []
    for c in period_cases():
        assert int(B.u32()) == 11
        P = c["n"][0] * c["n"][1] * c["n"][2]
        raw = B.f32(P)
        mm = B.f32(2)
        res.append(dict(raw=raw, minmax=mm, mapped=B.f32(P)))
    for c in mask_cases():
        assert int(B.u32()) == 12
        res.append(dict(lat=B.f32(len(c["lat"]))))
    assert B.o == len(blob)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    exe = MG.build_runner()
    job = os.path.join(args.out, "job_period_mask.bin")
    with open(job, "wb") as f:
        f.write(build_job())
    results = {}
    for var in ("sm103a", "ptx89"):
        out = os.path.join(args.out, f"out_period_mask_{var}.bin")
        subprocess.run([exe, MG.REF_DIR, var, MG.TABLES, job, out], check=True)
        with open(out, "rb") as f:
            results[var] = parse(f.read())
    bad = [f"{i}:{k}" for i, (a, b) in enumerate(zip(results["sm103a"], results["ptx89"])) for k in a
           if a[k].tobytes() != b[k].tobytes()]
    print("variant differences:", bad or "none")
    # The period field's PTX form leaves unrounded multiplies and adds that the
    # driver's JIT and the offline sm_103a assembler may fuse differently; the
    # fixtures keep the sm_103a build (this library's target) and record which
    # cases differ.  Any other difference is an error.
    if any(int(b.split(":")[0]) >= len(period_cases()) for b in bad):
        return 1
    d = {"variant_differs": np.array(sorted({int(b.split(":")[0]) for b in bad}), np.int32)}
    r = results["sm103a"]
    for i, c in enumerate(period_cases()):
        pre = f"period{i}/"
        d[pre + "params"] = np.array([*c["n"], *c["d"], *c["mean"], ord(c["axis"]), c["a1"], c["b1"]], np.float64)
        d[pre + "raw"] = r[i]["raw"]
        d[pre + "minmax"] = r[i]["minmax"]
        d[pre + "mapped"] = r[i]["mapped"]
    off = len(period_cases())
    for i, c in enumerate(mask_cases()):
        pre = f"mask{i}/"
        d[pre + "flags"] = np.array([c["fixed"], c["dynamic"]], np.int32)
        d[pre + "acc"] = c["acc"]
        d[pre + "prim"] = c["prim"]
        d[pre + "lat"] = c["lat"]
        d[pre + "out"] = r[off + i]["lat"]
    np.savez_compressed(os.path.join(args.out, "golden_period_mask.npz"), **d)
    print("wrote", os.path.join(args.out, "golden_period_mask.npz"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
