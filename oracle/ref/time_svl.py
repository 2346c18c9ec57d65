"""Times the reference's spatially variant lattice synthesis (its own kernels,
its host-synchronous conjugate-gradient loop, job kind 9 of ref_runner.cpp)
beside gcm_svl_lattice on the same grid, coefficients and settings.

Measurement infrastructure: runs on the GPU machine after
``oracle/ref/build_ref.py`` has built the reference's device code.

    python oracle/ref/time_svl.py [--n 64 64 64] [--coeff 62]

The reference's loop per coefficient also re-normalises and re-meshes the
lattice and draws a frame (src/main.cu:3972-4024); only the synthesis
(finding_phi_kernel, GPUCG_lattice, grating_kernel, svl_kernel) is timed here.
Prints one JSON line.
"""
import argparse
import json
import os
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, nargs=3, default=[64, 64, 64])
    ap.add_argument("--coeff", type=int, default=62)
    ap.add_argument("--period", type=float, default=12.0)
    args = ap.parse_args()
    import make_golden as MG
    import oracle as O
    import torch

    from gpucadforam_gb300.mesher import Context

    nx, ny, nz = args.n
    u = O.unit_cell(0, 61, 61, 61).reshape(61, 61, 61)
    coef = O.svl_dft(u, 2)
    P = nx * ny * nz
    b = MG._p("I", 9) + MG._p("3i", nx, ny, nz) + MG._p("3f", 1.0, 1.0, 1.0) + MG._p("I", ord("r"))
    b += MG._p("i", 0) + MG._p("4f", args.period, 8.0, 8.0, 8.0) + MG._p("2f", 0.0, 0.0) + MG._p("I", 0)
    b += MG._p("i", 2) + MG._p("2I", args.coeff, 500) + MG._p("f", 0.01)
    b += np.zeros(P, np.float32).tobytes() + coef.astype("<f4").tobytes()
    work = tempfile.mkdtemp(prefix="gcm_time_svl_")
    job, out = os.path.join(work, "job.bin"), os.path.join(work, "out.bin")
    with open(job, "wb") as f:
        f.write(MG._p("I", MG.MAGIC) + MG._p("I", 1) + b)
    exe = MG.build_runner()
    subprocess.run([exe, MG.REF_DIR, "sm103a", MG.TABLES, job, out], check=True)
    blob = open(out, "rb").read()
    ref_iters = np.frombuffer(blob, np.uint32, args.coeff, 4)
    ref_s = struct.unpack_from("<d", blob, 4 + 4 * args.coeff)[0]

    ctx = Context(0)
    d_coef = torch.from_numpy(coef).cuda()
    ctx.svl_lattice((nx, ny, nz), d_coef, "r", 0, args.period, n_coeff=args.coeff)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    svl, iters, _ = ctx.svl_lattice((nx, ny, nz), d_coef, "r", 0, args.period, n_coeff=args.coeff)
    torch.cuda.synchronize()
    ours_s = time.perf_counter() - t0
    print(json.dumps({"grid": [nx, ny, nz], "coefficients": args.coeff, "kind": "r",
                      "reference_s": ref_s, "gcm_s": ours_s, "speedup": ref_s / ours_s,
                      "steps_equal": [int(v) for v in ref_iters] == iters,
                      "cg_steps_total": int(sum(iters)), "cg_steps_max": int(max(iters))}))
    ctx.close()


if __name__ == "__main__":
    main()
