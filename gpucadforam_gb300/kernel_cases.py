"""Runs one of the library's kernels on a seeded input, a few times, so that a
profiler can capture it alone.

    python -m gpucadforam_gb300.kernel_cases CASE [--n 320] [--reps 3]

Cases (the kernel each one launches ``reps`` times after one warm-up call):

* ``unit_cell``      unit_cell_kernel: a gyroid unit cell of n^3 samples;
* ``lattice_rows``   lattice_rows_kernel: the graded TPMS lattice of a 16^3
                     control grid (periods U[16, 64], Euler angles U[-pi/4, pi/4],
                     thickness U[-0.6, 0.6], types gyroid/diamond/Schwarz-P);
* ``lattice_wide``   lattice_rows_kernel with one row per warp in opt-in shared
                     memory: the same with a 96 x 8 x 8 control grid;
* ``lattice_params`` lattice_params_kernel: the same with a 320 x 4 x 4 control
                     grid, wider than the row kernel stages;
* ``lattice_blend``  lattice_prep_kernel + lattice_blend_kernel: the 16^3 grid
                     in the blend grading;
* ``staged_mc``      mc_classify_kernel, scan_u32 (two exclusive scans),
                     mc_compact_kernel, mc_generate_kernel: the staged
                     extraction of the lattice_rows field at iso 0.

Each case prints one line with the sizes and the mean time per call from CUDA
events (not a bench number; the captures are what these runs are for).
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np


def _controls(ctrl, seed=0xD4A + 2):
    rng = np.random.default_rng(seed)
    n = int(np.prod(ctrl))
    period = rng.uniform(16, 64, n).astype(np.float32)
    euler = rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32)
    thick = rng.uniform(-0.6, 0.6, n).astype(np.float32)
    types = rng.choice(np.array([0, 1, 5], np.uint8), n)
    return period, euler, thick, types


def _timed(fn, reps):
    import torch

    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["unit_cell", "lattice_rows", "lattice_wide", "lattice_params", "lattice_blend",
                                     "staged_mc"])
    ap.add_argument("--n", type=int, default=320)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args(argv)

    import torch

    from .mesher import Context, Lattice

    n = args.n
    shape = (n, n, n)
    ctx = Context(0)
    info = {"case": args.case, "grid": n, "reps": args.reps}

    def lattice(mode, ctrl):
        period, euler, thick, types = _controls(ctrl)
        ctrl_xyz = (ctrl[0], ctrl[1], ctrl[2])
        return Lattice.from_numpy(mode, ctrl_xyz, period, euler, thick, types, ((n - 1) / 2,) * 3)

    if args.case == "unit_cell":
        info["ms"] = _timed(lambda: ctx.unit_cell(0, n, n, n), args.reps)
    elif args.case in ("lattice_rows", "lattice_wide", "lattice_params", "lattice_blend"):
        ctrl = {"lattice_wide": (96, 8, 8), "lattice_params": (min(320, n), 4, 4)}.get(args.case, (16, 16, 16))
        lat = lattice(1 if args.case == "lattice_blend" else 0, ctrl)
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
        s = ctx.lattice_struct(lat)
        import ctypes as C

        info["ms"] = _timed(lambda: ctx.check(ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), n, n, n,
                                                                          C.c_void_p(out.data_ptr()), None)),
                            args.reps)
    else:
        field = ctx.lattice_field(lattice(0, (16, 16, 16)), shape)
        torch.cuda.synchronize()

        def staged():
            verts, occ, _ = ctx.classify(field, 0.0)
            occ_scan, active = ctx.scan(occ)
            verts_scan, total = ctx.scan(verts)
            comp = ctx.compact(occ, occ_scan, active)
            pos, _ = ctx.generate(field, 0.0, comp, verts_scan, total)
            info["active_voxels"], info["verts"] = active, total

        info["ms"] = _timed(staged, args.reps)
    print(json.dumps(info))
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
