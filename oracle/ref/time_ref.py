"""Times the reference's own marching-cubes kernels on a GB300 beside this
project's fused kernel, on the same 512^3 graded-lattice field.

Test and measurement infrastructure: runs on the GPU machine after
``oracle/ref/build_ref.py`` has compiled the reference's device code into
``oracle/_ref/`` (done by ``__graft_entry__.build()`` where the reference
sources are present).  The field is the bench's graded TPMS lattice (16^3
control grid, seed 0xD4A + 2) evaluated by the oracle, shifted by +3 with the
isovalue moved to 3: the reference's plain generate kernel takes its cube index
as (f < iso) && (f > 0) (src/MarchingCubes_kernel.cu:3041-3170), so it needs a
positive field to agree with its classify kernel.

    python oracle/ref/time_ref.py [--grid 512] [--reps 5] [--field FILE]

``--field`` takes the field (grid^3 float32, x fastest, already shifted by +3)
from a file instead of evaluating it with the oracle; the bench writes its own
device field there, which is bit-identical to the oracle's.

Prints one JSON line: per-kernel median times of the reference (classify,
compaction, generate, launched by name from its compiled code; its thrust
exclusive scan, which cannot be launched by name, is timed by ref_scan.cu making
the same thrust call on as many voxels, and counted twice as the reference
scans twice), this project's fused kernel on the same field, and both as
achieved GB/s of the algorithmic bytes 4 P + 32 V.
"""
import argparse
import ctypes as C
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_DIR = os.path.join(REPO, "oracle", "_ref")
TABLES = os.path.join(REPO, "tests", "golden", "ref_tables.bin")
sys.path.insert(0, REPO)


def controls(n_ctrl=16, seed=0xD4A + 2):
    rng = np.random.default_rng(seed)
    n = n_ctrl ** 3
    period = rng.uniform(16, 64, n).astype(np.float32)
    euler = rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32)
    thick = rng.uniform(-0.6, 0.6, n).astype(np.float32)
    types = rng.choice(np.array([0, 1, 5], np.uint8), n)
    return period, euler, thick, types


def build_runner():
    exe = os.path.join(REF_DIR, "ref_runner")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(HERE, "ref_runner.cpp"), "-I",
                    os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64"), "-L",
                    os.path.join(cuda, "lib64", "stubs"), "-lcuda", "-o", exe], check=True)
    return exe


def build_scan():
    """The reference's thrust scan call, compiled with nvcc (ref_scan.cu)."""
    exe = os.path.join(REF_DIR, "ref_scan")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run([os.path.join(cuda, "bin", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                    "-std=c++17", os.path.join(HERE, "ref_scan.cu"), "-o", exe], check=True)
    return exe


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--work", default=None, help="scratch directory for the 4 P-byte job file (default: a temp dir)")
    ap.add_argument("--field", default=None, help="raw float32 field file (grid^3 samples, shifted by +3)")
    args = ap.parse_args()

    n = args.grid
    if args.field:
        f = np.fromfile(args.field, np.float32)
        assert f.size == n ** 3, (f.size, n)
        f = f.reshape(n, n, n)
    else:
        import oracle as O

        period, euler, thick, types = controls()
        f = O.lattice_field((n, n, n), 0, (16, 16, 16), period, euler, thick, types, origin=((n - 1) / 2,) * 3)
        f = (f + np.float32(3.0)).astype(np.float32)
    iso = 3.0
    work = args.work or tempfile.mkdtemp(prefix="gcm_time_ref_")
    os.makedirs(work, exist_ok=True)
    job = os.path.join(work, "time_job.bin")
    with open(job, "wb") as fh:
        fh.write(struct.pack("<III", 0x4A4D4347, 1, 6))
        fh.write(struct.pack("<IIIf", n, n, n, iso))
        fh.write(struct.pack("<ffffffI", 1, 1, 1, 0, 0, 0, args.reps))
        fh.write(np.ascontiguousarray(f).tobytes())
    out = os.path.join(work, "time_out.bin")
    exe = build_runner()
    subprocess.run([exe, REF_DIR, "sm103a", TABLES, job, out], check=True)
    b = open(out, "rb").read()
    kind, nvox, active, total, reps = struct.unpack_from("<IIIII", b, 0)
    t = np.frombuffer(b, np.float32, 3 * reps, 20).reshape(reps, 3)
    med = np.median(t, axis=0)
    # the reference's two thrust scans per extraction (vertex counts and
    # occupancy), each over all voxels
    scan_ms = None
    try:
        r = subprocess.run([build_scan(), str(nvox), str(args.reps)], check=True, capture_output=True, text=True)
        scan_ms = float(r.stdout.split()[1])
    except (OSError, subprocess.SubprocessError, ValueError, IndexError) as e:
        print(f"thrust scan not timed: {e}", file=sys.stderr)

    # this project's fused kernel, same field and isovalue
    import torch

    from gpucadforam_gb300.mesher import Context

    ctx = Context(0)
    d = torch.from_numpy(f).cuda()
    cnt = ctx.count_field(d, iso)
    pos = torch.empty((cnt.total_verts, 4), device="cuda")
    norm = torch.empty_like(pos)
    dc = torch.zeros(4, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    for _ in range(3):
        ctx.mesh_field_async(d, iso, pos, norm, dc)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ctx.mesh_field_async(d, iso, pos, norm, dc)
        e1.record(st)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    ours = float(np.median(ms))
    P = n ** 3
    alg = 4 * P + 32 * int(total)
    ref_ms = float(med.sum())
    print(json.dumps({
        "grid": n, "voxels": int(nvox), "active_voxels": int(active), "verts_reference": int(total),
        "verts_gcm": int(cnt.total_verts),
        "reps": int(reps), "reference_ms_per_rep": t.tolist(),
        "reference_ms": {"classifyVoxel_new": float(med[0]), "compactVoxels": float(med[1]),
                         "generateTriangles_lattice_kernel_3": float(med[2]), "sum_without_scans": ref_ms,
                         "thrust_exclusive_scan": scan_ms,
                         "sum_with_scans": ref_ms + 2 * scan_ms if scan_ms is not None else None},
        "gcm_fused_ms": ours,
        "algorithmic_bytes": alg,
        "reference_GBs": alg / ref_ms / 1e6, "gcm_GBs": (4 * P + 32 * int(cnt.total_verts)) / ours / 1e6,
        "speedup": ref_ms / ours}))
    ctx.close()


if __name__ == "__main__":
    main()
