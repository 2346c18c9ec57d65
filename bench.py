"""Benchmark of the field -> mesh hot path on GB300.

Default workload (the headline configuration): a spatially varying TPMS lattice
on a 512^3 FP32 grid.  Per control point of a 16^3 grid of seeded uniform values:
type in {gyroid, Schwarz-P, diamond}, period U[16,64] voxels, Euler angles
U[-pi/4, pi/4], thickness U[-0.6, 0.6]; parameters trilinear per voxel, type of
the nearest control point (GCM_GRADE_PARAMS), isovalue 0, unshared float4
position + normal triangles out.

One step = field evaluation + fused marching cubes over the whole grid.
`value` = voxels/s with the control grids resident in HBM; `e2e` = the same
through the C ABI with host buffers (control grids copied in, the mesh copied
out to pinned host memory, inside the timed region).  `--impl reference` times
the CPU restatement of the reference's algorithm (oracle/) on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gcm|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_GRID = 512
N_CTRL = 16
SEED = 0xD4A + 2
METRIC = "voxels/s & tris/s at 512^3 (%HBM roofline)"


def c2_controls(n_ctrl=N_CTRL, seed=SEED):
    rng = np.random.default_rng(seed)
    n = n_ctrl ** 3
    period = rng.uniform(16, 64, n).astype(np.float32)
    euler = rng.uniform(-np.pi / 4, np.pi / 4, 3 * n).astype(np.float32)
    thick = rng.uniform(-0.6, 0.6, n).astype(np.float32)
    types = rng.choice(np.array([0, 1, 5], np.uint8), n)
    return period, euler, thick, types


def workload_config(n=N_GRID):
    return {"workload": f"graded TPMS lattice {n}^3 FP32 (gyroid/Schwarz-P/diamond, period 16-64 vox, "
                        f"Euler +-pi/4, thickness +-0.6, {N_CTRL}^3 control grid, trilinear parameters)",
            "grid": [n, n, n], "control_grid": [N_CTRL] * 3, "grading": "params", "iso": 0.0,
            "l2": f"working set larger than L2 ({4 * n ** 3 / 2 ** 20:.0f} MiB field + mesh); no flush",
            "parallelism": "replicas"}


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel_key):
    """DRAM bytes per launch of one kernel from a committed ncu summary (a small
    JSON sidecar next to the text summary in profiles/), scaled to the workload
    by the summary itself; None when no capture exists."""
    p = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    v = d.get(kernel_key)
    return None if v is None else float(v)


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "gcm" else "gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg, torch=None):
    if torch is not None:
        torch.cuda.synchronize()
    if pg is not None:
        pg.barrier()


def allmax(pg, v, torch=None):
    if pg is None:
        return v
    import torch as T

    t = T.tensor([float(v)], dtype=T.float64, device="cuda" if torch is not None else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allsum(pg, v, torch=None):
    if pg is None:
        return v
    import torch as T

    t = T.tensor([float(v)], dtype=T.float64, device="cuda" if torch is not None else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ----------------------------------------------------------------------------- CPU


def cpu_sample(threads, n=N_GRID, planes=256):
    """Times the oracle's field evaluation + marching cubes (OpenMP) on a centred
    z-slab of `planes` sample planes of the workload (same control grid, origin
    and voxel numbering); returns voxels/s and the split."""
    import oracle as O

    period, euler, thick, types = c2_controls()
    planes = min(planes or n, n)
    z0 = (n - planes) // 2
    origin = ((n - 1) / 2,) * 3
    t0 = time.perf_counter()
    f = O.lattice_slab((n, n, n), z0, planes, 0, (N_CTRL,) * 3, period, euler, thick, types, origin, threads=threads)
    t1 = time.perf_counter()
    vox = (n - 1) * (n - 1) * (planes - 1)
    # the first pass sizes the output (it runs the whole pipeline, writing nothing)
    total, _, _, _ = O.mesh_field_omp(f, (1, 1, 1), (0, 0, 0), 0.0, 0, threads)
    t2 = time.perf_counter()
    total, active, _, _ = O.mesh_field_omp(f, (1, 1, 1), (0, 0, 0), 0.0, total, threads)
    t3 = time.perf_counter()
    field_s, mesh_s = t1 - t0, t3 - t2
    return {"voxels": vox, "verts": total, "active": active, "field_s": field_s, "mesh_s": mesh_s,
            "voxels_per_s": vox / (field_s + mesh_s)}


def csg_scene(seed, n_prims=64, n_sub=8):
    """Config C3: 64 seeded primitives (spheres r in [0.02, 0.15], z-axis capped
    cylinders, axis boxes with half-extents in [0.02, 0.12]) at uniform centres
    in [0, 1]^3, min-union with the last 8 subtracted."""
    rng = np.random.default_rng(seed)
    prims = []
    for i in range(n_prims):
        kind = int(rng.integers(0, 3))
        c = rng.uniform(0, 1, 3).astype(np.float32)
        op = 1 if i >= n_prims - n_sub else 0
        if kind == 0:
            prims.append(dict(kind=0, op=op, center=c, p=[rng.uniform(0.02, 0.15), 0.0]))
        elif kind == 1:
            r, hh = rng.uniform(0.02, 0.12, 2)
            prims.append(dict(kind=1, op=op, center=c, v3=(0.0, 0.0, 1.0), p=[r, 0.0, 2 * hh]))
        else:
            prims.append(dict(kind=2, op=op, center=c, v3=(0.0, 0.0, 0.0), p=list(2 * rng.uniform(0.02, 0.12, 3))))
    return prims


def run_configs(ctx, steps, warmup, cpu=True):
    """Configs C1 (128^3 uniform gyroid, period 32 voxels, over [0,1]^3) and C3
    (384^3 CSG scene): field and fused mesh per step from CUDA events, and the
    oracle on the host cores for the same config (all of C1; a centred slab of
    64 planes of C3)."""
    import torch

    import oracle as O
    from gpucadforam_gb300.mesher import Lattice, make_frame, make_grid, primitives_to_device

    peak, _ = measured_peaks()
    out = {}
    threads = os.cpu_count() or 1
    stream = torch.cuda.current_stream()
    cs = C.c_void_p(stream.cuda_stream)
    for name in ("C1", "C3"):
        if name == "C1":
            n = 128
            lat = Lattice.from_numpy(0, (1, 1, 1), np.array([32.0], np.float32), np.zeros(3, np.float32),
                                     np.zeros(1, np.float32), np.zeros(1, np.uint8), (0.0, 0.0, 0.0))
            s = ctx.lattice_struct(lat)
            field_call = lambda f: ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), n, n, n, C.c_void_p(f.data_ptr()), cs)
            desc = "uniform gyroid 128^3, period 32 voxels, over [0,1]^3, iso 0"
        else:
            n = 384
            prims = csg_scene(SEED + 1)
            d_prims = primitives_to_device(prims)
            h = np.float32(1.0 / (n - 1))
            frame = make_frame((0, 0, 0), (h, h, h))
            field_call = lambda f: ctx.lib.gcm_field_csg(ctx.h, C.c_void_p(d_prims.data_ptr()), len(prims),
                                                         C.byref(frame), n, n, n, C.c_void_p(f.data_ptr()), cs)
            desc = "CSG 384^3: 64 seeded spheres / capped cylinders / boxes in [0,1]^3, 8 subtracted, iso 0"
        vs = 1.0 / (n - 1)
        grid = make_grid((n, n, n), (vs, vs, vs))
        field = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
        ctx.check(field_call(field))
        cnt = ctx.count_field(field, 0.0)
        cap = max(cnt.total_verts, 1)
        pos = torch.empty((cap, 4), device="cuda")
        norm = torch.empty((cap, 4), device="cuda")
        d_counts = torch.zeros(4, dtype=torch.int64, device="cuda")

        def step(ev=None):
            if ev:
                ev[0].record(stream)
            ctx.check(field_call(field))
            if ev:
                ev[1].record(stream)
            ctx.check(ctx.lib.gcm_mesh_field_async(ctx.h, C.c_void_p(field.data_ptr()), C.byref(grid), 0.0,
                                                   C.c_void_p(pos.data_ptr()), C.c_void_p(norm.data_ptr()), cap,
                                                   C.c_void_p(d_counts.data_ptr()), cs))
            if ev:
                ev[2].record(stream)

        # both extraction paths; the line's mesh_ms is the one the workload's
        # own call takes by default (gcm_mesh_csg: sparse, lattices: fused)
        times = {}
        for path in ("fused", "sparse"):
            ctx.set_mesh_path(path)
            for _ in range(warmup):
                step()
            torch.cuda.synchronize()
            evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
            for k in range(steps):
                step(evs[k])
            torch.cuda.synchronize()
            times[path] = (statistics.mean(e[0].elapsed_time(e[1]) for e in evs),
                           statistics.mean(e[1].elapsed_time(e[2]) for e in evs))
        ctx.set_mesh_path("auto")
        # C3's own call: gcm_mesh_csg_async evaluates the field with its tile
        # states and extracts (the count pass skips the tasks whose tiles all
        # lie on one side of the isovalue)
        csg_ms = None
        if name == "C3":
            def csg_step():
                ctx.check(ctx.lib.gcm_mesh_csg_async(ctx.h, C.c_void_p(d_prims.data_ptr()), len(prims), C.byref(frame),
                                                     C.byref(grid), 0.0, C.c_void_p(pos.data_ptr()),
                                                     C.c_void_p(norm.data_ptr()), cap,
                                                     C.c_void_p(d_counts.data_ptr()), cs))

            for _ in range(warmup):
                csg_step()
            torch.cuda.synchronize()
            evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
            for k in range(steps):
                evs[k][0].record(stream)
                csg_step()
                evs[k][1].record(stream)
            torch.cuda.synchronize()
            csg_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in evs)
            chk = d_counts.cpu().numpy().view(np.uint64)
            assert int(chk[1]) == cnt.total_verts and int(chk[2] & 0xFFFFFFFF) == 0, chk
        chosen = "sparse" if name == "C3" else "fused"
        f_ms, m_ms = times[chosen]
        vox = (n - 1) ** 3
        alg = 4 * n ** 3 + 32 * cnt.total_verts
        r = {"workload": desc, "grid": [n, n, n], "verts": int(cnt.total_verts), "active_voxels": int(cnt.active_voxels),
             "field_ms": f_ms, "mesh_ms": m_ms, "mesh_path": chosen, "mesh_ms_fused": times["fused"][1],
             "mesh_ms_sparse": times["sparse"][1], "voxels_per_s": vox / ((f_ms + m_ms) / 1e3),
             "tris_per_s": cnt.total_verts / 3 / ((f_ms + m_ms) / 1e3), "mesh_GBs": alg / (m_ms / 1e3) / 1e9,
             "mesh_frac_of_measured": alg / (m_ms / 1e3) / 1e9 / peak}
        if csg_ms is not None:
            m2 = csg_ms - f_ms  # the extraction's share of the one call, the field timed alone
            r.update({"mesh_csg_ms": csg_ms, "mesh_csg_voxels_per_s": vox / (csg_ms / 1e3),
                      "mesh_ms_with_tile_states": m2, "mesh_frac_with_tile_states": alg / (m2 / 1e3) / 1e9 / peak,
                      "mesh_csg_note": "gcm_mesh_csg_async (field with tile states + windowed extraction) timed as "
                                       "one call; the extraction's share is that time less field_ms"})
        if cpu:
            t0 = time.perf_counter()
            if name == "C1":
                fo = O.lattice_field((n, n, n), 0, (1, 1, 1), np.array([32.0], np.float32), np.zeros(3, np.float32),
                                     np.zeros(1, np.float32), np.zeros(1, np.uint8), (0.0, 0.0, 0.0), threads=threads)
                planes = n
            else:
                planes = 64
                z0 = (n - planes) // 2
                fo = O.csg_field(prims, (n, n, planes), (0, 0, -z0), (h, h, h), threads=threads)
            t1 = time.perf_counter()
            tot, _, _, _ = O.mesh_field_omp(fo, (vs, vs, vs), (0, 0, 0), 0.0, 0, threads)
            t2 = time.perf_counter()
            O.mesh_field_omp(fo, (vs, vs, vs), (0, 0, 0), 0.0, tot, threads)
            t3 = time.perf_counter()
            cvox = (n - 1) ** 2 * (planes - 1)
            r["cpu_baseline"] = {"value": cvox / ((t1 - t0) + (t3 - t2)), "unit": "voxels/s", "cores": threads,
                                 "kind": "port", "sample": f"{planes} of {n} sample planes"}
        out[name] = r
        del field, pos, norm
    return out


def run_rows(ctx, steps, warmup, cpu=True):
    """The rows beside the hot path, each timed on the device (CUDA events on
    the launching stream) with its algorithmic bytes, and the oracle's rate on
    the host cores beside it:

    * retained CSG editing: 8 sphere fields (6 united, 2 subtracted) folded into
      a 256^3 accumulator (16 B read + 4 B field + 16 B written per sample and
      fold), then the region mesh (16 B per sample read, 32 B per vertex);
    * band mode: a 384^3 gyroid (period 32 voxels) normalised into label and
      band field (4 B read twice, 8 B written per sample), then the band mesh
      (8 B per sample read, 32 B per vertex), band [0.35, 0.65], iso 0.5;
    * .obj export of the 128^3 gyroid mesh: GPU weld (call to counts on the
      host) and the whole file written, against the oracle's restatement of
      the reference's serial writer."""
    import tempfile

    import torch

    import oracle as O
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import Lattice, make_frame, make_grid, primitives_to_device

    peak, _ = measured_peaks()
    threads = os.cpu_count() or 1
    stream = torch.cuda.current_stream()
    cs = C.c_void_p(stream.cuda_stream)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    out = {}

    # ---- retained CSG editing
    n = 256
    rng = np.random.default_rng(SEED + 5)
    h = np.float32(1.0 / (n - 1))
    frame = make_frame((0, 0, 0), (h, h, h))
    sph = [dict(kind=0, op=0, center=rng.uniform(0.2, 0.8, 3).astype(np.float32),
                p=[float(rng.uniform(0.1, 0.25)), 0.0]) for _ in range(8)]
    ops = ["union"] * 6 + ["subtract"] * 2
    fields = [ctx.csg_field(primitives_to_device([q]), 1, frame, (n, n, n)) for q in sph]
    acc = ctx.csg_accumulator((n, n, n))
    for f, op in zip(fields, ops):
        ctx.csg_retain(acc, f, op=op)
    cap = ctx.count_retained(acc).total_verts
    pos = torch.empty((max(cap, 1), 4), device="cuda")
    norm = torch.empty((max(cap, 1), 4), device="cuda")
    grid = make_grid((n, n, n))
    gc = N.GcmCounts()
    fold_ms, mesh_ms = [], []
    for k in range(warmup + steps):
        acc.zero_()
        e = [ev() for _ in range(len(fields) + 2)]
        e[0].record(stream)
        for i, (f, op) in enumerate(zip(fields, ops)):
            ctx.csg_retain(acc, f, op=op)
            e[i + 1].record(stream)
        ctx.check(ctx.lib.gcm_mesh_retained(ctx.h, C.c_void_p(acc.data_ptr()), None, 0, C.byref(grid), 0.0,
                                            C.c_void_p(pos.data_ptr()), C.c_void_p(norm.data_ptr()), cap,
                                            C.byref(gc), cs))
        e[-1].record(stream)
        torch.cuda.synchronize()
        if k >= warmup:
            fold_ms += [e[i].elapsed_time(e[i + 1]) for i in range(len(fields))]
            mesh_ms.append(e[-2].elapsed_time(e[-1]))
    P = n ** 3
    f_ms, m_ms = statistics.mean(fold_ms), statistics.mean(mesh_ms)
    r = {"workload": "8 sphere fields (6 united, 2 subtracted) folded into a 256^3 retained accumulator, then its "
                     "region mesh", "grid": [n, n, n], "verts": int(gc.total_verts),
         "fold_ms": f_ms, "fold_samples_per_s": P / (f_ms / 1e3), "fold_GBs": 36 * P / (f_ms / 1e3) / 1e9,
         "fold_frac_of_measured": 36 * P / (f_ms / 1e3) / 1e9 / peak,
         "mesh_ms": m_ms, "mesh_voxels_per_s": (n - 1) ** 3 / (m_ms / 1e3),
         "mesh_GBs": (16 * P + 32 * int(gc.total_verts)) / (m_ms / 1e3) / 1e9,
         "mesh_note": "gcm_mesh_retained returns counts to the host; its events include that sync"}
    if cpu:
        planes = 32
        z0 = (n - planes) // 2
        hf = [O.csg_field([q], (n, n, planes), (0, 0, -z0), (h, h, h), threads=threads) for q in sph]
        hacc = O.csg_accumulator((planes, n, n))
        t0 = time.perf_counter()
        for f, op in zip(hf, ops):
            O.csg_retain(hacc, f, op=op)
        t1 = time.perf_counter()
        O.mesh_retained(hacc, None, "union", (1, 1, 1), (0, 0, 0))
        t2 = time.perf_counter()
        r["cpu_baseline"] = {"fold_samples_per_s": len(hf) * n * n * planes / (t1 - t0) / len(hf),
                             "mesh_voxels_per_s": (n - 1) ** 2 * (planes - 1) / (t2 - t1), "cores": 1,
                             "kind": "port", "sample": f"{planes} of {n} sample planes (the oracle's retained kernels "
                                                       f"are single-threaded)"}
    out["retained_csg"] = r
    del fields, acc, pos, norm

    # ---- band mode
    n = 384
    lat = Lattice.from_numpy(0, (1, 1, 1), np.array([32.0], np.float32), np.zeros(3, np.float32),
                             np.zeros(1, np.float32), np.zeros(1, np.uint8), (0.0, 0.0, 0.0))
    f = ctx.lattice_field(lat, (n, n, n))
    label = torch.empty_like(f)
    nfield = torch.empty_like(f)
    iso, lo, hi = 0.5, 0.35, 0.65
    ctx.check(ctx.lib.gcm_normalise_band(ctx.h, C.c_void_p(f.data_ptr()), n, n, n, lo, hi,
                                         C.c_void_p(label.data_ptr()), C.c_void_p(nfield.data_ptr()), None, cs))
    cap = ctx.count_field(label, iso).total_verts
    pos = torch.empty((max(cap, 1), 4), device="cuda")
    norm = torch.empty((max(cap, 1), 4), device="cuda")
    d_counts = torch.zeros(4, dtype=torch.int64, device="cuda")
    grid = make_grid((n, n, n))
    norm_ms, band_ms = [], []
    for k in range(warmup + steps):
        e = [ev() for _ in range(3)]
        e[0].record(stream)
        ctx.check(ctx.lib.gcm_normalise_band(ctx.h, C.c_void_p(f.data_ptr()), n, n, n, lo, hi,
                                             C.c_void_p(label.data_ptr()), C.c_void_p(nfield.data_ptr()), None, cs))
        e[1].record(stream)
        ctx.check(ctx.lib.gcm_mesh_band_async(ctx.h, C.c_void_p(label.data_ptr()), C.c_void_p(nfield.data_ptr()),
                                              C.byref(grid), iso, lo, hi, C.c_void_p(pos.data_ptr()),
                                              C.c_void_p(norm.data_ptr()), cap, C.c_void_p(d_counts.data_ptr()), cs))
        e[2].record(stream)
        torch.cuda.synchronize()
        if k >= warmup:
            norm_ms.append(e[0].elapsed_time(e[1]))
            band_ms.append(e[1].elapsed_time(e[2]))
    P = n ** 3
    nv = int(d_counts[1])
    a_ms, b_ms = statistics.mean(norm_ms), statistics.mean(band_ms)
    r = {"workload": "384^3 gyroid (period 32 voxels) normalised into a band [0.35, 0.65], iso 0.5, and meshed",
         "grid": [n, n, n], "verts": nv, "normalise_ms": a_ms, "normalise_GBs": 16 * P / (a_ms / 1e3) / 1e9,
         "normalise_frac_of_measured": 16 * P / (a_ms / 1e3) / 1e9 / peak,
         "mesh_ms": b_ms, "mesh_voxels_per_s": (n - 1) ** 3 / (b_ms / 1e3),
         "mesh_GBs": (8 * P + 32 * nv) / (b_ms / 1e3) / 1e9,
         "mesh_frac_of_measured": (8 * P + 32 * nv) / (b_ms / 1e3) / 1e9 / peak}
    if cpu:
        planes = 64
        z0 = (n - planes) // 2
        hf = f[z0:z0 + planes].cpu().numpy()
        t0 = time.perf_counter()
        hl, hn, _ = O.normalise_band(hf, lo, hi)
        t1 = time.perf_counter()
        O.mesh_band(hl, hn, (1, 1, 1), (0, 0, 0), iso, lo, hi)
        t2 = time.perf_counter()
        r["cpu_baseline"] = {"normalise_samples_per_s": n * n * planes / (t1 - t0),
                             "mesh_voxels_per_s": (n - 1) ** 2 * (planes - 1) / (t2 - t1), "cores": 1,
                             "kind": "port", "sample": f"{planes} of {n} sample planes (the slab normalised on its "
                                                       f"own range)"}
    out["band"] = r
    del f, label, nfield, pos, norm

    # ---- .obj export
    n = 128
    lat = Lattice.from_numpy(0, (1, 1, 1), np.array([32.0], np.float32), np.zeros(3, np.float32),
                             np.zeros(1, np.float32), np.zeros(1, np.uint8), (0.0, 0.0, 0.0))
    f = ctx.lattice_field(lat, (n, n, n))
    vs = 1.0 / (n - 1)
    pos, _, cnt = ctx.mesh_field(f, 0.0, (vs, vs, vs))
    V = int(cnt.total_verts)
    nvo, nfo = C.c_uint64(0), C.c_uint64(0)
    d_v = torch.empty((V, 3), dtype=torch.float32, device="cuda")
    d_f = torch.empty((V // 3, 3), dtype=torch.int32, device="cuda")
    weld_s, write_s = [], []
    work = tempfile.mkdtemp(prefix="gcm_obj_")
    path = os.path.join(work, "mesh.obj")
    for k in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.check(ctx.lib.gcm_weld_obj(ctx.h, C.c_void_p(pos.data_ptr()), V, C.c_void_p(d_v.data_ptr()), V,
                                       C.c_void_p(d_f.data_ptr()), V // 3, C.byref(nvo), C.byref(nfo), cs))
        t1 = time.perf_counter()
        ctx.check(ctx.lib.gcm_write_obj(ctx.h, C.c_void_p(pos.data_ptr()), V, path.encode(), None, None, cs))
        t2 = time.perf_counter()
        if k >= warmup:
            weld_s.append(t1 - t0)
            write_s.append(t2 - t1)
    w_s, wr_s = statistics.median(weld_s), statistics.median(write_s)
    r = {"workload": "128^3 uniform gyroid mesh (period 32 voxels) welded and written as .obj", "verts": V,
         "obj_vertices": int(nvo.value), "obj_faces": int(nfo.value), "file_bytes": os.path.getsize(path),
         "weld_s": w_s, "weld_verts_per_s": V / w_s, "write_s": wr_s, "write_verts_per_s": V / wr_s}
    if cpu:
        hp = pos.cpu().numpy()
        opath = os.path.join(work, "oracle.obj")
        t0 = time.perf_counter()
        O.write_obj(hp, opath)
        t1 = time.perf_counter()
        with open(path, "rb") as a, open(opath, "rb") as b:
            r["identical_to_oracle"] = a.read() == b.read()
        r["cpu_baseline"] = {"write_verts_per_s": V / (t1 - t0), "cores": 1, "kind": "port",
                             "sample": "the whole mesh through the oracle's restatement of the reference's writer"}
        os.remove(opath)
    os.remove(path)
    os.rmdir(work)
    out["obj"] = r
    return out


def run_reference(args):
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    samples = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(threads, planes=args.cpu_planes)
        if i >= args.warmup:
            samples.append(r)
    v = statistics.median(s["voxels_per_s"] for s in samples)
    tris = statistics.median(s["verts"] / 3 / (s["field_s"] + s["mesh_s"]) for s in samples)
    ms = statistics.median((s["field_s"] + s["mesh_s"]) * 1e3 for s in samples)
    sample = (f"centred z-slab of {args.cpu_planes} of {N_GRID} sample planes of the same field per step "
              f"(field evaluation + classify + scans + compaction + generation)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "voxels/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(), "tris_per_s": tris,
            "cpu_baseline": {"value": v, "unit": "voxels/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- GPU


def run_reference_cuda(field, local, reps=5):
    """The reference's own plain marching-cubes kernels (classifyVoxel_new,
    compactVoxels, generateTriangles_lattice_kernel_3 of
    src/MarchingCubes_kernel.cu:3207-3249, 1594-1608, 3041-3170, compiled for
    sm_103a from its sources into oracle/_ref/) timed on this GPU on the bench
    field, in a subprocess (oracle/ref/time_ref.py) with its own clock samples.

    A reported baseline beside ``kernels_ms``, never the bench value.  The
    field is shifted by +3 with the isovalue at 3, because the reference's
    generate kernel indexes cubes by (f < iso) && (f > 0).  Its two thrust
    scans cannot be launched by name; the same thrust call on as many voxels is
    timed separately and reported beside the kernel sum."""
    import shutil
    import tempfile

    import torch

    here = os.path.dirname(os.path.abspath(__file__))
    ref_dir = os.path.join(here, "oracle", "_ref")
    need = [os.path.join(ref_dir, "ref_mc_sm103a.fatbin"), os.path.join(here, "tests", "golden", "ref_tables.bin")]
    missing = [os.path.relpath(p, here) for p in need if not os.path.exists(p)]
    if missing:
        return {"unavailable": "reference device code not built here: missing " + ", ".join(missing)}
    n = field.shape[0]
    work = tempfile.mkdtemp(prefix="gcm_ref_cuda_")
    try:
        path = os.path.join(work, "field.bin")
        (field + 3.0).cpu().numpy().tofile(path)
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        time.sleep(0.3)
        r = subprocess.run([sys.executable, os.path.join(here, "oracle", "ref", "time_ref.py"), "--grid", str(n),
                            "--reps", str(reps), "--field", path, "--work", work],
                           capture_output=True, text=True, timeout=600,
                           env=dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES", str(local))))
        clk = clocks.stop()
    except (OSError, subprocess.SubprocessError) as e:
        return {"unavailable": f"reference timing did not run: {type(e).__name__}: {e}"}
    finally:
        shutil.rmtree(work, ignore_errors=True)
    if r.returncode != 0:
        tail = (r.stderr or r.stdout).strip().splitlines()[-1:] or ["no output"]
        return {"unavailable": f"reference timing exited {r.returncode}: {tail[0][:200]}"}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    ms = d["reference_ms"]
    scan = ms.get("thrust_exclusive_scan")
    return {"classify_ms": ms["classifyVoxel_new"], "compact_ms": ms["compactVoxels"],
            "generate_ms": ms["generateTriangles_lattice_kernel_3"], "total_ms": ms["sum_without_scans"],
            "scan_ms": scan, "total_with_scans_ms": ms.get("sum_with_scans"),
            "speedup_mesh_with_scans": (ms["sum_with_scans"] / d["gcm_fused_ms"]) if ms.get("sum_with_scans") else None,
            "scans": "total_ms leaves out the reference's two thrust exclusive scans; scan_ms is the same thrust "
                     "call on as many voxels (oracle/ref/ref_scan.cu), counted twice in total_with_scans_ms",
            "reps": d["reps"], "statistic": "median over reps", "verts": d["verts_reference"],
            "gcm_mesh_ms_same_field": d["gcm_fused_ms"], "verts_gcm": d["verts_gcm"],
            "speedup_mesh": d["speedup"], "algorithmic_bytes": d["algorithmic_bytes"],
            "reference_GBs": d["reference_GBs"], "field": f"bench field + 3, iso 3, {n}^3",
            "clocks": clk}


def run_batched(ctx, steps, warmup, n_inst=256, seed=SEED + 2):
    """Config C4: n_inst graded lattices (sides U{32..256}, one type and one
    period U[8,48] per instance, thickness and rotation graded on an 8^3 control
    grid) meshed as one autotuned, graph-replayed batch, against the same
    instances meshed one at a time with gcm_mesh_lattice."""
    import torch

    from gpucadforam_gb300.mesher import Batch, random_batch_lattices

    lats, shapes = random_batch_lattices(n_inst, seed=seed)
    b = Batch(ctx, lats, shapes)
    verts, active, tot = b.count()
    cap = tot.total_verts
    pos, norm, offsets, counts = b.buffers(cap)
    threads, tile = b.tune(pos, norm)
    for _ in range(warmup):
        b.mesh_async(pos, norm, offsets, counts, graph=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.mesh_async(pos, norm, offsets, counts, graph=True)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / steps
    off = offsets.cpu().numpy().view(np.uint64)
    ref = pos[:: max(1, cap // 4096)].clone()
    # plain: one public call per instance, each synchronising for its counts
    sl = [(int(off[i]), int(off[i + 1])) for i in range(n_inst)]

    def plain_round():
        for i, (lat, shape) in enumerate(zip(lats, shapes)):
            a, e = sl[i]
            ctx.mesh_lattice(lat, shape, 0.0, pos=pos[a:e] if e > a else pos[:1], norm=norm[a:e] if e > a else norm[:1])

    for _ in range(max(1, warmup // 2)):
        plain_round()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        plain_round()
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3 / steps
    same = bool(torch.equal(pos[:: max(1, cap // 4096)], ref))
    points = sum(s[0] * s[1] * s[2] for s in shapes)
    b.close()
    return {"workload": f"{n_inst} graded lattices, sides U{{32..256}}, period U[8,48], 8^3 control grids",
            "instances": n_inst, "points": int(points), "verts": int(cap), "launch_shape": [threads, tile],
            "batched_ms": batched_ms, "plain_ms": plain_ms, "meshes_per_s": n_inst / (batched_ms / 1e3),
            "plain_meshes_per_s": n_inst / (plain_ms / 1e3), "speedup": plain_ms / batched_ms,
            "graph": True, "identical_to_plain": same}


def served_requests(seed, duration_s, rate, device="cuda"):
    """Config C5 request stream: Poisson arrivals, cubic grids with edges
    log-uniform in [64, 512], 70% graded TPMS lattices (blend grading against
    one of 8 resident 8^3 grading fields), 30% CSG scenes of U{8..64}
    primitives.  Returns (arrival_s, requests, resident lattices)."""
    from gpucadforam_gb300.mesher import Lattice, make_frame, primitives_to_device

    rng = np.random.default_rng(seed)
    nc = 8 ** 3
    resident = [Lattice.from_numpy(1, (8, 8, 8), rng.uniform(16, 64, nc).astype(np.float32),
                                   rng.uniform(-np.pi / 4, np.pi / 4, 3 * nc).astype(np.float32),
                                   rng.uniform(-0.6, 0.6, nc).astype(np.float32),
                                   rng.choice(np.array([0, 1, 5], np.uint8), nc), device=device) for _ in range(8)]
    t, arrivals, reqs = 0.0, [], []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration_s:
            break
        edge = int(round(np.exp(rng.uniform(np.log(64), np.log(512)))))
        shape = (edge, edge, edge)
        if rng.random() < 0.7:
            reqs.append(("lattice", resident[int(rng.integers(0, 8))], shape))
        else:
            k = int(rng.integers(8, 65))
            prims = []
            for j in range(k):
                kind = int(rng.integers(0, 3))
                c = rng.uniform(0, 1, 3)
                op = 1 if j >= k - max(1, k // 8) else 0
                if kind == 0:
                    prims.append(dict(kind=0, op=op, center=c, p=[rng.uniform(0.02, 0.15), 0.0]))
                elif kind == 1:
                    r, hh = rng.uniform(0.02, 0.12, 2)
                    prims.append(dict(kind=1, op=op, center=c, v3=(0, 0, 1), p=[r, 0.0, 2 * hh]))
                else:
                    prims.append(dict(kind=2, op=op, center=c, p=list(2 * rng.uniform(0.02, 0.12, 3))))
            h = np.float32(1.0 / (edge - 1))
            reqs.append(("csg", (primitives_to_device(prims, device), k, make_frame((0, 0, 0), (h, h, h))), shape))
        arrivals.append(t)
    return arrivals, reqs, resident


def serve_stream(arrivals, reqs, lanes, pool_bytes=64 << 30, host_bytes=16 << 30, saturate=False):
    """Runs the stream through a gcm_server; returns latency and throughput."""
    from gpucadforam_gb300.mesher import Server

    srv = Server(lanes=lanes, device_pool_bytes=pool_bytes, host_pool_bytes=host_bytes,
                 queue_capacity=max(64, len(reqs) + 1))
    done = {}
    t_sub = {}
    lock = threading.Lock()

    def submitter():
        t0 = time.perf_counter()
        for i, (arr, r) in enumerate(zip(arrivals, reqs)):
            if not saturate:
                dt = arr - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
            kind, payload, shape = r
            if kind == "lattice":
                rc, tk = srv.submit_lattice(payload, shape, 0.0, i)
            else:
                rc, tk = srv.submit_csg(payload[0], payload[1], payload[2], shape, 0.0, i)
            with lock:
                t_sub[i] = (rc, tk)

    th = threading.Thread(target=submitter)
    th.start()
    n_ok = n_bad = 0
    lat, tdone, tsub, verts = [], [], [], 0
    deadline = time.time() + 600
    while (th.is_alive() or n_ok + n_bad < len(reqs)) and time.time() < deadline:
        for res in srv.poll(timeout_us=20000):
            if res.status == 0:
                n_ok += 1
                lat.append(res.t_done - res.t_submit)
                tdone.append(res.t_done)
                tsub.append(res.t_submit)
                verts += res.total_verts
            else:
                n_bad += 1
            srv.release(res.ticket)
        with lock:
            n_bad += sum(1 for v in t_sub.values() if v[0] != 0)
            t_sub = {k: v for k, v in t_sub.items() if v[0] == 0}
    th.join()
    st = srv.stats()
    srv.close()
    span = (max(tdone) - min(tsub)) if tdone else float("nan")
    lat_ms = np.array(lat) * 1e3
    return {"lanes": lanes, "requests": len(reqs), "completed": n_ok, "failed_or_rejected": n_bad,
            "p50_ms": float(np.percentile(lat_ms, 50)) if n_ok else None,
            "p99_ms": float(np.percentile(lat_ms, 99)) if n_ok else None,
            "meshes_per_s": n_ok / span if n_ok else 0.0, "span_s": span, "verts": int(verts),
            "device_pool_peak_gb": st["device_pool_peak"] / 1e9}


def d2h_copy_rate(streams, total=2 << 30, reps=3):
    """Device -> pinned host copy rate (GB/s) of `total` bytes split over
    `streams` streams: the ceiling of a served stream whose meshes all go to
    host memory."""
    import torch

    src = torch.empty(total, dtype=torch.uint8, device="cuda")
    dst = torch.empty(total, dtype=torch.uint8).pin_memory()
    cuts = [total * i // streams for i in range(streams + 1)]
    ss = [torch.cuda.Stream() for _ in range(streams)]

    def go():
        for i, st in enumerate(ss):
            with torch.cuda.stream(st):
                dst[cuts[i]:cuts[i + 1]].copy_(src[cuts[i]:cuts[i + 1]], non_blocking=True)
        torch.cuda.synchronize()

    go()
    t0 = time.perf_counter()
    for _ in range(reps):
        go()
    dt = (time.perf_counter() - t0) / reps
    del src, dst
    return total / dt / 1e9


def run_served(duration_s=4.0, rate=200.0, lanes=6, seed=SEED + 3):
    arrivals, reqs, resident = served_requests(seed, duration_s, rate)
    served = serve_stream(arrivals, reqs, lanes)
    plain = serve_stream(arrivals, reqs, 1)
    sat_served = serve_stream(arrivals, reqs, lanes, saturate=True)
    sat_plain = serve_stream(arrivals, reqs, 1, saturate=True)
    # the copy floor: every mesh (32 B per vertex) crosses to pinned host memory
    rates = {"1_stream": d2h_copy_rate(1), f"{lanes}_streams": d2h_copy_rate(lanes)}
    best = max(rates.values())
    mesh_bytes = 32 * sat_served["verts"]
    floor = {"d2h_GBs": rates, "mesh_bytes": int(mesh_bytes),
             "copy_bound_meshes_per_s": sat_served["completed"] / (mesh_bytes / (best * 1e9)) if mesh_bytes else None}
    # the same streams with every mesh left in the device pool (a consumer on
    # the GPU takes the result): the GPU's own service rate, no copy floor
    dev_served = serve_stream(arrivals, reqs, lanes, host_bytes=0)
    dev_plain = serve_stream(arrivals, reqs, 1, host_bytes=0)
    dev_sat = serve_stream(arrivals, reqs, lanes, host_bytes=0, saturate=True)
    dev_sat_plain = serve_stream(arrivals, reqs, 1, host_bytes=0, saturate=True)
    device = {"served": dev_served, "plain_one_lane": dev_plain,
              "saturation_meshes_per_s": dev_sat["meshes_per_s"],
              "saturation_plain_meshes_per_s": dev_sat_plain["meshes_per_s"],
              "saturation_speedup": (dev_sat["meshes_per_s"] / dev_sat_plain["meshes_per_s"]
                                     if dev_sat_plain["meshes_per_s"] else None)}
    return {"workload": f"Poisson {rate:g} req/s for {duration_s:g} s, edges log-U[64,512], 70% graded TPMS "
                        f"(blend grading, 8 resident 8^3 grading fields) / 30% CSG (8-64 primitives), 64 GB pool, "
                        f"meshes copied to pinned host memory",
            "offered_rate": rate, "served": served, "plain_one_lane": plain,
            "saturation_meshes_per_s": sat_served["meshes_per_s"],
            "saturation_plain_meshes_per_s": sat_plain["meshes_per_s"],
            "saturation_speedup": (sat_served["meshes_per_s"] / sat_plain["meshes_per_s"]
                                   if sat_plain["meshes_per_s"] else None),
            "copy_floor": floor, "device_resident": device}


def run_gcm(args):
    import torch

    world, rank, local, pg = dist_setup(args)
    torch.cuda.set_device(local)
    from gpucadforam_gb300 import _native as N
    from gpucadforam_gb300.mesher import Context, Lattice, make_grid

    n = args.grid
    period, euler, thick, types = c2_controls()
    origin = ((n - 1) / 2,) * 3
    ctx = Context(local)
    lat = Lattice.from_numpy(0, (N_CTRL,) * 3, period, euler, thick, types, origin, device=f"cuda:{local}")
    s = ctx.lattice_struct(lat)
    grid = make_grid((n, n, n))
    stream = torch.cuda.current_stream()
    cs = C.c_void_p(stream.cuda_stream)
    field = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
    ctx.check(ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), n, n, n, C.c_void_p(field.data_ptr()), cs))
    cnt = ctx.count_field(field, 0.0)
    cap = cnt.total_verts
    pos = torch.empty((cap, 4), dtype=torch.float32, device="cuda")
    norm = torch.empty((cap, 4), dtype=torch.float32, device="cuda")
    d_counts = torch.zeros(4, dtype=torch.int64, device="cuda")
    ctx.reserve(n ** 3)
    vox = (n - 1) ** 3

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        ctx.check(ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), n, n, n, C.c_void_p(field.data_ptr()), cs))
        if ev:
            ev[1].record(stream)
        ctx.check(ctx.lib.gcm_mesh_field_async(ctx.h, C.c_void_p(field.data_ptr()), C.byref(grid), 0.0,
                                               C.c_void_p(pos.data_ptr()), C.c_void_p(norm.data_ptr()), cap,
                                               C.c_void_p(d_counts.data_ptr()), cs))
        if ev:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    chk = d_counts.cpu().numpy().view(np.uint64)
    assert int(chk[1]) == cap and int(chk[2] & 0xFFFFFFFF) == 0, chk

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(pg, torch)
    launches0 = ctx.launches
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t1.record(stream)
    barrier(pg, torch)
    launches = ctx.launches - launches0
    clk = clocks.stop()
    total_ms = t0.elapsed_time(t1)
    field_ms = [e[0].elapsed_time(e[1]) for e in evs]
    mc_ms = [e[1].elapsed_time(e[2]) for e in evs]
    total_ms = allmax(pg, total_ms, torch)
    ms_step = total_ms / args.steps
    value = allsum(pg, vox * args.steps, torch) / (total_ms / 1e3)
    tris = allsum(pg, cap / 3 * args.steps, torch) / (total_ms / 1e3)

    peak, peak_kind = measured_peaks()
    mc_bytes = 4 * n ** 3 + 32 * cap
    mc_avg = statistics.mean(mc_ms) / 1e3
    achieved = mc_bytes / mc_avg / 1e9
    traffic = profile_traffic("mc_mesh_kernel_512")

    # ---- e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        h_period = torch.from_numpy(period).pin_memory()
        h_euler = torch.from_numpy(euler).pin_memory()
        h_thick = torch.from_numpy(thick).pin_memory()
        h_types = torch.from_numpy(types).pin_memory()
        h_pos = torch.empty((cap, 4), dtype=torch.float32).pin_memory()
        h_norm = torch.empty((cap, 4), dtype=torch.float32).pin_memory()
        h_counts = torch.zeros(4, dtype=torch.int64).pin_memory()
        # Two device output buffers: step k's mesh is copied out (positions and
        # normals on two copy streams) while step k+1 computes into the other
        # buffer; a buffer is reused only after its copies have finished.
        bufs = [(pos, norm, torch.zeros(4, dtype=torch.int64, device="cuda")),
                (torch.empty_like(pos), torch.empty_like(norm), torch.zeros(4, dtype=torch.int64, device="cuda"))]
        copy_streams = [torch.cuda.Stream(), torch.cuda.Stream()]
        meshed = [torch.cuda.Event(), torch.cuda.Event()]
        copied = [[torch.cuda.Event(), torch.cuda.Event()] for _ in range(2)]
        n_e2e = [0]

        def e2e_step():
            b = n_e2e[0] % 2
            n_e2e[0] += 1
            d_pos, d_norm, d_cnt = bufs[b]
            lat.period.copy_(h_period, non_blocking=True)
            lat.euler.copy_(h_euler, non_blocking=True)
            lat.thickness.copy_(h_thick, non_blocking=True)
            lat.types.copy_(h_types, non_blocking=True)
            for e in copied[b]:
                stream.wait_event(e)
            ctx.check(ctx.lib.gcm_mesh_lattice_async(ctx.h, C.byref(s), C.byref(grid), 0.0,
                                                     C.c_void_p(d_pos.data_ptr()), C.c_void_p(d_norm.data_ptr()),
                                                     cap, C.c_void_p(d_cnt.data_ptr()), cs))
            meshed[b].record(stream)
            for j, (src, dst) in enumerate(((d_pos, h_pos), (d_norm, h_norm))):
                cst = copy_streams[j]
                cst.wait_event(meshed[b])
                with torch.cuda.stream(cst):
                    dst.copy_(src, non_blocking=True)
                    if j == 0:
                        h_counts.copy_(d_cnt, non_blocking=True)
                copied[b][j].record(cst)

        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        barrier(pg, torch)
        a = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        barrier(pg, torch)
        e2e_s = allmax(pg, time.perf_counter() - a, torch)
        assert int(h_counts[1]) == cap and int(h_counts[2]) == 0
        last = bufs[(n_e2e[0] - 1) % 2][0]
        assert h_pos[:16].numpy().tobytes() == last[:16].cpu().numpy().tobytes()
        del bufs[1]
        h2d = period.nbytes + euler.nbytes + thick.nbytes + types.nbytes
        e2e = {"value": allsum(pg, vox * args.steps, torch) / e2e_s, "unit": "voxels/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(32 * cap + 32),
               "ms_per_step": e2e_s / args.steps * 1e3,
               "overlap": "gcm_mesh_lattice_async into two device buffers: step k+1 computes while step k's "
                          "mesh is copied to pinned host memory"}

    batched = None
    if not args.no_batched:
        batched = run_batched(ctx, args.steps, args.warmup, n_inst=args.batch_instances)
    served = None
    if not args.no_served and rank == 0:
        served = run_served()
    configs = None
    if not args.no_configs:
        configs = run_configs(ctx, args.steps, args.warmup, cpu=(rank == 0 and not args.no_cpu))
    rows = None
    if not args.no_rows:
        rows = run_rows(ctx, args.steps, args.warmup, cpu=(rank == 0 and not args.no_cpu))

    reference_cuda = None
    if rank == 0 and not args.no_reference_cuda:
        ctx.check(ctx.lib.gcm_field_lattice(ctx.h, C.byref(s), n, n, n, C.c_void_p(field.data_ptr()), cs))
        reference_cuda = run_reference_cuda(field, local)

    cpu = None
    if rank == 0 and not args.no_cpu:
        r = cpu_sample(os.cpu_count() or 1, planes=args.cpu_planes)
        cpu = {"value": r["voxels_per_s"], "unit": "voxels/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"oracle OpenMP field + marching cubes on a centred z-slab of {args.cpu_planes} of {n} "
                         f"sample planes"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded control grid)",
                "config": workload_config(n), "tris_per_s": tris, "verts_per_step": cap,
                "active_voxels": cnt.active_voxels,
                "kernels_ms": {"lattice_rows_kernel": statistics.mean(field_ms),
                               "mc_mesh_kernel": statistics.mean(mc_ms)},
                "reference_cuda": reference_cuda,
                "roofline": {"bound": "hbm", "kernel": "mc_mesh_kernel", "achieved": achieved, "peak": peak,
                             "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                             "algorithmic_bytes": mc_bytes, "traffic": traffic},
                "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(launches),
                "batched": batched, "served": served, "configs": configs, "rows": rows}
        print(json.dumps(line))
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gcm", "reference"], default="gcm")
    ap.add_argument("--grid", type=int, default=N_GRID)
    ap.add_argument("--cpu-planes", type=int, default=256)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--no-rows", action="store_true", help="skip the retained-CSG, band and .obj lines")
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip timing the reference's own marching-cubes kernels on this GPU")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gcm(args)


if __name__ == "__main__":
    sys.exit(main())
