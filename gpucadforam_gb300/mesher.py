"""Python front end over the C ABI, with torch tensors as device buffers.

torch supplies device memory and streams only; every computation is a call into
libgcm.so.  Names follow the reference's operations (classify, scan, compact,
generate, normalise, mesh) so tests read like the reference's own pipeline
(src/Isosurface.cu:401-572).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N


@dataclass
class Counts:
    active_voxels: int
    total_verts: int
    status: int


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def make_grid(shape_zyx, voxel_size=(1.0, 1.0, 1.0), grid_center=(0.0, 0.0, 0.0)):
    nz, ny, nx = shape_zyx
    return N.GcmGrid(nx, ny, nz, (C.c_float * 3)(*voxel_size), (C.c_float * 3)(*grid_center))


class Context:
    """One gcm_ctx: scratch owner for a stream of calls (not thread-safe)."""

    def __init__(self, device: int = 0):
        self.lib = N.load()
        self.device = device
        h = C.c_void_p()
        rc = self.lib.gcm_ctx_create(device, C.byref(h))
        if rc != 0:
            raise N.GcmError(rc, "gcm_ctx_create failed")
        self.h = h

    def close(self):
        if self.h:
            self.lib.gcm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def check(self, rc, allow=()):
        if rc != 0 and rc not in allow:
            raise N.GcmError(rc, self.lib.gcm_ctx_last_error(self.h).decode())
        return rc

    @property
    def launches(self) -> int:
        return int(self.lib.gcm_ctx_launch_count(self.h))

    def set_wait_limit(self, ns: int):
        self.check(self.lib.gcm_ctx_set_wait_limit(self.h, int(ns)))

    def reserve(self, max_points: int):
        self.check(self.lib.gcm_ctx_reserve(self.h, int(max_points)))

    def set_mesh_path(self, path: str):
        """'auto' (sparse for CSG scenes), 'fused' or 'sparse' plain extraction."""
        self.check(self.lib.gcm_ctx_set_mesh_path(self.h, {"auto": 0, "fused": 1, "sparse": 2}[path]))

    def set_primitive_arith(self, reference_exact: bool):
        """CSG primitive fields bit for bit as the reference's kernels (powf
        squares) instead of the default correctly rounded squares."""
        self.check(self.lib.gcm_ctx_set_primitive_arith(self.h, 1 if reference_exact else 0))

    def set_launch_shape(self, threads: int, tile_voxels: int):
        self.check(self.lib.gcm_ctx_set_launch_shape(self.h, int(threads), int(tile_voxels)))

    # ------------------------------------------------------------ fused mesh
    def count_field(self, field, iso, stream=None) -> Counts:
        g = make_grid(field.shape)
        c = N.GcmCounts()
        self.check(self.lib.gcm_count_field(self.h, _ptr(field), C.byref(g), float(iso), C.byref(c), _stream(stream)))
        return Counts(c.active_voxels, c.total_verts, c.status)

    def mesh_field(self, field, iso, voxel_size=(1, 1, 1), grid_center=(0, 0, 0), capacity=None, pos=None, norm=None,
                   stream=None, allow_overflow=False):
        """Fused single-pass extraction.  Without buffers, counts first and
        allocates the exact output."""
        assert field.is_cuda and field.dtype == torch.float32 and field.dim() == 3
        if pos is None:
            if capacity is None:
                capacity = self.count_field(field, iso, stream).total_verts
            pos = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=field.device)
            norm = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=field.device)
        elif capacity is None:
            capacity = pos.shape[0]
        g = make_grid(field.shape, voxel_size, grid_center)
        c = N.GcmCounts()
        rc = self.lib.gcm_mesh_field(self.h, _ptr(field), C.byref(g), float(iso), _ptr(pos), _ptr(norm), int(capacity),
                                     C.byref(c), _stream(stream))
        self.check(rc, allow=(N.GCM_ERR_OUTPUT_OVERFLOW,) if allow_overflow else ())
        n = int(c.total_verts)
        return pos[: min(n, capacity)], norm[: min(n, capacity)], Counts(c.active_voxels, c.total_verts, c.status)

    def mesh_field_async(self, field, iso, pos, norm, d_counts, voxel_size=(1, 1, 1), grid_center=(0, 0, 0),
                         stream=None):
        g = make_grid(field.shape, voxel_size, grid_center)
        self.check(self.lib.gcm_mesh_field_async(self.h, _ptr(field), C.byref(g), float(iso), _ptr(pos), _ptr(norm),
                                                 int(pos.shape[0]), _ptr(d_counts), _stream(stream)))

    def mesh_band(self, label, norm_field, iso, lo, hi, voxel_size=(1, 1, 1), grid_center=(0, 0, 0), capacity=None,
                  stream=None):
        if capacity is None:
            capacity = self.count_field(label, iso, stream).total_verts
        pos = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=label.device)
        norm = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=label.device)
        g = make_grid(label.shape, voxel_size, grid_center)
        c = N.GcmCounts()
        self.check(self.lib.gcm_mesh_band(self.h, _ptr(label), _ptr(norm_field), C.byref(g), float(iso), float(lo),
                                          float(hi), _ptr(pos), _ptr(norm), int(capacity), C.byref(c),
                                          _stream(stream)))
        n = int(c.total_verts)
        return pos[:n], norm[:n], Counts(c.active_voxels, c.total_verts, c.status)

    # ------------------------------------------------------------ staged form
    def classify(self, field, iso, stream=None):
        nz, ny, nx = field.shape
        nv = (nx - 1) * (ny - 1) * (nz - 1)
        verts = torch.empty(nv, dtype=torch.int32, device=field.device)
        occ = torch.empty(nv, dtype=torch.int32, device=field.device)
        cube = torch.empty(nv, dtype=torch.uint8, device=field.device)
        g = make_grid(field.shape)
        self.check(self.lib.gcm_mc_classify(self.h, _ptr(field), C.byref(g), float(iso), _ptr(verts), _ptr(occ),
                                            _ptr(cube), _stream(stream)))
        return verts, occ, cube

    def scan(self, values, stream=None):
        out = torch.empty_like(values)
        tot = C.c_uint64(0)
        self.check(self.lib.gcm_scan_exclusive_u32(self.h, _ptr(values), _ptr(out), values.numel(), C.byref(tot),
                                                   _stream(stream)))
        return out, int(tot.value)

    def compact(self, occ, occ_scan, active, stream=None):
        out = torch.zeros(max(active, 1), dtype=torch.int32, device=occ.device)
        self.check(self.lib.gcm_mc_compact(self.h, _ptr(occ), _ptr(occ_scan), occ.numel(), _ptr(out), _stream(stream)))
        return out[:active]

    def generate(self, field, iso, compacted, verts_scan, total, voxel_size=(1, 1, 1), grid_center=(0, 0, 0),
                 stream=None):
        pos = torch.empty((max(total, 1), 4), dtype=torch.float32, device=field.device)
        norm = torch.empty((max(total, 1), 4), dtype=torch.float32, device=field.device)
        g = make_grid(field.shape, voxel_size, grid_center)
        self.check(self.lib.gcm_mc_generate(self.h, _ptr(field), C.byref(g), float(iso), _ptr(compacted),
                                            compacted.numel(), _ptr(verts_scan), _ptr(pos), _ptr(norm), int(total),
                                            _stream(stream)))
        return pos[:total], norm[:total]

    # ------------------------------------------------------------ fields
    def unit_cell(self, tpms_type, nx, ny, nz, stream=None):
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=f"cuda:{self.device}")
        self.check(self.lib.gcm_field_unit_cell(self.h, int(tpms_type), nx, ny, nz, _ptr(out), _stream(stream)))
        return out

    def normalise_band(self, field, lo, hi, stream=None):
        nz, ny, nx = field.shape
        label = torch.empty_like(field)
        nf = torch.empty_like(field)
        mm = (C.c_float * 2)()
        self.check(self.lib.gcm_normalise_band(self.h, _ptr(field), nx, ny, nz, float(lo), float(hi), _ptr(label),
                                               _ptr(nf), mm, _stream(stream)))
        return label, nf, (mm[0], mm[1])

    def normalise_range(self, field, range_lo, range_span, out=None, stream=None):
        """Min/max map into [range_lo, range_lo + range_span] (in place when out is field)."""
        if out is None:
            out = torch.empty_like(field)
        mm = (C.c_float * 2)()
        self.check(self.lib.gcm_normalise_range(self.h, _ptr(field), _ptr(out), field.numel(), float(range_lo),
                                                float(range_span), mm, _stream(stream)))
        return out, (mm[0], mm[1])

    def svl_period_field(self, shape_zyx, spacing, mean, axis="z", stream=None):
        nz, ny, nx = shape_zyx
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=f"cuda:{self.device}")
        self.check(self.lib.gcm_svl_period_field(self.h, _ptr(out), nx, ny, nz, *(float(v) for v in spacing),
                                                 *(float(v) for v in mean), axis.encode(), _stream(stream)))
        return out

    def lattice_mask(self, lattice, acc=None, primitive=None, fixed=False, dynamic=False, stream=None):
        """In place: lattice samples outside the retained model (fixed) or the
        live primitive (dynamic) become FLT_MAX."""
        nz, ny, nx = lattice.shape
        self.check(self.lib.gcm_lattice_mask(self.h, _ptr(acc) if acc is not None else None,
                                             _ptr(primitive) if primitive is not None else None, _ptr(lattice),
                                             nx, ny, nz, int(bool(fixed)), int(bool(dynamic)), _stream(stream)))
        return lattice

    def lattice_struct(self, lat):  # noqa: D401 - also used unbound by Server
        return N.GcmLattice(lat.mode, lat.ctrl[0], lat.ctrl[1], lat.ctrl[2], _ptr(lat.period), _ptr(lat.euler),
                            _ptr(lat.thickness), _ptr(lat.types), (C.c_float * 3)(*lat.origin))

    def lattice_field(self, lat, shape_zyx, stream=None):
        nz, ny, nx = shape_zyx
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=f"cuda:{self.device}")
        s = self.lattice_struct(lat)
        self.check(self.lib.gcm_field_lattice(self.h, C.byref(s), nx, ny, nz, _ptr(out), _stream(stream)))
        return out

    def mesh_lattice(self, lat, shape_zyx, iso, voxel_size=(1, 1, 1), grid_center=(0, 0, 0), pos=None, norm=None,
                     stream=None, allow_overflow=False):
        s = self.lattice_struct(lat)
        g = make_grid(shape_zyx, voxel_size, grid_center)
        c = N.GcmCounts()
        rc = self.lib.gcm_mesh_lattice(self.h, C.byref(s), C.byref(g), float(iso), _ptr(pos), _ptr(norm),
                                       int(pos.shape[0]) if pos is not None else 0, C.byref(c), _stream(stream))
        self.check(rc, allow=(N.GCM_ERR_OUTPUT_OVERFLOW,) if allow_overflow or pos is None else ())
        return Counts(c.active_voxels, c.total_verts, c.status)

    def mesh_lattice_async(self, lat, shape_zyx, iso, pos, norm, d_counts, voxel_size=(1, 1, 1),
                           grid_center=(0, 0, 0), stream=None):
        """Field + fused mesh, stream-ordered; counts go to d_counts (4 x int64 on the device)."""
        s = self.lattice_struct(lat)
        g = make_grid(shape_zyx, voxel_size, grid_center)
        self.check(self.lib.gcm_mesh_lattice_async(self.h, C.byref(s), C.byref(g), float(iso), _ptr(pos), _ptr(norm),
                                                   int(pos.shape[0]), _ptr(d_counts), _stream(stream)))

    def csg_field(self, prims_dev, n_prims, frame, shape_zyx, stream=None):
        nz, ny, nx = shape_zyx
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=f"cuda:{self.device}")
        self.check(self.lib.gcm_field_csg(self.h, _ptr(prims_dev), n_prims, C.byref(frame), nx, ny, nz, _ptr(out),
                                          _stream(stream)))
        return out

    # ------------------------------------------------- spatially variant lattices
    def svl_coefficients(self, unit_type, unit_n=61, rng=2, stream=None):
        """(2 rng + 1)^3 complex Fourier coefficients of a unit cell, as a
        complex64 tensor in the reference's order (i fastest)."""
        w = 2 * rng + 1
        out = torch.empty((w ** 3, 2), dtype=torch.float32, device=f"cuda:{self.device}")
        self.check(self.lib.gcm_svl_coefficients(self.h, int(unit_type), int(unit_n), int(rng), _ptr(out),
                                                 _stream(stream)))
        return out

    def svl_lattice(self, shape_xyz, coeff, kind="n", period_type=0, period=8.0, periods=(8.0, 8.0, 8.0),
                    d_period=None, spacing=(1.0, 1.0, 1.0), lcon=0.0, lcon_1=0.0, sinewave_z=False, rng=2,
                    n_coeff=62, max_iter=500, end_res=0.01, svl=None, want_phase=False, stream=None):
        """Adds the lattice of the first n_coeff coefficients to svl (created
        zeroed when None) on the 2x grid; returns (svl[2nz, 2ny, 2nx],
        iterations per solve, phases or None)."""
        nx, ny, nz = shape_xyz
        dev = f"cuda:{self.device}"
        if svl is None:
            svl = torch.zeros((2 * nz, 2 * ny, 2 * nx), dtype=torch.float32, device=dev)
        phase = torch.empty((n_coeff, nz, ny, nx), dtype=torch.float32, device=dev) if want_phase else None
        p = N.GcmSvlParams(nx, ny, nz, *spacing, ord(kind), period_type, period, *periods, lcon, lcon_1,
                           1 if sinewave_z else 0, rng, n_coeff, max_iter, end_res)
        iters = (C.c_uint32 * n_coeff)()
        self.check(self.lib.gcm_svl_lattice(self.h, C.byref(p), _ptr(d_period), _ptr(coeff), _ptr(svl), _ptr(phase),
                                            iters, _stream(stream)))
        return svl, list(iters), phase

    # ------------------------------------------------- retained CSG editing
    CSG_OPS = {"union": 0, "subtract": 1, "intersect": 2}

    def csg_accumulator(self, shape_zyx):
        """An empty retained model: int32 sign + 3 float32 fractions per sample,
        as an (nz, ny, nx, 4) int32 tensor (the fractions are float bits)."""
        return torch.zeros((*shape_zyx, 4), dtype=torch.int32, device=f"cuda:{self.device}")

    def csg_retain(self, acc, field, op="union", iso=0.0, band=None, stream=None):
        """Fold a field (or, with band = (lo, hi), a lattice band) into acc."""
        nz, ny, nx = field.shape
        assert tuple(acc.shape[:3]) == (nz, ny, nx) and acc.shape[3] == 4
        if band is None:
            self.check(self.lib.gcm_csg_retain(self.h, _ptr(acc), _ptr(field), nx, ny, nz, float(iso),
                                               self.CSG_OPS.get(op, op), _stream(stream)))
        else:
            self.check(self.lib.gcm_csg_retain_band(self.h, _ptr(acc), _ptr(field), nx, ny, nz, float(iso),
                                                    float(band[0]), float(band[1]), self.CSG_OPS.get(op, op),
                                                    _stream(stream)))

    def count_retained(self, acc, field=None, op="union", iso=0.0, stream=None) -> Counts:
        g = make_grid(acc.shape[:3])
        c = N.GcmCounts()
        self.check(self.lib.gcm_count_retained(self.h, _ptr(acc), _ptr(field), self.CSG_OPS.get(op, op), C.byref(g),
                                               float(iso), C.byref(c), _stream(stream)))
        return Counts(c.active_voxels, c.total_verts, c.status)

    def mesh_retained(self, acc, field=None, op="union", iso=0.0, voxel_size=(1, 1, 1), grid_center=(0, 0, 0),
                      capacity=None, stream=None):
        """Region mesh of the accumulator (field None) or the live model with
        one more primitive field combined by op."""
        if capacity is None:
            capacity = self.count_retained(acc, field, op, iso, stream).total_verts
        dev = acc.device
        pos = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=dev)
        norm = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=dev)
        g = make_grid(acc.shape[:3], voxel_size, grid_center)
        c = N.GcmCounts()
        self.check(self.lib.gcm_mesh_retained(self.h, _ptr(acc), _ptr(field), self.CSG_OPS.get(op, op), C.byref(g),
                                              float(iso), _ptr(pos), _ptr(norm), int(capacity), C.byref(c),
                                              _stream(stream)))
        n = int(c.total_verts)
        return pos[:n], norm[:n], Counts(c.active_voxels, c.total_verts, c.status)

    def mesh_lattice_preview(self, lattice, band, acc=None, field=None, op="union", iso=0.0, voxel_size=(1, 1, 1),
                             grid_center=(0, 0, 0), stream=None):
        """Lattice preview mesh: with field the "fixed" form (field and the
        lattice band), with acc the "dynamic" form (model and band)."""
        g = make_grid(lattice.shape, voxel_size, grid_center)
        c = N.GcmCounts()
        opn = self.CSG_OPS.get(op, op)
        args = (self.h, _ptr(acc), _ptr(field), _ptr(lattice), opn, C.byref(g), float(iso), float(band[0]),
                float(band[1]))
        self.check(self.lib.gcm_mesh_lattice_preview(*args, None, None, 0, C.byref(c), _stream(stream)))
        cap = int(c.total_verts)
        pos = torch.empty((max(cap, 1), 4), dtype=torch.float32, device=lattice.device)
        norm = torch.empty((max(cap, 1), 4), dtype=torch.float32, device=lattice.device)
        self.check(self.lib.gcm_mesh_lattice_preview(*args, _ptr(pos), _ptr(norm), max(cap, 1), C.byref(c),
                                                     _stream(stream)))
        n = int(c.total_verts)
        return pos[:n], norm[:n], Counts(c.active_voxels, c.total_verts, c.status)

    def mesh_csg_async(self, prims_dev, n_prims, frame, shape_zyx, iso, pos, norm, d_counts, voxel_size=(1, 1, 1),
                       grid_center=(0, 0, 0), stream=None):
        """gcm_mesh_csg_async: counts into the int64[4] device tensor d_counts."""
        g = make_grid(shape_zyx, voxel_size, grid_center)
        self.check(self.lib.gcm_mesh_csg_async(self.h, _ptr(prims_dev), n_prims, C.byref(frame), C.byref(g), float(iso),
                                               _ptr(pos), _ptr(norm), int(pos.shape[0]), _ptr(d_counts),
                                               _stream(stream)))

    def mesh_csg(self, prims_dev, n_prims, frame, shape_zyx, iso, voxel_size=(1, 1, 1), grid_center=(0, 0, 0),
                 pos=None, norm=None, stream=None, allow_overflow=False):
        g = make_grid(shape_zyx, voxel_size, grid_center)
        c = N.GcmCounts()
        rc = self.lib.gcm_mesh_csg(self.h, _ptr(prims_dev), n_prims, C.byref(frame), C.byref(g), float(iso), _ptr(pos),
                                   _ptr(norm), int(pos.shape[0]) if pos is not None else 0, C.byref(c),
                                   _stream(stream))
        self.check(rc, allow=(N.GCM_ERR_OUTPUT_OVERFLOW,) if allow_overflow or pos is None else ())
        return Counts(c.active_voxels, c.total_verts, c.status)


@dataclass
class Lattice:
    """Graded lattice description with device control arrays."""
    mode: int
    ctrl: tuple
    period: torch.Tensor
    euler: torch.Tensor | None
    thickness: torch.Tensor | None
    types: torch.Tensor
    origin: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def from_numpy(mode, ctrl, period, euler=None, thickness=None, types=None, origin=(0, 0, 0), device="cuda"):
        n = int(np.prod(ctrl))
        t = lambda a, dt: None if a is None else torch.from_numpy(np.ascontiguousarray(a, dt).reshape(-1)).to(device)
        if types is None:
            types = np.zeros(n, np.uint8)
        return Lattice(mode, tuple(int(c) for c in ctrl), t(period, np.float32), t(euler, np.float32),
                       t(thickness, np.float32), t(types, np.uint8), tuple(float(o) for o in origin))


def primitives_to_device(prims, device="cuda"):
    """prims: sequence of dicts (kind, op, flag, center, v3, p) -> device array."""
    arr = (N.GcmPrimitive * max(len(prims), 1))()
    for i, q in enumerate(prims):
        pp = list(q.get("p", ())) + [0.0] * (6 - len(q.get("p", ())))
        arr[i] = N.GcmPrimitive(q["kind"], q.get("op", 0), q.get("flag", 0), 0, (C.c_float * 3)(*q["center"]),
                                (C.c_float * 3)(*q.get("v3", (0, 0, 0))), (C.c_float * 6)(*pp))
    raw = np.frombuffer(bytes(arr), np.uint8).copy()
    return torch.from_numpy(raw).to(device)


def make_frame(origin, spacing):
    return N.GcmFrame((C.c_float * 3)(*origin), (C.c_float * 3)(*spacing))


class Batch:
    """Many graded lattices meshed in one field launch + one fused launch."""

    def __init__(self, ctx: Context, lattices, shapes_zyx, isos=None, voxel_sizes=None, grid_centers=None):
        self.ctx = ctx
        self.lattices = list(lattices)  # keeps the device control arrays alive
        n = len(self.lattices)
        arr = (N.GcmBatchInstance * n)()
        for i, lat in enumerate(self.lattices):
            vs = voxel_sizes[i] if voxel_sizes is not None else (1.0, 1.0, 1.0)
            gc = grid_centers[i] if grid_centers is not None else (0.0, 0.0, 0.0)
            arr[i] = N.GcmBatchInstance(ctx.lattice_struct(lat), make_grid(shapes_zyx[i], vs, gc),
                                        float(isos[i]) if isos is not None else 0.0, 0)
        self.n = n
        self.shapes = [tuple(s) for s in shapes_zyx]
        h = C.c_void_p()
        ctx.check(ctx.lib.gcm_batch_create(ctx.h, arr, n, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.ctx.lib.gcm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def count(self, stream=None):
        verts = (C.c_uint64 * self.n)()
        active = (C.c_uint64 * self.n)()
        c = N.GcmCounts()
        self.ctx.check(self.ctx.lib.gcm_batch_count(self.h, verts, active, C.byref(c), _stream(stream)))
        return list(verts), list(active), Counts(c.active_voxels, c.total_verts, c.status)

    def buffers(self, capacity, device="cuda"):
        pos = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=device)
        norm = torch.empty((max(capacity, 1), 4), dtype=torch.float32, device=device)
        offsets = torch.zeros(self.n + 1, dtype=torch.int64, device=device)
        counts = torch.zeros(4, dtype=torch.int64, device=device)
        return pos, norm, offsets, counts

    def mesh_async(self, pos, norm, offsets, counts, capacity=None, stream=None, graph=False):
        cap = pos.shape[0] if capacity is None else capacity
        fn = self.ctx.lib.gcm_batch_mesh_graph if graph else self.ctx.lib.gcm_batch_mesh_async
        self.ctx.check(fn(self.h, _ptr(pos), _ptr(norm), int(cap), _ptr(offsets), _ptr(counts), _stream(stream)))

    def tune(self, pos, norm, cache_path=None, stream=None):
        t = C.c_int(0)
        v = C.c_uint32(0)
        self.ctx.check(self.ctx.lib.gcm_batch_tune(self.h, _ptr(pos), _ptr(norm), int(pos.shape[0]),
                                                   cache_path.encode() if cache_path else None, C.byref(t),
                                                   C.byref(v), _stream(stream)))
        return int(t.value), int(v.value)


def random_batch_lattices(n, seed, dims=(32, 256), period=(8.0, 48.0), ctrl=8, blend_every=0, device="cuda"):
    """Config-C4-style instances: dims U{32..256} per axis, one lattice type and
    one period per instance, thickness and rotation graded on a ctrl^3 grid.
    Returns (lattices, shapes_zyx)."""
    rng = np.random.default_rng(seed)
    lats, shapes = [], []
    nc = ctrl ** 3
    for i in range(n):
        nx, ny, nz = (int(v) for v in rng.integers(dims[0], dims[1] + 1, 3))
        typ = int(rng.choice([0, 1, 5]))
        per = float(rng.uniform(*period))
        mode = 1 if (blend_every and i % blend_every == blend_every - 1) else 0
        lats.append(Lattice.from_numpy(
            mode, (ctrl, ctrl, ctrl), np.full(nc, per, np.float32),
            rng.uniform(-np.pi / 4, np.pi / 4, 3 * nc).astype(np.float32),
            rng.uniform(-0.6, 0.6, nc).astype(np.float32), np.full(nc, typ, np.uint8),
            origin=((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2), device=device))
        shapes.append((nz, ny, nx))
    return lats, shapes


class Server:
    """Continuous-batching mesh server (gcm_server)."""

    def __init__(self, lanes=4, device_pool_bytes=8 << 30, host_pool_bytes=4 << 30, queue_capacity=4096,
                 fault_flags=0, fault_param=0, device=0):
        self.lib = N.load()
        cfg = N.GcmServerConfig(device, lanes, queue_capacity, fault_flags, device_pool_bytes, host_pool_bytes,
                                fault_param, 0)
        h = C.c_void_p()
        rc = self.lib.gcm_server_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise N.GcmError(rc, "gcm_server_create failed")
        self.h = h
        self._keep = {}

    def close(self):
        if self.h:
            self.lib.gcm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def now(self):
        return float(self.lib.gcm_server_now(self.h))

    def submit_lattice(self, lat, shape_zyx, iso=0.0, tag=0, ctx=None):
        r = N.GcmRequest()
        r.kind = 0
        r.lattice = Context.lattice_struct(None, lat)
        r.grid = make_grid(shape_zyx)
        r.iso = float(iso)
        r.user_tag = tag
        return self._submit(r, lat)

    def submit_csg(self, prims_dev, n_prims, frame, shape_zyx, iso=0.0, tag=0):
        r = N.GcmRequest()
        r.kind = 1
        r.n_prims = n_prims
        r.d_prims = prims_dev.data_ptr()
        r.frame = frame
        r.grid = make_grid(shape_zyx)
        r.iso = float(iso)
        r.user_tag = tag
        return self._submit(r, prims_dev)

    def submit_field(self, field, iso=0.0, tag=0):
        r = N.GcmRequest()
        r.kind = 2
        r.d_field = field.data_ptr()
        r.grid = make_grid(field.shape)
        r.iso = float(iso)
        r.user_tag = tag
        return self._submit(r, field)

    def _submit(self, r, keep):
        t = C.c_uint64(0)
        rc = self.lib.gcm_server_submit(self.h, C.byref(r), C.byref(t))
        if rc != 0:
            return rc, None
        self._keep[int(t.value)] = keep
        return 0, int(t.value)

    def poll(self, max_results=256, timeout_us=100000):
        arr = (N.GcmResult * max_results)()
        n = C.c_uint32(0)
        rc = self.lib.gcm_server_poll(self.h, arr, max_results, C.byref(n), int(timeout_us))
        if rc != 0:
            raise N.GcmError(rc, "gcm_server_poll failed")
        return [arr[i] for i in range(n.value)]

    def result_arrays(self, res):
        """(pos, norm) numpy copies of a completed host result."""
        n = int(res.total_verts)
        if not res.on_host or n == 0:
            return np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32)
        pos = np.ctypeslib.as_array(C.cast(res.pos, C.POINTER(C.c_float)), shape=(n, 4)).copy()
        norm = np.ctypeslib.as_array(C.cast(res.norm, C.POINTER(C.c_float)), shape=(n, 4)).copy()
        return pos, norm

    def release(self, ticket):
        self._keep.pop(ticket, None)
        return self.lib.gcm_server_release(self.h, int(ticket))

    def cancel(self, ticket):
        return self.lib.gcm_server_cancel(self.h, int(ticket))

    def stats(self):
        s = N.GcmServerStats()
        self.lib.gcm_server_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def drain(self, tickets, timeout_s=120.0):
        """Waits for the given tickets; returns {ticket: (result, pos, norm)}."""
        want = set(tickets)
        out = {}
        t0 = time.time()
        while want and time.time() - t0 < timeout_s:
            for r in self.poll():
                if r.ticket in want:
                    pos, norm = self.result_arrays(r)
                    out[r.ticket] = (r, pos, norm)
                    want.discard(r.ticket)
                    self.release(r.ticket)
        return out
