"""ctypes front end of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``, to check and time against; the product
package never imports it.  Every function mirrors one reference routine; see oracle.cpp for
the file:line each one restates.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

F32P = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
U8P = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class OrcLattice(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("cx", C.c_uint32), ("cy", C.c_uint32), ("cz", C.c_uint32),
                ("period", C.c_void_p), ("euler", C.c_void_p), ("thickness", C.c_void_p), ("type", C.c_void_p),
                ("origin", C.c_float * 3)]


class OrcPrim(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("op", C.c_uint32), ("flag", C.c_uint32), ("pad", C.c_uint32),
                ("center", C.c_float * 3), ("v3", C.c_float * 3), ("p", C.c_float * 6)]


class OrcSvl(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("dx", C.c_float), ("dy", C.c_float),
                ("dz", C.c_float), ("kind", C.c_uint32), ("period_type", C.c_uint32), ("period", C.c_float),
                ("period_x", C.c_float), ("period_y", C.c_float), ("period_z", C.c_float), ("lcon", C.c_float),
                ("lcon_1", C.c_float), ("sinewave_z", C.c_uint32), ("range", C.c_uint32), ("n_coeff", C.c_uint32),
                ("max_iter", C.c_uint32), ("end_res", C.c_float)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_default_arith.restype = C.c_uint32
        L.orc_mc_classify.argtypes = [F32P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, U32P, U32P, U8P]
        L.orc_scan_exclusive_u32.argtypes = [U32P, U32P, C.c_uint64]
        L.orc_scan_exclusive_u32.restype = C.c_uint64
        L.orc_mc_compact.argtypes = [U32P, U32P, C.c_uint64, U32P]
        L.orc_mc_generate.argtypes = [F32P, C.c_uint32, C.c_uint32, C.c_uint32, F32P, F32P, C.c_float, U32P,
                                      C.c_uint64, U32P, C.c_uint64, F32P, F32P, C.c_uint32]
        L.orc_mc_generate_band.argtypes = [F32P, F32P, C.c_uint32, C.c_uint32, C.c_uint32, F32P, F32P, C.c_float,
                                           C.c_float, C.c_float, U32P, C.c_uint64, U32P, C.c_uint64, F32P, F32P,
                                           C.c_uint32]
        L.orc_mesh_field.argtypes = [F32P, C.c_uint32, C.c_uint32, C.c_uint32, F32P, F32P, C.c_float, C.c_void_p,
                                     C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64), C.c_int]
        L.orc_mesh_field.restype = C.c_uint64
        L.orc_unit_cell.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, F32P]
        L.orc_primitive.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, F32P,
                                    F32P, F32P, C.c_uint32, F32P]
        L.orc_lattice_field.argtypes = [C.POINTER(OrcLattice), C.c_uint32, C.c_uint32, C.c_uint32, F32P, C.c_int]
        L.orc_lattice_field_slab.argtypes = [C.POINTER(OrcLattice), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                             C.c_uint32, F32P, C.c_int]
        L.orc_lattice_field64_slab.argtypes = [C.POINTER(OrcLattice), C.c_uint32, C.c_uint32, C.c_uint32,
                                               C.c_uint32, C.c_uint32, F64P, C.c_int]
        L.orc_lattice_field64.argtypes = [C.POINTER(OrcLattice), C.c_uint32, C.c_uint32, C.c_uint32, F64P, C.c_int]
        L.orc_csg_field.argtypes = [C.POINTER(OrcPrim), C.c_uint32, F32P, F32P, C.c_uint32, C.c_uint32, C.c_uint32,
                                    F32P, C.c_int]
        L.orc_csg_field64.argtypes = [C.POINTER(OrcPrim), C.c_uint32, F32P, F32P, C.c_uint32, C.c_uint32,
                                      C.c_uint32, F64P, C.c_int]
        L.orc_svl_period_field.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, F32P, F32P, C.c_char, F32P]
        L.orc_normalise_range.argtypes = [F32P, F32P, C.c_uint64, C.c_float, C.c_float, F32P]
        L.orc_lattice_mask.argtypes = [C.c_void_p, C.c_void_p, F32P, C.c_uint64, C.c_int, C.c_int]
        L.orc_normalise_band.argtypes = [F32P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, F32P, F32P, F32P]
        L.orc_write_obj.argtypes = [F32P, C.c_uint64, C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_write_obj.restype = C.c_int
        L.orc_csg_retain.argtypes = [C.c_void_p, F32P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32]
        L.orc_csg_retain_band.argtypes = [C.c_void_p, F32P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_float,
                                          C.c_float, C.c_uint32]
        L.orc_mesh_retained.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                        F32P, F32P, C.c_float, C.c_void_p, C.c_void_p, C.c_uint64,
                                        C.POINTER(C.c_uint64)]
        L.orc_mesh_retained.restype = C.c_uint64
        L.orc_mesh_lattice_preview.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                               C.c_uint32, C.c_uint32, C.c_uint32, F32P, F32P, C.c_float, C.c_float,
                                               C.c_float, C.c_void_p, C.c_void_p, C.c_uint64,
                                               C.POINTER(C.c_uint64)]
        L.orc_mesh_lattice_preview.restype = C.c_uint64
        L.orc_svl_dft.argtypes = [F32P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, F32P]
        L.orc_svl_rhs.argtypes = [C.POINTER(OrcSvl), C.c_void_p, C.c_uint32, F32P]
        L.orc_svl_cg.argtypes = [C.POINTER(OrcSvl), F32P, F32P]
        L.orc_svl_cg.restype = C.c_uint32
        L.orc_svl_accumulate.argtypes = [C.POINTER(OrcSvl), F32P, F32P, F32P]
        _lib = L
    return _lib


def default_arith() -> int:
    return int(lib().orc_default_arith())


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))


def _dims(field):
    nz, ny, nx = field.shape
    return nx, ny, nz


def mc_classify(field, iso):
    field = np.ascontiguousarray(field, np.float32)
    nx, ny, nz = _dims(field)
    nv = (nx - 1) * (ny - 1) * (nz - 1)
    verts = np.zeros(nv, np.uint32)
    occ = np.zeros(nv, np.uint32)
    cube = np.zeros(nv, np.uint8)
    lib().orc_mc_classify(field, nx, ny, nz, iso, verts, occ, cube)
    return verts, occ, cube


def scan_exclusive(a):
    a = np.ascontiguousarray(a, np.uint32)
    out = np.zeros_like(a)
    total = lib().orc_scan_exclusive_u32(a, out, a.size)
    return out, int(total)


def mc_compact(occ, occ_scan):
    occ = np.ascontiguousarray(occ, np.uint32)
    occ_scan = np.ascontiguousarray(occ_scan, np.uint32)
    active = int(occ_scan[-1] + occ[-1]) if occ.size else 0
    out = np.zeros(max(active, 1), np.uint32)
    lib().orc_mc_compact(occ, occ_scan, occ.size, out)
    return out[:active]


def mc_generate(field, vs, gc, iso, compacted, verts_scan, total, arith=None, capacity=None):
    field = np.ascontiguousarray(field, np.float32)
    nx, ny, nz = _dims(field)
    cap = total if capacity is None else capacity
    pos = np.zeros((max(cap, 1), 4), np.float32)
    norm = np.zeros((max(cap, 1), 4), np.float32)
    comp = np.ascontiguousarray(compacted, np.uint32)
    if comp.size == 0:
        comp = np.zeros(1, np.uint32)
    lib().orc_mc_generate(field, nx, ny, nz, _f3(vs), _f3(gc), iso, comp, len(compacted),
                          np.ascontiguousarray(verts_scan, np.uint32), cap, pos.reshape(-1), norm.reshape(-1),
                          default_arith() if arith is None else arith)
    return pos[:cap], norm[:cap]


def mc_generate_band(label, normf, vs, gc, iso, lo, hi, compacted, verts_scan, total, arith=None):
    label = np.ascontiguousarray(label, np.float32)
    normf = np.ascontiguousarray(normf, np.float32)
    nx, ny, nz = _dims(label)
    pos = np.zeros((max(total, 1), 4), np.float32)
    norm = np.zeros((max(total, 1), 4), np.float32)
    comp = np.ascontiguousarray(compacted, np.uint32)
    if comp.size == 0:
        comp = np.zeros(1, np.uint32)
    lib().orc_mc_generate_band(label, normf, nx, ny, nz, _f3(vs), _f3(gc), iso, lo, hi, comp, len(compacted),
                               np.ascontiguousarray(verts_scan, np.uint32), total, pos.reshape(-1),
                               norm.reshape(-1), default_arith() if arith is None else arith)
    return pos[:total], norm[:total]


def mesh(field, vs, gc, iso):
    """Whole plain pipeline (classify, scans, compact, generate); returns
    (pos, norm, active_voxels) with the reference's vertex order."""
    verts, occ, _ = mc_classify(field, iso)
    occ_scan, active = scan_exclusive(occ)
    verts_scan, total = scan_exclusive(verts)
    comp = mc_compact(occ, occ_scan)
    pos, norm = mc_generate(field, vs, gc, iso, comp, verts_scan, total)
    return pos, norm, active


def mesh_band(label, normf, vs, gc, iso, lo, hi):
    verts, occ, _ = mc_classify(label, iso)
    occ_scan, active = scan_exclusive(occ)
    verts_scan, total = scan_exclusive(verts)
    comp = mc_compact(occ, occ_scan)
    pos, norm = mc_generate_band(label, normf, vs, gc, iso, lo, hi, comp, verts_scan, total)
    return pos, norm, active


def mesh_field_omp(field, vs, gc, iso, capacity, threads=0):
    """Multi-threaded whole pipeline (the timed CPU baseline).  Returns
    (total_verts, active_voxels, pos, norm)."""
    field = np.ascontiguousarray(field, np.float32)
    nx, ny, nz = _dims(field)
    pos = np.empty((max(capacity, 1), 4), np.float32)
    norm = np.empty((max(capacity, 1), 4), np.float32)
    act = C.c_uint64(0)
    total = lib().orc_mesh_field(field, nx, ny, nz, _f3(vs), _f3(gc), iso, pos.ctypes.data, norm.ctypes.data,
                                 capacity, C.byref(act), threads)
    return int(total), int(act.value), pos, norm


def unit_cell(tpms_type, nx, ny, nz):
    out = np.zeros(nx * ny * nz, np.float32)
    lib().orc_unit_cell(tpms_type, nx, ny, nz, out)
    return out.reshape(nz, ny, nx)


def primitive(kind, n, d, center, v3, p, flag):
    nx, ny, nz = n
    out = np.zeros(nx * ny * nz, np.float32)
    pp = np.zeros(6, np.float32)
    pp[: len(p)] = p
    lib().orc_primitive(kind, nx, ny, nz, d[0], d[1], d[2], _f3(center), _f3(v3), pp, flag, out)
    return out.reshape(nz, ny, nx)


def _lattice_struct(mode, ctrl, period, euler, thickness, types, origin):
    cx, cy, cz = ctrl
    keep = []

    def ptr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a.ctypes.data

    s = OrcLattice(mode, cx, cy, cz, ptr(period, np.float32), ptr(euler, np.float32), ptr(thickness, np.float32),
                   ptr(types, np.uint8), (C.c_float * 3)(*origin))
    return s, keep


def lattice_field(n, mode, ctrl, period, euler=None, thickness=None, types=None, origin=(0, 0, 0), threads=0,
                  fp64=False):
    nx, ny, nz = n
    if types is None:
        types = np.zeros(int(np.prod(ctrl)), np.uint8)
    s, keep = _lattice_struct(mode, ctrl, period, euler, thickness, types, origin)
    if fp64:
        out = np.zeros(nx * ny * nz, np.float64)
        lib().orc_lattice_field64(C.byref(s), nx, ny, nz, out, threads)
    else:
        out = np.zeros(nx * ny * nz, np.float32)
        lib().orc_lattice_field(C.byref(s), nx, ny, nz, out, threads)
    del keep
    return out.reshape(nz, ny, nx)


def lattice_slab(n, z0, nplanes, mode, ctrl, period, euler=None, thickness=None, types=None, origin=(0, 0, 0),
                 threads=0, fp64=False):
    """Planes z0..z0+nplanes-1 of the nx*ny*nz lattice field (same control mapping)."""
    nx, ny, nz = n
    if types is None:
        types = np.zeros(int(np.prod(ctrl)), np.uint8)
    s, keep = _lattice_struct(mode, ctrl, period, euler, thickness, types, origin)
    if fp64:
        out = np.zeros(nx * ny * nplanes, np.float64)
        lib().orc_lattice_field64_slab(C.byref(s), nx, ny, nz, z0, nplanes, out, threads)
    else:
        out = np.zeros(nx * ny * nplanes, np.float32)
        lib().orc_lattice_field_slab(C.byref(s), nx, ny, nz, z0, nplanes, out, threads)
    del keep
    return out.reshape(nplanes, ny, nx)


def prim_array(prims):
    """prims: sequence of dicts with kind, op, flag, center, v3, p."""
    arr = (OrcPrim * max(len(prims), 1))()
    for i, q in enumerate(prims):
        pp = list(q.get("p", ())) + [0.0] * (6 - len(q.get("p", ())))
        arr[i] = OrcPrim(q["kind"], q.get("op", 0), q.get("flag", 0), 0, (C.c_float * 3)(*q["center"]),
                         (C.c_float * 3)(*q.get("v3", (0, 0, 0))), (C.c_float * 6)(*pp))
    return arr


def csg_field(prims, n, origin, spacing, threads=0, fp64=False):
    nx, ny, nz = n
    arr = prim_array(prims)
    if fp64:
        out = np.zeros(nx * ny * nz, np.float64)
        lib().orc_csg_field64(arr, len(prims), _f3(origin), _f3(spacing), nx, ny, nz, out, threads)
    else:
        out = np.zeros(nx * ny * nz, np.float32)
        lib().orc_csg_field(arr, len(prims), _f3(origin), _f3(spacing), nx, ny, nz, out, threads)
    return out.reshape(nz, ny, nx)


def svl_period_field(n, d, mean, axis="z"):
    nx, ny, nz = n
    out = np.zeros(nx * ny * nz, np.float32)
    lib().orc_svl_period_field(nx, ny, nz, _f3(d), _f3(mean), axis.encode(), out)
    return out.reshape(nz, ny, nx)


def normalise_range(field, a1, b1):
    f = np.ascontiguousarray(field, np.float32).reshape(-1)
    out = np.empty_like(f)
    mm = np.zeros(2, np.float32)
    lib().orc_normalise_range(f, out, f.size, a1, b1, mm)
    return out.reshape(np.shape(field)), mm


def lattice_mask(lattice, acc=None, prim=None, fixed=False, dynamic=False):
    lat = np.array(lattice, np.float32).reshape(-1)
    a = None if acc is None else np.ascontiguousarray(acc)
    q = None if prim is None else np.ascontiguousarray(prim, np.float32)
    lib().orc_lattice_mask(None if a is None else a.ctypes.data, None if q is None else q.ctypes.data, lat, lat.size,
                           int(bool(fixed)), int(bool(dynamic)))
    return lat.reshape(np.shape(lattice))


def normalise_band(field, lo, hi):
    field = np.ascontiguousarray(field, np.float32)
    nx, ny, nz = _dims(field)
    label = np.zeros_like(field)
    nf = np.zeros_like(field)
    mm = np.zeros(2, np.float32)
    lib().orc_normalise_band(field.reshape(-1), nx, ny, nz, lo, hi, label.reshape(-1), nf.reshape(-1), mm)
    return label, nf, mm


def write_obj(pos, path):
    pos = np.ascontiguousarray(pos, np.float32)
    nv = C.c_uint64(0)
    nf = C.c_uint64(0)
    rc = lib().orc_write_obj(pos.reshape(-1), pos.shape[0], os.fsencode(path), C.byref(nv), C.byref(nf))
    if rc:
        raise OSError(f"orc_write_obj failed ({rc})")
    return int(nv.value), int(nf.value)


CSG_OPS = {"union": 0, "subtract": 1, "intersect": 2}


def csg_accumulator(shape_zyx):
    """Empty retained model: (nz, ny, nx, 4) int32 = sign + 3 fractions (float bits)."""
    return np.zeros((*shape_zyx, 4), np.int32)


def csg_retain(acc, field, op="union", iso=0.0, band=None):
    """classify_copy_Voxel (src/MarchingCubes_kernel.cu:158-447), in place: the
    static mode, or with band = (iso1, iso2) the lattice-band mode with field
    as the lattice."""
    assert acc.dtype == np.int32 and acc.flags.c_contiguous and acc.shape[3] == 4
    field = np.ascontiguousarray(field, np.float32)
    nz, ny, nx = field.shape
    assert acc.shape[:3] == field.shape
    if band is None:
        lib().orc_csg_retain(acc.ctypes.data, field, nx, ny, nz, iso, CSG_OPS.get(op, op))
    else:
        lib().orc_csg_retain_band(acc.ctypes.data, field, nx, ny, nz, iso, float(band[0]), float(band[1]),
                                  CSG_OPS.get(op, op))
    return acc


def mesh_retained(acc, field, op, vs, gc, iso=0.0):
    """Region mesh (field None) or live-model mesh of the accumulator; returns
    (pos, norm, active_voxels)."""
    nz, ny, nx = acc.shape[:3]
    g = None if field is None else np.ascontiguousarray(field, np.float32)
    L = lib()
    act = C.c_uint64(0)
    gp = None if g is None else g.ctypes.data
    total = L.orc_mesh_retained(acc.ctypes.data, gp, CSG_OPS.get(op, op), nx, ny, nz, _f3(vs), _f3(gc), iso,
                                None, None, 0, C.byref(act))
    pos = np.zeros((max(total, 1), 4), np.float32)
    norm = np.zeros((max(total, 1), 4), np.float32)
    L.orc_mesh_retained(acc.ctypes.data, gp, CSG_OPS.get(op, op), nx, ny, nz, _f3(vs), _f3(gc), iso,
                        pos.ctypes.data, norm.ctypes.data, total, C.byref(act))
    return pos[:total], norm[:total], int(act.value)


def mesh_lattice_preview(acc, field, lattice, band, op, vs, gc, iso=0.0):
    """Lattice preview mesh: with field (the primitive field; acc unused) the
    "fixed" form, with field None the "dynamic" form over acc; band = (iso1,
    iso2) on the lattice.  Returns (pos, norm, active_voxels)."""
    nz, ny, nx = lattice.shape
    lat = np.ascontiguousarray(lattice, np.float32)
    f = None if field is None else np.ascontiguousarray(field, np.float32)
    a = np.ascontiguousarray(acc) if acc is not None else np.zeros((nz, ny, nx, 4), np.int32)
    mode = 2 if f is not None else 3
    L = lib()
    act = C.c_uint64(0)
    fp = None if f is None else f.ctypes.data
    args = (a.ctypes.data, fp, lat.ctypes.data, mode, CSG_OPS.get(op, op), nx, ny, nz, _f3(vs), _f3(gc), iso,
            float(band[0]), float(band[1]))
    total = L.orc_mesh_lattice_preview(*args, None, None, 0, C.byref(act))
    pos = np.zeros((max(total, 1), 4), np.float32)
    norm = np.zeros((max(total, 1), 4), np.float32)
    L.orc_mesh_lattice_preview(*args, pos.ctypes.data, norm.ctypes.data, total, C.byref(act))
    return pos[:total], norm[:total], int(act.value)


def svl_params(shape_xyz, kind="n", period_type=0, period=8.0, periods=(8.0, 8.0, 8.0), spacing=(1.0, 1.0, 1.0),
               lcon=0.0, lcon_1=0.0, sinewave_z=False, rng=2, n_coeff=62, max_iter=500, end_res=0.01):
    return OrcSvl(*shape_xyz, *spacing, ord(kind), period_type, period, *periods, lcon, lcon_1,
                  1 if sinewave_z else 0, rng, n_coeff, max_iter, end_res)


def svl_dft(field, rng=2):
    """Unit-cell Fourier coefficients (w^3, 2) float32 in the reference's order."""
    f = np.ascontiguousarray(field, np.float32)
    nz, ny, nx = f.shape
    out = np.zeros(2 * (2 * rng + 1) ** 3, np.float32)
    lib().orc_svl_dft(f, nx, ny, nz, rng, out)
    return out.reshape(-1, 2)


def svl_rhs(p, m, period=None):
    out = np.zeros(p.nx * p.ny * p.nz, np.float32)
    per = None if period is None else np.ascontiguousarray(period, np.float32)
    lib().orc_svl_rhs(C.byref(p), None if per is None else per.ctypes.data, m, out)
    return out


def svl_cg(p, rhs):
    x = np.zeros(p.nx * p.ny * p.nz, np.float32)
    it = lib().orc_svl_cg(C.byref(p), np.ascontiguousarray(rhs, np.float32), x)
    return x, int(it)


def svl_accumulate(p, phases, coef, svl=None):
    if svl is None:
        svl = np.zeros(8 * p.nx * p.ny * p.nz, np.float32)
    svl = np.ascontiguousarray(svl, np.float32).copy()
    lib().orc_svl_accumulate(C.byref(p), np.ascontiguousarray(phases, np.float32),
                             np.ascontiguousarray(coef, np.float32).reshape(-1), svl)
    return svl


def svl_lattice(p, coef, period=None):
    """Whole SVL synthesis: (svl on the 2x grid, phases (n, P), iterations)."""
    P = p.nx * p.ny * p.nz
    phases = np.zeros((p.n_coeff, P), np.float32)
    iters = []
    for m in range(p.n_coeff):
        x, it = svl_cg(p, svl_rhs(p, m, period))
        phases[m] = x
        iters.append(it)
    return svl_accumulate(p, phases, coef), phases, iters

