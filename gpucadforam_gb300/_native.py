"""ctypes binding of libgcm.so (the C ABI in include/gcm.h).

The library is the product: there is no Python or CPU fallback.  Importing this
module loads ``gpucadforam_gb300/libgcm.so``; if it is missing the import fails
with a message that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgcm.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gcm.h")

GCM_OK = 0
STATUS = {
    0: "GCM_OK", 1: "GCM_ERR_INVALID_ARGUMENT", 2: "GCM_ERR_OUTPUT_OVERFLOW", 3: "GCM_ERR_DEVICE_TIMEOUT",
    4: "GCM_ERR_CUDA", 5: "GCM_ERR_OUT_OF_MEMORY", 6: "GCM_ERR_NOT_SUPPORTED", 7: "GCM_ERR_IO",
    8: "GCM_ERR_REJECTED", 9: "GCM_ERR_CANCELLED", 10: "GCM_ERR_BUSY",
}
GCM_ERR_INVALID_ARGUMENT = 1
GCM_ERR_OUTPUT_OVERFLOW = 2
GCM_ERR_DEVICE_TIMEOUT = 3
GCM_ERR_CUDA = 4
GCM_ERR_OUT_OF_MEMORY = 5
GCM_ERR_NOT_SUPPORTED = 6
GCM_ERR_IO = 7
GCM_ERR_REJECTED = 8
GCM_ERR_CANCELLED = 9
GCM_ERR_BUSY = 10


class GcmSvlParams(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("dx", C.c_float), ("dy", C.c_float),
                ("dz", C.c_float), ("kind", C.c_uint32), ("period_type", C.c_uint32), ("period", C.c_float),
                ("period_x", C.c_float), ("period_y", C.c_float), ("period_z", C.c_float), ("lcon", C.c_float),
                ("lcon_1", C.c_float), ("sinewave_z", C.c_uint32), ("range", C.c_uint32), ("n_coeff", C.c_uint32),
                ("max_iter", C.c_uint32), ("end_res", C.c_float)]


class GcmGrid(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("voxel_size", C.c_float * 3),
                ("grid_center", C.c_float * 3)]


class GcmCounts(C.Structure):
    _fields_ = [("active_voxels", C.c_uint64), ("total_verts", C.c_uint64), ("status", C.c_uint32),
                ("reserved", C.c_uint32)]


class GcmLattice(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("cx", C.c_uint32), ("cy", C.c_uint32), ("cz", C.c_uint32),
                ("d_period", C.c_void_p), ("d_euler", C.c_void_p), ("d_thickness", C.c_void_p),
                ("d_type", C.c_void_p), ("origin", C.c_float * 3)]


class GcmBatchInstance(C.Structure):
    _fields_ = [("lattice", GcmLattice), ("grid", GcmGrid), ("iso", C.c_float), ("reserved", C.c_uint32)]


class GcmServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("lanes", C.c_uint32), ("queue_capacity", C.c_uint32),
                ("fault_flags", C.c_uint32), ("device_pool_bytes", C.c_uint64), ("host_pool_bytes", C.c_uint64),
                ("fault_param", C.c_uint32), ("reserved", C.c_uint32)]


class GcmResult(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("user_tag", C.c_uint64), ("status", C.c_int32), ("lane", C.c_uint32),
                ("total_verts", C.c_uint64), ("active_voxels", C.c_uint64), ("pos", C.c_void_p),
                ("norm", C.c_void_p), ("on_host", C.c_uint32), ("reserved", C.c_uint32), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double)]


class GcmServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "rejected", "cancelled", "failed", "requeued",
                                          "pool_faults", "device_pool_peak", "device_pool_used",
                                          "host_pool_peak")] + [("lanes_alive", C.c_uint32), ("pending", C.c_uint32)]


class GcmPrimitive(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("op", C.c_uint32), ("flag", C.c_uint32), ("reserved", C.c_uint32),
                ("center", C.c_float * 3), ("v3", C.c_float * 3), ("p", C.c_float * 6)]


class GcmFrame(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("spacing", C.c_float * 3)]


class GcmRequest(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("n_prims", C.c_uint32), ("lattice", GcmLattice), ("d_prims", C.c_void_p),
                ("frame", GcmFrame), ("d_field", C.c_void_p), ("grid", GcmGrid), ("iso", C.c_float),
                ("reserved", C.c_uint32), ("user_tag", C.c_uint64)]


P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
F32 = C.c_float
I32 = C.c_int

# name -> (restype, argtypes)
PROTOTYPES = {
    "gcm_abi_version": (C.c_int, []),
    "gcm_status_string": (C.c_char_p, [I32]),
    "gcm_ctx_create": (I32, [I32, C.POINTER(P)]),
    "gcm_ctx_destroy": (I32, [P]),
    "gcm_ctx_last_error": (C.c_char_p, [P]),
    "gcm_ctx_reserve": (I32, [P, U64]),
    "gcm_ctx_set_wait_limit": (I32, [P, U64]),
    "gcm_ctx_launch_count": (U64, [P]),
    "gcm_ctx_set_primitive_arith": (I32, [P, I32]),
    "gcm_ctx_set_mesh_path": (I32, [P, I32]),
    "gcm_mesh_field": (I32, [P, P, C.POINTER(GcmGrid), F32, P, P, U64, C.POINTER(GcmCounts), P]),
    "gcm_mesh_field_async": (I32, [P, P, C.POINTER(GcmGrid), F32, P, P, U64, P, P]),
    "gcm_count_field": (I32, [P, P, C.POINTER(GcmGrid), F32, C.POINTER(GcmCounts), P]),
    "gcm_mc_classify": (I32, [P, P, C.POINTER(GcmGrid), F32, P, P, P, P]),
    "gcm_scan_exclusive_u32": (I32, [P, P, P, U64, C.POINTER(U64), P]),
    "gcm_mc_compact": (I32, [P, P, P, U64, P, P]),
    "gcm_mc_generate": (I32, [P, P, C.POINTER(GcmGrid), F32, P, U64, P, P, P, U64, P]),
    "gcm_normalise_band": (I32, [P, P, U32, U32, U32, F32, F32, P, P, C.POINTER(F32), P]),
    "gcm_normalise_range": (I32, [P, P, P, U64, F32, F32, C.POINTER(F32), P]),
    "gcm_lattice_mask": (I32, [P, P, P, P, U32, U32, U32, I32, I32, P]),
    "gcm_svl_period_field": (I32, [P, P, U32, U32, U32, F32, F32, F32, F32, F32, F32, C.c_char, P]),
    "gcm_mesh_band": (I32, [P, P, P, C.POINTER(GcmGrid), F32, F32, F32, P, P, U64, C.POINTER(GcmCounts), P]),
    "gcm_mesh_band_async": (I32, [P, P, P, C.POINTER(GcmGrid), F32, F32, F32, P, P, U64, P, P]),
    "gcm_field_unit_cell": (I32, [P, U32, U32, U32, U32, P, P]),
    "gcm_field_lattice": (I32, [P, C.POINTER(GcmLattice), U32, U32, U32, P, P]),
    "gcm_mesh_lattice": (I32, [P, C.POINTER(GcmLattice), C.POINTER(GcmGrid), F32, P, P, U64, C.POINTER(GcmCounts), P]),
    "gcm_mesh_lattice_async": (I32, [P, C.POINTER(GcmLattice), C.POINTER(GcmGrid), F32, P, P, U64, P, P]),
    "gcm_field_csg": (I32, [P, P, U32, C.POINTER(GcmFrame), U32, U32, U32, P, P]),
    "gcm_csg_retain": (I32, [P, P, P, U32, U32, U32, F32, U32, P]),
    "gcm_csg_retain_band": (I32, [P, P, P, U32, U32, U32, F32, F32, F32, U32, P]),
    "gcm_svl_coefficients": (I32, [P, U32, U32, U32, P, P]),
    "gcm_svl_lattice": (I32, [P, C.POINTER(GcmSvlParams), P, P, P, P, P, P]),
    "gcm_mesh_retained": (I32, [P, P, P, U32, C.POINTER(GcmGrid), F32, P, P, U64, C.POINTER(GcmCounts), P]),
    "gcm_count_retained": (I32, [P, P, P, U32, C.POINTER(GcmGrid), F32, C.POINTER(GcmCounts), P]),
    "gcm_mesh_lattice_preview": (I32, [P, P, P, P, U32, C.POINTER(GcmGrid), F32, F32, F32, P, P, U64,
                                      C.POINTER(GcmCounts), P]),
    "gcm_test_lookback_stall": (I32, [P, U32, U32, U64, P, P]),
    "gcm_batch_create": (I32, [P, P, U32, C.POINTER(P)]),
    "gcm_batch_destroy": (I32, [P]),
    "gcm_batch_count": (I32, [P, P, P, C.POINTER(GcmCounts), P]),
    "gcm_batch_mesh_async": (I32, [P, P, P, U64, P, P, P]),
    "gcm_batch_mesh_graph": (I32, [P, P, P, U64, P, P, P]),
    "gcm_batch_tune": (I32, [P, P, P, U64, C.c_char_p, C.POINTER(I32), C.POINTER(U32), P]),
    "gcm_ctx_set_launch_shape": (I32, [P, I32, U32]),
    "gcm_server_create": (I32, [C.POINTER(GcmServerConfig), C.POINTER(P)]),
    "gcm_server_destroy": (I32, [P]),
    "gcm_server_submit": (I32, [P, C.POINTER(GcmRequest), C.POINTER(U64)]),
    "gcm_server_poll": (I32, [P, P, U32, C.POINTER(U32), U64]),
    "gcm_server_release": (I32, [P, U64]),
    "gcm_server_cancel": (I32, [P, U64]),
    "gcm_server_get_stats": (I32, [P, C.POINTER(GcmServerStats)]),
    "gcm_server_now": (C.c_double, [P]),
    "gcm_test_pool_script": (C.c_int64, [U64, P, P, U32]),
    "gcm_weld_obj": (I32, [P, P, U64, P, U64, P, U64, C.POINTER(U64), C.POINTER(U64), P]),
    "gcm_write_obj": (I32, [P, P, U64, C.c_char_p, C.POINTER(U64), C.POINTER(U64), P]),
    "gcm_mesh_field_noalloc": (I32, [P, C.POINTER(GcmGrid), F32, P, P, U64, P, P]),
    "gcm_mesh_csg": (I32, [P, P, U32, C.POINTER(GcmFrame), C.POINTER(GcmGrid), F32, P, P, U64,
                           C.POINTER(GcmCounts), P]),
    "gcm_mesh_csg_async": (I32, [P, P, U32, C.POINTER(GcmFrame), C.POINTER(GcmGrid), F32, P, P, U64, P, P]),
}


def header_symbols() -> list[str]:
    """Every function declared in include/gcm.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gcm_[a-z0-9_]+)\s*\(", text)))


_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Loads libgcm.so (GCM_LIBRARY overrides the in-tree path)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("GCM_LIBRARY") or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class GcmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code
