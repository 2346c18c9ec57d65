"""A compiled C++ caller of the C ABI (tests/consumer/gcm_consumer.cpp), built
here with g++ against include/gcm.h and linked to libgcm.so.

* the size and every field offset of each public struct equal the ctypes
  layouts of gpucadforam_gb300/_native.py, so header and bindings cannot drift;
* argument checks that need no GPU return the documented statuses;
* on a GPU, the consumer's gcm_count_field + gcm_mesh_field of golden plain
  case 1 writes exactly the reference kernels' vertices (Isosurface.h:60-64 is
  the interface being replaced).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from gpucadforam_gb300 import _native as N
from tests.helpers import golden, plain_case

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "consumer", "gcm_consumer.cpp")
OUT = os.path.join(REPO, "tests", "consumer", "_build")


@pytest.fixture(scope="module")
def consumer():
    N.load()  # builds nothing; the library must exist
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "gcm_consumer")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    lib_dir = os.path.dirname(N.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-o", exe, SRC, "-I", os.path.join(REPO, "include"), "-I",
           os.path.join(cuda, "include"), "-L", lib_dir, "-lgcm", f"-Wl,-rpath,{lib_dir}", "-L",
           os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    subprocess.run(cmd, check=True)
    return exe


STRUCTS = {"gcm_grid": N.GcmGrid, "gcm_counts": N.GcmCounts, "gcm_lattice": N.GcmLattice,
           "gcm_primitive": N.GcmPrimitive, "gcm_frame": N.GcmFrame, "gcm_svl_params": N.GcmSvlParams,
           "gcm_batch_instance": N.GcmBatchInstance, "gcm_server_config": N.GcmServerConfig,
           "gcm_request": N.GcmRequest, "gcm_result": N.GcmResult, "gcm_server_stats": N.GcmServerStats}


def test_header_layouts_match_the_bindings(consumer):
    out = subprocess.run([consumer, "layout"], check=True, capture_output=True, text=True).stdout.split("\n")
    seen = set()
    for line in filter(None, out):
        name, field, off, size = line.split()
        off, size = int(off), int(size)
        if name == "gcm_csg_point":  # a 16-byte record of int32 + 3 floats, used as raw arrays in Python
            assert (field, off) in {("sizeof", 16), ("val", 0), ("t_x", 4), ("t_y", 8), ("t_z", 12)}
            continue
        S = STRUCTS[name]
        if field == "sizeof":
            assert C.sizeof(S) == off, name
        else:
            f = getattr(S, field)
            assert (f.offset, f.size) == (off, size), (name, field)
        seen.add((name, field))
    # every ctypes field was checked against the header
    for name, S in STRUCTS.items():
        for fname, _ in S._fields_:
            assert (name, fname) in seen, (name, fname)


def test_consumer_argument_checks(consumer):
    r = subprocess.run([consumer, "reject"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "abi 1 status0 ok" in r.stdout


@pytest.mark.gpu
def test_consumer_meshes_golden_case(consumer, tmp_path):
    MC = golden("golden_mc.npz")
    f, iso, vs, gc = plain_case(MC, 1)
    nz, ny, nx = f.shape
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        fh.write(np.array([nx, ny, nz], np.uint32).tobytes())
        fh.write(np.array([iso, *vs, *gc], np.float32).tobytes())
        fh.write(np.ascontiguousarray(f, np.float32).tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([consumer, "mesh", str(inp), str(out)], check=True)
    b = out.read_bytes()
    V = int(np.frombuffer(b[:8], np.uint64)[0])
    ref_pos, ref_norm = MC["sm103a/plain1/pos"], MC["sm103a/plain1/norm"]
    assert V == len(ref_pos)
    assert b[8:8 + 16 * V] == ref_pos.tobytes()
    assert b[8 + 16 * V:] == ref_norm.tobytes()
