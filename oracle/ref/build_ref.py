"""Recipe that compiles the reference's own hot-path CUDA files for the parity harness.

Test infrastructure only.  It reads the reference sources where they lie (the
``src`` directory of a reference checkout: ``GCM_REFERENCE_SRC``, by default
``/root/reference/src``), never copies them, and writes only into
``oracle/_ref/`` (git-ignored; it travels to the GPU machine with the rest of the
working tree).  Outputs:

* ``oracle/_ref/ref_<name>_sm103a.fatbin`` - device code compiled for sm_103a;
* ``oracle/_ref/ref_<name>_ptx89.fatbin``  - device code as the reference's own
  Makefile ships it (``-gencode arch=compute_89,code=compute_89``, PTX only, JIT
  compiled by the CUDA driver at load time), Makefile:46-48;
* ``tests/golden/ref_tables.bin`` - the reference's tables.h data, dumped by a tiny
  host program (``oracle/ref/dump_tables.cpp``);
* ``oracle/_ref/obj_ref_writer`` - the reference's own ``.obj`` writer
  (``File_output.cu``, host C++) linked with ``oracle/ref/obj_ref_driver.cpp``,
  which supplies a host-memory ``cudaMemcpy`` so it runs without a GPU; used
  here to make ``tests/golden/golden_obj.json``.

The reference files are compiled with nvcc's defaults (no fast-math; FMA
contraction on), as the reference Makefile does, but with ``--std=c++17`` instead of
its ``--std=c++14`` (Makefile:50): the thrust headers of CUDA 13 refuse anything
older.  The dialect does not change device arithmetic.  Two adjustments, both
outside the reference tree: ``oracle/ref/shim/helper_cuda.h`` stands in for the
CUDA-samples helper (the original names cuFFT enums removed in CUDA 13), and
``-D__IMGUIAPP_H__`` skips the GUI header that ``lattice_files/Gratings.h:6``
includes but never uses.

Host code is not built: the GPU machine is aarch64 and only receives the device
code.  ``oracle/ref/ref_runner.cpp`` (this project's own driver-API program) loads
these fatbins there and launches the reference kernels by name.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
REF_SRC = os.environ.get("GCM_REFERENCE_SRC", "/root/reference/src")
OUT = os.path.join(ORACLE, "_ref")

# (name, reference source file relative to src/)
UNITS = [
    ("mc", "MarchingCubes_kernel.cu"),
    ("modelling", "Modelling.cu"),
    ("fft", "lattice_files/Fft_lattice.cu"),
    ("gratings", "lattice_files/Gratings.cu"),
]

ARCHES = {
    "sm103a": ["-gencode", "arch=compute_103a,code=sm_103a"],
    "ptx89": ["-gencode", "arch=compute_89,code=compute_89"],
}


def available() -> bool:
    return os.path.isdir(REF_SRC)


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(name: str, rel: str, arch: str) -> str:
    out = os.path.join(OUT, f"ref_{name}_{arch}.fatbin")
    src = os.path.join(REF_SRC, rel)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = [_nvcc(), "-fatbin", *ARCHES[arch], "--std=c++17", "-D__IMGUIAPP_H__",
           "-I", os.path.join(HERE, "shim"), "-I", os.path.join(REF_SRC, "commons"),
           "-I", REF_SRC, "-o", out, src]
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return out


def dump_tables() -> str:
    out = os.path.join(REPO, "tests", "golden", "ref_tables.bin")
    exe = os.path.join(OUT, "dump_tables")
    cmd = ["g++", "-O0", "-o", exe, os.path.join(HERE, "dump_tables.cpp"),
           f'-DREF_TABLES_H="{os.path.join(REF_SRC, "tables.h")}"']
    subprocess.run(cmd, check=True)
    subprocess.run([exe, out], check=True)
    return out


def build_obj_writer() -> str:
    exe = os.path.join(OUT, "obj_ref_writer")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cmd = ["g++", "-O1", "-std=c++17", "-include", "cuda_runtime_api.h", "-I", cuda_inc, "-I", REF_SRC,
           "-x", "c++", os.path.join(REF_SRC, "File_output.cu"), "-x", "c++", os.path.join(HERE, "obj_ref_driver.cpp"),
           "-o", exe]
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return exe


def build() -> list[str]:
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    jobs = [(n, r, a) for n, r in UNITS for a in ARCHES]
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(lambda j: _compile(*j), jobs))
    outs.append(dump_tables())
    outs.append(build_obj_writer())
    return outs


if __name__ == "__main__":
    res = build()
    if not res:
        print("reference sources not present; nothing built", file=sys.stderr)
    for r in res:
        print(r)
