"""Builds the CPU oracle (oracle/oracle.cpp) into oracle/_build/liboracle.so.

Test infrastructure only.  Compiled with -ffp-contract=off so that each
floating-point operation rounds where the source says, and with OpenMP for the
timed CPU baseline.  Portable flags only (the GPU machine is aarch64).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.cpp")]
DEPS = SOURCES + [os.path.join(HERE, "oracle.h"),
                  os.path.join(os.path.dirname(HERE), "gpucadforam_gb300", "csrc", "mc_tables.h"),
                  os.path.join(os.path.dirname(HERE), "gpucadforam_gb300", "csrc", "angle_table.h")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, *SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
