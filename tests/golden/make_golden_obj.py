"""Runs the reference's own .obj writer (oracle/_ref/obj_ref_writer, built by
oracle/ref/build_ref.py from src/File_output.cu) on the buffers of
obj_inputs.py and records the SHA-256 and size of each file it writes, plus
its vertex and face line counts, in golden_obj.json.

    python oracle/ref/build_ref.py && python tests/golden/make_golden_obj.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import obj_inputs  # noqa: E402

EXE = os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref", "obj_ref_writer")


def main():
    res = {}
    with tempfile.TemporaryDirectory() as td:
        for name, pos in obj_inputs.cases():
            src = os.path.join(td, "p.f32")
            dst = os.path.join(td, "o.obj")
            pos.astype("<f4").tofile(src)
            subprocess.run([EXE, src, dst], check=True, stdout=subprocess.DEVNULL)
            b = open(dst, "rb").read()
            lines = b.split(b"\n")
            res[name] = {"sha256": hashlib.sha256(b).hexdigest(), "bytes": len(b), "nverts_in": int(pos.shape[0]),
                         "v": sum(1 for ln in lines if ln.startswith(b"v ")),
                         "f": sum(1 for ln in lines if ln.startswith(b" f "))}
    with open(os.path.join(HERE, "golden_obj.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
