"""The oracle's .obj writer reproduces the reference's own writer byte for byte.

tests/golden/golden_obj.json holds SHA-256 digests of the files the reference's
File_output::file_write_obj (src/File_output.cu:5-81) writes for the buffers of
tests/golden/obj_inputs.py (tests/golden/make_golden_obj.py made them)."""
import hashlib
import json
import os
import sys

import pytest

import oracle as O
from tests.helpers import GOLDEN

sys.path.insert(0, GOLDEN)
import obj_inputs  # noqa: E402

REF = json.load(open(os.path.join(GOLDEN, "golden_obj.json")))
CASES = obj_inputs.cases()


@pytest.mark.parametrize("name,pos", CASES, ids=[c[0] for c in CASES])
def test_oracle_obj_matches_reference_writer(tmp_path, name, pos):
    path = str(tmp_path / "o.obj")
    nv, nf = O.write_obj(pos, path)
    data = open(path, "rb").read()
    assert hashlib.sha256(data).hexdigest() == REF[name]["sha256"]
    assert (nv, nf) == (REF[name]["v"], REF[name]["f"])
