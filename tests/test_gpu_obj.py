"""GPU .obj welding and writing against the reference's own writer.

Files written by gcm_write_obj must be byte-identical to what the reference's
File_output::file_write_obj writes (SHA-256 digests in tests/golden/golden_obj.json,
from tests/golden/make_golden_obj.py), and to the oracle's restatement on a
full 128^3 gyroid mesh."""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np
import pytest
import torch

import oracle as O
from tests.helpers import GOLDEN

sys.path.insert(0, GOLDEN)
import obj_inputs  # noqa: E402

pytestmark = pytest.mark.gpu

REF = json.load(open(os.path.join(GOLDEN, "golden_obj.json")))
CASES = obj_inputs.cases()


@pytest.fixture(scope="module")
def ctx():
    from gpucadforam_gb300.mesher import Context

    c = Context(0)
    yield c
    c.close()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def write_obj(ctx, pos_dev, n, path):
    nv, nf = C.c_uint64(), C.c_uint64()
    rc = ctx.lib.gcm_write_obj(ctx.h, C.c_void_p(pos_dev.data_ptr()), n, os.fsencode(path), C.byref(nv),
                               C.byref(nf), _stream())
    return rc, int(nv.value), int(nf.value)


@pytest.mark.parametrize("name,pos", CASES, ids=[c[0] for c in CASES])
def test_gpu_obj_matches_reference_writer(ctx, tmp_path, name, pos):
    path = str(tmp_path / "g.obj")
    d = torch.from_numpy(pos.copy() if pos.size else np.zeros((1, 4), np.float32)).cuda()
    rc, nv, nf = write_obj(ctx, d, pos.shape[0], path)
    assert rc == 0, ctx.lib.gcm_ctx_last_error(ctx.h)
    data = open(path, "rb").read()
    assert hashlib.sha256(data).hexdigest() == REF[name]["sha256"]
    assert (nv, nf) == (REF[name]["v"], REF[name]["f"])


def test_weld_arrays_match_oracle_file(ctx, tmp_path):
    pos = dict(CASES)["lattice_dups"]
    d = torch.from_numpy(pos).cuda()
    nv, nf = C.c_uint64(), C.c_uint64()
    V = torch.empty((pos.shape[0], 3), dtype=torch.float32, device="cuda")
    F = torch.empty((pos.shape[0] // 3, 3), dtype=torch.int32, device="cuda")
    rc = ctx.lib.gcm_weld_obj(ctx.h, C.c_void_p(d.data_ptr()), pos.shape[0], C.c_void_p(V.data_ptr()), V.shape[0],
                              C.c_void_p(F.data_ptr()), F.shape[0], C.byref(nv), C.byref(nf), _stream())
    assert rc == 0
    path = str(tmp_path / "o.obj")
    O.write_obj(pos, path)
    lines = open(path).read().split("\n")
    ov = np.array([[float(t) for t in ln.split()[1:]] for ln in lines if ln.startswith("v ")], np.float32)
    of = np.array([[int(t) for t in ln.split()[1:]] for ln in lines if ln.startswith(" f ")], np.int64)
    assert (int(nv.value), int(nf.value)) == (len(ov), len(of))
    # printed with 6 significant digits: compare the reprinted values
    gv = V[: nv.value].cpu().numpy()
    assert np.array_equal(np.array([[float("%g" % x) for x in r] for r in gv], np.float32), ov)
    assert np.array_equal(F[: nf.value].cpu().numpy().astype(np.int64), of)


def test_full_gyroid_mesh_obj_equals_oracle(ctx, tmp_path):
    n = 128
    f = O.lattice_field((n, n, n), 0, (1, 1, 1), np.array([32.0], np.float32))
    h = np.float32(1.0 / 127.0)
    pos, norm, cnt = ctx.mesh_field(torch.from_numpy(f).cuda(), 0.0, (h, h, h), (0, 0, 0))
    gpath, opath = str(tmp_path / "g.obj"), str(tmp_path / "o.obj")
    rc, nv, nf = write_obj(ctx, pos, cnt.total_verts, gpath)
    assert rc == 0
    onv, onf = O.write_obj(pos.cpu().numpy(), opath)
    assert (nv, nf) == (onv, onf)
    assert open(gpath, "rb").read() == open(opath, "rb").read()


def test_out_of_range_coordinates_are_refused(ctx, tmp_path):
    pos = np.zeros((3, 4), np.float32)
    pos[1, 0] = 2000.0
    d = torch.from_numpy(pos).cuda()
    rc, _, _ = write_obj(ctx, d, 3, str(tmp_path / "x.obj"))
    assert rc == 6  # GCM_ERR_NOT_SUPPORTED
