"""The project's marching-cubes table equals the reference's src/tables.h data."""
import numpy as np

from gpucadforam_gb300.tables import tri_table, num_verts_table, edge_table
from tests.helpers import GOLDEN
import os


def _ref():
    b = open(os.path.join(GOLDEN, "ref_tables.bin"), "rb").read()
    assert len(b) == 512 + 4096 + 256
    edge = np.frombuffer(b[:512], "<u2")
    tri = np.frombuffer(b[512:4608], np.uint8).reshape(256, 16)
    nv = np.frombuffer(b[4608:], np.uint8)
    return edge, tri, nv


def test_tri_table_identical():
    _, tri, _ = _ref()
    assert np.array_equal(tri_table(), tri)


def test_num_verts_identical():
    _, _, nv = _ref()
    assert np.array_equal(num_verts_table(), nv)


def test_edge_table_identical():
    edge, _, _ = _ref()
    assert np.array_equal(edge_table(), edge)
