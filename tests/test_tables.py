"""The project's marching-cubes table equals the reference's src/tables.h data."""
import numpy as np

from gpucadforam_gb300 import tables as T
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


def test_rows_end_in_terminator_and_fit_five_triangles():
    """The fused kernel keeps each configuration's triangle count in the
    lowest nibble of its shared copy of the row and reads triangle j's edges
    as the 12-bit group starting at nibble 3j: every row must end in the 0xF
    terminator and list at most 5 triangles."""
    for ci, row in enumerate(T.tri_rows()):
        assert row & 0xF == 0xF, ci
        nib = [(row >> (4 * (15 - i))) & 0xF for i in range(16)]
        n = next(i for i, v in enumerate(nib) if v == 0xF)
        assert n % 3 == 0 and n <= 15 and all(v == 0xF for v in nib[n:]), ci
        for j in range(n // 3):
            g = (row >> (52 - 12 * j)) & 0xFFF
            assert [(g >> 8) & 0xF, (g >> 4) & 0xF, g & 0xF] == nib[3 * j:3 * j + 3]
