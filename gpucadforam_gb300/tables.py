"""Host-side view of the marching-cubes tables compiled into the CUDA library.

The data lives once, in ``csrc/mc_tables.h`` (one 64-bit nibble word per cube
configuration); this module parses that header so host code and tests read the
very words the kernels use.  The reference keeps the same data in three arrays
(src/tables.h:11 edgeTable, :49 triTable, :311 numVertsTable); the last two are
derived here from the triangle rows, the first from the cube index itself.
"""
from __future__ import annotations

import functools
import os
import re

import numpy as np

_HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "mc_tables.h")

# Corner offsets and edge endpoints, as in csrc/mc_tables.h.
CORNER_X = (0, 1, 1, 0, 0, 1, 1, 0)
CORNER_Y = (0, 0, 1, 1, 0, 0, 1, 1)
CORNER_Z = (0, 0, 0, 0, 1, 1, 1, 1)
EDGE_A = (0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3)
EDGE_B = (1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7)


@functools.lru_cache(maxsize=1)
def tri_rows() -> tuple[int, ...]:
    text = open(_HEADER).read()
    body = text[text.index("#define GCM_TRI_ROWS"):text.index("namespace gcm")]
    rows = tuple(int(h, 16) for h in re.findall(r"0x([0-9A-Fa-f]{16})ULL", body))
    if len(rows) != 256:
        raise RuntimeError(f"{_HEADER}: expected 256 table rows, found {len(rows)}")
    return rows


def tri_table() -> np.ndarray:
    """(256, 16) uint8, 255 marks the end of a list (the reference's X)."""
    out = np.empty((256, 16), np.uint8)
    for ci, w in enumerate(tri_rows()):
        for j in range(16):
            nib = (w >> (4 * (15 - j))) & 0xF
            out[ci, j] = 255 if nib == 0xF else nib
    return out


def num_verts_table() -> np.ndarray:
    t = tri_table()
    return (t != 255).sum(axis=1).astype(np.uint8)


def edge_table() -> np.ndarray:
    """Bit e set when edge e joins an inside corner to an outside one."""
    out = np.zeros(256, np.uint16)
    for ci in range(256):
        m = 0
        for e in range(12):
            if ((ci >> EDGE_A[e]) & 1) != ((ci >> EDGE_B[e]) & 1):
                m |= 1 << e
        out[ci] = m
    return out
