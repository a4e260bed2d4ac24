"""The marching-cubes tables: both generated copies identical, and the edge
masks / vertex counts are what the triangle lists imply (no reference tree
needed)."""
import os
import re

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EDGE_CORNERS = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4),
                (0, 4), (1, 5), (2, 6), (3, 7)]


def _parse(path, prefix):
    txt = open(path).read()

    def arr(name):
        m = re.search(prefix + name + r"[^=]*=\s*\{(.*?)\};", txt, re.S)
        body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
        return [int(v, 0) for v in re.findall(r"-?0x[0-9a-f]+|-?\d+", body)]

    tri = np.array(arr("tri_table"), dtype=np.int64).reshape(256, 16)
    edge = np.array(arr("edge_table"), dtype=np.int64)
    nv = np.array(arr("num_verts"), dtype=np.int64)
    sha = re.search(r'SHA256 "([0-9a-f]+)"', txt).group(1)
    return tri, edge, nv, sha


def load_tables():
    return _parse(os.path.join(REPO, "oracle", "mc_tables.h"), "orc_")


def test_copies_identical():
    a = _parse(os.path.join(REPO, "oracle", "mc_tables.h"), "orc_")
    b = _parse(os.path.join(REPO, "marching_cube_gb300", "csrc", "mc_tables.h"), "mcg_")
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert a[3] == b[3]


def test_derived_consistency():
    tri, edge, nv, _ = load_tables()
    for ci in range(256):
        row = tri[ci]
        n = int(np.argmax(row < 0)) if (row < 0).any() else 16
        assert (row[n:] == -1).all()
        assert n == nv[ci] and n % 3 == 0
        used = 0
        for e in row[:n]:
            used |= 1 << int(e)
        assert used == edge[ci]
        sign = 0
        for e, (a, b) in enumerate(EDGE_CORNERS):
            if ((ci >> a) & 1) != ((ci >> b) & 1):
                sign |= 1 << e
        assert sign == edge[ci]
    assert nv[0] == 0 and nv[255] == 0


def test_complement_symmetry():
    # case ci and its complement 255-ci cut the same edges
    _, edge, nv, _ = load_tables()
    for ci in range(256):
        assert edge[ci] == edge[255 - ci]
