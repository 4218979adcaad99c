"""The marching-cubes tables (the oracle's and, through the GPU tests, the
library's, built by the same rule) against the classic table the reference
carries in Mapping/Constant.h: for every configuration the same edge mask,
the same number of triangles and the same polygons -- the outline of its
triangles, with orientation -- so that only the split of polygons of four
or more vertices into triangles differs.  Runs where the reference sources
are present (the container the fixtures are made in)."""
import os
import re
from collections import Counter

import numpy as np
import pytest


def _reference_tables():
    from oracle.ref_shim import build_ref
    path = os.path.join(build_ref.REF, "Mapping", "Constant.h")
    if not os.path.exists(path):
        pytest.skip("reference sources not present")
    src = open(path).read()

    def arr(name):
        i = src.index(name)
        j = src.index("{", i)
        depth, k = 0, j
        while True:
            depth += {"{": 1, "}": -1}.get(src[k], 0)
            if depth == 0:
                break
            k += 1
        return np.array([int(x, 0) for x in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", src[j:k + 1])], np.int64)
    return arr("edgeTableHost"), arr("triangleTableHost").reshape(256, 16), arr("vertexTableHost")


def _triangles(row):
    out = []
    for q in range(0, 15, 3):
        if row[q] < 0:
            break
        out.append(tuple(int(x) for x in row[q:q + 3]))
    return out


def _outline(tris):
    c = Counter()
    for t in tris:
        for i in range(3):
            c[(t[i], t[(i + 1) % 3])] += 1
    return {e for e in c if c.get((e[1], e[0]), 0) == 0}


def test_tables_match_reference_polygons():
    from oracle import oracle as O
    edge_r, tri_r, nv_r = _reference_tables()
    tri, nv, edge = O.mc_tables()
    assert np.array_equal(edge, edge_r)
    assert np.array_equal(nv, nv_r)
    for ci in range(256):
        assert _outline(_triangles(tri[ci])) == _outline(_triangles(tri_r[ci])), "configuration %d" % ci
