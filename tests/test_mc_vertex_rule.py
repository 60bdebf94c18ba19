"""The marching-cubes vertex set by sign changes.

The reference places a vertex on every edge that a triangle of some cube
uses (the std::map of edge keys filled while the cubes' triangles are
emitted, TRIANGLE_MESH.cpp:4884-4948).  The device mesher instead marks the
edges whose endpoint signs differ, which is the same set except where the
reference's case 158 leaves out the three edges of its isolated corner
(edges 5, 6 and 10): every other case uses exactly its sign-change edges, and
an interior edge has another cube that uses it.  An omitted edge keeps no
vertex only when the case-158 cube is its one cube, which happens on three
lines of the grid: x-edges at (y, z) = (0, 0), y-edges at (x, z) = (X-1, 0)
and z-edges at (x, y) = (X-1, 0).  This checks that rule against the
table-driven set on random sign grids with planted case-158 cubes."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# edge id -> lower endpoint offset (x, y, z) and axis (TRIANGLE_MESH::getVertexTriplets)
OFF = [None, (0, 0, 0), (0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0), (1, 0, 0), (1, 0, 1),
       (1, 1, 0), (0, 1, 0), (0, 0, 0), (0, 0, 1), (0, 1, 1)]
AXIS = [None, 1, 2, 1, 2, 1, 2, 1, 2, 0, 0, 0, 0]


def cases():
    src = open(os.path.join(ROOT, "quijibo_gb300", "csrc", "mc_cases.h")).read()
    body = src[src.index("QJ_MC_CASES[256][16] = {"):]
    body = body[:body.index("};")].split("=", 1)[1]
    rows = re.findall(r"\{([0-9,]+)\}", body)
    return np.array([[int(v) for v in r.split(",")] for r in rows])


def flag_of(s, x, y, z):
    f = 0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                f |= int(s[z + dz, y + dy, x + dx]) << (4 * dx + 2 * dy + dz)
    return f


def table_vertices(s, tab):
    Z, Y, X = s.shape
    out = set()
    for z in range(Z - 1):
        for y in range(Y - 1):
            for x in range(X - 1):
                for e in tab[flag_of(s, x, y, z)]:
                    if e:
                        o = OFF[e]
                        out.add((x + o[0], y + o[1], z + o[2], AXIS[e]))
    return out


def rule_vertices(s):
    Z, Y, X = s.shape
    out = set()
    if min(X, Y, Z) < 2:
        return out
    for z in range(Z):
        for y in range(Y):
            for x in range(X):
                if x + 1 < X and s[z, y, x] != s[z, y, x + 1]:
                    if not (y == 0 and z == 0 and flag_of(s, x, 0, 0) == 158):
                        out.add((x, y, z, 0))
                if y + 1 < Y and s[z, y, x] != s[z, y + 1, x]:
                    if not (x == X - 1 and z == 0 and flag_of(s, X - 2, y, 0) == 158):
                        out.add((x, y, z, 1))
                if z + 1 < Z and s[z, y, x] != s[z + 1, y, x]:
                    if not (x == X - 1 and y == 0 and flag_of(s, X - 2, 0, z) == 158):
                        out.add((x, y, z, 2))
    return out


def plant(s, x, y, z, f):
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                s[z + dz, y + dy, x + dx] = f >> (4 * dx + 2 * dy + dz) & 1


def test_only_case_158_skips_sign_change_edges():
    tab = cases()
    for f in range(256):
        used = {int(e) for e in tab[f] if e}
        sc = set()
        for e in range(1, 13):
            o = list(OFF[e])
            o2 = list(o)
            o2[AXIS[e]] += 1
            if (f >> (4 * o[0] + 2 * o[1] + o[2]) & 1) != (f >> (4 * o2[0] + 2 * o2[1] + o2[2]) & 1):
                sc.add(e)
        assert used <= sc
        assert used == sc or (f == 158 and sc - used == {5, 6, 10})


@pytest.mark.parametrize("seed", range(12))
def test_sign_change_rule_equals_table_vertex_set(seed):
    tab = cases()
    rng = np.random.RandomState(seed)
    X, Y, Z = rng.randint(2, 7, size=3)
    s = (rng.uniform(size=(Z, Y, X)) < rng.uniform(0.2, 0.8)).astype(np.uint8)
    # case-158 cubes on the three boundary lines and at random places
    for _ in range(3):
        which = rng.randint(4)
        if which == 0:
            plant(s, rng.randint(X - 1), 0, 0, 158)
        elif which == 1:
            plant(s, X - 2, rng.randint(Y - 1), 0, 158)
        elif which == 2:
            plant(s, X - 2, 0, rng.randint(Z - 1), 158)
        else:
            plant(s, rng.randint(X - 1), rng.randint(Y - 1), rng.randint(Z - 1), 158)
    assert rule_vertices(s) == table_vertices(s, tab)


def test_rule_on_an_all_158_line():
    """A grid one cube wide and high whose cubes are all case 158."""
    tab = cases()
    for X, Y, Z in ((2, 2, 2), (2, 2, 5), (2, 3, 2)):
        s = np.zeros((Z, Y, X), dtype=np.uint8)
        for z in range(Z - 1):
            plant(s, X - 2, 0, z, 158)
        assert rule_vertices(s) == table_vertices(s, tab)
