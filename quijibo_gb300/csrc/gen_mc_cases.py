"""Generate ``mc_cases.h``, the marching-cubes case table shared by the CUDA
mesher and the CPU oracle.

The table must be identical to the reference's so that the emitted topology
(which edges carry vertices, which triangles each cube emits and in which
order) matches it exactly.  This script reads the reference's four case
includes (src/geometry/MARCHING_CUBES_{VERTICES,TRIANGLES}.include[.huge]),
checks that all four list the same triangles, checks the table against the
marching-cubes invariant (every edge whose corners differ in sign is used and
no other), and writes the triangles as edge ids 1..12 in a flat C array.

Usage:  python gen_mc_cases.py <reference root> <output header>
It runs only when the header is regenerated; the build uses the committed
header.
"""
import re
import sys

# edge id -> (corner offset of the lower endpoint, axis 0=x 1=y 2=z);
# follows TRIANGLE_MESH::getVertexTriplets (src/geometry/TRIANGLE_MESH.cpp:1569-1665)
EDGES = {
    1: ((0, 0, 0), 1), 2: ((0, 0, 0), 2), 3: ((0, 0, 1), 1), 4: ((0, 1, 0), 2),
    5: ((1, 0, 0), 1), 6: ((1, 0, 0), 2), 7: ((1, 0, 1), 1), 8: ((1, 1, 0), 2),
    9: ((0, 1, 0), 0), 10: ((0, 0, 0), 0), 11: ((0, 0, 1), 0), 12: ((0, 1, 1), 0),
}
# cube flag bit k <-> corner (x,y,z) offsets, TRIANGLE_MESH.cpp:4929-4931
CORNER_BIT = {(0, 0, 0): 0, (0, 0, 1): 1, (0, 1, 0): 2, (0, 1, 1): 3,
              (1, 0, 0): 4, (1, 0, 1): 5, (1, 1, 0): 6, (1, 1, 1): 7}


def parse(path, fn):
    table = {}
    call = re.compile(fn + r"\((\d+),(\d+),(\d+),index\)")
    # a line may hold several "case N:" labels; split the whole text on them
    parts = re.split(r"case\s+(\d+):", open(path).read())
    for label, body in zip(parts[1::2], parts[2::2]):
        tris = [tuple(int(v) for v in c) for c in call.findall(body)]
        assert int(label) not in table
        table[int(label)] = tris
    for c in range(256):
        table.setdefault(c, [])
    return table


def main(ref, out):
    g = ref.rstrip("/") + "/src/geometry/"
    tabs = [parse(g + "MARCHING_CUBES_TRIANGLES.include.huge", "addVertexTripletTriangle"),
            parse(g + "MARCHING_CUBES_VERTICES.include.huge", "addVertexTriplets"),
            parse(g + "MARCHING_CUBES_TRIANGLES.include", "addVertexPairTriangle"),
            parse(g + "MARCHING_CUBES_VERTICES.include", "addVertexPairs")]
    for t in tabs[1:]:
        assert t == tabs[0], "case includes disagree"
    tab = tabs[0]
    omitted = []
    for case in range(256):
        used = {e for tri in tab[case] for e in tri}
        crossing = set()
        for e, (off, ax) in EDGES.items():
            hi = list(off)
            hi[ax] += 1
            a = (case >> CORNER_BIT[off]) & 1
            b = (case >> CORNER_BIT[tuple(hi)]) & 1
            if a != b:
                crossing.add(e)
        # the table never places a vertex on an edge without a sign change;
        # it may omit some crossing edges (case 158 omits the triangle around
        # its isolated corner), and those omissions are kept as they are
        assert used <= crossing, (case, used, crossing)
        if used != crossing:
            omitted.append((case, sorted(crossing - used)))
        assert len(tab[case]) <= 5
    lines = [
        "// Marching-cubes case table: for each 8-bit cube flag, up to five",
        "// triangles as edge ids 1..12, zero-terminated.  Generated by",
        "// gen_mc_cases.py from the reference's case includes",
        "// (src/geometry/MARCHING_CUBES_TRIANGLES.include.huge); the triangles and",
        "// their order must match the reference for identical mesh topology.",
        "// Cases whose triangles skip crossing edges (kept as in the reference): %s" % (
            ", ".join("%d omits edges %s" % (c, "/".join(map(str, es))) for c, es in omitted) or "none"),
        "#pragma once",
        "#define QJ_MC_MAX_TRIS 5",
        "// CUDA code defines QJ_MC_STORAGE as __constant__ storage before including",
        "#ifndef QJ_MC_STORAGE",
        "#define QJ_MC_STORAGE static const",
        "#endif",
        "QJ_MC_STORAGE unsigned char QJ_MC_CASES[256][16] = {",
    ]
    for case in range(256):
        flat = [e for tri in tab[case] for e in tri]
        flat += [0] * (16 - len(flat))
        lines.append("  {" + ",".join(str(v) for v in flat) + "},  // %d" % case)
    lines.append("};")
    lines.append("// bit (e-1) set when case c places a vertex on edge e")
    lines.append("QJ_MC_STORAGE unsigned short QJ_MC_EDGEMASK[256] = {")
    masks = []
    for case in range(256):
        m = 0
        for tri in tab[case]:
            for e in tri:
                m |= 1 << (e - 1)
        masks.append("0x%03x" % m)
    for i in range(0, 256, 16):
        lines.append("  " + ",".join(masks[i:i + 16]) + ",")
    lines.append("};")
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
