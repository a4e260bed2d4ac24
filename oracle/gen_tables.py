"""Mechanical extraction of the marching-cubes lookup tables.

The triangulation of each of the 256 cube configurations is a fixed table
(the classic Lorensen-Cline / Bourke tables).  Topology parity with the
reference is only possible with *the same* table, so it is not retyped: this
script parses the three arrays out of the reference source
(cu_marching_cubes_v1.cu:471-505 edgeTable, :509-767 triTable,
:770-1028 numVertsTable), cross-checks that edgeTable and numVertsTable are
exactly what triTable implies, and writes two generated headers with a
checksum:

  oracle/mc_tables.h                       (used by the CPU oracle)
  marching_cube_gb300/csrc/mc_tables.h     (used by the CUDA kernels)

Both are committed, because the reference tree is not available where the
code is built for the GPU.  tests/test_tables.py re-derives the checks
without the reference.

usage:  python oracle/gen_tables.py path/to/cu_marching_cubes_v1.cu
"""
import hashlib
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

# corner pairs of the 12 cube edges, in the reference's vertlist order
# (cu_marching_cubes_v1.cu:304-315)
EDGE_CORNERS = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4),
                (0, 4), (1, 5), (2, 6), (3, 7)]


def _array_body(src, name):
    m = re.search(name + r"\s*(\[[^\]]*\])+\s*=\s*\{", src)
    if not m:
        raise SystemExit("table %s not found" % name)
    i = m.end()
    depth = 1
    j = i
    while depth:
        c = src[j]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        j += 1
    return src[i:j - 1]


def _ints(body):
    return [int(tok, 0) for tok in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", body)]


def parse(src_text):
    edge = _ints(_array_body(src_text, r"const int edgeTable"))
    tri = _ints(_array_body(src_text, r"const int triTable"))
    nv = _ints(_array_body(src_text, r"const int numVertsTable"))
    if len(edge) != 256 or len(tri) != 256 * 16 or len(nv) != 256:
        raise SystemExit("unexpected table sizes %d %d %d" % (len(edge), len(tri), len(nv)))
    tri = [tri[i * 16:(i + 1) * 16] for i in range(256)]
    return edge, tri, nv


def derive(tri):
    """edgeTable / numVertsTable implied by triTable."""
    edge, nv = [], []
    for row in tri:
        n = 0
        while n < 16 and row[n] >= 0:
            n += 1
        mask = 0
        for e in row[:n]:
            mask |= 1 << e
        edge.append(mask)
        nv.append(n)
    return edge, nv


def check(edge, tri, nv):
    d_edge, d_nv = derive(tri)
    assert d_nv == nv, "numVertsTable disagrees with triTable"
    assert d_edge == edge, "edgeTable disagrees with triTable"
    for ci in range(256):
        # every intersected edge (sign change between its corners) is used
        mask = 0
        for e, (a, b) in enumerate(EDGE_CORNERS):
            if ((ci >> a) & 1) != ((ci >> b) & 1):
                mask |= 1 << e
        assert mask == edge[ci], "edgeTable[%d] is not the sign-change set" % ci
        assert nv[ci] % 3 == 0


def digest(edge, tri, nv):
    h = hashlib.sha256()
    h.update(bytes(x & 0xFF for row in tri for x in row))
    h.update(b"".join(x.to_bytes(2, "little") for x in edge))
    h.update(bytes(nv))
    return h.hexdigest()


def render(edge, tri, nv, prefix):
    dig = digest(edge, tri, nv)
    out = []
    out.append("/* GENERATED by oracle/gen_tables.py -- do not edit.")
    out.append(" * Marching-cubes lookup tables, extracted mechanically from the reference")
    out.append(" * (cu_marching_cubes_v1.cu:471-1028) and cross-checked: edge mask and")
    out.append(" * vertex count of every case are re-derived from the triangle list.")
    out.append(" * sha256(tri|edge|nverts) = %s */" % dig)
    guard = prefix.upper() + "MC_TABLES_H"
    out.append("#ifndef %s" % guard)
    out.append("#define %s" % guard)
    out.append("#define %sMC_TABLES_SHA256 \"%s\"" % (prefix.upper(), dig))
    out.append("/* triangle edge lists per cube case, -1 terminated, 16 per case */")
    out.append("static const signed char %stri_table[256][16] = {" % prefix)
    for ci, row in enumerate(tri):
        out.append("  {" + ",".join("%d" % v for v in row) + "}," + "  /* %3d */" % ci)
    out.append("};")
    out.append("/* bit e set iff cube edge e is intersected */")
    out.append("static const unsigned short %sedge_table[256] = {" % prefix)
    for i in range(0, 256, 8):
        out.append("  " + ",".join("0x%03x" % v for v in edge[i:i + 8]) + ",")
    out.append("};")
    out.append("/* number of triangle vertices emitted per cube case */")
    out.append("static const unsigned char %snum_verts[256] = {" % prefix)
    for i in range(0, 256, 16):
        out.append("  " + ",".join("%d" % v for v in nv[i:i + 16]) + ",")
    out.append("};")
    if prefix == "mcg_":
        # the same lists as device data initialised with the module image (no
        # upload, nothing to redo after a device reset)
        out.append("#if defined(__CUDACC__) && defined(MCG_TABLES_DEVICE)")
        out.append("static __device__ __align__(16) signed char %stri_table_dev[256][16] = {" % prefix)
        for row in tri:
            out.append("  {" + ",".join("%d" % v for v in row) + "},")
        out.append("};")
        out.append("static __device__ unsigned char %snum_verts_dev[256] = {" % prefix)
        for i in range(0, 256, 16):
            out.append("  " + ",".join("%d" % v for v in nv[i:i + 16]) + ",")
        out.append("};")
        out.append("#endif")
    out.append("#endif")
    return "\n".join(out) + "\n"


def main(argv):
    if len(argv) != 2:
        raise SystemExit("usage: python oracle/gen_tables.py path/to/cu_marching_cubes_v1.cu")
    src = argv[1]
    with open(src, "r", encoding="latin-1") as f:
        text = f.read()
    edge, tri, nv = parse(text)
    check(edge, tri, nv)
    targets = [
        (os.path.join(HERE, "mc_tables.h"), "orc_"),
        (os.path.join(REPO, "marching_cube_gb300", "csrc", "mc_tables.h"), "mcg_"),
    ]
    for path, prefix in targets:
        with open(path, "w") as f:
            f.write(render(edge, tri, nv, prefix))
        print("wrote", path)
    print("sha256", digest(edge, tri, nv))


if __name__ == "__main__":
    main(sys.argv)
