"""Generate topology_tables.inc: the local combinatorics of the Freudenthal grid.

Every cell of the complex is owned by one "anchor" vertex, the minimum corner
of the cell's bounding box.  An anchor owns 1 vertex, 7 edges (families 0-6),
12 triangles (slots 0-11) and 6 tetrahedra (slots 0-5); the numbering of
families and slots is the reference's (main_3d.cu getEdgeID :917-1012,
getVerticesFromTriangleID :425-565, getVerticesFromTetrahedraID :672-740), so
a (anchor, slot) pair maps to the reference's cell id by a closed formula.

The tables list, for an unbounded grid, each cell's facets and cofaces as
(anchor offset, slot) pairs.  Coface lists of a triangle are in the order the
reference's get_cell_tetra (main_3d.cu:4363-4430) finds them: by stencil
direction index from the triangle's highest-id vertex.  Edge coface lists use
the same rule from the edge's highest-id vertex.

Run:  python gen_topology.py  (rewrites topology_tables.inc next to it)
"""
import itertools
import os

DIRS = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (-1, 1, 0), (1, -1, 0),
        (0, 1, 1), (0, -1, -1), (-1, 0, 1), (1, 0, -1), (-1, 1, 1), (1, -1, -1)]
DSET = set(DIRS)

EDGES = [((0, 0, 0), (1, 0, 0)), ((0, 0, 0), (0, 1, 0)), ((0, 0, 0), (0, 0, 1)), ((1, 0, 0), (0, 1, 0)),
         ((0, 0, 0), (0, 1, 1)), ((1, 0, 0), (0, 0, 1)), ((1, 0, 0), (0, 1, 1))]
FACES = [((0, 0, 0), (1, 0, 0), (0, 1, 0)), ((1, 1, 0), (1, 0, 0), (0, 1, 0)),
         ((0, 0, 0), (0, 1, 0), (0, 1, 1)), ((0, 0, 0), (0, 0, 1), (0, 1, 1)),
         ((0, 0, 0), (1, 0, 0), (0, 0, 1)), ((1, 0, 0), (0, 0, 1), (1, 0, 1)),
         ((0, 0, 0), (1, 0, 0), (0, 1, 1)), ((1, 0, 0), (0, 1, 0), (0, 1, 1)),
         ((1, 0, 0), (1, 1, 0), (0, 1, 1)), ((1, 0, 0), (0, 0, 1), (0, 1, 1)),
         ((1, 0, 0), (1, 0, 1), (0, 1, 1)), ((1, 0, 0), (0, 1, 1), (1, 1, 1))]
TETS = [((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 1, 1)), ((0, 0, 0), (1, 0, 0), (0, 0, 1), (0, 1, 1)),
        ((1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 1, 1)), ((1, 0, 0), (1, 1, 0), (0, 1, 1), (1, 1, 1)),
        ((1, 0, 0), (0, 0, 1), (1, 0, 1), (0, 1, 1)), ((1, 0, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1))]


def add(a, b):
    return tuple(x + y for x, y in zip(a, b))


def sub(a, b):
    return tuple(x - y for x, y in zip(a, b))


def idkey(p):
    """Order of vertex ids x + y*W + z*W*H for W, H >= 2: lexicographic in (z, y, x)."""
    return (p[2], p[1], p[0])


def canon(verts):
    """(anchor, frozenset of offsets relative to the anchor) of a cell given by absolute vertices."""
    a = tuple(min(v[i] for v in verts) for i in range(3))
    return a, frozenset(sub(v, a) for v in verts)


EDGE_OF = {frozenset(e): k for k, e in enumerate(EDGES)}
FACE_OF = {frozenset(f): s for s, f in enumerate(FACES)}
TET_OF = {frozenset(t): s for s, t in enumerate(TETS)}


def edge_cofaces(k):
    """Triangles containing edge k anchored at the origin, by direction index from its highest vertex."""
    p, q = sorted(EDGES[k], key=idkey, reverse=True)
    out = []
    for d in DIRS:
        n = add(p, d)
        if sub(n, q) not in DSET:
            continue
        a, rel = canon([p, q, n])
        out.append((a, FACE_OF[rel], n))
    return out


def face_cofaces(s):
    v1, v2, v3 = sorted(FACES[s], key=idkey, reverse=True)
    out = []
    for d in DIRS:
        n = add(v1, d)
        if sub(n, v2) not in DSET or sub(n, v3) not in DSET or n in (v1, v2, v3):
            continue
        a, rel = canon([v1, v2, v3, n])
        out.append((a, TET_OF[rel], n))
    return out


def face_edges(s):
    """edge opposite to vertex j (vertices sorted by id, descending)."""
    vs = sorted(FACES[s], key=idkey, reverse=True)
    out = []
    for j in range(3):
        rest = [v for i, v in enumerate(vs) if i != j]
        a, rel = canon(rest)
        k = EDGE_OF[rel]
        cof = edge_cofaces(k)
        idx = [i for i, (ca, cs, _) in enumerate(cof) if add(ca, a) == (0, 0, 0) and cs == s]
        assert len(idx) == 1
        out.append((a, k, idx[0]))
    return out


def tet_faces(s):
    vs = sorted(TETS[s], key=idkey, reverse=True)
    out = []
    for j in range(4):
        rest = [v for i, v in enumerate(vs) if i != j]
        a, rel = canon(rest)
        fs = FACE_OF[rel]
        cof = face_cofaces(fs)
        idx = [i for i, (ca, cs, _) in enumerate(cof) if add(ca, a) == (0, 0, 0) and cs == s]
        assert len(idx) == 1
        out.append((a, fs, idx[0]))
    return out


def corner(p):
    return p[0] + 2 * p[1] + 4 * p[2]


def emit():
    L = []
    w = L.append
    w("// Generated by gen_topology.py -- do not edit by hand.")
    w("// Local combinatorics of the Freudenthal grid, see gen_topology.py.")
    w("")
    w("#define DMTZ_MAX_EDGE_COF 6")
    w("#ifndef TOPO_QUAL")
    w("#define TOPO_QUAL static const")
    w("#endif")
    w(f"TOPO_QUAL signed char TOPO_DIRS[14][3] = {{{', '.join('{%d,%d,%d}' % d for d in DIRS)}}};")
    lut = [-1] * 27
    for i, d in enumerate(DIRS):
        lut[(d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1)] = i
    w(f"TOPO_QUAL signed char TOPO_DIR_LUT[27] = {{{', '.join(map(str, lut))}}};")
    # corners sorted by id descending
    ev = [sorted(e, key=idkey, reverse=True) for e in EDGES]
    fv = [sorted(f, key=idkey, reverse=True) for f in FACES]
    tv = [sorted(t, key=idkey, reverse=True) for t in TETS]
    w("// corners (dx + 2 dy + 4 dz) of each cell, highest vertex id first")
    w(f"TOPO_QUAL signed char TOPO_EDGE_V[7][2] = {{{', '.join('{%d,%d}' % tuple(corner(p) for p in e) for e in ev)}}};")
    w(f"TOPO_QUAL signed char TOPO_FACE_V[12][3] = {{{', '.join('{%d,%d,%d}' % tuple(corner(p) for p in f) for f in fv)}}};")
    w(f"TOPO_QUAL signed char TOPO_TET_V[6][4] = {{{', '.join('{%d,%d,%d,%d}' % tuple(corner(p) for p in t) for t in tv)}}};")
    # stencil direction from vertex a to vertex b inside a cell, by corner pair
    d88 = [[-1] * 8 for _ in range(8)]
    for a in range(8):
        for b in range(8):
            pa = (a & 1, (a >> 1) & 1, (a >> 2) & 1)
            pb = (b & 1, (b >> 1) & 1, (b >> 2) & 1)
            dd = sub(pb, pa)
            if dd in DSET:
                d88[a][b] = DIRS.index(dd)
    w("// stencil direction index from corner a to corner b (-1 if not adjacent)")
    w("TOPO_QUAL signed char TOPO_CORNER_DIR[8][8] = {" + ", ".join("{" + ",".join(map(str, r)) + "}" for r in d88) + "};")
    # edge cofaces
    ecn, ecf, ect = [], [], []
    for k in range(7):
        cof = edge_cofaces(k)
        ecn.append(len(cof))
        row = [(a[0], a[1], a[2], s) for a, s, _ in cof] + [(0, 0, 0, -1)] * (6 - len(cof))
        ecf.append(row)
        ect.append([n for _, _, n in cof] + [(0, 0, 0)] * (6 - len(cof)))
    w("// triangles containing each edge family: (anchor dx, dy, dz, face slot); third vertex offset")
    w(f"TOPO_QUAL signed char TOPO_EDGE_NCOF[7] = {{{', '.join(map(str, ecn))}}};")
    w("TOPO_QUAL signed char TOPO_EDGE_COF[7][6][4] = {" + ", ".join(
        "{" + ", ".join("{%d,%d,%d,%d}" % c for c in row) + "}" for row in ecf) + "};")
    w("TOPO_QUAL signed char TOPO_EDGE_THIRD[7][6][3] = {" + ", ".join(
        "{" + ", ".join("{%d,%d,%d}" % c for c in row) + "}" for row in ect) + "};")
    # face edges
    fe = [face_edges(s) for s in range(12)]
    w("// edge of each triangle opposite its vertex j (j by id, descending): (anchor dx,dy,dz, family, coface index)")
    w("TOPO_QUAL signed char TOPO_FACE_EDGE[12][3][5] = {" + ", ".join(
        "{" + ", ".join("{%d,%d,%d,%d,%d}" % (a[0], a[1], a[2], k, i) for a, k, i in row) + "}" for row in fe) + "};")
    # face cofaces
    fcn, fcf, fct = [], [], []
    for s in range(12):
        cof = face_cofaces(s)
        fcn.append(len(cof))
        fcf.append([(a[0], a[1], a[2], t) for a, t, _ in cof] + [(0, 0, 0, -1)] * (2 - len(cof)))
        fct.append([n for _, _, n in cof] + [(0, 0, 0)] * (2 - len(cof)))
    w("// tetrahedra containing each triangle slot in get_cell_tetra order: (anchor dx,dy,dz, tet slot); 4th vertex offset")
    w(f"TOPO_QUAL signed char TOPO_FACE_NCOF[12] = {{{', '.join(map(str, fcn))}}};")
    w("TOPO_QUAL signed char TOPO_FACE_COF[12][2][4] = {" + ", ".join(
        "{" + ", ".join("{%d,%d,%d,%d}" % c for c in row) + "}" for row in fcf) + "};")
    w("TOPO_QUAL signed char TOPO_FACE_FOURTH[12][2][3] = {" + ", ".join(
        "{" + ", ".join("{%d,%d,%d}" % c for c in row) + "}" for row in fct) + "};")
    te = [tet_faces(s) for s in range(6)]
    w("// triangle of each tetrahedron opposite its vertex j (j by id, descending): (anchor dx,dy,dz, slot, coface index)")
    w("TOPO_QUAL signed char TOPO_TET_FACE[6][4][5] = {" + ", ".join(
        "{" + ", ".join("{%d,%d,%d,%d,%d}" % (a[0], a[1], a[2], k, i) for a, k, i in row) + "}" for row in te) + "};")
    return "\n".join(L) + "\n"


if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "topology_tables.inc")
    with open(out, "w") as fh:
        fh.write(emit())
    print("wrote", out)
    for k in range(7):
        print("edge", k, "cofaces", len(edge_cofaces(k)))
    for s in range(12):
        print("face", s, "cofaces", len(face_cofaces(s)))
