"""Lattice tables generated from the crystal structures (no imported headers).

The reference emits its tables with a generator (GrossPitaevskii/GPBlocks.cpp:
38-301) on top of its own Delaunay / Hodge mesh library: the lattice points of a
3 x 3 x 3 region of unit cells (Mesh/DelaunayMesh.cpp:140-560, createXxxGrid)
are meshed by a Delaunay complex; the values live on its cells ("bodies") at the
cells' circumcentres; the cells whose circumcentre lies in the unit block
[0, width) are the block's nodes; two nodes are neighbours through every face
they share, with the DEC weight bodyHodge / faceHodge = |face| / (|dual edge|
|cell|) (:118-132, :201-248).  Cospherical points (cube, FCC, ...) make
polyhedral cells (a cube, an octahedron), not tetrahedra.

Here the same complex is computed from the periodic crystal with scipy's Qhull
Delaunay triangulation: the simplices of one merged (cospherical) Delaunay cell
share Qhull's hyperplane on the lifted paraboloid and are grouped by it; a cell's
volume is the sum of its simplices', its circumcentre the least-squares centre of
its vertices, a face the union of the triangles that separate two cells.  Nodes
are the periodic orbits of the circumcentres, wrapped into the block.

The result has the layout of the imported ``*.json`` tables.  For the seven
lattices of the reference it reproduces their node positions and stencil weights
to rounding (tests/test_lattice_generate.py), in the node order given by
``order`` (for example the imported tables' positions) or, by default, sorted by
position.  The dual-edge tables follow the reference generator's rule: an edge
runs from the lower-numbered node to the higher (a node's edges to its own
periodic images get one orientation), and both of its incidences carry the weight
seen from the edge's first node (:240-248).  Where cell volumes differ (A15, C15,
Z) the edge form therefore differs from the node stencil, as the reference's
tables do.
"""
from __future__ import annotations

import math

import numpy as np

S3 = math.sqrt(3.0)

# Crystal bases in fractions of the cell (the interior points of createXxxGrid),
# the reference's default cell widths (GPBlocks.cpp:25), and the cell aspect.
_C15_CU = [(1, 3, 7), (1, 1, 5), (3, 1, 7), (3, 3, 5), (1, 7, 3), (3, 7, 1), (3, 5, 3), (1, 5, 1),
           (5, 1, 1), (7, 3, 1), (5, 3, 3), (7, 1, 3), (5, 5, 5), (7, 5, 7), (7, 7, 5), (5, 7, 7)]
STRUCTURES = {
    # name: (basis, default width, aspect)
    "cube": ([(0, 0, 0)], 1.0, (1.0, 1.0, 1.0)),
    "bcc": ([(0, 0, 0), (0.5, 0.5, 0.5)], math.sqrt(8.0), (1.0, 1.0, 1.0)),
    "fcc": ([(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)], 2.51, (1.0, 1.0, 1.0)),
    "a15": ([(0, 0, 0), (0.5, 0.5, 0.5), (0.5, 0.25, 0), (0.5, 0.75, 0), (0.25, 0, 0.5), (0.75, 0, 0.5),
             (0, 0.5, 0.25), (0, 0.5, 0.75)], 3.91, (1.0, 1.0, 1.0)),
    "c15": ([(0, 0, 0), (0, 0.5, 0.5), (0.5, 0, 0.5), (0.5, 0.5, 0), (0.25, 0.75, 0.75), (0.75, 0.25, 0.75),
             (0.75, 0.75, 0.25), (0.25, 0.25, 0.25)] + [tuple(v / 8.0 for v in t) for t in _C15_CU], 5.39,
            (1.0, 1.0, 1.0)),
    "z": ([(0, 0, 0), (0.5, 0.5, 0), (0, 0, 0.5), (0.5, 0.5, 0.5), (0.25, 0.25, 0.75), (0.25, 0.75, 0.75),
           (0.75, 0.25, 0.75), (0.75, 0.75, 0.75), (0.5, 1 / 6, 0.25), (0.5, 5 / 6, 0.25), (0, 0.5, 0.75),
           (0, 1 / 3, 0.25), (0, 2 / 3, 0.25), (0.5, 0, 0.75)], 3.70, (1.0, S3, 1.0)),
}


def _origin(name: str, d: np.ndarray, width: float) -> np.ndarray:
    """Lattice origin inside the block, in fractions of the cell.  The reference
    meshes the region [-1.125, 1.875] x width (y: 1.875 sqrt3 for Z) starting its
    cells at p0 = (maxp + minp - 3 d) / 2 (DelaunayMesh.cpp:140-153, 511-520); the
    cube grid is created over [-1, 2] (GPBlocks.cpp:63)."""
    if name == "cube":
        return np.zeros(3)
    minp = width * np.array([-1.125, -1.125, -1.125])
    maxp = width * np.array([1.875, 1.875 * (S3 if name == "z" else 1.0), 1.875])
    p0 = 0.5 * (maxp + minp - 3.0 * d)
    return (p0 / d) % 1.0


def _circumcentre(P: np.ndarray) -> np.ndarray:
    A = 2.0 * (P[1:] - P[0])
    b = np.sum(P[1:] ** 2, axis=1) - np.sum(P[0] ** 2)
    return np.linalg.lstsq(A, b, rcond=None)[0]


def _complex(points: np.ndarray):
    """Delaunay cells of a point set: (cell of each simplex, cell volumes, cell
    circumcentres, {(cell_a, cell_b): face area}, simplices)."""
    from scipy.spatial import Delaunay

    tri = Delaunay(points)
    _, cell_of = np.unique(np.round(tri.equations, 9), axis=0, return_inverse=True)
    cell_of = np.asarray(cell_of).ravel()
    ncell = int(cell_of.max()) + 1
    S = tri.simplices
    P = points[S]
    vols = np.abs(np.linalg.det(P[:, 1:] - P[:, :1])) / 6.0
    vol = np.bincount(cell_of, weights=vols, minlength=ncell)
    members = [[] for _ in range(ncell)]
    for s, c in enumerate(cell_of):
        members[c].append(s)
    cen = np.zeros((ncell, 3))
    for c in range(ncell):
        cen[c] = _circumcentre(points[np.unique(S[members[c]])])
    face = {}
    for m in range(4):
        t = tri.neighbors[:, m]
        sel = np.where((t >= 0) & (cell_of[np.maximum(t, 0)] != cell_of))[0]
        tri3 = points[np.delete(S[sel], m, axis=1)]
        area = 0.5 * np.linalg.norm(np.cross(tri3[:, 1] - tri3[:, 0], tri3[:, 2] - tri3[:, 0]), axis=1)
        for s, a in zip(sel, area):
            key = (int(cell_of[s]), int(cell_of[t[s]]))
            face[key] = face.get(key, 0.0) + float(a)
    return cell_of, vol, cen, face


def generate(name: str, width: float | None = None, order=None, reach: int = 2) -> dict:
    """Tables of lattice `name` (a key of STRUCTURES) with cell width `width` (the
    reference's by default).  `order`: (V, 3) node positions to number the nodes
    by (each generated node takes the index of the nearest given position); by
    default nodes are sorted by (z, y, x).  `reach`: periodic images of the cell
    meshed on each side of the block."""
    basis, w0, aspect = STRUCTURES[name]
    width = float(w0 if width is None else width)
    d = width * np.asarray(aspect)
    shift = _origin(name, d, width)
    rng = range(-reach, reach + 1)
    cells = np.array([(i, j, k) for i in rng for j in rng for k in rng], dtype=np.float64)
    pts = ((np.asarray(basis, dtype=np.float64)[None, :, :] + cells[:, None, :] + shift) * d).reshape(-1, 3)
    cell_of, vol, cen, face = _complex(pts)

    tol = 1e-7 * width
    wrapped = cen - np.floor(cen / d) * d
    for ax in range(3):
        wrapped[np.abs(wrapped[:, ax] - d[ax]) < tol, ax] = 0.0
    off = np.rint((cen - wrapped) / d).astype(np.int64)
    inner = np.all(np.abs(off) <= reach - 1, axis=1)
    key = np.rint(wrapped / tol).astype(np.int64)
    orbit = {}
    for c in np.where(inner & np.all(off == 0, axis=1))[0]:
        orbit.setdefault(tuple(key[c]), int(c))
    reps = list(orbit.values())
    V = len(reps)
    pos = wrapped[reps]
    if order is not None:
        order = np.asarray(order, dtype=np.float64).reshape(-1, 3)
        if len(order) != V:
            raise ValueError("order has %d positions, the lattice has %d nodes" % (len(order), V))
        idx = [int(np.argmin(np.linalg.norm(order - p, axis=1))) for p in pos]
        if sorted(idx) != list(range(V)) or max(np.min(np.linalg.norm(order - p, axis=1)) for p in pos) > 1e-6 * width:
            raise ValueError("order does not match the generated node positions")
        rank = idx
    else:
        srt = np.lexsort((np.round(pos[:, 0], 9), np.round(pos[:, 1], 9), np.round(pos[:, 2], 9)))
        rank = [0] * V
        for r, i in enumerate(srt):
            rank[int(i)] = r
    node_of_key = {tuple(key[reps[i]]): rank[i] for i in range(V)}
    by_node = [reps[rank.index(n)] for n in range(V)]

    def node_at(c):
        k = key[c]
        for dk in ((0, 0, 0),) + tuple((a, b, e) for a in (-1, 0, 1) for b in (-1, 0, 1) for e in (-1, 0, 1)):
            n = node_of_key.get((k[0] + dk[0], k[1] + dk[1], k[2] + dk[2]))
            if n is not None:
                return n
        raise RuntimeError("a neighbour cell lies outside the meshed region: raise reach")

    nbrs = {}
    for (a, b), area in face.items():
        nbrs.setdefault(a, []).append((b, area))
    stencil, row_ptr, faces = [], [0], []
    for n, c in enumerate(by_node):
        row = []
        for b, area in nbrs.get(c, []):
            dual = float(np.linalg.norm(cen[b] - cen[c]))
            o = off[b] - off[c]
            row.append((int(o[0]), int(o[1]), int(o[2]), node_at(b), area / (dual * vol[c]), dual))
        row.sort()
        stencil += [list(r[:5]) for r in row]
        faces.append(row)
        row_ptr.append(len(stencil))
    degree = np.diff(row_ptr)
    out = {"name": name, "source": "generated", "nodes": V, "block_width": [float(v) for v in d],
           "volume": float(vol[by_node[0]]), "volumes": [float(vol[c]) for c in by_node],
           "dual_edge_length": float(faces[0][0][5]) if faces[0] else 0.0,
           "pos": [[float(v) for v in wrapped[c]] for c in by_node], "row_ptr": [int(v) for v in row_ptr],
           "stencil": stencil}
    if V and np.all(degree == degree[0]):
        edges, inc = [], [[] for _ in range(V)]
        seen = set()
        for n in range(V):
            for dx, dy, dz, m, h, _ in faces[n]:
                if m < n:
                    continue  # the edge was made from node m
                if m == n:
                    canon = (dx, dy, dz) if (dx, dy, dz) > (0, 0, 0) else (-dx, -dy, -dz)
                    if (n, canon) in seen:
                        continue
                    seen.add((n, canon))
                    dx, dy, dz = canon
                e = len(edges)
                edges.append([n, dx, dy, dz, m])
                inc[n].append([0, 0, 0, e, h])
                inc[m].append([-dx, -dy, -dz, e, -h])
        if all(len(r) == degree[0] for r in inc):
            out.update({"edge_count": len(edges), "edge_face_count": int(degree[0]), "edges": edges,
                        "incidence": [e for r in inc for e in r], "edge_block_width": out["block_width"]})
    return out
