"""Import the reference's generated lattice tables into this package's CSR format.

The reference (markus-kivioja/SpaceTime) discretises space with block cells whose
dual-node positions, neighbour lists and DEC Hodge weights are emitted by its table
generator (``GrossPitaevskii/GPBlocks.cpp:38-301``) into per-program ``mesh.h``
headers.  Results can only agree with the reference when the discretisation is the
same, so the numbers must be the same; this script reads those headers as text and
writes them out in this package's own format:

* ``pos``        -- V x 3 dual-node positions inside the unit block (``d_localPos`` /
                    ``getPositions``).
* ``stencil``    -- node Laplacian in CSR form: ``row_ptr`` (V+1) and per entry
                    ``(dx, dy, dz, node, hodge)``; the cell offsets replace the
                    reference's byte offsets (``int2``: ``GrossPitaevskiiGpuBcc/mesh.h:42-92``)
                    or explicit cell offsets (``int4``: ``Spin1GpeBCC/mesh.h:47-100``).
* ``edges``      -- dual-edge table ``(from, dx, dy, dz, to)`` (``d0``,
                    ``RelativisticSpin2Gpe/mesh.h:48-74``).
* ``incidence``  -- per node, FACE_COUNT entries ``(dx, dy, dz, edge, hodge)`` where
                    the sign of the incidence is folded into the hodge (``d1``,
                    ``RelativisticSpin2Gpe/mesh.h:76-233``).

Run it where the reference tree exists::

    python -m spacetime_gb300.lattices.import_mesh_tables /path/to/SpaceTime

It rewrites the ``*.json`` files next to this script.  The tables are data, not code:
the JSON layout, the parser and everything that consumes the tables are this
package's own.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# lattice name -> sources (relative to the reference root).  "stencil" files carry a
# node Laplacian (int2 byte offsets or int4 cell offsets); "edges" files carry d0/d1.
LATTICES = {
    "cube": {"stencil": "GrossPitaevskiiGpuCube/mesh.h", "edges": "RelativisticGpeCube/mesh.h"},
    "bcc": {"stencil": "Spin1GpeBCC/mesh.h", "edges": "RelativisticSpin2Gpe/mesh.h"},
    "bcc227": {"stencil": "GrossPitaevskiiGpuBcc/mesh.h", "edges": "RelativisticGpeBCC/mesh.h"},
    "fcc": {"stencil": "GrossPitaevskiiGpuFcc/mesh.h"},
    "a15": {"stencil": "GrossPitaevskiiGpuA15/mesh.h"},
    "c15": {"stencil": "GrossPitaevskiiGpuC15/mesh.h", "edges": "RelativisticGpeC15/mesh.h"},
    "z": {"stencil": "GrossPitaevskiiGpuZ/mesh.h"},
}

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _define(text: str, name: str):
    m = re.search(r"#define\s+%s\s+(%s)" % (name, _NUM), text)
    return None if m is None else float(m.group(1))


def _vec3(s: str):
    vals = [float(v) for v in re.findall(_NUM, s)]
    if len(vals) != 3:
        raise ValueError("expected 3 numbers in %r" % s)
    return vals


def _header(text: str) -> dict:
    out = {}
    for key in ("FACE_COUNT", "VALUES_IN_BLOCK", "EDGES_IN_BLOCK", "INDICES_PER_BLOCK", "DUAL_EDGE_LENGTH"):
        v = _define(text, key)
        if v is not None:
            out[key] = v
    m = re.search(r"BLOCK_WIDTH\s*=\s*(?:sqrt\(8\.0\)\s*\*\s*)?Vector3\(([^)]*)\)", text)
    out["BLOCK_WIDTH"] = _vec3(m.group(1))
    m = re.search(r"VOLUME\s*=\s*(%s)" % _NUM, text)
    out["VOLUME"] = float(m.group(1))
    return out


def _positions(text: str, nodes: int):
    pos = [None] * nodes
    for m in re.finditer(r"pos\[(\d+)\]\s*=\s*(?:Vector3\(([^)]*)\)|\{([^}]*)\})", text):
        i = int(m.group(1))
        body = m.group(2) if m.group(2) is not None else m.group(3)
        if i < nodes and pos[i] is None:
            pos[i] = _vec3(body)
    if any(p is None for p in pos):
        m = re.search(r"d_localPos\[[^\]]*\]\s*=\s*\{(.*?)\}\s*\};", text, re.S)
        if m is None:
            raise ValueError("no node positions found")
        triples = re.findall(r"\{([^{}]*)\}", m.group(1) + "}")
        pos = [_vec3(t) for t in triples[:nodes]]
    return pos


def _offset_expr(expr: str, names):
    """Decode a linear expression in the three stride names into (dx, dy, dz)."""
    expr = expr.strip()
    if expr in ("", "0"):
        return (0, 0, 0)
    sign = 1
    if expr.startswith("-(") and expr.endswith(")"):
        sign, expr = -1, expr[2:-1]
    env = {names[0]: 1, names[1]: 1000, names[2]: 1000000}
    val = sign * eval(expr, {"__builtins__": {}}, env)  # expression of three names only
    d = [0, 0, 0]
    for axis, unit in ((2, 1000000), (1, 1000), (0, 1)):
        q = int(round(val / unit))
        d[axis] = q
        val -= q * unit
    if val != 0:
        raise ValueError("cannot decode offset %r" % expr)
    return tuple(d)


def _last_assignments(text: str, pattern: str):
    """Return {index: groups} keeping the LAST assignment of each index.

    Some headers assign ``hodges`` twice (``RelativisticSpin2Gpe/mesh.h:138-233``);
    the second assignment is the one the reference program uses.
    """
    out = {}
    for m in re.finditer(pattern, text):
        out[int(m.group(1))] = m.groups()[1:]
    return out


def _hodges(text: str, count: int):
    h = _last_assignments(text, r"hodges\[(\d+)\]\s*=\s*(%s)\s*;" % _NUM)
    if len(h) != count:
        raise ValueError("expected %d hodges, found %d" % (count, len(h)))
    return [float(h[i][0]) for i in range(count)]


def parse_stencil(text: str) -> dict:
    hdr = _header(text)
    V = int(hdr["VALUES_IN_BLOCK"])
    n = int(hdr["INDICES_PER_BLOCK"])
    hod = _hodges(text, n)
    ent4 = _last_assignments(text, r"ind\[(\d+)\]\s*=\s*make_int4\(\s*(-?\d+)\s*,\s*(-?\d+)\s*,\s*(-?\d+)\s*,\s*(\d+)\s*\)")
    ent2 = _last_assignments(text, r"ind\[(\d+)\]\s*=\s*make_int2\(([^,]*),\s*(\d+)\s*\)")
    entries = []
    if ent4:
        for i in range(n):
            dx, dy, dz, node = ent4[i]
            entries.append([int(dx), int(dy), int(dz), int(node), hod[i]])
    else:
        for i in range(n):
            expr, node = ent2[i]
            dx, dy, dz = _offset_expr(expr, ("nx", "ny", "nz"))
            entries.append([dx, dy, dz, int(node), hod[i]])
    counts = _last_assignments(text, r"indicesAndFaceCounts\[(\d+)\]\s*=\s*make_int2\((\d+)\s*,\s*(\d+)\)")
    if counts:
        row_ptr = [int(counts[l][0]) for l in range(V)] + [n]
        for l in range(V):
            if row_ptr[l] + int(counts[l][1]) != row_ptr[l + 1]:
                raise ValueError("face counts are not contiguous")
    else:
        deg = n // V
        row_ptr = [l * deg for l in range(V + 1)]
    return {"header": hdr, "pos": _positions(text, V), "row_ptr": row_ptr, "stencil": entries}


def parse_edges(text: str) -> dict:
    hdr = _header(text)
    V = int(hdr["VALUES_IN_BLOCK"])
    E = int(hdr["EDGES_IN_BLOCK"])
    n = int(hdr["INDICES_PER_BLOCK"])
    hod = _hodges(text, n)
    d0 = _last_assignments(text, r"d0\[(\d+)\]\s*=\s*\{?\s*make_int3\(\s*(\d+)\s*,\s*([^,]*),\s*(\d+)\s*\)")
    d1 = _last_assignments(text, r"d1\[(\d+)\]\s*=\s*make_int2\((.*?),\s*(\d+)\s*\)\s*;")
    edges = []
    for e in range(E):
        frm, expr, to = d0[e]
        dx, dy, dz = _offset_expr(expr, ("d0x", "d0y", "d0z"))
        edges.append([int(frm), dx, dy, dz, int(to)])
    inc = []
    for i in range(n):
        expr, edge = d1[i]
        dx, dy, dz = _offset_expr(expr, ("d1x", "d1y", "d1z"))
        inc.append([dx, dy, dz, int(edge), hod[i]])
    return {"header": hdr, "pos": _positions(text, V), "edges": edges, "incidence": inc}


def import_all(ref_root: str, out_dir: str = HERE) -> list:
    written = []
    for name, src in LATTICES.items():
        with open(os.path.join(ref_root, src["stencil"])) as f:
            st = parse_stencil(f.read())
        hdr = st["header"]
        lat = {
            "name": name,
            "source": src,
            "nodes": int(hdr["VALUES_IN_BLOCK"]),
            "block_width": hdr["BLOCK_WIDTH"],
            "volume": hdr["VOLUME"],
            "dual_edge_length": hdr.get("DUAL_EDGE_LENGTH"),
            "pos": st["pos"],
            "row_ptr": st["row_ptr"],
            "stencil": st["stencil"],
        }
        if "edges" in src:
            with open(os.path.join(ref_root, src["edges"])) as f:
                ed = parse_edges(f.read())
            eh = ed["header"]
            if int(eh["VALUES_IN_BLOCK"]) != lat["nodes"]:
                raise ValueError("%s: node count mismatch between tables" % name)
            lat["edge_block_width"] = eh["BLOCK_WIDTH"]
            lat["edge_count"] = int(eh["EDGES_IN_BLOCK"])
            lat["edge_face_count"] = int(eh["FACE_COUNT"])
            lat["edges"] = ed["edges"]
            lat["incidence"] = ed["incidence"]
            lat["edge_pos"] = ed["pos"]
        path = os.path.join(out_dir, name + ".json")
        with open(path, "w") as f:
            json.dump(lat, f, indent=None, separators=(",", ":"))
            f.write("\n")
        written.append(path)
    return written


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPACETIME_REF", "")
    if not root or not os.path.isdir(root):
        sys.exit("usage: import_mesh_tables.py <reference root>")
    for p in import_all(root):
        print(p)
