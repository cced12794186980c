"""Lattice tables: structure, and agreement with the reference headers when present."""
import os

import numpy as np
import pytest

from spacetime_gb300 import capi
from spacetime_gb300.lattices import import_mesh_tables as imp

def _reference_root():
    """The reference tree: SPACETIME_REF, else where the oracle's build recipe
    found it (oracle/_ref/ref_root.txt); empty if neither is known."""
    env = os.environ.get("SPACETIME_REF", "")
    if env:
        return env
    rec = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "ref_root.txt")
    if os.path.exists(rec):
        with open(rec) as f:
            return f.read().strip()
    return ""


REF = _reference_root()


@pytest.mark.parametrize("name", capi.LATTICE_NAMES)
def test_stencil_symmetric_and_in_range(name):
    lat = capi.Lattice(name)
    rp = lat.row_ptr
    S = set()
    for l in range(lat.nodes):
        for dx, dy, dz, m, h in lat.data["stencil"][rp[l]:rp[l + 1]]:
            assert dx in (-1, 0, 1) and dy in (-1, 0, 1) and dz in (-1, 0, 1)
            assert 0 <= m < lat.nodes and h > 0
            S.add((l, (dx, dy, dz), m))
    for (l, d, m) in S:
        assert (m, (-d[0], -d[1], -d[2]), l) in S
    assert np.all(lat.pos >= 0) and np.all(lat.pos <= lat.block_width + 1e-9)


@pytest.mark.parametrize("name", [n for n in capi.LATTICE_NAMES if capi.Lattice(n).has_edges])
def test_edge_tables_consistent(name):
    """d1 incidence: +h on the 'from' node of a d0 edge, -h on the 'to' node, and the
    induced node graph equals the node stencil's graph."""
    lat = capi.Lattice(name)
    E = lat.data["edges"]
    F = lat.faces_per_node
    graph = set()
    for l in range(lat.nodes):
        for dx, dy, dz, eid, h in lat.data["incidence"][l * F:(l + 1) * F]:
            f, ex, ey, ez, t = E[eid]
            if h > 0:
                assert f == l and (dx, dy, dz) == (0, 0, 0)
                graph.add((l, (ex, ey, ez), t))
            else:
                assert t == l and (dx, dy, dz) == (-ex, -ey, -ez)
                graph.add((l, (-ex, -ey, -ez), f))
    rp = lat.row_ptr
    st = {(l, tuple(e[:3]), e[3]) for l in range(lat.nodes) for e in lat.data["stencil"][rp[l]:rp[l + 1]]}
    assert graph == st


def test_degrees():
    assert set(capi.Lattice("bcc").degree) == {4}
    assert set(capi.Lattice("cube").degree) == {6}
    assert set(capi.Lattice("fcc").degree) == {4, 8}  # GrossPitaevskiiGpuFcc/mesh.h:159-171
    assert capi.Lattice("c15").nodes == 136 and capi.Lattice("c15").edges == 272


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "Spin1GpeBCC")),
                    reason="reference tree not known (set SPACETIME_REF, or build the oracle with it present)")
def test_tables_match_reference_headers(tmp_path):
    written = imp.import_all(REF, str(tmp_path))
    import json

    for p in written:
        fresh = json.load(open(p))
        committed = json.load(open(os.path.join(capi.LATTICE_DIR, os.path.basename(p))))
        assert fresh == committed, os.path.basename(p)
