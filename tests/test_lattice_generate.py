"""Lattice tables generated from the crystal structures
(spacetime_gb300/lattices/generate.py, following the reference's generator
GrossPitaevskii/GPBlocks.cpp:38-301 and Mesh/DelaunayMesh.cpp:140-560) against the
reference's own generated tables (the imported ``*.json``): node positions, cell
volume, every stencil entry and weight, and the operator of the dual-edge tables.
CPU only."""
import numpy as np
import pytest

pytest.importorskip("scipy")

from spacetime_gb300 import capi  # noqa: E402
from spacetime_gb300.lattices import generate as gen  # noqa: E402

CASES = [("cube", "cube", None), ("bcc", "bcc", None), ("bcc", "bcc227", 2.27), ("fcc", "fcc", None),
         ("a15", "a15", None), ("c15", "c15", None), ("z", "z", None)]


def _edge_operator(t, n):
    """Coefficients of the q-form Laplacian at node n, sum over its incidences of
    w (psi(to) - psi(from)), keyed by (node, dx, dy, dz)."""
    F = t["edge_face_count"]
    out = {}
    for dx, dy, dz, e, w in t["incidence"][n * F:(n + 1) * F]:
        f, ex, ey, ez, to = t["edges"][e]
        for key, c in (((to, dx + ex, dy + ey, dz + ez), w), ((f, dx, dy, dz), -w)):
            out[key] = out.get(key, 0.0) + c
    return {k: v for k, v in out.items() if abs(v) > 1e-12}


@pytest.mark.parametrize("structure,name,width", CASES, ids=[c[1] for c in CASES])
def test_generated_tables_match_the_reference(structure, name, width):
    ref = capi.Lattice(name).data
    t = gen.generate(structure, width, order=ref["pos"])
    w = ref["block_width"][0]
    assert t["nodes"] == ref["nodes"]
    np.testing.assert_allclose(t["block_width"], ref["block_width"], rtol=1e-15)
    np.testing.assert_allclose(t["pos"], ref["pos"], atol=1e-12 * w)
    assert t["volume"] == pytest.approx(ref["volume"], rel=1e-12)
    assert t["row_ptr"] == ref["row_ptr"]
    for n in range(ref["nodes"]):
        a, b = ref["row_ptr"][n], ref["row_ptr"][n + 1]
        mine = sorted(map(tuple, t["stencil"][a:b]))
        theirs = sorted(map(tuple, ref["stencil"][a:b]))
        assert [r[:4] for r in mine] == [r[:4] for r in theirs], n
        np.testing.assert_allclose([r[4] for r in mine], [r[4] for r in theirs], rtol=1e-12)
    if "edges" in ref:
        assert t["edge_count"] == ref["edge_count"] and t["edge_face_count"] == ref["edge_face_count"]
        for n in range(ref["nodes"]):
            mine, theirs = _edge_operator(t, n), _edge_operator(ref, n)
            assert mine.keys() == theirs.keys(), n
            for k in mine:
                assert mine[k] == pytest.approx(theirs[k], rel=1e-12), (n, k)


def test_generated_lattice_builds_a_handle_description():
    """Generated tables (default node order) feed capi.Lattice like the files do."""
    lat = capi.Lattice("bcc-generated", tables=gen.generate("bcc"))
    assert lat.nodes == 12 and lat.has_edges and lat.edges == 24
    assert np.all(lat.degree == 4)
    # the default order sorts nodes by (z, y, x)
    p = np.round(lat.pos, 9)
    assert all(tuple(p[i][::-1]) <= tuple(p[i + 1][::-1]) for i in range(len(p) - 1))


def test_order_must_match():
    with pytest.raises(ValueError):
        gen.generate("bcc", order=np.zeros((12, 3)))


@pytest.mark.gpu
def test_generated_lattice_steps_like_the_imported_one(gpu):
    """A C15 spin-2 handle on generated tables (in the reference's node order)
    takes the same leapfrog steps as one on the imported tables (FP64, 1e-12)."""
    from spacetime_gb300 import states
    from spacetime_gb300.stepper import Stepper

    ref = capi.Lattice("c15")
    mine = capi.Lattice("c15-generated", tables=gen.generate("c15", order=ref.data["pos"]))
    out = []
    for lat in (ref, mine):
        p = capi.make_params(components=5, precision=capi.FP64, dims=(3, 2, 2), block_scale=0.3, dt=1e-4,
                             trap_offset=100.0, c0=120.0, c2=-7.0, c4=3.0, lattice=lat)
        psi = 0.2 * states.random_state(capi.buffer_shape(lat, p), seed=171)
        with Stepper(lat, p) as s:
            s.upload(capi.PSI_ODD, psi)
            s.start()
            s.step(4)
            out.append(s.download(s.current))
    scale = float(np.max(np.abs(out[0])))
    assert float(np.max(np.abs(out[1] - out[0]))) <= 1e-12 * scale
