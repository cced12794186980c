"""The FP64 oracle against the reference's own CPU stepper (golden fixture), and
the oracle's GPU-kernel form against its GPBlocks form."""
import os

import numpy as np
import pytest

from oracle import oracle
from spacetime_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "gpblocks_bcc.npz")


def _load():
    d = np.load(GOLDEN)
    X, Y, Z, V, deg, steps, iters = (int(v) for v in d["dims"])
    lapfac, lapfac0, g, volume, dt = (float(v) for v in d["scal"])
    return d, (X, Y, Z, V, deg, steps, iters), (lapfac, lapfac0, g, volume, dt)


def test_gpblocks_restatement_is_bit_exact():
    """orc_gpblocks_run reproduces integrateInTime's printed normsq/error exactly
    (GrossPitaevskii/GPBlocks.cpp:531-606)."""
    d, (X, Y, Z, V, deg, steps, iters), (lapfac, lapfac0, g, volume, dt) = _load()
    even, odd, psi0, pot = d["even"].copy(), d["odd"].copy(), d["psi0"].copy(), d["pot"].copy()
    bxsize = (X + 1) * V
    bxysize = (Y + 1) * bxsize
    ii0 = bxysize + bxsize + V
    vsize = ii0 + (Z + 1) * bxysize
    got = [oracle.gpblocks_norm(ii0, vsize, psi0, even, volume)]
    for _ in range(iters):
        oracle.gpblocks_run(X, Y, Z, V, deg, d["lapind"], lapfac, lapfac0, g, pot, even, odd, steps)
        got.append(oracle.gpblocks_norm(ii0, vsize, psi0, even, volume))
    got = np.array(got)
    ref = d["normsq_error"]
    assert got.shape == ref.shape
    assert np.array_equal(got, ref), (got, ref)


def _gp_to_ref_layout(a, X, Y, Z, V):
    """GPBlocks flat complex array -> reference file layout (Z+2, Y+2, X+2, V, 1, 2)."""
    n = (Z + 2) * (Y + 1) * (X + 1) * V
    c = a.reshape(-1, 2)[:n].reshape(Z + 2, Y + 1, X + 1, V, 2)
    out = np.zeros((Z + 2, Y + 2, X + 2, V, 1, 2))
    out[1:-1, 1:-1, 1:-1, :, 0, :] = c[1:Z + 1, 1:Y + 1, 1:X + 1]
    return out


def test_gpu_form_matches_gpblocks_form():
    """The node-stencil form the kernels use, sum w (psi_nb - psi) + (V + g|psi|^2) psi
    (GPUGrossPitaevskii_BCC.cu:176-202), against the GPBlocks sum-then-subtract form
    lapfac sum psi_nb + (lapfac0 + V + g|psi|^2) psi (GPBlocks.cpp:576-579), on the
    fixture's vortex state: equal to rounding (relative 1e-12)."""
    d, (X, Y, Z, V, deg, steps, iters), (lapfac, lapfac0, g, volume, dt) = _load()
    args = d["args"]
    bs, half = float(args[2]), float(args[3])
    lat = capi.Lattice("bcc")
    bw = lat.block_width
    p0 = [0.5 * (-half + half - bs * bw[i] * [X, Y, Z][i]) for i in range(3)]
    p = capi.make_params(components=1, precision=capi.FP64, dims=(X, Y, Z), block_scale=bs, p0=p0, dt=0.5 * dt,
                         c0=g / dt, trap_offset=0.0)
    even_ref = _gp_to_ref_layout(d["even"], X, Y, Z, V)
    odd_ref = _gp_to_ref_layout(d["odd"], X, Y, Z, V)
    nsteps = 6
    e, o = d["even"].copy(), d["odd"].copy()
    oracle.gpblocks_run(X, Y, Z, V, deg, d["lapind"], lapfac, lapfac0, g, d["pot"].copy(), e, o, nsteps // 2)
    newest = oracle.leapfrog_run(lat, p, even_ref, odd_ref, nsteps, fields=capi.make_fields())
    want = _gp_to_ref_layout(e, X, Y, Z, V)
    scale = np.abs(want).max()
    assert np.abs(newest - want).max() <= 1e-12 * scale


def test_golden_fixture_regenerates():
    """Where the reference tree and its compiled checker are present, a fresh run
    of the reference reproduces the committed fixture."""
    exe = os.path.join(os.path.dirname(oracle.HERE), "oracle", "_ref", "ref_gpblocks")
    if not os.path.exists(exe):
        pytest.skip("reference checker not built here")
    import subprocess
    import tempfile

    import importlib.util

    spec = importlib.util.spec_from_file_location("mg", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "dump.bin")
        subprocess.run([exe, out] + list(mg.CASES["gpblocks_bcc"]), check=True, cwd=tmp, capture_output=True)
        fresh = mg.read_dump(out)
    d = np.load(GOLDEN)
    for k in ("normsq_error", "psi0", "pot", "lapind"):
        assert np.array_equal(fresh[k], d[k]), k
