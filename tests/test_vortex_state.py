"""gpe_vortex_profile / gpe_vortex_sample (the reference's VortexState, host code)
against what the reference itself produced: tests/golden/gpblocks_bcc.npz holds
the initial state of the reference's CPU stepper, built by its own VortexState
(kappa = 1, g = 40, setRange(0, 4, 4, 0.1, 0.1), 400 relaxation sweeps, trap ratio
1; GPBlocks.cpp:460-486 sampled it at the BCC nodes of a 9^3-cell grid of block
scale 0.25 over [-3, 3]^3), and its odd state is that state times the phase
e^{i mu dt / 2} of the profile's mu (getPhase, VortexState.cpp:198-202;
GPBlocks.cpp:515-523).  Host code only: runs without a GPU."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from spacetime_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "gpblocks_bcc.npz")


@pytest.fixture(scope="module")
def lib():
    from spacetime_gb300 import build

    build.build()
    return capi.load_library()


def _gp_to_ref_layout(a, X, Y, Z, V):
    n = (Z + 2) * (Y + 1) * (X + 1) * V
    c = a.reshape(-1, 2)[:n].reshape(Z + 2, Y + 1, X + 1, V, 2)
    out = np.zeros((Z + 2, Y + 2, X + 2, V, 1, 2))
    out[1:-1, 1:-1, 1:-1, :, 0, :] = c[1:Z + 1, 1:Y + 1, 1:X + 1]
    return out


def test_vortex_state_is_the_references(lib):
    d = np.load(GOLDEN)
    X, Y, Z, V, deg, steps, iters = (int(v) for v in d["dims"])
    dt = float(d["scal"][4])
    kappa, g, bs, half, _, sweeps = (float(v) for v in d["args"])
    lat = capi.Lattice("bcc")
    bw = lat.block_width
    p0 = [0.5 * (-half + half - bs * bw[i] * [X, Y, Z][i]) for i in range(3)]
    p = capi.make_params(components=1, precision=capi.FP64, dims=(X, Y, Z), block_scale=bs, p0=p0, lattice=lat)
    psi, mu, taken = capi.vortex_state(lat, p, kappa=int(kappa), g=g, rmax=half + 1.0, zmax=half + 1.0, max_iters=int(sweeps),
                                       eps=1e-29)
    assert taken == int(sweeps)
    want = _gp_to_ref_layout(d["psi0"], X, Y, Z, V)
    scale = float(np.max(np.abs(want)))
    assert float(np.max(np.abs(psi - want))) <= 1e-13 * scale
    # mu from the phase between the reference's odd and even initial states
    e = d["even"].reshape(-1, 2)
    o = d["odd"].reshape(-1, 2)
    i = int(np.argmax(np.hypot(e[:, 0], e[:, 1])))
    angle = math.atan2(e[i, 0] * o[i, 1] - e[i, 1] * o[i, 0], e[i, 0] * o[i, 0] + e[i, 1] * o[i, 1])
    assert mu == pytest.approx(angle / (0.5 * dt), rel=1e-12)


def test_vortex_profile_converges_and_rejects(lib):
    """Run to convergence, the relaxation is a fixed point: mu settles, the
    profile is non-negative and vanishes on the axis; a bad grid is refused."""
    vp = capi.VortexParams(1, 40.0, 0.0, 4.0, 0.1, 4.0, 0.1, 1.0, 100000, 1e-26)
    rs, zs = C.c_uint32(), C.c_uint32()
    assert lib.gpe_vortex_profile(C.byref(vp), None, 0, C.byref(rs), C.byref(zs), None, None) == 0
    assert (rs.value, zs.value) == (40, 40)
    f = np.zeros(rs.value * zs.value)
    mu, it = C.c_double(), C.c_uint32()
    assert lib.gpe_vortex_profile(C.byref(vp), f.ctypes.data_as(C.POINTER(C.c_double)), f.size, None, None, C.byref(mu),
                                  C.byref(it)) == 0
    assert it.value < 100000 and np.all(f >= -1e-12) and np.all(f[:zs.value] == 0)
    vp.max_iters = it.value + 50
    mu2 = C.c_double()
    assert lib.gpe_vortex_profile(C.byref(vp), f.ctypes.data_as(C.POINTER(C.c_double)), f.size, None, None, C.byref(mu2),
                                  None) == 0
    assert mu2.value == pytest.approx(mu.value, rel=1e-10)
    bad = capi.VortexParams(1, 40.0, 2.0, 1.0, 0.1, 4.0, 0.1, 1.0, 10, 1e-26)
    assert lib.gpe_vortex_profile(C.byref(bad), None, 0, None, None, None, None) == 1
    assert lib.gpe_vortex_profile(C.byref(vp), f.ctypes.data_as(C.POINTER(C.c_double)), 10, None, None, None, None) == 1
