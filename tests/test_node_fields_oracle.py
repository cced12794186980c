"""The oracle's per-node output fields (orc_node_fields) on states with known
answers: localAvgSpinAndDensity (Spin1GpeBCC.cu:235-271), uvTheta (:273-326),
maxHamilton (:144-189) and the x/y-quantised projections (Spin1GpeBCC/utils.h:
177-193).  CPU only; tests/test_gpu_parity.py compares the kernels with it."""
import numpy as np
import pytest

from oracle import oracle
from spacetime_gb300 import capi, states


def _setup(C, seed=3):
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=C, precision=capi.FP64, dims=(3, 2, 2), block_scale=0.3, trap_offset=100.0,
                         c0=120.0, c2=-7.0, lattice=lat)
    return lat, p, 0.3 * states.random_state(capi.buffer_shape(lat, p), seed=seed)


def _interior(psi, C):
    u = psi[1:-1, 1:-1, 1:-1]
    return u[..., 0] + 1j * u[..., 1]


def test_projections_keep_the_density():
    lat, p, psi = _setup(3)
    rho = oracle.node_fields(lat, p, capi.make_fields(), 0.0, capi.FIELD_DENSITY, psi)[..., 0]
    for kind in (capi.FIELD_PROJ_X, capi.FIELD_PROJ_Y):
        q = oracle.node_fields(lat, p, capi.make_fields(), 0.0, kind, psi)
        np.testing.assert_allclose(q.sum(axis=-1), rho, rtol=1e-13)


@pytest.mark.parametrize("C", [3, 5])
def test_uv_theta_frame(C):
    """u and v are orthogonal, |u| >= |v|, |u|^2 + |v|^2 = |s1|^2 + |s0|^2 + |s_1|^2."""
    lat, p, psi = _setup(C)
    f = oracle.node_fields(lat, p, capi.make_fields(), 0.0, capi.FIELD_UV_THETA, psi)
    u, v, th = f[..., 0:3], f[..., 3:6], f[..., 6]
    c = _interior(psi, C)
    mid = c[..., 1:4] if C == 5 else c
    rho3 = np.sum(np.abs(mid) ** 2, axis=-1)
    np.testing.assert_allclose(np.sum(u * v, axis=-1), 0.0, atol=1e-13)
    assert np.all(np.linalg.norm(u, axis=-1) >= np.linalg.norm(v, axis=-1))
    np.testing.assert_allclose(np.sum(u * u + v * v, axis=-1), rho3, rtol=1e-12)
    if C == 3:
        assert np.all((th >= 0) & (th < np.pi))


def test_spin_of_polar_and_ferromagnetic_nodes():
    """Polar (0, a, 0): no spin.  Ferromagnetic (a, 0, 0): the normalised x, y
    components vanish and z = |a|^2 of the unnormalised spinor, so the reference's
    spin norm is rho * |a|^2 = rho^2."""
    lat, p, psi = _setup(3)
    pol = psi.copy()
    pol[..., 0, :] = 0.0
    pol[..., 2, :] = 0.0
    s = oracle.node_fields(lat, p, capi.make_fields(), 0.0, capi.FIELD_SPIN, pol)
    np.testing.assert_allclose(s[..., 0:4], 0.0, atol=1e-15)
    fer = psi.copy()
    fer[..., 1, :] = 0.0
    fer[..., 2, :] = 0.0
    s = oracle.node_fields(lat, p, capi.make_fields(), 0.0, capi.FIELD_SPIN, fer)
    rho = s[..., 4]
    np.testing.assert_allclose(s[..., 3], rho, rtol=1e-14)
    np.testing.assert_allclose(s[..., 0], rho * rho, rtol=1e-14)
    np.testing.assert_allclose(s[..., 1:3], 0.0, atol=1e-15)


def test_max_hamilton_bounds_the_potential():
    lat, p, psi = _setup(3)
    f = capi.make_fields(bq=0.2, bb=(0.1, -0.3, 0.5))
    h = oracle.node_fields(lat, p, f, 0.0, capi.FIELD_MAX_HAMILTON, psi)[..., 0]
    rho = oracle.node_fields(lat, p, f, 0.0, capi.FIELD_DENSITY, psi)[..., 0]
    r = states.node_positions(lat, p)
    pot = 0.5 * np.sum(r * r, axis=-1) + 100.0 + 120.0 * rho
    assert np.all(h >= pot)
    assert np.all(h <= pot + 10.0)


def test_rejects_fields_the_component_count_lacks():
    lat, p, psi = _setup(1)
    for kind in (capi.FIELD_SPIN, capi.FIELD_UV_THETA, capi.FIELD_MAX_HAMILTON):
        with pytest.raises(RuntimeError):
            oracle.node_fields(lat, p, capi.make_fields(), 0.0, kind, psi)
