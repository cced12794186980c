"""Host-side pieces of the adjoint path (no GPU): knot interpolation, the
monopole target state, and the ctypes signatures of the adjoint entry points."""
import math

import numpy as np
import torch

from spacetime_gb300 import capi, states
from spacetime_gb300.adjoint import BB_Z, BQ, RampControl, knot_matrix


def test_knot_matrix_rows_sum_to_one():
    W = knot_matrix(16, 2000)
    assert W.shape == (2000, 16)
    assert np.allclose(W.sum(axis=1), 1.0)
    assert W[0, 0] == 1.0 and W[-1, -1] == 1.0
    # a linear function of the knot position is reproduced exactly
    k = np.linspace(-1.0, 1.0, 16)
    assert np.allclose(W @ k, np.linspace(-1.0, 1.0, 2000))


def test_ramp_control_fields_layout():
    class _Dummy:
        pass

    rc = RampControl(_Dummy(), 100, 16, lambda: None, np.zeros(4))
    bq = torch.linspace(0.0, 1.0, 16, dtype=torch.float64)
    bz = torch.linspace(1.0, -1.0, 16, dtype=torch.float64)
    f = rc.fields(bq, bz)
    assert f.shape == (100, 4)
    assert torch.allclose(f[:, BQ], torch.linspace(0.0, 1.0, 100, dtype=torch.float64))
    assert torch.allclose(f[:, BB_Z], torch.linspace(1.0, -1.0, 100, dtype=torch.float64))
    assert float(f[:, 1].abs().max()) == 0.0 and float(f[:, 2].abs().max()) == 0.0


def test_monopole_state_is_a_normalised_hedgehog():
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=3, dims=(8, 8, 8), block_scale=0.25, c0=200.0, lattice=lat)
    psi = states.monopole_state(lat, p, noise=0.0)
    dv = p.block_scale ** 3 * lat.volume
    assert math.isclose(float(np.sum(psi ** 2)) * dv, 1.0, rel_tol=1e-12)
    # the local spin <F> of a polar state vanishes; its nematic director is r_hat:
    # psi_0 / |psi| = n_z
    r = states.node_positions(lat, p)
    u = psi[1:-1, 1:-1, 1:-1]
    c = u[..., 0] + 1j * u[..., 1]
    amp = np.sqrt(np.sum(np.abs(c) ** 2, axis=-1))
    fz = np.abs(c[..., 0]) ** 2 - np.abs(c[..., 2]) ** 2
    assert np.max(np.abs(fz)) < 1e-14
    nz = r[..., 2] / np.linalg.norm(r, axis=-1)
    mask = amp > 1e-3 * amp.max()
    assert np.allclose((c[..., 1].real / np.where(mask, amp, 1.0))[mask], nz[mask], atol=1e-12)


def test_adjoint_symbols_have_signatures():
    lib = capi.load_library()
    for name in ("gpe_adjoint_forward", "gpe_adjoint_backward"):
        assert getattr(lib, name).argtypes is not None
