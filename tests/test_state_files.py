"""Reference state files (raw host arrays of BlockPsis / BlockEdges cells with
their halo, Spin1GpeBCC.cu:1215-1237, 1690-1699; RelativisticSpin2Gpe.cu:
1428-1441, 1695-1706): byte-exact round trips on the host, and through a handle
on the GPU."""
import numpy as np
import pytest

from spacetime_gb300 import capi, states
from spacetime_gb300.stepper import Stepper


def _lat_params(C=3, prec=capi.FP64, scheme=capi.SCHEME_PARABOLIC):
    lat = capi.Lattice("bcc")
    return lat, capi.make_params(components=C, precision=prec, dims=(4, 3, 2), block_scale=0.3, scheme=scheme,
                                 sigma=0.01, lattice=lat)


def test_file_bytes_are_the_host_array(tmp_path):
    lat, p = _lat_params()
    psi = states.random_state(capi.buffer_shape(lat, p), seed=9)
    path = tmp_path / "state.dat"
    states.write_state_file(path, psi)
    raw = path.read_bytes()
    # what fs.write((char*)&h_psi[0], hostSize * sizeof(BlockPsis)) writes
    assert raw == psi.astype("<f8").tobytes()
    assert len(raw) == (4 + 2) * (3 + 2) * (2 + 2) * lat.nodes * 3 * 2 * 8
    back = states.read_state_file(path, lat, p)
    np.testing.assert_array_equal(back, psi)


def test_edge_file_and_size_check(tmp_path):
    lat, p = _lat_params(C=5, scheme=capi.SCHEME_HYPERBOLIC)
    q = states.random_state(capi.buffer_shape(lat, p, edges=True), seed=10)
    path = tmp_path / "q.dat"
    states.write_state_file(path, q)
    np.testing.assert_array_equal(states.read_state_file(path, lat, p, edges=True), q)
    with pytest.raises(ValueError):
        states.read_state_file(path, lat, p)  # a q file is not a psi file of this grid


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
def test_load_and_save_through_a_handle(gpu, tmp_path, prec):
    lat, p = _lat_params(prec=prec)
    psi = states.random_state(capi.buffer_shape(lat, p), seed=11)
    src, dst = tmp_path / "in.dat", tmp_path / "out.dat"
    states.write_state_file(src, psi)
    with Stepper(lat, p) as s:
        s.load_state(capi.PSI_ODD, str(src))
        s.save_state(capi.PSI_ODD, str(dst))
    want = psi if prec == capi.FP64 else psi.astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(states.read_state_file(dst, lat, p), want)
