"""gpe_observe_noalloc: observables of a caller-owned buffer with no device allocation.

It serves callers that cannot allocate device memory at the point where they
want the norm, energy and magnetisation of their state (memory owned by another
framework's pool, or a time loop that laid out every buffer up front).  Checked
through the C ABI against the handle-based gpe_observe on the same buffer, on two
calls in a row, within the FP64 reduction tolerance used by the other
observables tests (the two reductions add the same FP64 terms in a different
order).  This file is collected last so that a failing run has already run the
others; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from spacetime_gb300 import capi, states
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu

REL = 1e-11


def _noalloc(lib, lat, p, fields, t, pitched):
    o = capi.Observables()
    st = lib.gpe_observe_noalloc(C.byref(lat.desc), C.byref(p), C.byref(fields), t, pitched.ptr, pitched.pitch,
                                 pitched.slice_pitch, C.byref(o), None)
    return st, o.as_dict()


def _compare(a, b):
    for k in ("norm", "energy", "h_expect", "spin_norm", "max_abs"):
        assert a[k] == pytest.approx(b[k], rel=REL, abs=1e-13), k
    np.testing.assert_allclose(a["magnetization"], b["magnetization"], rtol=REL, atol=1e-13)
    np.testing.assert_allclose(a["com"], b["com"], rtol=REL, atol=1e-13)
    assert a["nonfinite"] == b["nonfinite"] == 0


@pytest.mark.parametrize("prec", [capi.FP32, capi.FP64])
@pytest.mark.parametrize("name,C,dims", [("bcc", 3, (9, 7, 5)), ("bcc", 5, (6, 5, 4)), ("c15", 1, (3, 3, 2)),
                                         ("bcc", 3, (96, 96, 8))])
def test_noalloc_matches_observe_twice(gpu, name, C, dims, prec):
    lib = gpu
    lat = capi.Lattice(name)
    p = capi.make_params(components=C, precision=prec, dims=dims, block_scale=0.3, dt=1e-4, trap_offset=100.0,
                         trap_lambda=(1.0, 1.1, 1.3), c0=120.0, c2=-7.0, c4=3.0, lattice=lat)
    fields = capi.make_fields(bq=0.3, bb=(0.1, -0.2, 0.5))
    ramp = capi.make_ramp(bq_segments=[(fields.bq, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[(tuple(fields.bb), 1e9, capi.RAMP_CONSTANT)])
    shape = capi.buffer_shape(lat, p)
    with Stepper(lat, p) as s:
        s.set_ramp(ramp, 0.0)
        pitched, _ = s.buffer(capi.PSI_EVEN)
        for call in range(2):
            psi = 0.2 * states.random_state(shape, seed=500 + call)
            s.upload(capi.PSI_EVEN, psi)
            want = s.observe(capi.PSI_EVEN, t=0.0)
            st, got = _noalloc(lib, lat, p, fields, 0.0, pitched)
            assert st == capi.GPE_OK, lib.gpe_last_error()
            _compare(got, want)


def test_noalloc_matches_observe_with_physics_switches(gpu):
    """The switches the no-alloc kernel builds into its own parameters by hand:
    quadratic Zeeman, quadrupole offset (non-zero bb_quad and bq_quad) and the
    trap switched off after trap_off_time, on two calls in a row either side of
    that time."""
    lib = gpu
    lat = capi.Lattice("bcc")
    flags = capi.FLAG_QUADRATIC_ZEEMAN | capi.FLAG_QUADRUPOLE_OFFSET | capi.FLAG_TRAP_OFF_AFTER
    p = capi.make_params(components=3, precision=capi.FP64, flags=flags, dims=(7, 6, 5), block_scale=0.3, dt=1e-4,
                         trap_offset=100.0, trap_off_time=0.5, trap_lambda=(1.0, 1.1, 1.3), c0=120.0, c2=-7.0,
                         quad_center=(0.1, -0.2, 0.3), lattice=lat)
    ramp = capi.make_ramp(bq_segments=[(0.3, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0.1, -0.2, 0.5), 1e9, capi.RAMP_CONSTANT)], bq_quad_scale=0.7, bb_quad_scale=0.4)
    shape = capi.buffer_shape(lat, p)
    with Stepper(lat, p) as s:
        s.set_ramp(ramp, 0.0)
        pitched, _ = s.buffer(capi.PSI_EVEN)
        for call, t in enumerate((0.25, 0.75)):
            fields = capi.Fields()
            assert lib.gpe_ramp_eval(C.byref(ramp), t, C.byref(fields)) == 0
            assert fields.bq_quad != 0 and any(fields.bb_quad[i] != 0 for i in range(3))
            s.upload(capi.PSI_EVEN, 0.2 * states.random_state(shape, seed=700 + call))
            want = s.observe(capi.PSI_EVEN, t=t)
            st, got = _noalloc(lib, lat, p, fields, t, pitched)
            assert st == capi.GPE_OK, lib.gpe_last_error()
            _compare(got, want)


def test_noalloc_during_expansion(gpu):
    """With condensate expansion the caller passes the current block scale
    bs(t) as block_scale; the integrals then carry dv = bs(t)^3 VOLUME where the
    handle keeps bs0^3 VOLUME."""
    lib = gpu
    lat = capi.Lattice("bcc")
    bs0, t0, rate = 0.3, 0.1, 2.0
    p = capi.make_params(components=3, precision=capi.FP64, dims=(7, 6, 5), block_scale=bs0, dt=1e-4, trap_offset=100.0,
                         c0=120.0, c2=-7.0, lattice=lat)
    fields = capi.make_fields(bq=0.3, bb=(0.1, -0.2, 0.5))
    ramp = capi.make_ramp(bq_segments=[(fields.bq, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[(tuple(fields.bb), 1e9, capi.RAMP_CONSTANT)])
    shape = capi.buffer_shape(lat, p)
    with Stepper(lat, p) as s:
        s.set_ramp(ramp, 0.0)
        s.set_expansion(t0, rate)
        pitched, _ = s.buffer(capi.PSI_EVEN)
        for call, t in enumerate((0.2, 0.4)):
            bs = bs0 * (1.0 + rate * (t - t0))
            # the box origin p0 stays where the handle set it; only the block scale grows
            q = capi.make_params(components=3, precision=capi.FP64, dims=(7, 6, 5), block_scale=bs, dt=1e-4,
                                 p0=tuple(p.p0), trap_offset=100.0, c0=120.0, c2=-7.0, lattice=lat)
            s.upload(capi.PSI_EVEN, 0.2 * states.random_state(shape, seed=800 + call))
            want = s.observe(capi.PSI_EVEN, t=t)
            st, got = _noalloc(lib, lat, q, fields, t, pitched)
            assert st == capi.GPE_OK, lib.gpe_last_error()
            k = (bs0 / bs) ** 3
            for key in ("norm", "energy", "h_expect", "spin_norm"):
                got[key] *= k
            got["magnetization"] = [m * k for m in got["magnetization"]]
            got["com"] = [c * k for c in got["com"]]
            _compare(got, want)


def test_noalloc_rejects_oversized_tables(gpu):
    lib = gpu
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=3, precision=capi.FP32, dims=(4, 4, 4), lattice=lat)
    with Stepper(lat, p) as s:
        pitched, _ = s.buffer(capi.PSI_EVEN)
        big = capi.LatticeDesc.from_buffer_copy(lat.desc)
        big.nodes = 161
        o = capi.Observables()
        st = lib.gpe_observe_noalloc(C.byref(big), C.byref(p), None, 0.0, pitched.ptr, pitched.pitch,
                                     pitched.slice_pitch, C.byref(o), None)
        assert st == 1 and b"static table size" in lib.gpe_last_error()
        q = capi.make_params(components=3, precision=capi.FP32, dims=(1 << 12, 1 << 10, 1 << 10), lattice=lat)
        st = lib.gpe_observe_noalloc(C.byref(lat.desc), C.byref(q), None, 0.0, pitched.ptr, pitched.pitch,
                                     pitched.slice_pitch, C.byref(o), None)
        assert st == 1 and b"2^32" in lib.gpe_last_error()
