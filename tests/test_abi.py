"""The C ABI: library loads, exports every declared symbol, host-side logic."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle
from spacetime_gb300 import capi

from conftest import has_gpu


@pytest.fixture(scope="module")
def lib():
    from spacetime_gb300 import build

    build.build()
    return capi.load_library()


def test_exports_every_declared_symbol(lib):
    names = capi.exported_symbols_from_header()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n


def test_version(lib):
    assert b"sm_103a" in lib.gpe_version()


def _ramps():
    yield capi.make_ramp(bq_segments=[(4.3, 10.0, capi.RAMP_LINEAR), (4.3, 192.03, capi.RAMP_CONSTANT), (0.0, 0.2, capi.RAMP_LINEAR), (0.0, 2000.0, capi.RAMP_CONSTANT)],
                         bb_segments=[((0, 0, 1.0), 10, capi.RAMP_CONSTANT), ((0, 0, 0.045), 10, capi.RAMP_LINEAR), ((0, 0, 0.045), 2.02, capi.RAMP_CONSTANT),
                                      ((0, 0, 0), 180, capi.RAMP_LINEAR), ((0, 0, 1.2), 0.5, capi.RAMP_SQRT), ((0, 0, 1.2), 2000.0, capi.RAMP_CONSTANT)],
                         time_scale=1.0, bq_scale=-0.37, bb_scale=-2.1, bq_quad_scale=0.5, bb_quad_scale=0.25)
    yield capi.make_ramp(bq_segments=[(0.2, 1e9, capi.RAMP_CONSTANT)],
                         bb_segments=[((0, 0, 0.5), 0.0, capi.RAMP_CONSTANT), ((0.1, -0.2, -0.5), 0.2, capi.RAMP_LINEAR), ((0, 0, -0.5), 1e9, capi.RAMP_CONSTANT)])
    yield capi.make_ramp()


@pytest.mark.parametrize("k", range(3))
def test_ramp_eval_matches_oracle(lib, k):
    """Host ramp evaluation (getSignal, AliceRingRamps.h:74-141) of the library
    equals the oracle's, at segment boundaries, inside segments and past the end."""
    ramp = list(_ramps())[k]
    for tau in [0.0, 1e-9, 5.0, 10.0, 15.0, 22.02, 100.0, 202.02, 202.3, 202.52, 203.0, 5000.0, 0.1, 0.2, 0.35]:
        a = capi.Fields()
        assert lib.gpe_ramp_eval(C.byref(ramp), tau, C.byref(a)) == 0
        b = oracle.ramp_eval(ramp, tau)
        for f in ("bq", "bq_quad"):
            assert getattr(a, f) == pytest.approx(getattr(b, f), rel=1e-15, abs=1e-15), (tau, f)
        for i in range(3):
            assert a.bb[i] == pytest.approx(b.bb[i], rel=1e-15, abs=1e-15)
            assert a.bb_quad[i] == pytest.approx(b.bb_quad[i], rel=1e-15, abs=1e-15)


def test_ramp_linear_values(lib):
    r = list(_ramps())[1]
    f = capi.Fields()
    lib.gpe_ramp_eval(C.byref(r), 0.1, C.byref(f))
    assert f.bq == pytest.approx(0.2)
    assert f.bb[2] == pytest.approx(0.0)  # halfway from 0.5 to -0.5
    assert f.bb[0] == pytest.approx(0.05)


def test_lattice_validation_rejects_bad_tables(lib):
    lat = capi.Lattice("bcc")
    h = C.c_void_p()
    assert lib.gpe_lattice_create(C.byref(lat.desc), C.byref(h)) == 0
    lib.gpe_lattice_destroy(h)
    # asymmetric stencil
    bad = capi.Lattice("bcc")
    bad._stencil[0].node = (bad._stencil[0].node + 1) % bad.nodes
    assert lib.gpe_lattice_create(C.byref(bad.desc), C.byref(h)) == 1
    assert b"symmetric" in lib.gpe_last_error()
    # offset out of range
    bad = capi.Lattice("bcc")
    bad._stencil[3].dx = 2
    assert lib.gpe_lattice_create(C.byref(bad.desc), C.byref(h)) == 1
    # node count out of range
    bad = capi.Lattice("bcc")
    bad.desc.nodes = 0
    assert lib.gpe_lattice_create(C.byref(bad.desc), C.byref(h)) == 1
    assert b"nodes" in lib.gpe_last_error()
    assert lib.gpe_lattice_create(None, C.byref(h)) == 1


def test_create_rejects_bad_params(lib):
    lat = capi.Lattice("bcc")
    L = C.c_void_p()
    assert lib.gpe_lattice_create(C.byref(lat.desc), C.byref(L)) == 0
    h = C.c_void_p()
    p = capi.make_params(components=2, lattice=lat)
    assert lib.gpe_create(L, C.byref(p), C.byref(h)) == 1
    p = capi.make_params(components=3, dims=(0, 4, 4), lattice=lat)
    assert lib.gpe_create(L, C.byref(p), C.byref(h)) == 1
    p = capi.make_params(components=3, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.0, lattice=lat)
    assert lib.gpe_create(L, C.byref(p), C.byref(h)) == 6
    lf = capi.Lattice("fcc")
    LF = C.c_void_p()
    assert lib.gpe_lattice_create(C.byref(lf.desc), C.byref(LF)) == 0
    p = capi.make_params(components=3, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01, lattice=lf)
    assert lib.gpe_create(LF, C.byref(p), C.byref(h)) == 6  # FCC has no d0/d1 tables
    p = capi.make_params(components=5, flags=capi.FLAG_QUADRATIC_ZEEMAN, lattice=lat)
    assert lib.gpe_create(L, C.byref(p), C.byref(h)) == 6
    if not has_gpu():
        p = capi.make_params(components=3, lattice=lat)
        assert lib.gpe_create(L, C.byref(p), C.byref(h)) == 7  # no device here: an error, never a CPU path
    lib.gpe_lattice_destroy(L)
    lib.gpe_lattice_destroy(LF)


def test_null_handles(lib):
    assert lib.gpe_step(None, 1, None) == 1
    assert lib.gpe_start(None, None) == 1
    assert lib.gpe_destroy(None) == 0
    assert lib.gpe_sites(None) == 0


def test_noalloc_rejects_bad_tables_and_alignment_on_host(lib):
    """gpe_observe_noalloc checks its tables and the buffer's alignment before it
    touches the GPU: a row table that does not start at 0 or that decreases would
    index the by-value stencil outside its rows, and a pointer or pitch off the
    complex value's size would make a misaligned vector load."""
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=3, precision=capi.FP32, dims=(4, 4, 4), lattice=lat)
    shape = capi.buffer_shape(lat, p)
    pitch = shape[2] * lat.nodes * 3 * 8
    slice_pitch = pitch * shape[1]
    o = capi.Observables()

    def call(desc, ptr, pt, sp, q=p):
        return lib.gpe_observe_noalloc(C.byref(desc), C.byref(q), None, 0.0, C.c_void_p(ptr), pt, sp, C.byref(o), None)

    for bad in ([1], [0, 4, 2]):
        rp = lat.row_ptr.copy()
        rp[:len(bad)] = bad
        d = capi.LatticeDesc.from_buffer_copy(lat.desc)
        d.row_ptr = rp.ctypes.data_as(C.POINTER(C.c_int32))
        assert call(d, 1 << 20, pitch, slice_pitch) == 1
        assert b"row_ptr" in lib.gpe_last_error()
    for ptr, pt, sp in (((1 << 20) + 4, pitch, slice_pitch), (1 << 20, pitch + 4, slice_pitch + 4 * shape[1]),
                        (1 << 20, pitch, slice_pitch + 4)):
        assert call(lat.desc, ptr, pt, sp) == 1
        assert b"multiples" in lib.gpe_last_error()
    p64 = capi.make_params(components=3, precision=capi.FP64, dims=(4, 4, 4), lattice=lat)
    assert call(lat.desc, (1 << 20) + 8, 2 * pitch, 2 * slice_pitch, p64) == 1


def test_python_constants_match_header_enums():
    """Every GPE_* enumerator of include/gpe.h that the Python front end names
    (tuning keys, batch keys, kernels, slots, flags) has the header's value."""
    import os
    import re

    hdr = open(os.path.join(os.path.dirname(capi.__file__), "..", "include", "gpe.h")).read()
    values = {}
    for body in re.findall(r"enum\s*\{([^}]*)\}", hdr):
        nxt = 0
        for item in re.sub(r"/\*.*?\*/", "", body, flags=re.S).split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, val = (x.strip() for x in item.split("="))
                nxt = int(val, 0)
            else:
                name = item
            values[name] = nxt
            nxt += 1
    pairs = {"GPE_TUNE_KERNEL": capi.TUNE_KERNEL, "GPE_TUNE_TIMING": capi.TUNE_TIMING,
             "GPE_TUNE_TRANSFER": capi.TUNE_TRANSFER, "GPE_TUNE_OBSERVE_ARITH": capi.TUNE_OBSERVE_ARITH,
             "GPE_BATCH_ITEM_NODES": capi.BATCH_ITEM_NODES, "GPE_BATCH_STEPS_PER_LAUNCH": capi.BATCH_STEPS_PER_LAUNCH,
             "GPE_BATCH_BLOCKS_PER_SM": capi.BATCH_BLOCKS_PER_SM, "GPE_BATCH_LAYOUT": capi.BATCH_LAYOUT,
             "GPE_BATCH_BARRIER_TIMEOUT_MS": capi.BATCH_BARRIER_TIMEOUT_MS}
    for name, v in pairs.items():
        assert values.get(name) == v, name
