"""Batched stepping (gpe_batch_*) against the members stepped one by one.

Members of different lattices, sizes, component counts, traps and ramps (one with
the trap switched off mid-run) are advanced by the persistent batch kernel --
directly, over several launches, and by CUDA-graph replay -- and compared with
the same members stepped by gpe_step with the one-node-per-thread kernel, which
computes the same per-node update: FP64 max |diff| <= 1e-12 * max|ref|, FP32
<= 2e-6 * max|ref| (the fields are evaluated on the device instead of the host).
"""
import ctypes as C

import numpy as np
import pytest
import torch

from spacetime_gb300 import capi, states
from spacetime_gb300.batch import Batch
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu

TOL = {capi.FP64: 1e-12, capi.FP32: 2e-6}

SPECS = [("bcc", 3, (7, 5, 4)), ("fcc", 1, (6, 5, 4)), ("a15", 3, (3, 4, 3)), ("c15", 1, (3, 2, 3)),
         ("bcc", 1, (5, 6, 7)), ("c15", 3, (2, 3, 2)), ("bcc227", 5, (4, 3, 3))]


def _member(spec, prec, idx, kernel=capi.KERNEL_GATHER):
    name, comps, dims = spec
    lat = capi.Lattice(name)
    flags = capi.FLAG_TRAP_OFF_AFTER if idx == 1 else 0
    p = capi.make_params(components=comps, precision=prec, dims=dims, block_scale=0.3, dt=2e-4, trap_offset=100.0,
                         trap_lambda=(0.8 + 0.05 * idx, 1.0, 1.2 - 0.04 * idx), c0=120.0 + 10 * idx, c2=-7.0, c4=3.0,
                         flags=flags, trap_off_time=1.5e-3, lattice=lat)
    s = Stepper(lat, p)
    s.set_tuning(capi.TUNE_KERNEL, kernel)
    s.upload(capi.PSI_ODD, 0.2 * states.random_state(capi.buffer_shape(lat, p), seed=100 + idx))
    ramp = capi.make_ramp(bq_segments=[(0.1 * idx, 0.0, capi.RAMP_CONSTANT), (0.3, 12 * 2e-4, capi.RAMP_LINEAR)],
                          bb_segments=[((0.0, 0.0, 0.5), 0.0, capi.RAMP_CONSTANT),
                                       ((0.1 * idx, -0.1, -0.5), 10 * 2e-4, capi.RAMP_LINEAR),
                                       ((0.2, 0.0, 0.3), 6 * 2e-4, capi.RAMP_SQRT)],
                          bq_quad_scale=0.5, bb_quad_scale=0.25)
    s.set_ramp(ramp, t0=1e-4 * idx)
    s.start()
    return s


def _pair(prec):
    return [_member(sp, prec, i) for i, sp in enumerate(SPECS)], [_member(sp, prec, i) for i, sp in enumerate(SPECS)]


def _compare(batched, ref, prec):
    for a, b in zip(batched, ref):
        assert a.current == b.current
        for slot in (capi.PSI_EVEN, capi.PSI_ODD):
            x, y = a.download(slot), b.download(slot)
            scale = float(np.max(np.abs(y)))
            err = float(np.max(np.abs(x - y)))
            assert err <= TOL[prec] * scale, (slot, err, scale)


def _close(ms):
    for m in ms:
        m.close()


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("per_launch", [0, 3])
def test_batch_step_matches_members(gpu, prec, per_launch):
    mem, ref = _pair(prec)
    try:
        with Batch(mem) as b:
            b.set_tuning(capi.BATCH_ITEM_NODES, 200)  # several items per member
            b.set_tuning(capi.BATCH_STEPS_PER_LAUNCH, per_launch)
            b.step(11)
            n0 = b.launches
            # FP32 spin-1 members of lattices up to 64 nodes a cell (not C15) are
            # stepped in the interleaved layout: 4 layout changes each per call
            n_il = sum(1 for sp in SPECS if sp[1] == 3 and sp[0] != "c15") if prec == capi.FP32 else 0
            assert b.get_tuning(capi.BATCH_LAYOUT) == 1
            assert n0 == (1 if per_launch == 0 else 4) + 4 * n_il
        for r in ref:
            r.step(11)
        _compare(mem, ref, prec)
    finally:
        _close(mem + ref)


def test_batch_graph_replay(gpu):
    prec = capi.FP32
    mem, ref = _pair(prec)
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    try:
        with Batch(mem) as b:
            b.stream = sp
            b.set_tuning(capi.BATCH_STEPS_PER_LAUNCH, 2)
            b.capture(5, sp)
            b.replay()
            b.replay()
            for m in mem:  # the members stay usable on their own between batched calls
                m.step(1)
            b.replay()
        for r in ref:
            r.step(16)
        _compare(mem, ref, prec)
    finally:
        _close(mem + ref)


def test_batch_layouts_agree(gpu):
    """FP32 spin-1 members stepped in the interleaved layout (GPE_BATCH_LAYOUT 1,
    FCC's rows of 4 and 8 and groups of 16 and 32 cells included) leave every
    member's two psi slots bit for bit as the handle layout (0) does, directly and
    through a captured graph."""
    specs = [("bcc", 3, (40, 3, 2)), ("fcc", 3, (35, 2, 3)), ("fcc", 3, (64, 2, 2)), ("a15", 3, (3, 2, 2)),
             ("c15", 3, (2, 2, 3)), ("bcc", 1, (5, 6, 7)), ("fcc", 5, (6, 3, 2)), ("bcc", 3, (50, 2, 2))]
    outs = []
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    for layout in (0, 1):
        mem = [_member(spec, capi.FP32, i) for i, spec in enumerate(specs)]
        try:
            with Batch(mem) as b:
                b.stream = sp
                b.set_tuning(capi.BATCH_LAYOUT, layout)
                assert b.get_tuning(capi.BATCH_LAYOUT) == layout
                b.set_tuning(capi.BATCH_ITEM_NODES, 300)
                b.step(6)
                b.capture(5, sp)
                b.replay()
            outs.append([(m.current, m.download(capi.PSI_EVEN), m.download(capi.PSI_ODD)) for m in mem])
        finally:
            _close(mem)
    for (ca, ea, oa), (cb, eb, ob) in zip(*outs):
        assert ca == cb
        np.testing.assert_array_equal(ea, eb)
        np.testing.assert_array_equal(oa, ob)


def test_batch_autotune_keeps_state(gpu):
    prec = capi.FP32
    mem, ref = _pair(prec)
    try:
        with Batch(mem) as b:
            rep = b.autotune(steps=2)
            assert len(rep) == 4 * 4 and all(r["ms_per_step"] > 0 for r in rep)  # 4 lattice keys x 4 sizes
            b.step(4)
        for r in ref:
            r.step(4)
        _compare(mem, ref, prec)
    finally:
        _close(mem + ref)


def test_batch_rejects(gpu):
    lat = capi.Lattice("bcc")
    p32 = capi.make_params(components=3, precision=capi.FP32, dims=(4, 4, 4), block_scale=0.3, dt=1e-4, lattice=lat)
    p64 = capi.make_params(components=3, precision=capi.FP64, dims=(4, 4, 4), block_scale=0.3, dt=1e-4, lattice=lat)
    a, b2 = Stepper(lat, p32), Stepper(lat, p64)
    try:
        with pytest.raises(capi.GpeError):
            Batch([a, b2])
        with pytest.raises(capi.GpeError):
            Batch([a, a])
        hl = capi.Lattice("bcc")
        ph = capi.make_params(components=3, scheme=capi.SCHEME_HYPERBOLIC, precision=capi.FP32, dims=(4, 4, 4),
                              block_scale=0.3, dt=1e-4, sigma=0.01, lattice=hl)
        try:
            h = Stepper(hl, ph)
        except capi.GpeError:
            h = None
        if h is not None:
            with pytest.raises(capi.GpeError) as e:
                Batch([a, h])
            assert e.value.status == 6  # GPE_ERR_UNSUPPORTED
            h.close()
    finally:
        a.close()
        b2.close()


def test_batch_barrier_timeout_is_reported(gpu):
    """The grid barrier's bounded wait: with one arrival that never comes every
    wait runs out after the set limit, the kernel returns, the call reports
    GPE_ERR_TIMEOUT, and the batch steps normally afterwards."""
    prec = capi.FP32
    mem, ref = _pair(prec)
    try:
        with Batch(mem) as b:
            b.set_tuning(capi.BATCH_BARRIER_TIMEOUT_MS, 50)
            b.set_tuning(capi.BATCH_TEST_EXTRA_ARRIVALS, 1)
            with pytest.raises(capi.GpeError) as e:
                b.step(2)
            assert e.value.status == 4  # GPE_ERR_TIMEOUT
            b.set_tuning(capi.BATCH_TEST_EXTRA_ARRIVALS, 0)
            for m in mem:  # the timed-out call left the members' states undefined: restart them
                m.upload(capi.PSI_ODD, 0.2 * states.random_state(capi.buffer_shape(m.lattice, m.params), seed=5))
            for r in ref:
                r.upload(capi.PSI_ODD, 0.2 * states.random_state(capi.buffer_shape(r.lattice, r.params), seed=5))
            for m, r in zip(mem, ref):
                m.start()
                r.start()
            b.step(3)
        for r in ref:
            r.step(3)
        _compare(mem, ref, prec)
    finally:
        _close(mem + ref)


def test_batch_constant_slots_exhausted(gpu):
    """An FP32 batch created while another live batch holds all 256 constant-memory
    slots of the device reads its members' constants from shared memory instead:
    the same states, bit for bit, as the constant-memory form."""
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=1, precision=capi.FP32, dims=(2, 2, 2), block_scale=0.3, dt=2e-4, lattice=lat)
    fillers = [Stepper(lat, p) for _ in range(256)]
    outs = []
    try:
        for hold in (True, False):
            mem = [_member(sp, capi.FP32, i) for i, sp in enumerate(SPECS)]
            holder = Batch(fillers) if hold else None
            try:
                with Batch(mem) as b:
                    b.step(7)
                outs.append([m.download(m.current) for m in mem])
            finally:
                if holder is not None:
                    holder.close()
                _close(mem)
    finally:
        _close(fillers)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
def test_batch_matches_oracle(gpu, prec):
    """A mixed batch (BCC spin-1, FCC scalar with the trap switched off mid-run,
    C15 scalar, A15 spin-1, FCC spin-1), every member against the FP64 CPU oracle's own time
    loop: forwardEuler at t0, then leapfrog steps with the member's ramp evaluated
    at t0 + (k+1) dt (Spin1GpeBCC.cu:1428-1603).  FP64 <= 1e-12 and FP32 <= 2e-5 of
    max|psi|, the parity tolerances of the single-condensate kernels."""
    from oracle import oracle

    specs = [("bcc", 3, (7, 5, 4)), ("fcc", 1, (6, 5, 4)), ("c15", 1, (3, 2, 3)), ("a15", 3, (3, 4, 3)),
             ("fcc", 3, (5, 3, 2))]
    n = 9
    members, init = [], []
    for i, sp in enumerate(specs):
        s = _member(sp, prec, i)
        init.append(s.download(capi.PSI_ODD))
        members.append(s)
    try:
        with Batch(members) as b:
            b.set_tuning(capi.BATCH_ITEM_NODES, 150)
            b.step(n)
        for i, (sp, s) in enumerate(zip(specs, members)):
            name, comps, dims = sp
            lat = capi.Lattice(name)
            flags = capi.FLAG_TRAP_OFF_AFTER if i == 1 else 0
            p = capi.make_params(components=comps, precision=capi.FP64, dims=dims, block_scale=0.3, dt=2e-4,
                                 trap_offset=100.0, trap_lambda=(0.8 + 0.05 * i, 1.0, 1.2 - 0.04 * i), c0=120.0 + 10 * i,
                                 c2=-7.0, c4=3.0, flags=flags, trap_off_time=1.5e-3, lattice=lat)
            ramp = capi.make_ramp(bq_segments=[(0.1 * i, 0.0, capi.RAMP_CONSTANT), (0.3, 12 * 2e-4, capi.RAMP_LINEAR)],
                                  bb_segments=[((0.0, 0.0, 0.5), 0.0, capi.RAMP_CONSTANT),
                                               ((0.1 * i, -0.1, -0.5), 10 * 2e-4, capi.RAMP_LINEAR),
                                               ((0.2, 0.0, 0.3), 6 * 2e-4, capi.RAMP_SQRT)],
                                  bq_quad_scale=0.5, bb_quad_scale=0.25)
            t0 = 1e-4 * i
            odd = init[i].copy()
            even = np.zeros_like(odd)
            oracle.parabolic_step(lat, p, oracle.ramp_eval(ramp, ramp.time_scale * t0), t0, oracle.EULER, even, odd)
            want = oracle.leapfrog_run(lat, p, even, odd, n, ramp=ramp, t0=t0)
            got = s.download(s.current)
            scale = float(np.max(np.abs(want)))
            err = float(np.max(np.abs(got - want)))
            tol = 1e-12 if prec == capi.FP64 else 2e-5
            assert err <= tol * scale, (name, comps, err, scale)
    finally:
        _close(members)
