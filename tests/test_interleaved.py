"""The interleaved step kernel (GPE_TUNE_KERNEL 6, and the automatic choice for
calls of 16 or more steps): the two psi slots are changed into a cell-interleaved
layout, stepped there and changed back.  Its arithmetic and order are those of the
gather kernel, so the states it leaves are compared with the gather kernel's bit
for bit, and with the FP64 oracle to the FP32 tolerance of the other parity tests.
"""
import numpy as np
import pytest

from oracle import oracle
from spacetime_gb300 import capi, states
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu

FIELDS = dict(bq=0.3, bb=(0.1, -0.2, 0.5), bq_quad=0.2, bb_quad=(0.05, 0.1, -0.3))


def _params(lat, C, dims, **kw):
    base = dict(components=C, precision=capi.FP32, dims=dims, block_scale=0.3, dt=2e-4, trap_offset=100.0,
                trap_lambda=(1.0, 1.1, 1.3), c0=120.0, c2=-7.0, c4=3.0, lattice=lat)
    base.update(kw)
    return capi.make_params(**base)


def _ramp(dt):
    return capi.make_ramp(bq_segments=[(0.3, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0.1, -0.2, 0.5), 0.0, capi.RAMP_CONSTANT),
                                       ((0.0, 0.1, -0.5), 30 * dt, capi.RAMP_LINEAR),
                                       ((0.0, 0.1, -0.5), 1e9, capi.RAMP_CONSTANT)], bq_quad_scale=0.5, bb_quad_scale=0.25)


def _state(lat, p, seed, amp=0.2):
    return amp * states.random_state(capi.buffer_shape(lat, p, False), seed=seed)


# (lattice, C, dims): X a multiple of 32, ragged (padding cells), and below 32
CASES = [("bcc", 3, (64, 3, 2)), ("bcc", 3, (40, 5, 3)), ("bcc", 1, (37, 4, 3)), ("bcc", 5, (33, 3, 2)),
         ("bcc", 3, (9, 4, 5)), ("a15", 3, (35, 2, 2)), ("a15", 1, (6, 3, 2)), ("c15", 1, (33, 2, 2)),
         ("c15", 5, (5, 2, 2)), ("z", 3, (34, 2, 2)), ("fcc", 3, (40, 3, 2)), ("fcc", 1, (33, 2, 3)),
         ("fcc", 5, (7, 3, 2)), ("fcc", 3, (64, 2, 2))]


@pytest.mark.parametrize("name,C,dims", CASES)
def test_interleaved_equals_gather(gpu, name, C, dims):
    """20 leapfrog steps with a ramp of the fields: the interleaved kernel leaves
    both psi slots bit for bit as the gather kernel does."""
    lat = capi.Lattice(name)
    flags = capi.FLAG_QUADRATIC_ZEEMAN | capi.FLAG_QUADRUPOLE_OFFSET if C == 3 else 0
    p = _params(lat, C, dims, flags=flags, quad_center=(0.1, -0.2, 0.05))
    psi = _state(lat, p, 7)
    ramp = _ramp(p.dt)
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        a.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_GATHER)
        b.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        assert b.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_INTERLEAVED
        b.set_tuning(capi.TUNE_TIMING, 1)
        for s in (a, b):
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(ramp, 0.0)
            s.start()
            s.step(20)
        t = b.step_timing()
        assert t["interleaved_calls"] == 1 and t["step_launches"] == 20 and t["convert_launches"] == 4
        assert a.current == b.current
        for slot in (capi.PSI_EVEN, capi.PSI_ODD):
            np.testing.assert_array_equal(a.download(slot), b.download(slot), err_msg="slot %d" % slot)


@pytest.mark.parametrize("name,C,dims", [("bcc", 3, (40, 3, 2)), ("a15", 1, (34, 2, 2)), ("bcc", 5, (9, 3, 2)),
                                         ("fcc", 3, (35, 2, 2))])
def test_interleaved_against_oracle(gpu, name, C, dims):
    """Three steps from two random states against the FP64 oracle's leapfrog
    (FP32 tolerance 2e-5 of the state's scale), through gpe_step with the
    interleaved kernel forced."""
    lat = capi.Lattice(name)
    p = _params(lat, C, dims)
    even, odd = _state(lat, p, 11), _state(lat, p, 12)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        s.set_ramp(None, 0.0)
        cur = s.current  # gpe_step reads this slot and writes the other
        s.step(3)
        ge, go = s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)
    b = {capi.PSI_EVEN: even.copy(), capi.PSI_ODD: odd.copy()}
    f = capi.make_fields()
    for n in range(3):
        prev, nxt = cur, (capi.PSI_ODD if cur == capi.PSI_EVEN else capi.PSI_EVEN)
        oracle.parabolic_step(lat, p, f, (n + 1) * p.dt, oracle.LEAPFROG, b[nxt], b[prev])
        cur = nxt
    for got, want in ((ge, b[capi.PSI_EVEN]), (go, b[capi.PSI_ODD])):
        scale = float(np.max(np.abs(want)))
        assert float(np.max(np.abs(got - want))) <= 2e-5 * scale


def test_automatic_choice_by_call_length(gpu):
    """The automatic choice steps calls of 16 or more steps in the interleaved
    layout and shorter calls with the gather kernel; the states agree."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, (40, 4, 3))
    psi = _state(lat, p, 21)
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        for s in (a, b):
            s.set_tuning(capi.TUNE_TIMING, 1)
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(_ramp(p.dt), 0.0)
            s.start()
        a.step(20)
        for _ in range(4):
            b.step(5)
        ta, tb = a.step_timing(), b.step_timing()
        assert ta["interleaved_calls"] == 1 and ta["calls"] == 1
        assert tb["interleaved_calls"] == 0 and tb["calls"] == 4 and tb["step_launches"] == 20
        assert tb["convert_launches"] == 0 and tb["step_ms"] > 0
        np.testing.assert_array_equal(a.download(a.current), b.download(b.current))


@pytest.mark.parametrize("name,C,dims", [("bcc", 3, (40, 5, 3)), ("c15", 1, (33, 2, 2)), ("bcc", 5, (34, 3, 2)),
                                         ("fcc", 3, (34, 3, 2))])
def test_interleaved_step_observe(gpu, name, C, dims):
    """gpe_step_observe(20) in the interleaved layout: the states of the gather
    kernel's plain steps to rounding (the observed step is another kernel, whose
    multiply-adds the compiler may contract differently: 1e-6 of the state's
    scale, as for the gather kernel's own observed step), and the observables of
    the state the last step reads equal gpe_observe of that state (FP32 node terms
    summed in another order: 2e-6 of the norm / energy scale)."""
    lat = capi.Lattice(name)
    p = _params(lat, C, dims)
    psi = _state(lat, p, 31)
    n = 20
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        a.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_GATHER)
        for s in (a, b):
            s.set_tuning(capi.TUNE_OBSERVE_ARITH, 1)
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(_ramp(p.dt), 0.0)
            s.start()
        b.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        b.set_tuning(capi.TUNE_TIMING, 1)
        a.step(n - 1)
        want = a.observe(a.current, n * p.dt)
        a.step(1)
        got = b.step_observe(n)
        t = b.step_timing()
        assert t["interleaved_calls"] == 1 and t["observed_launches"] == 1 and t["step_launches"] == n - 1
        assert a.current == b.current
        for slot in (capi.PSI_EVEN, capi.PSI_ODD):
            sa, sb = a.download(slot), b.download(slot)
            assert float(np.max(np.abs(sa - sb))) <= 1e-6 * float(np.max(np.abs(sa))), "slot %d" % slot
    scale = max(abs(want["norm"]), abs(want["h_expect"]))
    for k in ("norm", "energy", "h_expect", "spin_norm"):
        assert got[k] == pytest.approx(want[k], rel=2e-6, abs=2e-6 * scale), k
    np.testing.assert_allclose(got["magnetization"], want["magnetization"], rtol=2e-6, atol=2e-6 * scale)
    np.testing.assert_allclose(got["com"], want["com"], rtol=2e-6, atol=2e-5 * scale)
    assert got["max_abs"] == pytest.approx(want["max_abs"], rel=1e-6)
    assert got["nonfinite"] == 0


@pytest.mark.parametrize("name,C,want", [("bcc", 3, 1), ("a15", 3, 1), ("bcc", 5, 1), ("z", 5, 1), ("bcc", 1, 0),
                                         ("z", 3, 1), ("c15", 3, 1), ("c15", 5, 1), ("c15", 1, 0), ("a15", 1, 0),
                                         ("fcc", 3, 1), ("fcc", 5, 1), ("fcc", 1, 0)])
def test_automatic_choice_by_lattice(gpu, name, C, want):
    """The automatic choice takes the interleaved kernel for long calls on spinor
    handles (where it measured faster) and keeps the gather kernel for scalars;
    forced, it applies to scalars too, on every lattice with rows of 4 (or of 4 and
    8) entries."""
    lat = capi.Lattice(name)
    p = _params(lat, C, (33, 2, 2) if lat.nodes > 40 else (40, 3, 2))
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_TIMING, 1)
        s.upload(capi.PSI_ODD, _state(lat, p, 9))
        s.start()
        s.step(16)
        assert s.step_timing()["interleaved_calls"] == want
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        s.step(1)
        assert s.step_timing()["interleaved_calls"] == 1


def test_interleaved_rejected_where_it_does_not_apply(gpu):
    """FP64, the cube's rows of 6 entries (parabolic) and 6 edges per node
    (hyperbolic), the split scheme: no interleaved kernel; the automatic choice
    stays the gather kernel there."""
    cases = [("bcc", dict(precision=capi.FP64)), ("cube", {}), ("cube", dict(scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01)),
             ("bcc", dict(scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01, precision=capi.FP64))]
    for name, kw in cases:
        lat = capi.Lattice(name)
        with Stepper(lat, _params(lat, 3, (40, 3, 2), **kw)) as s:
            with pytest.raises(capi.GpeError):
                s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
            s.set_tuning(capi.TUNE_TIMING, 1)
            s.upload(capi.PSI_ODD, _state(lat, s.params, 3))
            s.start()
            s.step(20)
            assert s.step_timing()["interleaved_calls"] == 0


def test_explicit_kernels_keep_their_layout(gpu):
    """An explicitly chosen kernel (gather, row tile) is not replaced by the
    interleaved one on long calls."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, (40, 4, 3))
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_TIMING, 1)
        s.upload(capi.PSI_ODD, _state(lat, p, 5))
        s.start()
        for k in (capi.KERNEL_GATHER, capi.KERNEL_TILE):
            s.set_tuning(capi.TUNE_KERNEL, k)
            s.step(20)
            assert s.step_timing()["interleaved_calls"] == 0


# hyperbolic (psi + q): x edges giving groups of 16 (40, 33, 37, 48, 9) and of 32 cells (64, 20)
HYPER_CASES = [("bcc", 3, (40, 3, 2)), ("bcc", 3, (64, 2, 2)), ("bcc", 5, (33, 2, 2)), ("bcc", 1, (37, 3, 2)),
               ("c15", 5, (5, 2, 2)), ("c15", 5, (20, 1, 2)), ("c15", 3, (48, 2, 1)), ("bcc227", 3, (9, 3, 2))]


def _hyper_pair(name, C, dims, seed):
    lat = capi.Lattice(name)
    p = _params(lat, C, dims, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01)
    return lat, p, _state(lat, p, seed)


@pytest.mark.parametrize("name,C,dims", HYPER_CASES)
def test_interleaved_hyperbolic_equals_gather(gpu, name, C, dims):
    """20 fused hyperbolic steps (update_psi + update_q, RelativisticSpin2Gpe.cu:1873-1874)
    with a ramp: the interleaved kernel leaves psi and q, both slots of each, bit
    for bit as the gather kernel does; one call, 8 layout changes."""
    lat, p, psi = _hyper_pair(name, C, dims, 17)
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        a.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_GATHER)
        b.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        assert b.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_INTERLEAVED
        for s in (a, b):
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(_ramp(p.dt), 0.0)
            s.start()
        b.set_tuning(capi.TUNE_TIMING, 1)
        for s in (a, b):
            s.step(20)
        t = b.step_timing()
        assert t["interleaved_calls"] == 1 and t["step_launches"] == 20 and t["convert_launches"] == 8
        assert a.current == b.current
        for slot in (capi.PSI_EVEN, capi.PSI_ODD, capi.Q_EVEN, capi.Q_ODD):
            np.testing.assert_array_equal(a.download(slot), b.download(slot), err_msg="slot %d" % slot)


@pytest.mark.parametrize("name,C,dims", [("bcc", 3, (35, 2, 2)), ("c15", 5, (3, 2, 1))])
def test_interleaved_hyperbolic_against_oracle(gpu, name, C, dims):
    """gpe_start then 5 interleaved hyperbolic steps against the FP64 oracle's
    start and time loop (FP32 tolerance 2e-5 of the state's scale, psi and q)."""
    from oracle import oracle as orc
    lat, p, psi = _hyper_pair(name, C, dims, 23)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        s.upload(capi.PSI_ODD, psi)
        s.set_ramp(None, 0.0)
        s.start()
        s.step(5)
        got_p, got_q = s.download(s.current), s.download(capi.Q_EVEN if s.current == capi.PSI_EVEN else capi.Q_ODD)
    p64 = _params(lat, C, dims, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01, precision=capi.FP64)
    po, pe = psi.copy(), np.zeros_like(psi)
    qo = np.zeros(capi.buffer_shape(lat, p64, True))
    qe = np.zeros_like(qo)
    f0 = capi.make_fields()
    orc.q_step(lat, p64, orc.Q_PARA, qo, qo, po)
    orc.q_psi_step(lat, p64, f0, 0.0, orc.EULER, False, pe, po, qo)
    orc.q_step(lat, p64, orc.Q_PARA, qe, qe, pe)
    rp, rq = orc.hyper_run(lat, p64, pe, po, qe, qo, 5)
    for got, want in ((got_p, rp), (got_q, rq)):
        scale = float(np.max(np.abs(want)))
        assert float(np.max(np.abs(got - want))) <= 2e-5 * scale


def test_interleaved_hyperbolic_step_observe(gpu):
    """gpe_step_observe(20) on a hyperbolic spinor handle: 19 interleaved steps, the
    observables of the state the last step reads, then that step -- the states and
    observables of the gather kernel's call (the same kernels' arithmetic)."""
    lat, p, psi = _hyper_pair("bcc", 3, (40, 3, 2), 29)
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        a.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_GATHER)
        for s in (a, b):
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(_ramp(p.dt), 0.0)
            s.start()
        b.set_tuning(capi.TUNE_TIMING, 1)
        oa, ob = a.step_observe(20), b.step_observe(20)
        assert b.step_timing()["interleaved_calls"] == 1
        for slot in (capi.PSI_EVEN, capi.PSI_ODD, capi.Q_EVEN, capi.Q_ODD):
            np.testing.assert_array_equal(a.download(slot), b.download(slot))
        for k in ("norm", "energy", "h_expect"):
            assert oa[k] == ob[k], k


@pytest.mark.parametrize("C,want", [(3, 1), (5, 1), (1, 1)])
def test_interleaved_hyperbolic_automatic_choice(gpu, C, want):
    """Calls of 16 or more steps on hyperbolic handles take the interleaved kernel
    by themselves (it measured faster for every spin)."""
    lat, p, psi = _hyper_pair("bcc", C, (40, 3, 2), 31)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_TIMING, 1)
        s.upload(capi.PSI_ODD, psi)
        s.start()
        s.step(16)
        assert s.step_timing()["interleaved_calls"] == want


@pytest.mark.parametrize("name,C,dims", [("bcc", 3, (40, 3, 2)), ("fcc", 5, (9, 2, 2))])
def test_interleaved_with_expansion_and_trap_switch(gpu, name, C, dims):
    """Condensate expansion (the block scale growing from the 5th step on, weights h
    / bs(t)^2 and positions bs(t)) and the trap switched off mid-call: the
    interleaved kernel's states equal the gather kernel's bit for bit."""
    lat = capi.Lattice(name)
    p = _params(lat, C, dims, flags=capi.FLAG_TRAP_OFF_AFTER, trap_off_time=7.5 * 2e-4)
    psi = _state(lat, p, 37)
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        a.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_GATHER)
        b.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_INTERLEAVED)
        b.set_tuning(capi.TUNE_TIMING, 1)
        for s in (a, b):
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(_ramp(p.dt), 0.0)
            s.set_expansion(4 * p.dt, 30.0)
            s.start()
            s.step(20)
        assert b.step_timing()["interleaved_calls"] == 1
        for slot in (capi.PSI_EVEN, capi.PSI_ODD):
            np.testing.assert_array_equal(a.download(slot), b.download(slot), err_msg="slot %d" % slot)
