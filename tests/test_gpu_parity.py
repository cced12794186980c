"""CUDA kernels (through the C ABI) against the FP64 CPU oracle.

FP64 plain kernels: max |gpu - oracle| <= 1e-12 * max|oracle| (the kernels contract
multiply-adds, the oracle does not; differences are rounding only).
FP32 fused kernels: max |gpu - oracle| <= 2e-5 * max|oracle| after a few steps from
moderate random states (FP32 has a 6e-8 unit roundoff; a handful of steps of a
4-neighbour stencil stays well inside this bound).
"""
import numpy as np
import pytest

from oracle import oracle
from spacetime_gb300 import capi, states
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu

TOL = {capi.FP64: 1e-12, capi.FP32: 2e-5}

FIELDS = dict(bq=0.3, bb=(0.1, -0.2, 0.5), bq_quad=0.2, bb_quad=(0.05, 0.1, -0.3))


def _params(lat, C, prec, dims, **kw):
    base = dict(components=C, precision=prec, dims=dims, block_scale=0.3, dt=2e-4, trap_offset=100.0,
                trap_lambda=(1.0, 1.1, 1.3), c0=120.0, c2=-7.0, c4=3.0, lattice=lat)
    base.update(kw)
    return capi.make_params(**base)


def _rand(lat, p, seed, amp=0.2, edges=False):
    return amp * states.random_state(capi.buffer_shape(lat, p, edges), seed=seed)


def _close(gpu, ref, prec, what=""):
    scale = float(np.max(np.abs(ref)))
    err = float(np.max(np.abs(gpu - ref)))
    assert err <= TOL[prec] * max(scale, 1e-30), "%s: max|gpu-oracle| = %.3e, scale %.3e" % (what, err, scale)


CASES = [
    ("bcc", 1), ("bcc", 3), ("bcc", 5),
    ("bcc227", 1), ("cube", 1), ("cube", 3), ("cube", 5),
    ("fcc", 1), ("fcc", 3), ("fcc", 5), ("a15", 1), ("a15", 3), ("a15", 5), ("c15", 1), ("c15", 5), ("z", 1), ("z", 3),
]


@pytest.mark.parametrize("kernel", [capi.KERNEL_GATHER, capi.KERNEL_AUTO])
@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C", CASES)
def test_parabolic_leapfrog(gpu, name, C, prec, kernel):
    """leapfrog (Spin1GpeBCC.cu:793-917 / Spin2GpeBCC.cu:845-990 / BCC.cu:327-347),
    3 steps with external fields, ragged grid; both the gather kernel and the
    automatic choice (the TMA row-tile kernel wherever cells are 16-byte multiples)."""
    lat = capi.Lattice(name)
    dims = (5, 3, 4) if lat.nodes > 40 else (7, 5, 4)
    p = _params(lat, C, prec, dims)
    even, odd = _rand(lat, p, 11), _rand(lat, p, 12)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_KERNEL, kernel)
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        bufs = [capi.PSI_EVEN, capi.PSI_ODD]
        for n in range(3):
            s.step_explicit(bufs[(n + 1) % 2], bufs[n % 2], f, t=0.1 * n)
        got_e, got_o = s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)
    e, o = even.copy(), odd.copy()
    b = [e, o]
    for n in range(3):
        oracle.parabolic_step(lat, p, f, 0.1 * n, oracle.LEAPFROG, b[(n + 1) % 2], b[n % 2])
    _close(got_e, e, prec, "even")
    _close(got_o, o, prec, "odd")


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("flags", [capi.FLAG_THREE_BODY_LOSS, capi.FLAG_QUADRATIC_ZEEMAN, capi.FLAG_QUADRUPOLE_OFFSET,
                                   capi.FLAG_TRAP_OFF_AFTER | capi.FLAG_QUADRATIC_ZEEMAN | capi.FLAG_THREE_BODY_LOSS])
def test_spin1_physics_toggles(gpu, flags, prec):
    """Three-body loss (Spin1GpeBCC.cu:877-880), quadratic Zeeman (:897-912),
    quadrupole offset (:128-137), trap switched off after a time (:114)."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, prec, (6, 4, 3), flags=flags, alpha=0.7, quad_center=(-0.2, -0.49, -0.27), trap_off_time=0.05)
    even, odd = _rand(lat, p, 21), _rand(lat, p, 22)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN, f, t=0.1)
        got = s.download(capi.PSI_ODD)
    oracle.parabolic_step(lat, p, f, 0.1, oracle.LEAPFROG, odd, even)
    _close(got, odd, prec)


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("C", [1, 3, 5])
@pytest.mark.parametrize("mode", [capi.MODE_EULER, capi.MODE_ITP])
def test_euler_and_itp_modes(gpu, C, mode, prec):
    """forwardEuler (Spin1GpeBCC.cu:667-791) and itp (:554-662), H psi stored for ITP."""
    lat = capi.Lattice("bcc")
    p = _params(lat, C, prec, (5, 4, 3))
    prev = _rand(lat, p, 31)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_ODD, prev)
        s.step_explicit(capi.PSI_EVEN, capi.PSI_ODD, f, t=0.0, mode=mode)
        got = s.download(capi.PSI_EVEN)
        hp = s.download(capi.HPSI) if mode == capi.MODE_ITP else None
    nxt = np.zeros_like(prev)
    href = np.zeros_like(prev)
    oracle.parabolic_step(lat, p, f, 0.0, mode, nxt, prev, href)
    _close(got, nxt, prec, "next")
    if hp is not None:
        _close(hp, href, prec, "hpsi")


@pytest.mark.parametrize("kernel,tile", [(capi.KERNEL_GATHER, 0), (capi.KERNEL_AUTO, 0), (capi.KERNEL_AUTO, 4)])
@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C", [("bcc", 1), ("bcc", 3), ("bcc", 5), ("bcc227", 1), ("cube", 3), ("c15", 5), ("c15", 1)])
def test_hyperbolic_fused_step(gpu, name, C, prec, kernel, tile):
    """One fused launch = update_psi + update_q (RelativisticSpin2Gpe.cu:971-1132,
    RelativisticSpin1Gpe common/hyper kernels, RelativisticGpeBCC.cu:179-255): the
    gather kernel, the TMA row-tile kernel (automatic where cells are 16-byte
    multiples), and partial row tiles."""
    lat = capi.Lattice(name)
    dims = (4, 3, 3) if lat.nodes > 40 else (6, 5, 4)
    if tile and lat.nodes > 40:
        tile = 3
    p = _params(lat, C, prec, dims, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01)
    pe, po = _rand(lat, p, 41), _rand(lat, p, 42)
    qe, qo = _rand(lat, p, 43, edges=True), _rand(lat, p, 44, edges=True)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_KERNEL, kernel)
        if tile:
            s.set_tuning(capi.TUNE_TILE_CELLS, tile)
        for slot, a in ((capi.PSI_EVEN, pe), (capi.PSI_ODD, po), (capi.Q_EVEN, qe), (capi.Q_ODD, qo)):
            s.upload(slot, a)
        s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN, f, t=0.2)
        s.step_explicit(capi.PSI_EVEN, capi.PSI_ODD, f, t=0.3)
        got = [s.download(k) for k in (capi.PSI_EVEN, capi.PSI_ODD, capi.Q_EVEN, capi.Q_ODD)]
    oracle.q_psi_step(lat, p, f, 0.2, oracle.LEAPFROG, True, po, pe, qe)
    oracle.q_step(lat, p, oracle.Q_HYPER, qo, qe, pe)
    oracle.q_psi_step(lat, p, f, 0.3, oracle.LEAPFROG, True, pe, po, qo)
    oracle.q_step(lat, p, oracle.Q_HYPER, qe, qo, po)
    for g, r, w in zip(got, (pe, po, qe, qo), ("psi_even", "psi_odd", "q_even", "q_odd")):
        _close(g, r, prec, w)


@pytest.mark.parametrize("kernel", [capi.KERNEL_AUTO, capi.KERNEL_GATHER, capi.KERNEL_TILE])
@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("C", [1, 3, 5])
def test_hyperbolic_start_and_run(gpu, C, prec, kernel):
    """gpe_start (RelativisticSpin2Gpe.cu:1628-1630) then 6 fused steps with a ramp,
    with the automatic kernel choice, the gather kernel and the fused tile kernel."""
    lat = capi.Lattice("bcc")
    p = _params(lat, C, prec, (6, 4, 5), scheme=capi.SCHEME_HYPERBOLIC, sigma=0.02)
    psi = _rand(lat, p, 51)
    ramp = capi.make_ramp(bq_segments=[(0.25, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0, 0, 0.5), 0.0, capi.RAMP_CONSTANT), ((0, 0, -0.5), 4 * p.dt, capi.RAMP_LINEAR),
                                       ((0, 0, -0.5), 1e9, capi.RAMP_CONSTANT)])
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_KERNEL, kernel)
        assert s.get_tuning(capi.TUNE_KERNEL) == (kernel or (2 if C == 3 else 1))
        s.upload(capi.PSI_ODD, psi)
        s.set_ramp(ramp, 0.0)
        s.start()
        s.step(6)
        got_p, got_q = s.download(capi.PSI_EVEN), s.download(capi.Q_EVEN)
    po, pe = psi.copy(), np.zeros_like(psi)
    qo = np.zeros(capi.buffer_shape(lat, p, True))
    qe = np.zeros_like(qo)
    f0 = oracle.ramp_eval(ramp, 0.0)
    oracle.q_step(lat, p, oracle.Q_PARA, qo, qo, po)
    oracle.q_psi_step(lat, p, f0, 0.0, oracle.EULER, False, pe, po, qo)
    oracle.q_step(lat, p, oracle.Q_PARA, qe, qe, pe)
    rp, rq = oracle.hyper_run(lat, p, pe, po, qe, qo, 6, ramp=ramp)
    _close(got_p, rp, prec, "psi")
    _close(got_q, rq, prec, "q")


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C", [("bcc", 1), ("bcc", 3), ("bcc", 5), ("fcc", 3), ("c15", 5)])
def test_observables(gpu, name, C, prec):
    """FP64 reductions (density/energy/magnetisation/centre of mass) against the oracle."""
    lat = capi.Lattice(name)
    p = _params(lat, C, prec, (5, 4, 3))
    psi = _rand(lat, p, 61)
    if prec == capi.FP32:
        psi = psi.astype(np.float32).astype(np.float64)  # same stored values on both sides
    f = capi.make_fields(**FIELDS)
    ramp = capi.make_ramp(bq_segments=[(f.bq, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[(tuple(f.bb), 1e9, capi.RAMP_CONSTANT)])
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, psi)
        s.set_ramp(ramp, 0.0)
        got = s.observe(capi.PSI_EVEN, t=0.0)
    want = oracle.observe(lat, p, oracle.ramp_eval(ramp, 0.0), 0.0, psi)
    for k in ("norm", "energy", "h_expect", "spin_norm", "max_abs"):
        assert got[k] == pytest.approx(want[k], rel=1e-11, abs=1e-12), k
    for k in ("magnetization", "com"):
        np.testing.assert_allclose(got[k], want[k], rtol=1e-11, atol=1e-12)
    assert got["nonfinite"] == 0


@pytest.mark.parametrize("name,C", [("bcc", 1), ("bcc", 3), ("c15", 5)])
def test_observables_fp32_node_terms(gpu, name, C):
    """GPE_TUNE_OBSERVE_ARITH = 1: per-node terms in FP32, sums in FP64; within 1e-5
    (relative to the norm / energy scale) of the FP64 oracle on the same stored values."""
    lat = capi.Lattice(name)
    p = _params(lat, C, capi.FP32, (6, 5, 4))
    psi = _rand(lat, p, 62).astype(np.float32).astype(np.float64)
    f = capi.make_fields(**FIELDS)
    ramp = capi.make_ramp(bq_segments=[(f.bq, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[(tuple(f.bb), 1e9, capi.RAMP_CONSTANT)])
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, psi)
        s.set_ramp(ramp, 0.0)
        s.set_tuning(capi.TUNE_OBSERVE_ARITH, 1)
        assert s.get_tuning(capi.TUNE_OBSERVE_ARITH) == 1
        got = s.observe(capi.PSI_EVEN, t=0.0)
    want = oracle.observe(lat, p, oracle.ramp_eval(ramp, 0.0), 0.0, psi)
    for k in ("norm", "energy", "h_expect", "spin_norm"):
        assert got[k] == pytest.approx(want[k], rel=1e-5, abs=1e-5 * abs(want["h_expect"])), k
    np.testing.assert_allclose(got["magnetization"], want["magnetization"], rtol=1e-5, atol=1e-5 * want["norm"])
    np.testing.assert_allclose(got["com"], want["com"], rtol=1e-5, atol=1e-5 * want["norm"])


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
def test_imaginary_time(gpu, prec):
    """gpe_itp = itp + normalize, twice per iteration pair (Spin1GpeBCC.cu:1470-1490)."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, prec, (6, 5, 4), dt=1e-3)
    psi = np.abs(_rand(lat, p, 71)) + 0.0
    psi = states.normalize(psi, lat, p)
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_ODD, psi)
        mu = s.itp(4)
        assert s.current == capi.PSI_ODD  # 4 iterations from PSI_ODD end in PSI_ODD
        got = s.download(s.current)
        obs = s.observe(s.current)
    cur = psi.copy()
    hp = np.zeros_like(psi)
    for _ in range(4):
        nxt = np.zeros_like(psi)
        oracle.parabolic_step(lat, p, capi.make_fields(), 0.0, oracle.ITP, nxt, cur, hp)
        oracle.normalize(lat, p, nxt)
        cur = nxt
    dv = p.block_scale ** 3 * lat.volume
    mu_ref = float(np.sum(cur[1:-1, 1:-1, 1:-1] * hp[1:-1, 1:-1, 1:-1])) * dv
    _close(got, cur, prec)
    assert obs["norm"] == pytest.approx(1.0, rel=1e-10 if prec == capi.FP64 else 1e-6)
    assert mu == pytest.approx(mu_ref, rel=1e-11 if prec == capi.FP64 else 1e-5)


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C", [("bcc", 1), ("bcc", 3), ("bcc", 5), ("c15", 5), ("cube", 3)])
def test_hyperbolic_imaginary_time(gpu, name, C, prec):
    """gpe_itp on a hyperbolic handle: itp_q + itp_psi in one launch, then
    normalize_h, per iteration (RelativisticSpin2Gpe.cu:1712-1715), and H psi /
    mu of the last iteration."""
    lat = capi.Lattice(name)
    dims = (4, 3, 3) if lat.nodes > 40 else (6, 5, 4)
    p = _params(lat, C, prec, dims, dt=1e-3, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.1)
    po = states.normalize(_rand(lat, p, 81), lat, p)
    qo = _rand(lat, p, 82, edges=True)
    with Stepper(lat, p) as s:
        assert s.current == capi.PSI_ODD
        s.upload(capi.PSI_ODD, po)
        s.upload(capi.Q_ODD, qo)
        mu = s.itp(5)
        assert s.current == capi.PSI_EVEN
        got_p, got_q, got_h = s.download(capi.PSI_EVEN), s.download(capi.Q_EVEN), s.download(capi.HPSI)
        obs = s.observe(capi.PSI_EVEN)
    hp = np.zeros_like(po)
    rp, rq = oracle.hyper_itp_run(lat, p, po.copy(), np.zeros_like(po), qo.copy(), np.zeros_like(qo), 5, hpsi=hp)
    dv = p.block_scale ** 3 * lat.volume
    mu_ref = float(np.sum(rp[1:-1, 1:-1, 1:-1] * hp[1:-1, 1:-1, 1:-1])) * dv
    _close(got_p, rp, prec, "psi")
    _close(got_q, rq, prec, "q")
    _close(got_h, hp, prec, "H psi")
    assert obs["norm"] == pytest.approx(1.0, rel=1e-10 if prec == capi.FP64 else 1e-6)
    assert mu == pytest.approx(mu_ref, rel=1e-11 if prec == capi.FP64 else 1e-5)


def test_hyperbolic_itp_reaches_the_parabolic_ground_state(gpu):
    """Property at a size the oracle loop would take minutes for: the fixed point of
    the hyperbolic imaginary-time loop has q = d0 psi and H psi = mu psi with the
    d1 * d0 operator, which on BCC is the parabolic stencil away from the boundary;
    with the state confined well inside the grid both loops reach the same ground
    state (mu within 1e-8, overlap within 1e-5, q - d0 psi within 1e-5) from the
    same start after 8000 iterations."""
    lat = capi.Lattice("bcc")
    kw = dict(dims=(12, 12, 12), dt=1e-3, trap_offset=0.0, trap_lambda=(2.0, 2.0, 2.0), c0=50.0)
    pp = _params(lat, 1, capi.FP64, **kw)
    ph = _params(lat, 1, capi.FP64, scheme=capi.SCHEME_HYPERBOLIC, sigma=0.1, **kw)
    psi0 = np.abs(_rand(lat, pp, 7))
    for ax in range(3):
        idx = [slice(None)] * 3
        for end in (0, -1):
            idx[ax] = end
            psi0[tuple(idx)] = 0.0
    psi0 = states.normalize(psi0, lat, pp)
    n = 8000
    with Stepper(lat, pp) as s:
        s.upload(capi.PSI_ODD, psi0)
        s.itp(n - 1, want_mu=False)
        mu_p = s.itp(1)
        psi_p = s.download(s.current)
    with Stepper(lat, ph) as s:
        s.upload(capi.PSI_ODD, psi0)
        s.itp(n - 1, want_mu=False)
        mu_h = s.itp(1)
        psi_h, q_h = s.download(s.current), s.download(capi.Q_EVEN if s.current == capi.PSI_EVEN else capi.Q_ODD)
    dv = pp.block_scale ** 3 * lat.volume
    assert mu_h == pytest.approx(mu_p, rel=1e-8)
    assert float(np.sum(psi_h * psi_p)) * dv == pytest.approx(1.0, abs=1e-5)
    d0 = np.zeros_like(q_h)
    oracle.q_step(lat, ph, oracle.Q_PARA, d0, d0, psi_h)
    assert float(np.max(np.abs(q_h - d0))) <= 1e-5 * float(np.max(np.abs(d0)))  # q lags psi by ~sigma/dt steps


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("dims", [(2, 2, 2), (3, 1, 2), (1, 1, 1)])
def test_split_scheme(gpu, dims, prec):
    """C15 real/imaginary split scheme (RelativisticGpeC15/GPUGrossPitaevskii_C15.cu:
    90-155, 469-482): gpe_start's q_R start then 5 steps of two half-step launches."""
    lat = capi.Lattice("c15")
    p = _params(lat, 1, prec, dims, scheme=capi.SCHEME_SPLIT, sigma=0.01, dt=1e-3, trap_offset=0.0,
                trap_lambda=(1.0, 1.0, 1.0), c0=300.0)
    psi, q = _rand(lat, p, 91), _rand(lat, p, 92, edges=True)
    with Stepper(lat, p) as s:
        assert s.current == capi.PSI_EVEN
        s.upload(capi.PSI_EVEN, psi)
        s.upload(capi.Q_EVEN, q)
        n0 = s.launches
        s.start()
        s.step(5)
        assert s.launches - n0 == 11
        got_p, got_q = s.download(capi.PSI_EVEN), s.download(capi.Q_EVEN)
    oracle.split_run(lat, p, psi, q, 5)
    _close(got_p, psi, prec, "psi")
    _close(got_q, q, prec, "q")


def test_split_scheme_rejects(gpu):
    lat = capi.Lattice("c15")
    with pytest.raises(capi.GpeError):  # scalar only
        Stepper(lat, _params(lat, 3, capi.FP64, (2, 2, 2), scheme=capi.SCHEME_SPLIT, sigma=0.01))
    with pytest.raises(capi.GpeError):  # needs edge tables
        Stepper(capi.Lattice("fcc"), _params(capi.Lattice("fcc"), 1, capi.FP64, (2, 2, 2), scheme=capi.SCHEME_SPLIT,
                                             sigma=0.01))
    with Stepper(lat, _params(lat, 1, capi.FP64, (2, 2, 2), scheme=capi.SCHEME_SPLIT, sigma=0.01)) as s:
        with pytest.raises(capi.GpeError):
            s.itp(1)
        with pytest.raises(capi.GpeError):
            s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN)


FIELD_CASES = [(3, k) for k in (capi.FIELD_DENSITY, capi.FIELD_SPIN, capi.FIELD_UV_THETA, capi.FIELD_MAX_HAMILTON,
                                 capi.FIELD_PROJ_X, capi.FIELD_PROJ_Y)] + \
              [(5, capi.FIELD_SPIN), (5, capi.FIELD_UV_THETA), (1, capi.FIELD_DENSITY)]


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("C,kind", FIELD_CASES)
def test_node_fields(gpu, C, kind, prec):
    """gpe_node_fields against the oracle on the same stored values (FP64 fields
    from FP32 or FP64 storage): localAvgSpinAndDensity, uvTheta, maxHamilton,
    projections (Spin1GpeBCC.cu:144-326, Spin2GpeBCC.cu:192-306)."""
    lat = capi.Lattice("bcc")
    p = _params(lat, C, prec, (5, 4, 3))
    psi = _rand(lat, p, 151)
    if prec == capi.FP32:
        psi = psi.astype(np.float32).astype(np.float64)
    f = capi.make_fields(**FIELDS)
    ramp = capi.make_ramp(bq_segments=[(f.bq, 1e9, capi.RAMP_CONSTANT)], bb_segments=[(tuple(f.bb), 1e9, capi.RAMP_CONSTANT)])
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, psi)
        s.set_ramp(ramp, 0.0)
        got = s.node_fields(capi.PSI_EVEN, kind, t=0.0)
    want = oracle.node_fields(lat, p, oracle.ramp_eval(ramp, 0.0), 0.0, kind, psi)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * float(np.max(np.abs(want))))


@pytest.mark.parametrize("C,kind", [(3, capi.FIELD_DENSITY), (3, capi.FIELD_SPIN), (5, capi.FIELD_SPIN),
                                    (3, capi.FIELD_MAX_HAMILTON)])
def test_node_fields_reduce(gpu, C, kind):
    """gpe_node_fields_reduce: integrateSpinAndDensity's spin, density-weighted
    magnetisation and density (Spin1GpeBCC.cu:992-1020) and getMaxHamilton's
    maximum (:1022-1037), from the oracle's per-node fields."""
    lat = capi.Lattice("bcc")
    p = _params(lat, C, capi.FP64, (6, 5, 4))
    psi = _rand(lat, p, 152)
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_ODD, psi)
        got = s.node_fields_reduce(capi.PSI_ODD, kind)
    v = oracle.node_fields(lat, p, capi.make_fields(), 0.0, kind, psi).reshape(-1, oracle.FIELD_WIDTH[kind])
    dv = p.block_scale ** 3 * lat.volume
    if kind == capi.FIELD_SPIN:
        want = np.array([v[:, 0].sum(), (v[:, 4] * v[:, 1]).sum(), (v[:, 4] * v[:, 2]).sum(), (v[:, 4] * v[:, 3]).sum(),
                         v[:, 4].sum()]) * dv
    elif kind == capi.FIELD_MAX_HAMILTON:
        want = np.array([v[:, 0].max()])
    else:
        want = np.array([v[:, 0].sum() * dv])
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14)


def test_node_fields_rejects(gpu):
    lat = capi.Lattice("bcc")
    with Stepper(lat, _params(lat, 1, capi.FP64, (2, 2, 2))) as s:
        with pytest.raises(capi.GpeError):
            s.node_fields(capi.PSI_EVEN, capi.FIELD_SPIN)
        with pytest.raises(capi.GpeError):
            s.node_fields_reduce(capi.PSI_EVEN, capi.FIELD_UV_THETA)
        with pytest.raises(capi.GpeError):
            s.node_fields(capi.PSI_EVEN, 99)


def _bs_at(p, t, t0, rate):
    q = capi.Params.from_buffer_copy(p)
    if t >= t0:
        q.block_scale = p.block_scale * (1.0 + rate * (t - t0))
    return q


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("kernel", [capi.KERNEL_TILE, capi.KERNEL_GATHER, capi.KERNEL_ROWS])
def test_expansion_run(gpu, kernel, prec):
    """gpe_set_expansion: 8 leapfrog steps with a ramp, the block scale growing from
    the 3rd step on (Spin1GpeBCC.cu:1576-1588) and the trap off from then too
    (:112-116), against the oracle stepping with each step's block scale."""
    lat = capi.Lattice("bcc")
    dt = 2e-4
    t_exp, rate = 2.5 * dt, 40.0
    p = _params(lat, 3, prec, (8, 4, 4), dt=dt, flags=capi.FLAG_TRAP_OFF_AFTER, trap_off_time=t_exp)
    even, odd = _rand(lat, p, 161), _rand(lat, p, 162)
    ramp = capi.make_ramp(bq_segments=[(0.3, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0.1, 0.0, 0.5), 0.0, capi.RAMP_CONSTANT), ((0.0, 0.2, -0.5), 6 * dt, capi.RAMP_LINEAR)])
    with Stepper(lat, p) as s:
        try:
            s.set_tuning(capi.TUNE_KERNEL, kernel)
        except capi.GpeError:
            pytest.skip("kernel not available for this shape")
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        s.set_ramp(ramp, 0.0)
        s.set_expansion(t_exp, rate)
        s.step(8)
        got = s.download(s.current)
        obs = s.observe(s.current, t=8 * dt)
    bufs = [odd, even]  # a new handle's newest state is PSI_ODD: step 0 writes PSI_EVEN
    for n in range(8):
        t = (n + 1) * dt
        oracle.parabolic_step(lat, _bs_at(p, t, t_exp, rate), oracle.ramp_eval(ramp, ramp.time_scale * t), t, oracle.LEAPFROG,
                              bufs[(n + 1) % 2], bufs[n % 2])
    _close(got, bufs[8 % 2], prec, "psi")
    pe = _bs_at(p, 8 * dt, t_exp, rate)
    want = oracle.observe(lat, pe, oracle.ramp_eval(ramp, ramp.time_scale * 8 * dt), 8 * dt, bufs[0].astype(np.float32).astype(np.float64)
                          if prec == capi.FP32 else bufs[0])
    vol = (p.block_scale / pe.block_scale) ** 3  # dv stays bs0^3 VOLUME, as in the reference
    tol = 1e-10 if prec == capi.FP64 else 1e-4
    for k in ("norm", "energy", "h_expect"):
        assert obs[k] == pytest.approx(want[k] * vol, rel=tol), k


def test_expansion_rejects(gpu):
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP32, (4, 4, 4))
    with Stepper(lat, p) as s:
        with pytest.raises(capi.GpeError):
            s.set_expansion(0.0, -1.0)
        s.set_expansion(0.0, 10.0)
        with pytest.raises(capi.GpeError):
            s.adjoint_forward(np.zeros((2, 4)), _rand(lat, p, 1))
    ph = _params(lat, 3, capi.FP32, (4, 4, 4), scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01)
    with Stepper(lat, ph) as s:
        with pytest.raises(capi.GpeError):
            s.set_expansion(0.0, 10.0)


def test_leapfrog_run_with_ramp_matches_oracle(gpu):
    """gpe_start + gpe_step(n) with the device-side schedule of a ramp (config-2 shape:
    linear Bz ramp plus a quadrupole gradient) against the oracle time loop."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP64, (8, 6, 5), dt=5e-5, c0=2000.0, c2=-50.0, trap_lambda=(1, 1, 1))
    psi = states.spinor_state(lat, p, states.POLAR, seed=2, noise=1e-2)
    ramp = capi.make_ramp(bq_segments=[(0.2, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0, 0, 0.5), 0.0, capi.RAMP_CONSTANT), ((0, 0, -0.5), 30 * p.dt, capi.RAMP_LINEAR),
                                       ((0, 0, -0.5), 1e9, capi.RAMP_CONSTANT)])
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_ODD, psi)
        s.set_ramp(ramp)
        s.start()
        s.step(41)
        got = s.download(capi.PSI_ODD)
    po, pe = psi.copy(), np.zeros_like(psi)
    oracle.parabolic_step(lat, p, oracle.ramp_eval(ramp, 0.0), 0.0, oracle.EULER, pe, po)
    ref = oracle.leapfrog_run(lat, p, pe, po, 41, ramp=ramp)
    _close(got, ref, capi.FP64)


def test_edge_sizes(gpu):
    """1x1x1 grid and a long thin grid: halo handling at every face."""
    lat = capi.Lattice("bcc")
    for dims in ((1, 1, 1), (17, 1, 2), (1, 9, 1)):
        p = _params(lat, 3, capi.FP64, dims)
        even, odd = _rand(lat, p, 81), _rand(lat, p, 82)
        f = capi.make_fields(**FIELDS)
        with Stepper(lat, p) as s:
            s.upload(capi.PSI_EVEN, even)
            s.upload(capi.PSI_ODD, odd)
            s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN, f, t=0.0)
            got = s.download(capi.PSI_ODD)
        oracle.parabolic_step(lat, p, f, 0.0, oracle.LEAPFROG, odd, even)
        _close(got, odd, capi.FP64, str(dims))
        assert np.all(got[0] == 0) and np.all(got[-1] == 0) and np.all(got[:, 0] == 0) and np.all(got[:, :, -1] == 0)


def test_nonfinite_is_reported(gpu):
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP32, (4, 4, 4))
    psi = _rand(lat, p, 91)
    psi[2, 2, 2, 3, 1, 0] = np.nan
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, psi)
        with pytest.raises(capi.GpeError) as ei:
            s.observe(capi.PSI_EVEN)
        assert ei.value.status == 5


def test_launch_count(gpu):
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP32, (4, 4, 4))
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_ODD, _rand(lat, p, 1))
        n0 = s.launches
        s.start()
        s.step(10)
        assert s.launches - n0 == 11
        assert s.current == capi.PSI_EVEN


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C,tile", [("bcc", 3, 5), ("bcc", 3, 16), ("bcc", 1, 3), ("bcc", 5, 7), ("fcc", 3, 4),
                                         ("a15", 1, 2), ("z", 3, 1), ("c15", 5, 1)])
def test_tile_kernel_tile_lengths(gpu, name, C, tile, prec):
    """Row-tile kernel with tile lengths that do not divide X (partial last tile)."""
    lat = capi.Lattice(name)
    X = 17 if lat.nodes < 40 else 5
    p = _params(lat, C, prec, (X, 3, 2))
    even, odd = _rand(lat, p, 101), _rand(lat, p, 102)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_TILE)
        s.set_tuning(capi.TUNE_TILE_CELLS, min(tile, X))
        assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_TILE
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN, f, t=0.0)
        s.step_explicit(capi.PSI_EVEN, capi.PSI_ODD, f, t=0.1)
        ge, go = s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)
    oracle.parabolic_step(lat, p, f, 0.0, oracle.LEAPFROG, odd, even)
    oracle.parabolic_step(lat, p, f, 0.1, oracle.LEAPFROG, even, odd)
    _close(ge, even, prec, "even")
    _close(go, odd, prec, "odd")


def test_tile_kernel_rejected_for_unaligned_cells(gpu):
    lat = capi.Lattice("cube")  # 1 node: 24-byte FP32 spin-1 cells
    p = _params(lat, 3, capi.FP32, (4, 4, 4))
    with Stepper(lat, p) as s:
        with pytest.raises(capi.GpeError):
            s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_TILE)
        assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_GATHER


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C,dims,shape", [
    ("bcc", 3, (8, 4, 5), (4, 2, 2)),      # partial last z-chunk
    ("bcc", 3, (16, 6, 7), (8, 3, 3)),
    ("bcc", 1, (12, 4, 4), (6, 4, 4)),
    ("bcc", 5, (8, 4, 6), (8, 2, 5)),
    ("bcc227", 1, (6, 6, 3), (3, 1, 1)),
    ("fcc", 3, (8, 4, 5), (4, 2, 3)),       # per-node degree 4 or 8
    ("a15", 3, (4, 2, 3), (2, 1, 2)),
    ("z", 1, (4, 4, 3), (2, 2, 2)),
    ("c15", 1, (2, 2, 3), (1, 1, 2)),
])
def test_march_kernel(gpu, name, C, dims, shape, prec):
    """2.5-D z-march kernel (ring of shared-memory slabs filled by bulk copies)
    against the oracle over three steps, with explicit tile shapes."""
    lat = capi.Lattice(name)
    p = _params(lat, C, prec, dims)
    even, odd = _rand(lat, p, 111), _rand(lat, p, 112)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.set_tuning(capi.TUNE_TILE_CELLS, shape[0])
        s.set_tuning(capi.TUNE_TILE_ROWS, shape[1])
        s.set_tuning(capi.TUNE_ZCHUNK, shape[2])
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_MARCH)
        assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_MARCH
        assert s.get_tuning(capi.TUNE_TILE_ROWS) == shape[1]
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        bufs = [capi.PSI_EVEN, capi.PSI_ODD]
        for n in range(3):
            s.step_explicit(bufs[(n + 1) % 2], bufs[n % 2], f, t=0.1 * n)
        ge, go = s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)
    b = [even, odd]
    for n in range(3):
        oracle.parabolic_step(lat, p, f, 0.1 * n, oracle.LEAPFROG, b[(n + 1) % 2], b[n % 2])
    _close(ge, even, prec, "even")
    _close(go, odd, prec, "odd")


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C,dims,shape", [
    ("bcc", 3, (16, 8, 5), (8, 4)),        # whole tiles
    ("bcc", 3, (13, 7, 6), (8, 4)),        # ragged in x and y
    ("bcc", 3, (7, 5, 4), (0, 0)),         # automatic shape
    ("bcc", 1, (20, 9, 3), (16, 2)),
    ("bcc", 5, (9, 6, 4), (4, 2)),
    ("bcc", 3, (3, 2, 1), (0, 0)),         # one plane, a grid smaller than the default tile
    ("a15", 3, (5, 3, 4), (2, 2)),
    ("z", 1, (4, 5, 3), (2, 2)),
    ("c15", 1, (3, 2, 3), (1, 1)),
])
def test_slab_kernel(gpu, name, C, dims, shape, prec):
    """Slab-ring kernel (psi_prev planes in a ring of shared-memory slabs filled by
    bulk copies, the column marching up z) against the oracle over three steps."""
    lat = capi.Lattice(name)
    p = _params(lat, C, prec, dims)
    cell_bytes = lat.nodes * C * (16 if prec == capi.FP64 else 8)
    # four psi_prev slabs must fit in 110 KB
    while shape[0] and (shape[0] + 2) * (shape[1] + 2) * 4 * cell_bytes > 110 * 1024:
        shape = (max(1, shape[0] // 2), shape[1] if shape[0] > 1 else max(1, shape[1] // 2))
    even, odd = _rand(lat, p, 121), _rand(lat, p, 122)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        if shape[0]:
            s.set_tuning(capi.TUNE_TILE_CELLS, shape[0])
            s.set_tuning(capi.TUNE_TILE_ROWS, shape[1])
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_SLAB)
        assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_SLAB
        if shape[0]:
            assert (s.get_tuning(capi.TUNE_TILE_CELLS), s.get_tuning(capi.TUNE_TILE_ROWS)) == shape
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        bufs = [capi.PSI_EVEN, capi.PSI_ODD]
        for n in range(3):
            s.step_explicit(bufs[(n + 1) % 2], bufs[n % 2], f, t=0.1 * n)
        ge, go = s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)
    b = [even, odd]
    for n in range(3):
        oracle.parabolic_step(lat, p, f, 0.1 * n, oracle.LEAPFROG, b[(n + 1) % 2], b[n % 2])
    _close(ge, even, prec, "even")
    _close(go, odd, prec, "odd")


@pytest.mark.parametrize("C", [1, 3, 5])
def test_slab_kernel_matches_gather_to_rounding(gpu, C):
    """The slab kernel does the gather kernel's arithmetic in the same order (the
    compiler may contract a different multiply-add): a ramped run of 20 leapfrog
    steps agrees to a few FP32 ulps of the largest value."""
    lat = capi.Lattice("bcc")
    p = _params(lat, C, capi.FP32, (24, 17, 11))
    ramp = capi.make_ramp(bq_segments=[(0.2, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0, 0, 0.5), 0.0, capi.RAMP_CONSTANT), ((0, 0, -0.5), 20 * p.dt, capi.RAMP_LINEAR),
                                       ((0, 0, -0.5), 1e9, capi.RAMP_CONSTANT)])
    psi = _rand(lat, p, 123)
    out = []
    for kernel in (capi.KERNEL_GATHER, capi.KERNEL_SLAB):
        with Stepper(lat, p) as s:
            s.set_tuning(capi.TUNE_KERNEL, kernel)
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(ramp, 0.0)
            s.start()
            s.step(20)
            out.append((s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)))
    for a, b in zip(out[0], out[1]):
        scale = float(np.max(np.abs(a)))
        err = float(np.max(np.abs(a - b)))
        assert err <= 1e-6 * scale, "max|slab - gather| = %.3e, scale %.3e" % (err, scale)


def test_slab_kernel_rejected_where_it_does_not_apply(gpu):
    """FCC rows of 4 and 8 entries and the cube's 6: no slab kernel."""
    for name in ("fcc", "cube"):
        lat = capi.Lattice(name)
        with Stepper(lat, _params(lat, 3, capi.FP32, (6, 4, 4))) as s:
            with pytest.raises(capi.GpeError):
                s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_SLAB)
            assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_GATHER


@pytest.mark.parametrize("name,C,want", [("bcc", 1, capi.KERNEL_GATHER), ("bcc", 5, capi.KERNEL_GATHER),
                                         ("fcc", 3, capi.KERNEL_GATHER), ("a15", 3, capi.KERNEL_GATHER),
                                         ("c15", 5, capi.KERNEL_GATHER), ("fcc", 1, capi.KERNEL_GATHER)])
def test_automatic_kernel_choice(gpu, name, C, want):
    """The automatic choice is the grid-stride gather kernel on every lattice."""
    lat = capi.Lattice(name)
    with Stepper(lat, _params(lat, C, capi.FP32, (6, 4, 4))) as s:
        assert s.get_tuning(capi.TUNE_KERNEL) == want


def test_kernel_choice_on_config2_shape(gpu):
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP32, (96, 96, 96))
    with Stepper(lat, p) as s:
        assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_GATHER  # the grid-stride gather kernel
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_TILE)
        assert s.get_tuning(capi.TUNE_TILE_CELLS) == 16
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_ROWS)
        assert s.get_tuning(capi.TUNE_TILE_CELLS) == 8
        assert (s.get_tuning(capi.TUNE_TILE_ROWS), s.get_tuning(capi.TUNE_ZCHUNK)) == (2, 2)


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C,dims,tile", [("bcc", 3, (17, 3, 4), 5), ("bcc", 1, (7, 5, 4), 0), ("bcc", 5, (9, 3, 3), 4),
                                              ("fcc", 3, (7, 4, 3), 3), ("a15", 3, (5, 3, 2), 2), ("z", 1, (5, 3, 3), 0),
                                              ("c15", 5, (3, 2, 2), 1), ("c15", 1, (4, 3, 2), 2), ("bcc227", 1, (6, 4, 3), 6)])
@pytest.mark.parametrize("block", [(0, 0, 0), (1, 1, 0), (2, 1, 64), (1, 2, 32)])
def test_rows_kernel(gpu, name, C, dims, tile, prec, block):
    """Row-block kernel (every row the stencil touches staged in shared memory) over
    three steps; partial last tiles, per-node degrees 4/8 (FCC), explicit RY x RZ
    blocks and thread counts smaller than the node count included."""
    lat = capi.Lattice(name)
    p = _params(lat, C, prec, dims)
    even, odd = _rand(lat, p, 121), _rand(lat, p, 122)
    f = capi.make_fields(**FIELDS)
    ry, rz, threads = block
    if ry and (dims[1] % ry or dims[2] % rz):
        pytest.skip("block does not divide the grid")
    with Stepper(lat, p) as s:
        if tile:
            s.set_tuning(capi.TUNE_TILE_CELLS, tile)
        if ry:
            s.set_tuning(capi.TUNE_TILE_ROWS, ry)
            s.set_tuning(capi.TUNE_ZCHUNK, rz)
        if threads:
            s.set_tuning(capi.TUNE_THREADS, threads)
        try:
            s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_ROWS)
        except capi.GpeError as e:
            if e.status == 6 and (ry > 1 or rz > 1):
                pytest.skip("row block does not fit in shared memory")
            raise
        s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_ROWS)
        assert s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_ROWS
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        bufs = [capi.PSI_EVEN, capi.PSI_ODD]
        for n in range(3):
            s.step_explicit(bufs[(n + 1) % 2], bufs[n % 2], f, t=0.1 * n)
        ge, go = s.download(capi.PSI_EVEN), s.download(capi.PSI_ODD)
    b = [even, odd]
    for n in range(3):
        oracle.parabolic_step(lat, p, f, 0.1 * n, oracle.LEAPFROG, b[(n + 1) % 2], b[n % 2])
    _close(ge, even, prec, "even")
    _close(go, odd, prec, "odd")


def test_autotune_keeps_state_and_picks_a_kernel(gpu):
    """gpe_autotune restores the state, and stepping after it still matches the oracle."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP32, (16, 4, 4))
    even, odd = _rand(lat, p, 131), _rand(lat, p, 132)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, even)
        s.upload(capi.PSI_ODD, odd)
        rep = s.autotune(steps=3)
        assert len(rep) >= 3 and all(r["ms"] > 0 for r in rep)
        best = min(rep, key=lambda r: r["ms"])
        assert s.get_tuning(capi.TUNE_KERNEL) in (best["kernel"], capi.KERNEL_ROWS, capi.KERNEL_TILE, capi.KERNEL_GATHER)
        np.testing.assert_array_equal(s.download(capi.PSI_EVEN), even.astype(np.float32).astype(np.float64))
        s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN, f, t=0.0)
        got = s.download(capi.PSI_ODD)
    oracle.parabolic_step(lat, p, f, 0.0, oracle.LEAPFROG, odd, even)
    _close(got, odd, capi.FP32)


def test_autotune_keeps_hyperbolic_state(gpu):
    """gpe_autotune on a hyperbolic handle restores q even/odd as well as psi (its
    trial steps write both), and stepping after it still matches the oracle."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 5, capi.FP32, (8, 4, 4), scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01)
    pe, po = _rand(lat, p, 141), _rand(lat, p, 142)
    qe, qo = _rand(lat, p, 143, edges=True), _rand(lat, p, 144, edges=True)
    f = capi.make_fields(**FIELDS)
    with Stepper(lat, p) as s:
        for slot, a in ((capi.PSI_EVEN, pe), (capi.PSI_ODD, po), (capi.Q_EVEN, qe), (capi.Q_ODD, qo)):
            s.upload(slot, a)
        s.autotune(steps=2)
        for slot, a in ((capi.PSI_EVEN, pe), (capi.PSI_ODD, po), (capi.Q_EVEN, qe), (capi.Q_ODD, qo)):
            np.testing.assert_array_equal(s.download(slot), a.astype(np.float32).astype(np.float64))
        s.step_explicit(capi.PSI_ODD, capi.PSI_EVEN, f, t=0.2)
        got_p, got_q = s.download(capi.PSI_ODD), s.download(capi.Q_ODD)
    oracle.q_psi_step(lat, p, f, 0.2, oracle.LEAPFROG, True, po, pe, qe)
    oracle.q_step(lat, p, oracle.Q_HYPER, qo, qe, pe)
    _close(got_p, po, capi.FP32, "psi")
    _close(got_q, qo, capi.FP32, "q")


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C,kind", [("bcc", 1, "vortex"), ("bcc", 3, "polar"), ("c15", 5, "cyclic")])
def test_device_initial_state_matches_numpy(gpu, name, C, kind, prec):
    """gpe_init_state reproduces states.vortex_state / spinor_state (SplitMix64 +
    Box-Muller, same counters) to rounding."""
    lat = capi.Lattice(name)
    dims = (6, 5, 4) if lat.nodes < 40 else (3, 2, 2)
    p = _params(lat, C, prec, dims, c0=2000.0, trap_lambda=(1.0, 1.0, 1.0), block_scale=16.0 / (dims[0] * lat.block_width[0]))
    if kind == "vortex":
        want = states.vortex_state(lat, p, seed=5, noise=1e-2, kappa=1)
        init = capi.make_init(zeta=(1.0,), kappa=1, noise_abs=1e-2, seed=5)
    else:
        zeta = states.POLAR if kind == "polar" else states.CYCLIC
        want = states.spinor_state(lat, p, zeta, seed=6, noise=1e-2)
        init = capi.make_init(zeta=zeta, noise_rel=1e-2, seed=6)
    with Stepper(lat, p) as s:
        s.init_state(capi.PSI_ODD, init)
        assert s.current == capi.PSI_ODD
        got = s.download(capi.PSI_ODD)
        assert s.observe(capi.PSI_ODD)["norm"] == pytest.approx(1.0, rel=1e-12 if prec == capi.FP64 else 1e-6)
    tol = 1e-12 if prec == capi.FP64 else 1e-6
    assert np.max(np.abs(got - want)) <= tol * np.max(np.abs(want))


def _obs_close(got, want, rel, what):
    scale = max(abs(want["norm"]), abs(want["h_expect"]), 1e-30)
    for k in ("norm", "energy", "h_expect", "spin_norm"):
        assert got[k] == pytest.approx(want[k], rel=rel, abs=rel * scale), (what, k, got[k], want[k])
    np.testing.assert_allclose(got["magnetization"], want["magnetization"], rtol=rel, atol=rel * scale, err_msg=what)
    np.testing.assert_allclose(got["com"], want["com"], rtol=rel, atol=rel * scale * 10, err_msg=what)
    assert got["max_abs"] == pytest.approx(want["max_abs"], rel=1e-6 if rel > 1e-9 else 1e-15), what
    assert got["nonfinite"] == want["nonfinite"] == 0


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,C,dims", [("bcc", 3, (12, 7, 5)), ("bcc", 1, (9, 8, 3)), ("bcc", 5, (6, 5, 4)),
                                         ("fcc", 3, (6, 5, 4)), ("cube", 3, (20, 9, 7)), ("c15", 1, (3, 3, 2)),
                                         ("a15", 5, (3, 2, 3)), ("bcc", 3, (1, 1, 1))])
def test_step_observe_matches_step_and_observe(gpu, name, C, dims, prec):
    """gpe_step_observe(n): the observables of the state the last step reads,
    summed inside that step's kernel, equal gpe_observe of that state at the last
    step's time (FP64 handles to 1e-11: the same FP64 terms added in another
    order; FP32 handles against gpe_observe's FP32 node terms to 2e-6 of the
    norm / energy scale: FP32 terms rounded in another order), and the states
    equal plain stepping to rounding."""
    lat = capi.Lattice(name)
    flags = capi.FLAG_QUADRATIC_ZEEMAN | capi.FLAG_QUADRUPOLE_OFFSET if C == 3 else 0
    p = _params(lat, C, prec, dims, flags=flags, quad_center=(0.1, -0.2, 0.05))
    ramp = capi.make_ramp(bq_segments=[(0.3, 1e9, capi.RAMP_CONSTANT)],
                          bb_segments=[((0.1, -0.2, 0.5), 0.0, capi.RAMP_CONSTANT), ((0.0, 0.1, -0.5), 8 * p.dt, capi.RAMP_LINEAR),
                                       ((0.0, 0.1, -0.5), 1e9, capi.RAMP_CONSTANT)], bq_quad_scale=0.5, bb_quad_scale=0.25)
    psi = _rand(lat, p, 131)
    n = 5
    with Stepper(lat, p) as a, Stepper(lat, p) as b:
        for s in (a, b):
            s.set_tuning(capi.TUNE_OBSERVE_ARITH, 1 if prec == capi.FP32 else 0)
            s.upload(capi.PSI_ODD, psi)
            s.set_ramp(ramp, 0.0)
            s.start()
        a.step(n - 1)
        t_last = n * p.dt  # the start took step 0; the last of the n steps is step n
        want = a.observe(a.current, t_last)
        a.step(1)
        n0 = b.launches
        got = b.step_observe(n)
        assert b.launches - n0 == n + 1  # n step launches + the finalize
        assert a.current == b.current
        sa, sb = a.download(a.current), b.download(b.current)
    _obs_close(got, want, 1e-11 if prec == capi.FP64 else 2e-6, "%s C=%d" % (name, C))
    scale = float(np.max(np.abs(sa)))
    assert float(np.max(np.abs(sa - sb))) <= (1e-13 if prec == capi.FP64 else 1e-6) * scale


def test_step_observe_with_another_kernel_and_scheme(gpu):
    """Where the handle steps with a tile kernel or the hyperbolic scheme, the
    observables come from a separate pass; the numbers are the same."""
    for kind in ("tile", "hyper"):
        lat = capi.Lattice("bcc")
        kw = dict(scheme=capi.SCHEME_HYPERBOLIC, sigma=0.01) if kind == "hyper" else {}
        p = _params(lat, 3, capi.FP64, (8, 6, 5), **kw)
        psi = _rand(lat, p, 132)
        with Stepper(lat, p) as a, Stepper(lat, p) as b:
            for s in (a, b):
                if kind == "tile":
                    s.set_tuning(capi.TUNE_KERNEL, capi.KERNEL_TILE)
                s.upload(capi.PSI_ODD, psi)
                s.start()
            a.step(3)
            want = a.observe(a.current, 4 * p.dt)
            a.step(1)
            got = b.step_observe(4)
            assert np.array_equal(a.download(a.current), b.download(b.current))
        _obs_close(got, want, 1e-13, kind)
