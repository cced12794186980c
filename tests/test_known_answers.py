"""Known answers the reference prints, reproduced from scratch on the GPU.

The spin-1 program (Spin1GpeBCC/Spin1GpeBCC.cu) hard-codes the energy of its
imaginary-time ground state, E = 127.295 (:1421, "Computed with ITP"), which its
ground-state loop prints as <psi|H psi> (:1445-1494).  Its configuration: BCC,
domain [-12, 12]^3 with 112 block cells per edge (:49-55, 1812-1813), N = 2e5
atoms with a_0 = 101.8 and a_2 = 100.4 Bohr (:57-74), trap 126 Hz radially and
166 Hz axially with the +100 offset of `trap` (:59-66, 112-122).  Its a_2 < a_0
gives c2 < 0: the ground state is ferromagnetic, psi = (psi_1, 0, 0) with
<F> = (0, 0, rho), where the spin term adds c2 rho and the condensate feels
c0 + c2.  Started from the ferromagnetic Thomas-Fermi state the imaginary-time
loop converges to that ground state whatever its step size (the fixed point of
psi <- normalise(psi - dt H psi) is an eigenvector of H).  (From the polar state,
<F> = 0, the same loop converges to the polar state, about 0.05 higher.)
"""
import math

import numpy as np

import pytest

from spacetime_gb300 import capi
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu

PI = 3.1415926535897932385  # Types/Types.hpp


def spin1_program_params(precision):
    """The spin-1 program's constants, computed as its source does."""
    n_atoms, a_bohr, a0, a2 = 2e5, 5.2917721092e-11, 101.8, 100.4
    mass, hbar = 1.44316060e-25, 1.05457148e-34
    omega_r, omega_z = 126 * 2 * PI, 166 * 2 * PI
    a_r = math.sqrt(hbar / (mass * omega_r))
    c0 = 4 * PI * n_atoms * (a0 + 2 * a2) * a_bohr / (3 * a_r)
    c2 = 4 * PI * n_atoms * (a2 - a0) * a_bohr / (3 * a_r)
    lat = capi.Lattice("bcc")
    bw = lat.block_width[0]
    bs = (24.0 / 112.0) / bw                # targetBlockWidth / BLOCK_WIDTH_X
    cells = int(24.0 / (bs * bw))           # integrateInTime's xsize
    return lat, capi.make_params(components=3, precision=precision, dims=(cells,) * 3, block_scale=bs, dt=8e-4,
                                 trap_lambda=(1.0, 1.0, omega_z / omega_r), trap_offset=100.0, c0=c0, c2=c2,
                                 lattice=lat)


def test_spin1_ground_state_energy_is_the_programs():
    """gpe_itp from the ferromagnetic Thomas-Fermi state on the program's own grid
    (112^3 BCC cells, 16,859,136 nodes; FP32 storage, FP64 sums) converges to
    E = 127.295 to the digits the program prints (std::cout's six), and the state
    stays fully magnetised along z."""
    lat, p = spin1_program_params(capi.FP32)
    assert tuple(p.dims) == (112, 112, 112)
    with Stepper(lat, p) as s:
        s.init_state(s.current, capi.make_init(zeta=(1.0, 0.0, 0.0)))
        mus = []
        for _ in range(4):
            mus.append(s.itp(1500))
        assert abs(mus[-1] - mus[-2]) < 2e-5, mus           # converged
        assert float("%.6g" % mus[-1]) == 127.295, mus
        o = s.observe(s.current, 0.0)
        assert o["norm"] == pytest.approx(1.0, rel=1e-6)
        assert o["magnetization"][2] == pytest.approx(1.0, rel=1e-6)


def _small_spin1(scheme=capi.SCHEME_PARABOLIC, sigma=0.0, dims=(14, 14, 14), dt=1e-4):
    """A small spin-1 BCC condensate with the programs' trap shape (lambda_z =
    166/126, +100) and a moderate interaction, box [-6, 6]^3."""
    lat = capi.Lattice("bcc")
    bs = 12.0 / (dims[0] * lat.block_width[0])
    return lat, capi.make_params(components=3, scheme=scheme, precision=capi.FP64, dims=dims, block_scale=bs, dt=dt,
                                 trap_lambda=(1.0, 1.0, 166.0 / 126.0), trap_offset=100.0, c0=300.0, c2=-2.0,
                                 sigma=sigma, lattice=lat)


def test_ground_state_rotates_as_exp_minus_iEt():
    """The spin-1 program's analytic check (Spin1GpeBCC.cu:1611-1633 analyticStep;
    RelativisticSpin1Gpe.cu:876-897): a ground state from imaginary time, run
    forward in real time by the leapfrog stepper, stays psi_g exp(-i E t) with E the
    <psi|H psi> the imaginary-time loop returns.  Leapfrog turns an eigenstate by
    asin(E dt) per step, not E dt: against that phase the weighted difference
    sum |psi_g e^{-i n asin(E dt)} - psi_n|^2 dv stays below 1e-8 over 2000
    steps (what is left is the Euler start's parasitic mode); against the
    continuous e^{-iEt} it is the scheme's phase error, n (E dt)^3 / 6 squared."""
    lat, p = _small_spin1()
    dv = p.block_scale ** 3 * lat.volume
    _, pi = _small_spin1(dt=3e-3)  # imaginary time: a larger step, the same fixed point
    with Stepper(lat, pi) as g:
        g.init_state(g.current, capi.make_init(zeta=(1.0, 0.0, 0.0)))
        E = 0.0
        for _ in range(6):
            E_prev, E = E, g.itp(2000)
        assert abs(E - E_prev) < 1e-9 * abs(E)
        ground = g.download(g.current)
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_ODD, ground)
        s.start()
        n = 2000
        s.step(n - 1)  # the start took step 0: psi(t) with t = n dt
        psi = s.download(s.current)
    g = ground[..., 0] + 1j * ground[..., 1]
    w = psi[..., 0] + 1j * psi[..., 1]
    theta = n * math.asin(E * p.dt)
    err = float(np.sum(np.abs(g * np.exp(-1j * theta) - w) ** 2)) * dv
    assert err < 1e-8, (E, err)
    phase_err = n * (E * p.dt) ** 3 / 6
    err_t = float(np.sum(np.abs(g * np.exp(-1j * E * n * p.dt) - w) ** 2)) * dv
    assert err_t == pytest.approx(phase_err ** 2, rel=0.1), (err_t, phase_err ** 2)


def test_hyperbolic_tends_to_parabolic_as_sigma_shrinks():
    """The relativistic spin-1 program's comparison (RelativisticSpin1Gpe.cu:
    848-875): the same start run by the parabolic and by the hyperbolic scheme,
    weighted difference sum |psi_para - psi_hyper|^2 dv after 400 steps.  It
    falls with every halving of sigma, by a factor that grows towards 4 (the
    hyperbolic correction to psi is of order sigma, so the difference tends to
    sigma^2; with the trap's +100 the kinetic factor 1 + sigma (V + c0 rho) is
    still 1.1 at sigma = 5e-4, so the approach is slow)."""
    lat, p = _small_spin1()
    dv = p.block_scale ** 3 * lat.volume
    psi0 = None
    n = 400
    with Stepper(lat, p) as s:
        s.init_state(s.current, capi.make_init(zeta=(0.0, 1.0, 0.0), noise_rel=1e-2, seed=9))
        psi0 = s.download(s.current)
        s.upload(capi.PSI_ODD, psi0)
        s.start()
        s.step(n - 1)
        para = s.download(s.current)
    diffs = []
    for sigma in (4e-3, 2e-3, 1e-3, 5e-4):
        lat, q = _small_spin1(capi.SCHEME_HYPERBOLIC, sigma)
        with Stepper(lat, q) as s:
            s.upload(capi.PSI_ODD, psi0)
            s.start()
            s.step(n - 1)
            hyper = s.download(s.current)
        diffs.append(float(np.sum((hyper - para) ** 2)) * dv)
    ratios = [a / b for a, b in zip(diffs, diffs[1:])]
    assert all(r > 2.0 for r in ratios), (diffs, ratios)
    assert all(b > a for a, b in zip(ratios, ratios[1:])), (diffs, ratios)  # towards sigma^2
    assert ratios[-1] > 3.0, (diffs, ratios)
