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
