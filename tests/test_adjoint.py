"""Adjoint (reverse-time) kernel and its torch.autograd wrapper.

Checks, all on seeded small grids:
  - FP64 adjoint gradients against central finite differences (h = 1e-4) of the
    GPU FP64 forward run and of the FP64 CPU oracle's forward run: relative error
    <= 1e-6 (the adjoint is exact up to rounding; the differences are the FD
    truncation and cancellation error);
  - the FP32 adjoint against the FP64 adjoint: relative error of the gradient
    vector <= 1e-3;
  - checkpoint stride does not change the gradient (bit-identical in FP64);
  - overlap and magnetisation losses, scalar / spin-1 / spin-2 lattices and the
    physics switches (loss, quadratic Zeeman, quadrupole offset, trap switch-off);
  - RampControl (torch.autograd.Function): knot gradients against central
    differences on 8 knots.
"""
import numpy as np
import pytest
import torch

from oracle import oracle
from spacetime_gb300 import capi, states
from spacetime_gb300.adjoint import RampControl
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu

FD_H = 1e-4


def _params(lat, C, prec, dims, **kw):
    base = dict(components=C, precision=prec, dims=dims, block_scale=0.3, dt=5e-4, trap_offset=100.0,
                trap_lambda=(1.0, 1.1, 1.3), c0=120.0, c2=-7.0, c4=3.0, lattice=lat)
    base.update(kw)
    return capi.make_params(**base)


def _fields(n, seed):
    u = states.uniform01(seed, 4 * n).reshape(n, 4)
    return 2.0 * u - 1.0


def _initial(lat, p, C):
    zeta = {1: (1.0,), 3: states.POLAR, 5: states.CYCLIC}[C]
    return states.spinor_state(lat, p, zeta, seed=2, noise=1e-2)


def _target(lat, p, C):
    """A target with an O(1) overlap with the initial state, so that the loss
    gradients are far above the rounding floor of central differences."""
    zeta = {1: (1.0,), 3: (0.4, 0.8, 0.4j + 0.2), 5: (0.2, 0.3j, 0.8, 0.3, 0.36)}[C]
    z = np.asarray(zeta, dtype=np.complex128)
    return states.spinor_state(lat, p, z / np.linalg.norm(z), seed=5, noise=5e-2)


# L = Re<T|psi_N> - 0.7 Im<T|psi_N>: linear in the overlap, so dL/dB is not
# suppressed where the overlap is small.
LIN = np.array([1.0, -0.7, 0.0, 0.0, 0.0])


def _overlap_loss(out):
    return float(LIN[:2] @ np.asarray(out)[:2])


def _overlap_seed(out):
    return LIN


def _oracle_final(lat, p, psi0, fields):
    """The same run on the FP64 CPU oracle (forwardEuler + leapfrog)."""
    odd, even = psi0.copy(), np.zeros_like(psi0)
    bufs = [odd, even]
    t0 = 0.0
    rows = np.zeros((fields.shape[0], 8))
    rows[:, : fields.shape[1]] = fields

    def f(j):
        return capi.make_fields(bq=rows[j, 0], bb=tuple(rows[j, 1:4]), bq_quad=rows[j, 4], bb_quad=tuple(rows[j, 5:8]))

    oracle.parabolic_step(lat, p, f(0), t0, oracle.EULER, even, odd)
    for j in range(1, fields.shape[0]):
        oracle.parabolic_step(lat, p, f(j), t0 + j * p.dt, oracle.LEAPFROG, bufs[(j + 1) % 2], bufs[j % 2])
    return bufs[fields.shape[0] % 2]


def _oracle_out(lat, p, psi, target):
    dv = p.block_scale ** 3 * lat.volume
    T, u = target[1:-1, 1:-1, 1:-1], psi[1:-1, 1:-1, 1:-1]
    re = float(np.sum(T[..., 0] * u[..., 0] + T[..., 1] * u[..., 1])) * dv
    im = float(np.sum(T[..., 0] * u[..., 1] - T[..., 1] * u[..., 0])) * dv
    return np.array([re, im])


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


class Run:
    """A stepper with a fixed initial state and target; loss and gradient of a field table."""

    def __init__(self, lat, p, C, stride=0):
        self.lat, self.p = lat, p
        self.s = Stepper(lat, p)
        self.psi0 = _initial(lat, p, C)
        self.target = _target(lat, p, C)
        self.stride = stride

    def forward(self, fields):
        self.s.upload(capi.PSI_ODD, self.psi0)
        return self.s.adjoint_forward(fields, self.target, self.stride)

    def grad(self, fields, seed_fn=_overlap_seed):
        out = self.forward(fields)
        return out, self.s.adjoint_backward(seed_fn(out))

    def close(self):
        self.s.close()


CHECKS = [(0, 0), (0, 3), (1, 0), (5, 1), (11, 2), (17, 3), (23, 0), (23, 3)]


@pytest.mark.parametrize("name,C", [("bcc", 3), ("bcc", 1), ("cube", 5), ("fcc", 3)])
def test_adjoint_fp64_vs_fd(gpu, name, C):
    """dL/dB_j of the FP64 adjoint against central differences of the GPU FP64 run."""
    lat = capi.Lattice(name)
    p = _params(lat, C, capi.FP64, (6, 5, 4))
    fields = _fields(24, seed=41)
    r = Run(lat, p, C, stride=5)
    try:
        out, g = r.grad(fields)
        assert np.all(np.isfinite(g))
        for j, m in CHECKS:
            fp, fm = fields.copy(), fields.copy()
            fp[j, m] += FD_H
            fm[j, m] -= FD_H
            fd = (_overlap_loss(r.forward(fp)) - _overlap_loss(r.forward(fm))) / (2 * FD_H)
            if C == 1 and m > 0:
                assert abs(g[j, m]) == 0.0 and abs(fd) < 1e-12  # a scalar field ignores B
                continue
            assert abs(g[j, m] - fd) <= 1e-6 * abs(fd) + 1e-11, (j, m, g[j, m], fd)
    finally:
        r.close()


def test_adjoint_vs_oracle_fd(gpu):
    """The GPU FP64 adjoint against central differences of the FP64 CPU oracle's run
    (an independent forward: Spin1GpeBCC.cu's leapfrog restated in C)."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP64, (5, 4, 4))
    fields = _fields(16, seed=43)
    r = Run(lat, p, 3, stride=4)
    try:
        out, g = r.grad(fields)
        ref = _oracle_out(lat, p, _oracle_final(lat, p, r.psi0, fields), r.target)
        assert np.max(np.abs(out[:2] - ref)) <= 1e-12
        for j, m in [(0, 0), (3, 3), (8, 0), (15, 3), (9, 1)]:
            fp, fm = fields.copy(), fields.copy()
            fp[j, m] += FD_H
            fm[j, m] -= FD_H
            lp = _overlap_loss(_oracle_out(lat, p, _oracle_final(lat, p, r.psi0, fp), r.target))
            lm = _overlap_loss(_oracle_out(lat, p, _oracle_final(lat, p, r.psi0, fm), r.target))
            fd = (lp - lm) / (2 * FD_H)
            assert abs(g[j, m] - fd) <= 1e-6 * abs(fd) + 1e-11, (j, m, g[j, m], fd)
    finally:
        r.close()


@pytest.mark.parametrize("flags", [capi.FLAG_THREE_BODY_LOSS, capi.FLAG_QUADRATIC_ZEEMAN | capi.FLAG_QUADRUPOLE_OFFSET,
                                   capi.FLAG_TRAP_OFF_AFTER])
def test_adjoint_physics_toggles(gpu, flags):
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP64, (5, 4, 4), flags=flags, alpha=2.0, quad_center=(0.1, -0.2, 0.05),
                trap_off_time=6e-3)
    fields = _fields(20, seed=44)
    fields8 = np.zeros((20, 8))
    fields8[:, :4] = fields
    fields8[:, 4] = 0.3
    fields8[:, 5:8] = (0.1, -0.2, 0.4)
    r = Run(lat, p, 3, stride=3)
    try:
        out, g = r.grad(fields8)
        for j, m in [(0, 0), (7, 3), (13, 1), (19, 2)]:
            fp, fm = fields8.copy(), fields8.copy()
            fp[j, m] += FD_H
            fm[j, m] -= FD_H
            fd = (_overlap_loss(r.forward(fp)) - _overlap_loss(r.forward(fm))) / (2 * FD_H)
            assert abs(g[j, m] - fd) <= 1e-6 * abs(fd) + 1e-11, (flags, j, m, g[j, m], fd)
    finally:
        r.close()


@pytest.mark.parametrize("C", [3, 5])
def test_adjoint_magnetization_loss(gpu, C):
    """L = M_z + 0.5 M_x of the final state (seed on the magnetisation outputs)."""
    lat = capi.Lattice("bcc")
    p = _params(lat, C, capi.FP64, (5, 4, 4))
    fields = _fields(18, seed=45)
    r = Run(lat, p, C, stride=4)
    seed = np.array([0.0, 0.0, 0.5, 0.0, 1.0])
    try:
        out, g = r.grad(fields, seed_fn=lambda o: seed)
        for j, m in [(0, 3), (6, 0), (12, 1), (17, 3)]:
            fp, fm = fields.copy(), fields.copy()
            fp[j, m] += FD_H
            fm[j, m] -= FD_H
            lp, lm = r.forward(fp), r.forward(fm)
            fd = (seed @ lp - seed @ lm) / (2 * FD_H)
            assert abs(g[j, m] - fd) <= 1e-6 * abs(fd) + 1e-11, (j, m, g[j, m], fd)
    finally:
        r.close()


def test_adjoint_stride_invariance(gpu):
    """Checkpoint spacing changes memory and recomputation only: the FP64 gradients
    for strides 1, 3, 7, default (ceil sqrt N) and N are bit-identical."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP64, (6, 5, 4))
    fields = _fields(22, seed=46)
    ref = None
    for stride in (1, 3, 7, 0, 22):
        r = Run(lat, p, 3, stride=stride)
        try:
            _, g = r.grad(fields)
        finally:
            r.close()
        if ref is None:
            ref = g
        assert np.array_equal(g, ref), stride


@pytest.mark.parametrize("prec,kernel", [(capi.FP32, capi.KERNEL_GATHER), (capi.FP64, capi.KERNEL_TILE),
                                         (capi.FP32, capi.KERNEL_TILE), (capi.FP32, capi.KERNEL_AUTO),
                                         (capi.FP32, capi.KERNEL_INTERLEAVED)])
def test_adjoint_stride_invariance_kernels(gpu, prec, kernel):
    """The recomputation reproduces the forward run's states exactly with either
    step kernel: out of place for the gather kernel, a state copy and an in-place
    step for the row tile; forward segments run by the interleaved kernel (the
    automatic choice for the 16 steps of stride N, every segment when it is
    forced) are recomputed by the gather kernel.  Gradients for strides 1 (no
    recomputation), 4 and N are bit-identical."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, prec, (6, 5, 4))
    fields = _fields(17, seed=48)
    ref = None
    for stride in (1, 4, 17):
        r = Run(lat, p, 3, stride=stride)
        try:
            r.s.set_tuning(capi.TUNE_KERNEL, kernel)
            _, g = r.grad(fields)
        finally:
            r.close()
        if ref is None:
            ref = g
        assert np.array_equal(g, ref), stride


def test_adjoint_fp32_vs_fp64(gpu):
    """FP32 adjoint (FP32 states, FP64 reductions) against the FP64 adjoint."""
    lat = capi.Lattice("bcc")
    fields = _fields(40, seed=47)
    grads = {}
    for prec in (capi.FP64, capi.FP32):
        p = _params(lat, 3, prec, (8, 6, 6))
        r = Run(lat, p, 3)
        try:
            grads[prec] = r.grad(fields)[1]
        finally:
            r.close()
    assert _rel(grads[capi.FP32], grads[capi.FP64]) <= 1e-3


def test_adjoint_requires_forward(gpu):
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP64, (4, 4, 4))
    r = Run(lat, p, 3)
    try:
        with pytest.raises(capi.GpeError):
            r.s.adjoint_backward(np.ones(5))
        r.grad(_fields(6, seed=48))
        r.s.step(1)  # the state moved on: the recorded run is gone
        with pytest.raises(capi.GpeError):
            r.s.adjoint_backward(np.ones(5))
    finally:
        r.close()


def test_ramp_control_autograd(gpu):
    """Knot gradients of 1 - |<T|psi(T)>|^2 through torch autograd against central
    differences (h = 1e-4) on 8 random knots (target with an O(1) overlap)."""
    lat = capi.Lattice("bcc")
    p = _params(lat, 3, capi.FP64, (6, 6, 5))
    n_steps, n_knots = 60, 16
    s = Stepper(lat, p)
    psi0 = _initial(lat, p, 3)
    try:
        rc = RampControl(s, n_steps, n_knots, lambda: s.upload(capi.PSI_ODD, psi0), _target(lat, p, 3), stride=8)
        k = 2.0 * states.uniform01(4, 2 * n_knots).reshape(2, n_knots) - 1.0
        bq = torch.tensor(k[0], requires_grad=True)
        bz = torch.tensor(k[1], requires_grad=True)
        loss = rc.loss(bq, bz)
        loss.backward()
        rng = np.random.default_rng(4)
        picks = [(int(a), int(b)) for a, b in zip(rng.integers(0, 2, 8), rng.integers(0, n_knots, 8))]
        for which, i in picks:
            kp, km = k.copy(), k.copy()
            kp[which, i] += FD_H
            km[which, i] -= FD_H
            with torch.no_grad():
                lp = float(rc.loss(torch.tensor(kp[0]), torch.tensor(kp[1])))
                lm = float(rc.loss(torch.tensor(km[0]), torch.tensor(km[1])))
            fd = (lp - lm) / (2 * FD_H)
            got = float((bq.grad if which == 0 else bz.grad)[i])
            assert abs(got - fd) <= 1e-4 * abs(fd) + 1e-12, (which, i, got, fd)
    finally:
        s.close()

