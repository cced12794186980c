"""Python binding of the FP64 CPU oracle (oracle/gpe_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference arm of bench.py, as the checker.  The product
(spacetime_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from spacetime_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libgpe_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

LEAPFROG, EULER, ITP = 0, 1, 2
Q_HYPER, Q_PARA, Q_EULER_HYPER, Q_ITP = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP when available)."""
    src = os.path.join(HERE, "gpe_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "gpe_oracle.h"))
    ):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    base = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", src, "-o", LIB, "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        dp = P(C.c_double)
        L.orc_parabolic_step.argtypes = [P(capi.LatticeDesc), P(capi.Params), P(capi.Fields), C.c_double, C.c_int, dp, dp, dp, C.c_int]
        L.orc_q_psi_step.argtypes = [P(capi.LatticeDesc), P(capi.Params), P(capi.Fields), C.c_double, C.c_int, C.c_int, dp, dp, dp, dp, C.c_int]
        L.orc_q_step.argtypes = [P(capi.LatticeDesc), P(capi.Params), C.c_int, dp, dp, dp, C.c_int]
        L.orc_normalize.argtypes = [P(capi.LatticeDesc), P(capi.Params), dp]
        L.orc_normalize.restype = C.c_double
        L.orc_observe.argtypes = [P(capi.LatticeDesc), P(capi.Params), P(capi.Fields), C.c_double, dp, P(capi.Observables)]
        L.orc_ramp_eval.argtypes = [P(capi.Ramp), C.c_double, P(capi.Fields)]
        L.orc_ramp_eval.restype = None
        L.orc_node_fields.argtypes = [P(capi.LatticeDesc), P(capi.Params), P(capi.Fields), C.c_double, C.c_int, dp, dp]
        L.orc_node_fields.restype = C.c_int
        L.orc_split_step.argtypes = [P(capi.LatticeDesc), P(capi.Params), C.c_int, dp, dp, C.c_int]
        L.orc_split_step.restype = C.c_int
        L.orc_gpblocks_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_int64), C.c_double, C.c_double, C.c_double, dp, dp, dp, C.c_int]
        L.orc_gpblocks_run.restype = None
        L.orc_gpblocks_norm.argtypes = [C.c_size_t, C.c_size_t, dp, dp, C.c_double, dp]
        L.orc_gpblocks_norm.restype = None
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(st, where):
    if st != 0:
        raise RuntimeError("%s returned %d" % (where, st))


def parabolic_step(lat, params, fields, t, mode, nxt, prev, hpsi=None, threads=0):
    _check(lib().orc_parabolic_step(C.byref(lat.desc), C.byref(params), C.byref(fields), t, mode, _dp(nxt), _dp(prev), _dp(hpsi), threads), "orc_parabolic_step")


def q_psi_step(lat, params, fields, t, mode, hyperb, nxt, prev, q, threads=0, hpsi=None):
    _check(lib().orc_q_psi_step(C.byref(lat.desc), C.byref(params), C.byref(fields), t, mode, int(hyperb), _dp(nxt), _dp(prev), _dp(q), _dp(hpsi), threads), "orc_q_psi_step")


def q_step(lat, params, qmode, next_q, prev_q, psi, threads=0):
    _check(lib().orc_q_step(C.byref(lat.desc), C.byref(params), qmode, _dp(next_q), _dp(prev_q), _dp(psi), threads), "orc_q_step")


def normalize(lat, params, psi) -> float:
    return lib().orc_normalize(C.byref(lat.desc), C.byref(params), _dp(psi))


def observe(lat, params, fields, t, psi) -> dict:
    o = capi.Observables()
    _check(lib().orc_observe(C.byref(lat.desc), C.byref(params), C.byref(fields), t, _dp(psi), C.byref(o)), "orc_observe")
    return o.as_dict()


def ramp_eval(ramp, tau):
    f = capi.Fields()
    lib().orc_ramp_eval(C.byref(ramp), tau, C.byref(f))
    return f


# ---------------------------------------------------------------- time loops


def leapfrog_run(lat, params, even, odd, nsteps, ramp=None, t0=0.0, fields=None, threads=0):
    """Reference time loop: odd <- even, even <- odd, ... (Spin1GpeBCC.cu:1574-1603).
    Step n (0-based) uses the fields at t0 + (n+1)*dt.  Returns the buffer holding
    the newest state (even or odd)."""
    bufs = [even, odd]
    for n in range(nsteps):
        t = t0 + (n + 1) * params.dt
        f = fields if ramp is None else ramp_eval(ramp, ramp.time_scale * t)
        if f is None:
            f = capi.make_fields()
        nxt, prv = bufs[(n + 1) % 2], bufs[n % 2]
        parabolic_step(lat, params, f, t, LEAPFROG, nxt, prv, None, threads)
    return bufs[nsteps % 2]


def hyper_run(lat, params, psi_even, psi_odd, q_even, q_odd, nsteps, ramp=None, t0=0.0, fields=None, threads=0,
              hyperb=True):
    """Hyperbolic psi+q loop (RelativisticSpin2Gpe.cu:1859-1899).  Both updates of a
    step read the previous (psi, q) pair."""
    ps = [psi_even, psi_odd]
    qs = [q_even, q_odd]
    for n in range(nsteps):
        t = t0 + (n + 1) * params.dt
        f = fields if ramp is None else ramp_eval(ramp, ramp.time_scale * t)
        if f is None:
            f = capi.make_fields()
        a, b = n % 2, (n + 1) % 2
        q_psi_step(lat, params, f, t, LEAPFROG, hyperb, ps[b], ps[a], qs[a], threads)
        if hyperb:
            q_step(lat, params, Q_HYPER, qs[b], qs[a], ps[a], threads)
        else:
            q_step(lat, params, Q_PARA, qs[b], qs[b], ps[b], threads)
    return ps[nsteps % 2], qs[nsteps % 2]


FIELD_WIDTH = {0: 1, 1: 5, 2: 7, 3: 1, 4: 3, 5: 3}


def node_fields(lat, params, fields, t, kind, psi) -> np.ndarray:
    """Per-node output field, shape (Z, Y, X, V, K) (orc_node_fields)."""
    X, Y, Z = (int(params.dims[i]) for i in range(3))
    out = np.zeros((Z, Y, X, lat.nodes, FIELD_WIDTH[kind]))
    _check(lib().orc_node_fields(C.byref(lat.desc), C.byref(params), C.byref(fields), t, kind, _dp(psi), _dp(out)),
           "orc_node_fields")
    return out


def split_step(lat, params, part, psi, q, threads=0):
    _check(lib().orc_split_step(C.byref(lat.desc), C.byref(params), part, _dp(psi), _dp(q), threads), "orc_split_step")


def split_run(lat, params, psi, q, nsteps, start=True, threads=0):
    """Time loop of the real/imaginary split scheme (RelativisticGpeC15/
    GPUGrossPitaevskii_C15.cu:469-482): the q_R start, then per step the I half
    and the R half, in place on psi = R + iI and q = q_R + i q_I."""
    if start:
        split_step(lat, params, 2, psi, q, threads)
    for _ in range(nsteps):
        split_step(lat, params, 0, psi, q, threads)
        split_step(lat, params, 1, psi, q, threads)


def hyper_itp_run(lat, params, psi_even, psi_odd, q_even, q_odd, niter, hpsi=None, threads=0):
    """Imaginary-time loop of the hyperbolic scheme (RelativisticSpin2Gpe.cu:1712-1719;
    RelativisticSpin1Gpe.cu:687-697): per iteration itp_q and itp_psi both read the
    current (psi, q) pair and write the other one, then the new psi is renormalised.
    Starts from the even pair; returns the newest (psi, q).  hpsi, if given, holds
    H psi of the last iteration's input."""
    ps = [psi_even, psi_odd]
    qs = [q_even, q_odd]
    f = capi.make_fields()
    for n in range(niter):
        a, b = n % 2, (n + 1) % 2
        q_step(lat, params, Q_ITP, qs[b], qs[a], ps[a], threads)
        q_psi_step(lat, params, f, 0.0, ITP, False, ps[b], ps[a], qs[a], threads, hpsi=hpsi)
        normalize(lat, params, ps[b])
    return ps[niter % 2], qs[niter % 2]


def gpblocks_run(X, Y, Z, V, deg, lapind, lapfac, lapfac0, g, pot, even, odd, steps):
    lapind = np.ascontiguousarray(lapind, dtype=np.int64)
    lib().orc_gpblocks_run(X, Y, Z, V, deg, lapind.ctypes.data_as(C.POINTER(C.c_int64)), lapfac, lapfac0, g, _dp(pot), _dp(even), _dp(odd), steps)


def gpblocks_norm(ii0, vsize, psi0, even, volume):
    out = np.zeros(2)
    lib().orc_gpblocks_norm(ii0, vsize, _dp(psi0), _dp(even), volume, _dp(out))
    return out


def respin(psi, zeta):
    """The phase-preparation kernels of the reference, in place on a host state
    (file layout, halo untouched since it is zero): at every node each component
    becomes sqrt(rho * w_m) times the phase of zeta_m, rho the node's density and
    w_m = |zeta_m|^2 -- polarState / ferromagneticState / mixedState
    (Spin1GpeBCC.cu:463-551), unState / horizontalBnState / verticalBnState /
    cyclicState (Spin2GpeBCC.cu:417-558)."""
    zeta = np.asarray(zeta, dtype=np.complex128)
    rho = np.sum(psi[..., 0] ** 2 + psi[..., 1] ** 2, axis=-1)
    for m, z in enumerate(zeta):
        w = z.real * z.real + z.imag * z.imag
        a = np.sqrt(w)
        amp = np.sqrt(rho * w)
        psi[..., m, 0] = amp * (z.real / a if a > 0 else 0.0)
        psi[..., m, 1] = amp * (z.imag / a if a > 0 else 0.0)
    return psi
