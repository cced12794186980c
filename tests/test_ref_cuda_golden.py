"""Parity with the reference's own CUDA kernels (golden vectors).

tests/golden/ref_cuda_*.npz hold short runs of the reference's unmodified
kernels -- spin-1 leapfrog/forwardEuler with and without loss, quadratic Zeeman
and quadrupole offset (Spin1GpeBCC.cu:667-917) and with a growing block scale
(the expansion phase, :1576-1588), spin-2 (Spin2GpeBCC.cu:698-990),
relativistic spin-2 update_psi + update_q (RelativisticSpin2Gpe.cu:971-1132),
the C15 real/imaginary split scalar program (RelativisticGpeC15/
GPUGrossPitaevskii_C15.cu:90-155, 469-482), the hyperbolic imaginary-time pair
itp_q + itp_psi and get_Hpsi of the spin-2 and
spin-1 ground-state loops (RelativisticSpin2Gpe.cu:558-807;
RelativisticSpin1Gpe/hyper_kernels.h:4-40, common_kernels.h:17-94), and the
scalar BCC / C15 / A15 / FCC updates, and the spin-1 program's per-node output
kernels localAvgSpinAndDensity, uvTheta and maxHamilton (Spin1GpeBCC.cu:144-326)
and the phase-preparation kernels of the spin-1 and spin-2 programs
(Spin1GpeBCC.cu:463-551, Spin2GpeBCC.cu:417-558) -- made by
tests/golden/make_ref_cuda_golden.py on a GB300 from seeded inputs.

CPU: the FP64 oracle replays each run: max |oracle - reference| <= 1e-12 * max|reference|
(the reference contracts multiply-adds, the oracle does not; the scalar programs
fold dt into their tables).  GPU: libgpe's FP64 kernels replay it to the same
bound, its FP32 kernels to 2e-5 * max|reference|.
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle import oracle
from spacetime_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_cuda_*.npz")))
IDS = [os.path.basename(f)[9:-4] for f in FILES]


def _load(path):
    d = dict(np.load(path, allow_pickle=False))
    d["params"] = json.loads(str(d["params"]))
    d["kind"] = str(d["kind"])
    d["lattice"] = str(d["lattice"])
    return d


def _params(d, precision):
    pd = dict(d["params"])
    lat = capi.Lattice(d["lattice"])
    pd["precision"] = precision
    pd["dims"] = tuple(pd["dims"])
    pd["trap_lambda"] = tuple(pd["trap_lambda"])
    pd["quad_center"] = tuple(pd["quad_center"])
    return lat, capi.make_params(lattice=lat, **pd)


def _embed(a):
    out = np.zeros((a.shape[0] + 2, a.shape[1] + 2, a.shape[2] + 2) + a.shape[3:])
    out[1:-1, 1:-1, 1:-1] = a
    return out


def _fields(row):
    return capi.make_fields(bq=row[0], bb=tuple(row[1:4]), bq_quad=row[4], bb_quad=tuple(row[5:8]))


def _expanded(p, d, t):
    """The parameters of a step at time t of a run with condensate expansion: the
    oracle takes the step's block scale as the reference's launch does."""
    if "expansion" not in d:
        return p
    t0, rate = (float(v) for v in d["expansion"])
    q = capi.Params.from_buffer_copy(p)
    if t >= t0:
        q.block_scale = p.block_scale * (1.0 + rate * (t - t0))
    return q


def _check(got, want, tol, what):
    g = got[1:-1, 1:-1, 1:-1] if got.shape != want.shape else got
    scale = float(np.max(np.abs(want)))
    err = float(np.max(np.abs(g - want)))
    assert err <= tol * scale, "%s: max|diff| = %.3e, scale %.3e" % (what, err, scale)


def _fields_check(get, d, tol, uv=True):
    """The node-field kernels' outputs (localAvgSpinAndDensity, uvTheta,
    maxHamilton) against `get(kind, fields, t)` -> (Z, Y, X, V, K).  uv: also the
    u, v, theta frame (its orientation is ill-conditioned where |m| ~ |n|, so it
    is compared on FP64 states only)."""
    f = _fields(d["fields"][0])
    t = float(d["times"][0])
    spin = get(capi.FIELD_SPIN, f, t).reshape(-1, 5)
    _check(spin[:, 0], d["out_spin_norm"], tol, "spin norm")
    _check(spin[:, 1:4], d["out_avg_spin"], tol, "local average spin")
    _check(spin[:, 4], d["out_density"], tol, "density")
    if uv:
        uvt = get(capi.FIELD_UV_THETA, f, t).reshape(-1, 7)
        _check(uvt[:, 0:3], d["out_u"], tol, "u")
        _check(uvt[:, 3:6], d["out_v"], tol, "v")
        _check(uvt[:, 6], d["out_theta"], tol, "theta")
    _check(get(capi.FIELD_MAX_HAMILTON, f, t).reshape(-1), d["out_max_hamilton"], tol, "max Hamilton")


def test_golden_files_present():
    assert len(FILES) >= 17, "reference-kernel golden vectors missing"


@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_oracle_vs_reference_cuda(path):
    d = _load(path)
    lat, p = _params(d, capi.FP64)
    n = d["fields"].shape[0]
    if d["kind"] == "fields":
        psi = _embed(d["in_even"])
        _fields_check(lambda kind, f, t: oracle.node_fields(lat, p, f, t, kind, psi), d, 1e-12)
        return
    if d["kind"] == "respin":
        for zeta, want in zip(d["zetas"], d["out_states"]):
            _check(oracle.respin(_embed(d["in_even"]), zeta), want, 1e-14, str(zeta))
        return
    if d["kind"] == "spinor":
        even, odd = _embed(d["in_even"]), _embed(d["in_odd"])
        bufs = [odd, even]
        for j in range(n):
            mode = oracle.EULER if j == 0 else oracle.LEAPFROG
            pj = _expanded(p, d, float(d["times"][j]))
            oracle.parabolic_step(lat, pj, _fields(d["fields"][j]), float(d["times"][j]), mode, bufs[(j + 1) % 2], bufs[j % 2])
    elif d["kind"] == "scalar":
        even, odd = _embed(d["in_even"]), _embed(d["in_odd"])
        bufs = [even, odd]
        for j in range(n):
            oracle.parabolic_step(lat, p, capi.make_fields(), 0.0, oracle.LEAPFROG, bufs[(j + 1) % 2], bufs[j % 2])
    elif d["kind"] == "hyper":
        ps = [_embed(d["in_even"]), _embed(d["in_odd"])]
        qs = [_embed(d["in_qeven"]), _embed(d["in_qodd"])]
        for j in range(n):
            a, b = j % 2, (j + 1) % 2
            oracle.q_psi_step(lat, p, _fields(d["fields"][j]), 0.0, oracle.LEAPFROG, True, ps[b], ps[a], qs[a])
            oracle.q_step(lat, p, oracle.Q_HYPER, qs[b], qs[a], ps[a])
        even, odd = ps
        _check(qs[0], d["out_qeven"], 1e-12, "q even")
        _check(qs[1], d["out_qodd"], 1e-12, "q odd")
    elif d["kind"] == "split":  # the q_R start, then NSTEPS (I, q_I), (R, q_R) half-step pairs
        even, q = _embed(d["in_even"]), _embed(d["in_qeven"])
        oracle.split_run(lat, p, even, q, n)
        _check(q, d["out_qeven"], 1e-12, "q")
        _check(even, d["out_even"], 1e-12, "psi")
        return
    else:  # itp: itp_q + itp_psi per step, H psi of the last step's input
        ps = [_embed(d["in_even"]), _embed(d["in_odd"])]
        qs = [_embed(d["in_qeven"]), _embed(d["in_qodd"])]
        hpsi = np.zeros_like(ps[0])
        for j in range(n):
            a, b = j % 2, (j + 1) % 2
            oracle.q_step(lat, p, oracle.Q_ITP, qs[b], qs[a], ps[a])
            oracle.q_psi_step(lat, p, capi.make_fields(), 0.0, oracle.ITP, False, ps[b], ps[a], qs[a], hpsi=hpsi)
        even, odd = ps
        _check(qs[0], d["out_qeven"], 1e-12, "q even")
        _check(qs[1], d["out_qodd"], 1e-12, "q odd")
        _check(hpsi, d["out_hpsi"], 1e-12, "H psi")
    _check(even, d["out_even"], 1e-12, "even")
    _check(odd, d["out_odd"], 1e-12, "odd")


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_kernels_vs_reference_cuda(gpu, path, prec):
    from spacetime_gb300.stepper import Stepper

    d = _load(path)
    lat, p = _params(d, prec)
    tol = 1e-12 if prec == capi.FP64 else 2e-5
    n = d["fields"].shape[0]
    with Stepper(lat, p) as s:
        if d["kind"] == "fields":
            # FP64 fields from the stored values: FP32 storage rounds the state itself
            s.upload(capi.PSI_EVEN, _embed(d["in_even"]))

            def get(kind, f, t):
                s.set_ramp(capi.make_ramp(bq_segments=[(f.bq, 1e9, capi.RAMP_CONSTANT)],
                                          bb_segments=[(tuple(f.bb), 1e9, capi.RAMP_CONSTANT)]), 0.0)
                return s.node_fields(capi.PSI_EVEN, kind, t)

            _fields_check(get, d, 1e-12 if prec == capi.FP64 else 2e-5, uv=prec == capi.FP64)
            return
        if d["kind"] == "respin":
            for zeta, want in zip(d["zetas"], d["out_states"]):
                s.upload(capi.PSI_EVEN, _embed(d["in_even"]))
                s.respin(capi.PSI_EVEN, zeta)
                _check(s.download(capi.PSI_EVEN), want, 1e-14 if prec == capi.FP64 else 1e-6, str(zeta))
            return
        if d["kind"] == "split":
            s.upload(capi.PSI_EVEN, _embed(d["in_even"]))
            s.upload(capi.Q_EVEN, _embed(d["in_qeven"]))
            s.start()
            s.step(n)
            _check(s.download(capi.PSI_EVEN), d["out_even"], tol, "psi")
            _check(s.download(capi.Q_EVEN), d["out_qeven"], tol, "q")
            return
        s.upload(capi.PSI_EVEN, _embed(d["in_even"]))
        s.upload(capi.PSI_ODD, _embed(d["in_odd"]))
        if "expansion" in d:
            s.set_expansion(*(float(v) for v in d["expansion"]))
        if d["kind"] in ("hyper", "itp"):
            s.upload(capi.Q_EVEN, _embed(d["in_qeven"]))
            s.upload(capi.Q_ODD, _embed(d["in_qodd"]))
        for j in range(n):
            if d["kind"] == "itp":
                slots = [capi.PSI_EVEN, capi.PSI_ODD]
                s.step_explicit(slots[(j + 1) % 2], slots[j % 2], capi.make_fields(), 0.0, capi.MODE_ITP)
            elif d["kind"] == "spinor":
                slots = [capi.PSI_ODD, capi.PSI_EVEN]
                mode = capi.MODE_EULER if j == 0 else capi.MODE_LEAPFROG
                s.step_explicit(slots[(j + 1) % 2], slots[j % 2], _fields(d["fields"][j]), float(d["times"][j]), mode)
            else:
                slots = [capi.PSI_EVEN, capi.PSI_ODD]
                f = _fields(d["fields"][j]) if d["kind"] == "hyper" else capi.make_fields()
                s.step_explicit(slots[(j + 1) % 2], slots[j % 2], f, 0.0, capi.MODE_LEAPFROG)
        _check(s.download(capi.PSI_EVEN), d["out_even"], tol, "even")
        _check(s.download(capi.PSI_ODD), d["out_odd"], tol, "odd")
        if d["kind"] in ("hyper", "itp"):
            _check(s.download(capi.Q_EVEN), d["out_qeven"], tol, "q even")
            _check(s.download(capi.Q_ODD), d["out_qodd"], tol, "q odd")
        if d["kind"] == "itp":
            _check(s.download(capi.HPSI), d["out_hpsi"], tol, "H psi")
