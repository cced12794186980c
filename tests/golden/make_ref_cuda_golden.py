"""Golden vectors from the reference's own CUDA kernels (tests/golden/ref_cuda_*.npz).

Needs a GPU and the cubins of oracle/build_ref_cuda.sh (built from the reference
tree).  For every case it uploads seeded random states into an FP64 libgpe
handle (whose buffers have the reference's BlockPsis / BlockEdges layout), runs
a short sequence of the reference's kernels on those buffers through
oracle/ref_cuda.py with per-step fields and times, and stores the parameters,
the inputs and the outputs (interior cells only).  The ground-state (imaginary-time)
kernels of the hyperbolic spin-2 program come from rel_spin2_gs.cubin.  tests/test_ref_cuda_golden.py
replays every sequence with the oracle (CPU) and with libgpe's kernels (GPU).

    python tests/golden/make_ref_cuda_golden.py [outdir] [--all]

Cases whose file already exists in outdir are kept unless --all is given.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_cuda as R  # noqa: E402
from spacetime_gb300 import capi, states  # noqa: E402
from spacetime_gb300.stepper import Stepper  # noqa: E402

NSTEPS = 4


def fields_table(n, seed):
    u = states.uniform01(seed, 8 * n).reshape(n, 8)
    return 2.0 * u - 1.0  # bq, bb[3], bq_quad, bb_quad[3]


def as_fields(row):
    return capi.make_fields(bq=row[0], bb=tuple(row[1:4]), bq_quad=row[4], bb_quad=tuple(row[5:8]))


def interior(a):
    return np.ascontiguousarray(a[1:-1, 1:-1, 1:-1])


def params_dict(p):
    return {"components": p.components, "scheme": p.scheme, "flags": p.flags, "dims": list(p.dims),
            "block_scale": p.block_scale, "p0": list(p.p0), "dt": p.dt, "trap_lambda": list(p.trap_lambda),
            "trap_offset": p.trap_offset, "trap_off_time": p.trap_off_time, "c0": p.c0, "c2": p.c2, "c4": p.c4,
            "alpha": p.alpha, "sigma": p.sigma, "quad_center": list(p.quad_center)}


def spinor_case(drv, name, program, lattice, C, dims, flags, dt, c0, c2, c4, alpha, seed, expansion=None):
    """forwardEuler (odd -> even) then NSTEPS-1 leapfrog steps (Spin1GpeBCC.cu:1428-1603).
    expansion = (t_start, rate): the block scale passed to each launch grows as
    bs0 (1 + rate (t - t_start)) from t_start on, as the program's expansion phase
    passes its growing expansionBlockScale (:1576-1588)."""
    lat = capi.Lattice(lattice)
    p = capi.make_params(components=C, precision=capi.FP64, dims=dims, block_scale=0.3, dt=dt,
                         trap_lambda=(1.0, 1.0, R.LAMBDA_Z), trap_offset=R.TRAP_OFFSET, c0=c0, c2=c2, c4=c4,
                         alpha=alpha, flags=flags, quad_center=R.QUAD_CENTER, lattice=lat)
    s = Stepper(lat, p)
    shape = capi.buffer_shape(lat, p)
    even0 = 0.2 * states.random_state(shape, seed=seed)
    odd0 = 0.2 * states.random_state(shape, seed=seed + 1)
    s.upload(capi.PSI_EVEN, even0)
    s.upload(capi.PSI_ODD, odd0)
    ent, w = R.stencil_int4(lat)
    d_ent, d_w = drv.upload(ent), drv.upload(w)
    grid, block = R.spinor_grid(p, lat.nodes)
    F = fields_table(NSTEPS, seed + 7)
    times = 0.25 + np.arange(NSTEPS) * dt
    bufs = [R.pitched(s, capi.PSI_ODD), R.pitched(s, capi.PSI_EVEN)]  # u_j lives in bufs[j % 2]
    for j in range(NSTEPS):
        kern = "euler" if j == 0 else "leapfrog"
        nxt, prv = bufs[(j + 1) % 2], bufs[j % 2]
        bs = p.block_scale
        if expansion is not None and times[j] >= expansion[0]:
            bs = p.block_scale * (1.0 + expansion[1] * (times[j] - expansion[0]))
        common = [nxt, prv, R.C.c_void_p(d_ent), R.C.c_void_p(d_w), R.mag_fields(as_fields(F[j])), R.uint3(p),
                  R.C.c_double(bs), R.double3(p.p0), R.C.c_double(c0), R.C.c_double(c2)]
        if program == "spin1_bcc":
            args = common + [R.C.c_double(alpha), R.C.c_bool(bool(flags & capi.FLAG_THREE_BODY_LOSS)),
                             R.C.c_bool(bool(flags & capi.FLAG_QUADRATIC_ZEEMAN)),
                             R.C.c_bool(bool(flags & capi.FLAG_QUADRUPOLE_OFFSET)), R.C.c_double(dt),
                             R.C.c_double(times[j])]
        else:  # spin-2: dt is a compile-time constant of the program
            args = common + [R.C.c_double(c4), R.C.c_double(alpha), R.C.c_double(times[j])]
        drv.launch(drv.function(program, kern), grid, block, args)
    out = {"even": interior(s.download(capi.PSI_EVEN)), "odd": interior(s.download(capi.PSI_ODD))}
    s.close()
    extra = {} if expansion is None else {"expansion": np.array(expansion, dtype=np.float64)}
    return dict(kind="spinor", lattice=lattice, params=params_dict(p), fields=F, times=times,
                in_even=interior(even0), in_odd=interior(odd0), **{"out_" + k: v for k, v in out.items()}, **extra)


def rel_case(drv, name, lattice, dims, dt, sigma, c0, c2, c4, seed, program="rel_spin2_bcc", C=5):
    """NSTEPS hyperbolic steps: update_psi then update_q per step
    (RelativisticSpin2Gpe.cu:1859-1899; RelativisticSpin1Gpe.cu:830-850;
    RelativisticGpeBCC.cu:683-687).  The scalar program's psi increment is
    dt_ref (-i H) and its q increment i (dt_ref/sigma)(q + d0 psi): libgpe's
    2 dt and 2 dt/sigma with dt = dt_ref/2; its potential array holds the trap
    values libgpe computes."""
    lat = capi.Lattice(lattice)
    scalar = program == "rel_scalar_bcc"
    p = capi.make_params(components=C, scheme=capi.SCHEME_HYPERBOLIC, precision=capi.FP64, dims=dims, block_scale=0.3,
                         dt=dt, trap_lambda=(1.0, 1.1, 1.3) if scalar else (1.0, 1.0, R.LAMBDA_Z),
                         trap_offset=R.TRAP_OFFSET, c0=c0, c2=c2, c4=c4, sigma=sigma, lattice=lat)
    s = Stepper(lat, p)
    shape, qshape = capi.buffer_shape(lat, p), capi.buffer_shape(lat, p, edges=True)
    ins = {"in_even": 0.2 * states.random_state(shape, seed=seed), "in_odd": 0.2 * states.random_state(shape, seed=seed + 1),
           "in_qeven": 0.2 * states.random_state(qshape, seed=seed + 2),
           "in_qodd": 0.2 * states.random_state(qshape, seed=seed + 3)}
    s.upload(capi.PSI_EVEN, ins["in_even"])
    s.upload(capi.PSI_ODD, ins["in_odd"])
    s.upload(capi.Q_EVEN, ins["in_qeven"])
    s.upload(capi.Q_ODD, ins["in_qodd"])
    d0, d1, w = R.edge_tables(lat, s, p.block_scale)
    d_d0, d_d1, d_w = drv.upload(d0), drv.upload(d1), drv.upload(w)
    grid, pblock = R.spinor_grid(p, lat.nodes)
    egrid, eblock = grid, R.edge_grid(p, lat.edges)[1]
    if scalar:
        grid, pblock = R.scalar_grid(p, lat.nodes)
        egrid, eblock = R.scalar_grid(p, lat.edges)
        d_pot = R.pitched_upload(drv, R.node_potential(lat, p))
    F = fields_table(NSTEPS, seed + 7) if not scalar else np.zeros((NSTEPS, 8))
    psi = [R.pitched(s, capi.PSI_EVEN), R.pitched(s, capi.PSI_ODD)]
    q = [R.pitched(s, capi.Q_EVEN), R.pitched(s, capi.Q_ODD)]
    for j in range(NSTEPS):
        a, b = j % 2, (j + 1) % 2  # prev parity, next parity
        if scalar:
            drv.launch(drv.function(program, "update_psi"), grid, pblock,
                       [psi[b], psi[a], q[a], d_pot, R.C.c_void_p(d_d1), R.C.c_void_p(d_w), R.C.c_double(c0), R.uint3(p),
                        R.C.c_double(2 * dt)])
            drv.launch(drv.function(program, "update_q"), egrid, eblock,
                       [q[b], q[a], psi[a], R.C.c_void_p(d_d0), R.uint3(p), R.C.c_double(2 * dt / sigma)])
            continue
        head = [psi[b], psi[a], q[a], R.C.c_void_p(d_d1), R.C.c_void_p(d_w), R.mag_fields(as_fields(F[j])),
                R.uint3(p), R.C.c_double(p.block_scale), R.double3(p.p0), R.C.c_double(c0), R.C.c_double(c2)]
        tail = [R.C.c_double(dt), R.C.c_bool(True), R.C.c_double(sigma)]
        drv.launch(drv.function(program, "update_psi"), grid, pblock,
                   head + ([R.C.c_double(c4)] if C == 5 else []) + tail)
        if C == 5:
            drv.launch(drv.function(program, "update_q"), egrid, eblock,
                       [q[b], q[a], psi[a], R.C.c_void_p(d_d0), R.uint3(p), R.C.c_double(dt / sigma), R.C.c_bool(True)])
        else:
            drv.launch(drv.function(program, "update_q_hyper"), egrid, eblock,
                       [q[b], q[a], psi[a], R.C.c_void_p(d_d0), R.uint3(p), R.C.c_double(dt / sigma)])
    out = {"out_even": interior(s.download(capi.PSI_EVEN)), "out_odd": interior(s.download(capi.PSI_ODD)),
           "out_qeven": interior(s.download(capi.Q_EVEN)), "out_qodd": interior(s.download(capi.Q_ODD))}
    s.close()
    return dict(kind="hyper", lattice=lattice, params=params_dict(p), fields=F, times=np.zeros(NSTEPS),
                **{k: interior(v) for k, v in ins.items()}, **out)


def itp_case(drv, name, program, C, dims, dt, sigma, c0, c2, c4, seed):
    """NSTEPS imaginary-time steps of the hyperbolic ground-state loop without the
    renormalisation: itp_q then itp_psi per step, both reading the previous (psi, q)
    pair (RelativisticSpin2Gpe.cu:1712-1713 with rel_spin2_gs.cubin;
    RelativisticSpin1Gpe.cu:687-688).  out_hpsi is H psi of the last step's input:
    get_Hpsi on it for spin-2 (:1677), itp_psi's own H psi output for spin-1."""
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=C, scheme=capi.SCHEME_HYPERBOLIC, precision=capi.FP64, dims=dims, block_scale=0.3,
                         dt=dt, trap_lambda=(1.0, 1.0, R.LAMBDA_Z), trap_offset=R.TRAP_OFFSET, c0=c0, c2=c2, c4=c4,
                         sigma=sigma, lattice=lat)
    s = Stepper(lat, p)
    shape, qshape = capi.buffer_shape(lat, p), capi.buffer_shape(lat, p, edges=True)
    ins = {"in_even": 0.2 * states.random_state(shape, seed=seed), "in_odd": 0.2 * states.random_state(shape, seed=seed + 1),
           "in_qeven": 0.2 * states.random_state(qshape, seed=seed + 2),
           "in_qodd": 0.2 * states.random_state(qshape, seed=seed + 3)}
    s.upload(capi.PSI_EVEN, ins["in_even"])
    s.upload(capi.PSI_ODD, ins["in_odd"])
    s.upload(capi.Q_EVEN, ins["in_qeven"])
    s.upload(capi.Q_ODD, ins["in_qodd"])
    d0, d1, w = R.edge_tables(lat, s, p.block_scale)
    d_d0, d_d1, d_w = drv.upload(d0), drv.upload(d1), drv.upload(w)
    grid, pblock = R.spinor_grid(p, lat.nodes)
    eblock = R.edge_grid(p, lat.edges)[1]
    d_h = R.pitched_upload(drv, np.zeros(shape))
    psi = [R.pitched(s, capi.PSI_EVEN), R.pitched(s, capi.PSI_ODD)]
    q = [R.pitched(s, capi.Q_EVEN), R.pitched(s, capi.Q_ODD)]
    geo = [R.uint3(p), R.C.c_double(p.block_scale), R.double3(p.p0), R.C.c_double(c0), R.C.c_double(c2)]
    for j in range(NSTEPS):
        a, b = j % 2, (j + 1) % 2
        if C == 5:
            drv.launch(drv.function(program, "itp_q"), grid, eblock,
                       [q[b], q[a], psi[a], R.C.c_void_p(d_d0), R.uint3(p), R.C.c_double(dt / sigma)])
            drv.launch(drv.function(program, "itp_psi"), grid, pblock,
                       [psi[b], psi[a], q[a], R.C.c_void_p(d_d1), R.C.c_void_p(d_w)] + geo +
                       [R.C.c_double(c4), R.C.c_double(dt)])
        else:
            drv.launch(drv.function(program, "itp_q_hyper"), grid, eblock,
                       [q[b], q[a], psi[a], R.C.c_void_p(d_d0), R.uint3(p), R.C.c_double(dt / sigma)])
            drv.launch(drv.function(program, "itp_psi"), grid, pblock,
                       [d_h, psi[b], psi[a], q[a], R.C.c_void_p(d_d1), R.C.c_void_p(d_w),
                        R.mag_fields(capi.make_fields())] + geo + [R.C.c_double(dt)])
    if C == 5:
        a = (NSTEPS - 1) % 2
        drv.launch(drv.function(program, "get_Hpsi"), grid, pblock,
                   [d_h, psi[a], q[a], R.C.c_void_p(d_d1), R.C.c_void_p(d_w)] + geo + [R.C.c_double(c4)])
    out = {"out_even": interior(s.download(capi.PSI_EVEN)), "out_odd": interior(s.download(capi.PSI_ODD)),
           "out_qeven": interior(s.download(capi.Q_EVEN)), "out_qodd": interior(s.download(capi.Q_ODD)),
           "out_hpsi": interior(R.pitched_download(drv, d_h, shape))}
    s.close()
    return dict(kind="itp", lattice="bcc", params=params_dict(p), fields=np.zeros((NSTEPS, 8)), times=np.zeros(NSTEPS),
                **{k: interior(v) for k, v in ins.items()}, **out)


def split_case(drv, name, dims, dt, sigma, g, seed, program="rel_scalar_c15"):
    """The C15 real/imaginary split program: its q_R start, then NSTEPS steps of
    update_psi(I) + update_q(q_I) + update_psi(R) + update_q(q_R)
    (RelativisticGpeC15/GPUGrossPitaevskii_C15.cu:469-482) on separate R, I, q_R,
    q_I arrays, with dt folded into the potential, g and the Hodge weights as the
    program does (:282-286).  The potential array holds the trap values libgpe
    computes (lambda = 1, no offset: potentialV3).  Stored as complex pairs
    psi = R + iI, q = q_R + i q_I, libgpe's split-scheme layout."""
    lat = capi.Lattice("c15")
    p = capi.make_params(components=1, scheme=capi.SCHEME_SPLIT, precision=capi.FP64, dims=dims, block_scale=0.3,
                         dt=dt, trap_lambda=(1.0, 1.0, 1.0), trap_offset=0.0, c0=g, sigma=sigma, lattice=lat)
    shape, qshape = capi.buffer_shape(lat, p), capi.buffer_shape(lat, p, edges=True)
    psi = 0.2 * states.random_state(shape, seed=seed)
    q = 0.2 * states.random_state(qshape, seed=seed + 2)
    parts = [np.ascontiguousarray(psi[..., 0, 0]), np.ascontiguousarray(psi[..., 0, 1]),
             np.ascontiguousarray(q[..., 0, 0]), np.ascontiguousarray(q[..., 0, 1])]
    dR, dI, dqR, dqI = (R.pitched_upload(drv, a) for a in parts)
    d_pot = R.pitched_upload(drv, R.node_potential(lat, p) * dt)
    V, E = lat.nodes, lat.edges
    d0, d1, w = R.edge_tables_for(lat, p.block_scale, (V * 8, dR.pitch, dR.slicePitch), (E * 8, dqR.pitch, dqR.slicePitch))
    d_d0, d_d1, d_w = drv.upload(d0), drv.upload(d1), drv.upload(w * dt)
    grid, block = R.scalar_grid(p, V)
    egrid, eblock = R.scalar_grid(p, E)
    dts = dt / sigma
    dbl = R.C.c_double
    fq, fpsi = drv.function(program, "update_q"), drv.function(program, "update_psi")

    def upd_q(nq, pq, ps, coef, sign):
        drv.launch(fq, egrid, eblock, [nq, pq, ps, R.C.c_void_p(d_d0), R.uint3(p), dbl(coef), dbl(sign)])

    def upd_psi(nx, pv, qs, sign):
        drv.launch(fpsi, grid, block, [nx, pv, qs, d_pot, R.C.c_void_p(d_d1), R.C.c_void_p(d_w), dbl(g * dt), R.uint3(p),
                                       dbl(sign)])

    upd_q(dqR, dqR, dR, dts / (dt - dts), 1.0)
    for _ in range(NSTEPS):
        upd_psi(dI, dR, dqR, -1.0)
        upd_q(dqI, dqR, dR, dts, 1.0)
        upd_psi(dR, dI, dqI, 1.0)
        upd_q(dqR, dqI, dI, dts, -1.0)
    outp, outq = np.zeros_like(psi), np.zeros_like(q)
    outp[..., 0, 0] = R.pitched_download(drv, dR, parts[0].shape)
    outp[..., 0, 1] = R.pitched_download(drv, dI, parts[1].shape)
    outq[..., 0, 0] = R.pitched_download(drv, dqR, parts[2].shape)
    outq[..., 0, 1] = R.pitched_download(drv, dqI, parts[3].shape)
    return dict(kind="split", lattice="c15", params=params_dict(p), fields=np.zeros((NSTEPS, 8)), times=np.zeros(NSTEPS),
                in_even=interior(psi), in_qeven=interior(q), out_even=interior(outp), out_qeven=interior(outq))


def scalar_case(drv, name, program, lattice, dims, dt, g, seed):
    """NSTEPS leapfrog updates of the scalar programs.  Their update is
    next += dt_ref (-i H) (GPUGrossPitaevskii_BCC.cu:345-346); the C15/A15/FCC
    programs fold dt_ref into the weights, the potential and g
    (GPUGrossPitaevskii_C15.cu:241-246).  libgpe's step is next += 2 dt (-i H),
    so dt_ref = 2 dt.  The potential array holds the trap values libgpe computes."""
    lat = capi.Lattice(lattice)
    p = capi.make_params(components=1, precision=capi.FP64, dims=dims, block_scale=0.3, dt=dt,
                         trap_lambda=(1.0, 1.1, 1.3), trap_offset=R.TRAP_OFFSET, c0=g, lattice=lat)
    s = Stepper(lat, p)
    shape = capi.buffer_shape(lat, p)
    even0 = 0.2 * states.random_state(shape, seed=seed)
    odd0 = 0.2 * states.random_state(shape, seed=seed + 1)
    s.upload(capi.PSI_EVEN, even0)
    s.upload(capi.PSI_ODD, odd0)
    dt_ref = 2.0 * dt
    folded = program != "scalar_bcc"
    scale = 1.0 / (p.block_scale ** 2) * (dt_ref if folded else 1.0)
    ent, w = R.stencil_int2(lat, s, scale)
    pot = R.node_potential(lat, p) * (dt_ref if folded else 1.0)
    d_ent, d_w = drv.upload(ent), drv.upload(w)
    d_pot = R.pitched_upload(drv, pot)
    grid, block = R.scalar_grid(p, lat.nodes)
    bufs = [R.pitched(s, capi.PSI_EVEN), R.pitched(s, capi.PSI_ODD)]
    for j in range(NSTEPS):
        nxt, prv = bufs[(j + 1) % 2], bufs[j % 2]
        args = [nxt, prv, d_pot, R.C.c_void_p(d_ent), R.C.c_void_p(d_w)]
        if program == "scalar_fcc":
            rp = lat.row_ptr
            csr = np.stack([rp[:-1], np.diff(rp)], axis=1).astype(np.int32)
            args.append(R.C.c_void_p(drv.upload(csr)))
        args.append(R.C.c_double(g * dt_ref if folded else g))
        args.append(R.uint3(p))
        if not folded:
            args.append(R.C.c_double(dt_ref))
        drv.launch(drv.function(program, "update"), grid, block, args)
    out = {"out_even": interior(s.download(capi.PSI_EVEN)), "out_odd": interior(s.download(capi.PSI_ODD))}
    s.close()
    return dict(kind="scalar", lattice=lattice, params=params_dict(p), fields=np.zeros((NSTEPS, 8)),
                times=np.zeros(NSTEPS), in_even=interior(even0), in_odd=interior(odd0), **out)


def fields_case(drv, name, dims, c0, c2, seed, t=0.25):
    """The spin-1 program's per-node output kernels on one seeded state:
    localAvgSpinAndDensity (Spin1GpeBCC.cu:235-271), uvTheta (:273-326) and
    maxHamilton (:144-189, with the program's compiled-in trap at time t and one
    field row), each writing FP64 arrays in the order V (z X Y + y X + x) + l."""
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=3, precision=capi.FP64, dims=dims, block_scale=0.3, dt=2e-4,
                         trap_lambda=(1.0, 1.0, R.LAMBDA_Z), trap_offset=R.TRAP_OFFSET, c0=c0, c2=c2, lattice=lat)
    s = Stepper(lat, p)
    shape = capi.buffer_shape(lat, p)
    psi = 0.2 * states.random_state(shape, seed=seed)
    s.upload(capi.PSI_EVEN, psi)
    n = lat.nodes * dims[0] * dims[1] * dims[2]
    zeros = np.zeros(n)
    d_norm, d_spin, d_dens = drv.upload(zeros), drv.upload(np.zeros(3 * n)), drv.upload(zeros)
    d_u, d_v, d_th, d_h = drv.upload(np.zeros(3 * n)), drv.upload(np.zeros(3 * n)), drv.upload(zeros), drv.upload(zeros)
    grid, block = R.spinor_grid(p, lat.nodes)
    buf = R.pitched(s, capi.PSI_EVEN)
    F = fields_table(1, seed + 7)
    vp = R.C.c_void_p
    drv.launch(drv.function("spin1_bcc", "localAvgSpinAndDensity"), grid, block,
               [vp(d_norm), vp(d_spin), vp(d_dens), buf, R.uint3(p)])
    drv.launch(drv.function("spin1_bcc", "uvTheta"), grid, block, [vp(d_u), vp(d_v), vp(d_th), buf, R.uint3(p)])
    drv.launch(drv.function("spin1_bcc", "maxHamilton"), grid, block,
               [vp(d_h), buf, R.mag_fields(as_fields(F[0])), R.uint3(p), R.C.c_double(p.block_scale), R.double3(p.p0),
                R.C.c_double(c0), R.C.c_double(c2), R.C.c_double(0.0), R.C.c_double(t)])
    get = lambda d, k: drv.download(d, 8 * k * n).view(np.float64).reshape(n, k)  # noqa: E731
    out = {"out_spin_norm": get(d_norm, 1)[:, 0], "out_avg_spin": get(d_spin, 3), "out_density": get(d_dens, 1)[:, 0],
           "out_u": get(d_u, 3), "out_v": get(d_v, 3), "out_theta": get(d_th, 1)[:, 0], "out_max_hamilton": get(d_h, 1)[:, 0]}
    s.close()
    return dict(kind="fields", lattice="bcc", params=params_dict(p), fields=F, times=np.array([t]), in_even=interior(psi),
                **out)


def respin_case(drv, name, program, C, kernels, seed):
    """The programs' phase-preparation kernels, each applied to a fresh copy of one
    seeded state (Spin1GpeBCC.cu:463-551, Spin2GpeBCC.cu:417-558).  kernels:
    (kernel, phase argument or None, the spinor zeta it writes)."""
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=C, precision=capi.FP64, dims=(4, 3, 2), block_scale=0.3, lattice=lat)
    s = Stepper(lat, p)
    psi = 0.2 * states.random_state(capi.buffer_shape(lat, p), seed=seed)
    grid, block = R.spinor_grid(p, lat.nodes)
    outs, zetas = [], []
    for kern, phase, zeta in kernels:
        s.upload(capi.PSI_EVEN, psi)
        args = [R.pitched(s, capi.PSI_EVEN), R.uint3(p)]
        if phase is not None:
            args.append(R.C.c_double(phase))
        drv.launch(drv.function(program, kern), grid, block, args)
        outs.append(interior(s.download(capi.PSI_EVEN)))
        zetas.append(np.array(zeta, dtype=np.complex128))
    s.close()
    return dict(kind="respin", lattice="bcc", params=params_dict(p), fields=np.zeros((1, 8)), times=np.zeros(1),
                in_even=interior(psi), out_states=np.stack(outs), zetas=np.stack(zetas),
                kernels=np.array([k for k, _, _ in kernels]))


S2, S13, S23 = 0.5 ** 0.5, (1.0 / 3.0) ** 0.5, (2.0 / 3.0) ** 0.5
CASES = [
    ("spin1_bcc", lambda d: spinor_case(d, "spin1_bcc", "spin1_bcc", "bcc", 3, (5, 3, 2), 0, 2e-4, 120.0, -7.0, 0.0, 0.0, 11)),
    ("spin1_bcc_toggles", lambda d: spinor_case(d, "spin1_bcc_toggles", "spin1_bcc", "bcc", 3, (4, 3, 3),
                                                capi.FLAG_THREE_BODY_LOSS | capi.FLAG_QUADRATIC_ZEEMAN | capi.FLAG_QUADRUPOLE_OFFSET,
                                                2e-4, 120.0, -7.0, 0.0, 2.0, 21)),
    ("spin1_bcc_expansion", lambda d: spinor_case(d, "spin1_bcc_expansion", "spin1_bcc", "bcc", 3, (4, 3, 3), 0, 2e-4,
                                                  120.0, -7.0, 0.0, 0.0, 23, expansion=(0.2501, 50.0))),
    ("spin2_bcc", lambda d: spinor_case(d, "spin2_bcc", "spin2_bcc", "bcc", 5, (5, 3, 2), capi.FLAG_THREE_BODY_LOSS,
                                        R.SPIN2_DT, 120.0, -7.0, 3.0, 2.0, 31)),
    ("rel_spin2_bcc", lambda d: rel_case(d, "rel_spin2_bcc", "bcc", (4, 3, 2), 2e-4, 0.01, 120.0, -7.0, 3.0, 41)),
    ("rel_spin1_bcc", lambda d: rel_case(d, "rel_spin1_bcc", "bcc", (4, 3, 2), 2e-4, 0.01, 120.0, -7.0, 0.0, 43,
                                         program="rel_spin1_bcc", C=3)),
    ("rel_scalar_bcc", lambda d: rel_case(d, "rel_scalar_bcc", "bcc", (5, 3, 2), 1e-4, R.REL_SCALAR_SIGMA, 150.0, 0.0,
                                          0.0, 45, program="rel_scalar_bcc", C=1)),
    ("itp_rel_spin2_gs", lambda d: itp_case(d, "itp_rel_spin2_gs", "rel_spin2_gs", 5, (4, 3, 2), 1e-3, 0.1, 120.0, -7.0,
                                            3.0, 91)),
    ("itp_rel_spin1_bcc", lambda d: itp_case(d, "itp_rel_spin1_bcc", "rel_spin1_bcc", 3, (4, 3, 2), 1e-3, 0.1, 120.0,
                                             -7.0, 0.0, 93)),
    ("rel_scalar_c15", lambda d: split_case(d, "rel_scalar_c15", (2, 2, 2), 1e-3, 0.01, 300.0, 95)),
    ("scalar_bcc", lambda d: scalar_case(d, "scalar_bcc", "scalar_bcc", "bcc", (5, 3, 2), 2e-4, 150.0, 51)),
    ("scalar_c15", lambda d: scalar_case(d, "scalar_c15", "scalar_c15", "c15", (2, 2, 2), 2e-4, 150.0, 61)),
    ("scalar_a15", lambda d: scalar_case(d, "scalar_a15", "scalar_a15", "a15", (3, 2, 2), 2e-4, 150.0, 71)),
    ("scalar_fcc", lambda d: scalar_case(d, "scalar_fcc", "scalar_fcc", "fcc", (3, 3, 2), 2e-4, 150.0, 81)),
    ("fields_spin1_bcc", lambda d: fields_case(d, "fields_spin1_bcc", (4, 3, 2), 120.0, -7.0, 97)),
    ("respin_spin1_bcc", lambda d: respin_case(d, "respin_spin1_bcc", "spin1_bcc", 3, [
        ("polarState", None, (0, 1, 0)), ("ferromagneticState", None, (1, 0, 0)),
        ("mixedState", 0.3, (0.3 ** 0.5, 0.7 ** 0.5, 0))], 99)),
    ("respin_spin2_bcc", lambda d: respin_case(d, "respin_spin2_bcc", "spin2_bcc", 5, [
        ("unState", None, (0, 0, 1, 0, 0)),
        ("horizontalBnState", 0.7, (S2, 0, 0, 0, S2 * np.exp(0.7j))),
        ("verticalBnState", 1.1, (0, S2, 0, S2 * np.exp(1.1j), 0)),
        ("cyclicState", 0.4, (S13, 0, 0, S23 * np.exp(0.4j), 0))], 101)),
]


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    # a handle first: it makes the primary context current for the driver API
    warm = Stepper(capi.Lattice("bcc"), capi.make_params(components=1, precision=capi.FP64, dims=(2, 2, 2)))
    drv = R.Driver()
    try:
        for name, fn in CASES:
            program = (name.replace("_toggles", "").replace("_expansion", "").replace("itp_", "").replace("fields_", "")
                       .replace("respin_", ""))
            if os.path.exists(os.path.join(outdir, "ref_cuda_%s.npz" % name)) and "--all" not in sys.argv:
                continue  # keep the vectors already made
            if not R.available(program):
                print("skip %s: %s.cubin not built" % (name, program))
                continue
            case = fn(drv)
            case["params"] = json.dumps(case["params"])
            path = os.path.join(outdir, "ref_cuda_%s.npz" % name)
            np.savez_compressed(path, **case)
            print("wrote", path)
    finally:
        drv.close()
        warm.close()


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    main(args[0] if args else os.path.join(ROOT, "tests", "golden"))
