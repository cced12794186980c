"""FP32 fused stepper against an FP64 run of the reference's own spin-1 kernels.

CHECKER, not product: runs the reference's unmodified `forwardEuler` + `leapfrog`
(Spin1GpeBCC.cu:667-917, cubin from oracle/build_ref_cuda.sh) on an FP64
libgpe handle's buffers and libgpe's FP32 fused stepper on identical inputs --
the spin-1 BCC workload of bench.py (c0 = 2000, c2 = -50, polar state with
1e-3 relative noise, Bz ramp 0.5 -> -0.5 over 4000 steps, Bq = 0.2, dt = 5e-5,
box [-8, 8]^3) with the trap the reference program compiles in
(lambda = (1, 1, omega_z/omega_r), offset 100).  Both take the same steps with
the same fields and times (gpe_start + gpe_step's convention).  Every `every`
steps it records the FP64 observables of both states (gpe_observe, FP64
arithmetic) and at the end the max-abs wavefunction error.  Prints one JSON line.

    python -m oracle.ref_cuda_drift [--program spin1|scalar] [--cells N] [--steps N] [--every 100]

(spin1: 96^3, 10^4 steps by default; scalar: the scalar BCC 32^3 vortex, 1000 steps.)
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import ref_cuda as R  # noqa: E402


def run(cells=96, steps=10000, every=100, dt=5e-5, box=16.0):
    from spacetime_gb300 import capi, states
    from spacetime_gb300.stepper import Stepper

    lat = capi.Lattice("bcc")
    bs = box / (cells * lat.block_width[0])
    common = dict(components=3, dims=(cells, cells, cells), block_scale=bs, dt=dt, trap_lambda=(1.0, 1.0, R.LAMBDA_Z),
                  trap_offset=R.TRAP_OFFSET, c0=2000.0, c2=-50.0, lattice=lat)
    ramp = capi.make_ramp(bq_segments=[(0.2, 1e30, capi.RAMP_CONSTANT)],
                          bb_segments=[((0, 0, 0.5), 0.0, capi.RAMP_CONSTANT),
                                       ((0, 0, -0.5), 4000 * dt, capi.RAMP_LINEAR),
                                       ((0, 0, -0.5), 1e30, capi.RAMP_CONSTANT)])
    p64 = capi.make_params(precision=capi.FP64, **common)
    p32 = capi.make_params(precision=capi.FP32, **common)
    psi0 = states.spinor_state(lat, p64, states.POLAR, seed=2, noise=1e-3)
    ref = Stepper(lat, p64)   # buffers the reference kernels run on
    f32 = Stepper(lat, p32)
    drv = R.Driver()
    try:
        ref.upload(capi.PSI_ODD, psi0)
        ref.set_ramp(ramp, 0.0)  # only for observe's fields
        f32.upload(capi.PSI_ODD, psi0)
        f32.set_ramp(ramp, 0.0)
        ent, w = R.stencil_int4(lat)
        d_ent, d_w = drv.upload(ent), drv.upload(w)
        grid, block = R.spinor_grid(p64, lat.nodes)
        euler, leap = drv.function("spin1_bcc", "euler"), drv.function("spin1_bcc", "leapfrog")
        slots = [R.pitched(ref, capi.PSI_EVEN), R.pitched(ref, capi.PSI_ODD)]

        def ref_step(fn, nxt, prv, t):
            f = capi.Fields()
            capi.load_library().gpe_ramp_eval(C.byref(ramp), ramp.time_scale * t, C.byref(f))
            drv.launch(fn, grid, block, [nxt, prv, C.c_void_p(d_ent), C.c_void_p(d_w), R.mag_fields(f), R.uint3(p64),
                                         C.c_double(bs), R.double3(p64.p0), C.c_double(2000.0), C.c_double(-50.0),
                                         C.c_double(0.0), C.c_bool(False), C.c_bool(False), C.c_bool(False),
                                         C.c_double(dt), C.c_double(t)])

        t0 = time.perf_counter()
        ref_step(euler, slots[0], slots[1], 0.0)    # forwardEuler(even <- odd) at t0 (Spin1GpeBCC.cu:1433)
        f32.start()
        cur = 0                                     # the newest reference state is in slots[cur]
        rows = []

        def record(k):
            tk = k * dt
            a = ref.observe(capi.PSI_EVEN if cur == 0 else capi.PSI_ODD, tk)
            b = f32.observe(f32.current, tk)
            rows.append((k, a["energy"], b["energy"], a["norm"], b["norm"]))

        record(0)
        done32 = 0
        for k in range(steps):
            t = (k + 1) * dt
            ref_step(leap, slots[1 - cur], slots[cur], t)
            cur = 1 - cur
            if (k + 1) % every == 0 or k + 1 == steps:
                f32.step(k + 1 - done32)
                done32 = k + 1
                record(k + 1)
        elapsed = time.perf_counter() - t0
        a = ref.download(capi.PSI_EVEN if cur == 0 else capi.PSI_ODD)
        b = f32.download(f32.current)
        e = np.array(rows)
        return {"workload": "spin-1 BCC %d^3 cells, c0 2000, c2 -50, polar + 1e-3 noise, Bz 0.5->-0.5 over 4000 steps, "
                            "Bq 0.2, dt %g, trap lambda (1, 1, %.6f) + 100" % (cells, dt, R.LAMBDA_Z),
                "steps": steps, "every": every,
                "reference": "Spin1GpeBCC.cu forwardEuler + leapfrog, FP64, compiled unmodified for sm_103a",
                "psi_max_abs_err": float(np.max(np.abs(a - b))), "psi_max_abs": float(np.max(np.abs(a))),
                "energy_rel_diff_max": float(np.max(np.abs(e[:, 2] - e[:, 1]) / np.abs(e[:, 1]))),
                "norm_rel_diff_max": float(np.max(np.abs(e[:, 4] - e[:, 3]) / np.abs(e[:, 3]))),
                "energy_rel_drift_reference": float(abs(e[-1, 1] - e[0, 1]) / abs(e[0, 1])),
                "energy_rel_drift_fp32": float(abs(e[-1, 2] - e[0, 2]) / abs(e[0, 2])),
                "seconds": elapsed}
    finally:
        drv.close()
        ref.close()
        f32.close()


def run_scalar(cells=32, steps=1000, every=100, dt=1e-4, box=16.0, g=2000.0, trap_offset=R.TRAP_OFFSET):
    """The scalar workload (BCC 32^3, box [-8, 8]^3, trap omega = (1, 1, 1), g = 2000,
    Thomas-Fermi vortex + 1e-3 noise) on the reference's scalar BCC `update`
    (GPUGrossPitaevskii_BCC.cu:327-347): next += dt_ref (-i H prev) with
    dt_ref = 2 dt, its potential array holding libgpe's trap values; the start
    step is the same kernel with dt on a copy of the state (libgpe's forward
    Euler start)."""
    from spacetime_gb300 import capi, states
    from spacetime_gb300.stepper import Stepper

    lat = capi.Lattice("bcc")
    bs = box / (cells * lat.block_width[0])
    common = dict(components=1, dims=(cells, cells, cells), block_scale=bs, dt=dt, trap_offset=trap_offset, c0=g,
                  lattice=lat)
    p64 = capi.make_params(precision=capi.FP64, **common)
    p32 = capi.make_params(precision=capi.FP32, **common)
    psi0 = states.vortex_state(lat, p64, seed=1, noise=1e-3)
    ref, f32 = Stepper(lat, p64), Stepper(lat, p32)
    drv = R.Driver()
    try:
        ref.upload(capi.PSI_ODD, psi0)
        ref.upload(capi.PSI_EVEN, psi0)           # the start step updates a copy
        f32.upload(capi.PSI_ODD, psi0)
        ent, w = R.stencil_int2(lat, ref, 1.0 / (bs * bs))
        d_ent, d_w = drv.upload(ent), drv.upload(w)
        d_pot = R.pitched_upload(drv, R.node_potential(lat, p64))
        grid, block = R.scalar_grid(p64, lat.nodes)
        upd = drv.function("scalar_bcc", "update")
        slots = [R.pitched(ref, capi.PSI_EVEN), R.pitched(ref, capi.PSI_ODD)]

        def ref_step(nxt, prv, dt_ref):
            drv.launch(upd, grid, block, [nxt, prv, d_pot, C.c_void_p(d_ent), C.c_void_p(d_w), C.c_double(g), R.uint3(p64),
                                          C.c_double(dt_ref)])

        t0 = time.perf_counter()
        ref_step(slots[0], slots[1], dt)          # even = odd + dt (-i H odd)
        f32.start()
        cur, rows = 0, []

        def record(k):
            a = ref.observe(capi.PSI_EVEN if cur == 0 else capi.PSI_ODD, 0.0)
            b = f32.observe(f32.current, 0.0)
            rows.append((k, a["energy"], b["energy"], a["norm"], b["norm"]))

        record(0)
        done32 = 0
        for k in range(steps):
            ref_step(slots[1 - cur], slots[cur], 2 * dt)
            cur = 1 - cur
            if (k + 1) % every == 0 or k + 1 == steps:
                f32.step(k + 1 - done32)
                done32 = k + 1
                record(k + 1)
        elapsed = time.perf_counter() - t0
        a = ref.download(capi.PSI_EVEN if cur == 0 else capi.PSI_ODD)
        b = f32.download(f32.current)
        e = np.array(rows)
        return {"workload": "scalar BCC %d^3 cells, g %g, TF vortex + 1e-3 noise, dt %g (dt_ref %g), trap (1, 1, 1) + %g"
                            % (cells, g, dt, 2 * dt, trap_offset),
                "steps": steps, "every": every,
                "reference": "GPUGrossPitaevskii_BCC.cu update, FP64, compiled unmodified for sm_103a",
                "psi_max_abs_err": float(np.max(np.abs(a - b))), "psi_max_abs": float(np.max(np.abs(a))),
                "energy_rel_diff_max": float(np.max(np.abs(e[:, 2] - e[:, 1]) / np.abs(e[:, 1]))),
                "norm_rel_diff_max": float(np.max(np.abs(e[:, 4] - e[:, 3]) / np.abs(e[:, 3]))),
                "energy_rel_drift_reference": float(abs(e[-1, 1] - e[0, 1]) / abs(e[0, 1])),
                "energy_rel_drift_fp32": float(abs(e[-1, 2] - e[0, 2]) / abs(e[0, 2])),
                "seconds": elapsed}
    finally:
        drv.close()
        ref.close()
        f32.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--program", choices=["spin1", "scalar"], default="spin1")
    ap.add_argument("--cells", type=int, default=0)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--every", type=int, default=100)
    a = ap.parse_args()
    if a.program == "spin1":
        print(json.dumps(run(a.cells or 96, a.steps or 10000, a.every)))
    else:
        print(json.dumps(run_scalar(a.cells or 32, a.steps or 1000, a.every)))


if __name__ == "__main__":
    main()
