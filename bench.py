"""Benchmark: lattice site-updates/s of the fused FP32 stepper on one GB300.

Workload (the headline spin-1 configuration): spin-1 GPE on a BCC mesh of
96^3 block cells (10,616,832 dual nodes), box [-8, 8]^3, c0 = 2000, c2 = -50,
seeded polar state (0, 1, 0) with 1e-3 relative noise, linear Zeeman ramp
Bz 0.5 -> -0.5 over 4000 steps plus quadrupole gradient Bq = 0.2, dt = 5e-5.
Each psi buffer is 255 MB (FP32), larger than the 129 MB L2, so no L2 flush is
needed between iterations.

One bench "step" = one gpe_step_observe(100) call: 100 leapfrog steps (one fused
kernel each, in the cell-interleaved layout the call changes the state into and
back out of), the observables (norm, energy, magnetisation; FP32 node terms, FP64
sums) summed inside the last one.  value = sites * 100 * K / time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

INNER = 100                 # leapfrog steps per bench step
DIMS = (96, 96, 96)
BOX = 16.0
DT = 5e-5
C0, C2 = 2000.0, -50.0
RAMP_STEPS = 4000
BYTES_PER_SITE_FP32 = 72    # read psi_prev (24 B) + read/write psi_next (48 B), spin-1 FP32
BYTES_PER_SITE_FP64 = 144

# Optional legs (--workload): the other configurations of the benchmark plan.
#  scalar-bcc32: scalar GPE, BCC 32^3 cells, box [-8,8]^3, g = 2000, TF vortex + 1e-3 noise, dt = 1e-4
#  spin2-c15-128: relativistic spin-2, C15 128^3 cells (285,212,672 sites), hyperbolic psi+q,
#                 c0 = 2000, c2 = -20, c4 = 40, cyclic spinor + 1e-3 noise, sigma = 0.00225, dt = 2e-5
LEGS = {
    "scalar-bcc32": dict(lattice="bcc", C=1, dims=(32, 32, 32), c0=2000.0, c2=0.0, c4=0.0, dt=1e-4, scheme=0,
                         sigma=0.0, zeta=(1.0,), kappa=1, noise_abs=1e-3, noise_rel=0.0, bytes_fp32=24, seed=1,
                         trap_offset=0.0),
    "spin2-c15-128": dict(lattice="c15", C=5, dims=(128, 128, 128), c0=2000.0, c2=-20.0, c4=40.0, dt=2e-5, scheme=1,
                          sigma=0.00225, zeta=(math.sqrt(1 / 3), 0, 0, math.sqrt(2 / 3), 0), kappa=0, noise_abs=0.0,
                          noise_rel=1e-3, bytes_fp32=360, seed=3),
}
LEGS["spin2-c15-48"] = dict(LEGS["spin2-c15-128"], dims=(48, 48, 48))   # small case for profiling
#  scalar-hyper-bcc128: scalar hyperbolic psi+q (RelativisticGpeBCC), BCC 128^3 cells, c0 = 2000,
#                       sigma = 0.00225, dt = 2e-5; 72 B per site (psi 24 B + q 2 x 24 B, E/V = 2)
#  scalar-split-c15-64: the C15 real/imaginary split scheme (RelativisticGpeC15), C15 64^3 cells,
#                       two in-place half-step launches per step; 72 B per site (each half of
#                       psi and q read once and written once per step, E/V = 2)
LEGS["scalar-hyper-bcc128"] = dict(lattice="bcc", C=1, dims=(128, 128, 128), c0=2000.0, c2=0.0, c4=0.0, dt=2e-5,
                                   scheme=1, sigma=0.00225, zeta=(1.0,), kappa=1, noise_abs=1e-3, noise_rel=0.0,
                                   bytes_fp32=72, seed=6)
LEGS["scalar-split-c15-64"] = dict(lattice="c15", C=1, dims=(64, 64, 64), c0=2000.0, c2=0.0, c4=0.0, dt=2e-5,
                                   scheme=2, sigma=0.00225, zeta=(1.0,), kappa=1, noise_abs=1e-3, noise_rel=0.0,
                                   bytes_fp32=72, seed=7)
KERNEL_OF_SCHEME = {0: "leapfrog kernel (auto) C=%d", 1: "hyper_tile_kernel<float,%d> (fused tile)",
                    2: "split_step_kernel<float,PART> (C=%d, two launches per step)"}


def workload(precision):
    from spacetime_gb300 import capi, states

    lat = capi.Lattice("bcc")
    bs = BOX / (DIMS[0] * lat.block_width[0])
    p = capi.make_params(components=3, precision=precision, dims=DIMS, block_scale=bs, dt=DT, trap_offset=100.0,
                         c0=C0, c2=C2, lattice=lat)
    ramp = capi.make_ramp(bq_segments=[(0.2, 1e30, capi.RAMP_CONSTANT)],
                          bb_segments=[((0, 0, 0.5), 0.0, capi.RAMP_CONSTANT), ((0, 0, -0.5), RAMP_STEPS * DT, capi.RAMP_LINEAR),
                                       ((0, 0, -0.5), 1e30, capi.RAMP_CONSTANT)])
    psi0 = states.spinor_state(lat, p, states.POLAR, seed=2, noise=1e-3)
    return lat, p, ramp, psi0


def leg_params(w, prec, dims=None):
    """The leg's lattice and parameters (box [-8, 8]^3 along x) at `dims` (default
    the leg's own)."""
    from spacetime_gb300 import capi

    lat = capi.Lattice(w["lattice"])
    dims = tuple(dims or w["dims"])
    bs = BOX / (dims[0] * lat.block_width[0])
    p = capi.make_params(components=w["C"], scheme=w["scheme"], precision=prec, dims=dims, block_scale=bs, dt=w["dt"],
                         trap_offset=w.get("trap_offset", 100.0), c0=w["c0"], c2=w["c2"], c4=w["c4"], sigma=w["sigma"],
                         lattice=lat)
    return lat, p


def leg_init(w):
    from spacetime_gb300 import capi

    return capi.make_init(zeta=w["zeta"], kappa=w["kappa"], noise_abs=w["noise_abs"], noise_rel=w["noise_rel"],
                          seed=w["seed"])


def time_leg(w, steps, inner, warmup, kernel=0, dims=None):
    """A configuration on the device: seeded device-side initial state, start,
    `steps` x `inner` steps timed with CUDA events on the launching stream (the
    library's events give the step kernel's mean duration), and the observables
    (FP32 node terms, FP64 sums) after each bench step, inside the timed region."""
    import ctypes as C

    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    lat, p = leg_params(w, capi.FP32, dims)
    stream = torch.cuda.Stream()
    s = Stepper(lat, p)
    s.stream = C.c_void_p(stream.cuda_stream)
    # the per-bench-step observables as the headline's: FP32 node terms, FP64 sums
    s.set_tuning(capi.TUNE_OBSERVE_ARITH, 1)
    if kernel:
        s.set_tuning(capi.TUNE_KERNEL, kernel)
    with torch.cuda.stream(stream):
        s.init_state(s.current, leg_init(w))
        s.start()
        e0 = s.observe(s.current, 0.0)
        for _ in range(warmup):
            s.step(inner)
        torch.cuda.synchronize()
        n0 = s.launches
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        obs = []
        # the step launches' device time from the library's events on this stream
        # (layout changes of interleaved calls timed apart)
        s.set_tuning(capi.TUNE_TIMING, 1)
        s.step_timing(reset=True)
        with ClockSampler(0) as clk:
            a.record(stream)
            for _ in range(steps):
                s.step(inner)
                obs.append(s.observe(s.current))
            b.record(stream)
            torch.cuda.synchronize()
        timing = s.step_timing(reset=True)
        total_ms = a.elapsed_time(b)
        launches = s.launches - n0
    sites = s.sites
    gather = s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_GATHER
    interleaved = timing["interleaved_calls"] > 0
    s.close()
    launch_ms = timing["step_ms"] / timing["step_launches"]
    algo = w["bytes_fp32"] * sites
    peak, kind = measured_peak()
    name = KERNEL_OF_SCHEME[w["scheme"]] % w["C"]
    if w["scheme"] == 1 and gather:
        name = "hyper_step_kernel<float,%d> (gather form)" % w["C"]
    if w["scheme"] == 0 and gather:
        name = "parabolic_fixed_kernel<float,%d,LEAPFROG,4>" % w["C"]
    if interleaved and w["scheme"] == 1:
        name = "il_hyper_kernel<%d,%d>" % (w["C"], il_group_cells(p.dims[0]))
    elif interleaved:
        name = "il_step_kernel<%d,%d,%d>" % (w["C"], 8 if w["lattice"] == "fcc" else 4, il_group_cells(p.dims[0]))
    return {"metric": "lattice-site-updates/s", "value": sites * inner * steps / (total_ms * 1e-3),
            "unit": "lattice-site-updates/s", "steps": steps, "inner_steps_per_step": inner, "sites": sites,
            "ms_per_step": total_ms / steps, "dims": list(p.dims),
            "roofline": {"bound": "hbm", "achieved": algo / (launch_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (launch_ms * 1e-3) / 1e9 / peak, "peak_kind": kind, "kernel": name,
                         "algorithmic_bytes_per_launch": algo, "avg_launch_ms": launch_ms, "traffic": None},
            "gpu_launches": launches, "clocks": clk.summary(),
            "layout_change_ms_per_call": timing["convert_ms"] / timing["calls"] if interleaved else None,
            "energy_rel_drift": abs(obs[-1]["energy"] - e0["energy"]) / abs(e0["energy"]) if obs else None,
            "norm_last": obs[-1]["norm"] if obs else None}


def il_group_cells(x):
    """Cells per group of the interleaved layout for an x edge (the library's rule:
    32 unless 16 leaves fewer lanes idle)."""
    return 32 if 32 * ((x + 31) // 32) <= 16 * ((x + 15) // 16) else 16


def leg_e2e(w, steps, inner, dims=None, flight=1):
    """End to end through the C ABI with host buffers, every step: the FP64 host
    state (reference file layout, pinned) in, start (q from psi for the hyperbolic
    scheme), `inner` steps with the observables summed in the last one (or after it,
    on kernels without the fused form), the final FP64 state out into pinned host
    memory.  flight > 1: that many condensates in flight, one handle, stream, pinned
    host arrays and host thread each, the copies by DMA through the staging buffer
    (GPE_TUNE_TRANSFER 1) so that one condensate's copies run while another's kernels
    do; the value counts the steps of all, over the wall time of all."""
    import ctypes as C
    import threading

    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    lat, p = leg_params(w, capi.FP32, dims)
    runs = []
    for _ in range(flight):
        stream = torch.cuda.Stream()
        s = Stepper(lat, p)
        s.stream = C.c_void_p(stream.cuda_stream)
        if flight > 1:
            s.set_tuning(capi.TUNE_TRANSFER, 1)
        with torch.cuda.stream(stream):
            s.init_state(capi.PSI_ODD, leg_init(w))
            psi0 = s.download(capi.PSI_ODD)
        host = torch.from_numpy(psi0.ravel()).pin_memory().numpy().reshape(psi0.shape)
        out = torch.empty(psi0.size, dtype=torch.float64).pin_memory().numpy().reshape(psi0.shape)
        runs.append({"s": s, "stream": stream, "in": host, "out": out, "obs": None, "err": None})

    def work(r, n):
        try:
            s = r["s"]
            for _ in range(n):
                s.upload(capi.PSI_ODD, r["in"])
                s.start()
                r["obs"] = s.step_observe(inner)
                s.download(s.current, out=r["out"])
        except Exception as e:  # reported in the line
            r["err"] = "%s: %s" % (type(e).__name__, e)

    def all_runs(n):
        if flight == 1:
            work(runs[0], n)
            return
        ths = [threading.Thread(target=work, args=(r, n)) for r in runs]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    all_runs(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    all_runs(steps)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    sites = runs[0]["s"].sites
    nbytes = int(runs[0]["in"].nbytes)
    for r in runs:
        r["s"].close()
    res = {"value": flight * sites * inner * steps / el, "unit": "lattice-site-updates/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes + 96, "steps": flight * steps, "inner_steps_per_step": inner,
           "dims": list(p.dims), "condensates_in_flight": flight,
           "norm_last": runs[0]["obs"]["norm"] if runs[0]["obs"] else None,
           "path": "%d condensate(s) in flight, every step: gpe_upload (FP64 host, pinned) + gpe_start + "
                   "gpe_step_observe(%d) + gpe_download (FP64 host, pinned)" % (flight, inner)}
    errs = [r["err"] for r in runs if r["err"]]
    if errs:
        res["error"] = errs[0]
    return res


def run_leg(args):
    """--workload <leg>: one configuration's timing, printed as one JSON line."""
    w = LEGS[args.workload]
    inner = args.inner or INNER
    res = time_leg(w, args.steps, inner, args.warmup, args.kernel)
    res.update({"n_gpus": 1, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": dict(w, workload=args.workload, sites=res["sites"], inner_steps_per_step=inner)})
    if args.leg_drift:
        res["drift"] = leg_drift(w, None, args.drift_steps)
    print(json.dumps(res))
    return 0


def leg_drift(w, lat, nsteps, every=100, dims=None):
    """FP32 against FP64 on the leg's workload from the same seeded device state:
    observables (FP64 arithmetic) every `every` steps, and at the end the max-abs
    difference of the two states."""
    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    runs, last = {}, {}
    t0 = time.perf_counter()
    for prec in (capi.FP32, capi.FP64):
        lat, p = leg_params(w, prec, dims)
        s = Stepper(lat, p)
        s.init_state(s.current, leg_init(w))
        s.start()
        e = [s.observe(s.current, 0.0)]
        done = 0
        while done < nsteps:
            k = min(every, nsteps - done)
            s.step(k)
            done += k
            e.append(s.observe(s.current, done * w["dt"]))
        torch.cuda.synchronize()
        runs[prec] = e
        last[prec] = s.download(s.current)
        s.close()
    e32, e64 = runs[capi.FP32], runs[capi.FP64]
    return {"steps": nsteps, "every": every, "dims": list(dims or w["dims"]), "against": "libgpe FP64 (plain) stepper",
            "energy_rel_diff_max": max(abs(a["energy"] - b["energy"]) / abs(b["energy"]) for a, b in zip(e32, e64)),
            "norm_rel_diff_max": max(abs(a["norm"] - b["norm"]) / abs(b["norm"]) for a, b in zip(e32, e64)),
            "energy_rel_drift_fp32": abs(e32[-1]["energy"] - e32[0]["energy"]) / abs(e32[0]["energy"]),
            "energy_rel_drift_fp64": abs(e64[-1]["energy"] - e64[0]["energy"]) / abs(e64[0]["energy"]),
            "psi_max_abs_err": float(np.max(np.abs(last[capi.FP32] - last[capi.FP64]))),
            "psi_max_abs": float(np.max(np.abs(last[capi.FP64]))), "seconds": time.perf_counter() - t0}


# Adjoint ramp control: spin-1, BCC 64^3 cells, 2000 steps, Bz(t) and Bq(t) with 16
# piecewise-linear knots each (seeded uniform in [-1, 1]), loss 1 - |<T|psi(T)>|^2
# against a seeded hedgehog (monopole-like) target, 45-step checkpoints, central
# differences (h = 1e-4) of the FP64 run on 8 random knots.
ADJ = dict(dims=(64, 64, 64), steps=2000, stride=45, knots=16, fd_knots=8, h=1e-4, seed=4)


def run_adjoint(args):
    """--workload adjoint-bcc64: one JSON line."""
    print(json.dumps(adjoint_result(args.steps, args.adjoint_steps, args.fd_knots)))
    return 0


def adjoint_result(reps, n_steps, fd_knots):
    """Gradient of the ramp-control loss through the adjoint kernel (FP32 and
    FP64), timed from host knots to host gradient, and checked against central
    differences of the FP64 run."""
    import torch

    from spacetime_gb300 import capi, states
    from spacetime_gb300.adjoint import RampControl
    from spacetime_gb300.stepper import Stepper

    lat = capi.Lattice("bcc")
    dims = ADJ["dims"]
    bs = BOX / (dims[0] * lat.block_width[0])

    def params(prec):
        return capi.make_params(components=3, precision=prec, dims=dims, block_scale=bs, dt=DT, trap_offset=100.0,
                                c0=C0, c2=C2, lattice=lat)

    init = capi.make_init(zeta=states.POLAR, noise_rel=1e-3, seed=2)
    k = 2.0 * states.uniform01(ADJ["seed"], 2 * ADJ["knots"]).reshape(2, ADJ["knots"]) - 1.0
    target = states.monopole_state(lat, params(capi.FP64), seed=ADJ["seed"], noise=1e-3)
    out = {}
    for prec in (capi.FP32, capi.FP64):
        s = Stepper(lat, params(prec))
        rc = RampControl(s, n_steps, ADJ["knots"], lambda: s.init_state(capi.PSI_ODD, init), target,
                         stride=ADJ["stride"])
        reps = max(1, reps) if prec == capi.FP32 else 1
        fwd, bwd, grads, loss = [], [], None, None
        n0 = s.launches
        for it in range(reps + (1 if prec == capi.FP32 else 0)):
            bq = torch.tensor(k[0], requires_grad=True)
            bz = torch.tensor(k[1], requires_grad=True)
            t0 = time.perf_counter()
            loss = rc.loss(bq, bz)
            t1 = time.perf_counter()
            loss.backward()
            t2 = time.perf_counter()
            if prec == capi.FP32 and it == 0:
                n0 = s.launches
                continue  # warm-up
            fwd.append(t1 - t0)
            bwd.append(t2 - t1)
            grads = np.concatenate([bq.grad.numpy(), bz.grad.numpy()])
        launches = (s.launches - n0) / len(fwd)
        r = {"loss": float(loss.detach()), "grad": grads, "forward_s": statistics.median(fwd), "backward_s": statistics.median(bwd),
             "launches_per_gradient": launches}
        if prec == capi.FP64:
            rng = np.random.default_rng(ADJ["seed"])
            picks = rng.choice(2 * ADJ["knots"], fd_knots, replace=False)
            fd = []
            for i in picks:
                kp, km = k.copy().ravel(), k.copy().ravel()
                kp[i] += ADJ["h"]
                km[i] -= ADJ["h"]
                # central difference of L = 1 - |o|^2 taken as -(|o+|^2 - |o-|^2) / 2h: the
                # overlap of the polar state with the hedgehog is O(1e-4), and adding the
                # constant 1 first would round |o|^2 to a few digits
                with torch.no_grad():
                    op = rc.observables(torch.tensor(kp[:16]), torch.tensor(kp[16:]))
                    om = rc.observables(torch.tensor(km[:16]), torch.tensor(km[16:]))
                lp = -float(op[0] ** 2 + op[1] ** 2)
                lm = -float(om[0] ** 2 + om[1] ** 2)
                fd.append((lp - lm) / (2 * ADJ["h"]))
            r["fd_knots"] = [int(i) for i in picks]
            r["fd"] = fd
        out[prec] = r
        s.close()
    g32, g64 = out[capi.FP32]["grad"], out[capi.FP64]["grad"]
    picks, fd = out[capi.FP64]["fd_knots"], np.array(out[capi.FP64]["fd"], dtype=np.float64)
    rel_fd64 = np.abs(g64[picks] - fd) / np.maximum(np.abs(fd), 1e-300) if len(picks) else np.zeros(1)
    rel_fd32 = np.abs(g32[picks] - fd) / np.maximum(np.abs(fd), 1e-300) if len(picks) else np.zeros(1)
    sites = lat.nodes * dims[0] * dims[1] * dims[2]
    f32 = out[capi.FP32]
    grad_s = f32["forward_s"] + f32["backward_s"]
    res = {"metric": "adjoint gradient evaluations/s (forward + reverse run, %d steps)" % n_steps,
           "value": 1.0 / grad_s,
           "unit": "gradients/s", "n_gpus": 1, "steps": max(1, reps), "warmup": 1,
           "ms_per_step": 1e3 * grad_s, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "adjoint ramp control, spin-1 BCC 64^3 cells (%d sites), %d steps, %d+%d knots, "
                                  "%d-step checkpoints" % (sites, n_steps, ADJ["knots"], ADJ["knots"], ADJ["stride"]),
                      "dt": DT, "c0": C0, "c2": C2, "loss": "1 - |<monopole|psi(T)>|^2"},
           "forward_ms": 1e3 * f32["forward_s"], "backward_ms": 1e3 * f32["backward_s"],
           "reverse_site_updates_per_s": sites * n_steps / f32["backward_s"],
           "gpu_launches": f32["launches_per_gradient"],
           "loss_fp32": f32["loss"], "loss_fp64": out[capi.FP64]["loss"],
           "fp64_adjoint_vs_fd_max_rel": float(rel_fd64.max()), "fp32_adjoint_vs_fd_max_rel": float(rel_fd32.max()),
           "fp32_vs_fp64_adjoint_rel": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
           "fd_h": ADJ["h"], "fd_knots": [int(i) for i in picks], "fd": [float(x) for x in fd],
           "adjoint_fp64_at_fd_knots": [float(x) for x in g64[picks]],
           "fp64_forward_ms": 1e3 * out[capi.FP64]["forward_s"], "fp64_backward_ms": 1e3 * out[capi.FP64]["backward_s"]}
    # the timed call already runs through the public API from host arrays: the knots
    # in (the per-step fields and the FP64 target state uploaded by
    # gpe_adjoint_forward), the gradient out
    fields_bytes = n_steps * 8 * 8
    res["e2e"] = {"value": res["value"], "unit": "gradients/s", "h2d_bytes_per_step": int(fields_bytes + target.nbytes),
                  "d2h_bytes_per_step": int(5 * 8 + n_steps * 4 * 8),
                  "path": "torch knots -> gpe_adjoint_forward (fields + target from host) -> gpe_adjoint_backward "
                          "(gradient to host) -> torch"}
    return res


# Batched ensemble: 256 condensates, block-cell edge n ~ U{24..80}, lattice ~ U{BCC,
# FCC, A15, C15}, scalar or spin-1, trap omega ~ U[0.8, 1.2]^3, seeded ramps (Bz
# linear between two values in [-1, 1] over 2000 steps, Bq constant in [0, 0.5]),
# box [-8, 8]^3, dt = 5e-5, FP32 with FP64 observables; all advanced by the
# persistent batch kernel, n steps recorded in one CUDA graph.
ENS = dict(members=256, edge=(24, 80), lattices=("bcc", "fcc", "a15", "c15"), seed=5, dt=5e-5, ramp_steps=2000,
           steps=2000)


def ensemble_members(count=None):
    """The seeded ensemble: a list of (lattice, components, edge, omega, ramp) tuples."""
    from spacetime_gb300 import capi, states

    out = []
    for i in range(count or ENS["members"]):
        u = states.uniform01(ENS["seed"], 8, offset=8 * i)
        lo, hi = ENS["edge"]
        n = lo + min(int(u[0] * (hi - lo + 1)), hi - lo)
        lat = ENS["lattices"][min(int(u[1] * 4), 3)]
        comps = 1 if u[2] < 0.5 else 3
        omega = tuple(0.8 + 0.4 * u[3:6])
        bz0, bz1, bq = 2 * u[6] - 1, 2 * u[7] - 1, 0.5 * u[5]
        ramp = capi.make_ramp(bq_segments=[(bq, 1e30, capi.RAMP_CONSTANT)],
                              bb_segments=[((0, 0, bz0), 0.0, capi.RAMP_CONSTANT),
                                           ((0, 0, bz1), ENS["ramp_steps"] * ENS["dt"], capi.RAMP_LINEAR),
                                           ((0, 0, bz1), 1e30, capi.RAMP_CONSTANT)])
        out.append((lat, comps, n, omega, ramp))
    return out


def run_ensemble(args):
    """--workload ensemble-256: one JSON line."""
    print(json.dumps(ensemble_result(args.members, args.inner or 100, args.steps, args.warmup, args.batch_layout)))
    return 0


def ensemble_result(n_members, inner, replays, warmup, layout=1):
    """Every member advanced by the persistent batch kernel: `inner` steps in one
    persistent launch per CUDA-graph replay, `replays` replays timed with CUDA
    events (warm-up: `warmup` uncaptured 10-step batch calls).  layout 1: the
    spin-1 members in the interleaved layout (changed in and back inside every
    replay), 0: every member in its handle's layout."""
    import ctypes as C

    import torch

    from spacetime_gb300 import capi, states
    from spacetime_gb300.batch import Batch
    from spacetime_gb300.stepper import Stepper

    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    members, algo, state_bytes, specs = [], 0, 0, ensemble_members(n_members)
    t_setup = time.perf_counter()
    for i, (name, comps, n, omega, ramp) in enumerate(specs):
        lat = capi.Lattice(name)
        bs = BOX / (n * lat.block_width[0])
        p = capi.make_params(components=comps, precision=capi.FP32, dims=(n, n, n), block_scale=bs, dt=ENS["dt"],
                             trap_offset=100.0, trap_lambda=omega, c0=C0, c2=C2 if comps == 3 else 0.0, lattice=lat)
        s = Stepper(lat, p)
        s.stream = sp
        init = capi.make_init(zeta=states.POLAR, noise_rel=1e-3, seed=1000 + i) if comps == 3 else \
            capi.make_init(zeta=(1.0,), kappa=1, noise_abs=1e-3, seed=1000 + i)
        s.init_state(capi.PSI_ODD, init)
        s.set_ramp(ramp)
        s.start()
        members.append(s)
        algo += (72 if comps == 3 else 24) * s.sites
        state_bytes += (24 if comps == 3 else 8) * s.sites
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    b = Batch(members)
    b.stream = sp
    b.set_tuning(capi.BATCH_LAYOUT, layout)
    sites = b.sites
    tune = b.autotune(steps=2)
    e_first = [members[k].observe(members[k].current) for k in (0, len(members) // 2, len(members) - 1)]
    for _ in range(max(1, warmup)):
        b.step(10)
    b.capture(inner, sp)
    n0 = b.launches
    ev = []
    with ClockSampler(0) as clk:
        for _ in range(replays):
            x, y = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            x.record(stream)
            b.replay()
            y.record(stream)
            ev.append((x, y))
        torch.cuda.synchronize()
    ms = [x.elapsed_time(y) for x, y in ev]
    total_ms = sum(ms)
    launches = b.launches - n0
    e_last = [members[k].observe(members[k].current) for k in (0, len(members) // 2, len(members) - 1)]
    peak, kind = measured_peak()
    step_ms = total_ms / (replays * inner)
    counts = {}
    for name, comps, n, _, _ in specs:
        key = "%s/%s" % (name, "spin1" if comps == 3 else "scalar")
        counts[key] = counts.get(key, 0) + 1
    res = {"metric": "lattice-site-updates/s", "value": sites * inner * replays / (total_ms * 1e-3),
           "unit": "lattice-site-updates/s", "n_gpus": 1, "steps": replays, "warmup": max(1, warmup),
           "ms_per_step": total_ms / replays, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "ensemble of %d condensates (edge 24..80, BCC/FCC/A15/C15, scalar + spin-1), "
                                  "%d leapfrog steps in one persistent launch per CUDA-graph replay" % (len(members), inner),
                      "sites": sites, "members": counts, "dt": ENS["dt"],
                      "l2": "inputs larger than L2 (%.1f GB per state buffer set), no flush" % (state_bytes / 1e9)},
           "roofline": {"bound": "hbm", "achieved": algo / (step_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": algo / (step_ms * 1e-3) / 1e9 / peak, "peak_kind": kind, "kernel": "batch_kernel<float,3,true,%s>" % ("true" if layout else "false"),
                        "algorithmic_bytes_per_step": algo, "avg_step_ms": step_ms, "traffic": None},
           "gpu_launches": launches, "graph_replays": replays, "clocks": clk.summary(), "setup_s": setup_s,
           "autotune": tune,
           "norm_rel_change": [abs(b2["norm"] - a2["norm"]) / a2["norm"] for a2, b2 in zip(e_first, e_last)]}
    # end to end: each replay's graph copies the members' step state (ramp, time,
    # slot) from pinned host memory; after it every member's observables come back
    t0 = time.perf_counter()
    obs_all = [m.observe(m.current) for m in members]
    res["e2e"] = {"value": sites * inner * replays / (total_ms * 1e-3 + (time.perf_counter() - t0) * replays),
                  "unit": "lattice-site-updates/s", "h2d_bytes_per_step": len(members) * (C.sizeof(capi.Ramp) + 48),
                  "d2h_bytes_per_step": 96 * len(members),
                  "path": "gpe_batch_replay (graph: member state from pinned host memory, the interleaved members' "
                          "layout changes in, one persistent launch, layout changes out) + gpe_observe of every member",
                  "norm_min_max": [min(o["norm"] for o in obs_all), max(o["norm"] for o in obs_all)]}
    b.close()
    for s in members:
        s.close()
    return res


def config_dict():
    return {"workload": "spin-1 GPE, BCC 96^3 block cells (10,616,832 sites), leapfrog FP32 fused + observables "
                        "(FP32 node terms, FP64 sums) every 100 steps",
            "lattice": "bcc", "cells": list(DIMS), "components": 3, "dt": DT, "c0": C0, "c2": C2,
            "ramp": "Bz 0.5->-0.5 over 4000 steps, Bq 0.2", "inner_steps_per_step": INNER,
            "l2": "inputs larger than L2 (255 MB per psi buffer), no flush"}


# ------------------------------------------------------------------ clocks


class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------- CPU baseline


def cpu_baseline(seconds=10.0):
    """The FP64 CPU oracle (a restatement of Spin1GpeBCC.cu:793-917; the reference
    has no CPU spin-1 code) on the same workload, all host threads."""
    from oracle import oracle
    from spacetime_gb300 import capi

    lat, p, ramp, psi0 = workload(capi.FP64)
    p.precision = capi.FP64
    threads = os.cpu_count() or 1
    even = np.zeros_like(psi0)
    odd = psi0.copy()
    oracle.parabolic_step(lat, p, oracle.ramp_eval(ramp, 0.0), 0.0, oracle.EULER, even, odd, None, threads)
    sites = lat.nodes * DIMS[0] * DIMS[1] * DIMS[2]
    bufs = [even, odd]
    n = 0
    t0 = time.perf_counter()
    while True:
        t = (n + 1) * DT
        oracle.parabolic_step(lat, p, oracle.ramp_eval(ramp, t), t, oracle.LEAPFROG, bufs[(n + 1) % 2], bufs[n % 2], None, threads)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return {"value": sites * n / el, "unit": "lattice-site-updates/s", "cores": threads, "kind": "port",
            "sample": "%d leapfrog steps of the full 96^3 spin-1 BCC grid (FP64 oracle, OpenMP %d threads), %.1f s" % (n, threads, el)}


def _gpblocks_inputs(cells=32, g=2000.0, dt=1e-4):
    """Config 1 in the reference CPU stepper's own layout (GrossPitaevskii/
    GPBlocks.cpp:460-523): flat value arrays with the one-cell leading pad, the
    BCC index table, dt folded into lapfac, lapfac0, g and the potential
    V = |x|^2 / 2 (no offset) as integrateInTime does; the TF vortex + 1e-3 noise
    of the GPU leg as the even and odd states."""
    from spacetime_gb300 import capi, states

    w = LEGS["scalar-bcc32"]
    lat, p = leg_params(w, capi.FP64, (cells,) * 3)
    X = Y = Z = cells
    V = lat.nodes
    deg = int(lat.row_ptr[1] - lat.row_ptr[0])
    bsize, bxsize = V, (X + 1) * V
    bxysize = (Y + 1) * bxsize
    ii0 = bxysize + bxsize + bsize
    vsize = ii0 + (Z + 1) * bxysize
    st = lat.data["stencil"]
    lapind = np.array([e[2] * bxysize + e[1] * bxsize + e[0] * bsize + e[3] for e in st], dtype=np.int64)
    h = float(st[0][4])
    bs = p.block_scale
    dt_ref = 2 * dt  # one GPBlocks update advances by dt_ref / 2 (its odd buffer is shifted by -dt_ref / 2)
    lapfac = -0.5 * h / (bs * bs)
    lapfac0 = deg * (-lapfac)
    psi = states.vortex_state(lat, p, seed=w["seed"], noise=1e-3)  # (Z+2, Y+2, X+2, V, 1, 2)
    flat = np.zeros((vsize, 2))
    pot = np.zeros(vsize)
    r = states.node_positions(lat, p)  # (Z, Y, X, V, 3)
    for k in range(Z):
        for j in range(Y):
            base = ii0 + k * bxysize + j * bxsize
            flat[base:base + X * V] = psi[k + 1, j + 1, 1:X + 1, :, 0, :].reshape(-1, 2)
            pot[base:base + X * V] = 0.5 * np.sum(r[k, j] ** 2, axis=-1).ravel()
    return dict(X=X, Y=Y, Z=Z, V=V, deg=deg, lapind=lapind, lapfac=lapfac * dt_ref, lapfac0=lapfac0 * dt_ref,
                g=g * dt_ref, pot=pot * dt_ref, even=flat.ravel().copy(), odd=flat.ravel().copy())


def _gpblocks_worker(cells, steps, start_at):
    """One process of the whole-socket sample: set up its own copy of config 1,
    wait for the common start time, run `steps` GPBlocks steps (2 updates of every
    value each) and print (site-updates, start, end) as JSON."""
    from oracle import oracle

    d = _gpblocks_inputs(cells)
    while time.time() < start_at:
        time.sleep(0.01)
    t0 = time.time()
    oracle.gpblocks_run(d["X"], d["Y"], d["Z"], d["V"], d["deg"], d["lapind"], d["lapfac"], d["lapfac0"], d["g"], d["pot"],
                        d["even"], d["odd"], steps)
    t1 = time.time()
    print(json.dumps([d["X"] * d["Y"] * d["Z"] * d["V"] * 2 * steps, t0, t1]))


def cpu_gpblocks(seconds=5.0, cells=32):
    """Config 1 on the reference's CPU stepper (GPBlocks.cpp:560-606), in its
    bit-exact restatement orc_gpblocks_run (the reference's printed norms
    reproduced exactly, tests/test_oracle_golden.py): one core, then one copy per
    host core at once (separate processes) for the socket's aggregate."""
    from oracle import oracle

    d = _gpblocks_inputs(cells)
    sites = d["X"] * d["Y"] * d["Z"] * d["V"]
    oracle.gpblocks_run(d["X"], d["Y"], d["Z"], d["V"], d["deg"], d["lapind"], d["lapfac"], d["lapfac0"], d["g"], d["pot"],
                        d["even"], d["odd"], 2)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        oracle.gpblocks_run(d["X"], d["Y"], d["Z"], d["V"], d["deg"], d["lapind"], d["lapfac"], d["lapfac0"], d["g"],
                            d["pot"], d["even"], d["odd"], 5)
        n += 5
    el = time.perf_counter() - t0
    one = sites * 2 * n / el
    res = {"value": one, "unit": "lattice-site-updates/s", "cores": 1, "kind": "port",
           "sample": "%d GPBlocks steps (2 updates of every value each) of config 1 (%d^3 BCC cells), one thread, "
                     "%.1f s; orc_gpblocks_run restates integrateInTime's loop and reproduces the reference's printed "
                     "norms bit for bit" % (n, cells, el)}
    cores = os.cpu_count() or 1
    per = max(2, int(seconds * one / (2 * sites)))
    start_at = time.time() + 8.0
    code = "import bench; bench._gpblocks_worker(%d, %d, %r)" % (cells, per, start_at)
    procs = [subprocess.Popen([sys.executable, "-c", code], cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                              text=True) for _ in range(cores)]
    rows = []
    try:
        for pr in procs:
            out, _ = pr.communicate(timeout=8.0 + 20 * seconds + 60)
            if pr.returncode == 0 and out.strip():
                rows.append(json.loads(out.strip().splitlines()[-1]))
    except subprocess.TimeoutExpired:
        for pr in procs:
            pr.kill()
    if len(rows) == cores:
        wall = max(r[2] for r in rows) - min(r[1] for r in rows)
        res["all_cores"] = {"value": sum(r[0] for r in rows) / wall, "cores": cores,
                            "sample": "%d processes x %d steps at once, %.1f s from the first start to the last end "
                                      "(set-up excluded)" % (cores, per, wall)}
    else:
        res["all_cores"] = {"unavailable": "%d of %d worker processes reported" % (len(rows), cores)}
    return res


def cpu_oracle_leg(w, dims, seconds=5.0):
    """A leg's step on the FP64 oracle (all host threads), a bounded sample of the
    same workload at `dims`."""
    from oracle import oracle
    from spacetime_gb300 import capi, states

    lat, p = leg_params(w, capi.FP64, dims)
    threads = os.cpu_count() or 1
    sites = lat.nodes * int(np.prod(dims))
    if w["C"] == 1:
        psi = states.vortex_state(lat, p, seed=w["seed"], noise=1e-3, kappa=w["kappa"])
    else:
        psi = states.spinor_state(lat, p, w["zeta"], seed=w["seed"], noise=1e-3)
    f = capi.make_fields()
    n = 0
    if w["scheme"] == 0:
        bufs = [psi.copy(), psi.copy()]
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            oracle.parabolic_step(lat, p, f, 0.0, oracle.LEAPFROG, bufs[(n + 1) % 2], bufs[n % 2], None, threads)
            n += 1
        what = "FP64 oracle leapfrog (orc_parabolic_step)"
    else:
        qshape = capi.buffer_shape(lat, p, True)
        ps, qs = [psi.copy(), psi.copy()], [np.zeros(qshape), np.zeros(qshape)]
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            oracle.hyper_run(lat, p, ps[n % 2], ps[(n + 1) % 2], qs[n % 2], qs[(n + 1) % 2], 1, fields=f, threads=threads)
            n += 1
        what = "FP64 oracle hyperbolic psi + q step (orc_q_psi_step + orc_q_step)"
    el = time.perf_counter() - t0
    return {"value": sites * n / el, "unit": "lattice-site-updates/s", "cores": threads, "kind": "port",
            "sample": "%d steps of %s on %s %s, %d threads, %.1f s" % (n, what, w["lattice"], "x".join(map(str, dims)),
                                                                     threads, el)}


def cpu_adjoint(seconds=5.0):
    """Config 4 on the host: the CPU has no adjoint, so its gradient is central
    differences, two forward runs per knot.  The FP64 oracle's leapfrog step on the
    64^3 spin-1 workload is timed (all host threads) and the gradient rate derived
    as 1 / (2 x 32 knots x 2000 steps x the step time)."""
    from oracle import oracle
    from spacetime_gb300 import capi, states

    lat = capi.Lattice("bcc")
    dims = ADJ["dims"]
    bs = BOX / (dims[0] * lat.block_width[0])
    p = capi.make_params(components=3, precision=capi.FP64, dims=dims, block_scale=bs, dt=DT, trap_offset=100.0, c0=C0,
                         c2=C2, lattice=lat)
    psi = states.spinor_state(lat, p, states.POLAR, seed=2, noise=1e-3)
    bufs = [psi.copy(), psi.copy()]
    threads = os.cpu_count() or 1
    f = capi.make_fields(bq=0.2, bb=(0, 0, 0.5))
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        oracle.parabolic_step(lat, p, f, 0.0, oracle.LEAPFROG, bufs[(n + 1) % 2], bufs[n % 2], None, threads)
        n += 1
    t_step = (time.perf_counter() - t0) / n
    runs = 2 * 2 * ADJ["knots"]
    return {"value": 1.0 / (runs * ADJ["steps"] * t_step), "unit": "gradients/s", "cores": threads, "kind": "port",
            "sample": "%d FP64 oracle leapfrog steps of the 64^3 spin-1 grid, %d threads, %.3f s per step; a gradient "
                      "by central differences takes %d forward runs of %d steps" % (n, threads, t_step, runs, ADJ["steps"])}


def cpu_ensemble(seconds=5.0, count=4):
    """Config 5 on the host: the FP64 oracle's leapfrog on the first `count`
    members of the ensemble, each for an equal share of `seconds` (all host
    threads); site-updates per second over the sample."""
    from oracle import oracle
    from spacetime_gb300 import capi, states

    threads = os.cpu_count() or 1
    done, el = 0, 0.0
    names = []
    for i, (name, comps, n, omega, ramp) in enumerate(ensemble_members(count)):
        lat = capi.Lattice(name)
        bs = BOX / (n * lat.block_width[0])
        p = capi.make_params(components=comps, precision=capi.FP64, dims=(n, n, n), block_scale=bs, dt=ENS["dt"],
                             trap_offset=100.0, trap_lambda=omega, c0=C0, c2=C2 if comps == 3 else 0.0, lattice=lat)
        psi = states.spinor_state(lat, p, states.POLAR if comps == 3 else (1.0,), seed=1000 + i, noise=1e-3)
        bufs = [psi.copy(), psi.copy()]
        f = oracle.ramp_eval(ramp, 0.0)
        k, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < seconds / count:
            oracle.parabolic_step(lat, p, f, 0.0, oracle.LEAPFROG, bufs[(k + 1) % 2], bufs[k % 2], None, threads)
            k += 1
        el += time.perf_counter() - t0
        done += lat.nodes * n ** 3 * k
        names.append("%s/%s/%d^3" % (name, "spin1" if comps == 3 else "scalar", n))
    return {"value": done / el, "unit": "lattice-site-updates/s", "cores": threads, "kind": "port",
            "sample": "FP64 oracle leapfrog on members %s, %.1f s, %d threads" % (", ".join(names), el, threads)}


LEG_NAMES = ("scalar-bcc32", "spin2-c15", "adjoint-bcc64", "ensemble-256")


def run_legs(args):
    """The benchmark plan's other configurations, each with its own value,
    roofline, end-to-end number, CPU baseline and precision record:
      scalar-bcc32   config 1: scalar BCC 32^3, g = 2000, no trap offset, 1000 steps
                     per bench step; the reference CPU stepper (GPBlocks) as baseline
      spin2-c15      config 3: relativistic spin-2 C15 128^3; FP32 against FP64 over
                     10^4 steps at a smaller grid
      adjoint-bcc64  config 4: ramp-control gradients by the adjoint kernel
      ensemble-256   config 5: 256 uneven condensates, 2000 steps in one persistent
                     launch"""
    import torch

    sel = LEG_NAMES if args.legs == "all" else tuple(x for x in args.legs.split(",") if x)
    out = {}
    for name in sel:
        t0 = time.perf_counter()
        try:
            if name == "scalar-bcc32":
                w = LEGS["scalar-bcc32"]
                r = time_leg(w, steps=10, inner=100, warmup=3)
                r["config"] = {"workload": "scalar GPE, BCC 32^3 block cells, box [-8,8]^3, trap (1,1,1) without offset, "
                                           "g = 2000, TF vortex + 1e-3 noise, dt = 1e-4; 100 steps per bench step",
                               "l2": "L2-resident (3.8 MB per FP32 buffer): the fraction is of the HBM peak"}
                r["e2e"] = leg_e2e(w, steps=5, inner=1000)
                r["cpu_baseline"] = cpu_gpblocks(args.cpu_seconds / 2)
                r["drift"] = scalar_reference_drift()
            elif name == "spin2-c15":
                w = LEGS["spin2-c15-128"]
                r = time_leg(w, steps=2, inner=100, warmup=1)
                cells = args.c15_drift_cells
                r["config"] = {"workload": "relativistic spin-2 GPE (hyperbolic psi + q), C15 128^3 block cells "
                                           "(285,212,672 sites), c0 = 2000, c2 = -20, c4 = 40, cyclic + 1e-3 noise, "
                                           "sigma = 0.00225, dt = 2e-5; 100 steps per bench step (one call: the "
                                           "layout changes in and out of the interleaved kernel's call included)",
                               "l2": "inputs larger than L2 (68.5 GB of FP32 psi + q), no flush"}
                r["e2e"] = leg_e2e(w, steps=3, inner=100, dims=(48, 48, 48), flight=3)
                r["e2e_serial"] = leg_e2e(w, steps=3, inner=100, dims=(48, 48, 48))
                r["drift"] = leg_drift(w, None, args.c15_drift_steps, dims=(cells,) * 3)
                r["drift"]["note"] = ("no reference program runs spin-2 on C15; the FP64 run is libgpe's FP64 hyperbolic "
                                      "stepper, pinned to the reference's RelativisticSpin2Gpe kernels on BCC by golden vectors")
                r["cpu_baseline"] = cpu_oracle_leg(w, (24, 24, 24), args.cpu_seconds / 2)
            elif name == "adjoint-bcc64":
                r = adjoint_result(2, ADJ["steps"], ADJ["fd_knots"])
                r["cpu_baseline"] = cpu_adjoint(args.cpu_seconds / 2)
            elif name == "ensemble-256":
                r = ensemble_result(ENS["members"], ENS["steps"], 1, 1)
                r["cpu_baseline"] = cpu_ensemble(args.cpu_seconds / 2)
            else:
                r = {"error": "unknown leg"}
        except Exception as e:  # a failing leg is reported, the others still run
            r = {"error": "%s: %s" % (type(e).__name__, str(e)[:300])}
        r["wall_s"] = time.perf_counter() - t0
        out[name] = r
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


def scalar_reference_drift():
    """Config 1 in FP32 against an FP64 run of the reference's own scalar BCC
    kernel (GPUGrossPitaevskii_BCC.cu:327-347, compiled unmodified for sm_103a),
    1000 steps, observables every 100 (the checker of oracle/ref_cuda_drift.py)."""
    from oracle import ref_cuda, ref_cuda_drift

    if not ref_cuda.available("scalar_bcc"):
        return {"unavailable": "reference cubins not built (oracle/build_ref_cuda.sh needs the reference tree)"}
    d = ref_cuda_drift.run_scalar(32, 1000, 100, trap_offset=0.0)
    d["against"] = "the reference's FP64 scalar BCC update kernel"
    return d


def fp64_reference_timing(stream, launches=50):
    """The reference's own FP64 spin-1 leapfrog kernel (Spin1GpeBCC.cu:793-917,
    compiled unmodified for sm_103a by oracle/build_ref_cuda.sh, launched with its
    own launch shape Spin1GpeBCC.cu:1375-1380) on the headline grid, timed with CUDA
    events: the FP64 plain GPU stepper of the benchmark plan."""
    import ctypes as C

    import torch

    from oracle import ref_cuda as R
    from spacetime_gb300 import capi, states
    from spacetime_gb300.stepper import Stepper

    if not R.available("spin1_bcc"):
        return {"unavailable": "reference cubins not built (oracle/build_ref_cuda.sh needs the reference tree)"}
    lat = capi.Lattice("bcc")
    bs = BOX / (DIMS[0] * lat.block_width[0])
    p64 = capi.make_params(components=3, precision=capi.FP64, dims=DIMS, block_scale=bs, dt=DT,
                           trap_lambda=(1.0, 1.0, R.LAMBDA_Z), trap_offset=R.TRAP_OFFSET, c0=C0, c2=C2, lattice=lat)
    ref = Stepper(lat, p64)
    drv = R.Driver()
    try:
        psi0 = states.spinor_state(lat, p64, states.POLAR, seed=2, noise=1e-3)
        ref.upload(capi.PSI_ODD, psi0)
        ref.upload(capi.PSI_EVEN, psi0)
        ent, w = R.stencil_int4(lat)
        d_ent, d_w = drv.upload(ent), drv.upload(w)
        grid, block = R.spinor_grid(p64, lat.nodes)
        leap = drv.function("spin1_bcc", "leapfrog")
        slots = [R.pitched(ref, capi.PSI_EVEN), R.pitched(ref, capi.PSI_ODD)]
        f = capi.make_fields(bq=0.2, bb=(0.0, 0.0, 0.5))

        def step(k):
            drv.launch(leap, grid, block, [slots[(k + 1) % 2], slots[k % 2], C.c_void_p(d_ent), C.c_void_p(d_w),
                                           R.mag_fields(f), R.uint3(p64), C.c_double(bs), R.double3(p64.p0),
                                           C.c_double(C0), C.c_double(C2), C.c_double(0.0), C.c_bool(False),
                                           C.c_bool(False), C.c_bool(False), C.c_double(DT), C.c_double((k + 1) * DT)])

        for k in range(5):
            step(k)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()  # the driver API launches go to the legacy default stream
        for k in range(launches):
            step(k)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / launches
    finally:
        drv.close()
        ref.close()
    sites = lat.nodes * DIMS[0] * DIMS[1] * DIMS[2]
    return {"value": sites / (ms * 1e-3), "unit": "lattice-site-updates/s", "ms_per_launch": ms,
            "kernel": "Spin1GpeBCC.cu leapfrog, FP64, compiled unmodified for sm_103a",
            "launch": {"grid": list(grid), "block": list(block)}, "launches_timed": launches,
            "trap": "the program's compiled-in lambda (1, 1, %.6f) + %g" % (R.LAMBDA_Z, R.TRAP_OFFSET)}


def run_reference(args):
    """--impl reference: the CPU implementation of the path (the reference has no
    CPU code for spin-1, so its FP64 restatement, oracle/gpe_oracle.c) on the box's
    host cores, bounded samples of the same workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle
    from spacetime_gb300 import capi

    lat, p, ramp, psi0 = workload(capi.FP64)
    threads = os.cpu_count() or 1
    sites = lat.nodes * DIMS[0] * DIMS[1] * DIMS[2]
    even = np.zeros_like(psi0)
    odd = psi0.copy()
    oracle.parabolic_step(lat, p, oracle.ramp_eval(ramp, 0.0), 0.0, oracle.EULER, even, odd, None, threads)
    bufs = [even, odd]
    per_step = 2  # leapfrog steps per bench step (bounded sample)
    n = 0

    def one():
        nonlocal n
        for _ in range(per_step):
            t = (n + 1) * DT
            oracle.parabolic_step(lat, p, oracle.ramp_eval(ramp, t), t, oracle.LEAPFROG, bufs[(n + 1) % 2], bufs[n % 2], None, threads)
            n += 1

    for _ in range(args.warmup):
        one()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one()
    el = time.perf_counter() - t0
    value = sites * per_step * args.steps / el
    line = {"metric": "lattice-site-updates/s", "value": value, "unit": "lattice-site-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": dict(config_dict(), workload="spin-1 GPE, BCC 96^3 block cells, FP64 CPU leapfrog (2 steps per bench step)"),
            "cpu_baseline": {"value": value, "unit": "lattice-site-updates/s", "cores": threads, "kind": "port",
                             "sample": "%d bench steps x %d leapfrog steps of the full grid" % (args.steps, per_step)},
            "e2e": {"value": value, "unit": "lattice-site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU arm


def traffic_from_profile(kernel):
    """DRAM bytes per launch from the committed ncu capture, if it is of `kernel`."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        try:
            with open(path) as f:
                d = json.load(f)
            return d.get("bytes_per_launch") if d.get("kernel") == kernel else None
        except Exception:
            return None
    return None


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def replica_throughput(local_ms, units_per_rank, world, device="cpu"):
    """Replicas (one independent condensate per rank, no data-path collective):
    the job's time is the slowest rank's, and the job processed world x the units
    of one rank.  Returns (max over ranks of local_ms, units per second)."""
    import torch

    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    return ms, world * units_per_rank / (ms * 1e-3)


def run_gpu(args):
    import ctypes as C

    import torch
    import torch.distributed as dist

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    lat, p, ramp, psi0 = workload(capi.FP32)
    stream = torch.cuda.Stream()
    s = Stepper(lat, p)
    s.stream = C.c_void_p(stream.cuda_stream)
    sites = s.sites
    # per-step observables: FP32 node terms, FP64 sums (the FP64-arithmetic form is
    # kept for the drift check below and on request)
    s.set_tuning(capi.TUNE_OBSERVE_ARITH, 0 if args.observe_fp64 else 1)

    def cur_slot():
        return s.current

    s._nsteps = 0

    def advance():
        s.step(INNER)
        s._nsteps += INNER

    def advance_observed():
        """One bench step: INNER leapfrog steps in one gpe_step_observe call, the
        observables summed inside the last one (FP32 node terms, FP64 sums); with
        --observe-fp64 gpe_step(INNER) and a separate observe pass with FP64 node
        terms after it."""
        if args.observe_fp64:
            advance()
            return s.observe(cur_slot(), s._nsteps * DT)
        s._nsteps += INNER
        return s.step_observe(INNER)

    kernel_name = {capi.KERNEL_TILE: "leapfrog_tile_kernel<float,3>", capi.KERNEL_GATHER: "parabolic_fixed_kernel<float,3,LEAPFROG,4>",
                   capi.KERNEL_MARCH: "leapfrog_march_kernel<float,3>", capi.KERNEL_ROWS: "leapfrog_rows_kernel<float,3>",
                   capi.KERNEL_SLAB: "parabolic_slab_kernel<float,3,4>", capi.KERNEL_INTERLEAVED: "il_step_kernel<3,4,32>"}
    if args.kernel:
        s.set_tuning(capi.TUNE_KERNEL, args.kernel)
    for key, val in ((capi.TUNE_TILE_CELLS, args.tile), (capi.TUNE_TILE_ROWS, args.rows), (capi.TUNE_ZCHUNK, args.zchunk),
                     (capi.TUNE_THREADS, args.threads), (capi.TUNE_CARVEOUT, args.carveout)):
        if val:
            s.set_tuning(key, val)
    tuning_report = None
    if args.autotune:
        with torch.cuda.stream(stream):
            tuning_report = s.autotune(steps=10)
    chosen = s.get_tuning(capi.TUNE_KERNEL)
    tile = [s.get_tuning(capi.TUNE_TILE_CELLS), s.get_tuning(capi.TUNE_TILE_ROWS), s.get_tuning(capi.TUNE_ZCHUNK)]
    with torch.cuda.stream(stream):
        s.upload(capi.PSI_ODD, psi0)
        s.set_ramp(ramp, 0.0)
        s.start()
        for _ in range(args.warmup):
            advance_observed()
        barrier()
        launches0 = s.launches
        ev_start, ev_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        obs = []
        # the library's CUDA events on this stream time each call's plain step
        # launches, its observed step and its layout changes (gpe_get_step_timing)
        s.set_tuning(capi.TUNE_TIMING, 1)
        s.step_timing(reset=True)
        with ClockSampler(local) as clk:
            ev_start.record(stream)
            for k in range(args.steps):
                obs.append(advance_observed())
            ev_end.record(stream)
            barrier()
        timing = s.step_timing(reset=True)
        s.set_tuning(capi.TUNE_TIMING, 0)
        clocks = clk.summary()
        launches = s.launches - launches0
        total_ms = ev_start.elapsed_time(ev_end)
    total_ms, value = replica_throughput(total_ms, sites * INNER * args.steps, world, "cuda")
    # the step kernel's mean duration over the plain launches (INNER - 1 per bench
    # step; the observed step, with its finalize, and the layout changes are timed
    # on their own)
    plain_launches = int(timing["step_launches"])
    launch_ms = timing["step_ms"] / plain_launches
    observed_ms = timing["observed_ms"] / timing["observed_launches"] if timing["observed_launches"] else None
    if timing["interleaved_calls"]:
        chosen = capi.KERNEL_INTERLEAVED
    algo_bytes = BYTES_PER_SITE_FP32 * sites
    achieved = algo_bytes / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = traffic_from_profile(kernel_name[chosen])

    # ---- end to end through the C ABI with host buffers, every step: the FP64 host
    # state (reference file layout, pinned) in, start + 100 leapfrog steps with the
    # observables summed in the last one, and the final FP64 state back out into a
    # pinned host array (what a caller of the reference's time loop writes out at
    # every save, Spin1GpeBCC.cu:1688-1692).
    host = torch.from_numpy(psi0.ravel()).pin_memory()
    host_np = host.numpy().reshape(psi0.shape)
    out_host = torch.empty(psi0.size, dtype=torch.float64).pin_memory()
    out_np = out_host.numpy().reshape(psi0.shape)
    e2e_steps = max(3, min(args.steps, 10))

    def e2e_step():
        s.upload(capi.PSI_ODD, host_np)
        s.set_ramp(ramp, 0.0)
        s.start()
        s._nsteps = 0
        o = advance_observed()
        s.download(cur_slot(), out=out_np)
        return o

    with torch.cuda.stream(stream):
        for _ in range(2):
            e2e_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_obs = e2e_step()
        barrier()
        e2e_s = time.perf_counter() - t0
    e2e_value = world * sites * INNER * e2e_steps / e2e_s
    e2e_pipe = e2e_pipelined(lat, p, ramp, psi0, e2e_steps, args.observe_fp64, args.e2e_flight)

    # ---- FP64 plain stepper on the same workload (the "FP64 plain GPU stepper")
    lat64, p64, _, _ = workload(capi.FP64)
    s64 = Stepper(lat64, p64)
    s64.stream = C.c_void_p(stream.cuda_stream)
    with torch.cuda.stream(stream):
        s64.upload(capi.PSI_ODD, psi0)
        s64.set_ramp(ramp, 0.0)
        s64.start()
        s64.step(20)
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s64.step(200)
        b.record(stream)
        barrier()
        fp64_ms = a.elapsed_time(b) / 200
    s64.close()
    fp64_value = sites / (fp64_ms * 1e-3)

    # ---- the reference's own FP64 spin-1 leapfrog kernel on the same grid
    fp64_ref = fp64_reference_timing(stream) if rank == 0 and args.fp64_reference else None
    if fp64_ref and "value" in fp64_ref:
        fp64_ref["speedup_fp32_fused"] = (value / world) / fp64_ref["value"]

    # ---- precision: FP32 fused against an FP64 run of the reference's own kernels
    # (libgpe's FP64 stepper where the reference's cubins are not built)
    drift = None
    if args.drift_steps > 0 and rank == 0:
        drift = reference_drift(args.drift_steps)
        if drift is None:
            drift = measure_drift(args.drift_steps, stream)
            drift["against"] = "libgpe FP64 (plain) stepper"

    result = {
        "metric": "lattice-site-updates/s", "value": value, "unit": "lattice-site-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(),
        "parallelism": "replicas" if world > 1 else "single",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": kernel_name[chosen], "tile_cells_rows_zchunk": tile, "algorithmic_bytes_per_launch": algo_bytes,
                     "avg_launch_ms": launch_ms, "launches_timed": plain_launches},
        "observed_step_ms": observed_ms,
        "layout_change_ms_per_call": timing["convert_ms"] / timing["calls"] if timing["interleaved_calls"] else None,
        "step_timing": timing,
        "e2e": dict(e2e_pipe, value=world * e2e_pipe["value"]),
        "e2e_serial": {"value": e2e_value, "unit": "lattice-site-updates/s", "h2d_bytes_per_step": int(psi0.nbytes),
                       "d2h_bytes_per_step": int(psi0.nbytes) + 8 * 12, "steps": e2e_steps,
                       "path": "one condensate, one host thread: gpe_upload (FP64 host, pinned) + gpe_start + "
                               "gpe_step_observe(100) + gpe_download (FP64 host, pinned), each step after the last",
                       "norm_last": e2e_obs["norm"]},
        "observables": "FP64 node terms and sums (separate pass)" if args.observe_fp64 else
                       "summed inside the last step kernel of each bench step (FP32 node terms, FP64 sums)",
        "fp64_plain": {"value": fp64_value, "unit": "lattice-site-updates/s", "ms_per_launch": fp64_ms,
                       "speedup_fp32_fused": (value / world) / fp64_value},
        "gpu_launches": launches,
        "autotune": tuning_report,
        "clocks": clocks,
        "observables_last": obs[-1] if obs else None,
    }
    if fp64_ref is not None:
        result["fp64_reference"] = fp64_ref
    if drift is not None:
        result["drift"] = drift
    if rank == 0 and args.cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    s.close()
    if rank == 0 and args.legs != "none":
        result["legs"] = run_legs(args)
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()
    return 0


def e2e_pipelined(lat, p, ramp, psi0, steps, observe_fp64=False, flight=3):
    """End to end through the C ABI with host buffers, `flight` condensates of the
    workload in flight: each has its own handle, stream, pinned host arrays and host
    thread, and every one of its bench steps uploads its FP64 host state, starts,
    takes 100 steps with the observables summed in the last one and downloads the
    final FP64 state (gpe_upload / gpe_download by DMA through the staging buffer,
    GPE_TUNE_TRANSFER 1, so that one condensate's copies run while the other's
    kernels do).  Wall time from the threads' start to the last one's end; the
    value counts the steps of all."""
    import ctypes as C
    import threading

    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    runs = []
    for _ in range(flight):
        st = torch.cuda.Stream()
        s = Stepper(lat, p)
        s.stream = C.c_void_p(st.cuda_stream)
        s.set_tuning(capi.TUNE_OBSERVE_ARITH, 0 if observe_fp64 else 1)
        s.set_tuning(capi.TUNE_TRANSFER, 1)
        host = torch.from_numpy(psi0.ravel().copy()).pin_memory().numpy().reshape(psi0.shape)
        out = torch.empty(psi0.size, dtype=torch.float64).pin_memory().numpy().reshape(psi0.shape)
        runs.append({"s": s, "stream": st, "in": host, "out": out, "obs": None, "err": None})

    def work(r, n):
        try:
            s = r["s"]
            for _ in range(n):
                s.upload(capi.PSI_ODD, r["in"])
                s.set_ramp(ramp, 0.0)
                s.start()
                r["obs"] = s.step_observe(INNER)
                s.download(s.current, out=r["out"])
        except Exception as e:  # reported in the line
            r["err"] = "%s: %s" % (type(e).__name__, e)

    def both(n):
        ths = [threading.Thread(target=work, args=(r, n)) for r in runs]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    both(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    both(steps)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    sites = runs[0]["s"].sites
    res = {"value": flight * sites * INNER * steps / el, "unit": "lattice-site-updates/s",
           "h2d_bytes_per_step": int(psi0.nbytes), "d2h_bytes_per_step": int(psi0.nbytes) + 8 * 12,
           "steps": flight * steps, "condensates_in_flight": flight,
           "path": "%d condensates, one host thread and stream each, every bench step: gpe_upload (FP64 host, pinned, "
                   "DMA through the staging buffer) + gpe_start + gpe_step_observe(100) + gpe_download (FP64 host, "
                   "pinned, DMA)" % flight,
           "norm_last": [r["obs"]["norm"] if r["obs"] else None for r in runs]}
    errs = [r["err"] for r in runs if r["err"]]
    if errs:
        res["error"] = errs[0]
    for r in runs:
        r["s"].close()
    return res


def reference_drift(nsteps):
    """The headline workload in FP32 against an FP64 run of the reference's own
    forwardEuler + leapfrog (Spin1GpeBCC.cu:667-917, compiled unmodified), from the
    same state, with the trap the program compiles in: energy and norm every 100
    steps, the max-abs wavefunction error at the end (the checker of
    oracle/ref_cuda_drift.py).  None where the reference's cubins are not built."""
    from oracle import ref_cuda, ref_cuda_drift

    if not ref_cuda.available("spin1_bcc"):
        return None
    d = ref_cuda_drift.run(DIMS[0], nsteps, 100, DT, BOX)
    d["against"] = "the reference's FP64 spin-1 forwardEuler + leapfrog kernels"
    return d


def measure_drift(nsteps, stream):
    """FP32 fused vs FP64 plain from the same initial state: relative energy
    difference every 100 steps and the max-abs psi error at the end."""
    import ctypes as C

    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    out = {"steps": nsteps, "energy_rel_diff_max": 0.0, "norm_rel_diff_max": 0.0}
    runs = {}
    for prec in (capi.FP32, capi.FP64):
        lat, p, ramp, psi0 = workload(prec)
        st = Stepper(lat, p)
        st.stream = C.c_void_p(stream.cuda_stream)
        with torch.cuda.stream(stream):
            st.upload(capi.PSI_ODD, psi0)
            st.set_ramp(ramp, 0.0)
            st.start()
            e = [st.observe(capi.PSI_EVEN, 0.0)]
            done = 0
            while done < nsteps:
                st.step(100)
                done += 100
                e.append(st.observe(capi.PSI_EVEN if done % 2 == 0 else capi.PSI_ODD, done * DT))
            last = st.download(capi.PSI_EVEN if done % 2 == 0 else capi.PSI_ODD)
        st.close()
        runs[prec] = (e, last)
    e32, l32 = runs[capi.FP32]
    e64, l64 = runs[capi.FP64]
    out["energy_rel_diff_max"] = max(abs(a["energy"] - b["energy"]) / abs(b["energy"]) for a, b in zip(e32, e64))
    out["norm_rel_diff_max"] = max(abs(a["norm"] - b["norm"]) / abs(b["norm"]) for a, b in zip(e32, e64))
    out["energy_rel_drift_fp64"] = abs(e64[-1]["energy"] - e64[0]["energy"]) / abs(e64[0]["energy"])
    out["psi_max_abs_err"] = float(np.max(np.abs(l32 - l64)))
    out["psi_max_abs"] = float(np.max(np.abs(l64)))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--drift-steps", type=int, default=10000)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--kernel", type=int, default=0, help="0 auto, 1 gather, 2 row tile, 3 z-march, 4 multi-row tile, 5 slab ring")
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--rows", type=int, default=0)
    ap.add_argument("--zchunk", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--carveout", type=int, default=0, help="shared-memory carveout percent for the row-tile kernel")
    ap.add_argument("--autotune", action="store_true", help="run gpe_autotune before timing")
    ap.add_argument("--workload", default="spin1-bcc96", choices=["spin1-bcc96", "adjoint-bcc64", "ensemble-256"] + sorted(LEGS))
    ap.add_argument("--inner", type=int, default=0, help="leapfrog steps per bench step for --workload legs")
    ap.add_argument("--observe-fp64", action="store_true", help="FP64 arithmetic for the per-step observables")
    ap.add_argument("--leg-drift", action="store_true",
                    help="--workload legs: FP32 vs FP64 observables over --drift-steps steps (every 100)")
    ap.add_argument("--adjoint-steps", type=int, default=ADJ["steps"], help="adjoint-bcc64: steps of the recorded run")
    ap.add_argument("--fd-knots", type=int, default=ADJ["fd_knots"], help="adjoint-bcc64: knots checked by central differences")
    ap.add_argument("--members", type=int, default=ENS["members"], help="ensemble-256: members of the ensemble (a prefix)")
    ap.add_argument("--batch-layout", type=int, default=1, choices=[0, 1],
                    help="ensemble-256: 1 spinor members in the interleaved layout, 0 every member in its handle's")
    ap.add_argument("--legs", default="all",
                    help="default run: the other configurations to add to the line (all, none, or a comma list of %s)"
                    % ",".join(LEG_NAMES))
    ap.add_argument("--c15-drift-cells", type=int, default=32, help="spin2-c15 leg: grid edge of the 10^4-step FP32/FP64 run")
    ap.add_argument("--c15-drift-steps", type=int, default=10000, help="spin2-c15 leg: steps of the FP32/FP64 run")
    ap.add_argument("--no-fp64-reference", dest="fp64_reference", action="store_false",
                    help="skip timing the reference's FP64 kernel")
    ap.add_argument("--e2e-flight", type=int, default=3, help="condensates in flight in the end-to-end measurement")
    ap.add_argument("--quick", action="store_true",
                    help="headline only: no drift, CPU baseline or FP64 timings, and no legs unless --legs names some")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.quick:
        args.drift_steps, args.cpu_baseline, args.fp64_reference = 0, False, False
        if args.legs == "all":
            args.legs = "none"
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "adjoint-bcc64":
        return run_adjoint(args)
    if args.workload == "ensemble-256":
        return run_ensemble(args)
    if args.workload != "spin1-bcc96":
        return run_leg(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
