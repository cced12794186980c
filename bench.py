"""Benchmark: lattice site-updates/s of the fused FP32 stepper on one GB300.

Workload (the headline spin-1 configuration): spin-1 GPE on a BCC mesh of
96^3 block cells (10,616,832 dual nodes), box [-8, 8]^3, c0 = 2000, c2 = -50,
seeded polar state (0, 1, 0) with 1e-3 relative noise, linear Zeeman ramp
Bz 0.5 -> -0.5 over 4000 steps plus quadrupole gradient Bq = 0.2, dt = 5e-5.
Each psi buffer is 255 MB (FP32), larger than the 129 MB L2, so no L2 flush is
needed between iterations.

One bench "step" = 100 leapfrog steps (one fused kernel each) + one observables
pass (norm, energy, magnetisation; FP32 node terms, FP64 sums).  value = sites *
100 * K / time.

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
                         sigma=0.0, zeta=(1.0,), kappa=1, noise_abs=1e-3, noise_rel=0.0, bytes_fp32=24, seed=1),
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


def run_leg(args):
    """An optional configuration: device-side initial state, start, `steps` x 100
    steps timed with CUDA events, FP64 observables per bench step."""
    import ctypes as C

    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    w = LEGS[args.workload]
    lat = capi.Lattice(w["lattice"])
    bs = BOX / (w["dims"][0] * lat.block_width[0])
    p = capi.make_params(components=w["C"], scheme=w["scheme"], precision=capi.FP32, dims=w["dims"], block_scale=bs,
                         dt=w["dt"], trap_offset=100.0, c0=w["c0"], c2=w["c2"], c4=w["c4"], sigma=w["sigma"], lattice=lat)
    stream = torch.cuda.Stream()
    s = Stepper(lat, p)
    s.stream = C.c_void_p(stream.cuda_stream)
    if args.kernel:
        s.set_tuning(capi.TUNE_KERNEL, args.kernel)
    inner = args.inner or INNER
    with torch.cuda.stream(stream):
        s.init_state(s.current, capi.make_init(zeta=w["zeta"], kappa=w["kappa"], noise_abs=w["noise_abs"],
                                               noise_rel=w["noise_rel"], seed=w["seed"]))
        s.start()
        e0 = s.observe(s.current, 0.0)
        for _ in range(args.warmup):
            s.step(inner)
        torch.cuda.synchronize()
        n0 = s.launches
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        obs = []
        with ClockSampler(0) as clk:
            a.record(stream)
            step_ms = 0.0
            for _ in range(args.steps):
                x, y = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                x.record(stream)
                s.step(inner)
                y.record(stream)
                obs.append(s.observe(s.current))
                step_ms += x.elapsed_time(y)
            b.record(stream)
            torch.cuda.synchronize()
        total_ms = a.elapsed_time(b)
        launches = s.launches - n0
    sites = s.sites
    gather = s.get_tuning(capi.TUNE_KERNEL) == capi.KERNEL_GATHER
    s.close()
    drift = leg_drift(w, lat, args.drift_steps) if args.leg_drift else None
    launch_ms = step_ms / (inner * args.steps)
    algo = w["bytes_fp32"] * sites
    peak, kind = measured_peak()
    name = KERNEL_OF_SCHEME[w["scheme"]] % w["C"]
    if w["scheme"] == 1 and gather:
        name = "hyper_step_kernel<float,%d> (gather form)" % w["C"]
    res = {"metric": "lattice-site-updates/s", "value": sites * inner * args.steps / (total_ms * 1e-3),
           "unit": "lattice-site-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic", "config": dict(w, workload=args.workload, sites=sites, inner_steps_per_step=inner),
           "roofline": {"bound": "hbm", "achieved": algo / (launch_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": algo / (launch_ms * 1e-3) / 1e9 / peak, "peak_kind": kind, "kernel": name,
                        "algorithmic_bytes_per_launch": algo, "avg_launch_ms": launch_ms, "traffic": None},
           "gpu_launches": launches, "clocks": clk.summary(),
           "energy_rel_drift": abs(obs[-1]["energy"] - e0["energy"]) / abs(e0["energy"]) if obs else None,
           "norm_last": obs[-1]["norm"] if obs else None}
    if drift is not None:
        res["drift"] = drift
    print(json.dumps(res))
    return 0


def leg_drift(w, lat, nsteps, every=100):
    """FP32 against FP64 on the leg's workload from the same seeded device state:
    observables (FP64 arithmetic) every `every` steps."""
    import torch

    from spacetime_gb300 import capi
    from spacetime_gb300.stepper import Stepper

    bs = BOX / (w["dims"][0] * lat.block_width[0])
    runs = {}
    for prec in (capi.FP32, capi.FP64):
        p = capi.make_params(components=w["C"], scheme=w["scheme"], precision=prec, dims=w["dims"], block_scale=bs,
                             dt=w["dt"], trap_offset=100.0, c0=w["c0"], c2=w["c2"], c4=w["c4"], sigma=w["sigma"],
                             lattice=lat)
        s = Stepper(lat, p)
        s.init_state(s.current, capi.make_init(zeta=w["zeta"], kappa=w["kappa"], noise_abs=w["noise_abs"],
                                               noise_rel=w["noise_rel"], seed=w["seed"]))
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
        s.close()
    e32, e64 = runs[capi.FP32], runs[capi.FP64]
    return {"steps": nsteps, "every": every,
            "energy_rel_diff_max": max(abs(a["energy"] - b["energy"]) / abs(b["energy"]) for a, b in zip(e32, e64)),
            "norm_rel_diff_max": max(abs(a["norm"] - b["norm"]) / abs(b["norm"]) for a, b in zip(e32, e64)),
            "energy_rel_drift_fp32": abs(e32[-1]["energy"] - e32[0]["energy"]) / abs(e32[0]["energy"]),
            "energy_rel_drift_fp64": abs(e64[-1]["energy"] - e64[0]["energy"]) / abs(e64[0]["energy"])}


# Adjoint ramp control: spin-1, BCC 64^3 cells, 2000 steps, Bz(t) and Bq(t) with 16
# piecewise-linear knots each (seeded uniform in [-1, 1]), loss 1 - |<T|psi(T)>|^2
# against a seeded hedgehog (monopole-like) target, 45-step checkpoints, central
# differences (h = 1e-4) of the FP64 run on 8 random knots.
ADJ = dict(dims=(64, 64, 64), steps=2000, stride=45, knots=16, fd_knots=8, h=1e-4, seed=4)


def run_adjoint(args):
    """--workload adjoint-bcc64: gradient of the ramp-control loss through the adjoint
    kernel (FP32 and FP64), timed, and checked against central differences."""
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
        rc = RampControl(s, args.adjoint_steps, ADJ["knots"], lambda: s.init_state(capi.PSI_ODD, init), target,
                         stride=ADJ["stride"])
        reps = max(1, args.steps) if prec == capi.FP32 else 1
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
            picks = rng.choice(2 * ADJ["knots"], args.fd_knots, replace=False)
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
    res = {"metric": "adjoint gradient evaluations/s (forward + reverse run, %d steps)" % args.adjoint_steps,
           "value": 1.0 / grad_s,
           "unit": "gradients/s", "n_gpus": 1, "steps": max(1, args.steps), "warmup": 1,
           "ms_per_step": 1e3 * grad_s, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "adjoint ramp control, spin-1 BCC 64^3 cells (%d sites), %d steps, %d+%d knots, "
                                  "%d-step checkpoints" % (sites, args.adjoint_steps, ADJ["knots"], ADJ["knots"], ADJ["stride"]),
                      "dt": DT, "c0": C0, "c2": C2, "loss": "1 - |<monopole|psi(T)>|^2"},
           "forward_ms": 1e3 * f32["forward_s"], "backward_ms": 1e3 * f32["backward_s"],
           "reverse_site_updates_per_s": sites * args.adjoint_steps / f32["backward_s"],
           "gpu_launches": f32["launches_per_gradient"],
           "loss_fp32": f32["loss"], "loss_fp64": out[capi.FP64]["loss"],
           "fp64_adjoint_vs_fd_max_rel": float(rel_fd64.max()), "fp32_adjoint_vs_fd_max_rel": float(rel_fd32.max()),
           "fp32_vs_fp64_adjoint_rel": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
           "fd_h": ADJ["h"], "fd_knots": [int(i) for i in picks], "fd": [float(x) for x in fd],
           "adjoint_fp64_at_fd_knots": [float(x) for x in g64[picks]],
           "fp64_forward_ms": 1e3 * out[capi.FP64]["forward_s"], "fp64_backward_ms": 1e3 * out[capi.FP64]["backward_s"]}
    print(json.dumps(res))
    return 0


# Batched ensemble: 256 condensates, block-cell edge n ~ U{24..80}, lattice ~ U{BCC,
# FCC, A15, C15}, scalar or spin-1, trap omega ~ U[0.8, 1.2]^3, seeded ramps (Bz
# linear between two values in [-1, 1] over 2000 steps, Bq constant in [0, 0.5]),
# box [-8, 8]^3, dt = 5e-5, FP32 with FP64 observables; all advanced by the
# persistent batch kernel, n steps recorded in one CUDA graph.
ENS = dict(members=256, edge=(24, 80), lattices=("bcc", "fcc", "a15", "c15"), seed=5, dt=5e-5, ramp_steps=2000)


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
    """--workload ensemble-256: every member advanced by the persistent batch kernel,
    `inner` steps per graph replay, timed with CUDA events."""
    import ctypes as C

    import torch

    from spacetime_gb300 import capi, states
    from spacetime_gb300.batch import Batch
    from spacetime_gb300.stepper import Stepper

    inner = args.inner or 100
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    members, algo, state_bytes, specs = [], 0, 0, ensemble_members(args.members)
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
    sites = b.sites
    tune = b.autotune(steps=2)
    e_first = [members[k].observe(members[k].current) for k in (0, len(members) // 2, len(members) - 1)]
    b.capture(inner, sp)
    for _ in range(max(1, args.warmup)):
        b.replay()
    n0 = b.launches
    ev = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
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
    step_ms = total_ms / (args.steps * inner)
    counts = {}
    for name, comps, n, _, _ in specs:
        key = "%s/%s" % (name, "spin1" if comps == 3 else "scalar")
        counts[key] = counts.get(key, 0) + 1
    res = {"metric": "lattice-site-updates/s", "value": sites * inner * args.steps / (total_ms * 1e-3),
           "unit": "lattice-site-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": max(1, args.warmup),
           "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "ensemble of %d condensates (edge 24..80, BCC/FCC/A15/C15, scalar + spin-1), "
                                  "%d leapfrog steps per CUDA-graph replay" % (len(members), inner),
                      "sites": sites, "members": counts, "dt": ENS["dt"],
                      "l2": "inputs larger than L2 (%.1f GB per state buffer set), no flush" % (state_bytes / 1e9)},
           "roofline": {"bound": "hbm", "achieved": algo / (step_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": algo / (step_ms * 1e-3) / 1e9 / peak, "peak_kind": kind, "kernel": "batch_kernel<float,3>",
                        "algorithmic_bytes_per_step": algo, "avg_step_ms": step_ms, "traffic": None},
           "gpu_launches": launches, "graph_replays": args.steps, "clocks": clk.summary(), "setup_s": setup_s,
           "autotune": tune,
           "norm_rel_change": [abs(b2["norm"] - a2["norm"]) / a2["norm"] for a2, b2 in zip(e_first, e_last)]}
    b.close()
    for s in members:
        s.close()
    print(json.dumps(res))
    return 0


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

    def advance_observed(ev=None):
        """One bench step: INNER leapfrog steps, the observables summed inside the
        last one (FP32 node terms, FP64 sums); with --observe-fp64 a separate
        observe pass with FP64 node terms after the steps.  ev: three events
        recorded before the steps, after the INNER - 1 plain step launches, and
        after the observed step (its finalize included)."""
        if ev:
            ev[0].record(stream)
        if args.observe_fp64:
            advance()
            if ev:
                ev[1].record(stream)
            o = s.observe(cur_slot(), s._nsteps * DT)
        else:
            s.step(INNER - 1)
            if ev:
                ev[1].record(stream)
            s._nsteps += INNER
            o = s.step_observe(1)
        if ev:
            ev[2].record(stream)
        return o

    kernel_name = {capi.KERNEL_TILE: "leapfrog_tile_kernel<float,3>", capi.KERNEL_GATHER: "parabolic_fixed_kernel<float,3,LEAPFROG,4>",
                   capi.KERNEL_MARCH: "leapfrog_march_kernel<float,3>", capi.KERNEL_ROWS: "leapfrog_rows_kernel<float,3>",
                   capi.KERNEL_SLAB: "parabolic_slab_kernel<float,3,4>"}
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
        batch = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3)) for _ in range(args.steps)]
        obs = []
        with ClockSampler(local) as clk:
            ev_start.record(stream)
            for k in range(args.steps):
                obs.append(advance_observed(batch[k]))
            ev_end.record(stream)
            barrier()
        clocks = clk.summary()
        launches = s.launches - launches0
        total_ms = ev_start.elapsed_time(ev_end)
        plain_ms = sum(a.elapsed_time(b) for a, b, _ in batch)
        observed_ms = sum(b.elapsed_time(c) for _, b, c in batch) / args.steps
    total_ms, value = replica_throughput(total_ms, sites * INNER * args.steps, world, "cuda")
    # the step kernel's mean duration over the plain launches (INNER - 1 per bench
    # step; the observed step, with its finalize, is timed on its own)
    plain_launches = (INNER - (0 if args.observe_fp64 else 1)) * args.steps
    launch_ms = plain_ms / plain_launches
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

    drift = None
    if args.drift_steps > 0 and rank == 0:
        drift = measure_drift(args.drift_steps, stream)

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
        "e2e": {"value": e2e_value, "unit": "lattice-site-updates/s", "h2d_bytes_per_step": int(psi0.nbytes),
                "d2h_bytes_per_step": int(psi0.nbytes) + 8 * 12, "steps": e2e_steps,
                "path": "gpe_upload (FP64 host, pinned) + gpe_start + gpe_step_observe(100) + gpe_download (FP64 host, pinned)",
                "norm_last": e2e_obs["norm"]},
        "observables": "FP64 node terms and sums (separate pass)" if args.observe_fp64 else
                       "summed inside the last step kernel of each bench step (FP32 node terms, FP64 sums)",
        "fp64_plain": {"value": fp64_value, "unit": "lattice-site-updates/s", "ms_per_launch": fp64_ms,
                       "speedup_fp32_fused": (sites / (launch_ms * 1e-3)) / fp64_value},
        "gpu_launches": launches,
        "autotune": tuning_report,
        "clocks": clocks,
        "observables_last": obs[-1] if obs else None,
    }
    if drift is not None:
        result["drift"] = drift
    if rank == 0 and args.cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    s.close()
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()
    return 0


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
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
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
