"""Python front end of libgpe: one Stepper per condensate.

Mirrors the time loop of the reference programs (integrateInTime in
Spin1GpeBCC.cu:1105-1743, RelativisticSpin2Gpe.cu:1295-...): upload an initial
state into PSI_ODD, take the forward-Euler start step, then leapfrog steps with
the field ramp evaluated per step, and FP64 observables when wanted.  All the
work happens in libgpe's CUDA kernels; a missing library raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


class Stepper:
    def __init__(self, lattice, params: "capi.Params"):
        self.lib = capi.load_library()
        self.lattice = lattice if isinstance(lattice, capi.Lattice) else capi.Lattice(lattice)
        self.params = params
        self._lat = C.c_void_p()
        capi.check(self.lib.gpe_lattice_create(C.byref(self.lattice.desc), C.byref(self._lat)), "gpe_lattice_create")
        self._h = C.c_void_p()
        st = self.lib.gpe_create(self._lat, C.byref(params), C.byref(self._h))
        if st != capi.GPE_OK:
            self.lib.gpe_lattice_destroy(self._lat)
            self._lat = None
            capi.check(st, "gpe_create")
        self.stream = None

    # ------------------------------------------------------------- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self.lib.gpe_destroy(self._h)
            self._h = None
        if getattr(self, "_lat", None):
            self.lib.gpe_lattice_destroy(self._lat)
            self._lat = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ----------------------------------------------------------------- state
    def shape(self, edges=False):
        return capi.buffer_shape(self.lattice, self.params, edges)

    def upload(self, slot: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        capi.check(self.lib.gpe_upload(self._h, slot, a.ctypes.data_as(C.POINTER(C.c_double)), a.size, self.stream), "gpe_upload")

    def download(self, slot: int, out: np.ndarray | None = None) -> np.ndarray:
        """The slot's state as an FP64 host array in the reference file layout;
        `out` (C-contiguous float64 of that shape, pinned for full link speed) is
        filled in place when given."""
        edges = slot in (capi.Q_EVEN, capi.Q_ODD)
        if out is None:
            out = np.zeros(self.shape(edges))
        elif out.shape != tuple(self.shape(edges)) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("download: out must be a C-contiguous float64 array of shape %s" % (self.shape(edges),))
        capi.check(self.lib.gpe_download(self._h, slot, out.ctypes.data_as(C.POINTER(C.c_double)), out.size, self.stream), "gpe_download")
        return out

    def init_state(self, slot: int, init: "capi.Init"):
        """Seeded Thomas-Fermi state written on the device (gpe_init_state)."""
        capi.check(self.lib.gpe_init_state(self._h, slot, C.byref(init), self.stream), "gpe_init_state")

    def respin(self, slot: int, zeta):
        """Replace the spinor at every node, keeping the density (gpe_respin):
        psi_m <- sqrt(rho |zeta_m|^2) zeta_m / |zeta_m|."""
        z = np.zeros(2 * self.params.components)
        for m, c in enumerate(zeta):
            c = complex(c)
            z[2 * m], z[2 * m + 1] = c.real, c.imag
        capi.check(self.lib.gpe_respin(self._h, slot, z.ctypes.data_as(C.POINTER(C.c_double)), self.stream), "gpe_respin")

    def buffer(self, slot: int):
        p = capi.Pitched()
        cb = C.c_size_t()
        capi.check(self.lib.gpe_buffer(self._h, slot, C.byref(p), C.byref(cb)), "gpe_buffer")
        return p, cb.value

    # ------------------------------------------------------------------ time
    def set_ramp(self, ramp, t0: float = 0.0):
        capi.check(self.lib.gpe_set_ramp(self._h, C.byref(ramp) if ramp is not None else None, t0), "gpe_set_ramp")

    def start(self):
        capi.check(self.lib.gpe_start(self._h, self.stream), "gpe_start")

    def step(self, n: int = 1):
        capi.check(self.lib.gpe_step(self._h, n, self.stream), "gpe_step")

    def step_observe(self, n: int) -> dict:
        """n leapfrog steps; the observables of the state the last step reads (after
        n - 1 steps), summed inside that step's kernel (gpe_step_observe)."""
        o = capi.Observables()
        capi.check(self.lib.gpe_step_observe(self._h, n, C.byref(o), self.stream), "gpe_step_observe")
        return o.as_dict()

    def step_explicit(self, next_slot, prev_slot, fields=None, t=0.0, mode=capi.MODE_LEAPFROG):
        f = C.byref(fields) if fields is not None else None
        capi.check(self.lib.gpe_step_explicit(self._h, next_slot, prev_slot, f, t, mode, self.stream), "gpe_step_explicit")

    # --------------------------------------------------------------- adjoint
    def adjoint_forward(self, fields, target: np.ndarray, stride: int = 0) -> np.ndarray:
        """Recorded forward run from PSI_ODD (gpe_adjoint_forward).

        fields: (n, 4) = (bq, bb_x, bb_y, bb_z) or (n, 8) gpe_fields rows, one per
        step (row 0 drives the Euler start).  Returns (Re <T|psi_N>, Im <T|psi_N>,
        M_x, M_y, M_z)."""
        f = np.asarray(fields, dtype=np.float64)
        if f.ndim != 2 or f.shape[1] not in (4, 8) or f.shape[0] < 1:
            raise ValueError("fields must have shape (n, 4) or (n, 8)")
        rows = np.zeros((f.shape[0], 8))
        rows[:, : f.shape[1]] = f
        t = np.ascontiguousarray(target, dtype=np.float64)
        out = np.zeros(5)
        dp = C.POINTER(C.c_double)
        capi.check(self.lib.gpe_adjoint_forward(self._h, rows.shape[0], rows.ctypes.data_as(C.POINTER(capi.Fields)), stride,
                                                t.ctypes.data_as(dp), t.size, out.ctypes.data_as(dp), self.stream),
                   "gpe_adjoint_forward")
        self._adj_steps = rows.shape[0]
        return out

    def adjoint_backward(self, seed) -> np.ndarray:
        """dL/d(fields) of the recorded run, shape (n, 4) = (bq, bb_x, bb_y, bb_z),
        for seed = dL/d(the five numbers adjoint_forward returned)."""
        sd = np.zeros(5)
        s = np.asarray(seed, dtype=np.float64).ravel()
        sd[: s.size] = s
        n = getattr(self, "_adj_steps", 0)
        grad = np.zeros((max(n, 1), 4))
        dp = C.POINTER(C.c_double)
        capi.check(self.lib.gpe_adjoint_backward(self._h, sd.ctypes.data_as(dp), grad.ctypes.data_as(dp), self.stream),
                   "gpe_adjoint_backward")
        return grad[:n]

    def itp(self, n: int, want_mu: bool = True):
        mu = C.c_double(0.0)
        capi.check(self.lib.gpe_itp(self._h, n, C.byref(mu) if want_mu else None, self.stream), "gpe_itp")
        return mu.value

    def observe(self, slot: int, t: float = 0.0) -> dict:
        o = capi.Observables()
        capi.check(self.lib.gpe_observe(self._h, slot, t, C.byref(o), self.stream), "gpe_observe")
        return o.as_dict()

    def set_expansion(self, t_start: float, rate: float):
        """Condensate expansion: block scale bs0 (1 + rate (t - t_start)) from t_start on."""
        capi.check(self.lib.gpe_set_expansion(self._h, t_start, rate), "gpe_set_expansion")

    def load_state(self, slot: int, path: str):
        """Uploads a reference state file (states.read_state_file) into a slot."""
        from . import states

        self.upload(slot, states.read_state_file(path, self.lattice, self.params, slot in (capi.Q_EVEN, capi.Q_ODD)))

    def save_state(self, slot: int, path: str):
        """Writes a slot as a reference state file (states.write_state_file)."""
        from . import states

        states.write_state_file(path, self.download(slot))

    def node_fields(self, slot: int, kind: int, t: float = 0.0) -> np.ndarray:
        """Per-node output field (gpe_node_fields): shape (Z, Y, X, V, K)."""
        per, count = C.c_size_t(), C.c_size_t()
        capi.check(self.lib.gpe_node_field_count(self._h, kind, C.byref(per), C.byref(count)), "gpe_node_field_count")
        out = np.zeros(count.value)
        capi.check(self.lib.gpe_node_fields(self._h, slot, kind, t, out.ctypes.data_as(C.POINTER(C.c_double)), out.size,
                                            self.stream), "gpe_node_fields")
        X, Y, Z = (int(self.params.dims[i]) for i in range(3))
        return out.reshape(Z, Y, X, self.lattice.nodes, per.value)

    def node_fields_reduce(self, slot: int, kind: int, t: float = 0.0) -> np.ndarray:
        """Integral (or maximum, for FIELD_MAX_HAMILTON) of a field (gpe_node_fields_reduce)."""
        out = np.zeros(5)
        capi.check(self.lib.gpe_node_fields_reduce(self._h, slot, kind, t, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                   self.stream), "gpe_node_fields_reduce")
        return out[:5 if kind == capi.FIELD_SPIN else 1]

    def set_tuning(self, key: int, value: int):
        capi.check(self.lib.gpe_set_tuning(self._h, key, value), "gpe_set_tuning")

    def get_tuning(self, key: int) -> int:
        v = C.c_int32()
        capi.check(self.lib.gpe_get_tuning(self._h, key, C.byref(v)), "gpe_get_tuning")
        return v.value

    def step_timing(self, reset: bool = True) -> dict:
        """Device time of the gpe_step / gpe_step_observe calls made while
        TUNE_TIMING was 1 (gpe_get_step_timing); the sums restart when `reset`."""
        t = capi.StepTiming()
        capi.check(self.lib.gpe_get_step_timing(self._h, C.byref(t), 1 if reset else 0), "gpe_get_step_timing")
        return t.as_dict()

    def autotune(self, steps: int = 10) -> list:
        """Pick the fastest step kernel / tile shape for this handle (gpe_autotune)."""
        import json

        buf = C.create_string_buffer(1 << 16)
        capi.check(self.lib.gpe_autotune(self._h, steps, buf, len(buf), self.stream), "gpe_autotune")
        return json.loads(buf.value.decode() or "[]")

    @property
    def current(self) -> int:
        """Slot holding the newest state."""
        return int(self.lib.gpe_current_slot(self._h))

    @property
    def launches(self) -> int:
        return int(self.lib.gpe_launch_count(self._h))

    @property
    def sites(self) -> int:
        return int(self.lib.gpe_sites(self._h))
