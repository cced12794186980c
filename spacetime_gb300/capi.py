"""ctypes mirror of include/gpe.h and the loader for the in-tree libgpe.so.

The library is the product; this module only declares its C types and function
signatures.  ``load_library()`` raises if the CUDA library has not been built:
there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libgpe.so")
LATTICE_DIR = os.path.join(PKG_DIR, "lattices")

GPE_OK = 0
STATUS_NAMES = {
    0: "GPE_OK",
    1: "GPE_ERR_INVALID_ARG",
    2: "GPE_ERR_OOM",
    3: "GPE_ERR_CUDA",
    4: "GPE_ERR_TIMEOUT",
    5: "GPE_ERR_NONFINITE",
    6: "GPE_ERR_UNSUPPORTED",
    7: "GPE_ERR_NO_DEVICE",
}

SCHEME_PARABOLIC, SCHEME_HYPERBOLIC, SCHEME_SPLIT = 0, 1, 2
FP32, FP64 = 0, 1
FLAG_THREE_BODY_LOSS, FLAG_QUADRATIC_ZEEMAN, FLAG_QUADRUPOLE_OFFSET, FLAG_TRAP_OFF_AFTER = 1, 2, 4, 8
RAMP_CONSTANT, RAMP_LINEAR, RAMP_SQRT = 0, 1, 2
RAMP_MAX_SEGMENTS = 32
PSI_EVEN, PSI_ODD, Q_EVEN, Q_ODD, HPSI = 0, 1, 2, 3, 4
MODE_LEAPFROG, MODE_EULER, MODE_ITP = 0, 1, 2
TUNE_KERNEL, TUNE_TILE_CELLS, TUNE_TILE_ROWS, TUNE_ZCHUNK, TUNE_THREADS, TUNE_OBSERVE_ARITH, TUNE_CARVEOUT, TUNE_TIMING = (
    0, 1, 2, 3, 4, 5, 6, 7)
TUNE_TRANSFER = 8
FIELD_DENSITY, FIELD_SPIN, FIELD_UV_THETA, FIELD_MAX_HAMILTON, FIELD_PROJ_X, FIELD_PROJ_Y = 0, 1, 2, 3, 4, 5
KERNEL_AUTO, KERNEL_GATHER, KERNEL_TILE, KERNEL_MARCH, KERNEL_ROWS, KERNEL_SLAB, KERNEL_INTERLEAVED = 0, 1, 2, 3, 4, 5, 6
BATCH_ITEM_NODES, BATCH_STEPS_PER_LAUNCH, BATCH_BLOCKS_PER_SM, BATCH_BARRIER_TIMEOUT_MS, BATCH_TEST_EXTRA_ARRIVALS = 0, 1, 2, 3, 4
BATCH_LAYOUT = 5


class StencilEntry(C.Structure):
    _fields_ = [("dx", C.c_int32), ("dy", C.c_int32), ("dz", C.c_int32), ("node", C.c_int32), ("hodge", C.c_double)]


class Edge(C.Structure):
    _fields_ = [("frm", C.c_int32), ("dx", C.c_int32), ("dy", C.c_int32), ("dz", C.c_int32), ("to", C.c_int32)]


class Incidence(C.Structure):
    _fields_ = [("dx", C.c_int32), ("dy", C.c_int32), ("dz", C.c_int32), ("edge", C.c_int32), ("hodge", C.c_double)]


class LatticeDesc(C.Structure):
    _fields_ = [
        ("nodes", C.c_int32),
        ("block_width", C.c_double * 3),
        ("volume", C.c_double),
        ("pos", C.POINTER(C.c_double)),
        ("row_ptr", C.POINTER(C.c_int32)),
        ("stencil", C.POINTER(StencilEntry)),
        ("edges", C.c_int32),
        ("faces_per_node", C.c_int32),
        ("edge_table", C.POINTER(Edge)),
        ("incidence", C.POINTER(Incidence)),
    ]


class VortexParams(C.Structure):
    _fields_ = [
        ("kappa", C.c_uint32),
        ("g", C.c_double),
        ("rmin", C.c_double),
        ("rmax", C.c_double),
        ("rstep", C.c_double),
        ("zmax", C.c_double),
        ("zstep", C.c_double),
        ("trap_ratio", C.c_double),
        ("max_iters", C.c_uint32),
        ("eps", C.c_double),
    ]


class Params(C.Structure):
    _fields_ = [
        ("components", C.c_int32),
        ("scheme", C.c_int32),
        ("precision", C.c_int32),
        ("flags", C.c_int32),
        ("dims", C.c_uint32 * 3),
        ("block_scale", C.c_double),
        ("p0", C.c_double * 3),
        ("dt", C.c_double),
        ("trap_lambda", C.c_double * 3),
        ("trap_offset", C.c_double),
        ("trap_off_time", C.c_double),
        ("c0", C.c_double),
        ("c2", C.c_double),
        ("c4", C.c_double),
        ("alpha", C.c_double),
        ("sigma", C.c_double),
        ("quad_center", C.c_double * 3),
    ]


class Fields(C.Structure):
    _fields_ = [("bq", C.c_double), ("bb", C.c_double * 3), ("bq_quad", C.c_double), ("bb_quad", C.c_double * 3)]


class Ramp(C.Structure):
    _fields_ = [
        ("bq_segments", C.c_int32),
        ("bq_target", C.c_double * RAMP_MAX_SEGMENTS),
        ("bq_duration", C.c_double * RAMP_MAX_SEGMENTS),
        ("bq_type", C.c_int32 * RAMP_MAX_SEGMENTS),
        ("bb_segments", C.c_int32),
        ("bb_target", (C.c_double * 3) * RAMP_MAX_SEGMENTS),
        ("bb_duration", C.c_double * RAMP_MAX_SEGMENTS),
        ("bb_type", C.c_int32 * RAMP_MAX_SEGMENTS),
        ("time_scale", C.c_double),
        ("bq_scale", C.c_double),
        ("bb_scale", C.c_double),
        ("bq_quad_scale", C.c_double),
        ("bb_quad_scale", C.c_double),
    ]


class Init(C.Structure):
    _fields_ = [("zeta", (C.c_double * 2) * 5), ("vortex_kappa", C.c_int32), ("noise_abs", C.c_double),
                ("noise_rel", C.c_double), ("seed", C.c_uint64), ("normalize", C.c_int32)]


def make_init(zeta=(1.0,), kappa=0, noise_abs=0.0, noise_rel=0.0, seed=1, normalize=True) -> Init:
    it = Init()
    for m, z in enumerate(zeta):
        z = complex(z)
        it.zeta[m][0] = z.real
        it.zeta[m][1] = z.imag
    it.vortex_kappa = kappa
    it.noise_abs = noise_abs
    it.noise_rel = noise_rel
    it.seed = seed
    it.normalize = 1 if normalize else 0
    return it


class Pitched(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("pitch", C.c_size_t), ("slice_pitch", C.c_size_t)]


class Observables(C.Structure):
    _fields_ = [
        ("norm", C.c_double),
        ("energy", C.c_double),
        ("h_expect", C.c_double),
        ("magnetization", C.c_double * 3),
        ("spin_norm", C.c_double),
        ("com", C.c_double * 3),
        ("max_abs", C.c_double),
        ("nonfinite", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {
            "norm": self.norm,
            "energy": self.energy,
            "h_expect": self.h_expect,
            "magnetization": list(self.magnetization),
            "spin_norm": self.spin_norm,
            "com": list(self.com),
            "max_abs": self.max_abs,
            "nonfinite": self.nonfinite,
        }


class StepTiming(C.Structure):
    """gpe_step_timing: device time of the timed gpe_step / gpe_step_observe calls."""
    _fields_ = [
        ("calls", C.c_uint64),
        ("step_launches", C.c_uint64),
        ("step_ms", C.c_double),
        ("observed_launches", C.c_uint64),
        ("observed_ms", C.c_double),
        ("convert_launches", C.c_uint64),
        ("convert_ms", C.c_double),
        ("interleaved_calls", C.c_int32),
        ("reserved", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


# ------------------------------------------------------------------ lattices


class Lattice:
    """Lattice tables loaded from ``lattices/<name>.json`` with ctypes views that
    stay alive as long as this object does."""

    def __init__(self, name: str, tables: dict | None = None):
        """tables: tables in the same layout (e.g. lattices.generate.generate())
        instead of the file."""
        if tables is None:
            with open(os.path.join(LATTICE_DIR, name + ".json")) as f:
                d = json.load(f)
        else:
            d = tables
        self.name = name
        self.data = d
        self.nodes = int(d["nodes"])
        self.block_width = np.array(d["block_width"], dtype=np.float64)
        self.volume = float(d["volume"])
        self.pos = np.ascontiguousarray(np.array(d["pos"], dtype=np.float64).reshape(self.nodes, 3))
        self.row_ptr = np.array(d["row_ptr"], dtype=np.int32)
        st = d["stencil"]
        self._stencil = (StencilEntry * len(st))(*[StencilEntry(int(a), int(b), int(c), int(n), float(h)) for a, b, c, n, h in st])
        self.degree = np.diff(self.row_ptr)
        self.has_edges = "edges" in d
        self.edges = int(d.get("edge_count", 0))
        self.faces_per_node = int(d.get("edge_face_count", 0))
        if self.has_edges:
            ed = d["edges"]
            inc = d["incidence"]
            self._edges = (Edge * len(ed))(*[Edge(int(f), int(a), int(b), int(c), int(t)) for f, a, b, c, t in ed])
            self._inc = (Incidence * len(inc))(*[Incidence(int(a), int(b), int(c), int(e), float(h)) for a, b, c, e, h in inc])
        self.desc = LatticeDesc()
        self.desc.nodes = self.nodes
        for i in range(3):
            self.desc.block_width[i] = float(self.block_width[i])
        self.desc.volume = self.volume
        self.desc.pos = self.pos.ctypes.data_as(C.POINTER(C.c_double))
        self.desc.row_ptr = self.row_ptr.ctypes.data_as(C.POINTER(C.c_int32))
        self.desc.stencil = C.cast(self._stencil, C.POINTER(StencilEntry))
        if self.has_edges:
            self.desc.edges = self.edges
            self.desc.faces_per_node = self.faces_per_node
            self.desc.edge_table = C.cast(self._edges, C.POINTER(Edge))
            self.desc.incidence = C.cast(self._inc, C.POINTER(Incidence))
        else:
            self.desc.edges = 0
            self.desc.faces_per_node = 0

    def stencil_array(self) -> np.ndarray:
        return np.array(self.data["stencil"], dtype=np.float64)


LATTICE_NAMES = ("cube", "bcc", "bcc227", "fcc", "a15", "c15", "z")


def make_params(components=3, scheme=SCHEME_PARABOLIC, precision=FP32, flags=0, dims=(8, 8, 8), block_scale=0.1,
                p0=None, dt=1e-4, trap_lambda=(1.0, 1.0, 1.0), trap_offset=0.0, trap_off_time=0.0, c0=0.0, c2=0.0,
                c4=0.0, alpha=0.0, sigma=0.0, quad_center=(0.0, 0.0, 0.0), lattice: Lattice | None = None) -> Params:
    p = Params()
    p.components = components
    p.scheme = scheme
    p.precision = precision
    p.flags = flags
    for i in range(3):
        p.dims[i] = int(dims[i])
    p.block_scale = block_scale
    if p0 is None:
        # centre the box on the origin (Spin1GpeBCC.cu:1112)
        bw = lattice.block_width if lattice is not None else np.ones(3)
        p0 = [-0.5 * block_scale * bw[i] * dims[i] for i in range(3)]
    for i in range(3):
        p.p0[i] = float(p0[i])
        p.trap_lambda[i] = float(trap_lambda[i])
        p.quad_center[i] = float(quad_center[i])
    p.dt = dt
    p.trap_offset = trap_offset
    p.trap_off_time = trap_off_time
    p.c0, p.c2, p.c4 = c0, c2, c4
    p.alpha = alpha
    p.sigma = sigma
    return p


def make_fields(bq=0.0, bb=(0.0, 0.0, 0.0), bq_quad=0.0, bb_quad=(0.0, 0.0, 0.0)) -> Fields:
    f = Fields()
    f.bq = bq
    f.bq_quad = bq_quad
    for i in range(3):
        f.bb[i] = bb[i]
        f.bb_quad[i] = bb_quad[i]
    return f


def make_ramp(bq_segments=(), bb_segments=(), time_scale=1.0, bq_scale=1.0, bb_scale=1.0, bq_quad_scale=0.0,
              bb_quad_scale=0.0) -> Ramp:
    """Segments are (target, duration, type); bb targets are 3-vectors."""
    r = Ramp()
    if len(bq_segments) > RAMP_MAX_SEGMENTS or len(bb_segments) > RAMP_MAX_SEGMENTS:
        raise ValueError("too many ramp segments")
    r.bq_segments = len(bq_segments)
    for k, (tgt, dur, typ) in enumerate(bq_segments):
        r.bq_target[k] = tgt
        r.bq_duration[k] = dur
        r.bq_type[k] = typ
    r.bb_segments = len(bb_segments)
    for k, (tgt, dur, typ) in enumerate(bb_segments):
        for a in range(3):
            r.bb_target[k][a] = tgt[a]
        r.bb_duration[k] = dur
        r.bb_type[k] = typ
    r.time_scale = time_scale
    r.bq_scale, r.bb_scale, r.bq_quad_scale, r.bb_quad_scale = bq_scale, bb_scale, bq_quad_scale, bb_quad_scale
    return r


def buffer_shape(lat: Lattice, params: Params, edges: bool = False) -> tuple:
    """Shape of a host buffer in the reference file layout."""
    X, Y, Z = (int(params.dims[i]) for i in range(3))
    items = lat.edges if edges else lat.nodes
    return (Z + 2, Y + 2, X + 2, items, int(params.components), 2)


# ------------------------------------------------------------------- library

_lib = None


def load_library(path: str = LIB_PATH):
    """Load libgpe.so (the CUDA path).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libgpe.so not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "gpe_lattice_create": (C.c_int, [P(LatticeDesc), P(vp)]),
        "gpe_lattice_destroy": (None, [vp]),
        "gpe_create": (C.c_int, [vp, P(Params), P(vp)]),
        "gpe_destroy": (C.c_int, [vp]),
        "gpe_buffer": (C.c_int, [vp, C.c_int32, P(Pitched), P(C.c_size_t)]),
        "gpe_upload": (C.c_int, [vp, C.c_int32, P(C.c_double), C.c_size_t, vp]),
        "gpe_download": (C.c_int, [vp, C.c_int32, P(C.c_double), C.c_size_t, vp]),
        "gpe_set_ramp": (C.c_int, [vp, P(Ramp), C.c_double]),
        "gpe_ramp_eval": (C.c_int, [P(Ramp), C.c_double, P(Fields)]),
        "gpe_start": (C.c_int, [vp, vp]),
        "gpe_step": (C.c_int, [vp, C.c_int32, vp]),
        "gpe_step_explicit": (C.c_int, [vp, C.c_int32, C.c_int32, P(Fields), C.c_double, C.c_int32, vp]),
        "gpe_itp": (C.c_int, [vp, C.c_int32, P(C.c_double), vp]),
        "gpe_observe": (C.c_int, [vp, C.c_int32, C.c_double, P(Observables), vp]),
        "gpe_step_observe": (C.c_int, [vp, C.c_int32, P(Observables), vp]),
        "gpe_respin": (C.c_int, [vp, C.c_int32, P(C.c_double), vp]),
        "gpe_vortex_profile": (C.c_int, [P(VortexParams), P(C.c_double), C.c_size_t, P(C.c_uint32), P(C.c_uint32),
                                         P(C.c_double), P(C.c_uint32)]),
        "gpe_vortex_sample": (C.c_int, [P(VortexParams), P(C.c_double), P(LatticeDesc), P(Params), P(C.c_double),
                                        C.c_size_t]),
        "gpe_set_expansion": (C.c_int, [vp, C.c_double, C.c_double]),
        "gpe_node_field_count": (C.c_int, [vp, C.c_int32, P(C.c_size_t), P(C.c_size_t)]),
        "gpe_node_fields": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_double, P(C.c_double), C.c_size_t, vp]),
        "gpe_node_fields_reduce": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_double, P(C.c_double), vp]),
        "gpe_launch_count": (C.c_uint64, [vp]),
        "gpe_current_slot": (C.c_int32, [vp]),
        "gpe_set_tuning": (C.c_int, [vp, C.c_int32, C.c_int32]),
        "gpe_init_state": (C.c_int, [vp, C.c_int32, P(Init), vp]),
        "gpe_autotune": (C.c_int, [vp, C.c_int32, C.c_char_p, C.c_size_t, vp]),
        "gpe_observe_noalloc": (C.c_int, [P(LatticeDesc), P(Params), P(Fields), C.c_double, vp, C.c_size_t, C.c_size_t, P(Observables), vp]),
        "gpe_get_tuning": (C.c_int, [vp, C.c_int32, P(C.c_int32)]),
        "gpe_get_step_timing": (C.c_int, [vp, P(StepTiming), C.c_int32]),
        "gpe_adjoint_forward": (C.c_int, [vp, C.c_int32, P(Fields), C.c_int32, P(C.c_double), C.c_size_t, P(C.c_double), vp]),
        "gpe_adjoint_backward": (C.c_int, [vp, P(C.c_double), P(C.c_double), vp]),
        "gpe_batch_create": (C.c_int, [P(vp), C.c_int32, P(vp)]),
        "gpe_batch_destroy": (C.c_int, [vp]),
        "gpe_batch_step": (C.c_int, [vp, C.c_int32, vp]),
        "gpe_batch_capture": (C.c_int, [vp, C.c_int32, vp]),
        "gpe_batch_replay": (C.c_int, [vp, vp]),
        "gpe_batch_set_tuning": (C.c_int, [vp, C.c_int32, C.c_int32]),
        "gpe_batch_get_tuning": (C.c_int, [vp, C.c_int32, P(C.c_int32)]),
        "gpe_batch_autotune": (C.c_int, [vp, C.c_int32, C.c_char_p, C.c_size_t, vp]),
        "gpe_batch_sites": (C.c_uint64, [vp]),
        "gpe_batch_launch_count": (C.c_uint64, [vp]),
        "gpe_sites": (C.c_uint64, [vp]),
        "gpe_last_error": (C.c_char_p, []),
        "gpe_version": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GpeError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__("%s failed: %s %s" % (where, STATUS_NAMES.get(status, status), detail))


def check(status: int, where: str):
    if status != GPE_OK:
        detail = ""
        if _lib is not None:
            detail = (_lib.gpe_last_error() or b"").decode(errors="replace")
        raise GpeError(status, where, detail)


def exported_symbols_from_header(header: str | None = None) -> list:
    """Names of the functions declared in include/gpe.h (used by the ABI test)."""
    import re

    header = header or os.path.join(os.path.dirname(PKG_DIR), "include", "gpe.h")
    with open(header) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gpe_[a-z0-9_]+)\s*\(", text)))


def vortex_state(lat: "Lattice", params: "Params", kappa=1, g=None, rmin=0.0, rmax=None, zmax=None, rstep=0.1,
                 zstep=0.1, trap_ratio=1.0, max_iters=100000, eps=1e-28):
    """The relaxed vortex state Psi = f(r, z) e^{i kappa phi} (gpe_vortex_profile,
    the reference's VortexState) sampled at every node of the grid of `params`
    (gpe_vortex_sample): (host array in the file layout, mu, sweeps taken).
    g defaults to params.c0; rmax and zmax to the box's half-extent + 1, as the
    reference's CPU stepper sets them up."""
    lib = load_library()
    half = max(abs(params.p0[i]) for i in range(3))
    vp = VortexParams(kappa, params.c0 if g is None else g, rmin, half + 1.0 if rmax is None else rmax, rstep,
                      half + 1.0 if zmax is None else zmax, zstep, trap_ratio, max_iters, eps)
    rs, zs = C.c_uint32(), C.c_uint32()
    check(lib.gpe_vortex_profile(C.byref(vp), None, 0, C.byref(rs), C.byref(zs), None, None), "gpe_vortex_profile")
    f = np.zeros(rs.value * zs.value)
    mu, it = C.c_double(), C.c_uint32()
    check(lib.gpe_vortex_profile(C.byref(vp), f.ctypes.data_as(C.POINTER(C.c_double)), f.size, None, None, C.byref(mu),
                                 C.byref(it)), "gpe_vortex_profile")
    out = np.zeros(buffer_shape(lat, params))
    check(lib.gpe_vortex_sample(C.byref(vp), f.ctypes.data_as(C.POINTER(C.c_double)), C.byref(lat.desc), C.byref(params),
                                out.ctypes.data_as(C.POINTER(C.c_double)), out.size), "gpe_vortex_sample")
    return out, mu.value, it.value
