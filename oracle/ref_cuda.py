"""The reference's own CUDA kernels, run on device buffers: TEST INFRASTRUCTURE.

`oracle/build_ref_cuda.sh` compiles the device code of the reference programs on
the hot path, unmodified, to cubins in `oracle/_ref/`.  This module loads them
through the CUDA driver API (ctypes on libcuda) and launches the reference's
kernels with the reference's launch shapes on the pitched buffers of an FP64
libgpe handle, whose cell layout is the reference's BlockPsis / BlockEdges.  The
lattice tables are given in the reference's device formats (int4 / int2 / int3
byte-offset entries and host-scaled Hodge weights), built from this package's
lattice tables with the handle's pitches, exactly as each program's host code
builds them with `getLaplacian`.  Used only by tests/ and by
tests/golden/make_ref_cuda_golden.py, never by the library.

Kernels (names as the compiler exports them):
  spin1_bcc      leapfrog / forwardEuler       Spin1GpeBCC/Spin1GpeBCC.cu:667-917
                 maxHamilton, localAvgSpinAndDensity, uvTheta (node fields, :144-189, 235-326)
                 polarState, ferromagneticState, mixedState (:463-551)
  spin2_bcc      unState, horizontalBnState, verticalBnState, cyclicState (Spin2GpeBCC.cu:417-558)
  spin2_bcc      leapfrog / forwardEuler       Spin2GpeBCC/Spin2GpeBCC.cu:698-990
  rel_spin2_bcc  update_psi / update_q          RelativisticSpin2Gpe/RelativisticSpin2Gpe.cu:971-1132
  rel_spin1_bcc  update_psi / update_q_hyper    RelativisticSpin1Gpe/common_kernels.h:176-255, hyper_kernels.h:80-116
  rel_scalar_bcc update_psi / update_q          RelativisticGpeBCC/RelativisticGpeBCC.cu:179-255 (sigma = 0.001 compiled in)
  scalar_bcc     update                         GrossPitaevskiiGpuBcc/GPUGrossPitaevskii_BCC.cu:176-202, 327-347
  scalar_c15/a15 update (dt folded in)          GrossPitaevskiiGpuC15/GPUGrossPitaevskii_C15.cu:104-146
  scalar_fcc     update (CSR node table)        GrossPitaevskiiGpuFcc/GPUGrossPitaevskii_FCC.cu:104-150
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

# Compile-time constants of the reference programs that the kernels bake in.
PI = 3.1415926535897932385                                # Types/Types.hpp:24
LAMBDA_Z = (166 * 2 * PI) / (126 * 2 * PI)                # Spin1GpeBCC.cu: omega_z / omega_r
TRAP_OFFSET = 100.0                                       # Spin1GpeBCC.cu:121
QUAD_CENTER = (-0.20590789, -0.48902826, -0.27353409)     # Spin1GpeBCC.cu:124-126
SPIN2_DT = 1e-5                                           # Spin2GpeBCC.cu:159
TB_X, TB_Y = 16, 2                                        # THREAD_BLOCK_X/Y of the spinor programs
SCALAR_TB = 8                                             # THREAD_BLOCK_X/Y of the scalar programs
REL_SCALAR_SIGMA = 0.001                                  # RelativisticGpeBCC.cu:18

NAMES = {
    ("spin1_bcc", "leapfrog"): "_Z8leapfrog10PitchedPtrS_PK4int4PKd9MagFields5uint3d7double3dddbbbdd",
    ("spin1_bcc", "euler"): "_Z12forwardEuler10PitchedPtrS_P4int4Pd9MagFields5uint3d7double3dddbbbdd",
    ("spin1_bcc", "maxHamilton"): "_Z11maxHamiltonPd10PitchedPtr9MagFields5uint3d7double3dddd",
    ("spin1_bcc", "polarState"): "_Z10polarState10PitchedPtr5uint3",
    ("spin1_bcc", "ferromagneticState"): "_Z18ferromagneticState10PitchedPtr5uint3",
    ("spin1_bcc", "mixedState"): "_Z10mixedState10PitchedPtr5uint3d",
    ("spin2_bcc", "unState"): "_Z7unState10PitchedPtr5uint3",
    ("spin2_bcc", "horizontalBnState"): "_Z17horizontalBnState10PitchedPtr5uint3d",
    ("spin2_bcc", "verticalBnState"): "_Z15verticalBnState10PitchedPtr5uint3d",
    ("spin2_bcc", "cyclicState"): "_Z11cyclicState10PitchedPtr5uint3d",
    ("spin1_bcc", "localAvgSpinAndDensity"): "_Z22localAvgSpinAndDensityPdP7double3S_10PitchedPtr5uint3",
    ("spin1_bcc", "uvTheta"): "_Z7uvThetaP7double3S0_Pd10PitchedPtr5uint3",
    ("spin2_bcc", "leapfrog"): "_Z8leapfrog10PitchedPtrS_PK4int4PKd9MagFields5uint3d7double3ddddd",
    ("spin2_bcc", "euler"): "_Z12forwardEuler10PitchedPtrS_P4int4Pd9MagFields5uint3d7double3ddddd",
    ("rel_spin2_bcc", "update_psi"): "_Z10update_psi10PitchedPtrS_S_PK4int2PKd9MagFields5uint3d7double3ddddbd",
    ("rel_spin2_bcc", "update_q"): "_Z8update_q10PitchedPtrS_S_P4int35uint3db",
    ("rel_spin1_bcc", "update_psi"): "_Z10update_psi10PitchedPtrS_S_PK4int2PKd9MagFields5uint3d7double3dddbd",
    ("rel_spin1_bcc", "update_q_hyper"): "_Z14update_q_hyper10PitchedPtrS_S_P4int35uint3d",
    ("rel_spin1_bcc", "itp_q_hyper"): "_Z11itp_q_hyper10PitchedPtrS_S_P4int35uint3d",
    ("rel_spin1_bcc", "itp_psi"): "_Z7itp_psi10PitchedPtrS_S_S_PK4int2PKd9MagFields5uint3d7double3ddd",
    ("rel_spin2_gs", "itp_q"): "_Z5itp_q10PitchedPtrS_S_P4int35uint3d",
    ("rel_spin2_gs", "itp_psi"): "_Z7itp_psi10PitchedPtrS_S_PK4int2PKd5uint3d7double3dddd",
    ("rel_spin2_gs", "get_Hpsi"): "_Z8get_Hpsi10PitchedPtrS_S_PK4int2PKd5uint3d7double3ddd",
    ("rel_scalar_bcc", "update_psi"): "_Z10update_psi10PitchedPtrS_S_S_P4int2Pdd5uint3d",
    ("rel_scalar_bcc", "update_q"): "_Z8update_q10PitchedPtrS_S_P4int35uint3d",
    ("rel_scalar_c15", "update_psi"): "_Z10update_psi10PitchedPtrS_S_S_P4int2Pdd5uint3d",
    ("rel_scalar_c15", "update_q"): "_Z8update_q10PitchedPtrS_S_P4int35uint3dd",
    ("scalar_bcc", "update"): "_Z6update10PitchedPtrS_S_P4int2Pdd5uint3d",
    ("scalar_c15", "update"): "_Z6update10PitchedPtrS_S_P4int2Pdd5uint3",
    ("scalar_a15", "update"): "_Z6update10PitchedPtrS_S_P4int2Pdd5uint3",
    ("scalar_fcc", "update"): "_Z6update10PitchedPtrS_S_P4int2PdS1_d5uint3",
}


class PitchedPtr(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("pitch", C.c_size_t), ("slicePitch", C.c_size_t)]


class Double3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class Uint3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


class MagFields(C.Structure):
    _fields_ = [("Bq", C.c_double), ("Bb", Double3), ("BqQuad", C.c_double), ("BbQuad", Double3)]


def available(program: str) -> bool:
    return os.path.exists(os.path.join(REF_DIR, program + ".cubin"))


def mag_fields(f) -> MagFields:
    """gpe_fields -> the reference's MagFields (Spin1GpeBCC/utils.h:94-100)."""
    return MagFields(f.bq, Double3(*f.bb), f.bq_quad, Double3(*f.bb_quad))


class Driver:
    """Minimal CUDA driver API: modules, device memory, launches (current context)."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        ctx = C.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context (create a libgpe handle first)")
        self.cu.cuMemAlloc_v2.argtypes = [C.POINTER(C.c_uint64), C.c_size_t]
        self.cu.cuMemFree_v2.argtypes = [C.c_uint64]
        self.cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        self.cu.cuMemcpyDtoH_v2.argtypes = [C.c_void_p, C.c_uint64, C.c_size_t]
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                           C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]
        self.modules = {}
        self.allocs = []

    @staticmethod
    def _check(rc, where):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (where, rc))

    def function(self, program: str, kernel: str):
        if program not in self.modules:
            data = open(os.path.join(REF_DIR, program + ".cubin"), "rb").read()
            mod = C.c_void_p()
            self._check(self.cu.cuModuleLoadData(C.byref(mod), C.c_char_p(data)), "cuModuleLoadData")
            self.modules[program] = mod
        fn = C.c_void_p()
        self._check(self.cu.cuModuleGetFunction(C.byref(fn), self.modules[program],
                                                NAMES[(program, kernel)].encode()), "cuModuleGetFunction")
        return fn

    def upload(self, arr: np.ndarray) -> int:
        a = np.ascontiguousarray(arr)
        p = C.c_uint64()
        self._check(self.cu.cuMemAlloc_v2(C.byref(p), max(a.nbytes, 16)), "cuMemAlloc")
        self.allocs.append(p.value)
        self._check(self.cu.cuMemcpyHtoD_v2(p.value, a.ctypes.data, a.nbytes), "cuMemcpyHtoD")
        return p.value

    def download(self, ptr: int, nbytes: int) -> np.ndarray:
        out = np.empty(nbytes, dtype=np.uint8)
        self._check(self.cu.cuMemcpyDtoH_v2(out.ctypes.data, ptr, nbytes), "cuMemcpyDtoH")
        return out

    def launch(self, fn, grid, block, args):
        params = (C.c_void_p * len(args))(*[C.addressof(a) for a in args])
        self._check(self.cu.cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0, None,
                                           params, None), "cuLaunchKernel")
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def close(self):
        for p in self.allocs:
            self.cu.cuMemFree_v2(p)
        self.allocs = []
        for m in self.modules.values():
            self.cu.cuModuleUnload(m)
        self.modules = {}


def pitched(stepper, slot) -> PitchedPtr:
    p, _ = stepper.buffer(slot)
    return PitchedPtr(p.ptr, p.pitch, p.slice_pitch)


def cell_offset(dx, dy, dz, cell_bytes, pitch, slice_pitch) -> int:
    return int(dx * cell_bytes + dy * pitch + dz * slice_pitch)


def stencil_int4(lat) -> tuple:
    """getLaplacian of Spin1GpeBCC/mesh.h: int4 (dx, dy, dz, node) per entry and the
    host-scaled weights -0.5 * hodge (Spin1GpeBCC.cu:1169); node-major, FACE_COUNT
    entries per node."""
    st = lat.data["stencil"]  # rows (dx, dy, dz, node, hodge)
    ent = np.array([[int(dx), int(dy), int(dz), int(n)] for dx, dy, dz, n, _ in st], dtype=np.int32)
    return ent, -0.5 * np.array([float(h) for *_, h in st])


def stencil_int2(lat, stepper, scale) -> tuple:
    """int2 (byte offset, node) entries of the scalar programs' getLaplacian and the
    weights -0.5 * hodge * scale (scale = 1/bs^2, times dt where it is folded in)."""
    p, cell_bytes = stepper.buffer(0)
    st = lat.data["stencil"]  # rows (dx, dy, dz, node, hodge)
    ent = np.array([[cell_offset(dx, dy, dz, cell_bytes, p.pitch, p.slice_pitch), int(n)] for dx, dy, dz, n, _ in st],
                   dtype=np.int32)
    return ent, np.array([-0.5 * float(h) * scale for *_, h in st])


def edge_tables(lat, stepper, bs) -> tuple:
    """RelativisticSpin2Gpe/mesh.h getLaplacian: d0 int3 (from, byte offset of the
    to-cell in psi, to), d1 int2 (byte offset of the edge cell in q, edge) and the
    host-scaled incidence weights -0.5 * h / bs^2 (RelativisticSpin2Gpe.cu:1399)."""
    pp, cb = stepper.buffer(0)
    qp, qcb = stepper.buffer(2)
    return edge_tables_for(lat, bs, (cb, pp.pitch, pp.slice_pitch), (qcb, qp.pitch, qp.slice_pitch))


def edge_tables_for(lat, bs, psi_geom, q_geom) -> tuple:
    """edge_tables for buffers of the given (cell bytes, pitch, slice pitch)."""
    cb, pitch, slice_pitch = psi_geom
    qcb, qpitch, qslice = q_geom
    d0 = np.array([[int(f), cell_offset(dx, dy, dz, cb, pitch, slice_pitch), int(t)]
                   for f, dx, dy, dz, t in lat.data["edges"]], dtype=np.int32)  # rows (from, dx, dy, dz, to)
    inc = lat.data["incidence"]  # rows (dx, dy, dz, edge, hodge)
    d1 = np.array([[cell_offset(dx, dy, dz, qcb, qpitch, qslice), int(e)] for dx, dy, dz, e, _ in inc],
                  dtype=np.int32)
    w = np.array([-0.5 * float(h) / (bs * bs) for *_, h in inc])
    return d0, d1, w


def node_potential(lat, params) -> np.ndarray:
    """Trap potential 0.5 |lambda r|^2 + offset per interior node, in the reference's
    BlockPots layout with halo: shape (Z+2, Y+2, X+2, V)."""
    from spacetime_gb300 import states

    r = states.node_positions(lat, params)
    lam = [params.trap_lambda[i] for i in range(3)]
    x, y, z = r[..., 0] * lam[0], r[..., 1] * lam[1], r[..., 2] * lam[2]
    v = 0.5 * (x * x + y * y + z * z) + params.trap_offset
    out = np.zeros((v.shape[0] + 2, v.shape[1] + 2, v.shape[2] + 2, v.shape[3]))
    out[1:-1, 1:-1, 1:-1] = v
    return out


def pitched_upload(drv: Driver, host: np.ndarray, row_align: int = 256) -> PitchedPtr:
    """A pitched device copy of a (Z+2, Y+2, X+2, ...) host array; returns the
    interior PitchedPtr (one cell in on every axis)."""
    Z2, Y2, X2 = host.shape[:3]
    cell = int(np.prod(host.shape[3:])) * host.itemsize
    pitch = (X2 * cell + row_align - 1) // row_align * row_align
    buf = np.zeros((Z2, Y2, pitch), dtype=np.uint8)
    buf[:, :, : X2 * cell] = np.ascontiguousarray(host).view(np.uint8).reshape(Z2, Y2, X2 * cell)
    base = drv.upload(buf)
    slice_pitch = pitch * Y2
    return PitchedPtr(base + slice_pitch + pitch + cell, pitch, slice_pitch)


def pitched_download(drv: Driver, pp: PitchedPtr, shape, dtype=np.float64) -> np.ndarray:
    """Reads back a buffer made by pitched_upload: shape is the full
    (Z+2, Y+2, X+2, ...) host shape."""
    Z2, Y2, X2 = shape[:3]
    itemsize = np.dtype(dtype).itemsize
    cell = int(np.prod(shape[3:])) * itemsize
    base = pp.ptr - pp.slicePitch - pp.pitch - cell
    raw = drv.download(base, Z2 * pp.slicePitch).reshape(Z2, Y2, pp.pitch)
    return np.ascontiguousarray(raw[:, :, : X2 * cell]).view(dtype).reshape(shape)


def spinor_grid(params, V):
    X, Y, Z = (int(params.dims[i]) for i in range(3))
    return ((X + TB_X - 1) // TB_X, (Y + TB_Y - 1) // TB_Y, Z), (TB_X * V, TB_Y, 1)


def edge_grid(params, E):
    X, Y, Z = (int(params.dims[i]) for i in range(3))
    return ((X + TB_X - 1) // TB_X, (Y + TB_Y - 1) // TB_Y, Z), (TB_X * E, TB_Y, 1)


def scalar_grid(params, V):
    X, Y, Z = (int(params.dims[i]) for i in range(3))
    return ((X + SCALAR_TB - 1) // SCALAR_TB, (Y + SCALAR_TB - 1) // SCALAR_TB, Z * V), (SCALAR_TB, SCALAR_TB, 1)


def uint3(params) -> Uint3:
    return Uint3(int(params.dims[0]), int(params.dims[1]), int(params.dims[2]))


def double3(v) -> Double3:
    return Double3(float(v[0]), float(v[1]), float(v[2]))


__all__ = ["Driver", "available", "mag_fields", "pitched", "stencil_int4", "stencil_int2", "edge_tables",
           "edge_tables_for", "node_potential", "pitched_upload", "pitched_download", "spinor_grid", "edge_grid", "scalar_grid", "uint3", "double3",
           "LAMBDA_Z", "TRAP_OFFSET", "QUAD_CENTER", "SPIN2_DT", "math"]
