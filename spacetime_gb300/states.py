"""Seeded initial states in the reference file layout (FP64, halo included).

The reference prepares its states from an imaginary-time ground state loaded
from disk plus ``std::default_random_engine`` noise (Spin1GpeBCC.cu:1257-1292),
whose output is implementation defined.  These generators are deterministic on
every platform: SplitMix64 (Steele, Lea & Flood 2014; constants as published by
Vigna) feeding Box-Muller Gaussians, evaluated with numpy uint64/float64
arithmetic only.

Shapes: (Z+2, Y+2, X+2, V, C, 2) with the halo cells zero.
"""
from __future__ import annotations

import math

import numpy as np

from . import capi

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n consecutive SplitMix64 outputs of stream `seed` starting at `offset`."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """Uniform doubles in (0, 1]: ((z >> 11) + 1) * 2^-53."""
    z = splitmix64(seed, n, offset)
    return ((z >> np.uint64(11)).astype(np.float64) + 1.0) * (1.0 / 9007199254740992.0)


def gaussian_pairs(seed: int, n: int) -> np.ndarray:
    """n pairs of independent standard normals (Box-Muller), shape (n, 2)."""
    u = uniform01(seed, 2 * n).reshape(n, 2)
    r = np.sqrt(-2.0 * np.log(u[:, 0]))
    th = 2.0 * math.pi * u[:, 1]
    return np.stack([r * np.cos(th), r * np.sin(th)], axis=1)


def node_positions(lat: "capi.Lattice", params: "capi.Params") -> np.ndarray:
    """Physical positions of all interior nodes, shape (Z, Y, X, V, 3)
    (globalPos, Spin1GpeBCC.cu:871-874)."""
    X, Y, Z = (int(params.dims[i]) for i in range(3))
    bs = params.block_scale
    bw = lat.block_width
    p0 = np.array([params.p0[i] for i in range(3)])
    xs = np.arange(X)[None, None, :, None]
    ys = np.arange(Y)[None, :, None, None]
    zs = np.arange(Z)[:, None, None, None]
    lp = lat.pos[None, None, None, :, :]
    out = np.empty((Z, Y, X, lat.nodes, 3))
    out[..., 0] = p0[0] + bs * (xs * bw[0] + lp[..., 0])
    out[..., 1] = p0[1] + bs * (ys * bw[1] + lp[..., 1])
    out[..., 2] = p0[2] + bs * (zs * bw[2] + lp[..., 2])
    return out


def thomas_fermi_density(r: np.ndarray, c0: float, lam=(1.0, 1.0, 1.0)) -> np.ndarray:
    """rho_TF = max(mu - V, 0)/c0 for V = 0.5 |lambda r|^2, normalised to 1:
    mu = 0.5 (15 c0 lx ly lz / 4 pi)^(2/5)."""
    lx, ly, lz = lam
    mu = 0.5 * (15.0 * c0 * lx * ly * lz / (4.0 * math.pi)) ** 0.4
    V = 0.5 * ((lx * r[..., 0]) ** 2 + (ly * r[..., 1]) ** 2 + (lz * r[..., 2]) ** 2)
    return np.maximum(mu - V, 0.0) / c0


def _embed(interior: np.ndarray) -> np.ndarray:
    Z, Y, X = interior.shape[:3]
    out = np.zeros((Z + 2, Y + 2, X + 2) + interior.shape[3:])
    out[1:-1, 1:-1, 1:-1] = interior
    return out


def normalize(buf: np.ndarray, lat: "capi.Lattice", params: "capi.Params") -> np.ndarray:
    dv = params.block_scale ** 3 * lat.volume
    n = float(np.sum(buf[1:-1, 1:-1, 1:-1] ** 2)) * dv
    return buf / math.sqrt(n)


def tf_mu(c0: float, lam=(1.0, 1.0, 1.0)) -> float:
    lx, ly, lz = lam
    return 0.5 * (15.0 * c0 * lx * ly * lz / (4.0 * math.pi)) ** 0.4


def vortex_state(lat, params, seed=1, noise=1e-3, kappa=1) -> np.ndarray:
    """Scalar: Thomas-Fermi amplitude times exp(i kappa phi) (a straight z-vortex),
    plus complex Gaussian noise of amplitude noise * sqrt(mu/c0) (the TF peak
    amplitude), normalised to 1.  Same numbers as gpe_init_state."""
    r = node_positions(lat, params)
    lam = tuple(params.trap_lambda[i] for i in range(3))
    amp = np.sqrt(thomas_fermi_density(r, params.c0, lam))
    phi = np.arctan2(r[..., 1], r[..., 0])
    psi = np.empty(r.shape[:4] + (1, 2))
    psi[..., 0, 0] = amp * np.cos(kappa * phi)
    psi[..., 0, 1] = amp * np.sin(kappa * phi)
    if noise:
        g = gaussian_pairs(seed, psi[..., 0, 0].size).reshape(psi.shape[:4] + (2,))
        psi[..., 0, :] += noise * math.sqrt(tf_mu(params.c0, lam) / params.c0) * g
    return normalize(_embed(psi), lat, params)


def spinor_state(lat, params, zeta, seed=2, noise=1e-3) -> np.ndarray:
    """Spinor sqrt(rho_TF) * zeta plus the reference's relative noise
    psi_m += sqrt(rho) * noise * (g1 + i g2) (Spin1GpeBCC.cu:1272-1285),
    normalised to 1.  zeta: complex vector of length C (|zeta| = 1)."""
    zeta = np.asarray(zeta, dtype=np.complex128)
    C = zeta.size
    r = node_positions(lat, params)
    lam = tuple(params.trap_lambda[i] for i in range(3))
    rho = thomas_fermi_density(r, params.c0, lam)
    amp = np.sqrt(rho)
    psi = np.empty(r.shape[:4] + (C, 2))
    for m in range(C):
        psi[..., m, 0] = amp * zeta[m].real
        psi[..., m, 1] = amp * zeta[m].imag
    if noise:
        g = gaussian_pairs(seed, psi[..., 0].size).reshape(psi.shape)
        psi += noise * amp[..., None, None] * g
    return normalize(_embed(psi), lat, params)


def monopole_state(lat, params, seed=4, noise=1e-3, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Spin-1 hedgehog: at each node the polar spinor (0, 1, 0) rotated so that its
    director points along r_hat = (r - center)/|r - center|, i.e. components
    (m = +1, 0, -1) = (-(n_x - i n_y)/sqrt 2, n_z, (n_x + i n_y)/sqrt 2) for
    n = r_hat (the rotation D^1_{m0}(phi, theta, 0) of |1, 0>), times the
    Thomas-Fermi amplitude, plus seeded complex Gaussian noise of amplitude
    noise * sqrt(rho) per component; normalised to 1.  A target state for the
    ramp-control loss 1 - |<target|psi(T)>|^2."""
    r = node_positions(lat, params) - np.asarray(center, dtype=np.float64)
    lam = tuple(params.trap_lambda[i] for i in range(3))
    rho = thomas_fermi_density(r + np.asarray(center), params.c0, lam)
    amp = np.sqrt(rho)
    d = np.linalg.norm(r, axis=-1)
    safe = np.where(d > 0, d, 1.0)
    nx = np.where(d > 0, r[..., 0] / safe, 0.0)
    ny = np.where(d > 0, r[..., 1] / safe, 0.0)
    nz = np.where(d > 0, r[..., 2] / safe, 1.0)
    s = 1.0 / math.sqrt(2.0)
    psi = np.empty(r.shape[:4] + (3, 2))
    psi[..., 0, 0], psi[..., 0, 1] = -s * nx * amp, s * ny * amp
    psi[..., 1, 0], psi[..., 1, 1] = nz * amp, 0.0
    psi[..., 2, 0], psi[..., 2, 1] = s * nx * amp, s * ny * amp
    if noise:
        g = gaussian_pairs(seed, psi[..., 0].size).reshape(psi.shape)
        psi += noise * amp[..., None, None] * g
    return normalize(_embed(psi), lat, params)


POLAR = (0.0, 1.0, 0.0)                      # spin-1 polar (polarState, Spin1GpeBCC.cu:463-491)
FERRO = (1.0, 0.0, 0.0)                      # spin-1 ferromagnetic (Spin1GpeBCC.cu:493-521)
CYCLIC = (math.sqrt(1 / 3), 0, 0, math.sqrt(2 / 3), 0)  # spin-2 cyclic, phase 0 (Spin2GpeBCC.cu:523-558)


def random_state(shape, seed=7) -> np.ndarray:
    """Uniform random values in [-1, 1) on the interior (zero halo), for parity tests."""
    Z, Y, X = shape[0] - 2, shape[1] - 2, shape[2] - 2
    inner = (Z, Y, X) + tuple(shape[3:])
    v = 2.0 * uniform01(seed, int(np.prod(inner))).reshape(inner) - 1.0
    return _embed(v)


def read_state_file(path, lat: "capi.Lattice", params: "capi.Params", edges: bool = False) -> np.ndarray:
    """A state file of the reference programs: the raw host array of BlockPsis
    (or BlockEdges for q) cells with the one-cell zero halo, x fastest, written with
    ``fs.write`` and read back with ``fs.read`` (Spin1GpeBCC.cu:1215-1237, 1690-1699;
    RelativisticSpin2Gpe.cu:1428-1441, 1695-1706).  Returns the array in the layout
    gpe_upload takes, shape (Z+2, Y+2, X+2, V or E, C, 2).  The file must hold
    exactly that many little-endian doubles."""
    shape = capi.buffer_shape(lat, params, edges)
    data = np.fromfile(path, dtype="<f8")
    if data.size != int(np.prod(shape)):
        raise ValueError("%s holds %d doubles; a (%s) state of this grid has %d" %
                         (path, data.size, ", ".join(map(str, shape)), int(np.prod(shape))))
    return data.reshape(shape).astype(np.float64)


def write_state_file(path, state: np.ndarray) -> None:
    """Writes a state array (the layout gpe_download returns) as the reference's
    raw state file: the same bytes the reference's ``fs.write`` of its host array
    produces, so its programs can load it."""
    np.ascontiguousarray(state, dtype="<f8").tofile(path)
