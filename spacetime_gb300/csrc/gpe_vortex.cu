// gpe_vortex.cu -- the axisymmetric vortex state of a trapped scalar condensate
// (gpe_vortex_profile / gpe_vortex_sample in include/gpe.h): host code.
//
// Psi(r, phi, z) = f(r, z) e^{i kappa phi}, f on a regular (r, z) grid with f = 0
// at r = rmin, solved by the relaxation of the reference's VortexState
// (GrossPitaevskii/VortexState.cpp): Gauss-Seidel sweeps of the discretised
// radial + axial equation (-1/2 Laplacian + kappa^2 / 2r^2 + V + g f^2) f = mu f,
// each sweep followed by the Rayleigh quotient for mu and a renormalisation,
// until the squared change of a sweep falls below eps.  The reference runs it
// once on the host to build the initial state of its CPU stepper; it is a
// sequential recurrence, so it stays on the host here too.  The order of the
// arithmetic follows the reference so that the profile is the same to rounding.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gpe_handle.h"

namespace {

constexpr double kPi = 3.1415926535897932385;  // Types/Types.hpp
constexpr double kTwoPi = 2.0 * kPi;

// The grid of setRange (VortexState.cpp:42-47): sizes rounded to the nearest
// count, steps stretched to fit.
struct VGrid {
    uint32_t rsize, zsize;
    double rplug, rstep, zstep;
};

bool vortex_grid(const gpe_vortex_params* vp, VGrid* g) {
    if (!(vp->rstep > 0) || !(vp->zstep > 0) || !(vp->rmax > vp->rmin) || !(vp->zmax > 0) || !(vp->rmin >= 0))
        return false;
    const double rn = (vp->rmax - vp->rmin) / vp->rstep + 0.5, zn = vp->zmax / vp->zstep + 0.5;
    if (!(rn < 1e7) || !(zn < 1e7)) return false;
    const uint32_t rsize = (uint32_t)rn, zsize = (uint32_t)zn;
    // setDimensions clamps (VortexState.cpp:14-19)
    g->rsize = rsize > 1 ? rsize : 1;
    g->rstep = (vp->rmax - vp->rmin) / (double)rsize;
    if (!(g->rstep > 1e-13)) g->rstep = 1e-13;
    g->rplug = vp->rmin > 0.0 ? vp->rmin : 0.0;
    g->zsize = zsize > 1 ? zsize : 1;
    g->zstep = vp->zmax / (double)zsize;
    if (!(g->zstep > 1e-13)) g->zstep = 1e-13;
    return true;
}

inline double trap_rz(const gpe_vortex_params* vp, double r, double z) {
    return 0.5 * (r * r + vp->trap_ratio * vp->trap_ratio * z * z);  // potentialRZ, GPBlocks.cpp:28-31
}

// f(r, z) by bilinear interpolation, zero outside the grid and |z| mirrored
// (VortexState.cpp:220-236).
double profile_at(const VGrid& g, const double* f, double r, double z) {
    const double rr = (r - g.rplug) / g.rstep;
    if (rr < 0.0) return 0.0;
    const uint32_t ir = (uint32_t)rr;
    if (ir >= g.rsize) return 0.0;
    const double dr = rr - (double)ir;
    const double zz = std::fabs(z) / g.zstep;
    const uint32_t iz = (uint32_t)zz;
    if (iz >= g.zsize) return 0.0;
    const double dz = zz - (double)iz;
    const size_t n = (size_t)g.rsize * g.zsize;
    const size_t ii = (size_t)ir * g.zsize + iz;
    const double fr = ir + 1 < g.rsize ? f[ii + g.zsize] : 0.0;
    const double fz = iz + 1 < g.zsize ? f[ii + 1] : 0.0;
    const double frz = ii + g.zsize + 1 < n ? f[ii + g.zsize + 1] : 0.0;
    return (1.0 - dz) * ((1.0 - dr) * f[ii] + dr * fr) + dz * ((1.0 - dr) * fz + dr * frz);
}

}  // namespace

using namespace gpe;

extern "C" gpe_status gpe_vortex_profile(const gpe_vortex_params* vp, double* f, size_t count, uint32_t* rsize,
                                         uint32_t* zsize, double* mu, uint32_t* iterations) {
    if (!vp) return fail(GPE_ERR_INVALID_ARG, "null parameters");
    VGrid g;
    if (!vortex_grid(vp, &g)) return fail(GPE_ERR_INVALID_ARG, "vortex grid: rmax > rmin >= 0, zmax > 0, steps > 0");
    if (rsize) *rsize = g.rsize;
    if (zsize) *zsize = g.zsize;
    const size_t n = (size_t)g.rsize * g.zsize;
    if (!f) return GPE_OK;  // size query
    if (count < n) return fail(GPE_ERR_INVALID_ARG, "profile array smaller than rsize * zsize");
    if (!std::isfinite(vp->g) || !std::isfinite(vp->trap_ratio)) return fail(GPE_ERR_INVALID_ARG, "g and trap ratio");

    // initial guess (setDimensions, VortexState.cpp:21-38): a smooth bump vanishing
    // at r = rplug, normalised with the volume element 2 pi r dr dz over z >= 0
    // mirrored (rows j > 0 count twice)
    double prob = 0.0;
    for (uint32_t i = 0, ii = 0; i < g.rsize; i++) {
        const double fr = 1.0 - std::cos(i * kTwoPi / (double)g.rsize);
        const double r = g.rplug + i * g.rstep;
        uint32_t times = 1;
        for (uint32_t j = 0; j < g.zsize; j++, ii++) {
            f[ii] = (1.0 + std::cos(j * kPi / (double)g.zsize)) * fr;
            prob += times * f[ii] * f[ii] * r;
            times = 2;
        }
    }
    prob *= kTwoPi * g.rstep * g.zstep;
    {
        const double scale = 1.0 / std::sqrt(prob);
        for (size_t ii = 0; ii < n; ii++) f[ii] *= scale;
    }
    double m = 1.0;

    // relaxation (iterateSolution, VortexState.cpp:109-196)
    const double w2 = kTwoPi * g.rstep * g.zstep;
    const double kk = 0.5 * (double)(vp->kappa * vp->kappa);
    const double laplr = 0.5 / (g.rstep * g.rstep);
    const double laplz = g.zsize > 1 ? 0.5 / (g.zstep * g.zstep) : 0.0;
    const uint32_t Z = g.zsize;
    for (uint32_t j = 0; j < Z; j++) f[j] = 0.0;  // f = 0 at r = rplug
    uint32_t k = 0;
    for (; k < vp->max_iters; k++) {
        double diff = 0.0;
        for (uint32_t i = 1, ii = Z; i < g.rsize; i++) {
            const double r = g.rplug + i * g.rstep;
            const double lapl = kk / (r * r) + 2.0 * (laplr + laplz);
            const double gradr = 0.25 / (r * g.rstep);
            double dv = w2 * r;
            for (uint32_t j = 0; j < Z; j++, ii++) {
                const double pot = trap_rz(vp, r, j * g.zstep) + vp->g * f[ii] * f[ii];
                const double fout = i + 1 < g.rsize ? f[ii + Z] : 0.0;
                const double fin = f[ii - Z];
                const double fup = j + 1 < Z ? f[ii + 1] : 0.0;
                const double fdown = j > 0 ? f[ii - 1] : fup;  // mirror at z = 0
                double d = f[ii];
                f[ii] = (gradr * (fin - fout) - laplr * (fin + fout) - laplz * (fdown + fup)) / (m - lapl - pot);
                d -= f[ii];
                diff += d * d * dv;
                if (j == 0) dv *= 2.0;
            }
        }
        double p1 = 0.0, p2 = 0.0;
        for (uint32_t i = 1, ii = Z; i < g.rsize; i++) {
            const double r = g.rplug + i * g.rstep;
            const double lapl = kk / (r * r) + 2.0 * (laplr + laplz);
            const double gradr = 0.25 / (r * g.rstep);
            double dv = w2 * r;
            for (uint32_t j = 0; j < Z; j++, ii++) {
                const double pot = trap_rz(vp, r, j * g.zstep) + vp->g * f[ii] * f[ii];
                const double fout = i + 1 < g.rsize ? f[ii + Z] : 0.0;
                const double fin = f[ii - Z];
                const double fup = j + 1 < Z ? f[ii + 1] : 0.0;
                const double fdown = j > 0 ? f[ii - 1] : fup;
                p1 += f[ii] * f[ii] * dv;
                p2 += ((pot + lapl) * f[ii] + gradr * (fin - fout) - laplr * (fin + fout) - laplz * (fdown + fup)) * f[ii] *
                      dv;
                if (j == 0) dv *= 2.0;
            }
        }
        m = p2 / p1;
        const double scale = 1.0 / std::sqrt(p1);
        for (size_t ii = Z; ii < n; ii++) f[ii] *= scale;
        if (diff < vp->eps) break;
    }
    // the sign that makes f non-negative on the whole
    double sum = 0.0;
    for (size_t ii = Z; ii < n; ii++) sum += f[ii];
    if (sum < 0.0)
        for (size_t ii = Z; ii < n; ii++) f[ii] = -f[ii];
    if (!std::isfinite(m)) return fail(GPE_ERR_NONFINITE, "vortex relaxation diverged");
    if (mu) *mu = m;
    if (iterations) *iterations = k;
    return GPE_OK;
}

extern "C" gpe_status gpe_vortex_sample(const gpe_vortex_params* vp, const double* f, const gpe_lattice_desc* lat,
                                        const gpe_params* p, double* host, size_t count) {
    if (!vp || !f || !lat || !p || !host) return fail(GPE_ERR_INVALID_ARG, "null argument");
    VGrid g;
    if (!vortex_grid(vp, &g)) return fail(GPE_ERR_INVALID_ARG, "vortex grid: rmax > rmin >= 0, zmax > 0, steps > 0");
    const int V = lat->nodes, C = p->components;
    if (V <= 0 || !lat->pos || (C != 1 && C != 3 && C != 5)) return fail(GPE_ERR_INVALID_ARG, "lattice or components");
    const size_t X = p->dims[0], Y = p->dims[1], Z = p->dims[2];
    const size_t need = (X + 2) * (Y + 2) * (Z + 2) * (size_t)V * C * 2;
    if (count < need) return fail(GPE_ERR_INVALID_ARG, "host array smaller than the file layout of the grid");
    std::memset(host, 0, need * sizeof(double));
    const double bs = p->block_scale;
    for (size_t z = 0; z < Z; z++)
        for (size_t y = 0; y < Y; y++)
            for (size_t x = 0; x < X; x++)
                for (int l = 0; l < V; l++) {
                    // the node's position (GPBlocks.cpp:481), then getPsi (VortexState.cpp:204-212):
                    // f(r, z) times (x + iy)^kappa / r^kappa, zero on the axis
                    const double px = p->p0[0] + bs * (x * lat->block_width[0] + lat->pos[3 * l + 0]);
                    const double py = p->p0[1] + bs * (y * lat->block_width[1] + lat->pos[3 * l + 1]);
                    const double pz = p->p0[2] + bs * (z * lat->block_width[2] + lat->pos[3 * l + 2]);
                    const double r = std::sqrt(px * px + py * py);
                    double re = 0.0, im = 0.0;
                    if (!(r < 1e-30)) {
                        re = profile_at(g, f, r, pz);
                        const double nx = px / r, ny = py / r;
                        for (uint32_t j = 0; j < vp->kappa; j++) {
                            const double t = re * nx - im * ny;
                            im = re * ny + im * nx;
                            re = t;
                        }
                    }
                    double* out = host + ((((z + 1) * (Y + 2) + (y + 1)) * (X + 2) + (x + 1)) * V + l) * (size_t)C * 2;
                    out[0] = re;  // the scalar, or component 0 of a spinor (gpe_respin re-spins it)
                    out[1] = im;
                }
    return GPE_OK;
}
