/*
 * gpe_oracle.c -- FP64 CPU restatement of the reference's per-step kernels.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for libgpe's CUDA kernels and the timed
 * CPU baseline.  Each function follows the reference expression by expression
 * (operation order included) so that differences against the reference are
 * rounding-level only; the reference file:line is given at each function.
 * Build with -ffp-contract=off so that no multiply-add is fused.
 */
#include "gpe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y; } cplx;

static inline cplx c_make(double x, double y) { cplx r = {x, y}; return r; }
static inline cplx c_add(cplx a, cplx b) { return c_make(a.x + b.x, a.y + b.y); }
static inline cplx c_sub(cplx a, cplx b) { return c_make(a.x - b.x, a.y - b.y); }
static inline cplx c_scale(double s, cplx a) { return c_make(s * a.x, s * a.y); }
static inline cplx c_conj(cplx a) { return c_make(a.x, -a.y); }
/* complex product, same operation order as the reference's operator* (utils.h:71-74) */
static inline cplx c_mul(cplx a, cplx b) { return c_make(a.x * b.x - a.y * b.y, a.y * b.x + a.x * b.y); }

/* Constants exactly as the reference spells them (Spin1GpeBCC.cu:91-92). */
#define REF_SQRT_2 1.41421356237309
#define REF_INV_SQRT_2 0.70710678118655

/* ------------------------------------------------------------------ layout */

typedef struct {
    int X, Y, Z, V, C, E;
    size_t cell_vals;   /* doubles per psi cell */
    size_t qcell_vals;  /* doubles per q cell */
} geom;

static geom make_geom(const gpe_lattice_desc* lat, const gpe_params* p) {
    geom g;
    g.X = (int)p->dims[0];
    g.Y = (int)p->dims[1];
    g.Z = (int)p->dims[2];
    g.V = lat->nodes;
    g.C = p->components;
    g.E = lat->edges;
    g.cell_vals = (size_t)g.V * g.C * 2;
    g.qcell_vals = (size_t)g.E * g.C * 2;
    return g;
}

/* index of cell (x,y,z) (interior coordinates, may be -1 or dim) */
static inline size_t cell_index(const geom* g, int x, int y, int z) {
    return ((size_t)(z + 1) * (g->Y + 2) + (size_t)(y + 1)) * (g->X + 2) + (size_t)(x + 1);
}

static inline cplx load_c(const double* buf, size_t cell, size_t cell_vals, int item, int C, int s) {
    const double* v = buf + cell * cell_vals + ((size_t)item * C + s) * 2;
    return c_make(v[0], v[1]);
}

static inline void store_c(double* buf, size_t cell, size_t cell_vals, int item, int C, int s, cplx c) {
    double* v = buf + cell * cell_vals + ((size_t)item * C + s) * 2;
    v[0] = c.x;
    v[1] = c.y;
}

/* globalPos (Spin1GpeBCC.cu:871-874) */
static inline void node_pos(const gpe_lattice_desc* lat, const gpe_params* p, int x, int y, int z, int l,
                            double r[3]) {
    const double* lp = lat->pos + 3 * l;
    r[0] = p->p0[0] + p->block_scale * (x * lat->block_width[0] + lp[0]);
    r[1] = p->p0[1] + p->block_scale * (y * lat->block_width[1] + lp[1]);
    r[2] = p->p0[2] + p->block_scale * (z * lat->block_width[2] + lp[2]);
}

/* trap (Spin1GpeBCC.cu:112-122) */
static inline double trap(const gpe_params* p, const double r[3], double t) {
    if ((p->flags & GPE_FLAG_TRAP_OFF_AFTER) && t >= p->trap_off_time) return 0;
    double x = r[0] * p->trap_lambda[0];
    double y = r[1] * p->trap_lambda[1];
    double z = r[2] * p->trap_lambda[2];
    return 0.5 * (x * x + y * y + z * z) + p->trap_offset;
}

/* magneticField (Spin1GpeBCC.cu:128-142) */
static inline void mag_field(const gpe_params* p, const double r[3], double Bq, const double Bb[3], double B[3]) {
    if (p->flags & GPE_FLAG_QUADRUPOLE_OFFSET) {
        B[0] = Bq * (r[0] - p->quad_center[0]) + Bb[0];
        B[1] = Bq * (r[1] - p->quad_center[1]) + Bb[1];
        B[2] = -2 * Bq * (r[2] - p->quad_center[2]) + Bb[2];
    } else {
        B[0] = Bq * r[0] + Bb[0];
        B[1] = Bq * r[1] + Bb[1];
        B[2] = -2 * Bq * r[2] + Bb[2];
    }
}

/* ---------------------------------------------------- local (non-kinetic) H */

/* H += local terms for spin-1 (Spin1GpeBCC.cu:867-912; itp variant :631-653 uses
 * only c2<F> as B, selected by itp_fields). ps[0..2] = s1, s0, s_1. */
static void local_spin1(const gpe_params* p, const gpe_fields* Bs, const double r[3], double t, int itp_fields,
                        const cplx ps[3], cplx H[3], int allow_loss_qz) {
    const double normSq_s1 = ps[0].x * ps[0].x + ps[0].y * ps[0].y;
    const double normSq_s_1 = ps[2].x * ps[2].x + ps[2].y * ps[2].y;
    const double normSq = normSq_s1 + (ps[1].x * ps[1].x + ps[1].y * ps[1].y) + normSq_s_1;
    cplx totalPot = c_make(trap(p, r, t) + p->c0 * normSq, 0);
    if (allow_loss_qz && (p->flags & GPE_FLAG_THREE_BODY_LOSS)) totalPot.y = -p->alpha * normSq * normSq;
    H[0] = c_add(H[0], c_mul(totalPot, ps[0]));
    H[1] = c_add(H[1], c_mul(totalPot, ps[1]));
    H[2] = c_add(H[2], c_mul(totalPot, ps[2]));

    const cplx magXY = c_scale(REF_SQRT_2, c_add(c_mul(c_conj(ps[0]), ps[1]), c_mul(c_conj(ps[1]), ps[2])));
    double B[3];
    if (itp_fields) {
        B[0] = p->c2 * magXY.x;
        B[1] = p->c2 * magXY.y;
        B[2] = p->c2 * (normSq_s1 - normSq_s_1);
    } else {
        mag_field(p, r, Bs->bq, Bs->bb, B);
        B[0] += p->c2 * magXY.x;
        B[1] += p->c2 * magXY.y;
        B[2] += p->c2 * (normSq_s1 - normSq_s_1);
    }
    cplx Bxy = c_scale(REF_INV_SQRT_2, c_make(B[0], B[1]));
    cplx BxyConj = c_conj(Bxy);
    H[0] = c_add(H[0], c_add(c_scale(B[2], ps[0]), c_mul(BxyConj, ps[1])));
    H[1] = c_add(H[1], c_add(c_mul(Bxy, ps[0]), c_mul(BxyConj, ps[2])));
    H[2] = c_add(H[2], c_sub(c_mul(Bxy, ps[1]), c_scale(B[2], ps[2])));

    if (allow_loss_qz && (p->flags & GPE_FLAG_QUADRATIC_ZEEMAN)) {
        /* Spin1GpeBCC.cu:897-912 */
        double Q[3];
        mag_field(p, r, Bs->bq_quad, Bs->bb_quad, Q);
        Bxy = c_scale(REF_INV_SQRT_2, c_make(Q[0], Q[1]));
        BxyConj = c_conj(Bxy);
        const double BxyNormSq = c_mul(BxyConj, Bxy).x;
        const cplx BxySq = c_mul(Bxy, Bxy);
        const cplx BxyConjSq = c_mul(BxyConj, BxyConj);
        const double BzSq = Q[2] * Q[2];
        const cplx BzBxy = c_scale(Q[2], Bxy);
        const cplx BzBxyConj = c_scale(Q[2], BxyConj);
        H[0] = c_add(H[0], c_add(c_add(c_scale(BzSq + BxyNormSq, ps[0]), c_mul(BzBxyConj, ps[1])), c_mul(BxyConjSq, ps[2])));
        H[1] = c_add(H[1], c_sub(c_add(c_mul(BzBxy, ps[0]), c_scale(2 * BxyNormSq, ps[1])), c_mul(BzBxyConj, ps[2])));
        H[2] = c_add(H[2], c_add(c_sub(c_mul(BxySq, ps[0]), c_mul(BzBxy, ps[1])), c_scale(BzSq + BxyNormSq, ps[2])));
    }
}

/* spin-2 local terms after the kinetic part (Spin2GpeBCC.cu:923-970;
 * RelativisticSpin2Gpe.cu:1068-1125).  ps[0..4] = s2, s1, s0, s_1, s_2.
 * ab.x = trap + c0 rho (computed by the caller so that the hyperbolic c_K can
 * use it first), ab.y = -alpha rho^2 or 0. */
static void local_spin2(const gpe_params* p, const double B[3], cplx ab, const double n[5], const cplx ps[5],
                        cplx H[5]) {
    const double c2 = p->c2, c4 = p->c4;
    const double Fz = c2 * (2.0 * n[0] + n[1] - n[3] - 2.0 * n[4]);
    cplx d[5];
    d[0] = c_add(c_make(2.0 * Fz + 0.4 * c4 * n[4] - 2.0 * B[2], 0), ab);
    d[1] = c_add(c_make(Fz + 0.4 * c4 * n[3] - B[2], 0), ab);
    d[2] = c_add(c_make(0.2 * c4 * n[2], 0), ab);
    d[3] = c_add(c_make(-Fz + 0.4 * c4 * n[1] + B[2], 0), ab);
    d[4] = c_add(c_make(-2.0 * Fz + 0.4 * c4 * n[0] + 2.0 * B[2], 0), ab);
    for (int s = 0; s < 5; ++s) H[s] = c_add(H[s], c_mul(d[s], ps[s]));

    const cplx s2 = ps[0], s1 = ps[1], s0 = ps[2], s_1 = ps[3], s_2 = ps[4];
    const cplx denominator =
        c_sub(c_scale(c2, c_add(c_scale(2.0, c_add(c_mul(s2, c_conj(s1)), c_mul(s_1, c_conj(s_2)))),
                                c_scale(sqrt(6.0), c_add(c_mul(s1, c_conj(s0)), c_mul(s0, c_conj(s_1)))))),
              c_make(B[0], -B[1]));
    const cplx c12 = c_sub(denominator, c_mul(c_scale(0.4 * c4, s_1), c_conj(s_2)));
    const cplx c45 = c_sub(denominator, c_mul(c_scale(0.4 * c4, s2), c_conj(s1)));
    const cplx c13 = c_mul(c_scale(0.2 * c4, s0), c_conj(s_2));
    const cplx c35 = c_mul(c_scale(0.2 * c4, s2), c_conj(s0));
    const cplx c23 = c_sub(c_scale(sqrt(1.5), denominator), c_mul(c_scale(0.2 * c4, s0), c_conj(s_1)));
    const cplx c34 = c_sub(c_scale(sqrt(1.5), denominator), c_mul(c_scale(0.2 * c4, s1), c_conj(s0)));

    H[0] = c_add(H[0], c_add(c_mul(c12, s1), c_mul(c13, s0)));
    H[1] = c_add(H[1], c_add(c_mul(c_conj(c12), s2), c_mul(c23, s0)));
    H[2] = c_add(H[2], c_add(c_add(c_add(c_mul(c_conj(c13), s2), c_mul(c35, s_2)), c_mul(c34, s_1)), c_mul(c_conj(c23), s1)));
    H[3] = c_add(H[3], c_add(c_mul(c_conj(c34), s0), c_mul(c45, s_2)));
    H[4] = c_add(H[4], c_add(c_mul(c_conj(c35), s0), c_mul(c_conj(c45), s_1)));
}

static void spin2_norms(const cplx ps[5], double n[5], double* normSq) {
    for (int s = 0; s < 5; ++s) n[s] = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
    *normSq = n[0] + n[1] + n[2] + n[3] + n[4];
}

/* Apply the step update to one node (Spin1GpeBCC.cu:914-916, :788-790, :655-661). */
static void write_update(const geom* g, int mode, double dt, double* next, double* hpsi, size_t cell, int l,
                         const cplx* prev, const cplx* H) {
    for (int s = 0; s < g->C; ++s) {
        if (mode == ORC_LEAPFROG) {
            cplx n0 = load_c(next, cell, g->cell_vals, l, g->C, s);
            n0 = c_add(n0, c_scale(2 * dt, c_make(H[s].y, -H[s].x)));
            store_c(next, cell, g->cell_vals, l, g->C, s, n0);
        } else if (mode == ORC_EULER) {
            store_c(next, cell, g->cell_vals, l, g->C, s, c_add(prev[s], c_scale(dt, c_make(H[s].y, -H[s].x))));
        } else {
            if (hpsi) store_c(hpsi, cell, g->cell_vals, l, g->C, s, H[s]);
            store_c(next, cell, g->cell_vals, l, g->C, s, c_sub(prev[s], c_scale(dt, H[s])));
        }
    }
}

static int check_args(const gpe_lattice_desc* lat, const gpe_params* p) {
    if (!lat || !p) return GPE_ERR_INVALID_ARG;
    if (p->components != 1 && p->components != 3 && p->components != 5) return GPE_ERR_INVALID_ARG;
    if (p->dims[0] == 0 || p->dims[1] == 0 || p->dims[2] == 0) return GPE_ERR_INVALID_ARG;
    return GPE_OK;
}

static int nthreads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

/* ------------------------------------------------------------- parabolic step */

int orc_parabolic_step(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* Bs, double t,
                       int mode, double* next, const double* prev, double* hpsi, int threads) {
    int st = check_args(lat, p);
    if (st) return st;
    const geom g = make_geom(lat, p);
    const int C = g.C;
    const double bs2 = p->block_scale * p->block_scale;
    const int nt = nthreads(threads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int z = 0; z < g.Z; ++z) {
        for (int y = 0; y < g.Y; ++y) {
            for (int x = 0; x < g.X; ++x) {
                const size_t cell = cell_index(&g, x, y, z);
                for (int l = 0; l < g.V; ++l) {
                    cplx prv[5], H[5];
                    for (int s = 0; s < C; ++s) {
                        prv[s] = load_c(prev, cell, g.cell_vals, l, C, s);
                        H[s] = c_make(0, 0);
                    }
                    /* Laplacian (Spin1GpeBCC.cu:835-865; GPUGrossPitaevskii_BCC.cu:192-196) */
                    for (int f = lat->row_ptr[l]; f < lat->row_ptr[l + 1]; ++f) {
                        const gpe_stencil_entry* e = &lat->stencil[f];
                        const size_t ncell = cell_index(&g, x + e->dx, y + e->dy, z + e->dz);
                        const double hodge = (-0.5 * e->hodge) / bs2;
                        for (int s = 0; s < C; ++s) {
                            const cplx nb = load_c(prev, ncell, g.cell_vals, e->node, C, s);
                            H[s] = c_add(H[s], c_scale(hodge, c_sub(nb, prv[s])));
                        }
                    }
                    double r[3];
                    node_pos(lat, p, x, y, z, l, r);
                    if (C == 1) {
                        /* GPUGrossPitaevskii_BCC.cu:198-199 */
                        const double normsq = prv[0].x * prv[0].x + prv[0].y * prv[0].y;
                        cplx tp = c_make(trap(p, r, t) + p->c0 * normsq, 0);
                        if ((p->flags & GPE_FLAG_THREE_BODY_LOSS) && mode != ORC_ITP) tp.y = -p->alpha * normsq * normsq;
                        H[0] = c_add(H[0], c_mul(tp, prv[0]));
                    } else if (C == 3) {
                        local_spin1(p, Bs, r, t, mode == ORC_ITP, prv, H, mode != ORC_ITP);
                    } else {
                        double n[5], normSq, B[3];
                        spin2_norms(prv, n, &normSq);
                        cplx ab = c_make(trap(p, r, t) + p->c0 * normSq, 0);
                        if (p->flags & GPE_FLAG_THREE_BODY_LOSS) ab.y = -p->alpha * normSq * normSq;
                        if (mode == ORC_ITP) {
                            B[0] = B[1] = B[2] = 0;
                        } else {
                            mag_field(p, r, Bs->bq, Bs->bb, B);
                        }
                        local_spin2(p, B, ab, n, prv, H);
                    }
                    write_update(&g, mode, p->dt, next, hpsi, cell, l, prv, H);
                }
            }
        }
    }
    return GPE_OK;
}

/* --------------------------------------------------------- q-based psi step */

int orc_q_psi_step(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* Bs, double t, int mode,
                   int hyperb, double* next, const double* prev, const double* q, double* hpsi, int threads) {
    int st = check_args(lat, p);
    if (st) return st;
    if (lat->edges <= 0 || !lat->incidence) return GPE_ERR_UNSUPPORTED;
    const geom g = make_geom(lat, p);
    const int C = g.C;
    const int F = lat->faces_per_node;
    const double bs2 = p->block_scale * p->block_scale;
    const int nt = nthreads(threads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int z = 0; z < g.Z; ++z) {
        for (int y = 0; y < g.Y; ++y) {
            for (int x = 0; x < g.X; ++x) {
                const size_t cell = cell_index(&g, x, y, z);
                for (int l = 0; l < g.V; ++l) {
                    cplx prv[5], H[5];
                    for (int s = 0; s < C; ++s) {
                        prv[s] = load_c(prev, cell, g.cell_vals, l, C, s);
                        H[s] = c_make(0, 0);
                    }
                    /* d1 of q (RelativisticSpin2Gpe.cu:1051-1066) */
                    for (int k = 0; k < F; ++k) {
                        const gpe_incidence* e = &lat->incidence[l * F + k];
                        const size_t qcell = cell_index(&g, x + e->dx, y + e->dy, z + e->dz);
                        const double hodge = (-0.5 * e->hodge) / bs2;
                        for (int s = 0; s < C; ++s) {
                            const cplx qv = load_c(q, qcell, g.qcell_vals, e->edge, C, s);
                            H[s] = c_add(H[s], c_scale(hodge, qv));
                        }
                    }
                    double r[3];
                    node_pos(lat, p, x, y, z, l, r);
                    const double tr = trap(p, r, t);
                    if (C == 1) {
                        /* RelativisticGpeBCC.cu:244-253 */
                        const double normsq = c_mul(c_conj(prv[0]), prv[0]).x;
                        const double totalPot = tr + p->c0 * normsq;
                        if (hyperb) {
                            const double c_K = 1 + p->sigma * totalPot;
                            H[0] = c_scale(-c_K, H[0]);
                        }
                        H[0] = c_add(H[0], c_scale(totalPot, prv[0]));
                    } else if (C == 3) {
                        /* RelativisticSpin1Gpe/common_kernels.h:218-250 */
                        const double normSq_s1 = prv[0].x * prv[0].x + prv[0].y * prv[0].y;
                        const double normSq_s_1 = prv[2].x * prv[2].x + prv[2].y * prv[2].y;
                        const double normSq = normSq_s1 + (prv[1].x * prv[1].x + prv[1].y * prv[1].y) + normSq_s_1;
                        const cplx totalPot = c_make(tr + p->c0 * normSq, 0);
                        if (hyperb) {
                            const double c_K = 1 + p->sigma * totalPot.x;
                            for (int s = 0; s < 3; ++s) H[s] = c_scale(-c_K, H[s]);
                        }
                        for (int s = 0; s < 3; ++s) H[s] = c_add(H[s], c_mul(totalPot, prv[s]));
                        const cplx magXY = c_scale(REF_SQRT_2, c_add(c_mul(c_conj(prv[0]), prv[1]), c_mul(c_conj(prv[1]), prv[2])));
                        double B[3];
                        if (mode == ORC_ITP) {
                            B[0] = B[1] = B[2] = 0;
                        } else {
                            mag_field(p, r, Bs->bq, Bs->bb, B);
                        }
                        B[0] += p->c2 * magXY.x;
                        B[1] += p->c2 * magXY.y;
                        B[2] += p->c2 * (normSq_s1 - normSq_s_1);
                        const cplx Bxy = c_scale(REF_INV_SQRT_2, c_make(B[0], B[1]));
                        const cplx BxyConj = c_conj(Bxy);
                        H[0] = c_add(H[0], c_add(c_scale(B[2], prv[0]), c_mul(BxyConj, prv[1])));
                        H[1] = c_add(H[1], c_add(c_mul(Bxy, prv[0]), c_mul(BxyConj, prv[2])));
                        H[2] = c_add(H[2], c_sub(c_mul(Bxy, prv[1]), c_scale(B[2], prv[2])));
                    } else {
                        /* RelativisticSpin2Gpe.cu:1068-1125 */
                        double n[5], normSq, B[3];
                        spin2_norms(prv, n, &normSq);
                        const cplx ab = c_make(tr + p->c0 * normSq, 0);
                        if (hyperb) {
                            const double c_K = 1 + p->sigma * ab.x;
                            for (int s = 0; s < 5; ++s) H[s] = c_scale(-c_K, H[s]);
                        }
                        if (mode == ORC_ITP) {
                            B[0] = B[1] = B[2] = 0;
                        } else {
                            mag_field(p, r, Bs->bq, Bs->bb, B);
                        }
                        local_spin2(p, B, ab, n, prv, H);
                    }
                    write_update(&g, mode, p->dt, next, hpsi, cell, l, prv, H);
                }
            }
        }
    }
    return GPE_OK;
}

/* ----------------------------------------------------------------- q step */

int orc_q_step(const gpe_lattice_desc* lat, const gpe_params* p, int qmode, double* next_q, const double* prev_q,
               const double* psi, int threads) {
    int st = check_args(lat, p);
    if (st) return st;
    if (lat->edges <= 0 || !lat->edge_table) return GPE_ERR_UNSUPPORTED;
    const geom g = make_geom(lat, p);
    const int C = g.C;
    const double dt_per_sigma = p->dt / p->sigma;
    const int nt = nthreads(threads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int z = 0; z < g.Z; ++z) {
        for (int y = 0; y < g.Y; ++y) {
            for (int x = 0; x < g.X; ++x) {
                const size_t cell = cell_index(&g, x, y, z);
                for (int e = 0; e < g.E; ++e) {
                    const gpe_edge* d0 = &lat->edge_table[e];
                    const size_t ocell = cell_index(&g, x + d0->dx, y + d0->dy, z + d0->dz);
                    for (int s = 0; s < C; ++s) {
                        /* RelativisticSpin2Gpe.cu:988-995 */
                        const cplx thisPsi = load_c(psi, cell, g.cell_vals, d0->from, C, s);
                        const cplx otherPsi = load_c(psi, ocell, g.cell_vals, d0->to, C, s);
                        const cplx d0psi = c_sub(otherPsi, thisPsi);
                        if (qmode == ORC_Q_PARA) {
                            store_c(next_q, cell, g.qcell_vals, e, C, s, d0psi);
                        } else if (qmode == ORC_Q_HYPER) {
                            /* :1004-1014 */
                            const cplx pq = load_c(prev_q, cell, g.qcell_vals, e, C, s);
                            const cplx qq = c_scale(2 * dt_per_sigma, c_add(pq, d0psi));
                            cplx nq = load_c(next_q, cell, g.qcell_vals, e, C, s);
                            nq = c_add(nq, c_make(-qq.y, qq.x));
                            store_c(next_q, cell, g.qcell_vals, e, C, s, nq);
                        } else if (qmode == ORC_Q_ITP) {
                            /* itp_q, :589-599: q = (dt/sigma)(-d0 psi + prev_q); next_q = prev_q - q */
                            const cplx pq = load_c(prev_q, cell, g.qcell_vals, e, C, s);
                            const cplx qq = c_scale(dt_per_sigma, c_add(c_scale(-1.0, d0psi), pq));
                            store_c(next_q, cell, g.qcell_vals, e, C, s, c_sub(pq, qq));
                        } else {
                            /* forwardEuler_q, :841-851 */
                            const cplx pq = load_c(prev_q, cell, g.qcell_vals, e, C, s);
                            const cplx qq = c_scale(dt_per_sigma, c_add(pq, d0psi));
                            store_c(next_q, cell, g.qcell_vals, e, C, s, c_add(pq, c_make(-qq.y, qq.x)));
                        }
                    }
                }
            }
        }
    }
    return GPE_OK;
}

/* ------------------------------------------------------------ node fields */

/* Per-node output fields, interior nodes in the reference's order
 * idx = V (z X Y + y X + x) + l, GPE_FIELD_* values per node (see gpe.h).
 * DENSITY: density kernels (Spin1GpeBCC.cu:191-211, Spin2GpeBCC.cu:192-212).
 * SPIN: localAvgSpinAndDensity (Spin1GpeBCC.cu:235-271; Spin2GpeBCC.cu:214-254,
 *   which applies the spin-1 formula to s1, s0, s_1): psi normalised by sqrt(rho)
 *   for x, y, while z = |s1|^2 - |s_1|^2 of the unnormalised psi, as there.
 * UV_THETA: uvTheta (Spin1GpeBCC.cu:273-326, theta wrapped into [0, pi);
 *   Spin2GpeBCC.cu:256-306 on s1, s0, s_1, unwrapped).
 * MAX_HAMILTON: maxHamilton (Spin1GpeBCC.cu:144-189), field without quadrupole offset.
 * PROJ_X / PROJ_Y: |components|^2 in the x- / y-quantised basis (Spin1GpeBCC/utils.h:177-193). */
int orc_node_fields(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* Bs, double t, int kind,
                    const double* psi, double* out) {
    int st = check_args(lat, p);
    if (st) return st;
    const int C = p->components;
    const int per = kind == GPE_FIELD_DENSITY ? 1 : kind == GPE_FIELD_SPIN ? 5 : kind == GPE_FIELD_UV_THETA ? 7
                  : kind == GPE_FIELD_MAX_HAMILTON ? 1 : (kind == GPE_FIELD_PROJ_X || kind == GPE_FIELD_PROJ_Y) ? 3 : 0;
    if (per == 0) return GPE_ERR_INVALID_ARG;
    if ((kind == GPE_FIELD_SPIN || kind == GPE_FIELD_UV_THETA) && C == 1) return GPE_ERR_UNSUPPORTED;
    if ((kind == GPE_FIELD_MAX_HAMILTON || kind == GPE_FIELD_PROJ_X || kind == GPE_FIELD_PROJ_Y) && C != 3)
        return GPE_ERR_UNSUPPORTED;
    const geom g = make_geom(lat, p);
    const int o = C == 5 ? 1 : 0; /* s1, s0, s_1 */
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                const size_t cell = cell_index(&g, x, y, z);
                for (int l = 0; l < g.V; ++l) {
                    const size_t idx = (size_t)g.V * (((size_t)z * g.Y + y) * g.X + x) + l;
                    double* v = out + idx * per;
                    cplx ps[5];
                    double rho = 0;
                    for (int s = 0; s < C; ++s) {
                        ps[s] = load_c(psi, cell, g.cell_vals, l, C, s);
                        rho += ps[s].x * ps[s].x + ps[s].y * ps[s].y;
                    }
                    if (kind == GPE_FIELD_DENSITY) {
                        v[0] = rho;
                    } else if (kind == GPE_FIELD_SPIN) {
                        const double n1 = ps[o].x * ps[o].x + ps[o].y * ps[o].y;
                        const double nm1 = ps[o + 2].x * ps[o + 2].x + ps[o + 2].y * ps[o + 2].y;
                        const double sq = sqrt(rho);
                        const cplx a = c_make(ps[o].x / sq, ps[o].y / sq);
                        const cplx b = c_make(ps[o + 1].x / sq, ps[o + 1].y / sq);
                        const cplx c = c_make(ps[o + 2].x / sq, ps[o + 2].y / sq);
                        const cplx tmp = c_scale(REF_SQRT_2, c_add(c_mul(c_conj(a), b), c_mul(c_conj(b), c)));
                        const double sz = n1 - nm1;
                        v[0] = rho * sqrt(tmp.x * tmp.x + tmp.y * tmp.y + sz * sz);
                        v[1] = tmp.x;
                        v[2] = tmp.y;
                        v[3] = sz;
                        v[4] = rho;
                    } else if (kind == GPE_FIELD_UV_THETA) {
                        const cplx s1 = ps[o], s0 = ps[o + 1], sm1 = ps[o + 2];
                        const cplx ax = c_make((sm1.x - s1.x) / REF_SQRT_2, (sm1.y - s1.y) / REF_SQRT_2);
                        const cplx sum = c_add(sm1, s1);
                        const cplx ay = c_make(sum.y / REF_SQRT_2, -sum.x / REF_SQRT_2); /* -i (s_1 + s1) / sqrt2 */
                        const double m[3] = {ax.x, ay.x, s0.x}, n[3] = {ax.y, ay.y, s0.y};
                        const double mn = m[0] * n[0] + m[1] * n[1] + m[2] * n[2];
                        const double mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
                        const double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
                        double th = atan2(-2 * mn, mm - nn) / 2;
                        if (C == 3 && th < 0) th += 3.1415926535897932385;
                        const double sn = sin(th), cs = cos(th);
                        double u[3], w[3];
                        for (int k = 0; k < 3; ++k) {
                            u[k] = m[k] * cs - sn * n[k];
                            w[k] = m[k] * sn + cs * n[k];
                        }
                        const double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
                        const double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
                        const double* first = un >= wn ? u : w;
                        const double* second = un >= wn ? w : u;
                        for (int k = 0; k < 3; ++k) {
                            v[k] = first[k];
                            v[3 + k] = second[k];
                        }
                        v[6] = th;
                    } else if (kind == GPE_FIELD_MAX_HAMILTON) {
                        double r[3];
                        node_pos(lat, p, x, y, z, l, r);
                        const double n1 = ps[0].x * ps[0].x + ps[0].y * ps[0].y;
                        const double nm1 = ps[2].x * ps[2].x + ps[2].y * ps[2].y;
                        const double pot = trap(p, r, t) + p->c0 * rho;
                        const cplx tmp = c_scale(REF_SQRT_2, c_add(c_mul(c_conj(ps[0]), ps[1]), c_mul(c_conj(ps[1]), ps[2])));
                        double B[3] = {Bs->bq * r[0] + Bs->bb[0], Bs->bq * r[1] + Bs->bb[1], -2 * Bs->bq * r[2] + Bs->bb[2]};
                        B[0] += p->c2 * tmp.x;
                        B[1] += p->c2 * tmp.y;
                        B[2] += p->c2 * (n1 - nm1);
                        const double hx = pot + fabs(REF_INV_SQRT_2 * B[0]);
                        const double hy = pot + fabs(REF_INV_SQRT_2 * B[1]);
                        const double hz = pot + fabs(B[2]);
                        v[0] = fmax(hx, fmax(hy, hz));
                    } else {
                        const cplx s1 = ps[0], s0 = ps[1], sm1 = ps[2];
                        const double r2 = sqrt(2.0);
                        cplx q[3];
                        if (kind == GPE_FIELD_PROJ_X) {
                            q[0] = c_sub(c_scale(0.5, c_add(s1, sm1)), c_make(s0.x / r2, s0.y / r2));
                            q[1] = c_make((s1.x - sm1.x) / r2, (s1.y - sm1.y) / r2);
                            q[2] = c_add(c_scale(0.5, c_add(sm1, s1)), c_make(s0.x / r2, s0.y / r2));
                        } else {
                            const cplx ms0 = c_mul(s0, c_make(0, -1)); /* s0 (0, -1) */
                            const cplx ms = c_mul(c_add(s1, sm1), c_make(0, -1));
                            q[0] = c_add(c_scale(0.5, c_sub(s1, sm1)), c_make(ms0.x / r2, ms0.y / r2));
                            q[1] = c_make(ms.x / r2, ms.y / r2);
                            q[2] = c_add(c_scale(0.5, c_sub(sm1, s1)), c_make(ms0.x / r2, ms0.y / r2));
                        }
                        for (int k = 0; k < 3; ++k) v[k] = q[k].x * q[k].x + q[k].y * q[k].y;
                    }
                }
            }
    return GPE_OK;
}

/* ------------------------------------------------------- split scheme (C15) */

/* RelativisticGpeC15/GPUGrossPitaevskii_C15.cu: psi = R + iI, q = q_R + i q_I stored
 * as complex pairs.  The reference folds dt into the potential, g and the Hodge
 * weights (:282-286) and updates next += sign ((pot + g (prev^2 + next^2)) prev - d1q)
 * (update_psi :116-155) and next_q += sign dts (prev_q + d0 psi) (update_q :90-114);
 * the time loop (:477-482) is part 0 = (I, q_I) from (R, q_R) with sign -1 / +1 and
 * part 1 = (R, q_R) from (I, q_I) with sign +1 / -1; part 2 is the start (:469),
 * q_R += c (q_R + d0 R) with c = dts / (dt - dts). */
int orc_split_step(const gpe_lattice_desc* lat, const gpe_params* p, int part, double* psi, double* q, int threads) {
    int st = check_args(lat, p);
    if (st) return st;
    if (p->components != 1 || lat->edges <= 0 || !lat->incidence || !lat->edge_table) return GPE_ERR_UNSUPPORTED;
    if (part < 0 || part > 2) return GPE_ERR_INVALID_ARG;
    const geom g = make_geom(lat, p);
    const int F = lat->faces_per_node;
    const double dt = p->dt;
    const double dts = p->dt / p->sigma;
    const double bs2 = p->block_scale * p->block_scale;
    const double gdt = p->c0 * dt;
    const int rd = part == 1 ? 1 : 0; /* the half read: 0 = R / q_R, 1 = I / q_I */
    const int wr = 1 - rd;
    const int nt = nthreads(threads);
    (void)nt;
    if (part != 2) {
        const double sign = part == 0 ? -1.0 : 1.0;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int z = 0; z < g.Z; ++z)
            for (int y = 0; y < g.Y; ++y)
                for (int x = 0; x < g.X; ++x) {
                    const size_t cell = cell_index(&g, x, y, z);
                    for (int l = 0; l < g.V; ++l) {
                        double* own = psi + cell * g.cell_vals + 2 * l;
                        double d1q = 0;
                        for (int k = 0; k < F; ++k) {
                            const gpe_incidence* e = &lat->incidence[l * F + k];
                            const size_t qcell = cell_index(&g, x + e->dx, y + e->dy, z + e->dz);
                            const double hodge = -0.5 * e->hodge / bs2 * dt;
                            d1q += hodge * q[qcell * g.qcell_vals + 2 * e->edge + rd];
                        }
                        double r[3];
                        node_pos(lat, p, x, y, z, l, r);
                        const double pot = trap(p, r, 0.0) * dt;
                        const double prev = own[rd];
                        double next = own[wr];
                        const double normsq = prev * prev + next * next;
                        next += sign * ((pot + gdt * normsq) * prev - d1q);
                        own[wr] = next;
                    }
                }
    }
    const double qsign = part == 1 ? -1.0 : 1.0;
    const double coef = part == 2 ? dts / (dt - dts) : dts;
    const int qwr = part == 2 ? 0 : wr;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                const size_t cell = cell_index(&g, x, y, z);
                for (int e = 0; e < g.E; ++e) {
                    const gpe_edge* d0 = &lat->edge_table[e];
                    const size_t ocell = cell_index(&g, x + d0->dx, y + d0->dy, z + d0->dz);
                    const double d0psi = psi[ocell * g.cell_vals + 2 * d0->to + rd] - psi[cell * g.cell_vals + 2 * d0->from + rd];
                    double* qv = q + cell * g.qcell_vals + 2 * e;
                    qv[qwr] += qsign * coef * (qv[rd] + d0psi);
                }
            }
    return GPE_OK;
}

/* ------------------------------------------------------------ reductions */

static double cell_volume(const gpe_lattice_desc* lat, const gpe_params* p) {
    /* volume = bs^3 * VOLUME (Spin1GpeBCC.cu:1385) */
    return p->block_scale * p->block_scale * p->block_scale * lat->volume;
}

double orc_normalize(const gpe_lattice_desc* lat, const gpe_params* p, double* psi) {
    const geom g = make_geom(lat, p);
    const double dv = cell_volume(lat, p);
    double sum = 0;
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                const double* c = psi + cell_index(&g, x, y, z) * g.cell_vals;
                for (size_t i = 0; i < g.cell_vals; ++i) sum += c[i] * c[i];
            }
    const double norm = sum * dv;
    const double sq = sqrt(norm);
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                double* c = psi + cell_index(&g, x, y, z) * g.cell_vals;
                for (size_t i = 0; i < g.cell_vals; ++i) c[i] = c[i] / sq;
            }
    return norm;
}

/* Local H of one node with kinetic part zero; used for the energy split. */
static void local_h(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* Bs, const double r[3],
                    double t, int C, const cplx* ps, cplx* H, int with_external) {
    for (int s = 0; s < C; ++s) H[s] = c_make(0, 0);
    gpe_params q = *p;
    gpe_fields zero;
    memset(&zero, 0, sizeof zero);
    if (!with_external) {
        q.trap_lambda[0] = q.trap_lambda[1] = q.trap_lambda[2] = 0;
        q.trap_offset = 0;
        q.flags &= ~(GPE_FLAG_QUADRATIC_ZEEMAN | GPE_FLAG_THREE_BODY_LOSS | GPE_FLAG_QUADRUPOLE_OFFSET);
        Bs = &zero;
    }
    (void)lat;
    if (C == 1) {
        const double normsq = ps[0].x * ps[0].x + ps[0].y * ps[0].y;
        H[0] = c_scale(trap(&q, r, t) + q.c0 * normsq, ps[0]);
    } else if (C == 3) {
        local_spin1(&q, Bs, r, t, 0, ps, H, 1);
    } else {
        double n[5], normSq, B[3];
        spin2_norms(ps, n, &normSq);
        mag_field(&q, r, Bs->bq, Bs->bb, B);
        local_spin2(&q, B, c_make(trap(&q, r, t) + q.c0 * normSq, 0), n, ps, H);
    }
}

int orc_observe(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* Bs, double t, const double* psi,
                gpe_observables* out) {
    int st = check_args(lat, p);
    if (st) return st;
    const geom g = make_geom(lat, p);
    const int C = g.C;
    const double dv = cell_volume(lat, p);
    const double bs2 = p->block_scale * p->block_scale;
    double norm = 0, hexp = 0, eint = 0, kin = 0, mag[3] = {0, 0, 0}, spin = 0, com[3] = {0, 0, 0}, maxabs = 0;
    int nonfinite = 0;
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                const size_t cell = cell_index(&g, x, y, z);
                for (int l = 0; l < g.V; ++l) {
                    cplx ps[5], L[5], Hl[5], Hn[5];
                    double rho = 0;
                    for (int s = 0; s < C; ++s) {
                        ps[s] = load_c(psi, cell, g.cell_vals, l, C, s);
                        L[s] = c_make(0, 0);
                        const double a = sqrt(ps[s].x * ps[s].x + ps[s].y * ps[s].y);
                        if (!isfinite(ps[s].x) || !isfinite(ps[s].y)) nonfinite++;
                        if (a > maxabs) maxabs = a;
                        rho += ps[s].x * ps[s].x + ps[s].y * ps[s].y;
                    }
                    for (int f = lat->row_ptr[l]; f < lat->row_ptr[l + 1]; ++f) {
                        const gpe_stencil_entry* e = &lat->stencil[f];
                        const size_t ncell = cell_index(&g, x + e->dx, y + e->dy, z + e->dz);
                        const double hodge = (-0.5 * e->hodge) / bs2;
                        for (int s = 0; s < C; ++s)
                            L[s] = c_add(L[s], c_scale(hodge, c_sub(load_c(psi, ncell, g.cell_vals, e->node, C, s), ps[s])));
                    }
                    double r[3];
                    node_pos(lat, p, x, y, z, l, r);
                    local_h(lat, p, Bs, r, t, C, ps, Hl, 1);
                    local_h(lat, p, Bs, r, t, C, ps, Hn, 0);
                    double k = 0, hl = 0, hn = 0;
                    for (int s = 0; s < C; ++s) {
                        k += ps[s].x * L[s].x + ps[s].y * L[s].y;
                        hl += ps[s].x * Hl[s].x + ps[s].y * Hl[s].y;
                        hn += ps[s].x * Hn[s].x + ps[s].y * Hn[s].y;
                    }
                    kin += k;
                    hexp += k + hl;
                    eint += hn;
                    norm += rho;
                    com[0] += rho * r[0];
                    com[1] += rho * r[1];
                    com[2] += rho * r[2];
                    if (C == 3) {
                        const cplx m = c_scale(REF_SQRT_2, c_add(c_mul(c_conj(ps[0]), ps[1]), c_mul(c_conj(ps[1]), ps[2])));
                        const double fz = (ps[0].x * ps[0].x + ps[0].y * ps[0].y) - (ps[2].x * ps[2].x + ps[2].y * ps[2].y);
                        mag[0] += m.x;
                        mag[1] += m.y;
                        mag[2] += fz;
                        spin += sqrt(m.x * m.x + m.y * m.y + fz * fz);
                    } else if (C == 5) {
                        /* F+ = 2(s2* s1 + s_1* s_2) + sqrt6 (s1* s0 + s0* s_1), Fz = sum m |s_m|^2 */
                        const cplx fp = c_add(c_scale(2.0, c_add(c_mul(c_conj(ps[0]), ps[1]), c_mul(c_conj(ps[3]), ps[4]))),
                                              c_scale(sqrt(6.0), c_add(c_mul(c_conj(ps[1]), ps[2]), c_mul(c_conj(ps[2]), ps[3]))));
                        double n[5], ns;
                        spin2_norms(ps, n, &ns);
                        const double fz = 2 * n[0] + n[1] - n[3] - 2 * n[4];
                        mag[0] += fp.x;
                        mag[1] += fp.y;
                        mag[2] += fz;
                        spin += sqrt(fp.x * fp.x + fp.y * fp.y + fz * fz);
                    }
                }
            }
    memset(out, 0, sizeof *out);
    out->norm = norm * dv;
    out->h_expect = hexp * dv;
    out->energy = (hexp - 0.5 * eint) * dv;
    out->magnetization[0] = mag[0] * dv;
    out->magnetization[1] = mag[1] * dv;
    out->magnetization[2] = mag[2] * dv;
    out->spin_norm = spin * dv;
    out->com[0] = com[0] * dv;
    out->com[1] = com[1] * dv;
    out->com[2] = com[2] * dv;
    out->max_abs = maxabs;
    out->nonfinite = nonfinite;
    (void)kin;
    return GPE_OK;
}

/* ---------------------------------------------------------------- ramps */

void orc_ramp_eval(const gpe_ramp* r, double tau, gpe_fields* out) {
    /* getSignal (AliceRingRamps.h:74-141): walk the segment durations */
    double Bq = 0, Bb[3] = {0, 0, 0};
    {
        double t = tau;
        int k = 0;
        for (; k < r->bq_segments; ++k) {
            const double tin = t - r->bq_duration[k];
            if (tin < 0) break;
            t = tin;
        }
        if (k >= r->bq_segments) k = r->bq_segments - 1, t = r->bq_duration[k];
        if (k >= 0) {
            const double prev = k > 0 ? r->bq_target[k - 1] : 0.0;
            if (r->bq_type[k] == GPE_RAMP_CONSTANT) Bq = r->bq_target[k];
            else if (r->bq_type[k] == GPE_RAMP_LINEAR) Bq = prev + t * (r->bq_target[k] - prev) / r->bq_duration[k];
            else Bq = prev + (r->bq_target[k] - prev) * sqrt(t / r->bq_duration[k]);
        }
    }
    {
        double t = tau;
        int k = 0;
        for (; k < r->bb_segments; ++k) {
            const double tin = t - r->bb_duration[k];
            if (tin < 0) break;
            t = tin;
        }
        if (k >= r->bb_segments) k = r->bb_segments - 1, t = r->bb_duration[k];
        if (k >= 0) {
            for (int a = 0; a < 3; ++a) {
                const double prev = k > 0 ? r->bb_target[k - 1][a] : 0.0;
                if (r->bb_type[k] == GPE_RAMP_CONSTANT) Bb[a] = r->bb_target[k][a];
                else if (r->bb_type[k] == GPE_RAMP_LINEAR) Bb[a] = prev + t * (r->bb_target[k][a] - prev) / r->bb_duration[k];
                else Bb[a] = prev + (r->bb_target[k][a] - prev) * sqrt(t / r->bb_duration[k]);
            }
        }
    }
    /* Bs.Bq = BqScale * signal.Bq etc. (Spin1GpeBCC.cu:1583-1587) */
    out->bq = r->bq_scale * Bq;
    out->bq_quad = r->bq_quad_scale * Bq;
    for (int a = 0; a < 3; ++a) {
        out->bb[a] = r->bb_scale * Bb[a];
        out->bb_quad[a] = r->bb_quad_scale * Bb[a];
    }
}

/* ------------------------------------------------------------- GPBlocks */

void orc_gpblocks_run(int X, int Y, int Z, int V, int deg, const int64_t* lapind, double lapfac, double lapfac0,
                      double g, const double* pot, double* even, double* odd, int steps) {
    const size_t bsize = (size_t)V;
    const size_t bxsize = (size_t)(X + 1) * bsize;
    const size_t bxysize = (size_t)(Y + 1) * bxsize;
    const size_t ii0 = bxysize + bxsize + bsize;
    for (int step = 0; step < steps; ++step) {
        for (int pass = 0; pass < 2; ++pass) {
            /* pass 0: odd <- even; pass 1: even <- odd (GPBlocks.cpp:562-605) */
            const double* src = pass == 0 ? even : odd;
            double* dst = pass == 0 ? odd : even;
            for (int k = 0; k < Z; ++k)
                for (int j = 0; j < Y; ++j)
                    for (int i = 0; i < X; ++i) {
                        const size_t ii = ii0 + k * bxysize + j * bxsize + i * bsize;
                        size_t lapi = 0, lapimax = 0;
                        for (size_t l = 0; l < bsize; ++l) {
                            const size_t jj = ii + l;
                            lapimax += deg;
                            const int64_t o0 = lapind[lapi++];
                            cplx sum = c_make(src[2 * (ii + o0)], src[2 * (ii + o0) + 1]);
                            while (lapi < lapimax) {
                                const int64_t o = lapind[lapi++];
                                sum = c_add(sum, c_make(src[2 * (ii + o)], src[2 * (ii + o) + 1]));
                            }
                            const cplx pj = c_make(src[2 * jj], src[2 * jj + 1]);
                            const double nsq = pj.x * pj.x + pj.y * pj.y; /* Complex::normsq */
                            sum = c_add(c_scale(lapfac, sum), c_scale(lapfac0 + pot[jj] + g * nsq, pj));
                            dst[2 * jj] += sum.y;
                            dst[2 * jj + 1] += -sum.x;
                        }
                    }
        }
    }
}

void orc_gpblocks_norm(size_t ii0, size_t vsize, const double* psi0, const double* even, double volume, double out[2]) {
    /* GPBlocks.cpp:531-538 */
    double normsq = 0;
    cplx error = c_make(0, 0);
    for (size_t i = ii0; i < vsize; ++i) {
        const cplx e = c_make(even[2 * i], even[2 * i + 1]);
        const cplx p0 = c_make(psi0[2 * i], psi0[2 * i + 1]);
        normsq += (e.x * e.x + e.y * e.y) * volume;
        error = c_add(error, c_scale(volume, c_mul(c_conj(p0), e)));
    }
    out[0] = normsq;
    out[1] = normsq - sqrt(error.x * error.x + error.y * error.y);
}
