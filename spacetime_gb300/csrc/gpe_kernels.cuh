// gpe_kernels.cuh -- the per-step DEC stencil + nonlinear update kernels.
//
// One thread advances one dual node (all C spinor components) of one block cell;
// consecutive threads take consecutive nodes of consecutive cells along x, so a
// warp reads and writes one contiguous run of the reference's BlockPsis layout
// (coalesced 8-byte (re,im) accesses).  The node stencil, positions and weights
// live in shared memory; neighbour values are read through the read-only path
// and are served mostly by L1/L2 (each value is read from HBM once per step).
//
// Real = float is the fused FP32 stepper; Real = double the FP64 plain stepper
// that mirrors the reference kernels (Spin1GpeBCC.cu:793-917, Spin2GpeBCC.cu:845-990,
// GPUGrossPitaevskii_BCC.cu:327-347, RelativisticSpin2Gpe.cu:971-1132).
#pragma once

#include <algorithm>
#include <type_traits>

#include "gpe_internal.h"

namespace gpe {

// Constants exactly as the reference spells them (Spin1GpeBCC.cu:91-92).
#define GPE_REF_SQRT_2 1.41421356237309
#define GPE_REF_INV_SQRT_2 0.70710678118655

template <typename R>
struct Cx {
    R x, y;
};

template <typename R>
struct Vec2;
template <>
struct Vec2<float> {
    using type = float2;
};
template <>
struct Vec2<double> {
    using type = double2;
};

template <typename R>
__device__ __forceinline__ Cx<R> cx(R x, R y) {
    Cx<R> c;
    c.x = x;
    c.y = y;
    return c;
}
template <typename R>
__device__ __forceinline__ Cx<R> operator+(Cx<R> a, Cx<R> b) { return cx<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a, Cx<R> b) { return cx<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__device__ __forceinline__ Cx<R> operator*(R s, Cx<R> a) { return cx<R>(s * a.x, s * a.y); }
// complex product with the reference's operation order (utils.h:71-74)
template <typename R>
__device__ __forceinline__ Cx<R> operator*(Cx<R> a, Cx<R> b) { return cx<R>(a.x * b.x - a.y * b.y, a.y * b.x + a.x * b.y); }
template <typename R>
__device__ __forceinline__ Cx<R> conj(Cx<R> a) { return cx<R>(a.x, -a.y); }
template <typename R>
__device__ __forceinline__ void operator+=(Cx<R>& a, Cx<R> b) { a.x += b.x; a.y += b.y; }

template <typename R>
__device__ __forceinline__ Cx<R> ldc(const char* p) {
    if constexpr (sizeof(R) == 4) {
        float2 v = __ldg(reinterpret_cast<const float2*>(p));
        return cx<R>(v.x, v.y);
    } else {
        double2 v = __ldg(reinterpret_cast<const double2*>(p));
        return cx<R>(v.x, v.y);
    }
}
// plain (coherent) load for buffers the kernel also writes
template <typename R>
__device__ __forceinline__ Cx<R> ldc_rw(const char* p) {
    if constexpr (sizeof(R) == 4) {
        float2 v = *reinterpret_cast<const float2*>(p);
        return cx<R>(v.x, v.y);
    } else {
        double2 v = *reinterpret_cast<const double2*>(p);
        return cx<R>(v.x, v.y);
    }
}
template <typename R>
__device__ __forceinline__ void stc(char* p, Cx<R> c) {
    if constexpr (sizeof(R) == 4) {
        *reinterpret_cast<float2*>(p) = make_float2(c.x, c.y);
    } else {
        *reinterpret_cast<double2*>(p) = make_double2(c.x, c.y);
    }
}

// A whole node record of C complex values.  FP32 records of odd C > 1 (24 or 40
// bytes) start 8-byte aligned at a stride of 8C bytes, so each is (C-1)/2 aligned
// 16-byte loads plus one 8-byte load, in an order set by bit 3 of the address
// (which half of the record is 16-byte aligned): a warp's load instructions, and
// with them the L1 wavefronts they cost, drop from C to (C+1)/2 per record.
// NC: the read-only path (buffers the kernel does not write).
template <typename R, int C, bool NC>
__device__ __forceinline__ void ld_node(const char* p, Cx<R>* v) {
    if constexpr (sizeof(R) == 4 && C > 1 && (C % 2) == 1) {
        const bool odd = (reinterpret_cast<uintptr_t>(p) & 8) != 0;
        const char* q = p + (odd ? 8 : 0);
        const char* r = p + (odd ? 0 : 8 * (C - 1));
        float4 a[(C - 1) / 2];
#pragma unroll
        for (int k = 0; k < (C - 1) / 2; ++k) {
            if constexpr (NC) a[k] = __ldg(reinterpret_cast<const float4*>(q + 16 * k));
            else a[k] = *reinterpret_cast<const float4*>(q + 16 * k);
        }
        float2 b;
        if constexpr (NC) b = __ldg(reinterpret_cast<const float2*>(r));
        else b = *reinterpret_cast<const float2*>(r);
#pragma unroll
        for (int s = 0; s < C; ++s) {
            // even: a[0].xy a[0].zw a[1].xy ... b;  odd: b a[0].xy a[0].zw ...
            const int te = s, to = s - 1;
            const Cx<R> ve = s == C - 1 ? cx<R>(b.x, b.y)
                                        : ((te & 1) ? cx<R>(a[te / 2].z, a[te / 2].w) : cx<R>(a[te / 2].x, a[te / 2].y));
            const Cx<R> vo = s == 0 ? cx<R>(b.x, b.y)
                                    : ((to & 1) ? cx<R>(a[to / 2].z, a[to / 2].w) : cx<R>(a[to / 2].x, a[to / 2].y));
            v[s] = odd ? vo : ve;
        }
    } else {
#pragma unroll
        for (int s = 0; s < C; ++s) v[s] = NC ? ldc<R>(p + s * 2 * sizeof(R)) : ldc_rw<R>(p + s * 2 * sizeof(R));
    }
}

template <typename R, int C>
__device__ __forceinline__ void st_node(char* p, const Cx<R>* v) {
    if constexpr (sizeof(R) == 4 && C > 1 && (C % 2) == 1) {
        const bool odd = (reinterpret_cast<uintptr_t>(p) & 8) != 0;
        char* q = p + (odd ? 8 : 0);
        char* r = p + (odd ? 0 : 8 * (C - 1));
#pragma unroll
        for (int k = 0; k < (C - 1) / 2; ++k) {
            // component o + 2k and o + 2k + 1 (selected without dynamic indexing)
            Cx<R> lo = v[2 * k], hi = v[2 * k + 1];
            if (odd) {
                lo = v[2 * k + 1];
                hi = v[2 * k + 2];
            }
            *reinterpret_cast<float4*>(q + 16 * k) = make_float4(lo.x, lo.y, hi.x, hi.y);
        }
        const Cx<R> b = odd ? v[0] : v[C - 1];
        *reinterpret_cast<float2*>(r) = make_float2(b.x, b.y);
    } else {
#pragma unroll
        for (int s = 0; s < C; ++s) stc<R>(p + s * 2 * sizeof(R), v[s]);
    }
}

template <typename R>
__device__ __forceinline__ const PhysR<R>& make_phys(const StepArgs& a) {
    if constexpr (sizeof(R) == 4) return a.pf;
    else return a.pd;
}

// The per-step values of a PhysR (external fields bq, bb, bqq, bbq and the trap
// switch) are read from F where it is given, the constants from P: the batch
// kernel keeps its members' constants in constant memory and the fields of the
// step in shared memory.

// trap (Spin1GpeBCC.cu:112-122)
template <typename R>
__device__ __forceinline__ R trap(const PhysR<R>& P, const R r[3], const PhysR<R>* F = nullptr) {
    if (!(F ? F->trap_on : P.trap_on)) return (R)0;
    R x = r[0] * P.lambda[0];
    R y = r[1] * P.lambda[1];
    R z = r[2] * P.lambda[2];
    return (R)0.5 * (x * x + y * y + z * z) + P.trap_offset;
}

// magneticField (Spin1GpeBCC.cu:128-142)
template <typename R>
__device__ __forceinline__ void mag_field(const PhysR<R>& P, const R r[3], R Bq, const R Bb[3], R B[3]) {
    if (P.flags & GPE_FLAG_QUADRUPOLE_OFFSET) {
        B[0] = Bq * (r[0] - P.qc[0]) + Bb[0];
        B[1] = Bq * (r[1] - P.qc[1]) + Bb[1];
        B[2] = (R)-2 * Bq * (r[2] - P.qc[2]) + Bb[2];
    } else {
        B[0] = Bq * r[0] + Bb[0];
        B[1] = Bq * r[1] + Bb[1];
        B[2] = (R)-2 * Bq * r[2] + Bb[2];
    }
}

// Local (non-kinetic) part of H for spin-1 (Spin1GpeBCC.cu:867-912).  ext: use the
// external field (leapfrog / Euler); the imaginary-time kernel uses only c2<F>
// (Spin1GpeBCC.cu:645-646).  pot = trap value; lossqz: loss and quadratic Zeeman
// allowed.  totalPot_out receives trap + c0 rho for the hyperbolic c_K.
template <typename R>
__device__ __forceinline__ void local_spin1(const PhysR<R>& P, const R r[3], R pot, bool ext, bool lossqz,
                                            bool hyper, const Cx<R>* ps, Cx<R>* H, const PhysR<R>* F = nullptr) {
    const PhysR<R>& Fs = F ? *F : P;
    const R n1 = ps[0].x * ps[0].x + ps[0].y * ps[0].y;
    const R n_1 = ps[2].x * ps[2].x + ps[2].y * ps[2].y;
    const R normSq = n1 + (ps[1].x * ps[1].x + ps[1].y * ps[1].y) + n_1;
    Cx<R> totalPot = cx<R>(pot + P.c0 * normSq, (R)0);
    if (lossqz && (P.flags & GPE_FLAG_THREE_BODY_LOSS)) totalPot.y = -P.alpha * normSq * normSq;
    if (hyper) {
        // RelativisticSpin1Gpe/common_kernels.h:229-235
        const R cK = (R)1 + P.sigma * totalPot.x;
        for (int s = 0; s < 3; ++s) H[s] = (-cK) * H[s];
    }
    H[0] += totalPot * ps[0];
    H[1] += totalPot * ps[1];
    H[2] += totalPot * ps[2];
    const Cx<R> magXY = (R)GPE_REF_SQRT_2 * (conj(ps[0]) * ps[1] + conj(ps[1]) * ps[2]);
    R B[3];
    if (ext) {
        mag_field(P, r, Fs.bq, Fs.bb, B);
        B[0] += P.c2 * magXY.x;
        B[1] += P.c2 * magXY.y;
        B[2] += P.c2 * (n1 - n_1);
    } else {
        B[0] = P.c2 * magXY.x;
        B[1] = P.c2 * magXY.y;
        B[2] = P.c2 * (n1 - n_1);
    }
    Cx<R> Bxy = (R)GPE_REF_INV_SQRT_2 * cx<R>(B[0], B[1]);
    Cx<R> BxyConj = conj(Bxy);
    H[0] += (B[2] * ps[0] + BxyConj * ps[1]);
    H[1] += (Bxy * ps[0] + BxyConj * ps[2]);
    H[2] += (Bxy * ps[1] - B[2] * ps[2]);
    if (lossqz && (P.flags & GPE_FLAG_QUADRATIC_ZEEMAN)) {
        // Spin1GpeBCC.cu:897-912
        R Q[3];
        mag_field(P, r, Fs.bqq, Fs.bbq, Q);
        Bxy = (R)GPE_REF_INV_SQRT_2 * cx<R>(Q[0], Q[1]);
        BxyConj = conj(Bxy);
        const R BxyNormSq = (BxyConj * Bxy).x;
        const Cx<R> BxySq = Bxy * Bxy;
        const Cx<R> BxyConjSq = BxyConj * BxyConj;
        const R BzSq = Q[2] * Q[2];
        const Cx<R> BzBxy = Q[2] * Bxy;
        const Cx<R> BzBxyConj = Q[2] * BxyConj;
        H[0] += (BzSq + BxyNormSq) * ps[0] + BzBxyConj * ps[1] + BxyConjSq * ps[2];
        H[1] += BzBxy * ps[0] + ((R)2 * BxyNormSq) * ps[1] - BzBxyConj * ps[2];
        H[2] += BxySq * ps[0] - BzBxy * ps[1] + (BzSq + BxyNormSq) * ps[2];
    }
}

// Local part of H for spin-2 (Spin2GpeBCC.cu:923-970; RelativisticSpin2Gpe.cu:1068-1125).
template <typename R>
__device__ __forceinline__ void local_spin2(const PhysR<R>& P, const R r[3], R pot, bool ext, bool loss, bool hyper,
                                            const Cx<R>* ps, Cx<R>* H, const PhysR<R>* F = nullptr) {
    const PhysR<R>& Fs = F ? *F : P;
    R n[5];
    for (int s = 0; s < 5; ++s) n[s] = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
    const R normSq = n[0] + n[1] + n[2] + n[3] + n[4];
    Cx<R> ab = cx<R>(pot + P.c0 * normSq, (R)0);
    if (loss && (P.flags & GPE_FLAG_THREE_BODY_LOSS)) ab.y = -P.alpha * normSq * normSq;
    if (hyper) {
        const R cK = (R)1 + P.sigma * ab.x;
        for (int s = 0; s < 5; ++s) H[s] = (-cK) * H[s];
    }
    R B[3] = {(R)0, (R)0, (R)0};
    if (ext) mag_field(P, r, Fs.bq, Fs.bb, B);
    const R c2 = P.c2, c4 = P.c4;
    const R Fz = c2 * ((R)2 * n[0] + n[1] - n[3] - (R)2 * n[4]);
    Cx<R> d[5];
    d[0] = cx<R>((R)2 * Fz + (R)0.4 * c4 * n[4] - (R)2 * B[2], (R)0) + ab;
    d[1] = cx<R>(Fz + (R)0.4 * c4 * n[3] - B[2], (R)0) + ab;
    d[2] = cx<R>((R)0.2 * c4 * n[2], (R)0) + ab;
    d[3] = cx<R>(-Fz + (R)0.4 * c4 * n[1] + B[2], (R)0) + ab;
    d[4] = cx<R>((R)-2 * Fz + (R)0.4 * c4 * n[0] + (R)2 * B[2], (R)0) + ab;
    for (int s = 0; s < 5; ++s) H[s] += d[s] * ps[s];
    const Cx<R> s2 = ps[0], s1 = ps[1], s0 = ps[2], s_1 = ps[3], s_2 = ps[4];
    const R sq6 = (R)2.449489742783178098, sq15 = (R)1.224744871391589049;  // sqrt(6), sqrt(1.5)
    const Cx<R> den = c2 * ((R)2 * (s2 * conj(s1) + s_1 * conj(s_2)) + sq6 * (s1 * conj(s0) + s0 * conj(s_1))) -
                      cx<R>(B[0], -B[1]);
    const Cx<R> c12 = den - ((R)0.4 * c4 * s_1) * conj(s_2);
    const Cx<R> c45 = den - ((R)0.4 * c4 * s2) * conj(s1);
    const Cx<R> c13 = ((R)0.2 * c4 * s0) * conj(s_2);
    const Cx<R> c35 = ((R)0.2 * c4 * s2) * conj(s0);
    const Cx<R> c23 = sq15 * den - ((R)0.2 * c4 * s0) * conj(s_1);
    const Cx<R> c34 = sq15 * den - ((R)0.2 * c4 * s1) * conj(s0);
    H[0] += (c12 * s1 + c13 * s0);
    H[1] += (conj(c12) * s2 + c23 * s0);
    H[2] += (conj(c13) * s2 + c35 * s_2 + c34 * s_1 + conj(c23) * s1);
    H[3] += (conj(c34) * s0 + c45 * s_2);
    H[4] += (conj(c35) * s0 + conj(c45) * s_1);
}

template <typename R>
__device__ __forceinline__ void local_scalar(const PhysR<R>& P, R pot, bool loss, bool hyper, const Cx<R>* ps, Cx<R>* H) {
    // GPUGrossPitaevskii_BCC.cu:198-199; RelativisticGpeBCC.cu:244-253
    const R normsq = ps[0].x * ps[0].x + ps[0].y * ps[0].y;
    Cx<R> tp = cx<R>(pot + P.c0 * normsq, (R)0);
    if (loss && (P.flags & GPE_FLAG_THREE_BODY_LOSS)) tp.y = -P.alpha * normsq * normsq;
    if (hyper) {
        const R cK = (R)1 + P.sigma * tp.x;
        H[0] = (-cK) * H[0];
    }
    H[0] += tp * ps[0];
}

template <typename R, int C>
__device__ __forceinline__ void local_terms(const PhysR<R>& P, const R r[3], R pot, int mode, bool hyper, const Cx<R>* ps,
                                            Cx<R>* H, const PhysR<R>* F = nullptr) {
    const bool ext = (mode != GPE_MODE_ITP);
    if constexpr (C == 1) {
        local_scalar<R>(P, pot, ext, hyper, ps, H);
    } else if constexpr (C == 3) {
        local_spin1<R>(P, r, pot, ext, ext, hyper, ps, H, F);
    } else {
        local_spin2<R>(P, r, pot, ext, true, hyper, ps, H, F);
    }
}

// Shared-memory copy of the per-handle tables.
template <typename R>
struct __align__(16) SmemTables {
    int32_t nb_off[kMaxEntries];  // first and 16-byte aligned: a node's 4 entries load as one vector
    R w[kMaxEntries];
    R pos[kMaxNodes * 3];
    int32_t row_ptr[kMaxNodes + 1];
};

template <typename R>
__device__ __forceinline__ void load_tables(SmemTables<R>& s, const StepArgs& a) {
    const int V = a.g.V;
    const int n = a.tab.entries;
    const R ks = make_phys<R>(a).ks;  // condensate expansion: weights h / bs^2 of the step's bs
    for (int i = threadIdx.x; i <= V; i += blockDim.x) s.row_ptr[i] = a.tab.row_ptr[i];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s.nb_off[i] = a.tab.nb_off[i];
        if constexpr (sizeof(R) == 4) s.w[i] = a.tab.w32[i] * ks;
        else s.w[i] = a.tab.w64[i] * ks;
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) s.pos[i] = a.tab.pos32[i];
        else s.pos[i] = a.tab.pos64[i];
    }
}

// Apply the time update to one node (Spin1GpeBCC.cu:914-916, :788-790, :655-661).
template <typename R, int C>
__device__ __forceinline__ void write_update(int mode, R dt, char* nxt, char* hp, const Cx<R>* prv, const Cx<R>* H) {
#pragma unroll
    for (int s = 0; s < C; ++s) {
        char* p = nxt + s * 2 * sizeof(R);
        if (mode == GPE_MODE_LEAPFROG) {
            Cx<R> v = ldc_rw<R>(p);
            v += ((R)2 * dt) * cx<R>(H[s].y, -H[s].x);
            stc<R>(p, v);
        } else if (mode == GPE_MODE_EULER) {
            stc<R>(p, prv[s] + dt * cx<R>(H[s].y, -H[s].x));
        } else {
            if (hp) stc<R>(hp + s * 2 * sizeof(R), H[s]);
            stc<R>(p, prv[s] - dt * H[s]);
        }
    }
}

// ---------------------------------------------------------------- parabolic

// A node's stencil entries and position, for nodes with D entries each.
template <typename R, int D>
struct NodeTab {
    int32_t off[D];
    R w[D];
    R pos[3];
};

template <typename R, int D>
__device__ __forceinline__ NodeTab<R, D> node_tab(const SmemTables<R>& st, uint32_t l, int f0) {
    NodeTab<R, D> t;
    if constexpr (D % 4 == 0) {
        // f0 a multiple of 4: one 16-byte shared load per 4 offsets, one or two per 4 weights
#pragma unroll
        for (int q = 0; q < D; q += 4) {
            const int4 o4 = *reinterpret_cast<const int4*>(st.nb_off + f0 + q);
            t.off[q] = o4.x; t.off[q + 1] = o4.y; t.off[q + 2] = o4.z; t.off[q + 3] = o4.w;
            if constexpr (sizeof(R) == 4) {
                const float4 w4 = *reinterpret_cast<const float4*>(st.w + f0 + q);
                t.w[q] = w4.x; t.w[q + 1] = w4.y; t.w[q + 2] = w4.z; t.w[q + 3] = w4.w;
            } else {
                const double2 wa = *reinterpret_cast<const double2*>(st.w + f0 + q);
                const double2 wb = *reinterpret_cast<const double2*>(st.w + f0 + q + 2);
                t.w[q] = wa.x; t.w[q + 1] = wa.y; t.w[q + 2] = wb.x; t.w[q + 3] = wb.y;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            t.off[k] = st.nb_off[f0 + k];
            t.w[k] = st.w[f0 + k];
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) t.pos[k] = st.pos[3 * l + k];
    return t;
}

// Node l of a lattice whose nodes all have D entries.
template <typename R, int D>
__device__ __forceinline__ NodeTab<R, D> node_tab(const SmemTables<R>& st, uint32_t l) {
    return node_tab<R, D>(st, l, (int)l * D);
}

// The step kernels' default: no observables.
struct NoObs {
    template <typename R, int C>
    __device__ __forceinline__ void node(const PhysR<R>&, const R*, const Cx<R>*, const Cx<R>*) {}
};

// Observables of the state a step reads, summed by each thread over its nodes:
// the per-node terms of observe_kernel (density, <psi|H psi>, interaction energy,
// magnetisation, spin norm, centre of mass, max |psi_s|, non-finite count) in the
// storage precision R, from the step's own H psi (Laplacian + local terms at the
// step's time, already in registers), groups of kGroup nodes summed in R and each
// group added in FP64 (FP64 storage: every node in FP64).  The thread's FP64 sums
// live in shared memory (kObsSums x blockDim doubles, thread-major per sum), which
// keeps the step kernel's register count, and so its occupancy, near the plain
// step's.
constexpr int kObsSums = OBS_MAXABS;  // the summed observables come first in ObsIndex
static_assert(OBS_MAXABS + 2 == OBS_COUNT && OBS_NONFINITE == OBS_MAXABS + 1, "max and count last");
template <typename R>
struct ObsAcc {
    static constexpr int kGroup = sizeof(R) == 4 ? 8 : 1;
    double* sums;  // this thread's column of the block's kObsSums x blockDim array
    R grp[kObsSums];
    int in_group;
    R tmax;
    uint32_t nbad;
    __device__ __forceinline__ explicit ObsAcc(double* block_sums) : sums(block_sums + threadIdx.x), in_group(0), tmax((R)0), nbad(0) {
#pragma unroll
        for (int k = 0; k < kObsSums; ++k) {
            sums[k * blockDim.x] = 0.0;
            grp[k] = (R)0;
        }
    }
    template <typename RR, int C>
    __device__ __forceinline__ void node(const PhysR<R>& P, const R r[3], const Cx<R>* ps, const Cx<R>* H) {
        R v[kObsSums];
#pragma unroll
        for (int k = 0; k < kObsSums; ++k) v[k] = (R)0;
        R rho = 0, hexp = 0;
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const R n2 = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
            rho += n2;
            tmax = fmax(tmax, sqrt(n2));
            if (!isfinite(ps[s].x) || !isfinite(ps[s].y)) ++nbad;
            hexp += ps[s].x * H[s].x + ps[s].y * H[s].y;
        }
        v[OBS_NORM] = rho;
        v[OBS_HEXP] = hexp;
        v[OBS_COMX] = rho * r[0];
        v[OBS_COMY] = rho * r[1];
        v[OBS_COMZ] = rho * r[2];
        // interaction energy as observe_kernel: c0 n^2 (scalar), c0 n^2 + c2 |<F>|^2
        // (spin-1), psi^H (local terms without trap, fields, loss) psi (spin-2)
        if constexpr (C == 1) {
            v[OBS_EINT] = P.c0 * rho * rho;
        } else if constexpr (C == 3) {
            const Cx<R> m = (R)GPE_REF_SQRT_2 * (conj(ps[0]) * ps[1] + conj(ps[1]) * ps[2]);
            const R fz = (ps[0].x * ps[0].x + ps[0].y * ps[0].y) - (ps[2].x * ps[2].x + ps[2].y * ps[2].y);
            v[OBS_EINT] = P.c0 * rho * rho + P.c2 * (m.x * m.x + m.y * m.y + fz * fz);
            v[OBS_MAGX] = m.x;
            v[OBS_MAGY] = m.y;
            v[OBS_MAGZ] = fz;
            v[OBS_SPIN] = sqrt(m.x * m.x + m.y * m.y + fz * fz);
        } else {
            PhysR<R> Q = P;
            Q.bq = Q.bqq = 0;
            for (int k = 0; k < 3; ++k) Q.bb[k] = Q.bbq[k] = 0;
            Q.flags &= ~(GPE_FLAG_THREE_BODY_LOSS | GPE_FLAG_QUADRATIC_ZEEMAN | GPE_FLAG_QUADRUPOLE_OFFSET);
            Cx<R> Hn[5];
#pragma unroll
            for (int s = 0; s < 5; ++s) Hn[s] = cx<R>((R)0, (R)0);
            local_terms<R, C>(Q, r, (R)0, GPE_MODE_LEAPFROG, false, ps, Hn);
            R hn = 0;
#pragma unroll
            for (int s = 0; s < C; ++s) hn += ps[s].x * Hn[s].x + ps[s].y * Hn[s].y;
            v[OBS_EINT] = hn;
            const Cx<R> fp = (R)2 * (conj(ps[0]) * ps[1] + conj(ps[3]) * ps[4]) +
                             (R)2.449489742783178098 * (conj(ps[1]) * ps[2] + conj(ps[2]) * ps[3]);
            R n[5];
            for (int s = 0; s < 5; ++s) n[s] = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
            const R fz = (R)2 * n[0] + n[1] - n[3] - (R)2 * n[4];
            v[OBS_MAGX] = fp.x;
            v[OBS_MAGY] = fp.y;
            v[OBS_MAGZ] = fz;
            v[OBS_SPIN] = sqrt(fp.x * fp.x + fp.y * fp.y + fz * fz);
        }
#pragma unroll
        for (int k = 0; k < kObsSums; ++k) grp[k] += v[k];
        if (++in_group == kGroup) flush();
    }
    __device__ __forceinline__ void flush() {
#pragma unroll
        for (int k = 0; k < kObsSums; ++k) {
            sums[k * blockDim.x] += (double)grp[k];
            grp[k] = (R)0;
        }
        in_group = 0;
    }
    // the block's sums into partials[blockIdx.x]: warp shuffles, then shared memory
    // (red: 8 x OBS_COUNT doubles); every thread of the block must call it
    __device__ __forceinline__ void block_reduce(double (*red)[OBS_COUNT], double* partials) {
        flush();
        double acc[OBS_COUNT];
#pragma unroll
        for (int k = 0; k < kObsSums; ++k) acc[k] = sums[k * blockDim.x];
        acc[OBS_MAXABS] = (double)tmax;
        acc[OBS_NONFINITE] = (double)nbad;
#pragma unroll
        for (int k = 0; k < OBS_COUNT; ++k) {
            double v = acc[k];
            for (int o = 16; o > 0; o >>= 1) {
                const double u = __shfl_down_sync(0xffffffffu, v, o);
                v = (k == OBS_MAXABS) ? fmax(v, u) : v + u;
            }
            acc[k] = v;
        }
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < OBS_COUNT; ++k) red[warp][k] = acc[k];
        }
        __syncthreads();
        if (threadIdx.x < OBS_COUNT) {
            const int k = threadIdx.x;
            double v = red[0][k];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = (k == OBS_MAXABS) ? fmax(v, red[w][k]) : v + red[w][k];
            partials[(size_t)blockIdx.x * OBS_COUNT + k] = v;
        }
    }
};

// The accumulator of a step kernel: ObsAcc (its FP64 sums in the block's shared
// array) or NoObs.
template <bool OBS, typename R>
struct ObsOf {
    using type = NoObs;
    __device__ static NoObs make(double*) { return NoObs(); }
};
template <typename R>
struct ObsOf<true, R> {
    using type = ObsAcc<R>;
    __device__ static ObsAcc<R> make(double* sums) { return ObsAcc<R>(sums); }
};

// The local terms and the time update of one node, given its Laplacian sum in H
// (Spin1GpeBCC.cu:867-916).  nv: the old next record (leapfrog).  oa: where the
// observables of prv go (ObsAcc), or nothing (NoObs).
template <typename R, int C, int MODE, class OA = NoObs>
__device__ __forceinline__ void node_finish(const PhysR<R>& P, const R pos[3], uint32_t x, uint32_t y, uint32_t z,
                                            const Cx<R>* prv, Cx<R>* H, Cx<R>* nv, char* nxt, char* hp,
                                            const PhysR<R>* F = nullptr, OA* oa = nullptr) {
    R r[3];
    r[0] = P.p0[0] + P.bs * ((R)x * P.bw[0] + pos[0]);
    r[1] = P.p0[1] + P.bs * ((R)y * P.bw[1] + pos[1]);
    r[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + pos[2]);
    const R pot = trap<R>(P, r, F);
    local_terms<R, C>(P, r, pot, MODE, false, prv, H, F);
    if constexpr (!std::is_same<OA, NoObs>::value) oa->template node<R, C>(P, r, prv, H);
    if constexpr (MODE == GPE_MODE_LEAPFROG || MODE == kModeLeapfrogFrom) {
        // next = old + 2 dt (-i H), the whole record written at once
#pragma unroll
        for (int s = 0; s < C; ++s) nv[s] += ((R)2 * P.dt) * cx<R>(H[s].y, -H[s].x);
        st_node<R, C>(nxt, nv);
    } else {
        write_update<R, C>(MODE, P.dt, nxt, hp, prv, H);
    }
}

// One node of a parabolic step whose first D (> 0) stencil entries are given in t:
// the DEC Laplacian gather, the neighbour loads issued G at a time, then the local
// terms and the time update.  MORE: the node's further entries f_more .. f_end - 1
// (a multiple of 4 of them, f_more a multiple of 4) come from the shared tables, 4
// loads at a time (FCC's octahedra: 8 entries beside the tetrahedra's 4).
// prev/next/hpsi are the buffers' interior pointers; (x, y, z) the cell, l the node.
template <typename R, int C, int MODE, int D, int G = D, bool MORE = false, class OA = NoObs>
__device__ __forceinline__ void parabolic_node_t(const Grid& g, const NodeTab<R, D>& t, const PhysR<R>& P,
                                                 const char* prev, char* next, char* hpsi, uint32_t x, uint32_t y,
                                                 uint32_t z, uint32_t l, const SmemTables<R>* st = nullptr,
                                                 int f_more = 0, int f_end = 0, const PhysR<R>* F = nullptr,
                                                 OA* oa = nullptr) {
    const size_t cell_off = (size_t)z * g.slice + (size_t)y * g.pitch + (size_t)x * g.cell_bytes;
    const char* base = prev + cell_off;
    const uint32_t node_bytes = C * 2 * sizeof(R);
    Cx<R> prv[C], H[C], nv[C];
    ld_node<R, C, true>(base + l * node_bytes, prv);
    char* nxt = next + cell_off + l * node_bytes;
    // leapfrog: the old next record is loaded up front, in flight with the gathers
    if constexpr (MODE == GPE_MODE_LEAPFROG) ld_node<R, C, false>(nxt, nv);
    if constexpr (MODE == kModeLeapfrogFrom) ld_node<R, C, true>(hpsi + cell_off + l * node_bytes, nv);
    // DEC Laplacian, sum_f w_f (psi_nb - psi) in entry order (Spin1GpeBCC.cu:835-865)
#pragma unroll
    for (int s = 0; s < C; ++s) H[s] = cx<R>((R)0, (R)0);
#pragma unroll
    for (int k0 = 0; k0 < D; k0 += G) {
        Cx<R> v[G][C];
#pragma unroll
        for (int k = 0; k < G; ++k)
            if (k0 + k < D) ld_node<R, C, true>(base + t.off[k0 + k], v[k]);
#pragma unroll
        for (int k = 0; k < G; ++k) {
            if (k0 + k < D) {
#pragma unroll
                for (int s = 0; s < C; ++s) H[s] += t.w[k0 + k] * (v[k][s] - prv[s]);
            }
        }
    }
    if constexpr (MORE) {
        static_assert(4 % G == 0, "MORE: groups of 4 entries issued G at a time");
        for (int f = f_more; f < f_end; f += 4) {
            const int4 o4 = *reinterpret_cast<const int4*>(st->nb_off + f);
            const int32_t o[4] = {o4.x, o4.y, o4.z, o4.w};
            R w[4];
            if constexpr (sizeof(R) == 4) {
                const float4 w4 = *reinterpret_cast<const float4*>(st->w + f);
                w[0] = w4.x; w[1] = w4.y; w[2] = w4.z; w[3] = w4.w;
            } else {
                const double2 wa = *reinterpret_cast<const double2*>(st->w + f);
                const double2 wb = *reinterpret_cast<const double2*>(st->w + f + 2);
                w[0] = wa.x; w[1] = wa.y; w[2] = wb.x; w[3] = wb.y;
            }
#pragma unroll
            for (int h = 0; h < 4; h += G) {
                Cx<R> v[G][C];
#pragma unroll
                for (int k = 0; k < G; ++k) ld_node<R, C, true>(base + o[h + k], v[k]);
#pragma unroll
                for (int k = 0; k < G; ++k) {
#pragma unroll
                    for (int s = 0; s < C; ++s) H[s] += w[h + k] * (v[k][s] - prv[s]);
                }
            }
        }
    }
    char* hp = (MODE == GPE_MODE_ITP && hpsi) ? hpsi + cell_off + l * node_bytes : nullptr;
    node_finish<R, C, MODE, OA>(P, t.pos, x, y, z, prv, H, nv, nxt, hp, F, oa);
}

// One node of a parabolic step: the DEC Laplacian gather, the local terms and the
// time update (Spin1GpeBCC.cu:835-916).  prev/next/hpsi are the buffers' interior
// pointers; (x, y, z) the cell, l the node.  D > 0: every node has D stencil
// entries (MORE: a multiple of 4, the first D taken as the node's table), the
// neighbour loads issued G at a time.  F: where the step's fields come from (P if
// null).
template <typename R, int C, int MODE, int D = 0, int G = D, bool MORE = false, class OA = NoObs>
__device__ __forceinline__ void parabolic_node(const Grid& g, const SmemTables<R>& st, const PhysR<R>& P, const char* prev,
                                               char* next, char* hpsi, uint32_t x, uint32_t y, uint32_t z, uint32_t l,
                                               const PhysR<R>* F = nullptr, OA* oa = nullptr) {
    if constexpr (D > 0 && MORE) {
        const int f0 = st.row_ptr[l];
        parabolic_node_t<R, C, MODE, D, G, true, OA>(g, node_tab<R, D>(st, l, f0), P, prev, next, hpsi, x, y, z, l, &st,
                                                     f0 + D, st.row_ptr[l + 1], F, oa);
    } else if constexpr (D > 0) {
        parabolic_node_t<R, C, MODE, D, G, false, OA>(g, node_tab<R, D>(st, l), P, prev, next, hpsi, x, y, z, l, nullptr, 0,
                                                      0, F, oa);
    } else {
        const size_t cell_off = (size_t)z * g.slice + (size_t)y * g.pitch + (size_t)x * g.cell_bytes;
        const char* base = prev + cell_off;
        const uint32_t node_bytes = C * 2 * sizeof(R);
        Cx<R> prv[C], H[C], nv[C];
        ld_node<R, C, true>(base + l * node_bytes, prv);
#pragma unroll
        for (int s = 0; s < C; ++s) H[s] = cx<R>((R)0, (R)0);
        char* nxt = next + cell_off + l * node_bytes;
        if constexpr (MODE == GPE_MODE_LEAPFROG) ld_node<R, C, false>(nxt, nv);
        if constexpr (MODE == kModeLeapfrogFrom) ld_node<R, C, true>(hpsi + cell_off + l * node_bytes, nv);
        const int f0 = st.row_ptr[l], f1 = st.row_ptr[l + 1];
        if constexpr (C == 1) {
            // scalars: groups of 4 entries, the loads of a group issued together (rows
            // of mixed length, e.g. FCC's 4 and 8; for spinors the registers this
            // takes cost more occupancy than it gains)
            for (int f = f0; f < f1; f += 4) {
                Cx<R> v[4][C];
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (f + k < f1) ld_node<R, C, true>(base + st.nb_off[f + k], v[k]);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (f + k < f1) {
                        const R w = st.w[f + k];
#pragma unroll
                        for (int s = 0; s < C; ++s) H[s] += w * (v[k][s] - prv[s]);
                    }
                }
            }
        } else {
            for (int f = f0; f < f1; ++f) {
                Cx<R> v[C];
                ld_node<R, C, true>(base + st.nb_off[f], v);
                const R w = st.w[f];
#pragma unroll
                for (int s = 0; s < C; ++s) H[s] += w * (v[s] - prv[s]);
            }
        }
        const R pos[3] = {st.pos[3 * l + 0], st.pos[3 * l + 1], st.pos[3 * l + 2]};
        char* hp = (MODE == GPE_MODE_ITP && hpsi) ? hpsi + cell_off + l * node_bytes : nullptr;
        node_finish<R, C, MODE, OA>(P, pos, x, y, z, prv, H, nv, nxt, hp, F, oa);
    }
}

// MODE: GPE_MODE_LEAPFROG / EULER / ITP.  Grid-stride over the nodes, one node
// per thread per pass, on a fixed grid, so that each block stages the tables once.
template <typename R, int C, int MODE, int D, bool OBS>
__device__ __forceinline__ void parabolic_step_body(const StepArgs& a) {
    __shared__ SmemTables<R> st;
    load_tables<R>(st, a);
    __syncthreads();
    const PhysR<R>& P = make_phys<R>(a);
    using OA = typename ObsOf<OBS, R>::type;
    __shared__ double obs_sums[OBS ? kObsSums * 256 : 1];
    OA oa = ObsOf<OBS, R>::make(obs_sums);
    for (uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < a.total;
         gid += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)gid;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * a.g.V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        parabolic_node<R, C, MODE, D, D, false, OA>(a.g, st, P, a.prev, a.next, a.hpsi, x, y, z, l, nullptr, &oa);
    }
    if constexpr (OBS) {
        __shared__ double red[8][OBS_COUNT];
        oa.block_reduce(red, a.partials);
    }
}
template <typename R, int C, int MODE, int D>
__global__ void __launch_bounds__(256) parabolic_step_kernel(StepArgs a) {
    parabolic_step_body<R, C, MODE, D, false>(a);
}
// The same with the observables of the state it reads (three blocks per SM).
template <typename R, int C, int MODE, int D>
__global__ void __launch_bounds__(256, 3) parabolic_step_obs_kernel(StepArgs a) {
    parabolic_step_body<R, C, MODE, D, true>(a);
}

// The same update on a grid whose stride is a multiple of V: a thread keeps one
// node index l on every pass, so its first D entries and its position are loaded
// once into registers instead of from shared memory for every node.  Every node has
// D entries, or (MORE) a multiple of 4 of them, the entries past the first D read
// from the shared tables.  G: neighbour loads issued together.
template <typename R, int C, int MODE, int D, int G, bool MORE, bool OBS>
__device__ __forceinline__ void parabolic_fixed_body(const StepArgs& a) {
    __shared__ SmemTables<R> st;
    load_tables<R>(st, a);
    __syncthreads();
    const PhysR<R>& P = make_phys<R>(a);
    using OA = typename ObsOf<OBS, R>::type;
    __shared__ double obs_sums[OBS ? kObsSums * 256 : 1];
    OA oa = ObsOf<OBS, R>::make(obs_sums);
    uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (!OBS && gid >= a.total) return;
    const uint32_t l = (uint32_t)gid - fdiv((uint32_t)gid, a.divV) * a.g.V;
    const int f0 = MORE ? st.row_ptr[l] : (int)l * D;
    const int f_end = MORE ? st.row_ptr[l + 1] : 0;
    const NodeTab<R, D> t = node_tab<R, D>(st, gid < a.total ? l : 0u, gid < a.total ? f0 : 0);
    for (; gid < a.total; gid += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)gid;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t x = fdiv(i - row * a.row_items, a.divV);
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        parabolic_node_t<R, C, MODE, D, G, MORE, OA>(a.g, t, P, a.prev, a.next, a.hpsi, x, y, z, l, &st, f0 + D, f_end,
                                                     nullptr, &oa);
    }
    if constexpr (OBS) {
        __shared__ double red[8][OBS_COUNT];
        oa.block_reduce(red, a.partials);
    }
}
template <typename R, int C, int MODE, int D, int G, bool MORE>
__global__ void __launch_bounds__(256) parabolic_fixed_kernel(StepArgs a) {
    parabolic_fixed_body<R, C, MODE, D, G, MORE, false>(a);
}
// The same with the observables of the state it reads (three blocks per SM).
template <typename R, int C, int MODE, int D, int G, bool MORE>
__global__ void __launch_bounds__(256, 3) parabolic_fixed_obs_kernel(StepArgs a) {
    parabolic_fixed_body<R, C, MODE, D, G, MORE, true>(a);
}

// SM count of the current device (cached per device).
inline int device_sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (cache[dev] == 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = sms > 0 ? sms : 1;
    }
    return cache[dev];
}

// ---------------------------------------------------------------- hyperbolic

template <typename R>
struct __align__(16) SmemHyper {
    int32_t inc_off[kMaxNodes * kMaxFaces];  // first and 16-byte aligned: a node's 4 faces load as one vector
    R inc_w[kMaxNodes * kMaxFaces];
    int32_t e_from[kMaxEdges];
    int32_t e_to[kMaxEdges];
    R pos[kMaxNodes * 3];
};

// The 4 incidences of node l (offsets and weights) as two 16-byte shared loads
// (one 16-byte and two for FP64 weights), for lattices of 4 faces per node.
template <typename R>
__device__ __forceinline__ void incidences4(const SmemHyper<R>& sh, uint32_t l, int32_t off[4], R w[4]) {
    const int4 o = *reinterpret_cast<const int4*>(sh.inc_off + 4 * l);
    off[0] = o.x; off[1] = o.y; off[2] = o.z; off[3] = o.w;
    if constexpr (sizeof(R) == 4) {
        const float4 v = *reinterpret_cast<const float4*>(sh.inc_w + 4 * l);
        w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
    } else {
        const double2 a = *reinterpret_cast<const double2*>(sh.inc_w + 4 * l);
        const double2 b = *reinterpret_cast<const double2*>(sh.inc_w + 4 * l + 2);
        w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
    }
}

// Edge (q) update of one dual edge (RelativisticSpin2Gpe.cu:986-1019, :823-856, :573-598).
// QM: 0 hyperbolic leapfrog  next_q += i 2(dt/sigma)(prev_q + d0 psi)
//     1 parabolic            next_q  = d0 psi
//     2 forward Euler        next_q  = prev_q + i (dt/sigma)(prev_q + d0 psi)
//     3 imaginary time       next_q  = prev_q - (dt/sigma)(prev_q - d0 psi)
template <typename R, int C, int QM>
__device__ __forceinline__ void q_update(const StepArgs& a, const SmemHyper<R>& sh, uint32_t x, uint32_t y,
                                         uint32_t z, uint32_t e) {
    const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
    const size_t qcell_off = (size_t)z * a.g.qslice + (size_t)y * a.g.qpitch + (size_t)x * a.g.qcell_bytes;
    const char* pb = a.prev + cell_off;
    const char* thisp = pb + sh.e_from[e];
    const char* otherp = pb + sh.e_to[e];
    const uint32_t edge_bytes = C * 2 * sizeof(R);
    const char* qprev = a.q + qcell_off + e * edge_bytes;
    char* qnext = a.qnext + qcell_off + e * edge_bytes;
    const R dts = make_phys<R>(a).dts;
    // whole records: (C+1)/2 loads each in FP32
    Cx<R> to[C], from[C], pq[C], v[C];
    ld_node<R, C, true>(otherp, to);
    ld_node<R, C, true>(thisp, from);
    if constexpr (QM != 1) ld_node<R, C, false>(qprev, pq);
    if constexpr (QM == 0) ld_node<R, C, false>(qnext, v);
#pragma unroll
    for (int s = 0; s < C; ++s) {
        const Cx<R> d0psi = to[s] - from[s];
        if constexpr (QM == 1) {
            v[s] = d0psi;
        } else if constexpr (QM == 0) {
            const Cx<R> qq = ((R)2 * dts) * (pq[s] + d0psi);
            v[s] += cx<R>(-qq.y, qq.x);
        } else if constexpr (QM == 3) {
            v[s] = pq[s] - dts * (pq[s] - d0psi);
        } else {
            const Cx<R> qq = dts * (pq[s] + d0psi);
            v[s] = pq[s] + cx<R>(-qq.y, qq.x);
        }
    }
    st_node<R, C>(qnext, v);
}

// Fused psi + q step.  The reference launches update_psi then update_q, both
// reading the previous (psi, q) (RelativisticSpin2Gpe.cu:1873-1874); here one
// launch does both.  Blocks are interleaved in groups of 1 + E/V: the first block
// of a group updates 256 nodes, the next E/V blocks update the 256*E/V edges of
// the same cells, so both halves of a group read the same psi/q lines from L2.  The
// grid strides over these `vblocks` item blocks on one wave, so that each block
// stages the tables once.
// DO_PSI: psi update with MODE and HYPERB (-c_K scaling); QM < 0: no q update.
template <typename R, int C, bool DO_PSI, int MODE, bool HYPERB, int QM>
__global__ void __launch_bounds__(256) hyper_step_kernel(StepArgs a, uint32_t node_items, uint32_t edge_items,
                                                         uint32_t ratio, uint32_t vblocks) {
    __shared__ SmemHyper<R> sh;
    const int V = a.g.V, E = a.g.E, F = a.tab.faces;
    for (int i = threadIdx.x; i < V * F; i += blockDim.x) {
        sh.inc_off[i] = a.tab.inc_off[i];
        if constexpr (sizeof(R) == 4) sh.inc_w[i] = a.tab.inc_w32[i];
        else sh.inc_w[i] = a.tab.inc_w64[i];
    }
    for (int i = threadIdx.x; i < E; i += blockDim.x) {
        sh.e_from[i] = a.tab.e_from_off[i];
        sh.e_to[i] = a.tab.e_to_off[i];
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) sh.pos[i] = a.tab.pos32[i];
        else sh.pos[i] = a.tab.pos64[i];
    }
    __syncthreads();

    for (uint32_t vb = blockIdx.x; vb < vblocks; vb += gridDim.x) {
    uint32_t group, sub;
    if (DO_PSI && QM >= 0) {
        group = vb / (1 + ratio);
        sub = vb - group * (1 + ratio);
    } else if (DO_PSI) {
        group = vb;
        sub = 0;
    } else {
        group = 0;
        sub = 1 + vb;  // edge block index = sub - 1
    }
    if (DO_PSI && sub == 0) {
        const uint32_t i = group * blockDim.x + threadIdx.x;
        if (i >= node_items) continue;
        const PhysR<R>& P = make_phys<R>(a);
        const uint32_t node_bytes = C * 2 * sizeof(R);
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
        const size_t qcell_off = (size_t)z * a.g.qslice + (size_t)y * a.g.qpitch + (size_t)x * a.g.qcell_bytes;
        const char* own = a.prev + cell_off + l * node_bytes;
        Cx<R> prv[C], H[C];
        ld_node<R, C, true>(own, prv);
#pragma unroll
        for (int s = 0; s < C; ++s) H[s] = cx<R>((R)0, (R)0);
        // d1 of q (RelativisticSpin2Gpe.cu:1051-1066), whole edge records
        const char* qb = a.q + qcell_off;
        if (F == 4) {
            int32_t off[4];
            R w[4];
            incidences4<R>(sh, l, off, w);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                Cx<R> qv[C];
                ld_node<R, C, true>(qb + off[k], qv);
#pragma unroll
                for (int s = 0; s < C; ++s) H[s] += w[k] * qv[s];
            }
        } else {
            for (int k = 0; k < F; ++k) {
                Cx<R> qv[C];
                ld_node<R, C, true>(qb + sh.inc_off[l * F + k], qv);
                const R w = sh.inc_w[l * F + k];
#pragma unroll
                for (int s = 0; s < C; ++s) H[s] += w * qv[s];
            }
        }
        R r[3];
        r[0] = P.p0[0] + P.bs * ((R)x * P.bw[0] + sh.pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((R)y * P.bw[1] + sh.pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + sh.pos[3 * l + 2]);
        const R pot = trap<R>(P, r);
        if constexpr (C == 1) {
            local_scalar<R>(P, pot, false, HYPERB, prv, H);
        } else if constexpr (C == 3) {
            local_spin1<R>(P, r, pot, MODE != GPE_MODE_ITP, false, HYPERB, prv, H);
        } else {
            local_spin2<R>(P, r, pot, MODE != GPE_MODE_ITP, false, HYPERB, prv, H);
        }
        char* hp = (MODE == GPE_MODE_ITP && a.hpsi) ? a.hpsi + cell_off + l * node_bytes : nullptr;
        write_update<R, C>(MODE, P.dt, a.next + cell_off + l * node_bytes, hp, prv, H);
    } else if constexpr (QM >= 0) {
        const uint32_t eb = (DO_PSI ? group * ratio : 0) + (sub - 1);
        const uint32_t i = eb * blockDim.x + threadIdx.x;
        if (i >= edge_items) continue;
        const uint32_t row = fdiv(i, a.divRowE);
        const uint32_t within = i - row * a.row_items_e;
        const uint32_t x = fdiv(within, a.divE);
        const uint32_t e = within - x * E;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        q_update<R, C, QM>(a, sh, x, y, z, e);
    }
    }
}

}  // namespace gpe

namespace gpe {

// ---------------------------------------------------------------- observables

// Observables of one psi buffer with FP64 sums (density/integrate Spin1GpeBCC.cu:191-211,
// 328-348; energy GPUGrossPitaevskii_BCC.cu:204-226; localAvgSpinAndDensity
// Spin1GpeBCC.cu:235-271; com GPUGrossPitaevskii_BCC.cu:349-375).  Values are
// loaded in the storage precision R; the per-node terms are computed in A (FP64,
// or the FP32 storage precision when the handle asks for it) and accumulated in
// FP64.  Each block writes OBS_COUNT partial sums (warp shuffles, then shared
// memory); a one-block kernel adds the partials in a fixed order, so results are
// reproducible run to run.
template <typename R, int C, typename A>
__global__ void __launch_bounds__(256) observe_kernel(StepArgs a) {
    __shared__ SmemTables<A> st;
    __shared__ double red[8][OBS_COUNT];
    {
        const int V = a.g.V, n = a.tab.entries;
        for (int i = threadIdx.x; i <= V; i += blockDim.x) st.row_ptr[i] = a.tab.row_ptr[i];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            st.nb_off[i] = a.tab.nb_off[i];
            // condensate expansion: weights h / bs^2 of the step's bs
            if constexpr (sizeof(A) == 4) st.w[i] = a.tab.w32[i] * make_phys<A>(a).ks;
            else st.w[i] = a.tab.w64[i] * make_phys<A>(a).ks;
        }
        for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
            if constexpr (sizeof(A) == 4) st.pos[i] = a.tab.pos32[i];
            else st.pos[i] = a.tab.pos64[i];
        }
    }
    __syncthreads();
    double acc[OBS_COUNT];
#pragma unroll
    for (int k = 0; k < OBS_COUNT; ++k) acc[k] = 0.0;
    // grid-stride: each thread sums many nodes, so the FP64 warp reduction (which
    // runs on GB300's narrow FP64 pipe) is paid once per thread, not per node.  With
    // FP32 node terms, groups of kGroup nodes are summed in FP32 first and each group
    // sum is added in FP64 (the group sum's rounding is that of its FP32 terms).
    constexpr int kGroup = sizeof(A) == 4 ? 8 : 1;
    A grp[OBS_COUNT];
#pragma unroll
    for (int k = 0; k < OBS_COUNT; ++k) grp[k] = (A)0;
    int in_group = 0;
    // the thread's max |psi_s| and non-finite count, in A and an integer (exact), so
    // that no FP64 operation is paid per node for them
    A tmax = (A)0;
    uint32_t nbad = 0;
    for (uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < a.total;
         gid += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)gid;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * a.g.V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
        const char* base = a.prev + cell_off;
        const uint32_t node_bytes = C * 2 * sizeof(R);
        Cx<A> ps[C], L[C], Hl[C], Hn[C];
        A rho = 0;
        {
            Cx<R> pv[C];
            ld_node<R, C, true>(base + l * node_bytes, pv);  // whole records
#pragma unroll
            for (int s = 0; s < C; ++s) {
                ps[s] = cx<A>((A)pv[s].x, (A)pv[s].y);
                L[s] = Hl[s] = Hn[s] = cx<A>((A)0, (A)0);
                const A n2 = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
                rho += n2;
                tmax = fmax(tmax, sqrt(n2));
                if (!isfinite(ps[s].x) || !isfinite(ps[s].y)) ++nbad;
            }
        }
        if (a.tab.uniform_deg == 4) {
            // 4 entries: table vectors, the 4 neighbour loads issued together
            const NodeTab<A, 4> t = node_tab<A, 4>(st, l);
            Cx<R> nv[4][C];
#pragma unroll
            for (int k = 0; k < 4; ++k) ld_node<R, C, true>(base + t.off[k], nv[k]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
#pragma unroll
                for (int s = 0; s < C; ++s) L[s] += t.w[k] * (cx<A>((A)nv[k][s].x, (A)nv[k][s].y) - ps[s]);
            }
        } else {
            for (int f = st.row_ptr[l]; f < st.row_ptr[l + 1]; ++f) {
                Cx<R> nv[C];
                ld_node<R, C, true>(base + st.nb_off[f], nv);
#pragma unroll
                for (int s = 0; s < C; ++s) L[s] += st.w[f] * (cx<A>((A)nv[s].x, (A)nv[s].y) - ps[s]);
            }
        }
        const PhysR<A>& P = make_phys<A>(a);
        A r[3];
        r[0] = P.p0[0] + P.bs * ((A)x * P.bw[0] + st.pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((A)y * P.bw[1] + st.pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((A)z * P.bw[2] + st.pos[3 * l + 2]);
        local_terms<A, C>(P, r, trap<A>(P, r), GPE_MODE_LEAPFROG, false, ps, Hl);
        // interaction-only part: no trap, no external field, no loss / quadratic
        // Zeeman.  Scalars: psi^H (c0 n) psi = c0 n^2; spin-1: psi^H [c0 n +
        // c2 <F>.F] psi = c0 n^2 + c2 |<F>|^2 with <F> = (Re m, Im m, n_1 - n_-1),
        // m = sqrt2 (psi_1* psi_0 + psi_0* psi_-1); spin-2 through local_terms.
        A kin = 0, hl = 0, hn = 0;
        if constexpr (C == 1) {
            hn = P.c0 * rho * rho;
        } else if constexpr (C == 3) {
            const Cx<A> m = (A)GPE_REF_SQRT_2 * (conj(ps[0]) * ps[1] + conj(ps[1]) * ps[2]);
            const A fz = (ps[0].x * ps[0].x + ps[0].y * ps[0].y) - (ps[2].x * ps[2].x + ps[2].y * ps[2].y);
            hn = P.c0 * rho * rho + P.c2 * (m.x * m.x + m.y * m.y + fz * fz);
        } else {
            PhysR<A> Q = P;
            Q.bq = Q.bqq = 0;
            for (int k = 0; k < 3; ++k) Q.bb[k] = Q.bbq[k] = 0;
            Q.flags &= ~(GPE_FLAG_THREE_BODY_LOSS | GPE_FLAG_QUADRATIC_ZEEMAN | GPE_FLAG_QUADRUPOLE_OFFSET);
            local_terms<A, C>(Q, r, (A)0, GPE_MODE_LEAPFROG, false, ps, Hn);
#pragma unroll
            for (int s = 0; s < C; ++s) hn += ps[s].x * Hn[s].x + ps[s].y * Hn[s].y;
        }
#pragma unroll
        for (int s = 0; s < C; ++s) {
            kin += ps[s].x * L[s].x + ps[s].y * L[s].y;
            hl += ps[s].x * Hl[s].x + ps[s].y * Hl[s].y;
        }
        A v[OBS_COUNT];
#pragma unroll
        for (int k = 0; k < OBS_COUNT; ++k) v[k] = (A)0;
        v[OBS_NORM] = rho;
        v[OBS_HEXP] = kin + hl;
        v[OBS_EINT] = hn;
        v[OBS_COMX] = rho * r[0];
        v[OBS_COMY] = rho * r[1];
        v[OBS_COMZ] = rho * r[2];
        if constexpr (C == 3) {
            const Cx<A> m = (A)GPE_REF_SQRT_2 * (conj(ps[0]) * ps[1] + conj(ps[1]) * ps[2]);
            const A fz = (ps[0].x * ps[0].x + ps[0].y * ps[0].y) - (ps[2].x * ps[2].x + ps[2].y * ps[2].y);
            v[OBS_MAGX] = m.x;
            v[OBS_MAGY] = m.y;
            v[OBS_MAGZ] = fz;
            v[OBS_SPIN] = sqrt(m.x * m.x + m.y * m.y + fz * fz);
        } else if constexpr (C == 5) {
            const Cx<A> fp = (A)2 * (conj(ps[0]) * ps[1] + conj(ps[3]) * ps[4]) +
                             (A)2.449489742783178098 * (conj(ps[1]) * ps[2] + conj(ps[2]) * ps[3]);
            A n[5];
            for (int s = 0; s < 5; ++s) n[s] = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
            const A fz = (A)2 * n[0] + n[1] - n[3] - (A)2 * n[4];
            v[OBS_MAGX] = fp.x;
            v[OBS_MAGY] = fp.y;
            v[OBS_MAGZ] = fz;
            v[OBS_SPIN] = sqrt(fp.x * fp.x + fp.y * fp.y + fz * fz);
        }
        if constexpr (kGroup == 1) {
            // FP64 node terms: the sums as they were (kin + hl added in FP64)
#pragma unroll
            for (int k = 0; k < OBS_COUNT; ++k)
                if (k != OBS_MAXABS && k != OBS_NONFINITE) acc[k] += (double)v[k];
        } else {
#pragma unroll
            for (int k = 0; k < OBS_COUNT; ++k) grp[k] += v[k];
            if (++in_group == kGroup) {
#pragma unroll
                for (int k = 0; k < OBS_COUNT; ++k)
                    if (k != OBS_MAXABS && k != OBS_NONFINITE) acc[k] += (double)grp[k];
#pragma unroll
                for (int k = 0; k < OBS_COUNT; ++k) grp[k] = (A)0;
                in_group = 0;
            }
        }
    }
    if constexpr (kGroup > 1) {
#pragma unroll
        for (int k = 0; k < OBS_COUNT; ++k)
            if (k != OBS_MAXABS && k != OBS_NONFINITE) acc[k] += (double)grp[k];
    }
    acc[OBS_MAXABS] = (double)tmax;
    acc[OBS_NONFINITE] = (double)nbad;
    // warp reduction
#pragma unroll
    for (int k = 0; k < OBS_COUNT; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_down_sync(0xffffffffu, v, o);
            v = (k == OBS_MAXABS) ? fmax(v, u) : v + u;
        }
        acc[k] = v;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < OBS_COUNT; ++k) red[warp][k] = acc[k];
    }
    __syncthreads();
    if (threadIdx.x < OBS_COUNT) {
        const int k = threadIdx.x;
        double v = red[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = (k == OBS_MAXABS) ? fmax(v, red[w][k]) : v + red[w][k];
        a.partials[(size_t)blockIdx.x * OBS_COUNT + k] = v;
    }
}

// Adds nblocks x OBS_COUNT partials into out[OBS_COUNT] with one block of 256
// threads; the order of additions depends only on nblocks.
static __global__ void __launch_bounds__(256) observe_finalize_kernel(const double* partials, uint32_t nblocks, double* out) {
    __shared__ double red[256];
    for (int k = 0; k < OBS_COUNT; ++k) {
        double v = (k == OBS_MAXABS) ? 0.0 : 0.0;
        for (uint32_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
            const double u = partials[(size_t)b * OBS_COUNT + k];
            v = (k == OBS_MAXABS) ? fmax(v, u) : v + u;
        }
        red[threadIdx.x] = v;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s)
                red[threadIdx.x] = (k == OBS_MAXABS) ? fmax(red[threadIdx.x], red[threadIdx.x + s])
                                                     : red[threadIdx.x] + red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[k] = red[0];
        __syncthreads();
    }
}

// The squared norm sum_nodes |psi|^2 of a psi buffer alone (density + integrate,
// Spin1GpeBCC.cu:191-211, 328-348, for normalize_h :955-975): grid-stride, whole-
// record loads, the per-node terms in the storage precision (FP32 storage: groups
// of 8 nodes summed in FP32, each group added in FP64), FP64 block sums written to
// the OBS_NORM column of the partials (the other columns zero) for
// observe_finalize_kernel.
template <typename R, int C>
__global__ void __launch_bounds__(256) norm_kernel(StepArgs a) {
    __shared__ double red[8];
    constexpr int kGroup = sizeof(R) == 4 ? 8 : 1;
    double acc = 0.0;
    R grp = (R)0;
    int in_group = 0;
    const uint32_t node_bytes = C * 2 * sizeof(R);
    for (uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < a.total;
         gid += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)gid;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * a.g.V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        Cx<R> v[C];
        ld_node<R, C, true>(a.prev + (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes +
                                l * node_bytes, v);
        R n2 = 0;
#pragma unroll
        for (int s = 0; s < C; ++s) n2 += v[s].x * v[s].x + v[s].y * v[s].y;
        grp += n2;
        if (++in_group == kGroup) {
            acc += (double)grp;
            grp = (R)0;
            in_group = 0;
        }
    }
    acc += (double)grp;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x < OBS_COUNT) {
        double v = 0.0;
        if (threadIdx.x == OBS_NORM)
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
        a.partials[(size_t)blockIdx.x * OBS_COUNT + threadIdx.x] = v;
    }
}

// Scale every interior value of a psi buffer by 1/sqrt(norm) where norm is read
// from device memory (normalize, Spin1GpeBCC.cu:412-434: FP64 storage divides by
// the square root as the reference does; FP32 storage multiplies by its
// reciprocal, computed in FP64 and rounded once).
template <typename R, int C>
__global__ void __launch_bounds__(256) scale_kernel(StepArgs a, const double* norm_sum, double dv) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= a.total) return;
    const uint32_t i = (uint32_t)gid;
    const uint32_t row = fdiv(i, a.divRow);
    const uint32_t within = i - row * a.row_items;
    const uint32_t x = fdiv(within, a.divV);
    const uint32_t l = within - x * a.g.V;
    const uint32_t z = fdiv(row, a.divY);
    const uint32_t y = row - z * a.g.Y;
    const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
    char* p = a.next + cell_off + l * (C * 2 * sizeof(R));
    const double sq = sqrt(norm_sum[OBS_NORM] * dv);
    if constexpr (sizeof(R) == 8) {
#pragma unroll
        for (int s = 0; s < C; ++s) {
            Cx<R> v = ldc_rw<R>(p + s * 2 * sizeof(R));
            v.x = v.x / sq;
            v.y = v.y / sq;
            stc<R>(p + s * 2 * sizeof(R), v);
        }
    } else {
        const R inv = (R)(1.0 / sq);
        Cx<R> v[C];
        ld_node<R, C, false>(p, v);
#pragma unroll
        for (int s = 0; s < C; ++s) v[s] = inv * v[s];
        st_node<R, C>(p, v);
    }
}

// ---------------------------------------------------------------- launchers

inline unsigned nblocks(uint64_t items, unsigned bs) { return (unsigned)((items + bs - 1) / bs); }

// One wave of resident blocks (the kernel's occupancy x SMs), fewer for small grids.
// D > 0: the fixed-node kernel (see parabolic_fixed_kernel for D, G, MORE).
template <typename R, int C, int MODE, int D, int G, bool MORE, bool OBS = false>
cudaError_t launch_parabolic_m(const StepArgs& a, cudaStream_t s, unsigned* grid = nullptr) {
    if constexpr (D > 0) {
        // the largest multiple of V / gcd(V, 256) blocks within one wave: the grid
        // stride is then a multiple of V
        auto kf = OBS ? parabolic_fixed_obs_kernel<R, C, MODE, D, G, MORE> : parabolic_fixed_kernel<R, C, MODE, D, G, MORE>;
        static int occ_f = 0;
        if (occ_f == 0) {
            // a small shared-memory share leaves the rest of L1 to cache the gathers; the
            // observed step also holds its FP64 sums there (20 KB per block)
            cudaFuncSetAttribute(kf, cudaFuncAttributePreferredSharedMemoryCarveout, OBS ? 50 : 25);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, kf, 256, 0);
            if (occ_f < 1) occ_f = 1;
        }
        uint32_t gv = a.g.V, gb = 256;
        while (gb) {
            const uint32_t r = gv % gb;
            gv = gb;
            gb = r;
        }
        const uint32_t m = a.g.V / gv;
        const uint64_t wave = std::min<uint64_t>((uint64_t)occ_f * (unsigned)device_sm_count(), (a.total + 255) / 256);
        const unsigned nb = (unsigned)(wave / m * m);
        if (nb > 0) {
            kf<<<nb, 256, 0, s>>>(a);
            if (grid) *grid = nb;
            return cudaGetLastError();
        }
    }
    // grids smaller than V / gcd(V, 256) blocks: the grid-stride kernel (the
    // 4-entry form where every node has 4 entries)
    constexpr int DS = (D == 4 && !MORE) ? 4 : 0;
    auto ks = OBS ? parabolic_step_obs_kernel<R, C, MODE, DS> : parabolic_step_kernel<R, C, MODE, DS>;
    static int occ = 0;
    if (occ == 0) {
        // a small shared-memory share leaves the rest of L1 to cache the gathers
        cudaFuncSetAttribute(ks, cudaFuncAttributePreferredSharedMemoryCarveout, OBS ? 50 : 25);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ks, 256, 0);
        if (occ < 1) occ = 1;
    }
    const unsigned nb = std::min<unsigned>(nblocks(a.total, 256), (unsigned)occ * (unsigned)device_sm_count());
    if (nb) ks<<<nb, 256, 0, s>>>(a);
    if (grid) *grid = nb;
    return cudaGetLastError();
}

template <typename R, int C, int D, int G = D, bool MORE = false>
cudaError_t launch_parabolic_d(const StepArgs& a, int mode, cudaStream_t s) {
    switch (mode) {
        case GPE_MODE_LEAPFROG: return launch_parabolic_m<R, C, GPE_MODE_LEAPFROG, D, G, MORE>(a, s);
        case GPE_MODE_EULER: return launch_parabolic_m<R, C, GPE_MODE_EULER, D, G, MORE>(a, s);
        case kModeLeapfrogFrom: return launch_parabolic_m<R, C, kModeLeapfrogFrom, D, G, MORE>(a, s);
        default: return launch_parabolic_m<R, C, GPE_MODE_ITP, D, G, MORE>(a, s);
    }
}

// The kernel form by the lattice's row lengths: every node 4 entries (BCC, A15,
// C15, Z), every row a multiple of 4 long (FCC: 4 and 8), every node 6 entries
// (the cube); others the general grid-stride kernel.
template <typename R, int C>
cudaError_t launch_parabolic(const StepArgs& a, int mode, cudaStream_t s) {
    if (a.total == 0) return cudaSuccess;
    if constexpr (C <= 3) {
        if (a.tab.uniform_deg == 4) return launch_parabolic_d<R, C, 4>(a, mode, s);
        if (a.tab.quad_rows) return launch_parabolic_d<R, C, 4, 4, true>(a, mode, s);
        if (a.tab.uniform_deg == 6) return launch_parabolic_d<R, C, 6, (C == 1 ? 6 : 3)>(a, mode, s);
    } else {
        if (a.tab.uniform_deg == 4) return launch_parabolic_d<R, C, 4, 2>(a, mode, s);
        if (a.tab.quad_rows) return launch_parabolic_d<R, C, 4, 2, true>(a, mode, s);
        if (a.tab.uniform_deg == 6) return launch_parabolic_d<R, C, 6, 2>(a, mode, s);
    }
    return launch_parabolic_d<R, C, 0>(a, mode, s);
}

// A leapfrog step that also sums the observables of the state it reads (ObsAcc):
// block partials into a.partials, then the fixed-order finalize into out.
template <typename R, int C>
cudaError_t launch_parabolic_observe(const StepArgs& a, double* out, cudaStream_t s) {
    if (a.total == 0) return cudaErrorInvalidValue;
    unsigned nb = 0;
    cudaError_t e;
    constexpr int G4 = C <= 3 ? 4 : 2;
    if (a.tab.uniform_deg == 4) e = launch_parabolic_m<R, C, GPE_MODE_LEAPFROG, 4, G4, false, true>(a, s, &nb);
    else if (a.tab.quad_rows) e = launch_parabolic_m<R, C, GPE_MODE_LEAPFROG, 4, G4, true, true>(a, s, &nb);
    else if (a.tab.uniform_deg == 6)
        e = launch_parabolic_m<R, C, GPE_MODE_LEAPFROG, 6, (C == 1 ? 6 : (C == 3 ? 3 : 2)), false, true>(a, s, &nb);
    else e = launch_parabolic_m<R, C, GPE_MODE_LEAPFROG, 0, 0, false, true>(a, s, &nb);
    if (e != cudaSuccess) return e;
    observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    return cudaGetLastError();
}

// kinds of hyperbolic launches
enum HyperKind {
    HK_FUSED_LEAPFROG = 0,   // psi (hyperbolic, leapfrog) + q (hyperbolic leapfrog)
    HK_PSI_PARA_LEAPFROG,    // psi only, parabolic kinetic from q, leapfrog
    HK_PSI_PARA_EULER,       // psi only, parabolic, forward Euler (start step)
    HK_PSI_HYPER_EULER,      // psi only, hyperbolic, forward Euler
    HK_PSI_PARA_ITP,         // psi only, parabolic, imaginary time
    HK_Q_PARA,               // q = d0 psi
    HK_Q_EULER_HYPER,        // q = q + i dt/sigma (q + d0 psi)
    HK_Q_HYPER,              // q += i 2 dt/sigma (q + d0 psi)
    HK_FUSED_ITP             // psi (parabolic kinetic from q, imaginary time, H psi out) + q relaxation
};

// One hyper_step_kernel launch over vb item blocks, on at most one wave.
template <typename R, int C, bool DO_PSI, int MODE, bool HYPERB, int QM>
cudaError_t launch_hyper_k(const StepArgs& a, uint32_t nn, uint32_t ne, uint32_t ratio, unsigned vb, cudaStream_t s) {
    static int occ = 0;
    if (occ == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, hyper_step_kernel<R, C, DO_PSI, MODE, HYPERB, QM>, 256, 0);
        if (occ < 1) occ = 1;
    }
    const unsigned nb = std::min(vb, (unsigned)occ * (unsigned)device_sm_count());
    if (nb) hyper_step_kernel<R, C, DO_PSI, MODE, HYPERB, QM><<<nb, 256, 0, s>>>(a, nn, ne, ratio, vb);
    return cudaGetLastError();
}

template <typename R, int C>
cudaError_t launch_hyper(const StepArgs& a, int kind, cudaStream_t s) {
    const uint32_t nn = (uint32_t)((uint64_t)a.g.X * a.g.Y * a.g.Z * a.g.V);
    const uint32_t ne = (uint32_t)((uint64_t)a.g.X * a.g.Y * a.g.Z * a.g.E);
    const uint32_t ratio = a.g.V ? (a.g.E + a.g.V - 1) / a.g.V : 1;
    const unsigned nbn = nblocks(nn, 256), nbe = nblocks(ne, 256);
    // every group of (1 + ratio) blocks holds one node block and `ratio` edge blocks
    const unsigned groups = nbn > (nbe + ratio - 1) / ratio ? nbn : (nbe + ratio - 1) / ratio;
    switch (kind) {
        case HK_FUSED_LEAPFROG:
            return launch_hyper_k<R, C, true, GPE_MODE_LEAPFROG, true, 0>(a, nn, ne, ratio, groups * (1 + ratio), s);
        case HK_FUSED_ITP:
            return launch_hyper_k<R, C, true, GPE_MODE_ITP, false, 3>(a, nn, ne, ratio, groups * (1 + ratio), s);
        case HK_PSI_PARA_LEAPFROG: return launch_hyper_k<R, C, true, GPE_MODE_LEAPFROG, false, -1>(a, nn, ne, ratio, nbn, s);
        case HK_PSI_PARA_EULER: return launch_hyper_k<R, C, true, GPE_MODE_EULER, false, -1>(a, nn, ne, ratio, nbn, s);
        case HK_PSI_HYPER_EULER: return launch_hyper_k<R, C, true, GPE_MODE_EULER, true, -1>(a, nn, ne, ratio, nbn, s);
        case HK_PSI_PARA_ITP: return launch_hyper_k<R, C, true, GPE_MODE_ITP, false, -1>(a, nn, ne, ratio, nbn, s);
        case HK_Q_PARA: return launch_hyper_k<R, C, false, GPE_MODE_LEAPFROG, false, 1>(a, nn, ne, ratio, nbe, s);
        case HK_Q_EULER_HYPER: return launch_hyper_k<R, C, false, GPE_MODE_LEAPFROG, false, 2>(a, nn, ne, ratio, nbe, s);
        default: return launch_hyper_k<R, C, false, GPE_MODE_LEAPFROG, false, 0>(a, nn, ne, ratio, nbe, s);
    }
}

// Real/imaginary split scalar scheme on the dual edges (RelativisticGpeC15/
// GPUGrossPitaevskii_C15.cu:90-155, time loop :477-482).  psi = R + iI and q = q_R +
// i q_I are the two halves of one complex value (R and I staggered by half a step);
// a.next is the psi buffer and a.qnext the q buffer, both updated in place.
//   PART 0 (first half of a step):  I   -= dt [(V + g(R^2 + I^2)) R - sum_f w_f q_R],
//                                   q_I += (dt/sigma)(q_R + d0 R)
//   PART 1 (second half):           R   += dt [(V + g(I^2 + R^2)) I - sum_f w_f q_I],
//                                   q_R -= (dt/sigma)(q_I + d0 I)
//   PART 2 (start, :469):           q_R += c (q_R + d0 R),  c = qinit
// with w_f = -0.5 h_f / bs^2 (the reference folds dt into V, g and the Hodge weights).
// A half-step reads one half of every value and writes the other (a node also reads
// the half it writes, of its own value only), so the node and edge updates of a
// half-step share one launch, laid out in groups of 1 + E/V blocks of 256 items as
// the hyperbolic step is.  The grid strides over these `vblocks` item blocks on one
// wave, so that each block stages the tables once.  Plain loads: lines read here
// are written by the same launch.
template <typename R, int PART>
__global__ void __launch_bounds__(256) split_step_kernel(StepArgs a, uint32_t node_items, uint32_t edge_items,
                                                         uint32_t ratio, R qinit, uint32_t vblocks) {
    __shared__ SmemHyper<R> sh;
    const int V = a.g.V, E = a.g.E, F = a.tab.faces;
    for (int i = threadIdx.x; i < V * F; i += blockDim.x) {
        sh.inc_off[i] = a.tab.inc_off[i];
        if constexpr (sizeof(R) == 4) sh.inc_w[i] = a.tab.inc_w32[i];
        else sh.inc_w[i] = a.tab.inc_w64[i];
    }
    for (int i = threadIdx.x; i < E; i += blockDim.x) {
        sh.e_from[i] = a.tab.e_from_off[i];
        sh.e_to[i] = a.tab.e_to_off[i];
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) sh.pos[i] = a.tab.pos32[i];
        else sh.pos[i] = a.tab.pos64[i];
    }
    __syncthreads();
    constexpr bool kNodes = PART != 2;
    const PhysR<R>& P = make_phys<R>(a);
    // the half read by the psi update and by d0 (R for PARTs 0 and 2, I for PART 1)
    constexpr uint32_t rd = PART == 1 ? sizeof(R) : 0;
    constexpr uint32_t wr = sizeof(R) - rd;
    for (uint32_t vb = blockIdx.x; vb < vblocks; vb += gridDim.x) {
    uint32_t group, sub;
    if (kNodes) {
        group = vb / (1 + ratio);
        sub = vb - group * (1 + ratio);
    } else {
        group = 0;
        sub = 1 + vb;
    }
    if (kNodes && sub == 0) {
        const uint32_t i = group * blockDim.x + threadIdx.x;
        if (i >= node_items) continue;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
        const size_t qcell_off = (size_t)z * a.g.qslice + (size_t)y * a.g.qpitch + (size_t)x * a.g.qcell_bytes;
        char* own = a.next + cell_off + l * 2 * sizeof(R);
        const Cx<R> v = ldc_rw<R>(own);
        const char* qb = a.qnext + qcell_off + rd;
        R d1q = (R)0;
        if (F == 4) {
            // the 4 incident q values loaded together, tables as vectors
            int32_t off[4];
            R w[4], qv[4];
            incidences4<R>(sh, l, off, w);
#pragma unroll
            for (int k = 0; k < 4; ++k) qv[k] = *reinterpret_cast<const R*>(qb + off[k]);
#pragma unroll
            for (int k = 0; k < 4; ++k) d1q += w[k] * qv[k];
        } else {
            for (int k = 0; k < F; ++k) d1q += sh.inc_w[l * F + k] * *reinterpret_cast<const R*>(qb + sh.inc_off[l * F + k]);
        }
        R r[3];
        r[0] = P.p0[0] + P.bs * ((R)x * P.bw[0] + sh.pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((R)y * P.bw[1] + sh.pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + sh.pos[3 * l + 2]);
        const R tp = trap<R>(P, r) + P.c0 * (v.x * v.x + v.y * v.y);
        if constexpr (PART == 0) *reinterpret_cast<R*>(own + wr) = v.y - P.dt * (tp * v.x - d1q);
        else *reinterpret_cast<R*>(own + wr) = v.x + P.dt * (tp * v.y - d1q);
    } else {
        const uint32_t eb = (kNodes ? group * ratio : 0) + (sub - 1);
        const uint32_t i = eb * blockDim.x + threadIdx.x;
        if (i >= edge_items) continue;
        const uint32_t row = fdiv(i, a.divRowE);
        const uint32_t within = i - row * a.row_items_e;
        const uint32_t x = fdiv(within, a.divE);
        const uint32_t e = within - x * E;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
        const size_t qcell_off = (size_t)z * a.g.qslice + (size_t)y * a.g.qpitch + (size_t)x * a.g.qcell_bytes;
        const char* pb = a.next + cell_off + rd;
        const R d0 = *reinterpret_cast<const R*>(pb + sh.e_to[e]) - *reinterpret_cast<const R*>(pb + sh.e_from[e]);
        char* qe = a.qnext + qcell_off + e * 2 * sizeof(R);
        const R qr = *reinterpret_cast<const R*>(qe + rd);
        if constexpr (PART == 0) *reinterpret_cast<R*>(qe + wr) += P.dts * (qr + d0);
        else if constexpr (PART == 1) *reinterpret_cast<R*>(qe + wr) -= P.dts * (qr + d0);
        else *reinterpret_cast<R*>(qe) = qr + qinit * (qr + d0);
    }
    }
}

// part: 0/1 the two half-steps, 2 the start; qinit is PART 2's coefficient.
template <typename R>
cudaError_t launch_split(const StepArgs& a, int part, double qinit, cudaStream_t s) {
    const uint32_t nn = (uint32_t)((uint64_t)a.g.X * a.g.Y * a.g.Z * a.g.V);
    const uint32_t ne = (uint32_t)((uint64_t)a.g.X * a.g.Y * a.g.Z * a.g.E);
    const uint32_t ratio = a.g.V ? (a.g.E + a.g.V - 1) / a.g.V : 1;
    const unsigned nbn = nblocks(nn, 256), nbe = nblocks(ne, 256);
    const unsigned groups = nbn > (nbe + ratio - 1) / ratio ? nbn : (nbe + ratio - 1) / ratio;
    if (nn == 0) return cudaSuccess;
    static int occ = 0;
    if (occ == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, split_step_kernel<R, 0>, 256, 0);
        if (occ < 1) occ = 1;
    }
    const unsigned wave = (unsigned)occ * (unsigned)device_sm_count();
    const unsigned vb = part == 2 ? nbe : groups * (1 + ratio);
    const unsigned nb = std::min(vb, wave);
    switch (part) {
        case 0: split_step_kernel<R, 0><<<nb, 256, 0, s>>>(a, nn, ne, ratio, (R)0, vb); break;
        case 1: split_step_kernel<R, 1><<<nb, 256, 0, s>>>(a, nn, ne, ratio, (R)0, vb); break;
        default: split_step_kernel<R, 2><<<nb, 256, 0, s>>>(a, nn, ne, ratio, (R)qinit, vb); break;
    }
    return cudaGetLastError();
}

// node_fp32: per-node terms in FP32 (FP32 storage only); sums are FP64 either way.
template <typename R, int C>
cudaError_t launch_observe(const StepArgs& a, double* out, bool node_fp32, cudaStream_t s) {
    // one wave of resident blocks (fewer for small grids); the partial sums are added
    // in an order that depends only on the grid size
    static int occ32 = 0, occ64 = 0;
    if (occ32 == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ32, observe_kernel<R, C, float>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, observe_kernel<R, C, double>, 256, 0);
        occ32 = std::max(occ32, 1);
        occ64 = std::max(occ64, 1);
    }
    const bool f32 = sizeof(R) == 4 && node_fp32;
    const unsigned nb =
        std::min<unsigned>(nblocks(a.total, 256), (unsigned)(f32 ? occ32 : occ64) * (unsigned)device_sm_count());
    if (f32) observe_kernel<R, C, float><<<nb, 256, 0, s>>>(a);
    else observe_kernel<R, C, double><<<nb, 256, 0, s>>>(a);
    observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    return cudaGetLastError();
}

template <typename R, int C>
cudaError_t launch_norm(const StepArgs& a, double* out, cudaStream_t s) {
    static int occ = 0;
    if (occ == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, norm_kernel<R, C>, 256, 0);
        occ = std::max(occ, 1);
    }
    const unsigned nb = std::min<unsigned>(nblocks(a.total, 256), (unsigned)occ * (unsigned)device_sm_count());
    norm_kernel<R, C><<<nb, 256, 0, s>>>(a);
    observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    return cudaGetLastError();
}

template <typename R, int C>
cudaError_t launch_scale(const StepArgs& a, const double* norm_sum, double dv, cudaStream_t s) {
    scale_kernel<R, C><<<nblocks(a.total, 256), 256, 0, s>>>(a, norm_sum, dv);
    return cudaGetLastError();
}

#define GPE_INSTANTIATE(R, C)                                                               \
    template cudaError_t launch_parabolic<R, C>(const StepArgs&, int, cudaStream_t);       \
    template cudaError_t launch_parabolic_observe<R, C>(const StepArgs&, double*, cudaStream_t); \
    template cudaError_t launch_hyper<R, C>(const StepArgs&, int, cudaStream_t);           \
    template cudaError_t launch_observe<R, C>(const StepArgs&, double*, bool, cudaStream_t);     \
    template cudaError_t launch_scale<R, C>(const StepArgs&, const double*, double, cudaStream_t); \
    template cudaError_t launch_norm<R, C>(const StepArgs&, double*, cudaStream_t);

}  // namespace gpe

namespace gpe {

// sum_interior Re(conj(a) b) into partials[.][OBS_NORM] (innerProduct,
// Spin1GpeBCC.cu:213-233); a = StepArgs::prev, b = StepArgs::next.
template <typename R, int C>
__global__ void __launch_bounds__(256) dot_kernel(StepArgs a) {
    __shared__ double red[8];
    double acc = 0;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid < a.total) {
        const uint32_t i = (uint32_t)gid;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * a.g.V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        const size_t off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes + l * (C * 2 * sizeof(R));
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const Cx<R> u = ldc<R>(a.prev + off + s * 2 * sizeof(R));
            const Cx<R> v = ldc<R>(a.next + off + s * 2 * sizeof(R));
            acc += (double)u.x * (double)v.x + (double)u.y * (double)v.y;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < OBS_COUNT) {
        double v = 0;
        if (threadIdx.x == OBS_NORM)
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
        a.partials[(size_t)blockIdx.x * OBS_COUNT + threadIdx.x] = v;
    }
}

template <typename R, int C>
cudaError_t launch_dot_t(const StepArgs& a, double* out, cudaStream_t s) {
    const unsigned nb = nblocks(a.total, 256);
    dot_kernel<R, C><<<nb, 256, 0, s>>>(a);
    observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    return cudaGetLastError();
}

}  // namespace gpe

namespace gpe {

// Copy between a packed FP64 array in the reference file layout
// ((Z+2)(Y+2)(X+2) cells of `vals` doubles, halo included) and a pitched device
// buffer of storage type R.  TO_DEVICE: interior cells are converted, the device
// halo is left untouched (zero).  Otherwise the packed array receives the
// interior values and zeros in the halo.  `packed` may be device memory or pinned
// host memory (read and written over the host link).  W32: the element count
// fits 32 bits, and the index arithmetic uses 32-bit multiply-shift divisions.
template <typename R, bool TO_DEVICE, bool W32>
__global__ void __launch_bounds__(256) pack_kernel(double* packed, char* dev_base, uint32_t X, uint32_t Y, uint32_t Z,
                                                   uint32_t vals, size_t pitch, size_t slice, uint64_t total,
                                                   FastDiv dvals, FastDiv dx, FastDiv dy) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x, y, z, within;
        if constexpr (W32) {
            const uint32_t i32 = (uint32_t)i;
            const uint32_t cell = fdiv(i32, dvals);
            within = i32 - cell * vals;
            const uint32_t yz = fdiv(cell, dx);
            x = cell - yz * (X + 2);
            z = fdiv(yz, dy);
            y = yz - z * (Y + 2);
        } else {
            const uint64_t cell = i / vals;
            within = (uint32_t)(i - cell * vals);
            x = (uint32_t)(cell % (X + 2));
            const uint64_t yz = cell / (X + 2);
            y = (uint32_t)(yz % (Y + 2));
            z = (uint32_t)(yz / (Y + 2));
        }
        const bool halo = x == 0 || y == 0 || z == 0 || x == X + 1 || y == Y + 1 || z == Z + 1;
        R* d = reinterpret_cast<R*>(dev_base + (size_t)z * slice + (size_t)y * pitch + (size_t)x * vals * sizeof(R)) + within;
        if (TO_DEVICE) {
            if (!halo) *d = (R)packed[i];
        } else {
            packed[i] = halo ? 0.0 : (double)*d;
        }
    }
}

template <typename R>
cudaError_t launch_pack(double* packed, char* dev_base, uint32_t X, uint32_t Y, uint32_t Z, uint32_t vals, size_t pitch,
                        size_t slice, bool to_device, cudaStream_t s) {
    const uint64_t total = (uint64_t)(X + 2) * (Y + 2) * (Z + 2) * vals;
    const unsigned nb = (unsigned)((total + 255) / 256 < 152u * 64u ? (total + 255) / 256 : 152u * 64u);
    const FastDiv dv = make_fastdiv(vals), dx = make_fastdiv(X + 2), dy = make_fastdiv(Y + 2);
    if (total < (1ull << 32)) {
        if (to_device) pack_kernel<R, true, true><<<nb, 256, 0, s>>>(packed, dev_base, X, Y, Z, vals, pitch, slice, total, dv, dx, dy);
        else pack_kernel<R, false, true><<<nb, 256, 0, s>>>(packed, dev_base, X, Y, Z, vals, pitch, slice, total, dv, dx, dy);
    } else {
        if (to_device) pack_kernel<R, true, false><<<nb, 256, 0, s>>>(packed, dev_base, X, Y, Z, vals, pitch, slice, total, dv, dx, dy);
        else pack_kernel<R, false, false><<<nb, 256, 0, s>>>(packed, dev_base, X, Y, Z, vals, pitch, slice, total, dv, dx, dy);
    }
    return cudaGetLastError();
}

}  // namespace gpe

namespace gpe {

// ---------------------------------------------------------- TMA row tiles

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 1-D bulk copy global -> shared completing on an mbarrier (addresses 16-byte
// aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Bounded wait on an mbarrier phase; every thread of the block gets the same
// answer (false only if the copies did not land within the limit).
__device__ __forceinline__ bool block_wait(uint64_t* bar, uint32_t parity, int* err) {
    bool ok = false;
    for (uint32_t spin = 0; spin < (1u << 22) && !(ok = mbar_try_wait(bar, parity)); ++spin) {
    }
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0 && err) atomicExch(err, 1);
    return ok;
}

// Leapfrog step on a row tile of T cells (BCC spin-1 FP32: T = 16 cells,
// 192 nodes, one thread per node).  The previous state of cells [x0-1, x0+T]
// (the x halo included) and the old next state of [x0, x0+T) are brought into
// shared memory by two bulk copies; in-row neighbours (dy = dz = 0) are read
// from shared memory, off-row neighbours from global memory (L2); the updated
// tile goes back with one bulk store.  Requires cell_bytes % 16 == 0.
template <typename R, int C>
__global__ void __launch_bounds__(256) leapfrog_tile_kernel(StepArgs a, uint32_t T, uint32_t tiles_per_row) {
    extern __shared__ __align__(128) unsigned char dyn[];
    __shared__ __align__(8) uint64_t bar;
    const uint32_t cb = a.g.cell_bytes;
    const int V = a.g.V, n = a.tab.entries;
    char* s_prev = reinterpret_cast<char*>(dyn);
    char* s_next = s_prev + (size_t)(T + 2) * cb;
    int32_t* s_goff = reinterpret_cast<int32_t*>(s_next + (size_t)T * cb);
    int32_t* s_soff = s_goff + n;
    R* s_w = reinterpret_cast<R*>(s_soff + n);
    R* s_pos = s_w + n;
    int32_t* s_row = reinterpret_cast<int32_t*>(s_pos + 3 * V);

    const uint32_t tile = blockIdx.x % tiles_per_row;
    const uint32_t row = blockIdx.x / tiles_per_row;
    const uint32_t z = fdiv(row, a.divY);
    const uint32_t y = row - z * a.g.Y;
    const uint32_t x0 = tile * T;
    const uint32_t Tc = min(T, a.g.X - x0);
    const size_t row_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch;
    const char* g_prev = a.prev + row_off + (size_t)x0 * cb - cb;  // cell x0 - 1 (halo at x0 = 0)
    char* g_next = a.next + row_off + (size_t)x0 * cb;
    const uint32_t bytes_prev = (Tc + 2) * cb, bytes_next = Tc * cb;

    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_proxy_async_smem();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, bytes_prev + bytes_next);
        bulk_load(s_prev, g_prev, bytes_prev, &bar);
        bulk_load(s_next, g_next, bytes_next, &bar);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s_goff[i] = a.tab.nb_off[i];
        s_soff[i] = a.tab.nb_soff[i];
        // condensate expansion: weights h / bs^2 of the step's bs
        if constexpr (sizeof(R) == 4) s_w[i] = a.tab.w32[i] * make_phys<R>(a).ks;
        else s_w[i] = a.tab.w64[i] * make_phys<R>(a).ks;
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) s_pos[i] = a.tab.pos32[i];
        else s_pos[i] = a.tab.pos64[i];
    }
    for (int i = threadIdx.x; i <= V; i += blockDim.x) s_row[i] = a.tab.row_ptr[i];
    if (!block_wait(&bar, 0, a.err)) return;  // uniform across the block

    const uint32_t node_bytes = C * 2 * sizeof(R);
    const uint32_t i = threadIdx.x;
    if (i < Tc * V) {
        using V2 = typename Vec2<R>::type;
        const uint32_t xl = fdiv(i, a.divV);
        const uint32_t l = i - xl * V;
        const char* s_own = s_prev + (size_t)(xl + 1) * cb + l * node_bytes;
        const char* g_cell = g_prev + (size_t)(xl + 1) * cb;
        Cx<R> prv[C], H[C];
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const V2 v = reinterpret_cast<const V2*>(s_own)[s];
            prv[s] = cx<R>(v.x, v.y);
            H[s] = cx<R>((R)0, (R)0);
        }
        const char* s_cell = s_own - l * node_bytes;
        const int f0 = s_row[l], f1 = s_row[l + 1];
        for (int f = f0; f < f1; ++f) {
            const int32_t so = s_soff[f];
            const R w = s_w[f];
            if (so != INT32_MIN) {
                // in-row neighbour: shared memory (8- or 16-byte accesses)
                const V2* p = reinterpret_cast<const V2*>(s_cell + so);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const V2 v = p[c];
                    H[c] += w * (cx<R>(v.x, v.y) - prv[c]);
                }
            } else {
                // off-row neighbour: read-only global path (L2)
                const char* g = g_cell + s_goff[f];
#pragma unroll
                for (int c = 0; c < C; ++c) H[c] += w * (ldc<R>(g + c * 2 * sizeof(R)) - prv[c]);
            }
        }
        const PhysR<R>& P = make_phys<R>(a);
        const uint32_t x = x0 + xl;
        R r[3];
        r[0] = P.p0[0] + P.bs * ((R)x * P.bw[0] + s_pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((R)y * P.bw[1] + s_pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + s_pos[3 * l + 2]);
        const R pot = trap<R>(P, r);
        local_terms<R, C>(P, r, pot, GPE_MODE_LEAPFROG, false, prv, H);
        V2* q = reinterpret_cast<V2*>(s_next + (size_t)xl * cb + l * node_bytes);
        const R dt2 = (R)2 * P.dt;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            V2 v = q[c];
            v.x += dt2 * H[c].y;
            v.y += dt2 * -H[c].x;
            q[c] = v;
        }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        bulk_store(g_next, s_next, bytes_next);
        bulk_commit();
        bulk_wait_read_all();
    }
}

template <typename R, int C>
size_t tile_smem_bytes(const StepArgs& a, uint32_t T) {
    return (size_t)(2 * T + 2) * a.g.cell_bytes + (size_t)a.tab.entries * (8 + sizeof(R)) + 3 * a.g.V * sizeof(R) +
           (a.g.V + 1) * 4;
}

template <typename R, int C>
cudaError_t launch_leapfrog_tile(const StepArgs& a, uint32_t T, int carveout, cudaStream_t s) {
    const uint32_t tiles = (a.g.X + T - 1) / T;
    const uint32_t threads = ((T * a.g.V + 31) / 32) * 32;
    const size_t smem = tile_smem_bytes<R, C>(a, T);
    static bool configured = false;
    static int carve = -2;
    if (!configured) {
        cudaFuncSetAttribute(leapfrog_tile_kernel<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    if (carveout != carve) {  // shared-memory share of the unified L1 (the rest caches off-row gathers)
        cudaFuncSetAttribute(leapfrog_tile_kernel<R, C>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             carveout > 0 ? carveout : -1);
        carve = carveout;
    }
    const uint64_t blocks = (uint64_t)tiles * a.g.Y * a.g.Z;
    leapfrog_tile_kernel<R, C><<<(unsigned)blocks, threads, smem, s>>>(a, T, tiles);
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_TILE(R, C) template cudaError_t launch_leapfrog_tile<R, C>(const StepArgs&, uint32_t, int, cudaStream_t);

}  // namespace gpe

namespace gpe {

// ----------------------------------------------------------- 2.5-D z-march

// Packed stencil entry of the z-march kernel: the neighbour's plane (dz) and its
// byte offset inside a (TY+2) x (T+2)-cell slab relative to the own node's cell.
template <typename R>
struct __align__(16) MarchEntry {
    int32_t soff;
    int32_t dz;
    R w;
};
static_assert(sizeof(MarchEntry<float>) == 16 && sizeof(MarchEntry<double>) == 16, "16-byte stencil entries");

struct MarchArgs {
    uint32_t T, TY, ZC;          // cells per row tile, rows per tile, planes per block
    uint32_t tiles_x, tiles_y;   // tiles along x and y
    uint32_t nodes;              // T * TY * V
    FastDiv div_row_nodes;       // T * V
    uint32_t slab_bytes, tile_bytes;
    int uniform_deg;             // > 0: every node has this many entries (no row_ptr lookups)
};

// Leapfrog step, 2.5-D: block = T cells x TY rows of one z-chunk of ZC planes.
// A ring of four slabs holds psi_prev of planes z-1, z, z+1 and the prefetch of
// z+2, each slab the (TY+2) x (T+2) cells around the tile, brought in by TY+2
// bulk copies of contiguous row segments; the old psi_next of the tile is
// double-buffered.  Every neighbour is read from shared memory.  Requires
// cell_bytes % 16 == 0, T | X and TY | Y.
template <typename R, int C>
__global__ void __launch_bounds__(1024) leapfrog_march_kernel(StepArgs a, MarchArgs m) {
    extern __shared__ __align__(128) unsigned char dyn[];
    __shared__ __align__(8) uint64_t bar_slab[4];
    __shared__ __align__(8) uint64_t bar_tile[2];
    using V2 = typename Vec2<R>::type;
    const uint32_t cb = a.g.cell_bytes;
    const int V = a.g.V, n = a.tab.entries;
    char* slab = reinterpret_cast<char*>(dyn);
    char* tilebuf = slab + 4 * (size_t)m.slab_bytes;
    MarchEntry<R>* s_ent = reinterpret_cast<MarchEntry<R>*>(tilebuf + 2 * (size_t)m.tile_bytes);
    R* s_pos = reinterpret_cast<R*>(s_ent + n);
    int32_t* s_row = reinterpret_cast<int32_t*>(s_pos + 3 * V);

    const uint32_t tx = blockIdx.x % m.tiles_x;
    const uint32_t rest = blockIdx.x / m.tiles_x;
    const uint32_t ty = rest % m.tiles_y;
    const uint32_t tz = rest / m.tiles_y;
    const uint32_t x0 = tx * m.T, y0 = ty * m.TY, zb = tz * m.ZC;
    const uint32_t ze = min(zb + m.ZC, a.g.Z);
    const uint32_t seg_bytes = (m.T + 2) * cb;        // one row segment of a slab
    const uint32_t row_bytes = m.T * cb;              // one row of the tile

    // issue the copies of slab for plane zz (zz in [-1, Z]) into ring slot s
    auto load_slab = [&](int zz, int s) {
        mbar_expect_tx(&bar_slab[s], (m.TY + 2) * seg_bytes);
        for (uint32_t r = 0; r < m.TY + 2; ++r) {
            const char* src = a.prev + (ptrdiff_t)zz * (ptrdiff_t)a.g.slice + ((ptrdiff_t)y0 + r - 1) * (ptrdiff_t)a.g.pitch +
                              ((ptrdiff_t)x0 - 1) * cb;
            bulk_load(slab + (size_t)s * m.slab_bytes + (size_t)r * seg_bytes, src, seg_bytes, &bar_slab[s]);
        }
    };
    auto load_tile = [&](uint32_t zz, int s) {
        mbar_expect_tx(&bar_tile[s], m.TY * row_bytes);
        for (uint32_t r = 0; r < m.TY; ++r) {
            const char* src = a.next + (size_t)zz * a.g.slice + (size_t)(y0 + r) * a.g.pitch + (size_t)x0 * cb;
            bulk_load(tilebuf + (size_t)s * m.tile_bytes + (size_t)r * row_bytes, src, row_bytes, &bar_tile[s]);
        }
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < 4; ++s) mbar_init(&bar_slab[s], 1);
        for (int s = 0; s < 2; ++s) mbar_init(&bar_tile[s], 1);
        fence_proxy_async_smem();
    }
    __syncthreads();
    // prologue: slabs of planes zb-1, zb, zb+1 (ring slots 0, 1, 2) and the tile of zb
    if (threadIdx.x == 0) {
        load_slab((int)zb - 1, 0);
        load_slab((int)zb, 1);
        load_slab((int)zb + 1, 2);
        load_tile(zb, 0);
    }
    const uint32_t node_bytes = C * 2 * sizeof(R);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        // slab offset of the neighbour relative to the own cell: (dy (T+2) + dx) cells + node
        const int4 q = a.tab.ent4[i];
        MarchEntry<R> e;
        e.soff = (q.y * (int)(m.T + 2) + q.x) * (int)cb + q.w * (int)node_bytes;
        e.dz = q.z;
        // condensate expansion: weights h / bs^2 of the step's bs
        if constexpr (sizeof(R) == 4) e.w = a.tab.w32[i] * make_phys<R>(a).ks;
        else e.w = a.tab.w64[i] * make_phys<R>(a).ks;
        s_ent[i] = e;
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) s_pos[i] = a.tab.pos32[i];
        else s_pos[i] = a.tab.pos64[i];
    }
    for (int i = threadIdx.x; i <= V; i += blockDim.x) s_row[i] = a.tab.row_ptr[i];
    __syncthreads();

    const PhysR<R>& P = make_phys<R>(a);
    const R dt2 = (R)2 * P.dt;
    uint32_t slab_phase = 0;   // bit s: parity to wait for on slab slot s
    uint32_t tile_phase = 0;
    bool ok = true;
    for (uint32_t z = zb; z < ze; ++z) {
        const uint32_t k = z - zb;
        const int s_mid = (int)((k + 1) & 3), s_lo = (int)(k & 3), s_hi = (int)((k + 2) & 3), s_pre = (int)((k + 3) & 3);
        const int t_cur = (int)(k & 1), t_nxt = (int)((k + 1) & 1);
        if (threadIdx.x == 0) {
            // the store of plane z-1 used tile slot t_nxt: let it finish reading shared memory
            bulk_wait_read_all();
            // prefetch what the next iteration needs (plane z+2 <= Z: plane Z is the zero halo)
            if (z + 1 < ze) {
                load_slab((int)z + 2, s_pre);
                load_tile(z + 1, t_nxt);
            }
        }
        // wait for slab z+1 (slabs z-1 and z were waited for already) and tile z
        if (k == 0) {
            ok = ok && block_wait(&bar_slab[0], 0, a.err);
            ok = ok && block_wait(&bar_slab[1], 0, a.err);
            slab_phase ^= 0x3;
        }
        ok = ok && block_wait(&bar_slab[s_hi], (slab_phase >> s_hi) & 1, a.err);
        slab_phase ^= 1u << s_hi;
        ok = ok && block_wait(&bar_tile[t_cur], (tile_phase >> t_cur) & 1, a.err);
        tile_phase ^= 1u << t_cur;
        if (!ok) break;

        (void)s_lo;
        const char* sl_mid = slab + (size_t)s_mid * m.slab_bytes;
        char* tl = tilebuf + (size_t)t_cur * m.tile_bytes;
        for (uint32_t i = threadIdx.x; i < m.nodes; i += blockDim.x) {
            const uint32_t r = fdiv(i, m.div_row_nodes);
            const uint32_t j = i - r * (m.T * V);
            const uint32_t xl = fdiv(j, a.divV);
            const uint32_t l = j - xl * V;
            const size_t own_cell = ((size_t)(r + 1) * (m.T + 2) + (xl + 1)) * cb;
            const char* own = sl_mid + own_cell + l * node_bytes;
            Cx<R> prv[C], H[C];
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const V2 v = reinterpret_cast<const V2*>(own)[c];
                prv[c] = cx<R>(v.x, v.y);
                H[c] = cx<R>((R)0, (R)0);
            }
            int f0, f1;
            if (m.uniform_deg > 0) {
                f0 = (int)l * m.uniform_deg;
                f1 = f0 + m.uniform_deg;
            } else {
                f0 = s_row[l];
                f1 = s_row[l + 1];
            }
            for (int f = f0; f < f1; ++f) {
                const MarchEntry<R> e = s_ent[f];
                // plane z+dz sits in ring slot (s_mid + dz) mod 4
                const V2* p = reinterpret_cast<const V2*>(slab + (size_t)((s_mid + e.dz) & 3) * m.slab_bytes + own_cell + e.soff);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const V2 v = p[c];
                    H[c] += e.w * (cx<R>(v.x, v.y) - prv[c]);
                }
            }
            R rr[3];
            rr[0] = P.p0[0] + P.bs * ((R)(x0 + xl) * P.bw[0] + s_pos[3 * l + 0]);
            rr[1] = P.p0[1] + P.bs * ((R)(y0 + r) * P.bw[1] + s_pos[3 * l + 1]);
            rr[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + s_pos[3 * l + 2]);
            const R pot = trap<R>(P, rr);
            local_terms<R, C>(P, rr, pot, GPE_MODE_LEAPFROG, false, prv, H);
            V2* q = reinterpret_cast<V2*>(tl + ((size_t)r * m.T + xl) * cb + l * node_bytes);
#pragma unroll
            for (int c = 0; c < C; ++c) {
                V2 v = q[c];
                v.x += dt2 * H[c].y;
                v.y += dt2 * -H[c].x;
                q[c] = v;
            }
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t r = 0; r < m.TY; ++r) {
                char* dst = a.next + (size_t)z * a.g.slice + (size_t)(y0 + r) * a.g.pitch + (size_t)x0 * cb;
                bulk_store(dst, tl + (size_t)r * row_bytes, row_bytes);
            }
            bulk_commit();
        }
    }
    if (threadIdx.x == 0) bulk_wait_read_all();
    if (!ok) {
        // a wait ran out: give the copies in flight a bounded time to land before exiting
        for (int s = 0; s < 4; ++s)
            for (uint32_t spin = 0; spin < (1u << 16) && !mbar_try_wait(&bar_slab[s], (slab_phase >> s) & 1); ++spin) {
            }
    }
}

template <typename R, int C>
size_t march_smem_bytes(const StepArgs& a, const MarchArgs& m) {
    return 4 * (size_t)m.slab_bytes + 2 * (size_t)m.tile_bytes + (size_t)a.tab.entries * sizeof(MarchEntry<R>) +
           3 * a.g.V * sizeof(R) + (a.g.V + 1) * 4;
}

template <typename R, int C>
cudaError_t launch_leapfrog_march(const StepArgs& a, uint32_t T, uint32_t TY, uint32_t ZC, uint32_t threads,
                                  cudaStream_t s) {
    MarchArgs m;
    m.T = T;
    m.TY = TY;
    m.ZC = ZC;
    m.tiles_x = a.g.X / T;
    m.tiles_y = a.g.Y / TY;
    m.nodes = T * TY * a.g.V;
    m.div_row_nodes = make_fastdiv(T * a.g.V);
    m.slab_bytes = (TY + 2) * (T + 2) * a.g.cell_bytes;
    m.tile_bytes = TY * T * a.g.cell_bytes;
    m.uniform_deg = a.tab.uniform_deg;
    const size_t smem = march_smem_bytes<R, C>(a, m);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(leapfrog_march_kernel<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    const uint64_t blocks = (uint64_t)m.tiles_x * m.tiles_y * ((a.g.Z + ZC - 1) / ZC);
    leapfrog_march_kernel<R, C><<<(unsigned)blocks, threads, smem, s>>>(a, m);
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_MARCH(R, C) \
    template cudaError_t launch_leapfrog_march<R, C>(const StepArgs&, uint32_t, uint32_t, uint32_t, uint32_t, cudaStream_t);

}  // namespace gpe

namespace gpe {

// ------------------------------------------------------ multi-row tiles

// Packed stencil entry: byte offset of the neighbour relative to the own cell in
// row buffer 0, and the weight.
template <typename R>
struct __align__(8) RowsEntry {
    int32_t off;
    float w;
};
template <>
struct __align__(16) RowsEntry<double> {
    int32_t off;
    int32_t pad;
    double w;
};

struct RowsArgs {
    uint32_t T;             // cells per tile row
    uint32_t RY, RZ;        // output rows per block along y and z
    uint32_t tiles_x, tiles_y;
    uint32_t K;             // distinct (dy, dz) row offsets of the stencil, (0, 0) first
    uint32_t nbuf;          // row buffers staged per block
    uint32_t row_buf_bytes; // (T + 2) * cell_bytes
    FastDiv div_row_nodes;  // T * V
    const int32_t* blk;     // [nbuf dy][nbuf dz][RY*RZ*K buffer index of (own row, offset k)]
};

// Leapfrog step on a block of RY x RZ output rows (y, z) of T cells each.  Bulk
// copies bring psi_prev of cells [x0-1, x0+T] of every row the block's stencil
// touches (BCC, 2 x 2 rows: 14 rows, 3.5 per output row) into shared memory,
// plus the old psi_next of the block; every neighbour is then read from shared
// memory.  L2 supplies each psi_prev line a few times per step (the measured L2
// bandwidth is ~5x HBM); HBM still sees each value once.  Requires
// cell_bytes % 16 == 0, RY | Y and RZ | Z.
// Launch bounds of the row-block kernel: 384 threads; four resident blocks
// (<= 42 registers) for FP32 with up to three components, two otherwise.
template <typename R, int C>
struct RowsLB {
    static constexpr int threads = 384;
    static constexpr int blocks = (sizeof(R) == 4 && C <= 3) ? 4 : 2;
};

template <typename R, int C>
__global__ void __launch_bounds__(RowsLB<R, C>::threads, RowsLB<R, C>::blocks) leapfrog_rows_kernel(StepArgs a, RowsArgs m) {
    extern __shared__ __align__(128) unsigned char dyn[];
    __shared__ __align__(8) uint64_t bar;
    using V2 = typename Vec2<R>::type;
    const uint32_t cb = a.g.cell_bytes;
    const int V = a.g.V, n = a.tab.entries;
    const uint32_t own_rows = m.RY * m.RZ;
    char* s_rows = reinterpret_cast<char*>(dyn);
    char* s_next = s_rows + (size_t)m.nbuf * m.row_buf_bytes;
    RowsEntry<R>* s_ent = reinterpret_cast<RowsEntry<R>*>(s_next + (size_t)own_rows * m.T * cb);
    R* s_pos = reinterpret_cast<R*>(s_ent + n);
    int32_t* s_row = reinterpret_cast<int32_t*>(s_pos + 3 * V);
    int32_t* s_map = s_row + (V + 1);   // own_rows * K buffer indices

    const uint32_t tx = blockIdx.x % m.tiles_x;
    const uint32_t rest = blockIdx.x / m.tiles_x;
    const uint32_t ty = rest % m.tiles_y;
    const uint32_t tz = rest / m.tiles_y;
    const uint32_t x0 = tx * m.T, y0 = ty * m.RY, z0 = tz * m.RZ;
    const uint32_t Tc = min(m.T, a.g.X - x0);
    const uint32_t bytes_row = (Tc + 2) * cb, bytes_next = Tc * cb;

    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_proxy_async_smem();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, m.nbuf * bytes_row + own_rows * bytes_next);
        for (uint32_t b = 0; b < m.nbuf; ++b) {
            const int dy = m.blk[b], dz = m.blk[m.nbuf + b];
            const char* src = a.prev + ((ptrdiff_t)z0 + dz) * (ptrdiff_t)a.g.slice + ((ptrdiff_t)y0 + dy) * (ptrdiff_t)a.g.pitch +
                              ((ptrdiff_t)x0 - 1) * cb;
            bulk_load(s_rows + (size_t)b * m.row_buf_bytes, src, bytes_row, &bar);
        }
        for (uint32_t q = 0; q < own_rows; ++q) {
            const uint32_t ry = q % m.RY, rz = q / m.RY;
            const char* src = a.next + (size_t)(z0 + rz) * a.g.slice + (size_t)(y0 + ry) * a.g.pitch + (size_t)x0 * cb;
            bulk_load(s_next + (size_t)q * m.T * cb, src, bytes_next, &bar);
        }
    }
    const uint32_t node_bytes = C * 2 * sizeof(R);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int4 q = a.tab.ent4[i];
        RowsEntry<R> e;
        // offset k of (dy, dz) in the high byte, in-row byte offset below
        e.off = (a.tab.ent_row[i] << 24) + (q.x * (int)cb + q.w * (int)node_bytes + (1 << 23));
        // condensate expansion: weights h / bs^2 of the step's bs
        if constexpr (sizeof(R) == 4) e.w = a.tab.w32[i] * make_phys<R>(a).ks;
        else e.w = a.tab.w64[i] * make_phys<R>(a).ks;
        s_ent[i] = e;
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) s_pos[i] = a.tab.pos32[i];
        else s_pos[i] = a.tab.pos64[i];
    }
    for (int i = threadIdx.x; i <= V; i += blockDim.x) s_row[i] = a.tab.row_ptr[i];
    for (uint32_t i = threadIdx.x; i < own_rows * m.K; i += blockDim.x) s_map[i] = m.blk[2 * m.nbuf + i];
    if (!block_wait(&bar, 0, a.err)) return;  // uniform across the block

    const PhysR<R>& P = make_phys<R>(a);
    const R dt2 = (R)2 * P.dt;
    const uint32_t tile_nodes = Tc * V;
    for (uint32_t i = threadIdx.x; i < own_rows * m.T * V; i += blockDim.x) {
        const uint32_t q = fdiv(i, m.div_row_nodes);
        const uint32_t j = i - q * (m.T * V);
        if (j >= tile_nodes) continue;
        const uint32_t xl = fdiv(j, a.divV);
        const uint32_t l = j - xl * V;
        const int32_t* map = s_map + q * m.K;
        const size_t cell_in_row = (size_t)(xl + 1) * cb;
        const char* own = s_rows + (size_t)map[0] * m.row_buf_bytes + cell_in_row + l * node_bytes;
        Cx<R> prv[C], H[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const V2 v = reinterpret_cast<const V2*>(own)[c];
            prv[c] = cx<R>(v.x, v.y);
            H[c] = cx<R>((R)0, (R)0);
        }
        int f0, f1;
        if (a.tab.uniform_deg > 0) {
            f0 = (int)l * a.tab.uniform_deg;
            f1 = f0 + a.tab.uniform_deg;
        } else {
            f0 = s_row[l];
            f1 = s_row[l + 1];
        }
        for (int f = f0; f < f1; ++f) {
            const RowsEntry<R> e = s_ent[f];
            const int k = e.off >> 24;
            const int in_row = (e.off & 0xffffff) - (1 << 23);
            const V2* p = reinterpret_cast<const V2*>(s_rows + (size_t)map[k] * m.row_buf_bytes + cell_in_row + in_row);
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const V2 v = p[c];
                H[c] += (R)e.w * (cx<R>(v.x, v.y) - prv[c]);
            }
        }
        const uint32_t ry = q % m.RY, rz = q / m.RY;
        R r[3];
        r[0] = P.p0[0] + P.bs * ((R)(x0 + xl) * P.bw[0] + s_pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((R)(y0 + ry) * P.bw[1] + s_pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((R)(z0 + rz) * P.bw[2] + s_pos[3 * l + 2]);
        const R pot = trap<R>(P, r);
        local_terms<R, C>(P, r, pot, GPE_MODE_LEAPFROG, false, prv, H);
        V2* o = reinterpret_cast<V2*>(s_next + ((size_t)q * m.T + xl) * cb + l * node_bytes);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            V2 v = o[c];
            v.x += dt2 * H[c].y;
            v.y += dt2 * -H[c].x;
            o[c] = v;
        }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t q = 0; q < own_rows; ++q) {
            const uint32_t ry = q % m.RY, rz = q / m.RY;
            char* dst = a.next + (size_t)(z0 + rz) * a.g.slice + (size_t)(y0 + ry) * a.g.pitch + (size_t)x0 * cb;
            bulk_store(dst, s_next + (size_t)q * m.T * cb, bytes_next);
        }
        bulk_commit();
        bulk_wait_read_all();
    }
}

template <typename R, int C>
size_t rows_smem_bytes(const StepArgs& a, const RowsArgs& m) {
    return (size_t)m.nbuf * m.row_buf_bytes + (size_t)m.RY * m.RZ * m.T * a.g.cell_bytes +
           (size_t)a.tab.entries * sizeof(RowsEntry<R>) + 3 * a.g.V * sizeof(R) + (a.g.V + 1) * 4 + m.RY * m.RZ * m.K * 4;
}

// blk: device table [nbuf dy][nbuf dz][RY*RZ*K map], built by the host for this shape
template <typename R, int C>
cudaError_t launch_leapfrog_rows(const StepArgs& a, uint32_t T, uint32_t RY, uint32_t RZ, uint32_t K, uint32_t nbuf,
                                 const int32_t* blk, uint32_t threads, cudaStream_t s) {
    RowsArgs m;
    m.T = T;
    m.RY = RY;
    m.RZ = RZ;
    m.tiles_x = (a.g.X + T - 1) / T;
    m.tiles_y = a.g.Y / RY;
    m.K = K;
    m.nbuf = nbuf;
    m.row_buf_bytes = (T + 2) * a.g.cell_bytes;
    m.div_row_nodes = make_fastdiv(T * a.g.V);
    m.blk = blk;
    const size_t smem = rows_smem_bytes<R, C>(a, m);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(leapfrog_rows_kernel<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    const uint32_t nodes = RY * RZ * T * a.g.V;
    const uint32_t cap = RowsLB<R, C>::threads;
    if (threads == 0) threads = nodes >= cap ? cap : ((nodes + 31) / 32) * 32;
    if (threads > cap || threads % 32) return cudaErrorInvalidValue;
    const uint64_t blocks = (uint64_t)m.tiles_x * m.tiles_y * (a.g.Z / RZ);
    leapfrog_rows_kernel<R, C><<<(unsigned)blocks, threads, smem, s>>>(a, m);
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_ROWS(R, C)                                                                        \
    template cudaError_t launch_leapfrog_rows<R, C>(const StepArgs&, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, \
                                                    const int32_t*, uint32_t, cudaStream_t);

}  // namespace gpe

namespace gpe {

// ------------------------------------------------------------ initial states

struct InitArgs {
    double zeta[5][2];
    double mu, c0inv, noise_abs, noise_rel;
    int kappa;
    uint64_t seed;
};

// SplitMix64 (Steele, Lea & Flood 2014) output number `counter` (1-based) of stream `seed`.
__device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t counter) {
    uint64_t z = seed + counter * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01_at(uint64_t seed, uint64_t counter) {
    return ((double)(splitmix64_at(seed, counter) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

// Thomas-Fermi state psi_m = sqrt(rho_TF) zeta_m (times exp(i kappa phi)), plus
// noise (abs: noise_abs * N(0,1) per re/im; rel: sqrt(rho) noise_rel N(0,1)), the
// Gaussians drawn by Box-Muller from SplitMix64 pair number (node * C + m).
template <typename R, int C>
__global__ void __launch_bounds__(256) init_kernel(StepArgs a, InitArgs in) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= a.total) return;
    const uint32_t i = (uint32_t)gid;
    const uint32_t row = fdiv(i, a.divRow);
    const uint32_t within = i - row * a.row_items;
    const uint32_t x = fdiv(within, a.divV);
    const uint32_t l = within - x * a.g.V;
    const uint32_t z = fdiv(row, a.divY);
    const uint32_t y = row - z * a.g.Y;
    const PhysR<double>& P = a.pd;
    double r[3];
    r[0] = P.p0[0] + P.bs * ((double)x * P.bw[0] + a.tab.pos64[3 * l + 0]);
    r[1] = P.p0[1] + P.bs * ((double)y * P.bw[1] + a.tab.pos64[3 * l + 1]);
    r[2] = P.p0[2] + P.bs * ((double)z * P.bw[2] + a.tab.pos64[3 * l + 2]);
    const double lx = P.lambda[0] * r[0], ly = P.lambda[1] * r[1], lz = P.lambda[2] * r[2];
    const double V = 0.5 * (lx * lx + ly * ly + lz * lz);
    const double rho = fmax(in.mu - V, 0.0) * in.c0inv;
    const double amp = sqrt(rho);
    double cph = 1.0, sph = 0.0;
    if (in.kappa) {
        const double phi = atan2(r[1], r[0]);
        cph = cos(in.kappa * phi);
        sph = sin(in.kappa * phi);
    }
    const size_t off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes + l * (C * 2 * sizeof(R));
    const uint64_t node = gid;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const double zr = in.zeta[c][0] * cph - in.zeta[c][1] * sph;
        const double zi = in.zeta[c][0] * sph + in.zeta[c][1] * cph;
        double re = amp * zr, im = amp * zi;
        if (in.noise_abs != 0.0 || in.noise_rel != 0.0) {
            const uint64_t pair = node * C + c;
            const double u1 = uniform01_at(in.seed, 2 * pair + 1), u2 = uniform01_at(in.seed, 2 * pair + 2);
            const double rr = sqrt(-2.0 * log(u1));
            const double th = 6.283185307179586 * u2;
            const double g1 = rr * cos(th), g2 = rr * sin(th);
            const double s = in.noise_abs + in.noise_rel * amp;
            re += s * g1;
            im += s * g2;
        }
        stc<R>(a.next + off + c * 2 * sizeof(R), cx<R>((R)re, (R)im));
    }
}

template <typename R, int C>
cudaError_t launch_init(const StepArgs& a, const InitArgs& in, cudaStream_t s) {
    init_kernel<R, C><<<nblocks(a.total, 256), 256, 0, s>>>(a, in);
    return cudaGetLastError();
}

// The spinor of a state replaced at every node, its density kept: psi'_m =
// sqrt(rho w_m) u_m with rho = sum_m |psi_m|^2, w_m = |zeta_m|^2 and u_m =
// zeta_m / |zeta_m| (polarState / ferromagneticState / mixedState,
// Spin1GpeBCC.cu:463-551; unState / horizontalBnState / verticalBnState /
// cyclicState, Spin2GpeBCC.cu:417-558: each writes sqrt(rho x weight) times a
// phase into its fixed components).  a.next: the slot's interior pointer.
struct RespinArgs {
    double w[5];
    double u[5][2];
};

template <typename R, int C>
__global__ void __launch_bounds__(256) respin_kernel(StepArgs a, RespinArgs r) {
    const uint32_t node_bytes = C * 2 * sizeof(R);
    for (uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < a.total;
         gid += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)gid;
        const uint32_t row = fdiv(i, a.divRow);
        const uint32_t within = i - row * a.row_items;
        const uint32_t x = fdiv(within, a.divV);
        const uint32_t l = within - x * a.g.V;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * a.g.Y;
        char* p = a.next + (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes + l * node_bytes;
        Cx<R> v[C];
        ld_node<R, C, false>(p, v);
        R rho = 0;
#pragma unroll
        for (int m = 0; m < C; ++m) rho += v[m].x * v[m].x + v[m].y * v[m].y;
#pragma unroll
        for (int m = 0; m < C; ++m) {
            const R amp = sqrt(rho * (R)r.w[m]);
            v[m] = cx<R>(amp * (R)r.u[m][0], amp * (R)r.u[m][1]);
        }
        st_node<R, C>(p, v);
    }
}

template <typename R, int C>
cudaError_t launch_respin(const StepArgs& a, const RespinArgs& r, cudaStream_t s) {
    const unsigned nb = std::min<unsigned>(nblocks(a.total, 256), 8u * (unsigned)device_sm_count());
    if (nb) respin_kernel<R, C><<<nb, 256, 0, s>>>(a, r);
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_INIT(R, C)                                                                \
    template cudaError_t launch_init<R, C>(const StepArgs&, const InitArgs&, cudaStream_t);      \
    template cudaError_t launch_respin<R, C>(const StepArgs&, const RespinArgs&, cudaStream_t);

}  // namespace gpe

namespace gpe {

// ------------------------------------------------- hyperbolic row tiles (TMA)

// Fused hyperbolic psi+q leapfrog step on a row tile of T cells.  One bulk copy
// each brings psi_prev, q_prev, the old psi_next and the old q_next of cells
// [x0, x0+T) into shared memory; tasks [0, T*V) update nodes and tasks
// [T*V, T*(V+E)) update edges, looped over the block's threads.  Neighbours
// inside the tile (the d1 incidences of a node, the d0 end points of an edge) are
// read from shared memory, all others -- other rows, and the cells just outside
// the tile -- from global memory (L2): no halo cells are staged, which keeps the
// C15 tile (16 KB of psi+q per cell) small enough for several blocks per SM.
// Both updated tiles go back by bulk stores.  Requires cell_bytes and
// qcell_bytes to be multiples of 16.
constexpr uint32_t kHyperTileThreads = 224;
template <typename R, int C>
__global__ void __launch_bounds__(kHyperTileThreads, sizeof(R) == 4 ? 5 : 2)
    hyper_tile_kernel(StepArgs a, uint32_t T, uint32_t tiles_per_row) {
    extern __shared__ __align__(128) unsigned char dyn[];
    __shared__ __align__(8) uint64_t bar;
    using V2 = typename Vec2<R>::type;
    const uint32_t cb = a.g.cell_bytes, qb = a.g.qcell_bytes;
    const int V = a.g.V, E = a.g.E, F = a.tab.faces;
    char* s_psi = reinterpret_cast<char*>(dyn);                  // T psi cells
    char* s_q = s_psi + (size_t)T * cb;                          // T q cells
    char* s_psin = s_q + (size_t)T * qb;                         // T psi cells
    char* s_qn = s_psin + (size_t)T * cb;                        // T q cells
    int32_t* s_inc_soff = reinterpret_cast<int32_t*>(s_qn + (size_t)T * qb);  // V*F
    int32_t* s_inc_goff = s_inc_soff + V * F;
    R* s_inc_w = reinterpret_cast<R*>(s_inc_goff + V * F);
    int32_t* s_e_from = reinterpret_cast<int32_t*>(s_inc_w + V * F);          // E
    int32_t* s_e_tos = s_e_from + E;
    int32_t* s_e_tog = s_e_tos + E;
    R* s_pos = reinterpret_cast<R*>(s_e_tog + E + (E & 1));                    // 3V (8-aligned)

    const uint32_t tile = blockIdx.x % tiles_per_row;
    const uint32_t row = blockIdx.x / tiles_per_row;
    const uint32_t z = fdiv(row, a.divY);
    const uint32_t y = row - z * a.g.Y;
    const uint32_t x0 = tile * T;
    const uint32_t Tc = min(T, a.g.X - x0);
    const char* g_psi = a.prev + (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x0 * cb;
    const char* g_q = a.q + (size_t)z * a.g.qslice + (size_t)y * a.g.qpitch + (size_t)x0 * qb;
    char* g_psin = a.next + (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x0 * cb;
    char* g_qn = a.qnext + (size_t)z * a.g.qslice + (size_t)y * a.g.qpitch + (size_t)x0 * qb;

    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_proxy_async_smem();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, 2 * Tc * (cb + qb));
        bulk_load(s_psi, g_psi, Tc * cb, &bar);
        bulk_load(s_q, g_q, Tc * qb, &bar);
        bulk_load(s_psin, g_psin, Tc * cb, &bar);
        bulk_load(s_qn, g_qn, Tc * qb, &bar);
    }
    for (int i = threadIdx.x; i < V * F; i += blockDim.x) {
        s_inc_soff[i] = a.tab.inc_soff[i];
        s_inc_goff[i] = a.tab.inc_off[i];
        if constexpr (sizeof(R) == 4) s_inc_w[i] = a.tab.inc_w32[i];
        else s_inc_w[i] = a.tab.inc_w64[i];
    }
    for (int i = threadIdx.x; i < E; i += blockDim.x) {
        s_e_from[i] = a.tab.e_from_off[i];
        s_e_tos[i] = a.tab.e_to_soff[i];
        s_e_tog[i] = a.tab.e_to_off[i];
    }
    for (int i = threadIdx.x; i < 3 * V; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) s_pos[i] = a.tab.pos32[i];
        else s_pos[i] = a.tab.pos64[i];
    }
    if (!block_wait(&bar, 0, a.err)) return;  // uniform across the block

    const PhysR<R>& P = make_phys<R>(a);
    const uint32_t node_bytes = C * 2 * sizeof(R);
    for (uint32_t i = threadIdx.x; i < T * (V + E); i += blockDim.x) {
        if (i < T * V) {
            if (i >= Tc * V) continue;
            const uint32_t xl = fdiv(i, a.divV);
            const uint32_t l = i - xl * V;
            const char* own = s_psi + (size_t)xl * cb + l * node_bytes;
            Cx<R> prv[C], H[C];
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const V2 v = reinterpret_cast<const V2*>(own)[c];
                prv[c] = cx<R>(v.x, v.y);
                H[c] = cx<R>((R)0, (R)0);
            }
            // d1 of q (RelativisticSpin2Gpe.cu:1051-1066)
            const int32_t qrow = (int32_t)(xl * qb), qend = (int32_t)(Tc * qb);
            for (int k = 0; k < F; ++k) {
                const int so = s_inc_soff[l * F + k];
                const R w = s_inc_w[l * F + k];
                const int32_t tgt = qrow + so;  // byte offset from the tile's first q cell
                if (so != INT32_MIN && tgt >= 0 && tgt < qend) {
                    const V2* p = reinterpret_cast<const V2*>(s_q + tgt);
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        const V2 v = p[c];
                        H[c] += w * cx<R>(v.x, v.y);
                    }
                } else {
                    const char* g = so != INT32_MIN ? g_q + tgt : g_q + qrow + s_inc_goff[l * F + k];
#pragma unroll
                    for (int c = 0; c < C; ++c) H[c] += w * ldc<R>(g + c * 2 * sizeof(R));
                }
            }
            R r[3];
            r[0] = P.p0[0] + P.bs * ((R)(x0 + xl) * P.bw[0] + s_pos[3 * l + 0]);
            r[1] = P.p0[1] + P.bs * ((R)y * P.bw[1] + s_pos[3 * l + 1]);
            r[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + s_pos[3 * l + 2]);
            const R pot = trap<R>(P, r);
            if constexpr (C == 1) {
                local_scalar<R>(P, pot, false, true, prv, H);
            } else if constexpr (C == 3) {
                local_spin1<R>(P, r, pot, true, false, true, prv, H);
            } else {
                local_spin2<R>(P, r, pot, true, false, true, prv, H);
            }
            V2* o = reinterpret_cast<V2*>(s_psin + (size_t)xl * cb + l * node_bytes);
            const R dt2 = (R)2 * P.dt;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                V2 v = o[c];
                v.x += dt2 * H[c].y;
                v.y += dt2 * -H[c].x;
                o[c] = v;
            }
        } else {
            // q update (RelativisticSpin2Gpe.cu:986-1015)
            const uint32_t j = i - T * V;
            const uint32_t xl = fdiv(j, a.divE);
            if (xl >= Tc) continue;
            const uint32_t e = j - xl * E;
            const int32_t prow = (int32_t)(xl * cb);
            const char* thisp = s_psi + prow + s_e_from[e];
            const int ts = s_e_tos[e];
            const int32_t tgt = prow + ts;  // byte offset from the tile's first psi cell
            const bool to_in_row = ts != INT32_MIN && tgt >= 0 && tgt < (int32_t)(Tc * cb);
            const char* otherp = to_in_row ? s_psi + tgt : (ts != INT32_MIN ? g_psi + tgt : g_psi + prow + s_e_tog[e]);
            const char* qprev = s_q + (size_t)xl * qb + e * node_bytes;
            V2* qn = reinterpret_cast<V2*>(s_qn + (size_t)xl * qb + e * node_bytes);
            const R dts2 = (R)2 * P.dts;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const V2 tv = reinterpret_cast<const V2*>(thisp)[c];
                Cx<R> ov;
                if (to_in_row) {
                    const V2 w2 = reinterpret_cast<const V2*>(otherp)[c];
                    ov = cx<R>(w2.x, w2.y);
                } else {
                    ov = ldc<R>(otherp + c * 2 * sizeof(R));
                }
                const Cx<R> d0psi = ov - cx<R>(tv.x, tv.y);
                const V2 pq = reinterpret_cast<const V2*>(qprev)[c];
                const Cx<R> qq = dts2 * (cx<R>(pq.x, pq.y) + d0psi);
                V2 v = qn[c];
                v.x += -qq.y;
                v.y += qq.x;
                qn[c] = v;
            }
        }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        bulk_store(g_psin, s_psin, Tc * cb);
        bulk_store(g_qn, s_qn, Tc * qb);
        bulk_commit();
        bulk_wait_read_all();
    }
}

template <typename R, int C>
size_t hyper_tile_smem_bytes(const StepArgs& a, uint32_t T) {
    const int V = a.g.V, E = a.g.E, F = a.tab.faces;
    return (size_t)(2 * T) * (a.g.cell_bytes + a.g.qcell_bytes) + (size_t)V * F * (8 + sizeof(R)) +
           (size_t)(3 * E + (E & 1)) * 4 + 3 * V * sizeof(R);
}

template <typename R, int C>
cudaError_t launch_hyper_tile(const StepArgs& a, uint32_t T, cudaStream_t s) {
    const uint32_t tiles = (a.g.X + T - 1) / T;
    const uint32_t tasks = T * (a.g.V + a.g.E);
    // at most kHyperTileThreads threads (five blocks per SM in FP32); the tasks split
    // evenly into passes of the block
    const uint32_t passes = (tasks + kHyperTileThreads - 1) / kHyperTileThreads;
    const uint32_t threads = std::min(kHyperTileThreads, (((tasks + passes - 1) / passes) + 31) / 32 * 32);
    const size_t smem = hyper_tile_smem_bytes<R, C>(a, T);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(hyper_tile_kernel<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        // all of the unified L1 as shared memory: five ~44 KB C15 tiles per SM
        cudaFuncSetAttribute(hyper_tile_kernel<R, C>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        configured = smem;
    }
    const uint64_t blocks = (uint64_t)tiles * a.g.Y * a.g.Z;
    hyper_tile_kernel<R, C><<<(unsigned)blocks, threads, smem, s>>>(a, T, tiles);
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_HYPER_TILE(R, C) template cudaError_t launch_hyper_tile<R, C>(const StepArgs&, uint32_t, cudaStream_t);

}  // namespace gpe

#include "gpe_slab.cuh"
#include "gpe_il.cuh"
