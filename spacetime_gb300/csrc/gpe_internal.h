// gpe_internal.h -- shared host/device definitions of libgpe (not part of the ABI).
#pragma once

#include <cmath>
#include <cstddef>
#include <climits>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "../../include/gpe.h"

namespace gpe {

// Largest tables the kernels stage in shared memory.  C15 (V=136, 544 stencil
// entries, E=272) is the largest lattice of the reference.
// Internal step mode beside GPE_MODE_LEAPFROG / EULER / ITP: a leapfrog step that
// reads the old value from StepArgs::hpsi and writes next, leaving the old buffer
// as it was (the adjoint's recomputation keeps every state of a segment).
constexpr int kModeLeapfrogFrom = 3;

constexpr int kMaxNodes = 160;
constexpr int kMaxEntries = 640;
constexpr int kMaxEdges = 320;
constexpr int kMaxFaces = 8;

// Unsigned division by a run-time constant: q = umulhi(n, mul) >> shift
// (Granlund & Montgomery, "Division by invariant integers using multiplication", 1994).
struct FastDiv {
    uint32_t d, mul, shift;
};

inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    if (d == 1) {
        f.mul = 0;
        f.shift = 0;
        return f;
    }
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    // mul = floor(2^32 * (2^l - d) / d) + 1, shift = l - 1 for the "add" variant; we use
    // the 64-bit form q = (umulhi(n, m) + n) >> l which is exact for all 32-bit n.
    uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    f.mul = (uint32_t)m;
    f.shift = l;
    return f;
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    if (f.d == 1) return n;
    uint32_t t = __umulhi(n, f.mul);
    return (uint32_t)(((uint64_t)t + n) >> f.shift);
}
#endif

// Observables accumulated per block (FP64), in this order.
enum ObsIndex {
    OBS_NORM = 0,
    OBS_HEXP,
    OBS_EINT,
    OBS_MAGX,
    OBS_MAGY,
    OBS_MAGZ,
    OBS_SPIN,
    OBS_COMX,
    OBS_COMY,
    OBS_COMZ,
    OBS_MAXABS,
    OBS_NONFINITE,
    OBS_COUNT
};

// Geometry of one state buffer (bytes).
struct Grid {
    uint32_t X, Y, Z;
    uint32_t V, C, E;
    size_t pitch, slice;         // psi buffers
    size_t qpitch, qslice;       // q buffers
    uint32_t cell_bytes, qcell_bytes;
};

// Geometry of an FP32 state in the cell-interleaved layout.  Rows (y, z) run from
// -1 to Y and -1 to Z (the halo rows and planes are zero); a row holds GX groups of
// `cells` (32 or 16) consecutive cells along x; a group holds [node l][component
// s][cell of the group][re, im], so that node l's component s of a group's cells
// is one contiguous run of 8 cells bytes.  Cells x >= X of the last group, and the
// cells x = -1 and x = X, read as zero.  A warp takes node l of 32 / cells groups,
// the grid's groups counted row after row.  The group width is chosen per grid:
// 32 where that leaves no more lanes idle than 16 would (X a multiple of 32, or
// X mod 32 > 16), 16 otherwise.  Measured (FP32 leapfrog, fraction of the copy
// peak, 32 / 16): spin-1 BCC 96^3 0.860 / 0.833, A15 64^3 0.857 / 0.832, Z 56^3
// 0.774 / 0.750, C15 48^3 0.700 / 0.829; the 256-member ensemble 0.555 / 0.568.
struct ILGrid {
    uint32_t X, Y, Z, V, C, GX;
    uint32_t cells; // cells per group: 32 or 16
    size_t gb;      // bytes per group: V * C * cells * 8
    size_t row;     // bytes per row: GX * gb
    size_t bytes;   // the buffer: (Y + 2) (Z + 2) rows
};

inline uint32_t il_group_cells(uint32_t X) {
    const uint32_t g32 = (X + 31) / 32, g16 = (X + 15) / 16;
    return 32 * g32 <= 16 * g16 ? 32 : 16;
}

// The interleaved kernels keep a neighbour's offset from its group's base in 32
// bits: a plane of rows and two groups more must stay below 2^31 bytes.
inline bool il_offsets_fit(const ILGrid& G) {
    return (uint64_t)(G.Y + 3) * G.row + 2 * (uint64_t)G.gb < (uint64_t)INT32_MAX;
}

inline ILGrid make_il_grid(const Grid& g) {
    ILGrid G;
    G.X = g.X;
    G.Y = g.Y;
    G.Z = g.Z;
    G.V = g.V;
    G.C = g.C;
    G.cells = il_group_cells(g.X);
    G.GX = (g.X + G.cells - 1) / G.cells;
    G.gb = (size_t)g.V * g.C * G.cells * 8;
    G.row = G.GX * G.gb;
    G.bytes = (size_t)(g.Y + 2) * (g.Z + 2) * G.row;
    return G;
}

// Physics constants of a step (double; converted per kernel).
struct Phys {
    double p0[3];
    double bs;
    double bw[3];
    double dt;
    double lambda[3];
    double trap_offset;
    double trap_off_time;
    double c0, c2, c4, alpha, sigma;
    double quad_center[3];
    double ks;       // kinetic scale (bs0 / bs)^2 of the step's block scale bs (1 without expansion)
    int flags;
};

// Physics constants of a step in the arithmetic type of a kernel, prepared on the
// host so that kernels do no precision conversion (FP64 is slow on GB300).
template <typename R>
struct PhysR {
    R p0[3], bs, bw[3], lambda[3], trap_offset, c0, c2, c4, alpha, sigma, qc[3];
    R bq, bb[3], bqq, bbq[3];
    R dt, dts;       // dt and dt/sigma
    R ks;            // kinetic scale (bs0 / bs)^2; bs above is the step's block scale
    int trap_on;     // trap() is zero after trap_off_time (Spin1GpeBCC.cu:114)
    int flags;
};

// Per-handle device tables.  Byte offsets are relative to the base of the
// thread's own cell in the buffer being read.
struct DevTables {
    int32_t* row_ptr;     // V+1
    int32_t* nb_off;      // entries: byte offset of the neighbour value in prev
    int32_t* nb_soff;     // entries: offset inside a contiguous row of cells, INT32_MIN if the neighbour is off-row
    double* w64;          // entries: (-0.5*h)/bs^2
    float* w32;
    double* pos64;        // V*3
    float* pos32;
    int32_t* inc_off;     // V*F: byte offset of the incident edge value in q (relative to own q cell)
    double* inc_w64;      // V*F
    float* inc_w32;
    int32_t* e_from_off;  // E: byte offset of from-node in own psi cell
    int32_t* e_to_off;    // E: byte offset of to-node relative to own psi cell base
    int32_t* e_to_soff;   // E: the same inside a contiguous row of cells, INT32_MIN if off-row
    int32_t* inc_soff;    // V*F: incident edge inside a contiguous row of q cells, INT32_MIN if off-row
    int4* ent4;           // entries: (dx, dy, dz, node)
    int32_t* ent_row;     // entries: index of the (dy, dz) row in the multi-row tile
    int entries;
    int faces;
    int uniform_deg;      // > 0 when every node has the same number of entries
    int quad_rows;        // 1 when rows differ in length and every row is a positive multiple of 4 long
    int max_deg;          // the longest row
};

struct StepArgs {
    const char* prev;
    char* next;
    char* hpsi;
    const char* q;        // hyperbolic: q_prev
    char* qnext;          // hyperbolic: q_next
    Grid g;
    DevTables tab;
    Phys ph;
    gpe_fields B;
    double t;
    PhysR<float> pf;
    PhysR<double> pd;
    FastDiv divV, divRow, divY;   // nodes: within-row node index, X*V per row, rows
    FastDiv divE, divRowE;        // edges: within-row edge index, X*E per row
    uint32_t row_items;   // X*V
    uint32_t row_items_e; // X*E
    uint64_t total;       // total threads of work
    double* partials;     // observables
    int* err;             // device error flag (bounded waits that ran out)
};

#ifdef __CUDACC__
#define GPE_HD __host__ __device__
#else
#define GPE_HD
#endif

// getSignal + scaling (Spin1GpeBCC/AliceRingRamps.h:74-141): each channel walks its
// consecutive segment durations; inside segment k the value goes from the previous
// target (0 before the first) to target k by the segment's type; past the end the
// last target holds.  The same code runs on the host (gpe_ramp_eval) and on the
// device (batched stepping).  Segment counts must be in [0, GPE_RAMP_MAX_SEGMENTS].
GPE_HD inline void ramp_channel(int nseg, const double* tgt, int stride, const double* dur, const int32_t* type,
                                double tau, double* val, int dims) {
    for (int a = 0; a < dims; ++a) val[a] = 0;
    if (nseg <= 0) return;
    int k = 0;
    double t = tau;
    while (k < nseg && t - dur[k] >= 0) {
        t -= dur[k];
        ++k;
    }
    if (k == nseg) {
        k = nseg - 1;
        t = dur[k];
    }
    for (int a = 0; a < dims; ++a) {
        const double target = tgt[k * stride + a];
        const double prev = k > 0 ? tgt[(k - 1) * stride + a] : 0.0;
        if (type[k] == GPE_RAMP_CONSTANT) val[a] = target;
        else if (type[k] == GPE_RAMP_LINEAR) val[a] = prev + t * (target - prev) / dur[k];
        else val[a] = prev + (target - prev) * sqrt(t / dur[k]);
    }
}

GPE_HD inline void ramp_eval(const gpe_ramp& r, double tau, gpe_fields& out) {
    double bq = 0, bb[3];
    ramp_channel(r.bq_segments, r.bq_target, 1, r.bq_duration, r.bq_type, tau, &bq, 1);
    ramp_channel(r.bb_segments, &r.bb_target[0][0], 3, r.bb_duration, r.bb_type, tau, bb, 3);
    out.bq = r.bq_scale * bq;
    out.bq_quad = r.bq_quad_scale * bq;
    for (int a = 0; a < 3; ++a) {
        out.bb[a] = r.bb_scale * bb[a];
        out.bb_quad[a] = r.bb_quad_scale * bb[a];
    }
}

// Sets the text returned by gpe_last_error() for this thread (gpe_capi.cu).
void set_last_error(const std::string& msg);

}  // namespace gpe
