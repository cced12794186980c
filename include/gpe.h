/*
 * gpe.h -- C ABI of the GB300 Gross-Pitaevskii block-cell stepper (libgpe).
 *
 * The reference (markus-kivioja/SpaceTime) has no library API: its per-step
 * "operator" is a __global__ kernel launched from each program's time loop.
 * Every entry point below replaces one of those launches (or the host code
 * around it); the comment on each names the reference code it stands in for.
 *
 * Conventions shared by all entry points
 *  - One STEP advances one buffer by dt.  Leapfrog steps use
 *    next += 2*dt*(-i H prev), as in Spin1GpeBCC/Spin1GpeBCC.cu:914-916.  The scalar
 *    programs write next += dt_ref*(-i H prev) (GrossPitaevskiiGpuBcc/
 *    GPUGrossPitaevskii_BCC.cu:345-346); pass dt = dt_ref/2 to reproduce them.
 *  - State buffers keep the reference's block-cell layout: a pitched 3-D array of
 *    cells (x fastest) with a one-cell zero halo on every side; a cell holds
 *    V nodes x C components x (re, im) (BlockPsis, Spin1GpeBCC/utils.h:75-85),
 *    and an edge cell E edges x C components x (re, im) (BlockEdges,
 *    RelativisticSpin1Gpe/utils.h:91-94).  Host copies in and out use the unpadded
 *    reference file layout ((Z+2)(Y+2)(X+2) cells, FP64), so a reference
 *    "ground_state.dat" / "<t>.dat" dump can be loaded and written directly.
 *  - Every call returns a gpe_status and never exits the process.  Work is
 *    enqueued on the caller's stream; no call synchronises unless it says so.
 *  - Handles are not thread-safe; use one handle per host thread.
 */
#ifndef GPE_H
#define GPE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GPE_OK = 0,
    GPE_ERR_INVALID_ARG = 1,  /* bad pointer, size, table or parameter */
    GPE_ERR_OOM = 2,          /* device or host allocation failed */
    GPE_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    GPE_ERR_TIMEOUT = 4,      /* a bounded device wait ran out */
    GPE_ERR_NONFINITE = 5,    /* a reduction found NaN/Inf in the state */
    GPE_ERR_UNSUPPORTED = 6,  /* combination not built (e.g. C=5 on a lattice without edges) */
    GPE_ERR_NO_DEVICE = 7     /* no CUDA device visible */
} gpe_status;

/* ---------------------------------------------------------------- lattices */

/* One node-Laplacian entry: neighbour node `node` of the cell at offset
 * (dx,dy,dz) in {-1,0,1}^3, with DEC weight hodge = body hodge / face hodge.
 * Replaces the int2 byte-offset table (GrossPitaevskiiGpuBcc/mesh.h:42-92) and
 * the int4 cell-offset table (Spin1GpeBCC/mesh.h:47-100). */
typedef struct {
    int32_t dx, dy, dz;
    int32_t node;
    double hodge;
} gpe_stencil_entry;

/* One dual edge (d0 row, RelativisticSpin2Gpe/mesh.h:48-74): from node `from` of
 * this cell to node `to` of the cell at offset (dx,dy,dz).  d0 psi = psi[to]-psi[from]. */
typedef struct {
    int32_t from;
    int32_t dx, dy, dz;
    int32_t to;
} gpe_edge;

/* One node-edge incidence (d1 row, RelativisticSpin2Gpe/mesh.h:76-133): edge
 * `edge` of the edge cell at offset (dx,dy,dz), weight with the incidence sign
 * folded in (RelativisticSpin2Gpe/mesh.h:185-232). */
typedef struct {
    int32_t dx, dy, dz;
    int32_t edge;
    double hodge;
} gpe_incidence;

typedef struct {
    int32_t nodes;                      /* V (VALUES_IN_BLOCK) */
    double block_width[3];              /* BLOCK_WIDTH in unit-block units */
    double volume;                      /* VOLUME: dual-cell volume, unit-block units */
    const double* pos;                  /* V*3 node positions (d_localPos) */
    const int32_t* row_ptr;             /* V+1 CSR offsets into stencil */
    const gpe_stencil_entry* stencil;   /* row_ptr[V] entries */
    int32_t edges;                      /* E (EDGES_IN_BLOCK); 0 if no edge tables */
    int32_t faces_per_node;             /* incidence entries per node (FACE_COUNT) */
    const gpe_edge* edge_table;         /* E entries */
    const gpe_incidence* incidence;     /* V*faces_per_node entries */
} gpe_lattice_desc;

typedef struct gpe_lattice gpe_lattice;

/* Validates and copies the tables (symmetry, offsets in {-1,0,1}, node ids in
 * range).  Replaces the host getLaplacian(...) calls, e.g. Spin1GpeBCC.cu:1156. */
gpe_status gpe_lattice_create(const gpe_lattice_desc* desc, gpe_lattice** out);
void gpe_lattice_destroy(gpe_lattice* lat);

/* ----------------------------------------------------------------- physics */

/* PARABOLIC: node stencil, leapfrog (Spin1GpeBCC.cu, Spin2GpeBCC.cu, GrossPitaevskiiGpu*).
 * HYPERBOLIC: psi + dual-edge q, leapfrog (Relativistic{GpeBCC,Spin1Gpe,Spin2Gpe}).
 * SPLIT: scalar psi = R + iI and q = q_R + i q_I with R and I staggered by half a
 * step (RelativisticGpeC15/GPUGrossPitaevskii_C15.cu:90-155, loop :477-482); C = 1,
 * state in PSI_EVEN / Q_EVEN (the real part holds R, the imaginary part I); gpe_start
 * is the loop's q_R initialisation (:469), gpe_step two launches per step. */
enum { GPE_SCHEME_PARABOLIC = 0, GPE_SCHEME_HYPERBOLIC = 1, GPE_SCHEME_SPLIT = 2 };
enum { GPE_FP32 = 0, GPE_FP64 = 1 };
enum {
    GPE_FLAG_THREE_BODY_LOSS = 1,     /* -i alpha rho^2 (Spin1GpeBCC.cu:877-880) */
    GPE_FLAG_QUADRATIC_ZEEMAN = 2,    /* Spin1GpeBCC.cu:897-912 */
    GPE_FLAG_QUADRUPOLE_OFFSET = 4,   /* Spin1GpeBCC.cu:128-137 */
    GPE_FLAG_TRAP_OFF_AFTER = 8       /* trap() returns 0 for t >= trap_off_time (Spin1GpeBCC.cu:114) */
};

typedef struct {
    int32_t components;      /* C: 1 (scalar), 3 (spin-1) or 5 (spin-2) */
    int32_t scheme;          /* GPE_SCHEME_* */
    int32_t precision;       /* GPE_FP32 (fused fast path) or GPE_FP64 (plain) */
    int32_t flags;           /* GPE_FLAG_* */
    uint32_t dims[3];        /* interior cells X, Y, Z */
    double block_scale;      /* bs: physical width of a unit block / BLOCK_WIDTH */
    double p0[3];            /* physical position of the corner of cell (0,0,0) */
    double dt;               /* time step (code units) */
    double trap_lambda[3];   /* V = 0.5*|lambda .* r|^2 + trap_offset (Spin1GpeBCC.cu:112-122) */
    double trap_offset;      /* +100 in the spinor/GpuBcc programs, 0 in GPBlocks */
    double trap_off_time;    /* with GPE_FLAG_TRAP_OFF_AFTER */
    double c0;               /* density interaction (g for the scalar programs) */
    double c2;               /* spin interaction (spin-1: Fz/F+-; spin-2: c2 of Spin2GpeBCC.cu:128) */
    double c4;               /* spin-2 singlet interaction (Spin2GpeBCC.cu:129) */
    double alpha;            /* three-body loss */
    double sigma;            /* relativistic coefficient (RelativisticSpin2Gpe.cu:142) */
    double quad_center[3];   /* quadrupole centre with GPE_FLAG_QUADRUPOLE_OFFSET */
} gpe_params;

/* Magnetic fields of one step (MagFields, Spin1GpeBCC/utils.h:94-100):
 * B(r) = (Bq x + Bb.x, Bq y + Bb.y, -2 Bq z + Bb.z) (Spin1GpeBCC.cu:128-142). */
typedef struct {
    double bq;
    double bb[3];
    double bq_quad;
    double bb_quad[3];
} gpe_fields;

/* Piecewise field ramp, the device-side form of getSignal(t)
 * (Spin1GpeBCC/AliceRingRamps.h:74-141, KnotRamps.h:64-135).  Each channel is a
 * list of segments (target value, duration, type); inside segment k the value
 * goes from the previous target (0 before the first) to target k as
 *   CONSTANT: target;  LINEAR: prev + s*(target-prev);  SQRT: prev + sqrt(s)*(target-prev)
 * with s = time into segment / duration.  The field of step n is evaluated at
 * ramp time tau = time_scale * (t0 + (n+1)*dt) and scaled:
 *   Bq = bq_scale*signal.Bq, Bb = bb_scale*signal.Bb,
 *   BqQuad = bq_quad_scale*signal.Bq, BbQuad = bb_quad_scale*signal.Bb
 * (Spin1GpeBCC.cu:1583-1587). */
enum { GPE_RAMP_CONSTANT = 0, GPE_RAMP_LINEAR = 1, GPE_RAMP_SQRT = 2 };
#define GPE_RAMP_MAX_SEGMENTS 32
typedef struct {
    int32_t bq_segments;
    double bq_target[GPE_RAMP_MAX_SEGMENTS];
    double bq_duration[GPE_RAMP_MAX_SEGMENTS];
    int32_t bq_type[GPE_RAMP_MAX_SEGMENTS];
    int32_t bb_segments;
    double bb_target[GPE_RAMP_MAX_SEGMENTS][3];
    double bb_duration[GPE_RAMP_MAX_SEGMENTS];
    int32_t bb_type[GPE_RAMP_MAX_SEGMENTS];
    double time_scale;
    double bq_scale, bb_scale, bq_quad_scale, bb_quad_scale;
} gpe_ramp;

/* Host evaluation of a ramp at ramp time tau (getSignal + scaling). */
gpe_status gpe_ramp_eval(const gpe_ramp* ramp, double tau, gpe_fields* out);

/* ----------------------------------------------------------------- handles */

typedef struct gpe_handle gpe_handle;

/* Buffer slots of a handle. */
enum { GPE_PSI_EVEN = 0, GPE_PSI_ODD = 1, GPE_Q_EVEN = 2, GPE_Q_ODD = 3, GPE_HPSI = 4 };

/* A pitched device buffer in the reference layout; ptr is the interior cell
 * (0,0,0), one cell in from the allocation start in x, y and z (PitchedPtr,
 * Spin1GpeBCC.cu:1145-1147).  pitch/slice_pitch in bytes. */
typedef struct {
    void* ptr;
    size_t pitch;
    size_t slice_pitch;
} gpe_pitched;

/* Creates a stepper on the current CUDA device and allocates its buffers
 * (psi even/odd, plus q even/odd for the hyperbolic scheme), zero-filled.
 * Replaces the cudaMalloc3D/getLaplacian/host set-up of integrateInTime
 * (Spin1GpeBCC.cu:1105-1172, RelativisticSpin2Gpe.cu:1295-1403). */
gpe_status gpe_create(const gpe_lattice* lat, const gpe_params* params, gpe_handle** out);
gpe_status gpe_destroy(gpe_handle* h);

/* Describe one of the handle's device buffers (for a caller that wants to run
 * its own kernels on it, or to hand it to another library). */
gpe_status gpe_buffer(const gpe_handle* h, int32_t slot, gpe_pitched* out, size_t* cell_bytes);

/* Host <-> device copies in the reference file layout: (Z+2)(Y+2)(X+2) cells of
 * FP64 values, halo included (the ground_state.dat / "<t>.dat" format written at
 * Spin1GpeBCC.cu:1690-1699).  Halo cells are ignored on upload (kept zero).
 * count = number of doubles in host buffer.  These synchronise the stream.  A
 * page-locked (pinned, device-mapped) host array is read or written by the
 * conversion kernel directly over the host link; a pageable one goes through a
 * device staging buffer (allocated on first use).  With GPE_TUNE_TRANSFER 1 a
 * pinned array goes through the staging buffer too: a DMA copy by a copy engine
 * and a conversion at device-memory speed, so that the copy overlaps kernels that
 * other streams run (the direct form's conversion kernel holds SMs for the whole
 * transfer).  The results are the same. */
gpe_status gpe_upload(gpe_handle* h, int32_t slot, const double* host, size_t count, void* stream);
gpe_status gpe_download(gpe_handle* h, int32_t slot, double* host, size_t count, void* stream);

/* Seeded initial state written on the device (no host array): Thomas-Fermi
 * amplitude sqrt(max(mu - V, 0)/c0) for V = 0.5 |lambda r|^2 and
 * mu = 0.5 (15 c0 lx ly lz / 4 pi)^(2/5), times the spinor zeta and, if
 * vortex_kappa != 0, exp(i kappa phi) (a straight z-vortex); plus Gaussian noise
 * noise_abs * sqrt(mu/c0) * N(0,1) + noise_rel * sqrt(rho) * N(0,1) per re/im part
 * (the relative form is Spin1GpeBCC.cu:1272-1285's), drawn by Box-Muller from
 * SplitMix64 numbers 2k+1, 2k+2 of stream `seed` for pair k = node * C + m, with
 * nodes numbered ((z Y + y) X + x) V + l; then normalised to unit norm if
 * `normalize`.  Replaces the ground-state file + polarState/cyclicState set-up of
 * the reference (Spin1GpeBCC.cu:1228-1398, Spin2GpeBCC.cu:523-558), whose noise
 * comes from an implementation-defined std::default_random_engine. */
typedef struct {
    double zeta[5][2];
    int32_t vortex_kappa;
    double noise_abs;
    double noise_rel;
    uint64_t seed;
    int32_t normalize;
} gpe_init;
gpe_status gpe_init_state(gpe_handle* h, int32_t slot, const gpe_init* init, void* stream);

/* Re-spins a state in place, keeping its density: at every node
 * psi'_m = sqrt(rho |zeta_m|^2) zeta_m / |zeta_m| with rho = sum_m |psi_m|^2, for
 * zeta given as C (re, im) pairs (the density becomes rho sum_m |zeta_m|^2).
 * Replaces the reference's phase-preparation kernels applied to a loaded ground
 * state: polarState (zeta = (0, 1, 0)), ferromagneticState ((1, 0, 0)) and
 * mixedState ((sqrt(mix), sqrt(1 - mix), 0)), Spin1GpeBCC.cu:463-551, 1395-1407;
 * unState ((0, 0, 1, 0, 0)), horizontalBnState ((1, 0, 0, 0, e^{i phase}) /
 * sqrt 2), verticalBnState ((0, 1, 0, e^{i phase}, 0) / sqrt 2) and cyclicState
 * ((sqrt(1/3), 0, 0, sqrt(2/3) e^{i phase}, 0)), Spin2GpeBCC.cu:417-558. */
gpe_status gpe_respin(gpe_handle* h, int32_t slot, const double* zeta, void* stream);

/* Axisymmetric vortex state Psi = f(r, z) e^{i kappa phi} of a scalar condensate
 * in the trap V = (r^2 + trap_ratio^2 z^2) / 2, host code: the reference's
 * VortexState (GrossPitaevskii/VortexState.cpp:11-237), which builds the initial
 * state of its CPU stepper (GPBlocks.cpp:477-486, main).  The grid is setRange's:
 * r in [rmin, rmax) in rsize = round((rmax - rmin) / rstep) steps, z in [0, zmax)
 * in zsize = round(zmax / zstep) steps, mirrored at z = 0.
 * gpe_vortex_profile relaxes f from the reference's initial guess
 * (iterateSolution: Gauss-Seidel sweeps with the Rayleigh quotient for mu and a
 * renormalisation after each, until a sweep changes f by less than eps in the
 * weighted squared sense, at most max_iters sweeps) into f[i * zsize + j]; with
 * f = NULL it only reports rsize and zsize.  mu and the sweeps taken are
 * returned if the pointers are given.
 * gpe_vortex_sample evaluates Psi at every interior node of a grid (getPsi:
 * bilinear interpolation of f, times ((x + iy)/r)^kappa) into a host array in
 * the reference file layout (as gpe_upload takes it), into component 0 (the
 * scalar, or the first spinor component for gpe_respin to re-spin); the halo
 * and the other components are zero. */
typedef struct {
    uint32_t kappa;
    double g;
    double rmin, rmax, rstep;
    double zmax, zstep;
    double trap_ratio;
    uint32_t max_iters;
    double eps;
} gpe_vortex_params;
gpe_status gpe_vortex_profile(const gpe_vortex_params* vp, double* f, size_t count, uint32_t* rsize, uint32_t* zsize,
                              double* mu, uint32_t* iterations);
gpe_status gpe_vortex_sample(const gpe_vortex_params* vp, const double* f, const gpe_lattice_desc* lat,
                             const gpe_params* p, double* host, size_t count);

/* Install the field ramp used by gpe_step / gpe_start (device-side getSignal). */
gpe_status gpe_set_ramp(gpe_handle* h, const gpe_ramp* ramp, double t0);

/* Condensate expansion (Spin1GpeBCC.cu:1576-1582, 1590-1596): from t_start on,
 * every step at time t uses the block scale bs(t) = bs0 (1 + rate (t - t_start)),
 * for the node positions and the Laplacian weights h / bs^2, as the reference
 * passes its growing expansionBlockScale to leapfrog.  gpe_observe uses bs(t) for
 * positions and kinetic energy and keeps dv = bs0^3 VOLUME, as the reference's
 * volume.  The reference adds dt k bs0 per step from the first step whose time is
 * at or after EXPANSION_START: rate = k times its ms per code time unit, and
 * t_start = that step's time minus dt.  Pair it with GPE_FLAG_TRAP_OFF_AFTER at
 * the same time for the reference's trap switch-off (:112-116).  rate = 0 turns it
 * off.  Parabolic scheme only; the adjoint and batched stepping refuse handles
 * with expansion (GPE_ERR_UNSUPPORTED). */
gpe_status gpe_set_expansion(gpe_handle* h, double t_start, double rate);

/* Forward-Euler start step from PSI_ODD into PSI_EVEN at t0
 * (forwardEuler, Spin1GpeBCC.cu:667-791, launched at :1433; hyperbolic start
 * RelativisticSpin2Gpe.cu:1628-1630). */
gpe_status gpe_start(gpe_handle* h, void* stream);

/* n leapfrog steps, alternating odd<-even and even<-odd as the reference time loop
 * does (Spin1GpeBCC.cu:1574-1603; GPUGrossPitaevskii_BCC.cu:883-889;
 * hyperbolic psi+q RelativisticSpin2Gpe.cu:1859-1899, fused here into one kernel
 * per step).  Fields follow the installed ramp.  n may be odd: the handle tracks
 * which buffer holds the newest state. */
gpe_status gpe_step(gpe_handle* h, int32_t n, void* stream);

/* One step with explicit fields instead of the ramp: next <- prev, the
 * per-launch form of the reference loop (leapfrog<<<>>>(next, prev, ..., Bs, t),
 * Spin1GpeBCC.cu:1588).  mode: 0 leapfrog, 1 forward Euler, 2 imaginary time
 * (next = prev - dt*H prev, H prev stored in GPE_HPSI; Spin1GpeBCC.cu:554-662).
 * Hyperbolic scheme: modes 0 and 2; mode 2 is the ground-state pair itp_q +
 * itp_psi (RelativisticSpin2Gpe.cu:558-599, 706-807; RelativisticSpin1Gpe/
 * hyper_kernels.h:4-40, common_kernels.h:17-94): q_next = q_prev -
 * (dt/sigma)(q_prev - d0 psi_prev), psi_next = psi_prev - dt H(psi_prev, q_prev)
 * with B = 0 and H psi_prev stored in GPE_HPSI (get_Hpsi, :602-704).
 * next_slot and prev_slot must differ (GPE_ERR_INVALID_ARG). */
enum { GPE_MODE_LEAPFROG = 0, GPE_MODE_EULER = 1, GPE_MODE_ITP = 2 };
gpe_status gpe_step_explicit(gpe_handle* h, int32_t next_slot, int32_t prev_slot,
                             const gpe_fields* fields, double t, int32_t mode, void* stream);

/* Imaginary-time ground-state iterations: itp + renormalisation to norm 1, n
 * times, from the newest psi slot (Spin1GpeBCC.cu:1470-1478;
 * GPUGrossPitaevskii_BCC.cu:845-849).  Hyperbolic scheme: each iteration is the
 * mode-2 step of gpe_step_explicit on the (psi, q) pair, then normalize_h of the
 * new psi (RelativisticSpin2Gpe.cu:1712-1715); q is not renormalised.
 * If mu_out != NULL it receives <psi|H psi> of the last iteration (FP64, synchronises). */
gpe_status gpe_itp(gpe_handle* h, int32_t n, double* mu_out, void* stream);

/* FP64 observables of one psi slot, integrated with dv = bs^3*VOLUME
 * (density/integrate Spin1GpeBCC.cu:191-211,328-348; innerProduct :213-233;
 * localAvgSpinAndDensity + integrateSpinAndDensity :235-271, :992-1020;
 * com GPUGrossPitaevskii_BCC.cu:349-413).  Synchronises the stream. */
typedef struct {
    double norm;            /* sum |psi|^2 dv */
    double energy;          /* GP functional: kinetic + trap + c0/2 rho^2 + spin terms + Zeeman */
    double h_expect;        /* <psi|H psi> dv (the reference's `energy` kernel, BCC.cu:204-226) */
    double magnetization[3];/* sum <F> dv (unnormalised local spin times density) */
    double spin_norm;       /* sum rho |<F>/rho| dv */
    double com[3];          /* sum r |psi|^2 dv */
    double max_abs;         /* max |psi_component| */
    int32_t nonfinite;      /* number of non-finite values seen */
} gpe_observables;
gpe_status gpe_observe(gpe_handle* h, int32_t slot, double t, gpe_observables* out, void* stream);

/* Per-node output fields of a psi slot (PSI_EVEN, PSI_ODD or HPSI), FP64, interior
 * nodes in the reference's order idx = V (z X Y + y X + x) + l, K values per node:
 *   DENSITY (K = 1): |psi|^2 (density, Spin1GpeBCC.cu:191-211).
 *   SPIN (K = 5, C = 3 or 5): spin norm, local average spin x, y, z, density
 *     (localAvgSpinAndDensity, Spin1GpeBCC.cu:235-271; spin-2 Spin2GpeBCC.cu:214-254,
 *     which uses s1, s0, s_1).  As in the reference, x and y come from the spinor
 *     normalised by sqrt(density) and z = |s1|^2 - |s_1|^2 from the unnormalised one.
 *   UV_THETA (K = 7, C = 3 or 5): u x, y, z, v x, y, z, theta of a = m + i n
 *     (uvTheta, Spin1GpeBCC.cu:273-326, theta in [0, pi); Spin2GpeBCC.cu:256-306).
 *   MAX_HAMILTON (K = 1, C = 3): the local bound of maxHamilton (Spin1GpeBCC.cu:
 *     144-189) with the fields of the installed ramp at time t.
 *   PROJ_X, PROJ_Y (K = 3, C = 3): |component|^2 in the x- or y-quantised basis
 *     (the BASIS switch of the picture writer, Spin1GpeBCC/utils.h:177-193).
 * gpe_node_field_count gives K and the count of doubles `out` must hold.
 * gpe_node_fields copies the field to host memory and synchronises the stream.
 * gpe_node_fields_reduce integrates it (x dv = bs^3 VOLUME, FP64 sums, fixed
 * order): DENSITY -> out[1] = total norm; SPIN -> out[5] = spin, magnetisation
 * x, y, z, density, the quantities of integrateSpinAndDensity (Spin1GpeBCC.cu:
 * 992-1020; the magnetisation sums density x local average spin, so its z is
 * sum rho (|s1|^2 - |s_1|^2) dv there and here, unlike gpe_observe's sum F dv);
 * MAX_HAMILTON -> out[1] = the maximum over nodes (getMaxHamilton, :1022-1037,
 * the reference's dt bound). */
enum {
    GPE_FIELD_DENSITY = 0,
    GPE_FIELD_SPIN = 1,
    GPE_FIELD_UV_THETA = 2,
    GPE_FIELD_MAX_HAMILTON = 3,
    GPE_FIELD_PROJ_X = 4,
    GPE_FIELD_PROJ_Y = 5
};
gpe_status gpe_node_field_count(const gpe_handle* h, int32_t kind, size_t* per_node, size_t* count);
gpe_status gpe_node_fields(gpe_handle* h, int32_t slot, int32_t kind, double t, double* out, size_t count,
                           void* stream);
gpe_status gpe_node_fields_reduce(gpe_handle* h, int32_t slot, int32_t kind, double t, double* out, void* stream);

/* Kernel selection and tile shape (the autotuner's knobs).
 * GPE_TUNE_KERNEL: 0 = automatic, 1 = gather kernel (one node per thread per pass),
 *                  2 = row-tile kernel (TMA bulk copies of a row of cells into shared
 *                      memory; needs a cell size that is a multiple of 16 bytes),
 *                  3 = 2.5-D z-march kernel (tiles of T cells x TY rows streamed
 *                      along z through a ring of shared-memory slabs; needs 16-byte
 *                      cells, T | X and TY | Y),
 *                  4 = row-block kernel (a block of RY x RZ output rows; bulk copies
 *                      of every row the block's stencil touches; all gathers from
 *                      shared memory; needs 16-byte cells, RY | Y, RZ | Z),
 *                  5 = slab-ring kernel (one block per column of TILE_CELLS x
 *                      TILE_ROWS cells marching up z, the previous planes in a ring
 *                      of shared-memory slabs filled by bulk copies; lattices with
 *                      4 entries per node and 16-byte cells; ZCHUNK, if set, is the
 *                      number of slabs),
 *                  6 = interleaved kernel for every gpe_step / gpe_step_observe
 *                      call (FP32; the parabolic scheme on lattices with rows of 4
 *                      entries -- BCC, A15, C15, Z -- or of 4 and 8 -- FCC; the
 *                      hyperbolic scheme with 4 edges per node and 2 edges per
 *                      node of a cell -- BCC, C15).  The call changes the two psi
 *                      slots (and q) into a cell-interleaved layout (node l,
 *                      component s of 32 or 16 cells along x contiguous), steps
 *                      there and changes them back; the states are those of the
 *                      gather kernel, bit for bit.  Single explicit steps
 *                      (gpe_step_explicit, imaginary time) take the gather kernel.
 *                  The automatic choice (0) is the interleaved kernel for calls of
 *                  16 or more steps on the parabolic spinor handles and the
 *                  hyperbolic handles it applies to (faster there by 12-50 %; not
 *                  for parabolic scalars, whose 8-byte records already load as
 *                  coalesced runs; the layout changes cost a few steps per
 *                  call), else 1 (grid-stride gather, whole-record loads) -- which
 *                  gpe_get_tuning reports; 2-5 on request, and gpe_autotune may
 *                  pick any of 1-4 (it times single steps; its gather candidate is
 *                  recorded as 0).
 * GPE_TUNE_TILE_CELLS: cells per tile row (0 = automatic).
 * GPE_TUNE_TILE_ROWS: rows per tile along y (z-march TY, row-block RY; 0 = automatic).
 * GPE_TUNE_ZCHUNK: z-march planes per block, or row-block RZ (0 = automatic).
 * GPE_TUNE_THREADS: threads per row-block (a multiple of 32, at most 384; each
 *                   thread loops over the block's nodes; 0 = automatic).
 * GPE_TUNE_OBSERVE_ARITH: arithmetic of gpe_observe's per-node terms on an FP32
 *                   handle: 0 = FP64 (default; the same numbers as an FP64 run
 *                   on the stored values), 1 = FP32.  The sums over nodes are FP64
 *                   either way; mode 0 is bound by GB300's narrow FP64 pipe.
 * GPE_TUNE_CARVEOUT: shared-memory share (percent) of the unified L1 / shared
 *                   memory for the row-tile kernel; the rest caches its off-row
 *                   gathers (0 = driver default).
 * GPE_TUNE_TIMING: 1 = time every gpe_step / gpe_step_observe call with CUDA
 *                   events on its stream (each such call then synchronises the
 *                   stream at its end) and add the times to gpe_get_step_timing;
 *                   0 = off (default).
 * GPE_TUNE_TRANSFER: path of gpe_upload / gpe_download for pinned host arrays:
 *                   0 = the conversion kernel reads or writes the host array over
 *                   the host link (default; the fastest for a lone stream), 1 = a
 *                   DMA copy through the device staging buffer (overlaps other
 *                   streams' kernels). */
enum {
    GPE_TUNE_KERNEL = 0,
    GPE_TUNE_TILE_CELLS = 1,
    GPE_TUNE_TILE_ROWS = 2,
    GPE_TUNE_ZCHUNK = 3,
    GPE_TUNE_THREADS = 4,
    GPE_TUNE_OBSERVE_ARITH = 5,
    GPE_TUNE_CARVEOUT = 6,
    GPE_TUNE_TIMING = 7,
    GPE_TUNE_TRANSFER = 8
};
gpe_status gpe_set_tuning(gpe_handle* h, int32_t key, int32_t value);
gpe_status gpe_get_tuning(const gpe_handle* h, int32_t key, int32_t* value);

/* Device time of the gpe_step / gpe_step_observe calls made while GPE_TUNE_TIMING
 * was 1, from CUDA events on the calls' streams: the plain step launches, the
 * observed steps (their finalize included) and the layout changes of interleaved
 * calls.  `reset` non-zero zeroes the sums after reading.  No counterpart in the
 * reference (its programs time whole loops with host clocks). */
typedef struct {
    uint64_t calls;              /* calls timed */
    uint64_t step_launches;      /* plain step launches */
    double step_ms;              /* their device time */
    uint64_t observed_launches;  /* observed steps */
    double observed_ms;          /* their device time, finalize included */
    uint64_t convert_launches;   /* layout changes (interleaved calls: 4 per call) */
    double convert_ms;           /* their device time */
    int32_t interleaved_calls;   /* calls that ran the interleaved kernel */
    int32_t reserved;
} gpe_step_timing;
gpe_status gpe_get_step_timing(gpe_handle* h, gpe_step_timing* out, int32_t reset);

/* Autotuner: times every eligible step kernel and tile shape (cells per tile, rows
 * per block, threads per block) on this handle's own buffers with CUDA events,
 * `steps` leapfrog steps each, and keeps the fastest.  The psi buffers are saved
 * before and restored after the trials (temporary device copies).  `report`, if
 * given, receives a JSON list of the timings.  Synchronises `stream`.  No
 * counterpart in the reference (its launch shapes are compile-time #defines,
 * THREAD_BLOCK_X/Y/Z, Spin1GpeBCC.cu:39-41). */
gpe_status gpe_autotune(gpe_handle* h, int32_t steps, char* report, size_t report_len, void* stream);

/* n_steps leapfrog steps, as gpe_step, returning the observables of the state the
 * last step reads (the state after n_steps - 1 steps, at the last step's time):
 * the numbers gpe_observe(h, slot, t) gives for that state.  On the default
 * (gather) step kernel they are summed inside that step's kernel from its own
 * H psi, with no separate pass over the state: per-node terms in the storage
 * precision (FP32 handles: as GPE_TUNE_OBSERVE_ARITH = 1), sums in FP64.  With
 * another step kernel or scheme a separate observe pass runs before the last
 * step.  Replaces the reference's integrate / localAvgSpinAndDensity reductions
 * after a block of leapfrog launches (Spin1GpeBCC.cu:191-271, 992-1020, the save
 * step of its time loop :1611-1658).  Synchronises `stream`. */
gpe_status gpe_step_observe(gpe_handle* h, int32_t n_steps, gpe_observables* out, void* stream);

/* Slot (GPE_PSI_EVEN or GPE_PSI_ODD) holding the newest state after the last
 * gpe_start / gpe_step / gpe_itp call. */
int32_t gpe_current_slot(const gpe_handle* h);

/* Observables of a caller-owned psi buffer with no device allocation at all.
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory at the point where they want the norm, energy and magnetisation of
 * their state: memory owned by another framework's pool, or a time loop that
 * laid out all its buffers up front and must keep a fixed footprint.  No
 * handle is needed: psi is the interior cell (0,0,0) of a pitched buffer in the
 * reference layout (halo zero), in p->precision, and the results are the same
 * quantities gpe_observe computes.  The reduction scratch is one fixed-size
 * device array inside the library (2049 x 12 doubles, about 197 KB per GPU that
 * loads the library, held until the process exits); lattices larger than
 * 160 nodes / 640 stencil entries per cell, row_ptr tables that do not start
 * at 0 or that decrease, grids of 2^32 sites or more, and psi pointers, pitches
 * or slice pitches that are not multiples of one complex value's size (8 bytes
 * in FP32, 16 in FP64) are rejected with GPE_ERR_INVALID_ARG before the GPU is
 * touched.  During condensate expansion pass the current block scale bs(t) as
 * p->block_scale: positions and stencil weights then match the handle's step,
 * and the integrals use dv = bs(t)^3 VOLUME, where gpe_observe keeps the
 * initial bs0^3 VOLUME (multiply by (bs0/bs(t))^3 to compare).  The address
 * lookup does not survive cudaDeviceReset.  The first call on each device looks up
 * the scratch array's device address with that device current; make that first
 * call before any stream capture.  Calls share the scratch: calls that overlap on
 * the GPU race, so order them on one stream.  Synchronises `stream`; errors are
 * reported through gpe_last_error(). */
gpe_status gpe_observe_noalloc(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* fields,
                               double t, const void* psi, size_t pitch, size_t slice_pitch,
                               gpe_observables* out, void* stream);

/* Reverse-mode derivatives of a field-ramp run (parabolic scheme).  No
 * counterpart in the reference, which only runs forward; the forward run these
 * differentiate is its time loop (forwardEuler + leapfrog, Spin1GpeBCC.cu:1428-1603).
 *
 * gpe_adjoint_forward runs n_steps steps from the state in GPE_PSI_ODD: the
 * forward-Euler start (step 0) and n_steps-1 leapfrog steps, step j using
 * fields[j] at time t_j = t0 + j*dt (t0 from gpe_set_ramp, else 0) -- the same
 * steps gpe_start + gpe_step(n_steps-1) take with a ramp whose value at t_j is
 * fields[j].  It keeps checkpoints (u_{kS}, u_{kS+1}) every `stride` steps
 * (stride <= 0: ceil(sqrt(n_steps))) in device memory owned by the handle, and
 * writes out[5] = (Re <T|u_N>, Im <T|u_N>, M_x, M_y, M_z): the overlap with
 * `target` (host FP64, file layout, `count` doubles) and the magnetization of
 * the final state, integrated with dv as gpe_observe does.  Synchronises.
 *
 * gpe_adjoint_backward takes seed[5] = dL/d(out[k]) for a loss L of those five
 * numbers and writes grad[4*j + m] = dL/d(field m of step j) for
 * m = 0: bq, 1..3: bb[0..2] (n_steps x 4 doubles).  It recomputes the states of
 * one checkpoint segment at a time with the forward kernel and runs the adjoint
 * (reverse-time) kernel of the step back through it.  Valid while no other call
 * has written the handle's psi buffers since gpe_adjoint_forward; may be called
 * again with another seed.  Synchronises. */
gpe_status gpe_adjoint_forward(gpe_handle* h, int32_t n_steps, const gpe_fields* fields, int32_t stride,
                               const double* target, size_t count, double* out, void* stream);
gpe_status gpe_adjoint_backward(gpe_handle* h, const double* seed, double* grad, void* stream);

/* Batched stepping of many condensates (parabolic scheme).  No counterpart in the
 * reference, which runs one condensate per process and one kernel launch per step
 * (Spin1GpeBCC.cu:1574-1603).  A batch is built over existing handles of one
 * precision -- any lattices, grid sizes, component counts (1, 3, 5), traps and
 * ramps -- and advances all of them with one cooperative persistent kernel: the
 * members' rows are cut into work items of about GPE_BATCH_ITEM_NODES nodes, each
 * block of the persistent grid processes its share of items, evaluates the next
 * step's fields of the members from their own ramps on the device, and meets the
 * other blocks at a grid barrier whose wait is bounded in time (GPE_ERR_TIMEOUT).
 * Every member takes exactly the steps gpe_step would take (same time, fields,
 * trap switch and update), and the members' handles are updated as if gpe_step(n)
 * had been called on each, so gpe_observe / gpe_download / gpe_step keep working on
 * them.  The handles must outlive the batch and must not be used concurrently
 * with it; gpe_batch_step, _replay and _autotune synchronise the device before
 * they read the members' state, so earlier calls on any stream are complete.
 *
 * gpe_batch_step: n steps now (ceil(n / GPE_BATCH_STEPS_PER_LAUNCH) launches;
 *   0 = one launch).  Synchronises.
 * gpe_batch_capture: records an n-step call into a CUDA graph on `stream` (which
 *   must not be the legacy default stream); gpe_batch_replay launches it (one
 *   graph launch per n steps of every member) and synchronises.  The graph reads
 *   the members' current slot, step count and ramp at each replay.
 * gpe_batch_autotune: per lattice (nodes and stencil entries per cell), times
 *   `steps` steps of up to four of its members on scratch copies of their
 *   buffers, on a grid scaled so that each block has the work it has in the
 *   whole batch, for item sizes of 4K..256K nodes, and keeps the fastest; the
 *   members' states are untouched.  Within a step the blocks take items from
 *   one counter, so a block that finishes early takes more.
 *   `report` receives a JSON list of the timings.
 * An FP32 batch keeps its members' per-node constants in constant memory, one of
 * 256 slots per device and member, held until gpe_batch_destroy.  A batch created
 * while fewer slots are free (or an FP64 batch) reads them from shared memory
 * instead: the same results, about 5 % slower.  The members' parameters are read
 * once, at gpe_batch_create. */
typedef struct gpe_batch gpe_batch;
/* Batch tuning keys.  GPE_BATCH_BARRIER_TIMEOUT_MS bounds each grid-barrier wait
 * (default 10000).  GPE_BATCH_TEST_EXTRA_ARRIVALS is a test hook for the failure
 * path: the barrier then waits for that many arrivals that never come, every wait
 * runs out, the kernel returns and the call reports GPE_ERR_TIMEOUT (set it back
 * to 0 to step again).  GPE_BATCH_LAYOUT 1 (default): FP32 spin-1 members on
 * lattices with rows of 4 (or of 4 and 8) stencil entries are stepped in the
 * cell-interleaved layout of gpe_step's interleaved kernel -- each call changes
 * their two psi slots in and back (4 layout-change launches per member, in the
 * captured graph too) and the states are those of the gather form bit for bit;
 * 0: every member in its handle's layout.  Changing it drops a captured run. */
enum {
    GPE_BATCH_ITEM_NODES = 0,
    GPE_BATCH_STEPS_PER_LAUNCH = 1,
    GPE_BATCH_BLOCKS_PER_SM = 2,
    GPE_BATCH_BARRIER_TIMEOUT_MS = 3,
    GPE_BATCH_TEST_EXTRA_ARRIVALS = 4,
    GPE_BATCH_LAYOUT = 5
};
gpe_status gpe_batch_create(gpe_handle* const* members, int32_t count, gpe_batch** out);
gpe_status gpe_batch_destroy(gpe_batch* b);
gpe_status gpe_batch_step(gpe_batch* b, int32_t n, void* stream);
gpe_status gpe_batch_capture(gpe_batch* b, int32_t n, void* stream);
gpe_status gpe_batch_replay(gpe_batch* b, void* stream);
gpe_status gpe_batch_set_tuning(gpe_batch* b, int32_t key, int32_t value);
gpe_status gpe_batch_get_tuning(const gpe_batch* b, int32_t key, int32_t* value);
gpe_status gpe_batch_autotune(gpe_batch* b, int32_t steps, char* report, size_t report_len, void* stream);
uint64_t gpe_batch_sites(const gpe_batch* b);
uint64_t gpe_batch_launch_count(const gpe_batch* b);

/* Number of CUDA kernel launches this handle has issued (for accounting). */
uint64_t gpe_launch_count(const gpe_handle* h);

/* Sites (dual nodes) in the interior: V*X*Y*Z. */
uint64_t gpe_sites(const gpe_handle* h);

/* Last error text of this thread (static storage, never NULL). */
const char* gpe_last_error(void);

/* Library version string. */
const char* gpe_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GPE_H */
