// gpe_handle.h -- host-side definition of the libgpe handle (not part of the ABI).
// Shared by the translation units that implement entry points on a handle.
#pragma once

#include <string>
#include <vector>

#include "gpe_internal.h"

struct gpe_lattice {
    int V = 0;
    double bw[3] = {0, 0, 0};
    double volume = 0;
    std::vector<double> pos;
    std::vector<int32_t> row_ptr;
    std::vector<gpe_stencil_entry> stencil;
    int E = 0, F = 0;
    std::vector<gpe_edge> edges;
    std::vector<gpe_incidence> incidence;
};

namespace gpe {
// Device memory of the reverse-mode (adjoint) driver: checkpoints of the forward
// run, the recomputed states of one segment, two adjoint buffers and the target.
struct AdjointStore {
    int n = 0;                      // steps of the recorded forward run
    int stride = 0;                 // steps per checkpoint segment
    int segments = 0;
    double t0 = 0;
    std::vector<gpe_fields> fields; // per step
    std::vector<void*> ckpt;        // 2 per segment: (u_{kS}, u_{kS+1})
    std::vector<void*> seg;         // stride buffers for the recomputed segment
    void* adj[2] = {nullptr, nullptr};
    void* target = nullptr;
    size_t buf_bytes = 0;
    double* grad = nullptr;         // device, n x 4
    double* out = nullptr;          // device, 8
    double* part = nullptr;         // device, stride x blocks x 4: block partials of one segment
    size_t part_count = 0;
    double* wT64 = nullptr;         // transposed Laplacian weights
    float* wT32 = nullptr;
    bool valid = false;
    uint64_t epoch = 0;             // handle epoch at the end of the recorded forward run
};
}  // namespace gpe

struct gpe_handle {
    gpe_lattice lat;
    gpe_params p;
    int device = 0;
    size_t real_bytes = 4;
    gpe::Grid g{};
    void* alloc[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    char* interior[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    size_t alloc_bytes[5] = {0, 0, 0, 0, 0};
    gpe::DevTables tab{};
    std::vector<void*> dev_tables;
    double* partials = nullptr;
    size_t partial_blocks = 0;
    double* obs_out = nullptr;
    double* stage = nullptr;   // FP64 staging for uploads/downloads (allocated on first use)
    double* field_buf = nullptr;  // per-node output fields (gpe_node_fields; allocated on first use)
    size_t field_count = 0;
    size_t stage_count = 0;
    gpe_ramp ramp{};
    bool has_ramp = false;
    double exp_t0 = 0, exp_rate = 0;  // condensate expansion (gpe_set_expansion)
    double t0 = 0;
    int cur = 0;          // psi slot holding the newest state
    uint64_t nstep = 0;   // leapfrog steps since gpe_start / gpe_set_ramp
    uint64_t launches = 0;
    uint64_t epoch = 0;   // bumped by every call that writes a psi buffer
    int* err = nullptr;    // device error flag
    int tune_kernel = 0;   // GPE_TUNE_KERNEL
    int tune_tile = 0;     // GPE_TUNE_TILE_CELLS
    int tune_rows = 0;     // GPE_TUNE_TILE_ROWS
    int tune_zchunk = 0;   // GPE_TUNE_ZCHUNK
    int tune_threads = 0;  // GPE_TUNE_THREADS
    int tune_observe = 0;  // GPE_TUNE_OBSERVE_ARITH
    int tune_carveout = 0; // GPE_TUNE_CARVEOUT
    int tune_transfer = 0; // GPE_TUNE_TRANSFER
    uint32_t nrows = 0;    // multi-row tile kernel: (dy, dz) rows the stencil uses, own row first
    int32_t rdy[9] = {0}, rdz[9] = {0};
    int32_t* blk = nullptr;   // device row-block table of the current shape
    uint32_t blk_ry = 0, blk_rz = 0, blk_nbuf = 0;
    gpe::AdjointStore adj;
    // interleaved copies of the psi slots (index = slot) for multi-step calls,
    // allocated on first use
    char* il[2] = {nullptr, nullptr};
    gpe::ILGrid ilg{};
    // hyperbolic handles: interleaved copies of the q slots (index = slot - GPE_Q_EVEN)
    // and the interleaved offset tables of the fused step (il_hyper_tables)
    char* ilq[2] = {nullptr, nullptr};
    gpe::ILGrid ilgq{};
    int32_t* il_htab = nullptr;
    // device timing of gpe_step / gpe_step_observe calls (GPE_TUNE_TIMING)
    int tune_timing = 0;
    bool tev_ok = false;
    cudaEvent_t tev[5] = {};
    gpe_step_timing timing{};
};

namespace gpe {
gpe_status fail(gpe_status st, const std::string& msg);
gpe_status cuda_fail(cudaError_t e, const char* where);
StepArgs make_args(const gpe_handle* h, const gpe_fields& B, double t);
// One parabolic step on arbitrary buffers of the handle's geometry (interior
// pointers), with the same kernel choice as the slot-based steps.
gpe_status step_buffers(gpe_handle* h, char* next, const char* prev, const gpe_fields& B, double t, int mode,
                        cudaStream_t s);
// The leapfrog step next <- old + F(cur), leaving old as it was.  Only where the
// handle's step kernel is the gather kernel, whose in-place and out-of-place forms
// give identical states (false otherwise: nothing is launched).
bool leapfrog_from_supported(const gpe_handle* h);
gpe_status leapfrog_from(gpe_handle* h, char* next, const char* cur, const char* old, const gpe_fields& B, double t,
                         cudaStream_t s);
double cell_dv(const gpe_handle* h);
size_t host_count(const gpe_handle* h, bool is_q);
gpe_status ensure_stage(gpe_handle* h, size_t count);
gpe_status check_device_error(gpe_handle* h, cudaStream_t s);
cudaError_t launch_pack_any(int precision, double* packed, char* dev_base, uint32_t X, uint32_t Y, uint32_t Z,
                            uint32_t vals, size_t pitch, size_t slice, bool to_device, cudaStream_t s);
void adjoint_release(gpe_handle* h);
// The interleaved layout (gpe_il.cuh): the longest row the interleaved step takes
// on this handle's lattice (4, or 8 for rows of 4 and 8), 0 if it does not apply;
// and the handle's two interleaved psi copies, allocated (zeroed) on first use.
int il_stencil_deg(const gpe_handle* h);
gpe_status il_ensure(gpe_handle* h, cudaStream_t s);
// n parabolic leapfrog steps with explicit fields in the interleaved layout (both
// psi slots changed in and back), where the handle's kernel choice for a call of n
// steps is the interleaved kernel (il_leapfrog_applies); the states step_buffers
// would leave, bit for bit.
bool il_leapfrog_applies(const gpe_handle* h, int32_t n);
gpe_status il_leapfrog_explicit(gpe_handle* h, int first_prev, int32_t n, const gpe_fields* fields, double t_first,
                                double dt, cudaStream_t s);
}  // namespace gpe
