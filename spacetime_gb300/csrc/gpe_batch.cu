// gpe_batch.cu -- many condensates of uneven sizes, lattices and spin advanced
// together: one cooperative persistent kernel runs K leapfrog steps of every
// member per launch, and a run of n steps can be recorded into one CUDA graph.
//
// The reference runs one condensate per process, one kernel launch per step
// (Spin1GpeBCC.cu:1574-1603).  Here the members' interior rows are cut into work
// items of about `item_nodes` nodes (whole rows of cells, sorted by lattice and
// spin so that consecutive items mostly share a member); the blocks of the
// persistent grid take items in list order from one counter per step, process them with the
// same per-node update as the single-condensate gather kernel (parabolic_node),
// evaluates the next step's fields of its share of the members on the device
// (the members' own ramps, getSignal of AliceRingRamps.h:74-141), and meets the
// other blocks at a grid barrier.  The barrier's wait is bounded in time; a wait
// that runs out sets the batch's error flag and every block returns.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "gpe_handle.h"
#include "gpe_kernels.cuh"

namespace gpe {

// Per-member state the host refreshes before every batched call (the members'
// handles stay the source of truth: current slot, steps taken, ramp).
struct BatchState {
    gpe_ramp ramp;
    double t0, dt, trap_off_time;
    uint64_t nstep;
    int32_t cur;       // GPE_PSI_EVEN / GPE_PSI_ODD: slot of the newest state
    int32_t has_ramp;
    int32_t flags;
    int32_t pad;
};

// Per-member constants.
struct BatchMember {
    char* psi[2];       // interior pointers of GPE_PSI_EVEN, GPE_PSI_ODD
    Grid g;
    DevTables tab;
    PhysR<float> pf;    // constants; fields and trap switch filled per step
    PhysR<double> pd;
    FastDiv divV, divRow, divY;
    uint32_t row_items; // X * V
    int32_t C;
    int32_t cslot;      // slot of the member's MemberConst, or -1
    int32_t il_deg;     // 0: the handle's layout; 4 or 8: psi[] are the member's
                        // cell-interleaved copies, rows of at most il_deg entries
    ILGrid ilg;
    FastDiv divGX;
    const int32_t* il_off;  // interleaved entry offsets (il_offsets), or null
};

// The values an FP32 member's node loop reads for every node, kept in constant
// memory: read through the constant cache, they cost none of the L1 bandwidth the
// gathers are bound by (from shared memory they took about as many L1 wavefronts
// as the gathers).  The step's fields stay in shared memory.
struct MemberConst {
    PhysR<float> p;
    Grid g;
    FastDiv divV, divRow, divY;
    uint32_t row_items;
};
constexpr int kConstSlots = 256;
__constant__ MemberConst c_members[kConstSlots];

struct StepFieldsD {
    double bq, bb[3], bqq, bbq[3];
    int32_t trap_on, pad;
};

struct BatchItem {
    uint32_t member, row0, rows, pad;
};

struct BatchArgs {
    const BatchMember* members;
    const BatchState* state;
    StepFieldsD* fields;       // 2 x nmembers, by step parity
    const BatchItem* items;
    unsigned* next_item;       // one counter per step of the launch (zeroed before it)
    uint32_t nmembers, nitems;
    uint32_t nsteps;           // steps of this launch
    uint32_t step_base;        // steps of this call taken by earlier launches
    unsigned* bar;             // grid barrier: arrivals, generation
    int* err;
    unsigned expect;           // arrivals that release the barrier (gridDim.x; more only in tests)
    unsigned long long timeout_ns;
};

constexpr unsigned kBatchThreads = 256;
constexpr int32_t kMaxStepsPerLaunch = 4096;  // item counters held for one launch

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident).  The wait
// is bounded by the global timer; false means it ran out (or another block's did)
// and the error flag is set.
__device__ bool grid_barrier(unsigned* bar, int* err, unsigned expect, unsigned long long timeout_ns) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        if (atomicAdd(bar, 1u) + 1 == expect) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (*vgen == gen) {
                if (*(volatile int*)err) {
                    ok = 0;
                    break;
                }
                if (global_ns() - t0 > timeout_ns) {
                    atomicExch(err, 2);
                    ok = 0;
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Fields and trap switch of member m for step k of this call (gpe_step's
// convention: the leapfrog step after nstep steps runs at t0 + (nstep + 1) dt).
__device__ void batch_fields(const BatchArgs& A, uint32_t m, uint32_t k, StepFieldsD* out) {
    const BatchState& S = A.state[m];
    const double t = S.t0 + (double)(S.nstep + k + 1) * S.dt;
    gpe_fields B;
    B.bq = B.bq_quad = 0;
    for (int i = 0; i < 3; ++i) B.bb[i] = B.bb_quad[i] = 0;
    if (S.has_ramp) ramp_eval(S.ramp, S.ramp.time_scale * t, B);
    StepFieldsD f;
    f.bq = B.bq;
    f.bqq = B.bq_quad;
    for (int i = 0; i < 3; ++i) {
        f.bb[i] = B.bb[i];
        f.bbq[i] = B.bb_quad[i];
    }
    f.trap_on = !((S.flags & GPE_FLAG_TRAP_OFF_AFTER) && t >= S.trap_off_time);
    f.pad = 0;
    out[m] = f;
}

template <typename R>
__device__ __forceinline__ void set_fields(PhysR<R>& P, const StepFieldsD& f) {
    P.bq = (R)f.bq;
    P.bqq = (R)f.bqq;
    for (int i = 0; i < 3; ++i) {
        P.bb[i] = (R)f.bb[i];
        P.bbq[i] = (R)f.bbq[i];
    }
    P.trap_on = f.trap_on;
}

// Rows row0 .. row0 + rows - 1 of a member.  K: the member's grid and divisors
// (BatchMember in shared memory, or MemberConst in constant memory); P its
// constants; F where the step's fields are read from (P if null).
template <typename R, int C, int D, int G = D, bool MORE = false, typename MK>
__device__ __forceinline__ void batch_rows(const MK& M, const SmemTables<R>& st, const PhysR<R>& P,
                                           const PhysR<R>* F, const char* prev, char* next, uint32_t row0,
                                           uint32_t rows) {
    const uint32_t n = rows * M.row_items;
    for (uint32_t i = threadIdx.x; i < n; i += kBatchThreads) {
        const uint32_t rr = fdiv(i, M.divRow);
        const uint32_t within = i - rr * M.row_items;
        const uint32_t x = fdiv(within, M.divV);
        const uint32_t l = within - x * M.g.V;
        const uint32_t row = row0 + rr;
        const uint32_t z = fdiv(row, M.divY);
        const uint32_t y = row - z * M.g.Y;
        parabolic_node<R, C, GPE_MODE_LEAPFROG, D, G, MORE>(M.g, st, P, prev, next, nullptr, x, y, z, l, F);
    }
}

// Rows row0 .. row0 + rows - 1 of a scalar member whose nodes all have 4 entries,
// two nodes per thread and pass (i and i + kBatchThreads), the loads of both issued
// before either is computed: a scalar node's few loads leave the memory idle at the
// batch kernel's occupancy (the single-condensate gather kernel runs scalars at 48
// warps per SM, the batch kernel at 32).  Per node the arithmetic and its order are
// parabolic_node_t's (D = 4) and node_finish's.
template <typename R, typename MK>
__device__ __forceinline__ void batch_rows_c1x2(const MK& M, const SmemTables<R>& st, const PhysR<R>& P,
                                                const PhysR<R>* F, const char* prev, char* next, uint32_t row0,
                                                uint32_t rows) {
    constexpr uint32_t node_bytes = 2 * sizeof(R);
    const uint32_t n = rows * M.row_items;
    for (uint32_t i0 = threadIdx.x; i0 < n; i0 += 2 * kBatchThreads) {
        uint32_t x[2], y[2], z[2], l[2];
        bool ok[2];
        size_t own[2];
        Cx<R> prv[2][1], nv[2][1], v[2][4][1];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint32_t i = i0 + q * kBatchThreads;
            ok[q] = i < n;
            const uint32_t ii = ok[q] ? i : i0;   // a valid node either way; its results are not stored
            const uint32_t rr = fdiv(ii, M.divRow);
            const uint32_t within = ii - rr * M.row_items;
            x[q] = fdiv(within, M.divV);
            l[q] = within - x[q] * M.g.V;
            const uint32_t row = row0 + rr;
            z[q] = fdiv(row, M.divY);
            y[q] = row - z[q] * M.g.Y;
            const size_t cell_off = (size_t)z[q] * M.g.slice + (size_t)y[q] * M.g.pitch + (size_t)x[q] * M.g.cell_bytes;
            own[q] = cell_off + l[q] * node_bytes;
            const int4 o4 = *reinterpret_cast<const int4*>(st.nb_off + 4 * l[q]);
            const int32_t off[4] = {o4.x, o4.y, o4.z, o4.w};
            ld_node<R, 1, true>(prev + own[q], prv[q]);
            ld_node<R, 1, false>(next + own[q], nv[q]);
#pragma unroll
            for (int k = 0; k < 4; ++k) ld_node<R, 1, true>(prev + cell_off + off[k], v[q][k]);
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!ok[q]) continue;
            // the node's weights and position, read again from the shared tables
            const NodeTab<R, 4> t = node_tab<R, 4>(st, l[q]);
            Cx<R> H[1] = {cx<R>((R)0, (R)0)};
#pragma unroll
            for (int k = 0; k < 4; ++k) H[0] += t.w[k] * (v[q][k][0] - prv[q][0]);
            node_finish<R, 1, GPE_MODE_LEAPFROG>(P, t.pos, x[q], y[q], z[q], prv[q], H, nv[q], next + own[q], nullptr, F);
        }
    }
}

// Rows row0 .. row0 + rows - 1 of a member in the interleaved layout (FP32).
// Warp task t = u V + l within the item: node l of the item's u-th group
// (il_lane_group, counted row after row): the 8 warps of a block take
// consecutive nodes of the same groups, as the single-condensate interleaved
// kernel's warps do, so the neighbour records they gather are read while they are
// still in L2.  A node's stencil comes from the shared tables for every task:
// st.nb_off holds the member's interleaved entry offsets (il_offsets: rows, node
// and dx, with dx + 1 in the two low bits), to which each lane adds its own cell
// and, where x + dx leaves the group, the step to the neighbouring group.  The
// per-lane update is il_task, bit for bit the single-condensate kernel's.
template <int C, int D, int CELLS>
__device__ __forceinline__ void batch_il_rows(const BatchMember& M, const SmemTables<float>& st, const PhysR<float>& P,
                                              const PhysR<float>* F, const char* prev, char* next, uint32_t row0,
                                              uint32_t rows) {
    const ILGrid& G = M.ilg;
    const uint32_t sub = threadIdx.x & (CELLS - 1);
    constexpr uint32_t kWarps = kBatchThreads / 32;
    constexpr uint32_t kWG = 32 / CELLS;
    const uint32_t nq = rows * G.GX;
    const uint32_t tasks = (nq + kWG - 1) / kWG * G.V;
    const int32_t wrap = (int32_t)G.gb - CELLS * 8;
    NoObs no;
    for (uint32_t t = threadIdx.x >> 5; t < tasks; t += kWarps) {
        const uint32_t u = fdiv(t, M.divV);
        const uint32_t l = t - u * G.V;
        uint32_t gx, y, z;
        if (!il_lane_group<CELLS>(G, u, nq, row0, M.divGX, M.divY, gx, y, z)) continue;
        const int f0 = st.row_ptr[l];
        const int nd = D == 4 ? 4 : st.row_ptr[l + 1] - f0;
        int32_t off[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            off[k] = 1;
            if (k < nd) {
                const int32_t b = st.nb_off[f0 + k];
                const int xl = (int)sub + (b & 3) - 1;
                const int32_t gs = xl < 0 ? -1 : (xl >= CELLS ? 1 : 0);
                off[k] = ((b & ~3) + (int32_t)sub * 8 + gs * wrap) | (b & 3);
            }
        }
        il_task<C, D, CELLS, NoObs>(G, P, F, prev, next, off, st.w + f0, nd, st.pos + 3 * l, sub, l, gx, y, z, &no);
    }
}

// One work item: the member's kernel form by its spin and row lengths.  Members
// whose nodes all have 4 neighbours issue the 4 loads together; rows of 4 and 8
// (FCC) take their entries in vectors of 4.  Interleaved members (FP32 spin-1):
// batch_il_rows.
template <typename R, int CMASK, bool IL, typename MK>
__device__ __forceinline__ void batch_item(const BatchMember& M, const MK& K, const SmemTables<R>& st,
                                           const PhysR<R>& P, const PhysR<R>* F, const char* prev, char* next,
                                           uint32_t row0, uint32_t rows) {
    if constexpr (IL && sizeof(R) == 4) {
        if (M.il_deg) {
            const bool c32 = M.ilg.cells == 32;
            if ((CMASK & 2) && M.C == 3) {
                if (M.il_deg == 4) {
                    if (c32) batch_il_rows<3, 4, 32>(M, st, P, F, prev, next, row0, rows);
                    else batch_il_rows<3, 4, 16>(M, st, P, F, prev, next, row0, rows);
                } else {
                    if (c32) batch_il_rows<3, 8, 32>(M, st, P, F, prev, next, row0, rows);
                    else batch_il_rows<3, 8, 16>(M, st, P, F, prev, next, row0, rows);
                }
            }
            return;
        }
    }
    const bool d4 = M.tab.uniform_deg == 4, quad = M.tab.quad_rows != 0;
    if ((CMASK & 1) && M.C == 1) {
        if (d4) batch_rows_c1x2<R>(K, st, P, F, prev, next, row0, rows);
        else if (quad) batch_rows<R, 1, 4, 4, true>(K, st, P, F, prev, next, row0, rows);
        else batch_rows<R, 1, 0>(K, st, P, F, prev, next, row0, rows);
    } else if ((CMASK & 2) && M.C == 3) {
        if (d4) batch_rows<R, 3, 4>(K, st, P, F, prev, next, row0, rows);
        else if (quad) batch_rows<R, 3, 4, 4, true>(K, st, P, F, prev, next, row0, rows);
        else batch_rows<R, 3, 0>(K, st, P, F, prev, next, row0, rows);
    } else if (CMASK & 4) {
        batch_rows<R, 5, 0>(K, st, P, F, prev, next, row0, rows);
    }
}

// CMASK: which component counts the batch holds (bit 0: 1, bit 1: 3, bit 2: 5), so
// that a batch of scalar and spin-1 members does not carry spin-2 registers; such
// FP32 batches fit 64 registers, 4 blocks per SM.  CONSTP (FP32): every member has
// a MemberConst slot.  IL (FP32): some members are stepped in the interleaved
// layout.
template <typename R, int CMASK, bool CONSTP, bool IL>
__global__ void __launch_bounds__(kBatchThreads, sizeof(R) == 8 ? 1 : (CMASK & 4) ? 3 : 4) batch_kernel(BatchArgs A) {
    static_assert(!CONSTP || sizeof(R) == 4, "constant-memory members are FP32");
    __shared__ SmemTables<R> st;
    __shared__ PhysR<R> P;
    __shared__ BatchMember M;
    __shared__ uint32_t grabbed;
    const uint32_t gtid = blockIdx.x * kBatchThreads + threadIdx.x;
    const uint32_t gthreads = gridDim.x * kBatchThreads;
    for (uint32_t m = gtid; m < A.nmembers; m += gthreads) batch_fields(A, m, A.step_base, A.fields);
    if (!grid_barrier(A.bar, A.err, A.expect, A.timeout_ns)) return;
    for (uint32_t s = 0; s < A.nsteps; ++s) {
        const uint32_t k = A.step_base + s;
        const StepFieldsD* F = A.fields + (size_t)(s & 1) * A.nmembers;
        uint32_t loaded = 0xffffffffu;
        for (;;) {
            // items are handed out in list order by one counter per step, so blocks
            // that finish early take more and the step ends within about one item
            if (threadIdx.x == 0) grabbed = atomicAdd(A.next_item + s, 1u);
            __syncthreads();
            const uint32_t it = grabbed;
            __syncthreads();  // every thread has read `grabbed` before thread 0 rewrites it
            if (it >= A.nitems) break;
            const BatchItem w = A.items[it];
            // items of one member share the staged tables: the block synchronises
            // only where the member changes (w.member is the same in every thread)
            if (w.member != loaded) {
                __syncthreads();  // every warp is done with the previous member's tables
                if (threadIdx.x == 0) M = A.members[w.member];
                __syncthreads();
                const int V = M.g.V, nent = M.tab.entries;
                for (int i = threadIdx.x; i <= V; i += kBatchThreads) st.row_ptr[i] = M.tab.row_ptr[i];
                const int32_t* offs = IL && M.il_deg ? M.il_off : M.tab.nb_off;
                for (int i = threadIdx.x; i < nent; i += kBatchThreads) {
                    st.nb_off[i] = offs[i];
                    if constexpr (sizeof(R) == 4) st.w[i] = M.tab.w32[i];
                    else st.w[i] = M.tab.w64[i];
                }
                for (int i = threadIdx.x; i < 3 * V; i += kBatchThreads) {
                    if constexpr (sizeof(R) == 4) st.pos[i] = M.tab.pos32[i];
                    else st.pos[i] = M.tab.pos64[i];
                }
                if (threadIdx.x == 0) {
                    if constexpr (sizeof(R) == 4) P = M.pf;
                    else P = M.pd;
                    set_fields<R>(P, F[w.member]);
                }
                loaded = w.member;
                __syncthreads();
            }
            const int prev_slot = A.state[w.member].cur ^ (int)(k & 1);
            const char* prev = M.psi[prev_slot];
            char* next = M.psi[prev_slot ^ 1];
            if constexpr (CONSTP) {
                const MemberConst& K = c_members[M.cslot];
                batch_item<R, CMASK, IL>(M, K, st, K.p, &P, prev, next, w.row0, w.rows);
            } else {
                batch_item<R, CMASK, IL>(M, M, st, P, nullptr, prev, next, w.row0, w.rows);
            }
        }
        if (s + 1 < A.nsteps) {
            StepFieldsD* G = A.fields + (size_t)((s + 1) & 1) * A.nmembers;
            for (uint32_t m = gtid; m < A.nmembers; m += gthreads) batch_fields(A, m, k + 1, G);
        }
        if (!grid_barrier(A.bar, A.err, A.expect, A.timeout_ns)) return;
    }
}

template <typename R, int CMASK, bool CONSTP, bool IL = false>
static void* batch_kernel_ptr() {
    return reinterpret_cast<void*>(&batch_kernel<R, CMASK, CONSTP, IL>);
}

static void* batch_kernel_for(int precision, int cmask, bool constp, bool il) {
    typedef void* (*Fn)();
    static const Fn f32[8] = {nullptr, batch_kernel_ptr<float, 1, false>, batch_kernel_ptr<float, 2, false>,
                              batch_kernel_ptr<float, 3, false>, batch_kernel_ptr<float, 4, false>,
                              batch_kernel_ptr<float, 5, false>, batch_kernel_ptr<float, 6, false>,
                              batch_kernel_ptr<float, 7, false>};
    static const Fn f32c[8] = {nullptr, batch_kernel_ptr<float, 1, true>, batch_kernel_ptr<float, 2, true>,
                               batch_kernel_ptr<float, 3, true>, batch_kernel_ptr<float, 4, true>,
                               batch_kernel_ptr<float, 5, true>, batch_kernel_ptr<float, 6, true>,
                               batch_kernel_ptr<float, 7, true>};
    // interleaved members are spinors: masks with bit 1 or 2
    static const Fn f32i[8] = {nullptr, nullptr, batch_kernel_ptr<float, 2, false, true>,
                               batch_kernel_ptr<float, 3, false, true>, batch_kernel_ptr<float, 4, false, true>,
                               batch_kernel_ptr<float, 5, false, true>, batch_kernel_ptr<float, 6, false, true>,
                               batch_kernel_ptr<float, 7, false, true>};
    static const Fn f32ci[8] = {nullptr, nullptr, batch_kernel_ptr<float, 2, true, true>,
                                batch_kernel_ptr<float, 3, true, true>, batch_kernel_ptr<float, 4, true, true>,
                                batch_kernel_ptr<float, 5, true, true>, batch_kernel_ptr<float, 6, true, true>,
                                batch_kernel_ptr<float, 7, true, true>};
    static const Fn f64[8] = {nullptr, batch_kernel_ptr<double, 1, false>, batch_kernel_ptr<double, 2, false>,
                              batch_kernel_ptr<double, 3, false>, batch_kernel_ptr<double, 4, false>,
                              batch_kernel_ptr<double, 5, false>, batch_kernel_ptr<double, 6, false>,
                              batch_kernel_ptr<double, 7, false>};
    if (cmask < 1 || cmask > 7) return nullptr;
    if (precision == GPE_FP64) return f64[cmask]();
    const Fn* t = il ? (constp ? f32ci : f32i) : (constp ? f32c : f32);
    return t[cmask] ? t[cmask]() : nullptr;
}

// Constant-memory slots of FP32 members, per device.
std::mutex g_slot_mu;
constexpr int kSlotDevices = 64;
bool g_slot_used[kSlotDevices][kConstSlots];

// n free slots of the device, or none when fewer are free.
std::vector<int> take_slots(int device, int n) {
    std::vector<int> got;
    if (device < 0 || device >= kSlotDevices) return got;
    std::lock_guard<std::mutex> lock(g_slot_mu);
    for (int i = 0; i < kConstSlots && (int)got.size() < n; ++i)
        if (!g_slot_used[device][i]) got.push_back(i);
    if ((int)got.size() < n) return {};
    for (int i : got) g_slot_used[device][i] = true;
    return got;
}

void give_slots(int device, const std::vector<int>& slots) {
    if (device < 0 || device >= kSlotDevices) return;
    std::lock_guard<std::mutex> lock(g_slot_mu);
    for (int i : slots) g_slot_used[device][i] = false;
}

}  // namespace gpe

using namespace gpe;

struct gpe_batch {
    std::vector<gpe_handle*> members;
    int precision = GPE_FP32;
    int cmask = 0;
    int device = 0;
    int sms = 0;
    int blocks_per_sm = 0;      // occupancy of the kernel (cooperative limit)
    int grid = 0;
    int32_t tune_blocks_per_sm = 0;  // 0: occupancy limit
    int32_t steps_per_launch = 0;    // 0: all steps of a call in one launch
    std::vector<std::pair<uint64_t, int32_t>> item_nodes_by_lattice;  // (lattice key, target nodes per item)
    int32_t item_nodes = 16384;
    int32_t barrier_timeout_ms = 10000;
    int32_t extra_arrivals = 0;       // test hook: the barrier waits for arrivals that never come
    BatchMember* d_members = nullptr;
    BatchState* d_state = nullptr;
    BatchState* h_state = nullptr;   // pinned
    StepFieldsD* d_fields = nullptr;
    BatchItem* d_items = nullptr;
    size_t items_cap = 0;
    uint32_t nitems = 0;
    std::vector<uint64_t> item_cost;  // prefix sums of the items' nodes x components
    unsigned* d_next = nullptr;       // per-step item counters of one launch
    unsigned* d_bar = nullptr;
    int* d_err = nullptr;
    std::vector<int> cslots;         // FP32: one constant-memory slot per member, or none
    int32_t layout = 1;              // GPE_BATCH_LAYOUT
    std::vector<int> il_deg;         // per member: 0, or the interleaved rows (4 or 8)
    std::vector<void*> il_off;       // per member: device interleaved entry offsets, or null
    bool any_il = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int32_t graph_steps = 0;
    uint64_t launches = 0;
};

namespace {

gpe_status batch_fail_cuda(cudaError_t e, const char* where) { return cuda_fail(e, where); }

void member_constants(const gpe_handle* h, BatchMember& M) {
    gpe_fields zero;
    std::memset(&zero, 0, sizeof zero);
    StepArgs a = make_args(h, zero, 0.0);
    M.psi[GPE_PSI_EVEN] = h->interior[GPE_PSI_EVEN];
    M.psi[GPE_PSI_ODD] = h->interior[GPE_PSI_ODD];
    M.g = h->g;
    M.tab = h->tab;
    M.pf = a.pf;
    M.pd = a.pd;
    M.divV = a.divV;
    M.divRow = a.divRow;
    M.divY = a.divY;
    M.row_items = a.row_items;
    M.C = h->g.C;
    M.cslot = -1;
    M.il_deg = 0;
    M.ilg = make_il_grid(h->g);
    M.divGX = make_fastdiv(M.ilg.GX);
    M.il_off = nullptr;
}

// A member's stencil entries as byte offsets in the interleaved layout, relative to
// a group's base, for the group's first cell: the rows (dz, dy), the node and dx,
// with dx + 1 (|dx| <= 1) in the two low bits.  Empty if one does not fit 32 bits.
std::vector<int32_t> il_offsets(const gpe_handle* h) {
    const ILGrid G = make_il_grid(h->g);
    const int64_t node_run = (int64_t)G.C * G.cells * 8;
    std::vector<int32_t> out;
    for (const gpe_stencil_entry& e : h->lat.stencil) {
        const int64_t b = ((int64_t)e.dz * (G.Y + 2) + e.dy) * (int64_t)G.row + (int64_t)e.node * node_run + (int64_t)e.dx * 8;
        if (b > INT32_MAX - 3 || b < INT32_MIN) return {};
        out.push_back((int32_t)b | (e.dx + 1));
    }
    return out;
}

// The layout member m is stepped in: the interleaved one for FP32 spin-1 members on
// lattices of at most 64 nodes a cell with rows of 4 (or of 4 and 8) entries (BCC,
// FCC, A15, Z) when GPE_BATCH_LAYOUT is 1 (the default), the handle's own otherwise.  (Spin-2 members keep the handle's layout:
// their interleaved path does not fit the batch kernel's registers.)
int member_il_deg(const gpe_batch* b, const gpe_handle* h) {
    if (!b->layout || b->precision != GPE_FP32 || h->g.C != 3) return 0;
    // C15 (136 nodes a cell) measured faster in the handle's layout inside the batch
    // (the ensemble's 25 C15 spin-1 members: 7.22 against 7.52 ms per step)
    if (h->g.V > 64) return 0;
    return il_stencil_deg(h);
}

// Every member's BatchMember (constants, layout, constant-memory slot) into d_members.
gpe_status upload_members(gpe_batch* b) {
    const size_t n = b->members.size();
    std::vector<BatchMember> hm(n);
    b->il_deg.assign(n, 0);
    b->il_off.resize(n, nullptr);
    b->any_il = false;
    for (size_t i = 0; i < n; ++i) {
        gpe_handle* h = b->members[i];
        member_constants(h, hm[i]);
        if (!b->cslots.empty()) hm[i].cslot = b->cslots[i];
        const int deg = member_il_deg(b, h);
        const std::vector<int32_t> offs = deg ? il_offsets(h) : std::vector<int32_t>();
        if (deg && !offs.empty()) {
            if (gpe_status st = il_ensure(h, 0)) return st;
            if (!b->il_off[i]) {
                if (cudaMalloc(&b->il_off[i], offs.size() * sizeof(int32_t)) != cudaSuccess)
                    return fail(GPE_ERR_OOM, "cudaMalloc (batch interleaved offsets)");
                cudaError_t e = cudaMemcpy(b->il_off[i], offs.data(), offs.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
                if (e != cudaSuccess) return cuda_fail(e, "batch interleaved offsets");
            }
            hm[i].il_off = static_cast<const int32_t*>(b->il_off[i]);
            hm[i].il_deg = deg;
            hm[i].psi[GPE_PSI_EVEN] = h->il[GPE_PSI_EVEN];
            hm[i].psi[GPE_PSI_ODD] = h->il[GPE_PSI_ODD];
            b->il_deg[i] = deg;
            b->any_il = true;
        }
    }
    cudaError_t e = cudaMemcpy(b->d_members, hm.data(), n * sizeof(BatchMember), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "batch members upload");
    return GPE_OK;
}

// The interleaved members' two psi slots changed into (to_il) or out of their
// interleaved copies.
gpe_status convert_members(gpe_batch* b, bool to_il, cudaStream_t s) {
    for (size_t i = 0; i < b->members.size(); ++i) {
        if (!b->il_deg[i]) continue;
        gpe_handle* h = b->members[i];
        for (int k = GPE_PSI_EVEN; k <= GPE_PSI_ODD; ++k) {
            cudaError_t e = launch_il_convert(h->interior[k], h->g, h->il[k], h->ilg, to_il, s);
            if (e != cudaSuccess) return cuda_fail(e, to_il ? "batch layout change (in)" : "batch layout change (out)");
        }
    }
    return GPE_OK;
}

uint64_t convert_launch_count(const gpe_batch* b) {
    uint64_t n = 0;
    for (int d : b->il_deg) n += d ? 4 : 0;
    return n;
}

// A lattice is told apart by its node and stencil-entry counts per cell.
uint64_t lattice_key(const gpe_handle* h) { return ((uint64_t)h->g.V << 32) | (uint32_t)h->tab.entries; }

int32_t target_nodes(const gpe_batch* b, const gpe_handle* h) {
    for (const auto& kv : b->item_nodes_by_lattice)
        if (kv.first == lattice_key(h)) return kv.second;
    return b->item_nodes;
}

// Work items of the members `which` (indices into b->members), sorted by lattice
// (V) and spin so that consecutive items share tables.
std::vector<BatchItem> build_items(const gpe_batch* b, const std::vector<uint32_t>& which) {
    std::vector<uint32_t> order(which);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const gpe_handle* hx = b->members[x];
        const gpe_handle* hy = b->members[y];
        if (lattice_key(hx) != lattice_key(hy)) return lattice_key(hx) < lattice_key(hy);
        return hx->g.C < hy->g.C;
    });
    std::vector<BatchItem> items;
    for (uint32_t m : order) {
        const Grid& g = b->members[m]->g;
        const uint64_t row_nodes = (uint64_t)g.X * g.V;
        const uint32_t rows_total = g.Y * g.Z;
        uint32_t per = (uint32_t)std::max<uint64_t>(1, (uint64_t)target_nodes(b, b->members[m]) / row_nodes);
        per = std::min(per, rows_total);
        for (uint32_t r = 0; r < rows_total; r += per) items.push_back({m, r, std::min(per, rows_total - r), 0});
    }
    return items;
}

// Work of an item in the units the blocks are balanced in: nodes x components.
uint64_t item_cost(const Grid& g, const BatchItem& w) { return (uint64_t)w.rows * g.X * g.V * g.C; }

gpe_status upload_items(gpe_batch* b, const std::vector<BatchItem>& items, const std::vector<const Grid*>& grids) {
    b->item_cost.assign(items.size() + 1, 0);
    for (size_t i = 0; i < items.size(); ++i) b->item_cost[i + 1] = b->item_cost[i] + item_cost(*grids[items[i].member], items[i]);
    if (items.size() > b->items_cap) {
        if (b->d_items) cudaFree(b->d_items);
        b->d_items = nullptr;
        if (cudaMalloc(&b->d_items, items.size() * sizeof(BatchItem)) != cudaSuccess)
            return fail(GPE_ERR_OOM, "cudaMalloc (batch items)");
        b->items_cap = items.size();
    }
    cudaError_t e = cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return batch_fail_cuda(e, "cudaMemcpy (batch items)");
    b->nitems = (uint32_t)items.size();
    return GPE_OK;
}

std::vector<const Grid*> member_grids(const gpe_batch* b) {
    std::vector<const Grid*> g(b->members.size());
    for (size_t i = 0; i < g.size(); ++i) g[i] = &b->members[i]->g;
    return g;
}

gpe_status rebuild_items(gpe_batch* b) {
    std::vector<uint32_t> all(b->members.size());
    for (uint32_t i = 0; i < all.size(); ++i) all[i] = i;
    return upload_items(b, build_items(b, all), member_grids(b));
}

// Refreshes the per-member state; members stepped with condensate expansion
// (a block scale that changes in time) are refused, since the batch kernel
// keeps each member's block scale fixed.
gpe_status fill_state(gpe_batch* b) {
    for (size_t m = 0; m < b->members.size(); ++m) {
        const gpe_handle* h = b->members[m];
        if (h->exp_rate != 0) return fail(GPE_ERR_UNSUPPORTED, "batched stepping does not follow condensate expansion");
        BatchState& S = b->h_state[m];
        S.ramp = h->ramp;
        S.has_ramp = h->has_ramp ? 1 : 0;
        S.t0 = h->t0;
        S.dt = h->p.dt;
        S.trap_off_time = h->p.trap_off_time;
        S.nstep = h->nstep;
        S.cur = h->cur;
        S.flags = h->p.flags;
        S.pad = 0;
    }
    return GPE_OK;
}

gpe_status grid_size(gpe_batch* b) {
    void* fn = batch_kernel_for(b->precision, b->cmask, !b->cslots.empty(), b->any_il);
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kBatchThreads, 0);
    if (e != cudaSuccess) return batch_fail_cuda(e, "occupancy of the batch kernel");
    if (occ < 1) return fail(GPE_ERR_UNSUPPORTED, "the batch kernel does not fit on an SM");
    b->blocks_per_sm = occ;
    const int per = b->tune_blocks_per_sm > 0 ? std::min<int>(b->tune_blocks_per_sm, occ) : occ;
    b->grid = per * b->sms;
    return GPE_OK;
}

// Enqueues n steps of every member: the state upload, the interleaved members'
// layout change in (convert), ceil(n / K) persistent launches, and the layout
// change back.  Capturable into a CUDA graph (the state copy reads the pinned host
// array when the graph runs).
gpe_status enqueue_steps(gpe_batch* b, int32_t n, cudaStream_t s, const BatchMember* members, uint32_t nmembers,
                         const BatchState* h_state, int grid, bool convert) {
    cudaError_t e = cudaMemcpyAsync(b->d_state, h_state, nmembers * sizeof(BatchState), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return batch_fail_cuda(e, "batch state upload");
    if (convert)
        if (gpe_status st = convert_members(b, true, s)) return st;
    void* fn = batch_kernel_for(b->precision, b->cmask, !b->cslots.empty(), b->any_il);
    const int32_t K = std::min(b->steps_per_launch > 0 ? b->steps_per_launch : n, kMaxStepsPerLaunch);
    for (int32_t done = 0; done < n; done += K) {
        const int32_t steps = std::min(K, n - done);
        if ((e = cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned), s)) != cudaSuccess ||
            (e = cudaMemsetAsync(b->d_next, 0, (size_t)steps * sizeof(unsigned), s)) != cudaSuccess)
            return batch_fail_cuda(e, "batch barrier reset");
        BatchArgs A;
        A.members = members;
        A.state = b->d_state;
        A.fields = b->d_fields;
        A.items = b->d_items;
        A.next_item = b->d_next;
        A.nmembers = nmembers;
        A.nitems = b->nitems;
        A.nsteps = (uint32_t)steps;
        A.step_base = (uint32_t)done;
        A.bar = b->d_bar;
        A.err = b->d_err;
        A.expect = (unsigned)(grid + b->extra_arrivals);
        A.timeout_ns = (unsigned long long)b->barrier_timeout_ms * 1000000ull;
        void* args[] = {&A};
        cudaLaunchConfig_t cfg;
        std::memset(&cfg, 0, sizeof cfg);
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3(kBatchThreads);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if ((e = cudaLaunchKernelExC(&cfg, fn, args)) != cudaSuccess) return batch_fail_cuda(e, "batch kernel launch");
        b->launches += 1;
    }
    if (convert) {
        if (gpe_status st = convert_members(b, false, s)) return st;
        b->launches += convert_launch_count(b);
    }
    return GPE_OK;
}

gpe_status check_batch_error(gpe_batch* b, cudaStream_t s) {
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return batch_fail_cuda(e, "batch run");
    if (flag) {
        cudaMemsetAsync(b->d_err, 0, sizeof(int), s);
        return fail(GPE_ERR_TIMEOUT, "a grid barrier of the batch kernel ran out of time");
    }
    return GPE_OK;
}

void advance_members(gpe_batch* b, int32_t n) {
    for (gpe_handle* h : b->members) {
        if (n & 1) h->cur = h->cur == GPE_PSI_EVEN ? GPE_PSI_ODD : GPE_PSI_EVEN;
        h->nstep += (uint64_t)n;
        h->epoch += 1;
    }
}

void release_batch(gpe_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_members) cudaFree(b->d_members);
    if (b->d_state) cudaFree(b->d_state);
    if (b->h_state) cudaFreeHost(b->h_state);
    if (b->d_fields) cudaFree(b->d_fields);
    if (b->d_items) cudaFree(b->d_items);
    if (b->d_next) cudaFree(b->d_next);
    if (b->d_bar) cudaFree(b->d_bar);
    if (b->d_err) cudaFree(b->d_err);
    give_slots(b->device, b->cslots);
    b->cslots.clear();
    for (void* p : b->il_off)
        if (p) cudaFree(p);
    b->il_off.clear();
}

}  // namespace

extern "C" gpe_status gpe_batch_create(gpe_handle* const* members, int32_t count, gpe_batch** out) {
    if (!members || !out || count < 1) return fail(GPE_ERR_INVALID_ARG, "null argument or empty batch");
    *out = nullptr;
    gpe_batch* b = new (std::nothrow) gpe_batch();
    if (!b) return fail(GPE_ERR_OOM, "host allocation");
    b->members.assign(members, members + count);
    for (int32_t i = 0; i < count; ++i) {
        const gpe_handle* h = members[i];
        if (!h) {
            delete b;
            return fail(GPE_ERR_INVALID_ARG, "null member handle");
        }
        if (h->p.scheme != GPE_SCHEME_PARABOLIC) {
            delete b;
            return fail(GPE_ERR_UNSUPPORTED, "batched stepping is built for the parabolic scheme");
        }
        if (i == 0) {
            b->precision = h->p.precision;
            b->device = h->device;
        } else if (h->p.precision != b->precision || h->device != b->device) {
            delete b;
            return fail(GPE_ERR_INVALID_ARG, "batch members must share precision and device");
        }
        for (int32_t j = 0; j < i; ++j)
            if (members[j] == h) {
                delete b;
                return fail(GPE_ERR_INVALID_ARG, "a handle appears twice in the batch");
            }
        b->cmask |= h->g.C == 1 ? 1 : h->g.C == 3 ? 2 : 4;
    }
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, b->device);
    if (!coop) {
        delete b;
        return fail(GPE_ERR_UNSUPPORTED, "the device does not support cooperative launches");
    }
    std::vector<BatchMember> hm(count);
    for (int32_t i = 0; i < count; ++i) member_constants(members[i], hm[i]);
    gpe_status st = GPE_OK;
    if (b->precision == GPE_FP32) {
        // the members' per-node constants into constant memory, where slots are free
        b->cslots = take_slots(b->device, count);
        for (int32_t i = 0; i < (int32_t)b->cslots.size(); ++i) {
            MemberConst mc;
            std::memset(&mc, 0, sizeof mc);
            mc.p = hm[i].pf;
            mc.g = hm[i].g;
            mc.divV = hm[i].divV;
            mc.divRow = hm[i].divRow;
            mc.divY = hm[i].divY;
            mc.row_items = hm[i].row_items;
            hm[i].cslot = b->cslots[i];
            cudaError_t ce = cudaMemcpyToSymbol(c_members, &mc, sizeof mc, (size_t)b->cslots[i] * sizeof(MemberConst));
            if (ce != cudaSuccess) {
                release_batch(b);
                delete b;
                return cuda_fail(ce, "batch member constants");
            }
        }
    }
    if (cudaMalloc(&b->d_members, count * sizeof(BatchMember)) != cudaSuccess ||
        cudaMalloc(&b->d_state, count * sizeof(BatchState)) != cudaSuccess ||
        cudaMallocHost(&b->h_state, count * sizeof(BatchState)) != cudaSuccess ||
        cudaMalloc(&b->d_fields, 2 * (size_t)count * sizeof(StepFieldsD)) != cudaSuccess ||
        cudaMalloc(&b->d_bar, 2 * sizeof(unsigned)) != cudaSuccess || cudaMalloc(&b->d_err, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->d_next, kMaxStepsPerLaunch * sizeof(unsigned)) != cudaSuccess) {
        release_batch(b);
        delete b;
        return fail(GPE_ERR_OOM, "batch allocation");
    }
    cudaMemset(b->d_err, 0, sizeof(int));
    st = upload_members(b);
    if (!st) st = grid_size(b);
    if (!st) st = rebuild_items(b);
    if (st) {
        release_batch(b);
        delete b;
        return st;
    }
    *out = b;
    return GPE_OK;
}

extern "C" gpe_status gpe_batch_destroy(gpe_batch* b) {
    if (!b) return GPE_OK;
    release_batch(b);
    delete b;
    return GPE_OK;
}

extern "C" gpe_status gpe_batch_step(gpe_batch* b, int32_t n, void* stream) {
    if (!b) return fail(GPE_ERR_INVALID_ARG, "null batch");
    if (n < 0) return fail(GPE_ERR_INVALID_ARG, "negative step count");
    if (n == 0) return GPE_OK;
    cudaStream_t s = (cudaStream_t)stream;
    // the members' own calls may sit on other streams, and the pinned state array
    // may still feed a copy of an earlier call
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "batch step");
    if (gpe_status st = fill_state(b)) return st;
    gpe_status st = enqueue_steps(b, n, s, b->d_members, (uint32_t)b->members.size(), b->h_state, b->grid, true);
    if (st) return st;
    advance_members(b, n);
    return check_batch_error(b, s);
}

extern "C" gpe_status gpe_batch_capture(gpe_batch* b, int32_t n, void* stream) {
    if (!b) return fail(GPE_ERR_INVALID_ARG, "null batch");
    if (n < 1) return fail(GPE_ERR_INVALID_ARG, "a captured run needs at least one step");
    if (!stream) return fail(GPE_ERR_INVALID_ARG, "capture needs a non-default stream");
    cudaStream_t s = (cudaStream_t)stream;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_steps = 0;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    const uint64_t launches = b->launches;
    gpe_status st = enqueue_steps(b, n, s, b->d_members, (uint32_t)b->members.size(), b->h_state, b->grid, true);
    b->launches = launches;
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    b->graph = g;
    b->graph_steps = n;
    return GPE_OK;
}

extern "C" gpe_status gpe_batch_replay(gpe_batch* b, void* stream) {
    if (!b) return fail(GPE_ERR_INVALID_ARG, "null batch");
    if (!b->exec) return fail(GPE_ERR_INVALID_ARG, "no captured run (gpe_batch_capture)");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaDeviceSynchronize();  // see gpe_batch_step
    if (e != cudaSuccess) return cuda_fail(e, "batch replay");
    if (gpe_status st = fill_state(b)) return st;
    e = cudaGraphLaunch(b->exec, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    const int32_t K = std::min(b->steps_per_launch > 0 ? b->steps_per_launch : b->graph_steps, kMaxStepsPerLaunch);
    b->launches += (uint64_t)((b->graph_steps + K - 1) / K) + convert_launch_count(b);
    advance_members(b, b->graph_steps);
    return check_batch_error(b, s);
}

extern "C" gpe_status gpe_batch_set_tuning(gpe_batch* b, int32_t key, int32_t value) {
    if (!b) return fail(GPE_ERR_INVALID_ARG, "null batch");
    if (key == GPE_BATCH_ITEM_NODES) {
        if (value < 1) return fail(GPE_ERR_INVALID_ARG, "item nodes");
        b->item_nodes = value;
        b->item_nodes_by_lattice.clear();
        return rebuild_items(b);
    }
    if (key == GPE_BATCH_STEPS_PER_LAUNCH) {
        if (value < 0) return fail(GPE_ERR_INVALID_ARG, "steps per launch");
        b->steps_per_launch = value;
        return GPE_OK;
    }
    if (key == GPE_BATCH_BARRIER_TIMEOUT_MS) {
        if (value < 1) return fail(GPE_ERR_INVALID_ARG, "barrier timeout");
        b->barrier_timeout_ms = value;
        return GPE_OK;
    }
    if (key == GPE_BATCH_TEST_EXTRA_ARRIVALS) {
        if (value < 0) return fail(GPE_ERR_INVALID_ARG, "extra arrivals");
        b->extra_arrivals = value;
        return GPE_OK;
    }
    if (key == GPE_BATCH_BLOCKS_PER_SM) {
        if (value < 0) return fail(GPE_ERR_INVALID_ARG, "blocks per SM");
        b->tune_blocks_per_sm = value;
        return grid_size(b);
    }
    if (key == GPE_BATCH_LAYOUT) {
        if (value < 0 || value > 1) return fail(GPE_ERR_INVALID_ARG, "batch layout (0 or 1)");
        if (value == b->layout) return GPE_OK;
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "batch layout");
        // a captured run holds the old layout's kernel and layout changes
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        b->graph_steps = 0;
        b->layout = value;
        if (gpe_status st = upload_members(b)) return st;
        return grid_size(b);
    }
    return fail(GPE_ERR_INVALID_ARG, "unknown batch tuning key");
}

extern "C" gpe_status gpe_batch_get_tuning(const gpe_batch* b, int32_t key, int32_t* value) {
    if (!b || !value) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (key == GPE_BATCH_ITEM_NODES) *value = b->item_nodes;
    else if (key == GPE_BATCH_STEPS_PER_LAUNCH) *value = b->steps_per_launch;
    else if (key == GPE_BATCH_BLOCKS_PER_SM) *value = b->grid / (b->sms ? b->sms : 1);
    else if (key == GPE_BATCH_BARRIER_TIMEOUT_MS) *value = b->barrier_timeout_ms;
    else if (key == GPE_BATCH_TEST_EXTRA_ARRIVALS) *value = b->extra_arrivals;
    else if (key == GPE_BATCH_LAYOUT) *value = b->layout;
    else return fail(GPE_ERR_INVALID_ARG, "unknown batch tuning key");
    return GPE_OK;
}

// Per lattice (node and entry counts), times `steps` batched steps of up to four of its
// members -- run on scratch copies of their psi buffers, so the members' states
// are untouched -- for each candidate item size and keeps the fastest.
extern "C" gpe_status gpe_batch_autotune(gpe_batch* b, int32_t steps, char* report, size_t report_len, void* stream) {
    if (!b) return fail(GPE_ERR_INVALID_ARG, "null batch");
    if (steps <= 0) steps = 4;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaDeviceSynchronize();  // see gpe_batch_step
    if (e != cudaSuccess) return cuda_fail(e, "batch autotune");
    std::vector<uint64_t> keys;
    for (const gpe_handle* h : b->members)
        if (std::find(keys.begin(), keys.end(), lattice_key(h)) == keys.end()) keys.push_back(lattice_key(h));
    std::sort(keys.begin(), keys.end());
    const int32_t cands[4] = {4096, 16384, 65536, 262144};
    uint64_t full_cost = 0;
    for (const gpe_handle* h : b->members) full_cost += (uint64_t)h->g.X * h->g.Y * h->g.Z * h->g.V * h->g.C;
    std::string rep = "[";
    std::vector<std::pair<uint64_t, int32_t>> best_by_lattice;
    if (gpe_status st = fill_state(b)) return st;
    for (uint64_t key : keys) {
        const uint32_t V = (uint32_t)(key >> 32);
        std::vector<uint32_t> which;
        for (uint32_t m = 0; m < b->members.size() && which.size() < 4; ++m)
            if (lattice_key(b->members[m]) == key) which.push_back(m);
        // scratch members: copies of the psi buffers, same tables and constants
        std::vector<BatchMember> hm(which.size());
        std::vector<BatchState> hs(which.size());
        std::vector<void*> scratch;
        bool ok = true;
        for (size_t i = 0; i < which.size() && ok; ++i) {
            const gpe_handle* h = b->members[which[i]];
            member_constants(h, hm[i]);
            if (!b->cslots.empty()) hm[i].cslot = b->cslots[which[i]];
            hs[i] = b->h_state[which[i]];
            const int deg = b->il_deg[which[i]];
            for (int slot = 0; slot < 2 && ok; ++slot) {
                void* p = nullptr;
                if (deg) {
                    // interleaved members: a zeroed scratch copy in that layout
                    if (cudaMalloc(&p, h->ilg.bytes) != cudaSuccess) {
                        ok = false;
                        break;
                    }
                    scratch.push_back(p);
                    cudaMemsetAsync(p, 0, h->ilg.bytes, s);
                    if (launch_il_convert(h->interior[slot], h->g, static_cast<char*>(p), h->ilg, true, s) != cudaSuccess) {
                        ok = false;
                        break;
                    }
                    hm[i].psi[slot] = static_cast<char*>(p);
                    continue;
                }
                if (cudaMalloc(&p, h->alloc_bytes[slot]) != cudaSuccess) {
                    ok = false;
                    break;
                }
                scratch.push_back(p);
                cudaMemcpyAsync(p, h->alloc[slot], h->alloc_bytes[slot], cudaMemcpyDeviceToDevice, s);
                hm[i].psi[slot] = static_cast<char*>(p) + (h->interior[slot] - static_cast<char*>(h->alloc[slot]));
            }
            hm[i].il_deg = deg;
            hm[i].il_off = deg ? static_cast<const int32_t*>(b->il_off[which[i]]) : nullptr;
        }
        BatchMember* dm = nullptr;
        BatchState* ps = nullptr;
        if (ok && (cudaMalloc(&dm, hm.size() * sizeof(BatchMember)) != cudaSuccess ||
                   cudaMallocHost(&ps, hs.size() * sizeof(BatchState)) != cudaSuccess))
            ok = false;
        if (ok) {
            cudaMemcpy(dm, hm.data(), hm.size() * sizeof(BatchMember), cudaMemcpyHostToDevice);
            std::memcpy(ps, hs.data(), hs.size() * sizeof(BatchState));
        }
        float best_ms = 1e30f;
        int32_t best = b->item_nodes;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int32_t c : cands) {
            if (!ok) break;
            // items of the scratch members (member indices local to the scratch list)
            std::vector<BatchItem> items;
            for (uint32_t i = 0; i < which.size(); ++i) {
                const Grid& g = hm[i].g;
                const uint64_t row_nodes = (uint64_t)g.X * g.V;
                const uint32_t rows_total = g.Y * g.Z;
                uint32_t per = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1, (uint64_t)c / row_nodes), rows_total);
                for (uint32_t r = 0; r < rows_total; r += per) items.push_back({i, r, std::min(per, rows_total - r), 0});
            }
            std::vector<const Grid*> grids(which.size());
            for (size_t i = 0; i < which.size(); ++i) grids[i] = &hm[i].g;
            if (upload_items(b, items, grids) != GPE_OK) {
                ok = false;
                break;
            }
            // as many blocks as give each the work a block has in the whole batch
            const double share = (double)b->item_cost.back() / (double)full_cost;
            const int tgrid = std::max(1, std::min(b->grid, (int)std::lround(share * b->grid)));
            if (enqueue_steps(b, 1, s, dm, (uint32_t)which.size(), ps, tgrid, false) != GPE_OK) {
                ok = false;
                break;
            }
            cudaEventRecord(e0, s);
            gpe_status st = enqueue_steps(b, steps, s, dm, (uint32_t)which.size(), ps, tgrid, false);
            cudaEventRecord(e1, s);
            if (st != GPE_OK || cudaEventSynchronize(e1) != cudaSuccess) {
                ok = false;
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            char line[128];
            std::snprintf(line, sizeof line,
                          "%s{\"nodes_per_cell\":%u,\"entries\":%u,\"item_nodes\":%d,\"ms_per_step\":%.5f}",
                          rep.size() > 1 ? "," : "", V, (uint32_t)key, c, ms / steps);
            rep += line;
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaStreamSynchronize(s);
        for (void* p : scratch) cudaFree(p);
        if (dm) cudaFree(dm);
        if (ps) cudaFreeHost(ps);
        if (!ok) {
            rebuild_items(b);
            return fail(GPE_ERR_CUDA, "batch autotune trial failed");
        }
        best_by_lattice.push_back({key, best});
    }
    rep += "]";
    b->item_nodes_by_lattice = best_by_lattice;
    gpe_status st = rebuild_items(b);
    if (st) return st;
    if (report && report_len) std::snprintf(report, report_len, "%s", rep.c_str());
    return check_batch_error(b, s);
}

extern "C" uint64_t gpe_batch_sites(const gpe_batch* b) {
    if (!b) return 0;
    uint64_t n = 0;
    for (const gpe_handle* h : b->members) n += (uint64_t)h->g.X * h->g.Y * h->g.Z * h->g.V;
    return n;
}

extern "C" uint64_t gpe_batch_launch_count(const gpe_batch* b) { return b ? b->launches : 0; }
