// gpe_il.cuh -- the cell-interleaved layout of FP32 states and its leapfrog step.
//
// Why this layout.  In the handle's own layout a node's record (C complex FP32
// values) follows the previous node's, so a warp of 32 consecutive nodes reads
// 32 records 8C bytes apart: each neighbour gather becomes two requests (16 + 8
// bytes for spin-1) whose lanes straddle several 128-byte lines, and the spin-1
// BCC step is bound by the L1 data stage (85 % busy) with DRAM at 57 %.  Here a
// warp takes one node l of 32 consecutive cells along x.  The lattice's stencil
// is the same in every cell, so node l's k-th neighbour in those cells is node l'
// of 32 consecutive cells shifted by (dx, dy, dz): with the layout of ILGrid
// (gpe_internal.h) every load and store of the step -- own record, old next
// record, the neighbours, the update -- is one contiguous 256-byte run per
// component, a single line pair per request.
//
// The handle's slots stay in the handle's layout; a multi-step call converts the
// two psi slots in (il_convert_kernel), steps in this layout and converts both
// back.  The arithmetic and its order are those of parabolic_node_t + node_finish,
// so the state after the steps is the one the gather kernels give.
#pragma once

namespace gpe {

__host__ __device__ inline size_t il_row(const ILGrid& G, uint32_t y, uint32_t z) {
    return ((size_t)(z + 1) * (G.Y + 2) + (y + 1)) * G.row;
}

// Handle layout <-> interleaved layout of the interior cells, one tile of KG
// consecutive groups' cells (TC = KG cells of a row, contiguous in the handle's
// layout) x JT complex values (j = l C + s) per pass, staged in shared memory (TC x
// (JT + 1) float2, the padding against bank conflicts) so that both sides are read
// and written in contiguous 16-byte runs.  KG is as many groups as keep a thread's
// share of a tile within kIlConvLoads 16-byte loads (for J = 36, spin-1 BCC, three
// groups of 32 cells: one group per pass left 2 loads per thread and ran at half
// the copy rate).  aos: the slot's interior pointer.  J = V C and JT are even (every
// lattice with 4 entries per node has an even node count), so a cell's values and
// the tiles start on 16-byte boundaries.  Each thread issues all its loads of a
// tile before it stores any of them.  The interleaved halo rows and padding cells
// are not touched.
constexpr uint32_t kIlConvThreads = 256;
constexpr uint32_t kIlConvLoads = 8;  // 16-byte loads per thread and tile: TC x JT <= 4096 values
template <bool TO_IL>
__global__ void __launch_bounds__(kIlConvThreads, 4) il_convert_kernel(char* aos, Grid g, char* il, ILGrid G, uint32_t JT,
                                                                    uint32_t KG, uint32_t GXT, uint32_t jtiles,
                                                                    uint32_t tiles, FastDiv djt, FastDiv dgx,
                                                                    FastDiv dy) {
    extern __shared__ float2 il_tile[];  // TC x (JT + 1)
    const uint32_t J = G.V * G.C;
    const uint32_t cells = G.cells;
    const uint32_t TC = KG * cells, htc = TC / 2;
    const uint32_t ld = JT + 1;
    for (uint32_t w = blockIdx.x; w < tiles; w += gridDim.x) {
        const uint32_t r1 = fdiv(w, djt);
        const uint32_t jt = w - r1 * jtiles;
        const uint32_t r2 = fdiv(r1, dgx);
        const uint32_t gxt = r1 - r2 * GXT;
        const uint32_t z = fdiv(r2, dy);
        const uint32_t y = r2 - z * G.Y;
        const uint32_t j0 = jt * JT;
        const uint32_t nj = min(JT, J - j0);   // even
        const uint32_t x0 = gxt * TC;
        const uint32_t nc = min(TC, G.X - x0);
        const uint32_t half = nj / 2;          // 16-byte runs per cell of the tile
        char* arow = aos + (size_t)z * g.slice + (size_t)y * g.pitch + (size_t)x0 * g.cell_bytes + (size_t)j0 * 8;
        // cell c of the tile: group gxt KG + c / cells, cell c % cells of it
        char* irow = il + il_row(G, y, z) + (size_t)gxt * KG * G.gb + (size_t)j0 * cells * 8;
        float4 buf[kIlConvLoads];
        if (TO_IL) {
            // cell-major 16-byte runs of the handle's layout
            const uint32_t n4 = nc * half;
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                if (i < n4) {
                    const uint32_t c = i / half, q = i - c * half;
                    buf[k] = __ldg(reinterpret_cast<const float4*>(arow + (size_t)c * g.cell_bytes + (size_t)q * 16));
                }
            }
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                if (i < n4) {
                    const uint32_t c = i / half, q = i - c * half;
                    il_tile[c * ld + 2 * q] = make_float2(buf[k].x, buf[k].y);
                    il_tile[c * ld + 2 * q + 1] = make_float2(buf[k].z, buf[k].w);
                }
            }
            __syncthreads();
            // value-major pairs of cells of the interleaved layout
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                const uint32_t jj = i / htc, c = 2 * (i % htc);
                if (jj < nj && c < nc) {
                    const uint32_t gl = c / cells, cl = c - gl * cells;
                    const float2 a = il_tile[c * ld + jj];
                    char* dst = irow + (size_t)gl * G.gb + ((size_t)jj * cells + cl) * 8;
                    if (c + 1 < nc) {
                        const float2 b = il_tile[(c + 1) * ld + jj];
                        *reinterpret_cast<float4*>(dst) = make_float4(a.x, a.y, b.x, b.y);
                    } else {
                        *reinterpret_cast<float2*>(dst) = a;
                    }
                }
            }
        } else {
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                const uint32_t jj = i / htc, c = 2 * (i % htc);
                if (jj < nj && c < nc) {
                    const uint32_t gl = c / cells, cl = c - gl * cells;
                    buf[k] = __ldg(reinterpret_cast<const float4*>(irow + (size_t)gl * G.gb + ((size_t)jj * cells + cl) * 8));
                }
            }
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                const uint32_t jj = i / htc, c = 2 * (i % htc);
                if (jj < nj && c < nc) {
                    il_tile[c * ld + jj] = make_float2(buf[k].x, buf[k].y);
                    if (c + 1 < nc) il_tile[(c + 1) * ld + jj] = make_float2(buf[k].z, buf[k].w);
                }
            }
            __syncthreads();
            const uint32_t n4 = nc * half;
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                if (i < n4) {
                    const uint32_t c = i / half, q = i - c * half;
                    const float2 a = il_tile[c * ld + 2 * q], b = il_tile[c * ld + 2 * q + 1];
                    *reinterpret_cast<float4*>(arow + (size_t)c * g.cell_bytes + (size_t)q * 16) = make_float4(a.x, a.y, b.x, b.y);
                }
            }
        }
        __syncthreads();
    }
}

// Node l's stencil in the interleaved layout, for cell `sub` of a group (the
// lane's cell in its group): neighbour k is node e.w of the cells shifted by (dx,
// dy, dz), a fixed offset from the group base: the rows (dz, dy), the node, and
// sub + dx within the group or (first / last cell) the last / first cell of the
// group before / after it.  The offset is a multiple of 8, so its two low bits carry dx
// + 1 (|dx| <= 1, checked on the host) for the halo test of cells x + dx outside
// [0, X).  ent / wt: the node's table entries and weights; nd (4, or 4 or 8 for
// D = 8) of them.
template <int D, int CELLS>
__device__ __forceinline__ void il_node_stencil(const ILGrid& G, const int4* ent, const float* wt, int nd, uint32_t sub,
                                                int32_t* off, float* w) {
    const uint32_t node_run = G.C * CELLS * 8;   // bytes between nodes of a group
#pragma unroll
    for (int k = 0; k < D; ++k) {
        off[k] = 1;
        w[k] = 0.f;
        if (k < nd) {
            const int4 e = ent[k];
            const int xl = (int)sub + e.x;                        // -1 .. CELLS
            const int64_t gshift = xl < 0 ? -1 : (xl >= CELLS ? 1 : 0);
            const int64_t cell = xl - gshift * (int64_t)CELLS;
            off[k] = (int32_t)(((int64_t)e.z * (G.Y + 2) + e.y) * (int64_t)G.row + (int64_t)e.w * node_run +
                               gshift * (int64_t)G.gb + cell * 8) |
                     (e.x + 1);
            w[k] = wt[k];
        }
    }
}

// The group a lane works on in warp task u: the q-th group of the rows row0 ..
// (q = u 32 / CELLS + the lane's group within its warp, counted row after row),
// as (gx, y, z); false past the last group (nq groups).
template <int CELLS>
__device__ __forceinline__ bool il_lane_group(const ILGrid& G, uint32_t u, uint32_t nq, uint32_t row0, FastDiv dGX,
                                              FastDiv dY, uint32_t& gx, uint32_t& y, uint32_t& z) {
    const uint32_t q = (32 / CELLS) * u + (threadIdx.x & 31) / CELLS;
    if (q >= nq) return false;
    const uint32_t r = fdiv(q, dGX);
    gx = q - r * G.GX;
    const uint32_t row = row0 + r;
    z = fdiv(row, dY);
    y = row - z * G.Y;
    return true;
}

// One lane's node of an interleaved leapfrog step: node l of cell gx CELLS + sub
// of row (y, z), next <- next + 2 dt (-i H prev), with the arithmetic and its order of
// parabolic_node_t + node_finish.  F: where the step's fields come from (P if
// null); oa: where the observables of prev go.
template <int C, int D, int CELLS, class OA>
__device__ __forceinline__ void il_task(const ILGrid& G, const PhysR<float>& P, const PhysR<float>* F, const char* prev,
                                        char* next, const int32_t* off, const float* w, int nd, const float* pos,
                                        uint32_t sub, uint32_t l, uint32_t gx, uint32_t y, uint32_t z, OA* oa) {
    constexpr uint32_t kComp = CELLS * 8;   // bytes between a record's components
    const uint32_t x = gx * CELLS + sub;
    if (x >= G.X) return;
    const size_t gbase = il_row(G, y, z) + (size_t)gx * G.gb;
    const size_t own = gbase + (size_t)l * (G.C * kComp) + (size_t)sub * 8;
    Cx<float> prv[C], nv[C], H[C];
#pragma unroll
    for (int s = 0; s < C; ++s) {
        prv[s] = ldc<float>(prev + own + s * kComp);
        nv[s] = ldc_rw<float>(next + own + s * kComp);
    }
#pragma unroll
    for (int s = 0; s < C; ++s) H[s] = cx<float>(0.f, 0.f);
    // DEC Laplacian, sum_f w_f (psi_nb - psi) in entry order (Spin1GpeBCC.cu:835-865),
    // the loads of a group of 4 entries issued together; cells x + dx outside
    // [0, X) are the zero halo
#pragma unroll
    for (int k0 = 0; k0 < D; k0 += 4) {
        if (k0 >= nd) break;
        Cx<float> v[4][C];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int32_t o = off[k0 + k];
            const bool in = (unsigned)((int)x + (o & 3) - 1) < G.X;
            const char* p = prev + gbase + (in ? (o & ~3) : 0);
#pragma unroll
            for (int s = 0; s < C; ++s) v[k][s] = in ? ldc<float>(p + s * kComp) : cx<float>(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
            for (int s = 0; s < C; ++s) H[s] += w[k0 + k] * (v[k][s] - prv[s]);
        }
    }
    // local terms and the leapfrog update, as node_finish
    float rr[3];
    rr[0] = P.p0[0] + P.bs * ((float)x * P.bw[0] + pos[0]);
    rr[1] = P.p0[1] + P.bs * ((float)y * P.bw[1] + pos[1]);
    rr[2] = P.p0[2] + P.bs * ((float)z * P.bw[2] + pos[2]);
    const float pot = trap<float>(P, rr, F);
    local_terms<float, C>(P, rr, pot, GPE_MODE_LEAPFROG, false, prv, H, F);
    if constexpr (!std::is_same<OA, NoObs>::value) oa->template node<float, C>(P, rr, prv, H);
#pragma unroll
    for (int s = 0; s < C; ++s) {
        nv[s] += (2.f * P.dt) * cx<float>(H[s].y, -H[s].x);
        stc<float>(next + own + s * kComp, nv[s]);
    }
}

// Warp tasks per node of an interleaved step (the grid's groups counted row after
// row, 32 / cells per warp task).
__host__ __device__ inline uint32_t il_warp_tasks(const ILGrid& G) {
    const uint32_t wg = 32 / G.cells;
    return (G.Y * G.Z * G.GX + wg - 1) / wg;
}

// One FP32 leapfrog step in the interleaved layout: next <- next + 2 dt (-i H prev).
// D = 4: every node has 4 stencil entries (BCC, A15, C15, Z); D = 8: rows of 4 or 8
// entries (FCC's tetrahedra and octahedra).  Warp task t = u V + l: node l of the
// u-th group (il_lane_group).  The grid's warp count is a multiple
// of V, so a warp keeps its node, and with it its entries and position, in
// registers; the row length is the same in every lane of a warp, so the second
// group of 4 entries is a uniform branch.  OBS: the observables of prev are summed
// on the way (ObsAcc, as the gather kernels' observed step).
template <int C, int D, int CELLS, bool OBS>
__device__ __forceinline__ void il_step_body(const StepArgs& a, const ILGrid& G, uint32_t tasks, FastDiv dGX) {
    static_assert(D == 4 || D == 8, "rows of 4, or of 4 and 8 entries");
    const PhysR<float>& P = make_phys<float>(a);
    using OA = typename ObsOf<OBS, float>::type;
    __shared__ double obs_sums[OBS ? kObsSums * 256 : 1];
    OA oa = ObsOf<OBS, float>::make(obs_sums);
    const uint32_t sub = threadIdx.x & (CELLS - 1);
    const uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t l = warp - fdiv(warp, a.divV) * G.V;
    const uint32_t nq = G.Y * G.Z * G.GX;
    // the warp's node's table, read once from global memory (no shared tables: the
    // block then needs no shared memory, which left the plain kernel at 7 blocks per
    // SM); weights h / bs^2 of the step's block scale, as load_tables scales them
    const int f0 = a.tab.row_ptr[l];
    const int nd = D == 4 ? 4 : a.tab.row_ptr[l + 1] - f0;   // 4 or 8, the same in the whole warp
    float wt[D];
#pragma unroll
    for (int k = 0; k < D; ++k) wt[k] = k < nd ? a.tab.w32[f0 + k] * P.ks : 0.f;
    int32_t off[D];
    float w[D];
    il_node_stencil<D, CELLS>(G, a.tab.ent4 + f0, wt, nd, sub, off, w);
    const float pos[3] = {a.tab.pos32[3 * l], a.tab.pos32[3 * l + 1], a.tab.pos32[3 * l + 2]};
    for (uint32_t t = warp; t < tasks; t += nwarps) {
        const uint32_t u = fdiv(t, a.divV);
        uint32_t gx, y, z;
        if (il_lane_group<CELLS>(G, u, nq, 0, dGX, a.divY, gx, y, z))
            il_task<C, D, CELLS, OA>(G, P, nullptr, a.prev, a.next, off, w, nd, pos, sub, l, gx, y, z, &oa);
    }
    if constexpr (OBS) {
        __shared__ double red[8][OBS_COUNT];
        oa.block_reduce(red, a.partials);
    }
}

// Launch shapes: the plain step in blocks of kIlPlainThreads with at least
// IlBounds<C>::kMin of them per SM (the register cap that keeps the most warps in
// flight without spills), the observed step in blocks of 256 (its FP64 sums take
// shared memory per thread).
constexpr unsigned kIlPlainThreads = 128;
constexpr unsigned kIlObsThreads = 256;
template <int C, int D>
struct IlBounds {
    // D = 4: spin-1 BCC 96^3 (the cap 7 blocks lets it use 64 registers, 8 blocks):
    // 0.130 ms per step; capped at 72 registers before the offsets carried dx, 7
    // blocks 0.131, 8 (64) 0.147, 9 (56) 0.145; spin-2 BCC 96^3: 4 blocks (105)
    // 0.222 ms, 5 (96) 0.211, 6 (80) 0.218.  D = 8 keeps 12 more registers for the
    // second group of entries (FCC 96^3, fraction of the copy peak): spin-1 at 5
    // blocks (95 registers) 0.58, at 6 (80, 16 bytes of spills) 0.58, at 4 0.52;
    // spin-2 at 4 blocks (128) 0.58, at 3 0.52, at 5 0.49.
    static constexpr int kMin = D == 8 ? (C == 5 ? 4 : (C == 3 ? 5 : 8)) : (C == 5 ? 5 : (C == 3 ? 7 : 8));
    static constexpr int kMinObs = (C == 5 || (C == 3 && D == 8)) ? 2 : 3;
};

template <int C, int D, int CELLS>
__global__ void __launch_bounds__(kIlPlainThreads, IlBounds<C, D>::kMin) il_step_kernel(StepArgs a, ILGrid G, uint32_t tasks,
                                                                                    FastDiv dGX) {
    il_step_body<C, D, CELLS, false>(a, G, tasks, dGX);
}
template <int C, int D, int CELLS>
__global__ void __launch_bounds__(kIlObsThreads, IlBounds<C, D>::kMinObs) il_step_obs_kernel(StepArgs a, ILGrid G,
                                                                                        uint32_t tasks, FastDiv dGX) {
    il_step_body<C, D, CELLS, true>(a, G, tasks, dGX);
}

// Blocks of one interleaved step (rows of D entries at most): one wave at the
// kernel's occupancy or one warp per task if that is fewer, as a multiple of m =
// V / gcd(V, warps per block) (the grid's warp count a multiple of V), and at most
// `max_blocks` (the handle's partial-sum rows); 0 if no such grid.
template <int C, int D, int CELLS>
unsigned il_blocks_d(const ILGrid& G, bool obs, size_t max_blocks) {
    static int occ[2] = {0, 0};
    const unsigned threads = obs ? kIlObsThreads : kIlPlainThreads;
    const unsigned wpb = threads / 32;
    int& o = occ[obs ? 1 : 0];
    if (o == 0) {
        auto k = obs ? il_step_obs_kernel<C, D, CELLS> : il_step_kernel<C, D, CELLS>;
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, obs ? 50 : 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, (int)threads, 0);
        if (o < 1) o = 1;
    }
    uint32_t gv = G.V, gb = wpb;
    while (gb) {
        const uint32_t r = gv % gb;
        gv = gb;
        gb = r;
    }
    const uint64_t m = G.V / gv;
    const uint64_t tasks = (uint64_t)il_warp_tasks(G) * G.V;
    uint64_t nb = std::min<uint64_t>((uint64_t)o * (unsigned)device_sm_count(), (tasks + wpb - 1) / wpb);
    // rounded down (a block past the wave would start only when another ends);
    // grids of fewer tasks than m blocks' warps take m blocks, some warps idle
    nb = nb >= m ? nb / m * m : m;
    if (nb > max_blocks) nb = max_blocks / m * m;
    return (unsigned)nb;
}

template <int C>
unsigned il_blocks(const ILGrid& G, int deg, bool obs, size_t max_blocks) {
    if (G.cells == 32)
        return deg == 4 ? il_blocks_d<C, 4, 32>(G, obs, max_blocks) : il_blocks_d<C, 8, 32>(G, obs, max_blocks);
    return deg == 4 ? il_blocks_d<C, 4, 16>(G, obs, max_blocks) : il_blocks_d<C, 8, 16>(G, obs, max_blocks);
}

// One interleaved leapfrog step (a.prev / a.next: interleaved buffers) on rows of
// at most deg (4 or 8) entries; obs: sum the observables of a.prev into a.partials
// and finalize them into out.
template <int C, int D, int CELLS>
cudaError_t launch_il_step_d(const StepArgs& a, const ILGrid& G, size_t max_blocks, bool obs, double* out, cudaStream_t s) {
    const unsigned nb = il_blocks_d<C, D, CELLS>(G, obs, max_blocks);
    if (nb == 0) return cudaErrorInvalidConfiguration;
    const uint32_t tasks = il_warp_tasks(G) * G.V;
    const FastDiv dGX = make_fastdiv(G.GX);
    if (obs) {
        il_step_obs_kernel<C, D, CELLS><<<nb, kIlObsThreads, 0, s>>>(a, G, tasks, dGX);
        observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    } else {
        il_step_kernel<C, D, CELLS><<<nb, kIlPlainThreads, 0, s>>>(a, G, tasks, dGX);
    }
    return cudaGetLastError();
}

template <int C>
cudaError_t launch_il_step(const StepArgs& a, const ILGrid& G, int deg, size_t max_blocks, bool obs, double* out,
                           cudaStream_t s) {
    if (G.cells == 32) {
        if (deg == 4) return launch_il_step_d<C, 4, 32>(a, G, max_blocks, obs, out, s);
        if (deg == 8) return launch_il_step_d<C, 8, 32>(a, G, max_blocks, obs, out, s);
    } else if (G.cells == 16) {
        if (deg == 4) return launch_il_step_d<C, 4, 16>(a, G, max_blocks, obs, out, s);
        if (deg == 8) return launch_il_step_d<C, 8, 16>(a, G, max_blocks, obs, out, s);
    }
    return cudaErrorInvalidValue;
}

#define GPE_INSTANTIATE_IL(C)                                                                                           \
    template cudaError_t launch_il_step<C>(const StepArgs&, const ILGrid&, int, size_t, bool, double*, cudaStream_t); \
    template unsigned il_blocks<C>(const ILGrid&, int, bool, size_t);                                                 \
    template cudaError_t launch_il_hyper<C>(const StepArgs&, const ILGrid&, const ILGrid&, const int32_t*, cudaStream_t);

// ---------------------------------------------- hyperbolic (psi + q) leapfrog

// The fused hyperbolic leapfrog step (update_psi + update_q of
// RelativisticSpin2Gpe.cu:1873-1874, both reading the previous (psi, q)) in the
// interleaved layout: psi in G (V nodes per cell), q in Gq (the E = 2V edges of a
// cell in place of the nodes).  A warp keeps node j and edges 2j, 2j + 1 for the
// whole launch (the grid's warp count is a multiple of V): warp task t = u V + j
// updates node j of the u-th group from its 4 incident edges (d1 q,
// RelativisticSpin2Gpe.cu:1051-1066), then its two edges from their nodes (d0 psi,
// :986-1019).  Every warp does the same work, so the warps that read a group's psi
// and q lines stay together (a warp per node or edge let the edge warps run ahead
// of the node warps, and spin-2 then read 48 % more from DRAM than the algorithmic
// bytes).  tab: the handle's interleaved offset tables (il_hyper_tables: V*4
// incidences relative to the q group base, E to-nodes relative to the psi group
// base, both with dx + 1 in the two low bits, and E from-nodes).  The arithmetic
// and its order are hyper_step_kernel's (fused leapfrog), so the states are its
// states bit for bit.
template <int C, int CELLS>
__device__ __forceinline__ void il_hyper_body(const StepArgs& a, const ILGrid& G, const ILGrid& Gq, const int32_t* tab,
                                              uint32_t tasks, FastDiv dGX) {
    const uint32_t V = G.V, E = Gq.V;
    const uint32_t sub = threadIdx.x & (CELLS - 1);
    const uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t j = warp - fdiv(warp, a.divV) * V;
    const PhysR<float>& P = make_phys<float>(a);
    constexpr uint32_t kComp = CELLS * 8;
    const uint32_t nq = G.Y * G.Z * G.GX;
    // this lane's offsets (cell sub + dx, stepping into the next / previous group
    // where it leaves this one): the node's 4 incidences in q, its edges' to-nodes
    // in psi; the edges' from-nodes; the node's weights and position
    auto lane_off = [&](int32_t b, int32_t wrap) {
        const int xl = (int)sub + (b & 3) - 1;
        const int32_t gs = xl < 0 ? -1 : (xl >= CELLS ? 1 : 0);
        return ((b & ~3) + (int32_t)sub * 8 + gs * wrap) | (b & 3);
    };
    int32_t off[4], eto[2], efrom[2];
    float w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        off[k] = lane_off(tab[4 * j + k], (int32_t)Gq.gb - (int32_t)kComp);
        w[k] = a.tab.inc_w32[4 * j + k];
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        eto[r] = lane_off(tab[4 * V + 2 * j + r], (int32_t)G.gb - (int32_t)kComp);
        efrom[r] = tab[4 * V + E + 2 * j + r] + (int32_t)sub * 8;
    }
    const float pos[3] = {a.tab.pos32[3 * j], a.tab.pos32[3 * j + 1], a.tab.pos32[3 * j + 2]};
    const float dts = P.dts;
    for (uint32_t t = warp; t < tasks; t += nwarps) {
        const uint32_t u = fdiv(t, a.divV);
        uint32_t gx, y, z;
        if (!il_lane_group<CELLS>(G, u, nq, 0, dGX, a.divY, gx, y, z)) continue;
        const uint32_t x = gx * CELLS + sub;
        if (x >= G.X) continue;
        const size_t gbase = il_row(G, y, z) + (size_t)gx * G.gb;
        const size_t qbase = il_row(Gq, y, z) + (size_t)gx * Gq.gb;
        {
            // node j
            const size_t own = gbase + (size_t)j * (C * kComp) + (size_t)sub * 8;
            Cx<float> prv[C], H[C], nv[C];
#pragma unroll
            for (int s = 0; s < C; ++s) {
                prv[s] = ldc<float>(a.prev + own + s * kComp);
                nv[s] = ldc_rw<float>(a.next + own + s * kComp);   // in flight with the q loads
            }
#pragma unroll
            for (int s = 0; s < C; ++s) H[s] = cx<float>(0.f, 0.f);
            Cx<float> qv[4][C];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int32_t o = off[k];
                const bool in = (unsigned)((int)x + (o & 3) - 1) < G.X;
                const char* p = a.q + qbase + (in ? (o & ~3) : 0);
#pragma unroll
                for (int s = 0; s < C; ++s) qv[k][s] = in ? ldc<float>(p + s * kComp) : cx<float>(0.f, 0.f);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
#pragma unroll
                for (int s = 0; s < C; ++s) H[s] += w[k] * qv[k][s];
            }
            float r[3];
            r[0] = P.p0[0] + P.bs * ((float)x * P.bw[0] + pos[0]);
            r[1] = P.p0[1] + P.bs * ((float)y * P.bw[1] + pos[1]);
            r[2] = P.p0[2] + P.bs * ((float)z * P.bw[2] + pos[2]);
            const float pot = trap<float>(P, r);
            if constexpr (C == 1) {
                local_scalar<float>(P, pot, false, true, prv, H);
            } else if constexpr (C == 3) {
                local_spin1<float>(P, r, pot, true, false, true, prv, H);
            } else {
                local_spin2<float>(P, r, pot, true, false, true, prv, H);
            }
            // the leapfrog update, as write_update
#pragma unroll
            for (int s = 0; s < C; ++s) {
                nv[s] += (2.f * P.dt) * cx<float>(H[s].y, -H[s].x);
                stc<float>(a.next + own + s * kComp, nv[s]);
            }
        }
#pragma unroll 1
        for (int e = 0; e < 2; ++e) {
            // edge 2j + e: q_update, hyperbolic leapfrog: next_q += i 2 (dt/sigma)(prev_q + d0 psi)
            const size_t own = qbase + (size_t)(2 * j + e) * (C * kComp) + (size_t)sub * 8;
            Cx<float> to[C], fr[C], pq[C], v[C];
            const int32_t o = eto[e];
            const bool in = (unsigned)((int)x + (o & 3) - 1) < G.X;
            const char* pt = a.prev + gbase + (in ? (o & ~3) : 0);
#pragma unroll
            for (int s = 0; s < C; ++s) {
                to[s] = in ? ldc<float>(pt + s * kComp) : cx<float>(0.f, 0.f);
                fr[s] = ldc<float>(a.prev + gbase + efrom[e] + s * kComp);
                pq[s] = ldc<float>(a.q + own + s * kComp);
                v[s] = ldc_rw<float>(a.qnext + own + s * kComp);
            }
#pragma unroll
            for (int s = 0; s < C; ++s) {
                const Cx<float> d0psi = to[s] - fr[s];
                const Cx<float> qq = (2.f * dts) * (pq[s] + d0psi);
                v[s] += cx<float>(-qq.y, qq.x);
                stc<float>(a.qnext + own + s * kComp, v[s]);
            }
        }
    }
}

// Register caps: spin-2 at 5 blocks of 128 threads (96 registers, no spills),
// spin-1 at 6 (80 registers).  Measured against 6 blocks (80 registers) for
// spin-2: BCC 96^3 0.98 / 1.03, C15 48^3 0.93 / 0.97, but C15 128^3 (285 M sites)
// 0.87 / 0.73 of peak; spin-1 at 8 blocks (64 registers) within 1 %.
template <int C>
struct IlHyperBounds {
    static constexpr int kMin = C == 5 ? 5 : (C == 3 ? 6 : 8);
};

template <int C, int CELLS>
__global__ void __launch_bounds__(kIlPlainThreads, IlHyperBounds<C>::kMin)
    il_hyper_kernel(StepArgs a, ILGrid G, ILGrid Gq, const int32_t* tab, uint32_t tasks, FastDiv dGX) {
    il_hyper_body<C, CELLS>(a, G, Gq, tab, tasks, dGX);
}

template <int C, int CELLS>
unsigned il_hyper_blocks_c(const ILGrid& G, const ILGrid& Gq) {
    static int occ = 0;
    const unsigned wpb = kIlPlainThreads / 32;
    if (occ == 0) {
        cudaFuncSetAttribute(il_hyper_kernel<C, CELLS>, cudaFuncAttributePreferredSharedMemoryCarveout, 25);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, il_hyper_kernel<C, CELLS>, (int)kIlPlainThreads, 0);
        if (occ < 1) occ = 1;
    }
    const uint32_t items = G.V;
    uint32_t gv = items, gb = wpb;
    while (gb) {
        const uint32_t r = gv % gb;
        gv = gb;
        gb = r;
    }
    const uint64_t m = items / gv;
    const uint64_t tasks = (uint64_t)il_warp_tasks(G) * items;
    uint64_t nb = std::min<uint64_t>((uint64_t)occ * (unsigned)device_sm_count(), (tasks + wpb - 1) / wpb);
    nb = nb >= m ? nb / m * m : m;
    return (unsigned)nb;
}

// One fused hyperbolic leapfrog step in the interleaved layout (a.prev / a.next /
// a.q / a.qnext: interleaved buffers).
template <int C>
cudaError_t launch_il_hyper(const StepArgs& a, const ILGrid& G, const ILGrid& Gq, const int32_t* tab, cudaStream_t s) {
    const uint64_t tasks64 = (uint64_t)il_warp_tasks(G) * G.V;
    if (tasks64 > 0xffffffffu || G.cells != Gq.cells || G.GX != Gq.GX || Gq.V != 2 * G.V) return cudaErrorInvalidValue;
    const uint32_t tasks = (uint32_t)tasks64;
    const FastDiv dGX = make_fastdiv(G.GX);
    if (G.cells == 32) {
        const unsigned nb = il_hyper_blocks_c<C, 32>(G, Gq);
        il_hyper_kernel<C, 32><<<nb, kIlPlainThreads, 0, s>>>(a, G, Gq, tab, tasks, dGX);
    } else {
        const unsigned nb = il_hyper_blocks_c<C, 16>(G, Gq);
        il_hyper_kernel<C, 16><<<nb, kIlPlainThreads, 0, s>>>(a, G, Gq, tab, tasks, dGX);
    }
    return cudaGetLastError();
}

// Both directions of the layout change for one state buffer (interior pointer aos).
// Defined once (GPE_DEFINE_IL_CONVERT in one translation unit).
cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s);

#define GPE_DEFINE_IL_CONVERT                                                                                        \
    cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s) { \
        const uint32_t J = G.V * G.C;                                                                                \
        if (J % 2 || g.cell_bytes != J * 8) return cudaErrorInvalidValue;                                            \
        const uint32_t JT = J < 128 ? J : 128;                                                                       \
        const uint32_t jtiles = (J + JT - 1) / JT;                                                                   \
        /* groups per tile: TC JT <= 2 kIlConvLoads kIlConvThreads values, TC <= 1024 cells */                       \
        uint32_t KG = std::min<uint32_t>(2 * kIlConvLoads * kIlConvThreads / (G.cells * JT), 1024 / G.cells);      \
        KG = std::max<uint32_t>(1, std::min<uint32_t>(KG, G.GX));                                                   \
        const uint32_t GXT = (G.GX + KG - 1) / KG;                                                                   \
        const uint64_t tiles = (uint64_t)G.Y * G.Z * GXT * jtiles;                                                   \
        if (tiles == 0) return cudaSuccess;                                                                          \
        if (tiles > 0xffffffffu) return cudaErrorInvalidValue;                                                       \
        const size_t smem = (size_t)KG * G.cells * (JT + 1) * sizeof(float2);                                        \
        const unsigned nb = (unsigned)std::min<uint64_t>(tiles, (uint64_t)device_sm_count() * 8);                    \
        const FastDiv djt = make_fastdiv(jtiles), dgx = make_fastdiv(GXT), dy = make_fastdiv(G.Y);                   \
        if (to_il)                                                                                                   \
            il_convert_kernel<true><<<nb, kIlConvThreads, smem, s>>>(aos, g, il, G, JT, KG, GXT, jtiles, (uint32_t)tiles, \
                                                                     djt, dgx, dy);                                  \
        else                                                                                                         \
            il_convert_kernel<false><<<nb, kIlConvThreads, smem, s>>>(aos, g, il, G, JT, KG, GXT, jtiles,            \
                                                                      (uint32_t)tiles, djt, dgx, dy);                \
        return cudaGetLastError();                                                                                   \
    }

}  // namespace gpe
