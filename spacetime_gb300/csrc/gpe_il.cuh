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
// record, the four neighbours, the update -- is one contiguous 256-byte run per
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

// Handle layout <-> interleaved layout of the interior cells, one tile of 32
// cells x JT complex values (j = l C + s) per pass, staged in shared memory so
// that both sides are read and written in contiguous runs.  aos: the slot's
// interior pointer.  The interleaved halo rows and padding cells are not touched.
template <bool TO_IL>
__global__ void __launch_bounds__(256) il_convert_kernel(char* aos, Grid g, char* il, ILGrid G, uint32_t JT,
                                                         uint32_t jtiles, uint32_t tiles) {
    extern __shared__ float2 il_tile[];  // 32 x (JT + 1)
    const uint32_t J = G.V * G.C;
    const uint32_t ld = JT + 1;
    for (uint32_t w = blockIdx.x; w < tiles; w += gridDim.x) {
        uint32_t r = w;
        const uint32_t jt = r % jtiles;
        r /= jtiles;
        const uint32_t gx = r % G.GX;
        r /= G.GX;
        const uint32_t y = r % G.Y, z = r / G.Y;
        const uint32_t j0 = jt * JT;
        const uint32_t nj = min(JT, J - j0);
        const uint32_t nc = min(kIlCells, G.X - gx * kIlCells);
        char* arow = aos + (size_t)z * g.slice + (size_t)y * g.pitch + (size_t)gx * kIlCells * g.cell_bytes + (size_t)j0 * 8;
        char* irow = il + il_row(G, y, z) + (size_t)gx * G.gb + (size_t)j0 * kIlCells * 8;
        if (TO_IL) {
            for (uint32_t i = threadIdx.x; i < nc * nj; i += blockDim.x) {
                const uint32_t c = i / nj, jj = i - c * nj;
                il_tile[c * ld + jj] = *reinterpret_cast<const float2*>(arow + (size_t)c * g.cell_bytes + (size_t)jj * 8);
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < nj * kIlCells; i += blockDim.x) {
                const uint32_t jj = i / kIlCells, c = i % kIlCells;
                if (c < nc) *reinterpret_cast<float2*>(irow + (size_t)i * 8) = il_tile[c * ld + jj];
            }
        } else {
            for (uint32_t i = threadIdx.x; i < nj * kIlCells; i += blockDim.x) {
                const uint32_t jj = i / kIlCells, c = i % kIlCells;
                if (c < nc) il_tile[c * ld + jj] = *reinterpret_cast<const float2*>(irow + (size_t)i * 8);
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < nc * nj; i += blockDim.x) {
                const uint32_t c = i / nj, jj = i - c * nj;
                *reinterpret_cast<float2*>(arow + (size_t)c * g.cell_bytes + (size_t)jj * 8) = il_tile[c * ld + jj];
            }
        }
        __syncthreads();
    }
}

// One FP32 leapfrog step in the interleaved layout, lattices whose nodes all have
// 4 stencil entries (BCC, A15, C15, Z): next <- next + 2 dt (-i H prev).  Warp
// task t = ((z Y + y) GX + gx) V + l: node l of the cells gx*32 + lane of row
// (y, z).  The grid's warp count is a multiple of V, so a warp keeps its node, and
// with it its 4 entries and position, in registers.  OBS: the observables of prev
// are summed on the way (ObsAcc, as the gather kernels' observed step).
template <int C, bool OBS>
__device__ __forceinline__ void il_step_body(const StepArgs& a, const ILGrid& G, uint32_t tasks, FastDiv dGX) {
    __shared__ SmemTables<float> st;
    load_tables<float>(st, a);
    __syncthreads();
    const PhysR<float>& P = make_phys<float>(a);
    using OA = typename ObsOf<OBS, float>::type;
    __shared__ double obs_sums[OBS ? kObsSums * 256 : 1];
    OA oa = ObsOf<OBS, float>::make(obs_sums);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t l = warp - fdiv(warp, a.divV) * G.V;
    constexpr uint32_t kComp = kIlCells * 8;   // bytes between a record's components
    const uint32_t node_run = G.C * kComp;     // bytes between nodes of a group
    int dx[4];
    int32_t off[4];  // row and node part of each neighbour's address
    float w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int4 e = a.tab.ent4[l * 4 + k];
        dx[k] = e.x;
        off[k] = (int32_t)(((int64_t)e.z * (G.Y + 2) + e.y) * (int64_t)G.row + (int64_t)e.w * node_run);
        w[k] = st.w[l * 4 + k];
    }
    const float pos[3] = {st.pos[3 * l], st.pos[3 * l + 1], st.pos[3 * l + 2]};
    const char* prev = a.prev;
    char* next = a.next;
    for (uint32_t t = warp; t < tasks; t += nwarps) {
        const uint32_t r = fdiv(t, a.divV);
        const uint32_t row = fdiv(r, dGX);
        const uint32_t gx = r - row * G.GX;
        const uint32_t z = fdiv(row, a.divY);
        const uint32_t y = row - z * G.Y;
        const uint32_t x = gx * kIlCells + lane;
        if (x >= G.X) continue;
        const size_t rb = il_row(G, y, z);
        const size_t own = rb + (size_t)gx * G.gb + (size_t)l * node_run + (size_t)lane * 8;
        Cx<float> prv[C], nv[C], H[C];
#pragma unroll
        for (int s = 0; s < C; ++s) {
            prv[s] = ldc<float>(prev + own + s * kComp);
            nv[s] = ldc_rw<float>(next + own + s * kComp);
        }
#pragma unroll
        for (int s = 0; s < C; ++s) H[s] = cx<float>(0.f, 0.f);
        // DEC Laplacian, sum_f w_f (psi_nb - psi) in entry order (Spin1GpeBCC.cu:835-865);
        // cells x + dx outside [0, X) are the zero halo
        Cx<float> v[4][C];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int xx = (int)x + dx[k];
            const bool in = (unsigned)xx < G.X;
            const uint32_t xc = in ? (uint32_t)xx : x;
            const char* p = prev + rb + off[k] + (size_t)(xc / kIlCells) * G.gb + (size_t)(xc % kIlCells) * 8;
#pragma unroll
            for (int s = 0; s < C; ++s) v[k][s] = in ? ldc<float>(p + s * kComp) : cx<float>(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
            for (int s = 0; s < C; ++s) H[s] += w[k] * (v[k][s] - prv[s]);
        }
        // local terms and the leapfrog update, as node_finish
        float rr[3];
        rr[0] = P.p0[0] + P.bs * ((float)x * P.bw[0] + pos[0]);
        rr[1] = P.p0[1] + P.bs * ((float)y * P.bw[1] + pos[1]);
        rr[2] = P.p0[2] + P.bs * ((float)z * P.bw[2] + pos[2]);
        const float pot = trap<float>(P, rr, nullptr);
        local_terms<float, C>(P, rr, pot, GPE_MODE_LEAPFROG, false, prv, H, nullptr);
        if constexpr (OBS) oa.template node<float, C>(P, rr, prv, H);
#pragma unroll
        for (int s = 0; s < C; ++s) {
            nv[s] += (2.f * P.dt) * cx<float>(H[s].y, -H[s].x);
            stc<float>(next + own + s * kComp, nv[s]);
        }
    }
    if constexpr (OBS) {
        __shared__ double red[8][OBS_COUNT];
        oa.block_reduce(red, a.partials);
    }
}

// Blocks per SM the kernels are compiled for (registers: spin-2 holds 5 records).
template <int C>
struct IlBounds {
    static constexpr int kMin = C == 5 ? 2 : (C == 3 ? 3 : 4);
};

template <int C>
__global__ void __launch_bounds__(256, IlBounds<C>::kMin) il_step_kernel(StepArgs a, ILGrid G, uint32_t tasks, FastDiv dGX) {
    il_step_body<C, false>(a, G, tasks, dGX);
}
template <int C>
__global__ void __launch_bounds__(256, IlBounds<C>::kMin) il_step_obs_kernel(StepArgs a, ILGrid G, uint32_t tasks,
                                                                             FastDiv dGX) {
    il_step_body<C, true>(a, G, tasks, dGX);
}

// Blocks of one interleaved step: one wave at the kernel's occupancy, a multiple of
// V / gcd(V, 8) (the grid's warp count a multiple of V), at most one warp per task
// and at most `max_blocks` (the handle's partial-sum rows); 0 if no such grid.
template <int C>
unsigned il_blocks(const ILGrid& G, bool obs, size_t max_blocks) {
    static int occ[2] = {0, 0};
    int& o = occ[obs ? 1 : 0];
    if (o == 0) {
        auto k = obs ? il_step_obs_kernel<C> : il_step_kernel<C>;
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, obs ? 50 : 25);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, 256, 0);
        if (o < 1) o = 1;
    }
    uint32_t gv = G.V, gb = 8;
    while (gb) {
        const uint32_t r = gv % gb;
        gv = gb;
        gb = r;
    }
    const uint64_t m = G.V / gv;
    const uint64_t tasks = (uint64_t)G.Y * G.Z * G.GX * G.V;
    uint64_t nb = std::min<uint64_t>((uint64_t)o * (unsigned)device_sm_count(), (tasks + 7) / 8);
    nb = std::min<uint64_t>(nb, max_blocks);
    return (unsigned)(nb / m * m);
}

// One interleaved leapfrog step (a.prev / a.next: interleaved buffers); obs: sum
// the observables of a.prev into a.partials and finalize them into out.
template <int C>
cudaError_t launch_il_step(const StepArgs& a, const ILGrid& G, size_t max_blocks, bool obs, double* out, cudaStream_t s) {
    const unsigned nb = il_blocks<C>(G, obs, max_blocks);
    if (nb == 0) return cudaErrorInvalidConfiguration;
    const uint32_t tasks = G.Y * G.Z * G.GX * G.V;
    const FastDiv dGX = make_fastdiv(G.GX);
    if (obs) {
        il_step_obs_kernel<C><<<nb, 256, 0, s>>>(a, G, tasks, dGX);
        observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    } else {
        il_step_kernel<C><<<nb, 256, 0, s>>>(a, G, tasks, dGX);
    }
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_IL(C) \
    template cudaError_t launch_il_step<C>(const StepArgs&, const ILGrid&, size_t, bool, double*, cudaStream_t); \
    template unsigned il_blocks<C>(const ILGrid&, bool, size_t);

// Both directions of the layout change for one state buffer (interior pointer aos).
// Defined once (GPE_DEFINE_IL_CONVERT in one translation unit).
cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s);

#define GPE_DEFINE_IL_CONVERT                                                                                        \
    cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s) { \
        const uint32_t J = G.V * G.C;                                                                                \
        const uint32_t JT = J < 128 ? J : 128;                                                                       \
        const uint32_t jtiles = (J + JT - 1) / JT;                                                                   \
        const uint64_t tiles = (uint64_t)G.Y * G.Z * G.GX * jtiles;                                                  \
        if (tiles == 0) return cudaSuccess;                                                                          \
        if (tiles > 0xffffffffu) return cudaErrorInvalidValue;                                                       \
        const size_t smem = (size_t)kIlCells * (JT + 1) * sizeof(float2);                                            \
        const unsigned nb = (unsigned)std::min<uint64_t>(tiles, (uint64_t)device_sm_count() * 8);                    \
        if (to_il) il_convert_kernel<true><<<nb, 256, smem, s>>>(aos, g, il, G, JT, jtiles, (uint32_t)tiles);       \
        else il_convert_kernel<false><<<nb, 256, smem, s>>>(aos, g, il, G, JT, jtiles, (uint32_t)tiles);            \
        return cudaGetLastError();                                                                                   \
    }

}  // namespace gpe
