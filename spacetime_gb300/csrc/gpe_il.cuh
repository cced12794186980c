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
// cells x JT complex values (j = l C + s) per pass, staged in shared memory
// (32 x (JT + 1) float2, the padding against bank conflicts) so that both sides
// are read and written in contiguous 16-byte runs.  aos: the slot's interior
// pointer.  J = V C and JT are even (every lattice with 4 entries per node has an
// even node count), so a cell's values and the tiles start on 16-byte boundaries.
// Each thread issues all its loads of a tile (at most kIlConvLoads 16-byte loads)
// before it stores any of them.  The interleaved halo rows and padding cells are
// not touched.
constexpr uint32_t kIlConvThreads = 256;
constexpr uint32_t kIlConvLoads = 8;  // 32 cells x 128 values / 2 per load / 256 threads
template <bool TO_IL>
__global__ void __launch_bounds__(kIlConvThreads, 4) il_convert_kernel(char* aos, Grid g, char* il, ILGrid G, uint32_t JT,
                                                                    uint32_t jtiles, uint32_t tiles, FastDiv djt,
                                                                    FastDiv dgx, FastDiv dy) {
    extern __shared__ float2 il_tile[];  // 32 x (JT + 1)
    const uint32_t J = G.V * G.C;
    const uint32_t ld = JT + 1;
    for (uint32_t w = blockIdx.x; w < tiles; w += gridDim.x) {
        const uint32_t r1 = fdiv(w, djt);
        const uint32_t jt = w - r1 * jtiles;
        const uint32_t r2 = fdiv(r1, dgx);
        const uint32_t gx = r1 - r2 * G.GX;
        const uint32_t z = fdiv(r2, dy);
        const uint32_t y = r2 - z * G.Y;
        const uint32_t j0 = jt * JT;
        const uint32_t nj = min(JT, J - j0);   // even
        const uint32_t nc = min(kIlCells, G.X - gx * kIlCells);
        const uint32_t half = nj / 2;          // 16-byte runs per cell of the tile
        char* arow = aos + (size_t)z * g.slice + (size_t)y * g.pitch + (size_t)gx * kIlCells * g.cell_bytes + (size_t)j0 * 8;
        char* irow = il + il_row(G, y, z) + (size_t)gx * G.gb + (size_t)j0 * kIlCells * 8;
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
                const uint32_t jj = i / (kIlCells / 2), c = 2 * (i % (kIlCells / 2));
                if (jj < nj && c < nc) {
                    const float2 a = il_tile[c * ld + jj];
                    char* dst = irow + ((size_t)jj * kIlCells + c) * 8;
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
                const uint32_t jj = i / (kIlCells / 2), c = 2 * (i % (kIlCells / 2));
                if (jj < nj && c < nc) buf[k] = __ldg(reinterpret_cast<const float4*>(irow + ((size_t)jj * kIlCells + c) * 8));
            }
#pragma unroll
            for (uint32_t k = 0; k < kIlConvLoads; ++k) {
                const uint32_t i = threadIdx.x + k * kIlConvThreads;
                const uint32_t jj = i / (kIlCells / 2), c = 2 * (i % (kIlCells / 2));
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
    // neighbour k of node l: node e.w of the cells shifted by (dx, dy, dz); for
    // this lane the shift is a fixed offset from its own group's base: the rows
    // (dz, dy), the node, and lane + dx within the group or (lane 0 / 31) the last
    // / first cell of the group before / after it
    int dx[4];
    int32_t off[4];
    float w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int4 e = a.tab.ent4[l * 4 + k];
        dx[k] = e.x;
        const int xl = (int)lane + e.x;                       // -1 .. 32
        const int64_t gshift = xl < 0 ? -1 : (xl >= (int)kIlCells ? 1 : 0);
        const int64_t cell = xl - gshift * (int64_t)kIlCells;
        off[k] = (int32_t)(((int64_t)e.z * (G.Y + 2) + e.y) * (int64_t)G.row + (int64_t)e.w * node_run +
                           gshift * (int64_t)G.gb + cell * 8);
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
        const size_t gbase = il_row(G, y, z) + (size_t)gx * G.gb;
        const size_t own = gbase + (size_t)l * node_run + (size_t)lane * 8;
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
            const bool in = (unsigned)((int)x + dx[k]) < G.X;
            const char* p = prev + gbase + (in ? off[k] : 0);
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

// Launch shapes: the plain step in blocks of kIlPlainThreads with at least
// IlBounds<C>::kMin of them per SM (the register cap that keeps the most warps in
// flight without spills), the observed step in blocks of 256 (its FP64 sums take
// shared memory per thread).
constexpr unsigned kIlPlainThreads = 128;
constexpr unsigned kIlObsThreads = 256;
template <int C>
struct IlBounds {
    // spin-1 BCC 96^3: 7 blocks (72 registers) 0.131 ms per step, 8 (64) 0.147,
    // 9 (56) 0.145; spin-2 BCC 96^3: 4 blocks (105) 0.222 ms, 5 (96) 0.211, 6 (80) 0.218
    static constexpr int kMin = C == 5 ? 5 : (C == 3 ? 7 : 8);
    static constexpr int kMinObs = C == 5 ? 2 : 3;
};

template <int C>
__global__ void __launch_bounds__(kIlPlainThreads, IlBounds<C>::kMin) il_step_kernel(StepArgs a, ILGrid G, uint32_t tasks,
                                                                                    FastDiv dGX) {
    il_step_body<C, false>(a, G, tasks, dGX);
}
template <int C>
__global__ void __launch_bounds__(kIlObsThreads, IlBounds<C>::kMinObs) il_step_obs_kernel(StepArgs a, ILGrid G,
                                                                                        uint32_t tasks, FastDiv dGX) {
    il_step_body<C, true>(a, G, tasks, dGX);
}

// Blocks of one interleaved step: one wave at the kernel's occupancy, a multiple
// of V / gcd(V, warps per block) (the grid's warp count a multiple of V), at most
// one warp per task and at most `max_blocks` (the handle's partial-sum rows); 0 if
// no such grid.
template <int C>
unsigned il_blocks(const ILGrid& G, bool obs, size_t max_blocks) {
    static int occ[2] = {0, 0};
    const unsigned threads = obs ? kIlObsThreads : kIlPlainThreads;
    const unsigned wpb = threads / 32;
    int& o = occ[obs ? 1 : 0];
    if (o == 0) {
        auto k = obs ? il_step_obs_kernel<C> : il_step_kernel<C>;
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, obs ? 50 : 25);
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
    const uint64_t tasks = (uint64_t)G.Y * G.Z * G.GX * G.V;
    uint64_t nb = std::min<uint64_t>((uint64_t)o * (unsigned)device_sm_count(), (tasks + wpb - 1) / wpb);
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
        il_step_obs_kernel<C><<<nb, kIlObsThreads, 0, s>>>(a, G, tasks, dGX);
        observe_finalize_kernel<<<1, 256, 0, s>>>(a.partials, nb, out);
    } else {
        il_step_kernel<C><<<nb, kIlPlainThreads, 0, s>>>(a, G, tasks, dGX);
    }
    return cudaGetLastError();
}

#define GPE_INSTANTIATE_IL(C)                                                                                      \
    template cudaError_t launch_il_step<C>(const StepArgs&, const ILGrid&, size_t, bool, double*, cudaStream_t); \
    template unsigned il_blocks<C>(const ILGrid&, bool, size_t);

// Both directions of the layout change for one state buffer (interior pointer aos).
// Defined once (GPE_DEFINE_IL_CONVERT in one translation unit).
cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s);

#define GPE_DEFINE_IL_CONVERT                                                                                        \
    cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s) { \
        const uint32_t J = G.V * G.C;                                                                                \
        if (J % 2 || g.cell_bytes != J * 8) return cudaErrorInvalidValue;                                            \
        const uint32_t JT = J < 128 ? J : 128;                                                                       \
        const uint32_t jtiles = (J + JT - 1) / JT;                                                                   \
        const uint64_t tiles = (uint64_t)G.Y * G.Z * G.GX * jtiles;                                                  \
        if (tiles == 0) return cudaSuccess;                                                                          \
        if (tiles > 0xffffffffu) return cudaErrorInvalidValue;                                                       \
        const size_t smem = (size_t)kIlCells * (JT + 1) * sizeof(float2);                                            \
        const unsigned nb = (unsigned)std::min<uint64_t>(tiles, (uint64_t)device_sm_count() * 8);                    \
        const FastDiv djt = make_fastdiv(jtiles), dgx = make_fastdiv(G.GX), dy = make_fastdiv(G.Y);                  \
        if (to_il)                                                                                                   \
            il_convert_kernel<true><<<nb, kIlConvThreads, smem, s>>>(aos, g, il, G, JT, jtiles, (uint32_t)tiles, djt, dgx, dy); \
        else                                                                                                         \
            il_convert_kernel<false><<<nb, kIlConvThreads, smem, s>>>(aos, g, il, G, JT, jtiles, (uint32_t)tiles, djt, dgx, dy); \
        return cudaGetLastError();                                                                                   \
    }

}  // namespace gpe
