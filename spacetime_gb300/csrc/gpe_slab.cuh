// gpe_slab.cuh -- the slab-ring leapfrog kernel: one block per column of
// Tx x Ty block cells marching up z, every neighbour read from shared memory.
//
// Why this shape.  The gather kernels read each node's 4 neighbour records
// straight from global memory.  A warp's request for 32 scattered 24-byte
// records touches ~14 distinct 128-byte lines, and the L1 data stage spends about
// one wavefront per line and request: the spin-1 BCC step costs ~131 data-stage
// wavefronts per warp of 32 nodes and is bound there (85 % busy) while DRAM runs
// at 57 %.  Here the previous state arrives in shared memory by bulk copies
// (cp.async.bulk on an mbarrier: the async proxy, no LSU work), and a warp's
// shared-memory read of 32 records costs its bank-conflict degree, about 4 + 2
// wavefronts for a whole 24-byte record (16-byte + 8-byte loads).
//
// Pipeline.  Load i brings plane z = i - 1 of psi_prev (the Ty + 2 rows
// y0-1 .. y0+Ty, each the Tx + 2 cells x0-1 .. x0+Tx, one bulk copy per row) into
// ring slot i mod S; the step of plane z reads loads z, z+1, z+2 (planes z-1, z,
// z+1).  After the step of plane z every thread passes one block barrier and
// thread 0 reuses slot z mod S for load z + S, so S - 3 planes are in flight
// while a plane is computed.  Waits are bounded: a wait that runs out sets the
// handle's error flag, the block stops at the next barrier (all threads agree
// through __syncthreads_and) and lets its copies in flight land, with a bound,
// before it exits.
//
// The old psi_next values of the tile (Tx x Ty cells, no halo) arrive by bulk
// copies too, in a second ring of Sn tiles filled Sn - 1 planes ahead: a load of
// them from global memory at the start of each plane exposed a full DRAM latency
// per plane.  The updated record is stored straight from registers.  Each
// psi_next value is read and written once.  Thread 0 also asks L2 (bulk prefetch)
// for the psi_prev rows two loads beyond the ring, so the ring's copies find them
// there.  Arithmetic and its order are those of the gather
// kernels (parabolic_node_t + node_finish); the compiler may contract a
// different multiply-add, so the two agree to rounding, not bit for bit.
//
// Halo: the buffers carry a one-cell zero halo, so the rows and cells at -1 and
// X / Y / Z that a slab reaches exist.  Ragged tiles (X % Tx or Y % Ty non-zero)
// copy only their own cells plus the halo; threads outside the grid idle.
#pragma once

namespace gpe {

constexpr int kSlabMaxRing = 8;
constexpr int kSlabMaxThreads = 384;

struct SlabArgs {
    uint32_t Tx, Ty;       // cells of a tile along x, rows along y
    uint32_t S;            // psi_prev ring slots (4 .. kSlabMaxRing)
    uint32_t Sn;           // psi_next ring slots (2 .. kSlabMaxRing; 0: psi_next loaded per plane)
    uint32_t tiles_x;      // tiles along x (blocks = tiles_x * tiles_y)
    uint32_t seg_stride;   // bytes of one slab row: (Tx + 2) cells
    uint32_t slab_bytes;   // bytes of one slab: (Ty + 2) rows
    uint32_t tile_bytes;   // bytes of one psi_next tile: Ty rows of Tx cells
    uint32_t nodes;        // Tx * Ty * V (<= the block size)
};

// L2 prefetch of a contiguous range (16-byte aligned, a multiple of 16 bytes).
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// 16- and 8-byte shared-memory loads at a shared-window address (volatile: they
// must stay after the mbarrier wait that makes the data visible).
__device__ __forceinline__ float4 lds_f4(uint32_t a) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
    return v;
}
__device__ __forceinline__ float2 lds_f2(uint32_t a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ double2 lds_d2(uint32_t a) {
    double2 v;
    asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(a));
    return v;
}

// A whole node record from shared memory, in the split of ld_node: FP32 records of
// odd C > 1 as (C-1)/2 aligned 16-byte loads and one 8-byte load ordered by bit 3
// of the address; FP32 scalars one 8-byte load; FP64 one 16-byte load per value.
template <typename R, int C>
__device__ __forceinline__ void lds_node(uint32_t p, Cx<R>* v) {
    if constexpr (sizeof(R) == 4 && C > 1 && (C % 2) == 1) {
        const bool odd = (p & 8u) != 0;
        const uint32_t q = p + (odd ? 8u : 0u);
        const uint32_t r = p + (odd ? 0u : 8u * (C - 1));
        float4 a[(C - 1) / 2];
#pragma unroll
        for (int k = 0; k < (C - 1) / 2; ++k) a[k] = lds_f4(q + 16u * k);
        const float2 b = lds_f2(r);
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const int te = s, to = s - 1;
            const Cx<R> ve = s == C - 1 ? cx<R>(b.x, b.y)
                                        : ((te & 1) ? cx<R>(a[te / 2].z, a[te / 2].w) : cx<R>(a[te / 2].x, a[te / 2].y));
            const Cx<R> vo = s == 0 ? cx<R>(b.x, b.y)
                                    : ((to & 1) ? cx<R>(a[to / 2].z, a[to / 2].w) : cx<R>(a[to / 2].x, a[to / 2].y));
            v[s] = odd ? vo : ve;
        }
    } else if constexpr (sizeof(R) == 4) {
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const float2 b = lds_f2(p + 8u * s);
            v[s] = cx<R>(b.x, b.y);
        }
    } else {
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const double2 b = lds_d2(p + 16u * s);
            v[s] = cx<R>(b.x, b.y);
        }
    }
}

// Leapfrog step psi_next += 2 dt (-i H psi_prev) on lattices whose nodes all have
// D stencil entries.  Block = one Tx x Ty column of cells, all planes; thread t =
// node (t mod V) of tile cell t / V, the same node on every plane.
template <typename R, int C, int D>
__global__ void __launch_bounds__(kSlabMaxThreads, 2) parabolic_slab_kernel(StepArgs a, SlabArgs m) {
    extern __shared__ __align__(128) unsigned char dyn[];
    __shared__ __align__(8) uint64_t full[kSlabMaxRing];
    __shared__ __align__(8) uint64_t full_n[kSlabMaxRing];
    const uint32_t cb = a.g.cell_bytes;
    const uint32_t V = a.g.V;
    constexpr uint32_t nb = C * 2 * sizeof(R);
    const uint32_t t = threadIdx.x;
    const uint32_t cell = fdiv(t, a.divV);
    const uint32_t l = t - cell * V;
    const uint32_t uy = cell / m.Tx, ux = cell - uy * m.Tx;
    const uint32_t ty = blockIdx.x / m.tiles_x, tx = blockIdx.x - ty * m.tiles_x;
    const uint32_t x0 = tx * m.Tx, y0 = ty * m.Ty;
    const uint32_t wx = min(m.Tx, a.g.X - x0), wy = min(m.Ty, a.g.Y - y0);
    const bool active = t < m.nodes && ux < wx && uy < wy;
    const uint32_t seg_bytes = (wx + 2) * cb;
    const uint32_t plane_bytes = (wy + 2) * seg_bytes;
    const uint32_t S = m.S, Sn = m.Sn;
    const uint32_t Z = a.g.Z;
    const uint32_t nloads = Z + 2;
    const uint32_t slab0 = smem_u32(dyn);
    const uint32_t tile0 = slab0 + S * m.slab_bytes;
    const uint32_t row_bytes = wx * cb;  // one row of the tile's psi_next

    // the node's entries: offset inside a slab, plane (dz), weight h / bs^2 of the
    // step's block scale; its own record's offset; its position in the cell
    const uint32_t own = ((uy + 1) * (m.Tx + 2) + (ux + 1)) * cb + l * nb;
    int32_t soff[D];
    int32_t dzk[D];
    R w[D];
    const R ks = make_phys<R>(a).ks;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const int f = active ? (int)l * D + k : 0;
        const int4 e = a.tab.ent4[f];
        soff[k] = (int32_t)own + (e.y * (int32_t)(m.Tx + 2) + e.x) * (int32_t)cb + (e.w - (int32_t)l) * (int32_t)nb;
        dzk[k] = e.z;
        if constexpr (sizeof(R) == 4) w[k] = a.tab.w32[f] * ks;
        else w[k] = a.tab.w64[f] * ks;
    }
    R pos[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = active ? 3 * (int)l + k : k;
        if constexpr (sizeof(R) == 4) pos[k] = a.tab.pos32[i];
        else pos[k] = a.tab.pos64[i];
    }

    const uint32_t own_n = (uy * m.Tx + ux) * cb + l * nb;  // the node in a psi_next tile
    if (t == 0) {
        for (uint32_t s = 0; s < S; ++s) mbar_init(&full[s], 1);
        for (uint32_t s = 0; s < Sn; ++s) mbar_init(&full_n[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async_smem();
    }
    __syncthreads();

    // Ring positions advance by one slot per load, the mbarrier parity flipping at
    // each wrap (no division by the runtime ring size anywhere in the loop).
    struct Cursor {
        uint32_t slot, par, n;
        __device__ __forceinline__ void next() {
            if (++slot == n) {
                slot = 0;
                par ^= 1u;
            }
        }
    };
    const bool ring_n = Sn > 0;  // psi_next through the tile ring (else loaded per plane)

    // thread 0: load i brings plane i - 1 of psi_prev into the next slab slot;
    // tile load j plane j of psi_next into the next tile slot
    const char* src_p = a.prev + ((ptrdiff_t)y0 - 1) * (ptrdiff_t)a.g.pitch + ((ptrdiff_t)x0 - 1) * (ptrdiff_t)cb -
                        (ptrdiff_t)a.g.slice;
    const char* src_n = a.next + (size_t)y0 * a.g.pitch + (size_t)x0 * cb;
    const size_t slice = a.g.slice, pitch = a.g.pitch;
    Cursor ip{0, 0, S}, in{0, 0, ring_n ? Sn : 1u};
    uint32_t issued = 0, issued_n = 0;
    auto issue = [&]() {
        mbar_expect_tx(&full[ip.slot], plane_bytes);
        const char* src = src_p + (size_t)issued * slice;
        char* dst = reinterpret_cast<char*>(dyn) + (size_t)ip.slot * m.slab_bytes;
        for (uint32_t r = 0; r < wy + 2; ++r) bulk_load(dst + (size_t)r * m.seg_stride, src + r * pitch, seg_bytes, &full[ip.slot]);
        ip.next();
        ++issued;
    };
    auto prefetch = [&](uint32_t i) {
        const char* src = src_p + (size_t)i * slice;
        for (uint32_t r = 0; r < wy + 2; ++r) bulk_prefetch_l2(src + r * pitch, seg_bytes);
    };
    auto issue_n = [&]() {
        mbar_expect_tx(&full_n[in.slot], wy * row_bytes);
        const char* src = src_n + (size_t)issued_n * slice;
        char* dst = reinterpret_cast<char*>(dyn) + (size_t)S * m.slab_bytes + (size_t)in.slot * m.tile_bytes;
        for (uint32_t r = 0; r < wy; ++r) bulk_load(dst + (size_t)r * m.Tx * cb, src + r * pitch, row_bytes, &full_n[in.slot]);
        in.next();
        ++issued_n;
    };
    if (t == 0) {
        while (issued < S && issued < nloads) issue();
        if (ring_n)
            while (issued_n < Sn && issued_n < Z) issue_n();
        for (uint32_t i = issued; i < issued + 2 && i < nloads; ++i) prefetch(i);
    }

    const PhysR<R>& P = make_phys<R>(a);
    char* nxt = a.next + (size_t)(y0 + uy) * pitch + (size_t)(x0 + ux) * cb + l * nb;
    bool ok = true;
    Cursor wp{0, 0, S}, wn{0, 0, ring_n ? Sn : 1u};  // next load / tile load to wait for
    uint32_t waited = 0, waited_n = 0;
    // slab addresses of planes z-1, z, z+1 (loads z, z+1, z+2)
    uint32_t b0 = slab0, b1 = slab0 + m.slab_bytes, b2 = slab0 + 2 * m.slab_bytes;
    const uint32_t slab_end = slab0 + S * m.slab_bytes;
    uint32_t tb = tile0;
    const uint32_t tile_end = tile0 + (ring_n ? Sn : 1u) * m.tile_bytes;
    auto wait_on = [&](uint64_t* bar, uint32_t par) {
        bool got = false;
        for (uint32_t spin = 0; spin < (1u << 22) && !(got = mbar_try_wait(bar, par)); ++spin) {
        }
        return got;
    };
    for (uint32_t z = 0; z < Z; ++z) {
        Cx<R> nv[C];
        if (!ring_n && active) ld_node<R, C, false>(nxt, nv);
        // loads z, z+1, z+2 and tile load z must have landed
        while (ok && waited < z + 3) {
            ok = wait_on(&full[wp.slot], wp.par);
            if (ok) {
                wp.next();
                ++waited;
            }
        }
        if (ok && ring_n) {
            ok = wait_on(&full_n[wn.slot], wn.par);
            if (ok) {
                wn.next();
                ++waited_n;
            }
        }
        if (ok && active) {
            if (ring_n) lds_node<R, C>(tb + own_n, nv);
            Cx<R> prv[C], H[C];
            lds_node<R, C>(b1 + own, prv);
            Cx<R> v[D][C];
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const uint32_t base = dzk[k] < 0 ? b0 : (dzk[k] > 0 ? b2 : b1);
                lds_node<R, C>(base + (uint32_t)soff[k], v[k]);
            }
#pragma unroll
            for (int s = 0; s < C; ++s) H[s] = cx<R>((R)0, (R)0);
            // DEC Laplacian in entry order (Spin1GpeBCC.cu:835-865), as the gather kernels
#pragma unroll
            for (int k = 0; k < D; ++k) {
#pragma unroll
                for (int s = 0; s < C; ++s) H[s] += w[k] * (v[k][s] - prv[s]);
            }
            node_finish<R, C, GPE_MODE_LEAPFROG>(P, pos, x0 + ux, y0 + uy, z, prv, H, nv, nxt, nullptr);
        }
        nxt += slice;
        b0 = b1;
        b1 = b2;
        b2 += m.slab_bytes;
        if (b2 == slab_end) b2 = slab0;
        tb += m.tile_bytes;
        if (tb == tile_end) tb = tile0;
        // every thread is done with the slab of load z (plane z-1) and tile z
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        if (t == 0) {
            fence_proxy_async_smem();
            if (issued < nloads) issue();
            if (ring_n && issued_n < Z) issue_n();
            if (issued + 1 < nloads) prefetch(issued + 1);
        }
    }
    if (!ok && t == 0) {
        if (a.err) atomicExch(a.err, 1);
        // let the copies in flight land before the block's shared memory goes away
        for (; waited < issued; ++waited) {
            for (uint32_t spin = 0; spin < (1u << 16) && !mbar_try_wait(&full[wp.slot], wp.par); ++spin) {
            }
            wp.next();
        }
        for (; ring_n && waited_n < issued_n; ++waited_n) {
            for (uint32_t spin = 0; spin < (1u << 16) && !mbar_try_wait(&full_n[wn.slot], wn.par); ++spin) {
            }
            wn.next();
        }
    }
}

// Ring sizes within 110 KB, two blocks per SM inside 228 KB with the driver's
// reserve.  S_req > 0 asks for that many psi_prev slabs; the psi_next tile ring
// takes what is left (0 if fewer than two tiles fit: psi_next is then loaded from
// global memory per plane).  By default four slabs and as many tiles as fit (up to
// four), then a fifth slab, then more tiles.  Returns false if four slabs do not fit.
inline bool slab_rings(uint32_t slab_bytes, uint32_t tile_bytes, uint32_t S_req, uint32_t* S, uint32_t* Sn) {
    const uint64_t budget = 110u * 1024u;
    const auto fits = [&](uint64_t s, uint64_t sn) { return s * slab_bytes + sn * tile_bytes <= budget; };
    if (!slab_bytes || !tile_bytes || !fits(4, 0)) return false;
    uint32_t s = 4, sn = 0;
    if (S_req > 0) {
        if (S_req < 4 || S_req > (uint32_t)kSlabMaxRing || !fits(S_req, 0)) return false;
        s = S_req;
        while (sn < (uint32_t)kSlabMaxRing && fits(s, sn + 1)) ++sn;
    } else {
        while (sn < 4 && fits(s, sn + 1)) ++sn;
        while (s < 5 && fits(s + 1, sn)) ++s;
        while (sn < (uint32_t)kSlabMaxRing && fits(s, sn + 1)) ++sn;
    }
    *S = s;
    *Sn = sn >= 2 ? sn : 0;
    return true;
}

template <typename R, int C, int D>
cudaError_t launch_parabolic_slab_d(const StepArgs& a, SlabArgs m, cudaStream_t s) {
    const size_t smem = (size_t)m.S * m.slab_bytes + (size_t)m.Sn * m.tile_bytes;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e =
            cudaFuncSetAttribute(parabolic_slab_kernel<R, C, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        cudaFuncSetAttribute(parabolic_slab_kernel<R, C, D>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        configured = smem;
    }
    const uint32_t threads = (m.nodes + 31) / 32 * 32;
    const uint32_t blocks = m.tiles_x * ((a.g.Y + m.Ty - 1) / m.Ty);
    parabolic_slab_kernel<R, C, D><<<blocks, threads, smem, s>>>(a, m);
    return cudaGetLastError();
}

// Leapfrog step by the slab kernel: 4-entry lattices with 16-byte cells, tile
// Tx x Ty with Tx * Ty * V <= 384 threads.
template <typename R, int C>
cudaError_t launch_parabolic_slab(const StepArgs& a, uint32_t Tx, uint32_t Ty, uint32_t S, cudaStream_t s) {
    if (a.tab.uniform_deg != 4 || a.g.cell_bytes % 16 != 0 || Tx == 0 || Ty == 0) return cudaErrorInvalidValue;
    SlabArgs m;
    m.Tx = Tx;
    m.Ty = Ty;
    m.nodes = Tx * Ty * a.g.V;
    if (m.nodes > (uint32_t)kSlabMaxThreads) return cudaErrorInvalidValue;
    m.tiles_x = (a.g.X + Tx - 1) / Tx;
    m.seg_stride = (Tx + 2) * a.g.cell_bytes;
    m.slab_bytes = (Ty + 2) * m.seg_stride;
    m.tile_bytes = Tx * Ty * a.g.cell_bytes;
    if (!slab_rings(m.slab_bytes, m.tile_bytes, S, &m.S, &m.Sn)) return cudaErrorInvalidValue;
    return launch_parabolic_slab_d<R, C, 4>(a, m, s);
}

#define GPE_INSTANTIATE_SLAB(R, C) \
    template cudaError_t launch_parabolic_slab<R, C>(const StepArgs&, uint32_t, uint32_t, uint32_t, cudaStream_t);

}  // namespace gpe
