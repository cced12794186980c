// gpe_noalloc.cu -- observables of a caller-owned psi buffer without any device
// allocation (gpe_observe_noalloc in include/gpe.h).
//
// Some callers cannot allocate device memory when they want the norm, energy or
// magnetisation of their state: a simulation whose memory is owned by another
// framework's pool, or a time loop that has laid out every buffer up front and
// must keep a fixed footprint.  This entry point needs no handle: the stencil
// tables travel in the kernel's parameter block, and the reduction's scratch is
// one file-scope device array of fixed size, OBS_NOALLOC_BLOCKS x OBS_COUNT
// partial sums plus one result row (2049 x 12 doubles, about 197 KB), which every
// GPU that loads the library keeps until the process exits.
//
// The array is shared by all calls: overlapping calls on the GPU race on it, so
// callers must order them (one stream, or events).  Every block overwrites its
// own partial row on each call and the final kernel overwrites the result row, so
// nothing has to be cleared between calls.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "gpe_kernels.cuh"

namespace gpe {

constexpr int OBS_NOALLOC_BLOCKS = 2048;

static __device__ __align__(256) double g_obs_scratch[(OBS_NOALLOC_BLOCKS + 1) * OBS_COUNT];

// Stencil tables by value (kernel parameter block, < 32 KB).
struct NoAllocTables {
    int32_t row_ptr[kMaxNodes + 1];
    int32_t nb_off[kMaxEntries];
    double w[kMaxEntries];
    double pos[kMaxNodes * 3];
};

// Grid-stride version of observe_kernel: a fixed number of blocks, each thread
// accumulating over many nodes, block partials into the static scratch.
template <typename R, int C>
__global__ void __launch_bounds__(256) observe_noalloc_kernel(StepArgs a, NoAllocTables tab, double* partials) {
    __shared__ double red[8][OBS_COUNT];
    double acc[OBS_COUNT];
#pragma unroll
    for (int k = 0; k < OBS_COUNT; ++k) acc[k] = 0.0;
    const PhysR<double>& P = a.pd;
    PhysR<double> Q = P;
    Q.bq = Q.bqq = 0;
    for (int k = 0; k < 3; ++k) Q.bb[k] = Q.bbq[k] = 0;
    Q.flags &= ~(GPE_FLAG_THREE_BODY_LOSS | GPE_FLAG_QUADRATIC_ZEEMAN | GPE_FLAG_QUADRUPOLE_OFFSET);
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
        const char* base = a.prev + (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
        Cx<double> ps[C], L[C], Hl[C], Hn[C];
        double rho = 0, maxabs = 0, bad = 0;
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const Cx<R> v = ldc<R>(base + l * node_bytes + s * 2 * sizeof(R));
            ps[s] = cx<double>((double)v.x, (double)v.y);
            L[s] = Hl[s] = Hn[s] = cx<double>(0.0, 0.0);
            const double n2 = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
            rho += n2;
            maxabs = fmax(maxabs, sqrt(n2));
            if (!isfinite(ps[s].x) || !isfinite(ps[s].y)) bad += 1;
        }
        for (int f = tab.row_ptr[l]; f < tab.row_ptr[l + 1]; ++f) {
            const char* nb = base + tab.nb_off[f];
#pragma unroll
            for (int s = 0; s < C; ++s) {
                const Cx<R> v = ldc<R>(nb + s * 2 * sizeof(R));
                L[s] += tab.w[f] * (cx<double>((double)v.x, (double)v.y) - ps[s]);
            }
        }
        double r[3];
        r[0] = P.p0[0] + P.bs * ((double)x * P.bw[0] + tab.pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((double)y * P.bw[1] + tab.pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((double)z * P.bw[2] + tab.pos[3 * l + 2]);
        local_terms<double, C>(P, r, trap<double>(P, r), GPE_MODE_LEAPFROG, false, ps, Hl);
        local_terms<double, C>(Q, r, 0.0, GPE_MODE_LEAPFROG, false, ps, Hn);
        double kin = 0, hl = 0, hn = 0;
#pragma unroll
        for (int s = 0; s < C; ++s) {
            kin += ps[s].x * L[s].x + ps[s].y * L[s].y;
            hl += ps[s].x * Hl[s].x + ps[s].y * Hl[s].y;
            hn += ps[s].x * Hn[s].x + ps[s].y * Hn[s].y;
        }
        acc[OBS_NORM] += rho;
        acc[OBS_HEXP] += kin + hl;
        acc[OBS_EINT] += hn;
        acc[OBS_COMX] += rho * r[0];
        acc[OBS_COMY] += rho * r[1];
        acc[OBS_COMZ] += rho * r[2];
        acc[OBS_MAXABS] = fmax(acc[OBS_MAXABS], maxabs);
        acc[OBS_NONFINITE] += bad;
        if constexpr (C == 3) {
            const Cx<double> m = GPE_REF_SQRT_2 * (conj(ps[0]) * ps[1] + conj(ps[1]) * ps[2]);
            const double fz = (ps[0].x * ps[0].x + ps[0].y * ps[0].y) - (ps[2].x * ps[2].x + ps[2].y * ps[2].y);
            acc[OBS_MAGX] += m.x;
            acc[OBS_MAGY] += m.y;
            acc[OBS_MAGZ] += fz;
            acc[OBS_SPIN] += sqrt(m.x * m.x + m.y * m.y + fz * fz);
        } else if constexpr (C == 5) {
            const Cx<double> fp = 2.0 * (conj(ps[0]) * ps[1] + conj(ps[3]) * ps[4]) +
                                  2.449489742783178098 * (conj(ps[1]) * ps[2] + conj(ps[2]) * ps[3]);
            double n[5];
            for (int s = 0; s < 5; ++s) n[s] = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
            const double fz = 2 * n[0] + n[1] - n[3] - 2 * n[4];
            acc[OBS_MAGX] += fp.x;
            acc[OBS_MAGY] += fp.y;
            acc[OBS_MAGZ] += fz;
            acc[OBS_SPIN] += sqrt(fp.x * fp.x + fp.y * fp.y + fz * fz);
        }
    }
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

}  // namespace gpe

using namespace gpe;

namespace {

// Device address of g_obs_scratch per device ordinal, looked up once per device
// with that device current.  In host code the symbol's name only stands in for
// the device array; a kernel must be given this address.  The mutex makes the
// first calls from several host threads safe.  The cached address belongs to the
// device's current context: after cudaDeviceReset the module is loaded again and
// the address may change, so a process that resets a device must not call this
// entry point on that device afterwards.
constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

// Errors are reported through gpe_last_error().
gpe_status noalloc_fail(gpe_status st, const std::string& m) {
    gpe::set_last_error(m);
    return st;
}

}  // namespace

extern "C" gpe_status gpe_observe_noalloc(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* fields,
                                          double t, const void* psi, size_t pitch, size_t slice_pitch,
                                          gpe_observables* out, void* stream) {
    if (!lat || !p || !psi || !out) return noalloc_fail(GPE_ERR_INVALID_ARG, "null argument");
    if (p->components != 1 && p->components != 3 && p->components != 5)
        return noalloc_fail(GPE_ERR_INVALID_ARG, "components must be 1, 3 or 5");
    if (p->precision != GPE_FP32 && p->precision != GPE_FP64) return noalloc_fail(GPE_ERR_INVALID_ARG, "precision");
    const int V = lat->nodes;
    if (V <= 0 || V > kMaxNodes) return noalloc_fail(GPE_ERR_INVALID_ARG, "nodes beyond the static table size (160)");
    if (!lat->row_ptr || !lat->stencil || !lat->pos) return noalloc_fail(GPE_ERR_INVALID_ARG, "missing table");
    // The kernel walks row_ptr[l] .. row_ptr[l+1] of the by-value tables, so every
    // row must lie inside them: row_ptr starts at 0 and never decreases.
    if (lat->row_ptr[0] != 0) return noalloc_fail(GPE_ERR_INVALID_ARG, "row_ptr[0] must be 0");
    for (int l = 0; l < V; ++l)
        if (lat->row_ptr[l + 1] < lat->row_ptr[l]) return noalloc_fail(GPE_ERR_INVALID_ARG, "row_ptr must not decrease");
    const int n = lat->row_ptr[V];
    if (n <= 0 || n > kMaxEntries) return noalloc_fail(GPE_ERR_INVALID_ARG, "stencil beyond the static table size (640)");
    const uint64_t sites = (uint64_t)p->dims[0] * p->dims[1] * p->dims[2] * (uint64_t)V;
    if (sites == 0 || sites >= (1ull << 32)) return noalloc_fail(GPE_ERR_INVALID_ARG, "grid must hold 1 .. 2^32-1 sites");
    const size_t real_bytes = p->precision == GPE_FP64 ? 8 : 4;
    const size_t cell_bytes = (size_t)V * p->components * 2 * real_bytes;
    if (pitch < (p->dims[0] + 2) * cell_bytes || slice_pitch < pitch * (p->dims[1] + 2))
        return noalloc_fail(GPE_ERR_INVALID_ARG, "pitch or slice pitch smaller than the padded row or slice");
    // Complex values are read as float2 / double2 vectors: psi, the pitch and the
    // slice pitch must keep every value on a multiple of its own size.
    const size_t align = 2 * real_bytes;
    if (reinterpret_cast<uintptr_t>(psi) % align != 0 || pitch % align != 0 || slice_pitch % align != 0)
        return noalloc_fail(GPE_ERR_INVALID_ARG, "psi, pitch and slice pitch must be multiples of one complex value's size");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(GPE_ERR_NO_DEVICE, "no usable CUDA device");
    double* scratch = nullptr;
    {
        // Set-up on the first call on this device (this device is current here).
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void* addr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&addr, g_obs_scratch);
            if (e != cudaSuccess || !addr)
                return noalloc_fail(GPE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<double*>(addr);
        }
        scratch = g_scratch_addr[dev];
    }

    NoAllocTables tab;
    std::memset(&tab, 0, sizeof tab);
    const double bs2 = p->block_scale * p->block_scale;
    const size_t node_bytes = (size_t)p->components * 2 * real_bytes;
    for (int l = 0; l <= V; ++l) tab.row_ptr[l] = lat->row_ptr[l];
    for (int f = 0; f < n; ++f) {
        const gpe_stencil_entry& e = lat->stencil[f];
        if (e.dx < -1 || e.dx > 1 || e.dy < -1 || e.dy > 1 || e.dz < -1 || e.dz > 1 || e.node < 0 || e.node >= V)
            return noalloc_fail(GPE_ERR_INVALID_ARG, "stencil entry out of range");
        const long long off = (long long)e.dz * (long long)slice_pitch + (long long)e.dy * (long long)pitch +
                              (long long)e.dx * (long long)cell_bytes + (long long)e.node * (long long)node_bytes;
        if (off > INT32_MAX || off < INT32_MIN) return noalloc_fail(GPE_ERR_INVALID_ARG, "grid too large for 32-bit offsets");
        tab.nb_off[f] = (int32_t)off;
        tab.w[f] = (-0.5 * e.hodge) / bs2;
    }
    for (int i = 0; i < 3 * V; ++i) tab.pos[i] = lat->pos[i];

    StepArgs a;
    std::memset(&a, 0, sizeof a);
    a.prev = static_cast<const char*>(psi);
    a.g.X = p->dims[0];
    a.g.Y = p->dims[1];
    a.g.Z = p->dims[2];
    a.g.V = V;
    a.g.C = p->components;
    a.g.pitch = pitch;
    a.g.slice = slice_pitch;
    a.g.cell_bytes = (uint32_t)cell_bytes;
    a.row_items = a.g.X * a.g.V;
    a.divV = make_fastdiv(a.g.V);
    a.divRow = make_fastdiv(a.row_items);
    a.divY = make_fastdiv(a.g.Y);
    a.total = sites;
    PhysR<double>& P = a.pd;
    gpe_fields B;
    std::memset(&B, 0, sizeof B);
    if (fields) B = *fields;
    for (int i = 0; i < 3; ++i) {
        P.p0[i] = p->p0[i];
        P.bw[i] = lat->block_width[i];
        P.lambda[i] = p->trap_lambda[i];
        P.qc[i] = p->quad_center[i];
        P.bb[i] = B.bb[i];
        P.bbq[i] = B.bb_quad[i];
    }
    P.bs = p->block_scale;
    P.trap_offset = p->trap_offset;
    P.c0 = p->c0;
    P.c2 = p->c2;
    P.c4 = p->c4;
    P.alpha = p->alpha;
    P.sigma = p->sigma;
    P.bq = B.bq;
    P.bqq = B.bq_quad;
    P.dt = p->dt;
    P.flags = p->flags;
    P.trap_on = !((p->flags & GPE_FLAG_TRAP_OFF_AFTER) && t >= p->trap_off_time);

    const uint64_t want = (sites + 255) / 256;
    const unsigned nb = (unsigned)(want < (uint64_t)OBS_NOALLOC_BLOCKS ? want : (uint64_t)OBS_NOALLOC_BLOCKS);
    cudaStream_t s = (cudaStream_t)stream;
    double* result = scratch + (size_t)OBS_NOALLOC_BLOCKS * OBS_COUNT;
    const bool fp64 = p->precision == GPE_FP64;
    switch (p->components) {
        case 1:
            if (fp64) observe_noalloc_kernel<double, 1><<<nb, 256, 0, s>>>(a, tab, scratch);
            else observe_noalloc_kernel<float, 1><<<nb, 256, 0, s>>>(a, tab, scratch);
            break;
        case 3:
            if (fp64) observe_noalloc_kernel<double, 3><<<nb, 256, 0, s>>>(a, tab, scratch);
            else observe_noalloc_kernel<float, 3><<<nb, 256, 0, s>>>(a, tab, scratch);
            break;
        default:
            if (fp64) observe_noalloc_kernel<double, 5><<<nb, 256, 0, s>>>(a, tab, scratch);
            else observe_noalloc_kernel<float, 5><<<nb, 256, 0, s>>>(a, tab, scratch);
            break;
    }
    observe_finalize_kernel<<<1, 256, 0, s>>>(scratch, nb, result);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(GPE_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    double r[OBS_COUNT];
    e = cudaMemcpyAsync(r, result, sizeof r, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return noalloc_fail(GPE_ERR_CUDA, std::string("result copy: ") + cudaGetErrorString(e));
    const double dv = p->block_scale * p->block_scale * p->block_scale * lat->volume;
    std::memset(out, 0, sizeof *out);
    out->norm = r[OBS_NORM] * dv;
    out->h_expect = r[OBS_HEXP] * dv;
    out->energy = (r[OBS_HEXP] - 0.5 * r[OBS_EINT]) * dv;
    out->magnetization[0] = r[OBS_MAGX] * dv;
    out->magnetization[1] = r[OBS_MAGY] * dv;
    out->magnetization[2] = r[OBS_MAGZ] * dv;
    out->spin_norm = r[OBS_SPIN] * dv;
    out->com[0] = r[OBS_COMX] * dv;
    out->com[1] = r[OBS_COMY] * dv;
    out->com[2] = r[OBS_COMZ] * dv;
    out->max_abs = r[OBS_MAXABS];
    out->nonfinite = (int32_t)r[OBS_NONFINITE];
    if (out->nonfinite) return noalloc_fail(GPE_ERR_NONFINITE, "state holds non-finite values");
    return GPE_OK;
}
