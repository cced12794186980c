// gpe_capi.cu -- host implementation of the libgpe C ABI (include/gpe.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "gpe_handle.h"

namespace gpe {
template <typename R, int C>
cudaError_t launch_parabolic(const StepArgs& a, int mode, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_hyper(const StepArgs& a, int kind, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_observe(const StepArgs& a, double* out, bool node_fp32, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_scale(const StepArgs& a, const double* norm_sum, double dv, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_norm(const StepArgs& a, double* out, cudaStream_t s);
cudaError_t launch_dot(const StepArgs& a, int precision, int C, double* out, cudaStream_t s);
struct InitArgs {
    double zeta[5][2];
    double mu, c0inv, noise_abs, noise_rel;
    int kappa;
    uint64_t seed;
};
template <typename R, int C>
cudaError_t launch_init(const StepArgs& a, const InitArgs& in, cudaStream_t s);
struct RespinArgs {
    double w[5];
    double u[5][2];
};
template <typename R, int C>
cudaError_t launch_respin(const StepArgs& a, const RespinArgs& r, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_leapfrog_tile(const StepArgs& a, uint32_t T, int carveout, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_leapfrog_rows(const StepArgs& a, uint32_t T, uint32_t RY, uint32_t RZ, uint32_t K, uint32_t nbuf,
                                 const int32_t* blk, uint32_t threads, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_hyper_tile(const StepArgs& a, uint32_t T, cudaStream_t s);
template <typename R>
cudaError_t launch_split(const StepArgs& a, int part, double qinit, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_leapfrog_march(const StepArgs& a, uint32_t T, uint32_t TY, uint32_t ZC, uint32_t threads, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_parabolic_slab(const StepArgs& a, uint32_t Tx, uint32_t Ty, uint32_t S, cudaStream_t s);
template <typename R, int C>
cudaError_t launch_parabolic_observe(const StepArgs& a, double* out, cudaStream_t s);
template <int C>
cudaError_t launch_il_step(const StepArgs& a, const ILGrid& G, int deg, size_t max_blocks, bool obs, double* out,
                           cudaStream_t s);
template <int C>
unsigned il_blocks(const ILGrid& G, int deg, bool obs, size_t max_blocks);
cudaError_t launch_il_convert(char* aos, const Grid& g, char* il, const ILGrid& G, bool to_il, cudaStream_t s);
template <int C>
cudaError_t launch_il_hyper(const StepArgs& a, const ILGrid& G, const ILGrid& Gq, const int32_t* tab, cudaStream_t s);
enum HyperKind {
    HK_FUSED_LEAPFROG = 0,
    HK_PSI_PARA_LEAPFROG,
    HK_PSI_PARA_EULER,
    HK_PSI_HYPER_EULER,
    HK_PSI_PARA_ITP,
    HK_Q_PARA,
    HK_Q_EULER_HYPER,
    HK_Q_HYPER,
    HK_FUSED_ITP
};
}  // namespace gpe

using namespace gpe;

static thread_local std::string g_last_error = "";

gpe_status gpe::fail(gpe_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

gpe_status gpe::cuda_fail(cudaError_t e, const char* where) {
    return fail(GPE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(expr)                                    \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
    } while (0)

extern "C" const char* gpe_last_error(void) { return g_last_error.c_str(); }

void gpe::set_last_error(const std::string& msg) { g_last_error = msg; }
extern "C" const char* gpe_version(void) { return "libgpe 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ lattices

extern "C" gpe_status gpe_lattice_create(const gpe_lattice_desc* d, gpe_lattice** out) {
    if (!d || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (d->nodes <= 0 || d->nodes > kMaxNodes) return fail(GPE_ERR_INVALID_ARG, "nodes out of range");
    if (!d->pos || !d->row_ptr || !d->stencil) return fail(GPE_ERR_INVALID_ARG, "missing table");
    if (!(d->volume > 0) || !(d->block_width[0] > 0) || !(d->block_width[1] > 0) || !(d->block_width[2] > 0))
        return fail(GPE_ERR_INVALID_ARG, "bad block width or volume");
    const int V = d->nodes;
    if (d->row_ptr[0] != 0) return fail(GPE_ERR_INVALID_ARG, "row_ptr[0] != 0");
    for (int l = 0; l < V; ++l)
        if (d->row_ptr[l + 1] < d->row_ptr[l]) return fail(GPE_ERR_INVALID_ARG, "row_ptr not monotone");
    const int n = d->row_ptr[V];
    if (n <= 0 || n > kMaxEntries) return fail(GPE_ERR_INVALID_ARG, "stencil size out of range");
    auto off_ok = [](int a) { return a >= -1 && a <= 1; };
    for (int f = 0; f < n; ++f) {
        const gpe_stencil_entry& e = d->stencil[f];
        if (!off_ok(e.dx) || !off_ok(e.dy) || !off_ok(e.dz)) return fail(GPE_ERR_INVALID_ARG, "stencil offset not in {-1,0,1}");
        if (e.node < 0 || e.node >= V) return fail(GPE_ERR_INVALID_ARG, "stencil node out of range");
        if (!std::isfinite(e.hodge)) return fail(GPE_ERR_INVALID_ARG, "non-finite hodge");
    }
    // symmetry of the neighbour graph: (l -> d, m) implies (m -> -d, l)
    for (int l = 0; l < V; ++l)
        for (int f = d->row_ptr[l]; f < d->row_ptr[l + 1]; ++f) {
            const gpe_stencil_entry& e = d->stencil[f];
            bool found = false;
            for (int g = d->row_ptr[e.node]; g < d->row_ptr[e.node + 1] && !found; ++g) {
                const gpe_stencil_entry& r = d->stencil[g];
                found = r.node == l && r.dx == -e.dx && r.dy == -e.dy && r.dz == -e.dz;
            }
            if (!found) return fail(GPE_ERR_INVALID_ARG, "stencil is not symmetric");
        }
    gpe_lattice* L = new (std::nothrow) gpe_lattice();
    if (!L) return fail(GPE_ERR_OOM, "host allocation");
    L->V = V;
    for (int i = 0; i < 3; ++i) L->bw[i] = d->block_width[i];
    L->volume = d->volume;
    L->pos.assign(d->pos, d->pos + 3 * V);
    L->row_ptr.assign(d->row_ptr, d->row_ptr + V + 1);
    L->stencil.assign(d->stencil, d->stencil + n);
    if (d->edges > 0) {
        if (d->edges > kMaxEdges || d->faces_per_node <= 0 || d->faces_per_node > kMaxFaces || !d->edge_table ||
            !d->incidence) {
            delete L;
            return fail(GPE_ERR_INVALID_ARG, "bad edge tables");
        }
        for (int e = 0; e < d->edges; ++e) {
            const gpe_edge& r = d->edge_table[e];
            if (r.from < 0 || r.from >= V || r.to < 0 || r.to >= V || !off_ok(r.dx) || !off_ok(r.dy) || !off_ok(r.dz)) {
                delete L;
                return fail(GPE_ERR_INVALID_ARG, "edge table entry out of range");
            }
        }
        for (int i = 0; i < V * d->faces_per_node; ++i) {
            const gpe_incidence& r = d->incidence[i];
            if (r.edge < 0 || r.edge >= d->edges || !off_ok(r.dx) || !off_ok(r.dy) || !off_ok(r.dz)) {
                delete L;
                return fail(GPE_ERR_INVALID_ARG, "incidence entry out of range");
            }
        }
        L->E = d->edges;
        L->F = d->faces_per_node;
        L->edges.assign(d->edge_table, d->edge_table + d->edges);
        L->incidence.assign(d->incidence, d->incidence + V * d->faces_per_node);
    }
    *out = L;
    return GPE_OK;
}

extern "C" void gpe_lattice_destroy(gpe_lattice* lat) { delete lat; }

// ------------------------------------------------------------------- ramps

extern "C" gpe_status gpe_ramp_eval(const gpe_ramp* r, double tau, gpe_fields* out) {
    if (!r || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (r->bq_segments < 0 || r->bq_segments > GPE_RAMP_MAX_SEGMENTS || r->bb_segments < 0 ||
        r->bb_segments > GPE_RAMP_MAX_SEGMENTS)
        return fail(GPE_ERR_INVALID_ARG, "segment count out of range");
    ramp_eval(*r, tau, *out);
    return GPE_OK;
}

// ----------------------------------------------------------------- handles

static size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

template <typename T>
static gpe_status upload_table(gpe_handle* h, const std::vector<T>& v, T** out) {
    *out = nullptr;
    if (v.empty()) return GPE_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, v.size() * sizeof(T));
    if (e != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (tables)");
    h->dev_tables.push_back(p);
    e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy (tables)");
    *out = static_cast<T*>(p);
    return GPE_OK;
}

static void release(gpe_handle* h) {
    for (int i = 0; i < 5; ++i)
        if (h->alloc[i]) cudaFree(h->alloc[i]);
    for (void* p : h->dev_tables) cudaFree(p);
    if (h->partials) cudaFree(h->partials);
    if (h->obs_out) cudaFree(h->obs_out);
    if (h->stage) cudaFree(h->stage);
    if (h->field_buf) cudaFree(h->field_buf);
    if (h->err) cudaFree(h->err);
    if (h->blk) cudaFree(h->blk);
    for (char* b : h->il)
        if (b) cudaFree(b);
    for (char* b : h->ilq)
        if (b) cudaFree(b);
    if (h->il_htab) cudaFree(h->il_htab);
    if (h->tev_ok)
        for (cudaEvent_t ev : h->tev) cudaEventDestroy(ev);
    adjoint_release(h);
}

static gpe_status build_tables(gpe_handle* h) {
    const gpe_lattice& L = h->lat;
    const Grid& g = h->g;
    const double bs2 = h->p.block_scale * h->p.block_scale;
    const size_t node_bytes = (size_t)g.C * 2 * h->real_bytes;
    const int n = (int)L.stencil.size();
    std::vector<int32_t> nb_off(n), nb_soff(n);
    std::vector<double> w64(n);
    std::vector<float> w32(n);
    for (int f = 0; f < n; ++f) {
        const gpe_stencil_entry& e = L.stencil[f];
        const long long off = (long long)e.dz * (long long)g.slice + (long long)e.dy * (long long)g.pitch +
                              (long long)e.dx * g.cell_bytes + (long long)e.node * node_bytes;
        if (off > INT32_MAX || off < INT32_MIN) return fail(GPE_ERR_INVALID_ARG, "grid too large for 32-bit offsets");
        nb_off[f] = (int32_t)off;
        // offset inside a contiguous row of cells (row-tile kernel), or off-row marker
        nb_soff[f] = (e.dy == 0 && e.dz == 0) ? (int32_t)((long long)e.dx * g.cell_bytes + (long long)e.node * node_bytes)
                                              : INT32_MIN;
        w64[f] = (-0.5 * e.hodge) / bs2;  // hodges[i] = -0.5*hodges[i]; hodge/(bs*bs) (Spin1GpeBCC.cu:1169, :859)
        w32[f] = (float)w64[f];
    }
    std::vector<int4> ent4(n);
    for (int f = 0; f < n; ++f) ent4[f] = make_int4(L.stencil[f].dx, L.stencil[f].dy, L.stencil[f].dz, L.stencil[f].node);
    int udeg = L.row_ptr[1] - L.row_ptr[0];
    for (int l = 0; l < L.V; ++l)
        if (L.row_ptr[l + 1] - L.row_ptr[l] != udeg) udeg = 0;
    h->tab.uniform_deg = udeg;
    // rows of different lengths, all multiples of 4 (FCC's 4 and 8): read in vectors of 4
    bool quad = udeg == 0;
    for (int l = 0; l < L.V && quad; ++l) {
        const int len = L.row_ptr[l + 1] - L.row_ptr[l];
        quad = len > 0 && len % 4 == 0;
    }
    h->tab.quad_rows = quad ? 1 : 0;
    h->tab.max_deg = 0;
    for (int l = 0; l < L.V; ++l) h->tab.max_deg = std::max(h->tab.max_deg, L.row_ptr[l + 1] - L.row_ptr[l]);
    // rows (dy, dz) touched by the stencil, the own row first
    h->nrows = 1;
    h->rdy[0] = h->rdz[0] = 0;
    for (int f = 0; f < n; ++f) {
        const int dy = L.stencil[f].dy, dz = L.stencil[f].dz;
        bool seen = false;
        for (uint32_t r = 0; r < h->nrows; ++r) seen = seen || (h->rdy[r] == dy && h->rdz[r] == dz);
        if (!seen && h->nrows < 9) {
            h->rdy[h->nrows] = dy;
            h->rdz[h->nrows] = dz;
            h->nrows++;
        }
    }
    std::vector<double> pos64(L.pos);
    std::vector<float> pos32(L.pos.begin(), L.pos.end());
    gpe_status st;
    if ((st = upload_table(h, L.row_ptr, &h->tab.row_ptr))) return st;
    if ((st = upload_table(h, nb_off, &h->tab.nb_off))) return st;
    if ((st = upload_table(h, nb_soff, &h->tab.nb_soff))) return st;
    if ((st = upload_table(h, ent4, &h->tab.ent4))) return st;
    std::vector<int32_t> ent_row(n, 0);
    for (int f = 0; f < n; ++f)
        for (uint32_t r = 0; r < h->nrows; ++r)
            if (h->rdy[r] == L.stencil[f].dy && h->rdz[r] == L.stencil[f].dz) ent_row[f] = (int32_t)r;
    if ((st = upload_table(h, ent_row, &h->tab.ent_row))) return st;
    if ((st = upload_table(h, w64, &h->tab.w64))) return st;
    if ((st = upload_table(h, w32, &h->tab.w32))) return st;
    if ((st = upload_table(h, pos64, &h->tab.pos64))) return st;
    if ((st = upload_table(h, pos32, &h->tab.pos32))) return st;
    h->tab.entries = n;
    if (L.E > 0) {
        const int F = L.F;
        std::vector<int32_t> inc_off(L.V * F), efrom(L.E), eto(L.E), inc_soff(L.V * F), eto_s(L.E);
        std::vector<double> iw64(L.V * F);
        std::vector<float> iw32(L.V * F);
        for (int i = 0; i < L.V * F; ++i) {
            const gpe_incidence& r = L.incidence[i];
            const long long off = (long long)r.dz * (long long)g.qslice + (long long)r.dy * (long long)g.qpitch +
                                  (long long)r.dx * g.qcell_bytes + (long long)r.edge * node_bytes;
            if (off > INT32_MAX || off < INT32_MIN) return fail(GPE_ERR_INVALID_ARG, "grid too large for 32-bit offsets");
            inc_off[i] = (int32_t)off;
            inc_soff[i] = (r.dy == 0 && r.dz == 0) ? (int32_t)((long long)r.dx * g.qcell_bytes + (long long)r.edge * node_bytes)
                                                  : INT32_MIN;
            iw64[i] = (-0.5 * r.hodge) / bs2;
            iw32[i] = (float)iw64[i];
        }
        for (int e = 0; e < L.E; ++e) {
            const gpe_edge& r = L.edges[e];
            efrom[e] = (int32_t)(r.from * node_bytes);
            const long long off = (long long)r.dz * (long long)g.slice + (long long)r.dy * (long long)g.pitch +
                                  (long long)r.dx * g.cell_bytes + (long long)r.to * node_bytes;
            if (off > INT32_MAX || off < INT32_MIN) return fail(GPE_ERR_INVALID_ARG, "grid too large for 32-bit offsets");
            eto[e] = (int32_t)off;
            eto_s[e] = (r.dy == 0 && r.dz == 0) ? (int32_t)((long long)r.dx * g.cell_bytes + (long long)r.to * node_bytes)
                                                : INT32_MIN;
        }
        if ((st = upload_table(h, inc_off, &h->tab.inc_off))) return st;
        if ((st = upload_table(h, iw64, &h->tab.inc_w64))) return st;
        if ((st = upload_table(h, iw32, &h->tab.inc_w32))) return st;
        if ((st = upload_table(h, efrom, &h->tab.e_from_off))) return st;
        if ((st = upload_table(h, eto, &h->tab.e_to_off))) return st;
        if ((st = upload_table(h, eto_s, &h->tab.e_to_soff))) return st;
        if ((st = upload_table(h, inc_soff, &h->tab.inc_soff))) return st;
        h->tab.faces = F;
    }
    return GPE_OK;
}

extern "C" gpe_status gpe_create(const gpe_lattice* lat, const gpe_params* p, gpe_handle** out) {
    if (!lat || !p || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (p->components != 1 && p->components != 3 && p->components != 5)
        return fail(GPE_ERR_INVALID_ARG, "components must be 1, 3 or 5");
    if (p->precision != GPE_FP32 && p->precision != GPE_FP64) return fail(GPE_ERR_INVALID_ARG, "precision");
    if (p->scheme != GPE_SCHEME_PARABOLIC && p->scheme != GPE_SCHEME_HYPERBOLIC && p->scheme != GPE_SCHEME_SPLIT)
        return fail(GPE_ERR_INVALID_ARG, "scheme");
    if (p->dims[0] == 0 || p->dims[1] == 0 || p->dims[2] == 0) return fail(GPE_ERR_INVALID_ARG, "empty grid");
    if (!(p->block_scale > 0) || !std::isfinite(p->dt)) return fail(GPE_ERR_INVALID_ARG, "block_scale/dt");
    if (p->scheme == GPE_SCHEME_HYPERBOLIC && (lat->E == 0 || !(p->sigma > 0)))
        return fail(GPE_ERR_UNSUPPORTED, "hyperbolic scheme needs edge tables and sigma > 0");
    if (p->scheme == GPE_SCHEME_SPLIT && (lat->E == 0 || !(p->sigma > 0) || p->components != 1))
        return fail(GPE_ERR_UNSUPPORTED, "split scheme needs C = 1, edge tables and sigma > 0");
    if (p->components == 5 && (p->flags & GPE_FLAG_QUADRATIC_ZEEMAN))
        return fail(GPE_ERR_UNSUPPORTED, "quadratic Zeeman is not built for spin-2");
    const uint64_t sites = (uint64_t)p->dims[0] * p->dims[1] * p->dims[2] * (uint64_t)lat->V;
    const uint64_t esites = (uint64_t)p->dims[0] * p->dims[1] * p->dims[2] * (uint64_t)lat->E;
    if (sites >= (1ull << 32) || esites >= (1ull << 32)) return fail(GPE_ERR_INVALID_ARG, "grid exceeds 2^32 sites");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GPE_ERR_NO_DEVICE, "no CUDA device");

    gpe_handle* h = new (std::nothrow) gpe_handle();
    if (!h) return fail(GPE_ERR_OOM, "host allocation");
    h->lat = *lat;
    h->p = *p;
    cudaGetDevice(&h->device);
    h->real_bytes = p->precision == GPE_FP64 ? 8 : 4;
    Grid& g = h->g;
    g.X = p->dims[0];
    g.Y = p->dims[1];
    g.Z = p->dims[2];
    g.V = lat->V;
    g.C = p->components;
    g.E = lat->E;
    g.cell_bytes = (uint32_t)(g.V * g.C * 2 * h->real_bytes);
    g.qcell_bytes = (uint32_t)(g.E * g.C * 2 * h->real_bytes);
    g.pitch = round_up((size_t)(g.X + 2) * g.cell_bytes, 256);
    g.slice = g.pitch * (g.Y + 2);
    g.qpitch = g.E ? round_up((size_t)(g.X + 2) * g.qcell_bytes, 256) : 0;
    g.qslice = g.qpitch * (g.Y + 2);

    const bool hyper = p->scheme != GPE_SCHEME_PARABOLIC;  // q buffers
    for (int slot = 0; slot < 5; ++slot) {
        const bool is_q = slot == GPE_Q_EVEN || slot == GPE_Q_ODD;
        if (is_q && !hyper) continue;
        if (slot == GPE_HPSI) continue;  // allocated on first use (ITP)
        const size_t bytes = (is_q ? g.qslice : g.slice) * (g.Z + 2);
        cudaError_t e = cudaMalloc(&h->alloc[slot], bytes);
        if (e != cudaSuccess) {
            release(h);
            delete h;
            return fail(GPE_ERR_OOM, "cudaMalloc of a state buffer failed");
        }
        h->alloc_bytes[slot] = bytes;
        cudaMemset(h->alloc[slot], 0, bytes);
        h->interior[slot] = static_cast<char*>(h->alloc[slot]) + (is_q ? g.qslice + g.qpitch + g.qcell_bytes
                                                                          : g.slice + g.pitch + g.cell_bytes);
    }
    gpe_status st = build_tables(h);
    if (st != GPE_OK) {
        release(h);
        delete h;
        return st;
    }
    // block partial sums: one row per 256 sites, and at least a wave of the
    // interleaved observed step's blocks on small grids
    h->partial_blocks = std::max<size_t>((sites + 255) / 256, 2048);
    if (cudaMalloc(&h->partials, h->partial_blocks * OBS_COUNT * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->obs_out, OBS_COUNT * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->err, sizeof(int)) != cudaSuccess || cudaMemset(h->err, 0, sizeof(int)) != cudaSuccess) {
        release(h);
        delete h;
        return fail(GPE_ERR_OOM, "cudaMalloc of reduction scratch failed");
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        release(h);
        delete h;
        return cuda_fail(e, "gpe_create");
    }
    // the reference loads the initial state into the odd buffer (Spin1GpeBCC.cu:1236);
    // the split scheme keeps R + iI in PSI_EVEN and q_R + i q_I in Q_EVEN
    h->cur = p->scheme == GPE_SCHEME_SPLIT ? GPE_PSI_EVEN : GPE_PSI_ODD;
    *out = h;
    return GPE_OK;
}

extern "C" gpe_status gpe_destroy(gpe_handle* h) {
    if (!h) return GPE_OK;
    release(h);
    delete h;
    return GPE_OK;
}

static bool slot_ok(const gpe_handle* h, int slot) { return slot >= 0 && slot < 5 && h->alloc[slot] != nullptr; }

static gpe_status ensure_hpsi(gpe_handle* h) {
    if (h->alloc[GPE_HPSI]) return GPE_OK;
    const size_t bytes = h->g.slice * (h->g.Z + 2);
    if (cudaMalloc(&h->alloc[GPE_HPSI], bytes) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (H psi)");
    cudaMemset(h->alloc[GPE_HPSI], 0, bytes);
    h->alloc_bytes[GPE_HPSI] = bytes;
    h->interior[GPE_HPSI] = static_cast<char*>(h->alloc[GPE_HPSI]) + h->g.slice + h->g.pitch + h->g.cell_bytes;
    return GPE_OK;
}

extern "C" gpe_status gpe_buffer(const gpe_handle* h, int32_t slot, gpe_pitched* out, size_t* cell_bytes) {
    if (!h || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (!slot_ok(h, slot)) return fail(GPE_ERR_INVALID_ARG, "slot not allocated");
    const bool is_q = slot == GPE_Q_EVEN || slot == GPE_Q_ODD;
    out->ptr = h->interior[slot];
    out->pitch = is_q ? h->g.qpitch : h->g.pitch;
    out->slice_pitch = is_q ? h->g.qslice : h->g.slice;
    if (cell_bytes) *cell_bytes = is_q ? h->g.qcell_bytes : h->g.cell_bytes;
    return GPE_OK;
}

size_t gpe::host_count(const gpe_handle* h, bool is_q) {
    const Grid& g = h->g;
    return (size_t)(g.X + 2) * (g.Y + 2) * (g.Z + 2) * (is_q ? g.E : g.V) * g.C * 2;
}

// A bounded device wait that ran out sets the handle's error flag; surface it.
gpe_status gpe::check_device_error(gpe_handle* h, cudaStream_t s) {
    int flag = 0;
    CUDA_TRY(cudaMemcpyAsync(&flag, h->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (flag) {
        cudaMemsetAsync(h->err, 0, sizeof(int), s);
        return fail(GPE_ERR_TIMEOUT, "a bounded device wait ran out (bulk copy did not complete)");
    }
    return GPE_OK;
}

gpe_status gpe::ensure_stage(gpe_handle* h, size_t count) {
    if (h->stage_count >= count) return GPE_OK;
    if (h->stage) cudaFree(h->stage);
    h->stage = nullptr;
    h->stage_count = 0;
    if (cudaMalloc(&h->stage, count * sizeof(double)) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (staging)");
    h->stage_count = count;
    return GPE_OK;
}

// Host FP64 (reference file layout) <-> device buffer.  The host array is copied
// as is into a device FP64 staging buffer and converted/unpacked by a kernel, so
// a pinned host buffer moves at full link speed and no host-side conversion pass
// is needed.
static gpe_status transfer(gpe_handle* h, int32_t slot, double* host, size_t count, void* stream, bool up) {
    if (!h || !host) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (up) h->epoch += 1;
    if (up && slot == GPE_HPSI) {
        gpe_status st = ensure_hpsi(h);
        if (st) return st;
    }
    if (!slot_ok(h, slot)) return fail(GPE_ERR_INVALID_ARG, "slot not allocated");
    const bool is_q = slot == GPE_Q_EVEN || slot == GPE_Q_ODD;
    if (count != host_count(h, is_q)) return fail(GPE_ERR_INVALID_ARG, "host buffer size does not match the grid");
    const Grid& g = h->g;
    const uint32_t vals = (uint32_t)((is_q ? g.qcell_bytes : g.cell_bytes) / h->real_bytes);
    const size_t pitch = is_q ? g.qpitch : g.pitch;
    const size_t slice = is_q ? g.qslice : g.slice;
    cudaStream_t s = (cudaStream_t)stream;
    // pinned (page-locked, device-mapped) host arrays are read or written by the
    // pack kernel itself over the host link, without the staging copy
    // (GPE_TUNE_TRANSFER 1: a DMA copy through the staging buffer instead, which
    // leaves the SMs to other streams' kernels while the copy runs)
    double* mapped = nullptr;
    cudaPointerAttributes attr;
    if (h->tune_transfer == 0 && cudaPointerGetAttributes(&attr, host) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
        attr.devicePointer)
        mapped = static_cast<double*>(attr.devicePointer);
    else
        cudaGetLastError();  // an unregistered pointer is not an error here
    if (!mapped) {
        gpe_status st = ensure_stage(h, count);
        if (st) return st;
    }
    if (up && !mapped) CUDA_TRY(cudaMemcpyAsync(h->stage, host, count * sizeof(double), cudaMemcpyHostToDevice, s));
    cudaError_t e = launch_pack_any(h->p.precision, mapped ? mapped : h->stage, static_cast<char*>(h->alloc[slot]), g.X,
                                    g.Y, g.Z, vals, pitch, slice, up, s);
    if (e != cudaSuccess) return cuda_fail(e, "pack kernel");
    h->launches += 1;
    if (!up && !mapped) CUDA_TRY(cudaMemcpyAsync(host, h->stage, count * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    return up ? GPE_OK : check_device_error(h, s);
}

extern "C" gpe_status gpe_upload(gpe_handle* h, int32_t slot, const double* host, size_t count, void* stream) {
    return transfer(h, slot, const_cast<double*>(host), count, stream, true);
}

extern "C" gpe_status gpe_download(gpe_handle* h, int32_t slot, double* host, size_t count, void* stream) {
    return transfer(h, slot, host, count, stream, false);
}

extern "C" gpe_status gpe_set_ramp(gpe_handle* h, const gpe_ramp* ramp, double t0) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if (ramp) {
        gpe_fields tmp;
        gpe_status st = gpe_ramp_eval(ramp, 0.0, &tmp);
        if (st) return st;
        h->ramp = *ramp;
        h->has_ramp = true;
    } else {
        h->has_ramp = false;
    }
    h->t0 = t0;
    h->nstep = 0;
    return GPE_OK;
}

static gpe_fields fields_at(const gpe_handle* h, double t) {
    gpe_fields f;
    std::memset(&f, 0, sizeof f);
    if (h->has_ramp) gpe_ramp_eval(&h->ramp, h->ramp.time_scale * t, &f);
    return f;
}

template <typename R>
static void fill_phys(PhysR<R>& P, const Phys& ph, const gpe_fields& B, double t) {
    for (int i = 0; i < 3; ++i) {
        P.p0[i] = (R)ph.p0[i];
        P.bw[i] = (R)ph.bw[i];
        P.lambda[i] = (R)ph.lambda[i];
        P.qc[i] = (R)ph.quad_center[i];
        P.bb[i] = (R)B.bb[i];
        P.bbq[i] = (R)B.bb_quad[i];
    }
    P.bs = (R)ph.bs;
    P.trap_offset = (R)ph.trap_offset;
    P.c0 = (R)ph.c0;
    P.c2 = (R)ph.c2;
    P.c4 = (R)ph.c4;
    P.alpha = (R)ph.alpha;
    P.sigma = (R)ph.sigma;
    P.bq = (R)B.bq;
    P.bqq = (R)B.bq_quad;
    P.dt = (R)ph.dt;
    P.dts = ph.sigma > 0 ? (R)(ph.dt / ph.sigma) : (R)0;
    P.ks = (R)ph.ks;
    P.flags = ph.flags;
    P.trap_on = !((ph.flags & GPE_FLAG_TRAP_OFF_AFTER) && t >= ph.trap_off_time);
}

StepArgs gpe::make_args(const gpe_handle* h, const gpe_fields& B, double t) {
    StepArgs a;
    std::memset(&a, 0, sizeof a);
    a.g = h->g;
    a.tab = h->tab;
    const gpe_params& p = h->p;
    for (int i = 0; i < 3; ++i) {
        a.ph.p0[i] = p.p0[i];
        a.ph.bw[i] = h->lat.bw[i];
        a.ph.lambda[i] = p.trap_lambda[i];
        a.ph.quad_center[i] = p.quad_center[i];
    }
    // condensate expansion (Spin1GpeBCC.cu:1579-1582): block scale bs(t) = bs0 (1 +
    // rate (t - t_start)) from t_start on; positions use bs(t), the Laplacian h / bs^2
    a.ph.bs = p.block_scale;
    a.ph.ks = 1.0;
    if (h->exp_rate != 0 && t >= h->exp_t0) {
        a.ph.bs = p.block_scale * (1.0 + h->exp_rate * (t - h->exp_t0));
        a.ph.ks = (p.block_scale / a.ph.bs) * (p.block_scale / a.ph.bs);
    }
    a.ph.dt = p.dt;
    a.ph.trap_offset = p.trap_offset;
    a.ph.trap_off_time = p.trap_off_time;
    a.ph.c0 = p.c0;
    a.ph.c2 = p.c2;
    a.ph.c4 = p.c4;
    a.ph.alpha = p.alpha;
    a.ph.sigma = p.sigma;
    a.ph.flags = p.flags;
    a.B = B;
    a.t = t;
    const Grid& g = h->g;
    a.row_items = g.X * g.V;
    a.row_items_e = g.X * g.E;
    a.divV = make_fastdiv(g.V);
    a.divRow = make_fastdiv(a.row_items);
    a.divY = make_fastdiv(g.Y);
    a.divE = make_fastdiv(g.E ? g.E : 1);
    a.divRowE = make_fastdiv(a.row_items_e ? a.row_items_e : 1);
    a.total = (uint64_t)g.X * g.Y * g.Z * g.V;
    a.partials = h->partials;
    a.err = h->err;
    fill_phys(a.pf, a.ph, B, t);
    fill_phys(a.pd, a.ph, B, t);
    return a;
}

template <int C>
static cudaError_t dispatch_parabolic_c(const gpe_handle* h, const StepArgs& a, int mode, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_parabolic<double, C>(a, mode, s) : launch_parabolic<float, C>(a, mode, s);
}
static cudaError_t dispatch_parabolic(const gpe_handle* h, const StepArgs& a, int mode, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_parabolic_c<1>(h, a, mode, s);
        case 3: return dispatch_parabolic_c<3>(h, a, mode, s);
        default: return dispatch_parabolic_c<5>(h, a, mode, s);
    }
}
template <int C>
static cudaError_t dispatch_hyper_c(const gpe_handle* h, const StepArgs& a, int kind, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_hyper<double, C>(a, kind, s) : launch_hyper<float, C>(a, kind, s);
}
static cudaError_t dispatch_hyper(const gpe_handle* h, const StepArgs& a, int kind, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_hyper_c<1>(h, a, kind, s);
        case 3: return dispatch_hyper_c<3>(h, a, kind, s);
        default: return dispatch_hyper_c<5>(h, a, kind, s);
    }
}
// One launch of the split scheme on PSI_EVEN / Q_EVEN (part 0, 1: half-steps; 2: start).
static gpe_status split_launch(gpe_handle* h, int part, double t, cudaStream_t s) {
    gpe_fields zero;
    std::memset(&zero, 0, sizeof zero);
    StepArgs a = make_args(h, zero, t);
    a.prev = a.next = h->interior[GPE_PSI_EVEN];
    a.q = a.qnext = h->interior[GPE_Q_EVEN];
    const double dts = h->p.dt / h->p.sigma;
    const double qinit = dts / (h->p.dt - dts);
    cudaError_t e = h->real_bytes == 8 ? launch_split<double>(a, part, qinit, s) : launch_split<float>(a, part, qinit, s);
    h->launches += 1;
    if (e != cudaSuccess) return cuda_fail(e, "split-scheme launch");
    return GPE_OK;
}

template <int C>
static cudaError_t dispatch_observe_c(const gpe_handle* h, const StepArgs& a, double* out, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_observe<double, C>(a, out, false, s)
                              : launch_observe<float, C>(a, out, h->tune_observe != 0, s);
}
static cudaError_t dispatch_observe(const gpe_handle* h, const StepArgs& a, double* out, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_observe_c<1>(h, a, out, s);
        case 3: return dispatch_observe_c<3>(h, a, out, s);
        default: return dispatch_observe_c<5>(h, a, out, s);
    }
}
template <int C>
static cudaError_t dispatch_norm_c(const gpe_handle* h, const StepArgs& a, double* out, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_norm<double, C>(a, out, s) : launch_norm<float, C>(a, out, s);
}
// sum |psi|^2 of a.prev into out[OBS_NORM] (the other entries zero)
static cudaError_t dispatch_norm(const gpe_handle* h, const StepArgs& a, double* out, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_norm_c<1>(h, a, out, s);
        case 3: return dispatch_norm_c<3>(h, a, out, s);
        default: return dispatch_norm_c<5>(h, a, out, s);
    }
}
template <int C>
static cudaError_t dispatch_scale_c(const gpe_handle* h, const StepArgs& a, const double* n, double dv, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_scale<double, C>(a, n, dv, s) : launch_scale<float, C>(a, n, dv, s);
}
static cudaError_t dispatch_scale(const gpe_handle* h, const StepArgs& a, const double* n, double dv, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_scale_c<1>(h, a, n, dv, s);
        case 3: return dispatch_scale_c<3>(h, a, n, dv, s);
        default: return dispatch_scale_c<5>(h, a, n, dv, s);
    }
}

// Shape of the 2.5-D z-march kernel (T = 0: not used).
struct MarchShape {
    uint32_t T = 0, TY = 0, ZC = 0, threads = 0;
};

static size_t march_smem(const gpe_handle* h, uint32_t T, uint32_t TY) {
    const size_t cb = h->g.cell_bytes;
    const size_t ent = 16;
    return 4 * (size_t)(TY + 2) * (T + 2) * cb + 2 * (size_t)TY * T * cb + h->lat.stencil.size() * ent +
           3 * h->g.V * h->real_bytes + (h->g.V + 1) * 4;
}

static MarchShape march_shape(const gpe_handle* h) {
    MarchShape m;
    if (h->tune_kernel != 3) return m;  // only on request: the multi-row kernel is faster where both apply
    if (h->g.cell_bytes % 16 != 0) return m;
    const uint32_t X = h->g.X, Y = h->g.Y, Z = h->g.Z, V = h->g.V;
    const size_t limit = 200 * 1024;
    auto fits = [&](uint32_t T, uint32_t TY) {
        return T > 0 && TY > 0 && X % T == 0 && Y % TY == 0 && march_smem(h, T, TY) <= limit && T * TY * V <= 8192;
    };
    uint32_t T = 0, TY = 0;
    if (h->tune_tile > 0 && h->tune_rows > 0) {
        if (fits((uint32_t)h->tune_tile, (uint32_t)h->tune_rows)) {
            T = (uint32_t)h->tune_tile;
            TY = (uint32_t)h->tune_rows;
        }
    } else if (h->tune_kernel == 3 || (X >= 8 && Y >= 2 && Z >= 8)) {
        // prefer about 192-384 nodes per row, two rows, the smallest halo overhead that fits
        const uint32_t tcand[] = {16, 32, 24, 12, 8, 20, 6, 4, 3, 2, 1};
        const uint32_t ycand[] = {2, 4, 3, 1};
        for (uint32_t ty : ycand) {
            for (uint32_t t : tcand)
                if (fits(t, ty) && t * V <= 512) {
                    T = t;
                    TY = ty;
                    break;
                }
            if (T) break;
        }
    }
    if (!T) return m;
    m.T = T;
    m.TY = TY;
    m.ZC = h->tune_zchunk > 0 ? (uint32_t)h->tune_zchunk : (Z >= 64 ? 32u : Z);
    if (m.ZC > Z) m.ZC = Z;
    const uint32_t nodes = T * TY * V;
    m.threads = nodes >= 1024 ? 1024 : ((nodes + 31) / 32) * 32;
    return m;
}

template <int C>
static cudaError_t dispatch_march_c(const gpe_handle* h, const StepArgs& a, const MarchShape& m, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_leapfrog_march<double, C>(a, m.T, m.TY, m.ZC, m.threads, s)
                              : launch_leapfrog_march<float, C>(a, m.T, m.TY, m.ZC, m.threads, s);
}
static cudaError_t dispatch_march(const gpe_handle* h, const StepArgs& a, const MarchShape& m, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_march_c<1>(h, a, m, s);
        case 3: return dispatch_march_c<3>(h, a, m, s);
        default: return dispatch_march_c<5>(h, a, m, s);
    }
}

// Shape of the slab-ring kernel (Tx = 0: not used); S: psi_prev ring slots (0:
// automatic).
struct SlabShape {
    uint32_t Tx = 0, Ty = 0, S = 0;
};

// Whether the slab kernel's rings fit for a Tx x Ty tile at two blocks per SM:
// S (at least four) psi_prev slabs within 110 KB.
static bool slab_slots(const gpe_handle* h, uint32_t Tx, uint32_t Ty, uint32_t S = 4) {
    const uint64_t slab = (uint64_t)(Tx + 2) * (Ty + 2) * h->g.cell_bytes;
    return S >= 4 && S <= 8 && S * slab <= 110ull * 1024;
}

// The slab-ring kernel applies to leapfrog steps on lattices whose nodes all have
// 4 stencil entries, with 16-byte cells.  Tile: Tx x Ty cells with Tx * Ty * V <=
// 384 threads and at least four slabs per block at two blocks per SM; by default
// the shape with the least halo per cell, whole tiles preferred, then larger tiles.
// GPE_TUNE_ZCHUNK, if set, is the number of psi_prev slabs.
static SlabShape slab_shape(const gpe_handle* h) {
    SlabShape r;
    if (h->tune_kernel != 5) return r;
    if (h->tab.uniform_deg != 4 || h->g.cell_bytes % 16 != 0) return r;
    const uint32_t V = h->g.V, X = h->g.X, Y = h->g.Y;
    const uint32_t S = h->tune_zchunk > 0 ? (uint32_t)h->tune_zchunk : 4u;
    if (h->tune_tile > 0 && h->tune_rows > 0) {
        const uint32_t Tx = (uint32_t)h->tune_tile, Ty = (uint32_t)h->tune_rows;
        if (Tx * Ty * V <= 384 && slab_slots(h, Tx, Ty, S)) {
            r.Tx = Tx;
            r.Ty = Ty;
            r.S = h->tune_zchunk > 0 ? S : 0;
        }
        return r;
    }
    double best = 1e30;
    for (uint32_t Ty = 1; Ty <= Y && Ty <= 16; ++Ty)
        for (uint32_t Tx = 1; Tx <= X && Tx * Ty * V <= 384; ++Tx) {
            if (!slab_slots(h, Tx, Ty, S)) continue;
            const double halo = (double)(Tx + 2) * (Ty + 2) / ((double)Tx * Ty);
            const bool whole = X % Tx == 0 && Y % Ty == 0;
            const double score = halo * (whole ? 1.0 : 1.25) - 1e-3 * Tx * Ty - 1e-4 * Tx;
            if (score < best) {
                best = score;
                r.Tx = Tx;
                r.Ty = Ty;
                r.S = h->tune_zchunk > 0 ? S : 0;
            }
        }
    return r;
}

template <int C>
static cudaError_t dispatch_slab_c(const gpe_handle* h, const StepArgs& a, const SlabShape& m, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_parabolic_slab<double, C>(a, m.Tx, m.Ty, m.S, s)
                              : launch_parabolic_slab<float, C>(a, m.Tx, m.Ty, m.S, s);
}
static cudaError_t dispatch_slab(const gpe_handle* h, const StepArgs& a, const SlabShape& m, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_slab_c<1>(h, a, m, s);
        case 3: return dispatch_slab_c<3>(h, a, m, s);
        default: return dispatch_slab_c<5>(h, a, m, s);
    }
}

// Row buffers a block of RY x RZ output rows needs: the distinct (y, z) rows
// (relative to the block origin) reached by the stencil's (dy, dz) offsets.
static void row_block_table(const gpe_handle* h, uint32_t RY, uint32_t RZ, std::vector<int32_t>& dy,
                            std::vector<int32_t>& dz, std::vector<int32_t>& map) {
    dy.clear();
    dz.clear();
    map.assign((size_t)RY * RZ * h->nrows, 0);
    for (uint32_t rz = 0; rz < RZ; ++rz)
        for (uint32_t ry = 0; ry < RY; ++ry)
            for (uint32_t k = 0; k < h->nrows; ++k) {
                const int32_t y = (int32_t)ry + h->rdy[k], z = (int32_t)rz + h->rdz[k];
                int32_t b = -1;
                for (size_t i = 0; i < dy.size() && b < 0; ++i)
                    if (dy[i] == y && dz[i] == z) b = (int32_t)i;
                if (b < 0) {
                    b = (int32_t)dy.size();
                    dy.push_back(y);
                    dz.push_back(z);
                }
                map[((size_t)rz * RY + ry) * h->nrows + k] = b;
            }
}

struct RowsShape {
    uint32_t T = 0, RY = 0, RZ = 0, nbuf = 0;
};

static size_t rows_smem(const gpe_handle* h, uint32_t T, uint32_t RY, uint32_t RZ, uint32_t nbuf) {
    const size_t cb = h->g.cell_bytes;
    return (size_t)nbuf * (T + 2) * cb + (size_t)RY * RZ * T * cb + h->lat.stencil.size() * (h->real_bytes == 8 ? 16 : 8) +
           3 * h->g.V * h->real_bytes + (h->g.V + 1) * 4 + (size_t)RY * RZ * h->nrows * 4;
}

// Multi-row tile kernel shape (T = 0: not used).
static RowsShape rows_shape(const gpe_handle* h) {
    RowsShape r;
    if (h->tune_kernel != 4) return r;  // on request or by the autotuner (the row tile is faster on BCC)
    if (h->g.cell_bytes % 16 != 0 || h->nrows == 0) return r;
    uint32_t cand[4][2] = {{2, 2}, {2, 1}, {1, 2}, {1, 1}};
    if (h->tune_rows > 0) {
        // explicit: RY = tune_rows, RZ = tune_zchunk (or 1)
        cand[0][0] = (uint32_t)h->tune_rows;
        cand[0][1] = h->tune_zchunk > 0 ? (uint32_t)h->tune_zchunk : 1u;
        for (int i = 1; i < 4; ++i) cand[i][0] = cand[i][1] = 0;
    }
    for (auto& c : cand) {
        const uint32_t RY = c[0], RZ = c[1];
        if (!RY || !RZ || h->g.Y % RY || h->g.Z % RZ) continue;
        uint32_t T = (uint32_t)h->tune_tile;
        if (T == 0) {
            // about 384 nodes per block, preferring a divisor of X
            const uint32_t want = 384 / (RY * RZ * h->g.V) > 0 ? 384 / (RY * RZ * h->g.V) : 1;
            T = want >= h->g.X ? h->g.X : want;
            for (uint32_t t = T; t * 2 > T && t > 0; --t)
                if (h->g.X % t == 0) {
                    T = t;
                    break;
                }
        }
        if (T == 0 || T > h->g.X) continue;
        if ((uint64_t)RY * RZ * T * h->g.V > 4096) continue;
        std::vector<int32_t> dy, dz, map;
        row_block_table(h, RY, RZ, dy, dz, map);
        if (rows_smem(h, T, RY, RZ, (uint32_t)dy.size()) > 200 * 1024) continue;
        r.T = T;
        r.RY = RY;
        r.RZ = RZ;
        r.nbuf = (uint32_t)dy.size();
        return r;
    }
    return r;
}

static uint32_t rows_cells(const gpe_handle* h) { return rows_shape(h).T; }

// Device copy of the row-block table for the shape (rebuilt when the shape changes).
static gpe_status ensure_row_block(gpe_handle* h, const RowsShape& r) {
    if (h->blk && h->blk_ry == r.RY && h->blk_rz == r.RZ) return GPE_OK;
    std::vector<int32_t> dy, dz, map;
    row_block_table(h, r.RY, r.RZ, dy, dz, map);
    std::vector<int32_t> t;
    t.insert(t.end(), dy.begin(), dy.end());
    t.insert(t.end(), dz.begin(), dz.end());
    t.insert(t.end(), map.begin(), map.end());
    if (h->blk) cudaFree(h->blk);
    h->blk = nullptr;
    if (cudaMalloc(&h->blk, t.size() * sizeof(int32_t)) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (row table)");
    CUDA_TRY(cudaMemcpy(h->blk, t.data(), t.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    h->blk_ry = r.RY;
    h->blk_rz = r.RZ;
    h->blk_nbuf = (uint32_t)dy.size();
    return GPE_OK;
}

template <int C>
static cudaError_t dispatch_rows_c(const gpe_handle* h, const StepArgs& a, const RowsShape& r, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_leapfrog_rows<double, C>(a, r.T, r.RY, r.RZ, h->nrows, r.nbuf, h->blk, (uint32_t)h->tune_threads, s)
                              : launch_leapfrog_rows<float, C>(a, r.T, r.RY, r.RZ, h->nrows, r.nbuf, h->blk, (uint32_t)h->tune_threads, s);
}
static cudaError_t dispatch_rows(const gpe_handle* h, const StepArgs& a, const RowsShape& r, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_rows_c<1>(h, a, r, s);
        case 3: return dispatch_rows_c<3>(h, a, r, s);
        default: return dispatch_rows_c<5>(h, a, r, s);
    }
}

// Row-tile kernel eligibility and tile length (0 = use the gather kernel).  The
// automatic choice is the grid-stride gather kernel: on GB300 (FP32, 10^6-10^7
// sites) it is as fast as the row tile or faster on every lattice and spin.
static uint32_t tile_cells(const gpe_handle* h) {
    // only on request (2) or for the multi-row tile (4); the interleaved choice (6)
    // steps single steps and explicit-field steps with the gather kernel, whose
    // states its own equal bit for bit
    if (h->tune_kernel != 2 && h->tune_kernel != 4) return 0;
    if (h->g.cell_bytes % 16 != 0) return 0;
    const uint32_t V = h->g.V, X = h->g.X;
    uint32_t tmax = 256 / V;
    if (tmax == 0) tmax = 1;
    if (V * tmax > 256) return 0;
    if (h->tune_tile > 0) return (uint32_t)h->tune_tile <= X && (uint32_t)h->tune_tile * V <= 256 ? (uint32_t)h->tune_tile : 0;
    if (tmax >= X) return X;
    for (uint32_t t = tmax; t * 2 > tmax; --t)
        if (X % t == 0) return t;
    return tmax;
}

template <int C>
static cudaError_t dispatch_tile_c(const gpe_handle* h, const StepArgs& a, uint32_t T, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_leapfrog_tile<double, C>(a, T, h->tune_carveout, s)
                              : launch_leapfrog_tile<float, C>(a, T, h->tune_carveout, s);
}
static cudaError_t dispatch_tile(const gpe_handle* h, const StepArgs& a, uint32_t T, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_tile_c<1>(h, a, T, s);
        case 3: return dispatch_tile_c<3>(h, a, T, s);
        default: return dispatch_tile_c<5>(h, a, T, s);
    }
}

// Hyperbolic row-tile kernel eligibility and tile length (0 = gather kernel).
static uint32_t hyper_tile_cells(const gpe_handle* h) {
    if (h->tune_kernel == 1 || h->g.E == 0) return 0;
    // the automatic choice, by measurement (fraction of peak, gather against tile):
    // scalars BCC 128^3 0.64 / 0.45, C15 40^3 0.60 / 0.39; spin-2 C15 128^3 0.69 /
    // 0.69, C15 48^3 0.75 / 0.71, BCC 96^3 0.77 / 0.69; spin-1 C15 40^3 0.55 / 0.51
    // -- the gather kernel; spin-1 BCC 96^3 0.56 / 0.74 -- the tile.  The tile
    // is chosen for spin-1 on small cells (V <= 16) and on request.
    if (h->tune_kernel != 2 && !(h->g.C == 3 && h->g.V <= 16)) return 0;
    if (h->g.cell_bytes % 16 != 0 || h->g.qcell_bytes % 16 != 0) return 0;
    const uint32_t per = h->g.V + h->g.E;
    const size_t tables = (size_t)h->g.V * h->lat.F * (8 + h->real_bytes) + (size_t)(3 * h->g.E + 1) * 4 +
                          3 * h->g.V * h->real_bytes;
    const size_t per_cell = 2 * (size_t)(h->g.cell_bytes + h->g.qcell_bytes);  // psi, q, psi_next, q_next
    uint32_t T = h->tune_tile > 0 ? (uint32_t)h->tune_tile : 0;
    if (T == 0) {
        // the most cells that keep the block within ~48 KB of shared memory (four or
        // more blocks per SM) and 1024 tasks, preferring a divisor of X
        T = 1;
        while (T < h->g.X && tables + (T + 1) * per_cell <= 48 * 1024 && (T + 1) * per <= 1024) ++T;
        for (uint32_t t = T; t * 2 > T && t > 0; --t)
            if (h->g.X % t == 0) {
                T = t;
                break;
            }
    }
    if (T == 0 || T > h->g.X || (uint64_t)T * per > 4096) return 0;
    if (tables + T * per_cell > 200 * 1024) return 0;
    return T;
}

template <int C>
static cudaError_t dispatch_hyper_tile_c(const gpe_handle* h, const StepArgs& a, uint32_t T, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_hyper_tile<double, C>(a, T, s) : launch_hyper_tile<float, C>(a, T, s);
}
static cudaError_t dispatch_hyper_tile(const gpe_handle* h, const StepArgs& a, uint32_t T, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return dispatch_hyper_tile_c<1>(h, a, T, s);
        case 3: return dispatch_hyper_tile_c<3>(h, a, T, s);
        default: return dispatch_hyper_tile_c<5>(h, a, T, s);
    }
}

double gpe::cell_dv(const gpe_handle* h) {
    const double bs = h->p.block_scale;
    return bs * bs * bs * h->lat.volume;  // volume = bs^3 * VOLUME (Spin1GpeBCC.cu:1385)
}

// One parabolic step next <- prev on interior pointers of the handle's geometry.
gpe_status gpe::step_buffers(gpe_handle* h, char* next, const char* prev, const gpe_fields& B, double t, int mode,
                             cudaStream_t s) {
    StepArgs a = make_args(h, B, t);
    a.prev = prev;
    a.next = next;
    a.hpsi = mode == GPE_MODE_ITP ? h->interior[GPE_HPSI] : nullptr;
    const MarchShape ms = march_shape(h);
    const uint32_t T = tile_cells(h);
    const RowsShape rs = rows_shape(h);
    const SlabShape ss = slab_shape(h);
    cudaError_t e;
    if (mode == GPE_MODE_LEAPFROG && ss.Tx > 0) e = dispatch_slab(h, a, ss, s);
    else if (mode == GPE_MODE_LEAPFROG && rs.T > 0) {
        gpe_status bst = ensure_row_block(h, rs);
        if (bst) return bst;
        e = dispatch_rows(h, a, rs, s);
    }
    else if (mode == GPE_MODE_LEAPFROG && ms.T > 0) e = dispatch_march(h, a, ms, s);
    else if (mode == GPE_MODE_LEAPFROG && T > 0) e = dispatch_tile(h, a, T, s);
    else e = dispatch_parabolic(h, a, mode, s);
    h->launches += 1;
    h->epoch += 1;
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return GPE_OK;
}

bool gpe::leapfrog_from_supported(const gpe_handle* h) {
    return h->p.scheme == GPE_SCHEME_PARABOLIC && rows_shape(h).T == 0 && march_shape(h).T == 0 && tile_cells(h) == 0 &&
           slab_shape(h).Tx == 0;
}

gpe_status gpe::leapfrog_from(gpe_handle* h, char* next, const char* cur, const char* old, const gpe_fields& B,
                              double t, cudaStream_t s) {
    if (!leapfrog_from_supported(h)) return fail(GPE_ERR_UNSUPPORTED, "out-of-place leapfrog needs the gather kernel");
    StepArgs a = make_args(h, B, t);
    a.prev = cur;
    a.next = next;
    a.hpsi = const_cast<char*>(old);  // read only, by the kModeLeapfrogFrom kernels
    const cudaError_t e = dispatch_parabolic(h, a, kModeLeapfrogFrom, s);
    h->launches += 1;
    h->epoch += 1;
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return GPE_OK;
}

// psi[next] <- psi[prev] (and q when hyperbolic), one step at time t.  The
// hyperbolic imaginary-time step is itp_q + itp_psi of the ground-state loop
// (RelativisticSpin2Gpe.cu:1712-1713), both reading the (psi, q) pair of prev,
// in one launch that also stores H psi_prev in GPE_HPSI.
static gpe_status one_step(gpe_handle* h, int next, int prev, const gpe_fields& B, double t, int mode, cudaStream_t s) {
    if (h->p.scheme == GPE_SCHEME_PARABOLIC) return step_buffers(h, h->interior[next], h->interior[prev], B, t, mode, s);
    StepArgs a = make_args(h, B, t);
    a.prev = h->interior[prev];
    a.next = h->interior[next];
    if (mode == GPE_MODE_EULER) return fail(GPE_ERR_UNSUPPORTED, "hyperbolic scheme: explicit steps are leapfrog or imaginary time");
    const int qprev = prev == GPE_PSI_EVEN ? GPE_Q_EVEN : GPE_Q_ODD;
    const int qnext = next == GPE_PSI_EVEN ? GPE_Q_EVEN : GPE_Q_ODD;
    a.q = h->interior[qprev];
    a.qnext = h->interior[qnext];
    cudaError_t e;
    if (mode == GPE_MODE_ITP) {
        a.hpsi = h->interior[GPE_HPSI];
        e = dispatch_hyper(h, a, HK_FUSED_ITP, s);
    } else {
        const uint32_t T = hyper_tile_cells(h);
        e = T > 0 ? dispatch_hyper_tile(h, a, T, s) : dispatch_hyper(h, a, HK_FUSED_LEAPFROG, s);
    }
    h->launches += 1;
    h->epoch += 1;
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return GPE_OK;
}

extern "C" gpe_status gpe_step_explicit(gpe_handle* h, int32_t next_slot, int32_t prev_slot, const gpe_fields* fields,
                                        double t, int32_t mode, void* stream) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if ((next_slot != GPE_PSI_EVEN && next_slot != GPE_PSI_ODD) || (prev_slot != GPE_PSI_EVEN && prev_slot != GPE_PSI_ODD))
        return fail(GPE_ERR_INVALID_ARG, "psi slots must be PSI_EVEN or PSI_ODD");
    // every mode reads neighbours of prev while it writes next
    if (next_slot == prev_slot) return fail(GPE_ERR_INVALID_ARG, "next and prev must be different buffers");
    if (mode < 0 || mode > 2) return fail(GPE_ERR_INVALID_ARG, "mode");
    if (h->p.scheme == GPE_SCHEME_SPLIT) return fail(GPE_ERR_UNSUPPORTED, "the split scheme steps in place: use gpe_step");
    if (mode == GPE_MODE_ITP) {
        gpe_status st = ensure_hpsi(h);
        if (st) return st;
    }
    gpe_fields B;
    std::memset(&B, 0, sizeof B);
    if (fields) B = *fields;
    return one_step(h, next_slot, prev_slot, B, t, mode, (cudaStream_t)stream);
}

extern "C" gpe_status gpe_set_expansion(gpe_handle* h, double t_start, double rate) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if (h->p.scheme != GPE_SCHEME_PARABOLIC) return fail(GPE_ERR_UNSUPPORTED, "expansion is built for the parabolic scheme");
    if (!std::isfinite(t_start) || !std::isfinite(rate) || rate < 0)
        return fail(GPE_ERR_INVALID_ARG, "expansion: finite t_start and rate >= 0");
    h->exp_t0 = t_start;
    h->exp_rate = rate;
    return GPE_OK;
}

extern "C" gpe_status gpe_start(gpe_handle* h, void* stream) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    cudaStream_t s = (cudaStream_t)stream;
    const double t = h->t0;
    const gpe_fields B = fields_at(h, t);
    if (h->p.scheme == GPE_SCHEME_SPLIT) {
        // q_R += c (q_R + d0 R), c = (dt/sigma) / (dt - dt/sigma)
        // (RelativisticGpeC15/GPUGrossPitaevskii_C15.cu:469)
        gpe_status st = split_launch(h, 2, t, s);
        if (st) return st;
        h->epoch += 1;
    } else if (h->p.scheme == GPE_SCHEME_PARABOLIC) {
        // forwardEuler(even <- odd) at t0 (Spin1GpeBCC.cu:1428-1433)
        gpe_status st = one_step(h, GPE_PSI_EVEN, GPE_PSI_ODD, B, t, GPE_MODE_EULER, s);
        if (st) return st;
    } else {
        // q_odd = d0 psi_odd; psi_even = psi_odd + dt(-iH) (parabolic form); q_even = d0 psi_even
        // (RelativisticSpin2Gpe.cu:1628-1630)
        StepArgs a = make_args(h, B, t);
        cudaError_t e;
        a.prev = h->interior[GPE_PSI_ODD];
        a.qnext = h->interior[GPE_Q_ODD];
        a.q = h->interior[GPE_Q_ODD];
        if ((e = dispatch_hyper(h, a, HK_Q_PARA, s)) != cudaSuccess) return cuda_fail(e, "q init");
        a.next = h->interior[GPE_PSI_EVEN];
        if ((e = dispatch_hyper(h, a, HK_PSI_PARA_EULER, s)) != cudaSuccess) return cuda_fail(e, "Euler start");
        a.prev = h->interior[GPE_PSI_EVEN];
        a.q = h->interior[GPE_Q_EVEN];
        a.qnext = h->interior[GPE_Q_EVEN];
        if ((e = dispatch_hyper(h, a, HK_Q_PARA, s)) != cudaSuccess) return cuda_fail(e, "q init");
        h->launches += 3;
        h->epoch += 1;
    }
    h->cur = GPE_PSI_EVEN;
    h->nstep = 0;
    return GPE_OK;
}

// n steps in the handle's layout.
static gpe_status plain_steps(gpe_handle* h, int32_t n, cudaStream_t s) {
    if (h->p.scheme == GPE_SCHEME_SPLIT) {
        // update_psi(I) + update_q(q_I), then update_psi(R) + update_q(q_R)
        // (RelativisticGpeC15/GPUGrossPitaevskii_C15.cu:477-482), one launch each
        for (int32_t k = 0; k < n; ++k) {
            const double t = h->t0 + (double)(h->nstep + 1) * h->p.dt;
            gpe_status st = split_launch(h, 0, t, s);
            if (!st) st = split_launch(h, 1, t, s);
            if (st) return st;
            h->epoch += 1;
            h->nstep++;
        }
        return GPE_OK;
    }
    for (int32_t k = 0; k < n; ++k) {
        const double t = h->t0 + (double)(h->nstep + 1) * h->p.dt;
        const gpe_fields B = fields_at(h, t);
        const int prev = h->cur, next = h->cur == GPE_PSI_EVEN ? GPE_PSI_ODD : GPE_PSI_EVEN;
        gpe_status st = one_step(h, next, prev, B, t, GPE_MODE_LEAPFROG, s);
        if (st) return st;
        h->cur = next;
        h->nstep++;
    }
    return GPE_OK;
}

// ------------------------------------------------------- call timing (GPE_TUNE_TIMING)

// Events on the call's stream: 0 call start, 1 steps start (after the layout change
// in), 2 observed step start, 3 observed step end, 4 call end (after the layout
// change out).  finish() waits for event 4 and adds the intervals to h->timing.
struct StepTimer {
    gpe_handle* h;
    cudaStream_t s;
    bool on;
    StepTimer(gpe_handle* hh, cudaStream_t ss) : h(hh), s(ss), on(hh->tune_timing != 0) {
        if (on && !h->tev_ok) {
            for (cudaEvent_t& ev : h->tev)
                if (cudaEventCreate(&ev) != cudaSuccess) on = false;
            h->tev_ok = on;
            if (!on) cudaGetLastError();
        }
    }
    void mark(int i) {
        if (on) cudaEventRecord(h->tev[i], s);
    }
    void finish(uint64_t plain, uint64_t observed, uint64_t converts, bool interleaved) {
        if (!on || cudaEventSynchronize(h->tev[4]) != cudaSuccess) return;
        float ms[4] = {0, 0, 0, 0};
        for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&ms[i], h->tev[i], h->tev[i + 1]);
        gpe_step_timing& T = h->timing;
        T.calls += 1;
        T.step_launches += plain;
        T.step_ms += ms[1];
        T.observed_launches += observed;
        T.observed_ms += ms[2];
        T.convert_launches += converts;
        T.convert_ms += ms[0] + ms[3];
        T.interleaved_calls += interleaved ? 1 : 0;
    }
};

// ---------------------------------------------------------- interleaved steps

// Calls shorter than this stay in the handle's layout: the two layout changes in
// and the two out cost about as much as two steps.
constexpr int32_t kIlMinSteps = 16;

// Rows the interleaved kernel takes: 4 entries in every row (BCC, A15, C15, Z), or
// rows of 4 and 8 (FCC), every neighbour in an adjacent cell (|dx|, |dy|, |dz| <= 1);
// 0 otherwise.
namespace gpe {
int il_stencil_deg(const gpe_handle* h) {
    if (!il_offsets_fit(make_il_grid(h->g))) return 0;
    for (const gpe_stencil_entry& e : h->lat.stencil)
        if (e.dx < -1 || e.dx > 1 || e.dy < -1 || e.dy > 1 || e.dz < -1 || e.dz > 1) return 0;
    if (h->tab.uniform_deg == 4) return 4;
    if (h->tab.quad_rows && h->tab.max_deg == 8) return 8;
    return 0;
}
}  // namespace gpe

static int il_deg(const gpe_handle* h) { return il_stencil_deg(h); }

static unsigned il_grid_blocks(const gpe_handle* h, bool obs) {
    const ILGrid G = make_il_grid(h->g);
    const int deg = il_deg(h);
    switch (h->g.C) {
        case 1: return il_blocks<1>(G, deg, obs, h->partial_blocks);
        case 3: return il_blocks<3>(G, deg, obs, h->partial_blocks);
        default: return il_blocks<5>(G, deg, obs, h->partial_blocks);
    }
}

// The interleaved kernel applies: FP32, parabolic, rows of 4 (or of 4 and 8)
// entries with neighbours in adjacent cells.
static bool il_applies(const gpe_handle* h) {
    if (h->p.scheme != GPE_SCHEME_PARABOLIC || h->real_bytes != 4 || il_deg(h) == 0) return false;
    return il_grid_blocks(h, false) > 0 && il_grid_blocks(h, true) > 0;
}

// Where the automatic choice takes the interleaved kernel, by measurement (FP32
// leapfrog, one launch, fraction of the measured copy peak, gather / interleaved;
// BCC 96^3, A15 64^3, C15 48^3, Z 56^3): spin-1 BCC 0.68 / 0.85, A15 0.63 / 0.85,
// C15 0.62 / 0.70, Z 0.66 / 0.77; spin-2 BCC 0.66 / 0.89, A15 0.59 / 0.88, C15
// 0.60 / 0.72, Z 0.64 / 0.79.  Not for scalars (BCC 0.68 / 0.51, C15 0.64 / 0.40:
// an 8-byte record already loads as one coalesced run in the handle's layout).
static bool il_auto(const gpe_handle* h) { return h->g.C >= 3; }

// The q slots' geometry as a Grid whose "nodes" are the E edges of a cell.
static Grid q_grid(const gpe_handle* h) {
    Grid q = h->g;
    q.V = h->g.E;
    q.slice = h->g.qslice;
    q.pitch = h->g.qpitch;
    q.cell_bytes = h->g.qcell_bytes;
    return q;
}

// The interleaved hyperbolic step applies: FP32, the hyperbolic scheme, 4 edges
// per node and 2 edges per node of a cell (BCC, BCC-227, C15), an even number of
// complex values per psi and q cell, and every edge and incidence within adjacent
// cells.
static bool il_hyper_applies(const gpe_handle* h) {
    const Grid& g = h->g;
    if (h->p.scheme != GPE_SCHEME_HYPERBOLIC || h->real_bytes != 4 || h->lat.F != 4 || g.E != 2 * g.V) return false;
    if ((g.V * g.C) % 2 || (g.E * g.C) % 2) return false;
    if (g.cell_bytes != g.V * g.C * 8 || g.qcell_bytes != g.E * g.C * 8) return false;
    if (!il_offsets_fit(make_il_grid(g)) || !il_offsets_fit(make_il_grid(q_grid(h)))) return false;
    auto adj = [](int dx, int dy, int dz) { return dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1; };
    for (const gpe_edge& e : h->lat.edges)
        if (!adj(e.dx, e.dy, e.dz)) return false;
    for (const gpe_incidence& r : h->lat.incidence)
        if (!adj(r.dx, r.dy, r.dz)) return false;
    return true;
}

// Where the automatic choice takes the interleaved hyperbolic step: everywhere it
// applies, by measurement (FP32, one fused launch, fraction of the measured copy
// peak, gather / row tile / interleaved): scalar BCC 128^3 0.64 / 0.46 / 0.71,
// spin-1 BCC 96^3 0.56 / 0.74 / 0.97, C15 40^3 0.57 / 0.51 / 0.80, spin-2 BCC 96^3
// 0.77 / 0.69 / 0.99, C15 48^3 0.75 / 0.67 / 0.93, C15 128^3 0.69 / 0.69 / 0.86.
static bool il_hyper_auto(const gpe_handle*) { return true; }

static bool use_interleaved(const gpe_handle* h, int32_t n) {
    if (n < 1 || (h->tune_kernel != 0 && h->tune_kernel != 6)) return false;
    if (h->p.scheme == GPE_SCHEME_HYPERBOLIC) {
        if (h->tune_kernel == 0 && (n < kIlMinSteps || !il_hyper_auto(h))) return false;
        return il_hyper_applies(h);
    }
    if (h->tune_kernel == 0 && (n < kIlMinSteps || !il_auto(h))) return false;
    return il_applies(h);
}

namespace gpe {
gpe_status il_ensure(gpe_handle* h, cudaStream_t s) {
    const ILGrid G = make_il_grid(h->g);
    for (int k = 0; k < 2; ++k) {
        if (h->il[k]) continue;
        void* p = nullptr;
        if (cudaMalloc(&p, G.bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(GPE_ERR_OOM, "cudaMalloc (interleaved state)");
        }
        h->il[k] = static_cast<char*>(p);
        // the halo rows and the padding cells stay zero
        CUDA_TRY(cudaMemsetAsync(p, 0, G.bytes, s));
    }
    h->ilg = G;
    return GPE_OK;
}
}  // namespace gpe

static gpe_status ensure_il(gpe_handle* h, cudaStream_t s) { return il_ensure(h, s); }

// Hyperbolic handles: the interleaved q copies (zeroed) and the offset tables of
// il_hyper_kernel, on first use: V*4 incidences (edge `edge` of the cell at (dx, dy,
// dz)) relative to a q group's base, E to-nodes (node `to` of the cell at (dx, dy,
// dz)) relative to a psi group's base -- each for the group's first cell, with dx +
// 1 in the two low bits -- and E from-nodes.
static gpe_status ensure_il_hyper(gpe_handle* h, cudaStream_t s) {
    gpe_status st = ensure_il(h, s);
    if (st) return st;
    const ILGrid G = h->ilg;
    const ILGrid Gq = make_il_grid(q_grid(h));
    for (int k = 0; k < 2; ++k) {
        if (h->ilq[k]) continue;
        void* p = nullptr;
        if (cudaMalloc(&p, Gq.bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(GPE_ERR_OOM, "cudaMalloc (interleaved q)");
        }
        h->ilq[k] = static_cast<char*>(p);
        CUDA_TRY(cudaMemsetAsync(p, 0, Gq.bytes, s));
    }
    h->ilgq = Gq;
    if (h->il_htab) return GPE_OK;
    const int64_t run = (int64_t)h->g.C * G.cells * 8;   // bytes between nodes (edges) of a group
    std::vector<int32_t> tab;
    auto put = [&](int64_t b, int dx) {
        if (b > INT32_MAX - 3 || b < INT32_MIN) return false;
        tab.push_back((int32_t)b | (dx + 1));
        return true;
    };
    for (const gpe_incidence& r : h->lat.incidence)
        if (!put(((int64_t)r.dz * (Gq.Y + 2) + r.dy) * (int64_t)Gq.row + (int64_t)r.edge * run + (int64_t)r.dx * 8, r.dx))
            return fail(GPE_ERR_INVALID_ARG, "grid too large for 32-bit interleaved offsets");
    for (const gpe_edge& e : h->lat.edges)
        if (!put(((int64_t)e.dz * (G.Y + 2) + e.dy) * (int64_t)G.row + (int64_t)e.to * run + (int64_t)e.dx * 8, e.dx))
            return fail(GPE_ERR_INVALID_ARG, "grid too large for 32-bit interleaved offsets");
    for (const gpe_edge& e : h->lat.edges) tab.push_back((int32_t)(e.from * run));
    void* p = nullptr;
    if (cudaMalloc(&p, tab.size() * sizeof(int32_t)) != cudaSuccess) {
        cudaGetLastError();
        return fail(GPE_ERR_OOM, "cudaMalloc (interleaved hyperbolic tables)");
    }
    h->il_htab = static_cast<int32_t*>(p);
    CUDA_TRY(cudaMemcpy(p, tab.data(), tab.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return GPE_OK;
}

static cudaError_t dispatch_il_hyper(const gpe_handle* h, const StepArgs& a, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return launch_il_hyper<1>(a, h->ilg, h->ilgq, h->il_htab, s);
        case 3: return launch_il_hyper<3>(a, h->ilg, h->ilgq, h->il_htab, s);
        default: return launch_il_hyper<5>(a, h->ilg, h->ilgq, h->il_htab, s);
    }
}

// The layout change of the interleaved slots of a call: psi, and q on hyperbolic
// handles (4 or 8 launches).
static gpe_status il_convert_all(gpe_handle* h, bool to_il, cudaStream_t s) {
    for (int k = GPE_PSI_EVEN; k <= GPE_PSI_ODD; ++k) {
        cudaError_t e = launch_il_convert(h->interior[k], h->g, h->il[k], h->ilg, to_il, s);
        if (e != cudaSuccess) return cuda_fail(e, to_il ? "layout change (in)" : "layout change (out)");
    }
    h->launches += 2;
    if (h->p.scheme != GPE_SCHEME_HYPERBOLIC) return GPE_OK;
    const Grid gq = q_grid(h);
    for (int k = 0; k < 2; ++k) {
        cudaError_t e = launch_il_convert(h->interior[GPE_Q_EVEN + k], gq, h->ilq[k], h->ilgq, to_il, s);
        if (e != cudaSuccess) return cuda_fail(e, to_il ? "layout change (in)" : "layout change (out)");
    }
    h->launches += 2;
    return GPE_OK;
}

static cudaError_t dispatch_il_step(const gpe_handle* h, const StepArgs& a, bool obs, cudaStream_t s) {
    switch (h->g.C) {
        case 1: return launch_il_step<1>(a, h->ilg, il_deg(h), h->partial_blocks, obs, h->obs_out, s);
        case 3: return launch_il_step<3>(a, h->ilg, il_deg(h), h->partial_blocks, obs, h->obs_out, s);
        default: return launch_il_step<5>(a, h->ilg, il_deg(h), h->partial_blocks, obs, h->obs_out, s);
    }
}

static gpe_status fill_observables(const gpe_handle* h, const double* r, gpe_observables* out);

namespace gpe {
// n parabolic leapfrog steps through the interleaved layout with the fields of
// every step given: step k reads slot `first_prev` (k even) or the other slot (k
// odd), at time t_first + k dt with fields[k], as step_buffers does in the
// handle's layout -- the same states, bit for bit.  False (nothing run) where the
// interleaved kernel is not the handle's choice for a call of n steps.
bool il_leapfrog_applies(const gpe_handle* h, int32_t n) {
    return h->p.scheme == GPE_SCHEME_PARABOLIC && use_interleaved(h, n);
}

gpe_status il_leapfrog_explicit(gpe_handle* h, int first_prev, int32_t n, const gpe_fields* fields, double t_first,
                                double dt, cudaStream_t s) {
    if (!il_leapfrog_applies(h, n)) return fail(GPE_ERR_UNSUPPORTED, "the interleaved kernel does not apply");
    gpe_status st = ensure_il(h, s);
    if (st) return st;
    if ((st = il_convert_all(h, true, s))) return st;
    int prev = first_prev;
    for (int32_t k = 0; k < n; ++k) {
        const int next = prev == GPE_PSI_EVEN ? GPE_PSI_ODD : GPE_PSI_EVEN;
        StepArgs a = make_args(h, fields[k], t_first + k * dt);
        a.prev = h->il[prev];
        a.next = h->il[next];
        cudaError_t e = dispatch_il_step(h, a, false, s);
        if (e != cudaSuccess) return cuda_fail(e, "interleaved step launch");
        h->launches += 1;
        h->epoch += 1;
        prev = next;
    }
    return il_convert_all(h, false, s);
}
}  // namespace gpe

// n leapfrog steps through the interleaved layout: both psi slots changed in,
// the steps (the observables of the state the last one reads summed inside it when
// out is given), both slots changed back.
static gpe_status il_steps(gpe_handle* h, int32_t n, gpe_observables* out, cudaStream_t s) {
    const bool hyper = h->p.scheme == GPE_SCHEME_HYPERBOLIC;
    if (hyper && out) return fail(GPE_ERR_UNSUPPORTED, "hyperbolic interleaved steps sum no observables");
    gpe_status st = hyper ? ensure_il_hyper(h, s) : ensure_il(h, s);
    if (st) return st;
    StepTimer tm(h, s);
    tm.mark(0);
    if ((st = il_convert_all(h, true, s))) return st;
    tm.mark(1);
    const int32_t plain = out ? n - 1 : n;
    for (int32_t k = 0; k < n; ++k) {
        const bool obs = k == plain;
        if (obs) tm.mark(2);
        const double t = h->t0 + (double)(h->nstep + 1) * h->p.dt;
        const gpe_fields B = fields_at(h, t);
        const int prev = h->cur, next = h->cur == GPE_PSI_EVEN ? GPE_PSI_ODD : GPE_PSI_EVEN;
        StepArgs a = make_args(h, B, t);
        a.prev = h->il[prev];
        a.next = h->il[next];
        cudaError_t e;
        if (hyper) {
            // q slots follow the psi slots (GPE_Q_EVEN with GPE_PSI_EVEN)
            a.q = h->ilq[prev == GPE_PSI_EVEN ? 0 : 1];
            a.qnext = h->ilq[next == GPE_PSI_EVEN ? 0 : 1];
            e = dispatch_il_hyper(h, a, s);
        } else {
            e = dispatch_il_step(h, a, obs, s);
        }
        if (e != cudaSuccess) return cuda_fail(e, "interleaved step launch");
        h->launches += obs ? 2 : 1;
        h->epoch += 1;
        h->cur = next;
        h->nstep++;
    }
    if (!out) tm.mark(2);
    tm.mark(3);
    if ((st = il_convert_all(h, false, s))) return st;
    tm.mark(4);
    tm.finish(plain, out ? 1 : 0, hyper ? 8 : 4, true);
    if (!out) return GPE_OK;
    double r[OBS_COUNT];
    CUDA_TRY(cudaMemcpyAsync(r, h->obs_out, sizeof r, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    gpe_status dst = check_device_error(h, s);
    if (dst) return dst;
    return fill_observables(h, r, out);
}

extern "C" gpe_status gpe_get_step_timing(gpe_handle* h, gpe_step_timing* out, int32_t reset) {
    if (!h || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    *out = h->timing;
    if (reset) std::memset(&h->timing, 0, sizeof h->timing);
    return GPE_OK;
}

extern "C" gpe_status gpe_step(gpe_handle* h, int32_t n, void* stream) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if (n < 0) return fail(GPE_ERR_INVALID_ARG, "negative step count");
    cudaStream_t s = (cudaStream_t)stream;
    if (use_interleaved(h, n)) return il_steps(h, n, nullptr, s);
    StepTimer tm(h, s);
    tm.mark(0);
    tm.mark(1);
    gpe_status st = plain_steps(h, n, s);
    if (st) return st;
    tm.mark(2);
    tm.mark(3);
    tm.mark(4);
    tm.finish(n, 0, 0, false);
    return GPE_OK;
}

// The observables from the OBS_COUNT FP64 sums of an observe or observed-step
// launch (dv = bs0^3 VOLUME).
static gpe_status fill_observables(const gpe_handle* h, const double* r, gpe_observables* out) {
    const double dv = cell_dv(h);
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
    if (out->nonfinite) return fail(GPE_ERR_NONFINITE, "state holds non-finite values");
    return GPE_OK;
}

template <int C>
static cudaError_t dispatch_parabolic_observe_c(const gpe_handle* h, const StepArgs& a, double* out, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_parabolic_observe<double, C>(a, out, s) : launch_parabolic_observe<float, C>(a, out, s);
}

extern "C" gpe_status gpe_step_observe(gpe_handle* h, int32_t n, gpe_observables* out, void* stream) {
    if (!h || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (n < 1) return fail(GPE_ERR_INVALID_ARG, "step count must be at least 1");
    cudaStream_t s = (cudaStream_t)stream;
    int32_t pre = n - 1;  // steps before the observed one
    if (use_interleaved(h, n)) {
        if (h->p.scheme != GPE_SCHEME_HYPERBOLIC) return il_steps(h, n, out, s);
        // hyperbolic: the first n - 1 steps in the interleaved layout, the observed
        // step below
        if (use_interleaved(h, pre)) {
            gpe_status ist = il_steps(h, pre, nullptr, s);
            if (ist) return ist;
            pre = 0;
        }
    }
    StepTimer tm(h, s);
    tm.mark(0);
    tm.mark(1);
    gpe_status st = plain_steps(h, pre, s);
    if (st) return st;
    tm.mark(2);
    const double t = h->t0 + (double)(h->nstep + 1) * h->p.dt;
    if (!leapfrog_from_supported(h)) {
        // another step kernel (tile, slab, hyperbolic, split): a separate observe pass
        gpe_observables o;
        gpe_status ost = gpe_observe(h, h->cur, t, &o, stream);
        if (ost && ost != GPE_ERR_NONFINITE) return ost;
        st = plain_steps(h, 1, s);
        tm.mark(3);
        tm.mark(4);
        tm.finish(pre, 1, 0, false);
        *out = o;
        return st ? st : (ost ? fail(ost, "state holds non-finite values") : GPE_OK);
    }
    const gpe_fields B = fields_at(h, t);
    const int prev = h->cur, next = h->cur == GPE_PSI_EVEN ? GPE_PSI_ODD : GPE_PSI_EVEN;
    StepArgs a = make_args(h, B, t);
    a.prev = h->interior[prev];
    a.next = h->interior[next];
    cudaError_t e;
    switch (h->g.C) {
        case 1: e = dispatch_parabolic_observe_c<1>(h, a, h->obs_out, s); break;
        case 3: e = dispatch_parabolic_observe_c<3>(h, a, h->obs_out, s); break;
        default: e = dispatch_parabolic_observe_c<5>(h, a, h->obs_out, s); break;
    }
    h->launches += 2;
    h->epoch += 1;
    if (e != cudaSuccess) return cuda_fail(e, "observed step launch");
    h->cur = next;
    h->nstep++;
    tm.mark(3);
    tm.mark(4);
    tm.finish(pre, 1, 0, false);
    double r[OBS_COUNT];
    CUDA_TRY(cudaMemcpyAsync(r, h->obs_out, sizeof r, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    gpe_status dst = check_device_error(h, s);
    if (dst) return dst;
    return fill_observables(h, r, out);
}

extern "C" gpe_status gpe_observe(gpe_handle* h, int32_t slot, double t, gpe_observables* out, void* stream) {
    if (!h || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (!slot_ok(h, slot) || slot == GPE_Q_EVEN || slot == GPE_Q_ODD) return fail(GPE_ERR_INVALID_ARG, "psi slot");
    cudaStream_t s = (cudaStream_t)stream;
    StepArgs a = make_args(h, fields_at(h, t), t);
    a.prev = h->interior[slot];
    cudaError_t e = dispatch_observe(h, a, h->obs_out, s);
    if (e != cudaSuccess) return cuda_fail(e, "observe launch");
    h->launches += 2;
    double r[OBS_COUNT];
    CUDA_TRY(cudaMemcpyAsync(r, h->obs_out, sizeof r, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    gpe_status dst = check_device_error(h, s);
    if (dst) return dst;
    return fill_observables(h, r, out);
}

extern "C" gpe_status gpe_itp(gpe_handle* h, int32_t n, double* mu_out, void* stream) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if (h->p.scheme == GPE_SCHEME_SPLIT) return fail(GPE_ERR_UNSUPPORTED, "imaginary time is not built for the split scheme");
    gpe_status st = ensure_hpsi(h);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    gpe_fields zero;
    std::memset(&zero, 0, sizeof zero);
    const double dv = cell_dv(h);
    for (int32_t k = 0; k < n; ++k) {
        const int prev = h->cur, next = h->cur == GPE_PSI_EVEN ? GPE_PSI_ODD : GPE_PSI_EVEN;
        // itp(H psi, next <- prev) then normalize(next) (Spin1GpeBCC.cu:1470-1473;
        // hyperbolic: itp_q + itp_psi, normalize_h, RelativisticSpin2Gpe.cu:1712-1715)
        st = one_step(h, next, prev, zero, 0.0, GPE_MODE_ITP, s);
        if (st) return st;
        StepArgs a = make_args(h, zero, 0.0);
        a.prev = h->interior[next];
        a.next = h->interior[next];
        cudaError_t e = dispatch_norm(h, a, h->obs_out, s);
        if (e != cudaSuccess) return cuda_fail(e, "itp norm");
        e = dispatch_scale(h, a, h->obs_out, dv, s);
        if (e != cudaSuccess) return cuda_fail(e, "itp scale");
        h->launches += 3;
        h->cur = next;
    }
    if (mu_out) {
        // innerProduct(psi, H psi) + integrate (Spin1GpeBCC.cu:1481-1490)
        StepArgs a = make_args(h, zero, 0.0);
        a.prev = h->interior[h->cur];
        a.next = h->interior[GPE_HPSI];
        cudaError_t e = launch_dot(a, h->p.precision, h->g.C, h->obs_out, s);
        if (e != cudaSuccess) return cuda_fail(e, "itp dot");
        h->launches += 2;
        double r[OBS_COUNT];
        CUDA_TRY(cudaMemcpyAsync(r, h->obs_out, sizeof r, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        *mu_out = r[OBS_NORM] * dv;
    }
    return GPE_OK;
}

extern "C" gpe_status gpe_set_tuning(gpe_handle* h, int32_t key, int32_t value) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if (key == GPE_TUNE_KERNEL) {
        if (value < 0 || value > 6) return fail(GPE_ERR_INVALID_ARG, "kernel choice");
        if (value == 6) {
            if (!il_applies(h) && !il_hyper_applies(h))
                return fail(GPE_ERR_UNSUPPORTED, "the interleaved kernel needs FP32, the parabolic scheme with rows of 4 (or 4 and 8) "
                                                 "entries or the hyperbolic scheme with 4 edges per node, and neighbours in "
                                                 "adjacent cells");
            h->tune_kernel = 6;
            return GPE_OK;
        }
        if (value >= 2 && h->g.cell_bytes % 16 != 0) return fail(GPE_ERR_UNSUPPORTED, "tiled kernels need 16-byte cells");
        const int old = h->tune_kernel;
        h->tune_kernel = value;
        if (value == 3 && march_shape(h).T == 0) {
            h->tune_kernel = old;
            return fail(GPE_ERR_UNSUPPORTED, "no z-march tile shape divides the grid within the shared-memory limit");
        }
        if (value == 4 && rows_cells(h) == 0) {
            h->tune_kernel = old;
            return fail(GPE_ERR_UNSUPPORTED, "the multi-row tile does not fit in shared memory");
        }
        if (value == 5 && slab_shape(h).Tx == 0) {
            h->tune_kernel = old;
            return fail(GPE_ERR_UNSUPPORTED, "the slab kernel needs 4 entries per node and a tile whose slabs fit");
        }
        return GPE_OK;
    }
    if (key == GPE_TUNE_TIMING) {
        if (value != 0 && value != 1) return fail(GPE_ERR_INVALID_ARG, "timing: 0 (off) or 1 (on)");
        h->tune_timing = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_TRANSFER) {
        if (value != 0 && value != 1) return fail(GPE_ERR_INVALID_ARG, "transfer: 0 (direct) or 1 (DMA through staging)");
        h->tune_transfer = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_CARVEOUT) {
        if (value < 0 || value > 100) return fail(GPE_ERR_INVALID_ARG, "carveout: 0 (driver default) or 1..100 percent");
        h->tune_carveout = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_OBSERVE_ARITH) {
        if (value != 0 && value != 1) return fail(GPE_ERR_INVALID_ARG, "observe arithmetic: 0 (FP64) or 1 (storage precision)");
        h->tune_observe = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_TILE_ROWS) {
        if (value < 0 || (uint32_t)value > h->g.Y) return fail(GPE_ERR_INVALID_ARG, "tile rows");
        h->tune_rows = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_THREADS) {
        if (value < 0 || value > 1024 || value % 32) return fail(GPE_ERR_INVALID_ARG, "threads must be a multiple of 32");
        h->tune_threads = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_ZCHUNK) {
        if (value < 0 || (uint32_t)value > h->g.Z) return fail(GPE_ERR_INVALID_ARG, "z chunk");
        h->tune_zchunk = value;
        return GPE_OK;
    }
    if (key == GPE_TUNE_TILE_CELLS) {
        if (value < 0 || (uint32_t)value > h->g.X || (uint64_t)value * h->g.V > 1024)
            return fail(GPE_ERR_INVALID_ARG, "tile length");
        h->tune_tile = value;
        return GPE_OK;
    }
    return fail(GPE_ERR_INVALID_ARG, "unknown tuning key");
}

extern "C" gpe_status gpe_get_tuning(const gpe_handle* h, int32_t key, int32_t* value) {
    if (!h || !value) return fail(GPE_ERR_INVALID_ARG, "null argument");
    const MarchShape ms = march_shape(h);
    const uint32_t tr = rows_cells(h);
    if (h->p.scheme == GPE_SCHEME_HYPERBOLIC && (key == GPE_TUNE_KERNEL || key == GPE_TUNE_TILE_CELLS)) {
        // hyperbolic handles: the interleaved kernel on request, else the fused tile
        // kernel or the gather kernel (calls of 16 or more steps on spinor handles
        // take the interleaved kernel by themselves)
        const uint32_t T = hyper_tile_cells(h);
        *value = key == GPE_TUNE_KERNEL ? (h->tune_kernel == 6 ? 6 : (T > 0 ? 2 : 1)) : (int32_t)T;
        return GPE_OK;
    }
    const SlabShape ss = slab_shape(h);
    if (ss.Tx > 0 && (key == GPE_TUNE_KERNEL || key == GPE_TUNE_TILE_CELLS || key == GPE_TUNE_TILE_ROWS)) {
        *value = key == GPE_TUNE_KERNEL ? 5 : (int32_t)(key == GPE_TUNE_TILE_CELLS ? ss.Tx : ss.Ty);
        return GPE_OK;
    }
    if (key == GPE_TUNE_TIMING) {
        *value = h->tune_timing;
        return GPE_OK;
    }
    if (key == GPE_TUNE_TRANSFER) {
        *value = h->tune_transfer;
        return GPE_OK;
    }
    if (key == GPE_TUNE_KERNEL && h->tune_kernel == 6) {
        *value = 6;
        return GPE_OK;
    }
    if (key == GPE_TUNE_KERNEL) *value = tr > 0 ? 4 : ms.T > 0 ? 3 : (tile_cells(h) > 0 ? 2 : 1);
    else if (key == GPE_TUNE_TILE_CELLS) *value = (int32_t)(tr > 0 ? tr : ms.T > 0 ? ms.T : tile_cells(h));
    else if (key == GPE_TUNE_TILE_ROWS) *value = (int32_t)(tr > 0 ? rows_shape(h).RY : ms.TY);
    else if (key == GPE_TUNE_ZCHUNK) *value = (int32_t)(tr > 0 ? rows_shape(h).RZ : ms.ZC);
    else if (key == GPE_TUNE_THREADS) *value = h->tune_threads;
    else if (key == GPE_TUNE_OBSERVE_ARITH) *value = h->tune_observe;
    else if (key == GPE_TUNE_CARVEOUT) *value = h->tune_carveout;
    else return fail(GPE_ERR_INVALID_ARG, "unknown tuning key");
    return GPE_OK;
}

extern "C" int32_t gpe_current_slot(const gpe_handle* h) { return h ? h->cur : -1; }

extern "C" uint64_t gpe_launch_count(const gpe_handle* h) { return h ? h->launches : 0; }

extern "C" uint64_t gpe_sites(const gpe_handle* h) {
    return h ? (uint64_t)h->g.X * h->g.Y * h->g.Z * h->g.V : 0;
}

// ------------------------------------------------------------------ autotuner

// Times candidate step kernels and tile shapes on this handle's buffers and keeps
// the fastest (the tile shape and threads per block per lattice type).  The state
// is saved before and restored after the trials.
extern "C" gpe_status gpe_autotune(gpe_handle* h, int32_t steps, char* report, size_t report_len, void* stream) {
    if (!h) return fail(GPE_ERR_INVALID_ARG, "null handle");
    if (h->p.scheme == GPE_SCHEME_SPLIT) return fail(GPE_ERR_UNSUPPORTED, "the split scheme has one kernel: nothing to tune");
    if (steps <= 0) steps = 10;
    cudaStream_t s = (cudaStream_t)stream;
    struct Cand {
        int kernel, tile, rows, zchunk, threads;
    };
    std::vector<Cand> cands;
    // the gather kernel as the automatic choice (0), which also keeps the
    // interleaved kernel for long calls
    cands.push_back({0, 0, 0, 0, 0});
    if (h->g.cell_bytes % 16 == 0) {
        cands.push_back({2, 0, 0, 0, 0});
        const uint32_t ryz[4][2] = {{1, 1}, {2, 1}, {1, 2}, {2, 2}};
        for (auto& b : ryz) {
            if (h->g.Y % b[0] || h->g.Z % b[1]) continue;
            const uint32_t base = 384 / (b[0] * b[1] * h->g.V) > 0 ? 384 / (b[0] * b[1] * h->g.V) : 1;
            const uint32_t ts[3] = {base / 2, base, base * 2};
            for (uint32_t t : ts) {
                if (t == 0 || t > h->g.X) continue;
                for (int th : {0, 192, 256})
                    cands.push_back({4, (int)t, (int)b[0], (int)b[1], th});
            }
        }
    }
    const int saved_k = h->tune_kernel, saved_t = h->tune_tile, saved_r = h->tune_rows, saved_z = h->tune_zchunk,
              saved_th = h->tune_threads;
    // save the state buffers the trial steps overwrite: psi even/odd and, for the
    // hyperbolic scheme, q even/odd
    void* save[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int slot = GPE_PSI_EVEN; slot <= GPE_Q_ODD; ++slot) {
        if (!h->alloc[slot]) continue;
        if (cudaMalloc(&save[slot], h->alloc_bytes[slot]) != cudaSuccess) {
            for (void* p : save)
                if (p) cudaFree(p);
            return fail(GPE_ERR_OOM, "cudaMalloc (autotune save)");
        }
        CUDA_TRY(cudaMemcpyAsync(save[slot], h->alloc[slot], h->alloc_bytes[slot], cudaMemcpyDeviceToDevice, s));
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    gpe_fields B;
    std::memset(&B, 0, sizeof B);
    float best_ms = 1e30f;
    Cand best = {saved_k, saved_t, saved_r, saved_z, saved_th};
    std::string rep = "[";
    for (const Cand& c : cands) {
        h->tune_kernel = c.kernel;
        h->tune_tile = c.tile;
        h->tune_rows = c.rows;
        h->tune_zchunk = c.zchunk;
        h->tune_threads = c.threads;
        if (c.kernel == 4 && rows_shape(h).T == 0) continue;
        if (c.kernel == 2 && tile_cells(h) == 0) continue;
        bool ok = true;
        for (int k = 0; k < 2 && ok; ++k) ok = one_step(h, GPE_PSI_ODD, GPE_PSI_EVEN, B, 0.0, GPE_MODE_LEAPFROG, s) == GPE_OK;
        cudaEventRecord(e0, s);
        for (int k = 0; k < steps && ok; ++k)
            ok = one_step(h, (k & 1) ? GPE_PSI_EVEN : GPE_PSI_ODD, (k & 1) ? GPE_PSI_ODD : GPE_PSI_EVEN, B, 0.0,
                          GPE_MODE_LEAPFROG, s) == GPE_OK;
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess || !ok) {
            cudaGetLastError();
            continue;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)steps;
        char line[160];
        std::snprintf(line, sizeof line, "%s{\"kernel\":%d,\"tile\":%d,\"rows\":%d,\"zchunk\":%d,\"threads\":%d,\"ms\":%.5f}",
                      rep.size() > 1 ? "," : "", c.kernel, c.tile, c.rows, c.zchunk, c.threads, ms);
        rep += line;
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    rep += "]";
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->tune_kernel = best.kernel;
    h->tune_tile = best.tile;
    h->tune_rows = best.rows;
    h->tune_zchunk = best.zchunk;
    h->tune_threads = best.threads;
    for (int slot = GPE_PSI_EVEN; slot <= GPE_Q_ODD; ++slot)
        if (save[slot])
            CUDA_TRY(cudaMemcpyAsync(h->alloc[slot], save[slot], h->alloc_bytes[slot], cudaMemcpyDeviceToDevice, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    for (void* p : save)
        if (p) cudaFree(p);
    if (report && report_len) {
        std::snprintf(report, report_len, "%s", rep.c_str());
    }
    return GPE_OK;
}

// ---------------------------------------------------------------- init state

template <int C>
static cudaError_t dispatch_init_c(const gpe_handle* h, const StepArgs& a, const InitArgs& in, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_init<double, C>(a, in, s) : launch_init<float, C>(a, in, s);
}

template <int C>
static cudaError_t dispatch_respin_c(const gpe_handle* h, const StepArgs& a, const RespinArgs& r, cudaStream_t s) {
    return h->real_bytes == 8 ? launch_respin<double, C>(a, r, s) : launch_respin<float, C>(a, r, s);
}

extern "C" gpe_status gpe_respin(gpe_handle* h, int32_t slot, const double* zeta, void* stream) {
    if (!h || !zeta) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (slot != GPE_PSI_EVEN && slot != GPE_PSI_ODD) return fail(GPE_ERR_INVALID_ARG, "psi slot");
    RespinArgs r;
    std::memset(&r, 0, sizeof r);
    for (int m = 0; m < h->g.C; ++m) {
        const double re = zeta[2 * m], im = zeta[2 * m + 1];
        if (!std::isfinite(re) || !std::isfinite(im)) return fail(GPE_ERR_INVALID_ARG, "zeta must be finite");
        r.w[m] = re * re + im * im;
        const double a = std::sqrt(r.w[m]);
        r.u[m][0] = a > 0 ? re / a : 0.0;
        r.u[m][1] = a > 0 ? im / a : 0.0;
    }
    cudaStream_t s = (cudaStream_t)stream;
    gpe_fields zero;
    std::memset(&zero, 0, sizeof zero);
    StepArgs a = make_args(h, zero, 0.0);
    a.next = h->interior[slot];
    cudaError_t e;
    switch (h->g.C) {
        case 1: e = dispatch_respin_c<1>(h, a, r, s); break;
        case 3: e = dispatch_respin_c<3>(h, a, r, s); break;
        default: e = dispatch_respin_c<5>(h, a, r, s); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "respin kernel");
    h->launches += 1;
    h->epoch += 1;
    return GPE_OK;
}

extern "C" gpe_status gpe_init_state(gpe_handle* h, int32_t slot, const gpe_init* init, void* stream) {
    if (!h || !init) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (slot != GPE_PSI_EVEN && slot != GPE_PSI_ODD) return fail(GPE_ERR_INVALID_ARG, "psi slot");
    if (!(h->p.c0 > 0)) return fail(GPE_ERR_INVALID_ARG, "the Thomas-Fermi profile needs c0 > 0");
    cudaStream_t s = (cudaStream_t)stream;
    gpe_fields zero;
    std::memset(&zero, 0, sizeof zero);
    StepArgs a = make_args(h, zero, 0.0);
    a.next = h->interior[slot];
    InitArgs in;
    std::memset(&in, 0, sizeof in);
    for (int c = 0; c < 5; ++c) {
        in.zeta[c][0] = init->zeta[c][0];
        in.zeta[c][1] = init->zeta[c][1];
    }
    const double lx = h->p.trap_lambda[0], ly = h->p.trap_lambda[1], lz = h->p.trap_lambda[2];
    in.mu = 0.5 * std::pow(15.0 * h->p.c0 * lx * ly * lz / (4.0 * 3.141592653589793), 0.4);
    in.c0inv = 1.0 / h->p.c0;
    in.noise_abs = init->noise_abs * std::sqrt(in.mu * in.c0inv);
    in.noise_rel = init->noise_rel;
    in.kappa = init->vortex_kappa;
    in.seed = init->seed;
    cudaError_t e;
    switch (h->g.C) {
        case 1: e = dispatch_init_c<1>(h, a, in, s); break;
        case 3: e = dispatch_init_c<3>(h, a, in, s); break;
        default: e = dispatch_init_c<5>(h, a, in, s); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "init kernel");
    h->launches += 1;
    h->epoch += 1;
    if (init->normalize) {
        a.prev = h->interior[slot];
        e = dispatch_norm(h, a, h->obs_out, s);
        if (e == cudaSuccess) e = dispatch_scale(h, a, h->obs_out, cell_dv(h), s);
        if (e != cudaSuccess) return cuda_fail(e, "init normalisation");
        h->launches += 3;
    }
    h->cur = slot;
    return GPE_OK;
}
