// gpe_fields.cu -- per-node output fields of a psi slot (gpe_node_fields) and
// their reductions (gpe_node_fields_reduce).
//
// The reference computes these on the device after a step and copies them to the
// host for its state files and its dt control: the density kernels
// (Spin1GpeBCC.cu:191-211), localAvgSpinAndDensity + integrateSpinAndDensity
// (:235-271, :992-1020), uvTheta (:273-326) and maxHamilton + getMaxHamilton
// (:144-189, :1022-1037); Spin2GpeBCC.cu:192-306 applies the spin-1 spin and
// uvTheta formulas to s1, s0, s_1.  The x/y-quantised projections are the
// component densities its picture writer draws (Spin1GpeBCC/utils.h:177-193).
// Here one kernel writes the chosen field of every interior node in FP64 (from
// values stored in FP32 or FP64), in the reference's node order
// idx = V (z X Y + y X + x) + l; a second kernel reduces it with FP64 partial
// sums per block, added on the host in a fixed order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gpe_handle.h"
#include "gpe_kernels.cuh"

namespace gpe {

static int field_width(int kind) {
    switch (kind) {
        case GPE_FIELD_DENSITY: return 1;
        case GPE_FIELD_SPIN: return 5;
        case GPE_FIELD_UV_THETA: return 7;
        case GPE_FIELD_MAX_HAMILTON: return 1;
        case GPE_FIELD_PROJ_X:
        case GPE_FIELD_PROJ_Y: return 3;
        default: return 0;
    }
}

template <typename R, int C, int KIND>
__global__ void __launch_bounds__(256) node_fields_kernel(StepArgs a, double* out) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= a.total) return;
    const uint32_t i = (uint32_t)gid;
    const uint32_t row = fdiv(i, a.divRow);
    const uint32_t within = i - row * a.row_items;
    const uint32_t x = fdiv(within, a.divV);
    const uint32_t l = within - x * a.g.V;
    const uint32_t z = fdiv(row, a.divY);
    const uint32_t y = row - z * a.g.Y;
    const char* p = a.prev + (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes +
                    l * (C * 2 * sizeof(R));
    double re[C], im[C];
    double rho = 0;
#pragma unroll
    for (int s = 0; s < C; ++s) {
        const Cx<R> v = ldc<R>(p + s * 2 * sizeof(R));
        re[s] = (double)v.x;
        im[s] = (double)v.y;
        rho += re[s] * re[s] + im[s] * im[s];
    }
    constexpr int kWidth = KIND == GPE_FIELD_DENSITY ? 1 : KIND == GPE_FIELD_SPIN ? 5 : KIND == GPE_FIELD_UV_THETA ? 7
                         : KIND == GPE_FIELD_MAX_HAMILTON ? 1 : 3;
    double* o = out + (size_t)i * kWidth;
    constexpr int b = C == 5 ? 1 : 0;  // s1, s0, s_1
    if constexpr (KIND == GPE_FIELD_DENSITY) {
        o[0] = rho;
    } else if constexpr (KIND == GPE_FIELD_SPIN) {
        const double n1 = re[b] * re[b] + im[b] * im[b];
        const double nm1 = re[b + 2] * re[b + 2] + im[b + 2] * im[b + 2];
        const double sq = sqrt(rho);
        const double ax = re[b] / sq, ay = im[b] / sq, bx = re[b + 1] / sq, by = im[b + 1] / sq;
        const double cx_ = re[b + 2] / sq, cy_ = im[b + 2] / sq;
        // sqrt2 (conj(s1) s0 + conj(s0) s_1) of the normalised spinor
        const double tx = GPE_REF_SQRT_2 * ((ax * bx + ay * by) + (bx * cx_ + by * cy_));
        const double ty = GPE_REF_SQRT_2 * ((ax * by - ay * bx) + (bx * cy_ - by * cx_));
        const double sz = n1 - nm1;  // of the unnormalised spinor, as the reference computes it
        o[0] = rho * sqrt(tx * tx + ty * ty + sz * sz);
        o[1] = tx;
        o[2] = ty;
        o[3] = sz;
        o[4] = rho;
    } else if constexpr (KIND == GPE_FIELD_UV_THETA) {
        // a = m + i n with a = ((s_1 - s1)/sqrt2, -i (s_1 + s1)/sqrt2, s0)
        const double m[3] = {(re[b + 2] - re[b]) / GPE_REF_SQRT_2, (im[b + 2] + im[b]) / GPE_REF_SQRT_2, re[b + 1]};
        const double n[3] = {(im[b + 2] - im[b]) / GPE_REF_SQRT_2, -(re[b + 2] + re[b]) / GPE_REF_SQRT_2, im[b + 1]};
        const double mn = m[0] * n[0] + m[1] * n[1] + m[2] * n[2];
        const double mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
        const double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
        double th = atan2(-2 * mn, mm - nn) / 2;
        if (C == 3 && th < 0) th += 3.1415926535897932385;
        double sn, cs;
        sincos(th, &sn, &cs);
        double u[3], w[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            u[k] = m[k] * cs - sn * n[k];
            w[k] = m[k] * sn + cs * n[k];
        }
        const bool keep = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) >= sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            o[k] = keep ? u[k] : w[k];
            o[3 + k] = keep ? w[k] : u[k];
        }
        o[6] = th;
    } else if constexpr (KIND == GPE_FIELD_MAX_HAMILTON) {
        const PhysR<double>& P = a.pd;
        double r[3];
        r[0] = P.p0[0] + P.bs * ((double)x * P.bw[0] + a.tab.pos64[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((double)y * P.bw[1] + a.tab.pos64[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((double)z * P.bw[2] + a.tab.pos64[3 * l + 2]);
        const double pot = trap<double>(P, r) + P.c0 * rho;
        const double mx = GPE_REF_SQRT_2 * ((re[0] * re[1] + im[0] * im[1]) + (re[1] * re[2] + im[1] * im[2]));
        const double my = GPE_REF_SQRT_2 * ((re[0] * im[1] - im[0] * re[1]) + (re[1] * im[2] - im[1] * re[2]));
        const double mz = (re[0] * re[0] + im[0] * im[0]) - (re[2] * re[2] + im[2] * im[2]);
        // magneticField without the quadrupole offset, as maxHamilton calls it
        const double Bx = P.bq * r[0] + P.bb[0] + P.c2 * mx;
        const double By = P.bq * r[1] + P.bb[1] + P.c2 * my;
        const double Bz = -2 * P.bq * r[2] + P.bb[2] + P.c2 * mz;
        o[0] = fmax(pot + fabs(GPE_REF_INV_SQRT_2 * Bx), fmax(pot + fabs(GPE_REF_INV_SQRT_2 * By), pot + fabs(Bz)));
    } else {
        const double r2 = sqrt(2.0);
        double qr[3], qi[3];
        if constexpr (KIND == GPE_FIELD_PROJ_X) {
            qr[0] = 0.5 * (re[0] + re[2]) - re[1] / r2;
            qi[0] = 0.5 * (im[0] + im[2]) - im[1] / r2;
            qr[1] = (re[0] - re[2]) / r2;
            qi[1] = (im[0] - im[2]) / r2;
            qr[2] = 0.5 * (re[2] + re[0]) + re[1] / r2;
            qi[2] = 0.5 * (im[2] + im[0]) + im[1] / r2;
        } else {
            // s (0, -1) = (im, -re)
            qr[0] = 0.5 * (re[0] - re[2]) + im[1] / r2;
            qi[0] = 0.5 * (im[0] - im[2]) - re[1] / r2;
            qr[1] = (im[0] + im[2]) / r2;
            qi[1] = -(re[0] + re[2]) / r2;
            qr[2] = 0.5 * (re[2] - re[0]) + im[1] / r2;
            qi[2] = 0.5 * (im[2] - im[0]) - re[1] / r2;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) o[k] = qr[k] * qr[k] + qi[k] * qi[k];
    }
}

// Block partials of a field buffer: DENSITY sum; SPIN (spin norm, rho s_x, rho s_y,
// rho s_z, rho) sums, the weighting of integrateVecWithDensity; MAX_HAMILTON max.
__global__ void __launch_bounds__(256) fields_reduce_kernel(const double* buf, uint64_t n, int kind, double* partials) {
    __shared__ double red[8][5];
    const bool is_max = kind == GPE_FIELD_MAX_HAMILTON;
    double acc[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) acc[k] = is_max ? -INFINITY : 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (kind == GPE_FIELD_SPIN) {
            const double* v = buf + i * 5;
            acc[0] += v[0];
            acc[1] += v[4] * v[1];
            acc[2] += v[4] * v[2];
            acc[3] += v[4] * v[3];
            acc[4] += v[4];
        } else if (is_max) {
            acc[0] = fmax(acc[0], buf[i]);
        } else {
            acc[0] += buf[i];
        }
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        double v = acc[k];
        for (int off = 16; off > 0; off >>= 1) {
            const double u = __shfl_down_sync(0xffffffffu, v, off);
            v = is_max ? fmax(v, u) : v + u;
        }
        acc[k] = v;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 5; ++k) red[warp][k] = acc[k];
    __syncthreads();
    if (threadIdx.x < 5) {
        double v = red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = is_max ? fmax(v, red[w][threadIdx.x]) : v + red[w][threadIdx.x];
        partials[(size_t)blockIdx.x * 5 + threadIdx.x] = v;
    }
}

template <typename R, int C, int KIND>
static cudaError_t launch_fields_k(const StepArgs& a, double* out, cudaStream_t s) {
    const unsigned nb = (unsigned)((a.total + 255) / 256);
    if (nb) node_fields_kernel<R, C, KIND><<<nb, 256, 0, s>>>(a, out);
    return cudaGetLastError();
}

template <typename R, int C>
static cudaError_t launch_fields_c(const StepArgs& a, int kind, double* out, cudaStream_t s) {
    switch (kind) {
        case GPE_FIELD_DENSITY: return launch_fields_k<R, C, GPE_FIELD_DENSITY>(a, out, s);
        case GPE_FIELD_SPIN:
            if constexpr (C > 1) return launch_fields_k<R, C, GPE_FIELD_SPIN>(a, out, s);
            break;
        case GPE_FIELD_UV_THETA:
            if constexpr (C > 1) return launch_fields_k<R, C, GPE_FIELD_UV_THETA>(a, out, s);
            break;
        case GPE_FIELD_MAX_HAMILTON:
            if constexpr (C == 3) return launch_fields_k<R, C, GPE_FIELD_MAX_HAMILTON>(a, out, s);
            break;
        case GPE_FIELD_PROJ_X:
            if constexpr (C == 3) return launch_fields_k<R, C, GPE_FIELD_PROJ_X>(a, out, s);
            break;
        case GPE_FIELD_PROJ_Y:
            if constexpr (C == 3) return launch_fields_k<R, C, GPE_FIELD_PROJ_Y>(a, out, s);
            break;
        default: break;
    }
    return cudaErrorInvalidValue;
}

template <typename R>
static cudaError_t launch_fields(const StepArgs& a, int C, int kind, double* out, cudaStream_t s) {
    if (C == 1) return launch_fields_c<R, 1>(a, kind, out, s);
    if (C == 3) return launch_fields_c<R, 3>(a, kind, out, s);
    return launch_fields_c<R, 5>(a, kind, out, s);
}

// Checks the request and writes the field of every interior node into the
// handle's field buffer (grown on demand).
static gpe_status compute_fields(gpe_handle* h, int32_t slot, int32_t kind, double t, cudaStream_t s, int* width) {
    if (slot != GPE_PSI_EVEN && slot != GPE_PSI_ODD && slot != GPE_HPSI) return fail(GPE_ERR_INVALID_ARG, "psi slot");
    if (!h->alloc[slot]) return fail(GPE_ERR_INVALID_ARG, "slot not allocated");
    const int w = field_width(kind);
    if (w == 0) return fail(GPE_ERR_INVALID_ARG, "unknown field kind");
    const int C = h->g.C;
    if ((kind == GPE_FIELD_SPIN || kind == GPE_FIELD_UV_THETA) && C == 1)
        return fail(GPE_ERR_UNSUPPORTED, "spin fields need a spinor (C = 3 or 5)");
    if ((kind == GPE_FIELD_MAX_HAMILTON || kind == GPE_FIELD_PROJ_X || kind == GPE_FIELD_PROJ_Y) && C != 3)
        return fail(GPE_ERR_UNSUPPORTED, "this field is defined for spin-1 (C = 3)");
    const uint64_t nodes = (uint64_t)h->g.X * h->g.Y * h->g.Z * h->g.V;
    const size_t need = (size_t)nodes * w;
    if (need > h->field_count) {
        if (h->field_buf) cudaFree(h->field_buf);
        h->field_buf = nullptr;
        h->field_count = 0;
        if (cudaMalloc(&h->field_buf, need * sizeof(double)) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (node fields)");
        h->field_count = need;
    }
    gpe_fields B;
    std::memset(&B, 0, sizeof B);
    if (h->has_ramp) gpe_ramp_eval(&h->ramp, h->ramp.time_scale * t, &B);
    StepArgs a = make_args(h, B, t);
    a.prev = h->interior[slot];
    cudaError_t e = h->real_bytes == 8 ? launch_fields<double>(a, C, kind, h->field_buf, s)
                                       : launch_fields<float>(a, C, kind, h->field_buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "node fields launch");
    h->launches += 1;
    *width = w;
    return GPE_OK;
}

}  // namespace gpe

using namespace gpe;

extern "C" gpe_status gpe_node_field_count(const gpe_handle* h, int32_t kind, size_t* per_node, size_t* count) {
    if (!h || !per_node || !count) return fail(GPE_ERR_INVALID_ARG, "null argument");
    const int w = field_width(kind);
    if (w == 0) return fail(GPE_ERR_INVALID_ARG, "unknown field kind");
    *per_node = (size_t)w;
    *count = (size_t)h->g.X * h->g.Y * h->g.Z * h->g.V * (size_t)w;
    return GPE_OK;
}

extern "C" gpe_status gpe_node_fields(gpe_handle* h, int32_t slot, int32_t kind, double t, double* out, size_t count,
                                      void* stream) {
    if (!h || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    int w = 0;
    const uint64_t nodes = (uint64_t)h->g.X * h->g.Y * h->g.Z * h->g.V;
    if (field_width(kind) && count != (size_t)nodes * field_width(kind))
        return fail(GPE_ERR_INVALID_ARG, "count must be nodes x values per node (gpe_node_field_count)");
    gpe_status st = compute_fields(h, slot, kind, t, s, &w);
    if (st) return st;
    const cudaError_t e = cudaMemcpyAsync(out, h->field_buf, count * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "node fields copy");
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (e2 != cudaSuccess) return cuda_fail(e2, "node fields");
    return GPE_OK;
}

extern "C" gpe_status gpe_node_fields_reduce(gpe_handle* h, int32_t slot, int32_t kind, double t, double* out,
                                             void* stream) {
    if (!h || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (kind != GPE_FIELD_DENSITY && kind != GPE_FIELD_SPIN && kind != GPE_FIELD_MAX_HAMILTON)
        return fail(GPE_ERR_UNSUPPORTED, "reductions exist for DENSITY, SPIN and MAX_HAMILTON");
    cudaStream_t s = (cudaStream_t)stream;
    int w = 0;
    gpe_status st = compute_fields(h, slot, kind, t, s, &w);
    if (st) return st;
    const uint64_t nodes = (uint64_t)h->g.X * h->g.Y * h->g.Z * h->g.V;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned nb = (unsigned)std::min<uint64_t>((nodes + 255) / 256, 8ull * (uint64_t)(sms > 0 ? sms : 1));
    nb = (unsigned)std::min<size_t>(nb, h->partial_blocks * OBS_COUNT / 5);
    if (nb == 0) nb = 1;
    fields_reduce_kernel<<<nb, 256, 0, s>>>(h->field_buf, nodes, kind, h->partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "node fields reduction");
    h->launches += 1;
    std::vector<double> part((size_t)nb * 5);
    e = cudaMemcpyAsync(part.data(), h->partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "node fields reduction copy");
    const int nout = kind == GPE_FIELD_SPIN ? 5 : 1;
    const bool is_max = kind == GPE_FIELD_MAX_HAMILTON;
    const double dv = cell_dv(h);
    for (int k = 0; k < nout; ++k) {
        double v = is_max ? -INFINITY : 0.0;
        for (unsigned b = 0; b < nb; ++b) v = is_max ? std::fmax(v, part[(size_t)b * 5 + k]) : v + part[(size_t)b * 5 + k];
        out[k] = is_max ? v : v * dv;
    }
    return GPE_OK;
}
